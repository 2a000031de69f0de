"""GPU parity of gbr_superpose -- the per-frame fit of the rms / align actions
(Action_Rmsd::DoAction, Action_Align::DoAction) -- through the C ABI, against
cpptraj's own RMSD_CenteredRef(ref, U, Trans) + Trans_Rot_Trans output
(ref_superpose.npz) and the FP64 oracle.

Both sides compute in FP64, so the tolerances are FP64-level: RMSD 1e-9
Angstrom (2e-6 below 1e-5 Angstrom: for a frame fitted onto itself E0 - lambda
is FP64 rounding noise, sqrt(2 eps E0 / W) ~ 1e-6 Angstrom at these sizes,
which the reference's Jacobi path and QCP round differently), rotation
entries 1e-8 (QCP here, Jacobi in the reference),
translations 1e-10 Angstrom, moved coordinates 1e-8 Angstrom in FP64 and the
float32 rounding of the result (1e-5 Angstrom at these magnitudes) in FP32.
"""
import os

import numpy as np
import pytest

import oracle
from cpptraj_gb300 import gbrmsd, synth

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def h():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    hd = gbrmsd.Handle(0)
    yield hd
    hd.close()


def rmsd_close(got, want, tol_far=1e-9):
    got, want = np.asarray(got), np.asarray(want)
    tol = np.where(np.minimum(got, want) < 1e-5, 2e-6, tol_far)
    assert np.all(np.abs(got - want) <= tol), np.abs(got - want).max()


def close(got, want):
    rmsd, rot, tt, rt = got
    rmsd_close(rmsd, want[0])
    np.testing.assert_allclose(rot, want[1], rtol=0, atol=1e-8)
    np.testing.assert_allclose(tt, want[2], rtol=0, atol=1e-10)
    np.testing.assert_allclose(rt, want[3], rtol=0, atol=1e-10)


@pytest.mark.parametrize("wt", ["w", "u"])
def test_superpose_matches_reference_code(h, wt):
    g = np.load(os.path.join(GOLD, "ref_superpose.npz"))
    X = g["xyz"]
    m = g["mass"] if wt == "w" else None
    move = g["move"].copy()  # FP64 frames: the align move set is separate from the fit atoms
    got = h.superpose(X[5].astype(np.float64), X.astype(np.float64), mass=m, move=move)
    want = (g[f"rmsd_{wt}"], g[f"rot_{wt}"], g[f"tgt_trans_{wt}"], g[f"ref_trans_{wt}"])
    close(got, want)
    np.testing.assert_allclose(move, g[f"moved_{wt}"], rtol=0, atol=1e-8)


@pytest.mark.parametrize("F,N", [(1, 1), (3, 2), (37, 3), (65, 129), (300, 2000)])
@pytest.mark.parametrize("weighted", [True, False])
def test_superpose_vs_oracle(h, F, N, weighted):
    X, m = synth.trajectory(500 + F + N, F, N, 0.1, 3.0, np.float32, weighted)
    R = synth.trajectory(501 + N, 1, N, 0.5, 0.5, np.float32, False)[0][0]
    want = oracle.superpose_f64(R, X, mass=m)
    got = h.superpose(R, X, mass=m)
    # 1- to 3-atom frames (collinear or coplanar): a rank-deficient covariance,
    # whose zero eigenvalue enters the reference's RMSD as sig3*sqrt(|mu3|),
    # i.e. sqrt(eps)-level noise
    rmsd_close(got[0], want[0], 1e-9 if N >= 4 else 1e-6)
    if N >= 3:  # rotations of 1- and 2-atom frames are not unique
        np.testing.assert_allclose(got[1], want[1], rtol=0, atol=1e-8)
    np.testing.assert_allclose(got[2], want[2], rtol=0, atol=1e-10)
    np.testing.assert_allclose(got[3], want[3], rtol=0, atol=1e-10)


def test_superpose_fp32_move_in_place_on_device(h):
    torch = pytest.importorskip("torch")
    X, m = synth.trajectory(61, 500, 300, 0.2, 2.0, np.float32, True)
    full, _ = synth.trajectory(62, 500, 800, 0.5, 1.0, np.float32, False)
    rm = np.linspace(1.0, 2.0, 300)  # reference masses differ from the target's
    want = oracle.superpose_f64(X[17], X, ref_mass=rm, mass=m, move=full.astype(np.float64))
    dX, dmove = torch.from_numpy(X).cuda(), torch.from_numpy(full).cuda()
    got = h.superpose(torch.from_numpy(X[17]).cuda(), dX, mass=torch.from_numpy(m).cuda(),
                      ref_mass=torch.from_numpy(rm).cuda(), move=dmove)
    close(tuple(t.cpu().numpy() for t in got), want[:4])
    np.testing.assert_allclose(dmove.cpu().numpy(), want[4], rtol=0, atol=1e-4)
    # the reference is centred with its own masses, frame 17 with the target's:
    # the same coordinates are a nonzero RMSD apart here
    assert got[0][17].item() > 0.1


def test_superpose_nofit(h):
    X, m = synth.trajectory(71, 90, 64, 0.5, 1.5, np.float64, True)
    want = oracle.superpose_f64(X[0], X, mass=m, mode=oracle.NOFIT)
    move = X.copy()
    got = h.superpose(X[0], X, mass=m, mode="nofit", move=move)
    close(got, want[:4])
    np.testing.assert_array_equal(move, X)  # nofit moves nothing
    np.testing.assert_allclose(got[0], oracle.allpairs_f64(X[:1], X, tgt_mass=m, mode=oracle.NOFIT), atol=1e-9)


def test_superpose_errors(h):
    X = np.zeros((4, 5, 3), np.float32)
    with pytest.raises(gbrmsd.GbrError) as e:
        h.superpose(X[0], X, mass=np.zeros(5))
    assert e.value.code == 4
    with pytest.raises(gbrmsd.GbrError) as e:
        h.superpose(X[0], X, mode=2)  # DME is not a fit mode
    assert e.value.code == 1
    r = h.superpose(X[0], X[:0])
    assert r[0].shape == (0,)
