"""GPU parity of gbr_cluster_centroids -- Metric_RMS::CalculateCentroid
(src/Cluster/Metric_RMS.cpp:86-108) -- through the C ABI, against cpptraj's own
Frame code run in the same steps (ref_centroids.npz) and the FP64 oracle.

Tolerances: the kernel sums per atom in FP32 (centring, covariance; the
running sum is an FP32 hi + lo pair), solves the first 32 fits of a chain in
FP64 and the later ones in FP32, so a fitted centroid agrees with the FP64
chain to ~2e-7 of its coordinates' magnitude (2-3 FP32 ulps of the input):
1e-6 Angstrom + 3e-7 x max |coordinate| here.  No-fit centroids are sums kept
to ~1e-14 relative (FP64 inputs as FP32 hi + lo): 1e-10 Angstrom.
"""
import os

import numpy as np
import pytest

import oracle
from cpptraj_gb300 import gbrmsd, synth

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL_NOFIT = 1e-10


def tol_fit(want):
    return 1e-6 + 3e-7 * np.nanmax(np.abs(want))


@pytest.fixture(scope="module")
def h():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    hd = gbrmsd.Handle(0)
    yield hd
    hd.close()


def check(got, want, offsets, tol):
    sizes = np.diff(offsets)
    np.testing.assert_allclose(got[sizes > 0], want[sizes > 0], rtol=0, atol=tol)
    assert np.all(np.isnan(got[sizes == 0]))


@pytest.mark.parametrize("tag", ["fit_w", "fit_u", "nofit"])
def test_centroids_match_reference_code(h, tag):
    g = np.load(os.path.join(GOLD, "ref_centroids.npz"))
    m = g["mass"] if tag == "fit_w" else None
    mode = "nofit" if tag == "nofit" else "fit"
    got = h.cluster_centroids(g["xyz"], g["members"], g["offsets"], mass=m, mode=mode)
    check(got, g[tag], g["offsets"], TOL_NOFIT if tag == "nofit" else tol_fit(g[tag]))


@pytest.mark.parametrize("F,N,K", [(2000, 500, 20), (300, 3000, 3), (64, 4, 5), (257, 129, 1)])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("weighted", [True, False])
def test_centroids_vs_oracle(h, F, N, K, dtype, weighted):
    X, m = synth.trajectory(600 + F + N, F, N, 0.4, 2.0, dtype, weighted)
    labels = np.random.default_rng(F + K).integers(0, K, F)
    members, offsets = oracle.members_offsets(labels, K)
    for mode in ("fit", "nofit"):
        want = oracle.cluster_centroids_f64(X, members, offsets, mass=m,
                                            mode=oracle.FIT if mode == "fit" else oracle.NOFIT)
        got = h.cluster_centroids(X, members, offsets, mass=m, mode=mode)
        check(got, want, offsets, tol_fit(want) if mode == "fit" else TOL_NOFIT)


def test_centroids_member_order_and_device_buffers(h):
    torch = pytest.importorskip("torch")
    X, m = synth.trajectory(81, 400, 200, 0.5, 2.0, np.float32, True)
    # members in a scrambled (not increasing) order, a frame in two clusters
    rng = np.random.default_rng(5)
    members = np.concatenate([rng.permutation(400)[:150], rng.permutation(400)[:90], [3]]).astype(np.int32)
    offsets = np.array([0, 150, 150, 240, 241], np.int64)
    want = oracle.cluster_centroids_f64(X, members, offsets, mass=m)
    got = h.cluster_centroids(torch.from_numpy(X).cuda(), torch.from_numpy(members).cuda(),
                              torch.from_numpy(offsets).cuda(), mass=torch.from_numpy(m).cuda())
    assert got.is_cuda
    check(got.cpu().numpy(), want, offsets, tol_fit(want))
    # the order of the chain matters: reversing a cluster moves its centroid
    rev = members.copy()
    rev[:150] = rev[:150][::-1]
    other = oracle.cluster_centroids_f64(X, rev, offsets, mass=m)
    assert np.abs(other[0] - want[0]).max() > 10 * tol_fit(want)
    check(h.cluster_centroids(X, rev, offsets, mass=m), other, offsets, tol_fit(other))


def test_centroids_errors(h):
    X = np.zeros((4, 5, 3), np.float32)
    off = np.array([0, 2], np.int64)
    with pytest.raises(gbrmsd.GbrError) as e:
        h.cluster_centroids(X, np.array([0, 4], np.int32), off)  # frame 4 of 4
    assert e.value.code == 1
    with pytest.raises(gbrmsd.GbrError) as e:
        h.cluster_centroids(X, np.array([0, 1], np.int32), np.array([0, 2, 1], np.int64))
    assert e.value.code == 1
    with pytest.raises(gbrmsd.GbrError) as e:
        h.cluster_centroids(X, np.array([0, 1], np.int32), off, mass=np.zeros(5))
    assert e.value.code == 4
    # no-fit does not divide by the mass
    out = h.cluster_centroids(X, np.array([0, 1], np.int32), off, mass=np.zeros(5), mode="nofit")
    assert np.array_equal(out, np.zeros((1, 5, 3)))
    assert h.cluster_centroids(X, np.zeros(0, np.int32), np.zeros(1, np.int64)).shape == (0, 5, 3)
