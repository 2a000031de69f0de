"""GPU parity of the rms2d `dme` mode (Frame::DISTRMSD, src/Frame.cpp:1313-1344)
through the C ABI, against the reference's golden file, cpptraj's own Frame
code (ref_pairs.npz) and the FP64 oracle.

Tolerances: 1e-5 Angstrom for the FP32 kernels (FP32-rounded distances with
compensated sums; DME values here are 0.1-10 Angstrom), and float32 output
rounding (2e-6 relative) for GBR_PREC_FP64.
"""
import os

import numpy as np
import pytest

import oracle
from cpptraj_gb300 import gbrmsd, synth

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL32 = 1e-5


@pytest.fixture(scope="module")
def h():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    hd = gbrmsd.Handle(0)
    yield hd
    hd.close()


def square(tri, n):
    M = np.zeros((n, n))
    M[np.triu_indices(n, 1)] = tri
    return M + M.T


def fmt3(M):
    return np.array([[float("%8.3f" % v) for v in row] for row in M])


def check(got, want, precision):
    got = np.asarray(got, np.float64)
    if precision == "fp64":
        np.testing.assert_allclose(got, want, rtol=2e-6, atol=1e-7)
    else:
        np.testing.assert_allclose(got, want, rtol=0, atol=TOL32)


@pytest.mark.parametrize("precision", ["fp32", "tc", "fp64"])
def test_tz2_dme_golden(h, precision):
    # Test_2DRMS unit 4: `2drms crd1 :3-7 rmsout dme.dat dme` on tz2 frames 1-10
    tz2 = np.load(os.path.join(GOLD, "tz2_rms2d.npz"))
    X = tz2["fit_xyz"]
    out = h.allpairs(X, mode="dme", precision=precision)
    assert np.array_equal(fmt3(square(out, 10)), tz2["dme_save"])
    check(out, oracle.allpairs_f64(X, mode=oracle.DME), precision)
    assert h.stats()["precision"] == (2 if precision == "fp64" else 0)


def test_dme_matches_reference_frame_code(h):
    refp = np.load(os.path.join(GOLD, "ref_pairs.npz"))
    out = h.allpairs(refp["xyz"], mode="dme", precision="fp32")
    # cpptraj's own DISTRMSD output (float) and its FP64 restatement
    np.testing.assert_allclose(out, refp["tri_dme"], rtol=0, atol=TOL32)
    check(out, oracle.allpairs_f64(refp["xyz"], mode=oracle.DME), "fp32")


@pytest.mark.parametrize("F,N", [(2, 2), (3, 5), (65, 4), (67, 129), (129, 31), (200, 304)])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_dme_ragged_shapes(h, F, N, dtype):
    X, _ = synth.trajectory(300 + F + N, F, N, 0.3, 2.5, dtype, False)
    want = oracle.allpairs_f64(X, mode=oracle.DME)
    for precision in ("fp32", "fp64"):
        check(h.allpairs(X, mode="dme", precision=precision), want, precision)


def test_dme_one_atom_is_nan(h):
    # Nd = 0: the reference divides 0 by 0
    X = np.random.default_rng(1).normal(size=(5, 1, 3)).astype(np.float32)
    out = h.allpairs(X, mode="dme")
    assert out.shape == (10,) and np.all(np.isnan(out))
    assert np.all(np.isnan(oracle.allpairs(X, mode=oracle.DME)))


def test_dme_full_two_sets_and_row_ranges(h):
    A, _ = synth.trajectory(41, 70, 57, 0.2, 2.0, np.float32, False)
    B, _ = synth.trajectory(42, 133, 57, 0.2, 2.0, np.float32, False)
    want = oracle.allpairs_f64(A, B, mode=oracle.DME)  # FULL: index jt * n_ref + i
    full = h.allpairs(A, B, mode="dme")
    check(full, want, "fp32")
    # FULL rows are target frames; TRI rows reference frames
    parts = [h.allpairs(A, B, mode="dme", row_begin=a, row_end=b) for a, b in ((0, 50), (50, 51), (51, 133))]
    assert np.array_equal(np.concatenate(parts), full)
    tri = h.allpairs(B, mode="dme")
    parts = [h.allpairs(B, mode="dme", row_begin=a, row_end=b) for a, b in ((0, 64), (64, 100), (100, 133))]
    assert np.array_equal(np.concatenate(parts), tri)


def test_dme_device_buffers_and_identical_frames(h):
    torch = pytest.importorskip("torch")
    X, _ = synth.trajectory(7, 90, 64, 0.5, 1.5, np.float32, False)
    X[10] = X[3]  # identical frames: DME exactly 0
    dX = torch.from_numpy(X).cuda()
    out = h.allpairs(dX, mode="dme").cpu().numpy()
    np.testing.assert_array_equal(out, h.allpairs(X, mode="dme"))
    assert out[oracle.tri_index(90, 3, 10)] == 0.0
    check(out, oracle.allpairs_f64(X, mode=oracle.DME), "fp32")


def test_dme_chunked_atom_pairs(h):
    # 4,200 frames x 700 atoms: the FP32 distance planes (4,224 columns x
    # 244,650 atom pairs = 4.1 GB) exceed the 2 GB chunk budget, so the atom
    # pairs are processed in two chunks that accumulate into the same sums.
    X, _ = synth.trajectory(77, 4200, 700, 0.5, 2.0, np.float32, False)
    out = h.allpairs(X, mode="dme")
    assert h.stats()["kernel_launches"] == 5  # 2 x (distances + pairs) + final
    rng = np.random.default_rng(3)
    pi = rng.integers(0, 4199, 64)
    pj = np.array([rng.integers(i + 1, 4200) for i in pi])
    want = oracle.pairs_f64(X, pi, pj, mode=oracle.DME)
    got = out[[oracle.tri_index(4200, i, j) for i, j in zip(pi, pj)]]
    check(got, want, "fp32")
