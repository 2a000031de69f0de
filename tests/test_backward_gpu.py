"""Backward (gbr_rmsd_backward and the torch.autograd.Function) against the
FP64 oracle gradient and central finite differences (h = 1e-3 Angstrom).
Tolerance: 1e-5 relative, normwise -- against the FP64 gradient (largest
absolute error over the largest entry) and against finite differences (2-norm
over 64 sampled coordinates).  The gradient is FP32 and its per-atom terms are
assembled from FP32 sums: its absolute error is ~2-3e-7 of the largest entry,
so a coordinate 1000 times smaller than the largest carries a relative error
of up to a few 1e-4.  Per coordinate, the finite-difference test therefore
bounds coordinates of at least 1 % of the largest entry, at 1e-4."""
import numpy as np
import pytest

import oracle
from cpptraj_gb300 import gbrmsd, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def h():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    hd = gbrmsd.Handle(0)
    yield hd
    hd.close()


@pytest.mark.parametrize("weighted", [False, True])
def test_gradient_matches_fp64(h, weighted):
    X, m = synth.trajectory(4, 96, 180, 1.0, 1.0, np.float32, weighted)
    rng = np.random.default_rng(1)
    g = rng.uniform(0.5, 1.5, 96 * 95 // 2).astype(np.float32)
    grad = h.backward(X, mass=m, g=g)
    ref = oracle.grad_f64(X, mass=m, g=g)
    err = np.abs(grad - ref).max() / np.abs(ref).max()
    assert err <= 1e-5, err


def test_gradient_deep_stage_shape(h):
    # from 1,280 atoms the pair pass runs the deep-stage shape of the kernel
    X, m = synth.trajectory(5, 90, 1400, 0.5, 1.5, np.float32, True)
    rng = np.random.default_rng(3)
    g = rng.uniform(0.5, 1.5, 90 * 89 // 2).astype(np.float32)
    r = np.zeros(90 * 89 // 2, np.float32)
    grad = h.backward(X, mass=m, g=g, rmsd_out=r)
    ref = oracle.grad_f64(X, mass=m, g=g)
    err = np.abs(grad - ref).max() / np.abs(ref).max()
    assert err <= 1e-5, err
    assert np.abs(r - oracle.allpairs_f64(X, tgt_mass=m)).max() <= 1e-4


def test_gradient_matches_finite_differences(h):
    X, m = synth.trajectory(40, 128, 300, 1.0, 1.0, np.float32, False)
    grad = h.backward(X)
    rng = np.random.default_rng(2)
    gmax = float(np.abs(grad).max())
    got, fds = [], []
    for _ in range(64):
        f, a, p = int(rng.integers(0, 128)), int(rng.integers(0, 300)), int(rng.integers(0, 3))
        fds.append(oracle.fd_f64(X, f, a, p, 1e-3))
        got.append(float(grad[f, a, p]))
    got, fds = np.array(got), np.array(fds)
    rel = np.linalg.norm(got - fds) / np.linalg.norm(fds)
    assert rel <= 1e-5, rel
    big = np.abs(fds) >= 1e-2 * gmax
    assert big.sum() >= 32
    assert (np.abs(got - fds)[big] / np.abs(fds[big])).max() <= 1e-4


def test_forward_output_of_backward(h):
    X, _ = synth.trajectory(41, 70, 90, 0.5, 1.5, np.float32, False)
    r = np.zeros(70 * 69 // 2, np.float32)
    h.backward(X, rmsd_out=r)
    ref = oracle.allpairs_f64(X)
    assert np.abs(r - ref).max() <= 1e-4


def test_autograd_function():
    torch = pytest.importorskip("torch")
    from cpptraj_gb300.torch_ext import allpairs_rmsd
    X, _ = synth.trajectory(42, 64, 120, 1.0, 1.0, np.float32, False)
    x = torch.from_numpy(X).cuda().requires_grad_(True)
    tri = allpairs_rmsd(x, precision="fp32")
    w = torch.linspace(0.5, 1.5, tri.numel(), device="cuda")
    (tri * w).sum().backward()
    ref = oracle.grad_f64(X, g=w.cpu().numpy())
    err = np.abs(x.grad.cpu().numpy() - ref).max() / np.abs(ref).max()
    assert err <= 1e-5, err
    np.testing.assert_allclose(tri.detach().cpu().numpy(), oracle.allpairs_f64(X), atol=1e-4)
