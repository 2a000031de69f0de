"""gbr_allpairs_batched: many independent trajectories in one call (config 3
shape, reduced sizes), through the C ABI, against the oracle and against one
gbr_allpairs call per trajectory.  Covers host and device pointers, the
captured-graph replay of a repeated batch, and a changed batch."""
import ctypes

import numpy as np
import pytest

import oracle
from cpptraj_gb300 import gbrmsd, synth

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.fixture(scope="module")
def h():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    hd = gbrmsd.Handle(0)
    yield hd
    hd.close()


def make_batch(seed, n=12, frange=(2, 300), nrange=(1, 700)):
    rng = np.random.default_rng(seed)
    trajs, masses = [], []
    for t in range(n):
        F = int(rng.integers(frange[0], frange[1] + 1))
        N = int(rng.integers(nrange[0], nrange[1] + 1))
        X, m = synth.trajectory(seed * 1000 + t, F, N, 0.1, 3.0, np.float32, True)
        trajs.append(X)
        masses.append(m if t % 3 else None)
    return trajs, masses


def device_batch(h, trajs, masses, mode, precision):
    import torch
    dX = [torch.from_numpy(X).cuda() for X in trajs]
    dm = [None if m is None else torch.from_numpy(m).cuda() for m in masses]
    outs = [torch.zeros(max(X.shape[0] * (X.shape[0] - 1) // 2, 1), device="cuda") for X in trajs]
    n = len(trajs)
    P = ctypes.c_void_p * n
    xyz = P(*[x.data_ptr() for x in dX])
    nf = (ctypes.c_int64 * n)(*[X.shape[0] for X in trajs])
    na = (ctypes.c_int32 * n)(*[X.shape[1] for X in trajs])
    ms = P(*[None if m is None else m.data_ptr() for m in dm])
    op = P(*[o.data_ptr() for o in outs])
    m = gbrmsd.MODES[mode]
    p = gbrmsd.PRECISIONS[precision]

    def call():
        h._check(h.lib.gbr_allpairs_batched(h.h, n, ctypes.cast(xyz, ctypes.c_void_p), ctypes.cast(nf, ctypes.c_void_p),
                                            ctypes.cast(na, ctypes.c_void_p), ctypes.cast(ms, ctypes.c_void_p), m, p,
                                            ctypes.cast(op, ctypes.c_void_p)))
        return [o[: X.shape[0] * (X.shape[0] - 1) // 2].cpu().numpy() for o, X in zip(outs, trajs)]
    return call


@pytest.mark.parametrize("precision", ["fp32", "tc", "fp64"])
@pytest.mark.parametrize("mode", ["fit", "nofit"])
def test_batched_host_matches_oracle(h, precision, mode):
    trajs, masses = make_batch(3)
    try:
        outs = h.allpairs_batched(trajs, masses, mode=mode, precision=precision)
    except gbrmsd.GbrError as e:
        if e.code == 6:
            pytest.skip("tensor cores not available")
        raise
    for X, m, o in zip(trajs, masses, outs):
        ref = oracle.allpairs_f64(X, tgt_mass=m, mode=oracle.FIT if mode == "fit" else oracle.NOFIT)
        assert o.size == ref.size
        if ref.size:
            # FP64 mode: FP64 arithmetic, then the float32 store (half an ulp of the value)
            tol = 2e-6 + 6e-8 * np.abs(ref) if precision == "fp64" else TOL
            assert np.all(np.abs(o - ref) <= tol)


@pytest.mark.parametrize("precision", ["fp32", "tc"])
def test_batched_device_graph_replay(h, precision):
    trajs, masses = make_batch(5, n=20)
    call = device_batch(h, trajs, masses, "fit", precision)
    try:
        first = call()
    except gbrmsd.GbrError as e:
        if e.code == 6:
            pytest.skip("tensor cores not available")
        raise
    second = call()  # same signature: replays the captured graph
    for X, m, a, b in zip(trajs, masses, first, second):
        np.testing.assert_array_equal(a, b)
        ref = oracle.allpairs_f64(X, tgt_mass=m)
        if ref.size:
            assert np.abs(a - ref).max() <= TOL
    # a different batch (new signature) is captured again and still right
    trajs2, masses2 = make_batch(6, n=7)
    outs2 = device_batch(h, trajs2, masses2, "fit", precision)()
    for X, m, o in zip(trajs2, masses2, outs2):
        ref = oracle.allpairs_f64(X, tgt_mass=m)
        if ref.size:
            assert np.abs(o - ref).max() <= TOL


def test_batched_matches_single_calls(h):
    trajs, masses = make_batch(7, n=6, frange=(50, 200), nrange=(30, 400))
    outs = h.allpairs_batched(trajs, masses, precision="fp32")
    for X, m, o in zip(trajs, masses, outs):
        single = h.allpairs(X, tgt_mass=m, precision="fp32")
        assert np.abs(o - single).max() <= 2e-6


def test_batched_errors(h):
    trajs, masses = make_batch(8, n=3)
    masses[1] = np.zeros(trajs[1].shape[1])
    with pytest.raises(gbrmsd.GbrError) as e:
        h.allpairs_batched(trajs, masses)
    assert e.value.code == 4
