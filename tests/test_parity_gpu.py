"""GPU parity: libgbrmsd (through its C ABI) against the CPU oracle and the
reference's golden files.

Tolerances: 1e-4 Angstrom against the FP64 oracle for the FP32 and
tensor-core paths (the bar stated for this path); GBR_PREC_FP64 within 2e-6
(float32 output rounding plus QCP vs Jacobi eigen step).
"""
import os

import numpy as np
import pytest

import oracle
from cpptraj_gb300 import gbrmsd, synth

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL = 1e-4


def _precisions():
    return ["fp32", "tc", "fp64"]


@pytest.fixture(scope="module")
def h():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if not os.path.exists(gbrmsd.LIB_PATH):
        from cpptraj_gb300 import build
        build.build()
    hd = gbrmsd.Handle(0)
    yield hd
    hd.close()


def run(h, *a, precision="fp32", **k):
    try:
        return h.allpairs(*a, precision=precision, **k)
    except gbrmsd.GbrError as e:
        if e.code == 6 and precision == "tc":
            pytest.skip("tensor-core path not available")
        raise


def square(tri, n):
    M = np.zeros((n, n))
    M[np.triu_indices(n, 1)] = tri
    return M + M.T


def fmt3(M):
    return np.array([[float("%8.3f" % v) for v in row] for row in M])


@pytest.fixture(scope="module")
def tz2():
    return np.load(os.path.join(GOLD, "tz2_rms2d.npz"))


@pytest.mark.parametrize("precision", _precisions())
@pytest.mark.parametrize("save,xyz,mass,mode", [
    ("rmsd_save", "fit_xyz", None, "fit"),
    ("rmsd_mass_save", "fit_xyz", "fit_mass", "fit"),
    ("nofit_save", "nofit_xyz", None, "nofit"),
])
def test_tz2_golden(h, tz2, precision, save, xyz, mass, mode):
    out = run(h, tz2[xyz], tgt_mass=tz2[mass] if mass else None, mode=mode, precision=precision)
    ref = oracle.allpairs(tz2[xyz], tgt_mass=tz2[mass] if mass else None,
                          mode=oracle.FIT if mode == "fit" else oracle.NOFIT)
    assert np.abs(out - ref).max() <= TOL
    got = fmt3(square(out, 10))
    # printed at %8.3f: allow a last-digit flip only where the oracle sits on a rounding edge
    diff = np.abs(got - tz2[save])
    assert diff.max() <= 1.0001e-3
    assert (diff > 0).sum() <= 2


@pytest.mark.parametrize("precision", _precisions())
def test_tz2_full_ref_mask(h, tz2, precision):
    out = run(h, tz2["trp_ref_xyz"], tz2["trp_tgt_xyz"], precision=precision)
    M = np.asarray(out).reshape(10, 10)
    ref = oracle.allpairs(tz2["trp_ref_xyz"], tz2["trp_tgt_xyz"]).reshape(10, 10)
    assert np.abs(M - ref).max() <= TOL
    assert np.abs(fmt3(M) - tz2["trp_save"]).max() <= 1.0001e-3


def _check(h, X, m, precision, mode="fit", tol=TOL, **kw):
    out = run(h, X, tgt_mass=m, mode=mode, precision=precision, **kw)
    ref = oracle.allpairs_f64(X, tgt_mass=m, mode=oracle.FIT if mode == "fit" else oracle.NOFIT)
    err = np.abs(out.astype(np.float64) - ref)
    assert err.max() <= tol, (err.max(), h.stats())
    return err.max()


@pytest.mark.parametrize("precision", _precisions())
def test_c0_shape(h, precision):
    X, _ = synth.workload_c0()  # the stated 500 frames x 304 atoms, FP64
    _check(h, X, None, precision, tol=2e-6 if precision == "fp64" else TOL)


@pytest.mark.parametrize("precision", _precisions())
def test_c1_shape_mass_weighted(h, precision):
    X, m = synth.trajectory(1, 200, 2000, 0.1, 3.0, np.float32, True)
    _check(h, X, m, precision, tol=2e-6 if precision == "fp64" else TOL)


@pytest.mark.parametrize("precision", ["fp32", "tc"])
def test_clustered_frames(h, precision):
    X, lab = synth.clustered(2, 300, 500, 20, 0.8)
    _check(h, X, None, precision)
    assert h.stats()["n_refs"] >= 2


@pytest.mark.parametrize("pipeline", [1, 2, 3, 4])
@pytest.mark.parametrize("precision", ["fp32", "tc"])
def test_clustered_sorted_layout(h, pipeline, precision):
    # frames from 12 interleaved centroids: a whole triangle is computed over
    # frames re-ordered by reference, a row range over the original order
    X, _ = synth.clustered(5, 700, 300, 12, 0.8)
    ref = oracle.allpairs_f64(X)
    h.set_option(gbrmsd.OPT_TC_PIPELINE, pipeline)
    try:
        out = run(h, X, precision=precision)
        st = h.stats()
        assert st["n_refs"] >= 2
        assert np.abs(out - ref).max() <= TOL
        assert st["pairs_fixed"] <= st["pairs"] // 100, st
        part = run(h, X, precision=precision, row_begin=100, row_end=400)
        lo = 100 * 700 - 100 * 101 // 2
        hi = 400 * 700 - 400 * 401 // 2
        assert np.abs(part - ref[lo:hi]).max() <= TOL
    finally:
        h.set_option(gbrmsd.OPT_TC_PIPELINE, gbrmsd.TC_PIPELINE_DEFAULT)


@pytest.mark.parametrize("pipeline", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("precision", ["fp32", "tc"])
def test_clustered_full_row_ranges_bit_identical(h, pipeline, precision):
    # FULL output between two clustered sets: row ranges (target frames) shift
    # the tiles, so a pair whose references are its tile's reads the tile's
    # staged frame terms in one call and forms them from global memory in
    # another.  Both use the same rounded arithmetic: the same bits.
    X, _ = synth.clustered(5, 700, 300, 12, 0.8)
    A, B = X[:300], X[300:]
    h.set_option(gbrmsd.OPT_TC_PIPELINE, pipeline)
    try:
        whole = run(h, A, B, precision=precision)
        assert h.stats()["n_refs"] >= 2
        parts = [run(h, A, B, precision=precision, row_begin=a, row_end=b)
                 for a, b in ((0, 1), (1, 77), (77, 333), (333, 400))]
        np.testing.assert_array_equal(np.concatenate(parts), whole)
    finally:
        h.set_option(gbrmsd.OPT_TC_PIPELINE, gbrmsd.TC_PIPELINE_DEFAULT)


@pytest.mark.parametrize("pipeline", [0, 3, 4])
@pytest.mark.parametrize("precision", ["fp32", "tc"])
def test_clustered_tri_sorted_vs_rows(h, pipeline, precision):
    # A whole triangle over reference-sorted positions computes some pairs
    # with their two frames' roles exchanged (the RMSD is symmetric, its last
    # bit need not be); row ranges keep the original order.
    X, _ = synth.clustered(5, 700, 300, 12, 0.8)
    h.set_option(gbrmsd.OPT_TC_PIPELINE, pipeline)
    try:
        whole = run(h, X, precision=precision)
        parts = np.concatenate([run(h, X, precision=precision, row_begin=a, row_end=b)
                                for a, b in ((0, 1), (1, 250), (250, 699), (699, 700))])
        np.testing.assert_allclose(parts, whole, rtol=4e-7, atol=1e-7)
    finally:
        h.set_option(gbrmsd.OPT_TC_PIPELINE, gbrmsd.TC_PIPELINE_DEFAULT)


@pytest.mark.parametrize("precision", ["fp32", "tc"])
def test_many_references(h, precision):
    # widely scattered frames (independent displacements up to 3 A over 300
    # atoms): the k-centre choice goes past 32 references when allowed 64
    X, m = synth.trajectory(5, 3000, 300, 0.1, 3.0, np.float32, True)
    h.set_option(gbrmsd.OPT_MAX_REFS, 64)
    try:
        _check(h, X, m, precision)
        assert h.stats()["n_refs"] > 32, h.stats()
    finally:
        h.set_option(gbrmsd.OPT_MAX_REFS, 32)


@pytest.mark.parametrize("precision", ["fp32", "tc"])
def test_nofit_clustered(h, precision):
    # several references without fitting (the k-centre scans then fit every frame)
    X, _ = synth.clustered(7, 400, 200, 6, 0.8)
    _check(h, X, None, precision, mode="nofit")


@pytest.mark.parametrize("precision", _precisions())
def test_nofit(h, precision):
    X, m = synth.trajectory(8, 130, 77, 0.2, 2.0, np.float32, True)
    _check(h, X, m, precision, mode="nofit")


@pytest.mark.parametrize("precision", _precisions())
def test_full_different_masses(h, precision):
    rng = np.random.default_rng(3)
    A, _ = synth.trajectory(4, 70, 150, 0.3, 1.5, np.float32, False)
    B, _ = synth.trajectory(5, 90, 150, 0.3, 1.5, np.float32, False)
    mr = synth.masses(rng, 150)
    mt = synth.masses(rng, 150)
    out = run(h, A, B, ref_mass=mr, tgt_mass=mt, precision=precision)
    ref = oracle.allpairs(A, B, ref_mass=mr, tgt_mass=mt)
    assert np.abs(out - ref).max() <= TOL


@pytest.mark.parametrize("precision", ["fp32", "tc"])
def test_row_ranges(h, precision):
    X, m = synth.trajectory(6, 150, 120, 0.3, 2.0, np.float32, True)
    full = run(h, X, tgt_mass=m, precision=precision)
    parts = [run(h, X, tgt_mass=m, precision=precision, row_begin=a, row_end=b)
             for a, b in ((0, 1), (1, 64), (64, 149), (149, 150))]
    np.testing.assert_array_equal(np.concatenate(parts), full)
    A, B = X[:40], X[40:]
    fullf = run(h, A, B, tgt_mass=m, precision=precision)
    partf = [run(h, A, B, tgt_mass=m, precision=precision, row_begin=a, row_end=b) for a, b in ((0, 33), (33, 110))]
    np.testing.assert_array_equal(np.concatenate(partf), fullf)


@pytest.mark.parametrize("precision", _precisions())
@pytest.mark.parametrize("F,N", [(2, 1), (3, 2), (5, 3), (65, 4), (2, 65), (67, 129), (129, 31)])
def test_small_and_ragged(h, precision, F, N):
    X, _ = synth.trajectory(F * 100 + N, F, N, 0.5, 1.5, np.float64, False)
    _check(h, X, None, precision, tol=2e-6 if precision == "fp64" else TOL)


def test_single_frame_has_no_pairs(h):
    X = np.zeros((1, 10, 3), np.float32)
    out = h.allpairs(X)
    assert out.size == 0


def test_identical_frames_are_zero(h):
    X = np.repeat(synth.random_walk(np.random.default_rng(0), 50)[None], 6, axis=0).astype(np.float32)
    for p in ("fp32", "fp64"):
        out = run(h, X, precision=p)
        assert np.all(out == 0.0) or np.abs(out).max() < 1e-5


def test_errors_are_reported(h):
    X = np.zeros((4, 5, 3), np.float32)
    with pytest.raises(gbrmsd.GbrError) as e:
        h.allpairs(X, tgt_mass=np.zeros(5))
    assert e.value.code == 4
    with pytest.raises(gbrmsd.GbrError) as e:
        h.allpairs(np.zeros((4, 0, 3), np.float32))
    assert e.value.code == 1
    # the handle stays usable after errors
    Y, _ = synth.trajectory(9, 12, 30, 0.5, 1.0, np.float32, False)
    _check(h, Y, None, "fp32")


def test_device_pointers_match_host(h):
    import torch
    X, m = synth.trajectory(10, 100, 300, 0.2, 2.0, np.float32, True)
    host = h.allpairs(X, tgt_mass=m)
    dX = torch.from_numpy(X).cuda()
    dm = torch.from_numpy(m).cuda()
    dev = h.allpairs(dX, tgt_mass=dm)
    assert dev.is_cuda
    np.testing.assert_array_equal(dev.cpu().numpy(), host)


@pytest.mark.parametrize("precision", ["fp32", "tc"])
def test_device_deferred_reference_count(h, precision):
    # Device input and output: the one-reference assumption is checked on the
    # device; frames around 6 centroids need more references, so the call runs
    # again from its first scan.  A second call of the same shape decides on
    # the host at once (the handle remembers the last shape's count).  Both
    # must equal the host-input path bit for bit, and the oracle within the
    # tolerance.
    import torch
    X, _ = synth.clustered(11, 400, 320, 6, 0.8)
    ref = oracle.allpairs_f64(X)
    h.allpairs(synth.trajectory(3, 20, 20, 0.1, 1.0, np.float32, False)[0], precision=precision)  # other shape
    dX = torch.from_numpy(X).cuda()
    dev1 = run(h, dX, precision=precision).cpu().numpy()
    refs1 = h.stats()["n_refs"]
    dev2 = run(h, dX, precision=precision).cpu().numpy()
    refs2 = h.stats()["n_refs"]
    host = run(h, X, precision=precision)
    assert refs1 >= 2 and refs2 == refs1 and h.stats()["n_refs"] == refs1
    np.testing.assert_array_equal(dev1, host)
    np.testing.assert_array_equal(dev2, host)
    assert np.abs(host - ref).max() <= TOL


def test_tc_matches_fp32_closely(h):
    X, m = synth.trajectory(12, 256, 700, 0.1, 3.0, np.float32, True)
    a = run(h, X, tgt_mass=m, precision="fp32")
    b = run(h, X, tgt_mass=m, precision="tc")
    assert np.abs(a - b).max() <= TOL


@pytest.mark.parametrize("pipeline", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("F,N", [(67, 129), (300, 2000), (129, 31), (2, 65), (171, 200)])
def test_tc_pipeline_variants(h, pipeline, F, N):
    X, m = synth.trajectory(F * 7 + N, F, N, 0.1, 3.0, np.float32, True)
    h.set_option(gbrmsd.OPT_TC_PIPELINE, pipeline)
    try:
        _check(h, X, m, "tc")
        st = h.stats()
        # the contraction itself must be right: the FP64 re-check may only
        # touch the odd pair, not stand in for the tensor-core result
        assert st["pairs_fixed"] <= max(1, st["pairs"] // 100), st
    finally:
        h.set_option(gbrmsd.OPT_TC_PIPELINE, gbrmsd.TC_PIPELINE_DEFAULT)


@pytest.mark.parametrize("pipeline", [1, 2, 3, 4])
def test_tc_pipeline_full_and_rows(h, pipeline):
    R, m = synth.trajectory(77, 130, 257, 0.1, 3.0, np.float32, True)
    T, _ = synth.trajectory(78, 201, 257, 0.1, 3.0, np.float32, True)
    ref = oracle.allpairs_f64(R, T, tgt_mass=m).reshape(201, 130)
    tri_ref = oracle.allpairs_f64(R, tgt_mass=m)
    h.set_option(gbrmsd.OPT_TC_PIPELINE, pipeline)
    try:
        full = run(h, R, T, tgt_mass=m, precision="tc").reshape(201, 130)
        assert np.abs(full - ref).max() <= TOL
        assert h.stats()["pairs_fixed"] <= 201 * 130 // 100
        part = run(h, R, T, tgt_mass=m, precision="tc", row_begin=37, row_end=161).reshape(124, 130)
        assert np.abs(part - ref[37:161]).max() <= TOL
        tri = run(h, R, tgt_mass=m, precision="tc", row_begin=50, row_end=120)
        lo = 50 * 130 - 50 * 51 // 2
        hi = 120 * 130 - 120 * 121 // 2
        assert np.abs(tri - tri_ref[lo:hi]).max() <= TOL
    finally:
        h.set_option(gbrmsd.OPT_TC_PIPELINE, gbrmsd.TC_PIPELINE_DEFAULT)


@pytest.mark.parametrize("host_out", [1, 0])
@pytest.mark.parametrize("precision", ["tc", "fp32"])
def test_pinned_host_overlap(h, precision, host_out):
    # pinned host inputs (chunked copies overlapping the first prep pass) and a
    # pinned host result -- stored in place by the kernels (host_out 1) or in
    # row bands copied while later bands compute (host_out 0) -- must give
    # exactly what the device-resident call gives
    torch = pytest.importorskip("torch")
    h.set_option(gbrmsd.OPT_HOST_OUT, host_out)
    X, m = synth.trajectory(91, 4200, 800, 0.1, 3.0, np.float32, True)
    dev = run(h, torch.from_numpy(X).cuda(), tgt_mass=m, precision=precision).cpu().numpy()
    hX = torch.from_numpy(X).pin_memory()
    hout = torch.empty(dev.size, dtype=torch.float32).pin_memory()
    h.allpairs(hX, tgt_mass=m, precision=precision, out=hout)
    np.testing.assert_array_equal(hout.numpy(), dev)
    rng = np.random.default_rng(4)
    pi = rng.integers(0, 4199, 300)
    pj = pi + 1 + (rng.integers(0, 10**9, 300) % (4199 - pi))
    ref = oracle.pairs_f64(X, pi, pj, mass=m)
    k = pi * 4200 - pi * (pi + 1) // 2 + pj - pi - 1
    assert np.abs(hout.numpy()[k] - ref).max() <= TOL
    # FULL: two pinned sets, banded by target rows
    T, _ = synth.trajectory(92, 4200, 800, 0.1, 3.0, np.float32, True)
    R = X[:2100]
    devf = run(h, torch.from_numpy(R).cuda(), torch.from_numpy(T).cuda(), tgt_mass=m,
               precision=precision).cpu().numpy()
    houtf = torch.empty(devf.size, dtype=torch.float32).pin_memory()
    h.allpairs(torch.from_numpy(R).pin_memory(), torch.from_numpy(T).pin_memory(), tgt_mass=m,
               precision=precision, out=houtf)
    np.testing.assert_array_equal(houtf.numpy(), devf)
    h.set_option(gbrmsd.OPT_HOST_OUT, 1)


@pytest.mark.parametrize("precision", _precisions())
def test_qrmsd_maps_to_fit(h, precision):
    """rms2d `qrmsd` (QuaternionRMSD_CenteredRef) is passed to the library as
    GBR_FIT: same best-fit RMSD, QCP instead of Jacobi.  Check against
    cpptraj's own qrmsd triangle (ref_pairs.npz, its Frame/QCP code)."""
    refp = np.load(os.path.join(GOLD, "ref_pairs.npz"))
    out = run(h, refp["xyz"], tgt_mass=refp["mass"], mode="fit", precision=precision)
    tol = 2e-6 if precision == "fp64" else TOL
    assert np.abs(out.astype(np.float64) - refp["tri_qcp"]).max() <= tol


@pytest.mark.parametrize("overlap", [0, 1])
@pytest.mark.parametrize("sig_hi,expect_refs", [(1.0, 1), (6.0, None)])
def test_pinned_input_speculative_prep(h, sig_hi, expect_refs, overlap):
    # Chunked pinned host input: the operands are built for one reference as
    # the chunks land.  Tight frames keep that build (one reference); spread
    # frames need more references, and the call falls back to the general
    # path.  Either way the result equals the device-resident call bit for bit.
    torch = pytest.importorskip("torch")
    X, m = synth.trajectory(93, 3000, 1000, 0.1, sig_hi, np.float32, True)
    dev = run(h, torch.from_numpy(X).cuda(), tgt_mass=m, precision="tc").cpu().numpy()
    refs_dev = h.stats()["n_refs"]
    hX = torch.from_numpy(X).pin_memory()
    hout = torch.empty(dev.size, dtype=torch.float32).pin_memory()
    h.set_option(gbrmsd.OPT_INPUT_OVERLAP, overlap)
    try:
        run(h, hX, tgt_mass=m, precision="tc", out=hout)
    finally:
        h.set_option(gbrmsd.OPT_INPUT_OVERLAP, 1)  # the default
    assert h.stats()["n_refs"] == refs_dev
    if expect_refs is not None:
        assert refs_dev == expect_refs
    else:
        assert refs_dev > 1
    np.testing.assert_array_equal(hout.numpy(), dev)


@pytest.mark.parametrize("precision", ["tc", "fp32"])
def test_pageable_host_buffers(h, precision):
    # Pageable host input (chunk copies issued one by one between the chunks'
    # passes) and a pageable host result (row bands, each copied while the
    # next computes), with one reference and with several: bit for bit the
    # device-resident call.
    torch = pytest.importorskip("torch")
    X, m = synth.trajectory(96, 4200, 800, 0.1, 3.0, np.float32, True)
    dev = run(h, torch.from_numpy(X).cuda(), tgt_mass=m, precision=precision).cpu().numpy()
    out = np.full(dev.size, -1.0, np.float32)
    run(h, X, tgt_mass=m, precision=precision, out=out)
    np.testing.assert_array_equal(out, dev)
    T, _ = synth.trajectory(98, 3000, 1000, 0.1, 0.5, np.float32, True)  # one reference
    devt = run(h, torch.from_numpy(T).cuda(), precision=precision).cpu().numpy()
    assert h.stats()["n_refs"] == 1
    outt = run(h, T, precision=precision)
    assert h.stats()["n_refs"] == 1
    np.testing.assert_array_equal(outt, devt)
    C, _ = synth.clustered(97, 3000, 1000, 6, 0.8)
    devc = run(h, torch.from_numpy(C).cuda(), precision=precision).cpu().numpy()
    assert h.stats()["n_refs"] > 1
    outc = run(h, C, precision=precision)
    np.testing.assert_array_equal(outc, devc)
    # FULL, two pageable sets (chunks of both), the result in bands of target rows
    R = X[:2100]
    T2, _ = synth.trajectory(99, 4200, 800, 0.1, 3.0, np.float32, True)
    devf = run(h, torch.from_numpy(R).cuda(), torch.from_numpy(T2).cuda(), tgt_mass=m,
               precision=precision).cpu().numpy()
    outf = run(h, R, T2, tgt_mass=m, precision=precision)
    np.testing.assert_array_equal(outf, devf)


@pytest.mark.parametrize("precision", ["tc", "fp32"])
def test_pinned_clustered_result(h, precision):
    # Several references: the triangle is computed over reference-sorted
    # positions, whose results scatter over the whole output; bound for pinned
    # host memory it is computed into device memory and copied back whole.
    # The first pinned call speculates on one reference (and throws that
    # away), a repeated call of the same shape does not.  Both equal the
    # device-resident call bit for bit.
    torch = pytest.importorskip("torch")
    X, _ = synth.clustered(95, 3000, 400, 6, 0.8)
    dev = run(h, torch.from_numpy(X).cuda(), precision=precision).cpu().numpy()
    assert h.stats()["n_refs"] > 1
    run(h, synth.trajectory(3, 20, 20, 0.1, 1.0, np.float32, False)[0], precision=precision)  # other shape
    hX = torch.from_numpy(X).pin_memory()
    hout = torch.empty(dev.size, dtype=torch.float32).pin_memory()
    run(h, hX, precision=precision, out=hout)
    np.testing.assert_array_equal(hout.numpy(), dev)
    hout.fill_(-1.0)
    run(h, hX, precision=precision, out=hout)
    np.testing.assert_array_equal(hout.numpy(), dev)
    # a result buffer 4 bytes past a 16-byte boundary: copied back whole instead
    shifted = torch.full((dev.size + 1,), -1.0, dtype=torch.float32).pin_memory()[1:]
    run(h, hX, precision=precision, out=shifted)
    np.testing.assert_array_equal(shifted.numpy(), dev)
    ref = oracle.allpairs_f64(X[:600])
    k = np.concatenate([np.arange(i * 3000 - i * (i + 1) // 2, i * 3000 - i * (i + 1) // 2 + 599 - i)
                        for i in range(599)])
    assert np.abs(hout.numpy()[k] - ref).max() <= TOL


def test_pinned_input_late_speculation_failure(h):
    # With GBR_OPT_INPUT_OVERLAP (the default) the contraction starts on the
    # chunks that have landed; a far frame in the last chunk ends the speculation after
    # several stages already ran.  Their results are discarded and the general
    # path recomputes the whole triangle: bit-identical to the device-resident
    # call.
    torch = pytest.importorskip("torch")
    X, m = synth.trajectory(93, 3000, 1000, 0.1, 0.5, np.float32, True)
    Y, _ = synth.trajectory(94, 40, 1000, 0.1, 0.5, np.float32, True)
    X[2960:] = Y  # another chain: far more than tau from frame 0
    dev = run(h, torch.from_numpy(X).cuda(), tgt_mass=m, precision="tc").cpu().numpy()
    assert h.stats()["n_refs"] > 1
    hX = torch.from_numpy(X).pin_memory()
    hout = torch.empty(dev.size, dtype=torch.float32).pin_memory()
    h.set_option(gbrmsd.OPT_INPUT_OVERLAP, 1)
    try:
        run(h, hX, tgt_mass=m, precision="tc", out=hout)
        np.testing.assert_array_equal(hout.numpy(), dev)
        # one reference allowed: the speculation always stands
        h.set_option(gbrmsd.OPT_MAX_REFS, 1)
        dev1 = run(h, torch.from_numpy(X).cuda(), tgt_mass=m, precision="tc").cpu().numpy()
        run(h, hX, tgt_mass=m, precision="tc", out=hout)
        assert h.stats()["n_refs"] == 1
        np.testing.assert_array_equal(hout.numpy(), dev1)
    finally:
        h.set_option(gbrmsd.OPT_MAX_REFS, 32)
        h.set_option(gbrmsd.OPT_INPUT_OVERLAP, 1)  # the default
