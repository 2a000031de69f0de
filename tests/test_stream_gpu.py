"""Streamed triangles (gbr_allpairs_stream) for pairwise caches larger than
device memory, and the cluster-matrix file written through them.

- bands arrive in row order and cover the triangle; their values equal the
  row-range calls of gbr_allpairs bit for bit (the same unsorted frame
  layout) and the FP64 oracle within 1e-4 Angstrom;
- a forced small band size writes cpptraj's binary cluster-matrix file
  byte-identical in header and trailer to Cmatrix_Binary::WriteCmatrix's
  (src/Cluster/Cmatrix_Binary.cpp:141-188, tests/golden/tz2_cluster_cmatrix.npz);
- a band whose list of pairs for the FP64 re-check overflows is recomputed
  in FP64 on the device;
- a sink that stops the call makes it return GBR_ERR_IO."""
import os

import numpy as np
import pytest

import oracle
from cpptraj_gb300 import gbrmsd, synth

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "tz2_cluster_cmatrix.npz")
HEADER = 4 + 8 + 8 + 8
TOL = 1e-4


@pytest.fixture(scope="module")
def h():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    hd = gbrmsd.Handle(0)
    yield hd
    hd.close()


def _collect(h, X, m, precision, band, mode="fit"):
    bands = []

    def sink(rb, re, v):
        bands.append((rb, re, v.copy()))

    h.allpairs_stream(X, sink, mass=m, mode=mode, precision=precision, band_floats=band)
    return bands


@pytest.mark.parametrize("precision", ["tc", "fp32", "fp64"])
def test_stream_matches_row_ranges_and_oracle(h, precision):
    X, _ = synth.clustered(5, 700, 300, 12, 0.8)
    m = synth.masses(np.random.default_rng(1), 300)
    try:
        bands = _collect(h, X, m, precision, 20_000)
    except gbrmsd.GbrError as e:
        if e.code == 6:
            pytest.skip("tensor cores not available")
        raise
    st = h.stats()
    assert len(bands) > 5
    assert bands[0][0] == 0 and bands[-1][1] == 700
    for (a0, a1, _), (b0, b1, _) in zip(bands, bands[1:]):
        assert a1 == b0
    tri = np.concatenate([v for _, _, v in bands])
    assert tri.size == 700 * 699 // 2
    ref = oracle.allpairs_f64(X, tgt_mass=m)
    assert np.abs(tri.astype(np.float64) - ref).max() <= (2e-6 if precision == "fp64" else TOL)
    assert st["pairs"] == tri.size
    if precision != "fp64":  # the FP64 mode computes every pair directly, no references
        assert st["n_refs"] >= 2
    for rb, re, v in bands[:3] + bands[-2:]:
        want = h.allpairs(X, tgt_mass=m, precision=precision, row_begin=rb, row_end=re)
        np.testing.assert_array_equal(v, want)


def test_stream_md_like_recheck_per_band(h):
    X, m = synth.md_like(2006, 1200, 2000, weighted=True)
    try:
        bands = _collect(h, X, m, "tc", 50_000)
    except gbrmsd.GbrError as e:
        if e.code == 6:
            pytest.skip("tensor cores not available")
        raise
    st = h.stats()
    tri = np.concatenate([v for _, _, v in bands])
    ref = oracle.allpairs_f64(X, tgt_mass=m)
    assert np.abs(tri.astype(np.float64) - ref).max() <= TOL
    assert st["pairs_fixed"] > 0


def test_stream_flag_overflow_recomputes_band(h):
    # every pair flagged (tolerance 1e-12) in one band of 2.2M pairs, above
    # the per-band list capacity of 2^21: the band is recomputed in FP64
    X, _ = synth.trajectory(9, 2100, 50, 0.5, 2.0, np.float32, False)
    try:
        h.set_option(gbrmsd.OPT_TOL, 1e-12)
        bands = _collect(h, X, None, "fp32", 0)
        st = h.stats()
    finally:
        h.set_option(gbrmsd.OPT_TOL, 5e-5)
    assert len(bands) == 1
    assert st["pairs_fixed"] > (1 << 21)
    want = h.allpairs(X, precision="fp64")
    # FP64 results on both sides: equal but for the rare last-bit flip of the
    # float cast (the centres come from different prep passes); the FP32
    # kernel's values would differ in most pairs
    d = np.abs(bands[0][2].astype(np.float64) - want)
    assert d.max() <= 3e-7
    assert (d > 0).mean() < 1e-3


def test_sink_can_stop_the_call(h):
    X, _ = synth.trajectory(3, 300, 40, 0.5, 2.0, np.float32, False)
    seen = []

    def sink(rb, re, v):
        seen.append(rb)
        return False if len(seen) == 2 else None

    with pytest.raises(gbrmsd.GbrError) as e:
        h.allpairs_stream(X, sink, precision="fp32", band_floats=3000)
    assert e.value.code == 7
    assert len(seen) == 2
    # the handle works after a stopped call
    out = h.allpairs(X, precision="fp32")
    assert np.abs(out - oracle.allpairs_f64(X)).max() <= TOL


@pytest.mark.parametrize("tag", ["full", "sieve3"])
@pytest.mark.parametrize("precision", ["fp32", "tc"])
def test_cmatrix_in_small_bands_matches_reference_writer(h, tmp_path, tag, precision):
    z = np.load(GOLD)
    f2i = z[f"f2i_{tag}"]
    kept = np.nonzero(f2i >= 0)[0]
    X = np.ascontiguousarray(z["xyz"][kept])
    want = z[f"ctm_{tag}"].tobytes()
    path = str(tmp_path / f"{tag}.cmatrix")
    n = len(kept) * (len(kept) - 1) // 2
    h.set_option(gbrmsd.OPT_BAND_FLOATS, 700)  # several bands even for 101 frames
    try:
        h.write_cmatrix(path, X, mode="nofit", precision=precision,
                        frame_to_idx=None if tag == "full" else f2i, sieve=1 if tag == "full" else 3)
    except gbrmsd.GbrError as e:
        if e.code == 6:
            pytest.skip("tensor cores not available")
        raise
    finally:
        h.set_option(gbrmsd.OPT_BAND_FLOATS, 0)
    got = open(path, "rb").read()
    assert len(got) == len(want)
    assert got[:HEADER] == want[:HEADER]
    a = np.frombuffer(got[HEADER:HEADER + 4 * n], dtype=np.float32)
    b = np.frombuffer(want[HEADER:HEADER + 4 * n], dtype=np.float32)
    assert np.all(np.abs(a - b) <= TOL)
    assert got[HEADER + 4 * n:] == want[HEADER + 4 * n:]
