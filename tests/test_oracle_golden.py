"""The CPU oracle against the reference's own golden vectors (no GPU).

tz2 fixtures come from test/Test_2DRMS (printed at %8.3f); ref_pairs come from
cpptraj's Frame code compiled from its sources (tests/golden/make_golden.py).
"""
import os

import numpy as np
import pytest

import oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def square(tri, n):
    M = np.zeros((n, n))
    k = 0
    for i in range(n):
        for j in range(i + 1, n):
            M[i, j] = M[j, i] = tri[k]
            k += 1
    return M


def fmt3(M):
    return np.array([[float("%8.3f" % v) for v in row] for row in M])


@pytest.fixture(scope="module")
def tz2():
    return np.load(os.path.join(GOLD, "tz2_rms2d.npz"))


@pytest.mark.parametrize("save,xyz,mass,mode", [
    ("rmsd_save", "fit_xyz", None, oracle.FIT),           # unit 1
    ("rmsd_mass_save", "fit_xyz", "fit_mass", oracle.FIT),  # unit 2
    ("nofit_save", "nofit_xyz", None, oracle.NOFIT),      # unit 6
    ("rmsd_save", "fit_xyz", None, oracle.QCP),           # unit 8 (qrmsd)
    ("dme_save", "fit_xyz", None, oracle.DME),            # unit 4 (dme)
])
def test_tz2_triangle(tz2, save, xyz, mass, mode):
    out = oracle.allpairs(tz2[xyz], tgt_mass=tz2[mass] if mass else None, mode=mode)
    assert np.array_equal(fmt3(square(out, 10)), tz2[save])


def test_tz2_full_ref_mask(tz2):
    # unit 5: `2drms :2 :11` -> target mask :2, reference mask :11, FULL matrix
    out = oracle.allpairs(tz2["trp_ref_xyz"], tz2["trp_tgt_xyz"])
    M = out.reshape(10, 10)  # printed row = target frame, column = reference frame
    assert np.array_equal(fmt3(M), tz2["trp_save"])


@pytest.fixture(scope="module")
def refp():
    return np.load(os.path.join(GOLD, "ref_pairs.npz"))


@pytest.mark.parametrize("mode,tag", [(oracle.FIT, "fit"), (oracle.NOFIT, "nofit")])
@pytest.mark.parametrize("wt", ["w", "u"])
def test_pairs_match_reference_code(refp, mode, tag, wt):
    m = refp["mass"] if wt == "w" else None
    got = oracle.pairs_f64(refp["xyz"], refp["pi"], refp["pj"], mass=m, mode=mode)
    # rms2d centres the row frame, the cluster metric the second frame: the same
    # math, so agreement is at FP64 rounding level.
    np.testing.assert_allclose(got, refp[f"{tag}_{wt}"], rtol=0, atol=1e-9)


def test_dme_pairs_match_reference_code(refp):
    got = oracle.pairs_f64(refp["xyz"], refp["pi"], refp["pj"], mode=oracle.DME)
    np.testing.assert_allclose(got, refp["dme_u"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("mode,tag", [(oracle.FIT, "fit"), (oracle.QCP, "qcp"), (oracle.NOFIT, "nofit"),
                                      (oracle.DME, "dme")])
def test_tri_bitwise_vs_reference_code(refp, mode, tag):
    got = oracle.allpairs(refp["xyz"], tgt_mass=refp["mass"], mode=mode)
    assert np.array_equal(got, refp[f"tri_{tag}"])


def test_row_ranges_concatenate(refp):
    X, m = refp["xyz"], refp["mass"]
    full = oracle.allpairs(X, tgt_mass=m)
    parts = [oracle.allpairs(X, tgt_mass=m, row_begin=a, row_end=b) for a, b in ((0, 5), (5, 17), (17, 24))]
    assert np.array_equal(np.concatenate(parts), full)


def test_zero_mass_reports_error():
    X = np.random.default_rng(0).standard_normal((3, 4, 3))
    out = oracle.allpairs_f64(X, tgt_mass=np.zeros(4))
    assert np.all(out == -1.0)


@pytest.mark.skipif(not oracle.ref_available(), reason="reference sources not built here")
def test_live_reference_random():
    from cpptraj_gb300 import synth
    X, m = synth.trajectory(21, 40, 211, 0.1, 2.0, np.float64, True)
    for mode in (oracle.FIT, oracle.NOFIT, oracle.QCP):
        a = oracle.allpairs(X, tgt_mass=m, mode=mode)
        b = oracle.allpairs(X, tgt_mass=m, mode=mode, use_reference_code=True)
        assert np.array_equal(a, b)


def test_full_row_ranges_are_target_rows(refp):
    X, m = refp["xyz"], refp["mass"]
    A, B = X[:10], X[10:]
    full = oracle.allpairs(A, B, tgt_mass=m)
    assert full.size == 10 * 14
    parts = [oracle.allpairs(A, B, tgt_mass=m, row_begin=a, row_end=b) for a, b in ((0, 3), (3, 14))]
    assert np.array_equal(np.concatenate(parts), full)


def test_cluster_cmatrix_fixture_matches_oracle():
    # the cached distances in the reference-written file are the oracle's nofit RMSDs
    z = np.load(os.path.join(GOLD, "tz2_cluster_cmatrix.npz"))
    for tag in ("full", "sieve3"):
        f2i = z[f"f2i_{tag}"]
        kept = np.nonzero(f2i >= 0)[0]
        raw = z[f"ctm_{tag}"].tobytes()
        assert raw[:4] == b"CTM\x02"
        n_orig, nrows, sieve = np.frombuffer(raw[4:28], dtype=np.int64)
        assert (n_orig, nrows) == (len(f2i), len(kept))
        n = nrows * (nrows - 1) // 2
        tri = np.frombuffer(raw[28:28 + 4 * n], dtype=np.float32)
        mine = oracle.allpairs(np.ascontiguousarray(z["xyz"][kept]), mode=oracle.NOFIT)
        np.testing.assert_allclose(tri, mine, rtol=0, atol=1e-6)
        if sieve != 1:
            flags = raw[28 + 4 * n:]
            assert flags == b"".join(b"T" if v < 0 else b"F" for v in f2i)


@pytest.mark.parametrize("wt", ["w", "u"])
def test_superpose_matches_reference_code(wt):
    """rms / align per-frame fit: the restatement against cpptraj's own
    RMSD_CenteredRef(ref, U, Trans) + Trans_Rot_Trans output (ref_superpose.npz)."""
    g = np.load(os.path.join(GOLD, "ref_superpose.npz"))
    m = g["mass"] if wt == "w" else None
    r, rot, tt, rt, mv = oracle.superpose_f64(g["xyz"][5], g["xyz"], mass=m, move=g["move"])
    np.testing.assert_array_equal(r, g[f"rmsd_{wt}"])
    np.testing.assert_array_equal(rot, g[f"rot_{wt}"])
    np.testing.assert_array_equal(tt, g[f"tgt_trans_{wt}"])
    np.testing.assert_array_equal(rt, g[f"ref_trans_{wt}"])
    np.testing.assert_array_equal(mv, g[f"moved_{wt}"])
    assert r[5] < 1e-6  # the reference frame itself


@pytest.mark.parametrize("tag", ["fit_w", "fit_u", "nofit"])
def test_cluster_centroids_match_reference_code(tag):
    """Cluster centroids: the restatement against cpptraj's own Frame code run
    in the steps of Metric_RMS::CalculateCentroid (ref_centroids.npz)."""
    g = np.load(os.path.join(GOLD, "ref_centroids.npz"))
    m = g["mass"] if tag == "fit_w" else None
    mode = oracle.NOFIT if tag == "nofit" else oracle.FIT
    got = oracle.cluster_centroids_f64(g["xyz"], g["members"], g["offsets"], mass=m, mode=mode)
    sizes = np.diff(g["offsets"])
    np.testing.assert_allclose(got[sizes > 0], g[tag][sizes > 0], rtol=0, atol=1e-12)
    assert np.all(np.isnan(got[sizes == 0]))
    # a one-member cluster's centroid is that frame, centred when fitting
    one = oracle.cluster_centroids_f64(g["xyz"], np.array([7], np.int32), np.array([0, 1]), mass=m, mode=mode)
    want = g["xyz"][7].astype(np.float64)
    if mode == oracle.FIT:
        w = m if m is not None else np.ones(len(want))
        want = want - (w[:, None] * want).sum(0) / w.sum()
    np.testing.assert_allclose(one[0], want, rtol=0, atol=1e-12)
