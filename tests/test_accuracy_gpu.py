"""Accuracy on the data classes that stress the per-pair error bound, every
pair of the triangle against the FP64 oracle (1e-4 Angstrom, the bar of this
path).

- MD-like time-correlated frames (consecutive frames near-duplicates, the
  residuals correlated across atoms): on these the tensor-core contraction
  alone errs above 1e-4 Angstrom for some pairs, and only the FP64 re-check
  of the pairs whose a-priori bound exceeds the tolerance brings them in.
  The tests assert that the re-check engages.
- Near-identical frames (RMSD ~0.01 Angstrom) whose residuals against their
  pre-alignment reference are large (3 Angstrom), spread over at least 8
  references, frame order shuffled.

The per-pair arithmetic being checked is Frame::RMSD_CenteredRef
(src/Frame.cpp:1137-1273) with mass weighting.
"""
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


def _run(h, X, m, precision):
    try:
        out = h.allpairs(X, tgt_mass=m, precision=precision)
    except gbrmsd.GbrError as e:
        if e.code == 6 and precision == "tc":
            pytest.skip("tensor-core path not available")
        raise
    return out, h.stats()


@pytest.mark.parametrize("n_atom", [2000, 3000])
@pytest.mark.parametrize("precision", ["tc", "fp32"])
def test_md_like_every_pair(h, precision, n_atom):
    X, m = synth.md_like(6 + n_atom, 1200, n_atom, weighted=True)
    ref = oracle.allpairs_f64(X, tgt_mass=m)
    out, st = _run(h, X, m, precision)
    err = np.abs(out.astype(np.float64) - ref)
    assert st["pairs"] == len(ref)
    assert err.max() <= TOL, (float(err.max()), st)
    if precision == "tc":
        # the bound sends some pairs to the FP64 kernel on this data
        assert st["pairs_fixed"] > 0, st


@pytest.mark.parametrize("precision", ["tc", "fp32"])
def test_near_duplicates_far_from_references(h, precision):
    X, m, base = synth.near_duplicates(11, 8, 40, 4, 2000, resid=3.0, dup=0.01)
    ref = oracle.allpairs_f64(X, tgt_mass=m)
    out, st = _run(h, X, m, precision)
    assert st["n_refs"] >= 8, st
    err = np.abs(out.astype(np.float64) - ref)
    assert err.max() <= TOL, (float(err.max()), st)
    # the near-duplicate pairs themselves: RMSD ~0.014 Angstrom, still within the bar
    F = len(X)
    i, j = np.triu_indices(F, 1)
    same = base[i] == base[j]
    assert same.sum() >= 8 * 40 * 6
    assert ref[same].max() < 0.05
    assert err[same].max() <= TOL


def test_raw_tensor_contraction_needs_the_recheck(h):
    """With the re-check switched off (tolerance 1e9) the tensor-core result on
    MD-like frames is reported as is; with the shipped tolerance every pair is
    within the bar.  The raw error is recorded, not asserted above the bar:
    the test pins that the shipped result never depends on it."""
    X, m = synth.md_like(2006, 1200, 2000, weighted=True)
    ref = oracle.allpairs_f64(X, tgt_mass=m)
    try:
        h.set_option(gbrmsd.OPT_TOL, 1e9)
        raw, st_raw = _run(h, X, m, "tc")
        h.set_option(gbrmsd.OPT_TOL, 5e-5)
        shipped, st = _run(h, X, m, "tc")
    finally:
        h.set_option(gbrmsd.OPT_TOL, 5e-5)
    assert st_raw["pairs_fixed"] == 0
    raw_err = float(np.abs(raw.astype(np.float64) - ref).max())
    err = float(np.abs(shipped.astype(np.float64) - ref).max())
    assert err <= TOL, (err, raw_err, st)
    assert err <= raw_err + 1e-6
