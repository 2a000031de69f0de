"""gbr_write_cmatrix against cpptraj's own writer: the pairwise cache of
test/Test_Cluster's first unit (`:2-10`, nofit, 101 tz2 frames), full and with
a regular sieve of 3.  Header and sieve trailer must be byte-identical to the
file Cmatrix_Binary::WriteCmatrix wrote (tests/golden/tz2_cluster_cmatrix.npz);
the distances must agree within 1e-4 Angstrom (FP64 mode: float32 rounding)."""
import os

import numpy as np
import pytest

from cpptraj_gb300 import gbrmsd

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "tz2_cluster_cmatrix.npz")
HEADER = 4 + 8 + 8 + 8


@pytest.fixture(scope="module")
def h():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    hd = gbrmsd.Handle(0)
    yield hd
    hd.close()


@pytest.mark.parametrize("tag", ["full", "sieve3"])
@pytest.mark.parametrize("precision", ["fp32", "tc", "fp64"])
def test_cmatrix_matches_reference_writer(h, tmp_path, tag, precision):
    z = np.load(GOLD)
    f2i = z[f"f2i_{tag}"]
    kept = np.nonzero(f2i >= 0)[0]
    X = np.ascontiguousarray(z["xyz"][kept])
    want = z[f"ctm_{tag}"].tobytes()
    path = str(tmp_path / f"{tag}.cmatrix")
    try:
        h.write_cmatrix(path, X, mode="nofit", precision=precision,
                        frame_to_idx=None if tag == "full" else f2i, sieve=1 if tag == "full" else 3)
    except gbrmsd.GbrError as e:
        if e.code == 6:
            pytest.skip("tensor cores not available")
        raise
    got = open(path, "rb").read()
    assert len(got) == len(want)
    assert got[:HEADER] == want[:HEADER]
    n = len(kept) * (len(kept) - 1) // 2
    a = np.frombuffer(got[HEADER:HEADER + 4 * n], dtype=np.float32)
    b = np.frombuffer(want[HEADER:HEADER + 4 * n], dtype=np.float32)
    tol = 2e-6 + 6e-8 * np.abs(b) if precision == "fp64" else 1e-4
    assert np.all(np.abs(a - b) <= tol)
    assert got[HEADER + 4 * n:] == want[HEADER + 4 * n:]
