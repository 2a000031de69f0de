"""gbr_allpairs_fp64_static: the entry point for callers that cannot
allocate device memory (hosts that serve all device memory from their own
fixed pool, and plugins loaded into them).  It must give the same triangle as
the allocating entry point
gbr_allpairs(..., GBR_PREC_FP64), on two calls in a row that reuse the shared
scratch array.  This file is collected last so that a failure here leaves
every other test already run."""
import numpy as np
import pytest

from cpptraj_gb300 import gbrmsd, synth

pytestmark = pytest.mark.gpu
TOL = 2e-6  # the FP64 checking mode's tolerance in the parity tests


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_static_matches_allocating_entry_point_twice(torch_cuda):
    torch = torch_cuda
    h = gbrmsd.Handle(0)
    # two calls in a row with different sizes, weights and modes
    cases = [
        (synth.trajectory(51, 90, 140, 0.2, 2.0, np.float32, True), "fit"),
        (synth.trajectory(52, 61, 77, 0.5, 1.5, np.float64, False), "nofit"),
    ]
    for (X, m), mode in cases:
        want = h.allpairs(X, tgt_mass=m, mode=mode, precision="fp64")
        dX = torch.from_numpy(X).cuda()
        dm = torch.from_numpy(m).cuda() if m is not None else None
        got = gbrmsd.allpairs_fp64_static(dX, mass=dm, mode=mode)
        torch.cuda.synchronize()
        np.testing.assert_allclose(got.cpu().numpy(), want, rtol=0, atol=TOL)
    h.close()


def test_static_rejects_host_memory_and_oversize(torch_cuda):
    torch = torch_cuda
    X = np.zeros((4, 5, 3), np.float32)
    lib = gbrmsd.load()
    out = torch.zeros(6, device="cuda")
    assert lib.gbr_allpairs_fp64_static(X.ctypes.data, 0, 4, 5, None, 0, out.data_ptr(), None) == 1
    dX = torch.zeros((4, 5, 3), device="cuda")
    assert lib.gbr_allpairs_fp64_static(dX.data_ptr(), 0, 2_000_000, 5, None, 0, out.data_ptr(), None) == 3
