"""Device-side failure detection without a GPU fault.

The tensor-core pair kernels bound every mbarrier wait (about 2 s); when a
wait runs out the kernel records a site code, returns and the call fails with
GBR_ERR_DEVICE.  gbr_selftest_bounded_wait runs that same helper in a one-CTA
kernel (no TMA, no MMA, no peer CTA) on a barrier nothing arrives on, with a
short limit: the wait must give up, every thread must return, the code must
be recorded, and the context must stay usable for the next call."""
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


@pytest.mark.parametrize("limit", [20_000, 2_000_000])
def test_bounded_wait_gives_up_and_reports(h, limit):
    site, waited = h.selftest_bounded_wait(limit)
    assert site == 0x5E1F
    assert limit <= waited < limit + 5_000_000
    # the context is still usable: a normal call right after
    X, m = synth.trajectory(3, 40, 50, 0.2, 2.0, np.float32, True)
    out = h.allpairs(X, tgt_mass=m, precision="fp32")
    assert np.abs(out - oracle.allpairs_f64(X, tgt_mass=m)).max() <= 1e-4


def test_bounded_wait_limit_is_checked(h):
    with pytest.raises(gbrmsd.GbrError) as e:
        h.selftest_bounded_wait(10)
    assert e.value.code == 1
