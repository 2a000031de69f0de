"""Band partition of the streamed triangle (gbr_row_bands, host only): the
bands cover every TRI row once, in order, none holds more than the band
size, boundaries fall on multiples of the row alignment wherever a band
holds whole groups, and a band smaller than one row is refused."""
import numpy as np
import pytest

from cpptraj_gb300 import gbrmsd


def _before(n, r):
    return r * n - r * (r + 1) // 2


@pytest.mark.parametrize("n,band,align", [(101, 1000, 1), (101, 1000, 84), (700, 5000, 84), (5000, 10**6, 84),
                                          (5000, 5000, 64), (2, 1, 1), (3, 2, 7), (50000, 1 << 28, 84),
                                          (1234, 700_000, 84)])
def test_bands_cover_the_triangle(n, band, align):
    cuts = gbrmsd.row_bands(n, band, align)
    assert cuts[0] == 0 and cuts[-1] == n
    assert np.all(np.diff(cuts) > 0)
    sizes = np.array([_before(n, cuts[k + 1]) - _before(n, cuts[k]) for k in range(len(cuts) - 1)])
    assert sizes.max() <= band
    assert sizes.sum() == n * (n - 1) // 2
    group = _before(n, min(n, align)) - _before(n, 0)
    if group <= band:
        # the first band starts at row 0 and holds whole groups: aligned end
        assert cuts[1] % align == 0 or cuts[1] == n


def test_whole_triangle_is_one_band():
    assert list(gbrmsd.row_bands(10000, 1 << 28, 84)) == [0, 10000]


def test_band_smaller_than_a_row_is_refused():
    with pytest.raises(ValueError):
        gbrmsd.row_bands(1000, 998, 1)
    assert list(gbrmsd.row_bands(1000, 999, 1))[:2] == [0, 1]
