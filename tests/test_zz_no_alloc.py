"""cntc_calculate_noalloc (no device allocation, fixed device scratch) against cntc_calculate.

Collected last so that it also runs after every other GPU test of the session; it passes
alone as well (`pytest tests/test_zz_no_alloc.py -m gpu`)."""
import numpy as np
import pytest

import cases as C

pytestmark = pytest.mark.gpu


def _same(a, b):
    for k in ("fn", "fx", "fy", "mz", "pen", "itcg", "itgs", "ierror"):
        assert a[k] == b[k], k
    for k in ("pn", "px", "py", "igs"):
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("mixed", [0, 2])
def test_noalloc_matches_calculate_twice(cntc, mixed):
    case = C.config0(gausei=5, eps=1e-9, mx=41, my=37, mixed=mixed)
    cntc.setup_case(60, 1, case)
    assert cntc.calculate(60, 1) == 0
    ref = cntc.results(60, 1)
    for _ in range(2):                       # two calls in a row reuse the same scratch
        cntc.setup_case(61, 1, case)
        assert cntc.calculate_noalloc(61, 1) == 0
        _same(cntc.results(61, 1), ref)


@pytest.mark.parametrize("mx,my,group", [(128, 128, 0), (41, 37, 4)])
def test_noalloc_near_limit_and_grouped(cntc, mx, my, group):
    """A grid near the 16 MiB limit, and a patch group of 4 CTAs (its group scratch carved from
    the same array), each against cntc_calculate on two calls in a row."""
    case = dict(C.config0(gausei=5, eps=1e-8, mx=mx, my=my), group=group)
    cntc.setup_case(63, 1, case)
    assert cntc.calculate(63, 1) == 0
    ref = cntc.results(63, 1)
    for _ in range(2):
        cntc.setup_case(64, 1, case)
        assert cntc.calculate_noalloc(64, 1) == 0
        if group:
            assert int(cntc.getsolverstats(64, 1)["ctas"]) == group
        _same(cntc.results(64, 1), ref)


def test_noalloc_rejects_oversize(cntc):
    case = C.config0(gausei=5, eps=1e-8, mx=160, my=160)      # ~19 MB of device data > 16 MiB
    cntc.setup_case(62, 1, case)
    assert cntc.calculate_noalloc(62, 1) == cntc.CNTC_err_other
