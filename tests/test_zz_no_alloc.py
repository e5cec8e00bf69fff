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


def test_noalloc_rejects_oversize(cntc):
    case = C.config0(gausei=5, eps=1e-8, mx=160, my=160)      # ~19 MB of device data > 16 MiB
    cntc.setup_case(62, 1, case)
    assert cntc.calculate_noalloc(62, 1) == cntc.CNTC_err_other
