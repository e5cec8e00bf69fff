"""Non-identical materials (K != 0): the normal and tangential problems are coupled through the
influence coefficients xz, yz (zx = -xz, zy = -yz) and solved alternately until the tractions
settle (the Panagiotopoulos process, m_scontc.f90:356-553).  The library against the oracle on
the testbank cases that hold such a material pair."""
import numpy as np
import pytest

import cases as C
from test_gpu_parity import MIXED_FORCE_TOL, TRAC_TOL, assert_parity, run_gpu

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("icase", [9, 4])
def test_testbank_coupled(cntc, oracle, icase):
    """9: steady rolling, SteadyGS, Fx prescribed, K = 0.4, up to 10 outer passes (25 x 25);
    4: steady rolling on a 3 x 3 grid with one element in contact (G 200 against 1)."""
    case = C.testbank_case(icase)
    g = run_gpu(cntc, case, ire=90 + icase)
    o = C.oracle_solve(case)
    assert_parity(g, o, case)


def test_testbank_coupled_strip(cntc, oracle):
    """25: a shift of two very different bodies on a 251 x 1 strip, up to 30 outer passes with
    eps 1e-8 for the outer loop and for TangCG alike.  Each pass stops TangCG at |dp| <= eps |p|,
    and the outer loop stops when the tractions change by less than 5 eps (rms) between passes,
    so the pass at which it stops follows the solver's rounding: the first passes agree with the
    oracle to 1e-9 of pmax, the converged result to the outer tolerance."""
    case = C.testbank_case(25)
    g = run_gpu(cntc, case, ire=115)
    o = C.oracle_solve(case)
    assert g["ierror_call"] == o["ierror"]
    assert np.array_equal(g["igs"], o["igs"])
    assert abs(g["pen"] - o["pen"]) <= 1e-10 * abs(o["pen"])
    assert abs(g["fn"] - o["fn"]) <= 1e-10 * abs(o["fn"])
    pmax = np.abs(o["pn"]).max()
    for k in ("pn", "px", "py"):
        assert np.abs(g[k] - o[k]).max() <= 5e-7 * pmax, k
    for mo in (1, 2):
        c1 = dict(case, maxout=mo)
        g1 = run_gpu(cntc, c1, ire=116)
        o1 = C.oracle_solve(c1)
        assert (g1["itnorm"], g1["ittang"]) == (o1["itnorm"], o1["ittang"]) == (mo, mo)
        for k in ("pn", "px", "py"):
            assert np.abs(g1[k] - o1[k]).max() <= 1e-9 * pmax, (mo, k)


def test_coupled_steady_rolling_gdsteady(cntc, oracle):
    """Testbank case 9 by GDsteady (G = 5)."""
    case = dict(C.testbank_case(9), gausei=5, eps=1e-8)
    g = run_gpu(cntc, case, ire=99)
    o = C.oracle_solve(case)
    assert o["ierror"] >= 0
    assert_parity(g, o, case)


def test_coupled_mixed(cntc, oracle):
    """Testbank case 9 in the mixed-precision form: same element division, forces within 1e-8."""
    case = dict(C.testbank_case(9), eps=1e-9)
    o = C.oracle_solve(case)
    g = run_gpu(cntc, dict(case, mixed=1), ire=98)
    assert_parity(g, o, case, force_tol=MIXED_FORCE_TOL, trac_tol=TRAC_TOL, iterations=False)


def test_coupled_transient_refused(cntc):
    """Transient rolling (T = 2) of a material pair with K != 0 is refused, never solved as K = 0."""
    case = dict(C.testbank_case(9), tang=2, dq=1.1)
    cntc.setup_case(97, 1, case)
    assert cntc.calculate(97, 1) == cntc.CNTC_err_other
