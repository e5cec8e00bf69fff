"""Sensitivities on the GPU against the oracle (S digit, cntc_getsensitivities).

S >= 2 adds d Fn / d pen from one extra NormCG solve with the approach perturbed (sens_norm,
src/m_solvpn.f90:531-650); S = 3 adds d(Fx, Fy, Mz) / d(cksi, ceta, cphi) from one extra
tangential solve per creepage (sens_tang, src/m_solvpt.f90:544-798), each started from the
solution with the stopping rule on the change from it.  The oracle's own sensitivities are
checked against central differences of full solves (tests/test_oracle.py); here the GPU's
are held to them within 1e-6 relative (scaled by the largest entry of their row for entries
that vanish by symmetry): each is a difference quotient over a perturbation of 1e-4 of the
characteristic creepage, so the solves' rounding-level differences grow by about 1e4 in it.
"""
import pytest

import cases as C
from test_gpu_parity import assert_parity, run_gpu

pytestmark = pytest.mark.gpu


def _compare(g_s, o_s, rows, cols):
    for io in rows:
        scale = max(abs(o_s[io][j]) for j in cols)
        for ji in cols:
            assert abs(g_s[io, ji] - o_s[io][ji]) <= 1e-6 * max(abs(o_s[io][ji]), scale), (io, ji, g_s[io, ji],
                                                                                       o_s[io][ji])


@pytest.mark.parametrize("gausei", [0, 5])
def test_creepage_sensitivities(cntc, oracle, gausei):
    """S = 3 on the 25 x 25 Hertzian steady-rolling case, SteadyGS (G=0) and GDsteady (G=5)."""
    c = dict(C.config0(gausei=gausei, eps=1e-9, mx=25, my=25), sens=3, epsens=1e-8, mxsens=999)
    o = C.oracle_solve(c)
    g = run_gpu(cntc, c, ire=110)
    assert_parity(g, o, c)
    s = cntc.getsensitivities(110, 1)
    _compare(s, o["sens"], rows=(1, 2, 3), cols=(1, 2, 3))


def test_approach_sensitivity(cntc, oracle):
    """S = 2: d Fn / d pen of the normal problem with Fn prescribed (N=1) on a quadratic geometry."""
    q = C.catt_to_cart_case1()
    q.update(force3=0, cksi=0.0, tang=0, eps=1e-10, sens=2, epsens=1e-10, mxsens=200)
    o = C.oracle_solve(q)
    g = run_gpu(cntc, q, ire=111)
    assert_parity(g, o, q)
    s = cntc.getsensitivities(111, 1)
    assert abs(s[0, 0] - o["sens"][0][0]) <= 1e-6 * abs(o["sens"][0][0])


def test_shift_sensitivities_with_forces_prescribed(cntc, oracle):
    """S = 3 after a Newton-Raphson on prescribed Fx (catt_to_cart case 1, TangCG, T=1)."""
    c = dict(C.catt_to_cart_case1(), sens=3, eps=1e-9, epsens=1e-9, mxsens=300)
    o = C.oracle_solve(c)
    g = run_gpu(cntc, c, ire=112)
    assert_parity(g, o, c)
    s = cntc.getsensitivities(112, 1)
    _compare(s, o["sens"], rows=(1, 2, 3), cols=(1, 2, 3))
