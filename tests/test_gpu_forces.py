"""Total tangential forces prescribed (F=1: Fx, F=2: Fx and Fy) on the GPU against the oracle.

The reference meets prescribed forces by a Newton-Raphson iteration on the creepages (or
shifts) around the tangential solver, its derivatives the secants of its own steps
(solvpt, src/m_solvpt.f90:51-378).  The engine runs the same iteration inside the solve
kernel.  Each case is held to the FP64 parity bar against the oracle, which itself
reproduces the reference's printed Newton-Raphson rows (tests/test_oracle.py): element
division, forces, tractions and iteration counts, plus the creepages that the iteration
finds and the sensitivities it leaves (cntc_getsensitivities).
"""
import numpy as np
import pytest

import cases as C
from test_gpu_parity import assert_parity, run_gpu

pytestmark = pytest.mark.gpu


def _check(cntc, case, ire, creep_tol=1e-10):
    o = C.oracle_solve(case)
    g = run_gpu(cntc, case, ire=ire)
    assert o["ierror"] == 0
    assert_parity(g, o, case)
    cksi, ceta, _ = cntc.getcreepages(ire, 1)
    assert abs(cksi - o["cksi"]) <= creep_tol * max(abs(o["cksi"]), 1e-6)
    if case.get("force3", 0) >= 2:
        assert abs(ceta - o["ceta"]) <= creep_tol * max(abs(o["ceta"]), 1e-6)
    s = cntc.getsensitivities(ire, 1)
    for io, ji in ((1, 1), (2, 1), (1, 2), (2, 2)):
        assert abs(s[io, ji] - o["sens"][io][ji]) <= 1e-8 * max(abs(o["sens"][io][ji]), 1.0), (io, ji)
    return g, o


def test_cattaneo_fx_fy_prescribed(cntc, oracle):
    """examples/cattaneo.inp case 2 as the reference states it: shift (T=1, TangCG) with
    Fx = -0.875 mu Fn and Fy = 0 prescribed (F=2)."""
    g, o = _check(cntc, C.cattaneo_forces_case(), ire=81)
    assert len(o["nr"]) >= 3


def test_catt_to_cart_fx_prescribed(cntc, oracle):
    """examples/catt_to_cart.inp case 1: Cattaneo shift with Fx = -0.657 mu Fn (F=1)."""
    _check(cntc, C.catt_to_cart_case1(), ire=82)


def test_hertzian_shift_bound_fx_prescribed(cntc, oracle):
    """testbank case 13: the normal problem skipped for the elliptical traction bound (B=2)
    and Fx prescribed (F=1), TangCG on a 41x41 Hertzian grid."""
    _check(cntc, C.testbank_case(13), ire=83)


@pytest.mark.parametrize("gausei,f3", [(5, 1), (5, 2), (0, 1), (0, 2)])
def test_steady_rolling_forces_prescribed(cntc, oracle, gausei, f3):
    """Steady rolling (T=3) by GDsteady (G=5) or SteadyGS (G=0) with Fx (F=1) or Fx and Fy
    (F=2) prescribed on a 25x25 Hertzian grid."""
    base = C.config0(gausei=gausei, eps=1e-8, mx=25, my=25)
    case = dict(base, force3=1, fxrel=-0.6)
    del case["cksi"]
    if f3 == 2:
        case.update(force3=2, fyrel=0.3)
        del case["ceta"]
    g, o = _check(cntc, case, ire=84)
    mufn = case["fstat"] * case["fn"]
    assert g["fx"] == pytest.approx(-0.6 * mufn, rel=1e-14)
    assert abs(g["dx"] * g["dy"] * g["px"].sum() / mufn + 0.6) <= 1e-8


def test_forces_prescribed_mixed(cntc, oracle):
    """The mixed-precision form with Fx prescribed (GDsteady): same element division, forces
    and creepage within the mixed bar."""
    base = C.config0(gausei=5, eps=1e-10, mx=25, my=25)
    case = dict(base, force3=1, fxrel=-0.6)
    del case["cksi"]
    o = C.oracle_solve(case)
    g = run_gpu(cntc, dict(case, mixed=1), ire=85)
    assert_parity(g, o, case, force_tol=1e-8, trac_tol=1e-8, iterations=False)
    cksi, _, _ = cntc.getcreepages(85, 1)
    assert abs(cksi - o["cksi"]) <= 1e-8 * abs(o["cksi"])
