"""GB300 library (through its C-ABI) against the CPU oracle and the reference's golden outputs.

Parity bar (FP64 form):
  * element classification identical (exterior / adhesion / slip / plastic),
  * total forces Fn, Fx, Fy and Mz within 1e-10 relative; a force that cancels to below a
    thousandth of the friction bound mu*Fn is compared at that scale (1e-10 * 1e-3 mu Fn),
  * tractions pn, px, py within 1e-8 of the maximum pressure,
  * iteration counts equal to the oracle's where both follow the same iteration path.
Mixed form (FP32 bulk + FP64 refinement): same classification, forces within 1e-8 relative.
"""
import json
import os

import numpy as np
import pytest

import cases as C

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FORCE_TOL = 1e-10
TRAC_TOL = 1e-8
MIXED_FORCE_TOL = 1e-8


def run_gpu(cntc, case, ire=1, icp=1):
    cntc.setup_case(ire, icp, case)
    ierr = cntc.calculate(ire, icp)
    r = cntc.results(ire, icp)
    r["ierror_call"] = ierr
    return r


def force_err(g, o, fstat):
    """Relative errors: Fn; the tangential force vector (Fx, Fy), relative to its magnitude or,
    when that cancels to below a thousandth of the friction bound, to 1e-3 mu Fn; Mz relative
    to mu Fn times the half-width of the grid."""
    fn = abs(o["fn"])
    ft = float(np.hypot(o["fx"], o["fy"]))
    width = 0.5 * float(np.hypot(g["dx"] * g["mx"], g["dy"] * g["my"]))
    return {"fn": abs(g["fn"] - o["fn"]) / max(fn, 1e-300),
            "ft": float(np.hypot(g["fx"] - o["fx"], g["fy"] - o["fy"])) / max(ft, 1e-3 * fstat * fn, 1e-300),
            "mz": abs(g["mz"] - o["mz"]) / max(abs(o["mz"]), fstat * fn * width, 1e-300)}


def trac_err(g, o):
    pmax = max(np.abs(o["pn"]).max(), 1e-300)
    return max(np.abs(g[k] - o[k]).max() for k in ("pn", "px", "py")) / pmax


def assert_parity(g, o, case, force_tol=FORCE_TOL, trac_tol=TRAC_TOL, iterations=True):
    assert g["ierror_call"] == o["ierror"], (g["ierror_call"], o["ierror"])
    assert np.array_equal(g["igs"], o["igs"]), int((g["igs"] != o["igs"]).sum())
    fe = force_err(g, o, case.get("fstat", 0.3))
    assert max(fe.values()) <= force_tol, fe
    assert trac_err(g, o) <= trac_tol
    assert abs(g["pen"] - o["pen"]) <= 1e-10 * abs(o["pen"])
    if iterations:
        assert (g["itnorm"], g["ittang"], g["itcg"], g["itgs"]) == (o["itnorm"], o["ittang"], o["itcg"], o["itgs"])


@pytest.mark.parametrize("gausei,eps", [(5, 1e-10), (0, 1e-6)])
def test_hertz_steady_rolling_51(cntc, oracle, gausei, eps):
    """Hertzian steady rolling, 51x51, NormCG + GDsteady (G=5) or SteadyGS (G=0)."""
    case = C.config0(gausei=gausei, eps=eps)
    g = run_gpu(cntc, case)
    o = C.oracle_solve(case)
    assert o["ierror"] == 0
    assert_parity(g, o, case)
    assert g["solver"] == o["solver"]


def test_hertz_steady_rolling_mixed(cntc, oracle):
    """FP32 bulk + FP64 refinement against the FP64 oracle."""
    case = C.config0(gausei=5, eps=1e-10, mixed=1)
    g = run_gpu(cntc, case)
    o = C.oracle_solve(C.config0(gausei=5, eps=1e-10))
    assert_parity(g, o, case, force_tol=MIXED_FORCE_TOL, trac_tol=1e-8, iterations=False)
    st = cntc.getsolverstats(1, 1)
    assert st["nconv32"] > 0 and st["nconv64"] > 0


@pytest.mark.parametrize("mx,my", [(51, 51), (64, 40), (33, 97)])
def test_steadygs_mixed_rows(cntc, oracle, mx, my):
    """SteadyGS in the mixed form (an FP64 product per sweep, the sweep's own change applied in
    FP32 row by row) against the FP64 oracle: same classification, forces within 1e-8."""
    case = C.config0(gausei=0, eps=1e-10, mx=mx, my=my, mixed=1)
    g = run_gpu(cntc, case)
    o = C.oracle_solve(dict(case, mixed=0))
    assert o["ierror"] == 0 and o["solver"] == 4 and g["solver"] == 4
    assert_parity(g, o, case, force_tol=MIXED_FORCE_TOL, trac_tol=TRAC_TOL, iterations=False)
    assert cntc.getsolverstats(1, 1)["t_gs"] > 0
    # the sweeps are the reference's: the sweep count follows the FP64 one (a sweep that dropped
    # part of the in-sweep update would still converge, but in many more sweeps)
    assert abs(g["itgs"] - o["itgs"]) <= 2, (g["itgs"], o["itgs"])


@pytest.mark.parametrize("tang,dq", [(1, None), (2, 0.2)])
def test_tangcg_shift_and_transient(cntc, oracle, tang, dq):
    """TangCG for shift (T=1) and transient rolling (T=2)."""
    case = C.config0(gausei=0, eps=1e-8)
    case["tang"] = tang
    if dq is not None:
        case["dq"] = dq
    g = run_gpu(cntc, case)
    o = C.oracle_solve(case)
    assert o["solver"] == 2
    assert_parity(g, o, case)


@pytest.fixture(scope="module")
def tt_setup(oracle):
    gold = json.load(open(os.path.join(GOLD, "test_table_mx11.json")))
    rho, cp = [], []
    for iell in range(5):
        r = C.oracle_solve(C.test_table_base(iell))
        rho.append(r["rho"])
        cp.append(r["cp"])
    return gold, rho, cp


def test_table_subset_against_golden(cntc, tt_setup):
    """Every 11th case of src/test_table.f90 through cntc_calculate: the printed line of the
    reference (testbank/test_table_mx11.ref_fx) reproduced exactly, forces at parity with
    the oracle."""
    gold, rho, cp = tt_setup
    from test_oracle import fmt_tt
    bad = []
    for icase in range(0, 3220, 11):
        case, iell = C.test_table_case(icase, rho, cp)
        g = run_gpu(cntc, case, ire=2)
        ref = "Fx=%11.6f, Fy=%11.6f, Mz=%11.6f, %%Slip=%6.1f" % tuple(gold["cases"][icase])
        if fmt_tt(g, cp[iell]) != ref.replace("-0.000000", " 0.000000"):
            bad.append((icase, fmt_tt(g, cp[iell]), ref))
    assert not bad, bad[:5]


def test_table_cases_against_oracle(cntc, tt_setup):
    gold, rho, cp = tt_setup
    for icase in (0, 5, 100, 333, 700, 1500, 2222, 3000, 3219):
        case, _ = C.test_table_case(icase, rho, cp)
        g = run_gpu(cntc, case, ire=3)
        o = C.oracle_solve(case)
        assert_parity(g, o, case)


@pytest.mark.parametrize("icase", [1, 4, 12, 30])
def test_tractcurv_against_golden(cntc, oracle, icase):
    """examples/tractcurv.inp, first series: element-division picture, counts and iteration
    numbers as printed by the reference; forces at parity with the oracle."""
    gold = json.load(open(os.path.join(GOLD, "tractcurv_series1.json")))
    c = gold["cases"][icase - 1]
    case = C.tractcurv_case(c["cksi"])
    g = run_gpu(cntc, case, ire=4)
    sym = np.array([".", "*", "S", "P"])[g["igs"]].reshape(44, 48)
    assert ["".join(r) for r in sym] == [r.replace("o", ".") for r in c["picture"]]
    assert (g["ncon"], g["nadh"], g["nslip"]) == (c["ncon"], c["nadh"], c["nslip"])
    assert (g["itcg"], g["itgs"]) == (c["itcg"], c["itgs"])
    o = C.oracle_solve(case)
    assert_parity(g, o, case)


def test_nonhertzian_grid(cntc, oracle):
    """Element-wise undeformed distance (ibase 9) with seeded roughness, 96x96, GDsteady."""
    case = C.config1(96, seed=1, eps=1e-8)
    g = run_gpu(cntc, case)
    o = C.oracle_solve(case)
    assert_parity(g, o, case)


def test_batch_equals_single(cntc):
    """Patches of mixed sizes solved in one cntc_calculate_batch give bit-identical results to
    the same patches solved one by one."""
    cs = C.batch_patches(10, seed=11, mixed=1, eps=1e-8)
    for c in cs:
        c["potprm"] = [min(c["potprm"][0], 64), min(c["potprm"][1], 64)] + c["potprm"][2:]
    single = []
    for i, c in enumerate(cs):
        single.append(run_gpu(cntc, c, ire=20 + i))
    for i, c in enumerate(cs):
        cntc.setup_case(20 + i, 1, c)
    err = cntc.calculate_batch([20 + i for i in range(len(cs))], [1] * len(cs))
    for i in range(len(cs)):
        b = cntc.results(20 + i, 1)
        assert err[i] == single[i]["ierror_call"]
        for k in ("fn", "fx", "fy", "mz", "pen"):
            assert b[k] == single[i][k], (i, k)
        for k in ("pn", "px", "py", "igs"):
            assert np.array_equal(b[k], single[i][k]), (i, k)


def test_batch_mixed_against_oracle(cntc, oracle):
    """A few patches of the batched workload (mixed precision, eps 1e-8) against the FP64 oracle."""
    cs = [c for i, c in enumerate(C.batch_patches(4, seed=2, mixed=1, eps=1e-8)) if i in (0, 3)]
    for i, c in enumerate(cs):
        cntc.setup_case(40 + i, 1, c)
    err = cntc.calculate_batch([40 + i for i in range(len(cs))], [1] * len(cs))
    for i, c in enumerate(cs):
        g = cntc.results(40 + i, 1)
        g["ierror_call"] = int(err[i])
        o = C.oracle_solve(dict(c, mixed=0))
        assert_parity(g, o, c, force_tol=MIXED_FORCE_TOL, trac_tol=1e-7, iterations=False)


def test_repeat_is_deterministic(cntc):
    case = C.config0(gausei=5, eps=1e-10, mixed=1, mx=31, my=31)
    a = run_gpu(cntc, case, ire=5)
    b = run_gpu(cntc, case, ire=5)
    for k in ("fx", "fy", "fn", "mz"):
        assert a[k] == b[k]
    assert np.array_equal(a["px"], b["px"]) and np.array_equal(a["igs"], b["igs"])


def test_native_kernels_launched(cntc):
    before = cntc.kernel_launches()
    run_gpu(cntc, C.config0(gausei=5, eps=1e-8, mx=21, my=21), ire=6)
    assert cntc.kernel_launches() > before


@pytest.mark.parametrize("mx,my", [(2, 2), (3, 5), (7, 1), (11, 1), (4, 1)])
def test_tiny_grids(cntc, oracle, mx, my):
    """Degenerate grids follow the oracle (including its error codes)."""
    case = C.config0(gausei=5, eps=1e-8, mx=mx, my=my)
    g = run_gpu(cntc, case, ire=7)
    o = C.oracle_solve(case)
    assert g["ierror_call"] == o["ierror"]
    if o["ierror"] == 0:
        assert_parity(g, o, case, iterations=False)


def lateral_boundary_case(mx=40, my=24):
    """Quadratic gap on a grid that cuts the contact patch at its lateral sides only (the
    trailing column stays free, so steady rolling keeps GDsteady as its solver)."""
    xl, yl = -9.0, -3.6
    dx, dy = 18.0 / mx, 7.2 / my
    x = xl + (np.arange(mx) + 0.5) * dx
    y = yl + (np.arange(my) + 0.5) * dy
    X, Y = np.meshgrid(x, y)
    h = X ** 2 / (2 * 460.0) + Y ** 2 / (2 * 300.0)
    return dict(tang=3, norm=1, bound=0, gausei=5, maxgs=999, maxin=100, maxnr=30, maxout=1, eps=1e-8,
                poiss=C.NU_STEEL, gg=C.G_STEEL, fstat=0.3, veloc=10000.0, fn=1e5, cksi=0.002, ceta=0.0, cphi=0.0,
                ipotcn=1, potprm=[mx, my, xl, yl, dx, dy], h=h)


def test_contact_touching_boundary(cntc, oracle):
    """Contact on the lateral grid boundary: positive ierror = number of contact elements on the
    boundary of the potential contact area (contact_addon.f90:3754-3900)."""
    case = lateral_boundary_case()
    g = run_gpu(cntc, case, ire=8)
    o = C.oracle_solve(case)
    assert o["ierror"] > 0
    assert g["ierror_call"] == o["ierror"]
    assert_parity(g, o, case, iterations=False)


def test_contact_in_trailing_column_convexgs(cntc, oracle):
    """Contact in the trailing column selects ConvexGS in the reference (m_stang.f90 solver
    choice, src/m_solvpt.f90:2446-2821), with contact on the boundary of the potential contact
    (a positive ierror).  Same element division, forces, tractions and sweeps as the oracle."""
    case = C.config0(gausei=5, eps=1e-8, mx=21, my=21)
    case["potprm"] = [21, 21, 6.0, 4.0, 0.9]
    o = C.oracle_solve(case)
    g = run_gpu(cntc, case, ire=8)
    assert o["ierror"] > 0 and o["solver"] == 3 and g["solver"] == 3
    assert_parity(g, o, case)


@pytest.mark.parametrize("dq_dx", [1.0, 2.5, 5.0])
def test_convexgs_rolling_step(cntc, oracle, dq_dx):
    """ConvexGS chosen by its G digit (G=2) in steady rolling with a rolling step of dq_dx
    elements: the steady-rolling coefficients csv = cs - cv of one step, and for dq > dx the
    leading-edge estimate (subnd) on the elements within one step of the edge."""
    mx, my = 31, 21
    case = C.config0(gausei=2, eps=1e-8, mx=mx, my=my)
    case["dq"] = dq_dx * 2 * 1.1 * 6.0 / mx
    case["chi"] = 0.0
    o = C.oracle_solve(case)
    g = run_gpu(cntc, case, ire=11)
    assert o["ierror"] == 0 and o["solver"] == 3 and g["solver"] == 3
    assert_parity(g, o, case)


def test_convexgs_shift(cntc, oracle):
    """ConvexGS (G=2) for the shift problem (T=1): shifts through cs from the tractions."""
    case = C.config0(gausei=2, eps=1e-8, mx=21, my=21)
    case["tang"] = 1
    o = C.oracle_solve(case)
    g = run_gpu(cntc, case, ire=12)
    assert o["ierror"] == 0 and o["solver"] == 3 and g["solver"] == 3
    assert_parity(g, o, case)


def test_pure_spin_and_zero_creepage(cntc, oracle):
    for ck, cp_ in ((0.0, 0.0), (0.0, 5e-4)):
        case = C.config0(gausei=5, eps=1e-9, mx=41, my=41)
        case["cksi"], case["cphi"] = ck, cp_
        g = run_gpu(cntc, case, ire=9)
        o = C.oracle_solve(case)
        assert_parity(g, o, case, iterations=False)
        if cp_ == 0.0:
            assert g["fx"] == 0.0 and g["fy"] == 0.0


def test_unsupported_flags_rejected(cntc):
    """Options outside the GB300 engine (here: viscoelastic material M=1) are refused with
    CNTC_err_other, never a silent fallback."""
    case = C.config0(gausei=5, eps=1e-8, mx=21, my=21)
    cntc.setup_case(10, 1, case)
    cntc.setmaterialparameters(10, 1, 1, [0.28, 0.28, 82000.0, 82000.0, 0.0, 0.0, 0.0, 0.0])
    assert cntc.calculate(10, 1) == cntc.CNTC_err_other
