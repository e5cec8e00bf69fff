"""Patch groups: one patch solved by a cooperative grid of CTAs.

Grids whose FFT lines do not fit the per-warp shared-memory buffers of a single CTA (sides
above about 210: the 256^2 and 512^2 grids of the non-Hertzian sweep, the 1024^2 patch) are
solved by a group of CTAs that meet at grid barriers; its reductions combine per-CTA partials
in rank order.  On small grids the group form is forced (CNTC_if_groupctas) and held to the
parity bar of the single-CTA form against the oracle; on the large grids, where the oracle
takes minutes, the checks are properties that hold at any size: the prescribed total force,
the traction bound, the slip and adhesion conditions, and agreement of the mixed-precision
form with the FP64 form.
"""
import numpy as np
import pytest

import cases as C
from test_gpu_parity import FORCE_TOL, MIXED_FORCE_TOL, TRAC_TOL, assert_parity, force_err, run_gpu

pytestmark = pytest.mark.gpu

GROUP = 8


def ctas(cntc, ire, icp=1):
    return int(cntc.getsolverstats(ire, icp)["ctas"])


@pytest.mark.parametrize("gausei,eps,mixed", [(5, 1e-10, 0), (5, 1e-10, 1), (0, 1e-6, 0), (0, 1e-10, 1)])
def test_group_hertz_51_matches_oracle(cntc, oracle, gausei, eps, mixed):
    """The 51x51 Hertzian case (GDsteady, GDsteady mixed, SteadyGS, SteadyGS mixed) solved by 8
    CTAs."""
    case = C.config0(gausei=gausei, eps=eps, mixed=mixed)
    g = run_gpu(cntc, dict(case, group=GROUP), ire=70)
    assert ctas(cntc, 70) == GROUP
    o = C.oracle_solve(dict(case, mixed=0))
    assert o["ierror"] == 0
    if mixed:
        assert_parity(g, o, case, force_tol=MIXED_FORCE_TOL, trac_tol=TRAC_TOL, iterations=False)
    else:
        assert_parity(g, o, case)


def test_group_tangcg_shift(cntc, oracle):
    """TangCG (shift, T=1) solved by 6 CTAs."""
    case = C.config0(gausei=0, eps=1e-8)
    case["tang"] = 1
    g = run_gpu(cntc, dict(case, group=6), ire=71)
    assert ctas(cntc, 71) == 6
    o = C.oracle_solve(case)
    assert_parity(g, o, case)


def test_group_convexgs(cntc, oracle):
    """ConvexGS (contact in the trailing column and a rolling step of 2.5 elements) solved by 4
    CTAs: the steady-rolling coefficients and the leading-edge estimate in a patch group."""
    case = C.config0(gausei=2, eps=1e-8, mx=31, my=21)
    case["dq"] = 2.5 * 2 * 1.1 * 6.0 / 31
    g = run_gpu(cntc, dict(case, group=4), ire=75)
    assert ctas(cntc, 75) == 4
    o = C.oracle_solve(case)
    assert o["solver"] == 3 and g["solver"] == 3
    assert_parity(g, o, case)


def test_group_rough_96_matches_oracle(cntc, oracle):
    """Non-Hertzian rough surface, 96x96, element-wise h, 36 CTAs."""
    case = C.config1(96)
    g = run_gpu(cntc, dict(case, group=36), ire=72)
    assert ctas(cntc, 72) == 36
    o = C.oracle_solve(case)
    assert_parity(g, o, case)


def test_group_equals_single_cta(cntc):
    """Group and single-CTA solves of one problem agree to the FP64 parity bar."""
    case = C.config0(gausei=5, eps=1e-10, mx=64, my=48)
    a = run_gpu(cntc, dict(case, group=1), ire=73)
    assert ctas(cntc, 73) == 1
    b = run_gpu(cntc, dict(case, group=12), ire=74)
    assert ctas(cntc, 74) == 12
    assert np.array_equal(a["igs"], b["igs"])
    fe = force_err(b, a, case["fstat"])
    assert max(fe.values()) <= FORCE_TOL, fe


def check_solution(r, case, tol=1e-10):
    """Size-independent conditions of a steady-rolling solution with prescribed Fn."""
    igs, pn, px, py = r["igs"], r["pn"], r["px"], r["py"]
    assert r["ierror_call"] >= 0
    dxdy = r["dx"] * r["dy"]
    assert abs(dxdy * pn.sum() - case["fn"]) <= tol * case["fn"]
    pt = np.hypot(px, py)
    bound = case["fstat"] * pn
    pmax = pn.max()
    assert np.all(pn[igs == 0] == 0.0) and np.all(pn[igs >= 1] >= 0.0)
    assert np.all(pt <= bound + 1e-9 * pmax)
    slip = igs == 2
    assert np.all(np.abs(pt[slip] - bound[slip]) <= 1e-9 * pmax)
    # adhesion elements have no slip
    adh = igs == 1
    assert np.all(r["sx"][adh] == 0.0) and np.all(r["sy"][adh] == 0.0)


@pytest.fixture(scope="module")
def large256(cntc):
    case = C.config1(256)
    plain = run_gpu(cntc, dict(case, mixed=0), ire=75)
    n_plain = ctas(cntc, 75)
    mixed = run_gpu(cntc, dict(case, mixed=1), ire=76)
    n_mixed = ctas(cntc, 76)
    return case, plain, mixed, n_plain, n_mixed


def test_large_256_is_grouped_and_valid(large256):
    """256^2 rough-surface grid (configuration of the grid sweep): solved by a CTA group in
    FP64, the solution satisfies the contact conditions."""
    case, plain, mixed, n_plain, n_mixed = large256
    assert n_plain > 1 and n_mixed > 1
    check_solution(plain, case)
    check_solution(mixed, case)


def test_large_256_mixed_against_fp64(large256):
    """Mixed precision (FP32 convolutions, FP64 refinement) against the FP64 form at 256^2."""
    case, plain, mixed, _, _ = large256
    fe = force_err(mixed, plain, case["fstat"])
    assert fe["fn"] <= 1e-10 and fe["ft"] <= MIXED_FORCE_TOL * 10, fe
    assert int((mixed["igs"] != plain["igs"]).sum()) <= 2


def test_single_call_launch_shape(cntc, oracle):
    """With CNTC_if_groupctas = -1 a single cntc_calculate of a 96 x 96 patch (size class 2^13
    elements) takes the launch shape timed fastest for that class on this device, one CTA or a
    patch group; the result is the oracle's within the parity bar of a converged solution (a
    group sums its reductions in another order, so its GDsteady path differs at the rounding
    level), with the same element division."""
    case = C.config0(gausei=5, eps=1e-10, mx=96, my=96)
    g = run_gpu(cntc, dict(case, group=-1), ire=130)
    shapes = cntc.latency_shapes()
    assert 13 in shapes, shapes
    assert (ctas(cntc, 130) > 1) == shapes[13]
    o = C.oracle_solve(case)
    assert_parity(g, o, case, iterations=False)
    # the default keeps one CTA for a single call
    run_gpu(cntc, case, ire=131)
    assert ctas(cntc, 131) == 1
