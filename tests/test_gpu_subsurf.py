"""Subsurface stresses on the GPU (subs_addBlock / subs_calculate / subs_getResults, module 3)
against the reference's printed maxima of its own example (examples/subsurf.ref_out, fixture
tests/golden/subsurf.json) and against the oracle's two forms on the same tractions: the direct
sum at arbitrary points, and the influence-coefficient path at element centres."""
import json
import os

import numpy as np
import pytest

import cases as C

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# oracle column of each library column (oracle: ux uy uz sighyd sigvm sigtr sigma1..3 sig row by row)
ORC = {"ux": 0, "uy": 1, "uz": 2, "sighyd": 3, "sigvm": 4, "sigtr": 5, "sigma1": 6, "sigma2": 7, "sigma3": 8,
       "sigxx": 9, "sigxy": 10, "sigxz": 11, "sigyx": 12, "sigyy": 13, "sigyz": 14, "sigzx": 15, "sigzy": 16,
       "sigzz": 17}
FIELD = [c for c in ORC]
# The principal stresses come from the trigonometric (Cardano) solution of the characteristic
# cubic, as in the reference (m_subsurf.f90:2440-2490, Cardano's algorithm): near a
# repeated eigenvalue (sigma1 = sigma2 on the axis below a symmetric load) acos(r) with r
# close to +-1 turns a rounding difference dr into an angle of order sqrt(dr), so two
# evaluations of the same formula agree to about 1e-8 of the stresses there, not to 1e-11.
PRINCIPAL_TOL = {"sigma1": 5e-8, "sigma2": 5e-8, "sigma3": 5e-8, "sigtr": 5e-8}


def test_example_against_printed_table(cntc, oracle):
    """examples/subsurf.inp case 1 solved on the GPU (the normal problem on its single element:
    pressure 1 on 1 x 1 mm), then its field on the GPU at the example's two blocks: block 1 (a
    column below the centre) and block 2 (21 x 21 x 15 points).  The printed maxima of case 1
    (largest hydrostatic stress, von Mises, Tresca, principal stresses, sigma_xx, yy, zz) to
    the printed 3 decimals and at the printed position; every point within 1e-11 of the
    largest displacement (stress) of the oracle's direct sum of the same pressure (principal
    stresses near a repeated eigenvalue: 5e-8).  (Case 2 adds a
    traction found by ConvexGS on a single column, which is not on the device; its printed
    table is held against the oracle's own solve on the CPU.)"""
    import pyoracle as po
    with open(os.path.join(GOLD, "subsurf.json")) as f:
        g = json.load(f)
    ire, icp = 140, 1
    cntc.setup_case(ire, icp, C.subsurf_case(1))
    assert cntc.calculate(ire, icp) >= 0
    res = cntc.results(ire, icp)
    assert (res["mx"], res["my"]) == (1, 1)
    solve = [s for s in g["solves"] if s["case"] == 1][0]
    assert abs(res["pn"].max() - solve["pmax"]) <= 0.5e-4
    b1 = np.array([[float(v) for v in r[:3]] for r in g["block1"]])
    cntc.subs_addblock(ire, icp, 1, 9, [b1[0, 0]], [b1[0, 1]], b1[:, 2])
    cntc.subs_addblock(ire, icp, 2, 9, g["block2_x"], g["block2_y"], g["block2_z"])
    assert cntc.subs_calculate(ire, icp) == 0
    assert cntc.subs_getblocksize(ire, icp, 1) == (1, 1, len(b1))
    nx, ny, nz = len(g["block2_x"]), len(g["block2_y"]), len(g["block2_z"])
    assert cntc.subs_getblocksize(ire, icp, 2) == (nx, ny, nz)
    out = {1: cntc.subs_getresults(ire, icp, 1), 2: cntc.subs_getresults(ire, icp, 2)}
    pot = C.subsurf_case(1)["potprm"]                       # first corner, element size
    grid = (res["mx"], res["my"], res["dx"], res["dy"], pot[2] + 0.5 * pot[4], pot[3] + 0.5 * pot[5])
    for blk, r in out.items():
        pts = np.stack([r["x"], r["y"], r["z"]], 1)
        d = po.subsurf_points(grid, res["pn"], res["px"], res["py"], g["gg"], g["poiss"], pts)
        for name in FIELD:
            # against the largest value of the column's group (displacements, stresses): a
            # column that nearly vanishes (ux on the axis) carries the group's rounding
            grp = FIELD[:3] if name in FIELD[:3] else FIELD[3:]
            scale = max(np.abs(d[:, ORC[c]]).max() for c in grp)
            assert np.abs(r[name] - d[:, ORC[name]]).max() <= PRINCIPAL_TOL.get(name, 1e-11) * scale, (blk, name)
    # block 2 points: x fastest, then y, then z
    assert np.allclose(out[2]["x"][:nx], sorted(g["block2_x"]))
    summ = [s for s in g["summaries"] if s["case"] == 1]
    assert len(summ) == 16
    for s in summ:
        r = out[s["block"]]
        col = r[s["quantity"].lower()]
        i = int(np.argmax(np.abs(col)) if s["kind"] == "ABSMAX" else np.argmax(col) if s["kind"] == "MAX"
                else np.argmin(col))
        assert abs(col[i] - s["value"]) <= 0.5e-3 * (1 + 1e-9), s
        assert np.allclose(np.round([r["x"][i], r["y"][i], r["z"][i]], 3), s["at"]), s


def test_element_centres_and_points_against_oracle(cntc, oracle):
    """Hertzian steady rolling on 51 x 51 (GDsteady, FP64), then its field on the GPU: every
    element centre at four listed depths from the surface (block type 5), a subgrid of centres at listed
    depths (type 6), and explicit points in both bodies (type 9, z < 0 below the surface of body
    2).  Centres: the oracle's influence-coefficient path on the same tractions, within 1e-10 of
    each column's largest value (the GPU sums the tabulated coefficients directly, the oracle by
    FFT); points: the oracle's direct sum within 1e-11 of the largest displacement (stress)."""
    ire, icp = 141, 1
    case = C.config0(gausei=5, eps=1e-10)
    cntc.setup_case(ire, icp, case)
    assert cntc.calculate(ire, icp) >= 0
    res = cntc.results(ire, icp)
    mx, my = res["mx"], res["my"]
    zc = [0.0, 0.4, 1.0, 2.5]
    cntc.subs_addblock(ire, icp, 1, 5, [], [], zc)
    cntc.subs_addblock(ire, icp, 2, 6, [3, 4, 49], [10, 7, 40], [0.3, 1.2])
    px_, py_, pz_ = [-3.0, 0.1, 2.2], [-1.5, 0.0, 2.0], [-0.8, 0.05, 0.7]
    cntc.subs_addblock(ire, icp, 3, 9, px_, py_, pz_)
    assert cntc.subs_calculate(ire, icp) == 0
    r1 = cntc.subs_getresults(ire, icp, 1)
    assert cntc.subs_getblocksize(ire, icp, 1) == (mx, my, len(zc))
    xc1, yc1 = r1["x"][0], r1["y"][0]
    grid = (mx, my, res["dx"], res["dy"], xc1, yc1)
    gg, nu = case["gg"], case["poiss"]
    f = oracle.subsurf_depths(grid, res["pn"], res["px"], res["py"], gg, nu, np.array(zc))   # (nz, n, 18)
    for name in FIELD:
        got = r1[name].reshape(len(zc), mx * my)
        ref = f[:, :, ORC[name]]
        scale = np.abs(ref).max() + 1e-300
        assert np.abs(got - ref).max() <= 1e-10 * scale, (name, np.abs(got - ref).max() / scale)
    # type 6: ix 3, 7, ..., 47; iy 10, 17, ..., 38 at z 0.3, 1.2
    r2 = cntc.subs_getresults(ire, icp, 2)
    ixs, iys = list(range(3, 50, 4)), list(range(10, 41, 7))
    assert cntc.subs_getblocksize(ire, icp, 2) == (len(ixs), len(iys), 2)
    f2 = oracle.subsurf_depths(grid, res["pn"], res["px"], res["py"], gg, nu, np.array([0.3, 1.2]))
    sel = [(ix - 1) + (iy - 1) * mx for iy in iys for ix in ixs]
    for name in FIELD:
        ref = f2[:, sel, ORC[name]].ravel()
        scale = np.abs(ref).max() + 1e-300
        assert np.abs(r2[name] - ref).max() <= 1e-10 * scale, name
    # type 9: explicit points, x fastest, then y, then z (sorted)
    r3 = cntc.subs_getresults(ire, icp, 3)
    X, Y, Z = np.meshgrid(sorted(px_), sorted(py_), sorted(pz_), indexing="ij")
    pts = np.stack([X.transpose(2, 1, 0).ravel(), Y.transpose(2, 1, 0).ravel(), Z.transpose(2, 1, 0).ravel()], 1)
    assert np.allclose(np.stack([r3["x"], r3["y"], r3["z"]], 1), pts)
    d = oracle.subsurf_points(grid, res["pn"], res["px"], res["py"], gg, nu, pts)
    for name in FIELD:
        grp = FIELD[:3] if name in FIELD[:3] else FIELD[3:]
        scale = max(np.abs(d[:, ORC[c]]).max() for c in grp)
        assert np.abs(r3[name] - d[:, ORC[name]]).max() <= PRINCIPAL_TOL.get(name, 1e-11) * scale, name
