"""Subsurface stresses in the CPU oracle (oracle/orc_subsurf.hpp) against the reference's printed
field (examples/subsurf.ref_subs, .ref_out; fixture tests/golden/subsurf.json) of the oracle's
own solves of examples/subsurf.inp, against Love's closed form for the stress below a uniformly
loaded rectangle, and its FFT path (element centres, per-depth influence coefficients) against
its direct path.
"""
import json
import math
import os

import numpy as np
import pytest

import cases as C

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# fixture columns X Y Z UX UY UZ SIGHYD SIGVM SIGXX SIGXY SIGXZ SIGYY SIGYZ SIGZZ -> oracle columns
ORC = {"UX": 0, "UY": 1, "UZ": 2, "SIGHYD": 3, "SIGVM": 4, "SIGTR": 5, "SIGMA1": 6, "SIGMA3": 8, "SIGXX": 9,
       "SIGXY": 10, "SIGXZ": 11, "SIGYY": 13, "SIGYZ": 14, "SIGZZ": 17}


@pytest.fixture(scope="module")
def gold():
    with open(os.path.join(GOLD, "subsurf.json")) as f:
        return json.load(f)


def _half_unit(tok):
    """Half a unit of the last digit a value was printed with ('0.482073', '2.0902E-05')."""
    t = tok.upper()
    if "E" in t:
        mant, ex = t.split("E")
        return 0.5 * 10.0 ** (int(ex) - (len(mant.split(".")[1]) if "." in mant else 0))
    return 0.5 * 10.0 ** (-(len(t.split(".")[1]) if "." in t else 0))


_SOLVES = {}


def _solve(case):
    if case not in _SOLVES:
        _SOLVES[case] = C.oracle_solve(C.subsurf_case(case))
    return _SOLVES[case]


def _field(po, g, case, pts):
    """The field of the oracle's own solution of the example's case (1: pressure alone,
    2: pressure and the traction found by ConvexGS and Newton-Raphson)."""
    r = _solve(case)
    grid = (r["mx"], r["my"], r["dx"], r["dy"], r["xc1"], r["yc1"])
    return po.subsurf_points(grid, r["pn"], r["px"], r["py"], g["gg"], g["poiss"], pts)


def test_solves_of_the_example(oracle, gold):
    """The two solves of examples/subsurf.inp as printed: the normal problem, and steady rolling
    with Fx prescribed on the single element (ConvexGS inside a Newton-Raphson on cksi, three
    iterations of two sweeps): forces, moment, elastic energy, approach, pmax to 4 digits,
    counts and iterations exact, the Newton-Raphson rows and dFx/dcksi as printed."""
    for g in gold["solves"]:
        o = _solve(g["case"])
        assert o["ierror"] >= 0 and o["itcg"] == g["norm_itcg"]
        for key, gk in (("fn", "fn"), ("fx", "fx"), ("mz", "mz"), ("elen", "elen"), ("pen", "approach"),
                        ("pmax", "pmax")):
            gold_v = g[gk]
            unit = 0.5e-4 if gold_v == 0.0 else 0.5 * 10.0 ** (math.floor(math.log10(abs(gold_v))) - 3)
            assert abs(o[key] - gold_v) <= unit * (1 + 1e-9), (g["case"], key, o[key], gold_v)
        assert (o["ncon"], o["nadh"], o["nslip"]) == (g["ncon"], g["nadh"], g["nslip"])
        if "nr" in g:
            assert o["solver"] == 3 and o["itgs"] == g["tang_it"]
            assert [int(r[6]) for r in o["nr"]] == [r[5] for r in g["nr"]]
            for row, gr in zip(o["nr"], g["nr"]):
                for k, gk in ((2, 1), (3, 2)):
                    unit = 0.5 * 10.0 ** (math.floor(math.log10(abs(gr[gk]))) - 3)
                    assert abs(row[k] - gr[gk]) <= unit * (1 + 1e-9), (row, gr)
            assert abs(o["sens"][1][1] - g["sens"][1][1]) <= 0.005


def test_field_against_printed_table(oracle, gold):
    """All printed values of block 1 and of the 7x7 subgrid of block 2 (case 2: the pressure and
    traction of the oracle's solve, 1 and 0.999): displacements, hydrostatic and von Mises stress and the six
    stress components within half a unit of their last printed digit.  Components that vanish
    (the shear stresses on the free surface) print as rounding residues of order 1e-14; those
    are held to 1e-12 of their column's largest value instead."""
    import pyoracle as po
    cols = gold["columns"][3:]
    for rows in (gold["block1"], gold["block2_subgrid"]):
        pts = np.array([[float(v) for v in r[:3]] for r in rows])
        o = _field(po, gold, 2, pts)
        g = np.array([[float(v) for v in r[3:]] for r in rows])
        scale = np.abs(g).max(axis=0)
        for q, r in enumerate(rows):
            for c, name in enumerate(cols):
                tol = max(_half_unit(r[3 + c]) * (1 + 1e-9), 1e-12 * scale[c])
                assert abs(o[q, ORC[name]] - g[q, c]) <= tol, (r[:3], name, o[q, ORC[name]], r[3 + c])


def test_block_summaries(oracle, gold):
    """The printed maxima of both cases (pressure alone; pressure and traction) over both blocks:
    hydrostatic (largest magnitude), von Mises, Tresca, largest and smallest principal stress
    and sigma_xx, yy, zz (largest magnitude), to the printed 3 decimals and at the printed
    position."""
    import pyoracle as po
    b1 = np.array([[float(v) for v in r[:3]] for r in gold["block1"]])
    X, Y, Z = np.meshgrid(gold["block2_x"], gold["block2_y"], gold["block2_z"], indexing="xy")
    b2 = np.stack([X.transpose(2, 0, 1).ravel(), Y.transpose(2, 0, 1).ravel(), Z.transpose(2, 0, 1).ravel()], 1)
    fields = {(case, blk): (pts, _field(po, gold, case, pts)) for case in (1, 2) for blk, pts in ((1, b1), (2, b2))}
    assert len(gold["summaries"]) == 32
    for s in gold["summaries"]:
        pts, o = fields[(s["case"], s["block"])]
        col = o[:, ORC[s["quantity"]]]
        i = int(np.argmax(np.abs(col)) if s["kind"] == "ABSMAX" else np.argmax(col) if s["kind"] == "MAX"
                else np.argmin(col))
        assert abs(col[i] - s["value"]) <= 0.5e-3 * (1 + 1e-9), s
        assert np.allclose(np.round(pts[i], 3), s["at"]), (s, pts[i])


def test_love_rectangle_axis(oracle):
    """sigma_zz on the axis below a uniform pressure p on a 2a x 2b rectangle (Love 1929; the sum
    of four corner rectangles): -(2p/pi) [atan(ab/(zR)) + abz/R (1/(a^2+z^2) + 1/(b^2+z^2))],
    R^2 = a^2 + b^2 + z^2, independent of the material."""
    import pyoracle as po
    a, b = 0.5, 0.75
    z = np.array([0.05, 0.2, 0.5, 1.0, 3.0])
    pts = np.stack([np.zeros_like(z), np.zeros_like(z), z], 1)
    o = po.subsurf_points((1, 1, 2 * a, 2 * b, 0.0, 0.0), [2.0], [0.0], [0.0], 1.0, 0.3, pts)
    for k, zz in enumerate(z):
        r = math.sqrt(a * a + b * b + zz * zz)
        love = -(2 * 2.0 / math.pi) * (math.atan(a * b / (zz * r)) + a * b * zz / r * (1 / (a * a + zz * zz) +
                                                                                         1 / (b * b + zz * zz)))
        assert o[k, ORC["SIGZZ"]] == pytest.approx(love, rel=1e-9, abs=1e-12), (zz, o[k, ORC["SIGZZ"]], love)


def test_fft_path_equals_direct_path(oracle):
    """At the element centres of a real solution (examples/cattaneo.inp case 2: pressure and
    traction on 177 of 361 elements), the influence-coefficient + FFT path equals the direct
    sum to 1e-12 of each column's largest value below the surface.  On the surface the two
    differ by up to 1e-5: the FFT path's coefficients come from one quadrant by mirror
    symmetry, which the direct formula's perturbation of zero coordinates (5e-7 of the
    distance) does not have exactly."""
    import pyoracle as po
    r = C.oracle_solve(C.cattaneo_case(2, 0.008155))
    mx, my = r["mx"], r["my"]
    grid = (mx, my, r["dx"], r["dy"], r["xc1"], r["yc1"])
    z = np.array([0.0, 0.05, 0.2, 0.6, 1.5])
    f = po.subsurf_depths(grid, r["pn"], r["px"], r["py"], 200.0, 0.42, z)
    xs = r["xc1"] + r["dx"] * np.arange(mx)
    ys = r["yc1"] + r["dy"] * np.arange(my)
    XX, YY = np.meshgrid(xs, ys)
    pts = np.stack([np.tile(XX.ravel(), len(z)), np.tile(YY.ravel(), len(z)), np.repeat(z, mx * my)], 1)
    d = po.subsurf_points(grid, r["pn"], r["px"], r["py"], 200.0, 0.42, pts).reshape(len(z), mx * my, -1)
    scale = np.abs(d).max(axis=(0, 1)) + 1e-300
    err = (np.abs(f - d) / scale).max(axis=(1, 2))
    assert err[0] <= 1e-5 and (err[1:] <= 1e-12).all(), err


def test_spence35_sequence(oracle):
    """examples/spence35.inp replayed in order, all 35 load steps of Spence's problem: a body of
    one material (G 0.5) pressed into and lifted off one of another (G 1e5), the normal and
    tangential problems coupled (K != 0), each step continuing from the previous one (P=0).
    Every printed outer iteration (the change of the tractions and its tolerance, 4 digits)
    and their number, totals to 4 digits and counts where printed; and the printed maxima of
    the subsurface stresses along one grid row at z = 1e-6 (the element-centre FFT path) in
    steps 6, 18 and 35, to 3 decimals and at the printed position."""
    import pyoracle as po

    def p4(x, gold):
        if gold == 0.0:
            return abs(x) < 5e-4
        return abs(x - gold) <= 0.5 * 10.0 ** (math.floor(math.log10(abs(gold))) - 3) * (1 + 1e-9)

    with open(os.path.join(GOLD, "spence35.json")) as f:
        g = json.load(f)
    res = C.replay_oracle(g["inputs"])
    assert len(res) == len(g["cases"]) == 35
    nsum = 0
    for c, gc, o in zip(g["inputs"], g["cases"], res):
        assert o["ierror"] >= 0
        assert len(o["outer"]) == len(gc["outer"]), gc["case"]
        for k, (a, b) in enumerate(gc["outer"]):
            assert p4(o["outer"][k][0], a) and p4(o["outer"][k][1], b), (gc["case"], k)
        for key, gk in (("fn", "fn"), ("fx", "fx"), ("fy", "fy"), ("elen", "elen"), ("pen", "approach"),
                        ("pmax", "pmax")):
            assert p4(o[key], gc[gk]), (gc["case"], key, o[key], gc[gk])
        if "ncon" in gc:
            assert (o["ncon"], o["nadh"], o["nslip"]) == (gc["ncon"], gc["nadh"], gc["nslip"])
        if "subs" in gc:
            b = c["subs"][0]
            grid = (o["mx"], o["my"], o["dx"], o["dy"], o["xc1"], o["yc1"])
            f = po.subsurf_depths(grid, o["pn"], o["px"], o["py"], (c["gg"], c.get("gg2", c["gg"])),
                                  (c["poiss"], c.get("poiss2", c["poiss"])), b["z"])
            sel = [(ix - 1) + (iy - 1) * o["mx"] for iy in b["iy"] for ix in b["ix"]]
            pts = [(o["xc1"] + (ix - 1) * o["dx"], o["yc1"] + (iy - 1) * o["dy"]) for iy in b["iy"] for ix in b["ix"]]
            for s in gc["subs"]:
                col = f[0][sel, ORC[s["quantity"]]]
                i = int(np.argmax(np.abs(col)) if s["kind"] == "ABSMAX" else np.argmax(col) if s["kind"] == "MAX"
                        else np.argmin(col))
                assert abs(col[i] - s["value"]) <= 0.5e-3 * (1 + 1e-9), (gc["case"], s)
                assert np.allclose(np.round(pts[i], 3), s["at"][:2]), (gc["case"], s, pts[i])
                nsum += 1
    assert nsum == 24


def test_two_bodies_at_points(oracle):
    """testbank/testbank.inp case 3: the normal problem of two bodies (G 200 above, 1 below) with
    one element in contact, and the field at six points on both sides of the surface (z = -1 in
    the soft body, 0.2 and 1 in the stiff one): the approach and pmax as printed, every printed
    displacement, stress component, SigHyd and SigVM within half a unit of its last digit, and
    the block's maxima at their printed positions."""
    import pyoracle as po
    g = json.load(open(os.path.join(GOLD, "testbank_case3_subs.json")))
    o = C.oracle_solve(C.testbank_case(3))
    assert o["ierror"] == 0 and o["itcg"] == g["norm_itcg"] and o["ncon"] == 1
    assert abs(o["pen"] - g["approach"]) <= 0.5e-6 and abs(o["pmax"] - g["pmax"]) <= 0.5e-3
    pts = np.array([[float(v) for v in r[:3]] for r in g["points"]])
    f = po.subsurf_points((o["mx"], o["my"], o["dx"], o["dy"], o["xc1"], o["yc1"]), o["pn"], o["px"], o["py"],
                          [200.0, 1.0], [0.28, 0.28], pts)
    at = {n: k for k, n in enumerate(po.SUBS_COLS)}
    at.update(sigxx=at["sxx"], sigyy=at["syy"], sigzz=at["szz"])
    cols = ["ux", "uy", "uz", "sxx", "sxy", "sxz", "syx", "syy", "syz", "szx", "szy", "szz", "sighyd", "sigvm"]
    for q, r in enumerate(g["points"]):
        for c, name in enumerate(cols):
            assert abs(f[q, at[name]] - float(r[3 + c])) <= _half_unit(r[3 + c]) * (1 + 1e-9), (r[:3], name)
    for sm in g["summaries"]:
        col = f[:, at[sm["quantity"]]]
        i = int(np.argmax(np.abs(col)) if sm["kind"] == "ABSMAX" else np.argmax(col) if sm["kind"] == "MAX"
                else np.argmin(col))
        assert abs(col[i] - sm["value"]) <= 0.5e-3 * (1 + 1e-9) and np.allclose(pts[i], sm["at"]), sm
