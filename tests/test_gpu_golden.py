"""The GB300 library through its C-ABI against the reference's own printed outputs.

Beside the oracle tests of the same fixtures (tests/test_oracle.py), these run the reference's
call sequences through this library: src/test_caddon.f90's result element 1 in SPCK units
(lengths in m, forces on body 2), and the two cases of examples/cattaneo.inp (NormCG, and
TangCG on the shift problem) in CONTACT units.
"""
import ctypes
import json
import math
import os

import numpy as np
import pytest

import cases as C

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


def _near(x, gold, decimals):
    return abs(x - gold) <= 0.5 * 10.0 ** (-decimals) * (1 + 1e-9)


def _printed4(x, gold):
    if gold == 0.0:
        return abs(x) < 5e-4
    unit = 10.0 ** (math.floor(math.log10(abs(gold))) - 3)
    return abs(x - gold) <= 0.5 * unit * (1 + 1e-9)


def test_caddon_element1_spck_units(cntc):
    """src/test_caddon.f90:95-230 for result element 1, the same calls in SPCK units."""
    g = _load("test_caddon_re1.json")["result"]
    ire, icp = 41, 2
    cntc.setflags(ire, icp, [cntc.CNTC_if_units], [cntc.CNTC_un_spck])
    cntc.setreferencevelocity(ire, icp, 24.0)                       # m/s
    cntc.setrollingstepsize(ire, icp, 0.0, 0.0005)                  # m
    cntc.setcreepages(ire, icp, 0.001, 0.0, 0.4)                    # spin in rad/m
    cntc.setmaterialparameters(ire, icp, 0, [0.28, 0.28, 82000e6, 82000e6])
    cntc.setfrictionmethod(ire, icp, 0, [0.3, 0.3])
    cntc.setpenetration(ire, icp, 0.00005)
    cntc.sethertzcontact(ire, icp, -3, [21.0, 33.0, 0.00425, 0.007, 21.0 / 17.0])
    cntc.setsolverflags(ire, icp, 0, [999, 30, 30, 1], [0.0001])
    assert cntc.calculate(ire, icp) == 0
    dx, dy = cntc.getgriddiscretization(ire, icp)
    assert _near(dx, g["dx_m"], 5) and _near(dy, g["dy_m"], 5)
    assert cntc.getnumelements(ire, icp) == (g["mx"], g["my"])
    fn, fx, fy, mz = cntc.getcontactforces(ire, icp)
    assert _near(fn, g["tn"], 1) and _near(fx, g["fx"], 1) and _near(fy, g["fy"], 1) and _near(mz, g["mz_nm"], 1)
    carea, harea, sarea = cntc.getcontactpatchareas(ire, icp)
    assert _near(carea, g["carea_m2"], 6) and _near(harea, g["harea_m2"], 6) and _near(sarea, g["sarea_m2"], 6)
    assert _near(cntc.getmaximumpressure(ire, icp) / 1e6, g["pnmax_mpa"], 1)
    pt = ctypes.c_double()
    cntc.load().cntc_getmaximumtraction(ctypes.byref(ctypes.c_int(ire)), ctypes.byref(ctypes.c_int(icp)),
                                        ctypes.byref(pt))
    assert _near(pt.value / 1e6, g["ptmax_mpa"], 1)
    pn, px, py = cntc.gettractions(ire, icp)
    mx = g["mx"]
    for key, arr in (("pn_max", pn), ("px_max", px), ("py_max", py)):
        i = int(np.argmax(np.abs(arr)))
        assert [i % mx + 1, i // mx + 1] == g[key][:2], key
        assert _near(arr[i] / 1e6, g[key][2], 1), key
    cntc.finalize(ire)


@pytest.mark.parametrize("icase", [1, 2])
def test_cattaneo_cases(cntc, icase):
    """examples/cattaneo.inp: forces, approach, pmax to the printed 4 digits; element counts,
    NormCG iterations and the element-division picture exact."""
    g = [c for c in _load("cattaneo.json")["cases"] if c["case"] == icase][0]
    ire = 42
    cntc.setup_case(ire, 1, C.cattaneo_case(icase, g.get("cksi", 0.0)))
    assert cntc.calculate(ire, 1) == 0
    r = cntc.results(ire, 1)
    for key, gk in (("fn", "fn"), ("fx", "fx"), ("pen", "approach"), ("pmax", "pmax")):
        assert _printed4(r[key], g[gk]), (key, r[key], g[gk])
    assert (r["ncon"], r["nadh"], r["nslip"]) == (g["ncon"], g["nadh"], g["nslip"])
    assert r["itcg"] == g["norm_itcg"]
    sym = {0: ".", 1: "*", 2: "S", 3: "P"}
    pic = ["".join(sym[int(r["igs"][iy * 19 + ix])] for ix in range(19)) for iy in range(19)]
    assert pic == [row.replace("o", ".") for row in g["picture"]]
    cntc.finalize(ire)
