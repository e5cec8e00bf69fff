"""The reader of CONTACT's module-3 input files (contact_gb300.inp), on CPU.

Number forms of the program's readline, and the reference's own inputs read into the same
case dicts that the golden tests build by hand (examples/tractcurv.inp, cattaneo.inp,
testbank/testbank.inp), with the cases outside this library reported as unsupported.  The
inputs are the reference's files; where its tree is absent the file tests are skipped (the
performance inputs are also committed in parsed form, tests/golden/perfc_cases.json).
"""
import json
import math
import os

import numpy as np
import pytest

import cases as C
from contact_gb300 import inp

REF = os.environ.get("CONTACT_REFERENCE", "/root/reference")
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _read(rel):
    path = os.path.join(REF, rel)
    if not os.path.exists(path):
        pytest.skip("the reference's input files are not present on this machine")
    return inp.read_inp(open(path).read())


def test_number_forms():
    assert inp.parse_number(".1-07") == pytest.approx(1e-8)
    assert inp.parse_number("1d0") == 1.0 and inp.parse_number("2.5D-3") == 2.5e-3
    assert inp.parse_number("30000.") == 30000.0 and inp.parse_number("1e-5") == 1e-5
    assert inp.parse_number("180.0d", angle=True) == pytest.approx(math.pi)
    assert inp.parse_number("0.5r", angle=True) == 0.5
    with pytest.raises(ValueError):
        inp.parse_number("MAXGS")


KEYS = ("tang", "norm", "bound", "gausei", "maxgs", "maxin", "maxnr", "maxout", "eps", "poiss", "gg", "fstat",
        "fn", "pen", "cksi", "ceta", "cphi", "ipotcn", "dq", "force3", "fxrel", "fyrel")


def _same_case(a, b):
    for k in KEYS:
        if k in b or k in a:
            assert a.get(k) == pytest.approx(b.get(k)), k
    assert a["potprm"] == pytest.approx(b["potprm"])
    if "prmudf" in b:
        assert a["prmudf"] == pytest.approx(b["prmudf"])


def test_tractcurv_first_series():
    cs = _read("examples/tractcurv.inp")
    assert len([c for c in cs if "unsupported" not in c]) == 60
    for c in cs[:30]:
        _same_case(c, C.tractcurv_case(c["cksi"]))
    # series 2: an elastic interfacial layer (M=4), kept by the cases that repeat only the M digit,
    # and exponential falling friction with a friction memory
    for c in cs[30:60]:
        assert (c["mater"], c["gg3"], c["laythk"], c["tau_c0"]) == (4, 8200.0, 1.25, 0.0)
        assert (c["frclaw"], c["memdst"], c["mem_s0"]) == (4, 0.003, 1.0)
    assert "M=3" in cs[60]["unsupported"]                # series 3: FASTSIM
    assert "plastic" in _read("examples/plastic_3bl.inp")[1]["unsupported"]


def test_cattaneo_and_testbank():
    cs = _read("examples/cattaneo.inp")
    _same_case(cs[0], C.cattaneo_case(1))
    _same_case(cs[1], C.cattaneo_forces_case())
    _same_case(_read("examples/catt_to_cart.inp")[0], C.catt_to_cart_case1())
    _same_case(_read("examples/carter2d.inp")[0], C.carter2d_case())        # with an XFLOW line
    tb = _read("testbank/testbank.inp")
    _same_case(tb[0], C.testbank_case(1))
    assert "C=3" in tb[1]["unsupported"]                 # bilinear loading
    sp = _read("examples/spence35.inp")
    assert len(sp) == 35 and sp[1]["pvtime"] == 0 and sp[0]["subs"][0]["isubs"] == 2
    assert sp[0]["subs"][0]["iy"] == [23] and len(sp[0]["subs"][0]["ix"]) == 45 and sp[5]["subs"] == sp[0]["subs"]
    ss = _read("examples/subsurf.inp")
    assert [b["isubs"] for b in ss[0]["subs"]] == [9, 9] and len(ss[0]["subs"][1]["x"]) == 21
    b = _read("examples/bentall.inp")
    assert len(b) == 6 and all("unsupported" not in c for c in b)          # two materials: poiss2, gg2
    assert (b[0]["poiss"], b[0]["poiss2"], b[0]["gg"], b[0]["gg2"]) == (0.31, 0.28, 23000.0, 82000.0)
    assert b[0]["chi"] == pytest.approx(math.pi) and b[1]["iestim"] == 1 and b[1]["force3"] == 1


def test_perfc_fixture_matches_the_inputs():
    """The committed performance cases are the reader's output for the reference's files, and
    their IBASE-2 geometry evaluates to the undeformed distance of the grid."""
    gold = json.load(open(os.path.join(GOLD, "perfc_cases.json")))
    g = gold["cases"][0]
    c = inp.materialize(g["case"])
    assert c["h"].shape == (c["potprm"][0] * c["potprm"][1],) and np.isfinite(c["h"]).all()
    fresh = _read("perfc_test/%s.inp" % g["name"])[0]
    _same_case(fresh, g["case"])
    assert np.array_equal(fresh["h"], c["h"])


DECK = """
 3  MODULE
  {pbtnfs}      P-B-T-N-F-S
  022020        L-D-C-M-Z-E
  0000341     H-G-I-A-O-W-R
   200  100  30  1  1.0E-08           MAXGS, MAXIN, MAXNR, MAXOUT, EPS
   9.1954   {cksi}   0.0   0.0         FN, CKSI, CETA, CPHI
   0.4  0.4                            FSTAT, FKIN
{veloc}   0.42  0.42  200.  200.       POISS 1,2,  GG 1,2
   {ipotcn}                            IPOTCN
   {potline}
{geom}
 0  MODULE
"""


def _deck(ipotcn, potline, geom, tang=1, cksi=0.008155):
    veloc = "   0.0  0.13333  1000.       CHI, DQ, VELOC\n" if tang == 3 else ""
    return DECK.format(pbtnfs="20%d100" % tang, cksi=cksi, veloc=veloc, ipotcn=ipotcn, potline=potline, geom=geom)


QUAD = "   1   1                IBASE, IPLAN\n   0.01 0.0 0.01 0.0 0.0 0.0    B1..B6"


def test_potential_contact_forms_agree(oracle):
    """IPOTCN 1 (lower-left corner and spacing), 2 (corners), 3 (first centre and spacing)
    and 4 (first and last centres) describing the same 19x19 grid read into the same
    element centres, and the oracle gives the same solution for each."""
    forms = [(1, "19 19 -1.26667 -1.26667 0.13333 0.13333"),
             (2, "19 19 -1.26667 -1.26667 1.26660 1.26660"),
             (3, "19 19 -1.200005 -1.200005 0.13333 0.13333"),
             (4, "19 19 -1.200005 -1.200005 1.199935 1.199935")]
    res = []
    for ip, line in forms:
        c = inp.read_inp(_deck(ip, line, QUAD))[0]
        assert c["ipotcn"] == ip and c["tang"] == 1 and c["prmudf"] == pytest.approx([0.01, 0, 0.01, 0, 0, 0])
        res.append(C.oracle_solve(c))
    for r in res[1:]:
        assert np.array_equal(r["igs"], res[0]["igs"])
        assert r["fx"] == pytest.approx(res[0]["fx"], rel=1e-9) and r["fn"] == pytest.approx(res[0]["fn"], rel=1e-12)


def test_geometry_forms_agree(oracle):
    """IBASE 1 (quadratic), 3 (no sines, x^2/p7 + y^2/p8) and 9 (element-wise) describing
    the same undeformed distance give the same solution."""
    pot = "19 19 -1.26667 -1.26667 0.13333 0.13333"
    a = inp.read_inp(_deck(1, pot, QUAD))[0]
    b = inp.read_inp(_deck(1, pot, "   3   1     IBASE, IPLAN\n   0 0 0 0 0 0 100.0 100.0"))[0]
    x = -1.26667 + (np.arange(19) + 0.5) * 0.13333
    X, Y = np.meshgrid(x, x)
    h = 0.01 * X ** 2 + 0.01 * Y ** 2
    body = "\n".join(" ".join("%.17g" % v for v in h.ravel()[k:k + 5]) for k in range(0, 361, 5))
    c = inp.read_inp(_deck(1, pot, "   9   1     IBASE, IPLAN\n" + body))[0]
    assert np.allclose(b["h"], h.ravel(), rtol=0, atol=1e-15) and np.allclose(c["h"], h.ravel(), rtol=0, atol=0)
    ra, rb, rc = (C.oracle_solve(z) for z in (a, b, c))
    for r in (rb, rc):
        assert np.array_equal(r["igs"], ra["igs"]) and r["fx"] == pytest.approx(ra["fx"], rel=1e-9)


def test_rolling_case_reads_the_step_line():
    """T=3 reads CHI, DQ, VELOC; values a later case omits keep their previous value."""
    text = _deck(1, "19 19 -1.26667 -1.26667 0.13333 0.13333", QUAD, tang=3, cksi=-0.001)
    c = inp.read_inp(text)[0]
    assert c["tang"] == 3 and c["dq"] == pytest.approx(0.13333) and c["veloc"] == 1000.0 and "chi" not in c
    two = text.replace(" 0  MODULE", """ 3  MODULE
  203100      P-B-T-N-F-S
  000000      L-D-C-M-Z-E
  0100341     H-G-I-A-O-W-R
   9.1954  -0.002  0.0  0.0      FN, CKSI, CETA, CPHI
   0.3  0.3                      FSTAT, FKIN
 0  MODULE""")
    cs = inp.read_inp(two)
    assert len(cs) == 2 and cs[1]["cksi"] == -0.002 and cs[1]["fstat"] == 0.3
    assert cs[1]["maxgs"] == 200 and cs[1]["potprm"] == cs[0]["potprm"] and cs[1]["prmudf"] == cs[0]["prmudf"]
