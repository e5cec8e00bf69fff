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
        "fn", "pen", "cksi", "ceta", "cphi", "ipotcn", "dq")


def _same_case(a, b):
    for k in KEYS:
        if k in b or k in a:
            assert a.get(k) == pytest.approx(b.get(k)), k
    assert a["potprm"] == pytest.approx(b["potprm"])
    if "prmudf" in b:
        assert a["prmudf"] == pytest.approx(b["prmudf"])


def test_tractcurv_first_series():
    cs = _read("examples/tractcurv.inp")
    assert len([c for c in cs if "unsupported" not in c]) == 30
    assert "unsupported" in cs[30]                       # series 2: falling friction, interface layer
    for c in cs[:30]:
        _same_case(c, C.tractcurv_case(c["cksi"]))


def test_cattaneo_and_testbank():
    cs = _read("examples/cattaneo.inp")
    _same_case(cs[0], C.cattaneo_case(1))
    assert "total forces prescribed" in cs[1]["unsupported"]
    tb = _read("testbank/testbank.inp")
    _same_case(tb[0], C.testbank_case(1))
    assert "C=3" in tb[1]["unsupported"]                 # bilinear loading
    assert "different materials" in _read("examples/bentall.inp")[0]["unsupported"]


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
