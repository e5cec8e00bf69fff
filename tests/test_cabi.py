"""The C-ABI library on the host (CPU only, no compute calls).

Checks that libcontact_addon.so loads, exports every function declared in
include/contact_addon.h with the declared argument count, and that the setter/getter
state handling follows the reference (src/contact_addon.f90): silent return on invalid
input, N=1 after cntc_setnormalforce, N=0 after cntc_setpenetration, finalize forgets a
result element.
"""
import ctypes
import os
import re

import numpy as np
import pytest

import contact_gb300 as cg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "contact_addon.h")


def header_prototypes():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    protos = {}
    for m in re.finditer(r"\b(?:void|int|long long|double)\s+((?:cntc|subs)_\w+)\s*\(([^)]*)\)\s*;", text):
        args = m.group(2).strip()
        protos[m.group(1)] = 0 if args in ("", "void") else len(args.split(","))
    return protos


@pytest.fixture(scope="module")
def lib():
    return cg.load()


def _i(v):
    return ctypes.byref(ctypes.c_int(int(v)))


def getflags(ire, icp, flags):
    f = np.asarray(flags, dtype=np.int32)
    v = np.zeros(len(f), dtype=np.int32)
    cg.load().cntc_getflags(_i(ire), _i(icp), _i(len(f)), f.ctypes.data_as(cg._IP), v.ctypes.data_as(cg._IP))
    return v.tolist()


def test_header_parsed():
    protos = header_prototypes()
    assert len(protos) >= 45
    assert protos["cntc_calculate"] == 3 and protos["cntc_finalizelast"] == 0


def test_every_declared_symbol_exported(lib):
    protos = header_prototypes()
    missing = [name for name in protos if not hasattr(lib, name)]
    assert not missing, missing


def test_python_bindings_match_header():
    protos = header_prototypes()
    assert set(cg._PROTOS) == set(protos)
    for name, nargs in protos.items():
        assert len(cg._PROTOS[name]) == nargs, name


def test_flags_roundtrip(lib):
    ire, icp = 901, 1
    flags = [cg.CNTC_ic_tang, cg.CNTC_ic_bound, cg.CNTC_ic_iestim, cg.CNTC_if_mixedprec, cg.CNTC_if_groupctas]
    cg.setflags(ire, icp, flags, [1, 2, 3, 1, 12])
    assert getflags(ire, icp, flags) == [1, 2, 3, 1, 12]
    cg.setflags(ire, icp, [cg.CNTC_if_groupctas], [-4])          # negative: automatic
    assert getflags(ire, icp, [cg.CNTC_if_groupctas]) == [0]
    cg.finalize(ire)


def test_normal_problem_switch(lib):
    """cntc_setnormalforce sets N=1, cntc_setpenetration N=0 (contact_addon.f90:2294-2357)."""
    ire, icp = 902, 1
    cg.setnormalforce(ire, icp, 5e4)
    assert getflags(ire, icp, [cg.CNTC_ic_norm]) == [1]
    cg.setpenetration(ire, icp, 0.1)
    assert getflags(ire, icp, [cg.CNTC_ic_norm]) == [0]
    cg.finalize(ire)


def test_invalid_input_returns_silently(lib):
    """Setters ignore invalid input (contact_addon.f90:1162-1173): a Hertz call with the wrong
    number of parameters leaves the grid as it was."""
    ire, icp = 903, 1
    cg.sethertzcontact(ire, icp, -3, [31, 21, 6.0, 4.0, 1.1])
    assert cg.getnumelements(ire, icp) == (31, 21)
    cg.sethertzcontact(ire, icp, -3, [17, 17, 6.0, 4.0])          # nparam 4: invalid for ipotcn -3
    assert cg.getnumelements(ire, icp) == (31, 21)
    cg.sethertzcontact(ire, icp, -9, [17, 17, 6.0, 4.0, 1.1])     # no such ipotcn
    assert cg.getnumelements(ire, icp) == (31, 21)
    cg.finalize(ire)


def test_creepages_and_velocity_roundtrip(lib):
    ire, icp = 904, 2
    cg.setcreepages(ire, icp, 0.002, -0.001, 3e-4)
    cg.setreferencevelocity(ire, icp, 12345.0)
    vx, vy, phi = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    lib.cntc_getcreepages(_i(ire), _i(icp), ctypes.byref(vx), ctypes.byref(vy), ctypes.byref(phi))
    assert (vx.value, vy.value, phi.value) == (0.002, -0.001, 3e-4)
    v = ctypes.c_double()
    lib.cntc_getreferencevelocity(_i(ire), _i(icp), ctypes.byref(v))
    assert v.value == 12345.0
    cg.finalize(ire)


def test_finalize_forgets_problem(lib):
    ire, icp = 905, 1
    cg.setflags(ire, icp, [cg.CNTC_ic_tang], [1])
    assert getflags(ire, icp, [cg.CNTC_ic_tang]) == [1]
    cg.finalize(ire)
    assert getflags(ire, icp, [cg.CNTC_ic_tang]) == [0]


def test_unknown_problem_getters_leave_output(lib):
    """Getters on an unknown (ire, icp) write nothing."""
    fn = ctypes.c_double(-7.0)
    z = ctypes.c_double(-7.0)
    lib.cntc_getcontactforces(_i(999), _i(9), ctypes.byref(fn), ctypes.byref(z), ctypes.byref(z), ctypes.byref(z))
    assert fn.value == -7.0
