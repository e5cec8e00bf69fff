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

import cases as C
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
    cg.setflags(ire, icp, [cg.CNTC_if_groupctas], [-1])          # -1: tuned per size class
    assert getflags(ire, icp, [cg.CNTC_if_groupctas]) == [-1]
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


def _getparameters(lib, ire, icp, itask, n=30):
    v = np.full(n, -1.0)
    lib.cntc_getparameters(_i(ire), _i(icp), _i(itask), _i(n), v.ctypes.data_as(cg._DP))
    return v


def test_getparameters_material_friction_kinematics(lib):
    """cntc_getParameters (contact_addon.f90:4164-4258): itask 2 material with combin_mater's
    ga, nu and ak, itask 3 the Coulomb friction, itask 1 the kinematics; values in the
    selected units (SI: moduli in N/m^2, velocity in m/s)."""
    ire, icp = 906, 1
    cg.setmaterialparameters(ire, icp, 0, [0.3, 0.25, 80000.0, 90000.0])
    cg.setfrictionmethod(ire, icp, 0, [0.35, 0.3])
    cg.setreferencevelocity(ire, icp, 20000.0)
    m = _getparameters(lib, ire, icp, 2)
    ga = 2.0 / (1 / 80000.0 + 1 / 90000.0)
    assert m[:3] == pytest.approx([80000.0, 90000.0, ga])
    assert m[3:6] == pytest.approx([0.3, 0.25, ga * (0.3 / 80000.0 + 0.25 / 90000.0) / 2])
    assert m[6] == pytest.approx((ga / 4) * ((1 - 0.6) / 80000.0 - (1 - 0.5) / 90000.0))
    assert np.all(m[7:22] == 0.0) and np.all(m[22:] == -1.0)     # only 22 values are written
    f = _getparameters(lib, ire, icp, 3)
    # L = 0 keeps one coefficient, the smaller of fstat and fkin (contact_addon.f90:1817-1822)
    assert f[:7] == pytest.approx([0, 1, 0, 0, 0, 0.3, 0.3])
    k = _getparameters(lib, ire, icp, 1)
    assert k[0] == 20000.0 and np.all(k[6:] == -1.0)
    cg.setflags(ire, icp, [cg.CNTC_if_units], [cg.CNTC_un_si])
    assert _getparameters(lib, ire, icp, 2)[0] == pytest.approx(80000.0 * 1e6)
    assert _getparameters(lib, ire, icp, 1)[0] == pytest.approx(20.0)
    short = _getparameters(lib, ire, icp, 2, n=2)                 # lenarr bounds the output
    assert short.size == 2
    cg.finalize(ire)


def test_entry_points_outside_the_solve_path(lib):
    """Wheel-rail and input-file entry points exist and report 'not supported': outputs zeroed,
    ierror CNTC_err_other; metadata is accepted; temperatures are zero.  Subsurface stresses of
    a problem without a solution are refused (CNTC_err_other); an unknown block has no points
    and leaves the output array as it was (src/contact_addon.f90:6147-6150)."""
    ire, icp = 907, 1
    cg.setnormalforce(ire, icp, 1e4)
    ierr = ctypes.c_int(0)
    name = b"track.inp"
    lib.cntc_readinpfile(_i(ire), _i(1), name, _i(len(name)), ctypes.byref(ierr))
    assert ierr.value == cg.CNTC_err_other
    lib.subs_calculate(_i(ire), _i(icp), ctypes.byref(ierr))
    assert ierr.value == -99
    npatch = ctypes.c_int(5)
    lib.cntc_getnumcontactpatches(_i(ire), ctypes.byref(npatch))
    assert npatch.value == 0
    v = np.full(6, 3.0)
    lib.cntc_getcontactlocation(_i(ire), _i(icp), _i(6), v.ctypes.data_as(cg._DP))
    assert np.all(v == 0.0)
    nx, ny, nz = ctypes.c_int(1), ctypes.c_int(1), ctypes.c_int(1)
    lib.subs_getblocksize(_i(ire), _i(icp), _i(1), ctypes.byref(nx), ctypes.byref(ny), ctypes.byref(nz))
    assert (nx.value, ny.value, nz.value) == (0, 0, 0)
    w = np.full((2, 3), 4.0)
    icol = np.zeros(2, dtype=np.int32)
    lib.subs_getresults(_i(ire), _i(icp), _i(1), _i(3), _i(2), icol.ctypes.data_as(cg._IP), w.ctypes.data_as(cg._DP))
    assert np.all(w == 4.0)
    params = np.array([1], dtype=np.int32)
    vals = np.array([0.5])
    lib.cntc_setmetadata(_i(ire), _i(icp), _i(1), params.ctypes.data_as(cg._IP), vals.ctypes.data_as(cg._DP))
    t1, t2 = ctypes.c_double(-1), ctypes.c_double(-1)
    lib.cntc_getmaximumtemperature(_i(ire), _i(icp), ctypes.byref(t1), ctypes.byref(t2))
    assert (t1.value, t2.value) == (0.0, 0.0)
    cg.finalize(ire)


def _calc(lib, ire, icp):
    ierr = ctypes.c_int(12345)
    lib.cntc_calculate(_i(ire), _i(icp), ctypes.byref(ierr))
    return ierr.value


def test_unsupported_options_refused_before_any_device_work(lib):
    """Options outside the engine return CNTC_err_other from cntc_calculate (never a silent
    fallback); the refusal comes from the set-up, so it needs no device: bilinear loading
    (C=3), temperatures (H=3), viscoelastic material (M=1), prescribed total force (F=1)."""
    base = C.config0(gausei=5, eps=1e-8, mx=21, my=21)
    ire = 908
    cg.setup_case(ire, 1, base)
    cg.setflags(ire, 1, [cg.CNTC_ic_inflcf], [3])
    assert _calc(lib, ire, 1) == cg.CNTC_err_other
    cg.setup_case(ire, 2, base)
    lib.cntc_settemperaturedata(_i(ire), _i(2), _i(3), _i(9), np.zeros(9).ctypes.data_as(cg._DP))
    assert _calc(lib, ire, 2) == cg.CNTC_err_other
    cg.setup_case(ire, 3, base)
    cg.setmaterialparameters(ire, 3, 1, [0.28, 0.28, 82000.0, 82000.0, 0.0, 0.0, 0.0, 0.0])
    assert _calc(lib, ire, 3) == cg.CNTC_err_other
    cg.setup_case(ire, 4, base)
    cg.setflags(ire, 4, [cg.CNTC_ic_force], [1])
    assert _calc(lib, ire, 4) == cg.CNTC_err_other
    cg.finalize(ire)


def test_single_column_refused_for_tangential_problems(lib, capfd):
    """A grid of one column in rolling direction (mx = 1) is refused by the set-up for a
    tangential problem (the reference selects ConvexGS there) but passes it for the normal
    problem alone, which then reaches the engine (no device here)."""
    ire = 909
    roll = C.subsurf_case(2)
    roll.pop("force3"), roll.pop("fxrel")
    roll["cksi"] = 0.0
    cg.setglobalflags([cg.CNTC_if_idebug], [1])
    try:
        cg.setup_case(ire, 1, roll)
        capfd.readouterr()
        assert _calc(lib, ire, 1) == cg.CNTC_err_other
        assert "mx < 2" in capfd.readouterr().err
        cg.setup_case(ire, 2, C.subsurf_case(1))
        _calc(lib, ire, 2)
        assert "mx < 2" not in capfd.readouterr().err
    finally:
        cg.setglobalflags([cg.CNTC_if_idebug], [0])
        cg.finalize(ire)


def test_subsurface_block_with_empty_list_reads_no_parameters(lib):
    """subs_addBlock with a list of zero values (npx = 0 for explicit points) reads nothing
    from that list: a null array does not crash the call.  An invalid block type (4) and a
    wrong parameter count (type 2 needs three per direction) are refused without reading
    their (null) arrays."""
    ire, icp = 910, 1
    cg.setnormalforce(ire, icp, 1e4)
    y = np.array([0.0, 1.0])
    z = np.array([0.5])
    null = ctypes.POINTER(ctypes.c_double)()
    lib.subs_addblock(_i(ire), _i(icp), _i(1), _i(9), _i(0), _i(2), _i(1), null, y.ctypes.data_as(cg._DP),
                      z.ctypes.data_as(cg._DP))
    lib.subs_addblock(_i(ire), _i(icp), _i(2), _i(4), _i(0), _i(0), _i(1), null, null, z.ctypes.data_as(cg._DP))
    lib.subs_addblock(_i(ire), _i(icp), _i(2), _i(2), _i(2), _i(3), _i(1), null, null, z.ctypes.data_as(cg._DP))
    # blocks beyond the list are unknown: no points, the output is left as it was
    nx, ny, nz = ctypes.c_int(7), ctypes.c_int(7), ctypes.c_int(7)
    lib.subs_getblocksize(_i(ire), _i(icp), _i(2), ctypes.byref(nx), ctypes.byref(ny), ctypes.byref(nz))
    assert (nx.value, ny.value, nz.value) == (0, 0, 0)
    cg.finalize(ire)
