"""contact_gb300: GB300-native rolling-contact solve path with CONTACT's cntc_* C-ABI.

The shared library contact_gb300/_build/libcontact_addon.so exports the module-3
library interface of CONTACT (see include/contact_addon.h).  This module is a thin
ctypes front end with the function names of the reference's python_intfc package
(initialize, setflags, calculate, getcontactforces, ...), plus helpers used by the
tests and the benchmark.  Every solve runs on the GPU; there is no CPU fallback: if
the library is missing or no CUDA device is present, calls raise.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libcontact_addon.so")

# codes of src/caddon_flags.inc
CNTC_if_units, CNTC_un_cntc, CNTC_un_spck, CNTC_un_si = 1933, 1934, 1935, 1936
CNTC_ic_config, CNTC_ic_pvtime, CNTC_ic_bound, CNTC_ic_tang, CNTC_ic_norm = 1967, 1970, 1971, 1972, 1973
CNTC_ic_force, CNTC_ic_frclaw, CNTC_ic_inflcf, CNTC_ic_mater = 1974, 1976, 1978, 1979
CNTC_ic_exrhs, CNTC_ic_iestim, CNTC_ic_output, CNTC_ic_flow, CNTC_ic_matfil = 1980, 1983, 1984, 1985, 1987
CNTC_ic_sens = 1988
CNTC_if_idebug, CNTC_if_ncase = 2000, 2005
CNTC_if_mixedprec = 2010
CNTC_if_groupctas = 2011
CNTC_fld_h, CNTC_fld_mu, CNTC_fld_px, CNTC_fld_py, CNTC_fld_pn = 1, 2, 3, 4, 5
CNTC_fld_ux, CNTC_fld_uy, CNTC_fld_un, CNTC_fld_sx, CNTC_fld_sy = 7, 8, 9, 15, 16
CNTC_err_norm, CNTC_err_tang, CNTC_err_icp, CNTC_err_other = -27, -28, -31, -99

_lib = None
_I = ctypes.c_int
_D = ctypes.c_double
_IP = ctypes.POINTER(ctypes.c_int)
_DP = ctypes.POINTER(ctypes.c_double)
_CP = ctypes.c_char_p

# prototypes of include/contact_addon.h
_PROTOS = {
    "cntc_initializefirst": [_IP, _IP, _IP, _CP, _CP, _CP, _IP, _IP, _IP],
    "cntc_initializefirst_new": [_IP, _IP, _IP, _CP, _CP, _CP, _IP, _IP, _IP],
    "cntc_initialize": [_IP, _IP, _IP, _IP, _CP, _IP],
    "cntc_setglobalflags": [_IP, _IP, _IP],
    "cntc_setflags": [_IP, _IP, _IP, _IP, _IP],
    "cntc_setsolverflags": [_IP, _IP, _IP, _IP, _IP, _IP, _DP],
    "cntc_setmaterialparameters": [_IP, _IP, _IP, _IP, _DP],
    "cntc_settemperaturedata": [_IP, _IP, _IP, _IP, _DP],
    "cntc_settimestep": [_IP, _IP, _DP],
    "cntc_setreferencevelocity": [_IP, _IP, _DP],
    "cntc_setrollingstepsize": [_IP, _IP, _DP, _DP],
    "cntc_setfrictionmethod": [_IP, _IP, _IP, _IP, _DP],
    "cntc_sethertzcontact": [_IP, _IP, _IP, _IP, _DP],
    "cntc_setpotcontact": [_IP, _IP, _IP, _IP, _DP],
    "cntc_setpenetration": [_IP, _IP, _DP],
    "cntc_setnormalforce": [_IP, _IP, _DP],
    "cntc_setundeformeddistc": [_IP, _IP, _IP, _IP, _DP],
    "cntc_setcreepages": [_IP, _IP, _DP, _DP, _DP],
    "cntc_setextrarigidslip": [_IP, _IP, _IP, _DP, _DP],
    "cntc_settangentialforces": [_IP, _IP, _DP, _DP],
    "cntc_calculate": [_IP, _IP, _IP],
    "cntc_calculate_batch": [_IP, _IP, _IP, _IP],
    "cntc_calculate_noalloc": [_IP, _IP, _IP],
    "cntc_calculate_async": [_IP, _IP, _IP],
    "cntc_wait": [_IP, _IP, _IP],
    "cntc_gb300_wait_latency": [_IP, _IP, _IP, _DP],
    "cntc_gb300_setadmissionbudget": [_DP],
    "cntc_getflags": [_IP, _IP, _IP, _IP, _IP],
    "cntc_getreferencevelocity": [_IP, _IP, _DP],
    "cntc_gethertzcontact": [_IP, _IP, _IP, _DP],
    "cntc_getnumelements": [_IP, _IP, _IP, _IP],
    "cntc_getgriddiscretization": [_IP, _IP, _DP, _DP],
    "cntc_getpotcontact": [_IP, _IP, _IP, _DP],
    "cntc_getpenetration": [_IP, _IP, _DP],
    "cntc_getcreepages": [_IP, _IP, _DP, _DP, _DP],
    "cntc_getcontactforces": [_IP, _IP, _DP, _DP, _DP, _DP],
    "cntc_getcontactpatchareas": [_IP, _IP, _DP, _DP, _DP],
    "cntc_getelementdivision": [_IP, _IP, _IP, _IP],
    "cntc_getmaximumpressure": [_IP, _IP, _DP],
    "cntc_getmaximumtraction": [_IP, _IP, _DP],
    "cntc_getfielddata": [_IP, _IP, _IP, _IP, _DP],
    "cntc_gettractions": [_IP, _IP, _IP, _DP, _DP, _DP],
    "cntc_getmicroslip": [_IP, _IP, _IP, _DP, _DP],
    "cntc_getdisplacements": [_IP, _IP, _IP, _DP, _DP, _DP],
    "cntc_getsensitivities": [_IP, _IP, _IP, _IP, _DP],
    "cntc_getcalculationtime": [_IP, _IP, _DP, _DP],
    "cntc_resetcalculationtime": [_IP, _IP],
    "cntc_getiterationcounts": [_IP, _IP, _IP, _IP],
    "cntc_getparameters": [_IP, _IP, _IP, _IP, _DP],
    "cntc_setmetadata": [_IP, _IP, _IP, _IP, _DP],
    "cntc_getmaximumtemperature": [_IP, _IP, _DP, _DP],
    "cntc_readinpfile": [_IP, _IP, _CP, _IP, _IP],
    "cntc_setverticalforce": [_IP, _DP],
    "cntc_setprofileinputfname": [_IP, _CP, _IP, _IP, _IP, _IP, _DP],
    "cntc_setprofileinputvalues": [_IP, _IP, _DP, _IP, _IP, _IP, _DP],
    "cntc_settrackdimensions": [_IP, _IP, _IP, _DP],
    "cntc_setwheelsetdimensions": [_IP, _IP, _IP, _DP],
    "cntc_setwheelsetposition": [_IP, _IP, _IP, _DP],
    "cntc_setwheelsetvelocity": [_IP, _IP, _IP, _DP],
    "cntc_setwheelsetflexibility": [_IP, _IP, _IP, _DP],
    "cntc_getprofilevalues": [_IP, _IP, _IP, _IP, _IP, _DP, _IP, _DP],
    "cntc_getprofilevalues_new": [_IP, _IP, _IP, _IP, _IP, _DP, _IP, _DP],
    "cntc_getwheelsetposition": [_IP, _IP, _DP],
    "cntc_getwheelsetvelocity": [_IP, _IP, _DP],
    "cntc_getnumcontactpatches": [_IP, _IP],
    "cntc_getcontactlocation": [_IP, _IP, _IP, _DP],
    "cntc_getglobalforces": [_IP, _IP, _IP, _DP],
    "subs_addblock": [_IP, _IP, _IP, _IP, _IP, _IP, _IP, _DP, _DP, _DP],
    "subs_calculate": [_IP, _IP, _IP],
    "subs_getblocksize": [_IP, _IP, _IP, _IP, _IP, _IP],
    "subs_getresults": [_IP, _IP, _IP, _IP, _IP, _IP, _DP],
    "cntc_finalize": [_IP],
    "cntc_finalizelast": [],
    "cntc_gb300_kernel_launches": [],
    "cntc_gb300_getsolverstats": [_IP, _IP, _IP, _DP],
    "cntc_gb300_resident_setup": [_IP, _IP, _IP, _IP],
    "cntc_gb300_resident_solve": [_IP, _DP, _IP],
    "cntc_gb300_resident_collect": [_IP, _IP],
    "cntc_gb300_resident_release": [],
    "cntc_gb300_resident_depth": [_IP],
    "cntc_gb300_resident_graphs": [],
    "cntc_gb300_lastcopybytes": [ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)],
    "cntc_gb300_fmapeaks": [_DP],
    "cntc_gb300_latencyshapes": [_IP, _IP, _IP],
}


def load(path=None):
    """Load the shared library (building it first when it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        from . import build as _b
        _b.build()
    lib = ctypes.CDLL(p)
    for name, args in _PROTOS.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = {"cntc_gb300_kernel_launches": ctypes.c_longlong, "cntc_gb300_fmapeaks": ctypes.c_int,
                     "cntc_gb300_resident_graphs": ctypes.c_int, "cntc_gb300_latencyshapes": ctypes.c_int}.get(name)
    _lib = lib
    return lib


def exported_symbols():
    return list(_PROTOS)


def _i(v):
    return ctypes.byref(ctypes.c_int(int(v)))


def _d(v):
    return ctypes.byref(ctypes.c_double(float(v)))


def _iarr(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(_IP)


def _darr(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_DP)


def _require_gpu():
    import torch  # plumbing only: device presence
    if not torch.cuda.is_available():
        raise RuntimeError("contact_gb300: no CUDA device available; this library has no CPU path")


# ------------------------------------------------------------------------------------------
# python_intfc-style wrappers (same names as the reference's Python interface)
# ------------------------------------------------------------------------------------------
def initialize(ire, imodul=3):
    lib = load()
    ver, ierr = ctypes.c_int(0), ctypes.c_int(0)
    lib.cntc_initialize(_i(ire), _i(imodul), ctypes.byref(ver), ctypes.byref(ierr), b" ", _i(1))
    return ver.value, ierr.value


def setglobalflags(flags, values):
    f, fp = _iarr(flags)
    v, vp = _iarr(values)
    load().cntc_setglobalflags(_i(len(f)), fp, vp)


def setflags(ire, icp, flags, values):
    f, fp = _iarr(flags)
    v, vp = _iarr(values)
    load().cntc_setflags(_i(ire), _i(icp), _i(len(f)), fp, vp)


def setsolverflags(ire, icp, gdigit, iparam, rparam):
    ia, ip = _iarr(iparam)
    ra, rp = _darr(rparam)
    load().cntc_setsolverflags(_i(ire), _i(icp), _i(gdigit), _i(len(ia)), ip, _i(len(ra)), rp)


def setmaterialparameters(ire, icp, mdigit, rparam):
    ra, rp = _darr(rparam)
    load().cntc_setmaterialparameters(_i(ire), _i(icp), _i(mdigit), _i(len(ra)), rp)


def setfrictionmethod(ire, icp, imeth, params):
    ra, rp = _darr(params)
    load().cntc_setfrictionmethod(_i(ire), _i(icp), _i(imeth), _i(len(ra)), rp)


def setreferencevelocity(ire, icp, veloc):
    load().cntc_setreferencevelocity(_i(ire), _i(icp), _d(veloc))


def setrollingstepsize(ire, icp, chi, dq):
    load().cntc_setrollingstepsize(_i(ire), _i(icp), _d(chi), _d(dq))


def sethertzcontact(ire, icp, ipotcn, params):
    ra, rp = _darr(params)
    load().cntc_sethertzcontact(_i(ire), _i(icp), _i(ipotcn), _i(len(ra)), rp)


def setpotcontact(ire, icp, ipotcn, params):
    ra, rp = _darr(params)
    load().cntc_setpotcontact(_i(ire), _i(icp), _i(ipotcn), _i(len(ra)), rp)


def setpenetration(ire, icp, pen):
    load().cntc_setpenetration(_i(ire), _i(icp), _d(pen))


def setnormalforce(ire, icp, fn):
    load().cntc_setnormalforce(_i(ire), _i(icp), _d(fn))


def setundeformeddistc(ire, icp, ibase, prmudf):
    ra, rp = _darr(prmudf)
    load().cntc_setundeformeddistc(_i(ire), _i(icp), _i(ibase), _i(len(ra)), rp)


def setcreepages(ire, icp, vx, vy, phi):
    load().cntc_setcreepages(_i(ire), _i(icp), _d(vx), _d(vy), _d(phi))


def settangentialforces(ire, icp, fx, fy):
    """Total tangential forces relative to fstat Fn (used with the F digit 1 or 2)."""
    load().cntc_settangentialforces(_i(ire), _i(icp), _d(fx), _d(fy))


def calculate(ire, icp):
    _require_gpu()
    ierr = ctypes.c_int(0)
    load().cntc_calculate(_i(ire), _i(icp), ctypes.byref(ierr))
    return ierr.value


def calculate_noalloc(ire, icp):
    """cntc_calculate without device allocations (fixed 16 MiB device scratch)."""
    _require_gpu()
    ierr = ctypes.c_int(0)
    load().cntc_calculate_noalloc(_i(ire), _i(icp), ctypes.byref(ierr))
    return ierr.value


def calculate_async(ire, icp):
    """Queue a solve (serving); returns 0 when queued."""
    _require_gpu()
    ierr = ctypes.c_int(0)
    load().cntc_calculate_async(_i(ire), _i(icp), ctypes.byref(ierr))
    return ierr.value


def wait(ire, icp, with_latency=False):
    """Wait for a queued solve; returns ierror (and the queue-to-completion latency in s)."""
    ierr = ctypes.c_int(0)
    if with_latency:
        lat = ctypes.c_double(0.0)
        load().cntc_gb300_wait_latency(_i(ire), _i(icp), ctypes.byref(ierr), ctypes.byref(lat))
        return ierr.value, lat.value
    load().cntc_wait(_i(ire), _i(icp), ctypes.byref(ierr))
    return ierr.value


def setadmissionbudget(gbytes):
    load().cntc_gb300_setadmissionbudget(ctypes.byref(ctypes.c_double(float(gbytes))))


# ------------------------------------------------------------------------------------------
# subsurface stresses (subs_addBlock, subs_calculate, subs_getBlocksize, subs_getResults)
# ------------------------------------------------------------------------------------------
SUBS_COLUMNS = ("x", "y", "z", "ux", "uy", "uz", "sighyd", "sigvm", "sigtr", "sigma1", "sigma2", "sigma3",
                "sigxx", "sigyx", "sigzx", "sigxy", "sigyy", "sigzy", "sigxz", "sigyz", "sigzz")


def subs_addblock(ire, icp, iblk, isubs, xparam=(), yparam=(), zparam=()):
    """Block iblk of subsurface points (types 1-3, 5-7: element centres; 9: x, y lists)."""
    xa = np.ascontiguousarray(xparam, dtype=np.float64).reshape(-1)
    ya = np.ascontiguousarray(yparam, dtype=np.float64).reshape(-1)
    za = np.ascontiguousarray(zparam, dtype=np.float64).reshape(-1)
    dummy = np.zeros(1)
    ptr = lambda a: (a if a.size else dummy).ctypes.data_as(_DP)
    load().subs_addblock(_i(ire), _i(icp), _i(iblk), _i(isubs), _i(xa.size), _i(ya.size), _i(za.size),
                         ptr(xa), ptr(ya), ptr(za))


def subs_calculate(ire, icp):
    """Subsurface field of the last solution at all blocks of (ire, icp); returns ierror."""
    e = ctypes.c_int(0)
    load().subs_calculate(_i(ire), _i(icp), ctypes.byref(e))
    return e.value


def subs_getblocksize(ire, icp, iblk):
    nx, ny, nz = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
    load().subs_getblocksize(_i(ire), _i(icp), _i(iblk), ctypes.byref(nx), ctypes.byref(ny), ctypes.byref(nz))
    return nx.value, ny.value, nz.value


def subs_getresults(ire, icp, iblk, cols=SUBS_COLUMNS):
    """Results of block iblk as {column name: array of nx*ny*nz values (x fastest)}."""
    nx, ny, nz = subs_getblocksize(ire, icp, iblk)
    npt = nx * ny * nz
    icol = np.array([SUBS_COLUMNS.index(c) + 1 for c in cols], dtype=np.int32)
    vals = np.zeros((len(cols), max(npt, 1)))
    load().subs_getresults(_i(ire), _i(icp), _i(iblk), _i(max(npt, 1)), _i(len(cols)), icol.ctypes.data_as(_IP),
                           vals.ctypes.data_as(_DP))
    return {c: vals[k, :npt].copy() for k, c in enumerate(cols)}


def calculate_batch(ire_list, icp_list):
    _require_gpu()
    a, ap = _iarr(ire_list)
    b, bp = _iarr(icp_list)
    err = np.zeros(len(a), dtype=np.int32)
    load().cntc_calculate_batch(_i(len(a)), ap, bp, err.ctypes.data_as(_IP))
    return err


def getcontactforces(ire, icp):
    v = [ctypes.c_double() for _ in range(4)]
    load().cntc_getcontactforces(_i(ire), _i(icp), *[ctypes.byref(x) for x in v])
    return tuple(x.value for x in v)


def gethertzcontact(ire, icp, lenarr=10):
    out = np.zeros(lenarr)
    load().cntc_gethertzcontact(_i(ire), _i(icp), _i(lenarr), out.ctypes.data_as(_DP))
    return out


def getnumelements(ire, icp):
    mx, my = ctypes.c_int(), ctypes.c_int()
    load().cntc_getnumelements(_i(ire), _i(icp), ctypes.byref(mx), ctypes.byref(my))
    return mx.value, my.value


def getgriddiscretization(ire, icp):
    dx, dy = ctypes.c_double(), ctypes.c_double()
    load().cntc_getgriddiscretization(_i(ire), _i(icp), ctypes.byref(dx), ctypes.byref(dy))
    return dx.value, dy.value


def getpenetration(ire, icp):
    v = ctypes.c_double()
    load().cntc_getpenetration(_i(ire), _i(icp), ctypes.byref(v))
    return v.value


def getcreepages(ire, icp):
    """(cksi, ceta, cphi) of the problem; after a solve with prescribed total forces the
    creepages that the Newton-Raphson found."""
    a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    load().cntc_getcreepages(_i(ire), _i(icp), ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
    return a.value, b.value, c.value


def getsensitivities(ire, icp, lenout=4, lenin=4):
    """sens[iout, iin]: outputs fn, fx, fy, mz; inputs pen, cksi, ceta, cphi (caller's units)."""
    out = np.zeros(lenout * lenin)
    load().cntc_getsensitivities(_i(ire), _i(icp), _i(lenout), _i(lenin), out.ctypes.data_as(_DP))
    return out.reshape(lenin, lenout).T.copy()


def getcontactpatchareas(ire, icp):
    v = [ctypes.c_double() for _ in range(3)]
    load().cntc_getcontactpatchareas(_i(ire), _i(icp), *[ctypes.byref(x) for x in v])
    return tuple(x.value for x in v)


def getmaximumpressure(ire, icp):
    v = ctypes.c_double()
    load().cntc_getmaximumpressure(_i(ire), _i(icp), ctypes.byref(v))
    return v.value


def getelementdivision(ire, icp):
    mx, my = getnumelements(ire, icp)
    out = np.zeros(mx * my, dtype=np.int32)
    load().cntc_getelementdivision(_i(ire), _i(icp), _i(mx * my), out.ctypes.data_as(_IP))
    return out


def getfielddata(ire, icp, ifld):
    mx, my = getnumelements(ire, icp)
    out = np.zeros(mx * my)
    load().cntc_getfielddata(_i(ire), _i(icp), _i(ifld), _i(mx * my), out.ctypes.data_as(_DP))
    return out


def gettractions(ire, icp):
    mx, my = getnumelements(ire, icp)
    pn, px, py = np.zeros(mx * my), np.zeros(mx * my), np.zeros(mx * my)
    load().cntc_gettractions(_i(ire), _i(icp), _i(mx * my), pn.ctypes.data_as(_DP), px.ctypes.data_as(_DP),
                             py.ctypes.data_as(_DP))
    return pn, px, py


def getiterationcounts(ire, icp):
    out = np.zeros(6, dtype=np.int32)
    load().cntc_getiterationcounts(_i(ire), _i(icp), _i(6), out.ctypes.data_as(_IP))
    return dict(zip(("itnorm", "ittang", "itcg", "itgs", "solver", "ierror"), out.tolist()))


def finalize(ire):
    load().cntc_finalize(_i(ire))


def finalizelast():
    load().cntc_finalizelast()


def kernel_launches():
    return int(load().cntc_gb300_kernel_launches())


STAT_NAMES = ("nconv32", "nconv64", "nls", "status", "t_total", "t_conv", "t_ls", "t_diag", "t_gs", "t_norm",
              "t_tang", "t_scan", "t_conv32", "t_gsser", "conv_bytes", "t_start_ns", "t_end_ns", "ctas")


def lastcopybytes():
    """(host->device, device->host) bytes of this thread's last calculate call."""
    a, b = ctypes.c_longlong(), ctypes.c_longlong()
    load().cntc_gb300_lastcopybytes(ctypes.byref(a), ctypes.byref(b))
    return a.value, b.value


def latency_shapes():
    """Launch shapes tuned so far for single-patch calls: {size class c: True (patch group) or
    False (one CTA)} for grids of 2**c .. 2**(c+1) - 1 elements."""
    cls = (ctypes.c_int * 32)()
    grp = (ctypes.c_int * 32)()
    cap = ctypes.c_int(32)
    k = load().cntc_gb300_latencyshapes(ctypes.cast(cls, _IP), ctypes.cast(grp, _IP), ctypes.byref(cap))
    return {int(cls[i]): bool(grp[i]) for i in range(k)}


def fma_peaks():
    """Measured FMA peaks of the current device: {"fp64_tflops": .., "fp32_tflops": ..}."""
    _require_gpu()
    out = (ctypes.c_double * 2)()
    rc = load().cntc_gb300_fmapeaks(out)
    if rc != 0:
        raise RuntimeError("FMA peak measurement failed")
    return {"fp64_tflops": out[0], "fp32_tflops": out[1]}


def opt_fft_size(n):
    """FFT length used for a grid side n (m_aijpj.f90:1022-1119): start from the next power of two
    and trade factors (4 -> 3, 32 -> 27, 6 -> 5, 16 -> 15, 27 -> 25, 8 -> 7, 15 -> 14, 10 -> 9)
    while the product stays >= n."""
    trades = (((-2, 1, 0, 0), 4, 3), ((-5, 3, 0, 0), 32, 27), ((-1, -1, 1, 0), 6, 5), ((-4, 1, 1, 0), 16, 15),
              ((0, -3, 2, 0), 27, 25), ((-3, 0, 0, 1), 8, 7), ((1, -1, -1, 1), 15, 14), ((-1, 2, -1, 0), 10, 9))
    k2 = 0
    while (1 << k2) < n:
        k2 += 1
    k = [k2, 0, 0, 0]
    prod = 1 << k2
    changed = True
    while changed:
        changed = False
        for dk, den, num in trades:
            while all(k[f] + dk[f] >= 0 for f in range(4)) and num * prod >= den * n:
                k = [k[f] + dk[f] for f in range(4)]
                prod = num * prod // den
                changed = True
    return prod


class ResidentBatch:
    """Problems staged in device memory once and solved repeatedly (inputs resident in HBM).
    depth > 1 stages them in that many buffer sets so that consecutive passes overlap."""

    def __init__(self, ire_list, icp_list, depth=1):
        _require_gpu()
        load().cntc_gb300_resident_depth(_i(depth))
        self.n = len(ire_list)
        a, ap = _iarr(ire_list)
        b, bp = _iarr(icp_list)
        self._ids = (a, b)
        self.setup_errors = np.zeros(self.n, dtype=np.int32)
        load().cntc_gb300_resident_setup(_i(self.n), ap, bp, self.setup_errors.ctypes.data_as(_IP))

    def solve(self, nrep=1):
        """Run the engine nrep times; returns an (nrep, 4) array: device ms of the pass, ms in
        patch solves, ms in influence/spectrum kernels, launches."""
        t = np.zeros((nrep, 4))
        err = ctypes.c_int(0)
        load().cntc_gb300_resident_solve(_i(nrep), t.ctypes.data_as(_DP), ctypes.byref(err))
        if err.value != 0:
            raise RuntimeError("resident solve failed (%d)" % err.value)
        return t

    def graphs(self):
        """Buffer sets whose pass replays a captured CUDA graph."""
        return int(load().cntc_gb300_resident_graphs())

    def collect(self):
        err = np.zeros(self.n, dtype=np.int32)
        load().cntc_gb300_resident_collect(_i(self.n), err.ctypes.data_as(_IP))
        return err

    def release(self):
        load().cntc_gb300_resident_release()


def getsolverstats(ire, icp):
    """Engine statistics of the last solve: convolution counts, status bits and SM cycles per phase."""
    out = np.zeros(len(STAT_NAMES))
    load().cntc_gb300_getsolverstats(_i(ire), _i(icp), _i(len(out)), out.ctypes.data_as(_DP))
    return dict(zip(STAT_NAMES, out.tolist()))


# ------------------------------------------------------------------------------------------
# helpers: describe a case as a dict and drive the C-ABI with it
# ------------------------------------------------------------------------------------------
def setup_case(ire, icp, case):
    """Apply a case description (the same dict the tests hand to the oracle) to (ire, icp).

    Keys: tang, norm, bound, gausei, maxgs, maxin, maxnr, maxout, eps, gd (8 floats + kdowfb
    for G=5), poiss, gg (poiss2, gg2 for a different body 2), fstat, veloc, cksi, ceta, cphi,
    force3 with fxrel, fyrel (total forces prescribed), fn | pen, ipotcn, potprm,
    h (element-wise undeformed distance, optional), prmudf (6 coefficients of a quadratic
    undeformed distance, ibase 1, optional), mixed (0-4), dq and chi (optional), group (CTAs
    per patch: 0 automatic, 1 one CTA, n >= 2 a cooperative group of at most n)."""
    flags = [CNTC_ic_tang, CNTC_ic_bound, CNTC_ic_iestim, CNTC_if_mixedprec, CNTC_if_groupctas, CNTC_ic_pvtime,
             CNTC_ic_force, CNTC_ic_sens]
    values = [case.get("tang", 3), case.get("bound", 0), case.get("iestim", 0), case.get("mixed", 0),
              case.get("group", 0), case.get("pvtime", 2), case.get("force3", 0), case.get("sens", 1)]
    setflags(ire, icp, flags, values)
    setfrictionmethod(ire, icp, 0, [case.get("fstat", 0.3), case.get("fstat", 0.3)])
    nu = case.get("poiss", 0.28)
    g = case.get("gg", 82000.0)
    setmaterialparameters(ire, icp, 0, [nu, case.get("poiss2", nu), g, case.get("gg2", g)])
    if case.get("force3", 0) >= 1:
        settangentialforces(ire, icp, case.get("fxrel", 0.0), case.get("fyrel", 0.0))
    setreferencevelocity(ire, icp, case.get("veloc", 10000.0))
    gdig = case.get("gausei", 0)
    ip = [case.get("maxgs", 999), case.get("maxin", 100), case.get("maxnr", 30), case.get("maxout", 1)]
    if gdig == 5:
        gd = case.get("gd", dict(fdecay=0.9, betath=0.1, kdowfb=1, d_ifc=1.0, d_lin=1.0, d_cns=1.0, d_slp=1.0,
                                 pow_s=0.9))
        setsolverflags(ire, icp, 5, ip + [gd["kdowfb"]],
                       [case.get("eps", 1e-6), gd["fdecay"], gd["betath"], gd["d_ifc"], gd["d_lin"], gd["d_cns"],
                        gd["d_slp"], gd["pow_s"]])
    elif gdig in (2, 3):
        # ConvexGS / SteadyGS with their relaxation: [maxgs, maxin, maxnr, maxout, inislp],
        # [eps, omegah, omegas, omgslp]
        setsolverflags(ire, icp, gdig, ip + [case.get("inislp", 0)],
                       [case.get("eps", 1e-6), case.get("omegah", 0.9), case.get("omegas", 1.0),
                        case.get("omgslp", 0.5)])
    elif gdig == 4:
        setsolverflags(ire, icp, gdig, ip + [case.get("inislp", 0)], [case.get("eps", 1e-6), case.get("omgslp", 0.5)])
    else:
        setsolverflags(ire, icp, gdig, ip, [case.get("eps", 1e-6)])
    if "mxsens" in case or "epsens" in case:
        setsolverflags(ire, icp, 6, [case.get("mxsens", 30)], [case.get("epsens", 1e-4)])
    if "dq" in case:
        setrollingstepsize(ire, icp, case.get("chi", 0.0), case["dq"])
    ipot = case.get("ipotcn", -3)
    if ipot < 0:
        sethertzcontact(ire, icp, ipot, case["potprm"][:5])
    else:
        setpotcontact(ire, icp, ipot, case["potprm"][:6])
    if "h" in case:
        setundeformeddistc(ire, icp, 9, np.asarray(case["h"], dtype=np.float64).ravel())
    elif "prmudf" in case:
        setundeformeddistc(ire, icp, 1, np.asarray(case["prmudf"], dtype=np.float64))
    if case.get("norm", 1) == 1:
        setnormalforce(ire, icp, case["fn"])
    else:
        setpenetration(ire, icp, case["pen"])
    setcreepages(ire, icp, case.get("cksi", 0.0), case.get("ceta", 0.0), case.get("cphi", 0.0))


def results(ire, icp):
    """Forces, scalars and fields of the last solve of (ire, icp) as a dict."""
    fn, fx, fy, mz = getcontactforces(ire, icp)
    pn, px, py = gettractions(ire, icp)
    carea, harea, sarea = getcontactpatchareas(ire, icp)
    dx, dy = getgriddiscretization(ire, icp)
    mx, my = getnumelements(ire, icp)
    out = dict(fn=fn, fx=fx, fy=fy, mz=mz, pn=pn, px=px, py=py, pen=getpenetration(ire, icp), mx=mx, my=my,
               pmax=getmaximumpressure(ire, icp), igs=getelementdivision(ire, icp),
               ncon=int(round(carea / (dx * dy))), nadh=int(round(harea / (dx * dy))),
               nslip=int(round(sarea / (dx * dy))), dx=dx, dy=dy)
    out.update(getiterationcounts(ire, icp))
    out["un"] = getfielddata(ire, icp, CNTC_fld_un)
    out["ux"] = getfielddata(ire, icp, CNTC_fld_ux)
    out["uy"] = getfielddata(ire, icp, CNTC_fld_uy)
    out["sx"] = getfielddata(ire, icp, CNTC_fld_sx)
    out["sy"] = getfielddata(ire, icp, CNTC_fld_sy)
    out["hz"] = gethertzcontact(ire, icp)
    return out
