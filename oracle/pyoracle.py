"""CPU ORACLE -- test infrastructure only.

ctypes front end of oracle/_build/libcontact_oracle.so, the serial C++ restatement
of CONTACT's module-3 solve path.  Used by tests/ (the reference results), by
__graft_entry__.smoke() and by bench.py's CPU-baseline legs; never by the
product library.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libcontact_oracle.so")
_LIB_FAST_PATH = os.path.join(_HERE, "_build", "libcontact_oracle_fast.so")
_lib = None


class Problem(ctypes.Structure):
    _fields_ = [
        ("pvtime", ctypes.c_int), ("bound", ctypes.c_int), ("tang", ctypes.c_int),
        ("norm", ctypes.c_int), ("force3", ctypes.c_int), ("iestim", ctypes.c_int),
        ("gausei", ctypes.c_int),
        ("maxgs", ctypes.c_int), ("maxin", ctypes.c_int), ("maxnr", ctypes.c_int),
        ("maxout", ctypes.c_int),
        ("eps", ctypes.c_double),
        ("omegah", ctypes.c_double), ("omegas", ctypes.c_double),
        ("inislp", ctypes.c_int), ("omgslp", ctypes.c_double),
        ("kdowfb", ctypes.c_int),
        ("fdecay", ctypes.c_double), ("betath", ctypes.c_double), ("d_ifc", ctypes.c_double),
        ("d_lin", ctypes.c_double), ("d_cns", ctypes.c_double), ("d_slp", ctypes.c_double),
        ("pow_s", ctypes.c_double),
        ("poiss1", ctypes.c_double), ("poiss2", ctypes.c_double),
        ("gg1", ctypes.c_double), ("gg2", ctypes.c_double),
        ("fstat", ctypes.c_double), ("fkin", ctypes.c_double),
        ("veloc", ctypes.c_double), ("chi", ctypes.c_double), ("dq", ctypes.c_double),
        ("cksi", ctypes.c_double), ("ceta", ctypes.c_double), ("cphi", ctypes.c_double),
        ("fn", ctypes.c_double), ("pen", ctypes.c_double),
        ("fxrel", ctypes.c_double), ("fyrel", ctypes.c_double),
        ("ipotcn", ctypes.c_int),
        ("potprm", ctypes.c_double * 6),
        ("ibase", ctypes.c_int),
        ("nprmudf", ctypes.c_int),
        ("prmudf", ctypes.POINTER(ctypes.c_double)),
        ("igs_init", ctypes.POINTER(ctypes.c_int)),
        ("pn_init", ctypes.POINTER(ctypes.c_double)),
        ("px_init", ctypes.POINTER(ctypes.c_double)),
        ("py_init", ctypes.POINTER(ctypes.c_double)),
        ("sens", ctypes.c_int), ("mxsens", ctypes.c_int), ("epsens", ctypes.c_double),
        ("standalone", ctypes.c_int),
        ("sens_init", ctypes.POINTER(ctypes.c_double)),
        ("igv_init", ctypes.POINTER(ctypes.c_int)),
        ("pvn_init", ctypes.POINTER(ctypes.c_double)), ("pvx_init", ctypes.POINTER(ctypes.c_double)),
        ("pvy_init", ctypes.POINTER(ctypes.c_double)),
        ("frclaw", ctypes.c_int), ("flaw", ctypes.c_double * 5), ("memdst", ctypes.c_double),
        ("mem_s0", ctypes.c_double),
        ("mus_init", ctypes.POINTER(ctypes.c_double)), ("svx_init", ctypes.POINTER(ctypes.c_double)),
        ("svy_init", ctypes.POINTER(ctypes.c_double)),
        ("mater", ctypes.c_int), ("gg3", ctypes.c_double), ("laythk", ctypes.c_double),
        ("tau_c0", ctypes.c_double), ("k_tau", ctypes.c_double),
    ]


class Result(ctypes.Structure):
    _fields_ = [
        ("ierror", ctypes.c_int), ("itnorm", ctypes.c_int), ("ittang", ctypes.c_int),
        ("itcg", ctypes.c_int), ("itgs", ctypes.c_int), ("solver", ctypes.c_int),
        ("mx", ctypes.c_int), ("my", ctypes.c_int),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("xc1", ctypes.c_double),
        ("yc1", ctypes.c_double),
        ("fn", ctypes.c_double), ("fx", ctypes.c_double), ("fy", ctypes.c_double),
        ("mz", ctypes.c_double), ("pen", ctypes.c_double), ("elen", ctypes.c_double),
        ("pmax", ctypes.c_double),
        ("cksi", ctypes.c_double), ("ceta", ctypes.c_double), ("cphi", ctypes.c_double),
        ("a1", ctypes.c_double), ("b1", ctypes.c_double), ("aa", ctypes.c_double),
        ("bb", ctypes.c_double), ("rho", ctypes.c_double), ("cp", ctypes.c_double),
        ("aob", ctypes.c_double),
        ("ncon", ctypes.c_int), ("nadh", ctypes.c_int), ("nslip", ctypes.c_int),
        ("pn", ctypes.POINTER(ctypes.c_double)), ("px", ctypes.POINTER(ctypes.c_double)),
        ("py", ctypes.POINTER(ctypes.c_double)),
        ("un", ctypes.POINTER(ctypes.c_double)), ("ux", ctypes.POINTER(ctypes.c_double)),
        ("uy", ctypes.POINTER(ctypes.c_double)),
        ("sx", ctypes.POINTER(ctypes.c_double)), ("sy", ctypes.POINTER(ctypes.c_double)),
        ("h", ctypes.POINTER(ctypes.c_double)),
        ("igs", ctypes.POINTER(ctypes.c_int)),
        ("mus", ctypes.POINTER(ctypes.c_double)),
        ("sens", ctypes.c_double * 16),
        ("nr_cap", ctypes.c_int), ("nnr", ctypes.c_int), ("nr_hist", ctypes.POINTER(ctypes.c_double)),
        ("nout", ctypes.c_int), ("outer", ctypes.c_double * 128),
        ("nslp", ctypes.c_int), ("slp", ctypes.c_double * 256),
    ]


NR_CAP = 256


def build(quiet=True):
    """Compile the oracle with its Makefile (g++ only, no GPU)."""
    out = subprocess.run(["make", "-C", _HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


_libs = {}


def lib(fast=False):
    """The oracle library; fast=True the build with the Stockham FFT and real-input convolutions (the timed CPU
    baseline), otherwise the parity build."""
    global _lib
    key = bool(fast)
    if key not in _libs:
        path = _LIB_FAST_PATH if key else _LIB_PATH
        if not os.path.exists(path):
            build()
        _l = ctypes.CDLL(path)
        _setup(_l)
        _libs[key] = _l
        if not key:
            _lib = _l
    return _libs[key]


def _setup(_lib):
    """ctypes prototypes of the oracle's entry points."""
    if True:
        _lib.orc_calculate.argtypes = [ctypes.POINTER(Problem), ctypes.POINTER(Result)]
        _lib.orc_calculate.restype = ctypes.c_int
        _lib.orc_default_problem.argtypes = [ctypes.POINTER(Problem)]
        _lib.orc_opt_fft_size.argtypes = [ctypes.c_int]
        _lib.orc_opt_fft_size.restype = ctypes.c_int
        _lib.orc_eli.argtypes = [ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                                 ctypes.POINTER(ctypes.c_double)]
        _lib.orc_eli.restype = ctypes.c_double
        _dp = ctypes.POINTER(ctypes.c_double)
        _lib.orc_influence_coefficients.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                    ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                                    ctypes.c_double, ctypes.c_double, _dp]
        _lib.orc_convolve.argtypes = [ctypes.c_int, ctypes.c_int, _dp, ctypes.c_double, _dp, _dp]
        _lib.orc_convolve_direct.argtypes = [ctypes.c_int, ctypes.c_int, _dp, ctypes.c_double, _dp, _dp]
        _subs = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                 _dp, _dp, _dp, _dp, _dp, ctypes.c_int, _dp, _dp]
        _lib.orc_subsurf_points.argtypes = _subs
        _lib.orc_subsurf_depths.argtypes = _subs
    return _lib


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def default_problem():
    pb = Problem()
    lib().orc_default_problem(ctypes.byref(pb))
    return pb


def solve(pb, h=None, warm=None, fields=True, fast=False, prev=None):
    """Solve one case; returns a dict of scalars and (optionally) fields.

    h: element-wise undeformed distance (ibase 9); warm: dict(igs, pn, px, py[, sens])
    used as initial estimate when pb.iestim > 0; prev: dict(igs, pn, px, py), the previous
    time instance of a transient sequence (pb.pvtime 0 or 1); fast: the baseline build
    (Stockham FFT, real-input convolutions)."""
    keep = []
    if prev is not None:
        igv = np.ascontiguousarray(prev["igs"], dtype=np.int32)
        pvs = [np.ascontiguousarray(prev[k], dtype=np.float64) for k in ("pn", "px", "py")]
        keep += [igv] + pvs
        pb.igv_init = igv.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        pb.pvn_init, pb.pvx_init, pb.pvy_init = (_dptr(a) for a in pvs)
        if "mus" in prev:
            extra = [np.ascontiguousarray(prev[k], dtype=np.float64) for k in ("mus", "svx", "svy")]
            keep += extra
            pb.mus_init, pb.svx_init, pb.svy_init = (_dptr(a) for a in extra)
    if warm is not None and "sens" in warm:
        sv = np.ascontiguousarray(np.asarray(warm["sens"], dtype=np.float64).T.ravel())
        keep.append(sv)
        pb.sens_init = _dptr(sv)
    if h is not None:
        hh = np.ascontiguousarray(h, dtype=np.float64).ravel()
        keep.append(hh)
        pb.ibase = 9
        pb.nprmudf = hh.size
        pb.prmudf = _dptr(hh)
    if warm is not None:
        igs0 = np.ascontiguousarray(warm["igs"], dtype=np.int32)
        pn0 = np.ascontiguousarray(warm["pn"], dtype=np.float64)
        px0 = np.ascontiguousarray(warm["px"], dtype=np.float64)
        py0 = np.ascontiguousarray(warm["py"], dtype=np.float64)
        keep += [igs0, pn0, px0, py0]
        pb.igs_init = igs0.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        pb.pn_init, pb.px_init, pb.py_init = _dptr(pn0), _dptr(px0), _dptr(py0)
    mx = max(1, int(round(pb.potprm[0])))
    my = max(1, int(round(pb.potprm[1])))
    n = mx * my
    res = Result()
    arrs = {}
    if fields:
        for k in ("pn", "px", "py", "un", "ux", "uy", "sx", "sy", "h", "mus"):
            arrs[k] = np.zeros(n, dtype=np.float64)
            setattr(res, k, _dptr(arrs[k]))
        arrs["igs"] = np.zeros(n, dtype=np.int32)
        res.igs = arrs["igs"].ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    hist = np.zeros(NR_CAP * 7, dtype=np.float64)
    res.nr_cap = NR_CAP
    res.nr_hist = _dptr(hist)
    lib(fast).orc_calculate(ctypes.byref(pb), ctypes.byref(res))
    out = {k: getattr(res, k) for k, _ in Result._fields_ if k not in
           ("pn", "px", "py", "un", "ux", "uy", "sx", "sy", "h", "igs", "mus", "sens", "nr_cap", "nr_hist", "outer",
            "slp")}
    out["slp"] = np.array(res.slp[:4 * min(res.nslp, 64)], dtype=np.float64).reshape(-1, 4)
    out["outer"] = np.array(res.outer[:2 * min(res.nout, 64)], dtype=np.float64).reshape(-1, 2)
    # sens[iout][iin]: iout Fn, Fx, Fy, Mz; iin pen, cksi, ceta, cphi
    out["sens"] = np.array(res.sens[:], dtype=np.float64).reshape(4, 4).T.copy()
    out["nr"] = hist[:7 * min(res.nnr, NR_CAP)].reshape(-1, 7).copy()
    out.update(arrs)
    return out


def opt_fft_size(n):
    return lib().orc_opt_fft_size(int(n))


def eli(k):
    a = ctypes.c_double()
    b = ctypes.c_double()
    r = lib().orc_eli(float(k), ctypes.byref(a), ctypes.byref(b))
    return r, a.value, b.value


def influence_coefficients(mx, my, dx, dy, nu, ak=0.0, xshft=0.0, yshft=0.0):
    out = np.zeros(9 * 4 * mx * my, dtype=np.float64)
    lib().orc_influence_coefficients(mx, my, dx, dy, nu, ak, xshft, yshft, _dptr(out))
    # block (ik,jk) -> cf[ik-1, jk-1, iy+my, ix+mx]
    return out.reshape(3, 3, 2 * my, 2 * mx)


def convolve(cf_block, ga, p, direct=False):
    my, mx = p.shape
    cb = np.ascontiguousarray(cf_block, dtype=np.float64)
    pp = np.ascontiguousarray(p, dtype=np.float64)
    u = np.zeros_like(pp)
    fn = lib().orc_convolve_direct if direct else lib().orc_convolve
    fn(mx, my, _dptr(cb), float(ga), _dptr(pp), _dptr(u))
    return u


SUBS_COLS = ("ux", "uy", "uz", "sighyd", "sigvm", "sigtr", "sigma1", "sigma2", "sigma3",
             "sxx", "sxy", "sxz", "syx", "syy", "syz", "szx", "szy", "szz")


def _subs_args(grid, pn, px, py, gg, poiss):
    mx, my, dx, dy, xc1, yc1 = grid
    arrs = [np.ascontiguousarray(a, dtype=np.float64).ravel() for a in (pn, px, py)]
    g = np.ascontiguousarray(gg if np.ndim(gg) else (gg, gg), dtype=np.float64)
    nu = np.ascontiguousarray(poiss if np.ndim(poiss) else (poiss, poiss), dtype=np.float64)
    return [int(mx), int(my), float(dx), float(dy), float(xc1), float(yc1)] + [_dptr(a) for a in arrs] + \
        [_dptr(g), _dptr(nu)], arrs + [g, nu]


def subsurf_points(grid, pn, px, py, gg, poiss, xyz, fast=False):
    """Subsurface field at arbitrary points (direct sum); grid = (mx, my, dx, dy, xc1, yc1).
    Returns an (npts, 18) array with the columns SUBS_COLS."""
    args, keep = _subs_args(grid, pn, px, py, gg, poiss)
    pts = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    out = np.zeros((pts.shape[0], len(SUBS_COLS)))
    lib(fast).orc_subsurf_points(*args, pts.shape[0], _dptr(pts), _dptr(out))
    return out


def subsurf_depths(grid, pn, px, py, gg, poiss, z, fast=False):
    """Subsurface field at every element centre at each depth z (influence coefficients and
    FFT convolution).  Returns an (nz, my*mx, 18) array."""
    args, keep = _subs_args(grid, pn, px, py, gg, poiss)
    zz = np.ascontiguousarray(z, dtype=np.float64).ravel()
    out = np.zeros((zz.size, int(grid[0]) * int(grid[1]), len(SUBS_COLS)))
    lib(fast).orc_subsurf_depths(*args, zz.size, _dptr(zz), _dptr(out))
    return out
