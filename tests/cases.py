"""Case descriptions shared by the parity tests and the benchmark.

A case is a plain dict (see contact_gb300.setup_case for the keys).  The same dict
drives the GB300 library through its C-ABI and the CPU oracle, so both solve exactly
the same problem.
"""
import ctypes
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if os.path.join(ROOT, "oracle") not in sys.path:
    sys.path.insert(0, os.path.join(ROOT, "oracle"))

E_STEEL = 210000.0          # N/mm^2
NU_STEEL = 0.28
G_STEEL = E_STEEL / (2.0 * (1.0 + NU_STEEL))


def f32(v):
    return float(np.float32(v))


def config0(gausei=5, eps=1e-10, mixed=0, mx=51, my=51):
    """Plain FP64 Hertzian steady rolling: a=6 mm, b=4 mm, 51x51 over 1.1a x 1.1b, Fn=100 kN,
    creepage 0.001, mu=0.3, steel on steel."""
    return dict(tang=3, norm=1, bound=0, gausei=gausei, maxgs=999, maxin=100, maxnr=30, maxout=1, eps=eps,
                poiss=NU_STEEL, gg=G_STEEL, fstat=0.3, veloc=10000.0, fn=1e5, cksi=0.001, ceta=0.0, cphi=0.0,
                ipotcn=-3, potprm=[mx, my, 6.0, 4.0, 1.1], mixed=mixed)


# test_table (src/test_table.f90:60-292): 11x11 Hertz grids, SteadyGS, eps 1e-6
TT_ELLIP = [f32(0.2), f32(0.5), 1.0, 2.0, 5.0]
TT_AA = [4.0, 6.0, 9.0, 12.0, 20.0]
TT_SPIN = [0.0, 0.5, 1.0, 2.0]
TT_ANGL = [-math.pi / 2, -math.pi / 3, -math.pi / 6, 0.0, math.pi / 6, math.pi / 3, math.pi / 2]
TT_MAGN = [f32(v) for v in (0.0, 0.1, 0.2, 0.3, 0.4, 0.5, 0.7, 0.9, 1.1, 1.4, 1.7, 2.0, 2.5, 3.0, 3.5, 4.0, 5.0,
                            6.0, 7.0, 8.0, 9.0, 10., 12.)]
TT_MX = 11
TT_SCALE = f32(np.float32(TT_MX) / np.float32(TT_MX - 4))


def test_table_base(iell):
    return dict(tang=3, norm=1, bound=0, gausei=0, maxgs=299, maxin=1, maxnr=30, maxout=1, eps=1e-6,
                poiss=0.28, gg=82000.0, fstat=0.3, veloc=10000.0, fn=82000.0, cksi=0.0, ceta=0.0, cphi=0.0,
                ipotcn=-3, potprm=[TT_MX, TT_MX, TT_AA[iell], TT_AA[iell] / TT_ELLIP[iell], TT_SCALE])


def test_table_case(icase, rho, cp):
    """Case number icase (0-based) of test_table, with the Hertz rho, cp per ellipticity."""
    ivmgn = icase % 23
    irem = icase // 23
    ivang = irem % 7
    irem //= 7
    ispin = irem % 4
    irem //= 4
    iell = irem % 5
    c = test_table_base(iell)
    cmgn, cang = TT_MAGN[ivmgn], TT_ANGL[ivang]
    c["cksi"] = cmgn * 0.3 * math.cos(cang) * cp[iell] / rho[iell]
    c["ceta"] = cmgn * 0.3 * math.sin(cang) * cp[iell] / rho[iell]
    c["cphi"] = 0.3 * TT_SPIN[ispin] / rho[iell]
    return c, iell


def tractcurv_case(cksi):
    """First series of examples/tractcurv.inp: Hertz a1=0.0008/mm, a/b=0.5, 48x44, Fn=106.7 kN."""
    return dict(tang=3, norm=1, bound=0, gausei=0, maxgs=80, maxin=200, maxnr=5, maxout=1, eps=1e-6,
                poiss=0.28, gg=82000.0, fstat=0.33, veloc=10000.0, fn=106700.0, cksi=cksi, ceta=0.0, cphi=0.0,
                ipotcn=-2, potprm=[48, 44, 0.0008, 0.5, 1.1], dq=0.5)


def cattaneo_case(icase, cksi=0.0):
    """examples/cattaneo.inp, a polyethylene ball (G 200 N/mm^2, nu 0.42, mu 0.4) on a plane,
    19x19 grid, Fn 9.1954 N, eps 1e-4.  Case 1: Hertzian semi-axes 1 mm, normal problem only.
    Case 2: the same geometry as quadratic undeformed distance 0.01 x^2 + 0.01 y^2 on the grid
    from -1.26667 mm with spacing 0.13333 mm, and the shift problem (T=1, TangCG) with rigid
    shift cksi (the reference prescribes the force and finds the shift by Newton-Raphson)."""
    c = dict(tang=0, norm=1, bound=0, gausei=0, maxgs=100, maxin=100, maxnr=30, maxout=1, eps=1e-4,
             poiss=0.42, gg=200.0, fstat=0.4, veloc=1.0, fn=9.1954, cksi=0.0, ceta=0.0, cphi=0.0)
    if icase == 1:
        c.update(ipotcn=-3, potprm=[19, 19, 1.0, 1.0, 1.26667])
    else:
        c.update(tang=1, cksi=cksi, ipotcn=1, potprm=[19, 19, -1.26667, -1.26667, 0.13333, 0.13333],
                 prmudf=[0.01, 0.0, 0.01, 0.0, 0.0, 0.0])
    return c


def cattaneo_forces_case():
    """Case 2 of examples/cattaneo.inp as the reference states it: the tangential forces
    prescribed (F=2), Fx = -0.875 mu Fn and Fy = 0, met by Newton-Raphson on the shifts."""
    c = cattaneo_case(2)
    del c["cksi"], c["ceta"]
    c.update(force3=2, fxrel=-0.875, fyrel=0.0)
    return c


def catt_to_cart_case1():
    """Case 1 of examples/catt_to_cart.inp: Cattaneo shift of a ball (G 1, nu 0.28, mu 0.4013,
    Fn 0.4705) on a 34x33 grid from -4.125 mm with spacing 0.25 mm, quadratic geometry
    0.002963 (x^2 + y^2), Fx = -0.657 mu Fn prescribed (F=1), ceta 0, TangCG, eps 1e-7."""
    return dict(tang=1, norm=1, bound=0, gausei=0, maxgs=100, maxin=100, maxnr=30, maxout=1, eps=1e-7,
                poiss=0.28, gg=1.0, fstat=0.4013, veloc=1.0, fn=0.4705, ceta=0.0, cphi=0.0, force3=1,
                fxrel=-0.657, ipotcn=1, potprm=[34, 33, -4.125, -4.125, 0.25, 0.25],
                prmudf=[0.002963, 0.0, 0.002963, 0.0, 0.0, 0.0])


def testbank_chain(name):
    """Sequences of testbank/testbank.inp whose later cases continue from the previous time
    instance (P=0), to be replayed in order (replay_oracle).  'mindlin': case 10 then case 11,
    a shift with the approach 0.01131 mm prescribed and Fx = -0.875 mu Fn, Fy = 0 from case
    10's tractions.  'rolling': case 13 (Hertzian shift) then cases 14-16, transient rolling
    (dq 0.2 mm) with Fx prescribed and the previous solution as initial estimate, the last
    step with creepage -0.002124, dq 0.8 mm and the grid from curvature 0.2963e-2 and a/b 1.
    'tilted': case 25 then case 26, the same bodies with the surface tilted by -0.031816."""
    if name == "mindlin":
        c10 = testbank_case(10)
        c11 = dict(c10, pvtime=0, norm=0, pen=0.01131, force3=2, fxrel=-0.875, fyrel=0.0, standalone=True)
        del c11["fn"]
        return [dict(c10, standalone=True), c11]
    if name == "rolling":
        c13 = dict(testbank_case(13), standalone=True)
        c14 = dict(c13, pvtime=0, bound=0, tang=2, iestim=1, maxin=100, maxnr=30, dq=0.2, veloc=1000.0)
        c16 = dict(c14, force3=0, cksi=-0.002124, dq=0.8, ipotcn=-2, potprm=[41, 41, 0.2963e-2, 1.0, 1.17143])
        return [c13, c14, dict(c14), c16]
    if name == "tilted":
        c25 = testbank_case(25)
        c26 = dict(c25, pvtime=0, prmudf=[0.0, 0.0, 0.0, -0.031816, 0.0, 0.0])
        return [c25, c26]
    raise ValueError(name)


def subsurf_case(icase):
    """examples/subsurf.inp: one 1x1 mm element (first corner at -0.4999, -0.4998), G 1, nu
    0.28, mu 1, Fn 1, geometry 2.16 (x^2 + y^2), eps 1e-6.  Case 1: the normal problem alone.
    Case 2: steady rolling with Fx = 0.999 mu Fn prescribed (F=1); contact reaches the
    trailing column, so the reference solves it by ConvexGS."""
    c = dict(tang=0, norm=1, bound=0, gausei=0, maxgs=80, maxin=100, maxnr=30, maxout=1, eps=1e-6, poiss=0.28,
             gg=1.0, fstat=1.0, veloc=30000.0, fn=1.0, cksi=0.0, ceta=0.0, cphi=0.0,
             ipotcn=1, potprm=[1, 1, -0.4999, -0.4998, 1.0, 1.0], prmudf=[2.16, 0.0, 2.16, 0.0, 0.0, 0.0])
    if icase == 2:
        del c["cksi"]
        c.update(tang=3, force3=1, fxrel=0.999)
    return c


def carter2d_case():
    """examples/carter2d.inp: Carter's two-dimensional steady rolling (T=3, SteadyGS, eps 1e-5)
    on a 55x1 strip from x = -1.05 mm with dx 0.04 mm and dy 200 mm, steel (G 82000, nu
    0.28, mu 0.3), Fn 35780 N, creepage -0.00024, undeformed distance 0.001 x^2."""
    return dict(tang=3, norm=1, bound=0, gausei=0, maxgs=999, maxin=100, maxnr=30, maxout=1, eps=1e-5,
                poiss=0.28, gg=82000.0, fstat=0.3, veloc=30000.0, fn=35780.0, cksi=-0.00024, ceta=0.0, cphi=0.0,
                ipotcn=3, potprm=[55, 1, -1.05, 0.0, 0.04, 200.0], dq=0.0401,
                prmudf=[0.001, 0.0, 0.0, 0.0, 0.0, 0.0])


def test_caddon_element1():
    """Result element 1 of src/test_caddon.f90 in CONTACT units (mm, N, rad/mm): steel
    (G 82000 N/mm^2, nu 0.28, mu 0.3), Hertzian semi-axes 4.25 x 7 mm on a 21x33 grid (scale
    21/17), penetration 0.05 mm prescribed, creepage 0.001, spin 0.4 rad/m, rolling speed
    24 m/s, SteadyGS with maxgs 999, maxin 30, eps 1e-4."""
    return dict(tang=3, norm=0, bound=0, gausei=0, maxgs=999, maxin=30, maxnr=30, maxout=1, eps=1e-4,
                poiss=0.28, gg=82000.0, fstat=0.3, veloc=24000.0, pen=0.05, cksi=0.001, ceta=0.0, cphi=0.4e-3,
                ipotcn=-3, potprm=[21, 33, 4.25, 7.0, 21.0 / 17.0], dq=0.5)


def testbank_case(icase):
    """Cases of testbank/testbank.inp.  1: shift problem (T=1) with prescribed approach
    0.01131 mm and shift 0.00304 mm, steel, mu 0.3, quadratic geometry 0.0056566 (x^2 + y^2)
    on a 17x17 grid from -1.13333 mm with spacing 0.13333 mm, TangCG, eps 1e-8.
    6: Carter's strip (as examples/carter2d.inp, first centre at -1.045 mm) by ConvexGS (G=2,
    omegah = omegas = 0.8) with a rolling step dq of 0.2 mm = 5 dx.
    7: steady rolling, Fn 0.4705, creepage -0.00304, mu 0.4013, G 1, nu 0.28, dq 0.2 mm,
    quadratic geometry 0.002963 (x^2 + y^2) on a 41x41 grid from -4.1 mm with spacing 0.2 mm,
    SteadyGS with maxgs 80, maxin 30, eps 1e-6.
    9: steady rolling with different materials (nu 0.1 and 0.28, G 1 and 81000: K = 0.4, the
    normal and tangential problems coupled and solved alternately, maxout 10), Fn 2.468, Fx =
    -0.4718 mu Fn prescribed, spin 1e-4, mu 0.6, 25x25 grid, SteadyGS.
    17: transient rolling from rest (T=2, dq 0.4 mm) of case 7's geometry, Fx = 0.657 mu Fn
    prescribed, TangCG, maxin 30, maxnr 5.
    25: a shift (T=1) of two very different bodies (nu 0.5, G 2e7 against nu 0, G 200) pressed
    by Fn 400 kN on a flat 251x1 strip from x = -20 mm, dx 0.16 mm, mu 0.4, eps 1e-8, up to
    30 outer iterations of the coupled problems.
    10: case 1 with Fn 1722 N, Fx = -0.875 mu Fn and Fy = 0 prescribed (F=2), the grid given by
    its corners.  13: a Cattaneo shift on a 41x41 Hertzian grid (semi-axes 4.1 mm, scale
    1.17143) with the normal problem skipped for the elliptical traction bound (B=2), Fn
    0.7563, Fx = 0.657 mu Fn prescribed (F=1), G 1, nu 0.28, mu 0.4013, TangCG, eps 1e-6.
    4: steady rolling on a 3x3 Hertzian grid (semi-axes 0.5 mm, scale 3) with one element in
    contact, two materials (G 200 and 1, nu 0.28), Fn 1, Fx = 0.999 mu Fn prescribed (F=1), mu 1,
    SteadyGS, eps 1e-4, up to 10 outer iterations of the coupled problems."""
    if icase == 3:                # case 4's bodies and grid, normal problem only
        return dict(tang=0, norm=1, bound=0, gausei=0, maxgs=80, maxin=100, maxnr=30, maxout=1, eps=1e-4,
                    poiss=0.28, poiss2=0.28, gg=200.0, gg2=1.0, fstat=1.0, veloc=1.0, fn=1.0, cksi=0.0,
                    ceta=0.0, cphi=0.0, ipotcn=-3, potprm=[3, 3, 0.5, 0.5, 3.0], standalone=True)
    if icase == 4:
        return dict(tang=3, norm=1, bound=0, gausei=0, maxgs=80, maxin=100, maxnr=30, maxout=10, eps=1e-4,
                    poiss=0.28, poiss2=0.28, gg=200.0, gg2=1.0, fstat=1.0, veloc=1000.0, fn=1.0, ceta=0.0,
                    cphi=0.0, force3=1, fxrel=0.999, dq=1.0, ipotcn=-3, potprm=[3, 3, 0.5, 0.5, 3.0],
                    standalone=True)
    if icase == 6:
        return dict(tang=3, norm=1, bound=0, gausei=2, maxgs=999, maxin=100, maxnr=30, maxout=1, eps=1e-5,
                    omegah=0.8, omegas=0.8, poiss=0.28, gg=82000.0, fstat=0.3, veloc=30000.0, fn=35780.0,
                    cksi=-0.00024, ceta=0.0, cphi=0.0, dq=0.2, ipotcn=3, potprm=[55, 1, -1.045, 0.0, 0.04, 200.0],
                    prmudf=[0.001, 0.0, 0.0, 0.0, 0.0, 0.0])
    if icase == 9:
        return dict(tang=3, norm=1, bound=0, gausei=0, maxgs=80, maxin=100, maxnr=30, maxout=10, eps=1e-6,
                    poiss=0.1, poiss2=0.28, gg=1.0, gg2=0.81e5, fstat=0.6, veloc=1000.0, fn=2.468, ceta=0.0,
                    cphi=1e-4, force3=1, fxrel=-0.4718, dq=1.1, ipotcn=1,
                    potprm=[25, 25, -13.75, -13.75, 1.1, 1.1], prmudf=[0.3332e-3, 0.0, 0.3332e-3, 0.0, 0.0, 0.0])
    if icase == 17:
        return dict(tang=2, norm=1, bound=0, gausei=0, maxgs=80, maxin=30, maxnr=5, maxout=1, eps=1e-6, poiss=0.28,
                    gg=1.0, fstat=0.4013, veloc=1000.0, fn=0.4705, ceta=0.0, cphi=0.0, force3=1, fxrel=0.657, dq=0.4,
                    ipotcn=1, potprm=[41, 41, -4.1, -4.1, 0.2, 0.2], prmudf=[0.002963, 0.0, 0.002963, 0.0, 0.0, 0.0],
                    standalone=True)
    if icase == 25:
        return dict(tang=1, norm=1, bound=0, gausei=0, maxgs=100, maxin=100, maxnr=30, maxout=30, eps=1e-8,
                    poiss=0.5, poiss2=0.0, gg=2e7, gg2=200.0, fstat=0.4, veloc=1.0, fn=400000.0, cksi=0.0, ceta=0.0,
                    cphi=0.0, ipotcn=3, potprm=[251, 1, -20.0, 0.0, 0.16, 1000.0],
                    prmudf=[0.0, 0.0, 0.0, 0.0, 0.0, 0.0], standalone=True)
    if icase == 10:
        return dict(tang=1, norm=1, bound=0, gausei=0, maxgs=100, maxin=100, maxnr=30, maxout=1, eps=1e-8,
                    poiss=0.28, gg=82000.0, fstat=0.3, veloc=1.0, fn=1722.0, cphi=0.0, force3=2, fxrel=-0.875,
                    fyrel=0.0, ipotcn=2, potprm=[17, 17, -1.13333, -1.13333, 1.13333, 1.13333],
                    prmudf=[0.0056566, 0.0, 0.0056566, 0.0, 0.0, 0.0])
    if icase == 13:
        return dict(tang=1, norm=1, bound=2, gausei=0, maxgs=80, maxin=100, maxnr=30, maxout=1, eps=1e-6,
                    poiss=0.28, gg=1.0, fstat=0.4013, veloc=1.0, fn=0.7563, ceta=0.0, cphi=0.0, force3=1,
                    fxrel=0.657, ipotcn=-3, potprm=[41, 41, 4.1, 4.1, 1.17143])
    if icase == 1:
        return dict(tang=1, norm=0, bound=0, gausei=0, maxgs=100, maxin=100, maxnr=30, maxout=1, eps=1e-8,
                    poiss=0.28, gg=82000.0, fstat=0.3, veloc=1.0, pen=0.01131, cksi=0.00304, ceta=0.0, cphi=0.0,
                    ipotcn=1, potprm=[17, 17, -1.13333, -1.13333, 0.13333, 0.13333],
                    prmudf=[0.0056566, 0.0, 0.0056566, 0.0, 0.0, 0.0])
    return dict(tang=3, norm=1, bound=0, gausei=0, maxgs=80, maxin=30, maxnr=5, maxout=1, eps=1e-6,
                poiss=0.28, gg=1.0, fstat=0.4013, veloc=1000.0, fn=0.4705, cksi=-0.00304, ceta=0.0, cphi=0.0,
                dq=0.2, ipotcn=1, potprm=[41, 41, -4.1, -4.1, 0.2, 0.2],
                prmudf=[0.002963, 0.0, 0.002963, 0.0, 0.0, 0.0])


def rough_surface(mx, my, xl, yl, dx, dy, pen_hz, seed, rx=460.0, ry=300.0, nsin=8):
    """Non-Hertzian undeformed distance: x^2/(2Rx) + y^2/(2Ry) + a seeded sum of 8 sinusoids
    (wavelength 1-5 mm, total amplitude 5% of the Hertzian approach)."""
    rng = np.random.default_rng(seed)
    lam = rng.uniform(1.0, 5.0, nsin)
    th = rng.uniform(0.0, math.pi, nsin)
    ph = rng.uniform(0.0, 2 * math.pi, nsin)
    amp = rng.uniform(0.0, 1.0, nsin)
    amp = amp / amp.sum() * 0.05 * pen_hz
    x = xl + (np.arange(mx) + 0.5) * dx
    y = yl + (np.arange(my) + 0.5) * dy
    X, Y = np.meshgrid(x, y)
    h = X ** 2 / (2 * rx) + Y ** 2 / (2 * ry)
    for k in range(nsin):
        h = h + amp[k] * np.sin(2 * math.pi * (X * math.cos(th[k]) + Y * math.sin(th[k])) / lam[k] + ph[k])
    return h


def config1(m, seed=1, gausei=5, eps=1e-8, mixed=0, fn=1e5, cksi=0.002, ceta=0.001, cphi=2e-4, mu=0.3, maxgs=999):
    """Non-Hertzian grid case: square m x m grid over [-1.25a, 1.25a]^2 of the Hertz solution
    for Rx=460, Ry=300 mm; element-wise h with seeded roughness.  GDsteady needs more
    iterations as the grid grows (about 300 at 128^2): large grids raise maxgs."""
    a_est = 7.2 * (fn / 1e5) ** (1.0 / 3.0)
    half = 1.25 * a_est
    dx = 2 * half / m
    pen_hz = 0.16 * (fn / 1e5) ** (2.0 / 3.0)
    h = rough_surface(m, m, -half, -half, dx, dx, pen_hz, seed)
    return dict(tang=3, norm=1, bound=0, gausei=gausei, maxgs=maxgs, maxin=100, maxnr=30, maxout=1, eps=eps,
                poiss=NU_STEEL, gg=G_STEEL, fstat=mu, veloc=10000.0, fn=fn, cksi=cksi, ceta=ceta, cphi=cphi,
                ipotcn=1, potprm=[m, m, -half, -half, dx, dx], h=h, mixed=mixed)


def config4(seed=4, mixed=0, maxgs=5000, eps=1e-8):
    """Large single patch: 1024^2 rough-surface grid as config1, Fn=150 kN, creepages
    (0.003, 0, 0.3 rad/m), mu=0.25."""
    return config1(1024, seed=seed, fn=150e3, cksi=0.003, ceta=0.0, cphi=3e-4, mu=0.25, mixed=mixed, maxgs=maxgs,
                   eps=eps)


def batch_patches(n, seed=2, mixed=1, eps=1e-8):
    """Batched workload: n independent Hertzian patches, sides U{24..160}, semi-axes
    log-uniform 2-10 mm, Fn U[10,150] kN, creepages U[-0.005,0.005], spin U[-0.5,0.5] rad/m,
    mu U[0.2,0.4], GDsteady with FP32 bulk + FP64 refinement."""
    rng = np.random.default_rng(seed)
    cases = []
    for i in range(n):
        mx, my = int(rng.integers(24, 161)), int(rng.integers(24, 161))
        a = float(np.exp(rng.uniform(math.log(2.0), math.log(10.0))))
        b = float(np.exp(rng.uniform(math.log(2.0), math.log(10.0))))
        fn = float(rng.uniform(10e3, 150e3))
        cksi, ceta = float(rng.uniform(-0.005, 0.005)), float(rng.uniform(-0.005, 0.005))
        cphi = float(rng.uniform(-0.5, 0.5)) * 1e-3            # rad/m -> rad/mm
        mu = float(rng.uniform(0.2, 0.4))
        cases.append(dict(tang=3, norm=1, bound=0, gausei=5, maxgs=999, maxin=100, maxnr=30, maxout=1, eps=eps,
                          poiss=NU_STEEL, gg=G_STEEL, fstat=mu, veloc=10000.0, fn=fn, cksi=cksi, ceta=ceta,
                          cphi=cphi, ipotcn=-3, potprm=[mx, my, a, b, 1.1], mixed=mixed))
    return cases


def to_oracle(case):
    """Oracle problem for a case dict; returns (Problem, h or None)."""
    import pyoracle as po
    pb = po.default_problem()
    pb.tang = case.get("tang", 3)
    pb.norm = case.get("norm", 1)
    pb.bound = case.get("bound", 0)
    pb.gausei = case.get("gausei", 0)
    pb.maxgs = case.get("maxgs", 999)
    pb.maxin = case.get("maxin", 100)
    pb.maxnr = case.get("maxnr", 30)
    pb.maxout = case.get("maxout", 1)
    pb.eps = case.get("eps", 1e-6)
    nu = case.get("poiss", 0.28)
    g = case.get("gg", 82000.0)
    pb.poiss1, pb.poiss2 = nu, case.get("poiss2", nu)
    pb.gg1, pb.gg2 = g, case.get("gg2", g)
    pb.fstat = pb.fkin = case.get("fstat", 0.3)
    pb.veloc = case.get("veloc", 10000.0)
    if "dq" in case:
        pb.dq = case["dq"]
    if "chi" in case:
        pb.chi = case["chi"]
    pb.cksi, pb.ceta, pb.cphi = case.get("cksi", 0.0), case.get("ceta", 0.0), case.get("cphi", 0.0)
    pb.force3 = case.get("force3", 0)
    if "omegah" in case:
        pb.omegah, pb.omegas = case["omegah"], case["omegas"]
    if "inislp" in case:
        pb.inislp, pb.omgslp = case["inislp"], case["omgslp"]
    if case.get("frclaw", 0) >= 2:
        pb.frclaw = case["frclaw"]
        for k, v in enumerate(case["flaw"]):
            pb.flaw[k] = v
        pb.memdst, pb.mem_s0 = case.get("memdst", 0.0), case.get("mem_s0", 0.0)
    if case.get("mater", 0) == 4:
        pb.mater = 4
        pb.gg3, pb.laythk, pb.tau_c0, pb.k_tau = case["gg3"], case["laythk"], case["tau_c0"], case["k_tau"]
    pb.fxrel, pb.fyrel = case.get("fxrel", 0.0), case.get("fyrel", 0.0)
    pb.sens = case.get("sens", 1)
    if "mxsens" in case:
        pb.mxsens = case["mxsens"]
    if "epsens" in case:
        pb.epsens = case["epsens"]
    pb.standalone = int(case.get("standalone", False))
    pb.pvtime = case.get("pvtime", 2)
    if "iestim" in case:
        pb.iestim = case["iestim"]
    if pb.norm == 1:
        pb.fn = case["fn"]
    else:
        pb.pen = case["pen"]
    pb.ipotcn = case.get("ipotcn", -3)
    for k, v in enumerate(case["potprm"][:6]):
        pb.potprm[k] = v
    if pb.gausei == 5:
        gd = case.get("gd", dict(fdecay=0.9, betath=0.1, kdowfb=1, d_ifc=1.0, d_lin=1.0, d_cns=1.0, d_slp=1.0,
                                 pow_s=0.9))
        pb.fdecay, pb.betath, pb.kdowfb = gd["fdecay"], gd["betath"], gd["kdowfb"]
        pb.d_ifc, pb.d_lin, pb.d_cns, pb.d_slp, pb.pow_s = gd["d_ifc"], gd["d_lin"], gd["d_cns"], gd["d_slp"], gd["pow_s"]
    if "prmudf" in case:
        arr = np.ascontiguousarray(case["prmudf"], dtype=np.float64)
        pb.ibase = 1
        pb.nprmudf = arr.size
        pb.prmudf = arr.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        pb._keep = arr                       # alive until the solve returns
    return pb, case.get("h")


def _grid_of(case, prev):
    """(mx, my, dx, dy, xc1, yc1) of an explicit potential contact (IPOTCN 1..4, potcon_fill),
    or the previous solution's grid for a Hertzian one."""
    ip, pr = case.get("ipotcn", -3), case["potprm"]
    mx, my = int(pr[0]), int(pr[1])
    if ip == 1:
        return mx, my, pr[4], pr[5], pr[2] + 0.5 * pr[4], pr[3] + 0.5 * pr[5]
    if ip == 2:
        dx, dy = (pr[4] - pr[2]) / mx, (pr[5] - pr[3]) / my
        return mx, my, dx, dy, pr[2] + 0.5 * dx, pr[3] + 0.5 * dy
    if ip == 3:
        return mx, my, pr[4], pr[5], pr[2], pr[3]
    if ip == 4:
        return mx, my, (pr[4] - pr[2]) / max(1, mx - 1), (pr[5] - pr[3]) / max(1, my - 1), pr[2], pr[3]
    return prev["mx"], prev["my"], prev["dx"], prev["dy"], prev["xc1"], prev["yc1"]


def _on_grid(prev, grid):
    """The previous solution's element division and tractions carried to a grid of the same
    spacing shifted by whole elements (eldiv_resize, gf3_resize: m_gridfunc_sub.f90:21-159):
    exterior and zero where the old grid does not reach."""
    mx, my, dx, dy, xc1, yc1 = grid
    kx = int(round((xc1 - prev["xc1"]) / dx))
    ky = int(round((yc1 - prev["yc1"]) / dy))
    keys = ("pn", "px", "py", "mus", "svx", "svy")
    prev = dict(prev, svx=prev["sx"] * prev.get("dq_used", 1.0), svy=prev["sy"] * prev.get("dq_used", 1.0))
    out = {"igs": np.zeros(mx * my, dtype=np.int32)}
    for k in keys:
        out[k] = np.zeros(mx * my)
    for iy in range(my):
        jy = iy + ky
        if not 0 <= jy < prev["my"]:
            continue
        for ix in range(mx):
            jx = ix + kx
            if 0 <= jx < prev["mx"]:
                out["igs"][ix + iy * mx] = prev["igs"][jx + jy * prev["mx"]]
                for k in keys:
                    out[k][ix + iy * mx] = prev[k][jx + jy * prev["mx"]]
    return out


def _step(case):
    """The rolling step dq a case is solved with (check_roll_stepsize, m_sdis.f90:125-206):
    dx for steady rolling other than by ConvexGS, 1 for shifts."""
    grid = _grid_of(case, None) if case.get("ipotcn", -3) >= 1 else None
    if case.get("tang", 3) not in (2, 3):
        return 1.0
    if case.get("tang") == 3 and case.get("gausei", 0) != 2 and grid is not None:
        return grid[2]
    return case.get("dq", grid[2] if grid else 1.0)


def replay_oracle(case_list, fast=False):
    """Solve the cases of an input file (contact_gb300.inp.read_inp) in order through the
    oracle, carrying the state from case to case as the stand-alone program does: a case with
    an initial estimate (IESTIM 1) starts from the previous solution and its sensitivities;
    creepages that a case does not prescribe (total forces given) keep their previous value.
    In a transient sequence (P = 0, 1) the previous solution is the previous time instance.
    Where the potential contact moves by whole elements, the previous solution moves with it."""
    import pyoracle as po
    out, prev = [], None
    for case in case_list:
        c = dict(case)
        if prev is not None:
            if c.get("force3", 0) >= 1:
                c.setdefault("cksi", prev["cksi"])
            if c.get("force3", 0) >= 2:
                c.setdefault("ceta", prev["ceta"])
        pb, h = to_oracle(c)
        warm = pv = None
        if prev is not None and (c.get("iestim", 0) >= 1 or c.get("pvtime", 2) <= 1):
            moved = _on_grid(prev, _grid_of(c, prev))
            if c.get("iestim", 0) >= 1:
                warm = dict(moved, sens=prev["sens"])
            if c.get("pvtime", 2) <= 1:
                pv = moved
        prev = po.solve(pb, h=h, warm=warm, fast=fast, prev=pv)
        prev["dq_used"] = _step(c)
        out.append(prev)
    return out


def oracle_solve(case, fast=False):
    """The oracle's solve of a case; fast: its baseline build (Stockham FFT, real-input convolutions)."""
    import pyoracle as po
    pb, h = to_oracle(case)
    return po.solve(pb, h=h, fast=fast)
