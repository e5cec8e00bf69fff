"""The non-Hertzian grid sweep (seeded sinusoidal roughness on a quadratic gap, Fn 100 kN,
creepages (0.002, 0.001, 0.2 rad/m), mu 0.3) at its configured grid sizes, against the oracle.

128 x 128 is solved by the oracle inside the test (a few seconds); 256 x 256 and 512 x 512
(patch groups on the GPU) against the committed oracle fixtures tests/golden/config1_256.npz
and config1_512.npz, made by tests/golden/make_config1.py.  The bar is the FP64 parity bar of the other tests: identical
element division and iteration counts, forces within 1e-10, tractions within 1e-8 of pmax.
The case with the large patch's parameters (seed 4, Fn 150 kN, creepages (0.003, 0, 0.3
rad/m), mu 0.25) is held to the same bar at 128 x 128.
"""
import os

import numpy as np
import pytest

import cases as C
from test_gpu_parity import FORCE_TOL, MIXED_FORCE_TOL, TRAC_TOL, assert_parity, force_err, run_gpu

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("mixed", [0, 1])
def test_sweep_128_against_oracle(cntc, oracle, mixed):
    case = C.config1(128, seed=1, eps=1e-8)
    o = C.oracle_solve(case, fast=True)
    g = run_gpu(cntc, dict(case, mixed=mixed), ire=100)
    assert o["ierror"] == 0
    if mixed:
        assert_parity(g, o, case, force_tol=MIXED_FORCE_TOL, trac_tol=TRAC_TOL, iterations=False)
    else:
        assert_parity(g, o, case)


def test_large_patch_parameters_128_against_oracle(cntc, oracle):
    case = C.config1(128, seed=4, fn=150e3, cksi=0.003, ceta=0.0, cphi=3e-4, mu=0.25, eps=1e-8)
    o = C.oracle_solve(case, fast=True)
    g = run_gpu(cntc, case, ire=101)
    assert o["ierror"] == 0
    assert_parity(g, o, case)


@pytest.mark.parametrize("m", [256, 512])
def test_sweep_against_fixture(cntc, m):
    f = np.load(os.path.join(GOLD, "config1_%d.npz" % m))
    assert int(f["m"]) == m
    case = C.config1(m, seed=int(f["seed"]), eps=float(f["eps"]), maxgs=int(f["maxgs"]))
    g = run_gpu(cntc, case, ire=102)
    assert int(cntc.getsolverstats(102, 1)["ctas"]) > 1          # a patch group
    ierr, itnorm, ittang, itcg, itgs, solver = (int(v) for v in f["it"])
    assert g["ierror_call"] == ierr == 0
    assert np.array_equal(g["igs"], f["igs"].astype(np.int32))
    fn, fx, fy, mz, pen, pmax = (float(v) for v in f["scal"])
    o = dict(fn=fn, fx=fx, fy=fy, mz=mz)
    fe = force_err(g, o, case["fstat"])
    assert max(fe.values()) <= FORCE_TOL, fe
    assert abs(g["pen"] - pen) <= 1e-10 * abs(pen)
    sel = f["sel"]
    for k in ("pn", "px", "py"):
        assert np.abs(g[k][sel] - f[k]).max() <= TRAC_TOL * pmax, k
    assert (g["itnorm"], g["ittang"], g["itcg"], g["itgs"]) == (itnorm, ittang, itcg, itgs)
