"""Serving path: cntc_calculate_async / cntc_wait with continuous batching.

Each result must be the same when the patch is solved alone (cntc_calculate) and when it
shares device passes with other requests that arrive while earlier ones are running."""
import threading
import time

import numpy as np
import pytest

import cases as C

pytestmark = pytest.mark.gpu

FIELDS = ("pn", "px", "py", "igs")
SCALARS = ("fn", "fx", "fy", "mz", "pen", "itcg", "itgs", "ierror")


def _cases(n, seed):
    cs = C.batch_patches(n, seed=seed, mixed=1, eps=1e-8)
    for c in cs:
        c["potprm"] = [min(c["potprm"][0], 72), min(c["potprm"][1], 72)] + c["potprm"][2:]
    return cs


def _same(a, b):
    for k in SCALARS:
        assert a[k] == b[k], k
    for k in FIELDS:
        assert np.array_equal(a[k], b[k]), k


def test_async_results_equal_alone_and_in_mix(cntc):
    cs = _cases(10, seed=21)
    alone = []
    for i, c in enumerate(cs):
        cntc.setup_case(300 + i, 1, c)
        assert cntc.calculate(300 + i, 1) == 0
        alone.append(cntc.results(300 + i, 1))
    for i, c in enumerate(cs):
        cntc.setup_case(300 + i, 2, c)

    def submit(idx, delay):
        for i in idx:
            assert cntc.calculate_async(300 + i, 2) == 0
            time.sleep(delay)

    # two waves: the second arrives while the first is on the device
    t1 = threading.Thread(target=submit, args=(range(0, 5), 0.0))
    t1.start()
    t1.join()
    time.sleep(0.02)
    submit(range(5, 10), 0.005)
    for i in range(len(cs)):
        ierr, lat = cntc.wait(300 + i, 2, with_latency=True)
        assert ierr == 0 and lat > 0.0
    for i in range(len(cs)):
        _same(cntc.results(300 + i, 2), alone[i])


def test_async_refuses_duplicate_and_small_budget_completes(cntc):
    cs = _cases(3, seed=22)
    for i, c in enumerate(cs):
        cntc.setup_case(320 + i, 1, c)
    cntc.setadmissionbudget(1e-6)          # every request then runs alone
    try:
        for i in range(3):
            assert cntc.calculate_async(320 + i, 1) == 0
        # the problem is held by its request until cntc_wait returns (the reference refuses
        # concurrent use of one problem, m_caddon_data.f90:336-413)
        assert cntc.calculate_async(320, 1) == cntc.CNTC_err_other
        errs = [cntc.wait(320 + i, 1) for i in range(3)]
        assert errs == [0, 0, 0]
        assert cntc.calculate_async(320, 1) == 0
        assert cntc.wait(320, 1) == 0
    finally:
        cntc.setadmissionbudget(40.0)


def test_coefficient_cache_reused_and_exact(cntc):
    """Influence coefficients and spectra stay on the device per problem: a new time step
    with other creepages and Fn on the same grid launches only the solve kernel, and its
    result equals a fresh problem's; a new grid recomputes them."""
    c = C.config0(gausei=5, eps=1e-8, mx=40, my=36, mixed=1)
    cntc.setup_case(320, 1, c)
    assert cntc.calculate(320, 1) == 0
    step = dict(c, cksi=0.0012, ceta=-0.0004, fn=9.1e4)
    cntc.setcreepages(320, 1, step["cksi"], step["ceta"], step["cphi"])
    cntc.setnormalforce(320, 1, step["fn"])
    k0 = cntc.kernel_launches()
    assert cntc.calculate(320, 1) == 0
    assert cntc.kernel_launches() - k0 == 1          # solve only: coefficients reused
    cntc.setup_case(321, 1, step)
    k0 = cntc.kernel_launches()
    assert cntc.calculate(321, 1) == 0
    assert cntc.kernel_launches() - k0 == 3          # influence, spectra, solve
    _same(cntc.results(320, 1), cntc.results(321, 1))
    # another grid on the same problem: recomputed, equal to a fresh problem
    other = dict(step, potprm=[44, 30] + step["potprm"][2:])
    cntc.setup_case(320, 1, other)
    k0 = cntc.kernel_launches()
    assert cntc.calculate(320, 1) == 0
    assert cntc.kernel_launches() - k0 == 3
    cntc.setup_case(322, 1, other)
    assert cntc.calculate(322, 1) == 0
    _same(cntc.results(320, 1), cntc.results(322, 1))
