"""Sequences of solves on the GPU: continuation from the previous time instance (P = 0) and
initial estimates from the previous solution (IESTIM = 1), both read from the problem's device
copy of its last solution, against the oracle replaying the same sequences.

The reference keeps each problem's solution and, for shifts and transient rolling (T = 1, 2)
with P = 0, subtracts the displacements of the previous tractions from the shift of the new
time instance (set_prev_data, src/m_sdis.f90:208-312; stang_rhs, src/m_stang.f90:749-951).
The sequences are the testbank chains that the oracle reproduces at the reference's printed
digits (tests/test_oracle.py); each step is held to the FP64 parity bar against the oracle.
"""
import numpy as np
import pytest

import cases as C
from test_gpu_parity import assert_parity, run_gpu

pytestmark = pytest.mark.gpu


def _replay_gpu(cntc, seq, ire):
    """The sequence through the C-ABI on one problem.  A case that prescribes total forces and
    gives no creepage keeps the creepage of the previous solve (the stand-alone program's
    carry-over, as the oracle replay does), which the Newton-Raphson starts from."""
    out = []
    for c in seq:
        c = dict(c)
        if out and c.get("force3", 0) >= 1 and "cksi" not in c:
            c["cksi"] = out[-1]["creep"][0]
        if out and c.get("force3", 0) >= 2 and "ceta" not in c:
            c["ceta"] = out[-1]["creep"][1]
        out.append(run_gpu(cntc, c, ire=ire))
        out[-1]["creep"] = cntc.getcreepages(ire, 1)
    return out


@pytest.mark.parametrize("chain,steps", [("mindlin", 2), ("rolling", 3)])
def test_previous_time_instance_chain(cntc, oracle, chain, steps):
    """testbank chains: 'mindlin' (case 10, then case 11 continuing from it with the approach
    prescribed and Fx, Fy prescribed), 'rolling' (Hertzian shift of case 13, then transient
    rolling from it twice, warm-started, with Fx prescribed)."""
    # the chains' own tolerances (1e-6 .. 1e-8) leave their Newton-Raphson and TangCG stops at
    # rounding distance in places; both sides solve at eps 1e-10 to hold the parity bar
    seq = [dict(c, eps=1e-10) for c in C.testbank_chain(chain)[:steps]]
    o = C.replay_oracle(seq)
    g = _replay_gpu(cntc, seq, ire=90 if chain == "mindlin" else 91)
    for k, (gk, ok, ck) in enumerate(zip(g, o, seq)):
        assert ok["ierror"] >= 0, k
        assert_parity(gk, ok, ck)
        if ck.get("force3", 0) >= 1:
            assert abs(gk["creep"][0] - ok["cksi"]) <= 1e-10 * max(abs(ok["cksi"]), 1e-6), k


def test_warm_start_from_device_copy(cntc, oracle):
    """IESTIM = 1: the second solve starts from the first one's solution (the problem's device
    copy) with a changed creepage; same iteration path and solution as the oracle started
    from the oracle's first solution."""
    a = C.config0(gausei=5, eps=1e-9, mx=31, my=31)
    b = dict(a, cksi=0.0015, iestim=1)
    import pyoracle as po
    oa = C.oracle_solve(a)
    pb, h = C.to_oracle(b)
    ob = po.solve(pb, h=h, warm=dict(igs=oa["igs"], pn=oa["pn"], px=oa["px"], py=oa["py"]))
    ga = run_gpu(cntc, a, ire=92)
    assert_parity(ga, oa, a)
    gb = run_gpu(cntc, b, ire=92)
    assert_parity(gb, ob, b)


def test_moved_grid_refused(cntc):
    """P = 0 after a solve on another grid: the reference would move the previous tractions
    with the potential contact; this library refuses the case (CNTC_err_other)."""
    a = dict(C.config0(gausei=0, eps=1e-8, mx=21, my=21), tang=1)
    cntc.setup_case(93, 1, a)
    assert cntc.calculate(93, 1) == 0
    b = dict(a, pvtime=0, potprm=[23, 21, 6.0, 4.0, 1.1])
    cntc.setup_case(93, 1, b)
    assert cntc.calculate(93, 1) == cntc.CNTC_err_other
