"""Oracle solutions of the non-Hertzian grid sweep at the grid sizes the oracle takes tens of
seconds (256^2) to minutes (512^2) for, committed as fixtures for the GPU parity tests (tests/test_gpu_sweep.py).

Each fixture holds the oracle's (baseline build) solution of one seeded case: error code and
iteration counts, the element division of every element, the total forces, approach and
maximum pressure, and the tractions pn, px, py of every STRIDE-th element (the stride keeps the
file small; the parity bar holds element by element on that sample).

    python tests/golden/make_config1.py [256] [512]   # writes tests/golden/config1_<m>.npz
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))

import cases as C  # noqa: E402

STRIDE = 7


def make(m, path, maxgs=2000, stride=STRIDE):
    case = C.config1(m, seed=1, eps=1e-8, maxgs=maxgs)
    o = C.oracle_solve(case, fast=True)
    sel = np.arange(0, m * m, stride)
    np.savez_compressed(path, m=m, seed=1, eps=1e-8, maxgs=maxgs, stride=stride,
                        it=np.array([o["ierror"], o["itnorm"], o["ittang"], o["itcg"], o["itgs"], o["solver"]]),
                        scal=np.array([o["fn"], o["fx"], o["fy"], o["mz"], o["pen"], o["pmax"]]),
                        igs=o["igs"].astype(np.int8), sel=sel.astype(np.int32),
                        pn=o["pn"][sel], px=o["px"][sel], py=o["py"][sel])
    return o


if __name__ == "__main__":
    which = sys.argv[1:] or ["256", "512"]
    for m, maxgs, stride in ((256, 2000, STRIDE), (512, 5000, 29)):
        if str(m) not in which:
            continue
        o = make(m, os.path.join(HERE, "config1_%d.npz" % m), maxgs=maxgs, stride=stride)
        print("%d^2: ierror %d, itcg %d, itgs %d, Fx %.10g" % (m, o["ierror"], o["itcg"], o["itgs"], o["fx"]))
