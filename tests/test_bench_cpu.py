"""Host-side error measures of bench.py (CPU only): the per-patch comparison of two solution
forms of the same problems (tangential and normal force, maximum pressure, traction field,
element division) and its summary, on a fake library whose results are set by the test."""
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


class FakeLib:
    """Getters of contact_gb300 for problems (ire, icp) held in a dict."""

    def __init__(self, sols):
        self.sols = sols

    def getcontactforces(self, ire, icp):
        s = self.sols[(ire, icp)]
        return s["fn"], s["fx"], s["fy"], 0.0

    def gettractions(self, ire, icp):
        s = self.sols[(ire, icp)]
        return s["pn"], s["px"], s["py"]

    def getmaximumpressure(self, ire, icp):
        return float(self.sols[(ire, icp)]["pn"].max())

    def getelementdivision(self, ire, icp):
        return self.sols[(ire, icp)]["igs"]


def _sol(fn, fx, fy, pn, px, py, igs):
    return dict(fn=fn, fx=fx, fy=fy, pn=np.array(pn, float), px=np.array(px, float), py=np.array(py, float),
                igs=np.array(igs, np.int32))


def test_form_errors_and_summary():
    base = _sol(100.0, 30.0, 40.0, [1.0, 2.0, 0.0], [0.3, 0.6, 0.0], [0.0, 0.1, 0.0], [2, 2, 0])
    near = _sol(100.0 + 1e-7, 30.0 + 3e-8, 40.0 - 4e-8, [1.0, 2.0 + 2e-9, 0.0], [0.3, 0.6, 0.0],
                [0.0, 0.1 - 6e-9, 0.0], [2, 2, 0])
    # small tangential force: relative to 1e-3 mu Fn (mu 0.3, Fn 50), one element changes class
    small = _sol(50.0, 1e-4, 0.0, [4.0, 0.0], [0.0, 0.0], [0.0, 0.0], [2, 0])
    small2 = _sol(50.0, 1e-4 + 3e-10, 0.0, [4.0, 0.0], [0.0, 0.0], [0.0, 0.0], [3, 0])
    lib = FakeLib({(1, 1): near, (1, 2): base, (2, 1): small2, (2, 2): small})
    e = bench.form_errors(lib, [1, 2], 1, 2, [0.3, 0.3])
    assert abs(e["ft"][0] - math.hypot(3e-8, 4e-8) / 50.0) < 1e-15
    assert abs(e["ft"][1] - 3e-10 / (1e-3 * 0.3 * 50.0)) < 1e-16
    assert abs(e["fn"][0] - 1e-9) < 1e-15 and e["fn"][1] == 0.0
    assert abs(e["pmax"][0] - 2e-9 / 2.0) < 1e-15
    assert abs(e["tractions"][0] - 6e-9 / 2.0) < 1e-15          # largest |dp| of the three components
    assert list(e["eldiv"]) == [0, 1]
    s = bench.summarize_errors(e)
    assert s["eldiv"] == {"patches_differing": 1, "max_elements": 1}
    assert s["ft"]["above_1e-08"] == 1 and s["tractions"]["above_1e-08"] == 0
    assert s["fn"]["max"] == e["fn"].max()
