"""A C host (tests/c_host/cntc_host.c) compiled with gcc against include/contact_addon.h and
linked with the library: the header is valid C and the symbols resolve at link time.  On
CPU the host runs its set-up and getters; the GPU test runs cntc_calculate through the pure
C-ABI and compares with the oracle."""
import os
import subprocess

import numpy as np
import pytest

import contact_gb300 as cg
import cases as C

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def host_exe(tmp_path_factory):
    cg.load()
    exe = str(tmp_path_factory.mktemp("chost") / "cntc_host")
    libdir = os.path.dirname(cg.LIB_PATH)
    cmd = ["gcc", "-std=c99", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(HERE, "c_host", "cntc_host.c"), "-o", exe, "-L", libdir, "-lcontact_addon",
           "-Wl,-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_host_setup_and_getters(host_exe):
    r = subprocess.run([host_exe], capture_output=True, text=True, timeout=60,
                       env=dict(os.environ, CUDA_VISIBLE_DEVICES=""))
    assert r.returncode == 0, r.stdout + r.stderr
    assert "setup tang 3 norm 1 creep 0.001 0 0" in r.stdout


@pytest.mark.gpu
def test_c_host_solve_matches_oracle(host_exe, oracle):
    r = subprocess.run([host_exe, "solve", "21"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("solve ")][0].split()
    v = dict(zip(line[1::2], line[2::2]))
    o = C.oracle_solve(C.config0(gausei=5, eps=1e-10, mx=21, my=21))
    assert int(v["ierror"]) == o["ierror"] == 0
    for k in ("fn", "fx", "fy"):
        assert abs(float(v[k]) - o[k]) <= 1e-10 * max(abs(o[k]), 1e-3 * 0.3 * o["fn"]), k
    assert abs(float(v["pmax"]) - np.abs(o["pn"]).max()) <= 1e-8 * np.abs(o["pn"]).max()
    assert (int(v["nadh"]), int(v["nslip"])) == (o["nadh"], o["nslip"])
