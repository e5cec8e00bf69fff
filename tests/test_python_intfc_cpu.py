"""The reference's own Python binding (python_intfc) drives this library.

python_intfc binds every entry point of CONTACT's library interface with ctypes when it is
imported, so a drop-in must export all of them, including those outside the solve path.
The test lays out the binding's expected tree in a temporary directory (the package next to
bin/contact_addon_linux64.so, here a link to this library) and calls setters and getters
through the binding's own wrapper functions in a child process.  No solve is run: that
needs a GPU.  The binding is the reference's source; where its tree is absent (the GPU
machine) the test is skipped.
"""
import json
import os
import subprocess
import sys

import pytest

import contact_gb300 as cg

REF = os.environ.get("CONTACT_REFERENCE", "/root/reference")

SCRIPT = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
import python_intfc as cntc
CNTC, ifcver, ierr0 = cntc.initlibrary()
ver, ierr1 = cntc.initialize(1, 3)
cntc.setmaterialparameters(1, 1, 0, [0.28, 0.28, 82031.25, 82031.25])
cntc.setfrictionmethod(1, 1, 0, [0.3, 0.3])
cntc.setnormalforce(1, 1, 1.0e5)
cntc.setcreepages(1, 1, 0.001, -0.0002, 0.0)
cntc.sethertzcontact(1, 1, -3, [51, 51, 6.0, 4.0, 1.1])
vx, vy, phi = cntc.getcreepages(1, 1)
mat = cntc.getparameters(1, 1, 2)
fric = cntc.getparameters(1, 1, 3)
npatch = cntc.getnumcontactpatches(1)
t = cntc.getmaximumtemperature(1, 1)
cntc.finalize(1)
def plain(v):
    return v.tolist() if hasattr(v, "tolist") else (list(v) if isinstance(v, tuple) else v)
print("RESULT " + json.dumps({"ierr": [ierr0, ierr1], "creep": [vx, vy, phi], "gg": plain(mat["gg"]),
                               "poiss": plain(mat["poiss"]), "ak": plain(mat["ak"]),
                               "fric": {k: plain(v) for k, v in fric.items()}, "npatch": plain(npatch),
                               "temp": plain(t)}))
"""


@pytest.fixture(scope="module")
def intfc_root(tmp_path_factory):
    src = os.path.join(REF, "python_intfc")
    if not os.path.isdir(src):
        pytest.skip("the reference's python_intfc is not present on this machine")
    cg.load()
    root = tmp_path_factory.mktemp("intfc")
    os.symlink(src, root / "python_intfc")
    (root / "bin").mkdir()
    os.symlink(cg.LIB_PATH, root / "bin" / "contact_addon_linux64.so")
    return str(root)


def test_reference_binding_loads_and_drives_library(intfc_root):
    env = dict(os.environ, LD_LIBRARY_PATH=os.environ.get("LD_LIBRARY_PATH", "") or os.path.dirname(cg.LIB_PATH),
               CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "-c", SCRIPT, intfc_root], capture_output=True, text=True, timeout=120,
                       env=env, cwd=intfc_root)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("RESULT ")]
    assert line, r.stdout[-2000:]
    res = json.loads(line[0][len("RESULT "):])
    assert res["ierr"] == [0, 0]
    assert res["creep"] == pytest.approx([0.001, -0.0002, 0.0])
    assert res["gg"] == pytest.approx(82031.25) and res["poiss"] == pytest.approx(0.28) and res["ak"] == 0.0
    assert res["npatch"] == 0
    assert res["fric"]["fstat"] == pytest.approx([0.3]) and res["fric"]["fkin"] == pytest.approx([0.3])
    assert res["temp"] == [0.0, 0.0]
