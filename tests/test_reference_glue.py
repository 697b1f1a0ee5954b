"""The reference's own pybind11 module source (uammd_python.cpp) built
unchanged against doublyperiodicstokes_gb300/glue/dpstokes_glue_gb300.cpp
(DPStokesGlue on the C ABI), in both of its precisions.  Needs the
reference's source tree (DPST_REFERENCE_ROOT) and pybind11; skipped
otherwise.  Without a GPU, initialize() must raise RuntimeError the way the
reference module reports errors; with one, a small Mdot runs and is checked
against the oracle."""
import os
import subprocess
import sys
import sysconfig

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("DPST_REFERENCE_ROOT", "")
WRAP = os.path.join(REF, "source", "gpu", "python_wrapper")
LIBDIR = os.path.join(ROOT, "doublyperiodicstokes_gb300", "lib")

CHECK = r"""
import sys
import numpy as np
sys.path.insert(0, sys.argv[1])
sys.path.insert(0, sys.argv[2])
import uammd
import dpstokes_oracle as O
from doublyperiodicstokes_gb300 import workloads as W
print(uammd.getPrecision())
w = W.SMALL_BY_NAME["s_dpbw_f_top"]
X, F, _ = W.make_inputs(w)
hx = w.Lx / w.nx
c = w.radius / (w.wm * hx)
p = uammd.StokesParameters(viscosity=w.eta, Lx=w.Lx, Ly=w.Ly, zmin=0, zmax=w.Lz, w=w.wm, w_d=0,
                           alpha=w.radius / (2 * c * hx), alpha_d=0, beta=w.betam_hat * w.wm,
                           beta_d=0, nx=w.nx, ny=w.ny, nz=w.nz, mode="bottom")
s = uammd.DPStokes()
try:
    s.initialize(p, w.N)
except RuntimeError as e:
    print("RuntimeError", e)
    sys.exit(0)
real = np.float64 if uammd.getPrecision() == "double" else np.float32
MF = np.zeros(3 * w.N, dtype=real)
s.setPositions(real(X.ravel()))
s.Mdot(forces=real(F.ravel()), velocities=MF)
Vo, _ = O.mdot(O.Params(**w.oracle_params()), X, F)
err = np.linalg.norm(MF - Vo) / np.linalg.norm(Vo)
print("relerr", err)
sys.exit(0 if err < (1e-10 if real == np.float64 else 1e-5) else 1)
"""


def _build(tmp, double):
    pybind11 = pytest.importorskip("pybind11")
    out = os.path.join(tmp, "p%d" % double)
    os.makedirs(out, exist_ok=True)
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    cmd = ["g++", "-O1", "-std=c++14", "-shared", "-fPIC", "-I" + WRAP, "-I" + os.path.join(ROOT, "include"),
           "-I" + pybind11.get_include(), "-I" + sysconfig.get_paths()["include"],
           os.path.join(WRAP, "uammd_python.cpp"),
           os.path.join(ROOT, "doublyperiodicstokes_gb300", "glue", "dpstokes_glue_gb300.cpp"),
           "-L" + LIBDIR, "-ldpstokes_gb300", "-Wl,-rpath," + LIBDIR, "-o", os.path.join(out, "uammd" + ext)]
    if double:
        cmd.insert(5, "-DDOUBLE_PRECISION")
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


@pytest.mark.skipif(not os.path.isfile(os.path.join(WRAP, "uammd_python.cpp")),
                    reason="reference source tree not available")
@pytest.mark.parametrize("double", [0, 1])
def test_reference_module_builds_and_runs_on_glue(tmp_path, double):
    if not os.path.isfile(os.path.join(LIBDIR, "libdpstokes_gb300.so")):
        pytest.skip("library not built")
    out = _build(str(tmp_path), double)
    r = subprocess.run([sys.executable, "-c", CHECK, out, os.path.join(ROOT, "oracle")], capture_output=True,
                       text=True, cwd=ROOT, env=dict(os.environ, PYTHONPATH=ROOT))
    print(r.stdout, r.stderr[-2000:])
    assert r.returncode == 0
    lines = r.stdout.split("\n")
    assert lines[0] == ("double" if double else "single")
    assert lines[1].startswith("RuntimeError") or lines[1].startswith("relerr")
