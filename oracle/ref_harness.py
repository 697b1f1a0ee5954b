"""Runs the UNMODIFIED reference CPU path (source/cpu/python/FCM.py driving the
C++ libraries built by oracle/Makefile.ref) on explicit grid/kernel
parameters, in a child process, and returns its outputs.

Test infrastructure only (golden-fixture generation and oracle pinning).  It
needs the reference sources (REF_ROOT) and oracle/_ref/*.so built on this
machine; nothing in the product or in the GPU tests imports it.

How the reference is driven (no reference source is copied):
  * FCM(radP, kernTypes, domType, has_torque), SetUnitCell, Initialize,
    SetPositions, Mdot are the reference's own methods (FCM.py:80-441).
  * FCM.Initialize normally picks (h, beta, Nz, z0) from its polynomial fits
    (GridAndKernelConfig.py:4-427).  The explicit-parameter configurations of
    this project are injected by replacing the two configure_* names inside the
    FCM module namespace with functions that return the requested values; the
    rest of Initialize (BCs, grids, Stokes precompute, transforms) runs as is.
  * numpy 2 removed np.int / np.complex that the reference uses
    (GridAndKernelConfig.py:74, Chebyshev.py:60, FCM.py:322); they are aliased
    back before import.
  * `config.num_threads` (source/cpu/python/config.py) is provided by a
    generated module placed first on sys.path.
  * Stage outputs (spread grid, forward transform, solver output, backward
    transform) are recorded by wrapping Transformer/Stokes methods.
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("DPST_REFERENCE_ROOT", "")
REF_LIB = os.path.join(HERE, "_ref")


def reference_available():
    return (os.path.isdir(os.path.join(REF_ROOT, "source", "cpu", "python"))
            and os.path.exists(os.path.join(REF_LIB, "libdpTools.so")))


def _child_main(cfg_path, in_path, out_path):
    import numpy as np  # noqa: F811
    np.int = int
    np.complex = complex
    cfg = json.load(open(cfg_path))
    data = np.load(in_path)
    import Solvers
    orig_ints = Solvers.precomputeInts

    def precomputeInts(Nz, H):
        # Chebyshev.py:96-117 returns (1, Nz) row vectors; numpy 2 no longer
        # accepts `Cp[1] += 0.5 * pints @ Ch` (Solvers.py:680,701) with a
        # 1-element array, so the same values are handed back flattened.
        p, uv = orig_ints(Nz, H)
        return np.ravel(p), np.ravel(uv)

    Solvers.precomputeInts = precomputeInts
    import FCM as fcm_mod
    nP = int(cfg["nP"])
    Nx, Ny, Nz = int(cfg["Nx"]), int(cfg["Ny"]), int(cfg["Nz"])
    Lx, Ly, Lz, z0 = float(cfg["Lx"]), float(cfg["Ly"]), float(cfg["Lz"]), float(cfg["z0"])
    hx, hy = Lx / Nx, Ly / Ny
    R = float(cfg.get("radius", 1.0))
    wm = np.full(nP, int(cfg["wm"]), dtype=np.ushort)
    has_torque = bool(cfg["has_torque"])
    wd = np.full(nP, int(cfg["wd"]), dtype=np.ushort) if has_torque else [0]
    betam = np.full(nP, float(cfg["betam_hat"]))
    betad = np.full(nP, float(cfg["betad_hat"])) if has_torque else [0]
    cbm = R / (wm * hx)
    cbd = R / (wd * hx) if has_torque else 0

    def cfg_xy(*args, **kw):
        return (Lx, Ly, hx, hy, Nx, Ny, wm, wd, cbm, cbd, betam, betad)

    def cfg_z(*args, **kw):
        # the triply periodic grid is uniform in z with hz = Lz / Nz
        # (GridAndKernelConfig.py:380-393); the Chebyshev domains have hz = 0
        return (Lz, Lz / Nz if cfg["domType"] == "TP" else 0.0, Nz, z0)

    fcm_mod.configure_grid_and_kernels_xy = cfg_xy
    fcm_mod.configure_grid_and_kernels_z = cfg_z

    stages = {}
    want_stages = bool(cfg.get("stages", False))
    if want_stages:
        Tr = fcm_mod.Transformer
        orig_f, orig_b = Tr.Ftransform, Tr.Btransform

        def Ftransform(self, in_real):
            stages.setdefault("spread_grid", np.array(in_real, copy=True))
            orig_f(self, in_real)
            stages.setdefault("f_hat_r", np.array(self.out_real, copy=True))
            stages.setdefault("f_hat_i", np.array(self.out_imag, copy=True))

        def Btransform(self, in_real, in_imag):
            stages.setdefault("u_hat_r", np.array(in_real, copy=True).ravel())
            stages.setdefault("u_hat_i", np.array(in_imag, copy=True).ravel())
            orig_b(self, in_real, in_imag)
            stages.setdefault("u_grid", np.array(self.out_real, copy=True))

        Tr.Ftransform, Tr.Btransform = Ftransform, Btransform

    radP = np.full(nP, R)
    kern = np.zeros(nP, dtype=int)
    dom = cfg["domType"]
    solver = fcm_mod.FCM(radP, kern, dom, has_torque)
    solver.SetUnitCell([0.0, Lx], [0.0, Ly], [z0, z0 + Lz])
    solver.Initialize(float(cfg["eta"]), 0, useRegKernel=bool(cfg.get("reg_kernel", False)))
    X = np.array(data["X"], dtype=np.float64).ravel().copy()
    F = np.array(data["F"], dtype=np.float64).ravel().copy()
    T = np.array(data["T"], dtype=np.float64).ravel().copy() if has_torque else np.empty(0)
    solver.SetPositions(X)
    V, W = solver.Mdot(F, T)
    out = {"V": np.array(V, copy=True)}
    if has_torque:
        out["W"] = np.array(W, copy=True)
    n_calls = int(cfg.get("repeat", 1))
    for _ in range(n_calls - 1):  # repeated Mdot on the same positions
        V2, W2 = solver.Mdot(F, T)
        out["V_repeat"] = np.array(V2, copy=True)
    out.update(stages)
    np.savez(out_path, **out)


def run_reference(cfg, X, F, T=None, stages=False, repeat=1, threads=4, timeout=3600):
    """Run the reference Mdot in a child process.

    cfg keys: domType ('DP'|'DPBW'|'DPSC'|'TP'), Nx, Ny, Nz, Lx, Ly, Lz, z0, eta,
    wm, betam_hat, has_torque, wd, betad_hat, radius, reg_kernel (FCM's useRegKernel).  Returns a dict of numpy
    arrays (V, W and, with stages=True, the intermediate grids)."""
    if not reference_available():
        raise RuntimeError("reference sources or oracle/_ref libraries are missing")
    X = np.asarray(X, dtype=np.float64)
    cfg = dict(cfg)
    cfg["nP"] = X.size // 3
    cfg["stages"] = bool(stages)
    cfg["repeat"] = int(repeat)
    with tempfile.TemporaryDirectory() as td:
        cfg_path = os.path.join(td, "cfg.json")
        in_path = os.path.join(td, "in.npz")
        out_path = os.path.join(td, "out.npz")
        json.dump(cfg, open(cfg_path, "w"))
        T = np.zeros_like(X) if T is None else T
        np.savez(in_path, X=X, F=np.asarray(F, dtype=np.float64), T=np.asarray(T, dtype=np.float64))
        shim = os.path.join(td, "shimcfg")
        os.makedirs(shim)
        with open(os.path.join(shim, "config.py"), "w") as f:
            f.write("num_threads=%d\n" % threads)
        env = dict(os.environ)
        env["LD_LIBRARY_PATH"] = REF_LIB + os.pathsep + env.get("LD_LIBRARY_PATH", "")
        env["PYTHONPATH"] = os.pathsep.join(
            [shim, os.path.join(REF_ROOT, "source", "cpu", "python"), HERE])
        env["FCM_CPUCONFIG_LAUNCHED"] = "1"
        env["OMP_NUM_THREADS"] = str(threads)
        code = ("import sys; sys.argv=['x']; import ref_harness as h; "
                "h._child_main(%r, %r, %r)" % (cfg_path, in_path, out_path))
        r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True,
                           text=True, timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError("reference run failed:\n" + r.stdout[-3000:] + r.stderr[-3000:])
        res = dict(np.load(out_path))
    return res
