"""Device operator: the GB300 Mdot behind the C ABI, on torch tensors.

    op = DPStokes(StokesParams(...), n_particles)
    op.set_positions(X)          # [N,3] cuda tensor
    V, W = op.mdot(F, T)         # [N,3] cuda tensors (W is None without torques)

Tensors are passed by device pointer on torch's current CUDA stream; nothing
is copied through the host.  The arithmetic is selected by
StokesParams.precision: 'fp64' (every stage FP64; the drop-in for the
reference) or 'mixed' (FP32 spread / FFT / z transform / interpolation, FP64
per-wavenumber solves)."""
import ctypes
import math
from dataclasses import dataclass, asdict

import torch

from . import _lib


@dataclass
class StokesParams:
    """Explicit operator parameters (the fields of dpst_params).

    mode: 'nowall' | 'bottom' | 'slit' | 'periodic' (reference domType DP /
    DPBW / DPSC / TP).  z interval [zmin, zmax]; walls at zmin (bottom) and
    zmax (slit top); 'periodic': nz uniform points on the periodic [zmin, zmax).
    Kernels: w points per axis, ES beta (the reference's beta_hat * w) and
    alpha (physical half width).  reg_kernel: torques and angular velocities
    with the regular ES kernel of (w_d, beta_d, alpha_d) and spectral curls
    (the reference's useRegKernel=True) instead of the derivative kernels.
    solve: arithmetic of the per-wavenumber solve, 'default' (FP64 for the
    FP64 operator, double-float for the mixed one), 'fp64' or 'df64'."""
    mode: str
    nx: int
    ny: int
    nz: int
    Lx: float
    Ly: float
    zmin: float
    zmax: float
    viscosity: float
    w: int
    beta: float
    alpha: float
    has_torque: bool = False
    w_d: int = 6
    beta_d: float = 13.296
    alpha_d: float = 3.0
    precision: str = "fp64"
    reg_kernel: bool = False
    solve: str = "default"

    def to_c(self):
        return _lib.DpstParams(
            _lib.MODE[self.mode], int(self.nx), int(self.ny), int(self.nz), float(self.Lx),
            float(self.Ly), float(self.zmin), float(self.zmax), float(self.viscosity), int(self.w),
            float(self.beta), float(self.alpha), int(bool(self.has_torque)), int(self.w_d),
            float(self.beta_d), float(self.alpha_d), _lib.PREC[self.precision], int(bool(self.reg_kernel)),
            _lib.SOLVE[self.solve])

    def as_dict(self):
        return asdict(self)

    @staticmethod
    def kernel_alpha(radius, w, hx):
        """alpha of the reference's UseCbeta convention: c = R/(w hx),
        alpha = R/(2c) (GridAndKernelConfig.py:328-329, ParticleList.cpp:229)."""
        c = radius / (w * hx)
        return radius / (2 * c)

    @classmethod
    def from_workload(cls, wl, precision="fp64"):
        """Parameters of a doublyperiodicstokes_gb300.workloads.Workload."""
        mode = {"DP": "nowall", "DPBW": "bottom", "DPSC": "slit", "TP": "periodic"}[wl.domType]
        hx = wl.Lx / wl.nx
        return cls(mode=mode, nx=wl.nx, ny=wl.ny, nz=wl.nz, Lx=wl.Lx, Ly=wl.Ly, zmin=wl.z0,
                   zmax=wl.z0 + wl.Lz, viscosity=wl.eta, w=wl.wm, beta=wl.betam_hat * wl.wm,
                   alpha=cls.kernel_alpha(wl.radius, wl.wm, hx), has_torque=wl.has_torque,
                   w_d=wl.wd, beta_d=wl.betad_hat * wl.wd,
                   alpha_d=cls.kernel_alpha(wl.radius, wl.wd, hx), precision=precision,
                   reg_kernel=wl.reg_kernel)


def _dtype_code(t):
    if t.dtype == torch.float64:
        return _lib.F64
    if t.dtype == torch.float32:
        return _lib.F32
    raise TypeError("particle arrays must be float32 or float64")


def _stream_ptr(device):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


class DPStokes:
    """One operator instance (owns the device state of dpst_create)."""

    def __init__(self, params: StokesParams, n_particles: int, device=None):
        if not torch.cuda.is_available():
            raise RuntimeError("DPStokes needs a CUDA device")
        self.L = _lib.lib()
        self.params = params
        self.N = int(n_particles)
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None
                                   else torch.device(device).index or 0)
        self._h = ctypes.c_void_p()
        cp = params.to_c()
        _lib.check(self.L.dpst_create(ctypes.byref(cp), self.N, self.device.index,
                                      ctypes.byref(self._h)))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            torch.cuda.synchronize(self.device)
            _lib.check(self.L.dpst_destroy(self._h))
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        inf = _lib.DpstInfo()
        _lib.check(self.L.dpst_get_info(self._h, ctypes.byref(inf)))
        return {f: getattr(inf, f) for f, _ in inf._fields_}

    def _check_arr(self, t, name):
        if t.device != self.device:
            raise ValueError("%s must be on %s" % (name, self.device))
        if t.numel() != 3 * self.N:
            raise ValueError("%s must hold 3*N = %d values" % (name, 3 * self.N))
        return t.contiguous()

    def set_positions(self, X):
        X = self._check_arr(X, "positions")
        self._X = X
        _lib.check(self.L.dpst_set_positions(self._h, ctypes.c_void_p(X.data_ptr()),
                                             _dtype_code(X), _stream_ptr(self.device)))

    def mdot(self, F, T=None, out=None):
        """(V, W) = M (F, T).  W is None when the operator has no torques."""
        F = self._check_arr(F, "forces")
        dt = F.dtype
        if T is not None:
            if not self.params.has_torque:
                raise ValueError("operator was created without torques")
            T = self._check_arr(T, "torques")
            if T.dtype != dt:
                raise TypeError("forces and torques must have the same dtype")
        V = torch.empty_like(F) if out is None else out[0]
        W = None
        if self.params.has_torque:
            W = torch.empty_like(F) if out is None else out[1]
        _lib.check(self.L.dpst_mdot(self._h, ctypes.c_void_p(F.data_ptr()),
                                    ctypes.c_void_p(T.data_ptr() if T is not None else 0),
                                    ctypes.c_void_p(V.data_ptr()),
                                    ctypes.c_void_p(W.data_ptr() if W is not None else 0),
                                    _dtype_code(F), _stream_ptr(self.device)))
        return V, W

    def mdot_multi(self, F, T=None, out=None):
        """(V, W) = M (F, T) for K columns at once: F, T of shape (K, N, 3) (or
        (K, 3N)); the result has the same shape.  W is None when the operator
        has no torques.  Column k equals mdot(F[k], T[k])."""
        if F.dim() < 2:
            raise ValueError("forces must have a leading column dimension K")
        K = F.shape[0]
        if F.device != self.device:
            raise ValueError("forces must be on %s" % self.device)
        if F.numel() != 3 * self.N * K:
            raise ValueError("forces must hold K*3*N = %d values" % (3 * self.N * K))
        F = F.contiguous()
        dt = F.dtype
        if T is not None:
            if not self.params.has_torque:
                raise ValueError("operator was created without torques")
            if T.device != self.device or T.numel() != F.numel():
                raise ValueError("torques must match the forces' shape and device")
            if T.dtype != dt:
                raise TypeError("forces and torques must have the same dtype")
            T = T.contiguous()
        V = torch.empty_like(F) if out is None else out[0]
        W = None
        if self.params.has_torque:
            W = torch.empty_like(F) if out is None else out[1]
        _lib.check(self.L.dpst_mdot_multi(self._h, K, ctypes.c_void_p(F.data_ptr()),
                                          ctypes.c_void_p(T.data_ptr() if T is not None else 0),
                                          ctypes.c_void_p(V.data_ptr()),
                                          ctypes.c_void_p(W.data_ptr() if W is not None else 0),
                                          _dtype_code(F), _stream_ptr(self.device)))
        return V, W

    # ---- diagnostics -------------------------------------------------------
    STAGES = ("spread", "fft_fwd", "ztrans_fwd", "solve", "ztrans_inv", "fft_inv", "interp", "total")

    def _grid_buffer(self):
        dt = torch.float64 if self.params.precision == "fp64" else torch.float32
        p = self.params
        return torch.empty((3, p.nz, p.ny, p.nx), dtype=dt, device=self.device)

    def spread_grid(self, F, T=None):
        """Spread grid (forces + torque curl, boundary fold applied),
        [3][nz][ny][nx] with z index 0 at zmax."""
        F = self._check_arr(F, "forces")
        if T is not None:
            T = self._check_arr(T, "torques")
        out = self._grid_buffer()
        _lib.check(self.L.dpst_spread_grid(self._h, ctypes.c_void_p(F.data_ptr()),
                                           ctypes.c_void_p(T.data_ptr() if T is not None else 0),
                                           _dtype_code(F), ctypes.c_void_p(out.data_ptr()),
                                           _stream_ptr(self.device)))
        return out

    def velocity_grid(self):
        """Fluid velocity on the grid from the last mdot, [3][nz][ny][nx]."""
        out = self._grid_buffer()
        _lib.check(self.L.dpst_velocity_grid(self._h, ctypes.c_void_p(out.data_ptr()),
                                             _stream_ptr(self.device)))
        return out

    def mdot_timed(self, F, T=None):
        """mdot plus per-stage device milliseconds (dict keyed by STAGES)."""
        F = self._check_arr(F, "forces")
        if T is not None:
            T = self._check_arr(T, "torques")
        V = torch.empty_like(F)
        W = torch.empty_like(F) if self.params.has_torque else None
        ms = (ctypes.c_float * 8)()
        _lib.check(self.L.dpst_mdot_timed(self._h, ctypes.c_void_p(F.data_ptr()),
                                          ctypes.c_void_p(T.data_ptr() if T is not None else 0),
                                          ctypes.c_void_p(V.data_ptr()),
                                          ctypes.c_void_p(W.data_ptr() if W is not None else 0),
                                          _dtype_code(F), _stream_ptr(self.device), ms))
        return V, W, dict(zip(self.STAGES, list(ms)))

    # ---- backward pass -----------------------------------------------------
    def forward_serial(self):
        """Serial of the last single-column mdot whose velocity grid the
        handle still holds (0 if none); pass it to mdot_backward."""
        v = ctypes.c_uint64()
        _lib.check(self.L.dpst_forward_serial(self._h, ctypes.byref(v)))
        return int(v.value)

    def mdot_backward(self, F, T, gV, gW=None, need_F=True, need_T=False, need_X=True, forward_serial=0):
        """Vector-Jacobian product of mdot at the current positions.

        For l = <gV, V> + <gW, W> with (V, W) = mdot(F, T), returns
        (dl/dF, dl/dT, dl/dX), each [N, 3] or None when not requested.  T is
        the forward call's torques (None if it had none); F is needed only for
        dl/dX.  The forward's velocity grid is recomputed, unless
        forward_serial is forward_serial() read right after that mdot and the
        handle still holds its grid (then F, T must be unchanged since)."""
        gV = self._check_arr(gV, "gV")
        dt = gV.dtype
        args = {}
        for name, t in (("F", F), ("T", T), ("gW", gW)):
            if t is not None:
                t = self._check_arr(t, name)
                if t.dtype != dt:
                    raise TypeError("%s must have the dtype of gV" % name)
            args[name] = t
        if gW is not None and not self.params.has_torque:
            raise ValueError("gW given but the operator was created without torques")
        gF = torch.empty_like(gV) if need_F else None
        gT = torch.empty_like(gV) if (need_T and T is not None) else None
        gX = torch.empty_like(gV) if need_X else None

        def ptr(t):
            return ctypes.c_void_p(t.data_ptr() if t is not None else 0)

        reused = ctypes.c_int(0)
        _lib.check(self.L.dpst_mdot_backward_saved(self._h, int(forward_serial), ptr(args["F"]), ptr(args["T"]),
                                                   ptr(gV), ptr(args["gW"]), ptr(gF), ptr(gT), ptr(gX),
                                                   _dtype_code(gV), _stream_ptr(self.device),
                                                   ctypes.byref(reused)))
        self.last_backward_reused = bool(reused.value)
        return gF, gT, gX


class DPStokesBatch:
    """Many independent systems in one pipeline (dpst_batched_*): uneven
    particle counts and box sizes; shared nz, z interval, geometry,
    viscosity, precision and torque flag.  Arrays are the systems' [N_s, 3]
    arrays concatenated in the order of `params`."""

    def __init__(self, params, n_particles, device=None):
        if not torch.cuda.is_available():
            raise RuntimeError("DPStokesBatch needs a CUDA device")
        if len(params) != len(n_particles) or not params:
            raise ValueError("one particle count per system, at least one system")
        self.L = _lib.lib()
        self.params = list(params)
        self.n = [int(v) for v in n_particles]
        self.N = sum(self.n)
        self.has_torque = bool(params[0].has_torque)
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None
                                   else torch.device(device).index or 0)
        arr = (_lib.DpstParams * len(params))(*[p.to_c() for p in params])
        cnt = (ctypes.c_int64 * len(params))(*self.n)
        self._h = ctypes.c_void_p()
        _lib.check(self.L.dpst_batched_create(arr, cnt, len(params), self.device.index,
                                              ctypes.byref(self._h)))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            torch.cuda.synchronize(self.device)
            _lib.check(self.L.dpst_batched_destroy(self._h))
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        inf = _lib.DpstBatchInfo()
        _lib.check(self.L.dpst_batched_get_info(self._h, ctypes.byref(inf)))
        return {f: getattr(inf, f) for f, _ in inf._fields_}

    def _check_arr(self, t, name):
        if t.device != self.device:
            raise ValueError("%s must be on %s" % (name, self.device))
        if t.numel() != 3 * self.N:
            raise ValueError("%s must hold 3*sum(N) = %d values" % (name, 3 * self.N))
        return t.contiguous()

    def set_positions(self, X):
        X = self._check_arr(X, "positions")
        self._X = X
        _lib.check(self.L.dpst_batched_set_positions(self._h, ctypes.c_void_p(X.data_ptr()),
                                                     _dtype_code(X), _stream_ptr(self.device)))

    def mdot(self, F, T=None, out=None):
        """(V, W) for every system, concatenated; W is None without torques."""
        F = self._check_arr(F, "forces")
        if T is not None:
            if not self.has_torque:
                raise ValueError("batch was created without torques")
            T = self._check_arr(T, "torques")
        V = torch.empty_like(F) if out is None else out[0]
        W = None
        if self.has_torque:
            W = torch.empty_like(F) if out is None else out[1]
        _lib.check(self.L.dpst_batched_mdot(self._h, ctypes.c_void_p(F.data_ptr()),
                                            ctypes.c_void_p(T.data_ptr() if T is not None else 0),
                                            ctypes.c_void_p(V.data_ptr()),
                                            ctypes.c_void_p(W.data_ptr() if W is not None else 0),
                                            _dtype_code(F), _stream_ptr(self.device)))
        return V, W

    def split(self, A):
        """Split a concatenated [sum N, 3] array into the systems' arrays."""
        return list(torch.split(A.reshape(-1, 3), self.n))
