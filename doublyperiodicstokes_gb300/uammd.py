"""Drop-in replacement for the reference's GPU Python module `uammd`.

The reference's joint wrapper FCMJoint(device='gpu')
(python_interface/common_interface_wrapper.py:28-30, 76-101, 112-132) calls
exactly this surface of the pybind11 module built from
source/gpu/python_wrapper/uammd_python.cpp:59-129:

    uammd.getPrecision()                     -> 'single' | 'double'
    uammd.StokesParameters(viscosity, Lx, Ly, zmin, zmax, w, w_d, alpha,
                           alpha_d, beta, beta_d, nx, ny, nz, mode)
    uammd.DPStokes().initialize(par, N) / .setPositions(pos)
        / .Mdot(forces, torques, velocities, angularVelocities) / .clear()

Importing this module as `uammd` (put this package's directory first on
sys.path, or alias it in sys.modules) makes that wrapper run
on libdpstokes_gb300.so through its host-array C entry points, with host
NumPy arrays in and out exactly as the reference glue copies them
(uammd_wrapper.cu:136-170).  No torch is needed.

Parameter meaning (the UAMMD sources are not shipped with the reference, so
this follows how FCMJoint fills the parameters so that its GPU path
reproduces its CPU path):
  * beta, beta_d: the ES beta (FCMJoint passes beta_hat * w);
  * alpha, alpha_d: kernel half width in grid units (FCMJoint passes
    R/(2 c h) = w/2); the operator uses alpha * Lx/nx;
  * zmin, zmax: the Chebyshev interval, taken at face value; walls at zmin
    ('bottom', 'slit') and zmax ('slit');
  * mode: 'nowall' | 'bottom' | 'slit' | 'periodic'; an unknown string
    means 'nowall' (uammd_wrapper.cu:55-66); 'periodic' runs the triply
    periodic operator on nz uniform points of [zmin, zmax) (the reference
    module hands it to UAMMD's FCM, uammd_wrapper.cu:122-126);
  * torques: the operator is created with the dipole kernel when w_d, beta_d
    and alpha_d are all positive; an Mdot whose torque array holds fewer than
    3N values runs without torques (uammd_python.cpp:51-53).
Errors surface as RuntimeError, like the pybind11 module's std::runtime_error
(uammd_wrapper.cu:106, 208-211).
Precision: FP64 by default ('double'); set DPSTOKES_GB300_PRECISION=single to
get the mixed-precision operator with float32 arrays.
"""
import ctypes
import os

import numpy as np

from . import _lib


def getPrecision():
    """'double' (FP64 operator) unless DPSTOKES_GB300_PRECISION=single."""
    return "single" if os.environ.get("DPSTOKES_GB300_PRECISION", "double") == "single" else "double"


def _real():
    return np.float32 if getPrecision() == "single" else np.float64


class StokesParameters:
    """Same fields and defaults as uammd.StokesParameters (uammd_python.cpp:74-102)."""

    def __init__(self, viscosity=1.0, Lx=0.0, Ly=0.0, zmin=0.0, zmax=0.0, w=1.0, w_d=1.0,
                 alpha=-1.0, alpha_d=-1.0, beta=-1.0, beta_d=-1.0, nx=-1, ny=-1, nz=-1,
                 mode="none"):
        self.viscosity = viscosity
        self.Lx, self.Ly, self.zmin, self.zmax = Lx, Ly, zmin, zmax
        self.w, self.w_d = w, w_d
        self.alpha, self.alpha_d = alpha, alpha_d
        self.beta, self.beta_d = beta, beta_d
        self.nx, self.ny, self.nz = nx, ny, nz
        self.mode = mode

    def __str__(self):
        return ("viscosity = %f\nbox (L = %f,%f,%f:%f )\nNx = %d\nNy = %d\nnz = %d\nmode = %s\n"
                % (self.viscosity, self.Lx, self.Ly, self.zmin, self.zmax, self.nx, self.ny,
                   self.nz, self.mode))


_MODES = {"nowall": 0, "bottom": 1, "slit": 2, "periodic": 3}


class DPStokes:
    """uammd.DPStokes: initialize / setPositions / Mdot / clear."""

    def __init__(self):
        self._h = None
        self.N = 0

    def initialize(self, Parameters, numberParticles):
        self.clear()
        par = Parameters
        if par.nx <= 0 or par.ny <= 0 or par.nz <= 0:
            raise RuntimeError("nx, ny and nz must be given")
        h = par.Lx / par.nx
        torque = par.w_d > 0 and par.alpha_d > 0 and par.beta_d > 0
        c = _lib.DpstParams(
            _MODES.get(par.mode, 0), int(par.nx), int(par.ny), int(par.nz), float(par.Lx),
            float(par.Ly), float(par.zmin), float(par.zmax), float(par.viscosity), int(round(par.w)),
            float(par.beta), float(par.alpha) * h, int(torque),
            int(round(par.w_d)) if torque else 6, float(par.beta_d) if torque else 1.0,
            float(par.alpha_d) * h if torque else 1.0,
            _lib.PREC["mixed" if getPrecision() == "single" else "fp64"])
        L = _lib.lib()
        hd = ctypes.c_void_p()
        self._check(L.dpst_create(ctypes.byref(c), int(numberParticles), int(os.environ.get(
            "DPSTOKES_GB300_DEVICE", "0")), ctypes.byref(hd)))
        self._h = hd
        self.N = int(numberParticles)
        self._torque = torque

    def clear(self):
        if self._h is not None and self._h.value:
            _lib.lib().dpst_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.clear()
        except Exception:
            pass

    def _check(self, code):
        if code != 0:
            raise RuntimeError(_lib.lib().dpst_last_error().decode())

    def _ready(self):
        if self._h is None:
            raise RuntimeError("DPStokes is not initialized. Call Initialize first")

    def _arr(self, a):
        a = np.ascontiguousarray(a, dtype=_real())
        return a, a.ctypes.data_as(ctypes.c_void_p)

    def setPositions(self, positions):
        self._ready()
        pos, p = self._arr(positions)
        if pos.size != 3 * self.N:
            raise RuntimeError("positions must hold 3*numberParticles values")
        code = _lib.F32 if pos.dtype == np.float32 else _lib.F64
        self._check(_lib.lib().dpst_set_positions_host(self._h, p, code, None))

    def Mdot(self, forces, torques=np.empty(0), velocities=None, angularVelocities=np.empty(0)):
        """Writes M F (+ M T) into `velocities` and, with torques, the angular
        velocities into `angularVelocities` (both modified in place)."""
        self._ready()
        F, fp = self._arr(forces)
        if velocities is None or velocities.size < 3 * self.N:
            raise RuntimeError("velocities must hold 3*numberParticles values")
        if velocities.dtype != F.dtype or not velocities.flags.c_contiguous:
            raise RuntimeError("velocities must be a contiguous array of the library precision")
        use_t = torques is not None and np.size(torques) >= 3 * self.N and self._torque
        T, tp = self._arr(torques) if use_t else (None, None)
        want_w = use_t and angularVelocities is not None and angularVelocities.size >= 3 * self.N
        wp = angularVelocities.ctypes.data_as(ctypes.c_void_p) if want_w else None
        if want_w and (angularVelocities.dtype != F.dtype or not angularVelocities.flags.c_contiguous):
            raise RuntimeError("angularVelocities must be a contiguous array of the library precision")
        code = _lib.F32 if F.dtype == np.float32 else _lib.F64
        self._check(_lib.lib().dpst_mdot_host(self._h, fp, tp,
                                               velocities.ctypes.data_as(ctypes.c_void_p), wp,
                                               code, None))
