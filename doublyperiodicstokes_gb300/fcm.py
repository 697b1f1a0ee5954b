"""FCMJoint with device='gb300': the reference's joint wrapper interface
(python_interface/common_interface_wrapper.py:21-133) on this operator, with
the CPU path's conventions (FCM.py): positions in [xmin,xmax] x [ymin,ymax] x
[zmin,zmax], the Chebyshev interval starting at z0, BCs per domain type.

The reference chooses the grid and kernel (h, beta, Nz, z0) from polynomial
fits in GridAndKernelConfig.py; those tables are not part of this package, so
Initialize takes the grid explicitly (nx, ny, nz, kernel widths and
dimensionless betas, z0).  Everything else -- argument names, order, array
formats ([3N] interleaved xyz), return values -- follows FCMJoint.
"""
import numpy as np
import torch

from .operator import DPStokes, StokesParams

_MODE = {"DP": "nowall", "DPBW": "bottom", "DPSC": "slit"}


class FCMJoint:
    def __init__(self, device="gb300"):
        if device != "gb300":
            raise ValueError("this FCMJoint runs the GB300 operator only (device='gb300')")
        self.device = device
        self.precision = np.float64
        self.op = None

    def Initialize(self, numberParticles, hydrodynamicRadius, viscosity, domType, has_torque,
                   xmax, ymax, zmin, zmax, xmin=0, ymin=0, kernType=0, optInd=0, ref=False, *,
                   nx, ny, nz, w=6, beta_hat=None, w_d=6, beta_d_hat=2.2160, z0=None,
                   precision="fp64"):
        """Explicit-grid version of FCMJoint.Initialize.  beta_hat defaults to
        the reference's w=6 values (1.714 without torques, 1.3267 with)."""
        if domType not in _MODE:
            raise ValueError("domType must be DP, DPBW or DPSC (TP is not provided)")
        self.Clean()
        self.has_torque = bool(has_torque)
        self.N = int(numberParticles)
        self.xmin, self.ymin = xmin, ymin
        Lx, Ly = xmax - xmin, ymax - ymin
        self.z0 = zmin if z0 is None else z0
        if beta_hat is None:
            beta_hat = 1.3267 if has_torque else 1.714
        hx = Lx / nx
        a = StokesParams.kernel_alpha(hydrodynamicRadius, w, hx)
        ad = StokesParams.kernel_alpha(hydrodynamicRadius, w_d, hx)
        Lz = zmax - self.z0
        self.params = StokesParams(mode=_MODE[domType], nx=nx, ny=ny, nz=nz, Lx=Lx, Ly=Ly,
                                   zmin=self.z0, zmax=self.z0 + Lz, viscosity=viscosity, w=w,
                                   beta=beta_hat * w, alpha=a, has_torque=self.has_torque, w_d=w_d,
                                   beta_d=beta_d_hat * w_d, alpha_d=ad, precision=precision)
        self.precision = np.float64 if precision == "fp64" else np.float32
        self.op = DPStokes(self.params, self.N)

    def Clean(self):
        if self.op is not None:
            self.op.close()
            self.op = None

    def SetPositions(self, positions):
        X = torch.tensor(np.asarray(positions, dtype=np.float64).reshape(-1, 3), device=self.op.device)
        X[:, 0] -= self.xmin
        X[:, 1] -= self.ymin
        self.op.set_positions(X)

    def Mdot(self, forces, torques=np.empty(0)):
        dt = torch.float64 if self.precision == np.float64 else torch.float32
        F = torch.tensor(np.asarray(forces), dtype=dt, device=self.op.device)
        T = None
        if self.has_torque and np.size(torques) == 3 * self.N:
            T = torch.tensor(np.asarray(torques), dtype=dt, device=self.op.device)
        V, W = self.op.mdot(F, T)
        MF = V.cpu().numpy().ravel()
        MT = W.cpu().numpy().ravel() if (W is not None and T is not None) else np.empty(0)
        return MF, MT
