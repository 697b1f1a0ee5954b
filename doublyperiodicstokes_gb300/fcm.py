"""FCMJoint with device='gb300': the reference's joint wrapper interface
(python_interface/common_interface_wrapper.py:21-133) on this operator, with
the CPU path's conventions (FCM.py): positions in [xmin,xmax] x [ymin,ymax] x
[zmin,zmax], the Chebyshev interval starting at z0, BCs per domain type.

Without an explicit grid, Initialize chooses the grid and kernels exactly as
the reference does (gridconfig: GridAndKernelConfig.py's (h, beta, N) from the
hydrodynamic radius, kernel type and optInd; the z extent, Nz and floor from
the domain type), like the reference's GPU branch
(common_interface_wrapper.py:78-101) but with the Chebyshev interval at the
floor it returns, as the CPU path places it.  The keyword-only arguments (nx,
ny, nz, kernel widths, dimensionless betas, z0) override that choice.
Everything else -- argument names, order, array formats ([3N] interleaved
xyz), return values -- follows FCMJoint.
"""
import numpy as np
import torch

from . import gridconfig
from .operator import DPStokes, StokesParams

_MODE = {"DP": "nowall", "DPBW": "bottom", "DPSC": "slit", "TP": "periodic"}


class FCMJoint:
    def __init__(self, device="gb300"):
        if device != "gb300":
            raise ValueError("this FCMJoint runs the GB300 operator only (device='gb300')")
        self.device = device
        self.precision = np.float64
        self.op = None

    def Initialize(self, numberParticles, hydrodynamicRadius, viscosity, domType, has_torque,
                   xmax, ymax, zmin, zmax, xmin=0, ymin=0, kernType=0, optInd=0, ref=False, *,
                   nx=None, ny=None, nz=None, w=6, beta_hat=None, w_d=6, beta_d_hat=2.2160, z0=None,
                   precision="fp64", useRegKernel=False):
        """FCMJoint.Initialize.  With nx = None the grid and kernels are the
        reference's choice for (hydrodynamicRadius, kernType, optInd, ref);
        otherwise nx, ny, nz, w, beta_hat (default: the reference's w = 6
        value, 1.714 without torques, 1.3267 with), w_d, beta_d_hat and z0
        are taken as given.  useRegKernel selects the reference FCM's
        regular-kernel torque coupling (FCM.Initialize's argument of that
        name) instead of the derivative kernels."""
        if domType not in _MODE:
            raise ValueError("domType must be DP, DPBW, DPSC or TP")
        self.Clean()
        self.has_torque = bool(has_torque)
        self.N = int(numberParticles)
        self.xmin, self.ymin = xmin, ymin
        if nx is None:
            radP = hydrodynamicRadius * np.ones(self.N)
            kts = kernType * np.ones(self.N, dtype=int)
            Lx, Ly, hx, _, nx, ny, wm, wd, _, _, bm, bd = gridconfig.configure_grid_and_kernels_xy(
                xmax - xmin, ymax - ymin, radP, kts, optInd, self.has_torque, ref)
            Lz, _, nz, self.z0 = gridconfig.configure_grid_and_kernels_z(zmin, zmax, hx, wm, wd, domType,
                                                                        fac=1.5, ref=ref)
            w, beta_hat = int(wm[0]), float(bm[0])
            if self.has_torque:
                w_d, beta_d_hat = int(wd[0]), float(bd[0])
        else:
            if ny is None or nz is None:
                raise ValueError("an explicit grid needs nx, ny and nz")
            Lx, Ly = xmax - xmin, ymax - ymin
            hx = Lx / nx
            self.z0 = zmin if z0 is None else z0
            Lz = zmax - self.z0
            if beta_hat is None:
                beta_hat = 1.3267 if has_torque else 1.714
        a = StokesParams.kernel_alpha(hydrodynamicRadius, w, hx)
        ad = StokesParams.kernel_alpha(hydrodynamicRadius, w_d, hx)
        self.params = StokesParams(mode=_MODE[domType], nx=int(nx), ny=int(ny), nz=int(nz), Lx=Lx, Ly=Ly,
                                   zmin=self.z0, zmax=self.z0 + Lz, viscosity=viscosity, w=w,
                                   beta=beta_hat * w, alpha=a, has_torque=self.has_torque, w_d=w_d,
                                   beta_d=beta_d_hat * w_d, alpha_d=ad, precision=precision,
                                   reg_kernel=bool(useRegKernel))
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
