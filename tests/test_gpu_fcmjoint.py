"""FCMJoint(device='gb300') (doublyperiodicstokes_gb300.fcm) on the GPU: with no
explicit grid, Initialize takes the reference's grid and kernel choice
(gridconfig, pinned to GridAndKernelConfig.py by tests/test_gridconfig.py);
SetPositions / Mdot on that grid match the oracle run with the same derived
parameters (FP64, 1e-10), with and without torques."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import dpstokes_oracle as O  # noqa: E402
from conftest import rel_err  # noqa: E402
from doublyperiodicstokes_gb300 import gridconfig  # noqa: E402
from doublyperiodicstokes_gb300.fcm import FCMJoint  # noqa: E402

pytestmark = pytest.mark.gpu
ETA = 1.0 / (6.0 * np.pi)


@pytest.mark.parametrize("domType,has_torque,kern,opt", [("DPBW", False, 0, 0), ("DP", True, 0, 1),
                                                        ("DPSC", True, 3, 0)])
def test_auto_grid_mdot_matches_oracle(domType, has_torque, kern, opt):
    N, R, L = 24, 1.0, 16.0
    zmin, zmax = (0.0, 10.0) if domType != "DP" else (-4.0, 4.0)
    fj = FCMJoint("gb300")
    fj.Initialize(N, R, ETA, domType, has_torque, L, L, zmin, zmax, kernType=kern, optInd=opt)
    p = fj.params
    # the reference's choice, recomputed
    Lx, Ly, hx, _, nx, ny, wm, wd, _, _, bm, bd = gridconfig.configure_grid_and_kernels_xy(
        L, L, R * np.ones(N), kern * np.ones(N, dtype=int), opt, has_torque, False)
    Lz, _, nz, a = gridconfig.configure_grid_and_kernels_z(zmin, zmax, hx, wm, wd, domType, 1.5, False)
    assert (p.nx, p.ny, p.nz, p.w) == (nx, ny, nz, int(wm[0]))
    assert abs(p.beta - bm[0] * wm[0]) == 0 and p.zmin == a and abs(p.zmax - (a + Lz)) < 1e-12
    rng = np.random.default_rng(4)
    lo = zmin + 1.5 if domType != "DP" else zmin
    hi = zmax - 1.5 if domType == "DPSC" else zmax
    X = np.column_stack([rng.uniform(0, Lx, N), rng.uniform(0, Ly, N), rng.uniform(lo, hi, N)])
    F = rng.standard_normal(3 * N)
    T = rng.standard_normal(3 * N) if has_torque else np.empty(0)
    fj.SetPositions(X.ravel())
    MF, MT = fj.Mdot(F, T)
    op = O.Params(domType=domType, Nx=nx, Ny=ny, Nz=nz, Lx=Lx, Ly=Ly, Lz=Lz, z0=a, eta=ETA, wm=int(wm[0]),
                  betam_hat=float(bm[0]), has_torque=has_torque, wd=int(wd[0]) if has_torque else 6,
                  betad_hat=float(bd[0]) if has_torque else 2.2160, radius=R)
    Vo, Wo = O.mdot(op, X, F.reshape(-1, 3), T.reshape(-1, 3) if has_torque else None)
    print("%s grid %dx%dx%d w %d beta %.4f: V %.2e" % (domType, nx, ny, nz, wm[0], bm[0] * wm[0],
                                                       rel_err(MF, Vo)))
    assert rel_err(MF, Vo) < 1e-10
    if has_torque:
        assert rel_err(MT, Wo) < 1e-10
    fj.Clean()
