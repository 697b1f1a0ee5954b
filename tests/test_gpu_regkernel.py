"""Regular-kernel torque coupling (DPST_TORQUE_REG, the reference's
useRegKernel=True) on the GPU.  The reference's own outputs for the s_reg_*
cases are checked by test_gpu_parity.test_fp64_matches_reference (every golden
fixture); here: the force spread grid, the velocity grid and V, Omega against
the oracle (FP64: 1e-12 / 1e-10), mixed against FP64 (1e-5) in every geometry,
the symmetry of the triply periodic operator with torques
(<G, M F> = <F, M G>), linearity in the open domain at the c2 size, Mdot
without torques, multi-column Mdot, and the calls this coupling does not
provide (backward, batched systems)."""
import ctypes
import dataclasses

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import dpstokes_oracle as O  # noqa: E402
from conftest import rel_err  # noqa: E402
from doublyperiodicstokes_gb300 import DPStokes, StokesParams, _lib, workloads as W  # noqa: E402
from doublyperiodicstokes_gb300._lib import DPStokesError  # noqa: E402

pytestmark = pytest.mark.gpu
TOL_FP64 = 1e-10
TOL_MIXED = 1e-5


def _op(w, X, precision="fp64"):
    op = DPStokes(StokesParams.from_workload(w, precision), w.N)
    op.set_positions(torch.tensor(X, dtype=torch.float64, device=op.device))
    return op


def _mdot(op, F, T, dtype=torch.float64):
    Ft = torch.tensor(F, dtype=dtype, device=op.device)
    Tt = torch.tensor(T, dtype=dtype, device=op.device) if T is not None else None
    V, Wt = op.mdot(Ft, Tt)
    torch.cuda.synchronize()
    return V.double().cpu().numpy(), (Wt.double().cpu().numpy() if Wt is not None else None)


@pytest.mark.parametrize("name", [w.name for w in W.SMALL_REG])
def test_fp64_stages_match_oracle(name):
    w = W.SMALL_BY_NAME[name]
    X, F, T = W.make_inputs(w)
    op = _op(w, X)
    V, Wv = _mdot(op, F, T)
    vg = op.velocity_grid().cpu().numpy()
    sg = op.spread_grid(torch.tensor(F, device=op.device), torch.tensor(T, device=op.device)).cpu().numpy()
    st = {}
    o = O.Oracle(O.Params(**w.oracle_params()))
    o.set_positions(X)
    Vo, Wo = o.mdot(F, T, stages=st)
    e_s = rel_err(sg.transpose(2, 3, 1, 0), st["spread_grid"])
    e_u = rel_err(vg.transpose(2, 3, 1, 0), st["u_grid"])
    ev, ew = rel_err(V, Vo), rel_err(Wv, Wo)
    print("%s spread %.2e velocity grid %.2e V %.2e W %.2e" % (name, e_s, e_u, ev, ew))
    assert e_s < 1e-12
    assert e_u < TOL_FP64
    assert ev < TOL_FP64
    assert ew < TOL_FP64
    op.close()


@pytest.mark.parametrize("name", [w.name for w in W.SMALL_REG])
def test_mixed_close_to_fp64(name):
    w = W.SMALL_BY_NAME[name]
    X, F, T = W.make_inputs(w)
    V64, W64 = _mdot(_op(w, X), F, T)
    V32, W32 = _mdot(_op(w, X, "mixed"), F.astype(np.float32), T.astype(np.float32), torch.float32)
    ev, ew = rel_err(V32, V64), rel_err(W32, W64)
    print("%s mixed V %.2e W %.2e" % (name, ev, ew))
    assert ev < TOL_MIXED
    assert ew < TOL_MIXED


@pytest.mark.parametrize("name", ["s_reg_dpbw_t", "s_reg_tp_t"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_without_torques_matches_oracle(name, precision):
    w = W.SMALL_BY_NAME[name]
    X, F, _ = W.make_inputs(w)
    op = _op(w, X, precision)
    dt = torch.float64 if precision == "fp64" else torch.float32
    V, Wv = _mdot(op, F.astype(np.float32) if precision == "mixed" else F, None, dt)
    assert Wv is not None  # the vorticity of the force-driven flow
    Vo, Wo = O.mdot(O.Params(**w.oracle_params()), X, F, np.zeros_like(F))
    tol = TOL_FP64 if precision == "fp64" else TOL_MIXED
    assert rel_err(V, Vo) < tol
    assert rel_err(Wv, Wo) < tol
    op.close()


def _flat(V, Wv):
    return np.concatenate([V.ravel(), Wv.ravel()])


def test_tp_symmetry_and_dp_linearity_full_size():
    """t1 (512 x 512 x 64, N = 65,536) with regular-kernel torques: the triply
    periodic mobility is symmetric; c2 (open, 512^2 x 128): linearity, mixed
    against FP64."""
    w = dataclasses.replace(W.T1, name="t1_tp_n65536_reg", reg_kernel=True)
    X, F, T = W.make_inputs(w)
    rng = np.random.default_rng(5)
    G, S = rng.standard_normal(F.shape), rng.standard_normal(T.shape)
    op = _op(w, X)
    MF = _flat(*_mdot(op, F, T))
    MG = _flat(*_mdot(op, G, S))
    f, g = _flat(F, T), _flat(G, S)
    a, b = float(g @ MF), float(f @ MG)
    print("tp symmetry %.6e %.6e rel %.2e" % (a, b, abs(a - b) / abs(a)))
    assert abs(a - b) <= 1e-10 * np.sqrt(float(f @ MF) * float(g @ MG))
    op.close()
    w = dataclasses.replace(W.C2, name="c2_dp_n65536_reg", reg_kernel=True)
    X, F, T = W.make_inputs(w)
    G, S = rng.standard_normal(F.shape), rng.standard_normal(T.shape)
    op = _op(w, X)
    MF = _flat(*_mdot(op, F, T))
    MG = _flat(*_mdot(op, G, S))
    MH = _flat(*_mdot(op, 2.0 * F - 3.0 * G, 2.0 * T - 3.0 * S))
    e = rel_err(MH, 2.0 * MF - 3.0 * MG)
    print("dp linearity %.2e" % e)
    assert e < 1e-12
    op.close()
    opm = _op(w, X, "mixed")
    MFm = _flat(*_mdot(opm, F.astype(np.float32), T.astype(np.float32), torch.float32))
    em = rel_err(MFm, MF)
    print("c2 reg mixed %.2e" % em)
    assert em < TOL_MIXED
    opm.close()


def test_multi_columns_and_unsupported_calls():
    w = W.SMALL_BY_NAME["s_reg_dpsc_t"]
    X, F, T = W.make_inputs(w)
    op = _op(w, X)
    rng = np.random.default_rng(9)
    Fk, Tk = rng.standard_normal((2, w.N, 3)), rng.standard_normal((2, w.N, 3))
    Vm, Wm = op.mdot_multi(torch.tensor(Fk, device=op.device), torch.tensor(Tk, device=op.device))
    for k in range(2):
        Vs, Ws = _mdot(op, Fk[k], Tk[k])
        assert rel_err(Vm[k].cpu().numpy(), Vs) < 1e-13
        assert rel_err(Wm[k].cpu().numpy(), Ws) < 1e-13
    gV = torch.ones((w.N, 3), dtype=torch.float64, device=op.device)
    with pytest.raises(DPStokesError):
        op.mdot_backward(torch.tensor(F, device=op.device), torch.tensor(T, device=op.device), gV, gV)
    op.close()
    L = _lib.lib()
    prm = StokesParams.from_workload(w).to_c()
    n = (ctypes.c_int64 * 1)(w.N)
    b = ctypes.c_void_p()
    assert L.dpst_batched_create(ctypes.byref(prm), n, 1, 0, ctypes.byref(b)) == 5  # DPST_ERR_UNSUPPORTED


def test_fcmjoint_use_reg_kernel():
    """FCMJoint.Initialize(..., useRegKernel=True) with the reference's grid
    choice against the oracle on the same grid (bottom wall, torques)."""
    from doublyperiodicstokes_gb300.fcm import FCMJoint
    N, R, eta, L = 30, 1.0, 1.0 / (6 * np.pi), 24.0
    rng = np.random.default_rng(21)
    X = np.column_stack([rng.uniform(0, L, N), rng.uniform(0, L, N), rng.uniform(1.0, 9.0, N)])
    F, T = rng.standard_normal((N, 3)), rng.standard_normal((N, 3))
    fj = FCMJoint("gb300")
    fj.Initialize(N, R, eta, "DPBW", True, L, L, 0.0, 10.0, useRegKernel=True)
    p = fj.params
    assert p.reg_kernel
    fj.SetPositions(X.ravel())
    MF, MT = fj.Mdot(F.ravel(), T.ravel())
    h = p.Lx / p.nx
    op = O.Params("DPBW", p.nx, p.ny, p.nz, p.Lx, p.Ly, p.zmax - p.zmin, z0=p.zmin, eta=eta, wm=p.w,
                  betam_hat=p.beta / p.w, has_torque=True, wd=p.w_d, betad_hat=p.beta_d / p.w_d, radius=R,
                  reg_kernel=True)
    assert abs(op.alpha(p.w) - p.alpha) < 1e-12 * p.alpha and abs(h - op.hx) < 1e-15
    Xs = X.copy()
    Vo, Wo = O.mdot(op, Xs, F, T)
    assert rel_err(MF, Vo) < TOL_FP64
    assert rel_err(MT, Wo) < TOL_FP64
    fj.Clean()
