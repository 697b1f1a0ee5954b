"""Triply periodic mode (DPST_MODE_PERIODIC, the reference's domType 'TP') on
the GPU.  The reference's own outputs for the small TP cases and for
t0_tp_n2048 are checked by test_gpu_parity.test_fp64_matches_reference (every
golden fixture); here: the spread and velocity grids against the oracle stage
by stage (FP64, 1e-12 / 1e-10), the mixed operator against FP64 (1e-5), and at
the full t1_tp_n65536 size the properties that need no oracle run: symmetry
of the mobility (<G, M F> = <F, M G>, forces and torques), positivity,
linearity, invariance under shifts by whole grid cells (1e-10 FP64), mixed
against FP64 (1e-5).  Also FCMJoint(domType='TP') with the reference's grid
choice, the uammd shim's mode 'periodic', multi-column Mdot, and the calls
this mode does not provide."""
import ctypes

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


@pytest.mark.parametrize("name", [w.name for w in W.SMALL_TP])
def test_fp64_stages_match_oracle(name):
    w = W.SMALL_BY_NAME[name]
    X, F, T = W.make_inputs(w)
    op = _op(w, X)
    V, Wv = _mdot(op, F, T)
    vg = op.velocity_grid().cpu().numpy()
    sg = op.spread_grid(torch.tensor(F, device=op.device),
                        torch.tensor(T, device=op.device) if T is not None else None).cpu().numpy()
    st = {}
    o = O.Oracle(O.Params(**w.oracle_params()))
    o.set_positions(X)
    Vo, Wo = o.mdot(F, T, stages=st)
    e_s = rel_err(sg.transpose(2, 3, 1, 0), st["spread_grid"])
    e_u = rel_err(vg.transpose(2, 3, 1, 0), st["u_grid"])
    print("%s spread %.2e velocity grid %.2e V %.2e" % (name, e_s, e_u, rel_err(V, Vo)))
    assert e_s < 1e-12
    assert e_u < TOL_FP64
    assert rel_err(V, Vo) < TOL_FP64
    if T is not None:
        assert rel_err(Wv, Wo) < TOL_FP64
    op.close()


@pytest.mark.parametrize("name", [w.name for w in W.SMALL_TP] + ["t0_tp_n2048"])
def test_mixed_close_to_fp64(name):
    w = W.SMALL_BY_NAME.get(name) or W.by_name(name)
    X, F, T = W.make_inputs(w)
    V64, W64 = _mdot(_op(w, X), F, T)
    V32, W32 = _mdot(_op(w, X, "mixed"), F.astype(np.float32), None if T is None else T.astype(np.float32),
                     torch.float32)
    ev = rel_err(V32, V64)
    print("%s mixed V %.2e" % (name, ev))
    assert ev < TOL_MIXED
    if T is not None:
        assert rel_err(W32, W64) < TOL_MIXED


def test_unfused_particle_passes_match_oracle():
    # monopole w = 6, dipole w = 5: separate monopole and dipole passes
    import dataclasses
    w = dataclasses.replace(W.SMALL_BY_NAME["s_tp_t"], name="s_tp_t_wm6_wd5", wd=5, betad_hat=1.7584,
                            betam_hat=1.3261)
    X, F, T = W.make_inputs(w)
    op = _op(w, X)
    assert op.info()["fused_particle_passes"] == 0
    V, Wv = _mdot(op, F, T)
    Vo, Wo = O.mdot(O.Params(**w.oracle_params()), X, F, T)
    assert rel_err(V, Vo) < TOL_FP64
    assert rel_err(Wv, Wo) < TOL_FP64


def _flat(V, Wv):
    return np.concatenate([V.ravel(), Wv.ravel()]) if Wv is not None else V.ravel()


def test_full_size_properties():
    """t1_tp_n65536 (512 x 512 x 64, N = 65,536, torques): symmetry,
    positivity, linearity, periodic shift invariance; mixed vs FP64."""
    w = W.T1
    X, F, T = W.make_inputs(w)
    rng = np.random.default_rng(77)
    G, S = rng.standard_normal(F.shape), rng.standard_normal(T.shape)
    op = _op(w, X)
    MF = _flat(*_mdot(op, F, T))
    MG = _flat(*_mdot(op, G, S))
    f, g = _flat(F, T), _flat(G, S)
    # <G, M F> = <F, M G>: spread and interpolation are adjoint (weights hx hy hz)
    a, b = float(g @ MF), float(f @ MG)
    print("symmetry %.3e %.3e rel %.2e" % (a, b, abs(a - b) / abs(a)))
    assert abs(a - b) <= 1e-10 * np.sqrt(float(f @ MF) * float(g @ MG))
    assert float(f @ MF) > 0 and float(g @ MG) > 0
    # linearity
    MH = _flat(*_mdot(op, 2.0 * F - 3.0 * G, 2.0 * T - 3.0 * S))
    assert rel_err(MH, 2.0 * MF - 3.0 * MG) < 1e-12
    # shift by whole cells along x, y and z (wrapped into the box)
    Xs = X.copy()
    Xs[:, 0] = np.mod(Xs[:, 0] + 5 * w.Lx / w.nx, w.Lx)
    Xs[:, 1] = np.mod(Xs[:, 1] + 3 * w.Ly / w.ny, w.Ly)
    Xs[:, 2] = np.mod(Xs[:, 2] + 7 * w.Lz / w.nz, w.Lz)
    ops = _op(w, Xs)
    MFs = _flat(*_mdot(ops, F, T))
    e = rel_err(MFs, MF)
    print("shift %.2e" % e)
    assert e < TOL_FP64
    ops.close()
    # mixed precision
    opm = _op(w, X, "mixed")
    MFm = _flat(*_mdot(opm, F.astype(np.float32), T.astype(np.float32), torch.float32))
    em = rel_err(MFm, MF)
    print("mixed %.2e" % em)
    assert em < TOL_MIXED
    opm.close()
    op.close()


def test_info_multi_and_unsupported_calls():
    w = W.SMALL_BY_NAME["s_tp_t"]
    X, F, T = W.make_inputs(w)
    op = _op(w, X)
    inf = op.info()
    assert inf["n_modes"] == w.nz * w.ny * (w.nx // 2 + 1)
    assert inf["kernels_per_mdot"] == 3 and inf["fused_particle_passes"] == 1
    # K columns = K single calls (equal up to the order of the spread's atomic sums)
    rng = np.random.default_rng(3)
    Fk, Tk = rng.standard_normal((3, w.N, 3)), rng.standard_normal((3, w.N, 3))
    Vm, Wm = op.mdot_multi(torch.tensor(Fk, device=op.device), torch.tensor(Tk, device=op.device))
    for k in range(3):
        Vs, Ws = _mdot(op, Fk[k], Tk[k])
        assert rel_err(Vm[k].cpu().numpy(), Vs) < 1e-13
        assert rel_err(Wm[k].cpu().numpy(), Ws) < 1e-13
    op.close()
    # no backward with the regular-kernel coupling
    import dataclasses
    wr = dataclasses.replace(w, reg_kernel=True)
    opr = _op(wr, X)
    gV = torch.ones((w.N, 3), dtype=torch.float64, device=opr.device)
    with pytest.raises(DPStokesError):
        opr.mdot_backward(torch.tensor(F, device=opr.device), torch.tensor(T, device=opr.device), gV, gV)
    opr.close()
    # no batched systems in this mode
    L = _lib.lib()
    prm = StokesParams.from_workload(w).to_c()
    n = (ctypes.c_int64 * 1)(w.N)
    b = ctypes.c_void_p()
    code = L.dpst_batched_create(ctypes.byref(prm), n, 1, 0, ctypes.byref(b))
    assert code == 5  # DPST_ERR_UNSUPPORTED


def test_out_of_box_particle_rejected():
    w = W.SMALL_BY_NAME["s_tp_t"]
    X, _, _ = W.make_inputs(w)
    op = DPStokes(StokesParams.from_workload(w), w.N)
    X[3, 2] = w.Lz + 0.5
    with pytest.raises(DPStokesError):
        op.set_positions(torch.tensor(X, device=op.device))
    op.close()


def test_fcmjoint_tp_reference_grid():
    """FCMJoint(domType='TP') with the reference's (h, beta, N) choice, against
    the oracle on the same grid."""
    from doublyperiodicstokes_gb300 import gridconfig
    from doublyperiodicstokes_gb300.fcm import FCMJoint
    N, R, eta = 40, 1.0, 1.0 / (6 * np.pi)
    L, Lz = 30.0, 20.0
    rng = np.random.default_rng(12)
    X = np.column_stack([rng.uniform(0, L, N), rng.uniform(0, L, N), rng.uniform(0, Lz, N)])
    F, T = rng.standard_normal((N, 3)), rng.standard_normal((N, 3))
    fj = FCMJoint("gb300")
    fj.Initialize(N, R, eta, "TP", True, L, L, 0.0, Lz)
    p = fj.params
    fj.SetPositions(X.ravel())
    MF, MT = fj.Mdot(F.ravel(), T.ravel())
    Lx, Ly, hx, hy, nx, ny, wm, wd, _, _, bm, bd = gridconfig.configure_grid_and_kernels_xy(
        L, L, R * np.ones(N), np.zeros(N, dtype=int), 0, True)
    Lzc, hz, nz, z0 = gridconfig.configure_grid_and_kernels_z(0.0, Lz, hx, wm, wd, "TP")
    assert (p.nx, p.ny, p.nz) == (nx, ny, nz) and abs(p.zmax - p.zmin - Lzc) < 1e-12
    op = O.Params("TP", nx, ny, nz, Lx, Ly, Lzc, z0=z0, eta=eta, wm=int(wm[0]), betam_hat=float(bm[0]),
                  has_torque=True, wd=int(wd[0]), betad_hat=float(bd[0]), radius=R)
    Vo, Wo = O.mdot(op, X, F, T)
    assert rel_err(MF, Vo) < TOL_FP64
    assert rel_err(MT, Wo) < TOL_FP64
    fj.Clean()


def test_uammd_shim_periodic_mode():
    from doublyperiodicstokes_gb300 import uammd
    w = W.SMALL_BY_NAME["s_tp_t"]
    X, F, T = W.make_inputs(w)
    sp = StokesParams.from_workload(w)
    h = w.Lx / w.nx
    par = uammd.StokesParameters(viscosity=sp.viscosity, Lx=w.Lx, Ly=w.Ly, zmin=sp.zmin, zmax=sp.zmax, w=sp.w,
                                 w_d=sp.w_d, alpha=sp.alpha / h, alpha_d=sp.alpha_d / h, beta=sp.beta,
                                 beta_d=sp.beta_d, nx=w.nx, ny=w.ny, nz=w.nz, mode="periodic")
    m = uammd.DPStokes()
    m.initialize(par, w.N)
    m.setPositions(X.ravel())
    MF, MT = np.zeros(3 * w.N), np.zeros(3 * w.N)
    m.Mdot(forces=F.ravel(), torques=T.ravel(), velocities=MF, angularVelocities=MT)
    Vo, Wo = O.mdot(O.Params(**w.oracle_params()), X, F, T)
    assert rel_err(MF, Vo) < TOL_FP64
    assert rel_err(MT, Wo) < TOL_FP64
    m.clear()


@pytest.mark.parametrize("name", ["s_tp_t", "t0_tp_n2048", "t1_tp_n65536", "s_tp_f_odd"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fused_z_path_matches_cufft_path(name, precision, monkeypatch):
    """nz = 16, 32, 64: the fused z transform + solve kernel after 2-D x-y
    transforms (forced for FP64, the default for mixed) against cuFFT's 3-D
    transforms and the separate solve (FP64: 1e-12; mixed: 1e-6); nz = 13
    keeps the 3-D path."""
    w = W.SMALL_BY_NAME.get(name) or W.by_name(name)
    X, F, T = W.make_inputs(w)
    dt = torch.float64 if precision == "fp64" else torch.float32
    if T is not None and precision == "mixed":
        T = T.astype(np.float32)
    Fc = F.astype(np.float32) if precision == "mixed" else F
    out = {}
    for mode in ("fused", "cufft"):
        monkeypatch.setenv("DPSTOKES_GB300_TP_Z", mode)
        op = _op(w, X, precision)
        out[mode] = (_mdot(op, Fc, T, dt), op.info()["z_fused"])
        op.close()
    expect = 1 if w.nz in (16, 32, 64) else 0
    assert out["fused"][1] == expect and out["cufft"][1] == 0
    (Vf, Wf), (Vc, Wc) = out["fused"][0], out["cufft"][0]
    tol = 1e-12 if precision == "fp64" else 1e-6
    ev = rel_err(Vf, Vc)
    print("%s %s fused vs cufft V %.2e" % (name, precision, ev))
    assert ev < tol
    if Wc is not None:
        assert rel_err(Wf, Wc) < tol


@pytest.mark.parametrize("name", ["s_tp_t", "t0_tp_n2048"])
def test_backward_forces_torques(name):
    """dl/dF, dl/dT of l = <gV, V> + <gW, W>: the transpose identity
    <gV, V> + <gW, W> = <dl/dF, F> + <dl/dT, T> (FP64, 1e-12 of the terms'
    scale) and, per component, the oracle's M (gV, gW) (1e-10)."""
    w = W.SMALL_BY_NAME.get(name) or W.by_name(name)
    X, F, T = W.make_inputs(w)
    op = _op(w, X)
    d = op.device
    rng = np.random.default_rng(4)
    gV = rng.standard_normal(F.shape)
    gW = rng.standard_normal(F.shape) if T is not None else None
    V, Wv = _mdot(op, F, T)
    gF, gT, gX = op.mdot_backward(torch.tensor(F, device=d), torch.tensor(T, device=d) if T is not None else None,
                                  torch.tensor(gV, device=d), torch.tensor(gW, device=d) if gW is not None else None,
                                  need_F=True, need_T=T is not None, need_X=False)
    assert gX is None
    gF = gF.cpu().numpy()
    lhs = float(np.sum(gV * V.reshape(gV.shape)))
    rhs = float(np.sum(gF * F))
    if T is not None:
        gT = gT.cpu().numpy()
        lhs += float(np.sum(gW * Wv.reshape(gW.shape)))
        rhs += float(np.sum(gT * T))
    scale = float(np.linalg.norm(gF) * np.linalg.norm(F))
    print("%s transpose identity %.3e vs %.3e" % (name, lhs, rhs))
    assert abs(lhs - rhs) <= 1e-12 * scale
    Vo, Wo = O.mdot(O.Params(**w.oracle_params()), X, gV, gW)
    assert rel_err(gF, Vo) < TOL_FP64
    if T is not None:
        assert rel_err(gT, Wo) < TOL_FP64
    op.close()


@pytest.mark.parametrize("name", ["t0_tp_n2048", "t1_tp_n65536@128"])
def test_fp64_periodic_double_float_transforms(name, monkeypatch):
    """The triply periodic FP64 operator on the library's double-float 3-D
    transforms (x rows, y and z columns) against cuFFT's FP64 3-D transforms
    (1e-12), and the reference fixture where one exists (1e-10)."""
    import golden_io
    w = W.by_name(name)
    X, F, T = W.make_inputs(w)
    out = {}
    for which in ("own", "cufft"):
        monkeypatch.setenv("DPSTOKES_GB300_XY_FFT", which)
        op = DPStokes(StokesParams.from_workload(w, "fp64"), w.N)
        form = op.info()["xy_transform"]
        op.set_positions(torch.tensor(X, device=op.device))
        V, Wv = op.mdot(torch.tensor(F, device=op.device),
                        torch.tensor(T, device=op.device) if T is not None else None)
        torch.cuda.synchronize()
        out[which] = (form, V.cpu().numpy(), Wv.cpu().numpy() if Wv is not None else None)
        op.close()
    assert out["own"][0] == 3 and out["cufft"][0] == 0
    ev = rel_err(out["own"][1], out["cufft"][1])
    print("%s TP FP64 own double-float vs cuFFT V %.2e" % (name, ev))
    assert ev < 1e-12
    if T is not None:
        assert rel_err(out["own"][2], out["cufft"][2]) < 1e-12
    if name in golden_io.names():
        _, _, _, _, gd = golden_io.inputs(name)
        assert rel_err(golden_io.restrict(gd, out["own"][1]), gd["V"]) < 1e-10
