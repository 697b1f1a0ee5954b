"""GPU parity through the C ABI: the FP64 operator against the reference's own
outputs (tests/golden) and, stage by stage, against the oracle; the mixed
operator against the FP64 operator.  Tolerances: FP64 1e-10 relative (2-norm
over all 3N components), mixed 1e-5."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import dpstokes_oracle as O  # noqa: E402
import golden_io  # noqa: E402
from conftest import rel_err  # noqa: E402
from doublyperiodicstokes_gb300 import DPStokes, StokesParams, workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu
TOL_FP64 = 1e-10
TOL_MIXED = 1e-5


def _run(w, X, F, T, precision="fp64", dtype=torch.float64):
    op = DPStokes(StokesParams.from_workload(w, precision), w.N)
    dev = op.device
    op.set_positions(torch.tensor(X, dtype=torch.float64, device=dev))
    Ft = torch.tensor(F, dtype=dtype, device=dev)
    Tt = torch.tensor(T, dtype=dtype, device=dev) if T is not None else None
    V, Wt = op.mdot(Ft, Tt)
    torch.cuda.synchronize()
    return op, V.double().cpu().numpy(), (Wt.double().cpu().numpy() if Wt is not None else None)


@pytest.mark.parametrize("name", golden_io.names())
def test_fp64_matches_reference(name):
    w, X, F, T, g = golden_io.inputs(name)
    op, V, Wv = _run(w, X, F, T)
    ev = rel_err(golden_io.restrict(g, V), g["V"])
    print("%s V rel err %.3e" % (name, ev))
    assert ev < TOL_FP64
    if w.has_torque:
        ew = rel_err(golden_io.restrict(g, Wv), g["W"])
        print("%s W rel err %.3e" % (name, ew))
        assert ew < TOL_FP64


@pytest.mark.parametrize("name", [w.name for w in W.SMALL])
def test_fp64_stages_match_oracle(name):
    w = W.SMALL_BY_NAME[name]
    X, F, T = W.make_inputs(w)
    op, V, Wv = _run(w, X, F, T)
    vg = op.velocity_grid().cpu().numpy()
    dev = op.device
    sg = op.spread_grid(torch.tensor(F, device=dev),
                        torch.tensor(T, device=dev) if T is not None else None).cpu().numpy()
    st = {}
    o = O.Oracle(O.Params(**w.oracle_params()))
    o.set_positions(X)
    Vo, Wo = o.mdot(F, T, stages=st)
    # oracle grids are [ny][nx][nz][3]; the operator's [3][nz][ny][nx]
    e_s = rel_err(sg.transpose(2, 3, 1, 0), st["spread_grid"])
    e_u = rel_err(vg.transpose(2, 3, 1, 0), st["u_grid"])
    print("%s spread %.2e velocity grid %.2e V %.2e" % (name, e_s, e_u, rel_err(V, Vo)))
    assert e_s < 1e-12
    assert e_u < TOL_FP64
    assert rel_err(V, Vo) < TOL_FP64
    if T is not None:
        assert rel_err(Wv, Wo) < TOL_FP64


@pytest.mark.parametrize("name", [w.name for w in W.SMALL] + ["c0_dpbw_n2048", "c1_dpsc_n16384", "c2_dp_n65536"])
def test_mixed_close_to_fp64(name):
    w = W.SMALL_BY_NAME.get(name) or W.by_name(name)
    X, F, T = W.make_inputs(w)
    _, V64, W64 = _run(w, X, F, T)
    _, V32, W32 = _run(w, X, F, T, precision="mixed", dtype=torch.float32)
    ev = rel_err(V32, V64)
    print("%s mixed V rel err %.3e" % (name, ev))
    assert ev < TOL_MIXED
    if T is not None:
        ew = rel_err(W32, W64)
        print("%s mixed W rel err %.3e" % (name, ew))
        assert ew < TOL_MIXED


def test_repeated_mdot_is_identical_and_linear():
    w = W.SMALL_BY_NAME["s_dpsc_t"]
    X, F, T = W.make_inputs(w)
    op = DPStokes(StokesParams.from_workload(w), w.N)
    d = op.device
    op.set_positions(torch.tensor(X, device=d))
    Ft, Tt = torch.tensor(F, device=d), torch.tensor(T, device=d)
    V1, W1 = op.mdot(Ft, Tt)
    V2, W2 = op.mdot(Ft, Tt)
    assert torch.equal(V1, V2) or rel_err(V1.cpu(), V2.cpu()) < 1e-14
    V3, W3 = op.mdot(2 * Ft, 2 * Tt)
    assert rel_err(V3.cpu(), 2 * V1.cpu()) < 1e-13
    assert rel_err(W3.cpu(), 2 * W1.cpu()) < 1e-13


def test_host_entry_points_match_device_ones():
    import ctypes
    from doublyperiodicstokes_gb300 import _lib
    w = W.SMALL_BY_NAME["s_dpbw_t"]
    X, F, T = W.make_inputs(w)
    op, V, Wv = _run(w, X, F, T)
    L = _lib.lib()
    Xc, Fc, Tc = (np.ascontiguousarray(a) for a in (X, F, T))
    Vh, Wh = np.zeros_like(Fc), np.zeros_like(Fc)
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    _lib.check(L.dpst_set_positions_host(op._h, ptr(Xc), _lib.F64, None))
    _lib.check(L.dpst_mdot_host(op._h, ptr(Fc), ptr(Tc), ptr(Vh), ptr(Wh), _lib.F64, None))
    assert rel_err(Vh, V) < 1e-14
    assert rel_err(Wh, Wv) < 1e-14


def test_out_of_domain_is_an_error():
    from doublyperiodicstokes_gb300._lib import DPStokesError
    w = W.SMALL_BY_NAME["s_dpbw_t"]
    X, F, T = W.make_inputs(w)
    X[3, 2] = w.z0 + w.Lz + 0.5
    op = DPStokes(StokesParams.from_workload(w), w.N)
    with pytest.raises(DPStokesError) as e:
        op.set_positions(torch.tensor(X, device=op.device))
    assert e.value.code == 3
    with pytest.raises(DPStokesError) as e:
        op.mdot(torch.tensor(F, device=op.device), torch.tensor(T, device=op.device))
    assert e.value.code == 2


def test_asymmetric_ghost_extension_is_rejected():
    from doublyperiodicstokes_gb300._lib import DPStokesError
    w = W.small("asym", "DP", 4, 16, 19, 12.0, 5.0, 7.0, False)
    with pytest.raises(DPStokesError) as e:
        DPStokes(StokesParams.from_workload(w), w.N)
    assert e.value.code == 5


def _with_widths(base, wm, wd):
    import dataclasses
    return dataclasses.replace(W.SMALL_BY_NAME[base], name="%s_wm%d_wd%d" % (base, wm, wd), wm=wm, wd=wd)


@pytest.mark.parametrize("base,wm,wd,fused", [("s_dp_t", 6, 6, 1), ("s_dpsc_t", 6, 6, 1), ("s_dpbw_t", 6, 5, 0),
                                             ("s_dp_t", 5, 6, 0)])
def test_fused_and_separate_particle_passes(base, wm, wd, fused):
    """Equal kernel widths share one spread and one interpolation pass for
    forces and torques (the dipole's z windows nest in the monopole's);
    other widths keep separate passes.  Both match the oracle in FP64."""
    w = _with_widths(base, wm, wd)
    X, F, T = W.make_inputs(w)
    op, V, Wv = _run(w, X, F, T)
    assert op.info()["fused_particle_passes"] == fused
    Vo, Wo = O.mdot(O.Params(**w.oracle_params()), X, F, T)
    ev, ew = rel_err(V, Vo), rel_err(Wv, Wo)
    print("%s fused %d V %.2e W %.2e" % (w.name, fused, ev, ew))
    assert ev < TOL_FP64
    assert ew < TOL_FP64
    _, V32, W32 = _run(w, X, F, T, precision="mixed", dtype=torch.float32)
    assert rel_err(V32, V) < TOL_MIXED
    assert rel_err(W32, Wv) < TOL_MIXED


@pytest.mark.parametrize("name", ["s_dpbw_t", "s_tp_t"])
def test_periodic_seam_positions(name):
    """A particle at x = Lx, y = Ly (and, triply periodic, z = zmax) is the
    particle at 0 (the reference indexes past its extended grid there; this
    operator wraps)."""
    w = W.SMALL_BY_NAME[name]
    X, F, T = W.make_inputs(w)
    Xa, Xb = X.copy(), X.copy()
    Xa[0, :2], Xb[0, :2] = 0.0, (w.Lx, w.Ly)
    if w.domType == "TP":
        Xa[1, 2], Xb[1, 2] = w.z0, w.z0 + w.Lz
    _, Va, Wa = _run(w, Xa, F, T)
    _, Vb, Wb = _run(w, Xb, F, T)
    assert rel_err(Vb, Va) < 1e-13
    assert rel_err(Wb, Wa) < 1e-13
    Vo, Wo = O.mdot(O.Params(**w.oracle_params()), Xa, F, T)
    assert rel_err(Va, Vo) < TOL_FP64
