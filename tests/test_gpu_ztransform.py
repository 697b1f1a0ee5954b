"""The tcgen05 split-TF32 z transform of the mixed operator against the SIMT
transform and the FP64 operator (forced with DPSTOKES_GB300_ZTRANSFORM at
creation): Mdot outputs within 5e-6 of each other and 1e-5 of FP64, on the
small cases (odd and even nz, every geometry) and the open-domain c2
geometry on a 192^2 x 128 grid; the backward pass likewise.  The FP64
operator's double-float z transform against its FP64 one (1e-12) and the
reference fixtures (1e-10)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from conftest import rel_err  # noqa: E402
from doublyperiodicstokes_gb300 import DPStokes, StokesParams, workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu


def _op(w, precision, impl, monkeypatch):
    monkeypatch.setenv("DPSTOKES_GB300_ZTRANSFORM", impl)
    op = DPStokes(StokesParams.from_workload(w, precision), w.N)
    monkeypatch.delenv("DPSTOKES_GB300_ZTRANSFORM")
    return op


def _mdot(op, X, F, T, dtype):
    op.set_positions(torch.tensor(X, device="cuda"))
    V, Wv = op.mdot(torch.tensor(F, dtype=dtype, device="cuda"),
                    torch.tensor(T, dtype=dtype, device="cuda") if T is not None else None)
    torch.cuda.synchronize()
    return V.double().cpu().numpy(), (Wv.double().cpu().numpy() if Wv is not None else None)


CASES = [w.name for w in W.SMALL] + ["c2_dp_n65536@192"]


def _wl(name):
    return W.SMALL_BY_NAME.get(name) or W.by_name(name)


@pytest.mark.parametrize("name", CASES)
def test_tcgen05_ztransform_matches(name, monkeypatch):
    w = _wl(name)
    X, F, T = W.make_inputs(w)
    tc = _op(w, "mixed", "tcgen05", monkeypatch)
    info = tc.info()
    assert info["ztransform"] == 1, info
    si = _op(w, "mixed", "simt", monkeypatch)
    assert si.info()["ztransform"] == 0
    f64 = _op(w, "fp64", "auto", monkeypatch)
    Vt, Wt = _mdot(tc, X, F, T, torch.float32)
    Vs, Ws = _mdot(si, X, F, T, torch.float32)
    Vd, Wd = _mdot(f64, X, F, T, torch.float64)
    e_ts, e_td, e_sd = rel_err(Vt, Vs), rel_err(Vt, Vd), rel_err(Vs, Vd)
    print("%s tc-simt %.2e tc-fp64 %.2e simt-fp64 %.2e (ms simt %.3f tc %.3f)" %
          (name, e_ts, e_td, e_sd, info["ztransform_ms"][0], info["ztransform_ms"][1]))
    assert e_ts < 5e-6 and e_td < 1e-5
    if T is not None:
        assert rel_err(Wt, Ws) < 5e-6 and rel_err(Wt, Wd) < 1e-5


@pytest.mark.parametrize("name", ["s_dpbw_t", "s_dpsc_t", "s_dp_t_shift"])
def test_tcgen05_backward(name, monkeypatch):
    w = _wl(name)
    X, F, T = W.make_inputs(w)
    rng = np.random.default_rng(2)
    gV = rng.standard_normal((w.N, 3))
    gW = rng.standard_normal((w.N, 3)) if T is not None else None
    out = {}
    for key, prec, impl, dt in (("tc", "mixed", "tcgen05", torch.float32), ("d", "fp64", "auto", torch.float64)):
        op = _op(w, prec, impl, monkeypatch)
        op.set_positions(torch.tensor(X, device="cuda"))
        g = op.mdot_backward(torch.tensor(F, dtype=dt, device="cuda"),
                             torch.tensor(T, dtype=dt, device="cuda") if T is not None else None,
                             torch.tensor(gV, dtype=dt, device="cuda"),
                             torch.tensor(gW, dtype=dt, device="cuda") if gW is not None else None,
                             need_T=T is not None)
        torch.cuda.synchronize()
        out[key] = [x.double().cpu().numpy() if x is not None else None for x in g]
    for a, b in zip(out["tc"], out["d"]):
        if a is not None:
            assert rel_err(a, b) < 1e-4


@pytest.mark.parametrize("name", [w.name for w in W.SMALL] + ["c2_dp_n65536@192", "c0_dpbw_n2048"])
def test_fp64_double_float_ztransform(name, monkeypatch):
    """The FP64 operator's double-float z transform (FP32 pipes, compensated
    sums) against its FP64 transform: V, W to 1e-12; the backward pass too;
    and the reference fixtures (where one exists) to 1e-10."""
    import golden_io
    w = _wl(name)
    X, F, T = W.make_inputs(w)
    df = _op(w, "fp64", "df64", monkeypatch)
    info = df.info()
    assert info["ztransform"] == 2 and info["ztransform_inverse"] == 2, info
    fp = _op(w, "fp64", "simt", monkeypatch)
    assert fp.info()["ztransform"] == 0
    Va, Wa = _mdot(df, X, F, T, torch.float64)
    Vb, Wb = _mdot(fp, X, F, T, torch.float64)
    ev = rel_err(Va, Vb)
    print("%s df64-fp64 V %.2e (ms fp64 %.3f df64 %.3f)" % (name, ev, info["ztransform_ms"][0],
                                                           info["ztransform_ms"][1]))
    assert ev < 1e-12
    if T is not None:
        assert rel_err(Wa, Wb) < 1e-12
    g = np.random.default_rng(5).standard_normal(F.shape)
    grads = []
    for op in (df, fp):
        gF, _, gX = op.mdot_backward(torch.tensor(F, device="cuda"), torch.tensor(T, device="cuda") if T is not None
                                     else None, torch.tensor(g, device="cuda"), need_F=True, need_X=True)
        torch.cuda.synchronize()
        grads.append((gF.cpu().numpy(), gX.cpu().numpy()))
    assert rel_err(grads[0][0], grads[1][0]) < 1e-12 and rel_err(grads[0][1], grads[1][1]) < 1e-11
    if name in golden_io.names():
        _, _, _, _, gd = golden_io.inputs(name)
        er = rel_err(golden_io.restrict(gd, Va), gd["V"])
        print("%s df64 vs reference %.2e" % (name, er))
        assert er < 1e-10


def _variant(base, nz=None, nx=None, ny=None):
    from dataclasses import replace
    w = _wl(base)
    kw = {}
    if nz is not None:
        kw["nz"] = nz
    if nx is not None:
        kw.update(nx=nx, Lx=w.Lx * nx / w.nx)
    if ny is not None:
        kw.update(ny=ny, Ly=w.Ly * ny / w.ny)
    return replace(w, name="%s_nz%s" % (base, nz), **kw)


# (workload, nz): nz a multiple of 32, of 8, and neither (K padded, the last
# TMA block partly past nz); every geometry; partial last column tiles
TMA_CASES = [("c2_dp_n65536@192", None), ("c3_dpbw_n8192", None), ("s_dpsc_t", 37), ("s_dpbw_t_odd", 45),
             ("s_dp_t", 64), ("s_dpbw_t", 40)]


@pytest.mark.parametrize("base,nz", TMA_CASES)
def test_tma_ztransform_matches(base, nz, monkeypatch):
    """The TMA-fed tcgen05 z transform (T in tensor memory, blocks loaded and
    stored by cp.async.bulk.tensor) against the register-staged tcgen05
    transform (the same split products in the same order: 1e-6) and the FP64
    operator (1e-5), forward and backward."""
    w = _variant(base, nz) if nz else _wl(base)
    X, F, T = W.make_inputs(w)
    tm = _op(w, "mixed", "tma", monkeypatch)
    info = tm.info()
    assert info["ztransform"] == 3 and info["ztransform_inverse"] == 3, info
    tc = _op(w, "mixed", "tcgen05", monkeypatch)
    assert tc.info()["ztransform"] == 1
    f64 = _op(w, "fp64", "auto", monkeypatch)
    Vm, Wm = _mdot(tm, X, F, T, torch.float32)
    Vt, Wt = _mdot(tc, X, F, T, torch.float32)
    Vd, Wd = _mdot(f64, X, F, T, torch.float64)
    e_mt, e_md = rel_err(Vm, Vt), rel_err(Vm, Vd)
    print("%s nz %d tma-tc %.2e tma-fp64 %.2e (ms fwd tc %.3f tma %.3f, inv tc %.3f tma %.3f)" %
          (w.name, w.nz, e_mt, e_md, info["ztransform_ms"][1], info["ztransform_tma_ms"][0],
           info["ztransform_inverse_ms"][1], info["ztransform_tma_ms"][1]))
    print("  TMA variants (fwd 0-2, inv 0-2) ms", [round(x, 4) for x in info["ztransform_tma_variant_ms"]],
          "chosen", list(info["ztransform_tma_variant"]))
    assert e_mt < 1e-6 and e_md < 1e-5
    if T is not None:
        assert rel_err(Wm, Wt) < 1e-6 and rel_err(Wm, Wd) < 1e-5
    g = np.random.default_rng(7).standard_normal(F.shape)
    grads = []
    for op, dt in ((tm, torch.float32), (f64, torch.float64)):
        gF, _, gX = op.mdot_backward(torch.tensor(F, dtype=dt, device="cuda"),
                                     torch.tensor(T, dtype=dt, device="cuda") if T is not None else None,
                                     torch.tensor(g, dtype=dt, device="cuda"), need_F=True, need_X=True)
        torch.cuda.synchronize()
        grads.append((gF.double().cpu().numpy(), gX.double().cpu().numpy()))
    assert rel_err(grads[0][0], grads[1][0]) < 1e-5 and rel_err(grads[0][1], grads[1][1]) < 1e-4


@pytest.mark.parametrize("variant", [0, 1, 2])
def test_tma_ztransform_every_variant(variant, monkeypatch):
    """Each variant of the TMA-fed transform (ring and converted-stage
    counts), forced, against the register-staged tcgen05 transform."""
    w = _variant("s_dpbw_t", 45)
    X, F, T = W.make_inputs(w)
    monkeypatch.setenv("DPSTOKES_GB300_ZTMA_VARIANT", str(variant))
    tm = _op(w, "mixed", "tma", monkeypatch)
    monkeypatch.delenv("DPSTOKES_GB300_ZTMA_VARIANT")
    info = tm.info()
    assert info["ztransform"] == 3 and list(info["ztransform_tma_variant"]) == [variant, variant], info
    tc = _op(w, "mixed", "tcgen05", monkeypatch)
    Vm, Wm = _mdot(tm, X, F, T, torch.float32)
    Vt, Wt = _mdot(tc, X, F, T, torch.float32)
    assert rel_err(Vm, Vt) < 1e-6 and rel_err(Wm, Wt) < 1e-6


def test_tma_ztransform_unsupported_shape_falls_back(monkeypatch):
    """An odd number of modes (nx = 16, ny = 15: 9 x 15 = 135) gives rows that
    do not start on 16-byte boundaries: the TMA form is not chosen even when
    asked for, and the operator still matches FP64."""
    w = _variant("s_dp_t", 48, ny=15)
    X, F, T = W.make_inputs(w)
    tm = _op(w, "mixed", "tma", monkeypatch)
    info = tm.info()
    assert info["ztransform"] != 3 and info["ztransform_tma_ms"][0] == 0.0, info
    f64 = _op(w, "fp64", "auto", monkeypatch)
    Vm, _ = _mdot(tm, X, F, T, torch.float32)
    Vd, _ = _mdot(f64, X, F, T, torch.float64)
    assert rel_err(Vm, Vd) < 1e-5
