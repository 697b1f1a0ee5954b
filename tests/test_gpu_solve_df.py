"""The double-float per-wavenumber solve (DPST_SOLVE_DF64) against the FP64
solve.

The FP64 operator can run either solve with FP64 spectra in and out, which
isolates the solve's arithmetic: per wavenumber (kx, ky), the velocity
columns of the two runs (the velocity grid Fourier transformed in x and y,
all nz levels and three components, wall correction included) agree to
1e-12 relative to the column's own norm for the columns within 1e-2 of the
largest (5e-12 within 1e-3; every column within 5e-14 of the largest), and
V, W to 1e-12; the FP64
operator with the double-float solve still matches the reference's own
outputs to 1e-10.  The mixed operator (double-float solve by default) stays
within 5e-6 of the mixed operator with the FP64 solve (two mixed runs differ
at the FP32 level: the spreading's atomic sums run in another order on every
call) and within 1e-5 of the FP64 operator."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import golden_io  # noqa: E402
from conftest import rel_err  # noqa: E402
from doublyperiodicstokes_gb300 import DPStokes, StokesParams, workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu

CASES = [w.name for w in W.SMALL] + ["s_reg_dpbw_t", "s_dpbw_t_k3", "e_dpsc_t", "c0_dpbw_n2048",
                                     "c2_dp_n65536@64"]


def _wl(name):
    return W.SMALL_BY_NAME.get(name) or W.by_name(name)


def _run(w, precision, solve, X, F, T):
    prm = StokesParams.from_workload(w, precision)
    prm = StokesParams(**{**prm.as_dict(), "solve": solve})
    op = DPStokes(prm, w.N)
    d = op.device
    dt = torch.float64 if precision == "fp64" else torch.float32
    op.set_positions(torch.tensor(X, device=d))
    V, Wv = op.mdot(torch.tensor(F, dtype=dt, device=d), torch.tensor(T, dtype=dt, device=d) if T is not None else None)
    torch.cuda.synchronize()
    out = (V.double().cpu().numpy(), Wv.double().cpu().numpy() if Wv is not None else None,
           op.velocity_grid().double().cpu(), op.info()["solve_arith"])
    op.close()
    return out


@pytest.mark.parametrize("name", CASES)
def test_df64_solve_matches_fp64_solve_per_mode(name):
    w = _wl(name)
    X, F, T = W.make_inputs(w)
    V1, W1, g1, a1 = _run(w, "fp64", "fp64", X, F, T)
    V2, W2, g2, a2 = _run(w, "fp64", "df64", X, F, T)
    assert (a1, a2) == (1, 2)
    # per-wavenumber columns: [3][nz][ny][nx] -> x-y transform -> [ny][nxh][3 nz]
    c1 = torch.fft.rfft2(g1).permute(2, 3, 0, 1).reshape(w.ny, w.nx // 2 + 1, -1)
    c2 = torch.fft.rfft2(g2).permute(2, 3, 0, 1).reshape(w.ny, w.nx // 2 + 1, -1)
    n1 = torch.linalg.vector_norm(c1, dim=2)
    d = torch.linalg.vector_norm(c2 - c1, dim=2)
    nmax = float(n1.max())
    # the grid carries FP64 rounding of ~1e-16 of its largest values, which the
    # x-y transform spreads over every mode, and double-float rounds at 2^-48
    # (32 times FP64's unit): per-mode relative errors are bounded on the modes
    # within 1e-2 and 1e-3 of the largest, the rest against the largest
    big = n1 >= 1e-2 * nmax
    worst = float((d[big] / n1[big]).max())
    mid = n1 >= 1e-3 * nmax
    worst_mid = float((d[mid] / n1[mid]).max())
    worst_abs = float(d.max()) / nmax
    for lo, hi in ((1e-1, 1.1), (1e-2, 1e-1), (1e-3, 1e-2), (1e-5, 1e-3), (1e-8, 1e-5)):
        sel = (n1 >= lo * nmax) & (n1 < hi * nmax)
        if bool(sel.any()):
            print("  modes with norm in [%.0e, %.0e) of the largest: %5d, max rel err %.2e" %
                  (lo, hi, int(sel.sum()), float((d[sel] / n1[sel]).max())))
    ev, eg = rel_err(V2, V1), rel_err(g2.numpy(), g1.numpy())
    print("%s per-mode max %.2e (abs %.2e of the largest), grid %.2e, V %.2e" % (name, worst, worst_abs, eg, ev))
    assert worst < 1e-12
    assert worst_mid < 5e-12
    assert worst_abs < 5e-14
    assert ev < 1e-12
    if T is not None:
        assert rel_err(W2, W1) < 1e-12


@pytest.mark.parametrize("name", [n for n in golden_io.names() if n.startswith(("s_d", "e_d", "c0", "c1", "c2"))])
def test_fp64_operator_with_df64_solve_matches_reference(name):
    w, X, F, T, g = golden_io.inputs(name)
    V, Wv, _, _ = _run(w, "fp64", "df64", X, F, T)
    assert rel_err(golden_io.restrict(g, V), g["V"]) < 1e-10
    if w.has_torque:
        assert rel_err(golden_io.restrict(g, Wv), g["W"]) < 1e-10


@pytest.mark.parametrize("name", ["s_dpbw_t", "s_dp_t", "s_dpsc_t", "c1_dpsc_n16384", "c2_dp_n65536@192"])
def test_mixed_default_solve_is_df64(name):
    w = _wl(name)
    X, F, T = W.make_inputs(w)
    Vd, Wd, _, ad = _run(w, "mixed", "default", X, F, T)
    Vf, Wf, _, af = _run(w, "mixed", "fp64", X, F, T)
    V6, W6, _, _ = _run(w, "fp64", "fp64", X, F, T)
    assert (ad, af) == (2, 1)
    e1, e2 = rel_err(Vd, Vf), rel_err(Vd, V6)
    print("%s mixed df64 vs mixed fp64 solve %.2e, vs fp64 operator %.2e" % (name, e1, e2))
    assert e1 < 5e-6 and e2 < 1e-5
    if T is not None:
        assert rel_err(Wd, Wf) < 5e-6 and rel_err(Wd, W6) < 1e-5


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_every_solve_variant(variant, monkeypatch):
    """Each kernel variant of the double-float solve (the creation-time tuner
    picks one): the mixed operator against its FP64-solve form."""
    monkeypatch.setenv("DPSTOKES_GB300_SOLVE_VARIANT", str(variant))
    for name in ("s_dpsc_t", "s_dp_t", "c2_dp_n65536@64"):
        w = _wl(name)
        X, F, T = W.make_inputs(w)
        prm = StokesParams.from_workload(w, "mixed")
        op = DPStokes(prm, w.N)
        assert op.info()["solve_variant"] == variant
        op.close()
        Vd, Wd, _, _ = _run(w, "mixed", "df64", X, F, T)
        Vf, Wf, _, _ = _run(w, "mixed", "fp64", X, F, T)
        # two mixed handles differ at the FP32 level (the spreading's atomic
        # sums run in another order on every call)
        assert rel_err(Vd, Vf) < 5e-6 and rel_err(Wd, Wf) < 5e-6


@pytest.mark.parametrize("dom", ["DPBW", "DP", "DPSC"])
def test_batched_systems_df64_solve(dom):
    """The batched double-float solve (one launch over every system's modes):
    FP64 systems with it against the FP64 solve to 1e-12, and the mixed batch
    (double-float by default) against single mixed handles to 5e-6."""
    from doublyperiodicstokes_gb300 import DPStokesBatch
    ws = W.small_batch(dom, True)
    Xs, Fs, Ts = zip(*[W.make_inputs(w) for w in ws])
    cat = lambda a, dt: torch.tensor(np.concatenate(a), dtype=dt, device="cuda")  # noqa: E731

    def batch(precision, solve):
        prm = [StokesParams(**{**StokesParams.from_workload(w, precision).as_dict(), "solve": solve}) for w in ws]
        b = DPStokesBatch(prm, [w.N for w in ws])
        dt = torch.float64 if precision == "fp64" else torch.float32
        b.set_positions(cat(Xs, torch.float64))
        V, Wv = b.mdot(cat(Fs, dt), cat(Ts, dt))
        torch.cuda.synchronize()
        out = V.double().cpu().numpy(), Wv.double().cpu().numpy()
        b.close()
        return out

    V1, W1 = batch("fp64", "fp64")
    V2, W2 = batch("fp64", "df64")
    assert rel_err(V2, V1) < 1e-12 and rel_err(W2, W1) < 1e-12
    Vm, Wm = batch("mixed", "default")
    Vs = np.concatenate([_run(w, "mixed", "default", X, F, T)[0] for w, X, F, T in zip(ws, Xs, Fs, Ts)])
    assert rel_err(Vm, Vs) < 5e-6


def test_multi_column_df64_solve():
    """The multi-column Mdot with the batched double-float solve against
    single-column calls (mixed, 5e-6) and against its FP64-solve form."""
    w = _wl("c2_dp_n65536@64")
    X, F, T = W.make_inputs(w)
    rng = np.random.default_rng(5)
    K = 3
    Fk = rng.standard_normal((K, w.N, 3)).astype(np.float32)
    Tk = rng.standard_normal((K, w.N, 3)).astype(np.float32)
    res = {}
    for solve in ("default", "fp64"):
        prm = StokesParams(**{**StokesParams.from_workload(w, "mixed").as_dict(), "solve": solve})
        op = DPStokes(prm, w.N)
        op.set_positions(torch.tensor(X, device=op.device))
        Vk, Wk = op.mdot_multi(torch.tensor(Fk, device=op.device), torch.tensor(Tk, device=op.device))
        singles = [op.mdot(torch.tensor(Fk[k], device=op.device), torch.tensor(Tk[k], device=op.device))
                   for k in range(K)]
        torch.cuda.synchronize()
        for k in range(K):
            assert rel_err(Vk[k].double().cpu().numpy(), singles[k][0].double().cpu().numpy()) < 5e-6
            assert rel_err(Wk[k].double().cpu().numpy(), singles[k][1].double().cpu().numpy()) < 5e-6
        res[solve] = Vk.double().cpu().numpy()
        op.close()
    assert rel_err(res["default"], res["fp64"]) < 5e-6


@pytest.mark.parametrize("name", ["s_dpbw_t", "s_dp_t", "s_dpsc_t", "s_dpbw_t_odd", "s_dpsc_f_odd", "e_dp_t_shift",
                                  "c2_dp_n65536@64"])
def test_adjoint_df64_solve(name):
    """The backward pass with the double-float adjoint solve (FP64 I/O)
    against the FP64 adjoint (dl/dF, dl/dT, dl/dX to 1e-11), and its
    transpose identity <gV, V> + <gW, W> = <dl/dF, F> + <dl/dT, T>."""
    w = _wl(name)
    X, F, T = W.make_inputs(w)
    rng = np.random.default_rng(11)
    gV = rng.standard_normal(F.shape)
    gW = rng.standard_normal(F.shape) if T is not None else None
    out = {}
    for solve in ("fp64", "df64"):
        prm = StokesParams(**{**StokesParams.from_workload(w, "fp64").as_dict(), "solve": solve})
        op = DPStokes(prm, w.N)
        d = op.device
        op.set_positions(torch.tensor(X, device=d))
        Ft = torch.tensor(F, device=d)
        Tt = torch.tensor(T, device=d) if T is not None else None
        V, Wv = op.mdot(Ft, Tt)
        gF, gT, gX = op.mdot_backward(Ft, Tt, torch.tensor(gV, device=d),
                                      torch.tensor(gW, device=d) if gW is not None else None,
                                      need_F=True, need_T=T is not None, need_X=True)
        torch.cuda.synchronize()
        out[solve] = [None if a is None else a.cpu().numpy() for a in (V, Wv, gF, gT, gX)]
        op.close()
    V, Wv, gF, gT, gX = out["df64"]
    for a, b in zip(out["df64"][2:], out["fp64"][2:]):
        if a is not None:
            assert rel_err(a, b) < 1e-11
    lhs = np.sum(gV * V) + (np.sum(gW * Wv) if gW is not None else 0.0)
    rhs = np.sum(gF * F) + (np.sum(gT * T) if T is not None else 0.0)
    scale = np.sqrt(np.sum(gV * gV) * np.sum(V * V))
    print("%s transpose identity %.2e" % (name, abs(lhs - rhs) / scale))
    assert abs(lhs - rhs) < 1e-12 * scale


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_mixed_adjoint_every_variant(variant, monkeypatch):
    """The mixed operator's backward with each double-float adjoint variant
    (DPSTOKES_GB300_SOLVE_VARIANT) against the FP64 backward: dl/dF 1e-5,
    dl/dX 1e-4, on a bottom-wall case with torques."""
    w = _wl("c2_dp_n65536@64")
    X, F, T = W.make_inputs(w)
    rng = np.random.default_rng(21)
    gV = rng.standard_normal(F.shape)
    gW = rng.standard_normal(F.shape)
    res = {}
    for prec in ("fp64", "mixed"):
        if prec == "mixed":
            monkeypatch.setenv("DPSTOKES_GB300_SOLVE_VARIANT", str(variant))
        op = DPStokes(StokesParams.from_workload(w, prec), w.N)
        dt = torch.float64 if prec == "fp64" else torch.float32
        d = op.device
        op.set_positions(torch.tensor(X, device=d))
        out = op.mdot_backward(torch.tensor(F, dtype=dt, device=d), torch.tensor(T, dtype=dt, device=d),
                               torch.tensor(gV, dtype=dt, device=d), torch.tensor(gW, dtype=dt, device=d),
                               need_F=True, need_T=True, need_X=True)
        torch.cuda.synchronize()
        res[prec] = [a.double().cpu().numpy() for a in out]
        op.close()
        monkeypatch.delenv("DPSTOKES_GB300_SOLVE_VARIANT", raising=False)
    e = [rel_err(a, b) for a, b in zip(res["mixed"], res["fp64"])]
    print("variant %d mixed vs fp64 backward %s" % (variant, " ".join("%.2e" % x for x in e)))
    assert e[0] < 1e-5 and e[1] < 1e-5 and e[2] < 1e-4
