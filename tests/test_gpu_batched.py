"""Batched systems (dpst_batched_*, DPStokesBatch) on the GPU: every
system's V, W from the one-pipeline batch against the single-system
operator on the same inputs (FP64: 1e-12, equal up to the order of atomic
sums; mixed: 1e-6), one system against the oracle (1e-10), and a sample of
the 256-system bottom-wall configuration (mixed)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import dpstokes_oracle as O  # noqa: E402
from conftest import rel_err  # noqa: E402
from doublyperiodicstokes_gb300 import DPStokes, DPStokesBatch, StokesParams, _lib, workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu


def _inputs(ws, dtype):
    Xs, Fs, Ts = [], [], []
    for w in ws:
        X, F, T = W.make_inputs(w)
        Xs.append(X)
        Fs.append(F)
        Ts.append(T)
    cat = lambda a: torch.tensor(np.concatenate(a), dtype=dtype, device="cuda")  # noqa: E731
    return Xs, Fs, Ts, cat(Xs).double(), cat(Fs), (cat(Ts) if Ts[0] is not None else None)


class _ZTransform:
    """DPSTOKES_GB300_ZTRANSFORM for the handles created inside: batch and
    single handles compare like with like (the tensor-core transform differs
    from the SIMT one by ~1e-6, covered elsewhere)."""

    def __init__(self, which):
        self.which = which

    def __enter__(self):
        import os
        self.old = os.environ.get("DPSTOKES_GB300_ZTRANSFORM")
        if self.which:
            os.environ["DPSTOKES_GB300_ZTRANSFORM"] = self.which

    def __exit__(self, *exc):
        import os
        if self.old is None:
            os.environ.pop("DPSTOKES_GB300_ZTRANSFORM", None)
        else:
            os.environ["DPSTOKES_GB300_ZTRANSFORM"] = self.old


def _single(w, X, F, T, precision, dtype, zt="simt"):
    with _ZTransform(zt):
        op = DPStokes(StokesParams.from_workload(w, precision), w.N)
    op.set_positions(torch.tensor(X, device="cuda"))
    V, Wv = op.mdot(torch.tensor(F, dtype=dtype, device="cuda"),
                    torch.tensor(T, dtype=dtype, device="cuda") if T is not None else None)
    torch.cuda.synchronize()
    out = (V.double().cpu().numpy(), Wv.double().cpu().numpy() if Wv is not None else None)
    op.close()
    return out


def _run_batch(ws, precision, dtype, zt="simt"):
    with _ZTransform(zt):
        b = DPStokesBatch([StokesParams.from_workload(w, precision) for w in ws], [w.N for w in ws])
    Xs, Fs, Ts, X, F, T = _inputs(ws, dtype)
    b.set_positions(X)
    V, Wv = b.mdot(F, T)
    V2, W2 = b.mdot(F, T)  # graph replay
    torch.cuda.synchronize()
    Vs = [v.double().cpu().numpy() for v in b.split(V)]
    Ws = [v.double().cpu().numpy() for v in b.split(Wv)] if Wv is not None else None
    # replays agree up to the order of the spreading's atomic sums
    assert rel_err(V2.double().cpu().numpy(), V.double().cpu().numpy()) < (1e-12 if precision == "fp64" else 1e-6)
    return b, Xs, Fs, Ts, Vs, Ws


@pytest.mark.parametrize("dom,torque", [("DPBW", True), ("DP", True), ("DPSC", False), ("DPBW", False)])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_matches_single(dom, torque, precision):
    ws = W.small_batch(dom, torque)
    dtype = torch.float64 if precision == "fp64" else torch.float32
    b, Xs, Fs, Ts, Vs, Ws = _run_batch(ws, precision, dtype)
    info = b.info()
    assert info["n_systems"] == len(ws) and info["n_size_classes"] == 4
    tol = 1e-12 if precision == "fp64" else 1e-6
    for k, w in enumerate(ws):
        V1, W1 = _single(w, Xs[k], Fs[k], Ts[k], precision, dtype)
        ev = rel_err(Vs[k], V1)
        ew = rel_err(Ws[k], W1) if torque else 0.0
        print("%s %s V %.2e W %.2e" % (w.name, precision, ev, ew))
        assert ev < tol and ew < tol
    b.close()


def test_batched_system_matches_oracle():
    ws = W.small_batch("DPBW", True)
    b, Xs, Fs, Ts, Vs, Ws = _run_batch(ws, "fp64", torch.float64)
    k = 4  # the non-square grid
    Vo, Wo = O.mdot(O.Params(**ws[k].oracle_params()), Xs[k], Fs[k], Ts[k])
    assert rel_err(Vs[k], Vo) < 1e-10
    assert rel_err(Ws[k], Wo) < 1e-10
    b.close()


def test_batched_rejects_mismatched_systems():
    ws = W.small_batch("DPBW", False)
    ps = [StokesParams.from_workload(w) for w in ws]
    ps[2].nz = ps[2].nz + 1
    with pytest.raises(_lib.DPStokesError) as e:
        DPStokesBatch(ps, [w.N for w in ws])
    assert e.value.code == 1


def test_batched_c4_sample():
    """256 bottom-wall systems, N_i log-uniform in [64, 4096], L_i in
    [32, 128], mixed precision: sampled systems against the single operator."""
    ws = W.batched_c4()
    b, Xs, Fs, Ts, Vs, Ws = _run_batch(ws, "mixed", torch.float32)
    print(b.info())
    rng = np.random.default_rng(3)
    for k in rng.choice(len(ws), 6, replace=False):
        V1, _ = _single(ws[k], Xs[k], Fs[k], None, "mixed", torch.float32)
        e = rel_err(Vs[k], V1)
        print("%s N %d n %d: %.2e" % (ws[k].name, ws[k].N, ws[k].nx, e))
        assert e < 1e-6
    b.close()


@pytest.mark.parametrize("dom,torque", [("DPBW", True), ("DP", True), ("DPSC", False)])
def test_batched_tensor_core_ztransform(dom, torque):
    """The batch's tcgen05 z transform over all systems (one launch, tiles of
    every system): against single handles on the tcgen05 transform (1e-6),
    and against the FP64 batch (1e-5); the creation-time choice is reported."""
    ws = W.small_batch(dom, torque)
    b, Xs, Fs, Ts, Vs, Ws = _run_batch(ws, "mixed", torch.float32, zt="tcgen05")
    info = b.info()
    assert info["ztransform"] == 1 and info["ztransform_inverse"] == 1
    b64, _, _, _, V64, W64 = _run_batch(ws, "fp64", torch.float64)
    for k, w in enumerate(ws):
        V1, W1 = _single(w, Xs[k], Fs[k], Ts[k], "mixed", torch.float32, zt="tcgen05")
        ev = rel_err(Vs[k], V1)
        ew = rel_err(Ws[k], W1) if torque else 0.0
        e64 = rel_err(Vs[k], V64[k])
        print("%s tcgen05 V %.2e W %.2e vs fp64 %.2e" % (w.name, ev, ew, e64))
        # two FP32 runs (atomic order of the spreading, tile schedule of the
        # transforms): V within 1e-6, the vorticity within 2e-6
        assert ev < 1e-6 and ew < 2e-6 and e64 < 1e-5
    b.close()
    b64.close()
    b2, _, _, _, Va, _ = _run_batch(ws, "mixed", torch.float32, zt=None)
    info = b2.info()
    print("auto choice", info["ztransform"], info["ztransform_inverse"], list(info["ztransform_ms"]),
          list(info["ztransform_inverse_ms"]))
    for k in range(len(ws)):
        assert rel_err(Va[k], V64[k]) < 1e-5
    b2.close()


@pytest.mark.parametrize("dom,torque,nz", [("DPBW", True, 40), ("DP", True, 64), ("DPSC", False, 45)])
def test_batched_tma_ztransform(dom, torque, nz):
    """The batch's TMA-fed tcgen05 z transform (every system's spectrum
    through its own tensor maps, one launch): against single handles on the
    register-staged tcgen05 transform (1e-6 for V, 2e-6 for the vorticity)
    and against the FP64 batch (1e-5)."""
    from dataclasses import replace
    ws = [replace(w, nz=nz) for w in W.small_batch(dom, torque)]
    b, Xs, Fs, Ts, Vs, Ws = _run_batch(ws, "mixed", torch.float32, zt="tma")
    info = b.info()
    assert info["ztransform"] == 3 and info["ztransform_inverse"] == 3, info
    b64, _, _, _, V64, _ = _run_batch(ws, "fp64", torch.float64)
    for k, w in enumerate(ws):
        V1, W1 = _single(w, Xs[k], Fs[k], Ts[k], "mixed", torch.float32, zt="tcgen05")
        ev = rel_err(Vs[k], V1)
        ew = rel_err(Ws[k], W1) if torque else 0.0
        e64 = rel_err(Vs[k], V64[k])
        print("%s nz %d tma V %.2e W %.2e vs fp64 %.2e" % (w.name, nz, ev, ew, e64))
        assert ev < 1e-6 and ew < 2e-6 and e64 < 1e-5
    b.close()
    b64.close()


def test_batched_tma_ztransform_mixed_alignment():
    """Systems whose spectrum rows do not start on 16-byte boundaries (an odd
    mode count: nx = 16, ny = 15 gives 9 x 15) beside ones that do: the TMA
    launch takes the latter, the register-staged launch the former, and
    every system matches its single handle."""
    from dataclasses import replace
    ws = [replace(w, nz=48) for w in W.small_batch("DPBW", True)]
    ws[1] = replace(ws[1], nx=16, ny=15, Lx=16.0, Ly=15.0)
    b, Xs, Fs, Ts, Vs, Ws = _run_batch(ws, "mixed", torch.float32, zt="tma")
    info = b.info()
    assert info["ztransform"] == 3 and info["ztransform_inverse"] == 3, info
    for k, w in enumerate(ws):
        V1, W1 = _single(w, Xs[k], Fs[k], Ts[k], "mixed", torch.float32, zt="tcgen05")
        assert rel_err(Vs[k], V1) < 1e-6 and rel_err(Ws[k], W1) < 2e-6
    b.close()
