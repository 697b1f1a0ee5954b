"""Backward pass of Mdot on the GPU (dpst_mdot_backward and the autograd
wrapper doublyperiodicstokes_gb300.mdot).

For l = <gV, V> + <gW, W> with (V, W) = M(X) (F, T):
  * transpose identity <gV, V> + <gW, W> = <dl/dF, F> + <dl/dT, T> on every
    small case (each geometry including the triply periodic mode, torques,
    ghost-layer reuse at open ends, odd grids), FP64, to 1e-12 of the terms'
    scale;
  * dl/dF, dl/dT against the oracle's M^T g assembled column by column from
    the oracle's own forward (which matches the reference to ~1e-15), 1e-10;
  * dl/dX against central differences of the oracle's forward (step 1e-6),
    1e-6 relative (2-norm);
  * the autograd wrapper against the direct call, taking the forward's
    velocity grid from the handle (dpst_mdot_backward_saved);
  * the backward on a held forward grid against the recomputing backward
    (FP64 1e-13, mixed 5e-6: two runs of FP32 atomics), in every geometry
    and the triply periodic mode, and the serial's invalidation by position
    updates and multi-column Mdots;
  * the mixed-precision backward against the FP64 one;
  * the differentiation configuration (bottom wall, N = 8192, 192^2 x 64):
    transpose identity, sampled entries of M^T g from the FP64 forward and
    central differences for sampled coordinates.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import dpstokes_oracle as O  # noqa: E402
from conftest import rel_err  # noqa: E402
from doublyperiodicstokes_gb300 import DPStokes, StokesParams, mdot, workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu
FD_STEP = 1e-6


def _op(w, precision="fp64", n=None):
    return DPStokes(StokesParams.from_workload(w, precision), w.N if n is None else n)


def _dev(a, dtype=torch.float64):
    return None if a is None else torch.tensor(a, dtype=dtype, device="cuda")


def _np(t):
    return None if t is None else t.double().cpu().numpy()


def _grads(op, X, F, T, gV, gW, dtype=torch.float64, need_X=True):
    op.set_positions(_dev(X))
    gF, gT, gX = op.mdot_backward(_dev(F, dtype), _dev(T, dtype), _dev(gV, dtype), _dev(gW, dtype),
                                  need_F=True, need_T=T is not None, need_X=need_X)
    torch.cuda.synchronize()
    return _np(gF), _np(gT), _np(gX)


def _cotangents(w, seed=11):
    rng = np.random.default_rng(seed)
    gV = rng.standard_normal((w.N, 3))
    gW = rng.standard_normal((w.N, 3)) if w.has_torque else None
    return gV, gW


def _loss(V, Wv, gV, gW):
    l = float(np.sum(gV * np.reshape(V, gV.shape)))
    if gW is not None:
        l += float(np.sum(gW * np.reshape(Wv, gW.shape)))
    return l


@pytest.mark.parametrize("name", [w.name for w in W.SMALL + W.SMALL_TP])
def test_transpose_identity(name):
    w = W.SMALL_BY_NAME[name]
    X, F, T = W.make_inputs(w)
    gV, gW = _cotangents(w)
    op = _op(w)
    op.set_positions(_dev(X))
    V, Wv = op.mdot(_dev(F), _dev(T))
    V, Wv = _np(V), _np(Wv)
    gF, gT, _ = _grads(op, X, F, T, gV, gW, need_X=False)
    lhs = _loss(V, Wv, gV, gW)
    rhs = float(np.sum(gF * F)) + (float(np.sum(gT * T)) if T is not None else 0.0)
    scale = np.linalg.norm(gV) * np.linalg.norm(V) + (np.linalg.norm(gW) * np.linalg.norm(Wv)
                                                      if gW is not None else 0.0)
    print("%s <g,MF> %.15e <M^T g,F> %.15e rel %.2e" % (name, lhs, rhs, abs(lhs - rhs) / scale))
    assert abs(lhs - rhs) <= 1e-12 * scale


def _oracle_vjp(w, X, F, T, gV, gW):
    """M^T g from the oracle's forward, one column per input component."""
    o = O.Oracle(O.Params(**w.oracle_params()))
    o.set_positions(X)
    N = w.N
    zF = np.zeros((N, 3))
    gF = np.zeros((N, 3))
    gT = np.zeros((N, 3)) if T is not None else None
    for p in range(N):
        for d in range(3):
            e = np.zeros((N, 3))
            e[p, d] = 1.0
            V, Wv = o.mdot(e, zF if T is not None else None)
            gF[p, d] = _loss(V, Wv, gV, gW)
            if T is not None:
                V, Wv = o.mdot(zF, e)
                gT[p, d] = _loss(V, Wv, gV, gW)
    return gF, gT


def _oracle_fd(w, X, F, T, gV, gW, coords=None, h=FD_STEP):
    o = O.Oracle(O.Params(**w.oracle_params()))
    gX = np.zeros((w.N, 3))
    coords = [(p, d) for p in range(w.N) for d in range(3)] if coords is None else coords
    for p, d in coords:
        vals = []
        for s in (1.0, -1.0):
            Xs = X.copy()
            Xs[p, d] += s * h
            o.set_positions(Xs)
            V, Wv = o.mdot(F, T)
            vals.append(_loss(V, Wv, gV, gW))
        gX[p, d] = (vals[0] - vals[1]) / (2 * h)
    return gX


@pytest.mark.parametrize("name", [w.name for w in W.SMALL + W.SMALL_TP])
def test_gradients_match_oracle(name):
    w = W.SMALL_BY_NAME[name]
    X, F, T = W.make_inputs(w)
    gV, gW = _cotangents(w)
    gF, gT, gX = _grads(_op(w), X, F, T, gV, gW)
    oF, oT = _oracle_vjp(w, X, F, T, gV, gW)
    oX = _oracle_fd(w, X, F, T, gV, gW)
    eF = rel_err(gF, oF)
    eT = rel_err(gT, oT) if T is not None else 0.0
    eX = rel_err(gX, oX)
    print("%s dF %.2e dT %.2e dX %.2e (|dX| %.3e)" % (name, eF, eT, eX, np.linalg.norm(oX)))
    assert eF < 1e-10
    assert eT < 1e-10
    assert eX < 1e-6


def test_autograd_matches_direct():
    w = W.SMALL_BY_NAME["s_dpbw_t"]
    X, F, T = W.make_inputs(w)
    gV, gW = _cotangents(w)
    op = _op(w)
    Xt = _dev(X).requires_grad_(True)
    Ft = _dev(F).requires_grad_(True)
    Tt = _dev(T).requires_grad_(True)
    V, Wv = mdot(op, Xt, Ft, Tt)
    l = (V * _dev(gV)).sum() + (Wv * _dev(gW)).sum()
    l.backward()
    assert op.last_backward_reused
    dF, dT, dX = _grads(op, X, F, T, gV, gW)
    # equal up to the order of the spreading's atomic sums
    assert rel_err(_np(Ft.grad), dF) < 1e-12
    assert rel_err(_np(Tt.grad), dT) < 1e-12
    assert rel_err(_np(Xt.grad), dX) < 1e-12


@pytest.mark.parametrize("name", ["s_dpbw_t", "s_dp_t", "s_dpsc_t", "s_dpbw_f_top", "s_tp_t"])
def test_mixed_backward_matches_fp64(name):
    w = W.SMALL_BY_NAME[name]
    X, F, T = W.make_inputs(w)
    gV, gW = _cotangents(w)
    d64 = _grads(_op(w), X, F, T, gV, gW)
    d32 = _grads(_op(w, "mixed"), X, F, T, gV, gW, dtype=torch.float32)
    errs = [rel_err(a, b) for a, b in zip(d32, d64) if a is not None]
    print("%s mixed vs fp64: %s" % (name, " ".join("%.2e" % e for e in errs)))
    assert errs[0] < 1e-5  # dl/dF
    assert errs[-1] < 1e-4  # dl/dX


def test_differentiation_config():
    """Bottom wall, N = 8192, 192 x 192 x 64, forces only; l = <g, M(X) F>."""
    w = W.C3
    X, F, _ = W.make_inputs(w)
    gV, _ = _cotangents(w, seed=12)
    op = _op(w)
    Xd, Fd, gVd = _dev(X), _dev(F), _dev(gV)
    op.set_positions(Xd)
    V, _ = op.mdot(Fd)
    gF, _, gX = op.mdot_backward(Fd, None, gVd)
    V, gF, gX = _np(V), _np(gF), _np(gX)
    lhs, rhs = float(np.sum(gV * V)), float(np.sum(gF * F))
    scale = np.linalg.norm(gV) * np.linalg.norm(V)
    print("c3 transpose rel %.2e" % (abs(lhs - rhs) / scale))
    assert abs(lhs - rhs) <= 1e-12 * scale
    rng = np.random.default_rng(5)
    # sampled entries of M^T g from the forward: (M^T g)_j = <g, M e_j>
    for j in rng.choice(3 * w.N, 4, replace=False):
        e = torch.zeros_like(Fd)
        e.view(-1)[j] = 1.0
        Vj, _ = op.mdot(e)
        ref = float((gVd * Vj).sum())
        assert abs(gF.reshape(-1)[j] - ref) <= 1e-10 * max(abs(ref), 1e-3 * np.abs(gF).max())
    # central differences for sampled coordinates (lowest and highest
    # particles, whose kernels reach the wall and the open top, and random)
    zs = np.argsort(X[:, 2])
    picks = [(int(zs[0]), 2), (int(zs[-1]), 2), (int(zs[-1]), 0)]
    picks += [(int(p), int(d)) for p, d in zip(rng.choice(w.N, 5), rng.integers(0, 3, 5))]
    for p, d in picks:
        vals = []
        for s in (1.0, -1.0):
            Xs = X.copy()
            Xs[p, d] += s * FD_STEP
            op.set_positions(_dev(Xs))
            Vs, _ = op.mdot(Fd)
            vals.append(float((gVd * Vs).sum()))
        fd = (vals[0] - vals[1]) / (2 * FD_STEP)
        print("c3 dX[%d,%d] %.10e fd %.10e" % (p, d, gX[p, d], fd))
        assert abs(gX[p, d] - fd) <= 1e-6 * np.abs(gX).max()


@pytest.mark.parametrize("name,precision", [("s_dpbw_t", "fp64"), ("s_dp_t", "fp64"), ("s_dpsc_t", "fp64"),
                                            ("s_dpbw_f_top", "fp64"), ("s_tp_t", "fp64"), ("s_dpbw_t", "mixed"),
                                            ("s_tp_t", "mixed")])
def test_backward_on_held_forward_grid(name, precision):
    w = W.SMALL_BY_NAME[name]
    X, F, T = W.make_inputs(w)
    gV, gW = _cotangents(w)
    dt = torch.float64 if precision == "fp64" else torch.float32
    op = _op(w, precision)
    op.set_positions(_dev(X))
    assert op.forward_serial() == 0
    Fd, Td, gVd, gWd = _dev(F, dt), _dev(T, dt), _dev(gV, dt), _dev(gW, dt)
    ref = [_np(a) for a in op.mdot_backward(Fd, Td, gVd, gWd, need_F=True, need_T=T is not None, need_X=True)]
    assert not op.last_backward_reused
    op.mdot(Fd, Td)
    serial = op.forward_serial()
    assert serial != 0
    for _ in range(2):  # the held grid stays valid across backward calls
        got = [_np(a) for a in op.mdot_backward(Fd, Td, gVd, gWd, need_F=True, need_T=T is not None, need_X=True,
                                                forward_serial=serial)]
        assert op.last_backward_reused
        tol = 1e-13 if precision == "fp64" else 5e-6
        for a, b in zip(got, ref):
            if b is not None:
                assert rel_err(a, b) < tol
    # a position update forgets the held grid; a stale serial recomputes
    op.set_positions(_dev(X))
    assert op.forward_serial() == 0
    got = [_np(a) for a in op.mdot_backward(Fd, Td, gVd, gWd, need_F=True, need_T=T is not None, need_X=True,
                                            forward_serial=serial)]
    assert not op.last_backward_reused
    assert rel_err(got[-1], ref[-1]) < (1e-13 if precision == "fp64" else 5e-6)
    # a multi-column Mdot forgets it too
    op.mdot(Fd, Td)
    s2 = op.forward_serial()
    assert s2 > serial
    Fk = Fd.reshape(1, w.N, 3).repeat(2, 1, 1).contiguous()
    op.mdot_multi(Fk, Td.reshape(1, w.N, 3).repeat(2, 1, 1).contiguous() if Td is not None else None)
    assert op.forward_serial() == 0
    op.mdot_backward(Fd, Td, gVd, gWd, need_F=True, need_X=True, forward_serial=s2)
    assert not op.last_backward_reused
    op.close()
