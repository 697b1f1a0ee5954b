"""Multi-RHS Mdot (dpst_mdot_multi, DPStokes.mdot_multi) on the GPU: K force
(and torque) columns at the same positions against K single dpst_mdot calls
on the same handle (FP64: 1e-12, equal up to the order of the spreading's
atomic sums; mixed: 1e-6), one column against the oracle (FP64, 1e-10), on
small cases covering every geometry, torques and the open-end ghost layers;
buffer reuse with a smaller K and a position change between calls; the
argument errors."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import dpstokes_oracle as O  # noqa: E402
from conftest import rel_err  # noqa: E402
from doublyperiodicstokes_gb300 import DPStokes, StokesParams, _lib, workloads as W  # noqa: E402
from doublyperiodicstokes_gb300._lib import DPStokesError  # noqa: E402

pytestmark = pytest.mark.gpu


def _columns(w, K, seed=21):
    rng = np.random.default_rng(seed)
    F = rng.standard_normal((K, w.N, 3))
    T = rng.standard_normal((K, w.N, 3)) if w.has_torque else None
    return F, T


def _singles(op, F, T, dtype):
    Vs, Ws = [], []
    for k in range(F.shape[0]):
        V, Wv = op.mdot(torch.tensor(F[k], dtype=dtype, device="cuda"),
                        torch.tensor(T[k], dtype=dtype, device="cuda") if T is not None else None)
        Vs.append(V.double().cpu().numpy())
        Ws.append(Wv.double().cpu().numpy() if Wv is not None else None)
    return Vs, Ws


def _multi(op, F, T, dtype):
    V, Wv = op.mdot_multi(torch.tensor(F, dtype=dtype, device="cuda"),
                          torch.tensor(T, dtype=dtype, device="cuda") if T is not None else None)
    torch.cuda.synchronize()
    return V.double().cpu().numpy(), (Wv.double().cpu().numpy() if Wv is not None else None)


@pytest.mark.parametrize("name", ["s_dpbw_t", "s_dp_t", "s_dpsc_t", "s_dpbw_f_top", "s_dp_f_ends"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_multi_matches_single_columns(name, precision):
    w = W.SMALL_BY_NAME[name]
    X, _, _ = W.make_inputs(w)
    dtype = torch.float64 if precision == "fp64" else torch.float32
    tol = 1e-12 if precision == "fp64" else 1e-6
    op = DPStokes(StokesParams.from_workload(w, precision), w.N)
    op.set_positions(torch.tensor(X, device="cuda"))
    K = 3
    F, T = _columns(w, K)
    Vm, Wm = _multi(op, F, T, dtype)
    Vs, Ws = _singles(op, F, T, dtype)
    for k in range(K):
        ev = rel_err(Vm[k], Vs[k])
        print("%s %s column %d V %.2e" % (name, precision, k, ev))
        assert ev < tol
        if T is not None:
            assert rel_err(Wm[k], Ws[k]) < tol
    op.close()


def test_multi_column_matches_oracle():
    w = W.SMALL_BY_NAME["s_dpbw_t"]
    X, _, _ = W.make_inputs(w)
    op = DPStokes(StokesParams.from_workload(w), w.N)
    op.set_positions(torch.tensor(X, device="cuda"))
    F, T = _columns(w, 2, seed=5)
    Vm, Wm = _multi(op, F, T, torch.float64)
    for k in range(2):
        Vo, Wo = O.mdot(O.Params(**w.oracle_params()), X, F[k], T[k])
        assert rel_err(Vm[k], Vo) < 1e-10
        assert rel_err(Wm[k], Wo) < 1e-10
    op.close()


def test_multi_reuse_smaller_k_and_new_positions():
    w = W.SMALL_BY_NAME["s_dpbw_f_top"]
    X, _, _ = W.make_inputs(w)
    op = DPStokes(StokesParams.from_workload(w), w.N)
    op.set_positions(torch.tensor(X, device="cuda"))
    F, T = _columns(w, 4, seed=7)
    _multi(op, F, T, torch.float64)  # buffers for K = 4
    Vm, _ = _multi(op, F[:2], None, torch.float64)
    Vs, _ = _singles(op, F[:2], None, torch.float64)
    for k in range(2):
        assert rel_err(Vm[k], Vs[k]) < 1e-12
    # move every particle towards the open top: the ghost layers grow
    X2 = X.copy()
    X2[:, 2] = np.minimum(X2[:, 2] + 2.0, w.Lz - 0.05)
    op.set_positions(torch.tensor(X2, device="cuda"))
    Vm, _ = _multi(op, F[:3], None, torch.float64)
    Vs, _ = _singles(op, F[:3], None, torch.float64)
    for k in range(3):
        assert rel_err(Vm[k], Vs[k]) < 1e-12
    op.close()


def test_multi_argument_errors():
    w = W.SMALL_BY_NAME["s_dp_t"]
    X, _, _ = W.make_inputs(w)
    op = DPStokes(StokesParams.from_workload(w), w.N)
    op.set_positions(torch.tensor(X, device="cuda"))
    with pytest.raises(ValueError):
        op.mdot_multi(torch.zeros((2, w.N + 1, 3), dtype=torch.float64, device="cuda"))
    import ctypes
    code = op.L.dpst_mdot_multi(op._h, 0, ctypes.c_void_p(1), None, ctypes.c_void_p(1), None, _lib.F64, None)
    assert code != 0  # K < 1 is rejected before any device work
    with pytest.raises(DPStokesError):
        _lib.check(code)
    op.close()
