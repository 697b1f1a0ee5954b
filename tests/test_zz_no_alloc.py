"""dpst_mdot_noalloc: the allocation-free entry point, for callers that
cannot allocate device memory when they call the operator (inside a CUDA
stream capture in global capture mode, or under an allocator that has
reserved the device).  Its per-wavenumber solve uses a static device array
for scratch; here its results are checked, through the C ABI, against the
ordinary dpst_mdot on the same handle, on two calls in a row (the array
keeps the previous call's contents, which must not leak into the next), in
every geometry, with the regular-kernel coupling and in the triply periodic
mode (which needs no scratch).
This file sorts last so that a run stopping at the first failure has run
every other test first; it also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from doublyperiodicstokes_gb300 import DPStokes, StokesParams, _lib, workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = a.double().cpu().numpy().ravel()
    b = b.double().cpu().numpy().ravel()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("name,precision,tol", [("s_dpsc_t", "fp64", 1e-10), ("s_dpbw_t_odd", "fp64", 1e-10),
                                                ("s_dp_t", "mixed", 1e-5), ("s_reg_dpbw_t", "fp64", 1e-10),
                                                ("s_tp_t", "mixed", 1e-5)])
def test_noalloc_matches_mdot_on_two_calls(name, precision, tol):
    w = W.SMALL_BY_NAME[name]
    X, F, T = W.make_inputs(w)
    dt = torch.float64 if precision == "fp64" else torch.float32
    op = DPStokes(StokesParams.from_workload(w, precision), w.N)
    d = op.device
    op.set_positions(torch.tensor(X, device=d))
    Ft = torch.tensor(F, dtype=dt, device=d)
    Tt = torch.tensor(T, dtype=dt, device=d)
    V_ref, W_ref = op.mdot(Ft, Tt)
    L = _lib.lib()
    code = _lib.F64 if dt == torch.float64 else _lib.F32
    stream = ctypes.c_void_p(torch.cuda.current_stream(d).cuda_stream)
    for call in range(2):
        V = torch.full_like(Ft, float("nan"))
        Wt = torch.full_like(Ft, float("nan"))
        _lib.check(L.dpst_mdot_noalloc(op._h, ctypes.c_void_p(Ft.data_ptr()), ctypes.c_void_p(Tt.data_ptr()),
                                       ctypes.c_void_p(V.data_ptr()), ctypes.c_void_p(Wt.data_ptr()), code,
                                       stream))
        torch.cuda.synchronize()
        ev, ew = _rel(V, V_ref), _rel(Wt, W_ref)
        print("%s %s call %d: V %.2e W %.2e" % (name, precision, call, ev, ew))
        assert ev < tol and ew < tol
    op.close()
