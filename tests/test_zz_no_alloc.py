"""dpst_mdot_noalloc: the allocation-free entry point, for callers that
cannot allocate device memory when they call the operator (a host whose own
memory pool has reserved the device, or a time-critical loop that must not
pay for cudaMalloc / cudaFree).  Its per-wavenumber solve uses a static
device array for scratch; here its results are checked, through the C ABI,
against the ordinary dpst_mdot on the same handle, on two calls in a row (the
array keeps the previous call's contents, which must not leak into the next),
in every geometry, with the regular-kernel coupling, in the triply periodic
mode (which needs no scratch) and on a grid whose solve needs more CTAs than
the array holds (nz = 128 with walls: the launch is capped to the array and
each CTA takes a longer range of wavenumbers).  After a warm-up call, a call
must leave the device's free memory unchanged.
This file sorts last so that a run stopping at the first failure has run
every other test first; it also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from doublyperiodicstokes_gb300 import DPStokes, StokesParams, _lib, workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu

# nz = 128 on a 32 x 32 grid with a bottom wall (the c2 height): 544
# wavenumbers, 34 units of 16 for the ordinary solve's grid, against the
# 2^19 / (128 x 192) = 21 CTAs the static array holds
CAPPED = W.small("n_dpbw_t_nz128", "DPBW", 40, 32, 128, 41.0, 1.5, 39.5, True, seed=30)
CASES = {w.name: w for w in (CAPPED,)}


def _rel(a, b):
    a = a.double().cpu().numpy().ravel()
    b = b.double().cpu().numpy().ravel()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _noalloc(L, op, Ft, Tt, V, Wt, code, stream):
    _lib.check(L.dpst_mdot_noalloc(op._h, ctypes.c_void_p(Ft.data_ptr()), ctypes.c_void_p(Tt.data_ptr()),
                                   ctypes.c_void_p(V.data_ptr()), ctypes.c_void_p(Wt.data_ptr()), code, stream))


@pytest.mark.parametrize("name,precision,tol", [("s_dpsc_t", "fp64", 1e-10), ("s_dpbw_t_odd", "fp64", 1e-10),
                                                ("s_dp_t", "mixed", 1e-5), ("s_reg_dpbw_t", "fp64", 1e-10),
                                                ("s_tp_t", "mixed", 1e-5), ("n_dpbw_t_nz128", "fp64", 1e-10),
                                                ("n_dpbw_t_nz128", "mixed", 1e-5)])
def test_noalloc_matches_mdot_on_two_calls(name, precision, tol):
    w = CASES.get(name) or W.SMALL_BY_NAME[name]
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
        _noalloc(L, op, Ft, Tt, V, Wt, code, stream)
        torch.cuda.synchronize()
        ev, ew = _rel(V, V_ref), _rel(Wt, W_ref)
        print("%s %s call %d: V %.2e W %.2e" % (name, precision, call, ev, ew))
        assert ev < tol and ew < tol
    op.close()


def test_noalloc_call_leaves_free_memory_unchanged():
    w = CAPPED
    X, F, T = W.make_inputs(w)
    op = DPStokes(StokesParams.from_workload(w, "fp64"), w.N)
    d = op.device
    op.set_positions(torch.tensor(X, device=d))
    Ft = torch.tensor(F, device=d)
    Tt = torch.tensor(T, device=d)
    V = torch.empty_like(Ft)
    Wt = torch.empty_like(Ft)
    L = _lib.lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream(d).cuda_stream)
    _noalloc(L, op, Ft, Tt, V, Wt, _lib.F64, stream)  # warm-up: loads the kernels
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(d)
    for _ in range(3):
        _noalloc(L, op, Ft, Tt, V, Wt, _lib.F64, stream)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(d)
    assert free1 == free0, (free0, free1)
    op.close()
