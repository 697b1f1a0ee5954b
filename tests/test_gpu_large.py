"""Scale check past the headline size: l1_dp_n262144_1024 (open domain,
1024 x 1024 x 128, N = 262,144, torques; four times c2).  No oracle run at
this size; the properties that need none: linearity of the FP64 operator
(1e-12), invariance under a translation by whole grid cells in x and y
(1e-10), and the mixed operator within 1e-5 of the FP64 operator."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from conftest import rel_err  # noqa: E402
from doublyperiodicstokes_gb300 import DPStokes, StokesParams, workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu


def _run(op, X, F, T, dt):
    op.set_positions(torch.tensor(X, device=op.device))
    V, Wv = op.mdot(torch.tensor(F, dtype=dt, device=op.device), torch.tensor(T, dtype=dt, device=op.device))
    torch.cuda.synchronize()
    return np.concatenate([V.double().cpu().numpy().ravel(), Wv.double().cpu().numpy().ravel()])


def test_four_times_c2():
    w = W.L1
    X, F, T = W.make_inputs(w)
    op = DPStokes(StokesParams.from_workload(w, "fp64"), w.N)
    M1 = _run(op, X, F, T, torch.float64)
    M2 = _run(op, X, 2.0 * F, -T, torch.float64)
    M3 = _run(op, X, 3.0 * F, -T, torch.float64)
    assert rel_err(M3 - M2, _run(op, X, F, 0.0 * T, torch.float64)) < 1e-12
    Xs = X.copy()
    Xs[:, 0] = np.mod(Xs[:, 0] + 17 * w.Lx / w.nx, w.Lx)
    Xs[:, 1] = np.mod(Xs[:, 1] + 5 * w.Ly / w.ny, w.Ly)
    e = rel_err(_run(op, Xs, F, T, torch.float64), M1)
    print("shift %.2e" % e)
    assert e < 1e-10
    info = op.info()
    op.close()
    opm = DPStokes(StokesParams.from_workload(w, "mixed"), w.N)
    Mm = _run(opm, X, F.astype(np.float32), T.astype(np.float32), torch.float32)
    em = rel_err(Mm, M1)
    print("mixed vs fp64 %.2e, device bytes fp64 %.2f GB" % (em, info["device_bytes"] / 1e9))
    assert em < 1e-5
    opm.close()
