"""Position updates on one handle (the reference's ParticleList::update,
ParticleList.cpp:550-753, rebuilds its column lists incrementally; here
dpst_set_positions recomputes stencils, z windows, ghost layers and the tile
order on the GPU in O(N)).  A short explicit time-stepping loop X <- X + dt V
(periodic in x, y; particles drifting into and out of the open-end ghost
range) run on one handle matches fresh handles created at every step (FP64,
equal up to the order of atomic sums), and the last step matches the oracle."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import dpstokes_oracle as O  # noqa: E402
from conftest import rel_err  # noqa: E402
from doublyperiodicstokes_gb300 import DPStokes, StokesParams, workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["s_dpbw_f_top", "s_dp_t", "s_dpsc_t"])
def test_time_stepping_on_one_handle(name):
    w = W.SMALL_BY_NAME[name]
    X, F, T = W.make_inputs(w)
    prm = StokesParams.from_workload(w)
    op = DPStokes(prm, w.N)
    rng = np.random.default_rng(9)
    lo, hi = w.z0 + 0.3, w.z0 + w.Lz - 0.3
    for step in range(6):
        Xt = torch.tensor(X, device="cuda")
        op.set_positions(Xt)
        Ft = torch.tensor(F, device="cuda")
        Tt = torch.tensor(T, device="cuda") if T is not None else None
        V, Wv = op.mdot(Ft, Tt)
        fresh = DPStokes(prm, w.N)
        fresh.set_positions(Xt)
        V2, W2 = fresh.mdot(Ft, Tt)
        fresh.close()
        assert rel_err(V.cpu().numpy(), V2.cpu().numpy()) < 1e-13
        if Wv is not None:
            assert rel_err(Wv.cpu().numpy(), W2.cpu().numpy()) < 1e-13
        # step: drift plus a random kick, wrapped in x, y, kept inside z
        dX = 0.8 * V.cpu().numpy() / np.abs(V.cpu().numpy()).max() + 0.6 * rng.standard_normal(X.shape)
        X = X + dX
        X[:, 0] %= w.Lx
        X[:, 1] %= w.Ly
        X[:, 2] = np.clip(X[:, 2], lo, hi)
    op.set_positions(torch.tensor(X, device="cuda"))
    V, Wv = op.mdot(torch.tensor(F, device="cuda"), torch.tensor(T, device="cuda") if T is not None else None)
    Vo, Wo = O.mdot(O.Params(**w.oracle_params()), X, F, T)
    assert rel_err(V.cpu().numpy(), Vo) < 1e-10
    if T is not None:
        assert rel_err(Wv.cpu().numpy(), Wo) < 1e-10
    op.close()
