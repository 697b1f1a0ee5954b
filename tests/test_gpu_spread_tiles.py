"""The tile-owner spread of the mixed operator (k_spread_tiles: one CTA per
8 x 8-column tile writes its grid block once from shared memory; particles
whose window is not interior follow with atomics) against the
clear-and-atomics spread (the default; DPSTOKES_GB300_SPREAD=tiles selects
the tile-owner form) on the same inputs:
the spread grid to 1e-6 and V, W to 5e-6 (FP32 sums in another order), in
the open box, with walls (slit: particles near both walls take the atomic
path), with a grid that is not a multiple of the tile, and through the
multi-column Mdot; the operator with it stays within 1e-5 of the FP64
operator."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from conftest import rel_err  # noqa: E402
from doublyperiodicstokes_gb300 import DPStokes, StokesParams, workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu
CASES = ["c2_dp_n65536@128", "c1_dpsc_n16384@128", "c2_dp_n65536@100", "c1_dpsc_n16384@96"]


def _run(w, X, F, T, spread, monkeypatch, precision="mixed"):
    if spread:
        monkeypatch.setenv("DPSTOKES_GB300_SPREAD", spread)
    else:
        monkeypatch.delenv("DPSTOKES_GB300_SPREAD", raising=False)
    op = DPStokes(StokesParams.from_workload(w, precision), w.N)
    d = op.device
    dt = torch.float32 if precision == "mixed" else torch.float64
    op.set_positions(torch.tensor(X, device=d))
    Ft = torch.tensor(F, dtype=dt, device=d)
    Tt = torch.tensor(T, dtype=dt, device=d)
    grid = op.spread_grid(Ft, Tt).double().cpu().numpy()
    V, Wv = op.mdot(Ft, Tt)
    Vk, Wk = op.mdot_multi(torch.stack([Ft, 2 * Ft]), torch.stack([Tt, -Tt]))
    torch.cuda.synchronize()
    out = dict(tiles=op.info()["spread_tiles"], grid=grid, V=V.double().cpu().numpy(),
               W=Wv.double().cpu().numpy(), Vk=Vk.double().cpu().numpy(), Wk=Wk.double().cpu().numpy())
    op.close()
    return out


@pytest.mark.parametrize("name", CASES)
def test_tile_spread_matches_atomic_spread(name, monkeypatch):
    w = W.by_name(name)
    X, F, T = W.make_inputs(w)
    a = _run(w, X, F, T, "tiles", monkeypatch)
    b = _run(w, X, F, T, None, monkeypatch)
    assert a["tiles"] == 1 and b["tiles"] == 0
    eg = rel_err(a["grid"], b["grid"])
    ev, ew = rel_err(a["V"], b["V"]), rel_err(a["W"], b["W"])
    print("%s grid %.2e V %.2e W %.2e" % (name, eg, ev, ew))
    assert eg < 1e-6 and ev < 5e-6 and ew < 5e-6
    assert rel_err(a["Vk"], b["Vk"]) < 5e-6 and rel_err(a["Wk"], b["Wk"]) < 5e-6
    assert rel_err(a["Vk"][0], a["V"]) < 5e-6
    f = _run(w, X, F, T, "tiles", monkeypatch, precision="fp64")
    assert rel_err(a["V"], f["V"]) < 1e-5 and rel_err(a["W"], f["W"]) < 1e-5
