"""doublyperiodicstokes_gb300.gridconfig against the reference's own grid and
kernel configuration (golden vectors made by tests/golden/make_gridconfig_golden.py
from source/cpu/python/GridAndKernelConfig.py): identical (h, N, w, beta,
c(beta), z extent, Nz, floor) for every kernel type with and without torques,
the optimal and the candidate grids, the doubled reference grid, several
radii, every domain type; the same errors for unsupported kernel types."""
import json
import os

import numpy as np
import pytest

from doublyperiodicstokes_gb300 import gridconfig as G

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "gridconfig.json")) as f:
    GOLD = json.load(f)


def _same(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape
    assert np.array_equal(a, b), (a, b)


@pytest.mark.parametrize("case", GOLD["xy"], ids=lambda c: "%s-%s-opt%s-tq%s" % (c["args"][0], c["args"][3],
                                                                                c["args"][4], c["args"][5]))
def test_xy_matches_reference(case):
    Lx, Ly, radii, kts, opt, tq, ref = case["args"]
    if "error" in case:
        with pytest.raises(ValueError, match=case["error"]):
            G.configure_grid_and_kernels_xy(Lx, Ly, np.array(radii), np.array(kts), opt, tq, ref)
        return
    got = G.configure_grid_and_kernels_xy(Lx, Ly, np.array(radii), np.array(kts), opt, tq, ref)
    for g, r in zip(got, case["out"]):
        _same(g, r)


@pytest.mark.parametrize("case", GOLD["z"], ids=lambda c: "%s-%s" % (c["args"][5], c["args"][1]))
def test_z_matches_reference(case):
    minZ, maxZ, h, wm, wd, dom, ref = case["args"]
    got = G.configure_grid_and_kernels_z(minZ, maxZ, h, np.array(wm, dtype=np.ushort),
                                         np.array(wd, dtype=np.ushort), dom, 1.5, ref)
    if "error" in case:
        # the reference fails here (a triply periodic extent already an integer
        # number of cells: it calls .astype on a float); the intended result
        assert case["error"].startswith("AttributeError")
        assert got == (maxZ - minZ, h, int(round((maxZ - minZ) / h)), minZ)
        return
    for g, r in zip(got, case["out"]):
        _same(g, r)


def test_fft_friendly_sizes():
    assert list(G.fft_friendly_sizes(65, 100, 1)) == [64]
    assert all(G._valid(n) for n in G.fft_friendly_sizes(199, 100, 10))
