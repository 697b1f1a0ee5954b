"""The whole-Mdot CPU baseline (oracle/cpu_parallel.py: the oracle's Mdot on
worker processes, spreading by grid-column groups, the solve by wavenumber
blocks in banded form, DCT-I transforms) equals the oracle's own Mdot, in
every geometry, with torques, open-end ghost layers and odd grids."""
import numpy as np
import pytest

import cpu_parallel
import dpstokes_oracle as O
from conftest import rel_err
from doublyperiodicstokes_gb300 import workloads as W


@pytest.fixture(scope="module")
def cases():
    return ["s_dpbw_t", "s_dp_t", "s_dpsc_t", "e_dpsc_t", "e_dp_t_shift", "s_dpbw_t_odd", "s_dpsc_f_odd"]


def test_parallel_oracle_matches_oracle(cases):
    for name in cases:
        w = W.SMALL_BY_NAME[name]
        X, F, T = W.make_inputs(w)
        p = O.Params(**w.oracle_params())
        Vo, Wo = O.mdot(p, X, F, T)
        pm = cpu_parallel.ParallelMdot(p, X, workers=2)
        try:
            for _ in range(2):  # a second call on the same grids
                V, Wv = pm.mdot(F, T)
                assert rel_err(V, Vo) < 1e-13, name
                if Wo is not None:
                    assert rel_err(Wv, Wo) < 1e-13, name
            assert set(pm.stage_seconds) >= {"spread", "fft_fwd", "solve", "fft_bwd", "interp", "total"}
        finally:
            pm.close()


def test_banded_solver_matches_dense():
    p = O.Params(**W.SMALL_BY_NAME["s_dpsc_t"].oracle_params())
    rng = np.random.default_rng(3)
    nk = p.Nx * p.Ny
    fk = rng.standard_normal((nk, p.Nz, 3)) + 1j * rng.standard_normal((nk, p.Nz, 3))
    dense = O.DPSolver(p.Nx, p.Ny, p.Nz, p.Lx, p.Ly, p.Lz / 2, p.eta)
    band = cpu_parallel._BandedSolver(p.Nx, p.Ny, p.Nz, p.Lx, p.Ly, p.Lz / 2, p.eta)
    a, b = dense.solve_no_wall(fk), band.solve_no_wall(fk, chunk=37)
    assert rel_err(b.view(np.float64), a.view(np.float64)) < 1e-13
