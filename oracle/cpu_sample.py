"""Bounded CPU timing sample of the oracle's Mdot (test / benchmark
infrastructure: bench.py's CPU baseline of the triply periodic mode only;
the other geometries are timed on whole Mdots by oracle/cpu_parallel.py).

The sample times every stage of the same
configuration on a fixed fraction of its work and scales each stage back up
(all stages are linear in the sampled quantity):
  spread + interpolation   first N/pfrac particles            x pfrac
  forward / backward FFT   one of the three grid components   x 3
  per-wavenumber solve     every mfrac-th wavenumber (k != 0) x (modes/sampled)
Single-threaded numpy (cores = 1).
"""
import time

import numpy as np

import dpstokes_oracle as O


def _spread_nozero(g, kern, loc, Fp, deriv=None):
    """O.spread without its zeroing of the extended grid: the sample scales the
    spread of a particle subset to all particles, so the whole-grid zeroing
    (done once per Mdot whatever the particle count) is timed apart."""
    ext = g.ext_grid.reshape(-1, 3)
    for sl, lc in O._chunks(loc):
        delta = O.kernel_weights(kern, lc, deriv)
        idx = O._ext_indices(g, lc, kern.w).ravel()
        for d in range(3):
            np.add.at(ext[:, d], idx, (delta * Fp[sl, d][:, None, None, None]).ravel())


def _torque_spreads(p, T):
    """The torque spreads of one Mdot: three derivative kernels, or the
    regular kernel once."""
    if not p.has_torque or T is None:
        return ()
    return (None,) if p.reg_kernel else (0, 1, 2)


def _timed_spread(o, p, F, T):
    """(seconds of the particles' contributions, seconds of the passes done
    once per Mdot whatever the particle count -- zeroing the extended grids
    and the folds --, the folded force grid)."""
    tder = _torque_spreads(p, T)
    o.g.ext_grid[...] = 0.0
    if tder:
        o.tg.ext_grid[...] = 0.0
    t0 = time.perf_counter()
    _spread_nozero(o.g, o.km, o.loc, F)
    for d in tder:
        _spread_nozero(o.tg, o.kd, o.tloc, T, d)
    t_part = time.perf_counter() - t0
    t0 = time.perf_counter()
    o.g.ext_grid[...] = 0.0
    fG = O.fold(o.g, o.BCs)
    for d in tder:
        o.tg.ext_grid[...] = 0.0
        O.fold(o.tg, o.BCst if d == 2 else o.BCs)
    t_once = time.perf_counter() - t0
    return t_part, t_once, fG


def sample_mdot_seconds(p: O.Params, X, F, T=None, pfrac=16, mfrac=16):
    X = np.asarray(X, dtype=np.float64).reshape(-1, 3)
    F = np.asarray(F, dtype=np.float64).reshape(-1, 3)
    T = None if T is None else np.asarray(T, dtype=np.float64).reshape(-1, 3)
    N = X.shape[0]
    ns = max(1, N // pfrac)
    o = O.Oracle(p)
    o.set_positions(X[:ns])
    t_part, t_once, fG = _timed_spread(o, p, F[:ns], None if T is None else T[:ns])
    if p.domType == 'TP':
        return _sample_tp(p, o, fG, N, ns, t_part, t_once)
    # forward transform of one component
    one = np.ascontiguousarray(fG[..., :1])
    del fG
    t0 = time.perf_counter()
    fh = O.fc_forward(one)
    t_fwd = 3 * (time.perf_counter() - t0)
    # solve on a subset of wavenumbers
    nk = p.Nx * p.Ny
    modes = np.arange(1, nk, mfrac)
    rng = np.random.default_rng(0)
    fk = (rng.standard_normal((modes.size + 1, p.Nz, 3)) + 1j * rng.standard_normal((modes.size + 1, p.Nz, 3)))
    sol = O.DPSolver(p.Nx, p.Ny, p.Nz, p.Lx, p.Ly, p.Lz / 2, p.eta,
                     modes=np.concatenate(([0], modes)))
    t0 = time.perf_counter()
    U = sol.solve_no_wall(fk)
    if p.domType == 'DPBW':
        sol.correct_bottom(U, o.zpts)
    elif p.domType == 'DPSC':
        sol.correct_slit(U, o.zpts, p.Lz)
    t_solve = (time.perf_counter() - t0) * (nk - 1) / modes.size
    # backward transform of one component
    t0 = time.perf_counter()
    ug = O.fc_backward(fh)
    t_bwd = 3 * (time.perf_counter() - t0)
    del fh
    uG = np.repeat(ug, 3, axis=3)
    t0 = time.perf_counter()
    O.ghost_copy(o.g, uG, o.BCs)
    O.interpolate(o.g, o.km, o.loc)
    if p.has_torque:
        O.ghost_copy(o.tg, uG, o.BCs)
        O.interpolate(o.tg, o.kd, o.tloc, deriv=0)
        O.interpolate(o.tg, o.kd, o.tloc, deriv=1)
        O.ghost_copy(o.tg, uG, o.BCst)
        O.interpolate(o.tg, o.kd, o.tloc, deriv=2)
    t_interp = time.perf_counter() - t0
    scale = N / ns
    stages = dict(spread=t_part * scale + t_once, fft_fwd=t_fwd, solve=t_solve, fft_bwd=t_bwd,
                  interp=t_interp * scale)
    total = sum(stages.values())
    sample = ("oracle stages timed on %d of %d particles (x%.0f; the grid zeroing and folds once), "
              "1 of 3 grid components (x3), %d of %d wavenumbers (x%.1f); single-threaded numpy"
              % (ns, N, scale, modes.size, nk - 1, (nk - 1) / modes.size))
    return total, stages, sample


def _sample_tp(p, o, fG, N, ns, t_part, t_once):
    """Triply periodic stages: 3-D FFT of one component (x3), the full
    Fourier-space solve, inverse FFT of one component (x3), interpolation of
    the sampled particles."""
    t0 = time.perf_counter()
    fh1 = np.fft.fftn(np.ascontiguousarray(fG[..., 0]))
    t_fwd = 3 * (time.perf_counter() - t0)
    fh = np.repeat(fh1[..., None], 3, axis=3)
    del fG
    t0 = time.perf_counter()
    U = O.tp_solve(fh, p.Lx, p.Ly, p.Lz, p.eta)
    t_solve = time.perf_counter() - t0
    del fh
    t0 = time.perf_counter()
    ug = np.fft.ifftn(U[..., 0]).real
    t_bwd = 3 * (time.perf_counter() - t0)
    del U
    uG = np.repeat(ug[..., None], 3, axis=3)
    t0 = time.perf_counter()
    O.ghost_copy(o.g, uG, o.BCs)
    O.interpolate(o.g, o.km, o.loc)
    if p.has_torque:
        O.ghost_copy(o.tg, uG, o.BCs)
        O.interpolate(o.tg, o.kd, o.tloc, deriv=0)
        O.interpolate(o.tg, o.kd, o.tloc, deriv=1)
        O.interpolate(o.tg, o.kd, o.tloc, deriv=2)
    t_interp = time.perf_counter() - t0
    scale = N / ns
    stages = dict(spread=t_part * scale + t_once, fft_fwd=t_fwd, solve=t_solve, fft_bwd=t_bwd,
                  interp=t_interp * scale)
    total = sum(stages.values())
    sample = ("oracle stages timed on %d of %d particles (x%.0f; the grid zeroing and folds once), "
              "1 of 3 grid components (x3), every wavenumber; single-threaded numpy" % (ns, N, scale))
    return total, stages, sample
