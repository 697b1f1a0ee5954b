"""Bounded CPU timing sample of the oracle's Mdot (test / benchmark
infrastructure: bench.py's cpu_baseline and reference arm only).

A full oracle Mdot at the 65,536-particle, 512 x 512 x 128 configuration
takes minutes and ~15 GB.  The sample times every stage of the same
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


# --------------------------------------------------------------------------
# The same sample on every host core (bench.py's reference arm), timed the
# way the reference's OpenMP code divides the work (SpreadInterp.cpp:11-154,
# 302-600: independent groups of grid columns, no reduction): W worker
# processes each time the spread and the interpolation of their own 1/W of
# the particles and the solve of their own 1/W of the wavenumbers; a stage
# takes the slowest worker's time, plus the passes that are done once (the
# ghost fold / copy of the whole grid), timed in the parent; the transforms
# run on scipy.fft's threads.  Each worker samples 1/pfrac of its share of
# particles and 1/mfrac of its wavenumbers (scaled back).
# --------------------------------------------------------------------------
def _time_share(args):
    p, X, F, T, modes, seed = args
    o = O.Oracle(p)
    o.set_positions(X)
    torque = p.has_torque and T is not None
    t_spread, _, _ = _timed_spread(o, p, F, T)
    rng = np.random.default_rng(seed)
    o.g.ext_grid[...] = rng.standard_normal(o.g.ext_grid.shape)
    if torque:
        o.tg.ext_grid[...] = rng.standard_normal(o.tg.ext_grid.shape)
    t0 = time.perf_counter()
    O.interpolate(o.g, o.km, o.loc)
    if torque:
        for d in ((None,) if p.reg_kernel else (0, 1, 2)):
            O.interpolate(o.tg, o.kd, o.tloc, deriv=d)
    t_interp = time.perf_counter() - t0
    t_solve = 0.0
    if p.domType != 'TP' and modes.size:
        sol = O.DPSolver(p.Nx, p.Ny, p.Nz, p.Lx, p.Ly, p.Lz / 2, p.eta, modes=np.concatenate(([0], modes)))
        fk = rng.standard_normal((modes.size + 1, p.Nz, 3)) + 1j * rng.standard_normal((modes.size + 1, p.Nz, 3))
        t0 = time.perf_counter()
        U = sol.solve_no_wall(fk)
        if p.domType == 'DPBW':
            sol.correct_bottom(U, o.zpts)
        elif p.domType == 'DPSC':
            sol.correct_slit(U, o.zpts, p.Lz)
        t_solve = time.perf_counter() - t0
    return t_spread, t_interp, t_solve


def sample_mdot_seconds_parallel(p: O.Params, X, F, T=None, workers=None, pfrac=16, mfrac=16):
    """The sample on `workers` processes (default: the CPUs this process may
    run on).  Returns (seconds per Mdot estimate, stage seconds, sample
    description, workers)."""
    import multiprocessing as mp
    import os
    import scipy.fft as sfft
    if workers is None:
        workers = len(os.sched_getaffinity(0))
    X = np.asarray(X, dtype=np.float64).reshape(-1, 3)
    F = np.asarray(F, dtype=np.float64).reshape(-1, 3)
    T = None if T is None else np.asarray(T, dtype=np.float64).reshape(-1, 3)
    N = X.shape[0]
    share = (N + workers - 1) // workers
    ns = max(1, share // pfrac)  # sampled particles per worker
    nk = p.Nx * p.Ny
    modes = np.arange(1, nk, mfrac)
    mchunks = np.array_split(modes, workers)
    jobs = []
    for w in range(workers):
        a = w * share
        sl = slice(a, min(N, a + ns))
        jobs.append((p, X[sl], F[sl], None if T is None else T[sl], mchunks[w], w))
    ctx = mp.get_context("spawn")  # the caller may already hold a CUDA context
    # one BLAS / OpenMP thread per worker process (the workers are the threads)
    keys = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")
    saved = {k: os.environ.get(k) for k in keys}
    for k in keys:
        os.environ[k] = "1"
    try:
        with ctx.Pool(workers) as pool:
            res = pool.map(_time_share, jobs)
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    t_interp = max(r[1] for r in res) * (share / ns)
    t_solve = max(r[2] for r in res) * mfrac
    # the once-per-Mdot passes (grid zeroing, folds, ghost copies) and the
    # transforms, in this process
    o = O.Oracle(p)
    o.set_positions(X[:ns])
    torque = p.has_torque and T is not None
    _, t_once, fG = _timed_spread(o, p, F[:ns], None if T is None else T[:ns])
    t_spread = max(r[0] for r in res) * (share / ns) + t_once
    one = np.ascontiguousarray(fG[..., 0])
    del fG
    tp = p.domType == 'TP'
    t0 = time.perf_counter()
    if tp:
        fh1 = sfft.fftn(one, workers=workers)
    else:
        Nz = one.shape[2]
        fh1 = sfft.fftn(np.concatenate([one, one[:, :, Nz - 2:0:-1]], axis=2), workers=workers)[:, :, :Nz]
    t_fwd = 3 * (time.perf_counter() - t0)
    if tp:  # elementwise numpy, one thread
        fh = np.repeat(fh1[..., None], 3, axis=3)
        t0 = time.perf_counter()
        O.tp_solve(fh, p.Lx, p.Ly, p.Lz, p.eta)
        t_solve = time.perf_counter() - t0
        del fh
    t0 = time.perf_counter()
    if tp:
        ug = sfft.ifftn(fh1, workers=workers).real
    else:
        Nz = fh1.shape[2]
        ug = sfft.ifftn(np.concatenate([fh1, fh1[:, :, Nz - 2:0:-1]], axis=2), workers=workers)[:, :, :Nz].real
    t_bwd = 3 * (time.perf_counter() - t0)
    uG = np.repeat(np.ascontiguousarray(ug)[..., None], 3, axis=3)
    t0 = time.perf_counter()
    O.ghost_copy(o.g, uG, o.BCs)
    if torque:
        O.ghost_copy(o.tg, uG, o.BCs)
        if not p.reg_kernel:
            O.ghost_copy(o.tg, uG, o.BCst)
    t_interp += time.perf_counter() - t0
    stages = dict(spread=t_spread, fft_fwd=t_fwd, solve=t_solve, fft_bwd=t_bwd, interp=t_interp)
    total = sum(stages.values())
    sample = ("oracle on %d processes: spread and interpolation of each process's 1/%d of the particles "
              "(sampled 1 in %d), the solve of its 1/%d of the wavenumbers (sampled 1 in %d), the slowest "
              "process's time per stage plus the whole-grid fold / copy; transforms on %d scipy.fft threads "
              "(1 of 3 grid components, x3)%s"
              % (workers, workers, pfrac, workers, mfrac, workers,
                 "; the triply periodic solve elementwise on one thread" if tp else ""))
    return total, stages, sample, workers
