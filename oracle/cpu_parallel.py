"""Whole Mdots of the oracle (the reference CPU path restated in numpy) on
every host core -- test / benchmark infrastructure: bench.py's reference arm
and cpu_baseline only, never the product path.

Nothing is sampled or extrapolated: every call computes the full Mdot of the
configuration, with the work divided the way the reference's OpenMP code
divides it:
  * spreading: independent groups of grid columns (SpreadInterp.cpp:11-154,
    302-448): the particles are binned into x slabs of at least 2w + 2
    columns, and the even slabs, then the odd slabs, are spread by the worker
    processes straight into one shared extended grid (slabs of one phase
    touch disjoint columns, so no reduction is needed);
  * the boundary folds (BoundaryConditions.h): the ghost-region sums in the
    parent, the permuted copy of the interior with the torque curl added
    (FCM.py:353-371) by the workers, a block of y rows each;
  * the Fourier-Chebyshev transforms (Transform.cpp:107-304) on scipy.fft's
    threads: the DFT of the even extension in z of Nz real values is the
    type-I DCT of those values (X_k = x_0 + (-1)^k x_{Nz-1} +
    2 sum x_n cos(pi k n / (Nz - 1))), so the forward transform is a DCT-I in
    z then complex FFTs in x, y over the full spectrum the reference solves,
    and the inverse the complex inverse in x, y, its real part (the part the
    reference keeps) and a DCT-I in z over 2 Nz - 2 -- the values of the
    reference's complex 3-D DFTs of the extended array, without the
    extension;
  * the per-wavenumber solve (DPTools.cpp:81-877): each worker owns a
    contiguous block of wavenumbers, with its factors precomputed at set-up
    (the reference's DoublyPeriodicStokes_init), and applies the integration
    matrices through their few nonzero diagonals;
  * the ghost copies of the velocity grid: the permuted interior by the
    workers, a block of z levels each, the z-end rows in the parent;
  * interpolation (SpreadInterp.cpp:450-600): each worker a block of
    particles, reading the shared extended grids.
The workers are spawned processes that live as long as the object (like the
reference's OpenMP thread pool) and share the grids, spectra and particle
arrays through multiprocessing.shared_memory.  Results equal the oracle's
Mdot up to the order of floating-point sums.
"""
import multiprocessing as mp
import os
from multiprocessing import shared_memory

import numpy as np

import dpstokes_oracle as O

# --------------------------------------------------------------------------
# shared arrays
# --------------------------------------------------------------------------


class _Shared:
    def __init__(self):
        self.blocks = {}
        self.meta = {}

    def new(self, name, shape, dtype):
        nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        shm = shared_memory.SharedMemory(create=True, size=max(nbytes, 8))
        self.blocks[name] = shm
        self.meta[name] = (shm.name, tuple(shape), np.dtype(dtype).str)
        return np.ndarray(shape, dtype=dtype, buffer=shm.buf)

    def close(self):
        for shm in self.blocks.values():
            try:
                shm.close()
                shm.unlink()
            except FileNotFoundError:
                pass
        self.blocks = {}


def _attach(meta):
    out, keep = {}, []
    for name, (shm_name, shape, dtype) in meta.items():
        shm = shared_memory.SharedMemory(name=shm_name)
        keep.append(shm)
        out[name] = np.ndarray(shape, dtype=np.dtype(dtype), buffer=shm.buf)
    return out, keep


def _subset(loc, idx):
    return O.Located(loc.xclose[idx], loc.yclose[idx], loc.xun[idx], loc.yun[idx], loc.indl[idx], loc.wz[idx],
                     loc.zun[idx], loc.ptw[idx])


def _spread_into(ext, g, kern, loc, Fp, deriv=None):
    """O.spread without the zeroing: add the particles' kernels into ext."""
    flat = ext.reshape(-1, 3)
    for sl, lc in O._chunks(loc):
        delta = O.kernel_weights(kern, lc, deriv)
        idx = O._ext_indices(g, lc, kern.w).ravel()
        for d in range(3):
            np.add.at(flat[:, d], idx, (delta * Fp[sl, d][:, None, None, None]).ravel())


def _interp_from(ext, g, kern, loc, deriv=None):
    """O.interpolate on a given extended grid."""
    flat = ext.reshape(-1, 3)
    out = np.zeros((loc.xclose.shape[0], 3))
    for sl, lc in O._chunks(loc):
        delta = O.kernel_weights(kern, lc, deriv)
        idx = O._ext_indices(g, lc, kern.w)
        wgt = delta * lc.ptw[:, :, None, None]
        out[sl] = np.einsum('nkjid,nkji->nd', flat[idx], wgt)
    return out


def _band_plan(M):
    """The nonzero diagonals of a banded matrix M [n, m] as (offset, first row,
    values of the contiguous rows r0 .. r0 + len - 1)."""
    n, m = M.shape
    plan = []
    for d in range(-n + 1, m):
        rows = [r for r in range(n) if 0 <= r + d < m and M[r, r + d] != 0.0]
        if rows:
            r0, r1 = rows[0], rows[-1] + 1
            plan.append((d, r0, M[np.arange(r0, r1), np.arange(r0, r1) + d].copy()))
    return plan


def _band_apply(plan, x, n):
    """M x for x [m, k] (row-major over the wavenumbers) -> [n, k]."""
    out = np.zeros((n, x.shape[1]), dtype=x.dtype)
    for d, r0, vals in plan:
        r1 = r0 + vals.size
        out[r0:r1] += vals[:, None] * x[r0 + d:r1 + d]
    return out


class _BandedSolver(O.DPSolver):
    """The oracle's DPSolver computed with the wavenumbers as the contiguous
    axis ([row][wavenumber] arrays) and the integration matrices (SIMat,
    FIMat: three and two nonzero diagonals plus the border entries) applied
    through their diagonals instead of as dense products; same formulas
    otherwise (DPTools.cpp:81-345, LinearSolvers.h:76-141)."""

    def __post_init__(self):
        super().__post_init__()
        self._pS = _band_plan(self.SIMat)
        self._pF = _band_plan(self.FIMat)
        b = self.beta[1:].T  # [Nz + 1, k]
        Nz = self.Nz
        self._ib = np.ascontiguousarray(1.0 / np.where(b == 0, 1.0, b))
        mf = np.zeros((Nz, b.shape[1]))
        mf[2:] = self.dm2[1:, :Nz - 2].T / b[1:Nz - 1]
        self._mf = mf
        self._dp2 = np.ascontiguousarray(self.dp2[1:].T)
        self._AB = np.ascontiguousarray(self.AinvB[1:].transpose(2, 1, 0))  # [2, Nz, k]
        self._C = np.ascontiguousarray(self.C[1:].transpose(1, 2, 0))  # [2, Nz, k]
        self._Gi = np.ascontiguousarray(self.Ginv[1:].transpose(1, 2, 0))  # [2, 2, k]

    def _sweeps(self, rhs, cols):
        Nz = self.Nz
        x = rhs.copy()
        mf, ib, dp2 = self._mf[:, cols], self._ib[:, cols], self._dp2[:, cols]
        for i in range(2, Nz):
            x[i] -= mf[i] * x[i - 2]
        x[Nz - 1] *= ib[Nz]
        x[Nz - 2] *= ib[Nz - 1]
        for i in range(Nz - 3, -1, -1):
            x[i] = (x[i] - dp2[i] * x[i + 2]) * ib[i + 1]
        return x

    def solve_no_wall(self, fhat, chunk=1024):
        """U [k, Nz, 3] for fhat [k, Nz, 3] (row 0, k = 0, is left zero), in
        blocks of `chunk` wavenumbers so that the per-row arrays stay in cache."""
        U = np.zeros((fhat.shape[0], self.Nz, 3), dtype=np.complex128)
        n = fhat.shape[0] - 1
        for a in range(0, n, chunk):
            b = min(n, a + chunk)
            U[1 + a:1 + b] = self._solve_block(fhat[1 + a:1 + b], slice(a, b))
        return U

    def _solve_block(self, fk, cols):
        Nz, H, eta = self.Nz, self.H, self.eta
        f = np.ascontiguousarray(fk.transpose(2, 1, 0))  # [3, Nz, k]
        nk = f.shape[2]
        Dx, Dy = self.Dx[1:][cols], self.Dy[1:][cols]
        df = np.zeros((Nz, nk), dtype=np.complex128)
        df[Nz - 2] = ((Nz - 1) * 2 / H) * f[2, Nz - 1]
        for k in range(2, Nz):
            df[Nz - k - 1] = df[Nz - k + 1] + ((Nz - k) * 2 / H) * f[2, Nz - k]
        df[0] /= 2
        p_rhs = Dx * f[0] + Dy * f[1] + df
        AB, C, Gi = self._AB[:, :, cols], self._C[:, :, cols], self._Gi[:, :, cols]

        def solved(rhs, b0=0.0, b1=0.0):
            xp = self._sweeps(rhs, cols)
            y0 = np.sum(xp * C[0], axis=0) - b0
            y1 = np.sum(xp * C[1], axis=0) - b1
            g0 = Gi[0, 0] * y0 + Gi[0, 1] * y1
            g1 = Gi[1, 0] * y0 + Gi[1, 1] * y1
            x = np.empty((Nz + 2, nk), dtype=np.complex128)
            x[:Nz] = xp - (AB[0] * g0 + AB[1] * g1)
            x[Nz] = g0
            x[Nz + 1] = g1
            return x

        x = solved(p_rhs)
        cp = _band_apply(self._pS, x, Nz)
        dp = _band_apply(self._pF, x, Nz)
        sgn = np.power(-1.0, np.arange(Nz))
        ssum = np.sum(cp, axis=0)
        asum = np.sum(cp * sgn[:, None], axis=0)
        fac1 = 2 * eta
        fac = fac1 * self.K[1:][cols]
        bc = [(-Dx * ssum / fac, Dx * asum / fac), (-Dy * ssum / fac, Dy * asum / fac),
              (ssum / fac1, asum / fac1)]
        U = np.empty((nk, Nz, 3), dtype=np.complex128)
        rhs = ((Dx * cp - f[0]) / eta, (Dy * cp - f[1]) / eta, (dp - f[2]) / eta)
        for c in range(3):
            U[:, :, c] = _band_apply(self._pS, solved(rhs[c], *bc[c]), Nz).T
        return U


def _fold_edges(g, BCs):
    """The in-place part of the oracle's fold (DeGhostify,
    BoundaryConditions.h:22-361): ghost columns and rows added into the
    periodic interior, z-end ghost levels folded by the BCs.  The permuted
    copy of the interior is left to the workers."""
    e = g.ext_grid
    Nx, Ny, Nz = g.Nx, g.Ny, g.Nz
    lend = (g.Nxeff - Nx) // 2
    rbeg = g.Nxeff - lend
    bend = (g.Nyeff - Ny) // 2
    tbeg = g.Nyeff - bend
    dend = (g.Nzeff - Nz) // 2
    ubeg = g.Nzeff - dend
    e[:, :, Nx:Nx + lend, :] += e[:, :, 0:lend, :]
    e[:, :, rbeg - Nx:g.Nxeff - Nx, :] += e[:, :, rbeg:g.Nxeff, :]
    e[:, Ny:Ny + bend, :, :] += e[:, 0:bend, :, :]
    e[:, tbeg - Ny:g.Nyeff - Ny, :, :] += e[:, tbeg:g.Nyeff, :, :]
    for d in range(3):
        bc = BCs[12 + d]
        if bc != O.BC_NONE:
            s = 1.0 if bc == O.BC_MIRROR else -1.0
            src = np.arange(0, dend + 1)
            tmp = e[src, :, :, d].copy()
            e[2 * dend - src, :, :, d] += s * tmp
    for d in range(3):
        bc = BCs[15 + d]
        if bc != O.BC_NONE:
            s = 1.0 if bc == O.BC_MIRROR else -1.0
            src = np.arange(ubeg - 1, g.Nzeff)
            tmp = e[src, :, :, d].copy()
            e[2 * ubeg - src - 2, :, :, d] += s * tmp


def _interior(g, e):
    lend = (g.Nxeff - g.Nx) // 2
    bend = (g.Nyeff - g.Ny) // 2
    dend = (g.Nzeff - g.Nz) // 2
    return e[dend:g.Nzeff - dend, bend:g.Nyeff - bend, lend:g.Nxeff - lend, :]  # [Nz][Ny][Nx][3]


def _ghost_levels(g, e, uG, z0, z1):
    """The oracle's ghost_copy (Ghostify, BoundaryConditions.h:377-731) for
    interior levels [z0, z1): the permuted velocity and the periodic x, y
    ghost columns and rows of those levels."""
    Nx, Ny = g.Nx, g.Ny
    lend = (g.Nxeff - Nx) // 2
    rbeg = g.Nxeff - lend
    bend = (g.Nyeff - Ny) // 2
    tbeg = g.Nyeff - bend
    dend = (g.Nzeff - g.Nz) // 2
    zs = slice(dend + z0, dend + z1)
    e[zs, bend:tbeg, lend:rbeg, :] = uG[:, :, z0:z1, :].transpose(2, 0, 1, 3)
    e[zs, bend:tbeg, 0:lend, :] = e[zs, bend:tbeg, Nx:Nx + lend, :]
    e[zs, bend:tbeg, rbeg:g.Nxeff, :] = e[zs, bend:tbeg, rbeg - Nx:g.Nxeff - Nx, :]
    e[zs, tbeg:g.Nyeff, :, :] = e[zs, tbeg - Ny:g.Nyeff - Ny, :, :]
    e[zs, 0:bend, :, :] = e[zs, Ny:Ny + bend, :, :]


def _ghost_ends(g, e, BCs):
    """The z-end part of ghost_copy: ghost levels at active ends from the
    mirrored interior, the boundary node scaled by 1 + s."""
    dend = (g.Nzeff - g.Nz) // 2
    ubeg = g.Nzeff - dend
    for d in range(3):
        bc = BCs[12 + d]
        if bc != O.BC_NONE:
            s = 1.0 if bc == O.BC_MIRROR else -1.0
            k = np.arange(0, dend)
            e[k, :, :, d] = s * e[2 * dend - k, :, :, d]
            e[dend, :, :, d] += s * e[dend, :, :, d]
    for d in range(3):
        bc = BCs[15 + d]
        if bc != O.BC_NONE:
            s = 1.0 if bc == O.BC_MIRROR else -1.0
            k = np.arange(ubeg - 1, g.Nzeff)
            e[k, :, :, d] = s * e[2 * ubeg - k - 2, :, :, d]
            e[ubeg - 1, :, :, d] += s * e[ubeg - 1, :, :, d]


# --------------------------------------------------------------------------
# worker side
# --------------------------------------------------------------------------
_W = {}


def _worker_init(meta, state):
    arrs, keep = _attach(meta)
    _W.clear()
    _W.update(state)
    _W["arrs"] = arrs
    _W["keep"] = keep
    modes = state["modes"]
    p = state["p"]
    if modes is not None and modes.size:
        _W["solver"] = _BandedSolver(p.Nx, p.Ny, p.Nz, p.Lx, p.Ly, p.Lz / 2, p.eta,
                                     modes=np.concatenate(([0], modes)))


def _worker_task(task):
    kind, arg = task
    A = _W["arrs"]
    p = _W["p"]
    if kind == "zero":  # this worker's z levels of every extended grid
        for name in _W["grids"]:
            e = A[name]
            lo, hi = arg[name]
            e[lo:hi] = 0.0
        return 0
    if kind == "spread":
        for s in arg:
            idx_m, idx_d = _W["slabs_m"][s], _W["slabs_d"][s]
            if idx_m.size:
                _spread_into(A["g"], _W["g"], _W["km"], _subset(_W["loc"], idx_m), A["F"][idx_m])
            if _W["torque"] and idx_d.size:
                lc = _subset(_W["tloc"], idx_d)
                for d in range(3):
                    _spread_into(A["t%d" % d], _W["tg"], _W["kd"], lc, A["T"][idx_d], deriv=d)
        return 0
    if kind == "assemble":  # the folded force grid, y rows [a, b)
        ya, yb = arg
        Nz = p.Nz
        E = A["E"]
        gi = _interior(_W["g"], A["g"])[:, ya:yb]  # [Nz][rows][Nx][3]
        blk = gi.transpose(1, 2, 0, 3).copy()  # [rows][Nx][Nz][3]
        if _W["torque"]:
            tg = _W["tg"]
            dx = _interior(tg, A["t0"])[:, ya:yb].transpose(1, 2, 0, 3)
            dy = _interior(tg, A["t1"])[:, ya:yb].transpose(1, 2, 0, 3)
            dz = _interior(tg, A["t2"])[:, ya:yb].transpose(1, 2, 0, 3)
            blk[..., 1] -= 0.5 * dx[..., 2]  # addDx, SpreadInterpWrapper.cpp:66-79
            blk[..., 2] += 0.5 * dx[..., 1]
            blk[..., 0] += 0.5 * dy[..., 2]  # addDy :80-93
            blk[..., 2] -= 0.5 * dy[..., 0]
            blk[..., 0] -= 0.5 * dz[..., 1]  # addDz :94-107
            blk[..., 1] += 0.5 * dz[..., 0]
        E[ya:yb] = blk
        return 0
    if kind == "ghost":  # velocity grid into the extended grids, interior levels [a, b)
        z0, z1 = arg
        uG = A["uG"]
        _ghost_levels(_W["g"], A["g"], uG, z0, z1)
        if _W["torque"]:
            _ghost_levels(_W["tg"], A["t0"], uG, z0, z1)
            _ghost_levels(_W["tg"], A["t2"], uG, z0, z1)
        return 0
    if kind == "solve":
        modes = _W["modes"]
        if modes is None or not modes.size:
            return 0
        fk = A["fhat"].reshape(-1, p.Nz, 3)
        sub = np.concatenate((fk[:1], fk[modes]))
        s = _W["solver"]
        U = s.solve_no_wall(sub)
        if p.domType == 'DPBW':
            s.correct_bottom(U, _W["zpts"])
        elif p.domType == 'DPSC':
            s.correct_slit(U, _W["zpts"], p.Lz)
        A["U"].reshape(-1, p.Nz, 3)[modes] = U[1:]
        return 0
    if kind == "interp":
        a, b = arg
        if b <= a:
            return 0
        sl = np.arange(a, b)
        A["V"][a:b] = _interp_from(A["g"], _W["g"], _W["km"], _subset(_W["loc"], sl))
        if _W["torque"]:
            lc = _subset(_W["tloc"], sl)
            dxv = _interp_from(A["t0"], _W["tg"], _W["kd"], lc, deriv=0)
            dyv = _interp_from(A["t0"], _W["tg"], _W["kd"], lc, deriv=1)
            dzv = _interp_from(A["t2"], _W["tg"], _W["kd"], lc, deriv=2)
            Wv = A["W"]
            Wv[a:b, 0] = -1 / 2 * (dyv[:, 2] - dzv[:, 1])  # FCM.py:424-426
            Wv[a:b, 1] = -1 / 2 * (dzv[:, 0] - dxv[:, 2])
            Wv[a:b, 2] = -1 / 2 * (dxv[:, 1] - dyv[:, 0])
        return 0
    raise ValueError(kind)


# --------------------------------------------------------------------------
# parent side
# --------------------------------------------------------------------------
def _slabs(loc, g, w, nworkers):
    """Particle indices per x slab of the extended grid; slab width >= 2 w + 2
    so that slabs two apart never touch the same column."""
    lend = (g.Nxeff - g.Nx) // 2
    sw = max(2 * w + 2, -(-g.Nxeff // (2 * nworkers)))
    ns = -(-g.Nxeff // sw)
    c = loc.xclose + lend
    sid = np.minimum(c // sw, ns - 1)
    order = np.argsort(sid, kind="stable")
    bounds = np.searchsorted(sid[order], np.arange(ns + 1))
    return [order[bounds[s]:bounds[s + 1]] for s in range(ns)], sw


class ParallelMdot:
    """Oracle Mdot (the reference's DP / DPBW / DPSC path with the derivative-
    kernel torque coupling) on `workers` processes."""

    def __init__(self, p: O.Params, X, workers=None):
        if p.domType == 'TP' or p.reg_kernel:
            raise ValueError("the parallel oracle covers the DP, DPBW and DPSC paths with derivative kernels")
        self.p = p
        self.workers = workers or len(os.sched_getaffinity(0))
        o = O.Oracle(p)
        o.set_positions(X)
        self.o = o
        self.N = o.X.shape[0]
        self.torque = p.has_torque
        sh = self.sh = _Shared()
        A = {}
        A["g"] = sh.new("g", o.g.ext_grid.shape, np.float64)
        o.g.ext_grid = A["g"]
        grids = ["g"]
        if self.torque:
            for d in range(3):
                A["t%d" % d] = sh.new("t%d" % d, o.tg.ext_grid.shape, np.float64)
                grids.append("t%d" % d)
            o.tg.ext_grid = A["t0"]
        A["F"] = sh.new("F", (self.N, 3), np.float64)
        A["T"] = sh.new("T", (self.N, 3), np.float64)
        A["V"] = sh.new("V", (self.N, 3), np.float64)
        A["W"] = sh.new("W", (self.N, 3), np.float64)
        A["fhat"] = sh.new("fhat", (p.Ny, p.Nx, p.Nz, 3), np.complex128)
        A["U"] = sh.new("U", (p.Ny, p.Nx, p.Nz, 3), np.complex128)
        A["E"] = sh.new("E", (p.Ny, p.Nx, p.Nz, 3), np.float64)
        A["uG"] = sh.new("uG", (p.Ny, p.Nx, p.Nz, 3), np.float64)
        self.A = A
        W = self.workers
        slabs_m, sw_m = _slabs(o.loc, o.g, o.km.w, W)
        if self.torque:
            slabs_d, sw_d = _slabs(o.tloc, o.tg, o.kd.w, W)
            # one slab numbering for both kernels: the wider slabs
            if sw_d != sw_m or len(slabs_d) != len(slabs_m):
                slabs_m, _ = _slabs(o.loc, o.g, max(o.km.w, o.kd.w), W)
                slabs_d, _ = _slabs(o.tloc, o.tg, max(o.km.w, o.kd.w), W)
        else:
            slabs_d = [np.zeros(0, dtype=np.int64) for _ in slabs_m]
        ns = len(slabs_m)
        # phase 0: even slabs, phase 1: odd slabs, dealt round-robin to the workers
        self.phase_tasks = []
        for ph in (0, 1):
            own = [[] for _ in range(W)]
            for q, s in enumerate(range(ph, ns, 2)):
                own[q % W].append(s)
            self.phase_tasks.append([("spread", own[w]) for w in range(W) if own[w]])
        nk = p.Nx * p.Ny
        blocks = np.array_split(np.arange(1, nk), W)
        pb = np.linspace(0, self.N, W + 1).astype(int)
        self.interp_tasks = [("interp", (int(pb[w]), int(pb[w + 1]))) for w in range(W)]
        zs = {}
        for name in grids:
            nzeff = A[name].shape[0]
            zb = np.linspace(0, nzeff, W + 1).astype(int)
            zs[name] = zb
        self.zero_tasks = [("zero", {name: (int(zs[name][w]), int(zs[name][w + 1])) for name in grids})
                           for w in range(W)]
        yb = np.linspace(0, p.Ny, W + 1).astype(int)
        self.assemble_tasks = [("assemble", (int(yb[w]), int(yb[w + 1]))) for w in range(W) if yb[w + 1] > yb[w]]
        zb = np.linspace(0, p.Nz, W + 1).astype(int)
        self.ghost_tasks = [("ghost", (int(zb[w]), int(zb[w + 1]))) for w in range(W) if zb[w + 1] > zb[w]]
        ctx = mp.get_context("spawn")
        keys = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")
        saved = {k: os.environ.get(k) for k in keys}
        for k in keys:
            os.environ[k] = "1"
        try:
            base = dict(p=p, grids=grids, g=self._geom(o.g), km=o.km, loc=o.loc, torque=self.torque,
                        zpts=o.zpts, slabs_m=slabs_m, slabs_d=slabs_d)
            if self.torque:
                base.update(tg=self._geom(o.tg), kd=o.kd, tloc=o.tloc)
            # spreading / interpolation workers, and one process per
            # wavenumber block holding that block's factors
            self.pool = ctx.Pool(W, initializer=_worker_init, initargs=(sh.meta, dict(base, modes=None)))
            self.spool = [ctx.Pool(1, initializer=_worker_init, initargs=(sh.meta, dict(base, modes=blocks[w])))
                          for w in range(W)]
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v

    @staticmethod
    def _geom(g):
        import copy
        c = copy.copy(g)
        c.ext_grid = None
        return c

    def mdot(self, F, T=None):
        """V (and W) for forces F (torques T); self.stage_seconds holds the
        seconds of this call's stages (the split of the reference's
        mobility_bench.py:437-442: spreading, transforms, solve,
        interpolation)."""
        import time
        import scipy.fft as sfft
        p, o, A = self.p, self.o, self.A
        tm = [time.perf_counter()]
        A["F"][...] = np.asarray(F, dtype=np.float64).reshape(-1, 3)
        if self.torque:
            A["T"][...] = np.asarray(T, dtype=np.float64).reshape(-1, 3)
        pool = self.pool
        pool.map(_worker_task, self.zero_tasks)
        for tasks in self.phase_tasks:
            pool.map(_worker_task, tasks)
        tm.append(time.perf_counter())  # 1: spread
        # boundary folds: ghost regions here, the permuted interior with the
        # torque curl (FCM.py:353-371) in the workers
        _fold_edges(o.g, o.BCs)
        if self.torque:
            for d in range(3):
                o.tg.ext_grid = A["t%d" % d]
                _fold_edges(o.tg, o.BCst if d == 2 else o.BCs)
            o.tg.ext_grid = A["t0"]
        pool.map(_worker_task, self.assemble_tasks)
        tm.append(time.perf_counter())  # 2: folds
        # forward transform (Transform.cpp:107-152, 215-268): the z DFT of the
        # even extension is the DCT-I X_0 .. X_{Nz-1} (X_{Nu-k} = X_k), so the
        # Chebyshev fold (X_k + X_{Nu-k}) / Nu is 2 X_k / Nu
        W = self.workers
        Nz = p.Nz
        Nu = 2 * Nz - 2
        X = sfft.fftn(sfft.dct(A["E"], type=1, axis=2, workers=W), axes=(0, 1), workers=W, overwrite_x=True)
        scale = np.full(Nz, 2.0 / Nu)
        scale[0] = scale[Nz - 1] = 1.0 / Nu
        fh = A["fhat"]
        np.multiply(X, scale[None, None, :, None], out=fh)
        del X
        tm.append(time.perf_counter())  # 3: forward transform
        # per-wavenumber solve, every block at once
        res = [sp.apply_async(_worker_task, (("solve", None),)) for sp in self.spool]
        for r in res:
            r.get()
        U = A["U"]
        Uk = U.reshape(-1, Nz, 3)
        Uk[0] = 0.0
        if p.domType in ('DPBW', 'DPSC'):
            o.solver.correct_k0(Uk, fh.reshape(-1, Nz, 3)[0], slit=p.domType == 'DPSC')
        tm.append(time.perf_counter())  # 4: solve
        # inverse transform (Transform.cpp:154-213, 270-304): coefficients
        # scaled to the even extension's half spectrum, complex inverse in x, y,
        # real part, real inverse in z
        yscale = np.full(Nz, Nu / 2.0)
        yscale[0] = yscale[Nz - 1] = Nu
        U *= yscale[None, None, :, None]
        B = sfft.ifftn(U, axes=(0, 1), workers=W)
        A["uG"][...] = sfft.dct(B.real, type=1, axis=2, workers=W)
        del B
        A["uG"] *= 1.0 / Nu
        tm.append(time.perf_counter())  # 5: inverse transform
        # ghost copies: the interior levels in the workers, the z ends here; the
        # dipole grid's open-end ghost levels keep the last (z-derivative)
        # spread, as the reference's single torque grid does
        pool.map(_worker_task, self.ghost_tasks)
        _ghost_ends(o.g, A["g"], o.BCs)
        if self.torque:
            dend = (o.tg.Nzeff - o.tg.Nz) // 2
            if dend:
                A["t0"][:dend] = A["t2"][:dend]
                A["t0"][o.tg.Nzeff - dend:] = A["t2"][o.tg.Nzeff - dend:]
            _ghost_ends(o.tg, A["t0"], o.BCs)
            _ghost_ends(o.tg, A["t2"], o.BCst)
        tm.append(time.perf_counter())  # 6: ghost copies
        pool.map(_worker_task, self.interp_tasks)
        tm.append(time.perf_counter())  # 7: interpolation
        self.stage_seconds = dict(spread=tm[2] - tm[0], fft_fwd=tm[3] - tm[2], solve=tm[4] - tm[3],
                                  fft_bwd=tm[5] - tm[4], interp=tm[7] - tm[5], total=tm[7] - tm[0])
        V = A["V"].ravel().copy()
        Wv = A["W"].ravel().copy() if self.torque else None
        return V, Wv

    def close(self):
        for pl in [self.pool] + list(self.spool):
            pl.terminate()
            pl.join()
        self.sh.close()
