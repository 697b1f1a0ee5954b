"""CPU oracle for the doubly periodic Stokes mobility product Mdot.

TEST INFRASTRUCTURE ONLY.  This module is the checker: tests/, the smoke()
entry point and bench.py's cpu_baseline / reference arm may import it; the
GPU product never does.

It restates, in vectorised numpy/FP64, the reference CPU path that
FCMJoint(device='cpu').Mdot runs (stochasticHydroTools/DoublyPeriodicStokes,
source/cpu), keeping the reference's data flow so that its discretisation
quirks are reproduced exactly:
  * extended ("unwrapped") grid with ghost layers, spread into it, then the
    ghost fold (BoundaryConditions.h:22-361) / ghost copy before interpolation
    (BoundaryConditions.h:377-731);
  * per-grid extended-grid buffers that persist between the spread and the
    interpolation of one Mdot, exactly like the reference's Grid objects, so
    that ghost layers at open (BC 'none') z ends still hold the spread data
    when the interpolation reads them (the copy leaves them untouched);
  * clamping of out-of-support kernel offsets to +threshold
    (ParticleList.cpp:497-523);
  * Fourier-Chebyshev transform through an even extension in z
    (Transform.cpp:107-304);
  * per-wavenumber Schur/KBPENTA solve (DPTools.cpp:81-345,
    LinearSolvers.h:52-141), wall corrections (DPTools.cpp:590-877) and the
    k=0 corrections (Solvers.py:482-599);
  * triply periodic mode (domType 'TP'): uniform periodic z grid located like
    x and y (ParticleList.cpp:285-366), periodic z fold / copy, unnormalised
    3-D DFT and the Fourier-space solve (Solvers.py:197-258,
    TPTools.cpp:6-46).
Pinned against the reference itself (oracle/_ref, run through
oracle/ref_harness.py) by tests/golden/make_golden.py.
"""
import math
from dataclasses import dataclass, field

import numpy as np

BC_MIRROR, BC_MIRROR_INV, BC_NONE = 0, 1, 2  # common.h:11


# --------------------------------------------------------------------------
# Parameters
# --------------------------------------------------------------------------
@dataclass
class Params:
    """Explicit grid/kernel parameters of one Mdot configuration.

    betam_hat/betad_hat are the dimensionless ES betas (the kernel uses
    beta = beta_hat * w, SpreadInterp.h:123).  With UseCbeta
    (FCM.py:296-307) alpha = R / (2 * R / (w * hx)) = w*hx/2; the same
    floating-point formula is used (ParticleList.cpp:229).
    z0 is the floor of the Chebyshev interval [z0, z0+Lz] (FCM.py:170).
    domType 'TP' (triply periodic): Nz uniform points on the periodic
    interval [z0, z0+Lz), hz = Lz / Nz (GridAndKernelConfig.py:380-393).
    reg_kernel: the reference's useRegKernel torque coupling (FCM.py:372-396,
    427-439): torques spread with the regular ES kernel of the dipole's
    (w, beta, alpha), their curl and the fluid vorticity taken spectrally."""
    domType: str
    Nx: int
    Ny: int
    Nz: int
    Lx: float
    Ly: float
    Lz: float
    z0: float = 0.0
    eta: float = 1.0 / (6.0 * math.pi)
    wm: int = 6
    betam_hat: float = 1.714
    has_torque: bool = False
    wd: int = 6
    betad_hat: float = 2.2160
    radius: float = 1.0
    reg_kernel: bool = False  # torques with the regular kernel and spectral curls (useRegKernel)

    @property
    def hx(self):
        return self.Lx / self.Nx

    @property
    def hy(self):
        return self.Ly / self.Ny

    @property
    def hz(self):
        return self.Lz / self.Nz if self.domType == 'TP' else 0.0

    def alpha(self, w):
        cw = self.radius / (w * self.hx)  # GridAndKernelConfig.py:328-329
        return self.radius / (2 * cw)  # ParticleList.cpp:229

    def as_dict(self):
        return dict(domType=self.domType, Nx=self.Nx, Ny=self.Ny, Nz=self.Nz, Lx=self.Lx,
                    Ly=self.Ly, Lz=self.Lz, z0=self.z0, eta=self.eta, wm=self.wm,
                    betam_hat=self.betam_hat, has_torque=self.has_torque, wd=self.wd,
                    betad_hat=self.betad_hat, radius=self.radius, reg_kernel=self.reg_kernel)


def domain_bcs(domType):
    """Per-(axis end, component) BCs, FCM.py:211-229 and 244-248.
    Returns (BCs, BCst_z) as int arrays of length 18 = 6 ends x 3 dof;
    index 4*3+d is the z end at z=Lz (extended index 0), 5*3+d the end at z=0."""
    BCs = np.full(18, BC_NONE, dtype=np.int64)
    if domType == 'TP':  # periodic in z: the BCs are not used
        return BCs, BCs.copy()
    if domType == 'DPBW':
        BCs[15:18] = BC_MIRROR_INV
    elif domType == 'DPSC':
        BCs[12:15] = BC_MIRROR_INV
        BCs[15:18] = BC_MIRROR_INV
    elif domType != 'DP':
        raise ValueError('domType not supported')
    BCst = np.full(18, BC_NONE, dtype=np.int64)
    if domType in ('DPBW', 'DPSC'):
        BCst[15:18] = BC_MIRROR
        if domType == 'DPSC':
            BCst[12:15] = BC_MIRROR
    return BCs, BCst


# --------------------------------------------------------------------------
# Quadrature and kernels
# --------------------------------------------------------------------------
def clencurt(Np1, a, b):
    """Clenshaw-Curtis nodes (descending) and weights, Chebyshev.py:4-38 /
    Quadrature.cpp:11-46 (Trefethen's clencurt)."""
    N = Np1 - 1
    H = (b - a) / 2.0
    bpad2 = (b + a) / 2.0
    cpts = H * np.cos(np.pi * np.arange(0, Np1) / N) + bpad2
    cwts = np.zeros(Np1)
    if N % 2:
        w1 = H / (N * N)
        end = (N - 1) // 2 + 1
    else:
        w1 = H / (N * N - 1)
        end = N // 2
    cwts[0] = w1
    cwts[N] = w1
    v = np.ones(N - 1)
    ii = np.arange(1, N)
    for k in range(1, end):
        v -= 2 * np.cos(2.0 * k * np.pi * ii / N) / (4.0 * k * k - 1.0)
    if N % 2 == 0:
        v -= np.cos(N * np.pi * ii / N) / (N * N - 1)
    cwts[1:N] = 2 * H * v / N
    return cpts, cwts


def es_norm(beta, alpha):
    """1-D ES kernel integral by 1000-point Clenshaw-Curtis on [-alpha, alpha]
    (ParticleList.cpp:217-241)."""
    cpts, cwts = clencurt(1000, -alpha, alpha)
    f = np.exp(beta * (np.sqrt(1 - cpts * cpts / (alpha * alpha)) - 1))
    s = 0.0
    for a, b in zip(f, cwts):  # sequential accumulation, as in the reference
        s += a * b
    return s


def dipole_threshold(beta, alpha):
    """Largest |x| at which the ES-derivative kernel is used
    (ParticleList.cpp:260-265).  The csqrt argument is a real expression
    promoted to complex with +0 imaginary part, as in C99."""
    bw = float(beta)
    s = np.sqrt(complex(-12 * bw * bw + 81, 0.0))
    z = ((8 * bw * bw) + 12.0 * s - 108.0) * bw
    t = 6.0 * z ** (1.0 / 3.0) / bw + 24.0 * bw * z ** (-1.0 / 3.0) + 12.0
    return float((np.sqrt(t) * alpha / 6.0).real)


def cround(v):
    """std::round (half away from zero) for non-negative v."""
    return int(math.floor(v + 0.5))


class Kernel:
    """One ES kernel (monopole or dipole) as the ParticleList sees it."""

    def __init__(self, w, beta_hat, alpha, dipole):
        self.w = int(w)
        self.beta = beta_hat * w  # SpreadInterp.h:123 (betafPc * wfPc)
        self.alpha = alpha
        self.norm = es_norm(self.beta, alpha)
        self.thr = dipole_threshold(self.beta, alpha) if dipole else alpha
        self.dipole = dipole


# --------------------------------------------------------------------------
# Grid + particle locator (ParticleList.cpp:394-548)
# --------------------------------------------------------------------------
class GridState:
    """A reference Grid: interior grid [Ny][Nx][Nz][3], extended grid
    [Nzeff][Nyeff][Nxeff][3] (kept between spread and interpolation), and the
    extended Chebyshev z grid."""

    def __init__(self, p, zpts, zwts, thr_max, wmax):
        self.p = p
        self.Nx, self.Ny, self.Nz = p.Nx, p.Ny, p.Nz
        self.Nxeff = p.Nx + wmax + (wmax % 2)
        self.Nyeff = p.Ny + wmax + (wmax % 2)
        zG = zpts
        ext_up = 0
        i = 1
        while zG[0] - zG[i] <= thr_max:
            ext_up += 1
            i += 1
        ext_down = 0
        i = p.Nz - 2
        while zG[i] - zG[p.Nz - 1] <= thr_max:
            ext_down += 1
            i -= 1
        if ext_up != ext_down:
            raise ValueError('asymmetric z ghost extension is not supported')
        self.ext = ext_up
        self.Nzeff = p.Nz + ext_up + ext_down
        zext = np.zeros(self.Nzeff)
        wext = np.zeros(self.Nzeff)
        zext[ext_up:self.Nzeff - ext_down] = zG
        wext[ext_up:self.Nzeff - ext_down] = zwts
        j = 0
        for i in range(ext_up, 0, -1):
            zext[j] = 2.0 * zG[0] - zG[i]
            wext[j] = zwts[i]
            j += 1
        j = self.Nzeff - ext_down
        for i in range(p.Nz - 2, p.Nz - 2 - ext_down, -1):
            zext[j] = -1.0 * zG[i]
            wext[j] = zwts[i]
            j += 1
        self.zext, self.wext = zext, wext
        self.ext_grid = np.zeros((self.Nzeff, self.Nyeff, self.Nxeff, 3))
        self.periodic_z = False


class GridStateTP:
    """A reference Grid with uniform periodic z (hz > 0, Grid.cpp:26-29):
    the extended sizes of ParticleList::locateOnGridUnifZ
    (ParticleList.cpp:307-309), N + w + (w mod 2) on every axis."""

    def __init__(self, p, wmax, wzmax):
        self.p = p
        self.Nx, self.Ny, self.Nz = p.Nx, p.Ny, p.Nz
        self.Nxeff = p.Nx + wmax + (wmax % 2)
        self.Nyeff = p.Ny + wmax + (wmax % 2)
        self.Nzeff = p.Nz + wzmax + (wzmax % 2)
        self.ext = (self.Nzeff - self.Nz) // 2
        self.ext_grid = np.zeros((self.Nzeff, self.Nyeff, self.Nxeff, 3))
        self.periodic_z = True


@dataclass
class Located:
    xclose: np.ndarray
    yclose: np.ndarray
    xun: np.ndarray  # [N, w]
    yun: np.ndarray  # [N, w]
    indl: np.ndarray
    wz: np.ndarray
    zun: np.ndarray  # [N, wzmax] (0-padded)
    ptw: np.ndarray  # [N, wzmax] hx*hy*w_cc (0-padded)


def locate(p, g, kern, X):
    """Stencil of every particle (ParticleList.cpp:394-526).  X is [N,3]
    already shifted by (0, 0, z0)."""
    hx, hy = p.hx, p.hy
    w = kern.w
    thr = kern.thr
    x, y, z = X[:, 0], X[:, 1], X[:, 2]
    if (x < 0).any() or (x > p.Lx).any() or (y < 0).any() or (y > p.Ly).any() \
            or (z < 0).any() or (z > p.Lz).any():
        raise ValueError('Particles are outside of the unit cell.')
    wx = cround(2 * thr / hx)
    wy = cround(2 * thr / hy)
    if wx != w or wy != w:
        # the reference would use round(2*thr/h) as the stencil width
        w = wx
    evenx = -1 * (wx % 2) + 1
    eveny = -1 * (wy % 2) + 1
    xclose = (x / hx).astype(np.int64)
    yclose = (y / hy).astype(np.int64)
    xclose += ((wx % 2) & ((x / hx - xclose) > 0.5)).astype(np.int64)
    yclose += ((wy % 2) & ((y / hy - yclose) > 0.5)).astype(np.int64)
    j = np.arange(wx)
    xun = ((xclose[:, None].astype(np.float64) + j[None, :]) - (wx // 2) + evenx) * hx - x[:, None]
    xun = np.where((xun > thr) | (xun < -thr), thr, xun)
    j = np.arange(wy)
    yun = ((yclose[:, None].astype(np.float64) + j[None, :]) - (wy // 2) + eveny) * hy - y[:, None]
    yun = np.where((thr < yun) | (yun < -thr), thr, yun)
    # z window: lower_bound with std::greater on the descending extended grid
    asc = g.zext[::-1]
    n = g.Nzeff
    indl = n - np.searchsorted(asc, z + thr, side='right')
    high = n - np.searchsorted(asc, z - thr, side='right')
    indr = high.copy()
    at_end = indr == n
    indr[at_end] -= 1
    lt = ~at_end
    lt_idx = np.where(lt)[0]
    dec = (z[lt_idx] - thr) > g.zext[indr[lt_idx]]
    indr[lt_idx[dec]] -= 1
    wz = indr - indl + 1
    wzmax = int(wz.max())
    k = np.arange(wzmax)
    idx = indl[:, None] + k[None, :]
    valid = k[None, :] < wz[:, None]
    idxc = np.where(valid, idx, 0)
    zun = g.zext[idxc] - z[:, None]
    zun = np.where((thr < zun) | (zun < -thr), thr, zun)
    zun = np.where(valid, zun, 0.0)
    ptw = np.where(valid, hx * hy * g.wext[idxc], 0.0)
    return Located(xclose, yclose, xun, yun, indl, wz, zun, ptw)


def locate_tp(p, g, kern, X):
    """Stencil of every particle on the uniform periodic z grid
    (ParticleList.cpp:285-366): the z window is built like the x and y
    windows, round(2 thr / hz) points from the nearest node, its first entry
    at extended index zclose - wz/2 + evenz + (Nzeff - Nz)/2 (the zoffset of
    :357); interpolation weight hx*hy*hz (SpreadInterp.cpp:168).  X is [N,3]
    already shifted by (0, 0, z0)."""
    hx, hy, hz = p.hx, p.hy, p.hz
    thr = kern.thr
    x, y, z = X[:, 0], X[:, 1], X[:, 2]
    if (x < 0).any() or (x > p.Lx).any() or (y < 0).any() or (y > p.Ly).any() \
            or (z < 0).any() or (z > p.Lz).any():
        raise ValueError('Particles are outside of the unit cell.')
    wx, wy, wz = cround(2 * thr / hx), cround(2 * thr / hy), cround(2 * thr / hz)
    evenx, eveny, evenz = 1 - wx % 2, 1 - wy % 2, 1 - wz % 2
    xclose = (x / hx).astype(np.int64)
    yclose = (y / hy).astype(np.int64)
    zclose = (z / hz).astype(np.int64)
    xclose += ((wx % 2) & ((x / hx - xclose) > 0.5)).astype(np.int64)
    yclose += ((wy % 2) & ((y / hy - yclose) > 0.5)).astype(np.int64)
    zclose += ((wz % 2) & ((z / hz - zclose) > 0.5)).astype(np.int64)

    def offsets(close, w, even, h, c):
        j = np.arange(w)
        o = ((close[:, None].astype(np.float64) + j[None, :]) - (w // 2) + even) * h - c[:, None]
        return np.where((o > thr) | (o < -thr), thr, o)

    xun = offsets(xclose, wx, evenx, hx, x)
    yun = offsets(yclose, wy, eveny, hy, y)
    zun = offsets(zclose, wz, evenz, hz, z)
    n = X.shape[0]
    indl = zclose - wz // 2 + evenz + (g.Nzeff - g.Nz) // 2
    wzs = np.full(n, wz, dtype=np.int64)
    ptw = np.full((n, wz), hx * hy * hz)
    return Located(xclose, yclose, xun, yun, indl, wzs, zun, ptw)


def kernel_weights(kern, loc, deriv=None):
    """delta[N, wz, wy, wx] = esKernel(x)/norm^3 or its derivative along
    `deriv` (ESKernels.h:8-46, SpreadInterp.h:100-128); zero outside wz."""
    a2 = kern.alpha * kern.alpha
    b = kern.beta
    sx = np.sqrt(1 - loc.xun * loc.xun / a2)  # [N, wx]
    sy = np.sqrt(1 - loc.yun * loc.yun / a2)
    sz = np.sqrt(1 - loc.zun * loc.zun / a2)  # [N, wz]
    expo = b * (sx[:, None, None, :] + sy[:, None, :, None] + sz[:, :, None, None] - 3)
    val = np.exp(expo)
    if deriv is not None:
        if deriv == 0:
            xc = np.broadcast_to(loc.xun[:, None, None, :], val.shape)
            sc = np.broadcast_to(sx[:, None, None, :], val.shape)
        elif deriv == 1:
            xc = np.broadcast_to(loc.yun[:, None, :, None], val.shape)
            sc = np.broadcast_to(sy[:, None, :, None], val.shape)
        else:
            xc = np.broadcast_to(loc.zun[:, :, None, None], val.shape)
            sc = np.broadcast_to(sz[:, :, None, None], val.shape)
        val = -b * xc * val / (a2 * sc)
    norm = kern.norm
    norm3 = norm * norm * norm
    val = val / norm3
    k = np.arange(loc.zun.shape[1])
    valid = k[None, :] < loc.wz[:, None]
    return np.where(valid[:, :, None, None], val, 0.0)


def _ext_indices(g, loc, w):
    even = -1 * (w % 2) + 1
    lend = (g.Nxeff - g.Nx) // 2
    bend = (g.Nyeff - g.Ny) // 2
    ii = loc.xclose + lend
    jj = loc.yclose + bend
    j = np.arange(w)
    i3 = ii[:, None] + j[None, :] - w // 2 + even  # [N, w]
    j3 = jj[:, None] + j[None, :] - w // 2 + even
    k3 = loc.indl[:, None] + np.arange(loc.zun.shape[1])[None, :]
    k3 = np.minimum(k3, g.Nzeff - 1)  # padded entries carry zero weight
    if (i3 < 0).any() or (i3 >= g.Nxeff).any() or (j3 < 0).any() or (j3 >= g.Nyeff).any():
        raise ValueError('stencil outside the extended grid (particle at x=Lx or y=Ly)')
    flat = (k3[:, :, None, None] * g.Nyeff + j3[:, None, :, None]) * g.Nxeff + i3[:, None, None, :]
    return flat  # [N, wz, wy, wx]


def _chunks(loc, size=4096):
    n = loc.xclose.shape[0]
    for a in range(0, n, size):
        sl = slice(a, min(n, a + size))
        yield sl, Located(loc.xclose[sl], loc.yclose[sl], loc.xun[sl], loc.yun[sl],
                          loc.indl[sl], loc.wz[sl], loc.zun[sl], loc.ptw[sl])


def spread(g, kern, loc, Fp, deriv=None):
    """Zero the extended grid, spread Fp [N,3] into it (spreadNonUnifZ,
    SpreadInterp.cpp:302-448); the caller folds."""
    g.ext_grid[...] = 0.0
    ext = g.ext_grid.reshape(-1, 3)
    for sl, lc in _chunks(loc):
        delta = kernel_weights(kern, lc, deriv)
        idx = _ext_indices(g, lc, kern.w).ravel()
        for d in range(3):
            vals = (delta * Fp[sl, d][:, None, None, None]).ravel()
            np.add.at(ext[:, d], idx, vals)


def interpolate(g, kern, loc, deriv=None):
    """interpNonUnifZ (SpreadInterp.cpp:450-600): sum of extended-grid values
    x kernel x hx*hy*w_cc(z)."""
    ext = g.ext_grid.reshape(-1, 3)
    out = np.zeros((loc.xclose.shape[0], 3))
    for sl, lc in _chunks(loc):
        delta = kernel_weights(kern, lc, deriv)
        flat = _ext_indices(g, lc, kern.w)
        wgt = delta * lc.ptw[:, :, None, None]
        out[sl] = np.einsum('nkjid,nkji->nd', ext[flat], wgt)
    return out


def fold(g, BCs):
    """DeGhostify: BoundaryConditions.h:22-361 (x,y periodic; z per BC) and
    the permuted copy of the interior into fG [Ny][Nx][Nz][3]."""
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
    if g.periodic_z:  # BoundaryConditions.h:241-283
        e[Nz:Nz + dend] += e[0:dend]
        e[ubeg - Nz:g.Nzeff - Nz] += e[ubeg:g.Nzeff]
        inner = e[dend:ubeg, bend:tbeg, lend:rbeg, :]
        return np.ascontiguousarray(inner.transpose(1, 2, 0, 3))
    for d in range(3):
        bc = BCs[12 + d]
        if bc != BC_NONE:
            s = 1.0 if bc == BC_MIRROR else -1.0
            src = np.arange(0, dend + 1)
            dst = 2 * dend - src
            tmp = e[src, :, :, d].copy()
            e[dst, :, :, d] += s * tmp
    for d in range(3):
        bc = BCs[15 + d]
        if bc != BC_NONE:
            s = 1.0 if bc == BC_MIRROR else -1.0
            src = np.arange(ubeg - 1, g.Nzeff)
            dst = 2 * ubeg - src - 2
            tmp = e[src, :, :, d].copy()
            e[dst, :, :, d] += s * tmp
    inner = e[dend:ubeg, bend:tbeg, lend:rbeg, :]  # [Nz][Ny][Nx][3]
    return np.ascontiguousarray(inner.transpose(1, 2, 0, 3))


def ghost_copy(g, fG, BCs):
    """Ghostify: BoundaryConditions.h:377-731.  Ghost z layers at BC 'none'
    ends are left as they are (they still hold the last spread)."""
    e = g.ext_grid
    Nx, Ny, Nz = g.Nx, g.Ny, g.Nz
    lend = (g.Nxeff - Nx) // 2
    rbeg = g.Nxeff - lend
    bend = (g.Nyeff - Ny) // 2
    tbeg = g.Nyeff - bend
    dend = (g.Nzeff - Nz) // 2
    ubeg = g.Nzeff - dend
    e[dend:ubeg, bend:tbeg, lend:rbeg, :] = fG.transpose(2, 0, 1, 3)
    zs = slice(dend, ubeg)
    e[zs, bend:tbeg, 0:lend, :] = e[zs, bend:tbeg, Nx:Nx + lend, :]
    e[zs, bend:tbeg, rbeg:g.Nxeff, :] = e[zs, bend:tbeg, rbeg - Nx:g.Nxeff - Nx, :]
    e[zs, tbeg:g.Nyeff, :, :] = e[zs, tbeg - Ny:g.Nyeff - Ny, :, :]
    e[zs, 0:bend, :, :] = e[zs, Ny:Ny + bend, :, :]
    if g.periodic_z:  # BoundaryConditions.h:608-647
        e[ubeg:g.Nzeff] = e[ubeg - Nz:g.Nzeff - Nz]
        e[0:dend] = e[Nz:Nz + dend]
        return
    for d in range(3):
        bc = BCs[12 + d]
        if bc != BC_NONE:
            s = 1.0 if bc == BC_MIRROR else -1.0
            k = np.arange(0, dend)
            e[k, :, :, d] = s * e[2 * dend - k, :, :, d]
            e[dend, :, :, d] += s * e[dend, :, :, d]
    for d in range(3):
        bc = BCs[15 + d]
        if bc != BC_NONE:
            s = 1.0 if bc == BC_MIRROR else -1.0
            k = np.arange(ubeg - 1, g.Nzeff)
            e[k, :, :, d] = s * e[2 * ubeg - k - 2, :, :, d]
            e[ubeg - 1, :, :, d] += s * e[ubeg - 1, :, :, d]


# --------------------------------------------------------------------------
# Fourier-Chebyshev transform (Transform.cpp:107-304)
# --------------------------------------------------------------------------
def fc_forward(fG):
    """[Ny][Nx][Nz][3] real -> Fourier (unnormalised) x Chebyshev coefficients."""
    Ny, Nx, Nz, nd = fG.shape
    Nu = 2 * Nz - 2
    ext = np.concatenate([fG, fG[:, :, Nz - 2:0:-1, :]], axis=2)
    X = np.fft.fftn(ext, axes=(0, 1, 2))
    out = np.empty((Ny, Nx, Nz, nd), dtype=np.complex128)
    out[:, :, 0] = X[:, :, 0] / Nu
    out[:, :, 1:Nz - 1] = (X[:, :, 1:Nz - 1] + X[:, :, Nu - 1:Nz - 1:-1]) / Nu
    out[:, :, Nz - 1] = X[:, :, Nz - 1] / Nu
    return out


def fc_backward(U):
    """Chebyshev coefficients x Fourier -> real grid (real part)."""
    Ny, Nx, Nz, nd = U.shape
    Nu = 2 * Nz - 2
    Y = np.empty((Ny, Nx, Nu, nd), dtype=np.complex128)
    Y[:, :, 0] = Nu * U[:, :, 0]
    Y[:, :, 1:Nz - 1] = Nu * U[:, :, 1:Nz - 1] / 2
    Y[:, :, Nz - 1] = Nu * U[:, :, Nz - 1]
    Y[:, :, Nz:] = Nu * U[:, :, Nz - 2:0:-1] / 2
    u = np.fft.ifftn(Y, axes=(0, 1, 2))
    return np.ascontiguousarray(u[:, :, :Nz, :].real)


# --------------------------------------------------------------------------
# Doubly periodic solver (Solvers.py:258-347, 603-643; Chebyshev.py:96-160;
# LinearSolvers.*; DPTools.cpp)
# --------------------------------------------------------------------------
def first_integral_matrix(N, H):
    M = np.zeros((N, N + 2))
    jj = np.arange(2, N)
    colm1 = np.concatenate(([1], 1 / (2 * jj)))
    colp1 = np.concatenate(([0, -1 / 2], -1 / (2 * jj) * (jj < N - 1)))
    for r in range(1, N):
        M[r, r - 1] = colm1[r - 1]
    for r in range(0, N):
        if r + 1 < N + 2:
            M[r, r + 1] = colp1[r]
    M[0, N + 1] = 1
    return H * M


def second_integral_matrix(N, H):
    M = np.zeros((N, N + 2))
    jj = np.arange(3, N)
    colm2 = np.concatenate(([0.25], 1 / (2 * jj * (2 * jj - 2))))
    colp2 = np.concatenate(([0, 0.125, 1. / 24.], 1 / (2 * jj * (2 * jj + 2)) * (jj < N - 2)))
    col0 = np.concatenate(([0, -0.125, -1. / 8. - 1. / 24.],
                           -1 / (2 * jj * (2 * jj - 2)) - 1 / (2 * jj * (2 * jj + 2)) * (jj < N - 1)))
    for r in range(2, N):
        M[r, r - 2] = colm2[r - 2]
    for r in range(0, N):
        M[r, r] = col0[r]
        M[r, r + 2] = colp2[r]
    M[0, N] = 1
    M[1, N + 1] = 1
    return H ** 2 * M


def precompute_ints(Nz, H):
    theta = np.pi * np.arange(0, 1000).reshape(-1, 1) / 999
    _, zwts = clencurt(1000, 0, 2 * H)
    zwts = zwts.reshape(1, -1)
    pints = np.dot(zwts, np.cos(np.arange(0, Nz) * theta)).ravel()
    uvints = (H * np.dot(zwts, np.cos(np.arange(0, Nz) * theta) * np.cos(theta))).ravel()
    return pints, uvints


def no_wall_bcs(N):
    """BC rows, Solvers.py:603-643."""
    BCR1 = np.zeros(N + 2)
    BCR2 = np.zeros(N + 2)
    BCL1 = np.zeros(N + 2)
    BCL2 = np.zeros(N + 2)
    BCR1[N + 1] = 1; BCR2[N] = 1; BCR1[0] = 1; BCR1[2] = -1 / 2
    BCR2[N + 1] += 1; BCR2[1] = -1 / 8; BCR2[3] = 1 / 8
    BCR1[1] += 1 / 4; BCR1[3] -= 1 / 4; BCR2[0] += 1 / 4; BCR2[2] -= (1 / 8 + 1 / 24)
    BCR2[4] += 1 / 24
    BCL1[N + 1] = 1; BCL2[N] = -1; BCL1[0] = -1; BCL1[2] = 1 / 2
    BCL2[N + 1] += 1; BCL2[1] = -1 / 8; BCL2[3] = 1 / 8
    BCL1[1] += 1 / 4; BCL1[3] -= 1 / 4; BCL2[0] -= 1 / 4; BCL2[2] += 1 / 8 + 1 / 24
    BCL2[4] -= 1 / 24
    jj = np.arange(3, N)
    BCR1[2:N - 1] += 1 / (2 * jj)
    BCL1[2:N - 1] += np.power(-1, jj) / (2 * jj)
    BCR1[4:N + 1] -= 1 / (2 * jj) * (jj < N - 1)
    BCL1[4:N + 1] -= np.power(-1, jj) / (2 * jj) * (jj < N - 1)
    BCR2[1:N - 2] += 1 / (2 * jj) * 1 / (2 * jj - 2)
    BCL2[1:N - 2] -= 1 / (2 * jj) * 1 / (2 * jj - 2) * np.power(-1, jj)
    BCR2[5:N + 2] += 1 / (2 * jj) * 1 / (2 * jj + 2) * (jj < N - 2)
    BCL2[5:N + 2] -= 1 / (2 * jj) * 1 / (2 * jj + 2) * np.power(-1, jj) * (jj < N - 2)
    BCR2[3:N] -= (1 / (2 * jj) * 1 / (2 * jj - 2) + 1 / (2 * jj) * 1 / (2 * jj + 2) * (jj < N - 1))
    BCL2[3:N] += (1 / (2 * jj) * 1 / (2 * jj - 2) + 1 / (2 * jj) * 1 / (2 * jj + 2) * (jj < N - 1)) \
        * np.power(-1, jj)
    return BCR1, BCR2, BCL1, BCL2


@dataclass
class DPSolver:
    Nx: int
    Ny: int
    Nz: int
    Lx: float
    Ly: float
    H: float
    eta: float
    modes: np.ndarray = None  # optional subset of flattened wavenumbers (timing samples)
    Kx: np.ndarray = field(init=False)
    Ky: np.ndarray = field(init=False)

    def __post_init__(self):
        Nx, Ny, Nz, H = self.Nx, self.Ny, self.Nz, self.H
        kx = 2 * np.pi * np.concatenate((np.arange(0, np.floor(Nx / 2) + 1),
                                         np.arange(-1 * np.ceil(Nx / 2) + 1, 0))) / self.Lx
        ky = 2 * np.pi * np.concatenate((np.arange(0, np.floor(Ny / 2) + 1),
                                         np.arange(-1 * np.ceil(Ny / 2) + 1, 0))) / self.Ly
        Kx, Ky = [K.flatten() for K in np.meshgrid(kx, ky, indexing='xy')]
        Dx = 1j * Kx
        Dy = 1j * Ky
        if Nx % 2 == 0:
            Dx.reshape((Ny, Nx))[:, Nx // 2] = 0
        if Ny % 2 == 0:
            Dy.reshape((Ny, Nx))[Ny // 2, :] = 0
        if self.modes is not None:
            Kx, Ky, Dx, Dy = Kx[self.modes], Ky[self.modes], Dx[self.modes], Dy[self.modes]
        Ksq = Kx ** 2 + Ky ** 2
        self.Kx, self.Ky, self.K = Kx, Ky, np.sqrt(Ksq)
        self.Dx, self.Dy = Dx, Dy
        self.FIMat = first_integral_matrix(Nz, H)
        self.SIMat = second_integral_matrix(Nz, H)
        self.pints, self.uvints = precompute_ints(Nz, H)
        BCR1, BCR2, BCL1, BCL2 = no_wall_bcs(Nz)
        self.BCR1, self.BCR2, self.BCL1, self.BCL2 = BCR1, BCR2, BCL1, BCL2
        BCs_k0 = np.stack((BCR2, -BCL2), axis=0)
        BCs_k = np.einsum('ij, k->kij', np.stack((BCR2, BCL2), axis=0), H ** 2 * self.K)
        BCs_k += BCs_k0 + np.stack((H * BCR1 - BCR2, H * BCL1 + BCL2), axis=0)
        S = self.SIMat
        d0 = 1.0 - np.diag(S[:, :Nz])[None, :] * Ksq[:, None]
        dp2 = 0.0 - np.diag(S[:, :Nz], 2)[None, :] * Ksq[:, None]
        dm2 = 0.0 - np.diag(S[:, :Nz], -2)[None, :] * Ksq[:, None]
        B = -Ksq[:, None, None] * S[None, :, Nz:]  # [k, Nz, 2]
        C = BCs_k[:, :, :Nz]  # [k, 2, Nz]
        D = BCs_k[:, :, Nz:]  # [k, 2, 2] (row, col)
        nk = Kx.shape[0]
        beta = np.zeros((nk, Nz + 1))
        beta[:, 1] = d0[:, 0]
        beta[:, 2] = d0[:, 1]
        for i in range(3, Nz + 1):
            beta[:, i] = d0[:, i - 1] - dm2[:, i - 3] * dp2[:, i - 3] / beta[:, i - 2]
        self.beta, self.dp2, self.dm2 = beta, dp2, dm2
        with np.errstate(divide='ignore', invalid='ignore'):
            AinvB = np.stack([self._penta(B[:, :, c], real=True) for c in range(2)], axis=2)
        G = np.einsum('krj,kjc->krc', C, AinvB) - D
        Ginv = np.empty_like(G)
        with np.errstate(divide='ignore', invalid='ignore'):  # k=0 row is unused
            det = 1.0 / (G[:, 0, 0] * G[:, 1, 1] - G[:, 0, 1] * G[:, 1, 0])
            Ginv[:, 0, 0] = G[:, 1, 1] * det
            Ginv[:, 1, 0] = -G[:, 1, 0] * det
            Ginv[:, 0, 1] = -G[:, 0, 1] * det
            Ginv[:, 1, 1] = G[:, 0, 0] * det
        self.AinvB, self.C, self.Ginv = AinvB, C, Ginv
        self.C_k0 = BCs_k0[:, :Nz]
        D_k0 = -BCs_k0[:, Nz:]
        self.Ginv_k0 = 1.0 / (D_k0[0, 0] * D_k0[1, 1] - D_k0[0, 1] * D_k0[1, 0]) * \
            np.array([[D_k0[1, 1], -D_k0[0, 1]], [-D_k0[1, 0], D_k0[0, 0]]])

    def _penta(self, rhs, real=False, ks=slice(None)):
        """KBPENTA solve (LinearSolvers.h:76-141) for all k, rhs [k, Nz]."""
        Nz = self.Nz
        beta, dp2, dm2 = self.beta[ks], self.dp2[ks], self.dm2[ks]
        x = np.array(rhs, copy=True)
        for i in range(2, Nz):
            x[:, i] = rhs[:, i] - dm2[:, i - 2] * x[:, i - 2] / beta[:, i - 1]
        x[:, Nz - 1] /= beta[:, Nz]
        x[:, Nz - 2] /= beta[:, Nz - 1]
        for i in range(Nz - 3, -1, -1):
            x[:, i] = (x[:, i] - dp2[:, i] * x[:, i + 2]) / beta[:, i + 1]
        return x

    def solve_no_wall(self, fhat):
        """doublyPeriodicSolve_no_wall (DPTools.cpp:81-132) for k >= 1;
        fhat [k, Nz, 3] complex.  Returns U [k, Nz, 3] (k=0 row zero)."""
        Nz, H, eta = self.Nz, self.H, self.eta
        ks = slice(1, None)
        f = fhat[1:]
        Dx = self.Dx[1:][:, None]
        Dy = self.Dy[1:][:, None]
        # chebCoeffDiff (DPTools.cpp:134-174), z component
        df = np.zeros((f.shape[0], Nz), dtype=np.complex128)
        df[:, Nz - 2] = ((Nz - 1) * 2 / H) * f[:, Nz - 1, 2]
        for k in range(2, Nz):
            df[:, Nz - k - 1] = df[:, Nz - k + 1] + ((Nz - k) * 2 / H) * f[:, Nz - k, 2]
        df[:, 0] /= 2
        p_rhs = Dx * f[:, :, 0] + Dy * f[:, :, 1] + df
        AinvB, C, Ginv = self.AinvB[ks], self.C[ks], self.Ginv[ks]
        S, FI = self.SIMat, self.FIMat

        def schur(rhs):
            xp = self._penta(rhs, ks=ks)
            y0 = np.sum(xp * C[:, 0, :], axis=1)
            y1 = np.sum(xp * C[:, 1, :], axis=1)
            return xp, y0, y1

        xp, y0, y1 = schur(p_rhs)
        g0 = Ginv[:, 0, 0] * y0 + Ginv[:, 0, 1] * y1
        g1 = Ginv[:, 1, 0] * y0 + Ginv[:, 1, 1] * y1
        x = np.concatenate([xp - (AinvB[:, :, 0] * g0[:, None] + AinvB[:, :, 1] * g1[:, None]),
                            g0[:, None], g1[:, None]], axis=1)
        cp = x @ S.T
        dp = x @ FI.T
        u_rhs = np.stack([(Dx * cp - f[:, :, 0]) / eta, (Dy * cp - f[:, :, 1]) / eta,
                          (dp - f[:, :, 2]) / eta], axis=2)
        sgn = np.power(-1.0, np.arange(Nz))
        ssum = np.sum(cp, axis=1)
        asum = np.sum(cp * sgn[None, :], axis=1)
        fac1 = 2 * eta
        fac = fac1 * self.K[1:]
        Dxs, Dys = self.Dx[1:], self.Dy[1:]
        bc = [(-Dxs * ssum / fac, Dxs * asum / fac), (-Dys * ssum / fac, Dys * asum / fac),
              (ssum / fac1, asum / fac1)]
        U = np.zeros((fhat.shape[0], Nz, 3), dtype=np.complex128)
        for c in range(3):
            xp, y0, y1 = schur(u_rhs[:, :, c])
            b0, b1 = bc[c]
            g0 = Ginv[:, 0, 0] * (y0 - b0) + Ginv[:, 0, 1] * (y1 - b1)
            g1 = Ginv[:, 1, 0] * (y0 - b0) + Ginv[:, 1, 1] * (y1 - b1)
            x = np.concatenate([xp - (AinvB[:, :, 0] * g0[:, None] + AinvB[:, :, 1] * g1[:, None]),
                                g0[:, None], g1[:, None]], axis=1)
            U[1:, :, c] = x @ S.T
        return U

    def cheb_of_samples(self, vals):
        """Chebyshev coefficients of samples at the nodes through the even
        extension FFT (DPTools.cpp:643-697); vals [..., Nz]."""
        Nz = self.Nz
        n = 2 * Nz - 2
        ext = np.concatenate([vals, vals[..., Nz - 2:0:-1]], axis=-1)
        X = np.fft.fft(ext, axis=-1)
        out = np.empty(vals.shape, dtype=np.complex128)
        out[..., 0] = X[..., 0] / n
        out[..., 1:Nz - 1] = (X[..., 1:Nz - 1] + X[..., n - 1:Nz - 1:-1]) / n
        out[..., Nz - 1] = X[..., Nz - 1] / n
        return out

    def wall_values(self, U, theta):
        """evalTheta (DPTools.cpp:348-378)."""
        c = np.cos(np.arange(self.Nz) * theta)
        return np.einsum('kjd,j->kd', U, c)

    def correct_bottom(self, U, z):
        """evalCorrectionSol_bottomWall (DPTools.cpp:590-700), velocity only."""
        fh = -self.wall_values(U, np.pi)[1:]
        kx, ky, k = self.Kx[1:], self.Ky[1:], self.K[1:]
        alpha = kx * fh[:, 0] + ky * fh[:, 1] + 1j * k * fh[:, 2]
        enkz = np.exp(-k[:, None] * z[None, :])
        zenkz = z[None, :] * enkz
        a = alpha[:, None]
        Cu = -kx[:, None] * a * zenkz / k[:, None] + fh[:, 0:1] * enkz
        Cv = -ky[:, None] * a * zenkz / k[:, None] + fh[:, 1:2] * enkz
        Cw = -1j * a * zenkz + fh[:, 2:3] * enkz
        corr = self.cheb_of_samples(np.stack([Cu, Cv, Cw], axis=1))  # [k, 3, Nz]
        U[1:] += corr.transpose(0, 2, 1)

    def correct_slit(self, U, z, Hs):
        """evalCorrectionSol_slitChannel (DPTools.cpp:704-877), velocity only;
        Hs is the channel height (the caller passes Lz, Solvers.py:557)."""
        eta = self.eta
        fb = -self.wall_values(U, np.pi)[1:]
        ft = -self.wall_values(U, 0.0)[1:]
        kx, ky = self.Kx[1:], self.Ky[1:]
        k = np.sqrt(kx * kx + ky * ky)
        fac = 1.0 / 2.0 / eta
        nk = kx.shape[0]
        A = np.zeros((nk, 8, 8), dtype=np.complex128)
        enkh = np.exp(-k * Hs)
        A[:, 0, 0] = fac; A[:, 0, 1] = enkh * fac; A[:, 0, 6] = -k; A[:, 0, 7] = k * enkh
        A[:, 1, 0] = (1 - k * Hs) * enkh * fac; A[:, 1, 1] = (1 + k * Hs) * fac
        A[:, 1, 6] = -k * enkh; A[:, 1, 7] = k
        A[:, 2, 2] = 1; A[:, 2, 3] = enkh
        A[:, 3, 4] = 1; A[:, 3, 5] = enkh
        A[:, 4, 6] = 1; A[:, 4, 7] = enkh
        A[:, 5, 0] = -1j * kx * Hs * enkh * fac / k; A[:, 5, 1] = 1j * kx * Hs * fac / k
        A[:, 5, 2] = enkh; A[:, 5, 3] = 1
        A[:, 6, 0] = -1j * ky * Hs * enkh * fac / k; A[:, 6, 1] = 1j * ky * Hs * fac / k
        A[:, 6, 4] = enkh; A[:, 6, 5] = 1
        A[:, 7, 0] = Hs * enkh * fac; A[:, 7, 1] = Hs * fac; A[:, 7, 6] = enkh; A[:, 7, 7] = 1
        rhs = np.stack([-1j * kx * fb[:, 0] - 1j * ky * fb[:, 1], -1j * kx * ft[:, 0] - 1j * ky * ft[:, 1],
                        fb[:, 0], fb[:, 1], fb[:, 2], ft[:, 0], ft[:, 1], ft[:, 2]], axis=1)
        x = np.linalg.solve(A, rhs[:, :, None])[:, :, 0]
        enkz = np.exp(-k[:, None] * z[None, :])
        ekzmh = enkh[:, None] / enkz
        zekzmh = z[None, :] * ekzmh
        zenkz = z[None, :] * enkz
        X = [x[:, i:i + 1] for i in range(8)]
        kk = k[:, None]
        Cu = -1j * X[0] * kx[:, None] * zenkz * fac / kk + 1j * X[1] * kx[:, None] * zekzmh * fac / kk \
            + X[2] * enkz + X[3] * ekzmh
        Cv = -1j * X[0] * ky[:, None] * zenkz * fac / kk + 1j * X[1] * ky[:, None] * zekzmh * fac / kk \
            + X[4] * enkz + X[5] * ekzmh
        Cw = X[0] * zenkz * fac + X[1] * zekzmh * fac + X[6] * enkz + X[7] * ekzmh
        corr = self.cheb_of_samples(np.stack([Cu, Cv, Cw], axis=1))
        U[1:] += corr.transpose(0, 2, 1)

    def correct_k0(self, U, fhat0, slit):
        """k=0 velocity correction, Solvers.py:482-516 (bottom) and 563-599
        (slit; the reference builds both parts from the real part there, which
        changes only the discarded imaginary part, so the full value is used)."""
        Nz, H, eta = self.Nz, self.H, self.eta
        Cf, Cg = fhat0[:, 0], fhat0[:, 1]
        u_rhs = -Cf / eta
        v_rhs = -Cg / eta
        if slit:
            BC = np.stack((self.BCR2, self.BCL2), axis=0)
        else:
            BC = np.stack((self.BCR1, self.BCL2), axis=0)
        C = BC[:, :Nz]
        D = -BC[:, Nz:]
        Gi = 1.0 / (D[0, 0] * D[1, 1] - D[0, 1] * D[1, 0]) * \
            np.array([[D[1, 1], -D[0, 1]], [-D[1, 0], D[0, 0]]])
        au = np.concatenate((u_rhs, Gi @ (C @ u_rhs)))
        av = np.concatenate((v_rhs, Gi @ (C @ v_rhs)))
        U[0, :, 0] += self.SIMat @ au
        U[0, :, 1] += self.SIMat @ av


def cheb_coeff_diff(fh, H):
    """Chebyshev coefficients of d/dz of fh [..., Nz] (z last): the downward
    recurrence of chebCoeffDiff_perm
    (Chebyshev.py:68-94) for z in [a, a + 2H]."""
    Nz = fh.shape[-1]
    Df = np.zeros_like(fh)
    Df[..., Nz - 2] = 2 / H * (Nz - 1) * fh[..., Nz - 1]
    for j in range(2, Nz):
        Df[..., Nz - j - 1] = Df[..., Nz - j + 1] + 2 / H * (Nz - j) * fh[..., Nz - j]
    Df[..., 0] /= 2
    return Df


def spectral_curl(C, Dx, Dy, dz):
    """(Dy Cz - dz(Cy), dz(Cx) - Dx Cz, Dx Cy - Dy Cx) of the coefficient
    field C [..., 3] (FCM.py:372-396, Solvers.py:139-177); dz is the z
    derivative operator on one component."""
    Cx, Cy, Cz = C[..., 0], C[..., 1], C[..., 2]
    return np.stack([Dy * Cz - dz(Cy), -Dx * Cz + dz(Cx), Dx * Cy - Dy * Cx], axis=-1)


# --------------------------------------------------------------------------
# Triply periodic solver (Solvers.py:197-258, TPTools.cpp:6-46)
# --------------------------------------------------------------------------
def tp_wavenumbers(n, L):
    """2 pi [0, 1, ..., floor(n/2), -ceil(n/2)+1, ..., -1] / L (Solvers.py:202-209)."""
    return 2 * np.pi * np.concatenate((np.arange(0, np.floor(n / 2) + 1),
                                       np.arange(-1 * np.ceil(n / 2) + 1, 0))) / L


def tp_derivatives(Ny, Nx, Nz, Lx, Ly, Lz):
    """Ksq, Dx, Dy, Dz on [Ny, Nx, Nz] (Solvers.py:197-222)."""
    Ky, Kx, Kz = np.meshgrid(tp_wavenumbers(Ny, Ly), tp_wavenumbers(Nx, Lx),
                             tp_wavenumbers(Nz, Lz), indexing='ij')
    Ksq = Kx ** 2 + Ky ** 2 + Kz ** 2
    Dx, Dy, Dz = 1j * Kx, 1j * Ky, 1j * Kz
    if Nx % 2 == 0:
        Dx[:, Nx // 2, :] = 0
    if Ny % 2 == 0:
        Dy[Ny // 2, :, :] = 0
    if Nz % 2 == 0:
        Dz[:, :, Nz // 2] = 0
    return Ksq, Dx, Dy, Dz


def tp_solve(fhat, Lx, Ly, Lz, eta):
    """fhat [Ny,Nx,Nz,3] (unnormalised 3-D DFT) -> velocity coefficients:
    p = -(Dx f + Dy g + Dz h) / |k|^2, u = (f - Dx p) / (eta |k|^2) per mode,
    D = i k with the unpaired (Nyquist) plane of an even axis zeroed in D but
    not in |k|^2, and the k = 0 mode left at zero."""
    Ny, Nx, Nz, _ = fhat.shape
    Ksq, Dx, Dy, Dz = tp_derivatives(Ny, Nx, Nz, Lx, Ly, Lz)
    Ksq0 = Ksq.copy()
    Ksq0[0, 0, 0] = 1.0
    f, g, h = fhat[..., 0], fhat[..., 1], fhat[..., 2]
    ph = -(Dx * f + Dy * g + Dz * h) / Ksq0
    val = 1.0 / (eta * Ksq0)
    U = np.empty_like(fhat)
    U[..., 0] = val * (f - Dx * ph)
    U[..., 1] = val * (g - Dy * ph)
    U[..., 2] = val * (h - Dz * ph)
    U[0, 0, 0] = 0
    return U


# --------------------------------------------------------------------------
# The operator
# --------------------------------------------------------------------------
class Oracle:
    """FCM.Initialize / SetPositions / Mdot (FCM.py:149-441), derivative-kernel
    torque coupling (the reference default, useRegKernel=False)."""

    def __init__(self, p: Params):
        self.p = p
        self.BCs, self.BCst = domain_bcs(p.domType)
        self.tp = p.domType == 'TP'
        self.km = Kernel(p.wm, p.betam_hat, p.alpha(p.wm), dipole=False)
        self.kd = Kernel(p.wd, p.betad_hat, p.alpha(p.wd), dipole=not p.reg_kernel) if p.has_torque else None
        if self.tp:
            self.zpts = self.zwts = None
            self.solver = None
        else:
            self.zpts, self.zwts = clencurt(p.Nz, 0, p.Lz)
            self.solver = DPSolver(p.Nx, p.Ny, p.Nz, p.Lx, p.Ly, p.Lz / 2, p.eta)

    def _grid(self, kern):
        p = self.p
        if self.tp:
            return GridStateTP(p, cround(2 * kern.thr / p.hx), cround(2 * kern.thr / p.hz))
        return GridState(p, self.zpts, self.zwts, kern.thr, cround(2 * kern.thr / p.hx))

    def _locate(self, g, kern, X):
        return (locate_tp if self.tp else locate)(self.p, g, kern, X)

    def set_positions(self, X):
        p = self.p
        X = np.array(X, dtype=np.float64).reshape(-1, 3).copy()
        X[:, 2] -= p.z0
        self.X = X
        self.g = self._grid(self.km)
        self.loc = self._locate(self.g, self.km, X)
        if p.has_torque:
            self.tg = self._grid(self.kd)
            self.tloc = self._locate(self.tg, self.kd, X)

    def spread_all(self, F, T=None):
        """Spread grid incl. the torque curl (FCM.py:353-371)."""
        F = np.asarray(F, dtype=np.float64).reshape(-1, 3)
        spread(self.g, self.km, self.loc, F)
        fG = fold(self.g, self.BCs)
        if self.p.has_torque:
            T = np.asarray(T, dtype=np.float64).reshape(-1, 3)
            spread(self.tg, self.kd, self.tloc, T, deriv=0)
            dx = fold(self.tg, self.BCs)
            fG[..., 1] -= 0.5 * dx[..., 2]  # addDx, SpreadInterpWrapper.cpp:66-79
            fG[..., 2] += 0.5 * dx[..., 1]
            spread(self.tg, self.kd, self.tloc, T, deriv=1)
            dy = fold(self.tg, self.BCs)
            fG[..., 0] += 0.5 * dy[..., 2]  # addDy :80-93
            fG[..., 2] -= 0.5 * dy[..., 0]
            spread(self.tg, self.kd, self.tloc, T, deriv=2)
            dz = fold(self.tg, self.BCst)
            fG[..., 0] -= 0.5 * dz[..., 1]  # addDz :94-107
            fG[..., 1] += 0.5 * dz[..., 0]
        return fG

    def solve(self, fhat):
        """Solvers.py:99-131 for DP / DPBW / DPSC; fhat [Ny,Nx,Nz,3]."""
        p, s = self.p, self.solver
        if self.tp:
            return tp_solve(fhat, p.Lx, p.Ly, p.Lz, p.eta)
        fk = fhat.reshape(p.Nx * p.Ny, p.Nz, 3)
        U = s.solve_no_wall(fk)
        if p.domType == 'DPBW':
            s.correct_bottom(U, self.zpts)
            s.correct_k0(U, fk[0], slit=False)
        elif p.domType == 'DPSC':
            s.correct_slit(U, self.zpts, p.Lz)
            s.correct_k0(U, fk[0], slit=True)
        return U.reshape(p.Ny, p.Nx, p.Nz, 3)

    def _mdot_reg(self, F, T, stages):
        """useRegKernel torque coupling (FCM.py:372-396, 427-439): the torques
        spread with the regular kernel, 1/2 curl of their transform added to the
        forces' (Fourier derivatives in x, y; Chebyshev coefficient recurrence
        or Fourier derivative in z), the solve, the vorticity 1/2 curl u of the
        solution's coefficients (Solvers.py:134-177), both transformed back and
        interpolated (V with the monopole kernel, Omega with the regular dipole
        kernel on the torque grid, whose open-end ghost layers still hold the
        torque spread)."""
        p = self.p
        F = np.asarray(F, dtype=np.float64).reshape(-1, 3)
        T = np.zeros_like(F) if T is None else np.asarray(T, dtype=np.float64).reshape(-1, 3)
        spread(self.g, self.km, self.loc, F)
        fG = fold(self.g, self.BCs)
        spread(self.tg, self.kd, self.tloc, T)
        tG = fold(self.tg, self.BCs)
        if self.tp:
            _, Dx, Dy, Dz = tp_derivatives(p.Ny, p.Nx, p.Nz, p.Lx, p.Ly, p.Lz)
            fhat = np.fft.fftn(fG, axes=(0, 1, 2))
            that = np.fft.fftn(tG, axes=(0, 1, 2))
            dz = lambda C: Dz * C  # noqa: E731
        else:
            Dx = self.solver.Dx.reshape(p.Ny, p.Nx)[:, :, None]
            Dy = self.solver.Dy.reshape(p.Ny, p.Nx)[:, :, None]
            fhat = fc_forward(fG)
            that = fc_forward(tG)
            dz = lambda C: cheb_coeff_diff(C, p.Lz / 2)  # noqa: E731
        U = self.solve(fhat + 0.5 * spectral_curl(that, Dx, Dy, dz))
        Ut = 0.5 * spectral_curl(U, Dx, Dy, dz)
        if self.tp:
            uG = np.ascontiguousarray(np.fft.ifftn(U, axes=(0, 1, 2)).real)
            utG = np.ascontiguousarray(np.fft.ifftn(Ut, axes=(0, 1, 2)).real)
        else:
            uG = fc_backward(U)
            utG = fc_backward(Ut)
        if stages is not None:
            stages.update(spread_grid=fG, torque_grid=tG, u_hat=U, u_grid=uG, vort_grid=utG)
        ghost_copy(self.g, uG, self.BCs)
        V = interpolate(self.g, self.km, self.loc)
        ghost_copy(self.tg, utG, self.BCs)
        W = interpolate(self.tg, self.kd, self.tloc)
        return V.ravel(), W.ravel()

    def mdot(self, F, T=None, stages=None):
        p = self.p
        if p.has_torque and p.reg_kernel:
            return self._mdot_reg(F, T, stages)
        fG = self.spread_all(F, T)
        if self.tp:  # Transform type fourier (Transform.cpp:109-117, 273-281)
            fhat = np.fft.fftn(fG, axes=(0, 1, 2))
            U = self.solve(fhat)
            uG = np.ascontiguousarray(np.fft.ifftn(U, axes=(0, 1, 2)).real)
        else:
            fhat = fc_forward(fG)
            U = self.solve(fhat)
            uG = fc_backward(U)
        if stages is not None:
            stages.update(spread_grid=fG, f_hat=fhat, u_hat=U, u_grid=uG)
        ghost_copy(self.g, uG, self.BCs)
        V = interpolate(self.g, self.km, self.loc)
        if not p.has_torque:
            return V.ravel(), None
        ghost_copy(self.tg, uG, self.BCs)
        dxv = interpolate(self.tg, self.kd, self.tloc, deriv=0)
        dyv = interpolate(self.tg, self.kd, self.tloc, deriv=1)
        ghost_copy(self.tg, uG, self.BCst)
        dzv = interpolate(self.tg, self.kd, self.tloc, deriv=2)
        W = np.empty_like(V)
        W[:, 0] = -1 / 2 * (dyv[:, 2] - dzv[:, 1])  # FCM.py:424-426
        W[:, 1] = -1 / 2 * (dzv[:, 0] - dxv[:, 2])
        W[:, 2] = -1 / 2 * (dxv[:, 1] - dyv[:, 0])
        return V.ravel(), W.ravel()


def mdot(p: Params, X, F, T=None, stages=None):
    o = Oracle(p)
    o.set_positions(X)
    return o.mdot(F, T, stages=stages)
