"""Benchmark and parity workloads: explicit grid/kernel parameters and seeded
synthetic particle inputs for the five configurations the operator is
measured on, plus helpers for small parity cases.

All inputs are synthetic (no dataset exists for this operator): positions
uniform in the periodic box and in a z band, forces/torques i.i.d. standard
normal, drawn from numpy's PCG64 generator with a fixed seed in a fixed order
(x, y, z, then forces, then torques), so every machine regenerates the same
arrays.
"""
import math
from dataclasses import dataclass, asdict, replace

import numpy as np

ETA_DEFAULT = 1.0 / (6.0 * math.pi)


@dataclass(frozen=True)
class Workload:
    """One Mdot configuration.

    domType: 'DP' (open), 'DPBW' (bottom wall at z0), 'DPSC' (walls at z0 and z0+Lz),
    'TP' (triply periodic: nz uniform points on the periodic [z0, z0+Lz)).
    The Chebyshev interval is [z0, z0+Lz]; particle heights are drawn from
    [zlo, zhi].  beta = beta_hat * w for each kernel; alpha = w*h/2 (the
    reference's UseCbeta convention with c(beta) = R/(w h))."""
    name: str
    domType: str
    N: int
    Lx: float
    Ly: float
    nx: int
    ny: int
    nz: int
    z0: float
    Lz: float
    zlo: float
    zhi: float
    has_torque: bool
    wm: int = 6
    betam_hat: float = 1.714
    wd: int = 6
    betad_hat: float = 2.2160
    eta: float = ETA_DEFAULT
    radius: float = 1.0
    seed: int = 0
    reg_kernel: bool = False  # torques with the regular kernel and spectral curls (useRegKernel)
    layout: str = "uniform"   # particle positions: 'uniform' or 'edge' (edge_positions)

    def oracle_params(self):
        """Keyword arguments of the oracle's Params (same field meanings)."""
        return dict(domType=self.domType, Nx=self.nx, Ny=self.ny, Nz=self.nz, Lx=self.Lx,
                    Ly=self.Ly, Lz=self.Lz, z0=self.z0, eta=self.eta, wm=self.wm,
                    betam_hat=self.betam_hat, has_torque=self.has_torque, wd=self.wd,
                    betad_hat=self.betad_hat, radius=self.radius, reg_kernel=self.reg_kernel)

    def to_dict(self):
        return asdict(self)


def edge_positions(w: Workload, rng):
    """w.N positions at the edges of the unit cell and the grid: the cell's
    corner and z ends exactly (walls, open ends, the periodic seam), grid
    nodes exactly (x, y nodes; z Chebyshev nodes or uniform nodes),
    half-cell points (the rounding tie of odd-width stencils), two
    particles at one position, one just inside each z end; the rest uniform.
    x and y stay below Lx, Ly, and z below the top of a triply periodic
    box (at x = Lx, y = Ly or, uniform z with an even stencil, z = zmax the
    reference indexes past its extended grid; the wrapped seam is covered by
    the points at 0)."""
    hx, hy = w.Lx / w.nx, w.Ly / w.ny
    a, b = w.z0, w.z0 + w.Lz
    if w.domType == "TP":
        zn = w.z0 + np.arange(w.nz) * (w.Lz / w.nz)
    else:  # Chebyshev nodes on [z0, z0 + Lz] (Chebyshev.py:4-38)
        zn = w.z0 + w.Lz / 2 * np.cos(np.pi * np.arange(w.nz) / (w.nz - 1)) + w.Lz / 2
    top = b - 0.25 * (w.Lz / w.nz) if w.domType == "TP" else b
    pts = [(0.0, 0.0, a), (0.5 * hx, w.Ly - 0.25 * hy, top), (w.Lx / 2, w.Ly / 2, zn[2]),
           (w.Lx / 2, w.Ly / 2, zn[2]), (3 * hx, 5 * hy, zn[len(zn) // 2]), (2.5 * hx, 7.5 * hy, a + 0.3),
           (w.Lx - 0.5 * hx, 4 * hy, b - 0.3), (7 * hx, 0.0, zn[-3]), (0.0, 9.5 * hy, (a + b) / 2)]
    X = np.array(pts[:w.N], dtype=np.float64)
    n = w.N - X.shape[0]
    if n > 0:
        R = np.stack([rng.uniform(0.0, w.Lx, n), rng.uniform(0.0, w.Ly, n), rng.uniform(a, b, n)], axis=1)
        X = np.concatenate([X, R])
    return X


def make_inputs(w: Workload, dtype=np.float64):
    """Seeded synthetic positions [N,3], forces [N,3], torques [N,3] (or None)."""
    rng = np.random.default_rng(w.seed)
    if w.layout == "edge":
        X = edge_positions(w, rng)
    else:
        x = rng.uniform(0.0, w.Lx, w.N)
        y = rng.uniform(0.0, w.Ly, w.N)
        z = rng.uniform(w.zlo, w.zhi, w.N)
        X = np.stack([x, y, z], axis=1)
    F = rng.standard_normal((w.N, 3))
    T = rng.standard_normal((w.N, 3)) if w.has_torque else None
    if dtype != np.float64:
        F = F.astype(dtype)
        T = T.astype(dtype) if T is not None else None
    return X, F, T


# The five measured configurations (w = 6 everywhere; with torques the
# reference's w=6 monopole/dipole pair beta_m = 1.3267*6, beta_d = 2.2160*6).
C0 = Workload("c0_dpbw_n2048", "DPBW", 2048, 128.0, 128.0, 128, 128, 64, 0.0, 20.0, 1.5, 18.5,
              False, betam_hat=1.714)
C1 = Workload("c1_dpsc_n16384", "DPSC", 16384, 256.0, 256.0, 256, 256, 96, 0.0, 32.0, 1.5, 30.5,
              True, betam_hat=1.3267, betad_hat=2.2160)
C2 = Workload("c2_dp_n65536", "DP", 65536, 512.0, 512.0, 512, 512, 128, -20.5, 41.0, -16.0, 16.0,
              True, betam_hat=1.3267, betad_hat=2.2160)
C3 = Workload("c3_dpbw_n8192", "DPBW", 8192, 192.0, 192.0, 192, 192, 64, 0.0, 24.0, 1.5, 22.5,
              False, betam_hat=1.714)
# Triply periodic configurations (the reference's domType 'TP'): the c0 box
# and density on a 128 x 128 x 32 grid (reference fixture size), and the c2
# particle count, kernels and torques in a 512 x 512 x 64 periodic box (h = 1).
T0 = Workload("t0_tp_n2048", "TP", 2048, 128.0, 128.0, 128, 128, 32, 0.0, 32.0, 0.0, 32.0,
              False, betam_hat=1.714)
T1 = Workload("t1_tp_n65536", "TP", 65536, 512.0, 512.0, 512, 512, 64, 0.0, 64.0, 0.0, 64.0,
              True, betam_hat=1.3267, betad_hat=2.2160)
# Four times c2 (the same density and z geometry on a 1024 x 1024 x 128 grid,
# N = 262,144): a scale check of the index arithmetic and the solve's
# scheduling past the headline size (about 20 GB on the device with both
# operators).
L1 = Workload("l1_dp_n262144_1024", "DP", 262144, 1024.0, 1024.0, 1024, 1024, 128, -20.5, 41.0, -16.0, 16.0,
              True, betam_hat=1.3267, betad_hat=2.2160)
CONFIGS = {w.name: w for w in (C0, C1, C2, C3, T0, T1, L1)}


def scaled(w: Workload, n: int) -> Workload:
    """w with the same z geometry, grid spacing and particle density on an
    n x n grid (box side n h, N scaled by the area), named
    '<w.name>@<n>'; e.g. scaled(C2, 384) is the open 384 x 384 x 128 box with
    36,864 particles."""
    h = w.Lx / w.nx
    N = int(round(w.N * (n * n) / (w.nx * w.ny)))
    return replace(w, name="%s@%d" % (w.name, n), N=N, Lx=n * h, Ly=n * h, nx=n, ny=n)


def by_name(name: str) -> Workload:
    """A named configuration, or '<name>@<n>' for scaled(CONFIGS[name], n)."""
    if "@" in name:
        base, n = name.split("@", 1)
        return scaled(CONFIGS[base], int(n))
    return CONFIGS[name]


def fft_friendly(n):
    """Smallest integer >= n whose prime factors are all in {2,3,5,7}."""
    m = int(n)
    while True:
        k = m
        for p in (2, 3, 5, 7):
            while k % p == 0:
                k //= p
        if k == 1:
            return m
        m += 1


def batched_c4(n_systems=256, seed=1000):
    """The batched bottom-wall set: N_i log-uniform in [64, 4096], box side
    L_i ~ U[32, 128], n_i = fft_friendly(round(1.55 L_i)), h_i = L_i/n_i,
    Lz = 20, nz = 64, inputs drawn as for c0 with seed 1000+i."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_systems):
        N = int(round(math.exp(rng.uniform(math.log(64), math.log(4096)))))
        L = float(rng.uniform(32.0, 128.0))
        n = fft_friendly(int(round(1.55 * L)))
        out.append(Workload("c4_sys%03d" % i, "DPBW", N, L, L, n, n, 64, 0.0, 20.0, 1.5, 18.5,
                            False, betam_hat=1.714, seed=seed + i))
    return out


def small(name, domType, N, n, nz, Lz, zlo, zhi, has_torque, ny=None, Ly=None, z0=0.0, seed=0):
    """A small parity case with h = 1 (Lx = nx)."""
    ny = n if ny is None else ny
    Ly = float(ny) if Ly is None else Ly
    return Workload(name, domType, N, float(n), Ly, n, ny, nz, z0, Lz, zlo, zhi, has_torque,
                    betam_hat=1.3267 if has_torque else 1.714, seed=seed)


# Small parity cases: every geometry with and without torques, particles whose
# kernels reach open ends (the reference reuses spread data in the ghost
# layers there), odd and unequal grid sizes (Nyquist handling), a shifted z
# origin.
SMALL = [
    small("s_dpbw_t", "DPBW", 24, 16, 17, 10.0, 1.5, 8.5, True),
    small("s_dp_t", "DP", 24, 16, 19, 12.4, 3.0, 9.4, True, z0=0.0),
    small("s_dpsc_t", "DPSC", 24, 16, 21, 10.0, 1.0, 9.0, True),
    small("s_dpbw_f_top", "DPBW", 20, 20, 24, 12.0, 1.0, 11.5, False, seed=3),
    small("s_dp_f_ends", "DP", 18, 18, 16, 14.0, 0.5, 13.5, False, seed=4),
    small("s_dp_t_shift", "DP", 16, 16, 25, 10.0, -4.0, 4.0, True, z0=-5.0, seed=5),
    small("s_dpbw_t_odd", "DPBW", 20, 15, 22, 11.0, 0.8, 10.5, True, ny=18, Ly=18.0, seed=6),
    small("s_dpsc_f_odd", "DPSC", 20, 17, 20, 9.0, 0.3, 8.7, False, ny=14, Ly=14.0, seed=7),
]
# Small triply periodic cases: torques, odd and unequal grid sizes, a z
# spacing different from the x-y spacing (wider z stencil), odd-width kernels.
SMALL_TP = [
    small("s_tp_t", "TP", 24, 16, 16, 16.0, 0.0, 16.0, True, seed=8),
    small("s_tp_f_odd", "TP", 20, 15, 13, 13.0, 0.0, 13.0, False, ny=18, Ly=18.0, seed=9),
    small("s_tp_t_hz", "TP", 24, 16, 20, 16.0, 0.0, 16.0, True, seed=10),
    replace(small("s_tp_t_w5", "TP", 20, 17, 15, 15.0, 0.0, 15.0, True, seed=11),
            wm=5, wd=5, betam_hat=1.3055, betad_hat=2.2320),
]
# The regular-kernel torque coupling (useRegKernel) on torque cases of every
# geometry, including open ends reached by the kernels, an odd grid and a
# shifted z origin.
SMALL_REG = [replace(w, name=w.name.replace("s_", "s_reg_", 1), reg_kernel=True) for w in SMALL + SMALL_TP
             if w.name in ("s_dpbw_t", "s_dp_t", "s_dpsc_t", "s_dpbw_t_odd", "s_dp_t_shift", "s_tp_t", "s_tp_t_hz")]
# Edge positions (edge_positions) in every geometry, with torques, an odd
# kernel width and the regular-kernel coupling among them.
SMALL_EDGE = [
    replace(small("e_dpbw_t", "DPBW", 16, 16, 17, 10.0, 0.0, 10.0, True, seed=12), layout="edge"),
    replace(small("e_dpsc_t", "DPSC", 16, 16, 21, 10.0, 0.0, 10.0, True, seed=13), layout="edge"),
    replace(small("e_dp_f", "DP", 14, 16, 19, 12.4, 0.0, 12.4, False, seed=14), layout="edge"),
    replace(small("e_dp_t_shift", "DP", 16, 16, 25, 10.0, -5.0, 5.0, True, z0=-5.0, seed=15), layout="edge"),
    replace(small("e_tp_t", "TP", 16, 16, 16, 16.0, 0.0, 16.0, True, seed=16), layout="edge"),
    replace(small("e_tp_t_w5", "TP", 16, 17, 15, 15.0, 0.0, 15.0, True, seed=17), layout="edge",
            wm=5, wd=5, betam_hat=1.3055, betad_hat=2.2320),
    replace(small("e_dpbw_t_reg", "DPBW", 16, 16, 17, 10.0, 0.0, 10.0, True, seed=18), layout="edge",
            reg_kernel=True),
]
# Unequal monopole / dipole widths (the reference's torque kernel types 3, 4
# and 5: w_m / w_d = 6/5, 6/4, 5/4 with their betas, GridAndKernelConfig.py):
# separate monopole and dipole passes.
SMALL_KT = [
    replace(small("s_dpbw_t_k3", "DPBW", 24, 16, 17, 10.0, 1.5, 8.5, True, seed=19), wm=6, wd=5,
            betam_hat=1.3261, betad_hat=1.7584),
    replace(small("s_dpsc_t_k4", "DPSC", 24, 16, 21, 10.0, 1.0, 9.0, True, seed=20), wm=6, wd=4,
            betam_hat=1.5728, betad_hat=1.5115),
    replace(small("s_tp_t_k5", "TP", 24, 16, 16, 16.0, 0.0, 16.0, True, seed=21), wm=5, wd=4,
            betam_hat=1.3536, betad_hat=1.7147),
]
SMALL_BY_NAME = {w.name: w for w in SMALL + SMALL_TP + SMALL_REG + SMALL_EDGE + SMALL_KT}


def small_batch(domType, has_torque, seed=40):
    """A small batch sharing nz, the z interval and the geometry, with uneven
    boxes (one size class holding two systems, one non-square grid) and
    particle counts; h = 1 in every system."""
    z = {"DPBW": (17, 0.0, 10.0, 1.5, 8.5), "DP": (19, 0.0, 12.4, 3.0, 9.4),
         "DPSC": (20, 0.0, 9.0, 0.3, 8.7)}[domType]
    nz, z0, Lz, zlo, zhi = z
    shapes = [(16, 16, 24), (20, 20, 7), (16, 16, 30), (15, 15, 12), (18, 14, 20)]
    out = []
    for k, (nx, ny, N) in enumerate(shapes):
        out.append(Workload("b_%s_%d" % (domType.lower(), k), domType, N, float(nx), float(ny), nx, ny, nz, z0,
                            Lz, zlo, zhi, has_torque, betam_hat=1.3267 if has_torque else 1.714,
                            seed=seed + k))
    return out
