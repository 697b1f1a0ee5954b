"""Grid and kernel configuration from the hydrodynamic radius, as the
reference chooses it (source/cpu/python/GridAndKernelConfig.py): the x-y grid
spacing, grid sizes and ES kernel (w, beta) per kernel type, and the z extent,
Chebyshev size and floor per domain type.  FCMJoint.Initialize uses these
when no explicit grid is given, like the reference's GPU branch
(python_interface/common_interface_wrapper.py:78-101).

The choice rests on polynomial fits of the dimensionless radius
c(beta w) = R_h / (w h) of the ES kernels and of its inverse (the tables
below, GridAndKernelConfig.py:472-524); they are kept identical to the
reference's so that the same (h, beta, N) come out.  The reference's sampled
%-error curves only feed its printed diagnostics and are not needed here: the
selection itself depends on them only through the beta*w range check.
"""
import math

import numpy as np

# c(beta w) = R_h / (w h) and its inverse, monopole and dipole kernels,
# highest power first (numpy.poly1d order).
_CBETA_M = np.array([1.377360225705533e-14, -2.780166372816629e-12, 2.448353284693753e-10,
                     -1.237430413656322e-08, 3.979148502148348e-07, -8.561766184042201e-06,
                     0.0001272679847510219, -0.001354403465648405, 0.01097749452611932,
                     -0.07481288697153615, 0.5542048130466118])
_CBETA_D = np.array([-4.547131634839802e-15, 9.269149081395723e-13, -8.100791156357088e-11,
                     3.923458768903104e-09, -1.120891440829999e-07, 1.758862781905333e-06,
                     -6.91617984068661e-06, -0.0002952983095968742, 0.006854380595771486,
                     -0.07755569487992697, 0.6862730778816093])
_CBETA_M_INV = np.array([4131643418.193291, -10471683395.26777, 11833009228.6429, -7851132955.882548,
                         3388121732.651829, -994285251.2185925, 201183449.7086889, -27776767.88241613,
                         2515647.646492857, -136305.2970161326, 3445.959503226691])
_CBETA_D_INV = np.array([39129605.95992675, -141095001.9380851, 226461386.9399433, -213225975.7007014,
                         130589579.4920038, -54470021.75408537, 15723274.21737542, -3119398.842468358,
                         411336.473729197, -33239.91568304499, 1311.988715157221])

# kernel types (GridAndKernelConfig.py:54-66, 192-216): (w_m, beta_m / w_m, h_opt ratio) without
# torques; (w_m, w_d, beta_m / w_m, beta_d / w_d, h_opt ratio) with torques
_KERN_F = {0: (6, 1.714, 1.5539), 1: (5, 1.886, 1.3437), 2: (4, 1.785, 1.2047)}
_KERN_FT = {0: (6, 6, 1.3267, 2.2160, 1.7305), 1: (5, 5, 1.3055, 2.2320, 1.5598),
            3: (6, 5, 1.3261, 1.7584, 1.7309), 4: (6, 4, 1.5728, 1.5115, 1.6121),
            5: (5, 4, 1.3536, 1.7147, 1.5382)}
_BW_MIN, _BW_MAX = 4.0, 18.0  # beta*w range of the fits


def _valid(n):
    """True when n has no prime factors other than 2, 3, 5, 7 (:430-439)."""
    n = int(n)
    if n < 1:
        return False
    for p in (2, 3, 5, 7):
        while n % p == 0:
            n //= p
    return n == 1


def _nearest_friendly(n):
    """The FFT-friendly size nearest to n, looking up before down at each
    distance (:441-447); 0 when none is found."""
    for i in range(n):
        if _valid(n + i):
            return n + i
        if _valid(n - i):
            return n - i
    return 0


def fft_friendly_sizes(n, sep, count):
    """Up to count distinct nearest-friendly sizes of n, n+1, ..., n+sep-1
    (:449-459)."""
    out = []
    for i in range(n, n + sep):
        m = _nearest_friendly(i)
        if m not in out:
            if len(out) == count:
                break
            out.append(m)
    return np.array(out, dtype=np.int64)


def configure_grid_and_kernels_xy(Lx, Ly, radii, kern_types, opt_ind, has_torque=False, ref=False):
    """(Lx, Ly, hx, hy, Nx, Ny, wm, wd, cbeta_m, cbeta_d, beta_m, beta_d) as the
    reference returns them (GridAndKernelConfig.py:4-361): beta_* are per
    particle and dimensionless (beta / w); opt_ind = -1 selects the optimal
    grid with the extent adjusted to it, opt_ind >= 0 the corresponding
    FFT-friendly candidate for the given extent.  Raises ValueError for
    unsupported kernel types and out-of-range (h, beta)."""
    radii = np.asarray(radii, dtype=np.float64).ravel()
    kern_types = np.asarray(kern_types).ravel()
    nP = radii.size
    rmin = np.min(radii)
    poly_m, poly_d = np.poly1d(_CBETA_M), np.poly1d(_CBETA_D)
    inv_m, inv_d = np.poly1d(_CBETA_M_INV), np.poly1d(_CBETA_D_INV)
    wm = np.zeros(nP, dtype=np.ushort)
    beta_m = np.zeros(nP)
    h = np.zeros(nP)
    if not has_torque:
        for i in range(nP):
            if int(kern_types[i]) not in _KERN_F:
                raise ValueError("translation-only kernel type not supported")
            w, b, ratio = _KERN_F[int(kern_types[i])]
            wm[i], beta_m[i] = w, b
            hopt = rmin / ratio
            h[i] = radii[i] / (wm[i] * poly_m(beta_m[i] * wm[i]))
        wd = None
    else:
        wd = np.zeros(nP, dtype=np.ushort)
        beta_d = np.zeros(nP)
        for i in range(nP):
            if int(kern_types[i]) not in _KERN_FT:
                raise ValueError("translation-rotation kernel type not supported")
            w, w2, b, b2, ratio = _KERN_FT[int(kern_types[i])]
            wm[i], wd[i], beta_m[i], beta_d[i] = w, w2, b, b2
            hopt = rmin / ratio
            h[i] = radii[i] / (wm[i] * poly_m(beta_m[i] * wm[i]))
    h = np.min(h)
    # candidate sizes: the nearest FFT-friendly sizes from floor(Lx / h) up
    Nx = fft_friendly_sizes(int(np.floor(Lx / h)), 20 if has_torque else 100, 10)
    hx_c = Lx / Nx

    def in_range(bw):
        return _BW_MIN <= bw <= _BW_MAX

    # beta at the optimal spacing (must be in range) and at every candidate
    bm_opt = np.zeros(nP)
    bm_test = np.zeros((nP, len(Nx)))
    ok_test = np.ones(len(Nx), dtype=bool)
    if has_torque:
        bd_opt = np.zeros(nP)
        bd_test = np.zeros((nP, len(Nx)))
    for i in range(nP):
        bm_opt[i] = inv_m(radii[i] / (wm[i] * hopt)) / wm[i]
        bad = not in_range(bm_opt[i] * wm[i])
        if has_torque:
            bd_opt[i] = inv_d(radii[i] / (wd[i] * hopt)) / wd[i]
            bad = bad or not in_range(bd_opt[i] * wd[i])
        if bad:
            raise ValueError("Could not find optimal (h,beta) in range for particle #%d" % i)
        for j in range(len(hx_c)):
            bm_test[i, j] = inv_m(radii[i] / (wm[i] * hx_c[j])) / wm[i]
            good = in_range(bm_test[i, j] * wm[i])
            if has_torque:
                bd_test[i, j] = inv_d(radii[i] / (wd[i] * hx_c[j])) / wd[i]
                good = good and in_range(bd_test[i, j] * wd[i])
            ok_test[j] = ok_test[j] and good
    Nx_opt = int(np.round(Lx / hopt))
    Ny_opt = int(np.round(Ly / hopt))
    if opt_ind >= 0:
        if not ok_test[opt_ind]:
            raise ValueError("Out of range interpolation")
        beta_m = bm_test[:, opt_ind].copy()
        if has_torque:
            beta_d = bd_test[:, opt_ind].copy()
        Nx = Nx[opt_ind]
        hx = hy = hx_c[opt_ind]
        Ny = Ly / hy
        if np.round(Ny) != Ny:
            Ny = int(np.ceil(Ny))
            Ly = hy * Ny
    else:
        beta_m = bm_opt
        if has_torque:
            beta_d = bd_opt
        Lx, Ly = hopt * Nx_opt, hopt * Ny_opt
        Nx, Ny = Nx_opt, Ny_opt
        hx = hy = hopt
    cbeta_m = radii / (wm * hx)
    if has_torque:
        cbeta_d = radii / (wd * hx)
    else:
        cbeta_d, wd, beta_d = 0, [0], [0]
    if ref:
        hx, hy, Nx, Ny = hx / 2, hy / 2, Nx * 2, Ny * 2
    return Lx, Ly, hx, hy, int(Nx), int(Ny), wm, wd, cbeta_m, cbeta_d, beta_m, beta_d


def configure_grid_and_kernels_z(minZ, maxZ, h, wm, wd, domType, fac=1.5, ref=False):
    """(Lz, hz, Nz, a) as the reference returns them (:363-428): the z extent
    [a, a + Lz] with open-end margins fac * max(w_m) h / 2 (DP both ends, DPBW
    the top, none for DPSC / TP), and for the Chebyshev domains the smallest
    Nz resolving h at the ends with 2 (Nz - 1) FFT friendly."""
    if domType not in ("TP", "DP", "DPBW", "DPSC"):
        raise ValueError("domType is not supported")
    hz = h * (domType == "TP")
    half = fac * float(np.max(wm)) * h / 2
    down, up = {"TP": (0, 0), "DPSC": (0, 0), "DPBW": (0, half), "DP": (half, half)}[domType]
    if ref:
        down, up = down * 2.0, up * 2.0
    a = minZ - down
    Lz = (maxZ + up) - a
    if domType == "TP":
        Nz = Lz / hz
        if np.round(Nz) != Nz:
            Nz = int(np.ceil(Nz))
            Lz = hz * Nz
        return Lz, hz, int(Nz), a
    H = Lz / 2
    nz0 = int(np.ceil(math.pi / (np.arccos(-h / H) - math.pi / 2)))
    Nz = int(fft_friendly_sizes(nz0, 100, 1)[0]) + 1
    return Lz, hz, Nz, a
