// Wavenumber-space stages of Mdot:
//   k_zgemm       z transform as a batched GEMM over every (component, mode,
//                 re/im) column: Chebyshev coefficients from node values
//                 (forward) or node values from coefficients (inverse, with
//                 the wall correction added at the nodes and the 1/(nx ny)
//                 normalisation of the x-y inverse FFT folded in);
//   k_bvp_factors per-wavenumber factors of the Schur/KBPENTA solve;
//   k_bvp         per-wavenumber FP64 Stokes BVP + wall-correction
//                 coefficients + the k = 0 mode.
//
// Reference behaviour restated (stochasticHydroTools/DoublyPeriodicStokes):
//   transform normalisation  Transform.cpp:107-304 (DCT-I via even extension)
//   factors                  Solvers.py:258-347, LinearSolvers.cpp:11-60,
//                            LinearSolvers.h:52-103
//   no-wall solve            DPTools.cpp:81-345
//   bottom-wall correction   DPTools.cpp:590-700
//   slit correction          DPTools.cpp:704-877
//   k = 0                    Solvers.py:350-432 (open: zero),
//                            482-516 (bottom), 563-599 (slit)
// The Nyquist rows/columns: the reference solves the full spectrum and keeps
// the real part of the inverse transform, which equals the inverse transform
// of (U(k) + conj(U(-k)))/2.  The no-wall solution is Hermitian, the wall
// correction (built from Kx, Ky, not Dx, Dy) is not on Nyquist lines, so the
// correction of such a mode is averaged with the conjugate of the correction
// the reference computes at its partner index.
#include "dpst_internal.cuh"
#include <cuComplex.h>
#include <type_traits>

namespace dpst {



__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cscale(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
// i*k*a for real k
__device__ __forceinline__ double2 cik(double k, double2 a) { return make_double2(-k * a.y, k * a.x); }

__device__ __forceinline__ bool mode_is_hermitian(const KsArgs &a, int ix, int iy, double kx, double ky,
                                                  double &kxp, double &kyp) {
  int ixp = (a.nx - ix) % a.nx, iyp = (a.ny - iy) % a.ny;
  kxp = a.kvx[ixp];
  kyp = a.kvy[iyp];
  return (kxp == -kx) && (kyp == -ky);
}

// ---------------------------------------------------------------------------
// Per-wavenumber factors.  One thread per mode.
// ---------------------------------------------------------------------------
__global__ void k_bvp_factors(KsArgs a) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= a.nk) return;
  const int nz = a.nz;
  const int64_t nk = a.nk;
  int ix = (int)(i % a.nxh), iy = (int)(i / a.nxh);
  if (i == 0) {
    for (int j = 0; j < nz; ++j) {
      a.mfac[j * nk] = 0; a.invb[j * nk] = 1; a.dp2[j * nk] = 0;
      a.ab0[j * nk] = 0; a.ab1[j * nk] = 0; a.c0[j * nk] = 0; a.c1[j * nk] = 0;
    }
    a.invb[nz * nk] = 1;
    for (int q = 0; q < 4; ++q) a.ginv[q * nk] = 0;
    return;
  }
  const double kx = a.kvx[ix], ky = a.kvy[iy];
  const double K2 = kx * kx + ky * ky;
  const double K = sqrt(K2);
  // beta recursion (LinearSolvers.h:52-74) with d0 = 1 - S_jj K2,
  // dp2 = -S_{j,j+2} K2, dm2 = -S_{j+2,j} K2 (Solvers.py:321).  beta_j
  // (j = 1..nz) is kept in invb while A^{-1}B is formed with the reference's
  // divisions, then replaced by 1/beta_j for the per-Mdot sweeps.
  double *beta = a.invb;
  beta[0 * nk + i] = 0.0;
  beta[1 * nk + i] = 1.0 - a.s0[0] * K2;
  beta[2 * nk + i] = 1.0 - a.s0[1] * K2;
  for (int j = 3; j <= nz; ++j) {
    double d0 = 1.0 - a.s0[j - 1] * K2;
    double dm2 = 0.0 - a.sm2[j - 1] * K2;  // S[j-1][j-3]
    double dp2 = 0.0 - a.sp2[j - 3] * K2;  // S[j-3][j-1]
    beta[j * nk + i] = d0 - dm2 * dp2 / beta[(j - 2) * nk + i];
  }
  for (int j = 0; j < nz; ++j) a.dp2[j * nk + i] = (j < nz - 2) ? (0.0 - a.sp2[j] * K2) : 0.0;
  // A^{-1} B for the two border columns of B = -K2 * S[:, nz:nz+2]
  // (real KBPENTA, LinearSolvers.h:76-103), in place in ab0/ab1.
  for (int col = 0; col < 2; ++col) {
    double *x = col ? a.ab1 : a.ab0;
    for (int j = 0; j < nz; ++j) x[j * nk + i] = 0.0;
    x[col * nk + i] = (col == 0 ? a.se0 : a.se1) * (-K2);
    for (int j = 2; j < nz; ++j) {
      double dm2 = 0.0 - a.sm2[j] * K2;
      x[j * nk + i] = x[j * nk + i] - dm2 * x[(j - 2) * nk + i] / beta[(j - 1) * nk + i];
    }
    x[(nz - 1) * nk + i] /= beta[nz * nk + i];
    x[(nz - 2) * nk + i] /= beta[(nz - 1) * nk + i];
    for (int j = nz - 3; j >= 0; --j)
      x[j * nk + i] = (x[j * nk + i] - a.dp2[j * nk + i] * x[(j + 2) * nk + i]) / beta[(j + 1) * nk + i];
  }
  // multipliers of the forward sweep dm2[j-2]/beta[j-1], then 1/beta
  for (int j = 0; j < nz; ++j)
    a.mfac[j * nk + i] = (j >= 2) ? (0.0 - a.sm2[j] * K2) / beta[(j - 1) * nk + i] : 0.0;
  for (int j = 1; j <= nz; ++j) a.invb[j * nk + i] = 1.0 / beta[j * nk + i];
  a.invb[0 * nk + i] = 0.0;
  // BC rows at this k (Solvers.py:315-331) and G = C A^{-1}B - D, Ginv
  const double H = a.H, h2k = (H * H) * K;
  double G00 = 0, G01 = 0, G10 = 0, G11 = 0;
  for (int j = 0; j < nz; ++j) {
    double r0 = a.bcr2[j] * h2k + (a.bcr2[j] + (H * a.bcr1[j] - a.bcr2[j]));
    double r1 = a.bcl2[j] * h2k + (-a.bcl2[j] + (H * a.bcl1[j] + a.bcl2[j]));
    a.c0[j * nk + i] = r0;
    a.c1[j * nk + i] = r1;
    double x0 = a.ab0[j * nk + i], x1 = a.ab1[j * nk + i];
    G00 += r0 * x0; G01 += r0 * x1; G10 += r1 * x0; G11 += r1 * x1;
  }
  for (int c = 0; c < 2; ++c) {
    int j = nz + c;
    double r0 = a.bcr2[j] * h2k + (a.bcr2[j] + (H * a.bcr1[j] - a.bcr2[j]));
    double r1 = a.bcl2[j] * h2k + (-a.bcl2[j] + (H * a.bcl1[j] + a.bcl2[j]));
    if (c == 0) { G00 -= r0; G10 -= r1; } else { G01 -= r0; G11 -= r1; }
  }
  double det = 1.0 / (G00 * G11 - G01 * G10);
  a.ginv[0 * nk + i] = G11 * det;   // (0,0)
  a.ginv[1 * nk + i] = -G10 * det;  // (1,0)
  a.ginv[2 * nk + i] = -G01 * det;  // (0,1)
  a.ginv[3 * nk + i] = G00 * det;   // (1,1)
}

// ---------------------------------------------------------------------------
// 8x8 complex solve with partial pivoting on |re|+|im| (the LAPACK zgesv
// pivot rule), column-major A.
// ---------------------------------------------------------------------------
__device__ void zsolve8(double2 *A, double2 *x) {
  for (int k = 0; k < 8; ++k) {
    int piv = k;
    double best = -1.0;
    for (int r = k; r < 8; ++r) {
      double v = fabs(A[r + 8 * k].x) + fabs(A[r + 8 * k].y);
      if (v > best) { best = v; piv = r; }
    }
    if (piv != k) {
      for (int c = 0; c < 8; ++c) { double2 t = A[k + 8 * c]; A[k + 8 * c] = A[piv + 8 * c]; A[piv + 8 * c] = t; }
      double2 t = x[k]; x[k] = x[piv]; x[piv] = t;
    }
    double2 p = A[k + 8 * k];
    double den = p.x * p.x + p.y * p.y;
    for (int r = k + 1; r < 8; ++r) {
      double2 ar = A[r + 8 * k];
      double2 l = make_double2((ar.x * p.x + ar.y * p.y) / den, (ar.y * p.x - ar.x * p.y) / den);
      for (int c = k + 1; c < 8; ++c) A[r + 8 * c] = csub(A[r + 8 * c], cmul(l, A[k + 8 * c]));
      x[r] = csub(x[r], cmul(l, x[k]));
    }
  }
  for (int r = 7; r >= 0; --r) {
    double2 s = x[r];
    for (int c = r + 1; c < 8; ++c) s = csub(s, cmul(A[r + 8 * c], x[c]));
    double2 p = A[r + 8 * r];
    double den = p.x * p.x + p.y * p.y;
    x[r] = make_double2((s.x * p.x + s.y * p.y) / den, (s.y * p.x - s.x * p.y) / den);
  }
}

// Slit correction coefficients for wavevector (kx, ky), wall values fb (z=0)
// and ft (z=Hs) (DPTools.cpp:731-788).
__device__ void slit_coeffs(double kx, double ky, double Hs, double eta, const double2 fb[3],
                            const double2 ft[3], double2 c[8]) {
  double2 A[64];
  for (int q = 0; q < 64; ++q) A[q] = make_double2(0, 0);
  const double k = sqrt(kx * kx + ky * ky);
  const double fac = 1.0 / 2.0 / eta;
  const double enkh = exp(-k * Hs);
#define AT(r, cc) A[(r) + 8 * (cc)]
  AT(0, 0) = make_double2(fac, 0);
  AT(0, 1) = make_double2(enkh * fac, 0);
  AT(0, 6) = make_double2(-k, 0);
  AT(0, 7) = make_double2(k * enkh, 0);
  AT(1, 0) = make_double2((1 - k * Hs) * enkh * fac, 0);
  AT(1, 1) = make_double2((1 + k * Hs) * fac, 0);
  AT(1, 6) = make_double2(-k * enkh, 0);
  AT(1, 7) = make_double2(k, 0);
  AT(2, 2) = make_double2(1, 0);
  AT(2, 3) = make_double2(enkh, 0);
  AT(3, 4) = make_double2(1, 0);
  AT(3, 5) = make_double2(enkh, 0);
  AT(4, 6) = make_double2(1, 0);
  AT(4, 7) = make_double2(enkh, 0);
  AT(5, 0) = make_double2(0, -(kx * Hs * enkh * fac / k));
  AT(5, 1) = make_double2(0, kx * Hs * fac / k);
  AT(5, 2) = make_double2(enkh, 0);
  AT(5, 3) = make_double2(1, 0);
  AT(6, 0) = make_double2(0, -(ky * Hs * enkh * fac / k));
  AT(6, 1) = make_double2(0, ky * Hs * fac / k);
  AT(6, 4) = make_double2(enkh, 0);
  AT(6, 5) = make_double2(1, 0);
  AT(7, 0) = make_double2(Hs * enkh * fac, 0);
  AT(7, 1) = make_double2(Hs * fac, 0);
  AT(7, 6) = make_double2(enkh, 0);
  AT(7, 7) = make_double2(1, 0);
#undef AT
  // x0 = -i kx fbx - i ky fby ; x1 likewise for the top
  c[0] = csub(cik(-kx, fb[0]), cik(ky, fb[1]));
  c[1] = csub(cik(-kx, ft[0]), cik(ky, ft[1]));
  c[2] = fb[0]; c[3] = fb[1]; c[4] = fb[2];
  c[5] = ft[0]; c[6] = ft[1]; c[7] = ft[2];
  zsolve8(A, c);
}

// ---------------------------------------------------------------------------
// Per-wavenumber solve.  One thread per mode (persistent grid-stride loop);
// scratch holds three columns of nz+2 complex values per thread, laid out
// [array][j][thread] so that a warp's accesses are coalesced.
// spec: Chebyshev coefficients [3][nz][nk] complex (R), overwritten with the
// velocity coefficients.  corr: per mode 16 complex wall-correction
// coefficients (bottom: -u(0) in [0..2]; slit: c in [0..7], partner c' in
// [8..15]).
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(64) k_bvp(KsArgs a, R *spec, double2 *corr, double2 *scratch,
                                            int64_t nthreads) {
  typedef typename std::conditional<sizeof(R) == 8, double2, float2>::type C2;
  C2 *sp = reinterpret_cast<C2 *>(spec);
  const int nz = a.nz;
  const int64_t nk = a.nk;
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double2 *X = scratch + tid;
  double2 *CP = scratch + (int64_t)(nz + 2) * nthreads + tid;
  double2 *DP = scratch + (int64_t)2 * (nz + 2) * nthreads + tid;
  const int64_t st = nthreads;
  const double inv_eta = 1.0 / a.eta;
  for (int64_t i = tid; i < nk; i += nthreads) {
    auto ld = [&](int d, int j) -> double2 {
      C2 v = sp[((int64_t)d * nz + j) * nk + i];
      return make_double2((double)v.x, (double)v.y);
    };
    auto stv = [&](int d, int j, double2 v) {
      C2 o;
      o.x = (R)v.x;
      o.y = (R)v.y;
      sp[((int64_t)d * nz + j) * nk + i] = o;
    };
    const int ix = (int)(i % a.nxh), iy = (int)(i / a.nxh);
    if (i == 0) {
      // k = 0 mode
      if (a.mode == 0) {
        for (int d = 0; d < 3; ++d)
          for (int j = 0; j < nz; ++j) stv(d, j, make_double2(0, 0));
        continue;
      }
      for (int c = 0; c < 2; ++c) {
        double2 y0 = make_double2(0, 0), y1 = make_double2(0, 0);
        for (int j = 0; j < nz; ++j) {
          double2 r = cscale(-inv_eta, ld(c, j));
          X[j * st] = r;
          y0 = cadd(y0, cscale(a.k0c0[j], r));
          y1 = cadd(y1, cscale(a.k0c1[j], r));
        }
        double2 g0 = cadd(cscale(a.k0gi[0], y0), cscale(a.k0gi[1], y1));
        double2 g1 = cadd(cscale(a.k0gi[2], y0), cscale(a.k0gi[3], y1));
        for (int m = 0; m < nz; ++m) {
          double2 s = cscale(a.s0[m], X[m * st]);
          if (m >= 2) s = cadd(s, cscale(a.sm2[m], X[(m - 2) * st]));
          if (m + 2 < nz) s = cadd(s, cscale(a.sp2[m], X[(m + 2) * st]));
          if (m == 0) s = cadd(s, cscale(a.se0, g0));
          if (m == 1) s = cadd(s, cscale(a.se1, g1));
          CP[m * st] = s;
        }
        for (int m = 0; m < nz; ++m) stv(c, m, CP[m * st]);
      }
      for (int j = 0; j < nz; ++j) stv(2, j, make_double2(0, 0));
      continue;
    }
    const double kx = a.kvx[ix], ky = a.kvy[iy];
    const double Dx = ((a.nx % 2) == 0 && ix == a.nx / 2) ? 0.0 : kx;
    const double Dy = ((a.ny % 2) == 0 && iy == a.ny / 2) ? 0.0 : ky;
    const double K = sqrt(kx * kx + ky * ky);
    const double *mf = a.mfac + i, *ib = a.invb + i, *d2 = a.dp2 + i;
    const double *A0 = a.ab0 + i, *A1 = a.ab1 + i, *C0 = a.c0 + i, *C1 = a.c1 + i;
    const double G00 = a.ginv[i], G10 = a.ginv[nk + i], G01 = a.ginv[2 * nk + i],
                 G11 = a.ginv[3 * nk + i];

    // --- pressure RHS: Dx f + Dy g + d/dz h (DPTools.cpp:134-195) --------
    {
      double2 dfp1 = make_double2(0, 0), dfp2 = make_double2(0, 0);  // df[j+1], df[j+2]
      double2 fzn = make_double2(0, 0);                               // fz[j+1]
      for (int j = nz - 1; j >= 0; --j) {
        double2 df;
        if (j == nz - 1) df = make_double2(0, 0);
        else df = cadd(dfp2, cscale((double)((j + 1) * 2) / a.H, fzn));
        double2 fz = ld(2, j);
        double2 dfv = (j == 0) ? cscale(0.5, df) : df;
        double2 p = cadd(cadd(cik(Dx, ld(0, j)), cik(Dy, ld(1, j))), dfv);
        X[j * st] = p;
        dfp2 = dfp1;
        dfp1 = df;
        fzn = fz;
      }
    }
    // --- Schur solve for the pressure (DPTools.cpp:236-285) ---------------
    auto penta = [&](double2 &y0, double2 &y1) {
      // forward elimination (X[0], X[1] unchanged)
      double2 xm2 = X[0], xm1 = X[st];
      for (int j = 2; j < nz; ++j) {
        double2 v = csub(X[j * st], cscale(mf[j * nk], xm2));
        X[j * st] = v;
        xm2 = xm1;
        xm1 = v;
      }
      double2 xl = cscale(ib[nz * nk], X[(nz - 1) * st]);
      double2 xl2 = cscale(ib[(nz - 1) * nk], X[(nz - 2) * st]);
      X[(nz - 1) * st] = xl;
      X[(nz - 2) * st] = xl2;
      y0 = cadd(cscale(C0[(nz - 1) * nk], xl), cscale(C0[(nz - 2) * nk], xl2));
      y1 = cadd(cscale(C1[(nz - 1) * nk], xl), cscale(C1[(nz - 2) * nk], xl2));
      double2 xp2 = xl, xp1 = xl2;  // x[j+2], x[j+1]
      for (int j = nz - 3; j >= 0; --j) {
        double2 v = cscale(ib[(j + 1) * nk], csub(X[j * st], cscale(d2[j * nk], xp2)));
        X[j * st] = v;
        y0 = cadd(y0, cscale(C0[j * nk], v));
        y1 = cadd(y1, cscale(C1[j * nk], v));
        xp2 = xp1;
        xp1 = v;
      }
    };
    // x = xpenta - A^{-1}B g, then S [x; g] (and F [x; g]) for rows m
    auto border = [&](double2 g0, double2 g1) {
      for (int j = 0; j < nz; ++j)
        X[j * st] = csub(X[j * st], cadd(cscale(A0[j * nk], g0), cscale(A1[j * nk], g1)));
      X[nz * st] = g0;
      X[(nz + 1) * st] = g1;
    };
    double2 ssum = make_double2(0, 0), asum = make_double2(0, 0);
    {
      double2 y0, y1;
      penta(y0, y1);
      double2 g0 = cadd(cscale(G00, y0), cscale(G01, y1));
      double2 g1 = cadd(cscale(G10, y0), cscale(G11, y1));
      border(g0, g1);
      for (int m = 0; m < nz; ++m) {
        double2 c = cscale(a.s0[m], X[m * st]);
        if (m >= 2) c = cadd(cscale(a.sm2[m], X[(m - 2) * st]), c);
        c = cadd(c, cscale(a.sp2[m], X[(m + 2) * st]));
        if (m == 0) c = cadd(c, cscale(a.se0, g0));
        if (m == 1) c = cadd(c, cscale(a.se1, g1));
        double2 dpv = cscale(a.fp1[m], X[(m + 1) * st]);
        if (m >= 1) dpv = cadd(cscale(a.fm1[m], X[(m - 1) * st]), dpv);
        if (m == 0) dpv = cadd(dpv, cscale(a.fe, g1));
        CP[m * st] = c;
        DP[m * st] = dpv;
        ssum = cadd(ssum, c);
        asum = (m & 1) ? csub(asum, c) : cadd(asum, c);
      }
    }
    // --- velocity BC right-hand sides (DPTools.cpp:218-234) ----------------
    const double fac1 = 2.0 * a.eta, fac = fac1 * K;
    const double ifac = 1.0 / fac, ifac1 = 1.0 / fac1;
    double2 bc[6];
    bc[0] = cscale(-ifac, cik(Dx, ssum));
    bc[1] = cscale(ifac, cik(Dx, asum));
    bc[2] = cscale(-ifac, cik(Dy, ssum));
    bc[3] = cscale(ifac, cik(Dy, asum));
    bc[4] = cscale(ifac1, ssum);
    bc[5] = cscale(ifac1, asum);
    // --- three velocity Schur solves (DPTools.cpp:197-216, 287-345) --------
    double2 wtop[3], wbot[3];
    for (int c = 0; c < 3; ++c) {
      for (int j = 0; j < nz; ++j) {
        double2 f = ld(c, j);
        double2 r;
        if (c == 0) r = csub(cik(Dx, CP[j * st]), f);
        else if (c == 1) r = csub(cik(Dy, CP[j * st]), f);
        else r = csub(DP[j * st], f);
        X[j * st] = cscale(inv_eta, r);
      }
      double2 y0, y1;
      penta(y0, y1);
      double2 r0 = csub(y0, bc[2 * c]), r1 = csub(y1, bc[2 * c + 1]);
      double2 g0 = cadd(cscale(G00, r0), cscale(G01, r1));
      double2 g1 = cadd(cscale(G10, r0), cscale(G11, r1));
      border(g0, g1);
      double2 st_ = make_double2(0, 0), sb = make_double2(0, 0);
      for (int m = 0; m < nz; ++m) {
        double2 u = cscale(a.s0[m], X[m * st]);
        if (m >= 2) u = cadd(cscale(a.sm2[m], X[(m - 2) * st]), u);
        u = cadd(u, cscale(a.sp2[m], X[(m + 2) * st]));
        if (m == 0) u = cadd(u, cscale(a.se0, g0));
        if (m == 1) u = cadd(u, cscale(a.se1, g1));
        stv(c, m, u);
        st_ = cadd(st_, u);
        sb = (m & 1) ? csub(sb, u) : cadd(sb, u);
      }
      wtop[c] = st_;
      wbot[c] = sb;
    }
    // --- wall-correction coefficients --------------------------------------
    double2 *cr = corr + i * 16;
    if (a.mode == 1) {
      for (int c = 0; c < 3; ++c) cr[c] = make_double2(-wbot[c].x, -wbot[c].y);
    } else if (a.mode == 2) {
      double2 fb[3], ft[3], cf[8];
      for (int c = 0; c < 3; ++c) {
        fb[c] = make_double2(-wbot[c].x, -wbot[c].y);
        ft[c] = make_double2(-wtop[c].x, -wtop[c].y);
      }
      slit_coeffs(kx, ky, a.Lz, a.eta, fb, ft, cf);
      for (int q = 0; q < 8; ++q) cr[q] = cf[q];
      double kxp, kyp;
      if (!mode_is_hermitian(a, ix, iy, kx, ky, kxp, kyp)) {
        for (int c = 0; c < 3; ++c) {
          fb[c] = cconj(fb[c]);
          ft[c] = cconj(ft[c]);
        }
        slit_coeffs(kxp, kyp, a.Lz, a.eta, fb, ft, cf);
        for (int q = 0; q < 8; ++q) cr[8 + q] = cf[q];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// z transform GEMM.  OUT[r][col] = sum_m Tm[r][m] IN[m][col] for the real
// view of spec (per component: nz rows x ncols = 2*nk columns), in place.
// CTA: 256 threads, tile = all rows x 64 columns; each thread 4 columns x RPT
// rows.  The transform matrix sits in shared memory for the CTA's lifetime
// (persistent grid-stride over tiles).
// Inverse epilogue: add the wall correction at the node and scale.
// ---------------------------------------------------------------------------


template <typename R>
__device__ __forceinline__ void corr_value(const EpiArgs &e, int d, int m, int64_t mode, R &re, R &im) {
  re = 0;
  im = 0;
  const KsArgs &a = e.ks;
  if (a.mode == 0 || mode == 0) return;
  const int ix = (int)(mode % a.nxh), iy = (int)(mode / a.nxh);
  const double kx = a.kvx[ix], ky = a.kvy[iy];
  const double k = sqrt(kx * kx + ky * ky);
  double kxp, kyp;
  const bool herm = mode_is_hermitian(a, ix, iy, kx, ky, kxp, kyp);
  const double z = a.zn[m];
  const double2 *cr = e.corr + mode * 16;
  double2 acc = make_double2(0, 0);
  const int npass = herm ? 1 : 2;
  for (int pass = 0; pass < npass; ++pass) {
    const double qx = pass ? kxp : kx, qy = pass ? kyp : ky;
    double2 v;
    const double enkz = exp(-k * z);
    if (a.mode == 1) {
      // DPTools.cpp:627-641, velocity rows
      double2 f0 = cr[0], f1 = cr[1], f2 = cr[2];
      if (pass) { f0 = cconj(f0); f1 = cconj(f1); f2 = cconj(f2); }
      double2 al = cadd(cadd(cscale(qx, f0), cscale(qy, f1)), cik(k, f2));
      const double zenkz = z * enkz;
      if (d == 0) v = cadd(cscale(-qx * zenkz / k, al), cscale(enkz, f0));
      else if (d == 1) v = cadd(cscale(-qy * zenkz / k, al), cscale(enkz, f1));
      else v = cadd(cik(-zenkz, al), cscale(enkz, f2));
    } else {
      // DPTools.cpp:795-815 with e^{k(z-H)} evaluated directly
      const double2 *c = cr + 8 * pass;
      const double fac = 1.0 / 2.0 / a.eta;
      const double ekzmh = exp(k * (z - a.Lz));
      const double zenkz = z * enkz, zekzmh = z * ekzmh;
      if (d == 0)
        v = cadd(cadd(cik(-qx * zenkz * fac / k, c[0]), cik(qx * zekzmh * fac / k, c[1])),
                 cadd(cscale(enkz, c[2]), cscale(ekzmh, c[3])));
      else if (d == 1)
        v = cadd(cadd(cik(-qy * zenkz * fac / k, c[0]), cik(qy * zekzmh * fac / k, c[1])),
                 cadd(cscale(enkz, c[4]), cscale(ekzmh, c[5])));
      else
        v = cadd(cadd(cscale(zenkz * fac, c[0]), cscale(zekzmh * fac, c[1])),
                 cadd(cscale(enkz, c[6]), cscale(ekzmh, c[7])));
    }
    if (pass) v = cconj(v);
    acc = cadd(acc, v);
  }
  if (npass == 2) acc = cscale(0.5, acc);
  re = (R)acc.x;
  im = (R)acc.y;
}

template <typename R, int RPT>
__global__ void __launch_bounds__(256) k_zgemm(R *spec, int nz, int64_t ncols, const R *__restrict__ Tm,
                                              EpiArgs e) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R *Ts = reinterpret_cast<R *>(smem_raw);            // [16*RPT][nz+1]
  const int tstride = nz + 1;
  R *Bs = Ts + 16 * RPT * tstride;                     // [nz][64]
  const int tid = threadIdx.x;
  for (int idx = tid; idx < 16 * RPT * tstride; idx += 256) {
    int r = idx / tstride, m = idx % tstride;
    Ts[idx] = (r < nz && m < nz) ? Tm[r * nz + m] : (R)0;
  }
  const int tx = tid & 15, ty = tid >> 4;
  const int64_t tiles_per_comp = (ncols + 63) / 64;
  const int64_t ntiles = 3 * tiles_per_comp;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int d = (int)(t / tiles_per_comp);
    const int64_t c0 = (t % tiles_per_comp) * 64;
    R *B = spec + (int64_t)d * nz * ncols;
    __syncthreads();
    for (int idx = tid; idx < nz * 64; idx += 256) {
      int m = idx >> 6, c = idx & 63;
      Bs[idx] = (c0 + c < ncols) ? B[(int64_t)m * ncols + c0 + c] : (R)0;
    }
    __syncthreads();
    R acc[RPT][4];
#pragma unroll
    for (int q = 0; q < RPT; ++q)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[q][c] = 0;
    for (int m = 0; m < nz; ++m) {
      R b[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) b[c] = Bs[m * 64 + tx * 4 + c];
#pragma unroll
      for (int q = 0; q < RPT; ++q) {
        R av = Ts[(ty + 16 * q) * tstride + m];
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[q][c] = fma(av, b[c], acc[q][c]);
      }
    }
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
      const int r = ty + 16 * q;
      if (r >= nz) continue;
#pragma unroll
      for (int cp = 0; cp < 2; ++cp) {
        const int64_t col = c0 + tx * 4 + 2 * cp;  // even: real part of one mode
        if (col >= ncols) continue;
        R vr = acc[q][2 * cp], vi = acc[q][2 * cp + 1];
        if (e.inverse) {
          R cre, cim;
          corr_value<R>(e, d, r, col >> 1, cre, cim);
          vr = (vr + cre) * (R)e.scale;
          vi = (vi + cim) * (R)e.scale;
        }
        B[(int64_t)r * ncols + col] = vr;
        B[(int64_t)r * ncols + col + 1] = vi;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
void launch_bvp_factors(const KsArgs &a, cudaStream_t s) {
  int bs = 128;
  k_bvp_factors<<<(a.nk + bs - 1) / bs, bs, 0, s>>>(a);
}

template <typename R>
void launch_bvp(const KsArgs &a, R *spec, double2 *corr, double2 *scratch, int64_t nthreads,
                cudaStream_t s) {
  k_bvp<R><<<nthreads / 64, 64, 0, s>>>(a, spec, corr, scratch, nthreads);
}

template <typename R, int RPT>
static cudaError_t zgemm_rpt(R *spec, int nz, int64_t ncols, const R *Tm, const EpiArgs &e, int nsm,
                             cudaStream_t s) {
  size_t smem = (size_t)(16 * RPT * (nz + 1) + nz * 64) * sizeof(R);
  cudaError_t err = cudaFuncSetAttribute(k_zgemm<R, RPT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
  if (err != cudaSuccess) return err;
  int blocks_per_sm = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_zgemm<R, RPT>, 256, smem);
  if (err != cudaSuccess) return err;
  if (blocks_per_sm < 1) return cudaErrorInvalidConfiguration;
  int64_t ntiles = 3 * ((ncols + 63) / 64);
  int64_t grid = (int64_t)nsm * blocks_per_sm;
  if (grid > ntiles) grid = ntiles;
  k_zgemm<R, RPT><<<(unsigned)grid, 256, smem, s>>>(spec, nz, ncols, Tm, e);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_zgemm(R *spec, int nz, int64_t ncols, const R *Tm, const EpiArgs &e, int nsm,
                         cudaStream_t s) {
  int rpt = (nz + 15) / 16;
  if (rpt <= 2) return zgemm_rpt<R, 2>(spec, nz, ncols, Tm, e, nsm, s);
  if (rpt <= 4) return zgemm_rpt<R, 4>(spec, nz, ncols, Tm, e, nsm, s);
  if (rpt <= 6) return zgemm_rpt<R, 6>(spec, nz, ncols, Tm, e, nsm, s);
  if (rpt <= 8) return zgemm_rpt<R, 8>(spec, nz, ncols, Tm, e, nsm, s);
  return cudaErrorInvalidValue;
}

template void launch_bvp<float>(const KsArgs &, float *, double2 *, double2 *, int64_t, cudaStream_t);
template void launch_bvp<double>(const KsArgs &, double *, double2 *, double2 *, int64_t, cudaStream_t);
template cudaError_t launch_zgemm<float>(float *, int, int64_t, const float *, const EpiArgs &, int,
                                         cudaStream_t);
template cudaError_t launch_zgemm<double>(double *, int, int64_t, const double *, const EpiArgs &, int,
                                          cudaStream_t);

}  // namespace dpst
