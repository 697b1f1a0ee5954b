// Per-wavenumber Stokes BVP of the mixed operator in double-float arithmetic
// (the no-wall Schur/KBPENTA solve of DPTools.cpp:81-345 and the wall values
// the corrections of DPTools.cpp:590-877 start from), on the FP32 pipe.
//
// Same algorithm and factorisation as the FP64 solve (dpst_bvp.cu, bvp_mode):
// pressure right-hand side Dx f + Dy g + d/dz h, the KBPENTA forward and back
// sweeps with the border dots, the Schur correction with Ginv, the SIMat /
// FIMat window for the pressure coefficients and its z derivative, then the
// three velocity solves (z first) with the BC values from the pressure at
// z = +-1.  Every value is a double-float (dpst_df64.cuh, about 48
// significant bits); only the wall-correction coefficients of the slit
// channel (an 8 x 8 complex solve per mode) stay FP64.
//
// Scaled unknowns.  The matrix is A = I - K^2 S (S the second-integral bands)
// per parity chain, with pivots p_j and off-diagonals -K^2 sm2_j, -K^2 sp2_j.
// The sweeps run on u~_j = K^2 v_j / p_j (forward) and x~_j = K^2 x_j (back):
//   v_j = X_j + sm2_j u~_{j-2},  u~_j = kappa_j v_j,
//   x~_j = u~_j + kappa_j (sp2_j x~_{j+2}),   kappa_j = K^2 / p_j,
// so kappa is the only per-row factor the sweeps read (against the forward
// multiplier, pivot, upper band and both border rows of the unscaled form),
// the border rows C = h2k R2 + RA (H^2 K times one k-independent row plus
// another) are dotted as two k-independent sums, the Schur step takes
// g^ = K^2 g = Ginv (C x~ - K^2 bc), and the window outputs carry a factor
// K^2 that is removed once per output.  One wavenumber's factors shrink from
// 6 to 2 values per row, which keeps the re-reads of the four solves in L2.
//
// Work decomposition: four lanes per wavenumber.  The banded matrix couples
// row j with j +- 2 only, and its border columns act on rows of one parity
// each, so the sweeps split into an even and an odd chain; all operators
// have real coefficients, so real and imaginary parts split too.  Lane
// (part, parity) = (lane & 1, (lane >> 1) & 1) of a quad owns the rows of
// its parity of the real or imaginary part: a column of ceil(nz / 2)
// double-floats in shared memory ([row][lane], conflict-free).  The chains
// meet only in the border dots and coefficient sums (one shuffle each) and in
// the pressure window, whose z-derivative band reads the other parity's
// neighbours (the two lanes of a parity pair walk their rows in lockstep and
// exchange them by shuffles).  The pressure coefficients, read back by the
// other part's lane for the x and y velocity right-hand sides, go to an
// L2-resident global scratch [row][lane of the grid].  With half-length
// columns, 13 warps per SM fit at nz = 128 (the FP64 solve fits 6), enough to
// keep the FP32 pipe issuing through the double-float dependency chains.
#include "dpst_internal.cuh"
#include "dpst_kdev.cuh"
#include "dpst_df64.cuh"

namespace dpst {

constexpr int DFS_NZMAX = 128;
enum DfTab { DT_S0, DT_SM2, DT_SP2, DT_FM1, DT_FP1, DT_S0E, DT_SM2E, DT_SP2E, DT_BR2, DT_BRA, DT_DH };
// k-independent tables as double-floats, at fixed offsets (the first BC row
// as C0 = H^2 K BR2 + BRA); then the scalars se0, se1, fe, se0 / eta,
// se1 / eta, 1 / eta
__shared__ float2 dfs_tab[DT_DH * DFS_NZMAX + DFS_NZMAX + 1 + 6];
#define DTAB(t, j) df_lds(dfs_tab[(t) * DFS_NZMAX + (j)])
constexpr int DT_SCAL = DT_DH * DFS_NZMAX + DFS_NZMAX + 1;

struct DfCtx {
  float2 *Xs;         // this lane's column, row t at Xs[t * NT]
  float2 *CPs;        // this lane's pressure coefficients, row t at CPs[t * GT]
  const float2 *CPo;  // the other part's (same parity)
  int NT, GT;
};

// Row loops with their global loads read ahead of use: ld(t) is issued PF
// rows before body(t, value) runs (a ring of PF values in registers; loads
// past the end are clamped to row n - 1 and discarded).  Up: t = 0 .. n-1;
// down: t = n-1 .. 0.  n >= 1.
template <int PF, typename T, typename Ld, typename Body>
static __device__ __forceinline__ void rows_up(int n, Ld &&ld, Body &&body) {
  T ring[PF];
#pragma unroll
  for (int k = 0; k < PF; ++k) ring[k] = ld(min(k, n - 1));
  int t = 0;
  for (; t + PF <= n; t += PF) {
#pragma unroll
    for (int k = 0; k < PF; ++k) {
      const T v = ring[k];
      ring[k] = ld(min(t + PF + k, n - 1));
      body(t + k, v);
    }
  }
#pragma unroll
  for (int k = 0; k < PF - 1; ++k)
    if (t + k < n) body(t + k, ring[k]);
}
template <int PF, typename T, typename Ld, typename Body>
static __device__ __forceinline__ void rows_down(int n, Ld &&ld, Body &&body) {
  rows_up<PF, T>(n, [&](int s) { return ld(n - 1 - s); }, [&](int s, const T &v) { body(n - 1 - s, v); });
}

// Raw spectrum values (R) as double-float operands: FP32 values enter the
// FP32-operand forms directly; FP64 values (the FP64-I/O instantiation) are
// rounded to double-floats.
static __device__ __forceinline__ float df_v(float x) { return x; }
static __device__ __forceinline__ df64 df_v(double x) { return df_from_d(x); }
// the same as double-float values
static __device__ __forceinline__ df64 df_w(float x) { return df_from_f(x); }
static __device__ __forceinline__ df64 df_w(double x) { return df_from_d(x); }

template <typename R>
struct DfRhsP {  // pressure right-hand side inputs of one row
  R f, g, h;
};
template <typename R>
struct DfRhsV {  // velocity forward-sweep inputs of one row
  float2 k, cp;
  R f;
};
template <typename R>
struct DfWinP {  // pressure window inputs: A^{-1}B of row t + 1, f_z of row t
  float2 ab;
  R fz;
};

// Variants of the kernel: prefetch depths of the forward sweep, the back
// sweep and the windows (rows read ahead through register rings), and
// threads per CTA (13 warps with at most 128 registers, or 12 with 168).
// The fastest for a handle is chosen when it is created, by timing.
template <int F, int B, int W, int T>
struct DfCfg {
  static constexpr int PF_F = F, PF_B = B, PF_W = W, MAXT = T;
};
using DfV0 = DfCfg<4, 4, 4, 416>;
using DfV1 = DfCfg<8, 8, 4, 384>;
using DfV2 = DfCfg<8, 8, 8, 384>;
using DfV3 = DfCfg<4, 4, 4, 384>;
constexpr int DF_VARIANTS = 4;
constexpr int DF_MAXT = 416;  // the most threads of any variant

// Solve of wavenumber i by the quad of lanes this lane belongs to.
template <typename R, bool WALLS, typename CFG>
static __device__ __forceinline__ void dfs_mode(const KsArgs &a, R *__restrict__ spec, double2 *__restrict__ corr,
                                                float2 *__restrict__ corrf, int i, bool store, const DfCtx &c) {
  const int nz = a.nz;
  const int nk = (int)a.nk;  // nz * nk * 4 < 2^31 is checked at creation
  const int lane = threadIdx.x & 31;
  const int part = lane & 1, par = (lane >> 1) & 1;
  const int nzp = (nz + 1 - par) >> 1;  // rows of this parity
  const int nsteps = (nz + 1) >> 1;     // rows of parity 0: the lockstep length
  float2 *__restrict__ Xs = c.Xs;
  const int NT = c.NT, GT = c.GT;
#define XS(t) Xs[(t) * NT]
  const int rs = 2 * nk;  // spectrum row stride (R elements)
  R *__restrict__ sp_own = spec + 2 * i + part;
  const R *__restrict__ sp_oth = spec + 2 * i + (part ^ 1);
  const int ix = i % a.nxh, iy = i / a.nxh;
  // (i a)_part = sp a_(other part), sp = -1 for the real part
  const df64 dxs = part ? df_ld(a.dx2 + ix) : df_neg(df_ld(a.dx2 + ix));
  const df64 dys = part ? df_ld(a.dy2 + iy) : df_neg(df_ld(a.dy2 + iy));
  const float2 *__restrict__ kap0 = a.kap2 + i;
  const float2 *__restrict__ ab0 = a.ab2 + i;
  const float4 k2 = __ldg(a.km2 + i);
  const df64 K2 = df_make(k2.x, k2.y), iK2 = df_make(k2.z, k2.w);  // K^2, 1/K^2
  // g^ = Ginv r
  auto schur = [&](df64 r0, df64 r1, df64 &g0, df64 &g1) {
    g0 = df_fma(df_ld(a.gi2 + i), r0, df_mul(df_ld(a.gi2 + 2 * nk + i), r1));
    g1 = df_fma(df_ld(a.gi2 + nk + i), r0, df_mul(df_ld(a.gi2 + 3 * nk + i), r1));
  };

  // ---- pressure right-hand side over this chain, backward (DPTools.cpp:134-195):
  // X_j = Dx f + Dy g (other part) + d_j dh_j, with the Chebyshev derivative
  // dh_j = dh_{j+2} + (2 (j+1) / H) h_{j+1} (dh = 0 past the last row) and
  // d_0 = 1/2, d_j = 1 otherwise
  {
    df64 dh = df_zero();
    rows_down<CFG::PF_F, DfRhsP<R>>(
        nzp,
        [&](int t) {
          const int j = par + 2 * t;
          DfRhsP<R> v;
          v.f = sp_oth[j * rs];
          v.g = sp_oth[(nz + j) * rs];
          v.h = sp_own[(2 * nz + min(j + 1, nz - 1)) * rs];
          return v;
        },
        [&](int t, const DfRhsP<R> &v) {
          const int j = par + 2 * t;
          if (j + 1 < nz) dh = df_fma(DTAB(DT_DH, j + 1), df_v(v.h), dh);
          df64 X = df_mul(dxs, df_v(v.f));
          X = df_fma(dys, df_v(v.g), X);
          X = df_add(X, j == 0 ? df_scale2(dh, 0.5f) : dh);
          XS(t) = df_f2(X);
        });
  }

  // KBPENTA sweeps (LinearSolvers.h:106-141) on this chain in the scaled
  // unknowns, in place; returns y~ = C x~ summed over both chains.  The
  // forward sweep takes its right-hand side from XS or (x / y velocity) forms
  // Dc cp_other - f_c.
  const float4 k3 = __ldg(a.km3 + i);
  const df64 h2k = df_make(k3.x, k3.y);
  // The two BC rows are mirror images: bcl_j = -(-1)^j bcr_j for j < nz
  // (Solvers.py:603-643 builds them with the same magnitudes), so on one
  // parity chain C1 = sg C0 with sg = -1 (even rows) or +1 (odd rows), up to
  // the FP64 rounding of the reference's sums; one dot per chain gives both.
  const float sg = par ? 1.0f : -1.0f;
  auto back = [&](df64 &y0, df64 &y1) {
    df64 xn = df_zero();
    df_acc s1 = acc_zero(), s2 = acc_zero();
    rows_down<CFG::PF_B, float2>(
        nzp, [&](int t) { return __ldg(kap0 + (par + 2 * t) * nk); },
        [&](int t, const float2 &k) {
          const int j = par + 2 * t;
          const df64 x = df_fma(df_make(k.x, k.y), df_mul(DTAB(DT_SP2, j), xn), df_lds(XS(t)));
          XS(t) = df_f2(x);
          xn = x;
          acc_fma(s1, DTAB(DT_BR2, j), x);
          acc_fma(s2, DTAB(DT_BRA, j), x);
        });
    const df64 o0 = df_fma(h2k, acc_val(s1), acc_val(s2)), o1 = df_scale2(o0, sg);
    y0 = df_add(o0, df_shfl_xor(o0, 2));
    y1 = df_add(o1, df_shfl_xor(o1, 2));
  };
  auto penta_xs = [&](df64 &y0, df64 &y1) {
    df64 un = df_zero();
    rows_up<CFG::PF_F, float2>(
        nzp, [&](int t) { return __ldg(kap0 + (par + 2 * t) * nk); },
        [&](int t, const float2 &k) {
          const df64 u = df_mul(df_make(k.x, k.y), df_fma(DTAB(DT_SM2, par + 2 * t), un, df_lds(XS(t))));
          XS(t) = df_f2(u);
          un = u;
        });
    back(y0, y1);
  };
  auto penta_vel = [&](df64 dcs, const R *fs, df64 &y0, df64 &y1) {
    df64 un = df_zero();
    const float2 *cpo = c.CPo;
    rows_up<CFG::PF_F, DfRhsV<R>>(
        nzp,
        [&](int t) {
          const int j = par + 2 * t;
          DfRhsV<R> v;
          v.k = __ldg(kap0 + j * nk);
          v.cp = cpo[t * GT];
          v.f = fs[j * rs];
          return v;
        },
        [&](int t, const DfRhsV<R> &v) {
          const df64 X = df_fms(dcs, df_make(v.cp.x, v.cp.y), df_v(v.f));
          const df64 u = df_mul(df_make(v.k.x, v.k.y), df_fma(DTAB(DT_SM2, par + 2 * t), un, X));
          XS(t) = df_f2(u);
          un = u;
        });
    back(y0, y1);
  };
  const bool ext0 = (par + 2 * nzp == nz);  // this chain's extension is g0 (else g1)

  // ---- pressure: Schur solve, cp = S [x; g] (kept, times K^2, for the other
  // part's x, y velocity right-hand sides), dp = F [x; g] -> z-velocity
  // right-hand side.  The border-corrected solution of this chain, times K^2,
  // is x^_j = x~_j - (A^{-1}B)_j g^_par (column 0 on even rows, column 1 on
  // odd rows), extended by the border unknown that follows its last row
  // (x_nz = g0, x_nz+1 = g1).
  df_acc pacc = acc_zero();  // sum of this chain's pressure coefficients (x K^2)
  {
    df64 y0, y1, g0, g1;
    penta_xs(y0, y1);
    schur(y0, y1, g0, g1);
    const df64 gown = par ? g1 : g0, gext = ext0 ? g0 : g1;
    df64 xm = df_zero();
    df64 x0 = df_fnma(df_ld(ab0 + par * nk), gown, df_lds(XS(0)));
    float2 *cpw = c.CPs;
    rows_up<CFG::PF_W, DfWinP<R>>(
        nsteps,
        [&](int t) {
          DfWinP<R> v;
          v.ab = __ldg(ab0 + (par + 2 * min(t + 1, nzp - 1)) * nk);
          v.fz = sp_own[(2 * nz + par + 2 * min(t, nzp - 1)) * rs];
          return v;
        },
        [&](int t, const DfWinP<R> &v) {
          const int m = par + 2 * t;
          const df64 xp = (t + 1 < nzp)    ? df_fnma(df_make(v.ab.x, v.ab.y), gown, df_lds(XS(t + 1)))
                          : (t + 1 == nzp) ? gext
                                           : df_zero();
          // the other chain's neighbours x_{m-1}, x_{m+1}: parity 0 takes the
          // partner's x(t - 1), x(t); parity 1 its x(t), x(t + 1)
          const df64 px0 = df_shfl_xor(x0, 2), pside = df_shfl_xor(par ? xm : xp, 2);
          const df64 xl = par ? px0 : pside, xr = par ? pside : px0;
          if (t < nzp) {
            df64 cp = df_mul(DTAB(DT_S0, m), x0);
            if (m >= 2) cp = df_fma(DTAB(DT_SM2, m), xm, cp);
            cp = df_fma(DTAB(DT_SP2, m), xp, cp);
            if (m == 0) cp = df_fma(df_lds(dfs_tab[DT_SCAL]), g0, cp);
            if (m == 1) cp = df_fma(df_lds(dfs_tab[DT_SCAL + 1]), g1, cp);
            df64 dp = df_mul(DTAB(DT_FP1, m), xr);
            if (m >= 1) dp = df_fma(DTAB(DT_FM1, m), xl, dp);
            if (m == 0) dp = df_fma(df_lds(dfs_tab[DT_SCAL + 2]), g1, dp);
            cpw[t * GT] = df_f2(cp);
            acc_add(pacc, cp);
            // eta x z-velocity RHS (DPTools.cpp:214)
            XS(t) = df_f2(df_fms(dp, iK2, df_v(v.fz)));
          }
          xm = x0;
          x0 = xp;
        });
  }
  // velocity BC right-hand sides (DPTools.cpp:218-234): the pressure at
  // z = +-1 is the sum and the alternating sum of its coefficients; the
  // velocity solves run on eta x their right-hand sides (1/eta sits in the
  // window's SIMat bands), so the BC values are scaled by eta too; they enter
  // the Schur step times K^2
  df64 bc[6];
  {
    const df64 hK = df_make(k3.z, k3.w);  // 1 / (2 K)
    const df64 pown = df_mul(acc_val(pacc), iK2);
    const df64 poth = df_shfl_xor(pown, 2);
    const df64 pe = par ? poth : pown, po = par ? pown : poth;
    const df64 ssum = df_add(pe, po), asum = df_sub(pe, po);
    const df64 ssum_o = df_shfl_xor(ssum, 1), asum_o = df_shfl_xor(asum, 1);
    bc[0] = df_neg(df_mul(hK, df_mul(dxs, ssum_o)));
    bc[1] = df_mul(hK, df_mul(dxs, asum_o));
    bc[2] = df_neg(df_mul(hK, df_mul(dys, ssum_o)));
    bc[3] = df_mul(hK, df_mul(dys, asum_o));
    bc[4] = df_scale2(ssum, 0.5f);
    bc[5] = df_scale2(asum, 0.5f);
  }
  __syncwarp();  // the other part's pressure coefficients are read below

  // ---- velocity: three Schur solves (DPTools.cpp:197-216, 287-345); z first
  df64 wt[3], wb[3];
#pragma unroll
  for (int cc = 0; cc < 3; ++cc) {
    const int comp = (cc + 2) % 3;  // 2, 0, 1
    df64 y0, y1, g0, g1;
    if (comp == 2) penta_xs(y0, y1);
    else penta_vel(df_mul(comp == 0 ? dxs : dys, iK2), sp_own + comp * nz * rs, y0, y1);
    schur(df_fnma(K2, bc[2 * comp], y0), df_fnma(K2, bc[2 * comp + 1], y1), g0, g1);
    const df64 gown = par ? g1 : g0, gext = ext0 ? g0 : g1;
    df_acc uacc = acc_zero();
    R *us = sp_own + (comp * nz + par) * rs;
    df64 xm = df_zero();
    df64 x0 = df_fnma(df_ld(ab0 + par * nk), gown, df_lds(XS(0)));
    rows_up<CFG::PF_W, float2>(
        nzp, [&](int t) { return __ldg(ab0 + (par + 2 * min(t + 1, nzp - 1)) * nk); },
        [&](int t, const float2 &ab) {
          const int m = par + 2 * t;
          const df64 xp = (t + 1 < nzp) ? df_fnma(df_make(ab.x, ab.y), gown, df_lds(XS(t + 1))) : gext;
          df64 u = df_mul(DTAB(DT_S0E, m), x0);
          if (m >= 2) u = df_fma(DTAB(DT_SM2E, m), xm, u);
          u = df_fma(DTAB(DT_SP2E, m), xp, u);
          if (m == 0) u = df_fma(df_lds(dfs_tab[DT_SCAL + 3]), g0, u);
          if (m == 1) u = df_fma(df_lds(dfs_tab[DT_SCAL + 4]), g1, u);
          if (store) df_out(us + t * 2 * rs, df_mul(u, iK2));
          if (WALLS) acc_add(uacc, u);
          xm = x0;
          x0 = xp;
        });
    if (WALLS) {
      const df64 uown = df_mul(acc_val(uacc), iK2);
      const df64 uoth = df_shfl_xor(uown, 2);
      const df64 ue = par ? uoth : uown, uo = par ? uown : uoth;
      wt[comp] = df_add(ue, uo);  // u(z = 1), u(z = -1)
      wb[comp] = df_sub(ue, uo);
    }
  }
  if (!WALLS) {
    __syncwarp();  // column / pressure scratch reuse in the next mode
    return;
  }
  // wall-correction coefficients (evalTheta at z = 0 and z = Lz), FP64
  double wto[3], wbo[3], wtd[3], wbd[3];
  for (int q = 0; q < 3; ++q) {
    wtd[q] = df_to_d(wt[q]);
    wbd[q] = df_to_d(wb[q]);
    wto[q] = __shfl_xor_sync(0xffffffffu, wtd[q], 1);
    wbo[q] = __shfl_xor_sync(0xffffffffu, wbd[q], 1);
  }
  __syncwarp();  // column / pressure scratch reuse in the next mode
  if (!store || par != 0) return;
  double *crd = reinterpret_cast<double *>(corr + i * 16);
  if (a.mode == 1) {
    for (int q = 0; q < 3; ++q) crd[2 * q + part] = -wbd[q];
    if (corrf)
      for (int q = 0; q < 3; ++q) reinterpret_cast<float *>(corrf + i * 16)[2 * q + part] = (float)(-wbd[q]);
  } else if (a.mode == 2 && part == 0) {
    const double kx = __ldg(a.kvx + ix), ky = __ldg(a.kvy + iy);
    double2 fb[3], ft[3], cf[8];
    for (int q = 0; q < 3; ++q) {
      fb[q] = make_double2(-wbd[q], -wbo[q]);
      ft[q] = make_double2(-wtd[q], -wto[q]);
    }
    slit_coeffs(kx, ky, a.Lz, a.eta, fb, ft, cf);
    for (int r = 0; r < 8; ++r) corr[i * 16 + r] = cf[r];
    if (corrf)
      for (int r = 0; r < 8; ++r) corrf[i * 16 + r] = make_float2((float)cf[r].x, (float)cf[r].y);
    double kxp, kyp;
    if (!mode_is_hermitian(a, ix, iy, kx, ky, kxp, kyp)) {
      for (int q = 0; q < 3; ++q) {
        fb[q] = cconj(fb[q]);
        ft[q] = cconj(ft[q]);
      }
      slit_coeffs(kxp, kyp, a.Lz, a.eta, fb, ft, cf);
      for (int r = 0; r < 8; ++r) corr[i * 16 + 8 + r] = cf[r];
      if (corrf)
        for (int r = 0; r < 8; ++r) corrf[i * 16 + 8 + r] = make_float2((float)cf[r].x, (float)cf[r].y);
    }
  }
#undef XS
}

template <typename R>
cudaError_t launch_bvp_df(const KsArgs &a, R *spec, double2 *corr, float2 *scratch, int64_t grid, int variant,
                          cudaStream_t s);
template <typename R>
cudaError_t launch_bvp_df_b(const SysK<R> *sys, int S, const int64_t *mprefix, int64_t K, int nz, int mode,
                            float2 *scratch, int64_t grid, int variant, cudaStream_t s, int ncol = 0);
template <typename R>
cudaError_t launch_bvp_df_cols(const KsArgs &a, R *spec0, int64_t sstride, double2 *corr0, float2 *corrf0,
                               int64_t cstride, int ncol, float2 *scratch, int64_t grid, int variant,
                               cudaStream_t s);
template <typename R>
cudaError_t launch_adj_df(const KsArgs &a, R *spec, const double2 *cadj, float2 *scratch, int64_t grid, int variant,
                          cudaStream_t s);

// Persistent kernel: CTA b owns the units of 8 wavenumbers [b per_cta,
// (b+1) per_cta) and its warps take them from a shared-memory counter.
// The k-independent tables (every system of a batch shares nz, H and the BC
// rows) into static shared memory.
static __device__ __forceinline__ void dfs_tables(const KsArgs &a) {
  const int nz = a.nz, tid = threadIdx.x, NT = blockDim.x;
  const double inv_eta = 1.0 / a.eta;
  for (int t = tid; t < nz; t += NT) {
    dfs_tab[DT_S0 * DFS_NZMAX + t] = df_f2(df_from_d(a.s0[t]));
    dfs_tab[DT_SM2 * DFS_NZMAX + t] = df_f2(df_from_d(a.sm2[t]));
    dfs_tab[DT_SP2 * DFS_NZMAX + t] = df_f2(df_from_d(a.sp2[t]));
    dfs_tab[DT_FM1 * DFS_NZMAX + t] = df_f2(df_from_d(a.fm1[t]));
    dfs_tab[DT_FP1 * DFS_NZMAX + t] = df_f2(df_from_d(a.fp1[t]));
    dfs_tab[DT_S0E * DFS_NZMAX + t] = df_f2(df_from_d(a.s0[t] * inv_eta));
    dfs_tab[DT_SM2E * DFS_NZMAX + t] = df_f2(df_from_d(a.sm2[t] * inv_eta));
    dfs_tab[DT_SP2E * DFS_NZMAX + t] = df_f2(df_from_d(a.sp2[t] * inv_eta));
  }
  for (int t = tid; t < nz; t += NT) {
    // first BC row at k: C0 = bcr2 H^2 K + (bcr2 + (H bcr1 - bcr2))
    // (Solvers.py:315-331, as k_bvp_factors forms it)
    dfs_tab[DT_BR2 * DFS_NZMAX + t] = df_f2(df_from_d(a.bcr2[t]));
    dfs_tab[DT_BRA * DFS_NZMAX + t] = df_f2(df_from_d(a.bcr2[t] + (a.H * a.bcr1[t] - a.bcr2[t])));
  }
  for (int t = tid; t <= nz; t += NT) dfs_tab[DT_DH * DFS_NZMAX + t] = df_f2(df_from_d((double)(2 * t) / a.H));
  if (tid == 0) {
    dfs_tab[DT_SCAL] = df_f2(df_from_d(a.se0));
    dfs_tab[DT_SCAL + 1] = df_f2(df_from_d(a.se1));
    dfs_tab[DT_SCAL + 2] = df_f2(df_from_d(a.fe));
    dfs_tab[DT_SCAL + 3] = df_f2(df_from_d(a.se0 * inv_eta));
    dfs_tab[DT_SCAL + 4] = df_f2(df_from_d(a.se1 * inv_eta));
    dfs_tab[DT_SCAL + 5] = df_f2(df_from_d(inv_eta));
  }
}

static __device__ __forceinline__ DfCtx dfs_ctx(float2 *cols, float2 *cp_scratch) {
  const int tid = threadIdx.x, NT = blockDim.x;
  DfCtx c;
  c.NT = NT;
  c.GT = gridDim.x * NT;
  c.Xs = cols + tid;
  c.CPs = cp_scratch + (size_t)blockIdx.x * NT + tid;
  c.CPo = cp_scratch + (size_t)blockIdx.x * NT + (tid ^ 1);
  return c;
}

template <typename R, bool WALLS, typename CFG>
__global__ void __launch_bounds__(CFG::MAXT, 1) k_bvp_df(KsArgs a, R *__restrict__ spec, double2 *__restrict__ corr,
                                                         float2 *__restrict__ cp_scratch, int per_cta) {
  extern __shared__ float2 dfs_cols[];
  __shared__ int next_unit;
  dfs_tables(a);
  if (threadIdx.x == 0) next_unit = blockIdx.x * per_cta;
  __syncthreads();
  const DfCtx c = dfs_ctx(dfs_cols, cp_scratch);
  const int nk = (int)a.nk;
  const int units = (nk + 7) / 8;
  const int u_end = min((int)(blockIdx.x + 1) * per_cta, units);
  const int lane = threadIdx.x & 31;
  for (;;) {
    int u = 0;
    if (lane == 0) u = atomicAdd(&next_unit, 1);
    u = __shfl_sync(0xffffffffu, u, 0);
    if (u >= u_end) break;
    const int i_raw = u * 8 + (lane >> 2);
    const int i = i_raw < nk ? i_raw : nk - 1;
    const bool store = (i_raw < nk) && (i != 0);  // mode 0: k_bvp_k0
    dfs_mode<R, WALLS, CFG>(a, spec, corr, a.corrf, i, store, c);
  }
}

// Batched systems: units of 8 consecutive modes of the concatenated
// systems; a quad finds its system by binary search (all systems share nz,
// H and the geometry).  ncol > 0: the S systems are columns of one system,
// their modes interleaved wavenumber-major (k_bvp_df_cols does this with the
// system's arguments in the parameter space, which is faster).
template <typename R, bool WALLS, typename CFG>
__global__ void __launch_bounds__(CFG::MAXT, 1) k_bvp_df_b(const SysK<R> *__restrict__ sys, int S,
                                                           const int64_t *__restrict__ mprefix,
                                                           float2 *__restrict__ cp_scratch, int per_cta, int ncol) {
  extern __shared__ float2 dfs_cols[];
  __shared__ int next_unit;
  dfs_tables(sys[0].ks);
  if (threadIdx.x == 0) next_unit = blockIdx.x * per_cta;
  __syncthreads();
  const DfCtx c = dfs_ctx(dfs_cols, cp_scratch);
  const int64_t K = mprefix[S];
  const int units = (int)((K + 7) / 8);
  const int u_end = min((int)(blockIdx.x + 1) * per_cta, units);
  const int lane = threadIdx.x & 31;
  for (;;) {
    int u = 0;
    if (lane == 0) u = atomicAdd(&next_unit, 1);
    u = __shfl_sync(0xffffffffu, u, 0);
    if (u >= u_end) break;
    const int64_t g_raw = (int64_t)u * 8 + (lane >> 2);
    const int64_t g = g_raw < K ? g_raw : K - 1;
    int s, i;
    if (ncol > 0) {
      s = (int)(g % ncol);
      i = (int)(g / ncol);
    } else {
      s = find_sys(mprefix, S, g);
      i = (int)(g - mprefix[s]);
    }
    const SysK<R> &y = sys[s];
    const bool store = (g_raw < K) && (i != 0);  // mode 0 of each system: k_bvp_k0_b
    dfs_mode<R, WALLS, CFG>(y.ks, y.spec, y.corr, y.ks.corrf, i, store, c);
  }
}

// The K columns of a multi-RHS Mdot (one system: the same wavenumbers and
// factors; spectra, wall coefficients and their FP32 copies at fixed
// strides per column): mode g is column g % ncol of wavenumber g / ncol, so
// the quads of one warp that solve one wavenumber's columns share its factor
// reads, and the system's arguments stay in the parameter space.
template <typename R, bool WALLS, typename CFG>
__global__ void __launch_bounds__(CFG::MAXT, 1) k_bvp_df_cols(KsArgs a, R *__restrict__ spec0, int64_t sstride,
                                                              double2 *__restrict__ corr0,
                                                              float2 *__restrict__ corrf0, int64_t cstride,
                                                              int ncol, float2 *__restrict__ cp_scratch,
                                                              int per_cta) {
  extern __shared__ float2 dfs_cols[];
  __shared__ int next_unit;
  dfs_tables(a);
  if (threadIdx.x == 0) next_unit = blockIdx.x * per_cta;
  __syncthreads();
  const DfCtx c = dfs_ctx(dfs_cols, cp_scratch);
  const int64_t K = a.nk * ncol;
  const int units = (int)((K + 7) / 8);
  const int u_end = min((int)(blockIdx.x + 1) * per_cta, units);
  const int lane = threadIdx.x & 31;
  for (;;) {
    int u = 0;
    if (lane == 0) u = atomicAdd(&next_unit, 1);
    u = __shfl_sync(0xffffffffu, u, 0);
    if (u >= u_end) break;
    const int64_t g_raw = (int64_t)u * 8 + (lane >> 2);
    const int64_t g = g_raw < K ? g_raw : K - 1;
    const int col = (int)(g % ncol);
    const int i = (int)(g / ncol);
    const bool store = (g_raw < K) && (i != 0);  // mode 0 of each column: k_bvp_k0_b
    dfs_mode<R, WALLS, CFG>(a, spec0 + col * sstride, corr0 ? corr0 + col * cstride : nullptr,
                            corrf0 ? corrf0 + col * cstride : nullptr, i, store, c);
  }
}

// ---------------------------------------------------------------------------
// Adjoint of the solve (the backward pass's N_i^H, as k_bvp_adj_pairs in
// dpst_adjoint.cu computes it in FP64) in double-float arithmetic, with the
// same lanes, columns and K^2-scaled sweeps as the forward kernel.  Per
// velocity component (x, y, z): the transposed S window over the adjoint
// velocity (wall terms W^T included), the border adjoints gb = S_border^T v -
// (A^{-1}B)^T xbar, r = Ginv^T gb, then A^{-T} (xbar + C^T r) as
//   U^T: z~_j = kappa_j (X_j + sp2_{j-2} z~_{j-2})   (increasing j)
//   L^T: x~_j = z~_j + kappa_j sm2_{j+2} x~_{j+2}    (decreasing j)
// (z~, x~ the K^2-scaled unknowns); the adjoint right-hand sides feed the
// pressure's (i D_c cp -> the other part's rows) and the outputs -rhs/eta.
// Then the pressure: S^T cp_bar + F^T dp_bar (the z-derivative band from the
// other parity's rows), its border adjoints, A^{-T}, and the prhs adjoint
// into f0, f1 (-i Dx, -i Dy of the other part) and f2 (the transposed
// Chebyshev derivative recurrence, summed over the other parity's rows).
// Scratch: cp_bar and dp_bar, [row][lane of the grid] each.
// ---------------------------------------------------------------------------
template <typename R, typename CFG>
static __device__ __forceinline__ void dfs_adj_mode(const KsArgs &a, R *__restrict__ spec,
                                                    const double2 *__restrict__ cadj, int i, bool store,
                                                    const DfCtx &c, float2 *__restrict__ DPs,
                                                    const float2 *__restrict__ DPp) {
  const int nz = a.nz;
  const int nk = (int)a.nk;
  const int lane = threadIdx.x & 31;
  const int part = lane & 1, par = (lane >> 1) & 1;
  const int nzp = (nz + 1 - par) >> 1;
  float2 *__restrict__ Xs = c.Xs;
  const int NT = c.NT, GT = c.GT;
#define XS(t) Xs[(t) * NT]
#define XO(t) Xs[(t) * NT + (threadIdx.x ^ 1) - threadIdx.x]  // the other part, same row
#define XP(t) Xs[(t) * NT + (threadIdx.x ^ 2) - threadIdx.x]  // the other parity
  const int rs = 2 * nk;
  R *__restrict__ own = spec + 2 * i + part;
  const int ix = i % a.nxh, iy = i / a.nxh;
  const df64 dxs = part ? df_ld(a.dx2 + ix) : df_neg(df_ld(a.dx2 + ix));  // sp Dx
  const df64 dys = part ? df_ld(a.dy2 + iy) : df_neg(df_ld(a.dy2 + iy));
  const float2 *__restrict__ kap0 = a.kap2 + i;
  const float2 *__restrict__ ab0 = a.ab2 + i;
  const float4 k2 = __ldg(a.km2 + i), k3 = __ldg(a.km3 + i);
  const df64 iK2 = df_make(k2.z, k2.w), h2k = df_make(k3.x, k3.y), hK = df_make(k3.z, k3.w);
  const df64 inv_eta = df_lds(dfs_tab[DT_SCAL + 5]);
  const float sg = par ? 1.0f : -1.0f;    // C1 = sg C0 on this chain
  const float psg = par ? -1.0f : 1.0f;   // (-1)^j on this chain
  // r = Ginv^T gb
  auto schur_t = [&](df64 gb0, df64 gb1, df64 &r0, df64 &r1) {
    r0 = df_fma(df_ld(a.gi2 + i), gb0, df_mul(df_ld(a.gi2 + nk + i), gb1));
    r1 = df_fma(df_ld(a.gi2 + 2 * nk + i), gb0, df_mul(df_ld(a.gi2 + 3 * nk + i), gb1));
  };
  // A^{-T} (XS + C^T r) in place, leaving rhs_bar = x~ / K^2 in XS
  auto sweeps_t = [&](df64 rho) {
    const df64 rh = df_mul(h2k, rho);
    df64 zm = df_zero();
    rows_up<CFG::PF_F, float2>(
        nzp, [&](int t) { return __ldg(kap0 + (par + 2 * t) * nk); },
        [&](int t, const float2 &k) {
          const int j = par + 2 * t;
          df64 X = df_fma(DTAB(DT_BR2, j), rh, df_lds(XS(t)));
          X = df_fma(DTAB(DT_BRA, j), rho, X);
          if (t > 0) X = df_fma(DTAB(DT_SP2, j - 2), zm, X);
          const df64 z = df_mul(df_make(k.x, k.y), X);
          XS(t) = df_f2(z);
          zm = z;
        });
    df64 xn = df_zero();
    rows_down<CFG::PF_B, float2>(
        nzp, [&](int t) { return __ldg(kap0 + (par + 2 * t) * nk); },
        [&](int t, const float2 &k) {
          const int j = par + 2 * t;
          df64 x = df_lds(XS(t));
          if (t + 1 < nzp) x = df_fma(df_make(k.x, k.y), df_mul(DTAB(DT_SM2, j + 2), xn), x);
          xn = x;
          XS(t) = df_f2(df_mul(x, iK2));
        });
  };
  // transposed window over this chain's rows: XS(t) = (S^T v)_j [+ (F^T d)_j],
  // returning the border dot e = sum (A^{-1}B)_j xbar_j of this chain
  auto window_t = [&](auto &&vat, auto &&dat, bool with_d) -> df64 {
    df_acc e = acc_zero();
    df64 vm = df_zero(), v0 = vat(0);
    for (int t = 0; t < nzp; ++t) {
      const int j = par + 2 * t;
      const df64 vp = (t + 1 < nzp) ? vat(t + 1) : df_zero();
      df64 x = df_mul(DTAB(DT_S0, j), v0);
      if (j + 2 < nz) x = df_fma(DTAB(DT_SM2, j + 2), vp, x);
      if (j >= 2) x = df_fma(DTAB(DT_SP2, j - 2), vm, x);
      if (with_d) {
        if (j + 1 < nz) x = df_fma(DTAB(DT_FM1, j + 1), dat(j + 1), x);
        if (j >= 1) x = df_fma(DTAB(DT_FP1, j - 1), dat(j - 1), x);
      }
      XS(t) = df_f2(x);
      acc_fma(e, df_ld(ab0 + j * nk), x);
      vm = v0;
      v0 = vp;
    }
    return acc_val(e);
  };
  double wbb[3] = {0, 0, 0}, wtb[3] = {0, 0, 0};
  if (a.mode != 0 && i != 0) {
    const double *cd = reinterpret_cast<const double *>(cadj + (size_t)i * 6);
    for (int q = 0; q < 3; ++q) {
      wbb[q] = cd[2 * q + part];
      if (a.mode == 2) wtb[q] = cd[2 * (3 + q) + part];
    }
  }
  const df64 se0 = df_lds(dfs_tab[DT_SCAL]), se1 = df_lds(dfs_tab[DT_SCAL + 1]), fe = df_lds(dfs_tab[DT_SCAL + 2]);
  df64 bcbar[6];
#pragma unroll
  for (int comp = 0; comp < 3; ++comp) {
    R *us = own + comp * nz * rs;
    const df64 wterm = df_from_d((par ? -wbb[comp] : wbb[comp]) + wtb[comp]);
    auto vat = [&](int t) { return df_sub(df_w(us[(par + 2 * t) * rs]), wterm); };
    const df64 e_own = window_t(vat, [&](int) { return df_zero(); }, false);
    const df64 e_oth = df_shfl_xor(e_own, 2);
    const df64 vf = vat(0), vfo = df_shfl_xor(vf, 2);
    const df64 e0 = par ? e_oth : e_own, e1 = par ? e_own : e_oth;
    const df64 v0r = par ? vfo : vf, v1r = par ? vf : vfo;
    df64 r0, r1;
    schur_t(df_fnma(df_from_f(1.0f), e0, df_mul(se0, v0r)), df_fnma(df_from_f(1.0f), e1, df_mul(se1, v1r)), r0, r1);
    bcbar[2 * comp] = df_neg(r0);
    bcbar[2 * comp + 1] = df_neg(r1);
    sweeps_t(df_fma(df_from_f(sg), r1, r0));
    __syncwarp();  // the other part's rhs_bar is read below
    if (comp == 2) {
      for (int t = 0; t < nzp; ++t) {
        const df64 tj = df_mul(inv_eta, df_lds(XS(t)));
        DPs[t * GT] = df_f2(tj);
        if (store) df_out(us + (par + 2 * t) * rs, df_neg(tj));
      }
    } else {
      const df64 coef = df_neg(df_mul(comp == 0 ? dxs : dys, inv_eta));  // -sp D_c / eta
      for (int t = 0; t < nzp; ++t) {
        const df64 add = df_mul(coef, df_lds(XO(t)));
        float2 *cw = c.CPs + t * GT;
        *cw = df_f2(comp == 0 ? add : df_add(df_lds(*cw), add));
        if (store) df_out(us + (par + 2 * t) * rs, df_neg(df_mul(inv_eta, df_lds(XS(t)))));
      }
    }
    __syncwarp();  // XS is rewritten by the next window; DP / CP reads below
  }
  // bc adjoints -> ssum / asum adjoints (DPTools.cpp:218-234): bc0 = -(i Dx
  // ssum)/fac, bc1 = (i Dx asum)/fac, bc2, bc3 likewise with Dy, bc4 =
  // ssum/fac1, bc5 = asum/fac1, fac1 = 2 eta, fac = fac1 K
  const df64 ifac = df_mul(hK, inv_eta), ifac1 = df_scale2(inv_eta, 0.5f);
  const df64 b0o = df_shfl_xor(bcbar[0], 1), b1o = df_shfl_xor(bcbar[1], 1);
  const df64 b2o = df_shfl_xor(bcbar[2], 1), b3o = df_shfl_xor(bcbar[3], 1);
  const df64 ssb = df_fma(df_mul(dxs, ifac), b0o, df_fma(df_mul(dys, ifac), b2o, df_mul(ifac1, bcbar[4])));
  const df64 asb = df_fma(df_neg(df_mul(dxs, ifac)), b1o,
                          df_fma(df_neg(df_mul(dys, ifac)), b3o, df_mul(ifac1, bcbar[5])));
  const df64 cadd = df_fma(df_from_f(psg), asb, ssb);  // ssb + (-1)^j asb on this chain
  // pressure: S^T cp_bar + F^T dp_bar, dp_bar of the other parity at rows j +- 1
  {
    const int nzpp = (nz + 1 - (par ^ 1)) >> 1;  // rows of the other parity
    auto vat = [&](int t) { return df_add(df_lds(c.CPs[t * GT]), cadd); };
    auto dat = [&](int jj) {
      const int tp = (jj - (par ^ 1)) >> 1;  // row jj (other parity) in the other chain
      return (tp >= 0 && tp < nzpp) ? df_lds(DPp[tp * GT]) : df_zero();
    };
    const df64 e_own = window_t(vat, dat, true);
    const df64 e_oth = df_shfl_xor(e_own, 2);
    const df64 vf = vat(0), vfo = df_shfl_xor(vf, 2);
    const df64 e0 = par ? e_oth : e_own, e1 = par ? e_own : e_oth;
    const df64 v0r = par ? vfo : vf, v1r = par ? vf : vfo;
    const df64 d0 = par ? df_lds(DPp[0]) : df_lds(DPs[0]);
    df64 r0, r1;
    schur_t(df_fnma(df_from_f(1.0f), e0, df_mul(se0, v0r)),
            df_fnma(df_from_f(1.0f), e1, df_fma(fe, d0, df_mul(se1, v1r))), r0, r1);
    sweeps_t(df_fma(df_from_f(sg), r1, r0));  // XS = prhs_bar
  }
  __syncwarp();
  // prhs adjoint -> f0 += -i Dx prhs_bar, f1 += -i Dy prhs_bar (the other
  // part's rows), f2 += D^T of the derivative (DPTools.cpp:134-174): f2_j +=
  // (2 j / H) e_j, e_j the sum of prhs_bar over the other parity's rows below
  // j, the row-0 term halved
  if (store) {
    const df64 cx = df_neg(dxs), cy = df_neg(dys);
    R *f0 = own, *f1 = own + nz * rs, *f2 = own + 2 * nz * rs;
    df_acc e = acc_zero();
    // parity 1 rows start with the other chain's row 0 (halved); parity 0
    // rows sum the other chain's rows 1, 3, ... below them
    for (int t = 0; t < nzp; ++t) {
      const int j = par + 2 * t;
      const df64 po = df_lds(XO(t));
      df_out(f0 + j * rs, df_fma(cx, po, df_w(f0[j * rs])));
      df_out(f1 + j * rs, df_fma(cy, po, df_w(f1[j * rs])));
      if (par == 1) acc_add(e, t == 0 ? df_scale2(df_lds(XP(0)), 0.5f) : df_lds(XP(t)));
      if (j >= 1) df_out(f2 + j * rs, df_fma(DTAB(DT_DH, j), acc_val(e), df_w(f2[j * rs])));
      if (par == 0) acc_add(e, df_lds(XP(t)));
    }
  }
  __syncwarp();
#undef XS
#undef XO
#undef XP
}

template <typename R, typename CFG>
__global__ void __launch_bounds__(CFG::MAXT, 1) k_bvp_adj_df(KsArgs a, R *__restrict__ spec,
                                                             const double2 *__restrict__ cadj,
                                                             float2 *__restrict__ scratch, int per_cta) {
  extern __shared__ float2 dfs_cols[];
  __shared__ int next_unit;
  dfs_tables(a);
  if (threadIdx.x == 0) next_unit = blockIdx.x * per_cta;
  __syncthreads();
  const DfCtx c = dfs_ctx(dfs_cols, scratch);
  // dp_bar after cp_bar: [rows][lanes of the grid] each
  float2 *dp_base = scratch + (size_t)((a.nz + 1) / 2) * c.GT;
  float2 *DPs = dp_base + (size_t)blockIdx.x * c.NT + threadIdx.x;
  const float2 *DPp = dp_base + (size_t)blockIdx.x * c.NT + (threadIdx.x ^ 2);
  const int nk = (int)a.nk;
  const int units = (nk + 7) / 8;
  const int u_end = min((int)(blockIdx.x + 1) * per_cta, units);
  const int lane = threadIdx.x & 31;
  for (;;) {
    int u = 0;
    if (lane == 0) u = atomicAdd(&next_unit, 1);
    u = __shfl_sync(0xffffffffu, u, 0);
    if (u >= u_end) break;
    const int i_raw = u * 8 + (lane >> 2);
    const int i = i_raw < nk ? i_raw : nk - 1;
    const bool store = (i_raw < nk) && (i != 0);  // mode 0: k_bvp_adj_k0
    dfs_adj_mode<R, CFG>(a, spec, cadj, i, store, c, DPs, DPp);
  }
}

// Per-wavenumber data of the double-float solve (one thread per entry):
// kappa_j = K^2 / beta_{j+1} from the packed pivots, A^{-1}B, Ginv, the
// per-mode scalars and Dx, Dy.
__global__ void k_bvp_pack_df(KsArgs a) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nk = a.nk;
  auto k2_of = [&](int64_t i) {
    const int ix = (int)(i % a.nxh), iy = (int)(i / a.nxh);
    const double kx = a.kvx[ix], ky = a.kvy[iy];
    return kx * kx + ky * ky;
  };
  if (t < (int64_t)a.nz * nk) {
    const int64_t i = t % nk;
    a.kap2[t] = df_f2(df_from_d(k2_of(i) * a.bk[4 * t]));
    a.ab2[t] = df_f2(df_from_d(a.ab[t]));
  }
  if (t < 4 * nk) a.gi2[t] = df_f2(df_from_d(a.ginv[t]));
  if (t < nk) {
    const double K2 = k2_of(t), K = sqrt(K2);
    const df64 k2 = df_from_d(K2), ik2 = df_from_d(K2 > 0.0 ? 1.0 / K2 : 0.0);
    const df64 h2k = df_from_d((a.H * a.H) * K), hk = df_from_d(K > 0.0 ? 0.5 / K : 0.0);
    a.km2[t] = make_float4(k2.hi, k2.lo, ik2.hi, ik2.lo);
    a.km3[t] = make_float4(h2k.hi, h2k.lo, hk.hi, hk.lo);
  }
  if (t < a.nxh) {
    const double kx = a.kvx[t];
    a.dx2[t] = df_f2(df_from_d(((a.nx % 2) == 0 && t == a.nx / 2) ? 0.0 : kx));
  }
  if (t < a.ny) {
    const double ky = a.kvy[t];
    a.dy2[t] = df_f2(df_from_d(((a.ny % 2) == 0 && t == a.ny / 2) ? 0.0 : ky));
  }
}

void launch_bvp_pack_df(const KsArgs &a, cudaStream_t s) {
  int64_t tot = std::max<int64_t>((int64_t)a.nz * a.nk, 4 * a.nk);
  tot = std::max<int64_t>(tot, std::max(a.nxh, a.ny));
  k_bvp_pack_df<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(a);
}

// Threads per CTA of a variant for nz: as many warps as the columns
// (ceil(nz / 2) double-floats per lane) allow next to the static tables in
// 227 KB of shared memory, at most the variant's.
static int bvp_df_threads(int nz, int maxt) {
  const size_t per_warp = sizeof(float2) * (size_t)((nz + 1) / 2) * 32;
  const size_t stat = sizeof(dfs_tab) + 64;
  const size_t avail = (size_t)227 * 1024 - stat;
  int w = (int)(avail / per_warp);
  if (w > maxt / 32) w = maxt / 32;
  return w * 32;
}

template <typename CFG, typename R, bool WALLS>
static cudaError_t df_setup(int nz) {
  const int nt = bvp_df_threads(nz, CFG::MAXT);
  const size_t smem = sizeof(float2) * (size_t)((nz + 1) / 2) * nt;
  cudaError_t err = cudaFuncSetAttribute(k_bvp_df<R, WALLS, CFG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
  if (err == cudaSuccess)
    err = cudaFuncSetAttribute(k_bvp_df_cols<R, WALLS, CFG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  int per_sm = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bvp_df<R, WALLS, CFG>, nt, smem);
  if (err != cudaSuccess) return err;
  return per_sm < 1 ? cudaErrorInvalidConfiguration : cudaSuccess;
}

template <typename CFG, typename R, bool WALLS>
static cudaError_t df_setup_b(int nz) {
  const int nt = bvp_df_threads(nz, CFG::MAXT);
  const size_t smem = sizeof(float2) * (size_t)((nz + 1) / 2) * nt;
  return cudaFuncSetAttribute(k_bvp_df_b<R, WALLS, CFG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

template <typename CFG>
static cudaError_t df_setup_all(int nz) {
  cudaError_t e = df_setup<CFG, float, false>(nz);
  if (e == cudaSuccess) e = df_setup<CFG, float, true>(nz);
  if (e == cudaSuccess) e = df_setup_b<CFG, float, false>(nz);
  if (e == cudaSuccess) e = df_setup_b<CFG, float, true>(nz);
  return e;
}

int bvp_df_variants() { return DF_VARIANTS; }

// Grid (one CTA per SM, fewer when the units of 8 wavenumbers run out) and
// the bytes of the pressure scratch, for every variant.
cudaError_t bvp_df_plan(const KsArgs &a, int nsm, int64_t *grid, size_t *scratch_bytes) {
  if (a.nz > DFS_NZMAX) return cudaErrorInvalidValue;
  if ((int64_t)a.nz * a.nk * 4 >= ((int64_t)1 << 31)) return cudaErrorInvalidValue;
  cudaError_t err = df_setup_all<DfV0>(a.nz);
  if (err == cudaSuccess) err = df_setup_all<DfV1>(a.nz);
  if (err == cudaSuccess) err = df_setup_all<DfV2>(a.nz);
  if (err == cudaSuccess) err = df_setup_all<DfV3>(a.nz);
  if (err == cudaSuccess) err = df_setup<DfV1, double, false>(a.nz);
  if (err == cudaSuccess) err = df_setup<DfV1, double, true>(a.nz);
  if (err == cudaSuccess) err = df_setup_b<DfV1, double, false>(a.nz);
  if (err == cudaSuccess) err = df_setup_b<DfV1, double, true>(a.nz);
  if (err != cudaSuccess) return err;
  const int nt = bvp_df_threads(a.nz, DF_MAXT);
  int64_t g = nsm;
  const int64_t units = (a.nk + 7) / 8;
  const int64_t warps = nt / 32;
  if (g * warps > units) g = std::max<int64_t>(1, (units + warps - 1) / warps);
  *grid = g;
  *scratch_bytes = sizeof(float2) * (size_t)((a.nz + 1) / 2) * (size_t)g * nt;
  return cudaSuccess;
}

// Batched plan: the same for K modes in total with a shared nz (the tables
// of the first system stand for all).
cudaError_t bvp_df_plan_b(const KsArgs &a0, int64_t K, int nsm, int64_t *grid, size_t *scratch_bytes) {
  KsArgs a = a0;
  a.nk = K;
  if (a.nz > DFS_NZMAX) return cudaErrorInvalidValue;
  if (K >= ((int64_t)1 << 31)) return cudaErrorInvalidValue;
  a.nk = 1;  // the per-system bound is checked by each system's own plan
  cudaError_t err = bvp_df_plan(a, nsm, grid, scratch_bytes);
  if (err != cudaSuccess) return err;
  const int nt = bvp_df_threads(a.nz, DF_MAXT);
  int64_t g = nsm;
  const int64_t units = (K + 7) / 8;
  const int64_t warps = nt / 32;
  if (g * warps > units) g = std::max<int64_t>(1, (units + warps - 1) / warps);
  *grid = g;
  *scratch_bytes = sizeof(float2) * (size_t)((a.nz + 1) / 2) * (size_t)g * nt;
  return cudaSuccess;
}

template <typename CFG, typename R>
static cudaError_t df_launch_b(const SysK<R> *sys, int S, const int64_t *mprefix, int64_t K, int nz, int mode,
                               float2 *scratch, int64_t grid, int ncol, cudaStream_t s) {
  const int nt = bvp_df_threads(nz, CFG::MAXT);
  const size_t smem = sizeof(float2) * (size_t)((nz + 1) / 2) * nt;
  const int64_t units = (K + 7) / 8;
  const int per_cta = (int)((units + grid - 1) / grid);
  if (mode != 0)
    k_bvp_df_b<R, true, CFG><<<(unsigned)grid, nt, smem, s>>>(sys, S, mprefix, scratch, per_cta, ncol);
  else k_bvp_df_b<R, false, CFG><<<(unsigned)grid, nt, smem, s>>>(sys, S, mprefix, scratch, per_cta, ncol);
  return cudaGetLastError();
}

template <>
cudaError_t launch_bvp_df_b<float>(const SysK<float> *sys, int S, const int64_t *mprefix, int64_t K, int nz,
                                   int mode, float2 *scratch, int64_t grid, int variant, cudaStream_t s, int ncol) {
  switch (variant) {
    case 0: return df_launch_b<DfV0>(sys, S, mprefix, K, nz, mode, scratch, grid, ncol, s);
    case 2: return df_launch_b<DfV2>(sys, S, mprefix, K, nz, mode, scratch, grid, ncol, s);
    case 3: return df_launch_b<DfV3>(sys, S, mprefix, K, nz, mode, scratch, grid, ncol, s);
    default: return df_launch_b<DfV1>(sys, S, mprefix, K, nz, mode, scratch, grid, ncol, s);
  }
}
template <>
cudaError_t launch_bvp_df_b<double>(const SysK<double> *sys, int S, const int64_t *mprefix, int64_t K, int nz,
                                    int mode, float2 *scratch, int64_t grid, int variant, cudaStream_t s,
                                    int ncol) {
  (void)variant;
  return df_launch_b<DfV1>(sys, S, mprefix, K, nz, mode, scratch, grid, ncol, s);
}

template <typename CFG, typename R>
static cudaError_t adj_setup(int nz) {
  const int nt = bvp_df_threads(nz, CFG::MAXT);
  const size_t smem = sizeof(float2) * (size_t)((nz + 1) / 2) * nt;
  return cudaFuncSetAttribute(k_bvp_adj_df<R, CFG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

// The adjoint: the forward plan's grid, twice its scratch (cp_bar, dp_bar),
// sized for the largest variant.
cudaError_t bvp_adj_df_plan(const KsArgs &a, int nsm, int64_t *grid, size_t *scratch_bytes) {
  cudaError_t err = bvp_df_plan(a, nsm, grid, scratch_bytes);
  if (err == cudaSuccess) err = adj_setup<DfV0, float>(a.nz);
  if (err == cudaSuccess) err = adj_setup<DfV1, float>(a.nz);
  if (err == cudaSuccess) err = adj_setup<DfV2, float>(a.nz);
  if (err == cudaSuccess) err = adj_setup<DfV3, float>(a.nz);
  if (err == cudaSuccess) err = adj_setup<DfV1, double>(a.nz);
  if (err != cudaSuccess) return err;
  *scratch_bytes *= 2;
  return cudaSuccess;
}

template <typename CFG, typename R>
static cudaError_t adj_launch(const KsArgs &a, R *spec, const double2 *cadj, float2 *scratch, int64_t grid,
                              cudaStream_t s) {
  const int nt = bvp_df_threads(a.nz, CFG::MAXT);
  const size_t smem = sizeof(float2) * (size_t)((a.nz + 1) / 2) * nt;
  const int64_t units = (a.nk + 7) / 8;
  const int per_cta = (int)((units + grid - 1) / grid);
  k_bvp_adj_df<R, CFG><<<(unsigned)grid, nt, smem, s>>>(a, spec, cadj, scratch, per_cta);
  return cudaGetLastError();
}

// variant as for the forward solve (the FP64-I/O instantiation: variant 1)
template <>
cudaError_t launch_adj_df<float>(const KsArgs &a, float *spec, const double2 *cadj, float2 *scratch, int64_t grid,
                                 int variant, cudaStream_t s) {
  switch (variant) {
    case 0: return adj_launch<DfV0>(a, spec, cadj, scratch, grid, s);
    case 2: return adj_launch<DfV2>(a, spec, cadj, scratch, grid, s);
    case 3: return adj_launch<DfV3>(a, spec, cadj, scratch, grid, s);
    default: return adj_launch<DfV1>(a, spec, cadj, scratch, grid, s);
  }
}
template <>
cudaError_t launch_adj_df<double>(const KsArgs &a, double *spec, const double2 *cadj, float2 *scratch, int64_t grid,
                                  int variant, cudaStream_t s) {
  (void)variant;
  return adj_launch<DfV1>(a, spec, cadj, scratch, grid, s);
}

template <typename CFG, typename R>
static cudaError_t df_launch(const KsArgs &a, R *spec, double2 *corr, float2 *scratch, int64_t grid,
                             cudaStream_t s) {
  const int nt = bvp_df_threads(a.nz, CFG::MAXT);
  const size_t smem = sizeof(float2) * (size_t)((a.nz + 1) / 2) * nt;
  const int64_t units = (a.nk + 7) / 8;
  const int per_cta = (int)((units + grid - 1) / grid);
  if (a.mode != 0) k_bvp_df<R, true, CFG><<<(unsigned)grid, nt, smem, s>>>(a, spec, corr, scratch, per_cta);
  else k_bvp_df<R, false, CFG><<<(unsigned)grid, nt, smem, s>>>(a, spec, corr, scratch, per_cta);
  return cudaGetLastError();
}

template <typename CFG, typename R>
static cudaError_t df_launch_cols(const KsArgs &a, R *spec0, int64_t sstride, double2 *corr0, float2 *corrf0,
                                  int64_t cstride, int ncol, float2 *scratch, int64_t grid, cudaStream_t s) {
  const int nt = bvp_df_threads(a.nz, CFG::MAXT);
  const size_t smem = sizeof(float2) * (size_t)((a.nz + 1) / 2) * nt;
  const int64_t units = (a.nk * ncol + 7) / 8;
  const int per_cta = (int)((units + grid - 1) / grid);
  if (a.mode != 0)
    k_bvp_df_cols<R, true, CFG><<<(unsigned)grid, nt, smem, s>>>(a, spec0, sstride, corr0, corrf0, cstride, ncol,
                                                                   scratch, per_cta);
  else
    k_bvp_df_cols<R, false, CFG><<<(unsigned)grid, nt, smem, s>>>(a, spec0, sstride, corr0, corrf0, cstride, ncol,
                                                                    scratch, per_cta);
  return cudaGetLastError();
}

// ncol columns of one system (multi-RHS): spectra spec0 + c sstride (R
// elements), wall coefficients corr0 / corrf0 + c cstride; grid and scratch
// from bvp_df_plan_b over ncol nk modes.
template <>
cudaError_t launch_bvp_df_cols<float>(const KsArgs &a, float *spec0, int64_t sstride, double2 *corr0, float2 *corrf0,
                                      int64_t cstride, int ncol, float2 *scratch, int64_t grid, int variant,
                                      cudaStream_t s) {
  switch (variant) {
    case 0: return df_launch_cols<DfV0>(a, spec0, sstride, corr0, corrf0, cstride, ncol, scratch, grid, s);
    case 2: return df_launch_cols<DfV2>(a, spec0, sstride, corr0, corrf0, cstride, ncol, scratch, grid, s);
    case 3: return df_launch_cols<DfV3>(a, spec0, sstride, corr0, corrf0, cstride, ncol, scratch, grid, s);
    default: return df_launch_cols<DfV1>(a, spec0, sstride, corr0, corrf0, cstride, ncol, scratch, grid, s);
  }
}
template <>
cudaError_t launch_bvp_df_cols<double>(const KsArgs &a, double *spec0, int64_t sstride, double2 *corr0,
                                       float2 *corrf0, int64_t cstride, int ncol, float2 *scratch, int64_t grid,
                                       int variant, cudaStream_t s) {
  (void)variant;
  return df_launch_cols<DfV1>(a, spec0, sstride, corr0, corrf0, cstride, ncol, scratch, grid, s);
}

// variant in [0, bvp_df_variants()); the FP64-I/O instantiation (R = double,
// used to compare the solve with the FP64 one) exists in variant 1 only
template <>
cudaError_t launch_bvp_df<float>(const KsArgs &a, float *spec, double2 *corr, float2 *scratch, int64_t grid,
                                 int variant, cudaStream_t s) {
  switch (variant) {
    case 0: return df_launch<DfV0>(a, spec, corr, scratch, grid, s);
    case 2: return df_launch<DfV2>(a, spec, corr, scratch, grid, s);
    case 3: return df_launch<DfV3>(a, spec, corr, scratch, grid, s);
    default: return df_launch<DfV1>(a, spec, corr, scratch, grid, s);
  }
}
template <>
cudaError_t launch_bvp_df<double>(const KsArgs &a, double *spec, double2 *corr, float2 *scratch, int64_t grid,
                                  int variant, cudaStream_t s) {
  (void)variant;
  return df_launch<DfV1>(a, spec, corr, scratch, grid, s);
}

}  // namespace dpst
