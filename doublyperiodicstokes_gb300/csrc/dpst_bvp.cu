// Per-wavenumber Stokes BVP in FP64 (the no-wall Schur/KBPENTA solve of
// DPTools.cpp:81-345 plus the wall-correction coefficients of
// DPTools.cpp:590-877), and the k = 0 mode (Solvers.py:350-432, 482-516,
// 563-599).
//
// Work decomposition.  Every operator of the solve has real coefficients
// (the KBPENTA factors, the border columns, the BC rows, the integration
// matrices); real and imaginary parts couple only through the products with
// i kx and i ky.  A pair of adjacent lanes therefore owns one wavenumber:
// lane 2q the real part, lane 2q+1 the imaginary part, exchanging the few
// coupled values through shared memory, global scratch and warp shuffles.
// The penta / right-hand-side column of a lane (nz + 2 doubles) lives in
// shared memory laid out [row][lane], so every access is conflict-free; the
// pressure coefficients (nz doubles per lane, read back by the partner lane)
// live in an L2-resident global scratch laid out [row][lane of the grid];
// the pressure derivative is consumed as it is produced (the z velocity is
// solved first).  A CTA of 192 lanes solves 96 wavenumbers at a time and
// strides over all of them (persistent).  GB300 executes FP64 at 1/58 of its
// FP32 rate with the FP64 units split across the four SM sub-partitions, so
// the CTA is sized for six warps per SM and the per-wavenumber factors stream
// in through the read-only path ahead of the recurrences.
#include "dpst_internal.cuh"
#include "dpst_kdev.cuh"

#include <mutex>

namespace dpst {

constexpr int BVP_LANES = 192;  // 96 wavenumbers per CTA
constexpr int BVP_MODES = BVP_LANES / 2;

#define LDG(p) __ldg(p)

// The k-independent tables of the solve live in static shared memory at
// fixed offsets (nz <= BVP_NZMAX is checked at creation), so that the
// recurrences address them with immediates: the SIMat bands S0, SM2, SP2,
// the FIMat bands FM1, FP1, the SIMat bands / eta used by the velocity
// windows, and the Chebyshev derivative factors 2 j / H (nz + 1 entries).
constexpr int BVP_NZMAX = 128;
enum BvpTab { TB_S0, TB_SM2, TB_SP2, TB_FM1, TB_FP1, TB_S0E, TB_SM2E, TB_SP2E, TB_DH };
__shared__ double bvp_tab[TB_DH * BVP_NZMAX + BVP_NZMAX + 1];
#define TAB(t, j) bvp_tab[(t) * BVP_NZMAX + (j)]

// Column and pressure scratch of one lane of the solve.
struct BvpCtx {
  double *Xs;  // [(nz + 2)][BVP_LANES] penta / RHS columns in shared memory
  double *Xg;  // or this lane's column in global memory, row j at Xg[j * XGT]
  double *CPs;        // this lane's pressure coefficients, row j at CPs[j * GT]
  const double *CPo;  // the partner lane's
  int GT, XGT, tid;
};

// Load the tables (identical for every wavenumber) into shared memory.
// LANES threads per CTA, the first SL with their columns in shared memory
// ([nz + 2][SL]); the others (the hybrid kernel) keep theirs in xs_scratch,
// [nz + 2][(LANES - SL) x CTAs of the grid].
template <int LANES = BVP_LANES, int SL = BVP_LANES>
static __device__ __forceinline__ BvpCtx bvp_ctx(const KsArgs &a, double *bvp_sm, double *cp_scratch,
                                                 double *xs_scratch = nullptr) {
  const int nz = a.nz, tid = threadIdx.x;
  BvpCtx c;
  c.Xs = bvp_sm;
  c.XGT = gridDim.x * (LANES - SL);
  c.Xg = (LANES > SL && tid >= SL) ? xs_scratch + blockIdx.x * (LANES - SL) + (tid - SL) : nullptr;
  const double inv_eta = 1.0 / a.eta;
  for (int t = tid; t < nz; t += LANES) {
    TAB(TB_S0, t) = a.s0[t];
    TAB(TB_SM2, t) = a.sm2[t];
    TAB(TB_SP2, t) = a.sp2[t];
    TAB(TB_FM1, t) = a.fm1[t];
    TAB(TB_FP1, t) = a.fp1[t];
    TAB(TB_S0E, t) = a.s0[t] * inv_eta;
    TAB(TB_SM2E, t) = a.sm2[t] * inv_eta;
    TAB(TB_SP2E, t) = a.sp2[t] * inv_eta;
  }
  for (int t = tid; t <= nz; t += LANES) TAB(TB_DH, t) = (double)(2 * t) / a.H;
  // pressure coefficients of every lane of the grid, [nz][lanes of the grid]
  // in global memory (L2 resident: a few tens of MB)
  c.GT = gridDim.x * LANES;
  c.CPs = cp_scratch + blockIdx.x * LANES + tid;
  c.CPo = cp_scratch + blockIdx.x * LANES + (tid ^ 1);
  c.tid = tid;
  return c;
}

// The solve of one wavenumber i for this lane (lane 2q: real part, 2q + 1:
// imaginary part); both lanes of a pair run it together (shuffles).  The
// velocity solves run on the right-hand sides times eta (the 1/eta of
// DPTools.cpp:197-216 moves into the window's SIMat bands and the BC values
// are scaled by eta), which saves a multiply per row.  WALLS = false (open
// domain) skips the wall values that only the corrections use.
template <typename R, bool WALLS, int PF_F, int PF_B, bool GCOL = false, int SL = BVP_LANES, int PF_W = 4>
static __device__ __forceinline__ void bvp_mode(const KsArgs &a, R *__restrict__ spec, double2 *__restrict__ corr,
                                                int i, bool store, const BvpCtx &ctx) {
  const int nz = a.nz;
  const int nk = (int)a.nk;  // nz * nk * 4 < 2^31 is checked at creation
  constexpr int T = BVP_LANES;
  const int tid = ctx.tid, part = tid & 1;
  double *Xs = ctx.Xs;
  double *__restrict__ Xg = ctx.Xg;
  const int XGT = ctx.XGT;
  double *__restrict__ CPs = ctx.CPs;
  const double *__restrict__ CPo = ctx.CPo;
  const int GT = ctx.GT;
#define XS(j) (*(GCOL ? Xg + (j) * XGT : Xs + (j) * SL + tid))
  const double sp = part ? 1.0 : -1.0;  // (i a)_part = sp * a_(other part)
  const int rs = 2 * nk;  // spectrum row stride (R elements)
  // component d, row j, part pp of the spectrum: spec[(d nz + j) rs + 2 i + pp]
  R *__restrict__ sp_own = spec + 2 * i + part;
  const R *__restrict__ sp_oth = spec + 2 * i + (part ^ 1);
  const int ix = i % a.nxh, iy = i / a.nxh;
  const double kx = __ldg(a.kvx + ix), ky = __ldg(a.kvy + iy);
  const double Dx = ((a.nx % 2) == 0 && ix == a.nx / 2) ? 0.0 : kx;
  const double Dy = ((a.ny % 2) == 0 && iy == a.ny / 2) ? 0.0 : ky;
  const double K = sqrt(kx * kx + ky * ky);
  const double G00 = __ldg(a.ginv + i), G10 = __ldg(a.ginv + nk + i);
  const double G01 = __ldg(a.ginv + 2 * nk + i), G11 = __ldg(a.ginv + 3 * nk + i);
  const double *__restrict__ mf0 = a.mf + i;
  const double2 *__restrict__ bk0 = reinterpret_cast<const double2 *>(a.bk) + 2 * i;
  const double *__restrict__ ab0 = a.ab + i;

  // pressure RHS Dx f + Dy g + d/dz h (DPTools.cpp:134-195), backward in j;
  // the last row (df = 0) and row 0 (halved derivative) are peeled
  {
    const R *f0o = sp_oth + (nz - 1) * rs, *f1o = f0o + nz * rs;
    const R *f2s = sp_own + (2 * nz + nz - 1) * rs;
    const double dxs = Dx * sp, dys = Dy * sp;
    XS(nz - 1) = (dxs * ld_fp64(f0o) + dys * ld_fp64(f1o)) + 0.0;
    double fzn = ld_fp64(f2s);
    double dfp1 = 0.0, dfp2 = 0.0;
    f0o -= rs;
    f1o -= rs;
    f2s -= rs;
#pragma unroll 4
    for (int j = nz - 2; j >= 1; --j) {
      const double df = dfp2 + TAB(TB_DH, j + 1) * fzn;
      fzn = ld_fp64(f2s);
      XS(j) = (dxs * ld_fp64(f0o) + dys * ld_fp64(f1o)) + df;
      dfp2 = dfp1;
      dfp1 = df;
      f0o -= rs;
      f1o -= rs;
      f2s -= rs;
    }
    const double df0 = dfp2 + TAB(TB_DH, 1) * fzn;
    XS(0) = (dxs * ld_fp64(f0o) + dys * ld_fp64(f1o)) + 0.5 * df0;
  }
  // KBPENTA sweeps (LinearSolvers.h:106-141) in place on XS with the
  // border dots y = C x accumulated during the back sweep.  Rows 0, 1 of
  // mf and the dp2 of the last two rows are zero, so both loops are uniform.
  // The factor streams are read PF_F / PF_B rows ahead of the recurrence
  // through register rings (prefetch indices clamped into the table; the
  // depths follow the kernel's register budget, BvpRings), and
  // the border dots accumulate in two partial sums (rows of even and odd
  // distance from the last), which halves their FP64 dependency chains.
  auto penta = [&](double &y0, double &y1) {
    double xm2 = 0.0, xm1 = 0.0;
    double pm[PF_F];
#pragma unroll
    for (int k = 0; k < PF_F; ++k) pm[k] = __ldg(mf0 + min(k, nz - 1) * nk);
    int j = 0;
    for (; j + PF_F <= nz; j += PF_F) {
#pragma unroll
      for (int k = 0; k < PF_F; ++k) {
        const double m = pm[k];
        pm[k] = __ldg(mf0 + min(j + PF_F + k, nz - 1) * nk);
        const double v = XS(j + k) - m * xm2;
        XS(j + k) = v;
        xm2 = xm1;
        xm1 = v;
      }
    }
#pragma unroll
    for (int k = 0; k < PF_F - 1; ++k) {
      if (j + k < nz) {  // warp-uniform tail
        const double v = XS(j + k) - pm[k] * xm2;
        XS(j + k) = v;
        xm2 = xm1;
        xm1 = v;
      }
    }
    double xp2 = 0.0, xp1 = 0.0;
    double ya0 = 0.0, ya1 = 0.0, yb0 = 0.0, yb1 = 0.0;
    double2 pi[PF_B], pc[PF_B];
#pragma unroll
    for (int k = 0; k < PF_B; ++k) {
      const double2 *b = bk0 + max(nz - 1 - k, 0) * rs;
      pi[k] = __ldg(b);
      pc[k] = __ldg(b + 1);
    }
    j = nz - 1;
    for (; j - PF_B + 1 >= 0; j -= PF_B) {
#pragma unroll
      for (int k = 0; k < PF_B; ++k) {
        const double2 ibd = pi[k], cc = pc[k];
        const double2 *b = bk0 + max(j - k - PF_B, 0) * rs;
        pi[k] = __ldg(b);
        pc[k] = __ldg(b + 1);
        const double v = ibd.x * (XS(j - k) - ibd.y * xp2);
        XS(j - k) = v;
        if (k & 1) {
          yb0 += cc.x * v;
          yb1 += cc.y * v;
        } else {
          ya0 += cc.x * v;
          ya1 += cc.y * v;
        }
        xp2 = xp1;
        xp1 = v;
      }
    }
#pragma unroll
    for (int k = 0; k < PF_B - 1; ++k) {
      if (j - k >= 0) {  // warp-uniform tail
        const double v = pi[k].x * (XS(j - k) - pi[k].y * xp2);
        XS(j - k) = v;
        if (k & 1) {
          yb0 += pc[k].x * v;
          yb1 += pc[k].y * v;
        } else {
          ya0 += pc[k].x * v;
          ya1 += pc[k].y * v;
        }
        xp2 = xp1;
        xp1 = v;
      }
    }
    y0 = ya0 + yb0;
    y1 = ya1 + yb1;
  };
  // Window pass over the border-corrected solution x_m = X_m - (A^{-1}B g)_m
  // (x_nz = g0, x_nz+1 = g1): row m sees x_{m-2} .. x_{m+2} and applies
  // the SIMat / FIMat bands.  Rows 0, 1 (border columns) and nz-2, nz-1
  // (x_{m+2} is g) are peeled; the main loop takes rows in (even, odd)
  // pairs so that the parity of the border column is static, with the
  // A^{-1}B column read PF_W pairs ahead through a register ring.
  auto window = [&](double g0, double g1, auto &&row) {
    double xm2 = 0.0, xm1 = 0.0;
    double x0 = XS(0) - __ldg(ab0) * g0, x1 = XS(1) - __ldg(ab0 + nk) * g1;
    const double ab2 = __ldg(ab0 + min(2, nz - 1) * nk), ab3 = __ldg(ab0 + min(3, nz - 1) * nk);
    // ring slot q holds the A^{-1}B rows of main-loop pair q: 4 + 2q, 5 + 2q
    double pa[PF_W][2];
#pragma unroll
    for (int q = 0; q < PF_W; ++q) {
      pa[q][0] = __ldg(ab0 + min(4 + 2 * q, nz - 1) * nk);
      pa[q][1] = __ldg(ab0 + min(5 + 2 * q, nz - 1) * nk);
    }
    auto step = [&](int m, double x2, bool odd, int head) {
      row(m, xm2, xm1, x0, x1, x2, odd, head);
      xm2 = xm1;
      xm1 = x0;
      x0 = x1;
      x1 = x2;
    };
    step(0, XS(2) - ab2 * g0, false, 1);
    step(1, XS(3) - ab3 * g1, true, 2);
    int m = 2;
    for (; m + 2 * PF_W - 1 <= nz - 3; m += 2 * PF_W) {
#pragma unroll
      for (int q = 0; q < PF_W; ++q) {
        const int mm = m + 2 * q;
        const double a0 = pa[q][0], a1 = pa[q][1];
        pa[q][0] = __ldg(ab0 + min(mm + 2 + 2 * PF_W, nz - 1) * nk);
        pa[q][1] = __ldg(ab0 + min(mm + 3 + 2 * PF_W, nz - 1) * nk);
        step(mm, XS(mm + 2) - a0 * g0, false, 0);
        step(mm + 1, XS(mm + 3) - a1 * g1, true, 0);
      }
    }
#pragma unroll
    for (int q = 0; q < PF_W - 1; ++q) {
      if (m + 1 <= nz - 3) {  // warp-uniform tail pairs
        step(m, XS(m + 2) - pa[q][0] * g0, false, 0);
        step(m + 1, XS(m + 3) - pa[q][1] * g1, true, 0);
        m += 2;
      }
    }
    if (m <= nz - 3) {  // odd nz: one more even row
      step(m, XS(m + 2) - __ldg(ab0 + (m + 2) * nk) * g0, false, 0);
      ++m;
    }
    step(nz - 2, g0, ((nz - 2) & 1) != 0, 0);
    step(nz - 1, g1, ((nz - 1) & 1) != 0, 0);
  };

  // ---- pressure: Schur solve, cp = S [x; g] (kept), dp = F [x; g] used at
  // once for the z-velocity RHS, which overwrites XS behind the window
  double se = 0.0, so = 0.0;  // sums of the even and odd coefficients
  {
    double y0, y1;
    penta(y0, y1);
    const double g0 = G00 * y0 + G01 * y1, g1 = G10 * y0 + G11 * y1;
    const R *f2s = sp_own + 2 * nz * rs;
    double *cpw = CPs;
    window(g0, g1, [&](int m, double xm2, double xm1, double x0, double x1, double x2, bool odd, int head) {
      double c = TAB(TB_S0, m) * x0;
      if (head == 0) c = TAB(TB_SM2, m) * xm2 + c;
      c = c + TAB(TB_SP2, m) * x2;
      if (head == 1) c += a.se0 * g0;
      if (head == 2) c += a.se1 * g1;
      double dpv = TAB(TB_FP1, m) * x1;
      if (head != 1) dpv = TAB(TB_FM1, m) * xm1 + dpv;
      if (head == 1) dpv += a.fe * g1;
      *cpw = c;
      if (odd) so += c;
      else se += c;
      XS(m) = dpv - ld_fp64(f2s);  // eta x z-velocity RHS (DPTools.cpp:214)
      f2s += rs;
      cpw += GT;
    });
  }
  // velocity BC right-hand sides (DPTools.cpp:218-234): the pressure at
  // z = +-1 is the sum and the alternating sum of its coefficients
  const double ssum = se + so, asum = se - so;
  const double ssum_o = __shfl_xor_sync(0xffffffffu, ssum, 1);
  const double asum_o = __shfl_xor_sync(0xffffffffu, asum, 1);
  // eta x the BC values: 1/(2 eta K) -> 1/(2 K), 1/(2 eta) -> 1/2
  const double ifac = 0.5 / K, ifac1 = 0.5;
  double bc[6];
  bc[0] = -ifac * ((Dx * sp) * ssum_o);
  bc[1] = ifac * ((Dx * sp) * asum_o);
  bc[2] = -ifac * ((Dy * sp) * ssum_o);
  bc[3] = ifac * ((Dy * sp) * asum_o);
  bc[4] = ifac1 * ssum;
  bc[5] = ifac1 * asum;
  __syncwarp();  // the partner's pressure coefficients are read below

  // ---- velocity: three Schur solves (DPTools.cpp:197-216, 287-345); z first
  const double inv_eta_w = 1.0 / a.eta;
  double wt[3], wb[3];
#pragma unroll
  for (int cc = 0; cc < 3; ++cc) {
    const int c = (cc + 2) % 3;  // 2, 0, 1
    if (c != 2) {
      const double Dc = (c == 0 ? Dx : Dy) * sp;
      const R *fs = sp_own + c * nz * rs;
      const double *cpo = CPo;
#pragma unroll 4
      for (int j = 0; j < nz; ++j) {
        XS(j) = Dc * *cpo - ld_fp64(fs);
        fs += rs;
        cpo += GT;
      }
    }
    double y0, y1;
    penta(y0, y1);
    const double r0 = y0 - bc[2 * c], r1 = y1 - bc[2 * c + 1];
    const double g0 = G00 * r0 + G01 * r1, g1 = G10 * r0 + G11 * r1;
    double ue = 0.0, uo = 0.0;  // sums of the even and odd coefficients
    R *us = sp_own + c * nz * rs;
    const double se0e = a.se0 * inv_eta_w, se1e = a.se1 * inv_eta_w;
    window(g0, g1, [&](int m, double xm2, double xm1, double x0, double x1, double x2, bool odd, int head) {
      double u = TAB(TB_S0E, m) * x0;
      if (head == 0) u = TAB(TB_SM2E, m) * xm2 + u;
      u = u + TAB(TB_SP2E, m) * x2;
      if (head == 1) u += se0e * g0;
      if (head == 2) u += se1e * g1;
      if (store) *us = to_r<R>(u);
      if (WALLS) {
        if (odd) uo += u;
        else ue += u;
      }
      us += rs;
    });
    wt[c] = ue + uo;  // u(z = 1), u(z = -1)
    wb[c] = ue - uo;
  }
  if (!WALLS) {
    __syncwarp();  // XS/CPS reuse in the next tile
    return;
  }
  // wall-correction coefficients (evalTheta at z = 0 and z = Lz)
  double wto[3], wbo[3];
  for (int c = 0; c < 3; ++c) {
    wto[c] = __shfl_xor_sync(0xffffffffu, wt[c], 1);
    wbo[c] = __shfl_xor_sync(0xffffffffu, wb[c], 1);
  }
  __syncwarp();  // XS/CPS reuse in the next tile
  if (!store) return;
  double *crd = reinterpret_cast<double *>(corr + i * 16);
  if (a.mode == 1) {
    for (int c = 0; c < 3; ++c) crd[2 * c + part] = -wb[c];
    if (a.corrf)
      for (int c = 0; c < 3; ++c) reinterpret_cast<float *>(a.corrf + i * 16)[2 * c + part] = (float)(-wb[c]);
  } else if (a.mode == 2 && part == 0) {
    double2 fb[3], ft[3], cf[8];
    for (int c = 0; c < 3; ++c) {
      fb[c] = make_double2(-wb[c], -wbo[c]);
      ft[c] = make_double2(-wt[c], -wto[c]);
    }
    slit_coeffs(kx, ky, a.Lz, a.eta, fb, ft, cf);
    for (int r = 0; r < 8; ++r) corr[i * 16 + r] = cf[r];
    if (a.corrf)
      for (int r = 0; r < 8; ++r) a.corrf[i * 16 + r] = make_float2((float)cf[r].x, (float)cf[r].y);
    double kxp, kyp;
    if (!mode_is_hermitian(a, ix, iy, kx, ky, kxp, kyp)) {
      for (int c = 0; c < 3; ++c) {
        fb[c] = cconj(fb[c]);
        ft[c] = cconj(ft[c]);
      }
      slit_coeffs(kxp, kyp, a.Lz, a.eta, fb, ft, cf);
      for (int r = 0; r < 8; ++r) corr[i * 16 + 8 + r] = cf[r];
      if (a.corrf)
        for (int r = 0; r < 8; ++r) a.corrf[i * 16 + 8 + r] = make_float2((float)cf[r].x, (float)cf[r].y);
    }
  }
#undef XS
}

// Factor-ring depths (forward sweep, back sweep) of the kernel compiled for
// MINB CTAs per SM: one CTA (large nz, shared memory allows no more) has the
// whole register file and reads 16 / 8 rows ahead; two CTAs (small nz) keep
// under half of it with 8 / 2 rows.
template <int MINB>
struct BvpRings {
  static constexpr int F = MINB == 1 ? 16 : 8;
  static constexpr int B = MINB == 1 ? 8 : 2;
};

// Two CTAs per SM when their shared memory fits (228 KB per SM, 1 KB of it
// reserved per CTA).
static bool bvp_two_per_sm(int nz) {
  const size_t per_cta = sizeof(double) * ((size_t)(nz + 2) * BVP_LANES + TB_DH * BVP_NZMAX + BVP_NZMAX + 1) + 1024;
  return 2 * per_cta <= (size_t)228 * 1024;
}

// Work split: CTA b owns the contiguous modes [b per_cta, (b+1) per_cta),
// per_cta a multiple of 16 (the modes of one warp), and walks them 96 at a
// time; a warp whose 16 modes lie past the CTA's range skips the tile, so
// the last, partial tile of every CTA costs only the warps it needs.
template <typename R, int MINB>
__global__ void __launch_bounds__(BVP_LANES, MINB) k_bvp_pairs(KsArgs a, R *__restrict__ spec,
                                                            double2 *__restrict__ corr,
                                                            double *__restrict__ cp_scratch, int per_cta) {
  extern __shared__ double bvp_sm[];
  const BvpCtx ctx = bvp_ctx(a, bvp_sm, cp_scratch);
  __syncthreads();
  const int nk = (int)a.nk;
  const int tid = threadIdx.x, q = tid >> 1;
  const int cta_begin = blockIdx.x * per_cta;
  const int cta_end = min(cta_begin + per_cta, nk);
  for (int base = cta_begin; base < cta_end; base += BVP_MODES) {
    if (base + (tid >> 5) * 16 >= cta_end) continue;  // warp-uniform
    const int i_raw = base + q;
    const int i = i_raw < cta_end ? i_raw : cta_end - 1;
    const bool store = (i_raw < cta_end) && (i != 0);  // mode 0: k_bvp_k0
    if (a.mode != 0) bvp_mode<R, true, BvpRings<MINB>::F, BvpRings<MINB>::B>(a, spec, corr, i, store, ctx);
    else bvp_mode<R, false, BvpRings<MINB>::F, BvpRings<MINB>::B>(a, spec, corr, i, store, ctx);
  }
}

// Hybrid kernel: BVP_HYB_THREADS lanes per CTA, one CTA per SM; the first SL
// keep their penta columns in shared memory (SL = 2 BVP_LANES when those
// fit, else BVP_LANES), the others in an L2-resident global scratch.  The
// solve's limit is the factor loads in flight per SM, which grows with the
// warps (24 here: 3.2 ms on c2 against 4.4 ms with the 6 warps whose
// columns fit in shared memory), so every factor ring is one row deep and
// the register budget (85 per thread) goes to warps.  CTA b owns the units
// of 16 modes [b per_cta, (b+1) per_cta) and its warps take them from a
// shared-memory counter, so shared- and global-column warps share the work by
// their own speed.  Problems with fewer units than warps keep the plain
// kernel (deep factor rings, every SM busy).
constexpr int BVP_HYB_THREADS = 768;
template <typename R, int SL>
__global__ void __launch_bounds__(BVP_HYB_THREADS, 1) k_bvp_hybrid(KsArgs a, R *__restrict__ spec,
                                                                   double2 *__restrict__ corr,
                                                                   double *__restrict__ cp_scratch,
                                                                   double *__restrict__ xs_scratch, int per_cta) {
  extern __shared__ double bvp_sm[];
  __shared__ int next_unit;
  const BvpCtx ctx = bvp_ctx<BVP_HYB_THREADS, SL>(a, bvp_sm, cp_scratch, xs_scratch);
  if (threadIdx.x == 0) next_unit = blockIdx.x * per_cta;
  __syncthreads();
  const int nk = (int)a.nk;
  const int units = (nk + 15) / 16;
  const int u_end = min((int)(blockIdx.x + 1) * per_cta, units);
  const int tid = threadIdx.x, lane = tid & 31;
  const bool gcol = tid >= SL;  // warp-uniform
  for (;;) {
    int u = 0;
    if (lane == 0) u = atomicAdd(&next_unit, 1);
    u = __shfl_sync(0xffffffffu, u, 0);
    if (u >= u_end) break;
    const int base = u * 16;
    const int i_raw = base + (lane >> 1);
    const int i = i_raw < nk ? i_raw : nk - 1;
    const bool store = (i_raw < nk) && (i != 0);  // mode 0: k_bvp_k0
    if (gcol) {
      if (a.mode != 0) bvp_mode<R, true, 1, 1, true, SL, 1>(a, spec, corr, i, store, ctx);
      else bvp_mode<R, false, 1, 1, true, SL, 1>(a, spec, corr, i, store, ctx);
    } else {
      if (a.mode != 0) bvp_mode<R, true, 1, 1, false, SL, 1>(a, spec, corr, i, store, ctx);
      else bvp_mode<R, false, 1, 1, false, SL, 1>(a, spec, corr, i, store, ctx);
    }
  }
}

// Batched form of the hybrid kernel: units of 16 consecutive modes of the
// concatenated systems (a lane finds its system by binary search).
template <typename R, int SL>
__global__ void __launch_bounds__(BVP_HYB_THREADS, 1) k_bvp_hybrid_b(const SysK<R> *__restrict__ sys, int S,
                                                                     const int64_t *__restrict__ mprefix,
                                                                     double *__restrict__ cp_scratch,
                                                                     double *__restrict__ xs_scratch, int per_cta) {
  extern __shared__ double bvp_sm[];
  __shared__ int next_unit;
  const BvpCtx ctx = bvp_ctx<BVP_HYB_THREADS, SL>(sys[0].ks, bvp_sm, cp_scratch, xs_scratch);
  if (threadIdx.x == 0) next_unit = blockIdx.x * per_cta;
  __syncthreads();
  const int64_t K = mprefix[S];
  const int units = (int)((K + 15) / 16);
  const int u_end = min((int)(blockIdx.x + 1) * per_cta, units);
  const int tid = threadIdx.x, lane = tid & 31;
  const bool gcol = tid >= SL;  // warp-uniform
  for (;;) {
    int u = 0;
    if (lane == 0) u = atomicAdd(&next_unit, 1);
    u = __shfl_sync(0xffffffffu, u, 0);
    if (u >= u_end) break;
    const int64_t g_raw = (int64_t)u * 16 + (lane >> 1);
    const int64_t g = g_raw < K ? g_raw : K - 1;
    const int s = find_sys(mprefix, S, g);
    const SysK<R> &y = sys[s];
    const int i = (int)(g - mprefix[s]);
    const bool store = (g_raw < K) && (i != 0);
    if (gcol) {
      if (y.ks.mode != 0) bvp_mode<R, true, 1, 1, true, SL, 1>(y.ks, y.spec, y.corr, i, store, ctx);
      else bvp_mode<R, false, 1, 1, true, SL, 1>(y.ks, y.spec, y.corr, i, store, ctx);
    } else {
      if (y.ks.mode != 0) bvp_mode<R, true, 1, 1, false, SL, 1>(y.ks, y.spec, y.corr, i, store, ctx);
      else bvp_mode<R, false, 1, 1, false, SL, 1>(y.ks, y.spec, y.corr, i, store, ctx);
    }
  }
}

// Shared-memory lanes of the hybrid kernel for nz: 2 BVP_LANES when their
// columns and the tables fit in one CTA's shared memory, else BVP_LANES.
static int hybrid_smem_lanes(int nz) {
  const size_t tabs = sizeof(double) * (TB_DH * BVP_NZMAX + BVP_NZMAX + 1) + 64;  // + static slack
  return sizeof(double) * (size_t)(nz + 2) * 2 * BVP_LANES + tabs <= (size_t)227 * 1024 ? 2 * BVP_LANES
                                                                                       : BVP_LANES;
}

// Batched systems: global mode g of [0, mprefix[S]) belongs to system s with
// mprefix[s] <= g < mprefix[s+1]; every system has the same nz and H (the
// shared-memory tables), its own factors, spectrum and corrections.
template <typename R, int MINB>
__global__ void __launch_bounds__(BVP_LANES, MINB) k_bvp_pairs_b(const SysK<R> *__restrict__ sys, int S,
                                                              const int64_t *__restrict__ mprefix,
                                                              double *__restrict__ cp_scratch, int per_cta) {
  extern __shared__ double bvp_sm[];
  const BvpCtx ctx = bvp_ctx(sys[0].ks, bvp_sm, cp_scratch);
  __syncthreads();
  const int64_t K = mprefix[S];
  const int tid = threadIdx.x, q = tid >> 1;
  const int64_t cta_begin = (int64_t)blockIdx.x * per_cta;
  const int64_t cta_end = min(cta_begin + per_cta, K);
  for (int64_t base = cta_begin; base < cta_end; base += BVP_MODES) {
    if (base + (tid >> 5) * 16 >= cta_end) continue;  // warp-uniform
    const int64_t g_raw = base + q;
    const int64_t g = g_raw < cta_end ? g_raw : cta_end - 1;
    const int s = find_sys(mprefix, S, g);
    const SysK<R> &y = sys[s];
    const int i = (int)(g - mprefix[s]);
    const bool store = (g_raw < cta_end) && (i != 0);
    if (y.ks.mode != 0) bvp_mode<R, true, BvpRings<MINB>::F, BvpRings<MINB>::B>(y.ks, y.spec, y.corr, i, store, ctx);
    else bvp_mode<R, false, BvpRings<MINB>::F, BvpRings<MINB>::B>(y.ks, y.spec, y.corr, i, store, ctx);
  }
}

// k = 0: open domain -> zero; walls -> u, v from the k = 0 BVP with the
// reference's BC rows (u' = 0 or u = 0 at the top, u = 0 at the bottom), w = 0.
// One CTA of 2 x 128 threads: thread (part, j) owns row j of the real or
// imaginary part; the two BC dots are block reductions.
constexpr int K0_ROWS = 128;
template <typename R>
static __device__ __forceinline__ void bvp_k0_body(const KsArgs &a, R *__restrict__ spec) {
  __shared__ double X[2][K0_ROWS + 2];
  __shared__ double red[2][2][K0_ROWS / 32];
  const int part = threadIdx.x / K0_ROWS, j = threadIdx.x % K0_ROWS;
  const int nz = a.nz;
  const int64_t nk = a.nk;
  auto at = [&](int d, int r) -> R & { return spec[(((int64_t)d * nz + r) * nk) * 2 + part]; };
  if (a.mode == 0) {
    if (j < nz)
      for (int d = 0; d < 3; ++d) at(d, j) = (R)0;
    return;
  }
  const double inv_eta = 1.0 / a.eta;
  const int lane = j & 31, wid = j >> 5;
  for (int c = 0; c < 2; ++c) {
    const double r = (j < nz) ? -inv_eta * (double)at(c, j) : 0.0;
    X[part][j] = r;
    double y0 = (j < nz) ? a.k0c0[j] * r : 0.0, y1 = (j < nz) ? a.k0c1[j] * r : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      y0 += __shfl_xor_sync(0xffffffffu, y0, o);
      y1 += __shfl_xor_sync(0xffffffffu, y1, o);
    }
    if (lane == 0) {
      red[part][0][wid] = y0;
      red[part][1][wid] = y1;
    }
    __syncthreads();
    if (j == 0) {
      double s0 = 0.0, s1 = 0.0;
      for (int q = 0; q < K0_ROWS / 32; ++q) {
        s0 += red[part][0][q];
        s1 += red[part][1][q];
      }
      X[part][nz] = a.k0gi[0] * s0 + a.k0gi[1] * s1;
      X[part][nz + 1] = a.k0gi[2] * s0 + a.k0gi[3] * s1;
    }
    __syncthreads();
    if (j < nz) {
      double u = a.s0[j] * X[part][j];
      if (j >= 2) u = a.sm2[j] * X[part][j - 2] + u;
      u = u + a.sp2[j] * X[part][j + 2];
      if (j == 0) u += a.se0 * X[part][nz];
      if (j == 1) u += a.se1 * X[part][nz + 1];
      at(c, j) = (R)u;
    }
    __syncthreads();
  }
  if (j < nz) at(2, j) = (R)0;
}

template <typename R>
__global__ void __launch_bounds__(2 * K0_ROWS) k_bvp_k0(KsArgs a, R *__restrict__ spec) {
  bvp_k0_body<R>(a, spec);
}

// the k = 0 mode alone (after the double-float solve of the other modes)
template <typename R>
cudaError_t launch_bvp_k0(const KsArgs &a, R *spec, cudaStream_t s) {
  k_bvp_k0<R><<<1, 2 * K0_ROWS, 0, s>>>(a, spec);
  return cudaGetLastError();
}
template cudaError_t launch_bvp_k0<float>(const KsArgs &, float *, cudaStream_t);
template cudaError_t launch_bvp_k0<double>(const KsArgs &, double *, cudaStream_t);

template <typename R>
__global__ void __launch_bounds__(2 * K0_ROWS) k_bvp_k0_b(const SysK<R> *__restrict__ sys);
// the k = 0 mode of every system of a batch (after the double-float solve)
template <typename R>
cudaError_t launch_bvp_k0_b(const SysK<R> *sys, int S, cudaStream_t s) {
  k_bvp_k0_b<R><<<S, 2 * K0_ROWS, 0, s>>>(sys);
  return cudaGetLastError();
}

// Batched: one CTA per system.
template <typename R>
__global__ void __launch_bounds__(2 * K0_ROWS) k_bvp_k0_b(const SysK<R> *__restrict__ sys) {
  bvp_k0_body<R>(sys[blockIdx.x].ks, sys[blockIdx.x].spec);
}

// Grid of the persistent BVP kernel and the bytes of its pressure scratch.
template <typename R, int MINB>
static cudaError_t bvp_plan_v(const KsArgs &a, int nsm, int64_t *grid, size_t *scratch_bytes) {
  const size_t smem = sizeof(double) * ((size_t)(a.nz + 2) * BVP_LANES);
  cudaError_t err = cudaFuncSetAttribute(k_bvp_pairs<R, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  int per_sm = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bvp_pairs<R, MINB>, BVP_LANES, smem);
  if (err != cudaSuccess) return err;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  if ((int64_t)a.nz * a.nk * 4 >= ((int64_t)1 << 31)) return cudaErrorInvalidValue;
  int64_t g = (int64_t)nsm * per_sm;
  const int64_t warps_of_modes = (a.nk + 15) / 16;
  if (g > warps_of_modes) g = warps_of_modes;
  *grid = g;
  *scratch_bytes = sizeof(double) * (size_t)a.nz * (size_t)g * BVP_LANES;
  return cudaSuccess;
}

// Scratch of the hybrid kernel: pressure coefficients of all its lanes, the
// global-memory columns, the work counter.
static size_t hybrid_cp_doubles(int nz, int64_t grid) { return (size_t)nz * grid * BVP_HYB_THREADS; }
static size_t hybrid_xs_doubles(int nz, int64_t grid) {
  return (size_t)(nz + 2) * grid * (BVP_HYB_THREADS - hybrid_smem_lanes(nz));
}

template <typename R, int SL>
static cudaError_t hybrid_setup(size_t smem) {
  return cudaFuncSetAttribute(k_bvp_hybrid<R, SL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

// The planned grid and scratch serve both the hybrid kernel (ordinary calls)
// and the plain one (the allocation-free entry point).
template <typename R>
cudaError_t bvp_plan(const KsArgs &a, int nsm, int64_t *grid, size_t *scratch_bytes) {
  cudaError_t err = bvp_two_per_sm(a.nz) ? bvp_plan_v<R, 2>(a, nsm, grid, scratch_bytes)
                                         : bvp_plan_v<R, 1>(a, nsm, grid, scratch_bytes);
  if (err != cudaSuccess) return err;
  if ((a.nk + 15) / 16 < (int64_t)nsm * (BVP_HYB_THREADS / 32)) return cudaSuccess;  // plain kernel only
  const int sl = hybrid_smem_lanes(a.nz);
  const size_t smem = sizeof(double) * ((size_t)(a.nz + 2) * sl);
  err = sl == BVP_LANES ? hybrid_setup<R, BVP_LANES>(smem) : hybrid_setup<R, 2 * BVP_LANES>(smem);
  if (err != cudaSuccess) return err;
  int per_sm = 0;
  err = sl == BVP_LANES
            ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bvp_hybrid<R, BVP_LANES>, BVP_HYB_THREADS, smem)
            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bvp_hybrid<R, 2 * BVP_LANES>, BVP_HYB_THREADS,
                                                            smem);
  if (err != cudaSuccess) return err;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const int64_t hgrid = std::min<int64_t>(nsm, *grid);
  const size_t hy = sizeof(double) * (hybrid_cp_doubles(a.nz, hgrid) + hybrid_xs_doubles(a.nz, hgrid));
  if (hy > *scratch_bytes) *scratch_bytes = hy;
  return cudaSuccess;
}

// Batched solve: grid and scratch for K modes in total with a shared nz.
template <typename R, int MINB>
static cudaError_t bvp_plan_b_v(int nz, int64_t K, int nsm, int64_t *grid, size_t *scratch_bytes) {
  const size_t smem = sizeof(double) * ((size_t)(nz + 2) * BVP_LANES);
  cudaError_t err = cudaFuncSetAttribute(k_bvp_pairs_b<R, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  int per_sm = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bvp_pairs_b<R, MINB>, BVP_LANES, smem);
  if (err != cudaSuccess) return err;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int64_t g = (int64_t)nsm * per_sm;
  const int64_t warps_of_modes = (K + 15) / 16;
  if (g > warps_of_modes) g = warps_of_modes;
  if (g < 1) g = 1;
  *grid = g;
  *scratch_bytes = sizeof(double) * (size_t)nz * (size_t)g * BVP_LANES;
  return cudaSuccess;
}

template <typename R>
cudaError_t bvp_plan_b(int nz, int64_t K, int nsm, int64_t *grid, size_t *scratch_bytes) {
  cudaError_t err = bvp_two_per_sm(nz) ? bvp_plan_b_v<R, 2>(nz, K, nsm, grid, scratch_bytes)
                                       : bvp_plan_b_v<R, 1>(nz, K, nsm, grid, scratch_bytes);
  if (err != cudaSuccess) return err;
  if ((K + 15) / 16 < (int64_t)nsm * (BVP_HYB_THREADS / 32)) return cudaSuccess;  // plain kernel only
  const int sl = hybrid_smem_lanes(nz);
  const size_t smem = sizeof(double) * ((size_t)(nz + 2) * sl);
  err = sl == BVP_LANES
            ? cudaFuncSetAttribute(k_bvp_hybrid_b<R, BVP_LANES>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
            : cudaFuncSetAttribute(k_bvp_hybrid_b<R, 2 * BVP_LANES>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem);
  if (err != cudaSuccess) return err;
  const int64_t hgrid = std::min<int64_t>(nsm, *grid);
  const size_t hy = sizeof(double) * (hybrid_cp_doubles(nz, hgrid) + hybrid_xs_doubles(nz, hgrid));
  if (hy > *scratch_bytes) *scratch_bytes = hy;
  return cudaSuccess;
}

template <typename R>
cudaError_t launch_bvp_b(const SysK<R> *sys, int S, const int64_t *mprefix, int64_t K, int nz, double *scratch,
                         int64_t grid, cudaStream_t s) {
  const size_t smem = sizeof(double) * ((size_t)(nz + 2) * BVP_LANES);
  int nsm = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if ((K + 15) / 16 >= (int64_t)nsm * (BVP_HYB_THREADS / 32)) {
    const int64_t hgrid = std::min<int64_t>(nsm, grid);
    const int sl = hybrid_smem_lanes(nz);
    const size_t hsmem = sizeof(double) * ((size_t)(nz + 2) * sl);
    double *cp = scratch;
    double *xs = cp + hybrid_cp_doubles(nz, hgrid);
    const int64_t units = (K + 15) / 16;
    const int per_cta = (int)((units + hgrid - 1) / hgrid);
    if (sl == BVP_LANES)
      k_bvp_hybrid_b<R, BVP_LANES><<<(unsigned)hgrid, BVP_HYB_THREADS, hsmem, s>>>(sys, S, mprefix, cp, xs, per_cta);
    else
      k_bvp_hybrid_b<R, 2 * BVP_LANES><<<(unsigned)hgrid, BVP_HYB_THREADS, hsmem, s>>>(sys, S, mprefix, cp, xs,
                                                                                     per_cta);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    k_bvp_k0_b<R><<<S, 2 * K0_ROWS, 0, s>>>(sys);
    return cudaGetLastError();
  }
  const int64_t per = (K + grid - 1) / grid;
  const int per_cta = (int)((per + 15) / 16 * 16);
  if (bvp_two_per_sm(nz)) k_bvp_pairs_b<R, 2><<<(unsigned)grid, BVP_LANES, smem, s>>>(sys, S, mprefix, scratch, per_cta);
  else k_bvp_pairs_b<R, 1><<<(unsigned)grid, BVP_LANES, smem, s>>>(sys, S, mprefix, scratch, per_cta);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  k_bvp_k0_b<R><<<S, 2 * K0_ROWS, 0, s>>>(sys);
  return cudaGetLastError();
}

template cudaError_t bvp_plan_b<float>(int, int64_t, int, int64_t *, size_t *);
template cudaError_t bvp_plan_b<double>(int, int64_t, int, int64_t *, size_t *);
template cudaError_t launch_bvp_b<float>(const SysK<float> *, int, const int64_t *, int64_t, int, double *, int64_t,
                                         cudaStream_t);
template cudaError_t launch_bvp_b<double>(const SysK<double> *, int, const int64_t *, int64_t, int, double *,
                                          int64_t, cudaStream_t);

template <typename R>
cudaError_t launch_bvp(const KsArgs &a, R *spec, double2 *corr, double *scratch, int64_t grid,
                       cudaStream_t s, bool hybrid) {
  const size_t smem = sizeof(double) * ((size_t)(a.nz + 2) * BVP_LANES);
  int nsm = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  // the hybrid kernel when every warp of its grid gets at least one unit
  if (hybrid && (a.nk + 15) / 16 >= (int64_t)nsm * (BVP_HYB_THREADS / 32)) {
    const int64_t hgrid = std::min<int64_t>(nsm, grid);
    const int sl = hybrid_smem_lanes(a.nz);
    const size_t hsmem = sizeof(double) * ((size_t)(a.nz + 2) * sl);
    double *cp = scratch;
    double *xs = cp + hybrid_cp_doubles(a.nz, hgrid);
    const int64_t units = (a.nk + 15) / 16;
    const int per_cta = (int)((units + hgrid - 1) / hgrid);
    if (sl == BVP_LANES)
      k_bvp_hybrid<R, BVP_LANES><<<(unsigned)hgrid, BVP_HYB_THREADS, hsmem, s>>>(a, spec, corr, cp, xs, per_cta);
    else
      k_bvp_hybrid<R, 2 * BVP_LANES><<<(unsigned)hgrid, BVP_HYB_THREADS, hsmem, s>>>(a, spec, corr, cp, xs, per_cta);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    k_bvp_k0<R><<<1, 2 * K0_ROWS, 0, s>>>(a, spec);
    return cudaGetLastError();
  }
  const int64_t per = (a.nk + grid - 1) / grid;
  const int per_cta = (int)((per + 15) / 16 * 16);
  if (bvp_two_per_sm(a.nz)) k_bvp_pairs<R, 2><<<(unsigned)grid, BVP_LANES, smem, s>>>(a, spec, corr, scratch, per_cta);
  else k_bvp_pairs<R, 1><<<(unsigned)grid, BVP_LANES, smem, s>>>(a, spec, corr, scratch, per_cta);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  k_bvp_k0<R><<<1, 2 * K0_ROWS, 0, s>>>(a, spec);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Allocation-free launch of the same solve for dpst_mdot_noalloc.
//
// Some callers cannot allocate device memory at the moment they need the
// operator: a host application whose own memory pool has already reserved
// the device (a cudaMalloc from the library would fail, or take memory the
// pool counts on), or a time-critical loop that must not pay for cudaMalloc /
// cudaFree and the device-wide synchronisation cudaFree implies.  For them the
// solve's scratch (the pressure coefficients of every lane, nz doubles per
// lane) comes from the file-scope array below instead of memory owned by the
// handle.  The array is 4 MiB; every GPU that loads the library holds it
// until the process exits.  The solve writes each lane's scratch before
// reading it, so nothing needs clearing between calls, but all calls share
// the one array: calls that overlap on the GPU (other streams, other handles,
// other threads) race on it and must be serialised by the caller.  The kernel
// is launched on as many CTAs as the array holds (192 lanes x nz doubles
// each), at most the grid of the ordinary solve.
// ---------------------------------------------------------------------------
constexpr size_t NOALLOC_SCRATCH_DOUBLES = (size_t)1 << 19;  // 4 MiB
static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];

static std::mutex g_noalloc_mu;
static double *g_noalloc_ptr[256];  // device address of the array, per device

// The array's device address, looked up with the device current.  In host
// code the array's name is only a host-side stand-in and must never be
// passed to a kernel.  The first call on a device does this set-up, so it
// must come before any stream capture on that device; later calls look the
// address up again whenever the stream is not capturing (the module may
// have been reloaded at another address after a device reset) and use the
// address found last while it is.
static cudaError_t noalloc_scratch_ptr(cudaStream_t s, double **out) {
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  if (dev < 0 || dev >= 256) return cudaErrorInvalidDevice;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  err = cudaStreamIsCapturing(s, &cap);
  if (err != cudaSuccess) return err;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (cap == cudaStreamCaptureStatusNone || g_noalloc_ptr[dev] == nullptr) {
    void *p = nullptr;
    err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (err != cudaSuccess) return err;
    g_noalloc_ptr[dev] = static_cast<double *>(p);
  }
  *out = g_noalloc_ptr[dev];
  return cudaSuccess;
}

// Returns cudaErrorInvalidValue and sets *too_big when one CTA's scratch
// (nz x 192 doubles) exceeds the array.
template <typename R>
cudaError_t launch_bvp_noalloc(const KsArgs &a, R *spec, double2 *corr, int64_t planned_grid,
                               cudaStream_t s, bool *too_big) {
  *too_big = false;
  const size_t per_cta = (size_t)a.nz * BVP_LANES;
  if (per_cta > NOALLOC_SCRATCH_DOUBLES) {
    *too_big = true;
    return cudaErrorInvalidValue;
  }
  double *scratch = nullptr;
  cudaError_t err = noalloc_scratch_ptr(s, &scratch);
  if (err != cudaSuccess) return err;
  int64_t grid = (int64_t)(NOALLOC_SCRATCH_DOUBLES / per_cta);
  if (grid > planned_grid) grid = planned_grid;
  return launch_bvp<R>(a, spec, corr, scratch, grid, s, false);
}

size_t noalloc_scratch_bytes() { return NOALLOC_SCRATCH_DOUBLES * sizeof(double); }

template cudaError_t launch_bvp_k0_b<float>(const SysK<float> *, int, cudaStream_t);
template cudaError_t launch_bvp_k0_b<double>(const SysK<double> *, int, cudaStream_t);
template cudaError_t launch_bvp_noalloc<float>(const KsArgs &, float *, double2 *, int64_t, cudaStream_t, bool *);
template cudaError_t launch_bvp_noalloc<double>(const KsArgs &, double *, double2 *, int64_t, cudaStream_t, bool *);
template cudaError_t bvp_plan<float>(const KsArgs &, int, int64_t *, size_t *);
template cudaError_t bvp_plan<double>(const KsArgs &, int, int64_t *, size_t *);
template cudaError_t launch_bvp<float>(const KsArgs &, float *, double2 *, double *, int64_t, cudaStream_t, bool);
template cudaError_t launch_bvp<double>(const KsArgs &, double *, double2 *, double *, int64_t, cudaStream_t, bool);

}  // namespace dpst
