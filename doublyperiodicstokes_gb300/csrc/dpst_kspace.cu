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
#include "dpst_kdev.cuh"
#include "dpst_df64.cuh"
#include <cuComplex.h>
#include <type_traits>

namespace dpst {



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
// Repack the factors for the solve (layouts documented on KsArgs).
// ---------------------------------------------------------------------------
__global__ void k_bvp_pack(KsArgs a) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nk = a.nk;
  if (t >= (int64_t)a.nz * nk) return;
  const int j = (int)(t / nk);
  const int64_t i = t - (int64_t)j * nk;
  a.mf[t] = (j >= 2) ? a.mfac[t] : 0.0;
  double4_32a b;
  b.x = a.invb[(int64_t)(j + 1) * nk + i];
  b.y = (j < a.nz - 2) ? a.dp2[t] : 0.0;
  b.z = a.c0[t];
  b.w = a.c1[t];
  reinterpret_cast<double4_32a *>(a.bk)[t] = b;
  a.ab[t] = (j & 1) ? a.ab1[t] : a.ab0[t];
}

// ---------------------------------------------------------------------------
// z transform GEMM.  OUT[r][col] = sum_m Tm[r][m] IN[m][col] for the real
// view of spec (per component: nz rows x ncols = 2*nk columns), in place.
// CTA: 256 threads, tile = all rows x 64 columns; each thread 4 columns x RPT
// rows.  The transform matrix sits in shared memory for the CTA's lifetime
// (persistent grid-stride over tiles).
// Inverse epilogue: add the wall correction at the node and scale.
// ---------------------------------------------------------------------------


// Folded z transform.  The DCT-I matrices are symmetric under reversing the
// node index: T[j][N-1-m] = (-1)^j T[j][m] for the coefficient-from-nodes
// type (Tf and Ti^T) and T[N-1-m][j] = (-1)^j T[m][j] for the
// nodes-from-coefficients type (Ti and Tf^T), N = nz.  Either halves the
// multiply-adds:
//   ZFOLD_IN  (node-space input): with P_m = x_m + x_{N-1-m},
//             Q_m = x_m - x_{N-1-m} (m < N/2) and the middle node for odd N,
//             even rows are T[j][0..h] . P, odd rows T[j][0..h] . Q;
//   ZFOLD_OUT (node-space output): E_m = sum_{j even} T[m][j] x_j,
//             O_m = sum_{j odd} T[m][j] x_j for m < ceil(N/2), then
//             y_m = E_m + O_m and y_{N-1-m} = E_m - O_m.
// Only the first half of the stored matrix is read.  CTA: 256 threads, tile =
// all rows x 64 columns, each thread 4 columns x RPT rows; rows of one thread
// share a parity (r = ty + 16 q).  Persistent grid-stride over tiles; the
// inverse epilogue adds the wall correction at the node and scales.
constexpr int ZFOLD_IN = 1, ZFOLD_OUT = 2;

// Shared-memory state of a z-transform CTA: the (first half of the) matrix
// and the staged tile.
template <typename R, int RPT, int FOLD>
static __device__ __forceinline__ void zgemm_load_matrix(int nz, const R *__restrict__ Tm, R *Ts) {
  const int h = nz / 2, odd_n = nz & 1;
  const int kf = h + odd_n;
  const int tcols = (FOLD == ZFOLD_IN) ? kf : nz;
  const int tstride = tcols + 1;
  const int trows = (FOLD == ZFOLD_IN) ? nz : kf;
  for (int idx = threadIdx.x; idx < 16 * RPT * tstride; idx += 256) {
    const int r = idx / tstride, m = idx % tstride;
    Ts[idx] = (r < trows && m < tcols) ? Tm[r * nz + m] : (R)0;
  }
}

// One tile: columns [c0, c0 + 64) of component d of the spectrum block B
// (nz rows, row stride ncols), in place.
template <typename R, int RPT, int FOLD>
static __device__ __forceinline__ void zgemm_tile(R *B, int nz, int64_t ncols, int64_t c0, int d, const R *Ts,
                                                  R *Bs, const EpiArgs &e) {
  const int h = nz / 2, odd_n = nz & 1;
  const int kf = h + odd_n;
  const int tcols = (FOLD == ZFOLD_IN) ? kf : nz;
  const int tstride = tcols + 1;
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  __syncthreads();
  if (FOLD == ZFOLD_IN) {
    for (int idx = tid; idx < kf * 64; idx += 256) {
      const int m = idx >> 6, c = idx & 63;
      R pv = 0, qv = 0;
      if (c0 + c < ncols) {
        const R xa = B[(int64_t)m * ncols + c0 + c];
        if (m < h) {
          const R xb = B[(int64_t)(nz - 1 - m) * ncols + c0 + c];
          pv = xa + xb;
          qv = xa - xb;
        } else {
          pv = xa;  // middle node (odd nz)
        }
      }
      Bs[idx] = pv;
      Bs[kf * 64 + idx] = qv;
    }
  } else {
    for (int idx = tid; idx < nz * 64; idx += 256) {
      const int m = idx >> 6, c = idx & 63;
      Bs[idx] = (c0 + c < ncols) ? B[(int64_t)m * ncols + c0 + c] : (R)0;
    }
  }
  __syncthreads();
  if (FOLD == ZFOLD_IN) {
    R acc[RPT][4];
#pragma unroll
    for (int q = 0; q < RPT; ++q)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[q][c] = 0;
    const R *Bp = Bs + ((ty & 1) ? kf * 64 : 0);  // odd rows read Q
    for (int m = 0; m < kf; ++m) {
      R b[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) b[c] = Bp[m * 64 + tx * 4 + c];
#pragma unroll
      for (int q = 0; q < RPT; ++q) {
        const R av = Ts[(ty + 16 * q) * tstride + m];
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
        const int64_t col = c0 + tx * 4 + 2 * cp;
        if (col >= ncols) continue;
        R vr = acc[q][2 * cp], vi = acc[q][2 * cp + 1];
        if (e.inverse) {
          R cre, cim;
          corr_any<R>(e, d, r, col >> 1, cre, cim);
          vr = (vr + cre) * (R)e.scale;
          vi = (vi + cim) * (R)e.scale;
        }
        B[(int64_t)r * ncols + col] = vr;
        B[(int64_t)r * ncols + col + 1] = vi;
      }
    }
  } else {
    R ae[RPT][4], ao[RPT][4];
#pragma unroll
    for (int q = 0; q < RPT; ++q)
#pragma unroll
      for (int c = 0; c < 4; ++c) ae[q][c] = ao[q][c] = 0;
    int j = 0;
    for (; j + 1 < nz; j += 2) {
      R be[4], bo[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        be[c] = Bs[j * 64 + tx * 4 + c];
        bo[c] = Bs[(j + 1) * 64 + tx * 4 + c];
      }
#pragma unroll
      for (int q = 0; q < RPT; ++q) {
        const R te = Ts[(ty + 16 * q) * tstride + j], to = Ts[(ty + 16 * q) * tstride + j + 1];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          ae[q][c] = fma(te, be[c], ae[q][c]);
          ao[q][c] = fma(to, bo[c], ao[q][c]);
        }
      }
    }
    if (j < nz) {  // odd nz: last (even) coefficient
      R be[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) be[c] = Bs[j * 64 + tx * 4 + c];
#pragma unroll
      for (int q = 0; q < RPT; ++q) {
        const R te = Ts[(ty + 16 * q) * tstride + j];
#pragma unroll
        for (int c = 0; c < 4; ++c) ae[q][c] = fma(te, be[c], ae[q][c]);
      }
    }
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
      const int m = ty + 16 * q;
      if (m >= kf) continue;
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        const int r = half ? nz - 1 - m : m;
        if (half && r == m) continue;  // middle node
#pragma unroll
        for (int cp = 0; cp < 2; ++cp) {
          const int64_t col = c0 + tx * 4 + 2 * cp;
          if (col >= ncols) continue;
          R vr = half ? ae[q][2 * cp] - ao[q][2 * cp] : ae[q][2 * cp] + ao[q][2 * cp];
          R vi = half ? ae[q][2 * cp + 1] - ao[q][2 * cp + 1] : ae[q][2 * cp + 1] + ao[q][2 * cp + 1];
          if (e.inverse) {
            R cre, cim;
            corr_any<R>(e, d, r, col >> 1, cre, cim);
            vr = (vr + cre) * (R)e.scale;
            vi = (vi + cim) * (R)e.scale;
          }
          B[(int64_t)r * ncols + col] = vr;
          B[(int64_t)r * ncols + col + 1] = vi;
        }
      }
    }
  }

}

template <typename R, int RPT, int FOLD>
__global__ void __launch_bounds__(256) k_zgemm(R *spec, int nz, int64_t ncols, const R *__restrict__ Tm,
                                              EpiArgs e) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int kf = nz / 2 + (nz & 1);
  const int tcols = (FOLD == ZFOLD_IN) ? kf : nz;
  R *Ts = reinterpret_cast<R *>(smem_raw);  // [16*RPT][tcols+1]
  R *Bs = Ts + 16 * RPT * (tcols + 1);
  zgemm_load_matrix<R, RPT, FOLD>(nz, Tm, Ts);
  const int64_t tiles_per_comp = (ncols + 63) / 64;
  const int64_t ntiles = 3 * tiles_per_comp;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int d = (int)(t / tiles_per_comp);
    const int64_t c0 = (t % tiles_per_comp) * 64;
    zgemm_tile<R, RPT, FOLD>(spec + (int64_t)d * nz * ncols, nz, ncols, c0, d, Ts, Bs, e);
  }
}

// Batched: the tiles of every segment (one system's spectrum each), tprefix
// the first tile of each segment.
template <typename R, int RPT, int FOLD>
__global__ void __launch_bounds__(256) k_zgemm_b(const ZSeg<R> *__restrict__ segs, const int64_t *__restrict__ tprefix,
                                                int S, int nz, const R *__restrict__ Tm) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int kf = nz / 2 + (nz & 1);
  const int tcols = (FOLD == ZFOLD_IN) ? kf : nz;
  R *Ts = reinterpret_cast<R *>(smem_raw);
  R *Bs = Ts + 16 * RPT * (tcols + 1);
  zgemm_load_matrix<R, RPT, FOLD>(nz, Tm, Ts);
  const int64_t ntiles = tprefix[S];
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int sg = find_sys(tprefix, S, t);
    const ZSeg<R> &z = segs[sg];
    const int64_t lt = t - tprefix[sg];
    const int64_t tiles_per_comp = (z.ncols + 63) / 64;
    const int d = (int)(lt / tiles_per_comp);
    const int64_t c0 = (lt % tiles_per_comp) * 64;
    zgemm_tile<R, RPT, FOLD>(z.spec + (int64_t)d * nz * z.ncols, nz, z.ncols, c0, d, Ts, Bs, z.e);
  }
}


// ---------------------------------------------------------------------------
// The FP64 operator's z transform in double-float arithmetic on the FP32
// pipes (FP64 runs at 1/64 of the FP32 rate on this GPU): the folded GEMM of
// zgemm_tile with the matrix and the staged tile held as double-float pairs
// in shared memory and every sum accumulated with the compensated
// (Ogita-Rump-Oishi Dot2) scheme, 12 FP32 operations per multiply-add.  The
// folds (P, Q) are formed in FP64 before the rounding to double-float, and
// the epilogue (wall correction, scale) runs in FP64.  Error ~ 2^-48 times
// the sum of the terms' magnitudes plus the double-float rounding of the
// inputs: about 1e-14 relative against the FP64 GEMM.
// ---------------------------------------------------------------------------
template <int RPT, int FOLD>
__global__ void __launch_bounds__(256) k_zgemm_df(double *spec, int nz, int64_t ncols, const double *__restrict__ Tm,
                                                 EpiArgs e) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int h = nz / 2, odd_n = nz & 1;
  const int kf = h + odd_n;
  const int tcols = (FOLD == ZFOLD_IN) ? kf : nz;
  const int tstride = tcols + 1;
  const int trows = (FOLD == ZFOLD_IN) ? nz : kf;
  float2 *Ts = reinterpret_cast<float2 *>(smem_raw);  // [16 RPT][tcols + 1]
  float2 *Bs = Ts + 16 * RPT * tstride;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  for (int idx = tid; idx < 16 * RPT * tstride; idx += 256) {
    const int r = idx / tstride, m = idx % tstride;
    const df64 v = df_from_d((r < trows && m < tcols) ? Tm[r * nz + m] : 0.0);
    Ts[idx] = make_float2(v.hi, v.lo);
  }
  const int64_t tiles_per_comp = (ncols + 63) / 64;
  const int64_t ntiles = 3 * tiles_per_comp;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int d = (int)(t / tiles_per_comp);
    const int64_t c0 = (t % tiles_per_comp) * 64;
    double *B = spec + (int64_t)d * nz * ncols;
    __syncthreads();
    if (FOLD == ZFOLD_IN) {
      for (int idx = tid; idx < kf * 64; idx += 256) {
        const int m = idx >> 6, c = idx & 63;
        double pv = 0.0, qv = 0.0;
        if (c0 + c < ncols) {
          const double xa = B[(int64_t)m * ncols + c0 + c];
          if (m < h) {
            const double xb = B[(int64_t)(nz - 1 - m) * ncols + c0 + c];
            pv = xa + xb;
            qv = xa - xb;
          } else {
            pv = xa;  // middle node (odd nz)
          }
        }
        const df64 dp = df_from_d(pv), dq = df_from_d(qv);
        Bs[idx] = make_float2(dp.hi, dp.lo);
        Bs[kf * 64 + idx] = make_float2(dq.hi, dq.lo);
      }
    } else {
      for (int idx = tid; idx < nz * 64; idx += 256) {
        const int m = idx >> 6, c = idx & 63;
        const df64 v = df_from_d((c0 + c < ncols) ? B[(int64_t)m * ncols + c0 + c] : 0.0);
        Bs[idx] = make_float2(v.hi, v.lo);
      }
    }
    __syncthreads();
    auto store = [&](int r, int64_t col, df64 re_, df64 im_) {
      double vr = df_to_d(re_), vi = df_to_d(im_);
      if (e.inverse) {
        double cre, cim;
        corr_any<double>(e, d, r, col >> 1, cre, cim);
        vr = (vr + cre) * e.scale;
        vi = (vi + cim) * e.scale;
      }
      B[(int64_t)r * ncols + col] = vr;
      B[(int64_t)r * ncols + col + 1] = vi;
    };
    if (FOLD == ZFOLD_IN) {
      df_acc acc[RPT][4];
#pragma unroll
      for (int q = 0; q < RPT; ++q)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[q][c] = acc_zero();
      const float2 *Bp = Bs + ((ty & 1) ? kf * 64 : 0);  // odd rows read Q
      for (int m = 0; m < kf; ++m) {
        df64 b[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) b[c] = df_lds(Bp[m * 64 + tx * 4 + c]);
#pragma unroll
        for (int q = 0; q < RPT; ++q) {
          const df64 av = df_lds(Ts[(ty + 16 * q) * tstride + m]);
#pragma unroll
          for (int c = 0; c < 4; ++c) acc_fma(acc[q][c], av, b[c]);
        }
      }
#pragma unroll
      for (int q = 0; q < RPT; ++q) {
        const int r = ty + 16 * q;
        if (r >= nz) continue;
#pragma unroll
        for (int cp = 0; cp < 2; ++cp) {
          const int64_t col = c0 + tx * 4 + 2 * cp;
          if (col >= ncols) continue;
          store(r, col, acc_val(acc[q][2 * cp]), acc_val(acc[q][2 * cp + 1]));
        }
      }
    } else {
      df_acc ae[RPT][4], ao[RPT][4];
#pragma unroll
      for (int q = 0; q < RPT; ++q)
#pragma unroll
        for (int c = 0; c < 4; ++c) ae[q][c] = ao[q][c] = acc_zero();
      int j = 0;
      for (; j + 1 < nz; j += 2) {
        df64 be[4], bo[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          be[c] = df_lds(Bs[j * 64 + tx * 4 + c]);
          bo[c] = df_lds(Bs[(j + 1) * 64 + tx * 4 + c]);
        }
#pragma unroll
        for (int q = 0; q < RPT; ++q) {
          const df64 te = df_lds(Ts[(ty + 16 * q) * tstride + j]), to = df_lds(Ts[(ty + 16 * q) * tstride + j + 1]);
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            acc_fma(ae[q][c], te, be[c]);
            acc_fma(ao[q][c], to, bo[c]);
          }
        }
      }
      if (j < nz) {  // odd nz: last (even) coefficient
        df64 be[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) be[c] = df_lds(Bs[j * 64 + tx * 4 + c]);
#pragma unroll
        for (int q = 0; q < RPT; ++q) {
          const df64 te = df_lds(Ts[(ty + 16 * q) * tstride + j]);
#pragma unroll
          for (int c = 0; c < 4; ++c) acc_fma(ae[q][c], te, be[c]);
        }
      }
#pragma unroll
      for (int q = 0; q < RPT; ++q) {
        const int m = ty + 16 * q;
        if (m >= kf) continue;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const df64 E = acc_val(ae[q][c]), O = acc_val(ao[q][c]);
          ae[q][c].s = E.hi;  // keep E and O as value pairs for the store below
          ae[q][c].e = E.lo;
          ao[q][c].s = O.hi;
          ao[q][c].e = O.lo;
        }
#pragma unroll
        for (int half = 0; half < 2; ++half) {
          const int r = half ? nz - 1 - m : m;
          if (half && r == m) continue;  // middle node
#pragma unroll
          for (int cp = 0; cp < 2; ++cp) {
            const int64_t col = c0 + tx * 4 + 2 * cp;
            if (col >= ncols) continue;
            const df64 er = df_make(ae[q][2 * cp].s, ae[q][2 * cp].e), orr = df_make(ao[q][2 * cp].s, ao[q][2 * cp].e);
            const df64 ei = df_make(ae[q][2 * cp + 1].s, ae[q][2 * cp + 1].e);
            const df64 oi = df_make(ao[q][2 * cp + 1].s, ao[q][2 * cp + 1].e);
            store(r, col, half ? df_sub(er, orr) : df_add(er, orr), half ? df_sub(ei, oi) : df_add(ei, oi));
          }
        }
      }
    }
  }
}

template <int RPT, int FOLD>
static cudaError_t zgemm_df_rpt(double *spec, int nz, int64_t ncols, const double *Tm, const EpiArgs &e, int nsm,
                                cudaStream_t s) {
  const int kf = nz / 2 + (nz & 1);
  const size_t tcols = (FOLD == ZFOLD_IN) ? kf : nz;
  const size_t bs = (FOLD == ZFOLD_IN) ? 2 * (size_t)kf * 64 : (size_t)nz * 64;
  const size_t smem = (16 * RPT * (tcols + 1) + bs) * sizeof(float2);
  cudaError_t err = cudaFuncSetAttribute(k_zgemm_df<RPT, FOLD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
  if (err != cudaSuccess) return err;
  int blocks_per_sm = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_zgemm_df<RPT, FOLD>, 256, smem);
  if (err != cudaSuccess) return err;
  if (blocks_per_sm < 1) return cudaErrorInvalidConfiguration;
  int64_t ntiles = 3 * ((ncols + 63) / 64);
  int64_t grid = (int64_t)nsm * blocks_per_sm;
  if (grid > ntiles) grid = ntiles;
  k_zgemm_df<RPT, FOLD><<<(unsigned)grid, 256, smem, s>>>(spec, nz, ncols, Tm, e);
  return cudaGetLastError();
}

template <int FOLD>
static cudaError_t zgemm_df_fold(double *spec, int nz, int64_t ncols, const double *Tm, const EpiArgs &e, int nsm,
                                 cudaStream_t s) {
  const int rows = (FOLD == ZFOLD_IN) ? nz : nz / 2 + (nz & 1);
  const int rpt = (rows + 15) / 16;
  if (rpt <= 2) return zgemm_df_rpt<2, FOLD>(spec, nz, ncols, Tm, e, nsm, s);
  if (rpt <= 4) return zgemm_df_rpt<4, FOLD>(spec, nz, ncols, Tm, e, nsm, s);
  if (rpt <= 6) return zgemm_df_rpt<6, FOLD>(spec, nz, ncols, Tm, e, nsm, s);
  if (rpt <= 8) return zgemm_df_rpt<8, FOLD>(spec, nz, ncols, Tm, e, nsm, s);
  return cudaErrorInvalidValue;
}

// The double-float z transform of an FP64 spectrum (same arguments as
// launch_zgemm<double>).
cudaError_t launch_zgemm_df(double *spec, int nz, int64_t ncols, const double *Tm, const EpiArgs &e, int nsm,
                            cudaStream_t s, bool fold_out) {
  return fold_out ? zgemm_df_fold<ZFOLD_OUT>(spec, nz, ncols, Tm, e, nsm, s)
                  : zgemm_df_fold<ZFOLD_IN>(spec, nz, ncols, Tm, e, nsm, s);
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
void launch_bvp_factors(const KsArgs &a, cudaStream_t s) {
  int bs = 128;
  k_bvp_factors<<<(a.nk + bs - 1) / bs, bs, 0, s>>>(a);
  int64_t tot = (int64_t)a.nz * a.nk;
  k_bvp_pack<<<(tot + 255) / 256, 256, 0, s>>>(a);
}


template <typename R, int RPT, int FOLD>
static cudaError_t zgemm_rpt(R *spec, int nz, int64_t ncols, const R *Tm, const EpiArgs &e, int nsm,
                             cudaStream_t s) {
  const int kf = nz / 2 + (nz & 1);
  const size_t tcols = (FOLD == ZFOLD_IN) ? kf : nz;
  const size_t bs = (FOLD == ZFOLD_IN) ? 2 * (size_t)kf * 64 : (size_t)nz * 64;
  size_t smem = (16 * RPT * (tcols + 1) + bs) * sizeof(R);
  cudaError_t err = cudaFuncSetAttribute(k_zgemm<R, RPT, FOLD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
  if (err != cudaSuccess) return err;
  int blocks_per_sm = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_zgemm<R, RPT, FOLD>, 256, smem);
  if (err != cudaSuccess) return err;
  if (blocks_per_sm < 1) return cudaErrorInvalidConfiguration;
  int64_t ntiles = 3 * ((ncols + 63) / 64);
  int64_t grid = (int64_t)nsm * blocks_per_sm;
  if (grid > ntiles) grid = ntiles;
  k_zgemm<R, RPT, FOLD><<<(unsigned)grid, 256, smem, s>>>(spec, nz, ncols, Tm, e);
  return cudaGetLastError();
}

// fold_out = false: Tm is of the coefficient-from-nodes type (Tf, Ti^T);
// true: nodes-from-coefficients (Ti, Tf^T).
template <typename R, int FOLD>
static cudaError_t zgemm_fold(R *spec, int nz, int64_t ncols, const R *Tm, const EpiArgs &e, int nsm,
                              cudaStream_t s) {
  const int rows = (FOLD == ZFOLD_IN) ? nz : nz / 2 + (nz & 1);
  const int rpt = (rows + 15) / 16;
  if (rpt <= 2) return zgemm_rpt<R, 2, FOLD>(spec, nz, ncols, Tm, e, nsm, s);
  if (rpt <= 4) return zgemm_rpt<R, 4, FOLD>(spec, nz, ncols, Tm, e, nsm, s);
  if (rpt <= 6) return zgemm_rpt<R, 6, FOLD>(spec, nz, ncols, Tm, e, nsm, s);
  if (rpt <= 8) return zgemm_rpt<R, 8, FOLD>(spec, nz, ncols, Tm, e, nsm, s);
  return cudaErrorInvalidValue;
}

template <typename R>
cudaError_t launch_zgemm(R *spec, int nz, int64_t ncols, const R *Tm, const EpiArgs &e, int nsm, cudaStream_t s,
                         bool fold_out) {
  return fold_out ? zgemm_fold<R, ZFOLD_OUT>(spec, nz, ncols, Tm, e, nsm, s)
                  : zgemm_fold<R, ZFOLD_IN>(spec, nz, ncols, Tm, e, nsm, s);
}

template <typename R, int RPT, int FOLD>
static cudaError_t zgemm_rpt_b(const ZSeg<R> *segs, const int64_t *tprefix, int S, int64_t ntiles, int nz,
                               const R *Tm, int nsm, cudaStream_t s) {
  const int kf = nz / 2 + (nz & 1);
  const size_t tcols = (FOLD == ZFOLD_IN) ? kf : nz;
  const size_t bs = (FOLD == ZFOLD_IN) ? 2 * (size_t)kf * 64 : (size_t)nz * 64;
  size_t smem = (16 * RPT * (tcols + 1) + bs) * sizeof(R);
  cudaError_t err = cudaFuncSetAttribute(k_zgemm_b<R, RPT, FOLD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
  if (err != cudaSuccess) return err;
  int blocks_per_sm = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_zgemm_b<R, RPT, FOLD>, 256, smem);
  if (err != cudaSuccess) return err;
  if (blocks_per_sm < 1) return cudaErrorInvalidConfiguration;
  int64_t grid = (int64_t)nsm * blocks_per_sm;
  if (grid > ntiles) grid = ntiles;
  if (grid < 1) return cudaSuccess;
  k_zgemm_b<R, RPT, FOLD><<<(unsigned)grid, 256, smem, s>>>(segs, tprefix, S, nz, Tm);
  return cudaGetLastError();
}

template <typename R, int FOLD>
static cudaError_t zgemm_fold_b(const ZSeg<R> *segs, const int64_t *tprefix, int S, int64_t ntiles, int nz,
                                const R *Tm, int nsm, cudaStream_t s) {
  const int rows = (FOLD == ZFOLD_IN) ? nz : nz / 2 + (nz & 1);
  const int rpt = (rows + 15) / 16;
  if (rpt <= 2) return zgemm_rpt_b<R, 2, FOLD>(segs, tprefix, S, ntiles, nz, Tm, nsm, s);
  if (rpt <= 4) return zgemm_rpt_b<R, 4, FOLD>(segs, tprefix, S, ntiles, nz, Tm, nsm, s);
  if (rpt <= 6) return zgemm_rpt_b<R, 6, FOLD>(segs, tprefix, S, ntiles, nz, Tm, nsm, s);
  if (rpt <= 8) return zgemm_rpt_b<R, 8, FOLD>(segs, tprefix, S, ntiles, nz, Tm, nsm, s);
  return cudaErrorInvalidValue;
}

// Batched z transform over the segments' tiles (tprefix[S] = ntiles).
template <typename R>
cudaError_t launch_zgemm_b(const ZSeg<R> *segs, const int64_t *tprefix, int S, int64_t ntiles, int nz, const R *Tm,
                           int nsm, cudaStream_t s, bool fold_out) {
  return fold_out ? zgemm_fold_b<R, ZFOLD_OUT>(segs, tprefix, S, ntiles, nz, Tm, nsm, s)
                  : zgemm_fold_b<R, ZFOLD_IN>(segs, tprefix, S, ntiles, nz, Tm, nsm, s);
}
template cudaError_t launch_zgemm_b<float>(const ZSeg<float> *, const int64_t *, int, int64_t, int, const float *,
                                           int, cudaStream_t, bool);
template cudaError_t launch_zgemm_b<double>(const ZSeg<double> *, const int64_t *, int, int64_t, int,
                                            const double *, int, cudaStream_t, bool);

// ---------------------------------------------------------------------------
// Spectral curl of a 3-component field in x-y Fourier / z Chebyshev
// coefficients (the regular-kernel torque coupling, FCM.py:372-396 and
// Solvers.py:159-177):
//   c = 1/2 (Dy Sz - dz Sy, dz Sx - Dx Sz, Dx Sy - Dy Sx),
// D = i k with the unpaired Nyquist line of an even axis zeroed
// (Solvers.py:300-304), dz the downward coefficient recurrence of
// chebCoeffDiff_perm (Chebyshev.py:68-94) on [a, a + 2H]:
//   (dz S)_m = (dz S)_{m+2} + (2/H)(m+1) S_{m+1},  (dz S)_{nz-1} = 0, then / 2 at m = 0.
// ACC: dst += c (the torque curl added to the forces' coefficients); else
// dst = c (the vorticity; dst may alias src: level m is read before it is
// written and the recurrence only looks at levels above).  One thread per
// wavenumber; spectrum layout [3][nz][nk] complex.
// ---------------------------------------------------------------------------
template <typename R, bool ACC>
__global__ void k_spec_curl(const R *src, R *dst, int nz, int64_t nk, int nx, int ny, int nxh,
                            const double *__restrict__ kvx, const double *__restrict__ kvy, double H) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= nk) return;
  const int ix = (int)(k % nxh), iy = (int)(k / nxh);
  const R dx = (2 * ix == nx) ? (R)0 : (R)kvx[ix];
  const R dy = (2 * iy == ny) ? (R)0 : (R)kvy[iy];
  const R half = (R)0.5;
  auto idx = [&](int d, int m) { return (((int64_t)d * nz + m) * nk + k) * 2; };
  // f1: S at level m+1 (x, y); g1, g2: dz S at levels m+1, m+2
  R fxr = 0, fxi = 0, fyr = 0, fyi = 0;
  R gx1r = 0, gx1i = 0, gy1r = 0, gy1i = 0, gx2r = 0, gx2i = 0, gy2r = 0, gy2i = 0;
  for (int m = nz - 1; m >= 0; --m) {
    const R c = (R)(2.0 / H * (double)(m + 1));
    R gxr = gx2r + c * fxr, gxi = gx2i + c * fxi;
    R gyr = gy2r + c * fyr, gyi = gy2i + c * fyi;
    gx2r = gx1r; gx2i = gx1i; gy2r = gy1r; gy2i = gy1i;
    gx1r = gxr; gx1i = gxi; gy1r = gyr; gy1i = gyi;
    if (m == 0) {
      gxr /= 2; gxi /= 2; gyr /= 2; gyi /= 2;
    }
    const R sxr = src[idx(0, m)], sxi = src[idx(0, m) + 1];
    const R syr = src[idx(1, m)], syi = src[idx(1, m) + 1];
    const R szr = src[idx(2, m)], szi = src[idx(2, m) + 1];
    // i dy Sz - dz Sy, dz Sx - i dx Sz, i dx Sy - i dy Sx
    const R cxr = half * (-dy * szi - gyr), cxi = half * (dy * szr - gyi);
    const R cyr = half * (gxr + dx * szi), cyi = half * (gxi - dx * szr);
    const R czr = half * (-dx * syi + dy * sxi), czi = half * (dx * syr - dy * sxr);
    fxr = sxr; fxi = sxi; fyr = syr; fyi = syi;
    if (ACC) {
      dst[idx(0, m)] += cxr; dst[idx(0, m) + 1] += cxi;
      dst[idx(1, m)] += cyr; dst[idx(1, m) + 1] += cyi;
      dst[idx(2, m)] += czr; dst[idx(2, m) + 1] += czi;
    } else {
      dst[idx(0, m)] = cxr; dst[idx(0, m) + 1] = cxi;
      dst[idx(1, m)] = cyr; dst[idx(1, m) + 1] = cyi;
      dst[idx(2, m)] = czr; dst[idx(2, m) + 1] = czi;
    }
  }
}

template <typename R>
void launch_spec_curl(const R *src, R *dst, bool accumulate, int nz, int64_t nk, int nx, int ny, int nxh,
                      const double *kvx, const double *kvy, double H, cudaStream_t s) {
  const int bs = 128;
  const int64_t nb = (nk + bs - 1) / bs;
  if (accumulate) k_spec_curl<R, true><<<nb, bs, 0, s>>>(src, dst, nz, nk, nx, ny, nxh, kvx, kvy, H);
  else k_spec_curl<R, false><<<nb, bs, 0, s>>>(src, dst, nz, nk, nx, ny, nxh, kvx, kvy, H);
}
template void launch_spec_curl<float>(const float *, float *, bool, int, int64_t, int, int, int, const double *,
                                      const double *, double, cudaStream_t);
template void launch_spec_curl<double>(const double *, double *, bool, int, int64_t, int, int, int,
                                       const double *, const double *, double, cudaStream_t);

template cudaError_t launch_zgemm<float>(float *, int, int64_t, const float *, const EpiArgs &, int,
                                         cudaStream_t, bool);
template cudaError_t launch_zgemm<double>(double *, int, int64_t, const double *, const EpiArgs &, int,
                                          cudaStream_t, bool);

}  // namespace dpst
