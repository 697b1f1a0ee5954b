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
// coupled values through shared memory and warp shuffles.  The three working
// columns of a lane (penta solution / border solution, pressure
// coefficients, pressure derivative coefficients: 3 nz + 2 doubles) live in
// shared memory laid out [row][lane], so every access is conflict-free.  A
// CTA of 64 lanes solves 32 wavenumbers at a time and strides over all of
// them (persistent).  GB300 executes FP64 at 1/58 of its FP32 rate, so a
// few warps per SM keep the FP64 pipe busy; the kernel is built to issue
// nothing but the recurrence arithmetic on that pipe.
#include "dpst_internal.cuh"
#include "dpst_kdev.cuh"

namespace dpst {

constexpr int BVP_LANES = 64;

template <typename R>
__global__ void __launch_bounds__(BVP_LANES) k_bvp_pairs(KsArgs a, R *__restrict__ spec,
                                                         double2 *__restrict__ corr) {
  extern __shared__ double bvp_sm[];
  const int nz = a.nz;
  const int64_t nk = a.nk;
  const int tid = threadIdx.x, part = tid & 1, q = tid >> 1;
  const int T = BVP_LANES;
  double *Xs = bvp_sm;                 // [(nz + 2)][T]
  double *CPs = bvp_sm + (nz + 2) * T;  // [nz][T]
  double *DPs = CPs + nz * T;           // [nz][T]
#define XS(j) Xs[(j) * T + tid]
#define CPS(j) CPs[(j) * T + tid]
#define CPO(j) CPs[(j) * T + (tid ^ 1)]
#define DPS(j) DPs[(j) * T + tid]
  const double sp = part ? 1.0 : -1.0;  // (i a)_part = sp * a_(other part)
  const double inv_eta = 1.0 / a.eta;
  const double *s0 = a.s0, *sp2 = a.sp2, *sm2 = a.sm2, *fm1 = a.fm1, *fp1 = a.fp1;
  const int64_t ntiles = (nk + 31) / 32;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t i_raw = tile * 32 + q;
    const int64_t i = i_raw < nk ? i_raw : nk - 1;
    const bool store = (i_raw < nk) && (i != 0);  // mode 0 is solved by k_bvp_k0
    // element (d, j, mode, part) of the spectrum as a real array
    auto ldp = [&](int d, int j, int pp) -> double {
      return (double)spec[(((int64_t)d * nz + j) * nk + i) * 2 + pp];
    };
    const int ix = (int)(i % a.nxh), iy = (int)(i / a.nxh);
    const double kx = a.kvx[ix], ky = a.kvy[iy];
    const double Dx = ((a.nx % 2) == 0 && ix == a.nx / 2) ? 0.0 : kx;
    const double Dy = ((a.ny % 2) == 0 && iy == a.ny / 2) ? 0.0 : ky;
    const double K = sqrt(kx * kx + ky * ky);
    const double *mf = a.mfac + i, *ib = a.invb + i, *d2 = a.dp2 + i;
    const double *A0 = a.ab0 + i, *A1 = a.ab1 + i, *C0 = a.c0 + i, *C1 = a.c1 + i;
    const double G00 = a.ginv[i], G10 = a.ginv[nk + i], G01 = a.ginv[2 * nk + i], G11 = a.ginv[3 * nk + i];

    // pressure RHS Dx f + Dy g + d/dz h (DPTools.cpp:134-195), backward in j
    {
      double dfp1 = 0.0, dfp2 = 0.0, fzn = 0.0;
      for (int j = nz - 1; j >= 0; --j) {
        const double df = (j == nz - 1) ? 0.0 : dfp2 + ((double)((j + 1) * 2) / a.H) * fzn;
        const double fz = ldp(2, j, part);
        const double dfv = (j == 0) ? 0.5 * df : df;
        XS(j) = ((Dx * sp) * ldp(0, j, part ^ 1) + (Dy * sp) * ldp(1, j, part ^ 1)) + dfv;
        dfp2 = dfp1;
        dfp1 = df;
        fzn = fz;
      }
    }
    // KBPENTA sweeps (LinearSolvers.h:106-141) in place on XS, with the
    // border dots y = C x accumulated during the back sweep
    auto penta = [&](double &y0, double &y1) {
      double xm2 = XS(0), xm1 = XS(1);
#pragma unroll 4
      for (int j = 2; j < nz; ++j) {
        const double v = XS(j) - mf[j * nk] * xm2;
        XS(j) = v;
        xm2 = xm1;
        xm1 = v;
      }
      const double xl = ib[nz * nk] * XS(nz - 1);
      const double xl2 = ib[(nz - 1) * nk] * XS(nz - 2);
      XS(nz - 1) = xl;
      XS(nz - 2) = xl2;
      y0 = C0[(nz - 1) * nk] * xl + C0[(nz - 2) * nk] * xl2;
      y1 = C1[(nz - 1) * nk] * xl + C1[(nz - 2) * nk] * xl2;
      double xp2 = xl, xp1 = xl2;
#pragma unroll 4
      for (int j = nz - 3; j >= 0; --j) {
        const double v = ib[(j + 1) * nk] * (XS(j) - d2[j * nk] * xp2);
        XS(j) = v;
        y0 += C0[j * nk] * v;
        y1 += C1[j * nk] * v;
        xp2 = xp1;
        xp1 = v;
      }
    };
    auto border = [&](double g0, double g1) {
#pragma unroll 4
      for (int j = 0; j < nz; ++j) XS(j) -= A0[j * nk] * g0 + A1[j * nk] * g1;
      XS(nz) = g0;
      XS(nz + 1) = g1;
    };
    // S [x; g] for row m (SIMat, Chebyshev.py:139-160)
    auto srow = [&](int m, double g0, double g1) {
      double c = s0[m] * XS(m);
      if (m >= 2) c = sm2[m] * XS(m - 2) + c;
      c = c + sp2[m] * XS(m + 2);
      if (m == 0) c += a.se0 * g0;
      if (m == 1) c += a.se1 * g1;
      return c;
    };

    // pressure: Schur solve, then cp = S [x; g], dp = F [x; g]
    double ssum = 0.0, asum = 0.0;
    {
      double y0, y1;
      penta(y0, y1);
      const double g0 = G00 * y0 + G01 * y1, g1 = G10 * y0 + G11 * y1;
      border(g0, g1);
      for (int m = 0; m < nz; ++m) {
        const double c = srow(m, g0, g1);
        double dpv = fp1[m] * XS(m + 1);
        if (m >= 1) dpv = fm1[m] * XS(m - 1) + dpv;
        if (m == 0) dpv += a.fe * g1;
        CPS(m) = c;
        DPS(m) = dpv;
        ssum += c;
        asum += (m & 1) ? -c : c;
      }
    }
    // velocity BC right-hand sides (DPTools.cpp:218-234)
    const double ssum_o = __shfl_xor_sync(0xffffffffu, ssum, 1);
    const double asum_o = __shfl_xor_sync(0xffffffffu, asum, 1);
    const double fac1 = 2.0 * a.eta, fac = fac1 * K;
    const double ifac = 1.0 / fac, ifac1 = 1.0 / fac1;
    double bc[6];
    bc[0] = -ifac * ((Dx * sp) * ssum_o);
    bc[1] = ifac * ((Dx * sp) * asum_o);
    bc[2] = -ifac * ((Dy * sp) * ssum_o);
    bc[3] = ifac * ((Dy * sp) * asum_o);
    bc[4] = ifac1 * ssum;
    bc[5] = ifac1 * asum;
    __syncwarp();  // the partner's pressure coefficients are read below

    // velocity: three Schur solves (DPTools.cpp:197-216, 287-345)
    double wt[3], wb[3];
    for (int c = 0; c < 3; ++c) {
      for (int j = 0; j < nz; ++j) {
        const double f = ldp(c, j, part);
        double r;
        if (c == 0) r = (Dx * sp) * CPO(j) - f;
        else if (c == 1) r = (Dy * sp) * CPO(j) - f;
        else r = DPS(j) - f;
        XS(j) = inv_eta * r;
      }
      double y0, y1;
      penta(y0, y1);
      const double r0 = y0 - bc[2 * c], r1 = y1 - bc[2 * c + 1];
      const double g0 = G00 * r0 + G01 * r1, g1 = G10 * r0 + G11 * r1;
      border(g0, g1);
      double st = 0.0, sb = 0.0;
      for (int m = 0; m < nz; ++m) {
        const double u = srow(m, g0, g1);
        if (store) spec[(((int64_t)c * nz + m) * nk + i) * 2 + part] = (R)u;
        st += u;
        sb += (m & 1) ? -u : u;
      }
      wt[c] = st;
      wb[c] = sb;
    }
    // wall-correction coefficients (evalTheta at z = 0 and z = Lz)
    double wto[3], wbo[3];
    for (int c = 0; c < 3; ++c) {
      wto[c] = __shfl_xor_sync(0xffffffffu, wt[c], 1);
      wbo[c] = __shfl_xor_sync(0xffffffffu, wb[c], 1);
    }
    __syncwarp();  // XS/CPS reuse in the next tile
    if (!store) continue;
    double *crd = reinterpret_cast<double *>(corr + i * 16);
    if (a.mode == 1) {
      for (int c = 0; c < 3; ++c) crd[2 * c + part] = -wb[c];
    } else if (a.mode == 2 && part == 0) {
      double2 fb[3], ft[3], cf[8];
      for (int c = 0; c < 3; ++c) {
        fb[c] = make_double2(-wb[c], -wbo[c]);
        ft[c] = make_double2(-wt[c], -wto[c]);
      }
      slit_coeffs(kx, ky, a.Lz, a.eta, fb, ft, cf);
      for (int r = 0; r < 8; ++r) corr[i * 16 + r] = cf[r];
      double kxp, kyp;
      if (!mode_is_hermitian(a, ix, iy, kx, ky, kxp, kyp)) {
        for (int c = 0; c < 3; ++c) {
          fb[c] = cconj(fb[c]);
          ft[c] = cconj(ft[c]);
        }
        slit_coeffs(kxp, kyp, a.Lz, a.eta, fb, ft, cf);
        for (int r = 0; r < 8; ++r) corr[i * 16 + 8 + r] = cf[r];
      }
    }
  }
#undef XS
#undef CPS
#undef CPO
#undef DPS
}

// k = 0: open domain -> zero; walls -> u, v from the k = 0 BVP with the
// reference's BC rows (u' = 0 or u = 0 at the top, u = 0 at the bottom), w = 0.
template <typename R>
__global__ void k_bvp_k0(KsArgs a, R *__restrict__ spec) {
  const int part = threadIdx.x;  // 0: real part, 1: imaginary part
  if (part > 1) return;
  const int nz = a.nz;
  const int64_t nk = a.nk;
  auto at = [&](int d, int j) -> R & { return spec[(((int64_t)d * nz + j) * nk) * 2 + part]; };
  double X[130], U[128];
  if (a.mode == 0) {
    for (int d = 0; d < 3; ++d)
      for (int j = 0; j < nz; ++j) at(d, j) = (R)0;
    return;
  }
  const double inv_eta = 1.0 / a.eta;
  for (int c = 0; c < 2; ++c) {
    double y0 = 0.0, y1 = 0.0;
    for (int j = 0; j < nz; ++j) {
      const double r = -inv_eta * (double)at(c, j);
      X[j] = r;
      y0 += a.k0c0[j] * r;
      y1 += a.k0c1[j] * r;
    }
    const double g0 = a.k0gi[0] * y0 + a.k0gi[1] * y1;
    const double g1 = a.k0gi[2] * y0 + a.k0gi[3] * y1;
    X[nz] = g0;
    X[nz + 1] = g1;
    for (int m = 0; m < nz; ++m) {
      double s = a.s0[m] * X[m];
      if (m >= 2) s = a.sm2[m] * X[m - 2] + s;
      s = s + a.sp2[m] * X[m + 2];
      if (m == 0) s += a.se0 * g0;
      if (m == 1) s += a.se1 * g1;
      U[m] = s;
    }
    for (int m = 0; m < nz; ++m) at(c, m) = (R)U[m];
  }
  for (int j = 0; j < nz; ++j) at(2, j) = (R)0;
}

template <typename R>
cudaError_t launch_bvp(const KsArgs &a, R *spec, double2 *corr, int nsm, cudaStream_t s) {
  const size_t smem = sizeof(double) * (size_t)(3 * a.nz + 2) * BVP_LANES;
  cudaError_t err = cudaFuncSetAttribute(k_bvp_pairs<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  int per_sm = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bvp_pairs<R>, BVP_LANES, smem);
  if (err != cudaSuccess) return err;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int64_t ntiles = (a.nk + 31) / 32;
  int64_t grid = (int64_t)nsm * per_sm;
  if (grid > ntiles) grid = ntiles;
  k_bvp_pairs<R><<<(unsigned)grid, BVP_LANES, smem, s>>>(a, spec, corr);
  err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  k_bvp_k0<R><<<1, 32, 0, s>>>(a, spec);
  return cudaGetLastError();
}

template cudaError_t launch_bvp<float>(const KsArgs &, float *, double2 *, int, cudaStream_t);
template cudaError_t launch_bvp<double>(const KsArgs &, double *, double2 *, int, cudaStream_t);

}  // namespace dpst
