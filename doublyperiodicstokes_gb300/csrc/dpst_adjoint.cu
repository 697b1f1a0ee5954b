// Transpose of the wavenumber-space stages of Mdot, for the backward pass.
//
// The grid operator L of Mdot (spread grid -> velocity grid) is real and
// translation invariant in x-y.  With the x-y transforms unnormalised and the
// 1/(nx ny) folded into the per-mode map, L = C2R o B o R2C where, per
// half-spectrum mode i,
//     B_i = (1/(nx ny)) [Ti + Zeff_i W] N_i Tf
// (Tf / Ti the forward / inverse DCT-I matrices, N_i the no-wall solve of
// DPTools.cpp:81-345, W the wall evaluation with the sign the correction
// uses, Zeff_i the wall-correction profiles at the nodes of
// DPTools.cpp:590-877 averaged with the conjugate of the partner mode's on
// the self-conjugate columns).  The operators of the partner mode are the
// conjugates of mode i's, so L^T = C2R o B^H o R2C with
//     B_i^H = (1/(nx ny)) Tf^T N_i^H [Ti^T + W^T Zeff_i^H].
// This file holds the mode-local pieces:
//   k_corr_adj       Zeff_i^H applied to the node-space adjoint field
//   k_bvp_adj_pairs  N_i^H (with the W^T term added to its input); a lane
//                    pair per wavenumber as in the forward solve; the
//                    transposed KBPENTA sweeps reuse the forward factors
//                    (A = L U, so A^{-T} = L^{-T} U^{-T})
//   k_bvp_adj_k0     the k = 0 mode
// Every step is the transpose of the forward kernels' arithmetic, so
// <g, L f> = <L^T g, f> holds to rounding for any f, g.
#include "dpst_internal.cuh"
#include "dpst_kdev.cuh"

namespace dpst {

constexpr int ADJ_LANES = 192;
constexpr int ADJ_MODES = ADJ_LANES / 2;

// ---------------------------------------------------------------------------
// Zeff_i^H g per wavenumber from the node-space adjoint spectrum (x-y
// transform of the adjoint grid, before any z transform).  Output per mode:
// cadj[0..2] the adjoint of the bottom wall values, cadj[3..5] of the top
// wall values (slit).  For each pass the forward map is Z(q) (main pass,
// q = (kx, ky)) or conj(Z(q')) (partner pass, Nyquist lines only), so the
// adjoint applies Z(q)^H or Z(q')^T: the imaginary entries of Z are
// conjugated on the main pass only.
// CADJ_G lanes per mode split the nodes and combine their sums with
// shuffles; the node profiles and the sums are evaluated in the operator's
// arithmetic CT (as the forward's correction epilogue does; FP32 for the
// mixed operator, whose FP64 work runs at 1/64 of the FP32 rate here), the
// slit's 8x8 solve in FP64.  The partner pass runs when any mode of the warp
// needs it (a warp vote keeps the shuffles warp-uniform) and contributes only
// where the mode needs it.
// ---------------------------------------------------------------------------
constexpr int CADJ_G = 8;

template <typename V>
static __device__ __forceinline__ V group_sum(V v) {
  for (int o = CADJ_G / 2; o > 0; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  return v;
}

// complex helpers in the sums' type (float2 or double2)
template <typename V, typename S>
static __device__ __forceinline__ V vmk(S x, S y) {
  V r;
  r.x = x;
  r.y = y;
  return r;
}
template <typename V, typename S>
static __device__ __forceinline__ V vadd(V a, V b) { return vmk<V, S>(a.x + b.x, a.y + b.y); }
template <typename V, typename S>
static __device__ __forceinline__ V vscale(S s, V a) { return vmk<V, S>(s * a.x, s * a.y); }
template <typename V, typename S>
static __device__ __forceinline__ V vik(S s, V a) { return vmk<V, S>(-s * a.y, s * a.x); }  // i s a

template <typename R>
__global__ void __launch_bounds__(256) k_corr_adj(KsArgs a, const R *__restrict__ spec, double2 *__restrict__ cadj) {
  typedef R CT;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i_raw = t / CADJ_G;
  const int sub = (int)(t % CADJ_G);
  const int nz = a.nz;
  const int64_t nk = a.nk;
  const int64_t i = i_raw < nk ? i_raw : nk - 1;
  const bool store = (i_raw < nk) && sub == 0;
  const int ix = (int)(i % a.nxh), iy = (int)(i / a.nxh);
  const double kx = a.kvx[ix], ky = a.kvy[iy];
  const double k = sqrt(kx * kx + ky * ky);
  double kxp, kyp;
  const bool herm = mode_is_hermitian(a, ix, iy, kx, ky, kxp, kyp);
  const CT kc = (CT)k;
  typedef typename std::conditional<sizeof(CT) == 4, float2, double2>::type V;  // sums in CT
  auto g = [&](int d, int m) -> V {
    const R *p = spec + (((int64_t)d * nz + m) * nk + i) * 2;
    return vmk<V, CT>((CT)p[0], (CT)p[1]);
  };
  auto d2 = [](V v) { return make_double2((double)v.x, (double)v.y); };
  double2 acc[6];
  for (int q = 0; q < 6; ++q) acc[q] = make_double2(0, 0);
  const bool any_partner = __any_sync(0xffffffffu, !herm && i_raw < nk);
  for (int pass = 0; pass < (any_partner ? 2 : 1); ++pass) {
    const bool use = (pass == 0) || !herm;
    const double qx = pass ? kxp : kx, qy = pass ? kyp : ky;
    const CT qxc = (CT)qx, qyc = (CT)qy;
    // an entry i c of Z enters as i c (partner pass) or -i c (main pass)
    const double cs = pass ? 1.0 : -1.0;
    if (a.mode == 1) {
      // Z (DPTools.cpp:627-641) per node, symmetric 3x3:
      //   [e - qx^2 ze/k, -qx qy ze/k, -i qx ze; ., e - qy^2 ze/k, -i qy ze; ., ., e + k ze]
      V s0 = vmk<V, CT>(0, 0), s1 = s0, s2 = s0;
      const CT csc = (CT)cs;
      for (int m = sub; m < nz; m += CADJ_G) {
        const CT z = (CT)a.zn[m];
        const CT e = exp(-kc * z), ze = z * e;
        const V g0 = g(0, m), g1 = g(1, m), g2 = g(2, m);
        const CT z00 = e - qxc * qxc * ze / kc, z01 = -qxc * qyc * ze / kc;
        const CT z11 = e - qyc * qyc * ze / kc, z22 = e + kc * ze;
        const CT ix_ = csc * (-qxc * ze), iy_ = csc * (-qyc * ze);
        s0 = vadd<V, CT>(s0, vadd<V, CT>(vadd<V, CT>(vscale<V, CT>(z00, g0), vscale<V, CT>(z01, g1)),
                                          vik<V, CT>(ix_, g2)));
        s1 = vadd<V, CT>(s1, vadd<V, CT>(vadd<V, CT>(vscale<V, CT>(z01, g0), vscale<V, CT>(z11, g1)),
                                          vik<V, CT>(iy_, g2)));
        s2 = vadd<V, CT>(s2, vadd<V, CT>(vadd<V, CT>(vik<V, CT>(ix_, g0), vik<V, CT>(iy_, g1)),
                                          vscale<V, CT>(z22, g2)));
      }
      s0 = group_sum(s0);
      s1 = group_sum(s1);
      s2 = group_sum(s2);
      if (use) {
        acc[0] = cadd(acc[0], d2(s0));
        acc[1] = cadd(acc[1], d2(s1));
        acc[2] = cadd(acc[2], d2(s2));
      }
    } else {
      // Z = P A^{-1} R (DPTools.cpp:731-815): R maps (fb, ft) to the right
      // side of the 8x8 system A, P maps its solution to node values
      const double fac = 1.0 / 2.0 / a.eta, Hs = a.Lz;
      const CT facc = (CT)fac, Hc = (CT)Hs;
      V pv[8];
      for (int q = 0; q < 8; ++q) pv[q] = vmk<V, CT>(0, 0);
      const CT csc = (CT)cs;
      for (int m = sub; m < nz; m += CADJ_G) {
        const CT z = (CT)a.zn[m];
        const CT e = exp(-kc * z), e2 = exp(kc * (z - Hc));
        const CT ze = z * e, ze2 = z * e2;
        const V g0 = g(0, m), g1 = g(1, m), g2 = g(2, m);
        // P rows: v0 = -i qx ze fac/k c0 + i qx ze2 fac/k c1 + e c2 + e2 c3,
        // v1 likewise with qy, c4, c5; v2 = ze fac c0 + ze2 fac c1 + e c6 + e2 c7
        const CT a0 = csc * (-qxc * ze * facc / kc), a1 = csc * (-qyc * ze * facc / kc);
        const CT b0 = csc * (qxc * ze2 * facc / kc), b1 = csc * (qyc * ze2 * facc / kc);
        pv[0] = vadd<V, CT>(pv[0], vadd<V, CT>(vadd<V, CT>(vik<V, CT>(a0, g0), vik<V, CT>(a1, g1)),
                                                vscale<V, CT>(ze * facc, g2)));
        pv[1] = vadd<V, CT>(pv[1], vadd<V, CT>(vadd<V, CT>(vik<V, CT>(b0, g0), vik<V, CT>(b1, g1)),
                                                vscale<V, CT>(ze2 * facc, g2)));
        pv[2] = vadd<V, CT>(pv[2], vscale<V, CT>(e, g0));
        pv[3] = vadd<V, CT>(pv[3], vscale<V, CT>(e2, g0));
        pv[4] = vadd<V, CT>(pv[4], vscale<V, CT>(e, g1));
        pv[5] = vadd<V, CT>(pv[5], vscale<V, CT>(e2, g1));
        pv[6] = vadd<V, CT>(pv[6], vscale<V, CT>(e, g2));
        pv[7] = vadd<V, CT>(pv[7], vscale<V, CT>(e2, g2));
      }
      double2 p[8];
      for (int q = 0; q < 8; ++q) p[q] = d2(group_sum(pv[q]));
      if (use && sub == 0) {
        // A^{-H} (main) / A^{-T} (partner)
        double2 A[64], At[64];
        slit_matrix(qx, qy, Hs, a.eta, A);
        for (int r = 0; r < 8; ++r)
          for (int c = 0; c < 8; ++c) {
            const double2 v = A[r + 8 * c];
            At[c + 8 * r] = pass ? v : cconj(v);
          }
        zsolve8(At, p);
        // R: x0 = -i qx fb0 - i qy fb1, x1 likewise for the top, x2..x4 = fb,
        // x5..x7 = ft
        acc[0] = cadd(acc[0], cadd(cik(cs * (-qx), p[0]), p[2]));
        acc[1] = cadd(acc[1], cadd(cik(cs * (-qy), p[0]), p[3]));
        acc[2] = cadd(acc[2], p[4]);
        acc[3] = cadd(acc[3], cadd(cik(cs * (-qx), p[1]), p[5]));
        acc[4] = cadd(acc[4], cadd(cik(cs * (-qy), p[1]), p[6]));
        acc[5] = cadd(acc[5], p[7]);
      }
    }
  }
  if (!store) return;
  double2 *out = cadj + i * 6;
  const double wgt = herm ? 1.0 : 0.5;
  for (int q = 0; q < 6; ++q) out[q] = (i == 0) ? make_double2(0, 0) : cscale(wgt, acc[q]);  // k = 0: none
}

// ---------------------------------------------------------------------------
// N_i^H per wavenumber, in place on the coefficient-space spectrum (in: the
// adjoint of the velocity coefficients, Ti^T g; out: the adjoint of the force
// coefficients).  The W^T term is added to the input as it is read: the
// forward's wall values are fb = -sum_m (-1)^m u_m (z = 0) and
// ft = -sum_m u_m (z = Lz).  Lane pair per wavenumber (real / imaginary
// part).  Scratch: cp_bar and dp_bar, each [nz][lanes of the grid].
//
// Forward structure (per velocity component c; every operator real):
//   X = A^{-1} rhs_c, y = C X, g = Ginv (y - bc_c), x = X - AB g,
//   u_c = S [x; g];  rhs_c = (i D_c cp - f_c)/eta (c = 0, 1),
//   rhs_2 = (dp - f_2)/eta;
//   pressure: X = A^{-1} prhs, g = Ginv C X, x = X - AB g, cp = S [x; g],
//   dp = F [x; g];  prhs = i Dx f0 + i Dy f1 + D f2 (Chebyshev derivative);
//   bc from ssum = sum cp and asum = sum (-1)^m cp.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(ADJ_LANES) k_bvp_adj_pairs(KsArgs a, R *__restrict__ spec,
                                                            const double2 *__restrict__ cadj,
                                                            double *__restrict__ scratch, int per_cta) {
  extern __shared__ double adj_sm[];
  const int nz = a.nz;
  const int nk = (int)a.nk;
  const int tid = threadIdx.x, part = tid & 1, q = tid >> 1;
  constexpr int T = ADJ_LANES;
  double *Xs = adj_sm;  // [(nz + 2)][T]
  double *S0 = adj_sm + (nz + 2) * T, *SM2 = S0 + nz, *SP2 = SM2 + nz, *FM1 = SP2 + nz, *FP1 = FM1 + nz;
  double *DH = FP1 + nz;  // 2 j / H, j = 0..nz
  for (int t = tid; t < nz; t += T) {
    S0[t] = a.s0[t];
    SM2[t] = a.sm2[t];
    SP2[t] = a.sp2[t];
    FM1[t] = a.fm1[t];
    FP1[t] = a.fp1[t];
  }
  for (int t = tid; t <= nz; t += T) DH[t] = (double)(2 * t) / a.H;
  __syncthreads();
  const int GT = gridDim.x * T;
  double *__restrict__ CPb = scratch + blockIdx.x * T + tid;                    // row j at CPb[j * GT]
  double *__restrict__ DPb = scratch + (size_t)nz * GT + blockIdx.x * T + tid;  // row j at DPb[j * GT]
#define XS(j) Xs[(j) * T + tid]
#define XO(j) Xs[(j) * T + (tid ^ 1)]
  // (i a)_part = sp * a_(other part); (-i a)_part = -sp * a_(other part)
  const double sp = part ? 1.0 : -1.0;
  const double inv_eta = 1.0 / a.eta;
  const int rs = 2 * nk;  // spectrum row stride (R elements) = bk row stride (double2)
  // work split as in k_bvp_pairs: contiguous per-CTA ranges, whole warps
  const int cta_begin = blockIdx.x * per_cta;
  const int cta_end = min(cta_begin + per_cta, nk);
  for (int base = cta_begin; base < cta_end; base += ADJ_MODES) {
    if (base + (tid >> 5) * 16 >= cta_end) continue;  // warp-uniform
    const int i_raw = base + q;
    const int i = i_raw < cta_end ? i_raw : cta_end - 1;
    const bool store = (i_raw < cta_end) && (i != 0);  // mode 0: k_bvp_adj_k0
    R *__restrict__ own = spec + 2 * i + part;
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
    double wb_bar[3] = {0, 0, 0}, wt_bar[3] = {0, 0, 0};
    if (a.mode != 0 && i != 0) {
      const double *cd = reinterpret_cast<const double *>(cadj + (size_t)i * 6);
      for (int c = 0; c < 3; ++c) {
        wb_bar[c] = cd[2 * c + part];
        if (a.mode == 2) wt_bar[c] = cd[2 * (3 + c) + part];
      }
    }
    // A^{-T} (XS + C^T r) in place on XS: U^T z = b forward, then
    // L^T x = z backward, with U[j][j] = beta_{j+1}, U[j][j+2] = dp2_j and
    // L[j][j-2] = mf_j the forward's factors.
    auto penta_t = [&](double r0, double r1) {
      double zm2 = 0.0, zm1 = 0.0, d2m2 = 0.0, d2m1 = 0.0;
      const double2 *b = bk0;
#pragma unroll 4
      for (int j = 0; j < nz; ++j) {
        const double2 ibd = __ldg(b), cc = __ldg(b + 1);
        const double v = ibd.x * ((XS(j) + (cc.x * r0 + cc.y * r1)) - d2m2 * zm2);
        XS(j) = v;
        zm2 = zm1;
        zm1 = v;
        d2m2 = d2m1;
        d2m1 = ibd.y;
        b += rs;
      }
      double xp2 = 0.0, xp1 = 0.0, mp2 = 0.0, mp1 = 0.0;
      const double *mp = mf0 + (size_t)(nz - 1) * nk;
#pragma unroll 4
      for (int j = nz - 1; j >= 0; --j) {
        const double v = XS(j) - mp2 * xp2;
        XS(j) = v;
        xp2 = xp1;
        xp1 = v;
        mp2 = mp1;
        mp1 = __ldg(mp);  // mf_j, used two rows up
        mp -= nk;
      }
    };

    // Transposed window: XS(j) = (S^T v)_j [+ (F^T d)_j] on the interior rows
    // with the border-column dots e0 (even rows: column 0 of A^{-1}B) and e1
    // (odd rows: column 1).  v_j and d_j are fetched in increasing j.  Rows
    // 0, 1 and nz-2, nz-1 (incomplete bands) are peeled; the main loop takes
    // (even, odd) pairs so that the parity is static.
    auto st_window = [&](auto &&fetch_v, auto &&fetch_d, bool with_d, double &e0, double &e1) {
      double vm2 = 0.0, vm1 = 0.0, v0 = fetch_v(0), v1 = fetch_v(1);
      double dm1 = 0.0, d0 = with_d ? fetch_d(0) : 0.0, d1 = with_d ? fetch_d(1) : 0.0;
      const double *abp = ab0;
      // kind: 0 interior, 1 row 0, 2 row 1, 3 row nz-2, 4 row nz-1
      auto row = [&](int j, double v2, double d2, int kind, bool odd) {
        double x = S0[j] * v0;
        if (kind <= 2) x += SM2[j + 2] * v2;
        if (kind == 0 || kind >= 3) x += SP2[j - 2] * vm2;
        if (with_d) {
          if (kind != 4) x += FM1[j + 1] * d1;
          if (kind != 1) x += FP1[j - 1] * dm1;
        }
        XS(j) = x;
        const double t = __ldg(abp) * x;
        if (odd) e1 += t;
        else e0 += t;
        abp += nk;
        vm2 = vm1;
        vm1 = v0;
        v0 = v1;
        v1 = v2;
        dm1 = d0;
        d0 = d1;
        d1 = d2;
      };
      row(0, fetch_v(2), with_d ? fetch_d(2) : 0.0, 1, false);
      row(1, fetch_v(3), with_d ? fetch_d(3) : 0.0, 2, true);
      int j = 2;
#pragma unroll 2
      for (; j + 1 <= nz - 3; j += 2) {
        row(j, fetch_v(j + 2), with_d ? fetch_d(j + 2) : 0.0, 0, false);
        row(j + 1, fetch_v(j + 3), with_d ? fetch_d(j + 3) : 0.0, 0, true);
      }
      if (j <= nz - 3) {  // odd nz: one more even row
        row(j, fetch_v(j + 2), with_d ? fetch_d(j + 2) : 0.0, 0, false);
        ++j;
      }
      row(nz - 2, 0.0, 0.0, 3, ((nz - 2) & 1) != 0);
      row(nz - 1, 0.0, 0.0, 4, ((nz - 1) & 1) != 0);
    };
    auto no_d = [&](int) { return 0.0; };

    double bcbar[6];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      R *us = own + c * nz * rs;
      const double wbb = wb_bar[c], wtb = wt_bar[c];
      // x_bar = S^T u_bar, u_bar including the W^T term, then the border adjoints
      double e0 = 0.0, e1 = 0.0;
      auto fetch_u = [&](int j) { return ld_fp64(us + (size_t)j * rs) - ((j & 1) ? -wbb : wbb) - wtb; };
      const double ub0 = fetch_u(0), ub1 = fetch_u(1);
      st_window(fetch_u, no_d, false, e0, e1);
      const double gb0 = a.se0 * ub0 - e0, gb1 = a.se1 * ub1 - e1;
      const double r0 = G00 * gb0 + G10 * gb1, r1 = G01 * gb0 + G11 * gb1;
      bcbar[2 * c] = -r0;
      bcbar[2 * c + 1] = -r1;
      penta_t(r0, r1);  // XS = adjoint of rhs_c
      __syncwarp();
      if (c == 2) {
        double *dpw = DPb;
        R *fw = us;
#pragma unroll 4
        for (int j = 0; j < nz; ++j) {
          const double t = inv_eta * XS(j);
          *dpw = t;
          if (store) *fw = to_r<R>(-t);
          dpw += GT;
          fw += rs;
        }
      } else {
        const double coef = -sp * (c == 0 ? Dx : Dy) * inv_eta;
        double *cpw = CPb;
        R *fw = us;
#pragma unroll 4
        for (int j = 0; j < nz; ++j) {
          const double add = coef * XO(j);
          *cpw = (c == 0) ? add : *cpw + add;
          if (store) *fw = to_r<R>(-(inv_eta * XS(j)));
          cpw += GT;
          fw += rs;
        }
      }
      __syncwarp();
    }
    // bc adjoint -> ssum / asum adjoints; the forward's bc0 = -(i Dx ssum)/fac,
    // bc1 = (i Dx asum)/fac, bc2, bc3 likewise with Dy, bc4 = ssum/fac1,
    // bc5 = asum/fac1 (DPTools.cpp:218-234)
    const double fac1 = 2.0 * a.eta, fac = fac1 * K;
    const double ifac = 1.0 / fac, ifac1 = 1.0 / fac1;
    const double b0o = __shfl_xor_sync(0xffffffffu, bcbar[0], 1);
    const double b1o = __shfl_xor_sync(0xffffffffu, bcbar[1], 1);
    const double b2o = __shfl_xor_sync(0xffffffffu, bcbar[2], 1);
    const double b3o = __shfl_xor_sync(0xffffffffu, bcbar[3], 1);
    const double ssb = (sp * Dx * ifac) * b0o + (sp * Dy * ifac) * b2o + ifac1 * bcbar[4];
    const double asb = (-sp * Dx * ifac) * b1o + (-sp * Dy * ifac) * b3o + ifac1 * bcbar[5];
    // pressure: x_bar = S^T cp_bar + F^T dp_bar, border adjoints, A^{-T}
    {
      double e0 = 0.0, e1 = 0.0;
      auto fetch_c = [&](int j) { return CPb[(size_t)j * GT] + ssb + ((j & 1) ? -asb : asb); };
      auto fetch_dp = [&](int j) { return DPb[(size_t)j * GT]; };
      const double c0v = fetch_c(0), c1v = fetch_c(1), d0v = fetch_dp(0);
      st_window(fetch_c, fetch_dp, true, e0, e1);
      const double gb0 = a.se0 * c0v - e0;
      const double gb1 = a.se1 * c1v + a.fe * d0v - e1;
      const double r0 = G00 * gb0 + G10 * gb1, r1 = G01 * gb0 + G11 * gb1;
      penta_t(r0, r1);  // XS = adjoint of prhs
    }
    __syncwarp();
    // prhs adjoint -> f0 += -i Dx prb, f1 += -i Dy prb, f2 += D^T (df adjoint)
    // with df_j = sum_{i = j+1, j+3, ...} (2 i / H) f2_i and row 0 halved
    // (DPTools.cpp:134-174)
    if (store) {
      R *f0 = own, *f1 = own + nz * rs, *f2 = own + 2 * nz * rs;
      const double cx = -sp * Dx, cy = -sp * Dy;
      {
        const double prb_o = XO(0);
        *f0 = to_r<R>(ld_fp64(f0) + cx * prb_o);
        *f1 = to_r<R>(ld_fp64(f1) + cy * prb_o);
      }
      double em2 = 0.0, em1 = 0.5 * XS(0);  // e_0 = 0, e_1 = df_bar_0
#pragma unroll 4
      for (int j = 1; j < nz; ++j) {
        f0 += rs;
        f1 += rs;
        f2 += rs;
        const double prb_o = XO(j);
        *f0 = to_r<R>(ld_fp64(f0) + cx * prb_o);
        *f1 = to_r<R>(ld_fp64(f1) + cy * prb_o);
        const double e = em1;  // e_j
        *f2 = to_r<R>(ld_fp64(f2) + DH[j] * e);
        em1 = em2 + XS(j);  // e_{j+1} = e_{j-1} + df_bar_j
        em2 = e;
      }
    }
    __syncwarp();
  }
#undef XS
#undef XO
}

// k = 0 (walls): U_c = S [r; Gi C r] with r = -f_c/eta (c = 0, 1), U_2 = 0;
// open domain: zero.  Transposed in place; thread (part, j) owns row j.
constexpr int ADJ_K0_ROWS = 128;
template <typename R>
__global__ void __launch_bounds__(2 * ADJ_K0_ROWS) k_bvp_adj_k0(KsArgs a, R *__restrict__ spec) {
  __shared__ double U[2][ADJ_K0_ROWS];
  const int part = threadIdx.x / ADJ_K0_ROWS, j = threadIdx.x % ADJ_K0_ROWS;
  const int nz = a.nz;
  const int64_t nk = a.nk;
  auto at = [&](int d, int r) -> R & { return spec[(((int64_t)d * nz + r) * nk) * 2 + part]; };
  if (a.mode == 0) {
    if (j < nz)
      for (int d = 0; d < 3; ++d) at(d, j) = (R)0;
    return;
  }
  const double inv_eta = 1.0 / a.eta;
  for (int c = 0; c < 2; ++c) {
    if (j < nz) U[part][j] = (double)at(c, j);
    __syncthreads();
    if (j < nz) {
      double x = a.s0[j] * U[part][j];
      if (j + 2 < nz) x += a.sm2[j + 2] * U[part][j + 2];
      if (j >= 2) x += a.sp2[j - 2] * U[part][j - 2];
      const double gb0 = a.se0 * U[part][0], gb1 = a.se1 * U[part][1];
      // Gi row-major: g0 = Gi00 y0 + Gi01 y1, g1 = Gi10 y0 + Gi11 y1
      const double t0 = a.k0gi[0] * gb0 + a.k0gi[2] * gb1, t1 = a.k0gi[1] * gb0 + a.k0gi[3] * gb1;
      at(c, j) = (R)(-inv_eta * (x + a.k0c0[j] * t0 + a.k0c1[j] * t1));
    }
    __syncthreads();
  }
  if (j < nz) at(2, j) = (R)0;
}

template <typename R>
cudaError_t adj_plan(const KsArgs &a, int nsm, int64_t *grid, size_t *scratch_bytes) {
  const size_t smem = sizeof(double) * ((size_t)(a.nz + 2) * ADJ_LANES + 6 * (size_t)a.nz + 1);
  cudaError_t err = cudaFuncSetAttribute(k_bvp_adj_pairs<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  int per_sm = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bvp_adj_pairs<R>, ADJ_LANES, smem);
  if (err != cudaSuccess) return err;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int64_t g = (int64_t)nsm * per_sm;
  const int64_t warps_of_modes = (a.nk + 15) / 16;
  if (g > warps_of_modes) g = warps_of_modes;
  *grid = g;
  *scratch_bytes = sizeof(double) * 2 * (size_t)a.nz * (size_t)g * ADJ_LANES;
  return cudaSuccess;
}

template <typename R>
cudaError_t launch_adj_solve(const KsArgs &a, R *spec, const double2 *cadj, double *scratch, int64_t grid,
                             cudaStream_t s) {
  const size_t smem = sizeof(double) * ((size_t)(a.nz + 2) * ADJ_LANES + 6 * (size_t)a.nz + 1);
  const int64_t per = (a.nk + grid - 1) / grid;
  const int per_cta = (int)((per + 15) / 16 * 16);
  k_bvp_adj_pairs<R><<<(unsigned)grid, ADJ_LANES, smem, s>>>(a, spec, cadj, scratch, per_cta);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  k_bvp_adj_k0<R><<<1, 2 * ADJ_K0_ROWS, 0, s>>>(a, spec);
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_corr_adj(const KsArgs &a, const R *spec, double2 *cadj, cudaStream_t s) {
  if (a.mode == 0) return cudaSuccess;
  const int64_t threads = a.nk * CADJ_G;
  k_corr_adj<R><<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(a, spec, cadj);
  return cudaGetLastError();
}

// the k = 0 mode alone (after the double-float adjoint of the other modes)
template <typename R>
cudaError_t launch_adj_k0(const KsArgs &a, R *spec, cudaStream_t s) {
  k_bvp_adj_k0<R><<<1, 2 * ADJ_K0_ROWS, 0, s>>>(a, spec);
  return cudaGetLastError();
}
template cudaError_t launch_adj_k0<float>(const KsArgs &, float *, cudaStream_t);
template cudaError_t launch_adj_k0<double>(const KsArgs &, double *, cudaStream_t);

template cudaError_t adj_plan<float>(const KsArgs &, int, int64_t *, size_t *);
template cudaError_t adj_plan<double>(const KsArgs &, int, int64_t *, size_t *);
template cudaError_t launch_adj_solve<float>(const KsArgs &, float *, const double2 *, double *, int64_t,
                                             cudaStream_t);
template cudaError_t launch_adj_solve<double>(const KsArgs &, double *, const double2 *, double *, int64_t,
                                              cudaStream_t);
template cudaError_t launch_corr_adj<float>(const KsArgs &, const float *, double2 *, cudaStream_t);
template cudaError_t launch_corr_adj<double>(const KsArgs &, const double *, double2 *, cudaStream_t);

}  // namespace dpst
