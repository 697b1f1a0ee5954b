// Device helpers shared by the wavenumber-space kernels (dpst_kspace.cu,
// dpst_bvp.cu): complex arithmetic on double2, the Hermitian-partner test of
// a half-spectrum mode, and the slit-channel correction coefficients.
#pragma once
#include "dpst_internal.cuh"

namespace dpst {

static __device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
static __device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
static __device__ __forceinline__ double2 cscale(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
static __device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
static __device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
// i*k*a for real k
static __device__ __forceinline__ double2 cik(double k, double2 a) { return make_double2(-k * a.y, k * a.x); }

// FP32 <-> FP64 conversions with integer instructions, for kernels whose
// FP64 pipe is the bottleneck (GB300 executes FP64, conversions included, at
// a small fraction of its integer rate).
// f2d_int: exact for normal numbers, zeros, infinities and NaNs; FP32
// subnormals become signed zeros.
static __device__ __forceinline__ double f2d_int(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned sign = b & 0x80000000u;
  const unsigned e = (b >> 23) & 0xffu;
  const unsigned m = b & 0x7fffffu;
  const unsigned e2 = (e == 255u) ? 2047u : e + 896u;
  const unsigned hi = (e == 0u) ? sign : (sign | (e2 << 20) | (m >> 3));
  const unsigned lo = (e == 0u) ? 0u : (m << 29);
  return __hiloint2double((int)hi, (int)lo);
}
// d2f_int: round to nearest even, computed with integer instructions when the
// result is a normal FP32 number or overflows to infinity by rounding;
// every other input takes the hardware conversion.
static __device__ __forceinline__ float d2f_int(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const int e = (int)((hi >> 20) & 0x7ffu) - 896;
  if (e >= 1 && e <= 254) {
    const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rem = lo & 0x1fffffffu;
    unsigned r = ((unsigned)e << 23) | m;
    r += (rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) ? 1u : 0u;
    return __uint_as_float((hi & 0x80000000u) | r);
  }
  return __double2float_rn(d);
}
template <typename R>
static __device__ __forceinline__ double ld_fp64(const R *p) { return (double)*p; }
template <>
__device__ __forceinline__ double ld_fp64<float>(const float *p) { return f2d_int(*p); }
template <typename R>
static __device__ __forceinline__ R to_r(double v) { return (R)v; }
template <>
__device__ __forceinline__ float to_r<float>(double v) { return d2f_int(v); }

static __device__ __forceinline__ bool mode_is_hermitian(const KsArgs &a, int ix, int iy, double kx, double ky,
                                                  double &kxp, double &kyp) {
  int ixp = (a.nx - ix) % a.nx, iyp = (a.ny - iy) % a.ny;
  kxp = a.kvx[ixp];
  kyp = a.kvy[iyp];
  return (kxp == -kx) && (kyp == -ky);
}

// ---------------------------------------------------------------------------
// 8x8 complex solve with partial pivoting on |re|+|im| (the LAPACK zgesv
// pivot rule), column-major A.
// ---------------------------------------------------------------------------
static __device__ void zsolve8(double2 *A, double2 *x) {
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

// Matrix of the slit-channel correction system for wavevector (kx, ky),
// column-major 8x8 (DPTools.cpp:742-768).
static __device__ void slit_matrix(double kx, double ky, double Hs, double eta, double2 *A) {
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
}

// Slit correction coefficients for wavevector (kx, ky), wall values fb (z=0)
// and ft (z=Hs) (DPTools.cpp:731-788).
static __device__ void slit_coeffs(double kx, double ky, double Hs, double eta, const double2 fb[3],
                            const double2 ft[3], double2 c[8]) {
  double2 A[64];
  slit_matrix(kx, ky, Hs, eta, A);
  // x0 = -i kx fbx - i ky fby ; x1 likewise for the top
  c[0] = csub(cik(-kx, fb[0]), cik(ky, fb[1]));
  c[1] = csub(cik(-kx, ft[0]), cik(ky, ft[1]));
  c[2] = fb[0]; c[3] = fb[1]; c[4] = fb[2];
  c[5] = ft[0]; c[6] = ft[1]; c[7] = ft[2];
  zsolve8(A, c);
}

// Wall correction of one mode at node m for component d, evaluated in the
// operator's arithmetic CT (FP64 for the plain operator, FP32 for the mixed
// one); the coefficients themselves come from the FP64 solve.
template <typename CT>
struct cplx {
  CT x, y;
};
template <typename CT>
static __device__ __forceinline__ cplx<CT> mk(CT x, CT y) { cplx<CT> r; r.x = x; r.y = y; return r; }
template <typename CT>
static __device__ __forceinline__ cplx<CT> operator+(cplx<CT> a, cplx<CT> b) { return mk(a.x + b.x, a.y + b.y); }
template <typename CT>
static __device__ __forceinline__ cplx<CT> operator*(CT s, cplx<CT> a) { return mk(s * a.x, s * a.y); }
template <typename CT>
static __device__ __forceinline__ cplx<CT> ik(CT k, cplx<CT> a) { return mk(-k * a.y, k * a.x); }
template <typename CT>
static __device__ __forceinline__ cplx<CT> conj(cplx<CT> a) { return mk(a.x, -a.y); }
template <typename CT>
static __device__ __forceinline__ cplx<CT> ld(const double2 &v) { return mk((CT)v.x, (CT)v.y); }

template <typename R>
static __device__ __forceinline__ void corr_value(const EpiArgs &e, int d, int m, int64_t mode, R &re, R &im) {
  typedef R CT;
  re = 0;
  im = 0;
  const KsArgs &a = e.ks;
  if (a.mode == 0 || mode == 0) return;
  const int ix = (int)(mode % a.nxh), iy = (int)(mode / a.nxh);
  const double kxd = a.kvx[ix], kyd = a.kvy[iy];
  double kxpd, kypd;
  const bool herm = mode_is_hermitian(a, ix, iy, kxd, kyd, kxpd, kypd);
  const CT k = (CT)sqrt(kxd * kxd + kyd * kyd);
  const CT z = (CT)a.zn[m];
  const double2 *cr = e.corr + mode * 16;
  const CT enkz = exp(-k * z);
  const CT zenkz = z * enkz;
  cplx<CT> acc = mk<CT>(0, 0);
  const int npass = herm ? 1 : 2;
  for (int pass = 0; pass < npass; ++pass) {
    const CT qx = (CT)(pass ? kxpd : kxd), qy = (CT)(pass ? kypd : kyd);
    cplx<CT> v;
    if (a.mode == 1) {
      // DPTools.cpp:627-641, velocity rows
      cplx<CT> f0 = ld<CT>(cr[0]), f1 = ld<CT>(cr[1]), f2 = ld<CT>(cr[2]);
      if (pass) { f0 = conj(f0); f1 = conj(f1); f2 = conj(f2); }
      const cplx<CT> al = (qx * f0 + qy * f1) + ik(k, f2);
      if (d == 0) v = (-qx * zenkz / k) * al + enkz * f0;
      else if (d == 1) v = (-qy * zenkz / k) * al + enkz * f1;
      else v = ik(-zenkz, al) + enkz * f2;
    } else {
      // DPTools.cpp:795-815 with e^{k(z-H)} evaluated directly
      const double2 *c = cr + 8 * pass;
      const CT fac = (CT)(1.0 / 2.0 / a.eta);
      const CT ekzmh = exp(k * (z - (CT)a.Lz));
      const CT zekzmh = z * ekzmh;
      if (d == 0)
        v = (ik(-qx * zenkz * fac / k, ld<CT>(c[0])) + ik(qx * zekzmh * fac / k, ld<CT>(c[1]))) +
            (enkz * ld<CT>(c[2]) + ekzmh * ld<CT>(c[3]));
      else if (d == 1)
        v = (ik(-qy * zenkz * fac / k, ld<CT>(c[0])) + ik(qy * zekzmh * fac / k, ld<CT>(c[1]))) +
            (enkz * ld<CT>(c[4]) + ekzmh * ld<CT>(c[5]));
      else
        v = ((zenkz * fac) * ld<CT>(c[0]) + (zekzmh * fac) * ld<CT>(c[1])) +
            (enkz * ld<CT>(c[6]) + ekzmh * ld<CT>(c[7]));
    }
    if (pass) v = conj(v);
    acc = acc + v;
  }
  if (npass == 2) acc = (CT)0.5 * acc;
  re = acc.x;
  im = acc.y;
}

// corr_value of the mixed operator from FP32 tables only (EpiArgs' corrf,
// cmode, znf): the same values as corr_value<float> (every FP64 input there
// is rounded to FP32 before use), without its per-element FP64 work
// (wavenumber lookups, square root, conversions), which runs at 1/64 of the
// FP32 rate on this GPU.
static __device__ __forceinline__ void corr_value_f(const EpiArgs &e, int d, int m, int64_t mode, float &re,
                                                    float &im) {
  typedef float CT;
  re = 0;
  im = 0;
  const KsArgs &a = e.ks;
  if (a.mode == 0 || mode == 0) return;
  const float4 m0 = e.cmode[2 * mode];
  const CT k = m0.x;
  const CT z = e.znf[m];
  const float2 *cr = e.corrf + mode * 16;
  const CT enkz = expf(-k * z);
  const CT zenkz = z * enkz;
  cplx<CT> acc = mk<CT>(0, 0);
  const int npass = m0.w != 0.0f ? 1 : 2;
  for (int pass = 0; pass < npass; ++pass) {
    CT qx = m0.y, qy = m0.z;
    if (pass) {
      const float4 m1 = e.cmode[2 * mode + 1];
      qx = m1.x;
      qy = m1.y;
    }
    cplx<CT> v;
    if (a.mode == 1) {
      cplx<CT> f0 = mk<CT>(cr[0].x, cr[0].y), f1 = mk<CT>(cr[1].x, cr[1].y), f2 = mk<CT>(cr[2].x, cr[2].y);
      if (pass) { f0 = conj(f0); f1 = conj(f1); f2 = conj(f2); }
      const cplx<CT> al = (qx * f0 + qy * f1) + ik(k, f2);
      if (d == 0) v = (-qx * zenkz / k) * al + enkz * f0;
      else if (d == 1) v = (-qy * zenkz / k) * al + enkz * f1;
      else v = ik(-zenkz, al) + enkz * f2;
    } else {
      const float2 *c = cr + 8 * pass;
      auto C = [&](int r) { return mk<CT>(c[r].x, c[r].y); };
      const CT fac = e.fac;
      const CT ekzmh = expf(k * (z - (CT)a.Lz));
      const CT zekzmh = z * ekzmh;
      if (d == 0)
        v = (ik(-qx * zenkz * fac / k, C(0)) + ik(qx * zekzmh * fac / k, C(1))) + (enkz * C(2) + ekzmh * C(3));
      else if (d == 1)
        v = (ik(-qy * zenkz * fac / k, C(0)) + ik(qy * zekzmh * fac / k, C(1))) + (enkz * C(4) + ekzmh * C(5));
      else
        v = ((zenkz * fac) * C(0) + (zekzmh * fac) * C(1)) + (enkz * C(6) + ekzmh * C(7));
    }
    if (pass) v = conj(v);
    acc = acc + v;
  }
  if (npass == 2) acc = (CT)0.5 * acc;
  re = acc.x;
  im = acc.y;
}

// The correction at (component d, node m, mode): from the FP32 tables when
// the epilogue has them (mixed operator), else corr_value.
template <typename R>
static __device__ __forceinline__ void corr_any(const EpiArgs &e, int d, int m, int64_t mode, R &re, R &im) {
  if constexpr (sizeof(R) == 4) {
    if (e.corrf != nullptr) {
      corr_value_f(e, d, m, mode, re, im);
      return;
    }
  }
  corr_value<R>(e, d, m, mode, re, im);
}

}  // namespace dpst
