// Double-float arithmetic ("df64") for the per-wavenumber solve of the mixed
// operator.
//
// A value is the unevaluated sum hi + lo of two FP32 numbers with
// |lo| <= ulp(hi) / 2: about 48 significant bits (relative rounding error
// near 2^-48 = 3.6e-15 per operation, against 2^-53 for FP64), with FP32's
// exponent range.  GB300 executes FP64 at 1/64 of its FP32 rate, so a
// double-float operation of 5-15 FP32 instructions on the FP32 pipe is
// several times faster than the FP64 operation it replaces.
//
// Building blocks (published algorithms, written here from their
// definitions):
//   two_sum     Knuth's TwoSum: s + e = a + b exactly (6 operations);
//   fast_two_sum Dekker's Fast2Sum, exact when the exponent of a is not
//               below the exponent of b (3 operations);
//   products    the FMA form of Dekker's TwoProduct: p + e = a * b exactly
//               for p = fl(a b), e = fma(a, b, -p) (2 operations);
//   df_mul      a double-word product with the lo * lo term dropped
//               (Joldes, Muller, Popescu, "Tight and rigorous error bounds
//               for basic building blocks of double-word arithmetic", ACM
//               TOMS 44(2), 2017, algorithm DWTimesDW with FMA);
//   df_add      their "sloppy" double-word sum: the error is bounded
//               relative to |a| + |b| (not to |a + b| when the operands
//               cancel), the same kind of bound FP64 gives an unfused
//               multiply-add;
//   df_fma      a * b + c as the FMA-based product of hi parts plus both
//               cross terms, added to c with one TwoSum and renormalised
//               once (15 operations; error ~ 2^-48 (|a b| + |c|)).
// Every step uses the round-to-nearest intrinsics (__fadd_rn, __fmul_rn,
// __fmaf_rn), which the compiler never contracts or reassociates, so the
// error-free transformations stay exact.
#pragma once
#include <cuda_runtime.h>

namespace dpst {

struct df64 {
  float hi, lo;
};

static __device__ __forceinline__ df64 df_make(float h, float l) {
  df64 r;
  r.hi = h;
  r.lo = l;
  return r;
}
static __device__ __forceinline__ df64 df_zero() { return df_make(0.0f, 0.0f); }
static __device__ __forceinline__ df64 df_from_f(float x) { return df_make(x, 0.0f); }
// nearest double-float to a double (hi = fl32(x), lo = fl32(x - hi))
static __device__ __forceinline__ df64 df_from_d(double x) {
  const float h = __double2float_rn(x);
  return df_make(h, __double2float_rn(x - (double)h));
}
static __device__ __forceinline__ double df_to_d(df64 a) { return (double)a.hi + (double)a.lo; }
static __device__ __forceinline__ float df_to_f(df64 a) { return __fadd_rn(a.hi, a.lo); }
static __device__ __forceinline__ df64 df_ld(const float2 *p) {
  const float2 v = __ldg(p);
  return df_make(v.x, v.y);
}
static __device__ __forceinline__ df64 df_lds(const float2 &v) { return df_make(v.x, v.y); }
static __device__ __forceinline__ float2 df_f2(df64 a) { return make_float2(a.hi, a.lo); }

static __device__ __forceinline__ df64 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df_make(s, e);
}
static __device__ __forceinline__ df64 fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return df_make(s, __fsub_rn(b, __fsub_rn(s, a)));
}

static __device__ __forceinline__ df64 df_neg(df64 a) { return df_make(-a.hi, -a.lo); }
// exact scaling by a power of two
static __device__ __forceinline__ df64 df_scale2(df64 a, float p2) { return df_make(a.hi * p2, a.lo * p2); }

static __device__ __forceinline__ df64 df_add(df64 a, df64 b) {
  const df64 s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
static __device__ __forceinline__ df64 df_add(df64 a, float b) {
  const df64 s = two_sum(a.hi, b);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}
static __device__ __forceinline__ df64 df_sub(df64 a, df64 b) { return df_add(a, df_neg(b)); }
static __device__ __forceinline__ df64 df_sub(df64 a, float b) { return df_add(a, -b); }

static __device__ __forceinline__ df64 df_mul(df64 a, df64 b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
static __device__ __forceinline__ df64 df_mul(df64 a, float b) {
  const float p = __fmul_rn(a.hi, b);
  float e = __fmaf_rn(a.hi, b, -p);
  e = __fmaf_rn(a.lo, b, e);
  return fast_two_sum(p, e);
}

// a * b + c
static __device__ __forceinline__ df64 df_fma(df64 a, df64 b, df64 c) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const df64 s = two_sum(p, c.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(e, c.lo)));
}
static __device__ __forceinline__ df64 df_fma(df64 a, float b, df64 c) {
  const float p = __fmul_rn(a.hi, b);
  float e = __fmaf_rn(a.hi, b, -p);
  e = __fmaf_rn(a.lo, b, e);
  const df64 s = two_sum(p, c.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(e, c.lo)));
}
// c - a * b
static __device__ __forceinline__ df64 df_fnma(df64 a, df64 b, df64 c) { return df_fma(df_neg(a), b, c); }
// a * b - c for an FP32 or double-float c
static __device__ __forceinline__ df64 df_fms(df64 a, df64 b, float c) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const df64 s = two_sum(p, -c);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, e));
}
static __device__ __forceinline__ df64 df_fms(df64 a, df64 b, df64 c) { return df_fma(a, b, df_neg(c)); }

// Compensated accumulator of a sum of double-float terms or products (the
// scheme of Ogita, Rump and Oishi's Dot2): the hi parts are summed with
// TwoSum and every rounding error and lo part is collected in one FP32
// correction, normalised once at the end; 8 (sum) or 12 (product)
// operations per term instead of 10 or 15 for a renormalised double-float.
struct df_acc {
  float s, e;
};
static __device__ __forceinline__ df_acc acc_zero() {
  df_acc a;
  a.s = 0.0f;
  a.e = 0.0f;
  return a;
}
static __device__ __forceinline__ void acc_add(df_acc &a, df64 x) {
  const df64 t = two_sum(a.s, x.hi);
  a.s = t.hi;
  a.e = __fadd_rn(a.e, __fadd_rn(t.lo, x.lo));
}
static __device__ __forceinline__ void acc_fma(df_acc &a, df64 x, df64 y) {
  const float p = __fmul_rn(x.hi, y.hi);
  float e = __fmaf_rn(x.hi, y.hi, -p);
  e = __fmaf_rn(x.hi, y.lo, e);
  e = __fmaf_rn(x.lo, y.hi, e);
  const df64 t = two_sum(a.s, p);
  a.s = t.hi;
  a.e = __fadd_rn(a.e, __fadd_rn(t.lo, e));
}
static __device__ __forceinline__ df64 acc_val(df_acc a) { return two_sum(a.s, a.e); }

static __device__ __forceinline__ df64 df_shfl_xor(df64 a, int m) {
  return df_make(__shfl_xor_sync(0xffffffffu, a.hi, m), __shfl_xor_sync(0xffffffffu, a.lo, m));
}

// Spectrum elements as operands: FP32 elements enter the FP32-operand forms
// directly; FP64 elements (the FP64-I/O instantiation used to compare the
// solve with the FP64 one) are rounded to double-float first.
static __device__ __forceinline__ float df_in(const float *p) { return *p; }
static __device__ __forceinline__ df64 df_in(const double *p) { return df_from_d(*p); }
static __device__ __forceinline__ void df_out(float *p, df64 v) { *p = df_to_f(v); }
static __device__ __forceinline__ void df_out(double *p, df64 v) { *p = df_to_d(v); }

}  // namespace dpst
