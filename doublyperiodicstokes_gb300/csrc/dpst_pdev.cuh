// Device helpers shared by the particle-side kernels of the forward
// operator (dpst_particles.cu) and of its backward pass (dpst_grad.cu): the
// 1-D ES factor and its derivatives, the z-index map that applies the
// reference's ghost fold / copy rules (BoundaryConditions.h:22-731), and the
// grid read with those rules.
#pragma once
#include "dpst_internal.cuh"

namespace dpst {

static __device__ __forceinline__ int wrapi(int i, int n) {
  int r = i % n;
  return r < 0 ? r + n : r;
}

static __device__ __forceinline__ double es1(double x, double beta, double alpha2) {
  return exp(beta * (sqrt(1.0 - x * x / alpha2) - 1.0));
}

static __device__ __forceinline__ double des1(double x, double beta, double alpha2) {
  double s = sqrt(1.0 - x * x / alpha2);
  return -beta * x * exp(beta * (s - 1.0)) / (alpha2 * s);
}

// The factor and its derivative in a stencil's storage type R: FP64 for
// the FP64 operator (the reference's arithmetic); for the mixed operator the
// offset (computed in FP64) is rounded to FP32 and the factor evaluated in
// FP32, as the stored weights are FP32 anyway (FP64 exp and sqrt run at a
// small fraction of the FP32 rate on this GPU).  The clamped offset of an
// out-of-support node equals the threshold, so 1 - o^2/alpha^2 may round
// below 0 in FP32: it is clamped at 0 (the factor there is exp(-beta)).
template <typename R>
static __device__ __forceinline__ R es1r(double o, const KernelDesc &kd) {
  if constexpr (sizeof(R) == 8) {
    return es1(o, kd.beta, kd.alpha2);
  } else {
    const float x = (float)o, a2 = (float)kd.alpha2, b = (float)kd.beta;
    const float q = fmaxf(0.0f, 1.0f - x * x / a2);
    return expf(b * (sqrtf(q) - 1.0f));
  }
}

template <typename R>
static __device__ __forceinline__ R des1r(double o, const KernelDesc &kd) {
  if constexpr (sizeof(R) == 8) {
    return des1(o, kd.beta, kd.alpha2);
  } else {
    const float x = (float)o, a2 = (float)kd.alpha2, b = (float)kd.beta;
    const float s = sqrtf(fmaxf(0.0f, 1.0f - x * x / a2));
    return (s > 0.0f) ? -b * x * expf(b * (s - 1.0f)) / (a2 * s) : 0.0f;
  }
}

// es_pos_derivs for the mixed operator's FP32 stencils: 1 - o^2/alpha^2 in
// FP64 (it cancels near the support's edge; o^2 times the FP64 reciprocal
// 1/alpha^2 rather than an FP64 division, which costs dozens of FP64-pipe
// instructions), the square root, exponential and quotients in FP32.
static __device__ __forceinline__ void es_pos_derivs_f(double o, double beta, double alpha2, double inv_alpha2,
                                                       float &g1, float &g2) {
  const double qd = o * o * inv_alpha2;
  const double s2d = 1.0 - qd;
  if (!(s2d > 0.0)) {
    g1 = 0.0f;
    g2 = 0.0f;
    return;
  }
  const float x = (float)o, a2 = (float)alpha2, b = (float)beta;
  const float s2 = (float)s2d, q = (float)qd, s = sqrtf(s2);
  const float phi = expf(b * (s - 1.0f));
  g1 = b * x * phi / (a2 * s);
  g2 = (b / a2) * phi * (1.0f / s - b * q / s2 + q / (s2 * s));
}

// Position derivatives of one stencil factor.  The forward evaluates
// phi(o) (and phi'(o) for the dipole kernel) at o = node - x, so
// d/dx phi(o) = -phi'(o) -> g1 and d/dx phi'(o) = -phi''(o) -> g2, with
//   phi'  = -beta o phi / (alpha^2 s),  s = sqrt(1 - o^2/alpha^2),
//   phi'' = -(beta/alpha^2) phi (1/s - beta o^2/(alpha^2 s^2) + o^2/(alpha^2 s^3)).
// At |o| = alpha (s = 0) the one-sided derivative is unbounded; 0 is
// returned there.
static __device__ __forceinline__ void es_pos_derivs(double o, double beta, double alpha2, double &g1,
                                                     double &g2) {
  const double s2 = 1.0 - o * o / alpha2;
  if (!(s2 > 0.0)) {
    g1 = 0.0;
    g2 = 0.0;
    return;
  }
  const double s = sqrt(s2);
  const double phi = exp(beta * (s - 1.0));
  const double q = o * o / alpha2;
  g1 = beta * o * phi / (alpha2 * s);
  g2 = (beta / alpha2) * phi * (1.0 / s - beta * q / s2 + q / (s2 * s));
}

// Where extended z index kk lands on the interior grid under one BC set.
// Returns the interior index m (descending z, m = 0 at zmax; for a periodic
// uniform z grid ascending, m = 0 at zmin) and the weight
// (1 interior, s at a folded ghost, 1+s at an active boundary node).  A
// ghost layer at an inactive end returns m = -1 (top) or -2 (bottom) and its
// level in the ghost buffer.
struct ZMap {
  int m;
  int level;
  double wgt;
};

static __device__ __forceinline__ ZMap zmap(int kk, int dend, int nz, const ZEnds &b) {
  ZMap r;
  r.level = 0;
  if (b.periodic) {  // BoundaryConditions.h:241-283, 608-647: wrap by nz
    r.m = kk - dend;
    if (r.m < 0) r.m += nz;
    else if (r.m >= nz) r.m -= nz;
    r.wgt = 1.0;
    return r;
  }
  const int ubeg = dend + nz;
  if (kk < dend) {
    if (b.top_active) { r.m = dend - kk; r.wgt = b.s_top; }
    else { r.m = -1; r.level = kk; r.wgt = 1.0; }
  } else if (kk >= ubeg) {
    if (b.bot_active) { r.m = 2 * nz + dend - 2 - kk; r.wgt = b.s_bot; }
    else { r.m = -2; r.level = kk - ubeg; r.wgt = 1.0; }
  } else {
    r.m = kk - dend;
    r.wgt = 1.0;
    if (r.m == 0 && b.top_active) r.wgt = 1.0 + b.s_top;
    if (r.m == nz - 1 && b.bot_active) r.wgt = 1.0 + b.s_bot;
  }
  return r;
}

template <typename R>
static __device__ __forceinline__ void atomic_add(R *a, R v) { atomicAdd(a, v); }

// Value of component d at extended z index kk for a particle column, with the
// reference's ghost copy applied (BoundaryConditions.h:377-731): interior and
// active-end layers come from the interior grid (periodic in x, y, mirrored
// with sign at walls, boundary node times 1+s); inactive-end ghost layers come
// from the ghost buffer at the extended column (ie, je).
template <typename R>
static __device__ __forceinline__ void grid_value3(const R *__restrict__ grid, const ZMap &zm, int64_t col,
                                            int64_t plane, int64_t comp, const Ghosts<R> &gh,
                                            const KernelDesc &kd, int ie, int je, R out[3]) {
  if (zm.m >= 0) {
    const R *src = grid + zm.m * plane + col;
    const R w = (R)zm.wgt;
    out[0] = w * src[0];
    out[1] = w * src[comp];
    out[2] = w * src[2 * comp];
  } else {
    const R *buf = (zm.m == -1) ? gh.top : gh.bot;
    if (buf == nullptr || ie < 0 || ie >= kd.nxeff || je < 0 || je >= kd.nyeff) {
      out[0] = out[1] = out[2] = (R)0;
      return;
    }
    const R *src = buf + (((int64_t)zm.level * kd.nyeff + je) * kd.nxeff + ie) * 3;
    out[0] = src[0];
    out[1] = src[1];
    out[2] = src[2];
  }
}

template <typename R>
static __device__ __forceinline__ R warp_sum(R v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace dpst
