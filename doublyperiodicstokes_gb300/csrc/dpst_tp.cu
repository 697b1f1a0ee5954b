// Triply periodic operator (DPST_MODE_PERIODIC): the reference's CPU domType
// 'TP' (FCM.py:149-441 with Transformer type fourier and the TP solver) and
// the mode 'periodic' of its GPU module (uammd_wrapper.cu:122-126).
//
// Mdot pipeline:
//   zero grid -> spread F (+ torque curl) with z wrapped like x and y
//   -> 3-D real FFT -> Fourier-space Stokes solve (one thread per mode)
//   -> inverse 3-D real FFT -> interpolate V (+ W).
// The particle kernels are the ones of the doubly periodic geometries
// (dpst_particles.cu) with a uniform z window (ParticleList.cpp:285-366) and
// the periodic z map; the grid layout is [3][nz][ny][nx] with z ascending
// from zmin (node m at zmin + m hz).
//
// Reference behaviour restated (source/cpu of stochasticHydroTools/
// DoublyPeriodicStokes):
//   wavenumbers   Solvers.py:197-222 (FFT order, 2 pi m / L; the unpaired
//                 Nyquist plane of an even axis zeroed in the derivative but
//                 kept in |k|^2)
//   solve         TPTools.cpp:6-46: p = -(Dx f + Dy g + Dz h) / |k|^2,
//                 u = (f - Dx p) / (eta |k|^2), k = 0 left at zero
//   transforms    Transform.cpp:109-117 (unnormalised forward), 273-281
//                 (backward divided by Nx Ny Nz); the real part is kept, so
//                 the Hermitian half spectrum of a real-to-complex transform
//                 carries the same result.
#include <cuda_runtime.h>
#include <cufft.h>

#include <climits>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/dpstokes_gb300.h"
#include "dpst_host.cuh"
#include "dpst_internal.cuh"
#include "dpst_launch.cuh"

namespace dpst {
bool own_fft_df_supported(int nx, int ny);
std::vector<float4> fft_twiddles_df(int n);
cudaError_t fft_setup_df(int nx, int ny);
cudaError_t fft_rows_df(bool inverse, const double *grid_in, double2 *spec_out, const double2 *spec_in,
                        double *grid_out, int nx, int64_t rows, const float4 *twx, cudaStream_t s);
cudaError_t fft_cols_df(bool inverse, double2 *spec, int ny, int nxh, int64_t planes, const float4 *twy,
                        cudaStream_t s);
}  // namespace dpst

namespace dpst {

// backward-pass kernels (dpst_grad.cu)
template <typename R>
void launch_locate_grad(bool dipole, const double *pos, int64_t N, const KernelDesc &kd, const double *zext,
                        const double *wext, const GridArgs &g, const Stencils<R> &st, const GradStencils<R> &gs,
                        cudaStream_t s);
template <typename R, typename RG>
void launch_adj_spread_dip(const RG *gW, int64_t N, const KernelDesc &kd, const GridArgs &g, const Stencils<R> &st,
                           R *grid, const Ghosts<R> &gh, cudaStream_t s);
template <typename R, typename RF>
void launch_gather_mono(const R *u, const R *psi, int64_t N, const KernelDesc &kd, const GridArgs &g,
                        const Stencils<R> &st, const GradStencils<R> &gs, const Ghosts<R> &ghu,
                        const Ghosts<R> &ghp, const RF *F, const RF *gV, RF *gF, RF *gX, cudaStream_t s);
template <typename R, typename RF>
void launch_gather_dip(const R *u, const R *psi, int64_t N, const KernelDesc &kd, const GridArgs &g,
                       const Stencils<R> &st, const GradStencils<R> &gs, const Ghosts<R> &ghu,
                       const Ghosts<R> &ghp, const RF *T, const RF *gW, RF *gT, RF *gX, cudaStream_t s);

template <typename R>
struct Cplx;
template <>
struct Cplx<float> {
  typedef float2 T;
};
template <>
struct Cplx<double> {
  typedef double2 T;
};

// One thread per mode of the half spectrum [3][nz][ny][nxh] (component
// stride M = nz ny nxh), in place.  scale = 1 / (nx ny nz) folds the inverse
// transform's normalisation into the solve.
template <typename R>
__global__ void k_tp_solve(typename Cplx<R>::T *__restrict__ spec, int64_t M, int nx, int ny, int nz, int nxh,
                           const double *__restrict__ kvx, const double *__restrict__ kvy,
                           const double *__restrict__ kvz, R eta, R scale) {
  typedef typename Cplx<R>::T C;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= M) return;
  C *u = spec + t;
  if (t == 0) {  // k = 0: the net force on the cell is ignored
    const C z = {(R)0, (R)0};
    u[0] = z;
    u[M] = z;
    u[2 * M] = z;
    return;
  }
  const int ix = (int)(t % nxh);
  const int64_t r = t / nxh;
  const int iy = (int)(r % ny), iz = (int)(r / ny);
  const R kx = (R)__ldg(kvx + ix), ky = (R)__ldg(kvy + iy), kz = (R)__ldg(kvz + iz);
  const R dx = (2 * ix == nx) ? (R)0 : kx;
  const R dy = (2 * iy == ny) ? (R)0 : ky;
  const R dz = (2 * iz == nz) ? (R)0 : kz;
  const R ksq = kx * kx + ky * ky + kz * kz;
  const C f = u[0], g = u[M], h = u[2 * M];
  // p = -(i dx f + i dy g + i dz h) / ksq
  const R pr = (dx * f.y + dy * g.y + dz * h.y) / ksq;
  const R pi = -(dx * f.x + dy * g.x + dz * h.x) / ksq;
  const R v = scale / (eta * ksq);
  C a, b, c;
  a.x = v * (f.x + dx * pi);
  a.y = v * (f.y - dx * pr);
  b.x = v * (g.x + dy * pi);
  b.y = v * (g.y - dy * pr);
  c.x = v * (h.x + dz * pi);
  c.y = v * (h.y - dz * pr);
  u[0] = a;
  u[M] = b;
  u[2 * M] = c;
}

// The regular-kernel torque coupling (FCM.py:372-396, 427-439, Solvers.py:
// 139-156): with torques, 1/2 curl of the torque spectrum t (tspec) is added
// to the force spectrum first; after the solve, u goes to spec and the
// vorticity 1/2 curl u to tspec (both scaled like u).  curl c = (Dy cz - Dz cy,
// Dz cx - Dx cz, Dx cy - Dy cx) with the same zeroed Nyquist planes.
template <typename R>
__global__ void k_tp_solve_reg(typename Cplx<R>::T *__restrict__ spec, typename Cplx<R>::T *__restrict__ tspec,
                               int torque, int64_t M, int nx, int ny, int nz, int nxh, const double *__restrict__ kvx,
                               const double *__restrict__ kvy, const double *__restrict__ kvz, R eta, R scale) {
  typedef typename Cplx<R>::T C;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= M) return;
  C *u = spec + t, *w = tspec + t;
  if (t == 0) {
    const C z = {(R)0, (R)0};
    u[0] = z; u[M] = z; u[2 * M] = z;
    w[0] = z; w[M] = z; w[2 * M] = z;
    return;
  }
  const int ix = (int)(t % nxh);
  const int64_t r = t / nxh;
  const int iy = (int)(r % ny), iz = (int)(r / ny);
  const R kx = (R)__ldg(kvx + ix), ky = (R)__ldg(kvy + iy), kz = (R)__ldg(kvz + iz);
  const R dx = (2 * ix == nx) ? (R)0 : kx;
  const R dy = (2 * iy == ny) ? (R)0 : ky;
  const R dz = (2 * iz == nz) ? (R)0 : kz;
  const R ksq = kx * kx + ky * ky + kz * kz;
  const R half = (R)0.5;
  // 1/2 curl of (a, b, c) with D = i k: i (dy c - dz b, dz a - dx c, dx b - dy a) / 2
  auto curl = [&](const C &a, const C &b, const C &c, C &x, C &y, C &z) {
    x.x = half * (-dy * c.y - (-dz * b.y)); x.y = half * (dy * c.x - dz * b.x);
    y.x = half * (-dz * a.y - (-dx * c.y)); y.y = half * (dz * a.x - dx * c.x);
    z.x = half * (-dx * b.y - (-dy * a.y)); z.y = half * (dx * b.x - dy * a.x);
  };
  C f = u[0], g = u[M], h = u[2 * M];
  if (torque) {
    C cx, cy, cz;
    curl(w[0], w[M], w[2 * M], cx, cy, cz);
    f.x += cx.x; f.y += cx.y;
    g.x += cy.x; g.y += cy.y;
    h.x += cz.x; h.y += cz.y;
  }
  const R pr = (dx * f.y + dy * g.y + dz * h.y) / ksq;
  const R pi = -(dx * f.x + dy * g.x + dz * h.x) / ksq;
  const R v = scale / (eta * ksq);
  C a, b, c;
  a.x = v * (f.x + dx * pi);
  a.y = v * (f.y - dx * pr);
  b.x = v * (g.x + dy * pi);
  b.y = v * (g.y - dy * pr);
  c.x = v * (h.x + dz * pi);
  c.y = v * (h.y - dz * pr);
  u[0] = a; u[M] = b; u[2 * M] = c;
  C ox, oy, oz;
  curl(a, b, c, ox, oy, oz);
  w[0] = ox; w[M] = oy; w[2 * M] = oz;
}

// ---------------------------------------------------------------------------
// Fused z transform and solve (nz = R1 x R2, powers of two up to 64): after
// the x-y real transforms of every z plane, one CTA takes ZF_CB consecutive
// columns (kx, ky) of all three components into shared memory, transforms
// each column along z (two passes of small DFTs in registers: n = R2 n1 +
// n2, k = k1 + R1 k2; pass 1 DFT_R1 over n1 and the twiddle W^(n2 k1), pass
// 2 DFT_R2 over n2, each thread writing back the slots it read, so the
// spectrum ends in digit-reversed order: slot R2 k1 + k2 holds kz = k1 + R1
// k2), solves every (kz, column) mode, transforms back in the reverse order
// (unnormalised; the 1/(nx ny nz) is in the solve) and stores.  The same
// arithmetic as the 3-D transform's z passes plus k_tp_solve, with one read
// and one write of the spectrum instead of three of each.
// ---------------------------------------------------------------------------
constexpr int ZF_CB = 16;  // columns per CTA

template <typename C>
static __device__ __forceinline__ C cadd(C a, C b) { return C{a.x + b.x, a.y + b.y}; }
template <typename C>
static __device__ __forceinline__ C csub(C a, C b) { return C{a.x - b.x, a.y - b.y}; }
template <typename C>
static __device__ __forceinline__ C cmul(C a, C b) { return C{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
template <typename C>
static __device__ __forceinline__ C cmulc(C a, C b) { return C{a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y}; }  // a conj(b)

template <int N>
static constexpr int bitrev(int i) {
  int r = 0;
  for (int b = 1; b < N; b <<= 1) r = (r << 1) | ((i & b) ? 1 : 0);
  return r;
}

// b W_8^e (forward) or b conj(W_8^e) (INV) for W_8 = exp(-2 pi i / 8),
// e = 0..3, without a table: W_8^2 = -i, W_8^(1, 3) = (+-1 - i) / sqrt(2).
template <typename C, int E, bool INV>
static __device__ __forceinline__ C mul_w8(C b) {
  typedef decltype(b.x) R;
  const R c = (R)0.70710678118654752440;  // 1 / sqrt(2)
  if (E == 0) return b;
  if (E == 2) return INV ? C{-b.y, b.x} : C{b.y, -b.x};
  if (E == 1) return INV ? C{c * (b.x - b.y), c * (b.x + b.y)} : C{c * (b.x + b.y), c * (b.y - b.x)};
  return INV ? C{-c * (b.x + b.y), c * (b.x - b.y)} : C{c * (b.y - b.x), -c * (b.x + b.y)};
}

// In-place DFT of N (2, 4 or 8) values in registers, natural order in and
// out.  INV: the unnormalised inverse.  Iterative radix-2 with the input
// taken in bit-reversed order; the twiddles W_len^k = W_8^(k 8 / len) are
// applied by mul_w8 (indices and exponents are compile-time constants).
template <typename C, int N, bool INV>
static __device__ __forceinline__ void dft_small(C (&v)[N]) {
  static_assert(N == 2 || N == 4 || N == 8, "small DFT sizes");
  C u[N];
#pragma unroll
  for (int i = 0; i < N; ++i) u[i] = v[bitrev<N>(i)];
#pragma unroll
  for (int len = 2; len <= N; len <<= 1) {
#pragma unroll
    for (int i = 0; i < N; i += len) {
#pragma unroll
      for (int k = 0; k < len / 2; ++k) {
        const int e = k * (8 / len);
        C b = u[i + k + len / 2];
        b = (e == 0) ? b : (e == 1) ? mul_w8<C, 1, INV>(b) : (e == 2) ? mul_w8<C, 2, INV>(b) : mul_w8<C, 3, INV>(b);
        const C a = u[i + k];
        u[i + k] = cadd(a, b);
        u[i + k + len / 2] = csub(a, b);
      }
    }
  }
#pragma unroll
  for (int i = 0; i < N; ++i) v[i] = u[i];
}

// NS = 3: the force spectrum (derivative-kernel coupling).  NS = 6 (the
// regular-kernel coupling): the force spectrum in spec and the torque
// spectrum in tspec; with torques, 1/2 curl of the torque coefficients is
// added before the solve (k_tp_solve_reg's arithmetic), and the vorticity
// 1/2 curl u goes back to tspec.
template <typename R, int R1, int R2, int NS>
__global__ void __launch_bounds__(ZF_CB * NS * (R1 > R2 ? R1 : R2))
    k_tp_zfused(typename Cplx<R>::T *__restrict__ spec, typename Cplx<R>::T *__restrict__ tspec, int torque,
                int64_t nk, int nx, int ny, int nxh, const double *__restrict__ kvx, const double *__restrict__ kvy,
                const double *__restrict__ kvz, const typename Cplx<R>::T *__restrict__ twg, R eta, R scale) {
  typedef typename Cplx<R>::T C;
  constexpr int NZ = R1 * R2;
  constexpr int CB = ZF_CB;
  constexpr int CS = NZ * CB;  // component stride in shared memory
  extern __shared__ __align__(16) unsigned char zf_smem[];
  C *buf = reinterpret_cast<C *>(zf_smem);  // [NS][NZ][CB]
  __shared__ C tw[NZ];
  const int tid = threadIdx.x, nth = blockDim.x;
  const int64_t c0 = (int64_t)blockIdx.x * CB;
  for (int i = tid; i < NZ; i += nth) tw[i] = twg[i];
  for (int e = tid; e < NS * CS; e += nth) {
    const int col = e % CB, r = e / CB;
    const C *src = (r < 3 * NZ) ? spec + (int64_t)r * nk : tspec + (int64_t)(r - 3 * NZ) * nk;
    buf[e] = (c0 + col < nk && (r < 3 * NZ || torque)) ? src[c0 + col] : C{(R)0, (R)0};
  }
  __syncthreads();
  const int col = tid % CB, q = tid / CB, comp = q % NS, j = q / NS;
  C *s = buf + comp * CS + col;
  if (j < R2) {  // pass 1: n2 = j
    C v[R1];
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) v[n1] = s[(R2 * n1 + j) * CB];
    dft_small<C, R1, false>(v);
    s[j * CB] = v[0];
#pragma unroll
    for (int k1 = 1; k1 < R1; ++k1) s[(R2 * k1 + j) * CB] = cmul(v[k1], tw[(j * k1) % NZ]);
  }
  __syncthreads();
  if (j < R1) {  // pass 2: k1 = j
    C v[R2];
#pragma unroll
    for (int n2 = 0; n2 < R2; ++n2) v[n2] = s[(R2 * j + n2) * CB];
    dft_small<C, R2, false>(v);
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) s[(R2 * j + k2) * CB] = v[k2];
  }
  __syncthreads();
  // solve every (slot, column): slot R2 k1 + k2 holds kz index k1 + R1 k2
  for (int e = tid; e < CS; e += nth) {
    const int cc = e % CB, slot = e / CB;
    const int64_t kc = c0 + cc;
    if (kc >= nk) continue;
    const int iz = slot / R2 + R1 * (slot % R2);
    C *u = buf + slot * CB + cc;
    const int ix = (int)(kc % nxh), iy = (int)(kc / nxh);
    if (ix == 0 && iy == 0 && iz == 0) {
#pragma unroll
      for (int c = 0; c < NS; ++c) u[c * CS] = C{(R)0, (R)0};
      continue;
    }
    const R kx = (R)__ldg(kvx + ix), ky = (R)__ldg(kvy + iy), kz = (R)__ldg(kvz + iz);
    const R dx = (2 * ix == nx) ? (R)0 : kx;
    const R dy = (2 * iy == ny) ? (R)0 : ky;
    const R dz = (2 * iz == NZ) ? (R)0 : kz;
    const R ksq = kx * kx + ky * ky + kz * kz;
    const R half = (R)0.5;
    C f = u[0], g = u[CS], h = u[2 * CS];
    if (NS == 6 && torque) {  // + 1/2 curl t, with i k: i (dy tz - dz ty, dz tx - dx tz, dx ty - dy tx)
      const C a = u[3 * CS], b = u[4 * CS], c = u[5 * CS];
      f.x += half * (-dy * c.y - (-dz * b.y)); f.y += half * (dy * c.x - dz * b.x);
      g.x += half * (-dz * a.y - (-dx * c.y)); g.y += half * (dz * a.x - dx * c.x);
      h.x += half * (-dx * b.y - (-dy * a.y)); h.y += half * (dx * b.x - dy * a.x);
    }
    const R ik = (R)1 / ksq;
    const R pr = (dx * f.y + dy * g.y + dz * h.y) * ik;
    const R pi = -(dx * f.x + dy * g.x + dz * h.x) * ik;
    const R v = scale * ik / eta;
    const C a = C{v * (f.x + dx * pi), v * (f.y - dx * pr)};
    const C b = C{v * (g.x + dy * pi), v * (g.y - dy * pr)};
    const C c = C{v * (h.x + dz * pi), v * (h.y - dz * pr)};
    u[0] = a;
    u[CS] = b;
    u[2 * CS] = c;
    if (NS == 6) {  // vorticity 1/2 curl u
      u[3 * CS] = C{half * (-dy * c.y - (-dz * b.y)), half * (dy * c.x - dz * b.x)};
      u[4 * CS] = C{half * (-dz * a.y - (-dx * c.y)), half * (dz * a.x - dx * c.x)};
      u[5 * CS] = C{half * (-dx * b.y - (-dy * a.y)), half * (dx * b.x - dy * a.x)};
    }
  }
  __syncthreads();
  if (j < R1) {  // inverse of pass 2
    C v[R2];
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) v[k2] = s[(R2 * j + k2) * CB];
    dft_small<C, R2, true>(v);
#pragma unroll
    for (int n2 = 0; n2 < R2; ++n2) s[(R2 * j + n2) * CB] = v[n2];
  }
  __syncthreads();
  if (j < R2) {  // inverse of pass 1
    C v[R1];
    v[0] = s[j * CB];
#pragma unroll
    for (int k1 = 1; k1 < R1; ++k1) v[k1] = cmulc(s[(R2 * k1 + j) * CB], tw[(j * k1) % NZ]);
    dft_small<C, R1, true>(v);
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) s[(R2 * n1 + j) * CB] = v[n1];
  }
  __syncthreads();
  for (int e = tid; e < NS * CS; e += nth) {
    const int cc = e % CB, r = e / CB;
    if (c0 + cc >= nk) continue;
    C *dst = (r < 3 * NZ) ? spec + (int64_t)r * nk : tspec + (int64_t)(r - 3 * NZ) * nk;
    dst[c0 + cc] = buf[e];
  }
}

template <typename R, int R1, int R2, int NS>
static void launch_tp_zfused(typename Cplx<R>::T *spec, typename Cplx<R>::T *tspec, bool torque, int64_t nk, int nx,
                             int ny, int nxh, const double *kvx, const double *kvy, const double *kvz,
                             const typename Cplx<R>::T *tw, R eta, R scale, cudaStream_t s) {
  constexpr int threads = ZF_CB * NS * (R1 > R2 ? R1 : R2);
  const size_t smem = sizeof(typename Cplx<R>::T) * NS * R1 * R2 * ZF_CB;
  static bool attr = false;
  if (!attr) {
    DPST_CUDA(cudaFuncSetAttribute(k_tp_zfused<R, R1, R2, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
    attr = true;
  }
  const int64_t blocks = (nk + ZF_CB - 1) / ZF_CB;
  k_tp_zfused<R, R1, R2, NS><<<(unsigned)blocks, threads, smem, s>>>(spec, tspec, torque ? 1 : 0, nk, nx, ny, nxh,
                                                                     kvx, kvy, kvz, tw, eta, scale);
}

template <typename R, int NS>
static void launch_tp_zfused_nz(int nz, typename Cplx<R>::T *spec, typename Cplx<R>::T *tspec, bool torque,
                                int64_t nk, int nx, int ny, int nxh, const double *kvx, const double *kvy,
                                const double *kvz, const typename Cplx<R>::T *tw, R eta, R scale, cudaStream_t s) {
  if (nz == 64) launch_tp_zfused<R, 8, 8, NS>(spec, tspec, torque, nk, nx, ny, nxh, kvx, kvy, kvz, tw, eta, scale, s);
  else if (nz == 32) launch_tp_zfused<R, 8, 4, NS>(spec, tspec, torque, nk, nx, ny, nxh, kvx, kvy, kvz, tw, eta, scale, s);
  else launch_tp_zfused<R, 4, 4, NS>(spec, tspec, torque, nk, nx, ny, nxh, kvx, kvy, kvz, tw, eta, scale, s);
}

template <typename R>
struct EngineTP : EngineBase {
  typedef typename std::conditional<sizeof(R) == 8, cufftDoubleComplex, cufftComplex>::type CR;
  int nx, ny, nz, nxh;
  int64_t M;  // modes of the half spectrum
  double hx, hy, hz, Lz;
  KernelHost km, kd;
  bool fused = false;
  bool reg = false;  // torques with the regular kernel and spectral curls (DPST_TORQUE_REG)
  GridArgs g;
  DevBuf grid, spec, kvx, kvy, kvz, pos64, flags, ord_count, ord_start, perm, dphzw_buf;
  DevBuf gridT, specT;  // reg: torque grid and spectrum, then the vorticity's
  DevBuf st_m[8], st_d[8];
  Stencils<R> stm, std_;
  Ghosts<R> none;  // no ghost layers: z wraps
  bool positioned = false;
  cufftHandle plan_f = 0, plan_b = 0;
  bool plans = false;
  cudaEvent_t ev[8] = {};
  bool have_events = false;
  // fused z transform + solve (k_tp_zfused) for nz = 16, 32, 64: x-y
  // transforms by cuFFT, z in the kernel (six components with the
  // regular-kernel coupling).
  // Chosen for the mixed operator (HBM-bound there); the FP64 operator keeps
  // cuFFT's 3-D transforms (its z passes are FP64-pipe bound, and cuFFT's
  // are the faster of the two).  DPSTOKES_GB300_TP_Z = cufft | fused | auto
  // (default) overrides the choice.
  bool zfused = false;
  DevBuf twz;  // exp(-2 pi i m / nz), m < nz, in R
  // FP64 operator on the 3-D path: the library's double-float transforms
  // (x rows, y columns, z columns) when faster than cuFFT's FP64 3-D ones at
  // creation; timings {cuFFT, own} of a forward + inverse pair
  bool own3d = false;
  DevBuf twxd, twyd, twzd;
  float own3d_ms[2] = {0.0f, 0.0f};
  cudaStream_t cur_stream = 0;

  EngineTP(const dpst_params &prm, int64_t n, int dev) {
    p = prm;
    N = n;
    device = dev;
    DPST_CUDA(cudaSetDevice(dev));
    nx = p.nx; ny = p.ny; nz = p.nz;
    nxh = nx / 2 + 1;
    M = (int64_t)nz * ny * nxh;
    hx = p.Lx / nx;
    hy = p.Ly / ny;
    Lz = p.zmax - p.zmin;
    hz = Lz / nz;
    km = make_kernel_tp(p.w, p.beta, p.alpha, false, hx, hy, hz, nx, ny, nz, "monopole kernel");
    reg = p.has_torque && p.torque_kernel == DPST_TORQUE_REG;
    if (p.has_torque)
      kd = make_kernel_tp(p.w_d, p.beta_d, p.alpha_d, !reg, hx, hy, hz, nx, ny, nz, "dipole kernel");
    fused = p.has_torque && !reg && fused_supports(km.d, kd.d);
    memset(&g, 0, sizeof(g));
    g.nx = nx; g.ny = ny; g.nz = nz;
    g.hx = hx; g.hy = hy; g.Lx = p.Lx; g.Ly = p.Ly; g.Lz = Lz;
    bc_sets(DPST_MODE_PERIODIC, g);
    memset(&none, 0, sizeof(none));
    upload(kvx, wavenumbers(nx, p.Lx));
    upload(kvy, wavenumbers(ny, p.Ly));
    upload(kvz, wavenumbers(nz, Lz));
    grid.alloc(sizeof(R) * 3 * (size_t)nz * ny * nx);
    spec.alloc(sizeof(CR) * 3 * (size_t)M);
    pos64.alloc(sizeof(double) * 3 * std::max<int64_t>(N, 1));
    flags.alloc(sizeof(int) * 8);
    alloc_stencils(km.d, false, st_m, stm);
    if (p.has_torque) alloc_stencils(kd.d, !reg, st_d, std_);
    if (reg) {
      gridT.alloc(grid.bytes);
      specT.alloc(spec.bytes);
    }
    ord_count.alloc(sizeof(int) * tile_order_tiles(nx, ny));
    ord_start.alloc(sizeof(int) * (tile_order_tiles(nx, ny) + 1));
    perm.alloc(sizeof(int) * std::max<int64_t>(N, 1));
    const char *zenv = getenv("DPSTOKES_GB300_TP_Z");
    const std::string zwant = zenv ? zenv : "auto";
    zfused = (nz == 16 || nz == 32 || nz == 64) && (zwant == "fused" || (zwant != "cufft" && sizeof(R) == 4));
    if (zfused) {
      // 2-D real transforms over (y, x) of every (component, z) plane
      std::vector<R> t(2 * (size_t)nz);
      for (int m = 0; m < nz; ++m) {
        t[2 * m] = (R)std::cos(2.0 * M_PI * m / nz);
        t[2 * m + 1] = (R)(-std::sin(2.0 * M_PI * m / nz));
      }
      upload(twz, t);
      int n2[2] = {ny, nx};
      int inem[2] = {ny, nx}, onem[2] = {ny, nxh};
      const int64_t nk = (int64_t)ny * nxh;
      DPST_CUFFT(cufftPlanMany(&plan_f, 2, n2, inem, 1, ny * nx, onem, 1, (int)nk,
                               sizeof(R) == 8 ? CUFFT_D2Z : CUFFT_R2C, 3 * nz));
      DPST_CUFFT(cufftPlanMany(&plan_b, 2, n2, onem, 1, (int)nk, inem, 1, ny * nx,
                               sizeof(R) == 8 ? CUFFT_Z2D : CUFFT_C2R, 3 * nz));
    } else {
      // 3-D real transforms over (z, y, x), one per component
      int n3[3] = {nz, ny, nx};
      int inem[3] = {nz, ny, nx}, onem[3] = {nz, ny, nxh};
      DPST_CUFFT(cufftPlanMany(&plan_f, 3, n3, inem, 1, nz * ny * nx, onem, 1, (int)M,
                               sizeof(R) == 8 ? CUFFT_D2Z : CUFFT_R2C, 3));
      DPST_CUFFT(cufftPlanMany(&plan_b, 3, n3, onem, 1, (int)M, inem, 1, nz * ny * nx,
                               sizeof(R) == 8 ? CUFFT_Z2D : CUFFT_C2R, 3));
    }
    plans = true;
    if (sizeof(R) == 8 && !zfused && own_fft_df_supported(nx, ny) && own_fft_df_supported(nx, nz) &&
        !(getenv("DPSTOKES_GB300_XY_FFT") && std::string(getenv("DPSTOKES_GB300_XY_FFT")) == "cufft")) {
      upload(twxd, fft_twiddles_df(nx));
      upload(twyd, fft_twiddles_df(ny));
      upload(twzd, fft_twiddles_df(nz));
      DPST_CUDA(fft_setup_df(nx, ny));
      DPST_CUDA(fft_setup_df(nx, nz));
      const char *env = getenv("DPSTOKES_GB300_XY_FFT");
      tune_own3d(env && std::string(env) == "own");
    }
    DPST_CUDA(cudaDeviceSynchronize());
  }

  // cuFFT's FP64 3-D pair against the double-float kernels' pair on the
  // grid and spectrum buffers (one warm-up, best of three)
  void tune_own3d(bool force) {
    cudaEvent_t e0, e1;
    DPST_CUDA(cudaEventCreate(&e0));
    DPST_CUDA(cudaEventCreate(&e1));
    DPST_CUDA(cudaMemset(grid.p, 0, grid.bytes));
    cur_stream = 0;
    DPST_CUFFT(cufftSetStream(plan_f, 0));
    DPST_CUFFT(cufftSetStream(plan_b, 0));
    for (int form = 0; form < 2; ++form) {
      own3d = form == 1;
      float best = 1e30f;
      for (int r = 0; r < 4; ++r) {
        DPST_CUDA(cudaEventRecord(e0, 0));
        exec_fwd(grid.as<R>(), spec.as<CR>());
        exec_inv(spec.as<CR>(), grid.as<R>());
        DPST_CUDA(cudaEventRecord(e1, 0));
        DPST_CUDA(cudaEventSynchronize(e1));
        float ms = 0.0f;
        DPST_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (r > 0) best = std::min(best, ms);
      }
      own3d_ms[form] = best;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    own3d = force || own3d_ms[1] < own3d_ms[0];
    DPST_CUDA(cudaMemset(grid.p, 0, grid.bytes));
  }

  ~EngineTP() override {
    cudaSetDevice(device);
    cudaDeviceSynchronize();
    if (have_events)
      for (int i = 0; i < 8; ++i) cudaEventDestroy(ev[i]);
    if (plans) {
      cufftDestroy(plan_f);
      cufftDestroy(plan_b);
    }
  }

  void alloc_stencils(const KernelDesc &d, bool dip, DevBuf *b, Stencils<R> &s) {
    const size_t n = (size_t)std::max<int64_t>(N, 1);
    b[0].alloc(sizeof(int4) * n);
    b[1].alloc(sizeof(R) * n * d.wx);
    b[2].alloc(sizeof(R) * n * d.wy);
    b[3].alloc(sizeof(R) * n * d.wz_max);
    b[4].alloc(sizeof(R) * n * d.wz_max);
    memset(&s, 0, sizeof(s));
    s.cell = b[0].as<int4>();
    s.phx = b[1].as<R>();
    s.phy = b[2].as<R>();
    s.phz = b[3].as<R>();
    s.phzw = b[4].as<R>();
    if (dip) {
      b[5].alloc(sizeof(R) * n * d.wx);
      b[6].alloc(sizeof(R) * n * d.wy);
      b[7].alloc(sizeof(R) * n * d.wz_max);
      dphzw_buf.alloc(sizeof(R) * n * d.wz_max);
      s.dphx = b[5].as<R>();
      s.dphy = b[6].as<R>();
      s.dphz = b[7].as<R>();
      s.dphzw = dphzw_buf.as<R>();
    }
  }

  void set_positions(const void *pos, int dtype, cudaStream_t s) override {
    if (N == 0) { positioned = true; return; }
    if (pos == nullptr) throw Error(DPST_ERR_INVALID_ARG, "positions pointer is NULL");
    launch_prep_positions(pos, dtype, N, p.zmin, pos64.as<double>(), s);
    int init[8] = {0, INT_MAX, -1, INT_MAX, -1, 0, 0, 0};
    int *fl = flags.as<int>();
    DPST_CUDA(cudaMemcpyAsync(fl, init, sizeof(init), cudaMemcpyHostToDevice, s));
    launch_locate<R>(false, pos64.as<double>(), N, km.d, nullptr, nullptr, g, stm, fl, fl + 1, s);
    if (p.has_torque) launch_locate<R>(!reg, pos64.as<double>(), N, kd.d, nullptr, nullptr, g, std_, fl, fl + 3, s);
    DPST_CUDA(cudaGetLastError());
    launch_tile_order<R>(N, g, stm, ord_count.as<int>(), ord_start.as<int>(), perm.as<int>(), s);
    DPST_CUDA(cudaGetLastError());
    int out[8];
    DPST_CUDA(cudaMemcpyAsync(out, fl, sizeof(out), cudaMemcpyDeviceToHost, s));
    DPST_CUDA(cudaStreamSynchronize(s));
    if (out[0] & 1) {
      positioned = false;
      throw Error(DPST_ERR_OUT_OF_DOMAIN, "a particle lies outside [0,Lx]x[0,Ly]x[zmin,zmax] (or is NaN)");
    }
    positioned = true;
  }

  void mark(int k, cudaStream_t s) {
    if (!stage_ms) return;
    if (!have_events) {
      for (int i = 0; i < 8; ++i) DPST_CUDA(cudaEventCreate(&ev[i]));
      have_events = true;
    }
    DPST_CUDA(cudaEventRecord(ev[k], s));
  }

  template <typename RF>
  void spread_stage(const RF *F, const RF *T, cudaStream_t s) {
    R *gr = grid.as<R>();
    const bool torque = p.has_torque && T != nullptr;
    DPST_CUDA(cudaMemsetAsync(gr, 0, grid.bytes, s));
    if (reg) {  // the torques go to their own grid with the regular kernel
      launch_spread<R, RF>(false, F, N, km.d, g, stm, gr, none, s, perm.as<int>());
      if (torque) {
        DPST_CUDA(cudaMemsetAsync(gridT.p, 0, gridT.bytes, s));
        launch_spread<R, RF>(false, T, N, kd.d, g, std_, gridT.as<R>(), none, s, perm.as<int>());
      }
    } else if (torque && fused) {
      launch_spread_fused<R, RF>(F, T, N, km.d, kd.d, g, stm, std_, gr, none, none, s, perm.as<int>());
    } else {
      launch_spread<R, RF>(false, F, N, km.d, g, stm, gr, none, s, perm.as<int>());
      if (torque) launch_spread<R, RF>(true, T, N, kd.d, g, std_, gr, none, s, perm.as<int>());
    }
    DPST_CUDA(cudaGetLastError());
  }

  void exec_fwd(R *gr, CR *sp) {
    if constexpr (sizeof(R) == 8) {
      if (own3d) {  // x rows, y columns over every (component, z) plane, then z columns per component
        DPST_CUDA(fft_rows_df(false, reinterpret_cast<const double *>(gr), reinterpret_cast<double2 *>(sp), nullptr,
                              nullptr, nx, 3 * (int64_t)nz * ny, twxd.as<float4>(), cur_stream));
        DPST_CUDA(fft_cols_df(false, reinterpret_cast<double2 *>(sp), ny, nxh, 3 * (int64_t)nz, twyd.as<float4>(),
                              cur_stream));
        DPST_CUDA(fft_cols_df(false, reinterpret_cast<double2 *>(sp), nz, ny * nxh, 3, twzd.as<float4>(),
                              cur_stream));
        return;
      }
    }
    if (sizeof(R) == 8)
      DPST_CUFFT(cufftExecD2Z(plan_f, (cufftDoubleReal *)gr, (cufftDoubleComplex *)sp));
    else
      DPST_CUFFT(cufftExecR2C(plan_f, (cufftReal *)gr, (cufftComplex *)sp));
  }
  void exec_inv(CR *sp, R *gr) {
    if constexpr (sizeof(R) == 8) {
      if (own3d) {
        DPST_CUDA(fft_cols_df(true, reinterpret_cast<double2 *>(sp), nz, ny * nxh, 3, twzd.as<float4>(),
                              cur_stream));
        DPST_CUDA(fft_cols_df(true, reinterpret_cast<double2 *>(sp), ny, nxh, 3 * (int64_t)nz, twyd.as<float4>(),
                              cur_stream));
        DPST_CUDA(fft_rows_df(true, nullptr, nullptr, reinterpret_cast<const double2 *>(sp),
                              reinterpret_cast<double *>(gr), nx, 3 * (int64_t)nz * ny, twxd.as<float4>(),
                              cur_stream));
        return;
      }
    }
    if (sizeof(R) == 8)
      DPST_CUFFT(cufftExecZ2D(plan_b, (cufftDoubleComplex *)sp, (cufftDoubleReal *)gr));
    else
      DPST_CUFFT(cufftExecC2R(plan_b, (cufftComplex *)sp, (cufftReal *)gr));
  }

  // torque: the torque grid holds spread torques (regular-kernel coupling);
  // on: the grid to solve in place (default: the operator's grid)
  void solve_stage(bool torque, cudaStream_t s, R *on = nullptr) {
    R *gr = on ? on : grid.as<R>();
    CR *sp = spec.as<CR>();
    cur_stream = s;
    DPST_CUFFT(cufftSetStream(plan_f, s));
    exec_fwd(gr, sp);
    if (reg && torque) exec_fwd(gridT.as<R>(), specT.as<CR>());
    mark(2, s);
    mark(3, s);  // no z transform in this mode
    const int bs = 256;
    typedef typename Cplx<R>::T C;
    const R scale = (R)(1.0 / ((double)nx * ny * nz));
    if (zfused) {
      const int64_t nk = (int64_t)ny * nxh;
      C *spc = reinterpret_cast<C *>(sp);
      const double *kx = kvx.as<double>(), *ky = kvy.as<double>(), *kz = kvz.as<double>();
      const C *tw = twz.as<C>();
      const R eta = (R)p.viscosity;
      if (reg)
        launch_tp_zfused_nz<R, 6>(nz, spc, specT.as<C>(), torque, nk, nx, ny, nxh, kx, ky, kz, tw, eta, scale, s);
      else
        launch_tp_zfused_nz<R, 3>(nz, spc, nullptr, false, nk, nx, ny, nxh, kx, ky, kz, tw, eta, scale, s);
    } else if (reg)
      k_tp_solve_reg<R><<<(M + bs - 1) / bs, bs, 0, s>>>(reinterpret_cast<C *>(sp), specT.as<C>(), torque ? 1 : 0, M,
                                                        nx, ny, nz, nxh, kvx.as<double>(), kvy.as<double>(),
                                                        kvz.as<double>(), (R)p.viscosity,
                                                        (R)(1.0 / ((double)nx * ny * nz)));
    else
      k_tp_solve<R><<<(M + bs - 1) / bs, bs, 0, s>>>(reinterpret_cast<C *>(sp), M, nx, ny, nz, nxh, kvx.as<double>(),
                                                    kvy.as<double>(), kvz.as<double>(), (R)p.viscosity,
                                                    (R)(1.0 / ((double)nx * ny * nz)));
    DPST_CUDA(cudaGetLastError());
    mark(4, s);
    mark(5, s);
    DPST_CUFFT(cufftSetStream(plan_b, s));
    exec_inv(sp, gr);
    if (reg) exec_inv(specT.as<CR>(), gridT.as<R>());
    mark(6, s);
  }

  template <typename RF>
  void interp_stage(bool torque, RF *V, RF *W, cudaStream_t s) {
    const R *gr = grid.as<R>();
    (void)torque;
    if (reg) {  // V from the velocity grid, Omega from the vorticity grid (regular kernels)
      launch_interp<R, RF>(false, gr, N, km.d, g, stm, none, V, s, perm.as<int>());
      if (W != nullptr) launch_interp<R, RF>(false, gridT.as<R>(), N, kd.d, g, std_, none, W, s, perm.as<int>());
    } else if (p.has_torque && W != nullptr) {
      if (fused) {
        launch_interp_fused<R, RF>(gr, N, km.d, kd.d, g, stm, std_, none, none, V, W, s, perm.as<int>());
      } else {
        launch_interp<R, RF>(false, gr, N, km.d, g, stm, none, V, s, perm.as<int>());
        launch_interp<R, RF>(true, gr, N, kd.d, g, std_, none, W, s, perm.as<int>());
      }
    } else {
      launch_interp<R, RF>(false, gr, N, km.d, g, stm, none, V, s, perm.as<int>());
    }
    DPST_CUDA(cudaGetLastError());
  }

  template <typename RF>
  void run(const RF *F, const RF *T, RF *V, RF *W, cudaStream_t s) {
    const bool torque = p.has_torque && T != nullptr;
    mark(0, s);
    spread_stage<RF>(F, T, s);
    mark(1, s);
    solve_stage(torque, s);
    interp_stage<RF>(torque, V, W, s);
    mark(7, s);
    if (stage_ms) {
      DPST_CUDA(cudaEventSynchronize(ev[7]));
      const int from[8] = {0, 1, 2, 3, 4, 5, 6, 0}, to[8] = {1, 2, 3, 4, 5, 6, 7, 7};
      for (int k = 0; k < 8; ++k) DPST_CUDA(cudaEventElapsedTime(&stage_ms[k], ev[from[k]], ev[to[k]]));
    }
  }

  void mdot(const void *F, const void *T, void *V, void *W, int dtype, cudaStream_t s) override {
    if (!positioned) throw Error(DPST_ERR_NOT_READY, "positions have not been set");
    if (N == 0) return;
    if (F == nullptr || V == nullptr) throw Error(DPST_ERR_INVALID_ARG, "F and V must not be NULL");
    if (dtype == DPST_F64)
      run<double>((const double *)F, (const double *)T, (double *)V, (double *)W, s);
    else if (dtype == DPST_F32)
      run<float>((const float *)F, (const float *)T, (float *)V, (float *)W, s);
    else
      throw Error(DPST_ERR_INVALID_ARG, "dtype must be DPST_F64 or DPST_F32");
  }

  // K columns at the same positions: one Mdot per column (the triply
  // periodic solve has no per-wavenumber factors to share)
  void mdot_multi(int K, const void *F, const void *T, void *V, void *W, int dtype, cudaStream_t s) override {
    if (!positioned) throw Error(DPST_ERR_NOT_READY, "positions have not been set");
    if (K < 1) throw Error(DPST_ERR_INVALID_ARG, "K must be at least 1");
    if (N == 0) return;
    if (F == nullptr || V == nullptr) throw Error(DPST_ERR_INVALID_ARG, "F and V must not be NULL");
    if (dtype != DPST_F64 && dtype != DPST_F32) throw Error(DPST_ERR_INVALID_ARG, "dtype must be DPST_F64 or DPST_F32");
    const size_t col = 3 * (size_t)N * (dtype == DPST_F64 ? 8 : 4);
    for (int k = 0; k < K; ++k) {
      const char *Fk = (const char *)F + k * col;
      const char *Tk = T ? (const char *)T + k * col : nullptr;
      char *Vk = (char *)V + k * col;
      char *Wk = W ? (char *)W + k * col : nullptr;
      mdot(Fk, Tk, Vk, Wk, dtype, s);
    }
  }

  void spread_grid(const void *F, const void *T, int dtype, void *out, cudaStream_t s) override {
    if (!positioned) throw Error(DPST_ERR_NOT_READY, "positions have not been set");
    if (!F || !out) throw Error(DPST_ERR_INVALID_ARG, "F and grid_out must not be NULL");
    if (dtype == DPST_F64) spread_stage<double>((const double *)F, (const double *)T, s);
    else if (dtype == DPST_F32) spread_stage<float>((const float *)F, (const float *)T, s);
    else throw Error(DPST_ERR_INVALID_ARG, "dtype must be DPST_F64 or DPST_F32");
    DPST_CUDA(cudaMemcpyAsync(out, grid.p, grid.bytes, cudaMemcpyDeviceToDevice, s));
  }

  void velocity_grid(void *out, cudaStream_t s) override {
    if (!out) throw Error(DPST_ERR_INVALID_ARG, "grid_out must not be NULL");
    DPST_CUDA(cudaMemcpyAsync(out, grid.p, grid.bytes, cudaMemcpyDeviceToDevice, s));
  }

  // ---- backward pass ---------------------------------------------------------
  // The same structure as the doubly periodic backward (dpst_engine.cu): the
  // adjoint source J^T (gV, gW) spread with the interpolation's weights, the
  // adjoint of the grid-to-grid map applied to it, the gathers S^T psi (dl/dF,
  // dl/dT) and, for dl/dX, the derivatives of the stencil factors against the
  // recomputed forward grid u and psi.  The triply periodic grid-to-grid map
  // (real transforms, the Fourier solve, 1/(nx ny nz)) is self-adjoint, so psi
  // is the forward solve of the adjoint source.
  DevBuf grid2, gs_m[4], gs_d[8];
  GradStencils<R> gsm, gsd;
  bool grad_ready = false;

  void ensure_grad() {
    if (grad_ready) return;
    grid2.alloc(grid.bytes);
    const size_t n = (size_t)std::max<int64_t>(N, 1);
    memset(&gsm, 0, sizeof(gsm));
    memset(&gsd, 0, sizeof(gsd));
    gs_m[0].alloc(sizeof(R) * n * km.d.wx);
    gs_m[1].alloc(sizeof(R) * n * km.d.wy);
    gs_m[2].alloc(sizeof(R) * n * km.d.wz_max);
    gs_m[3].alloc(sizeof(R) * n * km.d.wz_max);
    gsm.gx = gs_m[0].as<R>();
    gsm.gy = gs_m[1].as<R>();
    gsm.gz = gs_m[2].as<R>();
    gsm.gzw = gs_m[3].as<R>();
    if (p.has_torque) {
      const KernelDesc &d = kd.d;
      const int w[8] = {d.wx, d.wy, d.wz_max, d.wz_max, d.wx, d.wy, d.wz_max, d.wz_max};
      for (int q = 0; q < 8; ++q) gs_d[q].alloc(sizeof(R) * n * w[q]);
      gsd.gx = gs_d[0].as<R>();
      gsd.gy = gs_d[1].as<R>();
      gsd.gz = gs_d[2].as<R>();
      gsd.gzw = gs_d[3].as<R>();
      gsd.gdx = gs_d[4].as<R>();
      gsd.gdy = gs_d[5].as<R>();
      gsd.gdz = gs_d[6].as<R>();
      gsd.gdzw = gs_d[7].as<R>();
    }
    grad_ready = true;
  }

  template <typename RF>
  void run_backward(const RF *F, const RF *T, const RF *gV, const RF *gW, RF *gF, RF *gT, RF *gX,
                    cudaStream_t s) {
    const bool torque = p.has_torque && T != nullptr;
    const bool want_x = gX != nullptr;
    ensure_grad();
    R *gr = grid.as<R>(), *g2 = grid2.as<R>();
    if (want_x) {
      launch_locate_grad<R>(false, pos64.as<double>(), N, km.d, nullptr, nullptr, g, stm, gsm, s);
      if (p.has_torque) launch_locate_grad<R>(true, pos64.as<double>(), N, kd.d, nullptr, nullptr, g, std_, gsd, s);
      if (!reuse_forward) {  // the forward's velocity grid, unless the handle still holds it
        spread_stage<RF>(F, T, s);
        solve_stage(false, s);
      }
    }
    DPST_CUDA(cudaMemsetAsync(g2, 0, grid2.bytes, s));
    Stencils<R> sw = stm;
    sw.phz = stm.phzw;  // the interpolation's weights
    if (gW && fused) {
      // J_dip^T gW = 1/2 grad(w) x gW at the interpolation's weights: the
      // form of the torque spread, and the periodic z map has no ghost
      // layers, so the fused spread applies it with gW in place of T
      Stencils<R> swd = std_;
      swd.phz = std_.phzw;
      swd.dphz = std_.dphzw;
      launch_spread_fused<R, RF>(gV, gW, N, km.d, kd.d, g, sw, swd, g2, none, none, s, perm.as<int>());
    } else {
      launch_spread<R, RF>(false, gV, N, km.d, g, sw, g2, none, s, perm.as<int>());
      if (gW) launch_adj_spread_dip<R, RF>(gW, N, kd.d, g, std_, g2, none, s);
    }
    DPST_CUDA(cudaGetLastError());
    solve_stage(false, s, g2);  // psi
    if (gF || want_x)
      launch_gather_mono<R, RF>(want_x ? gr : nullptr, g2, N, km.d, g, stm, gsm, none, none, F, gV, gF, gX, s);
    if (p.has_torque && (gT || (want_x && (torque || gW))))
      launch_gather_dip<R, RF>(want_x ? gr : nullptr, g2, N, kd.d, g, std_, gsd, none, none, torque ? T : nullptr, gW,
                               gT, gX, s);
    DPST_CUDA(cudaGetLastError());
  }

  void backward(const void *F, const void *T, const void *gV, const void *gW, void *gF, void *gT, void *gX,
                int dtype, cudaStream_t s) override {
    if (!positioned) throw Error(DPST_ERR_NOT_READY, "positions have not been set");
    if (N == 0) return;
    if (gV == nullptr) throw Error(DPST_ERR_INVALID_ARG, "gV must not be NULL");
    if (reg)
      throw Error(DPST_ERR_UNSUPPORTED, "the backward pass is available for the derivative-kernel torque coupling");
    if (gX != nullptr && F == nullptr)
      throw Error(DPST_ERR_INVALID_ARG, "the position gradient needs the forces F of the forward call");
    if (gW != nullptr && !p.has_torque) throw Error(DPST_ERR_INVALID_ARG, "gW needs an operator created with torques");
    if (gT != nullptr && (T == nullptr || !p.has_torque))
      throw Error(DPST_ERR_INVALID_ARG, "gT needs an operator created with torques and the torques T");
    if (dtype == DPST_F64)
      run_backward<double>((const double *)F, (const double *)T, (const double *)gV, (const double *)gW,
                           (double *)gF, (double *)gT, (double *)gX, s);
    else if (dtype == DPST_F32)
      run_backward<float>((const float *)F, (const float *)T, (const float *)gV, (const float *)gW, (float *)gF,
                          (float *)gT, (float *)gX, s);
    else
      throw Error(DPST_ERR_INVALID_ARG, "dtype must be DPST_F64 or DPST_F32");
  }

  void info(dpst_info *o) const override {
    memset(o, 0, sizeof(*o));
    o->nxh = nxh;
    o->n_modes = (int)M;
    o->nzeff_m = km.d.nzeff;
    o->nzeff_d = p.has_torque ? kd.d.nzeff : 0;
    o->ghost_m = km.d.dend;
    o->ghost_d = p.has_torque ? kd.d.dend : 0;
    o->wz_max_m = km.d.wz_max;
    o->wz_max_d = p.has_torque ? kd.d.wz_max : 0;
    o->thr_m = km.d.thr;
    o->thr_d = p.has_torque ? kd.d.thr : 0;
    o->norm_m = km.d.norm;
    o->norm_d = p.has_torque ? kd.d.norm : 0;
    o->n_particles = N;
    // spread (mono [+ dip]), Fourier solve, interp (mono [+ dip])
    const int particle_passes = (p.has_torque && !fused) ? 2 : 1;
    o->kernels_per_mdot = particle_passes + 1 + particle_passes;
    o->fused_particle_passes = fused ? 1 : 0;
    o->z_fused = zfused ? 1 : 0;
    o->xy_transform = own3d ? 3 : 0;
    o->xy_ms[0] = own3d_ms[0];
    o->xy_ms[1] = own3d_ms[1];
    int64_t b = 0;
    const DevBuf *all[] = {&grid, &spec, &kvx, &kvy, &kvz, &pos64, &flags, &ord_count, &ord_start, &perm, &dphzw_buf,
                           &gridT, &specT, &twz, &grid2};
    for (const DevBuf *d : all) b += d->bytes;
    for (int i = 0; i < 8; ++i) b += st_m[i].bytes + st_d[i].bytes;
    o->device_bytes = b;
  }
};

EngineBase *make_engine_tp(const dpst_params &p, int64_t n, int device) {
  if (p.precision == DPST_PREC_FP64) return new EngineTP<double>(p, n, device);
  return new EngineTP<float>(p, n, device);
}

}  // namespace dpst
