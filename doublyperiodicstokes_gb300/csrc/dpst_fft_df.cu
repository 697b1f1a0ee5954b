// x-y Fourier transforms of the FP64 operator in double-float arithmetic on
// the FP32 pipes (FP64 runs at 1/64 of the FP32 rate on this GPU, and the
// FP64 FFT passes are FP64-pipe bound): the same two-pass structure, index
// maps and real-to-complex split as the FP32 kernels of dpst_fft.cu, with
// every value a double-float complex (hi + lo pairs, about 48 significant
// bits; dpst_df64.cuh) and the twiddles rounded from FP64 to double-float.
// Input and output stay FP64 in memory: a value is split into a
// double-float pair when loaded and summed back when stored.  Error about
// 2^-48 log2(n) relative to the transform's magnitude (~1e-14 for n = 512),
// against ~1e-16 for an FP64 FFT; the FP64 operator's results move by about
// 1e-14 relative.  Powers of two with 64 <= nx <= 1024 and 32 <= ny <= 512.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <vector>

#include "dpst_df64.cuh"

namespace dpst {

struct dcx {
  df64 x, y;
};

static __device__ __forceinline__ dcx dc_make(df64 x, df64 y) {
  dcx r;
  r.x = x;
  r.y = y;
  return r;
}
static __device__ __forceinline__ dcx dc_add(dcx a, dcx b) { return dc_make(df_add(a.x, b.x), df_add(a.y, b.y)); }
static __device__ __forceinline__ dcx dc_sub(dcx a, dcx b) { return dc_make(df_sub(a.x, b.x), df_sub(a.y, b.y)); }
static __device__ __forceinline__ dcx dc_conj(dcx a) { return dc_make(a.x, df_neg(a.y)); }
static __device__ __forceinline__ dcx dc_half(dcx a) { return dc_make(df_scale2(a.x, 0.5f), df_scale2(a.y, 0.5f)); }
// a w
static __device__ __forceinline__ dcx dc_mul(dcx a, dcx w) {
  return dc_make(df_fma(a.x, w.x, df_neg(df_mul(a.y, w.y))), df_fma(a.x, w.y, df_mul(a.y, w.x)));
}
static __device__ __forceinline__ dcx dc_ld(const double2 *p) {
  const double2 v = __ldcg(p);
  return dc_make(df_from_d(v.x), df_from_d(v.y));
}
static __device__ __forceinline__ void dc_st(double2 *p, dcx v) { *p = make_double2(df_to_d(v.x), df_to_d(v.y)); }
// twiddle tables: float4 {re.hi, re.lo, im.hi, im.lo}
static __device__ __forceinline__ dcx tw_ld(const float4 *t) {
  const float4 v = __ldg(t);
  return dc_make(df_make(v.x, v.y), df_make(v.z, v.w));
}

// e^{-2 pi i m / 32} in double-float: the in-register DFTs' twiddles
__constant__ float4 c_tw32d[32];

// In place DFT of S values, left in bit-reversed order (the radix-2
// decimation in frequency of dft_reg in dpst_fft.cu).
template <int S, int DIR>
static __device__ __forceinline__ void dft_reg_d(dcx (&v)[S]) {
#pragma unroll
  for (int len = S; len >= 2; len >>= 1) {
#pragma unroll
    for (int i = 0; i < S; i += len) {
#pragma unroll
      for (int k = 0; k < len / 2; ++k) {
        const dcx a = v[i + k], b = v[i + k + len / 2];
        v[i + k] = dc_add(a, b);
        const dcx d = dc_sub(a, b);
        if (k == 0) {
          v[i + k + len / 2] = d;
        } else if (4 * k == len) {  // w = -i (forward) or +i: exact, no multiply
          v[i + k + len / 2] = DIR < 0 ? dc_make(d.y, df_neg(d.x)) : dc_make(df_neg(d.y), d.x);
        } else {
          const float4 t = c_tw32d[k * (32 / len)];
          dcx w = dc_make(df_make(t.x, t.y), df_make(t.z, t.w));
          if (DIR > 0) w = dc_conj(w);
          v[i + k + len / 2] = dc_mul(d, w);
        }
      }
    }
  }
}

template <int S>
static __host__ __device__ constexpr int brev_d(int j) {
  int r = 0;
  for (int m = S >> 1, b = 1; m > 0; m >>= 1, b <<= 1)
    if (j & m) r |= b;
  return r;
}

template <int L, int P>
struct RowCfgD {
  static constexpr int Q = L / P;
  static constexpr int BUF = (Q * (P + 1) > L + 1) ? Q * (P + 1) : L + 1;
  static constexpr int cap = (48 * 1024) / (BUF * (int)sizeof(dcx));
  static constexpr int RPC = (256 / P) <= cap ? (256 / P) : (cap >= 16 ? 16 : cap >= 8 ? 8 : cap >= 4 ? 4 : 2);
  static constexpr int T = RPC * P;
};

// rows: real FP64 rows of N = 2L -> half spectrum rows of L + 1 (see the FP32
// kernel for the split)
template <int L, int P>
__global__ void __launch_bounds__(RowCfgD<L, P>::T) k_fft_rows_r2c_d(const double *__restrict__ in,
                                                                     double2 *__restrict__ out, int64_t rows,
                                                                     const float4 *__restrict__ twN) {
  constexpr int Q = L / P, RPC = RowCfgD<L, P>::RPC, N = 2 * L, R = Q / P;
  __shared__ dcx sbuf[RPC * RowCfgD<L, P>::BUF];
  const int g = threadIdx.x / P, p = threadIdx.x % P;
  const int64_t row = (int64_t)blockIdx.x * RPC + g;
  const bool live = row < rows;
  const int64_t r = live ? row : rows - 1;
  const double2 *x = reinterpret_cast<const double2 *>(in + r * N);
  dcx v[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) v[q] = dc_ld(x + p + P * q);
  dcx *sm = sbuf + g * RowCfgD<L, P>::BUF;
  dft_reg_d<Q, -1>(v);
#pragma unroll
  for (int k1 = 0; k1 < Q; ++k1) {
    dcx y = v[brev_d<Q>(k1)];
    if (k1 != 0 && p != 0) y = dc_mul(y, tw_ld(twN + 2 * p * k1));
    sm[k1 * (P + 1) + p] = y;
  }
  __syncwarp();
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int k1 = p * R + i;
    dcx u[P];
#pragma unroll
    for (int q = 0; q < P; ++q) u[q] = sm[k1 * (P + 1) + q];
    dft_reg_d<P, -1>(u);
#pragma unroll
    for (int k2 = 0; k2 < P; ++k2) v[i * P + k2] = u[brev_d<P>(k2)];
  }
  __syncwarp();
#pragma unroll
  for (int i = 0; i < R; ++i)
#pragma unroll
    for (int k2 = 0; k2 < P; ++k2) sm[(p * R + i) + Q * k2] = v[i * P + k2];
  __syncwarp();
  if (p == 0) sm[L] = sm[0];
  __syncwarp();
  if (live) {
    double2 *o = out + r * (L + 1);
    for (int k = p; k <= L; k += P) {
      const dcx zk = sm[k], zm = dc_conj(sm[L - k]);
      const dcx e = dc_half(dc_add(zk, zm));
      // O_k = (Z_k - conj Z_{L-k}) / 2i
      const dcx d = dc_half(dc_sub(zk, zm));
      const dcx od = dc_make(d.y, df_neg(d.x));
      const dcx wo = (k == L) ? dc_make(df_neg(od.x), df_neg(od.y)) : dc_mul(tw_ld(twN + k), od);
      dc_st(o + k, dc_add(e, wo));
    }
  }
}

template <int L, int P>
__global__ void __launch_bounds__(RowCfgD<L, P>::T) k_fft_rows_c2r_d(const double2 *__restrict__ in,
                                                                     double *__restrict__ out, int64_t rows,
                                                                     const float4 *__restrict__ twN) {
  constexpr int Q = L / P, RPC = RowCfgD<L, P>::RPC, N = 2 * L, R = Q / P;
  __shared__ dcx sbuf[RPC * RowCfgD<L, P>::BUF];
  const int g = threadIdx.x / P, p = threadIdx.x % P;
  const int64_t row = (int64_t)blockIdx.x * RPC + g;
  const bool live = row < rows;
  const int64_t r = live ? row : rows - 1;
  dcx *sm = sbuf + g * RowCfgD<L, P>::BUF;
  const double2 *xr = in + r * (L + 1);
  {
    dcx t[Q];
#pragma unroll
    for (int m = 0; m < Q; ++m) t[m] = dc_ld(xr + p + P * m);
    const dcx last = dc_ld(xr + L);
#pragma unroll
    for (int m = 0; m < Q; ++m) sm[p + P * m] = t[m];
    if (p == 0) {  // kx = 0 and Nyquist terms by their real parts
      sm[0].y = df_zero();
      sm[L] = dc_make(last.x, df_zero());
    }
  }
  __syncwarp();
  dcx v[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int k = p + P * q;
    const dcx xk = sm[k], xm = dc_conj(sm[L - k]);
    const dcx e = dc_add(xk, xm), d = dc_sub(xk, xm);
    // O'_k = d w_N^{-k}; Z^_k = E'_k + i O'_k
    const dcx o = (k == 0) ? d : dc_mul(d, dc_conj(tw_ld(twN + k)));
    v[q] = dc_make(df_sub(e.x, o.y), df_add(e.y, o.x));
  }
  __syncwarp();
  dft_reg_d<Q, 1>(v);
#pragma unroll
  for (int k1 = 0; k1 < Q; ++k1) {
    dcx y = v[brev_d<Q>(k1)];
    if (k1 != 0 && p != 0) y = dc_mul(y, dc_conj(tw_ld(twN + 2 * p * k1)));
    sm[k1 * (P + 1) + p] = y;
  }
  __syncwarp();
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int k1 = p * R + i;
    dcx u[P];
#pragma unroll
    for (int q = 0; q < P; ++q) u[q] = sm[k1 * (P + 1) + q];
    dft_reg_d<P, 1>(u);
#pragma unroll
    for (int k2 = 0; k2 < P; ++k2) v[i * P + k2] = u[brev_d<P>(k2)];
  }
  __syncwarp();
#pragma unroll
  for (int i = 0; i < R; ++i)
#pragma unroll
    for (int k2 = 0; k2 < P; ++k2) sm[(p * R + i) + Q * k2] = v[i * P + k2];
  __syncwarp();
  if (live) {
    double2 *o = reinterpret_cast<double2 *>(out + r * N);
    for (int n = p; n < L; n += P) o[n] = make_double2(df_to_d(sm[n].x), df_to_d(sm[n].y));  // (x_2n, x_2n+1)
  }
}

// columns: complex FFT of length L along y, CW columns per CTA, in place
constexpr int FFTD_CW = 16;
template <int L, int P>
__host__ __device__ constexpr int col_stride_d() {
  return ((L / P) * (P + 1)) | 1;
}

template <int L, int P, int DIR>
__global__ void __launch_bounds__(FFTD_CW * P, 1) k_fft_cols_d(double2 *__restrict__ data, int64_t planes, int nxh,
                                                               const float4 *__restrict__ twL) {
  constexpr int Q = L / P, R = Q / P;
  extern __shared__ dcx cbufd[];  // [CW][col_stride]
  const int c = threadIdx.x % FFTD_CW, p = threadIdx.x / FFTD_CW;
  const int tiles = (nxh + FFTD_CW - 1) / FFTD_CW;
  const int64_t t = blockIdx.x;
  const int64_t plane = t / tiles;
  const int kx = (int)(t % tiles) * FFTD_CW + c;
  if (plane >= planes) return;
  const bool live = kx < nxh;
  double2 *base = data + plane * (int64_t)L * nxh + (live ? kx : nxh - 1);
  dcx v[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) v[q] = dc_ld(base + (int64_t)(p + P * q) * nxh);
  dcx *sm = cbufd + c * col_stride_d<L, P>();
  dft_reg_d<Q, DIR>(v);
#pragma unroll
  for (int k1 = 0; k1 < Q; ++k1) {
    dcx y = v[brev_d<Q>(k1)];
    if (k1 != 0 && p != 0) {
      dcx w = tw_ld(twL + p * k1);
      if (DIR > 0) w = dc_conj(w);
      y = dc_mul(y, w);
    }
    sm[k1 * (P + 1) + p] = y;
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int k1 = p * R + i;
    dcx u[P];
#pragma unroll
    for (int q = 0; q < P; ++q) u[q] = sm[k1 * (P + 1) + q];
    dft_reg_d<P, DIR>(u);
    if (live) {
#pragma unroll
      for (int k2 = 0; k2 < P; ++k2) dc_st(base + (int64_t)(k1 + Q * k2) * nxh, u[brev_d<P>(k2)]);
    }
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static bool pow2d(int n) { return n > 0 && (n & (n - 1)) == 0; }

bool own_fft_df_supported(int nx, int ny) {
  return pow2d(nx) && pow2d(ny) && nx >= 64 && nx <= 1024 && ny >= 32 && ny <= 512;
}

// e^{-2 pi i j / n} in double-float, float4 {re.hi, re.lo, im.hi, im.lo}
std::vector<float4> fft_twiddles_df(int n) {
  std::vector<float4> t(n);
  for (int j = 0; j < n; ++j) {
    const double a = -2.0 * M_PI * (double)j / (double)n;
    const double c = std::cos(a), s = std::sin(a);
    const float ch = (float)c, sh = (float)s;
    t[j] = make_float4(ch, (float)(c - (double)ch), sh, (float)(s - (double)sh));
  }
  return t;
}

template <int L, int P>
static cudaError_t cols_attr_d() {
  const int smem = (int)(sizeof(dcx) * FFTD_CW * col_stride_d<L, P>());
  cudaError_t e = cudaFuncSetAttribute(k_fft_cols_d<L, P, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_fft_cols_d<L, P, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  return e;
}

cudaError_t fft_setup_df(int nx, int ny) {
  (void)nx;
  static bool done[256] = {false};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (!(dev >= 0 && dev < 256 && done[dev])) {
    const std::vector<float4> t = fft_twiddles_df(32);
    e = cudaMemcpyToSymbol(c_tw32d, t.data(), sizeof(float4) * 32);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 256) done[dev] = true;
  }
  switch (ny) {
    case 32: return cols_attr_d<32, 4>();
    case 64: return cols_attr_d<64, 8>();
    case 128: return cols_attr_d<128, 8>();
    case 256: return cols_attr_d<256, 16>();
    case 512: return cols_attr_d<512, 16>();
  }
  return cudaErrorInvalidValue;
}

template <int L, int P>
static void rows_d(bool inverse, const double *gin, double2 *sout, const double2 *sin, double *gout, int64_t rows,
                   const float4 *tw, cudaStream_t s) {
  constexpr int RPC = RowCfgD<L, P>::RPC;
  const unsigned nb = (unsigned)((rows + RPC - 1) / RPC);
  if (inverse) k_fft_rows_c2r_d<L, P><<<nb, RowCfgD<L, P>::T, 0, s>>>(sin, gout, rows, tw);
  else k_fft_rows_r2c_d<L, P><<<nb, RowCfgD<L, P>::T, 0, s>>>(gin, sout, rows, tw);
}

template <int L, int P>
static void cols_d(bool inverse, double2 *data, int64_t planes, int nxh, const float4 *tw, cudaStream_t s) {
  const int tiles = (nxh + FFTD_CW - 1) / FFTD_CW;
  const size_t smem = sizeof(dcx) * FFTD_CW * col_stride_d<L, P>();
  if (inverse) k_fft_cols_d<L, P, 1><<<(unsigned)(planes * tiles), FFTD_CW * P, smem, s>>>(data, planes, nxh, tw);
  else k_fft_cols_d<L, P, -1><<<(unsigned)(planes * tiles), FFTD_CW * P, smem, s>>>(data, planes, nxh, tw);
}

// Row pass over rows = planes x ny rows; twx: fft_twiddles_df(nx).
cudaError_t fft_rows_df(bool inverse, const double *grid_in, double2 *spec_out, const double2 *spec_in,
                        double *grid_out, int nx, int64_t rows, const float4 *twx, cudaStream_t s) {
  switch (nx) {
#define ROWSD_CASE(NX, P)                                                                  \
  case NX:                                                                                 \
    rows_d<NX / 2, P>(inverse, grid_in, spec_out, spec_in, grid_out, rows, twx, s);        \
    break;
    ROWSD_CASE(64, 4)
    ROWSD_CASE(128, 8)
    ROWSD_CASE(256, 8)
    ROWSD_CASE(512, 16)
    ROWSD_CASE(1024, 16)
#undef ROWSD_CASE
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// Column pass over planes of ny x nxh, in place; twy: fft_twiddles_df(ny).
cudaError_t fft_cols_df(bool inverse, double2 *spec, int ny, int nxh, int64_t planes, const float4 *twy,
                        cudaStream_t s) {
  switch (ny) {
#define COLSD_CASE(NY, P)                                   \
  case NY:                                                  \
    cols_d<NY, P>(inverse, spec, planes, nxh, twy, s);      \
    break;
    COLSD_CASE(32, 4)
    COLSD_CASE(64, 8)
    COLSD_CASE(128, 8)
    COLSD_CASE(256, 16)
    COLSD_CASE(512, 16)
#undef COLSD_CASE
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace dpst
