// x-y Fourier transforms of the mixed operator (FP32): the unnormalised
// real-to-complex transform of every (component, level) plane of the grid
// [planes][ny][nx] into the half spectrum [planes][ny][nx/2 + 1] and back,
// the x-y part of the reference's Fourier-Chebyshev transform
// (Transform.cpp:107-304: an unnormalised DFT forward, the inverse divided by
// the point count -- here the 1/(nx ny) sits in the inverse z transform).
//
// Two passes per direction, each one read and one write of the data:
//   rows (x): the real-to-complex transform of a row of N = nx reals as the
//     complex FFT of length L = N/2 of z_n = x_2n + i x_2n+1 followed by the
//     split X_k = E_k + w_N^k O_k, E_k = (Z_k + conj Z_{L-k}) / 2,
//     O_k = (Z_k - conj Z_{L-k}) / 2i; the inverse forms
//     Z^_k = E'_k + i O'_k, E'_k = X_k + conj X_{L-k},
//     O'_k = (X_k - conj X_{L-k}) w_N^-k and takes the unnormalised inverse
//     FFT of length L, whose real and imaginary parts are the even and odd
//     reals;
//   columns (y): the complex FFT of length ny along every column of the half
//     spectrum, in place, 16 columns per CTA so that every row access is a
//     128-byte segment.
// Each length L = P x Q transform runs on P threads holding Q values each:
// a radix-Q DFT in registers (stride P), the twiddles w_L^{p k1}, one
// exchange through shared memory, Q/P radix-P DFTs in registers (Cooley-Tukey
// with the four-step index map k = k1 + Q k2).  Powers of two with
// 64 <= nx <= 2048 and 32 <= ny <= 1024; other sizes keep cuFFT.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <vector>

namespace dpst {

// e^{-2 pi i m / 32}: the twiddles of the in-register DFTs (sizes dividing 32)
__constant__ float2 c_tw32[32];

static __device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(__fmaf_rn(a.x, b.x, -a.y * b.y), __fmaf_rn(a.x, b.y, a.y * b.x));
}
static __device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }

// In place DFT of S values (S a power of two dividing 32): V_k = sum_j v_j
// w^{jk}, w = e^{-2 pi i / S} (DIR = -1) or its conjugate (DIR = +1), left
// in bit-reversed order: v[j] = V[brev(j)].  Radix-2 decimation in
// frequency, in place (S values in registers, no copies); every index is a
// compile-time constant after unrolling.
template <int S, int DIR>
static __device__ __forceinline__ void dft_reg(float2 (&v)[S]) {
#pragma unroll
  for (int len = S; len >= 2; len >>= 1) {
#pragma unroll
    for (int i = 0; i < S; i += len) {
#pragma unroll
      for (int k = 0; k < len / 2; ++k) {
        const float2 a = v[i + k], b = v[i + k + len / 2];
        v[i + k] = make_float2(a.x + b.x, a.y + b.y);
        const float2 d = make_float2(a.x - b.x, a.y - b.y);
        if (k == 0) {
          v[i + k + len / 2] = d;
        } else {
          float2 w = c_tw32[k * (32 / len)];
          if (DIR > 0) w = conjf2(w);
          v[i + k + len / 2] = cmulf(d, w);
        }
      }
    }
  }
}

// bit reversal of j within log2(S) bits
template <int S>
static __host__ __device__ constexpr int brev(int j) {
  int r = 0;
  for (int m = S >> 1, b = 1; m > 0; m >>= 1, b <<= 1)
    if (j & m) r |= b;
  return r;
}

// ---------------------------------------------------------------------------
// rows: real-to-complex (forward) and complex-to-real (inverse) along x
// ---------------------------------------------------------------------------
// rows per CTA: 256 threads' worth, at most 48 KB of rows in shared memory
// Exchange layout of a group's shared memory: value (k1, p) at k1 (P + 1) + p,
// so that the stage-2 reads (P values of one k1 per thread, threads P + 1
// apart) fall in different banks; the natural-order pass uses the first
// L + 1 entries.
template <int L, int P>
struct RowCfg {
  static constexpr int Q = L / P;
  static constexpr int BUF = (Q * (P + 1) > L + 1) ? Q * (P + 1) : L + 1;
  static constexpr int cap = (48 * 1024) / (BUF * 8);
  static constexpr int RPC = (256 / P) <= cap ? (256 / P) : (cap >= 16 ? 16 : cap >= 8 ? 8 : cap >= 4 ? 4 : 2);
  static constexpr int T = RPC * P;
};

template <int L, int P>
__global__ void __launch_bounds__(RowCfg<L, P>::T) k_fft_rows_r2c(const float *__restrict__ in,
                                                                  float2 *__restrict__ out, int64_t rows,
                                                                  const float2 *__restrict__ twN) {
  constexpr int Q = L / P, RPC = RowCfg<L, P>::RPC, N = 2 * L, R = Q / P;
  __shared__ float2 sbuf[RPC][RowCfg<L, P>::BUF];
  const int g = threadIdx.x / P, p = threadIdx.x % P;
  const int64_t row = (int64_t)blockIdx.x * RPC + g;
  const bool live = row < rows;
  const int64_t r = live ? row : rows - 1;
  const float2 *x = reinterpret_cast<const float2 *>(in + r * N);
  float2 v[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) v[q] = __ldg(x + p + P * q);
  float2 *sm = sbuf[g];
  {
    // stage 1 / exchange / stage 2, w_L^j = w_N^{2j} from the w_N table
    constexpr int DIR = -1;
    dft_reg<Q, DIR>(v);
#pragma unroll
    for (int k1 = 0; k1 < Q; ++k1) {
      float2 y = v[brev<Q>(k1)];
      if (k1 != 0 && p != 0) y = cmulf(y, __ldg(twN + 2 * p * k1));
      sm[k1 * (P + 1) + p] = y;
    }
    __syncwarp();
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int k1 = p * R + i;
      float2 u[P];
#pragma unroll
      for (int q = 0; q < P; ++q) u[q] = sm[k1 * (P + 1) + q];
      dft_reg<P, DIR>(u);
#pragma unroll
      for (int k2 = 0; k2 < P; ++k2) v[i * P + k2] = u[brev<P>(k2)];
    }
    __syncwarp();
  }
  // Z in natural order, Z_L = Z_0
#pragma unroll
  for (int i = 0; i < R; ++i)
#pragma unroll
    for (int k2 = 0; k2 < P; ++k2) sm[(p * R + i) + Q * k2] = v[i * P + k2];
  __syncwarp();
  if (p == 0) sm[L] = sm[0];
  __syncwarp();
  if (live) {
    float2 *o = out + r * (L + 1);
    for (int k = p; k <= L; k += P) {
      const float2 zk = sm[k], zm = conjf2(sm[L - k]);
      const float2 e = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y + zm.y));
      // O_k = (Z_k - conj Z_{L-k}) / 2i
      const float2 d = make_float2(0.5f * (zk.x - zm.x), 0.5f * (zk.y - zm.y));
      const float2 od = make_float2(d.y, -d.x);
      const float2 w = __ldg(twN + (k == L ? 0 : k));
      const float2 wo = (k == L) ? make_float2(-od.x, -od.y) : cmulf(w, od);
      o[k] = make_float2(e.x + wo.x, e.y + wo.y);
    }
  }
}

template <int L, int P>
__global__ void __launch_bounds__(RowCfg<L, P>::T) k_fft_rows_c2r(const float2 *__restrict__ in,
                                                                  float *__restrict__ out, int64_t rows,
                                                                  const float2 *__restrict__ twN) {
  constexpr int Q = L / P, RPC = RowCfg<L, P>::RPC, N = 2 * L, R = Q / P;
  __shared__ float2 sbuf[RPC][RowCfg<L, P>::BUF];
  const int g = threadIdx.x / P, p = threadIdx.x % P;
  const int64_t row = (int64_t)blockIdx.x * RPC + g;
  const bool live = row < rows;
  const int64_t r = live ? row : rows - 1;
  float2 *sm = sbuf[g];
  const float2 *xr = in + r * (L + 1);
  // the kx = 0 and Nyquist terms enter through their real parts (the real
  // part of the full complex inverse, as a complex-to-real transform takes it)
  {
    float2 t[Q];
#pragma unroll
    for (int m = 0; m < Q; ++m) t[m] = __ldg(xr + p + P * m);
    const float2 last = __ldg(xr + L);
#pragma unroll
    for (int m = 0; m < Q; ++m) sm[p + P * m] = t[m];
    if (p == 0) {
      sm[0].y = 0.0f;
      sm[L] = make_float2(last.x, 0.0f);
    }
  }
  __syncwarp();
  float2 v[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int k = p + P * q;
    const float2 xk = sm[k], xm = conjf2(sm[L - k]);
    const float2 e = make_float2(xk.x + xm.x, xk.y + xm.y);
    const float2 d = make_float2(xk.x - xm.x, xk.y - xm.y);
    // O'_k = d w_N^{-k}; Z^_k = E'_k + i O'_k
    const float2 o = (k == 0) ? d : cmulf(d, conjf2(__ldg(twN + k)));
    v[q] = make_float2(e.x - o.y, e.y + o.x);
  }
  __syncwarp();
  {
    constexpr int DIR = 1;
    dft_reg<Q, DIR>(v);
#pragma unroll
    for (int k1 = 0; k1 < Q; ++k1) {
      float2 y = v[brev<Q>(k1)];
      if (k1 != 0 && p != 0) y = cmulf(y, conjf2(__ldg(twN + 2 * p * k1)));
      sm[k1 * (P + 1) + p] = y;
    }
    __syncwarp();
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int k1 = p * R + i;
      float2 u[P];
#pragma unroll
      for (int q = 0; q < P; ++q) u[q] = sm[k1 * (P + 1) + q];
      dft_reg<P, DIR>(u);
#pragma unroll
      for (int k2 = 0; k2 < P; ++k2) v[i * P + k2] = u[brev<P>(k2)];
    }
    __syncwarp();
  }
#pragma unroll
  for (int i = 0; i < R; ++i)
#pragma unroll
    for (int k2 = 0; k2 < P; ++k2) sm[(p * R + i) + Q * k2] = v[i * P + k2];
  __syncwarp();
  if (live) {
    float2 *o = reinterpret_cast<float2 *>(out + r * N);
    for (int n = p; n < L; n += P) o[n] = sm[n];  // (x_2n, x_2n+1)
  }
}

// ---------------------------------------------------------------------------
// columns: complex FFT of length L along y for CW columns of the half
// spectrum per CTA, in place
// ---------------------------------------------------------------------------
constexpr int FFT_CW = 16;
// per-column exchange buffer: Q (P + 1) values, its stride odd so that the
// 16 columns of a warp's access fall in different banks
template <int L, int P>
constexpr int col_stride() {
  return ((L / P) * (P + 1)) | 1;
}

template <int L, int P, int DIR>
__global__ void __launch_bounds__(FFT_CW * P, (FFT_CW * P) <= 256 ? 3 : 1) k_fft_cols(float2 *__restrict__ data, int64_t planes, int nxh,
                                                         const float2 *__restrict__ twL) {
  constexpr int Q = L / P, R = Q / P;
  extern __shared__ float2 cbuf[];  // [CW][col_stride]
  const int c = threadIdx.x % FFT_CW, p = threadIdx.x / FFT_CW;
  const int tiles = (nxh + FFT_CW - 1) / FFT_CW;
  const int64_t t = blockIdx.x;
  const int64_t plane = t / tiles;
  const int kx = (int)(t % tiles) * FFT_CW + c;
  if (plane >= planes) return;
  const bool live = kx < nxh;
  float2 *base = data + plane * (int64_t)L * nxh + (live ? kx : nxh - 1);
  float2 v[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) v[q] = base[(int64_t)(p + P * q) * nxh];
  float2 *sm = cbuf + c * col_stride<L, P>();
  dft_reg<Q, DIR>(v);
#pragma unroll
  for (int k1 = 0; k1 < Q; ++k1) {
    float2 y = v[brev<Q>(k1)];
    if (k1 != 0 && p != 0) {
      float2 w = __ldg(twL + p * k1);
      if (DIR > 0) w = conjf2(w);
      y = cmulf(y, w);
    }
    sm[k1 * (P + 1) + p] = y;
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int k1 = p * R + i;
    float2 u[P];
#pragma unroll
    for (int q = 0; q < P; ++q) u[q] = sm[k1 * (P + 1) + q];
    dft_reg<P, DIR>(u);
    if (live) {
#pragma unroll
      for (int k2 = 0; k2 < P; ++k2) base[(int64_t)(k1 + Q * k2) * nxh] = u[brev<P>(k2)];
    }
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static bool pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

bool own_fft_supported(int nx, int ny) { return pow2(nx) && pow2(ny) && nx >= 64 && nx <= 2048 && ny >= 32 && ny <= 1024; }

// e^{-2 pi i j / n}, j < n, from FP64
std::vector<float2> fft_twiddles(int n) {
  std::vector<float2> t(n);
  for (int j = 0; j < n; ++j) {
    const double a = -2.0 * M_PI * (double)j / (double)n;
    t[j] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  return t;
}

static cudaError_t upload_tw32() {
  static bool done[256] = {false};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 0 && dev < 256 && done[dev]) return cudaSuccess;
  const std::vector<float2> t = fft_twiddles(32);
  e = cudaMemcpyToSymbol(c_tw32, t.data(), sizeof(float2) * 32);
  if (e == cudaSuccess && dev >= 0 && dev < 256) done[dev] = true;
  return e;
}

cudaError_t fft_setup(int nx, int ny) {
  (void)nx;
  cudaError_t e = upload_tw32();
  if (e != cudaSuccess) return e;
  auto cols_smem = [](int stride) { return (int)(sizeof(float2) * FFT_CW * stride); };
  // the column kernels' shared memory above 48 KB
  switch (ny) {
    case 512:
      e = cudaFuncSetAttribute(k_fft_cols<512, 16, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               cols_smem(col_stride<512, 16>()));
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_fft_cols<512, 16, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 cols_smem(col_stride<512, 16>()));
      break;
    case 1024:
      e = cudaFuncSetAttribute(k_fft_cols<1024, 32, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               cols_smem(col_stride<1024, 32>()));
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_fft_cols<1024, 32, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 cols_smem(col_stride<1024, 32>()));
      break;
    default:
      break;
  }
  return e;
}

template <int L, int P>
static void rows_r2c(const float *in, float2 *out, int64_t rows, const float2 *tw, cudaStream_t s) {
  constexpr int RPC = RowCfg<L, P>::RPC;
  k_fft_rows_r2c<L, P><<<(unsigned)((rows + RPC - 1) / RPC), RowCfg<L, P>::T, 0, s>>>(in, out, rows, tw);
}
template <int L, int P>
static void rows_c2r(const float2 *in, float *out, int64_t rows, const float2 *tw, cudaStream_t s) {
  constexpr int RPC = RowCfg<L, P>::RPC;
  k_fft_rows_c2r<L, P><<<(unsigned)((rows + RPC - 1) / RPC), RowCfg<L, P>::T, 0, s>>>(in, out, rows, tw);
}
template <int L, int P, int DIR>
static void cols(float2 *data, int64_t planes, int nxh, const float2 *tw, cudaStream_t s) {
  const int tiles = (nxh + FFT_CW - 1) / FFT_CW;
  const size_t smem = sizeof(float2) * FFT_CW * col_stride<L, P>();
  k_fft_cols<L, P, DIR><<<(unsigned)(planes * tiles), FFT_CW * P, smem, s>>>(data, planes, nxh, tw);
}

// Row pass: rows = planes x ny real rows of nx (forward) or half-spectrum
// rows of nx/2 + 1 (inverse).  twx: fft_twiddles(nx).
cudaError_t fft_rows(bool inverse, const float *grid_in, float2 *spec_out, const float2 *spec_in, float *grid_out,
                     int nx, int64_t rows, const float2 *twx, cudaStream_t s) {
  switch (nx) {
#define ROWS_CASE(NX, P)                                                \
  case NX:                                                              \
    if (inverse) rows_c2r<NX / 2, P>(spec_in, grid_out, rows, twx, s);   \
    else rows_r2c<NX / 2, P>(grid_in, spec_out, rows, twx, s);           \
    break;
    ROWS_CASE(64, 4)
    ROWS_CASE(128, 8)
    ROWS_CASE(256, 8)
    ROWS_CASE(512, 16)
    ROWS_CASE(1024, 16)
    ROWS_CASE(2048, 32)
#undef ROWS_CASE
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// Column pass over planes planes of ny x nxh, in place.  twy: fft_twiddles(ny).
cudaError_t fft_cols(bool inverse, float2 *spec, int ny, int nxh, int64_t planes, const float2 *twy,
                     cudaStream_t s) {
  switch (ny) {
#define COLS_CASE(NY, P)                                   \
  case NY:                                                 \
    if (inverse) cols<NY, P, 1>(spec, planes, nxh, twy, s); \
    else cols<NY, P, -1>(spec, planes, nxh, twy, s);        \
    break;
    COLS_CASE(32, 4)
    COLS_CASE(64, 8)
    COLS_CASE(128, 8)
    COLS_CASE(256, 16)
    COLS_CASE(512, 16)
    COLS_CASE(1024, 32)
#undef COLS_CASE
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace dpst
