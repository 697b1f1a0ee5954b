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
// e^{-2 pi i m / 1024}: the column passes' stage twiddles for every length L
// <= 1024 (w_L^j = entry j 1024 / L, the same FP32 values as a length-L
// table).  A warp of a column pass reads two distinct entries per access (its
// two thread rows), which the constant cache serves without the load pipe.
constexpr int FFT_TWC = 1024;
__constant__ float2 c_twc[FFT_TWC];

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
        } else if (4 * k == len) {  // w = -i (forward) or +i: exact, no multiply
          v[i + k + len / 2] = DIR < 0 ? make_float2(d.y, -d.x) : make_float2(-d.y, d.x);
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

// One CTA's rows [row0, row0 + RPC) (threads beyond RowCfg::T idle); sbuf:
// RPC x BUF values.  Data loads bypass L1 (another CTA of the same launch may
// have written them).
template <int L, int P>
static __device__ __forceinline__ void rows_r2c_body(const float *__restrict__ in, float2 *__restrict__ out,
                                                     int64_t rows, int64_t row0, const float2 *__restrict__ twN,
                                                     float2 *sbuf, const float2 *tws, int tss) {
  constexpr int Q = L / P, N = 2 * L, R = Q / P;
  if (threadIdx.x >= RowCfg<L, P>::T) return;
  const int g = threadIdx.x / P, p = threadIdx.x % P;
  const int64_t row = row0 + g;
  const bool live = row < rows;
  const int64_t r = live ? row : rows - 1;
  const float2 *x = reinterpret_cast<const float2 *>(in + r * N);
  float2 v[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) v[q] = __ldcg(x + p + P * q);
  float2 *sm = sbuf + g * RowCfg<L, P>::BUF;
  {
    // stage 1 / exchange / stage 2, w_L^j = w_N^{2j} from the w_N table
    constexpr int DIR = -1;
    dft_reg<Q, DIR>(v);
#pragma unroll
    for (int k1 = 0; k1 < Q; ++k1) {
      float2 y = v[brev<Q>(k1)];
      if (k1 != 0 && p != 0) y = cmulf(y, tws[p * k1 * tss]);
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
__global__ void __launch_bounds__(RowCfg<L, P>::T) k_fft_rows_r2c(const float *__restrict__ in,
                                                                  float2 *__restrict__ out, int64_t rows,
                                                                  const float2 *__restrict__ twN) {
  __shared__ float2 sbuf[RowCfg<L, P>::RPC * RowCfg<L, P>::BUF];
  __shared__ float2 tws[L];  // w_L^j = w_N^{2j}: the stage twiddles, read at 16 distinct entries per warp
  for (int j = threadIdx.x; j < L; j += blockDim.x) tws[j] = __ldg(twN + 2 * j);
  __syncthreads();
  rows_r2c_body<L, P>(in, out, rows, (int64_t)blockIdx.x * RowCfg<L, P>::RPC, twN, sbuf, tws, 1);
}

template <int L, int P>
static __device__ __forceinline__ void rows_c2r_body(const float2 *__restrict__ in, float *__restrict__ out,
                                                     int64_t rows, int64_t row0, const float2 *__restrict__ twN,
                                                     float2 *sbuf, const float2 *tws, int tss) {
  constexpr int Q = L / P, N = 2 * L, R = Q / P;
  if (threadIdx.x >= RowCfg<L, P>::T) return;
  const int g = threadIdx.x / P, p = threadIdx.x % P;
  const int64_t row = row0 + g;
  const bool live = row < rows;
  const int64_t r = live ? row : rows - 1;
  float2 *sm = sbuf + g * RowCfg<L, P>::BUF;
  const float2 *xr = in + r * (L + 1);
  // the kx = 0 and Nyquist terms enter through their real parts (the real
  // part of the full complex inverse, as a complex-to-real transform takes it)
  {
    float2 t[Q];
#pragma unroll
    for (int m = 0; m < Q; ++m) t[m] = __ldcg(xr + p + P * m);
    const float2 last = __ldcg(xr + L);
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
      if (k1 != 0 && p != 0) y = cmulf(y, conjf2(tws[p * k1 * tss]));
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

template <int L, int P>
__global__ void __launch_bounds__(RowCfg<L, P>::T) k_fft_rows_c2r(const float2 *__restrict__ in,
                                                                  float *__restrict__ out, int64_t rows,
                                                                  const float2 *__restrict__ twN) {
  __shared__ float2 sbuf[RowCfg<L, P>::RPC * RowCfg<L, P>::BUF];
  __shared__ float2 tws[L];  // w_L^j = w_N^{2j}, as in k_fft_rows_r2c
  for (int j = threadIdx.x; j < L; j += blockDim.x) tws[j] = __ldg(twN + 2 * j);
  __syncthreads();
  rows_c2r_body<L, P>(in, out, rows, (int64_t)blockIdx.x * RowCfg<L, P>::RPC, twN, sbuf, tws, 1);
}

// ---------------------------------------------------------------------------
// columns: complex FFT of length L along y for CW columns of the half
// spectrum per CTA, in place
// ---------------------------------------------------------------------------
constexpr int FFT_CW = 16;
// per-column exchange buffer: Q (P + 1) values, its stride odd so that the
// 16 columns of a warp's access fall in different banks
template <int L, int P>
__host__ __device__ constexpr int col_stride() {
  return ((L / P) * (P + 1)) | 1;
}

// Column tile `tile` (FFT_CW columns from kx = tile FFT_CW) of plane `plane`,
// in place; every thread of the CTA reaches the one barrier, threads beyond
// FFT_CW P idle.  cbuf: FFT_CW x col_stride values.
template <int L, int P, int DIR>
static __device__ __forceinline__ void cols_body(float2 *__restrict__ data, int64_t plane, int tile, int nxh,
                                                 const float2 *__restrict__ twL, float2 *cbuf) {
  constexpr int Q = L / P, R = Q / P;
  const bool act = threadIdx.x < FFT_CW * P;
  const int c = threadIdx.x % FFT_CW, p = threadIdx.x / FFT_CW;
  const int kx = tile * FFT_CW + c;
  const bool live = act && kx < nxh;
  float2 *base = data + plane * (int64_t)L * nxh + (kx < nxh ? kx : nxh - 1);
  float2 *sm = cbuf + c * col_stride<L, P>();
  if (act) {
    float2 v[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) v[q] = __ldcg(base + (int64_t)(p + P * q) * nxh);
    dft_reg<Q, DIR>(v);
#pragma unroll
    for (int k1 = 0; k1 < Q; ++k1) {
      float2 y = v[brev<Q>(k1)];
      if (k1 != 0 && p != 0) {
        float2 w = c_twc[p * k1 * (FFT_TWC / L)];
        if (DIR > 0) w = conjf2(w);
        y = cmulf(y, w);
      }
      sm[k1 * (P + 1) + p] = y;
    }
  }
  __syncthreads();
  if (act) {
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
}

template <int L, int P, int DIR>
__global__ void __launch_bounds__(FFT_CW * P, (FFT_CW * P) <= 256 ? 3 : 1) k_fft_cols(float2 *__restrict__ data, int64_t planes, int nxh,
                                                         const float2 *__restrict__ twL) {
  extern __shared__ float2 cbuf[];  // [CW][col_stride]
  const int tiles = (nxh + FFT_CW - 1) / FFT_CW;
  const int64_t t = blockIdx.x;
  const int64_t plane = t / tiles;
  if (plane >= planes) return;
  cols_body<L, P, DIR>(data, plane, (int)(t % tiles), nxh, twL, cbuf);
}

// ---------------------------------------------------------------------------
// both passes in one persistent launch, the intermediate kept in L2
// ---------------------------------------------------------------------------
// The two-pass form reads and writes the whole spectrum twice per direction
// (0.8 GB each way on a 512 x 512 x 384-plane grid, four times L2).  Here the
// CTAs take tasks from one counter in an order that runs the first pass of
// plane j beside the second pass of plane j - lag: rows (forward) or columns
// (inverse) of a plane are written to L2, and the other pass reads them back
// from L2 lag planes later, so DRAM sees one read and one write per direction.
// A second-pass task waits until every first-pass task of its plane has
// published (per-plane counter, release / acquire).  Those tasks were taken
// from the counter before it and never wait themselves, so every wait ends
// however many CTAs are resident; each wait still gives up after
// FFT_WAIT_NS, records the error in ctr[2] and skips its task.  The last CTA
// to finish resets the counters for the next launch (ctr[2] is sticky).
// ctr (ints): [1] CTAs finished, [2] error, [4..5] next task (64-bit),
// [6 + plane] first-pass tasks done.
constexpr unsigned long long FFT_WAIT_NS = 1000000000ull;

static __device__ __forceinline__ unsigned long long fft_clock_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
static __device__ __forceinline__ int ld_acquire_gpu(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

template <int NX>
struct RowP {
  static constexpr int P = NX <= 64 ? 4 : NX <= 256 ? 8 : NX <= 1024 ? 16 : 32;
};
template <int NY>
struct ColP {
  static constexpr int P = NY <= 32 ? 4 : NY <= 128 ? 8 : NY <= 512 ? 16 : 32;
};

template <int NX, int NY>
struct XyCfg {
  static constexpr int L = NX / 2, P = RowP<NX>::P, PY = ColP<NY>::P;
  static constexpr int TR = RowCfg<L, P>::T, TC = FFT_CW * PY;
  static constexpr int T = TR > TC ? TR : TC;
  static constexpr int MINB = T <= 256 ? 3 : 1;  // CTAs per SM the registers are sized for
  static constexpr int SR = RowCfg<L, P>::RPC * RowCfg<L, P>::BUF, SC = FFT_CW * col_stride<NY, PY>();
  static constexpr int SMEM = (SR > SC ? SR : SC) * (int)sizeof(float2);
  static constexpr int RT = NY / RowCfg<L, P>::RPC;          // row tasks per plane
  static constexpr int CT = (L + 1 + FFT_CW - 1) / FFT_CW;   // column tasks per plane
};

// INV = false: forward, grid -> spectrum (rows first); true: inverse,
// spectrum -> grid (columns first, in place on the spectrum).
template <int NX, int NY, bool INV>
__global__ void __launch_bounds__(XyCfg<NX, NY>::T, XyCfg<NX, NY>::MINB) k_fft_xy(const float *__restrict__ gin, float2 *spec,
                                                             float *__restrict__ gout, int64_t planes,
                                                             const float2 *__restrict__ twx,
                                                             const float2 *__restrict__ twy, int *ctr, int lag) {
  using C = XyCfg<NX, NY>;
  constexpr int NA = INV ? C::CT : C::RT, NB = INV ? C::RT : C::CT;
  constexpr int L = C::L, RPC = RowCfg<L, C::P>::RPC;
  extern __shared__ float2 xsm[];
  __shared__ int64_t s_task;
  __shared__ int s_ok;
  const int64_t D = lag < planes ? lag : planes;
  const int64_t s1 = D * NA, s2 = s1 + (planes - D) * (NA + NB), total = planes * (NA + NB);
  const int64_t rows = planes * NY;
  for (;;) {
    __syncthreads();  // the previous task's shared-memory reads are done
    if (threadIdx.x == 0) s_task = atomicAdd(reinterpret_cast<unsigned long long *>(ctr + 4), 1ull);
    __syncthreads();
    const int64_t t = s_task;
    if (t >= total) break;
    bool first;
    int64_t plane;
    int idx;
    if (t < s1) {
      first = true, plane = t / NA, idx = (int)(t % NA);
    } else if (t < s2) {
      const int64_t u = t - s1, j = D + u / (NA + NB);
      const int r = (int)(u % (NA + NB));
      first = r < NA;
      plane = first ? j : j - D;
      idx = first ? r : r - NA;
    } else {
      const int64_t u = t - s2;
      first = false, plane = planes + u / NB - D, idx = (int)(u % NB);
    }
    if (!first) {
      if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned long long t0 = fft_clock_ns();
        for (int spin = 0; ld_acquire_gpu(ctr + 6 + plane) < NA; ++spin) {
          if ((spin & 15) == 15 && fft_clock_ns() - t0 > FFT_WAIT_NS) {
            atomicOr(ctr + 2, 1);
            ok = 0;
            break;
          }
          __nanosleep(100);
        }
        s_ok = ok;
      }
      __syncthreads();
      if (!s_ok) continue;
    }
    const bool rowtask = (first != INV);
    if (rowtask) {
      if (!INV) rows_r2c_body<L, C::P>(gin, spec, rows, plane * NY + (int64_t)idx * RPC, twx, xsm, twx, 2);
      else rows_c2r_body<L, C::P>(spec, gout, rows, plane * NY + (int64_t)idx * RPC, twx, xsm, twx, 2);
    } else {
      cols_body<NY, C::PY, INV ? 1 : -1>(spec, plane, idx, L + 1, twy, xsm);
    }
    if (first) {
      __syncthreads();  // every thread's stores precede the release
      if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(ctr + 6 + plane, 1);
      }
    }
  }
  // the last CTA out resets the counters
  __shared__ int s_last;
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(ctr + 1, 1) == (int)gridDim.x - 1;
  }
  __syncthreads();
  if (s_last) {
    for (int64_t p = threadIdx.x; p < planes; p += blockDim.x) ctr[6 + p] = 0;
    if (threadIdx.x == 0) {
      *reinterpret_cast<unsigned long long *>(ctr + 4) = 0ull;
      ctr[1] = 0;
      __threadfence();
    }
  }
}

// ---------------------------------------------------------------------------
// both passes in one launch, the plane held across a thread-block cluster
// ---------------------------------------------------------------------------
// A cluster of FFT_CL CTAs transforms one (component, level) plane at a time,
// the plane's rows split evenly among its CTAs (RC = ny / FFT_CL rows each,
// in shared memory with a 16-byte row pitch), so that HBM sees one read of
// the input and one write of the output per direction:
//   forward: the CTA's RC real rows arrive by bulk asynchronous copies (one
//     mbarrier, the rows' byte count); each row's real-to-complex transform
//     runs in place; after a cluster barrier each CTA takes column tiles
//     rank, rank + FFT_CL, ... (FFT_CW columns each), gathers the tile's ny
//     rows from the owning CTAs' shared memory (distributed shared memory),
//     transforms along y and stores the tile to the spectrum;
//   inverse: each CTA loads its column tiles from the spectrum, transforms
//     along y and stores every row of the tile into the owning CTA's shared
//     memory; after a cluster barrier each CTA runs the complex-to-real
//     transform of its rows and stores them to the grid.
// A cluster barrier closes every plane, so no CTA writes a row buffer that
// another is still reading, and none exits while its memory may be read.
// Every CTA of a cluster takes the same planes, so all reach the same
// barriers; the one mbarrier wait gives up after FFT_WAIT_NS (error word set,
// the plane's results undefined) and the CTA still takes every barrier.
constexpr int FFT_CL = 8;

template <int NX, int NY>
struct XcCfg {
  static constexpr int L = NX / 2, NXH = L + 1;
  static constexpr int PITCH = (NXH + 1) & ~1;  // float2 per row in shared memory
  static constexpr int RC = NY / FFT_CL;        // rows per CTA
  static constexpr int PR = (L >= 256) ? 16 : 8;  // row transform: threads per row
  static constexpr int PC = 16;                 // column transform: threads per column
  static constexpr int T = 256;
  static constexpr int RPP = T / PR;            // rows per row pass
  static constexpr int BUF = RowCfg<L, PR>::BUF;
  static constexpr size_t ROWB = (size_t)RC * PITCH * 8;
  static constexpr size_t CB = (size_t)FFT_CW * col_stride<NY, PC>() * 8;
  static constexpr size_t SB = (size_t)RPP * BUF * 8;
  static constexpr size_t XB = CB > SB ? CB : SB;
  static constexpr size_t SMEM = ROWB + XB + 16;
  static_assert(RC % RPP == 0 && (L / PR) >= PR && (NY / PC) >= PC && FFT_CW * PC == T, "cluster x-y transform");
  static_assert(ROWB % 16 == 0 && (NX * 4) % 16 == 0, "16-byte rows");
};

static __device__ __forceinline__ uint32_t xc_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
static __device__ __forceinline__ void xc_cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
static __device__ __forceinline__ uint32_t xc_mapa(uint32_t a, uint32_t rank) {
  uint32_t d;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(rank));
  return d;
}
static __device__ __forceinline__ float2 xc_ld_remote(uint32_t a) {
  float2 v;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a) : "memory");
  return v;
}
static __device__ __forceinline__ void xc_st_remote(uint32_t a, float2 v) {
  asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(a), "f"(v.x), "f"(v.y) : "memory");
}

// In-place real-to-complex transform of one row in shared memory: L float2
// (the 2L reals) in, L + 1 values out; the P threads of the row (lane p of
// the row's group, all in one warp) exchange through sm (BUF values).
template <int L, int P>
static __device__ __forceinline__ void row_r2c_sm(float2 *row, const float2 *__restrict__ twN, float2 *sm, int p) {
  constexpr int Q = L / P, R = Q / P;
  float2 v[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) v[q] = row[p + P * q];
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
#pragma unroll
  for (int i = 0; i < R; ++i)
#pragma unroll
    for (int k2 = 0; k2 < P; ++k2) sm[(p * R + i) + Q * k2] = v[i * P + k2];
  __syncwarp();
  if (p == 0) sm[L] = sm[0];
  __syncwarp();
  for (int k = p; k <= L; k += P) {
    const float2 zk = sm[k], zm = conjf2(sm[L - k]);
    const float2 e = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y + zm.y));
    const float2 d = make_float2(0.5f * (zk.x - zm.x), 0.5f * (zk.y - zm.y));
    const float2 od = make_float2(d.y, -d.x);
    const float2 w = __ldg(twN + (k == L ? 0 : k));
    const float2 wo = (k == L) ? make_float2(-od.x, -od.y) : cmulf(w, od);
    row[k] = make_float2(e.x + wo.x, e.y + wo.y);
  }
  __syncwarp();
}

// Complex-to-real transform of one row in shared memory (L + 1 values) to
// the 2L reals at out (global).
template <int L, int P>
static __device__ __forceinline__ void row_c2r_sm(const float2 *row, float *__restrict__ out,
                                                  const float2 *__restrict__ twN, float2 *sm, int p) {
  constexpr int Q = L / P, R = Q / P;
  {
    float2 t[Q];
#pragma unroll
    for (int m = 0; m < Q; ++m) t[m] = row[p + P * m];
    const float2 last = row[L];
    __syncwarp();
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
    const float2 o = (k == 0) ? d : cmulf(d, conjf2(__ldg(twN + k)));
    v[q] = make_float2(e.x - o.y, e.y + o.x);
  }
  __syncwarp();
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
#pragma unroll
  for (int i = 0; i < R; ++i)
#pragma unroll
    for (int k2 = 0; k2 < P; ++k2) sm[(p * R + i) + Q * k2] = v[i * P + k2];
  __syncwarp();
  float2 *o = reinterpret_cast<float2 *>(out);
  for (int n = p; n < L; n += P) __stcs(o + n, sm[n]);  // (x_2n, x_2n+1)
  __syncwarp();
}

// Column tile `tile` of one plane: rows gathered from (INV = false) or
// scattered to (INV = true) the cluster's row buffers (rows_sa: this CTA's
// row buffer, shared-memory address; row y in CTA y / RC at row y % RC);
// the spectrum plane sp [NY][nxh] is written (forward) or read (inverse).
// Every thread of the CTA takes the one barrier.
template <int NX, int NY, bool INV>
static __device__ __forceinline__ void col_tile_cl(float2 *__restrict__ sp, int tile, uint32_t rows_sa,
                                                   const float2 *__restrict__ twL, float2 *cbuf) {
  using C = XcCfg<NX, NY>;
  constexpr int L = NY, P = C::PC, Q = L / P, R = Q / P, DIR = INV ? 1 : -1;
  constexpr int nxh = C::NXH;
  const int c = threadIdx.x % FFT_CW, p = threadIdx.x / FFT_CW;
  const int kx = tile * FFT_CW + c;
  const bool live = kx < nxh;
  const int kxc = live ? kx : nxh - 1;
  float2 *sm = cbuf + c * col_stride<L, P>();
  float2 v[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int y = p + P * q;
    if (INV) {
      v[q] = __ldcg(sp + (int64_t)y * nxh + kxc);
    } else {
      const uint32_t a = rows_sa + (uint32_t)(((y % C::RC) * C::PITCH + kxc) * 8);
      v[q] = xc_ld_remote(xc_mapa(a, (uint32_t)(y / C::RC)));
    }
  }
  dft_reg<Q, DIR>(v);
#pragma unroll
  for (int k1 = 0; k1 < Q; ++k1) {
    float2 y = v[brev<Q>(k1)];
    if (k1 != 0 && p != 0) {
      float2 w = c_twc[p * k1 * (FFT_TWC / L)];
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
      for (int k2 = 0; k2 < P; ++k2) {
        const int y = k1 + Q * k2;
        if (INV) {
          const uint32_t a = rows_sa + (uint32_t)(((y % C::RC) * C::PITCH + kx) * 8);
          xc_st_remote(xc_mapa(a, (uint32_t)(y / C::RC)), u[brev<P>(k2)]);
        } else {
          __stcs(sp + (int64_t)y * nxh + kx, u[brev<P>(k2)]);
        }
      }
    }
  }
  __syncthreads();  // cbuf reused by the next tile
}

template <int NX, int NY, bool INV>
__global__ void __cluster_dims__(FFT_CL, 1, 1) __launch_bounds__(256, 1)
    k_fft_xy_cl(const float *__restrict__ gin, float2 *spec, float *__restrict__ gout, int64_t planes,
                const float2 *__restrict__ twx, const float2 *__restrict__ twy, int *err) {
  using C = XcCfg<NX, NY>;
  extern __shared__ __align__(16) unsigned char xc_sm[];
  float2 *rows = reinterpret_cast<float2 *>(xc_sm);
  float2 *xb = reinterpret_cast<float2 *>(xc_sm + C::ROWB);
  uint64_t *bar = reinterpret_cast<uint64_t *>(xc_sm + C::ROWB + C::XB);
  const uint32_t rows_sa = (uint32_t)__cvta_generic_to_shared(rows);
  const uint32_t bar_sa = (uint32_t)__cvta_generic_to_shared(bar);
  const uint32_t rank = xc_rank();
  const int64_t cl = blockIdx.x / FFT_CL, ncl = gridDim.x / FFT_CL;
  constexpr int ntiles = (C::NXH + FFT_CW - 1) / FFT_CW;
  const int tid = threadIdx.x;
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_sa));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  xc_cluster_sync();  // every CTA of the cluster runs before any remote access
  int it = 0;
  for (int64_t pl = cl; pl < planes; pl += ncl, ++it) {
    const int64_t row0 = pl * NY + (int64_t)rank * C::RC;  // this CTA's first row of the plane
    if (!INV) {
      if (tid == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_sa),
                     "r"((uint32_t)(C::RC * NX * 4))
                     : "memory");
        for (int i = 0; i < C::RC; ++i)
          asm volatile(
              "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                  rows_sa + (uint32_t)(i * C::PITCH * 8)),
              "l"(gin + (row0 + i) * NX), "r"((uint32_t)(NX * 4)), "r"(bar_sa)
              : "memory");
      }
      {
        const unsigned long long t0 = fft_clock_ns();
        for (int spin = 0;; ++spin) {
          uint32_t done;
          asm volatile(
              "{\n\t.reg .pred q;\n\tmbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n\tselp.b32 %0, 1, 0, "
              "q;\n\t}"
              : "=r"(done)
              : "r"(bar_sa), "r"((uint32_t)(it & 1))
              : "memory");
          if (done) break;
          if ((spin & 63) == 63 && fft_clock_ns() - t0 > FFT_WAIT_NS) {
            if (tid == 0) atomicOr(err, 1);
            break;
          }
        }
      }
      for (int r0 = 0; r0 < C::RC; r0 += C::RPP)
        row_r2c_sm<C::L, C::PR>(rows + (r0 + tid / C::PR) * C::PITCH, twx, xb + (tid / C::PR) * C::BUF,
                                tid % C::PR);
      xc_cluster_sync();
      for (int tile = (int)rank; tile < ntiles; tile += FFT_CL)
        col_tile_cl<NX, NY, false>(spec + pl * (int64_t)NY * C::NXH, tile, rows_sa, twy, xb);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // row writes before the next copies
      xc_cluster_sync();
    } else {
      for (int tile = (int)rank; tile < ntiles; tile += FFT_CL)
        col_tile_cl<NX, NY, true>(spec + pl * (int64_t)NY * C::NXH, tile, rows_sa, twy, xb);
      xc_cluster_sync();
      for (int r0 = 0; r0 < C::RC; r0 += C::RPP) {
        const int r = r0 + tid / C::PR;
        row_c2r_sm<C::L, C::PR>(rows + r * C::PITCH, gout + (row0 + r) * NX, twx, xb + (tid / C::PR) * C::BUF,
                                tid % C::PR);
      }
      xc_cluster_sync();
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
  if (e == cudaSuccess) {
    const std::vector<float2> tc = fft_twiddles(FFT_TWC);
    e = cudaMemcpyToSymbol(c_twc, tc.data(), sizeof(float2) * FFT_TWC);
  }
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

// ---------------------------------------------------------------------------
// the one-launch form: sizes, counters, launch
// ---------------------------------------------------------------------------
bool fft_xy_fused_supported(int nx, int ny) {
  return nx == ny && (nx == 128 || nx == 256 || nx == 512 || nx == 1024);
}
int64_t fft_xy_counter_ints(int64_t planes) { return 6 + planes; }

template <int NX, int NY>
static cudaError_t xy_setup(int *grid) {
  using C = XyCfg<NX, NY>;
  cudaError_t e = cudaFuncSetAttribute(k_fft_xy<NX, NY, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_fft_xy<NX, NY, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
  int per_sm = 0, nsm = 0, dev = 0;
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fft_xy<NX, NY, false>, C::T, C::SMEM);
  if (e == cudaSuccess) e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) *grid = (per_sm > 0 ? per_sm : 1) * nsm;
  return e;
}

// ---- the cluster form ----
bool fft_xy_cluster_supported(int nx, int ny) { return nx == ny && (nx == 256 || nx == 512); }

template <int NX, int NY>
static cudaError_t xc_setup(int *grid) {
  using C = XcCfg<NX, NY>;
  cudaError_t e = cudaFuncSetAttribute(k_fft_xy_cl<NX, NY, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)C::SMEM);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_fft_xy_cl<NX, NY, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::SMEM);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(FFT_CL * 64, 1, 1);
  cfg.blockDim = dim3(C::T, 1, 1);
  cfg.dynamicSmemBytes = C::SMEM;
  int ncl = 0;
  e = cudaOccupancyMaxActiveClusters(&ncl, (void *)k_fft_xy_cl<NX, NY, false>, &cfg);
  if (e != cudaSuccess) return e;
  *grid = ncl * FFT_CL;
  return cudaSuccess;
}

// Shared-memory attributes and the grid (clusters resident at once x FFT_CL
// CTAs); grid 0: the cluster form cannot run here.
cudaError_t fft_xy_cluster_setup(int nx, int ny, int *grid) {
  *grid = 0;
  if (!fft_xy_cluster_supported(nx, ny)) return cudaErrorInvalidValue;
  cudaError_t e = upload_tw32();
  if (e != cudaSuccess) return e;
  if (nx == 256) return xc_setup<256, 256>(grid);
  return xc_setup<512, 512>(grid);
}

// Forward (grid_in -> spec) or inverse (spec -> grid_out, spec overwritten)
// x-y transform of `planes` planes in one launch of clusters; err: an int
// set (never cleared) when a wait gave up.
cudaError_t fft_xy_cluster(bool inverse, const float *grid_in, float2 *spec, float *grid_out, int nx, int ny,
                           int64_t planes, const float2 *twx, const float2 *twy, int *err, int grid, cudaStream_t s) {
  if (!fft_xy_cluster_supported(nx, ny) || grid < FFT_CL || planes <= 0) return cudaErrorInvalidValue;
  int64_t g = (int64_t)(grid / FFT_CL) * FFT_CL;
  if (g > planes * FFT_CL) g = planes * FFT_CL;
#define XC_LAUNCH(N)                                                                                            \
  if (inverse)                                                                                                 \
    k_fft_xy_cl<N, N, true><<<(unsigned)g, XcCfg<N, N>::T, XcCfg<N, N>::SMEM, s>>>(grid_in, spec, grid_out, planes, \
                                                                                 twx, twy, err);               \
  else                                                                                                         \
    k_fft_xy_cl<N, N, false><<<(unsigned)g, XcCfg<N, N>::T, XcCfg<N, N>::SMEM, s>>>(grid_in, spec, grid_out,     \
                                                                                  planes, twx, twy, err);
  if (nx == 256) {
    XC_LAUNCH(256)
  } else {
    XC_LAUNCH(512)
  }
#undef XC_LAUNCH
  return cudaGetLastError();
}

// Shared-memory attributes and the persistent grid (CTAs resident at once).
cudaError_t fft_xy_setup(int nx, int ny, int *grid) {
  if (!fft_xy_fused_supported(nx, ny)) return cudaErrorInvalidValue;
  cudaError_t e = upload_tw32();
  if (e != cudaSuccess) return e;
  switch (nx) {
    case 128: return xy_setup<128, 128>(grid);
    case 256: return xy_setup<256, 256>(grid);
    case 512: return xy_setup<512, 512>(grid);
    case 1024: return xy_setup<1024, 1024>(grid);
  }
  return cudaErrorInvalidValue;
}

template <int NX, int NY>
static void xy_launch(bool inverse, const float *gin, float2 *spec, float *gout, int64_t planes, const float2 *twx,
                      const float2 *twy, int *ctr, int grid, int lag, cudaStream_t s) {
  using C = XyCfg<NX, NY>;
  if (inverse) k_fft_xy<NX, NY, true><<<grid, C::T, C::SMEM, s>>>(gin, spec, gout, planes, twx, twy, ctr, lag);
  else k_fft_xy<NX, NY, false><<<grid, C::T, C::SMEM, s>>>(gin, spec, gout, planes, twx, twy, ctr, lag);
}

// Forward (grid_in -> spec) or inverse (spec -> grid_out, spec overwritten)
// x-y transform of `planes` planes in one launch; ctr: fft_xy_counter_ints
// (planes) zeroed ints (left zeroed, but for the sticky error at ctr[2]).
cudaError_t fft_xy_fused(bool inverse, const float *grid_in, float2 *spec, float *grid_out, int nx, int ny,
                         int64_t planes, const float2 *twx, const float2 *twy, int *ctr, int grid, int lag,
                         cudaStream_t s) {
  if (!fft_xy_fused_supported(nx, ny) || grid <= 0 || planes <= 0) return cudaErrorInvalidValue;
  switch (nx) {
    case 128: xy_launch<128, 128>(inverse, grid_in, spec, grid_out, planes, twx, twy, ctr, grid, lag, s); break;
    case 256: xy_launch<256, 256>(inverse, grid_in, spec, grid_out, planes, twx, twy, ctr, grid, lag, s); break;
    case 512: xy_launch<512, 512>(inverse, grid_in, spec, grid_out, planes, twx, twy, ctr, grid, lag, s); break;
    case 1024: xy_launch<1024, 1024>(inverse, grid_in, spec, grid_out, planes, twx, twy, ctr, grid, lag, s); break;
  }
  return cudaGetLastError();
}

}  // namespace dpst
