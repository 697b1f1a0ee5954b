// z transform of the mixed-precision operator on the 5th-generation tensor
// cores (tcgen05), split-TF32 with FP32 accumulation in tensor memory.
//
// The transform is OUT[r][col] = sum_m T[r][m] IN[m][col] over every real
// column of the spectrum (per component: nz rows x 2 nk columns, in place),
// with the inverse's epilogue adding the wall correction and scaling
// (corr_any, as k_zgemm does).  Per tile: M = 128 rows (nz padded with zero
// rows of T), N = 128 columns, K = nz padded to a multiple of 8 and streamed
// through shared memory in stages of 32 rows.  Each FP32
// operand x is split as x = hi + lo with hi = tf32(x), lo = tf32(x - hi) and
// the product is accumulated as hi*hi + hi*lo + lo*hi (three
// tcgen05.mma.kind::tf32 per K step of 8), which keeps the FP32-level
// accuracy of the SIMT transform.
//
// One persistent CTA per SM, warp-specialised so that loads, products and
// stores of successive tiles overlap:
//   * 8 producer warps read 32-row x 128-column blocks from HBM (three
//     blocks in flight per thread in registers), split them into TF32 hi /
//     lo and write them, in the canonical K-major no-swizzle layout (8-row x
//     16-byte core matrices, LBO = 128 B along K, SBO = 1 KB along N), into
//     one of two shared-memory stages, then arrive on the stage's "full"
//     mbarrier;
//   * one thread issues the MMAs of a stage (M = 128, N = 128, K = 8: large
//     enough that the per-instruction issue cost does not bound the kernel)
//     into one of two tensor-memory accumulators and commits them to the
//     stage's "empty" mbarrier, and after the tile's last stage to the
//     accumulator's "full" mbarrier;
//   * 4 epilogue warps (one per tensor-memory lane quadrant) read the
//     accumulator 32 columns at a time with tcgen05.ld, release it, transpose
//     each 32 x 32 block through shared memory and store whole rows.
// T (hi, lo) stays in shared memory for the CTA's lifetime.  Every wait has
// an iteration deadline: on expiry the waiting thread records the error and
// raises a shared abort flag that ends every role; the MMA thread then waits
// (bounded) for its issued products before the tensor memory is freed.
#include <cuda.h>

#include <mutex>
#include <vector>

#include "dpst_internal.cuh"
#include "dpst_kdev.cuh"

namespace dpst {

constexpr int ZTC_N = 128;                                     // columns per tile (MMA N)
constexpr int ZTC_KC = 32;                                     // K rows per shared-memory stage
constexpr int ZTC_STAGES = 2;                                  // B (hi, lo) stages
constexpr int ZTC_ACC = 2;                                     // tensor-memory accumulators
constexpr int ZTC_PROD_WARPS = 8;
constexpr int ZTC_EPI_WARPS = 4;                               // one per lane quadrant
constexpr int ZTC_MMA_WARP = ZTC_PROD_WARPS + ZTC_EPI_WARPS;   // warp 12
constexpr int ZTC_THREADS = 32 * (ZTC_MMA_WARP + 1);
constexpr int ZTC_TMEM_COLS = ZTC_ACC * ZTC_N;
constexpr int ZTC_DEPTH = 3;                                   // stages of loads in flight per producer
constexpr int ZTC_PGROUPS = 32 * ZTC_PROD_WARPS / ZTC_N;       // producer threads per column (2)
constexpr int ZTC_QPT = ZTC_KC / 4 / ZTC_PGROUPS;              // row quads per producer thread per stage (4)
constexpr int ZTC_STG = 32 + 4;                                // epilogue staging pitch (floats, 16-B rows)
constexpr unsigned long long ZTC_WAIT_NS = 2000000000ull;      // 2 s
static_assert(ZTC_EPI_WARPS == 4 && ZTC_PROD_WARPS % 4 == 0, "epilogue warp w must own lane quadrant w % 4");

static __device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

static __device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm volatile("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// K-major, no-swizzle shared-memory matrix descriptor (tcgen05 format:
// start >> 4 in [0,14), LBO >> 4 in [16,30), SBO >> 4 in [32,46), version 1
// in [46,48), layout type 0 = no swizzle in [61,64)).
static __device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::tf32: D FP32 (bits 4-5 = 1), A and B TF32
// (bits 7-9 and 10-12 = 2), both K-major, N >> 3 in bits 17-22, M >> 4 in
// bits 24-28.
static __host__ __device__ constexpr uint32_t ztc_idesc(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

static __device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t idesc,
                                                uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}

// Element offset (in 32-bit words) of (row, k) in the core-matrix layout.
static __device__ __forceinline__ int cm_off(int row, int k, int kq) {
  return (row >> 3) * (kq * 32) + (k >> 2) * 32 + (row & 7) * 4 + (k & 3);
}

static __device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

static __device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.b32 %0, 1, 0, p;\n\t}\n"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

static __device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

static __device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

static __device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

// Bounded wait for the completion of the mbarrier phase of the given parity.
// Returns false once the deadline passes (recording the error and raising
// the abort flag) or, when watch_abort, once another thread has aborted.
static __device__ bool ztc_wait(uint32_t bar, uint32_t parity, volatile int *abort_flag, int *err,
                                bool watch_abort = true) {
  const unsigned long long t0 = globaltimer();
  for (int spin = 0;; ++spin) {
    if (mbar_try(bar, parity)) return true;
    if ((spin & 63) == 63) {
      if (watch_abort && *abort_flag) return false;
      if (globaltimer() - t0 > ZTC_WAIT_NS) {
        *abort_flag = 1;
        atomicOr(err, 1);
        return false;
      }
    }
  }
}

// Shared-memory bytes: T hi / lo, the B stages, the epilogue staging, the
// mbarriers, the tensor-memory address slot and the abort flag.
static __host__ __device__ constexpr size_t ztc_off_b(int kp) { return (size_t)2 * 128 * kp * 4; }
static __host__ __device__ constexpr size_t ztc_off_stg(int kp) {
  return ztc_off_b(kp) + (size_t)ZTC_STAGES * 2 * ZTC_N * ZTC_KC * 4;
}
static __host__ __device__ constexpr size_t ztc_off_bar(int kp) {
  return ztc_off_stg(kp) + (size_t)ZTC_EPI_WARPS * 32 * ZTC_STG * 4;
}
constexpr int ZTC_NBARS = 2 * ZTC_STAGES + 2 * ZTC_ACC + 1;

size_t ztc_smem_bytes(int nz) {
  const int kp = (nz + 7) & ~7;
  return ztc_off_bar(kp) + ZTC_NBARS * 8 + 16;
}
// batched: after the single-system layout, one EpiArgs per epilogue warp
// (the tile's segment's epilogue arguments, copied from global memory)
static __host__ __device__ constexpr size_t ztc_off_epi(int kp) {
  return (ztc_off_bar(kp) + ZTC_NBARS * 8 + 16 + 15) & ~(size_t)15;
}
static size_t ztc_smem_bytes_b(int nz) {
  const int kp = (nz + 7) & ~7;
  return ztc_off_epi(kp) + ZTC_EPI_WARPS * sizeof(EpiArgs);
}

// A tile's data: its spectrum component block B ([nz][ncols] real columns),
// the component d, the first column, and the epilogue arguments.  BATCH: the
// tiles of the S segments (systems) are numbered by the prefix `tprefix` of
// 3 ceil(ncols_s / ZTC_N) tiles each; the segment is found by binary search.
struct ZtcTile {
  float *B;
  int64_t ncols, col0;
  int d, seg;
};

template <bool BATCH>
static __device__ __forceinline__ ZtcTile ztc_tile(int64_t t, float *spec, int nz, int64_t ncols,
                                                   const ZSeg<float> *__restrict__ segs,
                                                   const int64_t *__restrict__ tprefix, int S) {
  ZtcTile z;
  int64_t tl = t;
  z.seg = 0;
  if (BATCH) {
    int lo = 0, hi = S - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (tprefix[mid] <= t) lo = mid;
      else hi = mid - 1;
    }
    z.seg = lo;
    tl = t - tprefix[lo];
    spec = segs[lo].spec;
    ncols = segs[lo].ncols;
  }
  const int64_t tpc = (ncols + ZTC_N - 1) / ZTC_N;
  z.d = (int)(tl / tpc);
  z.col0 = (tl % tpc) * ZTC_N;
  z.ncols = ncols;
  z.B = spec + (int64_t)z.d * nz * ncols;
  return z;
}

// CORR: the epilogue may add the wall correction (inverse with walls); the
// inverse's 1/(nx ny) scale is applied in either instantiation.
template <bool CORR, bool BATCH>
__global__ void __launch_bounds__(ZTC_THREADS, 1) k_zgemm_tc(float *spec, int nz, int64_t ncols,
                                                             const float *__restrict__ Tm, EpiArgs e, int *err,
                                                             const ZSeg<float> *__restrict__ segs,
                                                             const int64_t *__restrict__ tprefix, int S,
                                                             int64_t ntiles_b) {
  extern __shared__ __align__(1024) unsigned char ztc_sm[];
  const int kp = (nz + 7) & ~7;  // K padded to the MMA step
  const int kq = kp / 4;         // core matrices along K
  uint32_t *Ahi = reinterpret_cast<uint32_t *>(ztc_sm);  // 128 x kp
  uint32_t *Alo = Ahi + 128 * kp;
  uint32_t *Bst = reinterpret_cast<uint32_t *>(ztc_sm + ztc_off_b(kp));  // stage s: hi, lo (ZTC_N x kp each)
  float *stg = reinterpret_cast<float *>(ztc_sm + ztc_off_stg(kp));
  uint64_t *bars = reinterpret_cast<uint64_t *>(ztc_sm + ztc_off_bar(kp));
  const uint32_t bar0 = smem_u32(bars);
  auto full_bar = [&](int s) { return bar0 + 8u * (uint32_t)s; };
  auto empty_bar = [&](int s) { return bar0 + 8u * (uint32_t)(ZTC_STAGES + s); };
  auto accf_bar = [&](int a) { return bar0 + 8u * (uint32_t)(2 * ZTC_STAGES + a); };
  auto acce_bar = [&](int a) { return bar0 + 8u * (uint32_t)(2 * ZTC_STAGES + ZTC_ACC + a); };
  const uint32_t drain_bar = bar0 + 8u * (uint32_t)(ZTC_NBARS - 1);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + ZTC_NBARS);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // A = T split into tf32 hi / lo, rows >= nz and columns >= nz zero
  for (int idx = tid; idx < 128 * kp; idx += ZTC_THREADS) {
    const int r = idx / kp, k = idx % kp;
    const float v = (r < nz && k < nz) ? Tm[r * nz + k] : 0.0f;
    const uint32_t h = to_tf32(v);
    Ahi[cm_off(r, k, kq)] = h;
    Alo[cm_off(r, k, kq)] = to_tf32(v - __uint_as_float(h));
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(ZTC_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int s = 0; s < ZTC_STAGES; ++s) {
      mbar_init(full_bar(s), ZTC_PROD_WARPS);
      mbar_init(empty_bar(s), 1);
    }
    for (int a = 0; a < ZTC_ACC; ++a) {
      mbar_init(accf_bar(a), 1);
      mbar_init(acce_bar(a), ZTC_EPI_WARPS);
    }
    mbar_init(drain_bar, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("fence.proxy.async.shared::cta;");
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;

  const int64_t ntiles = BATCH ? ntiles_b : 3 * ((ncols + ZTC_N - 1) / ZTC_N);
  const int64_t G = gridDim.x;
  const int my_tiles = (blockIdx.x < ntiles) ? (int)((ntiles - 1 - blockIdx.x) / G + 1) : 0;
  const int nkc = (kp + ZTC_KC - 1) / ZTC_KC;  // stages per tile
  const int my_steps = my_tiles * nkc;         // step u = (tile u / nkc, K chunk u % nkc)
  constexpr int SKQ = ZTC_KC / 4;              // core matrices along K in a stage

  if (warp < ZTC_PROD_WARPS) {
    // ---- producers: column n, row quads q = qg + ZTC_PGROUPS i of the chunk
    const int n = tid % ZTC_N, qg = tid / ZTC_N;
    float b0[ZTC_QPT][4], b1[ZTC_QPT][4], b2[ZTC_QPT][4];
    int cur_j = -1;  // the tile whose data `cur` holds (steps come in increasing order)
    ZtcTile cur;
    cur.B = spec;
    cur.ncols = ncols;
    cur.col0 = 0;
    const int64_t tpc = (ncols + ZTC_N - 1) / ZTC_N;  // single system: tiles per component
    auto load_step = [&](int u, float (&br)[ZTC_QPT][4]) {
      const bool valid = u < my_steps;
      const int j = valid ? u / nkc : 0, c = valid ? u - j * nkc : 0;
      int64_t col;
      const float *B;
      int64_t nc;
      if constexpr (BATCH) {
        if (valid && j != cur_j) {
          cur = ztc_tile<BATCH>(blockIdx.x + (int64_t)j * G, spec, nz, ncols, segs, tprefix, S);
          cur_j = j;
        }
        col = valid ? cur.col0 + n : 0;
        B = cur.B;
        nc = cur.ncols;
      } else {
        const int64_t t = blockIdx.x + (int64_t)j * G;
        const int d = valid ? (int)(t / tpc) : 0;
        col = valid ? (t % tpc) * ZTC_N + n : 0;
        B = spec + (int64_t)d * nz * ncols;
        nc = ncols;
      }
#pragma unroll
      for (int i = 0; i < ZTC_QPT; ++i) {
        const int q = qg + ZTC_PGROUPS * i;
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          const int k = ZTC_KC * c + 4 * q + jj;
          br[i][jj] = (valid && k < nz && col < nc) ? __ldcs(B + (int64_t)k * nc + col) : 0.0f;
        }
      }
    };
    auto step = [&](int u, float (&br)[ZTC_QPT][4]) -> bool {
      const int s = u % ZTC_STAGES;
      bool ok = ztc_wait(empty_bar(s), (uint32_t)(((u / ZTC_STAGES) & 1) ^ 1), abort_flag, err);
      if (!__all_sync(0xffffffffu, ok)) return false;
      uint32_t *Bhi = Bst + (size_t)s * 2 * ZTC_N * ZTC_KC, *Blo = Bhi + ZTC_N * ZTC_KC;
#pragma unroll
      for (int i = 0; i < ZTC_QPT; ++i) {
        const int q = qg + ZTC_PGROUPS * i;
        uint4 h, l;
        h.x = to_tf32(br[i][0]);
        h.y = to_tf32(br[i][1]);
        h.z = to_tf32(br[i][2]);
        h.w = to_tf32(br[i][3]);
        l.x = to_tf32(br[i][0] - __uint_as_float(h.x));
        l.y = to_tf32(br[i][1] - __uint_as_float(h.y));
        l.z = to_tf32(br[i][2] - __uint_as_float(h.z));
        l.w = to_tf32(br[i][3] - __uint_as_float(h.w));
        const int o = cm_off(n, 4 * q, SKQ);
        *reinterpret_cast<uint4 *>(Bhi + o) = h;
        *reinterpret_cast<uint4 *>(Blo + o) = l;
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(full_bar(s));
      load_step(u + ZTC_DEPTH, br);
      return true;
    };
    load_step(0, b0);
    load_step(1, b1);
    load_step(2, b2);
    for (int u = 0; u < my_steps; u += 3) {
      if (!step(u, b0)) break;
      if (u + 1 < my_steps && !step(u + 1, b1)) break;
      if (u + 2 < my_steps && !step(u + 2, b2)) break;
    }
  } else if (warp < ZTC_MMA_WARP) {
    // ---- epilogue: warp owns lane quadrant qd = rows 32 qd .. 32 qd + 31.
    // The accumulator is read 32 columns at a time; the next block's
    // tcgen05.ld is in flight while the current block is stored.
    const int qd = warp & 3;
    float *st = stg + (size_t)(warp - ZTC_PROD_WARPS) * 32 * ZTC_STG;
    EpiArgs *eslot = reinterpret_cast<EpiArgs *>(ztc_sm + ztc_off_epi(kp)) + (warp - ZTC_PROD_WARPS);
    int eseg = -1;  // the segment whose arguments eslot holds
    uint32_t v[32];
    auto tmem_ld = [&](uint32_t taddr) {
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
          "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
            "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]),
            "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
            "=r"(v[30]), "=r"(v[31])
          : "r"(taddr)
          : "memory");
    };
    for (int j = 0; j < my_tiles; ++j) {
      const int a = j % ZTC_ACC;
      bool ok = ztc_wait(accf_bar(a), (uint32_t)((j / ZTC_ACC) & 1), abort_flag, err);
      if (!__all_sync(0xffffffffu, ok)) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const int64_t t = blockIdx.x + (int64_t)j * G;
      const ZtcTile zt = ztc_tile<BATCH>(t, spec, nz, ncols, segs, tprefix, S);
      const int d = zt.d;
      const int64_t ncols_t = zt.ncols;
      if (BATCH && zt.seg != eseg) {
        // the segment's epilogue arguments into this warp's shared slot
        const int *src = reinterpret_cast<const int *>(&segs[zt.seg].e);
        int *dst = reinterpret_cast<int *>(eslot);
        for (int w = lane; w < (int)(sizeof(EpiArgs) / 4); w += 32) dst[w] = src[w];
        __syncwarp();
        eseg = zt.seg;
      }
      const EpiArgs &et = BATCH ? *eslot : e;
      const bool v4 = (ncols_t & 3) == 0;  // 16-byte aligned rows
      const bool corr = CORR && et.inverse && et.ks.mode != 0 && et.corr != nullptr;
      const float scale = et.inverse ? (float)et.scale : 1.0f;
      const uint32_t tbase = tmem + ((uint32_t)(32 * qd) << 16) + (uint32_t)(a * ZTC_N);
      tmem_ld(tbase);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      for (int sb = 0; sb < ZTC_N / 32; ++sb) {
        // row `lane` of the block -> staging (8 x 16 B, conflict-free per quarter warp)
        float4 *srow = reinterpret_cast<float4 *>(st + lane * ZTC_STG);
#pragma unroll
        for (int c = 0; c < 8; ++c)
          srow[c] = make_float4(__uint_as_float(v[4 * c]), __uint_as_float(v[4 * c + 1]),
                                __uint_as_float(v[4 * c + 2]), __uint_as_float(v[4 * c + 3]));
        __syncwarp();
        if (sb + 1 < ZTC_N / 32) tmem_ld(tbase + (uint32_t)(32 * (sb + 1)));
        // 4 rows x 128 B per store instruction
        const int64_t col = zt.col0 + 32 * sb + 4 * (lane & 7);
#pragma unroll 4
        for (int i = 0; i < 8; ++i) {
          const int rl = 4 * i + (lane >> 3);
          const int r = 32 * qd + rl;
          if (r < nz && col < ncols_t) {
            float4 q = *reinterpret_cast<const float4 *>(st + rl * ZTC_STG + 4 * (lane & 7));
            if (corr) {
              float c0r, c0i, c1r, c1i;
              corr_any<float>(et, d, r, col >> 1, c0r, c0i);
              if (col + 2 < ncols_t) corr_any<float>(et, d, r, (col >> 1) + 1, c1r, c1i);
              else c1r = c1i = 0.0f;
              q.x += c0r;
              q.y += c0i;
              q.z += c1r;
              q.w += c1i;
            }
            q.x *= scale;
            q.y *= scale;
            q.z *= scale;
            q.w *= scale;
            float *g = zt.B + (int64_t)r * ncols_t + col;
            if (v4) {
              __stcs(reinterpret_cast<float4 *>(g), q);
            } else {
              __stcs(reinterpret_cast<float2 *>(g), make_float2(q.x, q.y));
              if (col + 2 < ncols_t) __stcs(reinterpret_cast<float2 *>(g + 2), make_float2(q.z, q.w));
            }
          }
        }
        if (sb + 1 < ZTC_N / 32) {
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          if (sb + 2 == ZTC_N / 32) {  // the last block is in registers: release the accumulator
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncwarp();
            if (lane == 0) mbar_arrive(acce_bar(a));
          }
        }
        __syncwarp();  // staging reused by the next block
      }
    }
  } else {
    // ---- MMA warp: every lane takes the waits (warp vote), lane 0 issues
    const uint32_t idesc = ztc_idesc(128, ZTC_N);
    const uint32_t a_hi = smem_u32(Ahi), a_lo = smem_u32(Alo);
    const uint32_t sbo_a = kq * 128, sbo_b = SKQ * 128;
    for (int u = 0; u < my_steps; ++u) {
      const int j = u / nkc, c = u - j * nkc;
      const int s = u % ZTC_STAGES, a = j % ZTC_ACC;
      bool ok = ztc_wait(full_bar(s), (uint32_t)((u / ZTC_STAGES) & 1), abort_flag, err);
      if (!__all_sync(0xffffffffu, ok)) break;
      if (c == 0) {
        ok = ztc_wait(acce_bar(a), (uint32_t)(((j / ZTC_ACC) & 1) ^ 1), abort_flag, err);
        if (!__all_sync(0xffffffffu, ok)) break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      if (lane == 0) {
        const uint32_t b_hi = smem_u32(Bst + (size_t)s * 2 * ZTC_N * ZTC_KC);
        const uint32_t b_lo = b_hi + (uint32_t)(ZTC_N * ZTC_KC * 4);
        const uint32_t dt = tmem + (uint32_t)(a * ZTC_N);
        const int ksteps = min(ZTC_KC, kp - ZTC_KC * c) / 8;
        for (int ks = 0; ks < ksteps; ++ks) {
          const uint32_t offa = (uint32_t)(ZTC_KC / 8 * c + ks) * 256u, offb = (uint32_t)ks * 256u;
          const uint64_t ah = smem_desc(a_hi + offa, 128, sbo_a), al = smem_desc(a_lo + offa, 128, sbo_a);
          const uint64_t bh = smem_desc(b_hi + offb, 128, sbo_b), bl = smem_desc(b_lo + offb, 128, sbo_b);
          mma_tf32(dt, ah, bh, idesc, (c > 0 || ks > 0) ? 1u : 0u);
          mma_tf32(dt, ah, bl, idesc, 1u);
          mma_tf32(dt, al, bh, idesc, 1u);
        }
        tc_commit(empty_bar(s));                     // the stage is free once these products are done
        if (c == nkc - 1) tc_commit(accf_bar(a));    // and after the last stage, the accumulator
      }
      __syncwarp();
    }
    // every issued product completes before the tensor memory is freed
    if (lane == 0) tc_commit(drain_bar);
    __syncwarp();
    ztc_wait(drain_bar, 0u, abort_flag, err, false);
    __syncwarp();
  }
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ZTC_TMEM_COLS));
  }
}

template <bool BATCH>
static cudaError_t ztc_launch(float *spec, int nz, int64_t ncols, const float *Tm, const EpiArgs &e, int nsm, int *err,
                              const ZSeg<float> *segs, const int64_t *tprefix, int S, int64_t ntiles, bool corr,
                              cudaStream_t s) {
  if (nz > 128) return cudaErrorInvalidValue;
  const size_t smem = BATCH ? ztc_smem_bytes_b(nz) : ztc_smem_bytes(nz);
  cudaError_t r;
  if (corr)
    r = cudaFuncSetAttribute(k_zgemm_tc<true, BATCH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  else r = cudaFuncSetAttribute(k_zgemm_tc<false, BATCH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (r != cudaSuccess) return r;
  int per_sm = 0;
  if (corr)
    r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_zgemm_tc<true, BATCH>, ZTC_THREADS, smem);
  else r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_zgemm_tc<false, BATCH>, ZTC_THREADS, smem);
  if (r != cudaSuccess) return r;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  if (per_sm > 2) per_sm = 2;  // 2 x 256 tensor-memory columns: allocation never waits
  int64_t grid = (int64_t)nsm * per_sm;
  if (grid > ntiles) grid = ntiles;
  if (grid < 1) return cudaSuccess;
  if (corr)
    k_zgemm_tc<true, BATCH><<<(unsigned)grid, ZTC_THREADS, smem, s>>>(spec, nz, ncols, Tm, e, err, segs, tprefix, S,
                                                                      ntiles);
  else
    k_zgemm_tc<false, BATCH><<<(unsigned)grid, ZTC_THREADS, smem, s>>>(spec, nz, ncols, Tm, e, err, segs, tprefix, S,
                                                                       ntiles);
  return cudaGetLastError();
}

cudaError_t launch_zgemm_tc(float *spec, int nz, int64_t ncols, const float *Tm, const EpiArgs &e, int nsm,
                            int *err, cudaStream_t s) {
  const int64_t ntiles = 3 * ((ncols + ZTC_N - 1) / ZTC_N);
  const bool corr = e.inverse != 0 && e.ks.mode != 0 && e.corr != nullptr;
  return ztc_launch<false>(spec, nz, ncols, Tm, e, nsm, err, nullptr, nullptr, 0, ntiles, corr, s);
}

// Batched systems: one launch over the tiles of every segment (system);
// tprefix: S + 1 prefix counts of 3 ceil(ncols_s / 128) tiles, in device
// memory, ntiles = tprefix[S].  Segments share nz and T.
int64_t ztc_tiles(int64_t ncols) { return 3 * ((ncols + ZTC_N - 1) / ZTC_N); }
// corr: some segment's epilogue adds a wall correction (else the lighter
// instantiation runs; each segment's EpiArgs says whether it is an inverse).
cudaError_t launch_zgemm_tc_b(const ZSeg<float> *segs, const int64_t *tprefix, int S, int64_t ntiles, int nz,
                              const float *Tm, bool corr, int nsm, int *err, cudaStream_t s) {
  EpiArgs e;
  memset(&e, 0, sizeof(e));
  return ztc_launch<true>(nullptr, nz, 0, Tm, e, nsm, err, segs, tprefix, S, ntiles, corr, s);
}

// ---------------------------------------------------------------------------
// The same transform fed by the tensor memory accelerator (TMA).
//
// Differences from k_zgemm_tc:
//   * T (hi, lo) is the MMA's A operand in tensor memory (columns 256-383
//     hi, 384-511 lo; lane = row), written once with tcgen05.st, so shared
//     memory holds only the streamed B operand and staging;
//   * one thread issues cp.async.bulk.tensor loads of 32-row x 128-column
//     FP32 blocks ([32][128] row-major, zero-filled past nz and ncols) into
//     a ring of RS stages, each completing on its mbarrier with the
//     block's byte count; no register holds a load in flight;
//   * 8 converter warps read a block from the ring, split it into TF32
//     hi / lo and write the canonical K-major stages the MMAs read;
//   * 4 epilogue warps scale the accumulator's 32 x 32 blocks into
//     128-byte-swizzled staging (two buffers per warp) and store each block
//     with one cp.async.bulk.tensor store (rows >= nz and columns >= ncols
//     clipped by the tensor map).
// The spectrum is one 3-D tensor [3][nz][ncols] (ncols a multiple of 4, so
// that its rows start on 16-byte boundaries; every x coordinate is a
// multiple of 32 columns).  No wall-correction epilogue: the inverse with
// walls runs k_corr_add afterwards, as for the other tcgen05 form.
// ---------------------------------------------------------------------------
constexpr int ZTM_CONV_WARPS = 8;
constexpr int ZTM_EPI_WARPS = 4;
constexpr int ZTM_MMA_WARP = ZTM_CONV_WARPS + ZTM_EPI_WARPS;  // warp 12
constexpr int ZTM_TMA_WARP = ZTM_MMA_WARP + 1;                // warp 13
constexpr int ZTM_THREADS = 32 * (ZTM_TMA_WARP + 1);
constexpr int ZTM_TMEM_COLS = 512;                            // 2 accumulators, T hi, T lo
constexpr uint32_t ZTM_COL_AHI = 2 * ZTC_N, ZTM_COL_ALO = 3 * ZTC_N;
constexpr uint32_t ZTM_RAW_BYTES = ZTC_KC * ZTC_N * 4;        // 16 KB
constexpr uint32_t ZTM_HL_BYTES = 2 * ZTC_N * ZTC_KC * 4;     // hi + lo, 32 KB
constexpr uint32_t ZTM_STG_BYTES = 32 * 32 * 4;               // one 32 x 32 block, 4 KB
constexpr int ZTM_TP = 128 + 4;                               // T's row pitch in shared memory (floats)
// Shared-memory layout of a variant: RS ring stages of raw blocks, HL
// converted (hi, lo) stages, the epilogue's staging, the mbarriers.
template <int RS, int HL>
struct ZtmCfg {
  static constexpr size_t off_hl = (size_t)RS * ZTM_RAW_BYTES;
  static constexpr size_t off_stg = off_hl + (size_t)HL * ZTM_HL_BYTES;
  static constexpr size_t off_bar = off_stg + (size_t)ZTM_EPI_WARPS * 2 * ZTM_STG_BYTES;
  static constexpr int nbars = 2 * RS + 2 * HL + 2 * ZTC_ACC + 1;
  static constexpr size_t smem = off_bar + nbars * 8 + 16 + 1024;  // + alignment slack
  static_assert(smem <= 227 * 1024, "TMA z transform: shared memory");
  static_assert(off_hl % 1024 == 0 && off_stg % 1024 == 0, "1024-byte aligned regions");
  static_assert(off_bar - off_hl >= (size_t)128 * ZTM_TP * 4, "T staged over the converted stages and staging");
};

static __device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

static __device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int x, int y, int z,
                                                   uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

static __device__ __forceinline__ void tma_store_3d(const CUtensorMap *map, uint32_t src, int x, int y, int z) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(src), "r"(x), "r"(y), "r"(z)
               : "memory");
}

// D += A B with A (128 x 8 TF32) in tensor memory, B by descriptor
static __device__ __forceinline__ void mma_tf32_ta(uint32_t dtmem, uint32_t atmem, uint64_t bd, uint32_t idesc,
                                                   uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "r"(atmem), "l"(bd), "r"(idesc), "r"(acc));
}

// BATCH: the tiles of S segments (systems) numbered by the prefix tprefix of
// 3 ceil(ncols_s / 128) tiles each; segment s's load and store maps are
// gmaps[2 s], gmaps[2 s + 1] (global memory) and its scale is its EpiArgs'.
struct ZtmTile {
  int64_t col0;
  int d, seg;
};
template <bool BATCH>
static __device__ __forceinline__ ZtmTile ztm_tile(int64_t t, int64_t ncols, const ZSeg<float> *__restrict__ segs,
                                                   const int64_t *__restrict__ tprefix, int S) {
  ZtmTile z;
  z.seg = 0;
  if (BATCH) {
    int lo = 0, hi = S - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (tprefix[mid] <= t) lo = mid;
      else hi = mid - 1;
    }
    z.seg = lo;
    t -= tprefix[lo];
    ncols = segs[lo].ncols;
  }
  const int64_t tpc = (ncols + ZTC_N - 1) / ZTC_N;
  z.d = (int)(t / tpc);
  z.col0 = (t % tpc) * ZTC_N;
  return z;
}

static __device__ __forceinline__ void tmap_acquire(const CUtensorMap *m) {
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(reinterpret_cast<uint64_t>(m))
               : "memory");
}

template <int RS, int HL, bool BATCH>
__global__ void __launch_bounds__(ZTM_THREADS, 1)
    k_zgemm_tma(const __grid_constant__ CUtensorMap map_ld, const __grid_constant__ CUtensorMap map_st, int nz,
                int64_t ncols, const float *__restrict__ Tm, float scale, int *err, const CUtensorMap *gmaps,
                const ZSeg<float> *__restrict__ segs, const int64_t *__restrict__ tprefix, int S, int64_t ntiles_b) {
  using Cfg = ZtmCfg<RS, HL>;
  extern __shared__ unsigned char ztm_raw_sm[];
  // 1024-byte alignment of the swizzled staging (the dynamic window's base
  // alignment is not guaranteed beyond 16 bytes)
  unsigned char *sm = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(ztm_raw_sm) + 1023) & ~static_cast<uintptr_t>(1023));
  const int kp = (nz + 7) & ~7;
  const uint32_t raw0 = smem_u32(sm);
  uint32_t *Hst = reinterpret_cast<uint32_t *>(sm + Cfg::off_hl);
  const float *rawf = reinterpret_cast<const float *>(sm);
  float *stg = reinterpret_cast<float *>(sm + Cfg::off_stg);
  uint64_t *bars = reinterpret_cast<uint64_t *>(sm + Cfg::off_bar);
  const uint32_t bar0 = smem_u32(bars);
  auto rfull_bar = [&](int s) { return bar0 + 8u * (uint32_t)s; };
  auto rempty_bar = [&](int s) { return bar0 + 8u * (uint32_t)(RS + s); };
  auto full_bar = [&](int s) { return bar0 + 8u * (uint32_t)(2 * RS + s); };
  auto empty_bar = [&](int s) { return bar0 + 8u * (uint32_t)(2 * RS + HL + s); };
  auto accf_bar = [&](int a) { return bar0 + 8u * (uint32_t)(2 * RS + 2 * HL + a); };
  auto acce_bar = [&](int a) { return bar0 + 8u * (uint32_t)(2 * RS + 2 * HL + ZTC_ACC + a); };
  const uint32_t drain_bar = bar0 + 8u * (uint32_t)(Cfg::nbars - 1);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + Cfg::nbars);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(ZTM_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int s = 0; s < RS; ++s) {
      mbar_init(rfull_bar(s), 1);
      mbar_init(rempty_bar(s), ZTM_CONV_WARPS);
    }
    for (int s = 0; s < HL; ++s) {
      mbar_init(full_bar(s), ZTM_CONV_WARPS);
      mbar_init(empty_bar(s), 1);
    }
    for (int a = 0; a < ZTC_ACC; ++a) {
      mbar_init(accf_bar(a), 1);
      mbar_init(acce_bar(a), ZTM_EPI_WARPS);
    }
    mbar_init(drain_bar, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (!BATCH && warp == ZTM_TMA_WARP && lane == 0) {  // (BATCH: the parameter maps are unused)
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&map_ld)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&map_st)) : "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;");
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;

  const int64_t ntiles = BATCH ? ntiles_b : 3 * ((ncols + ZTC_N - 1) / ZTC_N);
  const int64_t G = gridDim.x;
  const int my_tiles = (blockIdx.x < ntiles) ? (int)((ntiles - 1 - blockIdx.x) / G + 1) : 0;
  const int nkc = (kp + ZTC_KC - 1) / ZTC_KC;  // stages per tile
  const int my_steps = my_tiles * nkc;         // step u = (tile u / nkc, K chunk u % nkc)
  constexpr int SKQ = ZTC_KC / 4;

  // TMA: step u's block into ring stage u % RS once the stage is free
  int issued = 0, ld_j = -1, ld_seg = -1;
  ZtmTile ld_t;
  ld_t.col0 = 0;
  ld_t.d = ld_t.seg = 0;
  auto tma_issue = [&](int u) -> bool {
    const int rs = u % RS;
    if (!ztc_wait(rempty_bar(rs), (uint32_t)(((u / RS) & 1) ^ 1), abort_flag, err)) return false;
    const int j = u / nkc, c = u - j * nkc;
    if (j != ld_j) {
      ld_t = ztm_tile<BATCH>(blockIdx.x + (int64_t)j * G, ncols, segs, tprefix, S);
      ld_j = j;
    }
    const CUtensorMap *m = &map_ld;
    if (BATCH) {
      m = gmaps + 2 * ld_t.seg;
      if (ld_t.seg != ld_seg) {
        tmap_acquire(m);
        ld_seg = ld_t.seg;
      }
    }
    mbar_expect_tx(rfull_bar(rs), ZTM_RAW_BYTES);
    tma_load_3d(raw0 + (uint32_t)rs * ZTM_RAW_BYTES, m, (int)ld_t.col0, ZTC_KC * c, ld_t.d, rfull_bar(rs));
    issued = u + 1;
    return true;
  };
  // the first ring stages are filled while T is set up
  if (warp == ZTM_TMA_WARP && lane == 0)
    for (int u = 0; u < min(RS, my_steps); ++u)
      if (!tma_issue(u)) break;

  // T through shared memory ([128][ZTM_TP] floats over the converted stages
  // and the staging, not yet in use): coalesced loads by every thread, then
  // each epilogue warp splits its lane quadrant's rows into tf32 hi / lo,
  // 8 columns per tcgen05.st; rows and columns >= nz zero
  float *tsm = reinterpret_cast<float *>(sm + Cfg::off_hl);
  for (int idx = tid; idx < 128 * kp; idx += ZTM_THREADS) {
    const int r = idx / kp, k = idx - (idx / kp) * kp;
    tsm[r * ZTM_TP + k] = (r < nz && k < nz) ? Tm[r * nz + k] : 0.0f;
  }
  __syncthreads();
  if (warp >= ZTM_CONV_WARPS && warp < ZTM_MMA_WARP) {
    const int r = 32 * (warp & 3) + lane;
    const uint32_t trow = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
    for (int k0 = 0; k0 < kp; k0 += 8) {
      uint32_t h[8], l[8];
      const float4 va = *reinterpret_cast<const float4 *>(tsm + r * ZTM_TP + k0);
      const float4 vb = *reinterpret_cast<const float4 *>(tsm + r * ZTM_TP + k0 + 4);
      const float tv[8] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z, vb.w};
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        h[i] = to_tf32(tv[i]);
        l[i] = to_tf32(tv[i] - __uint_as_float(h[i]));
      }
      asm volatile(
          "tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(
              trow + ZTM_COL_AHI + (uint32_t)k0),
          "r"(h[0]), "r"(h[1]), "r"(h[2]), "r"(h[3]), "r"(h[4]), "r"(h[5]), "r"(h[6]), "r"(h[7])
          : "memory");
      asm volatile(
          "tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(
              trow + ZTM_COL_ALO + (uint32_t)k0),
          "r"(l[0]), "r"(l[1]), "r"(l[2]), "r"(l[3]), "r"(l[4]), "r"(l[5]), "r"(l[6]), "r"(l[7])
          : "memory");
    }
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");

  if (warp < ZTM_CONV_WARPS) {
    // ---- converters: column n, row quads q = qg + ZTC_PGROUPS i of the chunk
    const int n = tid % ZTC_N, qg = tid / ZTC_N;
    for (int u = 0; u < my_steps; ++u) {
      const int rs = u % RS;
      bool ok = ztc_wait(rfull_bar(rs), (uint32_t)((u / RS) & 1), abort_flag, err);
      if (!__all_sync(0xffffffffu, ok)) break;
      const float *rb = rawf + (size_t)rs * (ZTC_KC * ZTC_N);
      float br[ZTC_QPT][4];
#pragma unroll
      for (int i = 0; i < ZTC_QPT; ++i) {
        const int q = qg + ZTC_PGROUPS * i;
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) br[i][jj] = rb[(4 * q + jj) * ZTC_N + n];
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(rempty_bar(rs));
      const int s = u % HL;
      ok = ztc_wait(empty_bar(s), (uint32_t)(((u / HL) & 1) ^ 1), abort_flag, err);
      if (!__all_sync(0xffffffffu, ok)) break;
      uint32_t *Bhi = Hst + (size_t)s * 2 * ZTC_N * ZTC_KC, *Blo = Bhi + ZTC_N * ZTC_KC;
#pragma unroll
      for (int i = 0; i < ZTC_QPT; ++i) {
        const int q = qg + ZTC_PGROUPS * i;
        uint4 h, l;
        h.x = to_tf32(br[i][0]);
        h.y = to_tf32(br[i][1]);
        h.z = to_tf32(br[i][2]);
        h.w = to_tf32(br[i][3]);
        l.x = to_tf32(br[i][0] - __uint_as_float(h.x));
        l.y = to_tf32(br[i][1] - __uint_as_float(h.y));
        l.z = to_tf32(br[i][2] - __uint_as_float(h.z));
        l.w = to_tf32(br[i][3] - __uint_as_float(h.w));
        const int o = cm_off(n, 4 * q, SKQ);
        *reinterpret_cast<uint4 *>(Bhi + o) = h;
        *reinterpret_cast<uint4 *>(Blo + o) = l;
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(full_bar(s));
    }
  } else if (warp < ZTM_MMA_WARP) {
    // ---- epilogue: warp owns lane quadrant qd = rows 32 qd .. 32 qd + 31
    const int qd = warp & 3;
    float *st0 = stg + (size_t)(warp - ZTM_CONV_WARPS) * 2 * (ZTM_STG_BYTES / 4);
    uint32_t v[32];
    auto tmem_ld = [&](uint32_t taddr) {
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
          "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
            "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]),
            "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
            "=r"(v[30]), "=r"(v[31])
          : "r"(taddr)
          : "memory");
    };
    const bool rows_live = 32 * qd < nz;
    int nst = 0;  // blocks stored by this warp (staging buffer nst & 1)
    int st_seg = -1;
    const CUtensorMap *mst = &map_st;
    int64_t ncols_t = ncols;
    for (int j = 0; j < my_tiles; ++j) {
      const int a = j % ZTC_ACC;
      bool ok = ztc_wait(accf_bar(a), (uint32_t)((j / ZTC_ACC) & 1), abort_flag, err);
      if (!__all_sync(0xffffffffu, ok)) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const ZtmTile zt = ztm_tile<BATCH>(blockIdx.x + (int64_t)j * G, ncols, segs, tprefix, S);
      const int d = zt.d;
      const int64_t col0 = zt.col0;
      if (BATCH && zt.seg != st_seg) {
        st_seg = zt.seg;
        mst = gmaps + 2 * st_seg + 1;
        ncols_t = segs[st_seg].ncols;
        scale = segs[st_seg].e.inverse ? (float)segs[st_seg].e.scale : 1.0f;
        if (lane == 0) tmap_acquire(mst);
        __syncwarp();
      }
      const uint32_t tbase = tmem + ((uint32_t)(32 * qd) << 16) + (uint32_t)(a * ZTC_N);
      tmem_ld(tbase);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      for (int sb = 0; sb < ZTC_N / 32; ++sb) {
        const bool live = rows_live && col0 + 32 * sb < ncols_t;
        float *st = st0 + (size_t)(nst & 1) * (ZTM_STG_BYTES / 4);
        if (live) {
          // the buffer's store of two blocks ago has read its source
          if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
          __syncwarp();
          // row `lane`: 16-byte chunk c at chunk position c ^ (lane & 7)
          // (the 128-byte swizzle of the store's tensor map)
          float4 *srow = reinterpret_cast<float4 *>(st + lane * 32);
#pragma unroll
          for (int c = 0; c < 8; ++c)
            srow[c ^ (lane & 7)] =
                make_float4(__uint_as_float(v[4 * c]) * scale, __uint_as_float(v[4 * c + 1]) * scale,
                            __uint_as_float(v[4 * c + 2]) * scale, __uint_as_float(v[4 * c + 3]) * scale);
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          __syncwarp();
        }
        if (sb + 1 < ZTC_N / 32) tmem_ld(tbase + (uint32_t)(32 * (sb + 1)));
        if (live) {
          if (lane == 0) {
            tma_store_3d(mst, smem_u32(st), (int)(col0 + 32 * sb), 32 * qd, d);
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
          }
          ++nst;
        }
        if (sb + 1 < ZTC_N / 32) {
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          if (sb + 2 == ZTC_N / 32) {  // the last block is in registers: release the accumulator
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncwarp();
            if (lane == 0) mbar_arrive(acce_bar(a));
          }
        }
      }
    }
    if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    __syncwarp();
  } else if (warp == ZTM_MMA_WARP) {
    // ---- MMA warp: every lane takes the waits (warp vote), lane 0 issues
    const uint32_t idesc = ztc_idesc(128, ZTC_N);
    const uint32_t sbo_b = SKQ * 128;
    for (int u = 0; u < my_steps; ++u) {
      const int j = u / nkc, c = u - j * nkc;
      const int s = u % HL, a = j % ZTC_ACC;
      bool ok = ztc_wait(full_bar(s), (uint32_t)((u / HL) & 1), abort_flag, err);
      if (!__all_sync(0xffffffffu, ok)) break;
      if (c == 0) {
        ok = ztc_wait(acce_bar(a), (uint32_t)(((j / ZTC_ACC) & 1) ^ 1), abort_flag, err);
        if (!__all_sync(0xffffffffu, ok)) break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      if (lane == 0) {
        const uint32_t b_hi = smem_u32(Hst + (size_t)s * 2 * ZTC_N * ZTC_KC);
        const uint32_t b_lo = b_hi + (uint32_t)(ZTC_N * ZTC_KC * 4);
        const uint32_t dt = tmem + (uint32_t)(a * ZTC_N);
        const int ksteps = min(ZTC_KC, kp - ZTC_KC * c) / 8;
        for (int ks = 0; ks < ksteps; ++ks) {
          const uint32_t acol = (uint32_t)(ZTC_KC * c + 8 * ks), offb = (uint32_t)ks * 256u;
          const uint64_t bh = smem_desc(b_hi + offb, 128, sbo_b), bl = smem_desc(b_lo + offb, 128, sbo_b);
          mma_tf32_ta(dt, tmem + ZTM_COL_AHI + acol, bh, idesc, (c > 0 || ks > 0) ? 1u : 0u);
          mma_tf32_ta(dt, tmem + ZTM_COL_AHI + acol, bl, idesc, 1u);
          mma_tf32_ta(dt, tmem + ZTM_COL_ALO + acol, bh, idesc, 1u);
        }
        tc_commit(empty_bar(s));
        if (c == nkc - 1) tc_commit(accf_bar(a));
      }
      __syncwarp();
    }
    if (lane == 0) tc_commit(drain_bar);
    __syncwarp();
    ztc_wait(drain_bar, 0u, abort_flag, err, false);
    __syncwarp();
  } else {
    // ---- TMA warp: lane 0 streams the blocks of this CTA's tiles
    if (lane == 0) {
      if (issued == min(RS, my_steps))
        for (int u = issued; u < my_steps; ++u)
          if (!tma_issue(u)) break;
      // every issued load has landed before the shared memory is released
      for (int u = max(0, issued - RS); u < issued; ++u)
        ztc_wait(rfull_bar(u % RS), (uint32_t)((u / RS) & 1), abort_flag, err, false);
    }
    __syncwarp();
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ZTM_TMEM_COLS));
  }
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library)
typedef CUresult (*ztm_encode_fn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static ztm_encode_fn ztm_encoder() {
  static ztm_encode_fn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<ztm_encode_fn>(p);
  });
  return fn;
}

// The load (128 x 32 blocks, no swizzle) and store (32 x 32 blocks, 128-byte
// swizzle) maps of the tensor [3][nz][ncols] at spec, encoded once per
// (device, spec, nz, ncols) and kept in a small cache (a launch then costs
// no driver call beyond the launch itself).
static bool ztm_encode(float *spec, int nz, int64_t ncols, CUtensorMap &mld, CUtensorMap &mst) {
  const cuuint64_t dims[3] = {(cuuint64_t)ncols, (cuuint64_t)nz, 3};
  const cuuint64_t strides[2] = {(cuuint64_t)ncols * 4, (cuuint64_t)ncols * 4 * (cuuint64_t)nz};
  const cuuint32_t box_ld[3] = {ZTC_N, ZTC_KC, 1}, box_st[3] = {32, 32, 1}, es[3] = {1, 1, 1};
  ztm_encode_fn enc = ztm_encoder();
  if (enc == nullptr) return false;
  if (enc(&mld, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, spec, dims, strides, box_ld, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  return enc(&mst, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, spec, dims, strides, box_st, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_NONE,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
struct ZtmMaps {
  CUtensorMap ld, st;
  const void *p;
  int64_t ncols;
  int nz, dev;
};
static bool ztm_maps(float *spec, int nz, int64_t ncols, CUtensorMap &mld, CUtensorMap &mst) {
  static std::mutex mu;
  static ZtmMaps cache[8];
  static int used = 0, next = 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  std::lock_guard<std::mutex> lock(mu);
  for (int i = 0; i < used; ++i)
    if (cache[i].p == spec && cache[i].nz == nz && cache[i].ncols == ncols && cache[i].dev == dev) {
      mld = cache[i].ld;
      mst = cache[i].st;
      return true;
    }
  if (!ztm_encode(spec, nz, ncols, mld, mst)) return false;
  ZtmMaps &c = cache[next];
  next = (next + 1) % 8;
  if (used < 8) ++used;
  c.ld = mld;
  c.st = mst;
  c.p = spec;
  c.nz = nz;
  c.ncols = ncols;
  c.dev = dev;
  return true;
}

// The spectrum qualifies: 16-byte aligned base, 4 | ncols (16-byte row
// pitch), 32 <= nz <= 128, an encoder available.
bool ztm_supported(const float *spec, int nz, int64_t ncols) {
  return nz >= 32 && nz <= 128 && ncols > 0 && (ncols & 3) == 0 && ncols < (int64_t(1) << 31) &&
         (reinterpret_cast<uintptr_t>(spec) & 15) == 0 && ztm_encoder() != nullptr;
}

template <int RS, int HL, bool BATCH = false>
static cudaError_t ztm_launch(const CUtensorMap &mld, const CUtensorMap &mst, int nz, int64_t ncols, const float *Tm,
                              float scale, int64_t grid, int *err, cudaStream_t s, const CUtensorMap *gmaps = nullptr,
                              const ZSeg<float> *segs = nullptr, const int64_t *tprefix = nullptr, int S = 0,
                              int64_t ntiles_b = 0) {
  cudaError_t r = cudaFuncSetAttribute(k_zgemm_tma<RS, HL, BATCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)ZtmCfg<RS, HL>::smem);
  if (r != cudaSuccess) return r;
  k_zgemm_tma<RS, HL, BATCH><<<(unsigned)grid, ZTM_THREADS, ZtmCfg<RS, HL>::smem, s>>>(
      mld, mst, nz, ncols, Tm, scale, err, gmaps, segs, tprefix, S, ntiles_b);
  return cudaGetLastError();
}

// variant: (ring stages, converted stages) = (6, 2), (4, 3), (7, 2)
int ztm_variants() { return 3; }

cudaError_t launch_zgemm_tma(float *spec, int nz, int64_t ncols, const float *Tm, const EpiArgs &e, int nsm, int *err,
                             int variant, cudaStream_t s) {
  if (!ztm_supported(spec, nz, ncols)) return cudaErrorNotSupported;
  CUtensorMap mld, mst;
  if (!ztm_maps(spec, nz, ncols, mld, mst)) return cudaErrorInvalidValue;
  const int64_t ntiles = 3 * ((ncols + ZTC_N - 1) / ZTC_N);
  int64_t grid = nsm;  // one CTA per SM: all 512 tensor-memory columns
  if (grid > ntiles) grid = ntiles;
  const float scale = e.inverse ? (float)e.scale : 1.0f;
  switch (variant) {
    case 1: return ztm_launch<4, 3>(mld, mst, nz, ncols, Tm, scale, grid, err, s);
    case 2: return ztm_launch<7, 2>(mld, mst, nz, ncols, Tm, scale, grid, err, s);
    default: return ztm_launch<6, 2>(mld, mst, nz, ncols, Tm, scale, grid, err, s);
  }
}

// Batched systems: every segment's load and store maps, in segment order
// (2 S maps, for device memory), when every segment qualifies.
bool ztm_maps_b(const ZSeg<float> *segs, int S, int nz, std::vector<CUtensorMap> &out) {
  out.assign(2 * (size_t)S, CUtensorMap{});
  for (int i = 0; i < S; ++i) {
    if (!ztm_supported(segs[i].spec, nz, segs[i].ncols)) return false;
    if (!ztm_encode(segs[i].spec, nz, segs[i].ncols, out[2 * i], out[2 * i + 1])) return false;
  }
  return true;
}

// One launch over the tiles of every segment (tprefix as launch_zgemm_tc_b,
// device memory); gmaps: ztm_maps_b's maps in device memory.  The epilogue
// only scales (each segment's EpiArgs); the inverse's wall correction is the
// caller's separate pass.
cudaError_t launch_zgemm_tma_b(const ZSeg<float> *segs, const int64_t *tprefix, int S, int64_t ntiles, int nz,
                               const float *Tm, const CUtensorMap *gmaps, int nsm, int *err, cudaStream_t s) {
  if (nz < 32 || nz > 128 || ntiles <= 0) return cudaErrorInvalidValue;
  CUtensorMap unused;
  memset(&unused, 0, sizeof(unused));
  int64_t grid = nsm;
  if (grid > ntiles) grid = ntiles;
  return ztm_launch<6, 2, true>(unused, unused, nz, 0, Tm, 1.0f, grid, err, s, gmaps, segs, tprefix, S, ntiles);
}

// ---------------------------------------------------------------------------
// The wall correction as its own pass after an inverse z transform run
// without it: spec[d][m][mode] += corr_d(z_m, mode) scale for every
// component d and node m, one thread per mode (its coefficients read once,
// the node loop in the thread; consecutive threads take consecutive modes,
// so every access of a node row is coalesced).  The tcgen05 kernel's
// epilogue has only four warps per CTA for this arithmetic; the pass
// spreads it over the whole GPU.  BATCH: modes of the S segments by their
// prefix mprefix (nk_s each); ks.mode == 0 or corr == nullptr: nothing.
// ---------------------------------------------------------------------------
// WM: 1 bottom wall (three coefficients per mode), 2 slit (eight per pass).
// Threads: K modes x ceil(nz / CORR_NODES) node blocks (consecutive threads,
// consecutive modes of one node block).
constexpr int CORR_NODES = 16;
template <bool BATCH, int WM>
__global__ void __launch_bounds__(128) k_corr_add(float *spec, int nz, int64_t nk, EpiArgs e,
                                                  const ZSeg<float> *__restrict__ segs,
                                                  const int64_t *__restrict__ mprefix, int S, int64_t K) {
  const int64_t tt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int nblk = (nz + CORR_NODES - 1) / CORR_NODES;
  if (tt >= K * nblk) return;
  const int64_t t = tt % K;
  const int m_beg = (int)(tt / K) * CORR_NODES, m_end = min(m_beg + CORR_NODES, nz);
  int64_t mode = t;
  const EpiArgs *ep = &e;
  if (BATCH) {
    int lo = 0, hi = S - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (mprefix[mid] <= t) lo = mid;
      else hi = mid - 1;
    }
    mode = t - mprefix[lo];
    ep = &segs[lo].e;
    spec = segs[lo].spec;
    nk = segs[lo].ncols / 2;
  }
  const EpiArgs &ea = *ep;
  if (ea.corr == nullptr || mode == 0) return;
  const float scale = (float)ea.scale;
  float2 *__restrict__ g0 = reinterpret_cast<float2 *>(spec) + mode;
  if (ea.corrf == nullptr) {  // no FP32 tables: the general per-value form
    for (int d = 0; d < 3; ++d)
      for (int m = m_beg; m < m_end; ++m) {
        float re, im;
        corr_any<float>(ea, d, m, mode, re, im);
        float2 *g = g0 + ((int64_t)d * nz + m) * nk;
        float2 v = *g;
        v.x += re * scale;
        v.y += im * scale;
        *g = v;
      }
    return;
  }
  // corr_value_f for the three components at once, the mode's table entries
  // read once into registers, four nodes' values loaded ahead of their update
  typedef float CT;
  constexpr int NC = WM == 1 ? 3 : 16;
  const float4 m0 = ea.cmode[2 * mode];
  const CT k = m0.x;
  const int npass = m0.w != 0.0f ? 1 : 2;
  const float4 m1 = npass == 2 ? ea.cmode[2 * mode + 1] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const float2 *cr = ea.corrf + mode * 16;
  const int ncoef = WM == 1 ? 3 : 8 * npass;
  cplx<CT> c[NC];
#pragma unroll
  for (int r = 0; r < NC; ++r) c[r] = r < ncoef ? mk<CT>(cr[r].x, cr[r].y) : mk<CT>(0, 0);
  const CT fac = ea.fac, Lz = (CT)ea.ks.Lz;
  const float *__restrict__ znf = ea.znf;
  const int64_t dstride = (int64_t)nz * nk;
  // the node-independent parts of each pass, hoisted out of the node loop:
  //   bottom wall: v_x = (-qx/k) z e^{-kz} al + e^{-kz} f0, v_y likewise,
  //     v_z = -i z e^{-kz} al + e^{-kz} f2, al = qx f0 + qy f1 + i k f2
  //     (f conjugated in the Nyquist partner's pass);
  //   slit: the same with fac / k and the top wall's e^{k(z - Lz)} terms.
  cplx<CT> al[2], f[2][3];
  CT ax[2], ay[2];
#pragma unroll
  for (int pass = 0; pass < 2; ++pass) {
    const CT qx = pass ? m1.x : m0.y, qy = pass ? m1.y : m0.z;
    if constexpr (WM == 1) {
      f[pass][0] = pass ? conj(c[0]) : c[0];
      f[pass][1] = pass ? conj(c[1]) : c[1];
      f[pass][2] = pass ? conj(c[2]) : c[2];
      al[pass] = (qx * f[pass][0] + qy * f[pass][1]) + ik(k, f[pass][2]);
      ax[pass] = -qx / k;
      ay[pass] = -qy / k;
    } else {
      ax[pass] = qx * fac / k;
      ay[pass] = qy * fac / k;
    }
  }
  constexpr int U = 4;
  for (int mb = m_beg; mb < m_end; mb += U) {
    float2 vin[U][3];
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int d = 0; d < 3; ++d)
        vin[u][d] = (mb + u < m_end) ? g0[d * dstride + (int64_t)(mb + u) * nk] : make_float2(0.0f, 0.0f);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int m = mb + u;
      if (m >= m_end) break;
      const CT z = znf[m];
      const CT enkz = expf(-k * z);
      const CT zenkz = z * enkz;
      CT ekzmh = 0, zekzmh = 0;
      if constexpr (WM != 1) {
        ekzmh = expf(k * (z - Lz));
        zekzmh = z * ekzmh;
      }
      cplx<CT> acc[3] = {mk<CT>(0, 0), mk<CT>(0, 0), mk<CT>(0, 0)};
#pragma unroll
      for (int pass = 0; pass < 2; ++pass) {
        if (pass >= npass) break;
        cplx<CT> v[3];
        if constexpr (WM == 1) {
          v[0] = (ax[pass] * zenkz) * al[pass] + enkz * f[pass][0];
          v[1] = (ay[pass] * zenkz) * al[pass] + enkz * f[pass][1];
          v[2] = ik(-zenkz, al[pass]) + enkz * f[pass][2];
        } else {
          const int o = 8 * pass;
          v[0] = (ik(-ax[pass] * zenkz, c[o + 0]) + ik(ax[pass] * zekzmh, c[o + 1])) +
                 (enkz * c[o + 2] + ekzmh * c[o + 3]);
          v[1] = (ik(-ay[pass] * zenkz, c[o + 0]) + ik(ay[pass] * zekzmh, c[o + 1])) +
                 (enkz * c[o + 4] + ekzmh * c[o + 5]);
          v[2] = ((zenkz * fac) * c[o + 0] + (zekzmh * fac) * c[o + 1]) + (enkz * c[o + 6] + ekzmh * c[o + 7]);
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) acc[d] = acc[d] + (pass ? conj(v[d]) : v[d]);
      }
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        if (npass == 2) acc[d] = (CT)0.5 * acc[d];
        float2 vv = vin[u][d];
        vv.x += acc[d].x * scale;
        vv.y += acc[d].y * scale;
        g0[d * dstride + (int64_t)m * nk] = vv;
      }
    }
  }
}

cudaError_t launch_corr_add(float *spec, int nz, int64_t nk, const EpiArgs &e, cudaStream_t s) {
  if (nk <= 0 || e.ks.mode == 0) return cudaSuccess;
  const int bs = 128;
  const int64_t nt = nk * ((nz + CORR_NODES - 1) / CORR_NODES);
  const unsigned nb = (unsigned)((nt + bs - 1) / bs);
  if (e.ks.mode == 1) k_corr_add<false, 1><<<nb, bs, 0, s>>>(spec, nz, nk, e, nullptr, nullptr, 0, nk);
  else k_corr_add<false, 2><<<nb, bs, 0, s>>>(spec, nz, nk, e, nullptr, nullptr, 0, nk);
  return cudaGetLastError();
}

// wall: the systems' common geometry (1 bottom wall, 2 slit)
cudaError_t launch_corr_add_b(const ZSeg<float> *segs, const int64_t *mprefix, int S, int64_t K, int nz, int wall,
                              cudaStream_t s) {
  if (K <= 0 || wall == 0) return cudaSuccess;
  EpiArgs e;
  memset(&e, 0, sizeof(e));
  const int bs = 128;
  const int64_t nt = K * ((nz + CORR_NODES - 1) / CORR_NODES);
  const unsigned nb = (unsigned)((nt + bs - 1) / bs);
  if (wall == 1) k_corr_add<true, 1><<<nb, bs, 0, s>>>(nullptr, nz, 0, e, segs, mprefix, S, K);
  else k_corr_add<true, 2><<<nb, bs, 0, s>>>(nullptr, nz, 0, e, segs, mprefix, S, K);
  return cudaGetLastError();
}

}  // namespace dpst
