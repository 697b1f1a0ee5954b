// z transform of the mixed-precision operator on the 5th-generation tensor
// cores (tcgen05), split-TF32 with FP32 accumulation in tensor memory.
//
// The transform is OUT[r][col] = sum_m T[r][m] IN[m][col] over every real
// column of the spectrum (per component: nz rows x 2 nk columns, in place),
// with the inverse's epilogue adding the wall correction and scaling
// (corr_value, as k_zgemm does).  Per CTA tile: M = 128 rows (nz padded with
// zero rows of T), N = 64 columns, K = nz padded to a multiple of 8.  Each
// FP32 operand x is split as x = hi + lo with hi = tf32(x), lo = tf32(x - hi)
// and the product is accumulated as hi*hi + hi*lo + lo*hi (three
// tcgen05.mma.kind::tf32 per K step of 8), which keeps the FP32-level
// accuracy of the SIMT transform.
//
// Shared memory holds A = T (hi, lo) for the CTA's lifetime and B = the
// current tile (hi, lo) in the canonical K-major layout without swizzle:
// 8-row x 16-byte core matrices, consecutive along K (LBO = 128 B), 8-row
// groups SBO = (Kp / 4) * 128 B apart.  One thread issues the MMAs and
// commits them to an mbarrier; every thread waits on it with an iteration
// limit (on expiry the kernel records the error, stops and still frees its
// tensor memory).  While the MMAs of tile t run, the threads load tile t+1
// into registers.  The accumulator (128 lanes x 64 FP32 columns) is read
// back with tcgen05.ld by the warp owning each lane quadrant.
#include "dpst_internal.cuh"
#include "dpst_kdev.cuh"

namespace dpst {

constexpr int ZTC_N = 64;         // columns per tile
constexpr int ZTC_THREADS = 256;  // 8 warps: two per TMEM lane quadrant
constexpr int ZTC_TMEM_COLS = 64;
constexpr unsigned long long ZTC_WAIT_NS = 2000000000ull;  // 2 s

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

// Bytes of the B operand (hi, lo) region, which the epilogue reuses as its
// [128][ZTC_N + 1] FP32 staging.
static __host__ __device__ constexpr size_t ztc_b_region(int kp) {
  return (2 * (size_t)ZTC_N * kp * 4 > (size_t)128 * (ZTC_N + 1) * 4) ? 2 * (size_t)ZTC_N * kp * 4
                                                                      : (size_t)128 * (ZTC_N + 1) * 4;
}

// Element offset (in 32-bit words) of (row, k) in the core-matrix layout.
static __device__ __forceinline__ int cm_off(int row, int k, int kq) {
  return (row >> 3) * (kq * 32) + (k >> 2) * 32 + (row & 7) * 4 + (k & 3);
}

template <bool INVERSE>
__global__ void __launch_bounds__(ZTC_THREADS) k_zgemm_tc(float *spec, int nz, int64_t ncols,
                                                          const float *__restrict__ Tm, EpiArgs e, int *err) {
  extern __shared__ __align__(1024) unsigned char ztc_sm[];
  const int kp = (nz + 7) & ~7;  // K padded to the MMA step
  const int kq = kp / 4;         // core matrices along K
  uint32_t *Ahi = reinterpret_cast<uint32_t *>(ztc_sm);  // 128 x kp
  uint32_t *Alo = Ahi + 128 * kp;
  uint32_t *Bhi = Alo + 128 * kp;  // 64 x kp; reused as the epilogue's staging
  uint32_t *Blo = Bhi + ZTC_N * kp;
  float *stg = reinterpret_cast<float *>(Bhi);  // [128][ZTC_N + 1]
  uint64_t *mbar = reinterpret_cast<uint64_t *>(reinterpret_cast<unsigned char *>(Bhi) + ztc_b_region(kp));
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mbar + 1);
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
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("fence.proxy.async.shared::cta;");
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;

  const int64_t tiles_per_comp = (ncols + ZTC_N - 1) / ZTC_N;
  const int64_t ntiles = 3 * tiles_per_comp;
  // loader mapping: column n = tid % 64, row quads q = tid / 64 + 4 i
  const int ln = tid % ZTC_N, lq0 = tid / ZTC_N;
  constexpr int QPT = 128 / 4 / (ZTC_THREADS / ZTC_N);  // row quads per thread (kp <= 128)
  // two tiles in flight in registers: tile t (being consumed) and t + G
  float b0[QPT][4], b1[QPT][4];
  auto load_tile = [&](int64_t t, float (&br)[QPT][4]) {
    const int d = (int)(t / tiles_per_comp);
    const int64_t col = (t % tiles_per_comp) * ZTC_N + ln;
    const float *B = spec + (int64_t)d * nz * ncols;
#pragma unroll
    for (int i = 0; i < QPT; ++i) {
      const int q = lq0 + 4 * i;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int k = 4 * q + j;
        br[i][j] = (q < kq && k < nz && col < ncols && t < ntiles) ? __ldcs(B + (int64_t)k * ncols + col) : 0.0f;
      }
    }
  };
  auto split_tile = [&](const float (&br)[QPT][4]) {
#pragma unroll
    for (int i = 0; i < QPT; ++i) {
      const int q = lq0 + 4 * i;
      if (q >= kq) continue;
      uint4 h, l;
      h.x = to_tf32(br[i][0]);
      h.y = to_tf32(br[i][1]);
      h.z = to_tf32(br[i][2]);
      h.w = to_tf32(br[i][3]);
      l.x = to_tf32(br[i][0] - __uint_as_float(h.x));
      l.y = to_tf32(br[i][1] - __uint_as_float(h.y));
      l.z = to_tf32(br[i][2] - __uint_as_float(h.z));
      l.w = to_tf32(br[i][3] - __uint_as_float(h.w));
      const int o = cm_off(ln, 4 * q, kq);
      *reinterpret_cast<uint4 *>(Bhi + o) = h;
      *reinterpret_cast<uint4 *>(Blo + o) = l;
    }
  };
  const uint32_t idesc = ztc_idesc(128, ZTC_N);
  const uint32_t a_hi = smem_u32(Ahi), a_lo = smem_u32(Alo), b_hi = smem_u32(Bhi), b_lo = smem_u32(Blo);
  const uint32_t sbo = kq * 128;
  const int64_t G = gridDim.x;
  uint32_t phase = 0;
  bool ok = true;
  int64_t t = blockIdx.x;
  load_tile(t, b0);
  load_tile(t + G, b1);
  for (int it = 0; t < ntiles && ok; t += G, ++it) {
    if (it & 1) split_tile(b1);
    else split_tile(b0);
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      for (int s = 0; s < kp / 8; ++s) {
        const uint32_t off = (uint32_t)s * 256u;  // two core matrices along K
        const uint64_t ah = smem_desc(a_hi + off, 128, sbo), al = smem_desc(a_lo + off, 128, sbo);
        const uint64_t bh = smem_desc(b_hi + off, 128, sbo), bl = smem_desc(b_lo + off, 128, sbo);
        mma_tf32(tmem, ah, bh, idesc, s > 0 ? 1u : 0u);
        mma_tf32(tmem, ah, bl, idesc, 1u);
        mma_tf32(tmem, al, bh, idesc, 1u);
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(mbar)));
    }
    // the registers of tile t are free: start tile t + 2G
    if (it & 1) load_tile(t + 2 * G, b1);
    else load_tile(t + 2 * G, b0);
    // wait for the accumulator, at most ZTC_WAIT_NS; the verdict is taken
    // block-wide so that every thread leaves the loop together
    uint32_t done = 0;
    {
      unsigned long long t0, now;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
      for (int spin = 0; !done; ++spin) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(smem_u32(mbar)), "r"(phase));
        if (!done && (spin & 255) == 255) {
          asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
          if (now - t0 > ZTC_WAIT_NS) break;
        }
      }
    }
    if (!__syncthreads_and(done != 0)) {
      if (tid == 0) atomicOr(err, 1);
      ok = false;
      break;
    }
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;");
    // accumulator -> staging (the B operand's shared memory is free now):
    // warp w reads lanes 32 (w % 4) .. + 31, columns 32 (w / 4) .. + 31
    {
      uint32_t v[32];
      const uint32_t taddr = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(32 * (warp >> 2));
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
          "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
            "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]),
            "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
            "=r"(v[30]), "=r"(v[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;");
      float *row = stg + (32 * (warp & 3) + lane) * (ZTC_N + 1) + 32 * (warp >> 2);
#pragma unroll
      for (int j = 0; j < 32; ++j) row[j] = __uint_as_float(v[j]);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    // coalesced epilogue: warp w writes rows w, w + 8, ...; lane = column pair
    {
      const int d = (int)(t / tiles_per_comp);
      const int64_t col = (t % tiles_per_comp) * ZTC_N + 2 * lane;
      if (col < ncols) {
        for (int r = warp; r < nz; r += ZTC_THREADS / 32) {
          float vr = stg[r * (ZTC_N + 1) + 2 * lane], vi = stg[r * (ZTC_N + 1) + 2 * lane + 1];
          if (INVERSE) {
            float cre, cim;
            corr_value<float>(e, d, r, col >> 1, cre, cim);
            vr = (vr + cre) * (float)e.scale;
            vi = (vi + cim) * (float)e.scale;
          }
          __stcs(reinterpret_cast<float2 *>(spec + ((int64_t)d * nz + r) * ncols + col), make_float2(vr, vi));
        }
      }
    }
    __syncthreads();  // staging consumed before the next split overwrites it
  }
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ZTC_TMEM_COLS));
  }
}

size_t ztc_smem_bytes(int nz) {
  const int kp = (nz + 7) & ~7;
  return (size_t)2 * 128 * kp * 4 + ztc_b_region(kp) + 16;
}

cudaError_t launch_zgemm_tc(float *spec, int nz, int64_t ncols, const float *Tm, const EpiArgs &e, int nsm,
                            int *err, cudaStream_t s) {
  if (nz > 128) return cudaErrorInvalidValue;
  const size_t smem = ztc_smem_bytes(nz);
  cudaError_t r;
  if (e.inverse) r = cudaFuncSetAttribute(k_zgemm_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  else r = cudaFuncSetAttribute(k_zgemm_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (r != cudaSuccess) return r;
  const int64_t ntiles = 3 * ((ncols + ZTC_N - 1) / ZTC_N);
  int per_sm = 0;
  if (e.inverse) r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_zgemm_tc<true>, ZTC_THREADS, smem);
  else r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_zgemm_tc<false>, ZTC_THREADS, smem);
  if (r != cudaSuccess) return r;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  if (per_sm > 4) per_sm = 4;  // 4 x 64 tensor-memory columns: allocation never waits
  int64_t grid = (int64_t)nsm * per_sm;
  if (grid > ntiles) grid = ntiles;
  if (grid < 1) return cudaSuccess;
  if (e.inverse) k_zgemm_tc<true><<<(unsigned)grid, ZTC_THREADS, smem, s>>>(spec, nz, ncols, Tm, e, err);
  else k_zgemm_tc<false><<<(unsigned)grid, ZTC_THREADS, smem, s>>>(spec, nz, ncols, Tm, e, err);
  return cudaGetLastError();
}

}  // namespace dpst
