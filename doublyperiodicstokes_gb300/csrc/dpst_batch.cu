// Batched systems (dpst_batched_*, include/dpstokes_gb300.h): many
// independent doubly periodic systems with uneven particle counts and box
// sizes, run as one pipeline.  No counterpart in the reference (which runs
// one system per FCM / DPStokes instance); each system's result is the same
// operator dpst_mdot applies to it alone.
//
// Layout: particles concatenated in the caller's order; grids and spectra
// concatenated with systems sorted by (nx, ny), so systems of one size class
// are contiguous and one cuFFT plan (batch = systems x 3 x nz planes) covers
// the class.  Every other stage is one launch over all systems through
// per-system tables (SysP for the particle kernels, SysK for the per-mode
// solve, ZSeg for the z transform) with prefix counts of their work items.
// The Mdot pipeline is captured once per (dtype, torques, vorticity) into a
// CUDA graph over fixed staging buffers and replayed: one graph launch per
// batched Mdot.
// Shared across the batch (checked at creation): nz, zmin, zmax, geometry,
// viscosity, precision, torque flag.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <climits>
#include <map>
#include <memory>
#include <numeric>
#include <string>

#include "dpst_host.cuh"

namespace dpst {

void launch_bvp_factors(const KsArgs &a, cudaStream_t s);
template <typename R>
void launch_locate_b(bool dipole, const double *pos, int64_t total, const SysP<R> *sys, const int64_t *pprefix,
                     int S, const double *zext, const double *wext, int *err, int *reach, cudaStream_t s);
template <typename R, typename RF>
void launch_spread_b(bool dipole, const RF *FT, int64_t items, const SysP<R> *sys, const int64_t *iprefix, int S,
                     cudaStream_t s);
template <typename R>
void launch_ghost_fold_b(bool yaxis, const FoldJob<R> *jobs, const int64_t *jprefix, int J, int64_t items,
                         cudaStream_t s);
template <typename R, typename RV>
void launch_interp_b(bool dipole, int64_t total, const SysP<R> *sys, const int64_t *pprefix, int S, RV *out,
                     bool dip_ghosts, cudaStream_t s);
template <typename R>
cudaError_t bvp_plan_b(int nz, int64_t K, int nsm, int64_t *grid, size_t *scratch_bytes);
void launch_bvp_pack_df(const KsArgs &a, cudaStream_t s);
int bvp_df_variants();
cudaError_t bvp_df_plan_b(const KsArgs &a0, int64_t K, int nsm, int64_t *grid, size_t *scratch_bytes);
template <typename R>
cudaError_t launch_bvp_df_b(const SysK<R> *sys, int S, const int64_t *mprefix, int64_t K, int nz, int mode,
                            float2 *scratch, int64_t grid, int variant, cudaStream_t s, int ncol = 0);
template <typename R>
cudaError_t launch_bvp_k0_b(const SysK<R> *sys, int S, cudaStream_t s);
template <typename R>
cudaError_t launch_bvp_b(const SysK<R> *sys, int S, const int64_t *mprefix, int64_t K, int nz, double *scratch,
                         int64_t grid, cudaStream_t s);
template <typename R>
cudaError_t launch_zgemm_b(const ZSeg<R> *segs, const int64_t *tprefix, int S, int64_t ntiles, int nz, const R *Tm,
                           int nsm, cudaStream_t s, bool fold_out);
int64_t ztc_tiles(int64_t ncols);
cudaError_t launch_zgemm_tc_b(const ZSeg<float> *segs, const int64_t *tprefix, int S, int64_t ntiles, int nz,
                              const float *Tm, bool corr, int nsm, int *err, cudaStream_t s);
cudaError_t launch_corr_add_b(const ZSeg<float> *segs, const int64_t *mprefix, int S, int64_t K, int nz, int wall,
                              cudaStream_t s);
bool ztm_maps_b(const ZSeg<float> *segs, int S, int nz, std::vector<CUtensorMap> &out);
cudaError_t launch_zgemm_tma_b(const ZSeg<float> *segs, const int64_t *tprefix, int S, int64_t ntiles, int nz,
                               const float *Tm, const CUtensorMap *gmaps, int nsm, int *err, cudaStream_t s);

template <typename RP>
__global__ void k_prep_pos_b(const RP *pos, int64_t N, double zmin, double *out) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= N) return;
  out[3 * p] = (double)pos[3 * p];
  out[3 * p + 1] = (double)pos[3 * p + 1];
  out[3 * p + 2] = (double)pos[3 * p + 2] - zmin;
}

struct BatchBase {
  virtual ~BatchBase() {}
  virtual void set_positions(const void *pos, int dtype, cudaStream_t s) = 0;
  virtual void mdot(const void *F, const void *T, void *V, void *W, int dtype, cudaStream_t s) = 0;
  virtual void info(dpst_batch_info *o) const = 0;
  int device = 0;
};

template <typename T>
static void upload_vec(DevBuf &b, const std::vector<T> &v) {
  upload(b, v);
}

template <typename R>
struct BatchEngine : BatchBase {
  typedef typename std::conditional<sizeof(R) == 8, cufftDoubleComplex, cufftComplex>::type CR;
  int S = 0, nz = 0, mode = 0, nsm = 0;
  bool torque_op = false;
  double zmin = 0, Lz = 0, H = 0;
  int64_t Ntot = 0, K = 0, grid_elems = 0, spec_elems = 0;
  std::vector<int64_t> npart, pbase;
  std::vector<int> order;  // systems sorted by (nx, ny)
  // device tables
  DevBuf d_sysp, d_sysk, d_segf, d_segi, d_pprefix, d_ipm, d_ipd, d_mprefix, d_tprefix;
  // tcgen05 z transform over every system (mixed operator): its tile prefix,
  // tile count, error word, the choice per direction {forward, inverse} and
  // the creation-time timings {SIMT, tcgen05} per direction
  DevBuf d_tprefix_tc, ztc_err, d_segi_nc;  // d_segi_nc: the inverse segments without the wall correction
  int64_t ntiles_tc = 0;
  // per direction: 0 SIMT, 1 tcgen05 (register-staged operands), 3 tcgen05
  // fed by TMA (every system's spectrum through its own tensor maps, d_tmaps)
  int ztc_use[2] = {0, 0};
  float ztc_ms[2][2] = {{0.0f, 0.0f}, {0.0f, 0.0f}};
  float ztm_ms[2] = {0.0f, 0.0f};
  // the TMA form runs over the systems whose spectrum rows start on 16-byte
  // boundaries (an even mode count; "a" tables: forward segments, inverse
  // segments without the correction, tile prefix, the tensor maps) and the
  // register-staged form over the others ("b" tables)
  DevBuf d_tmaps, d_segf_a, d_segi_a, d_tp_a, d_segf_b, d_segi_b, d_tp_b;
  int S_a = 0, S_b = 0;
  int64_t ntiles_a = 0, ntiles_b = 0;
  bool tma_ok = false;
  DevBuf d_jobs_m, d_jobs_d, d_jpx_m, d_jpy_m, d_jpx_d, d_jpy_d, d_reach, d_flags;
  int64_t items_m = 0, items_d = 0, ntiles = 0;
  int njobs_m = 0, njobs_d = 0;
  int64_t fold_x_m = 0, fold_y_m = 0, fold_x_d = 0, fold_y_d = 0;
  // device data
  DevBuf grid, spec, corr, zext, wext, zn, bands, bcrows, k0rows, Tf, Ti, kvs;
  DevBuf corrf, cmode, znf;  // FP32 correction tables (mixed operator, walls)
  DevBuf f_mf, f_bk, f_ab, f_g;
  // double-float solve (default for the mixed operator): per-system tables
  bool dfsolve = false;
  int df_variant = 1;
  DevBuf df_kap, df_ab, df_gi, df_km, df_km3, df_dxy;
  DevBuf st_cell_m, st_x_m, st_y_m, st_z_m, st_zw_m;
  DevBuf st_cell_d, st_x_d, st_y_d, st_z_d, st_zw_d, st_dx_d, st_dy_d, st_dz_d, st_dzw_d;
  DevBuf ghost_buf, pos64, bvp_scratch, fft_work;
  DevBuf sF, sT, sV, sW;  // staging (the graph's fixed inputs / outputs)
  int64_t bvp_grid = 0;
  struct FftClass {
    cufftHandle f = 0, b = 0;
    R *grid;
    CR *spec;
    int nx, ny, count;
  };
  std::vector<FftClass> classes;
  cudaStream_t cap = nullptr;
  std::map<int, cudaGraphExec_t> graphs;
  std::vector<SysP<R>> sysp_h;
  bool positioned = false;
  int kernels_per_mdot = 0;

  // the per-wavenumber solve of every system (+ their k = 0 modes)
  void solve(cudaStream_t s) {
    if (dfsolve) {
      DPST_CUDA(launch_bvp_df_b<R>(d_sysk.as<SysK<R>>(), S, d_mprefix.as<int64_t>(), K, nz, mode,
                                   bvp_scratch.as<float2>(), bvp_grid, df_variant, s));
      DPST_CUDA(launch_bvp_k0_b<R>(d_sysk.as<SysK<R>>(), S, s));
    } else {
      DPST_CUDA(launch_bvp_b<R>(d_sysk.as<SysK<R>>(), S, d_mprefix.as<int64_t>(), K, nz, bvp_scratch.as<double>(),
                                bvp_grid, s));
    }
  }

  // z transforms of every system in one launch: SIMT (folded) or tcgen05
  void ztrans(bool inverse, cudaStream_t s) {
    const ZSeg<R> *segs = (inverse ? d_segi : d_segf).template as<ZSeg<R>>();
    const R *Tm = (inverse ? Ti : Tf).template as<R>();
    if constexpr (sizeof(R) == 4) {
      if (ztc_use[inverse ? 1 : 0]) {
        // the inverse's wall correction as its own pass (the tcgen05
        // epilogue's four warps are too few for its arithmetic)
        const bool walls = inverse && mode != DPST_MODE_NOWALL;
        const ZSeg<R> *tsegs = walls ? d_segi_nc.template as<ZSeg<R>>() : segs;
        // no segment's epilogue corrects (the correction is its own pass)
        if (ztc_use[inverse ? 1 : 0] == 3 && tma_ok) {
          DPST_CUDA(launch_zgemm_tma_b((inverse ? d_segi_a : d_segf_a).as<ZSeg<float>>(), d_tp_a.as<int64_t>(), S_a,
                                       ntiles_a, nz, reinterpret_cast<const float *>(Tm),
                                       d_tmaps.as<CUtensorMap>(), nsm, ztc_err.as<int>(), s));
          if (S_b > 0)
            DPST_CUDA(launch_zgemm_tc_b((inverse ? d_segi_b : d_segf_b).as<ZSeg<float>>(), d_tp_b.as<int64_t>(), S_b,
                                        ntiles_b, nz, reinterpret_cast<const float *>(Tm), false, nsm,
                                        ztc_err.as<int>(), s));
        } else
          DPST_CUDA(launch_zgemm_tc_b(reinterpret_cast<const ZSeg<float> *>(tsegs), d_tprefix_tc.as<int64_t>(), S,
                                      ntiles_tc, nz, reinterpret_cast<const float *>(Tm), false, nsm,
                                      ztc_err.as<int>(), s));
        if (walls)
          DPST_CUDA(launch_corr_add_b(reinterpret_cast<const ZSeg<float> *>(segs), d_mprefix.as<int64_t>(), S, K, nz,
                                      mode, s));
        return;
      }
    }
    DPST_CUDA(launch_zgemm_b<R>(segs, d_tprefix.as<int64_t>(), S, ntiles, nz, Tm, nsm, s, inverse));
  }

  // Per direction, the SIMT, tcgen05 and TMA-fed tcgen05 transforms are
  // timed on the spectrum buffer (one warm-up, three runs) and the fastest
  // kept; a tensor-core run whose waits timed out is never kept.
  // DPSTOKES_GB300_ZTRANSFORM=simt|tcgen05|tma forces one.
  void tune_ztransform() {
    if (sizeof(R) != 4 || nz > 128) return;
    ztc_err.alloc(sizeof(int));
    DPST_CUDA(cudaMemset(ztc_err.p, 0, sizeof(int)));
    const char *env = getenv("DPSTOKES_GB300_ZTRANSFORM");
    const std::string want = env ? std::string(env) : std::string();
    DPST_CUDA(cudaMemset(spec.p, 0, spec.bytes));
    if (corr.p) DPST_CUDA(cudaMemset(corr.p, 0, corr.bytes));
    if (corrf.p) DPST_CUDA(cudaMemset(corrf.p, 0, corrf.bytes));
    cudaEvent_t a, b;
    DPST_CUDA(cudaEventCreate(&a));
    DPST_CUDA(cudaEventCreate(&b));
    for (int dir = 0; dir < 2; ++dir) {
      for (int k = 0; k < 3; ++k) {
        if (k == 2 && !tma_ok) continue;
        ztc_use[dir] = k == 2 ? 3 : k;
        ztrans(dir == 1, 0);
        DPST_CUDA(cudaEventRecord(a, 0));
        for (int rep = 0; rep < 3; ++rep) ztrans(dir == 1, 0);
        DPST_CUDA(cudaEventRecord(b, 0));
        DPST_CUDA(cudaEventSynchronize(b));
        float ms = 0.0f;
        DPST_CUDA(cudaEventElapsedTime(&ms, a, b));
        (k == 2 ? ztm_ms[dir] : ztc_ms[dir][k]) = ms / 3.0f;
      }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    int err = 0;
    DPST_CUDA(cudaMemcpy(&err, ztc_err.p, sizeof(int), cudaMemcpyDeviceToHost));
    for (int dir = 0; dir < 2; ++dir) {
      if (want == "tma" && tma_ok) ztc_use[dir] = 3;
      else if (want == "tcgen05") ztc_use[dir] = 1;
      else if (want == "simt") ztc_use[dir] = 0;
      else {
        float best = ztc_ms[dir][0];
        ztc_use[dir] = 0;
        if (ztc_ms[dir][1] < best) {
          best = ztc_ms[dir][1];
          ztc_use[dir] = 1;
        }
        if (tma_ok && ztm_ms[dir] < best) ztc_use[dir] = 3;
      }
      if (err != 0) ztc_use[dir] = 0;
    }
    DPST_CUDA(cudaMemset(spec.p, 0, spec.bytes));
  }

  // the double-float solve's kernel variant, timed on the spectrum buffer as
  // the single-system engine does (DPSTOKES_GB300_SOLVE_VARIANT fixes it)
  void tune_solve() {
    const char *env = getenv("DPSTOKES_GB300_SOLVE_VARIANT");
    if (env && *env) {
      const int v = atoi(env);
      if (v < 0 || v >= bvp_df_variants()) throw Error(DPST_ERR_INVALID_ARG, "DPSTOKES_GB300_SOLVE_VARIANT out of range");
      df_variant = v;
      return;
    }
    if (sizeof(R) != 4) return;
    DPST_CUDA(cudaMemset(spec.p, 0, spec.bytes));
    if (corr.p) DPST_CUDA(cudaMemset(corr.p, 0, corr.bytes));
    cudaEvent_t a, b;
    DPST_CUDA(cudaEventCreate(&a));
    DPST_CUDA(cudaEventCreate(&b));
    float best = 0.0f;
    for (int v = 0; v < bvp_df_variants(); ++v) {
      auto run = [&] {
        DPST_CUDA(launch_bvp_df_b<R>(d_sysk.as<SysK<R>>(), S, d_mprefix.as<int64_t>(), K, nz, mode,
                                     bvp_scratch.as<float2>(), bvp_grid, v, 0));
      };
      run();
      DPST_CUDA(cudaEventRecord(a, 0));
      for (int rep = 0; rep < 3; ++rep) run();
      DPST_CUDA(cudaEventRecord(b, 0));
      DPST_CUDA(cudaEventSynchronize(b));
      float ms = 0.0f;
      DPST_CUDA(cudaEventElapsedTime(&ms, a, b));
      if (v == 0 || ms < best) {
        best = ms;
        df_variant = v;
      }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }

  BatchEngine(const dpst_params *prm, const int64_t *n, int count, int dev) {
    device = dev;
    S = count;
    DPST_CUDA(cudaSetDevice(dev));
    DPST_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const dpst_params &p0 = prm[0];
    for (int s = 0; s < S; ++s) {
      validate(&prm[s], n[s]);
      const dpst_params &p = prm[s];
      if (p.nz != p0.nz || p.zmin != p0.zmin || p.zmax != p0.zmax || p.mode != p0.mode ||
          p.viscosity != p0.viscosity || p.precision != p0.precision || p.has_torque != p0.has_torque ||
          p.solve_arith != p0.solve_arith)
        throw Error(DPST_ERR_INVALID_ARG, "systems of a batch must share nz, zmin, zmax, mode, viscosity, "
                                          "precision, has_torque and solve_arith");
    }
    nz = p0.nz;
    mode = p0.mode;
    torque_op = p0.has_torque != 0;
    zmin = p0.zmin;
    Lz = p0.zmax - p0.zmin;
    H = Lz / 2;
    npart.assign(n, n + S);
    pbase.assign(S + 1, 0);
    for (int s = 0; s < S; ++s) pbase[s + 1] = pbase[s] + npart[s];
    Ntot = pbase[S];
    order.resize(S);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
      return prm[a].ny != prm[b].ny ? prm[a].ny < prm[b].ny : prm[a].nx < prm[b].nx;
    });
    std::vector<double> zG, zW;
    clencurt(nz, 0.0, Lz, zG, zW);
    upload(zn, zG);
    const ZTables zt = make_ztables(nz, H, mode);
    upload(bands, zt.bands);
    upload(bcrows, zt.bcrows);
    upload(k0rows, zt.k0rows);
    std::vector<double> tf, ti;
    dct_matrices(nz, tf, ti);
    upload(Tf, std::vector<R>(tf.begin(), tf.end()));
    upload(Ti, std::vector<R>(ti.begin(), ti.end()));

    // ---- per-system kernels, grids, offsets (in sorted order for grids/spectra)
    std::vector<KernelHost> km(S), kd(S);
    std::vector<GridArgs> ga(S);
    std::vector<double> ze, we, kv;
    std::vector<int64_t> goff(S), soff(S), koff(S), kvoff(S), moff(S);
    int64_t gtot = 0, stot = 0, ktot = 0;
    for (int oi = 0; oi < S; ++oi) {
      const int s = order[oi];
      const dpst_params &p = prm[s];
      const double hx = p.Lx / p.nx, hy = p.Ly / p.ny;
      km[s] = make_kernel(p.w, p.beta, p.alpha, false, hx, hy, p.nx, p.ny, zG, zW, "monopole kernel");
      km[s].d.zext_off = (int)ze.size();
      ze.insert(ze.end(), km[s].zext.begin(), km[s].zext.end());
      we.insert(we.end(), km[s].wext.begin(), km[s].wext.end());
      if (torque_op) {
        kd[s] = make_kernel(p.w_d, p.beta_d, p.alpha_d, true, hx, hy, p.nx, p.ny, zG, zW, "dipole kernel");
        kd[s].d.zext_off = (int)ze.size();
        ze.insert(ze.end(), kd[s].zext.begin(), kd[s].zext.end());
        we.insert(we.end(), kd[s].wext.begin(), kd[s].wext.end());
      } else {
        memset(&kd[s].d, 0, sizeof(KernelDesc));
      }
      GridArgs &g = ga[s];
      memset(&g, 0, sizeof(g));
      g.nx = p.nx;
      g.ny = p.ny;
      g.nz = nz;
      g.hx = hx;
      g.hy = hy;
      g.Lx = p.Lx;
      g.Ly = p.Ly;
      g.Lz = Lz;
      bc_sets(mode, g);
      const int64_t nk = (int64_t)p.ny * (p.nx / 2 + 1);
      if ((int64_t)nz * nk * 4 >= ((int64_t)1 << 31)) throw Error(DPST_ERR_UNSUPPORTED, "system grid too large");
      // a new size class starts on a 256-byte boundary (cuFFT wants aligned
      // base pointers); systems of one class are contiguous (one plan)
      if (oi > 0 && (prm[order[oi - 1]].nx != p.nx || prm[order[oi - 1]].ny != p.ny)) {
        const int64_t ag = 256 / sizeof(R), as = 256 / sizeof(CR);
        gtot = (gtot + ag - 1) / ag * ag;
        stot = (stot + as - 1) / as * as;
      }
      goff[s] = gtot;
      gtot += 3 * (int64_t)nz * p.ny * p.nx;
      soff[s] = stot;
      stot += 3 * (int64_t)nz * nk;
      moff[s] = ktot;
      ktot += nk;
      kvoff[s] = (int64_t)kv.size();
      const std::vector<double> kx = wavenumbers(p.nx, p.Lx), ky = wavenumbers(p.ny, p.Ly);
      kv.insert(kv.end(), kx.begin(), kx.end());
      kv.insert(kv.end(), ky.begin(), ky.end());
    }
    grid_elems = gtot;
    spec_elems = stot;
    K = ktot;
    upload(zext, ze);
    upload(wext, we);
    upload(kvs, kv);
    grid.alloc(sizeof(R) * gtot);
    spec.alloc(sizeof(CR) * stot);
    if (mode != DPST_MODE_NOWALL) corr.alloc(sizeof(double2) * 16 * (size_t)K);
    if (mode != DPST_MODE_NOWALL && sizeof(R) == 4) {
      // FP32 tables of the mixed operator's correction epilogue, per system
      // at its mode offset: the solve's coefficients in FP32, per mode {k, kx,
      // ky, Hermitian} and the partner index's {kx', ky'}; the shared nodes
      corrf.alloc(sizeof(float2) * 16 * (size_t)K);
      std::vector<float> cm(8 * (size_t)K, 0.0f);
      for (int s = 0; s < S; ++s) {
        const dpst_params &p = prm[s];
        const int nxh = p.nx / 2 + 1;
        const int64_t nk = (int64_t)p.ny * nxh;
        const double *kx = kv.data() + kvoff[s], *ky = kx + p.nx;
        for (int64_t i = 0; i < nk; ++i) {
          const int ix = (int)(i % nxh), iy = (int)(i / nxh);
          const double kxi = kx[ix], kyi = ky[iy];
          const double kxp = kx[(p.nx - ix) % p.nx], kyp = ky[(p.ny - iy) % p.ny];
          float *r = &cm[8 * (size_t)(moff[s] + i)];
          r[0] = (float)std::sqrt(kxi * kxi + kyi * kyi);
          r[1] = (float)kxi;
          r[2] = (float)kyi;
          r[3] = (kxp == -kxi && kyp == -kyi) ? 1.0f : 0.0f;
          r[4] = (float)kxp;
          r[5] = (float)kyp;
        }
      }
      upload(cmode, cm);
      const std::vector<float> zf(zG.begin(), zG.end());
      upload(znf, zf);
    }

    // ---- per-mode factors of every system (working arrays reused)
    int64_t nk_max = 0;
    for (int s = 0; s < S; ++s) nk_max = std::max<int64_t>(nk_max, (int64_t)prm[s].ny * (prm[s].nx / 2 + 1));
    f_mf.alloc(sizeof(double) * nz * K);
    f_bk.alloc(sizeof(double) * 4 * nz * K);
    f_ab.alloc(sizeof(double) * nz * K);
    f_g.alloc(sizeof(double) * 4 * K);
    dfsolve = p0.solve_arith == DPST_SOLVE_DF64 || (p0.solve_arith == DPST_SOLVE_DEFAULT && sizeof(R) == 4);
    if (dfsolve) {
      df_kap.alloc(sizeof(float2) * nz * K);
      df_ab.alloc(sizeof(float2) * nz * K);
      df_gi.alloc(sizeof(float2) * 4 * K);
      df_km.alloc(sizeof(float4) * K);
      df_km3.alloc(sizeof(float4) * K);
      df_dxy.alloc(sizeof(float2) * kvs.bytes / sizeof(double));
    }
    std::vector<SysK<R>> sysk(S);
    {
      DevBuf w_m, w_i, w_d, w_a0, w_a1, w_c0, w_c1;
      w_m.alloc(sizeof(double) * nz * nk_max);
      w_i.alloc(sizeof(double) * (nz + 1) * nk_max);
      w_d.alloc(sizeof(double) * nz * nk_max);
      w_a0.alloc(sizeof(double) * nz * nk_max);
      w_a1.alloc(sizeof(double) * nz * nk_max);
      w_c0.alloc(sizeof(double) * nz * nk_max);
      w_c1.alloc(sizeof(double) * nz * nk_max);
      const double *bd = bands.as<double>(), *bcd = bcrows.as<double>();
      const int N2 = nz + 2;
      for (int oi = 0; oi < S; ++oi) {
        const int s = order[oi];
        const dpst_params &p = prm[s];
        KsArgs ks;
        memset(&ks, 0, sizeof(ks));
        ks.nx = p.nx;
        ks.ny = p.ny;
        ks.nz = nz;
        ks.nxh = p.nx / 2 + 1;
        ks.nk = (int64_t)p.ny * ks.nxh;
        ks.H = H;
        ks.eta = p.viscosity;
        ks.Lz = Lz;
        ks.mode = mode;
        ks.kvx = kvs.as<double>() + kvoff[s];
        ks.kvy = kvs.as<double>() + kvoff[s] + p.nx;
        ks.zn = zn.as<double>();
        ks.s0 = bd;
        ks.sp2 = bd + nz;
        ks.sm2 = bd + 2 * nz;
        ks.fm1 = bd + 3 * nz;
        ks.fp1 = bd + 4 * nz;
        ks.se0 = H * H;
        ks.se1 = H * H;
        ks.fe = H;
        ks.bcr1 = bcd;
        ks.bcr2 = bcd + N2;
        ks.bcl1 = bcd + 2 * N2;
        ks.bcl2 = bcd + 3 * N2;
        ks.k0c0 = k0rows.as<double>();
        ks.k0c1 = k0rows.as<double>() + nz;
        for (int q = 0; q < 4; ++q) ks.k0gi[q] = zt.k0gi[q];
        ks.mfac = w_m.as<double>();
        ks.invb = w_i.as<double>();
        ks.dp2 = w_d.as<double>();
        ks.ab0 = w_a0.as<double>();
        ks.ab1 = w_a1.as<double>();
        ks.c0 = w_c0.as<double>();
        ks.c1 = w_c1.as<double>();
        ks.ginv = f_g.as<double>() + 4 * moff[s];
        ks.mf = f_mf.as<double>() + nz * moff[s];
        ks.bk = f_bk.as<double>() + 4 * nz * moff[s];
        ks.ab = f_ab.as<double>() + nz * moff[s];
        ks.corrf = corrf.p != nullptr ? corrf.as<float2>() + 16 * moff[s] : nullptr;
        launch_bvp_factors(ks, 0);
        DPST_CUDA(cudaGetLastError());
        ks.mfac = ks.invb = ks.dp2 = ks.ab0 = ks.ab1 = ks.c0 = ks.c1 = nullptr;
        if (dfsolve) {
          ks.kap2 = df_kap.as<float2>() + nz * moff[s];
          ks.ab2 = df_ab.as<float2>() + nz * moff[s];
          ks.gi2 = df_gi.as<float2>() + 4 * moff[s];
          ks.km2 = df_km.as<float4>() + moff[s];
          ks.km3 = df_km3.as<float4>() + moff[s];
          ks.dx2 = df_dxy.as<float2>() + kvoff[s];
          ks.dy2 = df_dxy.as<float2>() + kvoff[s] + p.nx;
          launch_bvp_pack_df(ks, 0);
          DPST_CUDA(cudaGetLastError());
        }
        sysk[s].ks = ks;
        sysk[s].spec = reinterpret_cast<R *>(spec.as<CR>() + soff[s]);
        sysk[s].corr = (mode != DPST_MODE_NOWALL) ? corr.as<double2>() + 16 * moff[s] : nullptr;
      }
      DPST_CUDA(cudaDeviceSynchronize());
    }
    // tables in sorted order (BVP modes, z-transform segments)
    std::vector<SysK<R>> sysk_sorted(S);
    std::vector<int64_t> mprefix(S + 1, 0), tprefix(S + 1, 0);
    std::vector<ZSeg<R>> segf(S), segi(S);
    for (int oi = 0; oi < S; ++oi) {
      const int s = order[oi];
      sysk_sorted[oi] = sysk[s];
      mprefix[oi + 1] = mprefix[oi] + sysk[s].ks.nk;
      const int64_t ncols = 2 * sysk[s].ks.nk;
      tprefix[oi + 1] = tprefix[oi] + 3 * ((ncols + 63) / 64);
      memset(&segf[oi], 0, sizeof(ZSeg<R>));
      segf[oi].spec = sysk[s].spec;
      segf[oi].ncols = ncols;
      segf[oi].e.inverse = 0;
      segf[oi].e.scale = 1.0;
      segf[oi].e.ks = sysk[s].ks;
      segi[oi] = segf[oi];
      segi[oi].e.inverse = 1;
      segi[oi].e.scale = 1.0 / ((double)prm[s].nx * (double)prm[s].ny);
      segi[oi].e.corr = sysk[s].corr;
      if (corrf.p != nullptr) {
        segi[oi].e.corrf = corrf.as<float2>() + 16 * moff[s];
        segi[oi].e.cmode = cmode.as<float4>() + 2 * moff[s];
        segi[oi].e.znf = znf.as<float>();
        segi[oi].e.fac = (float)(1.0 / 2.0 / prm[s].viscosity);
      }
    }
    ntiles = tprefix[S];
    upload(d_sysk, sysk_sorted);
    upload(d_mprefix, mprefix);
    upload(d_tprefix, tprefix);
    {
      std::vector<int64_t> tp(S + 1, 0);
      for (int oi = 0; oi < S; ++oi) tp[oi + 1] = tp[oi] + ztc_tiles(segf[oi].ncols);
      ntiles_tc = tp[S];
      upload(d_tprefix_tc, tp);
    }
    upload(d_segf, segf);
    upload(d_segi, segi);
    {
      std::vector<ZSeg<R>> nc = segi;
      for (ZSeg<R> &g : nc) {
        g.e.corr = nullptr;
        g.e.corrf = nullptr;
      }
      upload(d_segi_nc, nc);
    }
    if (sizeof(R) == 4 && nz >= 32 && nz <= 128) {
      // the systems the TMA form takes and their tensor maps (the same
      // spectra in both directions); the others keep the register-staged form
      std::vector<ZSeg<R>> fa, ia, fb, ib;
      std::vector<int64_t> pa(1, 0), pb(1, 0);
      for (int oi = 0; oi < S; ++oi) {
        ZSeg<R> inc = segi[oi];
        inc.e.corr = nullptr;
        inc.e.corrf = nullptr;
        std::vector<CUtensorMap> one;
        const bool a = ztm_maps_b(reinterpret_cast<const ZSeg<float> *>(&segf[oi]), 1, nz, one);
        (a ? fa : fb).push_back(segf[oi]);
        (a ? ia : ib).push_back(inc);
        std::vector<int64_t> &pp = a ? pa : pb;
        pp.push_back(pp.back() + ztc_tiles(segf[oi].ncols));
      }
      S_a = (int)fa.size();
      S_b = (int)fb.size();
      std::vector<CUtensorMap> maps;
      tma_ok = S_a > 0 && ztm_maps_b(reinterpret_cast<const ZSeg<float> *>(fa.data()), S_a, nz, maps);
      if (tma_ok) {
        upload(d_tmaps, maps);
        upload(d_segf_a, fa);
        upload(d_segi_a, ia);
        upload(d_tp_a, pa);
        ntiles_a = pa.back();
        if (S_b > 0) {
          upload(d_segf_b, fb);
          upload(d_segi_b, ib);
          upload(d_tp_b, pb);
          ntiles_b = pb.back();
        }
      }
    }
    size_t bvp_bytes = 0;
    if (dfsolve) {
      DPST_CUDA(bvp_df_plan_b(sysk[0].ks, K, nsm, &bvp_grid, &bvp_bytes));
    } else {
      DPST_CUDA(bvp_plan_b<R>(nz, K, nsm, &bvp_grid, &bvp_bytes));
    }
    bvp_scratch.alloc(bvp_bytes);
    if (dfsolve) tune_solve();
    tune_ztransform();

    // ---- particles: stencils, ghost layers, per-system particle tables
    auto total = [&](const std::vector<KernelHost> &kk, int which) {
      int64_t t = 0;
      for (int s = 0; s < S; ++s) {
        const KernelDesc &d = kk[s].d;
        t += npart[s] * (which == 0 ? d.wx : which == 1 ? d.wy : d.wz_max);
      }
      return std::max<int64_t>(t, 1);
    };
    const size_t N1 = (size_t)std::max<int64_t>(Ntot, 1);
    st_cell_m.alloc(sizeof(int4) * N1);
    st_x_m.alloc(sizeof(R) * total(km, 0));
    st_y_m.alloc(sizeof(R) * total(km, 1));
    st_z_m.alloc(sizeof(R) * total(km, 2));
    st_zw_m.alloc(sizeof(R) * total(km, 2));
    if (torque_op) {
      st_cell_d.alloc(sizeof(int4) * N1);
      st_x_d.alloc(sizeof(R) * total(kd, 0));
      st_y_d.alloc(sizeof(R) * total(kd, 1));
      st_z_d.alloc(sizeof(R) * total(kd, 2));
      st_zw_d.alloc(sizeof(R) * total(kd, 2));
      st_dx_d.alloc(sizeof(R) * total(kd, 0));
      st_dy_d.alloc(sizeof(R) * total(kd, 1));
      st_dz_d.alloc(sizeof(R) * total(kd, 2));
      st_dzw_d.alloc(sizeof(R) * total(kd, 2));
    }
    // ghost layers at every open end of every system (levels = dend), so the
    // pipeline does not depend on where the particles are
    auto ghost_levels = [&](const KernelDesc &d, bool top) -> int {
      const ZEnds &ends = ga[0].bcA;  // both BC sets have the same active ends
      return (top ? !ends.top_active : !ends.bot_active) ? d.dend : 0;
    };
    int64_t gh_total = 0;
    for (int s = 0; s < S; ++s)
      for (int kind = 0; kind < (torque_op ? 2 : 1); ++kind) {
        const KernelDesc &d = kind ? kd[s].d : km[s].d;
        const int64_t lev = (int64_t)d.nyeff * d.nxeff * 3;
        gh_total += lev * (ghost_levels(d, true) + ghost_levels(d, false));
      }
    ghost_buf.alloc(sizeof(R) * std::max<int64_t>(gh_total, 1));
    sysp_h.resize(S);
    std::vector<int64_t> ipm(S + 1, 0), ipd(S + 1, 0);
    std::vector<FoldJob<R>> jobs_m, jobs_d;
    int64_t o_x_m = 0, o_y_m = 0, o_z_m = 0, o_x_d = 0, o_y_d = 0, o_z_d = 0, o_gh = 0;
    for (int s = 0; s < S; ++s) {
      SysP<R> &y = sysp_h[s];
      memset(&y, 0, sizeof(y));
      y.km = km[s].d;
      y.kd = kd[s].d;
      y.g = ga[s];
      y.pbase = pbase[s];
      y.n = npart[s];
      y.grid = grid.as<R>() + goff[s];
      y.stm.cell = st_cell_m.as<int4>() + pbase[s];
      y.stm.phx = st_x_m.as<R>() + o_x_m;
      y.stm.phy = st_y_m.as<R>() + o_y_m;
      y.stm.phz = st_z_m.as<R>() + o_z_m;
      y.stm.phzw = st_zw_m.as<R>() + o_z_m;
      o_x_m += npart[s] * km[s].d.wx;
      o_y_m += npart[s] * km[s].d.wy;
      o_z_m += npart[s] * km[s].d.wz_max;
      if (torque_op) {
        y.std_.cell = st_cell_d.as<int4>() + pbase[s];
        y.std_.phx = st_x_d.as<R>() + o_x_d;
        y.std_.dphx = st_dx_d.as<R>() + o_x_d;
        y.std_.phy = st_y_d.as<R>() + o_y_d;
        y.std_.dphy = st_dy_d.as<R>() + o_y_d;
        y.std_.phz = st_z_d.as<R>() + o_z_d;
        y.std_.phzw = st_zw_d.as<R>() + o_z_d;
        y.std_.dphz = st_dz_d.as<R>() + o_z_d;
        y.std_.dphzw = st_dzw_d.as<R>() + o_z_d;
        o_x_d += npart[s] * kd[s].d.wx;
        o_y_d += npart[s] * kd[s].d.wy;
        o_z_d += npart[s] * kd[s].d.wz_max;
      }
      for (int kind = 0; kind < (torque_op ? 2 : 1); ++kind) {
        const KernelDesc &d = kind ? kd[s].d : km[s].d;
        Ghosts<R> &gh = kind ? y.ghd : y.ghm;
        const int64_t lev = (int64_t)d.nyeff * d.nxeff * 3;
        for (int top = 1; top >= 0; --top) {
          const int L = ghost_levels(d, top != 0);
          if (L == 0) continue;
          R *b = ghost_buf.as<R>() + o_gh;
          o_gh += lev * L;
          if (top) {
            gh.top = b;
            gh.ntop = L;
          } else {
            gh.bot = b;
            gh.nbot = L;
          }
          FoldJob<R> f;
          f.buf = b;
          f.levels = L;
          f.nx = prm[s].nx;
          f.ny = prm[s].ny;
          f.kd = d;
          (kind ? jobs_d : jobs_m).push_back(f);
        }
      }
      ipm[s + 1] = ipm[s] + npart[s] * km[s].d.wx * km[s].d.wy;
      ipd[s + 1] = ipd[s] + (torque_op ? npart[s] * kd[s].d.wx * kd[s].d.wy : 0);
    }
    items_m = ipm[S];
    items_d = ipd[S];
    upload(d_sysp, sysp_h);
    upload(d_pprefix, pbase);
    upload(d_ipm, ipm);
    upload(d_ipd, ipd);
    auto fold_tables = [&](const std::vector<FoldJob<R>> &jobs, DevBuf &dj, DevBuf &dpx, DevBuf &dpy, int64_t &nx_,
                           int64_t &ny_) {
      std::vector<int64_t> px(jobs.size() + 1, 0), py(jobs.size() + 1, 0);
      for (size_t j = 0; j < jobs.size(); ++j) {
        const FoldJob<R> &f = jobs[j];
        px[j + 1] = px[j] + (int64_t)f.levels * f.kd.nyeff * f.kd.lend * 3 * 2;
        py[j + 1] = py[j] + (int64_t)f.levels * f.kd.bend * f.kd.nxeff * 3 * 2;
      }
      nx_ = px.back();
      ny_ = py.back();
      if (!jobs.empty()) upload(dj, jobs);
      upload(dpx, px);
      upload(dpy, py);
    };
    njobs_m = (int)jobs_m.size();
    njobs_d = (int)jobs_d.size();
    fold_tables(jobs_m, d_jobs_m, d_jpx_m, d_jpy_m, fold_x_m, fold_y_m);
    fold_tables(jobs_d, d_jobs_d, d_jpx_d, d_jpy_d, fold_x_d, fold_y_d);
    d_reach.alloc(sizeof(int) * 2 * std::max(S, 1));
    d_flags.alloc(sizeof(int) * 8);
    pos64.alloc(sizeof(double) * 3 * N1);
    for (DevBuf *b : {&sF, &sT, &sV, &sW}) b->alloc(sizeof(double) * 3 * N1);

    // ---- cuFFT: one plan pair per size class (systems contiguous in sorted order)
    for (int oi = 0; oi < S;) {
      const int s0 = order[oi];
      int oj = oi;
      while (oj < S && prm[order[oj]].nx == prm[s0].nx && prm[order[oj]].ny == prm[s0].ny) ++oj;
      const int cnt = oj - oi;
      const int nx = prm[s0].nx, ny = prm[s0].ny, nxh = nx / 2 + 1;
      int n2[2] = {ny, nx}, inem[2] = {ny, nx}, onem[2] = {ny, nxh};
      const int batch = cnt * 3 * nz;
      FftClass c;
      c.grid = grid.as<R>() + goff[s0];
      c.nx = nx;
      c.ny = ny;
      c.count = cnt;
      c.spec = spec.as<CR>() + soff[s0];
      DPST_CUFFT(cufftPlanMany(&c.f, 2, n2, inem, 1, ny * nx, onem, 1, ny * nxh,
                               sizeof(R) == 8 ? CUFFT_D2Z : CUFFT_R2C, batch));
      DPST_CUFFT(cufftPlanMany(&c.b, 2, n2, onem, 1, ny * nxh, inem, 1, ny * nx,
                               sizeof(R) == 8 ? CUFFT_Z2D : CUFFT_C2R, batch));
      classes.push_back(c);
      oi = oj;
    }
    DPST_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    DPST_CUDA(cudaDeviceSynchronize());
  }

  ~BatchEngine() override {
    cudaSetDevice(device);
    cudaDeviceSynchronize();
    for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
    for (FftClass &c : classes) {
      if (c.f) cufftDestroy(c.f);
      if (c.b) cufftDestroy(c.b);
    }
    if (cap) cudaStreamDestroy(cap);
  }

  void set_positions(const void *pos, int dtype, cudaStream_t s) override {
    positioned = false;
    if (Ntot == 0) {
      positioned = true;
      return;
    }
    if (!pos) throw Error(DPST_ERR_INVALID_ARG, "positions pointer is NULL");
    const int bs = 256;
    const int64_t nb = (Ntot + bs - 1) / bs;
    if (dtype == DPST_F64) k_prep_pos_b<double><<<nb, bs, 0, s>>>((const double *)pos, Ntot, zmin, pos64.as<double>());
    else if (dtype == DPST_F32) k_prep_pos_b<float><<<nb, bs, 0, s>>>((const float *)pos, Ntot, zmin, pos64.as<double>());
    else throw Error(DPST_ERR_INVALID_ARG, "dtype must be DPST_F64 or DPST_F32");
    DPST_CUDA(cudaGetLastError());
    DPST_CUDA(cudaMemsetAsync(d_flags.p, 0, d_flags.bytes, s));
    const SysP<R> *sy = d_sysp.as<SysP<R>>();
    launch_locate_b<R>(false, pos64.as<double>(), Ntot, sy, d_pprefix.as<int64_t>(), S, zext.as<double>(),
                       wext.as<double>(), d_flags.as<int>(), d_reach.as<int>(), s);
    if (torque_op)
      launch_locate_b<R>(true, pos64.as<double>(), Ntot, sy, d_pprefix.as<int64_t>(), S, zext.as<double>(),
                         wext.as<double>(), d_flags.as<int>(), d_reach.as<int>(), s);
    DPST_CUDA(cudaGetLastError());
    int fl = 0;
    DPST_CUDA(cudaMemcpyAsync(&fl, d_flags.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    DPST_CUDA(cudaStreamSynchronize(s));
    if (fl & 1) throw Error(DPST_ERR_OUT_OF_DOMAIN, "a particle lies outside its system's box (or is NaN)");
    if (fl & 2) throw Error(DPST_ERR_CUDA, "internal: z window longer than its bound");
    positioned = true;
  }

  // The Mdot pipeline on fixed buffers (staged F, T in; V, W out).
  template <typename RF>
  void pipeline(bool torque, bool want_w, cudaStream_t s) {
    const SysP<R> *sy = d_sysp.as<SysP<R>>();
    DPST_CUDA(cudaMemsetAsync(grid.p, 0, grid.bytes, s));
    DPST_CUDA(cudaMemsetAsync(ghost_buf.p, 0, ghost_buf.bytes, s));
    launch_spread_b<R, RF>(false, sF.as<RF>(), items_m, sy, d_ipm.as<int64_t>(), S, s);
    if (torque) launch_spread_b<R, RF>(true, sT.as<RF>(), items_d, sy, d_ipd.as<int64_t>(), S, s);
    launch_ghost_fold_b<R>(false, d_jobs_m.as<FoldJob<R>>(), d_jpx_m.as<int64_t>(), njobs_m, fold_x_m, s);
    launch_ghost_fold_b<R>(true, d_jobs_m.as<FoldJob<R>>(), d_jpy_m.as<int64_t>(), njobs_m, fold_y_m, s);
    if (torque) {
      launch_ghost_fold_b<R>(false, d_jobs_d.as<FoldJob<R>>(), d_jpx_d.as<int64_t>(), njobs_d, fold_x_d, s);
      launch_ghost_fold_b<R>(true, d_jobs_d.as<FoldJob<R>>(), d_jpy_d.as<int64_t>(), njobs_d, fold_y_d, s);
    }
    DPST_CUDA(cudaGetLastError());
    for (size_t ci = 0; ci < classes.size(); ++ci) {
      FftClass &c = classes[ci];
      DPST_CUFFT(cufftSetStream(c.f, s));
      const cufftResult r = (sizeof(R) == 8)
                                ? cufftExecD2Z(c.f, (cufftDoubleReal *)c.grid, (cufftDoubleComplex *)c.spec)
                                : cufftExecR2C(c.f, (cufftReal *)c.grid, (cufftComplex *)c.spec);
      if (r != CUFFT_SUCCESS)
        throw Error(DPST_ERR_CUDA, "x-y transform of size class " + std::to_string(ci) + " (" +
                                       std::to_string(c.nx) + " x " + std::to_string(c.ny) + ", " +
                                       std::to_string(c.count) + " systems, grid offset " +
                                       std::to_string(c.grid - grid.as<R>()) + "): cuFFT error " +
                                       std::to_string((int)r));
    }
    ztrans(false, s);
    solve(s);
    ztrans(true, s);
    for (FftClass &c : classes) {
      DPST_CUFFT(cufftSetStream(c.b, s));
      if (sizeof(R) == 8)
        DPST_CUFFT(cufftExecZ2D(c.b, (cufftDoubleComplex *)c.spec, (cufftDoubleReal *)c.grid));
      else
        DPST_CUFFT(cufftExecC2R(c.b, (cufftComplex *)c.spec, (cufftReal *)c.grid));
    }
    launch_interp_b<R, RF>(false, Ntot, sy, d_pprefix.as<int64_t>(), S, sV.as<RF>(), false, s);
    if (want_w) launch_interp_b<R, RF>(true, Ntot, sy, d_pprefix.as<int64_t>(), S, sW.as<RF>(), torque, s);
    DPST_CUDA(cudaGetLastError());
    kernels_per_mdot = 2 + (torque ? 2 : 0) + (njobs_m ? 2 : 0) + (torque && njobs_d ? 2 : 0) + 2 + 2 +
                       (want_w ? 2 : 1);
  }

  template <typename RF>
  cudaGraphExec_t graph_for(bool torque, bool want_w) {
    const int key = (sizeof(RF) == 8 ? 1 : 0) | (torque ? 2 : 0) | (want_w ? 4 : 0);
    auto it = graphs.find(key);
    if (it != graphs.end()) return it->second;
    // one eager run first: library and kernel initialisation happens outside
    // the capture (its results are overwritten by the first replay)
    pipeline<RF>(torque, want_w, cap);
    DPST_CUDA(cudaStreamSynchronize(cap));
    cudaGraph_t g = nullptr;
    DPST_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeRelaxed));
    try {
      pipeline<RF>(torque, want_w, cap);
    } catch (...) {
      cudaStreamEndCapture(cap, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    DPST_CUDA(cudaStreamEndCapture(cap, &g));
    cudaGraphExec_t ex = nullptr;
    cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    DPST_CUDA(e);
    graphs[key] = ex;
    return ex;
  }

  template <typename RF>
  void run(const RF *F, const RF *T, RF *V, RF *W, cudaStream_t s) {
    const bool torque = torque_op && T != nullptr;
    const bool want_w = torque_op && W != nullptr;
    const size_t b = sizeof(RF) * 3 * (size_t)Ntot;
    cudaGraphExec_t ex = graph_for<RF>(torque, want_w);
    DPST_CUDA(cudaMemcpyAsync(sF.p, F, b, cudaMemcpyDeviceToDevice, s));
    if (torque) DPST_CUDA(cudaMemcpyAsync(sT.p, T, b, cudaMemcpyDeviceToDevice, s));
    DPST_CUDA(cudaGraphLaunch(ex, s));
    DPST_CUDA(cudaMemcpyAsync(V, sV.p, b, cudaMemcpyDeviceToDevice, s));
    if (want_w) DPST_CUDA(cudaMemcpyAsync(W, sW.p, b, cudaMemcpyDeviceToDevice, s));
  }

  void mdot(const void *F, const void *T, void *V, void *W, int dtype, cudaStream_t s) override {
    if (!positioned) throw Error(DPST_ERR_NOT_READY, "positions have not been set");
    if (Ntot == 0) return;
    if (F == nullptr || V == nullptr) throw Error(DPST_ERR_INVALID_ARG, "F and V must not be NULL");
    if (dtype == DPST_F64) run<double>((const double *)F, (const double *)T, (double *)V, (double *)W, s);
    else if (dtype == DPST_F32) run<float>((const float *)F, (const float *)T, (float *)V, (float *)W, s);
    else throw Error(DPST_ERR_INVALID_ARG, "dtype must be DPST_F64 or DPST_F32");
  }

  void info(dpst_batch_info *o) const override {
    memset(o, 0, sizeof(*o));
    o->n_systems = S;
    o->n_size_classes = (int)classes.size();
    o->n_particles = Ntot;
    o->n_modes = K;
    o->kernels_per_mdot = kernels_per_mdot;
    // the TMA form's second launch over the systems it does not take
    for (int d = 0; d < 2; ++d)
      if (kernels_per_mdot > 0 && ztc_use[d] == 3 && tma_ok && S_b > 0) o->kernels_per_mdot += 1;
    o->fft_plans = 2 * (int)classes.size();
    o->ztransform = ztc_use[0];
    o->ztransform_inverse = ztc_use[1];
    for (int k = 0; k < 2; ++k) {
      o->ztransform_ms[k] = ztc_ms[0][k];
      o->ztransform_inverse_ms[k] = ztc_ms[1][k];
      o->ztransform_tma_ms[k] = ztm_ms[k];
    }
    int64_t bytes = 0;
    const DevBuf *all[] = {&d_sysp, &d_sysk, &d_segf, &d_segi, &d_pprefix, &d_ipm, &d_ipd, &d_mprefix, &d_tprefix,
                           &d_tprefix_tc, &ztc_err, &d_segi_nc, &d_tmaps, &d_segf_a, &d_segi_a, &d_tp_a,
                           &d_segf_b, &d_segi_b, &d_tp_b,
                           &d_jobs_m, &d_jobs_d, &grid, &spec, &corr, &zext, &wext, &zn, &bands, &bcrows, &k0rows,
                           &Tf, &Ti, &kvs, &f_mf, &f_bk, &f_ab, &f_g, &st_cell_m, &st_x_m, &st_y_m, &st_z_m,
                           &st_zw_m, &st_cell_d, &st_x_d, &st_y_d, &st_z_d, &st_zw_d, &st_dx_d, &st_dy_d,
                           &st_dz_d, &st_dzw_d, &ghost_buf, &pos64, &bvp_scratch, &fft_work, &sF, &sT, &sV, &sW,
                           &df_kap, &df_ab, &df_gi, &df_km, &df_km3, &df_dxy,
                           &corrf, &cmode, &znf};
    for (const DevBuf *d : all) bytes += d->bytes;
    o->device_bytes = bytes;
  }
};

}  // namespace dpst

struct dpst_batch_engine {
  std::unique_ptr<dpst::BatchBase> e;
};

using dpst::Error;

extern "C" {

int dpst_batched_create(const dpst_params *params, const int64_t *n_particles, int n_systems, int device,
                        dpst_batch *out) {
  return dpst::guarded([&] {
    if (!out || !params || !n_particles) throw Error(DPST_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    if (n_systems < 1) throw Error(DPST_ERR_INVALID_ARG, "n_systems must be >= 1");
    std::unique_ptr<dpst_batch_engine> h(new dpst_batch_engine());
    if (params[0].precision == DPST_PREC_FP64)
      h->e.reset(new dpst::BatchEngine<double>(params, n_particles, n_systems, device));
    else
      h->e.reset(new dpst::BatchEngine<float>(params, n_particles, n_systems, device));
    *out = h.release();
  });
}

int dpst_batched_destroy(dpst_batch b) {
  return dpst::guarded([&] { delete b; });
}

int dpst_batched_set_positions(dpst_batch b, const void *pos, int dtype, void *stream) {
  return dpst::guarded([&] {
    if (!b) throw Error(DPST_ERR_INVALID_ARG, "handle is NULL");
    DPST_CUDA(cudaSetDevice(b->e->device));
    b->e->set_positions(pos, dtype, (cudaStream_t)stream);
  });
}

int dpst_batched_mdot(dpst_batch b, const void *F, const void *T, void *V, void *W, int dtype, void *stream) {
  return dpst::guarded([&] {
    if (!b) throw Error(DPST_ERR_INVALID_ARG, "handle is NULL");
    DPST_CUDA(cudaSetDevice(b->e->device));
    b->e->mdot(F, T, V, W, dtype, (cudaStream_t)stream);
  });
}

int dpst_batched_get_info(dpst_batch b, dpst_batch_info *out) {
  return dpst::guarded([&] {
    if (!b || !out) throw Error(DPST_ERR_INVALID_ARG, "NULL argument");
    b->e->info(out);
  });
}

}  // extern "C"
