// Engine and C ABI of libdpstokes_gb300.so (declared in include/dpstokes_gb300.h).
//
// Host side of the operator: validates parameters, reproduces the
// reference's set-up arithmetic (Chebyshev grid and weights, kernel
// normalisation and truncation threshold, extended z grid, BC rows,
// integration matrices, DCT-I matrices; stochasticHydroTools/
// DoublyPeriodicStokes source/cpu: Chebyshev.py:4-160, Quadrature.cpp:11-46,
// ParticleList.cpp:211-276 and 394-451, Solvers.py:258-347 and 603-643,
// FCM.py:211-248), owns the device buffers and cuFFT plans, and runs the
// Mdot pipeline:
//   zero grid -> spread F (+ torque curl) -> [fold open-end ghost layers]
//   -> x-y FFT -> z DCT-I -> per-k BVP -> inverse z DCT-I (+ wall correction)
//   -> inverse x-y FFT -> interpolate V (+ W);
// with the regular-kernel torque coupling (run_reg) the torques take their
// own grid and their curl and the vorticity are taken in wavenumber space.
// The triply periodic mode has its own engine (dpst_tp.cu).
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <climits>
#include <cstdlib>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/dpstokes_gb300.h"
#include "dpst_host.cuh"
#include "dpst_internal.cuh"
#include "dpst_launch.cuh"

namespace dpst {

// ---- declarations of the kernel launchers (dpst_particles.cu, dpst_kspace.cu)
template <typename R>
cudaError_t bvp_plan_b(int nz, int64_t K, int nsm, int64_t *grid, size_t *scratch_bytes);
template <typename R>
cudaError_t launch_bvp_b(const SysK<R> *sys, int S, const int64_t *mprefix, int64_t K, int nz, double *scratch,
                         int64_t grid, cudaStream_t s);


void launch_bvp_factors(const KsArgs &a, cudaStream_t s);
template <typename R>
cudaError_t bvp_plan(const KsArgs &a, int nsm, int64_t *grid, size_t *scratch_bytes);
template <typename R>
cudaError_t launch_bvp(const KsArgs &a, R *spec, double2 *corr, double *scratch, int64_t grid,
                       cudaStream_t s, bool hybrid = true);
template <typename R>
cudaError_t launch_bvp_noalloc(const KsArgs &a, R *spec, double2 *corr, int64_t planned_grid,
                               cudaStream_t s, bool *too_big);
size_t noalloc_scratch_bytes();
template <typename R>
cudaError_t launch_bvp_k0(const KsArgs &a, R *spec, cudaStream_t s);
// double-float solve of the mixed operator (dpst_bvp_df.cu)
void launch_bvp_pack_df(const KsArgs &a, cudaStream_t s);
cudaError_t bvp_df_plan(const KsArgs &a, int nsm, int64_t *grid, size_t *scratch_bytes);
int bvp_df_variants();
template <typename R>
cudaError_t launch_bvp_df(const KsArgs &a, R *spec, double2 *corr, float2 *scratch, int64_t grid, int variant,
                          cudaStream_t s);
cudaError_t bvp_df_plan_b(const KsArgs &a0, int64_t K, int nsm, int64_t *grid, size_t *scratch_bytes);
template <typename R>
cudaError_t launch_bvp_df_b(const SysK<R> *sys, int S, const int64_t *mprefix, int64_t K, int nz, int mode,
                            float2 *scratch, int64_t grid, int variant, cudaStream_t s, int ncol = 0);
template <typename R>
cudaError_t launch_bvp_df_cols(const KsArgs &a, R *spec0, int64_t sstride, double2 *corr0, float2 *corrf0,
                               int64_t cstride, int ncol, float2 *scratch, int64_t grid, int variant,
                               cudaStream_t s);
template <typename R>
cudaError_t launch_bvp_k0_b(const SysK<R> *sys, int S, cudaStream_t s);
// double-float adjoint solve (dpst_bvp_df.cu) and the FP64 k = 0 adjoint
cudaError_t bvp_adj_df_plan(const KsArgs &a, int nsm, int64_t *grid, size_t *scratch_bytes);
template <typename R>
cudaError_t launch_adj_df(const KsArgs &a, R *spec, const double2 *cadj, float2 *scratch, int64_t grid, int variant,
                          cudaStream_t s);
template <typename R>
cudaError_t launch_adj_k0(const KsArgs &a, R *spec, cudaStream_t s);
// x-y transforms of the mixed operator (dpst_fft.cu)
bool own_fft_supported(int nx, int ny);
std::vector<float2> fft_twiddles(int n);
cudaError_t fft_setup(int nx, int ny);
cudaError_t fft_rows(bool inverse, const float *grid_in, float2 *spec_out, const float2 *spec_in, float *grid_out,
                     int nx, int64_t rows, const float2 *twx, cudaStream_t s);
cudaError_t fft_cols(bool inverse, float2 *spec, int ny, int nxh, int64_t planes, const float2 *twy, cudaStream_t s);
bool fft_xy_fused_supported(int nx, int ny);
bool fft_xy_cluster_supported(int nx, int ny);
cudaError_t fft_xy_cluster_setup(int nx, int ny, int *grid);
cudaError_t fft_xy_cluster(bool inverse, const float *grid_in, float2 *spec, float *grid_out, int nx, int ny,
                           int64_t planes, const float2 *twx, const float2 *twy, int *err, int grid, cudaStream_t s);
int64_t fft_xy_counter_ints(int64_t planes);
bool own_fft_df_supported(int nx, int ny);
std::vector<float4> fft_twiddles_df(int n);
cudaError_t fft_setup_df(int nx, int ny);
cudaError_t fft_rows_df(bool inverse, const double *grid_in, double2 *spec_out, const double2 *spec_in,
                        double *grid_out, int nx, int64_t rows, const float4 *twx, cudaStream_t s);
cudaError_t fft_cols_df(bool inverse, double2 *spec, int ny, int nxh, int64_t planes, const float4 *twy,
                        cudaStream_t s);
// planes between the one-launch transform's two passes: 16, or
// DPSTOKES_GB300_XY_LAG (1 ... 4096)
static int xy_lag_setting() {
  const char *env = getenv("DPSTOKES_GB300_XY_LAG");
  const int v = env ? atoi(env) : 16;
  return (v >= 1 && v <= 4096) ? v : 16;
}
cudaError_t fft_xy_setup(int nx, int ny, int *grid);
cudaError_t fft_xy_fused(bool inverse, const float *grid_in, float2 *spec, float *grid_out, int nx, int ny,
                         int64_t planes, const float2 *twx, const float2 *twy, int *ctr, int grid, int lag,
                         cudaStream_t s);
template <typename R>
void launch_spec_curl(const R *src, R *dst, bool accumulate, int nz, int64_t nk, int nx, int ny, int nxh,
                      const double *kvx, const double *kvy, double H, cudaStream_t s);
template <typename R>
cudaError_t launch_zgemm(R *spec, int nz, int64_t ncols, const R *Tm, const EpiArgs &e, int nsm,
                         cudaStream_t s, bool fold_out);
// tensor-core z transform of the mixed operator (dpst_ztc.cu)
cudaError_t launch_zgemm_tc(float *spec, int nz, int64_t ncols, const float *Tm, const EpiArgs &e, int nsm,
                            int *err, cudaStream_t s);
cudaError_t launch_zgemm_df(double *spec, int nz, int64_t ncols, const double *Tm, const EpiArgs &e, int nsm,
                            cudaStream_t s, bool fold_out);
cudaError_t launch_corr_add(float *spec, int nz, int64_t nk, const EpiArgs &e, cudaStream_t s);
bool ztm_supported(const float *spec, int nz, int64_t ncols);
int ztm_variants();
cudaError_t launch_zgemm_tma(float *spec, int nz, int64_t ncols, const float *Tm, const EpiArgs &e, int nsm, int *err,
                             int variant, cudaStream_t s);
bool tile_spread_supported(const KernelDesc &km, const KernelDesc &kd, int nx, int ny, int nz);
cudaError_t tile_spread_setup(int nz);
template <typename R>
void launch_edge_list(int64_t N, const Stencils<R> &sm, const KernelDesc &km, int nz, int *count, int *list,
                      cudaStream_t s);
template <typename RF>
void launch_spread_tiles(const RF *F, const RF *T, const KernelDesc &km, const KernelDesc &kd, const GridArgs &g,
                         const Stencils<float> &sm, const Stencils<float> &sd, float *grid, const Ghosts<float> &ghm,
                         const Ghosts<float> &ghd, const int *perm, const int *tstart, const int *edge,
                         int64_t n_edge, cudaStream_t s);
// backward pass (dpst_adjoint.cu, dpst_grad.cu)
template <typename R>
cudaError_t adj_plan(const KsArgs &a, int nsm, int64_t *grid, size_t *scratch_bytes);
template <typename R>
cudaError_t launch_adj_solve(const KsArgs &a, R *spec, const double2 *cadj, double *scratch, int64_t grid,
                             cudaStream_t s);
template <typename R>
cudaError_t launch_corr_adj(const KsArgs &a, const R *spec, double2 *cadj, cudaStream_t s);
template <typename R>
void launch_locate_grad(bool dipole, const double *pos, int64_t N, const KernelDesc &kd, const double *zext,
                        const double *wext, const GridArgs &g, const Stencils<R> &st, const GradStencils<R> &gs,
                        cudaStream_t s);
template <typename R, typename RG>
void launch_adj_spread_dip(const RG *gW, int64_t N, const KernelDesc &kd, const GridArgs &g, const Stencils<R> &st,
                           R *grid, const Ghosts<R> &gh, cudaStream_t s);
template <typename R>
void launch_ghost_fold_t(R *buf, int levels, int nx, int ny, const KernelDesc &kd, cudaStream_t s);
template <typename R, typename RF>
void launch_gather_mono(const R *u, const R *psi, int64_t N, const KernelDesc &kd, const GridArgs &g,
                        const Stencils<R> &st, const GradStencils<R> &gs, const Ghosts<R> &ghu,
                        const Ghosts<R> &ghp, const RF *F, const RF *gV, RF *gF, RF *gX, cudaStream_t s);
template <typename R, typename RF>
void launch_gather_dip(const R *u, const R *psi, int64_t N, const KernelDesc &kd, const GridArgs &g,
                       const Stencils<R> &st, const GradStencils<R> &gs, const Ghosts<R> &ghu,
                       const Ghosts<R> &ghp, const RF *T, const RF *gW, RF *gT, RF *gX, cudaStream_t s);

thread_local std::string g_last_error;

// ---- the engine -----------------------------------------------------------------

template <typename R>
struct Engine : EngineBase {
  typedef typename std::conditional<sizeof(R) == 8, cufftDoubleComplex, cufftComplex>::type CR;
  int nx, ny, nz, nxh, nsm;
  int64_t nk;
  double hx, hy, Lz, H;
  KernelHost km, kd;
  bool fused = false;  // monopole and dipole share one spread and one interpolation pass
  // tile-owner spread (mixed operator, fused pair): the grid written once per
  // tile, no clearing, no HBM atomics; edge particles (windows not interior)
  // from their list with atomics afterwards
  bool tile_spread = false;
  DevBuf edge_list;
  int64_t n_edge = 0;
  bool reg = false;    // torques with the regular kernel and spectral curls (DPST_TORQUE_REG)
  DevBuf gridT, specT; // reg: torque grid and spectrum, then the vorticity's
  GridArgs g;
  KsArgs ks;
  // device buffers
  DevBuf bvp_scratch;
  int64_t bvp_grid = 0;
  // double-float solve (DPST_SOLVE_DF64): factor copies and pressure scratch
  bool dfsolve = false;
  DevBuf df_mf, df_bk, df_ab, df_gi, df_km, df_dx, df_dy, bvp_df_scratch;
  int64_t bvp_df_grid = 0;
  int df_variant = 1;              // kernel variant chosen by tune_solve
  float df_ms[4] = {0, 0, 0, 0};   // its creation-time timings
  DevBuf grid, spec, corr, zext, wext, kvx, kvy, zn, bands, bcrows, k0rows, Tf, Ti;
  DevBuf fac_m, fac_i, fac_d, fac_a0, fac_a1, fac_c0, fac_c1, fac_g, fac_pm, fac_pb, fac_pa;
  DevBuf pos64, flags;
  DevBuf ord_count, ord_start, perm;  // particles sorted by grid tile
  DevBuf corrf, cmode, znf;           // FP32 correction tables (mixed operator, walls)
  DevBuf st_m[8], st_d[8];
  DevBuf gh_m[2], gh_d[2];
  DevBuf hF, hT, hV, hW;  // staging for the host-array entry points
  Stencils<R> stm, std_;
  Ghosts<R> ghm, ghd;
  int reach_m[2], reach_d[2];
  bool positioned = false;
  cufftHandle plan_f = 0, plan_b = 0;
  bool plans = false;
  // the library's own x-y transforms (mixed operator, power-of-two nx, ny);
  // cuFFT otherwise
  bool ownfft = false;
  DevBuf twx, twy;
  // one-launch x-y transforms (both passes, the intermediate in L2): per-plane
  // counters for up to xy_planes planes, the persistent grid, the plane lag,
  // and the creation-time timings {two-pass, one-launch} of a forward +
  // inverse pair
  bool xyfused = false;
  // the cluster form (one launch per direction, a plane across a cluster's
  // shared memory): chosen when faster at creation; its grid and error word
  bool xycl = false;
  int xycl_grid = 0;
  DevBuf xycl_err;
  float xycl_ms = 0.0f;
  // FP64 operator: the library's double-float x-y transforms (when faster
  // than cuFFT's FP64 ones at creation) and their timings {cuFFT, own}
  bool ownfft_d = false;
  DevBuf twxd, twyd;
  float xyd_ms[2] = {0.0f, 0.0f};
  DevBuf xyctr;
  int64_t xy_planes = 0;
  int xy_grid = 0, xy_lag = xy_lag_setting();
  float xy_ms[2] = {0.0f, 0.0f};

  Engine(const dpst_params &prm, int64_t n, int dev) {
    p = prm;
    N = n;
    device = dev;
    DPST_CUDA(cudaSetDevice(dev));
    DPST_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    nx = p.nx; ny = p.ny; nz = p.nz;
    nxh = nx / 2 + 1;
    nk = (int64_t)ny * nxh;
    hx = p.Lx / nx;
    hy = p.Ly / ny;
    Lz = p.zmax - p.zmin;
    H = Lz / 2;
    // Chebyshev grid on [0, Lz], descending (Chebyshev.py:4-38, FCM.py:207)
    std::vector<double> zG, zW;
    clencurt(nz, 0.0, Lz, zG, zW);
    km = make_kernel(p.w, p.beta, p.alpha, false, hx, hy, nx, ny, zG, zW, "monopole kernel");
    reg = p.has_torque && p.torque_kernel == DPST_TORQUE_REG;
    if (p.has_torque) kd = make_kernel(p.w_d, p.beta_d, p.alpha_d, !reg, hx, hy, nx, ny, zG, zW, "dipole kernel");
    fused = p.has_torque && !reg && fused_supports(km.d, kd.d);
    {
      // measured on c2: 0.45 ms against 0.25 ms for the clear-and-atomics
      // spread (latency-bound gather phase at two CTAs per SM), so it runs
      // only when asked for
      const char *env = getenv("DPSTOKES_GB300_SPREAD");
      const bool want_tiles = env && std::string(env) == "tiles";
      tile_spread = sizeof(R) == 4 && fused && want_tiles && tile_spread_supported(km.d, kd.d, nx, ny, nz);
    }
    km.d.zext_off = 0;
    kd.d.zext_off = (int)km.zext.size();
    std::vector<double> ze = km.zext, we = km.wext;
    ze.insert(ze.end(), kd.zext.begin(), kd.zext.end());
    we.insert(we.end(), kd.wext.begin(), kd.wext.end());
    upload(zext, ze);
    upload(wext, we);
    upload(zn, zG);
    // grid arguments + BC sets (FCM.py:215-248)
    memset(&g, 0, sizeof(g));
    g.nx = nx; g.ny = ny; g.nz = nz;
    g.hx = hx; g.hy = hy; g.Lx = p.Lx; g.Ly = p.Ly; g.Lz = Lz;
    bc_sets(p.mode, g);
    const std::vector<double> kx = wavenumbers(nx, p.Lx), ky = wavenumbers(ny, p.Ly);
    upload(kvx, kx);
    upload(kvy, ky);
    const ZTables zt = make_ztables(nz, H, p.mode);
    const double H2 = H * H;
    const int N2 = nz + 2;
    upload(bands, zt.bands);
    upload(bcrows, zt.bcrows);
    const std::vector<double> &k0r = zt.k0rows;
    const double *k0gi = zt.k0gi;
    upload(k0rows, k0r);
    // DCT-I matrices (Transform.cpp:107-304): forward = Chebyshev
    // coefficients from node values, inverse = node values from coefficients
    std::vector<double> tf, ti;
    dct_matrices(nz, tf, ti);
    std::vector<R> tfr(tf.begin(), tf.end()), tir(ti.begin(), ti.end());
    upload(Tf, tfr);
    upload(Ti, tir);
    // per-wavenumber factors
    fac_m.alloc(sizeof(double) * nz * nk);
    fac_i.alloc(sizeof(double) * (nz + 1) * nk);
    fac_d.alloc(sizeof(double) * nz * nk);
    fac_a0.alloc(sizeof(double) * nz * nk);
    fac_a1.alloc(sizeof(double) * nz * nk);
    fac_c0.alloc(sizeof(double) * nz * nk);
    fac_c1.alloc(sizeof(double) * nz * nk);
    fac_g.alloc(sizeof(double) * 4 * nk);
    memset(&ks, 0, sizeof(ks));
    ks.nx = nx; ks.ny = ny; ks.nz = nz; ks.nxh = nxh; ks.nk = nk;
    ks.H = H; ks.eta = p.viscosity; ks.Lz = Lz;
    ks.mode = p.mode;
    ks.kvx = kvx.as<double>(); ks.kvy = kvy.as<double>(); ks.zn = zn.as<double>();
    const double *bd = bands.as<double>();
    ks.s0 = bd; ks.sp2 = bd + nz; ks.sm2 = bd + 2 * nz; ks.fm1 = bd + 3 * nz; ks.fp1 = bd + 4 * nz;
    ks.se0 = H2; ks.se1 = H2; ks.fe = H;
    const double *bcd = bcrows.as<double>();
    ks.bcr1 = bcd; ks.bcr2 = bcd + N2; ks.bcl1 = bcd + 2 * N2; ks.bcl2 = bcd + 3 * N2;
    ks.mfac = fac_m.as<double>(); ks.invb = fac_i.as<double>(); ks.dp2 = fac_d.as<double>();
    ks.ab0 = fac_a0.as<double>(); ks.ab1 = fac_a1.as<double>();
    ks.c0 = fac_c0.as<double>(); ks.c1 = fac_c1.as<double>(); ks.ginv = fac_g.as<double>();
    ks.k0c0 = k0rows.as<double>(); ks.k0c1 = k0rows.as<double>() + nz;
    for (int q = 0; q < 4; ++q) ks.k0gi[q] = k0gi[q];
    fac_pm.alloc(sizeof(double) * nz * nk);
    fac_pb.alloc(sizeof(double) * 4 * nz * nk);
    fac_pa.alloc(sizeof(double) * nz * nk);
    ks.mf = fac_pm.as<double>();
    ks.bk = fac_pb.as<double>();
    ks.ab = fac_pa.as<double>();
    launch_bvp_factors(ks, 0);
    DPST_CUDA(cudaGetLastError());
    DPST_CUDA(cudaDeviceSynchronize());
    // the unpacked working arrays are no longer needed
    for (DevBuf *b : {&fac_m, &fac_i, &fac_d, &fac_a0, &fac_a1, &fac_c0, &fac_c1}) b->release();
    ks.mfac = ks.invb = ks.dp2 = ks.ab0 = ks.ab1 = ks.c0 = ks.c1 = nullptr;
    // grids, spectrum, correction coefficients, BVP scratch
    grid.alloc(sizeof(R) * 3 * (size_t)nz * ny * nx);
    spec.alloc(sizeof(CR) * 3 * (size_t)nz * nk);
    if (p.mode != DPST_MODE_NOWALL) corr.alloc(sizeof(double2) * 16 * (size_t)nk);
    if (p.mode != DPST_MODE_NOWALL && sizeof(R) == 4) {
      // FP32 tables of the mixed operator's correction epilogue: the solve's
      // coefficients in FP32, per mode {k, kx, ky, Hermitian} and the partner
      // index's {kx', ky'} (as mode_is_hermitian finds them), the nodes
      corrf.alloc(sizeof(float2) * 16 * (size_t)nk);
      std::vector<float> cm(8 * (size_t)nk, 0.0f);
      for (int64_t i = 0; i < nk; ++i) {
        const int ix = (int)(i % nxh), iy = (int)(i / nxh);
        const double kxi = kx[ix], kyi = ky[iy];
        const double kxp = kx[(nx - ix) % nx], kyp = ky[(ny - iy) % ny];
        float *r = &cm[8 * (size_t)i];
        r[0] = (float)std::sqrt(kxi * kxi + kyi * kyi);
        r[1] = (float)kxi;
        r[2] = (float)kyi;
        r[3] = (kxp == -kxi && kyp == -kyi) ? 1.0f : 0.0f;
        r[4] = (float)kxp;
        r[5] = (float)kyp;
      }
      upload(cmode, cm);
      const std::vector<float> zf(zG.begin(), zG.end());
      upload(znf, zf);
      ks.corrf = corrf.as<float2>();
    }
    size_t bvp_bytes = 0;
    DPST_CUDA(bvp_plan<R>(ks, nsm, &bvp_grid, &bvp_bytes));
    bvp_scratch.alloc(bvp_bytes);
    // the double-float solve: by default for the mixed operator
    dfsolve = p.solve_arith == DPST_SOLVE_DF64 || (p.solve_arith == DPST_SOLVE_DEFAULT && sizeof(R) == 4);
    if (dfsolve) {
      df_mf.alloc(sizeof(float2) * nz * nk);
      df_ab.alloc(sizeof(float2) * nz * nk);
      df_bk.alloc(sizeof(float4) * nk);
      df_gi.alloc(sizeof(float2) * 4 * nk);
      df_km.alloc(sizeof(float4) * nk);
      df_dx.alloc(sizeof(float2) * nxh);
      df_dy.alloc(sizeof(float2) * ny);
      ks.kap2 = df_mf.as<float2>();
      ks.ab2 = df_ab.as<float2>();
      ks.km3 = df_bk.as<float4>();
      ks.gi2 = df_gi.as<float2>();
      ks.km2 = df_km.as<float4>();
      ks.dx2 = df_dx.as<float2>();
      ks.dy2 = df_dy.as<float2>();
      launch_bvp_pack_df(ks, 0);
      DPST_CUDA(cudaGetLastError());
      size_t df_bytes = 0;
      DPST_CUDA(bvp_df_plan(ks, nsm, &bvp_df_grid, &df_bytes));
      bvp_df_scratch.alloc(df_bytes);
      DPST_CUDA(cudaDeviceSynchronize());
    }
    // particle buffers
    pos64.alloc(sizeof(double) * 3 * std::max<int64_t>(N, 1));
    flags.alloc(sizeof(int) * 8);
    alloc_stencils(km.d, false, st_m, stm);
    if (p.has_torque) alloc_stencils(kd.d, !reg, st_d, std_);
    if (reg) {  // torque grid / spectrum, then the vorticity's
      gridT.alloc(grid.bytes);
      specT.alloc(spec.bytes);
    }
    // particle order by grid tile (set_positions), used by the spread and
    // interpolation kernels
    if (tile_spread) {
      DPST_CUDA(tile_spread_setup(nz));
      edge_list.alloc(sizeof(int) * std::max<int64_t>(N, 1));
    }
    ord_count.alloc(sizeof(int) * tile_order_tiles(nx, ny));
    ord_start.alloc(sizeof(int) * (tile_order_tiles(nx, ny) + 1));
    perm.alloc(sizeof(int) * std::max<int64_t>(N, 1));
    memset(&ghm, 0, sizeof(ghm));
    memset(&ghd, 0, sizeof(ghd));
    // FFT plans: batched 2-D over (y, x) for each (component, z) plane
    int n2[2] = {ny, nx};
    int inem[2] = {ny, nx}, onem[2] = {ny, nxh};
    const int batch = 3 * nz;
    DPST_CUFFT(cufftPlanMany(&plan_f, 2, n2, inem, 1, ny * nx, onem, 1, (int)nk,
                             sizeof(R) == 8 ? CUFFT_D2Z : CUFFT_R2C, batch));
    DPST_CUFFT(cufftPlanMany(&plan_b, 2, n2, onem, 1, (int)nk, inem, 1, ny * nx,
                             sizeof(R) == 8 ? CUFFT_Z2D : CUFFT_C2R, batch));
    plans = true;
    {
      const char *env = getenv("DPSTOKES_GB300_XY_FFT");
      const bool want_cufft = env && std::string(env) == "cufft";  // or "twopass" / "fused"
      if (sizeof(R) == 4 && !want_cufft && own_fft_supported(nx, ny)) {
        ownfft = true;
        upload(twx, fft_twiddles(nx));
        upload(twy, fft_twiddles(ny));
        DPST_CUDA(fft_setup(nx, ny));
        if (fft_xy_fused_supported(nx, ny) && !(env && std::string(env) == "twopass")) {
          DPST_CUDA(fft_xy_setup(nx, ny, &xy_grid));
          grow_xy_counters(3 * (int64_t)nz);
        }
        if (fft_xy_cluster_supported(nx, ny) && !(env && std::string(env) == "twopass")) {
          DPST_CUDA(fft_xy_cluster_setup(nx, ny, &xycl_grid));
          if (xycl_grid > 0) {
            xycl_err.alloc(sizeof(int));
            DPST_CUDA(cudaMemset(xycl_err.p, 0, sizeof(int)));
          }
        }
      }
      if (sizeof(R) == 8 && !want_cufft && own_fft_df_supported(nx, ny)) {
        upload(twxd, fft_twiddles_df(nx));
        upload(twyd, fft_twiddles_df(ny));
        DPST_CUDA(fft_setup_df(nx, ny));
        tune_xy_d(env && std::string(env) == "own");
      }
    }
    DPST_CUDA(cudaDeviceSynchronize());
    tune_xy();
    tune_ztransform();
    tune_solve();
  }

  // FP64 operator: cuFFT's FP64 pair against the double-float kernels' pair
  // on the grid and spectrum buffers (one warm-up, best of three); force:
  // DPSTOKES_GB300_XY_FFT=own (or =cufft, which skips this).
  void tune_xy_d(bool force) {
    cudaEvent_t e0, e1;
    DPST_CUDA(cudaEventCreate(&e0));
    DPST_CUDA(cudaEventCreate(&e1));
    DPST_CUDA(cudaMemset(grid.p, 0, grid.bytes));
    for (int form = 0; form < 2; ++form) {
      ownfft_d = form == 1;
      float best = 1e30f;
      for (int r = 0; r < 4; ++r) {
        DPST_CUDA(cudaEventRecord(e0, 0));
        exec_fwd(grid.as<R>(), spec.as<CR>(), 0);
        exec_inv(spec.as<CR>(), grid.as<R>(), 0);
        DPST_CUDA(cudaEventRecord(e1, 0));
        DPST_CUDA(cudaEventSynchronize(e1));
        float ms = 0.0f;
        DPST_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (r > 0) best = std::min(best, ms);
      }
      xyd_ms[form] = best;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ownfft_d = force || xyd_ms[1] < xyd_ms[0];
    DPST_CUDA(cudaMemset(grid.p, 0, grid.bytes));
  }

  void grow_xy_counters(int64_t planes) {
    if (planes <= xy_planes) return;
    xyctr.alloc(sizeof(int) * fft_xy_counter_ints(planes));
    DPST_CUDA(cudaMemset(xyctr.p, 0, sizeof(int) * fft_xy_counter_ints(planes)));
    xy_planes = planes;
  }

  // The x-y transform's form: the two-pass kernels, the one-launch kernel and
  // the cluster kernel each run a forward + inverse pair on the grid and
  // spectrum buffers (one warm-up, best of three), and the fastest is kept;
  // a one-launch or cluster run whose waits gave up (error word set) is never
  // kept.  DPSTOKES_GB300_XY_FFT= fused | cluster | twopass fixes the choice.
  void tune_xy() {
    if (!ownfft || (xy_planes == 0 && xycl_grid == 0)) return;
    const char *env = getenv("DPSTOKES_GB300_XY_FFT");
    const std::string want = env ? std::string(env) : std::string();
    cudaStream_t s = 0;
    cudaEvent_t e0, e1;
    DPST_CUDA(cudaEventCreate(&e0));
    DPST_CUDA(cudaEventCreate(&e1));
    for (int form = 0; form < 3; ++form) {
      if (form == 1 && xy_planes == 0) continue;
      if (form == 2 && xycl_grid == 0) continue;
      xyfused = form == 1;
      xycl = form == 2;
      float best = 1e30f;
      for (int r = 0; r < 4; ++r) {
        DPST_CUDA(cudaEventRecord(e0, s));
        exec_fwd(grid.as<R>(), spec.as<CR>(), s);
        exec_inv(spec.as<CR>(), grid.as<R>(), s);
        DPST_CUDA(cudaEventRecord(e1, s));
        DPST_CUDA(cudaEventSynchronize(e1));
        float ms = 0.0f;
        DPST_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (r > 0) best = std::min(best, ms);
      }
      (form == 2 ? xycl_ms : xy_ms[form]) = best;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    int err = 0, errc = 0;
    if (xy_planes > 0) DPST_CUDA(cudaMemcpy(&err, xyctr.as<int>() + 2, sizeof(int), cudaMemcpyDeviceToHost));
    if (xycl_grid > 0) DPST_CUDA(cudaMemcpy(&errc, xycl_err.p, sizeof(int), cudaMemcpyDeviceToHost));
    const bool ok1 = xy_planes > 0 && err == 0, ok2 = xycl_grid > 0 && errc == 0;
    xyfused = xycl = false;
    if (want == "fused" && ok1) xyfused = true;
    else if (want == "cluster" && ok2) xycl = true;
    else if (want != "twopass") {
      float best = xy_ms[0];
      if (ok1 && xy_ms[1] < best) {
        best = xy_ms[1];
        xyfused = true;
      }
      if (ok2 && xycl_ms < best) {
        xyfused = false;
        xycl = true;
      }
    }
    DPST_CUDA(cudaMemset(grid.p, 0, grid.bytes));
  }

  // The double-float solve's kernel variant (prefetch depths, warps per SM):
  // each is timed on the spectrum buffer (3 runs after a warm-up) and the
  // fastest kept; DPSTOKES_GB300_SOLVE_VARIANT=<v> fixes it instead.
  void tune_solve() {
    if (!dfsolve || sizeof(R) != 4) return;
    const char *env = getenv("DPSTOKES_GB300_SOLVE_VARIANT");
    if (env && *env) {
      const int v = atoi(env);
      if (v < 0 || v >= bvp_df_variants()) throw Error(DPST_ERR_INVALID_ARG, "DPSTOKES_GB300_SOLVE_VARIANT out of range");
      df_variant = v;
      return;
    }
    R *sp = reinterpret_cast<R *>(spec.p);
    DPST_CUDA(cudaMemset(spec.p, 0, spec.bytes));
    if (corr.p) DPST_CUDA(cudaMemset(corr.p, 0, corr.bytes));
    cudaEvent_t a, b;
    DPST_CUDA(cudaEventCreate(&a));
    DPST_CUDA(cudaEventCreate(&b));
    float best = 0.0f;
    for (int v = 0; v < bvp_df_variants() && v < 4; ++v) {
      DPST_CUDA(launch_bvp_df<R>(ks, sp, corr.as<double2>(), bvp_df_scratch.as<float2>(), bvp_df_grid, v, 0));
      DPST_CUDA(cudaEventRecord(a, 0));
      for (int rep = 0; rep < 3; ++rep)
        DPST_CUDA(launch_bvp_df<R>(ks, sp, corr.as<double2>(), bvp_df_scratch.as<float2>(), bvp_df_grid, v, 0));
      DPST_CUDA(cudaEventRecord(b, 0));
      DPST_CUDA(cudaEventSynchronize(b));
      DPST_CUDA(cudaEventElapsedTime(&df_ms[v], a, b));
      df_ms[v] /= 3.0f;
      if (v == 0 || df_ms[v] < best) {
        best = df_ms[v];
        df_variant = v;
      }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }

  ~Engine() override {
    cudaSetDevice(device);
    cudaDeviceSynchronize();
    if (have_events)
      for (int i = 0; i < 8; ++i) cudaEventDestroy(ev[i]);
    if (plans) {
      cufftDestroy(plan_f);
      cufftDestroy(plan_b);
    }
    if (planK_f) cufftDestroy(planK_f);
    if (planK_b) cufftDestroy(planK_b);
  }

  void alloc_stencils(const KernelDesc &d, bool dip, DevBuf *b, Stencils<R> &s) {
    const size_t n = (size_t)std::max<int64_t>(N, 1);
    b[0].alloc(sizeof(int4) * n);
    b[1].alloc(sizeof(R) * n * d.wx);
    b[2].alloc(sizeof(R) * n * d.wy);
    b[3].alloc(sizeof(R) * n * d.wz_max);
    b[4].alloc(sizeof(R) * n * d.wz_max);
    if (dip) {
      b[5].alloc(sizeof(R) * n * d.wx);
      b[6].alloc(sizeof(R) * n * d.wy);
      b[7].alloc(sizeof(R) * n * d.wz_max);
    }
    s.cell = b[0].as<int4>();
    s.phx = b[1].as<R>();
    s.phy = b[2].as<R>();
    s.phz = b[3].as<R>();
    s.phzw = b[4].as<R>();
    s.dphx = dip ? b[5].as<R>() : nullptr;
    s.dphy = dip ? b[6].as<R>() : nullptr;
    s.dphz = dip ? b[7].as<R>() : nullptr;
    s.dphzw = nullptr;
    if (dip) {
      dphzw_buf.alloc(sizeof(R) * n * d.wz_max);
      s.dphzw = dphzw_buf.as<R>();
    }
  }
  DevBuf dphzw_buf;

  // Ghost layers at open z ends that some particle reaches (see Ghosts).
  void setup_ghosts(const KernelDesc &d, const ZEnds &ends, const int reach[2], DevBuf *b, Ghosts<R> &gh) {
    const size_t lev = (size_t)d.nyeff * d.nxeff * 3;
    gh.top = gh.bot = nullptr;
    gh.ntop = gh.nbot = 0;
    if (!ends.top_active && reach[0] < d.dend) {
      gh.ntop = d.dend;
      if (b[0].bytes < sizeof(R) * lev * d.dend) b[0].alloc(sizeof(R) * lev * d.dend);
      gh.top = b[0].as<R>();
    }
    const int ubeg = d.dend + nz;
    if (!ends.bot_active && reach[1] >= ubeg) {
      gh.nbot = d.dend;
      if (b[1].bytes < sizeof(R) * lev * d.dend) b[1].alloc(sizeof(R) * lev * d.dend);
      gh.bot = b[1].as<R>();
    }
  }

  void set_positions(const void *pos, int dtype, cudaStream_t s) override {
    if (N == 0) { positioned = true; return; }
    if (pos == nullptr) throw Error(DPST_ERR_INVALID_ARG, "positions pointer is NULL");
    convert_positions(pos, dtype, s);
    int init[8] = {0, INT_MAX, -1, INT_MAX, -1, 0, 0, 0};
    int *fl = flags.as<int>();
    DPST_CUDA(cudaMemcpyAsync(fl, init, sizeof(init), cudaMemcpyHostToDevice, s));
    launch_locate<R>(false, pos64.as<double>(), N, km.d, zext.as<double>(), wext.as<double>(), g, stm, fl,
                     fl + 1, s);
    if (p.has_torque)
      launch_locate<R>(!reg, pos64.as<double>(), N, kd.d, zext.as<double>(), wext.as<double>(), g, std_, fl,
                       fl + 3, s);
    DPST_CUDA(cudaGetLastError());
    int out[8];
    launch_tile_order<R>(N, g, stm, ord_count.as<int>(), ord_start.as<int>(), perm.as<int>(), s);
    if (tile_spread) launch_edge_list<R>(N, stm, km.d, nz, fl + 5, edge_list.as<int>(), s);
    DPST_CUDA(cudaGetLastError());
    DPST_CUDA(cudaMemcpyAsync(out, fl, sizeof(out), cudaMemcpyDeviceToHost, s));
    DPST_CUDA(cudaStreamSynchronize(s));
    if (out[0] & 1) {
      positioned = false;
      throw Error(DPST_ERR_OUT_OF_DOMAIN, "a particle lies outside [0,Lx]x[0,Ly]x[zmin,zmax] (or is NaN)");
    }
    if (out[0] & 2) {
      positioned = false;
      throw Error(DPST_ERR_CUDA, "internal: z window longer than its bound");
    }
    n_edge = tile_spread ? out[5] : 0;
    reach_m[0] = out[1]; reach_m[1] = out[2];
    reach_d[0] = out[3]; reach_d[1] = out[4];
    setup_ghosts(km.d, g.bcA, reach_m, gh_m, ghm);
    if (p.has_torque) setup_ghosts(kd.d, reg ? g.bcA : g.bcB, reach_d, gh_d, ghd);
    positioned = true;
  }

  void convert_positions(const void *pos, int dtype, cudaStream_t s);

  cudaEvent_t ev[8] = {};
  bool have_events = false;
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
    // regular-kernel torques are curled in wavenumber space: the grid holds the forces only
    spread_into<RF>(F, reg ? nullptr : T, grid.as<R>(), ghm, ghd, s);
  }

  // spread F (+ the torque curl) into the grid gr with the ghost layers gm, gd
  template <typename RF>
  void spread_into(const RF *F, const RF *T, R *gr, const Ghosts<R> &gm, const Ghosts<R> &gd, cudaStream_t s) {
    const bool torque = p.has_torque && T != nullptr;
    const bool tiles = tile_spread && torque;
    if (!tiles) DPST_CUDA(cudaMemsetAsync(gr, 0, grid.bytes, s));
    for (const Ghosts<R> *gh : {&gm, &gd}) {
      const KernelDesc &d = (gh == &gm) ? km.d : kd.d;
      const size_t lev = (size_t)d.nyeff * d.nxeff * 3 * sizeof(R);
      if (gh->top) DPST_CUDA(cudaMemsetAsync(gh->top, 0, lev * gh->ntop, s));
      if (gh->bot) DPST_CUDA(cudaMemsetAsync(gh->bot, 0, lev * gh->nbot, s));
    }
    if (tiles) {
      if constexpr (sizeof(R) == 4)
        launch_spread_tiles<RF>(F, T, km.d, kd.d, g, stm, std_, gr, gm, gd, perm.as<int>(), ord_start.as<int>(),
                                edge_list.as<int>(), n_edge, s);
    } else if (torque && fused) {
      launch_spread_fused<R, RF>(F, T, N, km.d, kd.d, g, stm, std_, gr, gm, gd, s, perm.as<int>());
    } else {
      launch_spread<R, RF>(false, F, N, km.d, g, stm, gr, gm, s, perm.as<int>());
      if (torque) launch_spread<R, RF>(true, T, N, kd.d, g, std_, gr, gd, s, perm.as<int>());
    }
    launch_ghost_fold<R>(gm.top, gm.ntop, nx, ny, km.d, s);
    launch_ghost_fold<R>(gm.bot, gm.nbot, nx, ny, km.d, s);
    if (torque) {
      launch_ghost_fold<R>(gd.top, gd.ntop, nx, ny, kd.d, s);
      launch_ghost_fold<R>(gd.bot, gd.nbot, nx, ny, kd.d, s);
    }
    DPST_CUDA(cudaGetLastError());
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

  // ---- z transform kernel choice (creation-time autotuner) -----------------
  // 0: SIMT even/odd-folded GEMM (FP32 or FP64); 1: tcgen05 split-TF32 (FP32
  // data only, nz <= 128), operands staged through registers; 3: the same
  // fed by TMA (nz >= 32, an even number of modes).  Chosen separately for
  // the plain transforms (ztc[0]: forward, and the backward's adjoint
  // transforms) and for the inverse with its wall correction (ztc[1]), each
  // timed on this handle's buffers.  DPSTOKES_GB300_ZTRANSFORM = simt |
  // tcgen05 | tma | auto (default) overrides the choice, and
  // DPSTOKES_GB300_ZTMA_VARIANT = 0 | 1 | 2 the TMA-fed form's variant.
  int ztc[2] = {0, 0};
  float ztc_ms[2][2] = {{0.f, 0.f}, {0.f, 0.f}};  // [direction][impl]
  float ztm_ms[2] = {0.f, 0.f};                   // [direction]: the TMA-fed form, its best variant
  int ztm_var[2] = {0, 0};                        // [direction]: that variant (ring and converted stages)
  float ztm_vms[2][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};  // [direction][variant]
  DevBuf ztc_err;

  // the wall-correction inputs of the inverse transform's epilogue
  void epi_corr(EpiArgs &e) const {
    e.corr = corr.as<double2>();
    if (corrf.p != nullptr) {
      e.corrf = corrf.as<float2>();
      e.cmode = cmode.as<float4>();
      e.znf = znf.as<float>();
      e.fac = (float)(1.0 / 2.0 / p.viscosity);
    }
  }

  // impl < 0: the tuned kernel for e's direction; 0 SIMT in the operator's
  // arithmetic, 1 tcgen05 split-TF32 (FP32 spectra), 2 double-float SIMT
  // (FP64 spectra), 3 tcgen05 split-TF32 fed by TMA (FP32 spectra)
  cudaError_t zgemm(R *sp, const R *T, const EpiArgs &e, bool fold_out, cudaStream_t s, int impl = -1) {
    if (impl < 0) impl = ztc[e.inverse ? 1 : 0];
    if constexpr (sizeof(R) == 8) {
      if (impl == 2)
        return launch_zgemm_df(reinterpret_cast<double *>(sp), nz, 2 * nk, reinterpret_cast<const double *>(T), e,
                               nsm, s, fold_out);
    }
    if ((impl == 1 || impl == 3) && sizeof(R) == 4) {
      float *fs = reinterpret_cast<float *>(sp);
      const float *fT = reinterpret_cast<const float *>(T);
      const bool tma = impl == 3 && ztm_supported(fs, nz, 2 * nk);
      if (e.inverse && e.ks.mode != 0 && e.corr != nullptr) {
        // the wall correction as its own pass: the tcgen05 epilogue's four
        // warps are too few for its arithmetic
        EpiArgs e2 = e;
        e2.corr = nullptr;
        e2.corrf = nullptr;
        cudaError_t r = tma ? launch_zgemm_tma(fs, nz, 2 * nk, fT, e2, nsm, ztc_err.as<int>(), ztm_var[1], s)
                            : launch_zgemm_tc(fs, nz, 2 * nk, fT, e2, nsm, ztc_err.as<int>(), s);
        if (r == cudaSuccess) r = launch_corr_add(fs, nz, nk, e, s);
        return r;
      }
      return tma ? launch_zgemm_tma(fs, nz, 2 * nk, fT, e, nsm, ztc_err.as<int>(), ztm_var[e.inverse ? 1 : 0], s)
                 : launch_zgemm_tc(fs, nz, 2 * nk, fT, e, nsm, ztc_err.as<int>(), s);
    }
    return launch_zgemm<R>(sp, nz, 2 * nk, T, e, nsm, s, fold_out);
  }

  // The FP64 operator: the FP64 and the double-float SIMT transforms per
  // direction, timed like the FP32 pair (one warm-up, three runs), the faster
  // kept; DPSTOKES_GB300_ZTRANSFORM=simt | df64 fixes one.
  void tune_ztransform_fp64(const std::string &want) {
    if (want == "simt") return;
    R *sp = reinterpret_cast<R *>(spec.p);
    DPST_CUDA(cudaMemset(spec.p, 0, spec.bytes));
    DPST_CUDA(cudaMemset(corr.p, 0, corr.bytes));
    cudaEvent_t a, b;
    DPST_CUDA(cudaEventCreate(&a));
    DPST_CUDA(cudaEventCreate(&b));
    for (int dir = 0; dir < 2; ++dir) {
      EpiArgs e;
      memset(&e, 0, sizeof(e));
      e.ks = ks;
      e.inverse = dir;
      e.scale = dir ? 1.0 / ((double)nx * (double)ny) : 1.0;
      if (dir) epi_corr(e);
      const R *T = dir ? Ti.as<R>() : Tf.as<R>();
      for (int k = 0; k < 2; ++k) {
        const int impl = k ? 2 : 0;
        DPST_CUDA(zgemm(sp, T, e, dir == 1, 0, impl));  // warm-up
        DPST_CUDA(cudaEventRecord(a, 0));
        for (int rep = 0; rep < 3; ++rep) DPST_CUDA(zgemm(sp, T, e, dir == 1, 0, impl));
        DPST_CUDA(cudaEventRecord(b, 0));
        DPST_CUDA(cudaEventSynchronize(b));
        DPST_CUDA(cudaEventElapsedTime(&ztc_ms[dir][k], a, b));
        ztc_ms[dir][k] /= 3.0f;
      }
      ztc[dir] = (want == "df64" || ztc_ms[dir][1] < ztc_ms[dir][0]) ? 2 : 0;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    DPST_CUDA(cudaMemset(spec.p, 0, spec.bytes));
  }

  void tune_ztransform() {
    ztc_err.alloc(sizeof(int));
    DPST_CUDA(cudaMemset(ztc_err.p, 0, sizeof(int)));
    const char *env = getenv("DPSTOKES_GB300_ZTRANSFORM");
    const std::string want = env ? env : "auto";
    if (sizeof(R) == 8) {
      tune_ztransform_fp64(want);
      return;
    }
    if (nz > 128 || want == "simt") return;
    R *sp = reinterpret_cast<R *>(spec.p);
    const bool tma_ok = want != "tcgen05" && ztm_supported(reinterpret_cast<const float *>(sp), nz, 2 * nk);
    DPST_CUDA(cudaMemset(spec.p, 0, spec.bytes));
    DPST_CUDA(cudaMemset(corr.p, 0, corr.bytes));
    cudaEvent_t a, b;
    DPST_CUDA(cudaEventCreate(&a));
    DPST_CUDA(cudaEventCreate(&b));
    for (int dir = 0; dir < 2; ++dir) {
      EpiArgs e;
      memset(&e, 0, sizeof(e));
      e.ks = ks;
      e.inverse = dir;
      e.scale = dir ? 1.0 / ((double)nx * (double)ny) : 1.0;
      if (dir) epi_corr(e);
      const R *T = dir ? Ti.as<R>() : Tf.as<R>();
      // SIMT, tcgen05, then each variant of the TMA-fed form
      const int nv = tma_ok ? ztm_variants() : 0;
      int best_var = 0;
      for (int k = 0; k < 2 + nv; ++k) {
        const int impl = k >= 2 ? 3 : k;
        if (impl == 3) ztm_var[dir] = k - 2;
        float ms = 0.0f;
        DPST_CUDA(zgemm(sp, T, e, dir == 1, 0, impl));  // warm-up
        DPST_CUDA(cudaEventRecord(a, 0));
        for (int rep = 0; rep < 3; ++rep) DPST_CUDA(zgemm(sp, T, e, dir == 1, 0, impl));
        DPST_CUDA(cudaEventRecord(b, 0));
        DPST_CUDA(cudaEventSynchronize(b));
        DPST_CUDA(cudaEventElapsedTime(&ms, a, b));
        ms /= 3.0f;
        if (impl != 3) ztc_ms[dir][impl] = ms;
        else ztm_vms[dir][k - 2] = ms;
        if (impl == 3 && (k == 2 || ms < ztm_ms[dir])) {
          ztm_ms[dir] = ms;
          best_var = k - 2;
        }
      }
      ztm_var[dir] = best_var;
      if (const char *ev = getenv("DPSTOKES_GB300_ZTMA_VARIANT")) {
        const int v = atoi(ev);
        if (v >= 0 && v < nv) ztm_var[dir] = v;
      }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    int err = 0;
    DPST_CUDA(cudaMemcpy(&err, ztc_err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) {  // the tensor-core kernel gave up waiting: keep the SIMT kernel
      ztc[0] = ztc[1] = 0;
      DPST_CUDA(cudaMemset(ztc_err.p, 0, sizeof(int)));
      return;
    }
    for (int dir = 0; dir < 2; ++dir) {
      if (want == "tma" && tma_ok) ztc[dir] = 3;
      else if (want == "tcgen05") ztc[dir] = 1;
      else {
        float best = ztc_ms[dir][0];
        ztc[dir] = 0;
        if (ztc_ms[dir][1] < best) {
          best = ztc_ms[dir][1];
          ztc[dir] = 1;
        }
        if (tma_ok && ztm_ms[dir] < best) ztc[dir] = 3;
      }
    }
  }

  // grid (spread forces) -> grid (velocities): x-y FFT, z transform, per-k
  // solve, inverse z transform with the wall correction, inverse x-y FFT
  void solve_stage(cudaStream_t s) {
    R *gr = grid.as<R>();
    CR *sp = spec.as<CR>();
    exec_fwd(gr, sp, s);
    mark(2, s);
    EpiArgs ef;
    memset(&ef, 0, sizeof(ef));
    ef.inverse = 0;
    ef.scale = 1.0;
    ef.ks = ks;
    DPST_CUDA(zgemm((R *)sp, Tf.as<R>(), ef, false, s));
    mark(3, s);
    bvp_stage(sp, s);
    mark(4, s);
    EpiArgs eb = ef;
    eb.inverse = 1;
    eb.scale = 1.0 / ((double)nx * (double)ny);
    epi_corr(eb);
    DPST_CUDA(zgemm((R *)sp, Ti.as<R>(), eb, true, s));
    mark(5, s);
    exec_inv(sp, gr, s);
    mark(6, s);
  }

  template <typename RF>
  void run(const RF *F, const RF *T, RF *V, RF *W, cudaStream_t s) {
    if (reg) {
      run_reg<RF>(F, T, V, W, s);
      return;
    }
    const bool torque = p.has_torque && T != nullptr;
    R *gr = grid.as<R>();
    mark(0, s);
    spread_stage<RF>(F, T, s);
    mark(1, s);
    solve_stage(s);
    interp_from<RF>(gr, ghm, ghd, torque, V, W, s);
    mark(7, s);
    if (stage_ms) {
      DPST_CUDA(cudaEventSynchronize(ev[7]));
      const int from[8] = {0, 1, 2, 3, 4, 5, 6, 0}, to[8] = {1, 2, 3, 4, 5, 6, 7, 7};
      for (int k = 0; k < 8; ++k) DPST_CUDA(cudaEventElapsedTime(&stage_ms[k], ev[from[k]], ev[to[k]]));
    }
  }

  // ---- regular-kernel torque coupling (DPST_TORQUE_REG) ----------------------
  // The reference's useRegKernel path (FCM.py:372-396, 427-439): the torques
  // spread with the regular kernel of (w_d, beta_d, alpha_d) into their own
  // grid (BC set A, its own open-end ghost layers); after the forward
  // transforms, 1/2 curl of the torque coefficients is added to the forces'
  // (k_spec_curl); the solve; the vorticity 1/2 curl u (Solvers.py:159-177)
  // of the solution's coefficients (open domain) or, with walls, of the
  // corrected velocity's coefficients (the reference's U_hat: the velocity
  // nodes with the wall correction transformed forward again); both go
  // through the inverse z and x-y transforms; V is
  // interpolated with the monopole kernel, Omega with the regular dipole
  // kernel from the vorticity grid and the torque grid's ghost layers.
  template <typename RF>
  void run_reg(const RF *F, const RF *T, RF *V, RF *W, cudaStream_t s) {
    const bool torque = T != nullptr;
    R *gr = grid.as<R>(), *gt = gridT.as<R>();
    CR *sp = spec.as<CR>(), *st = specT.as<CR>();
    mark(0, s);
    spread_into<RF>(F, nullptr, gr, ghm, ghd, s);  // also clears the torque ghost layers
    if (torque) {
      DPST_CUDA(cudaMemsetAsync(gt, 0, gridT.bytes, s));
      launch_spread<R, RF>(false, T, N, kd.d, g, std_, gt, ghd, s, perm.as<int>());
      launch_ghost_fold<R>(ghd.top, ghd.ntop, nx, ny, kd.d, s);
      launch_ghost_fold<R>(ghd.bot, ghd.nbot, nx, ny, kd.d, s);
      DPST_CUDA(cudaGetLastError());
    }
    mark(1, s);
    exec_fwd(gr, sp, s);
    if (torque) exec_fwd(gt, st, s);
    mark(2, s);
    EpiArgs ef;
    memset(&ef, 0, sizeof(ef));
    ef.inverse = 0;
    ef.scale = 1.0;
    ef.ks = ks;
    DPST_CUDA(zgemm((R *)sp, Tf.as<R>(), ef, false, s));
    if (torque) {
      DPST_CUDA(zgemm((R *)st, Tf.as<R>(), ef, false, s));
      launch_spec_curl<R>((const R *)st, (R *)sp, true, nz, nk, nx, ny, nxh, kvx.as<double>(), kvy.as<double>(),
                          H, s);
      DPST_CUDA(cudaGetLastError());
    }
    mark(3, s);
    bvp_stage(sp, s);
    mark(4, s);
    EpiArgs eb = ef;
    eb.inverse = 1;
    eb.scale = 1.0 / ((double)nx * (double)ny);
    epi_corr(eb);
    EpiArgs ew = ef;
    ew.inverse = 1;
    ew.ks.mode = 0;  // the vorticity's inverse transform adds no wall correction
    if (p.mode == DPST_MODE_NOWALL) {
      // no correction: the vorticity straight from the solution's coefficients
      launch_spec_curl<R>((const R *)sp, (R *)st, false, nz, nk, nx, ny, nxh, kvx.as<double>(), kvy.as<double>(),
                          H, s);
      DPST_CUDA(cudaGetLastError());
      DPST_CUDA(zgemm((R *)sp, Ti.as<R>(), eb, true, s));
      ew.scale = eb.scale;
      DPST_CUDA(zgemm((R *)st, Ti.as<R>(), ew, true, s));
    } else {
      // walls: the correction is added at the nodes; the corrected velocity's
      // coefficients (the reference's U_hat) come from transforming them forward
      DPST_CUDA(zgemm((R *)sp, Ti.as<R>(), eb, true, s));
      DPST_CUDA(cudaMemcpyAsync(st, sp, spec.bytes, cudaMemcpyDeviceToDevice, s));
      DPST_CUDA(zgemm((R *)st, Tf.as<R>(), ef, false, s));
      launch_spec_curl<R>((const R *)st, (R *)st, false, nz, nk, nx, ny, nxh, kvx.as<double>(), kvy.as<double>(),
                          H, s);
      DPST_CUDA(cudaGetLastError());
      DPST_CUDA(zgemm((R *)st, Ti.as<R>(), ew, true, s));
    }
    mark(5, s);
    exec_inv(sp, gr, s);
    exec_inv(st, gt, s);
    mark(6, s);
    launch_interp<R, RF>(false, gr, N, km.d, g, stm, ghm, V, s, perm.as<int>());
    if (W != nullptr) {
      Ghosts<R> gz = ghd;
      if (!torque) { gz.top = nullptr; gz.bot = nullptr; }
      launch_interp<R, RF>(false, gt, N, kd.d, g, std_, gz, W, s, perm.as<int>());
    }
    DPST_CUDA(cudaGetLastError());
    mark(7, s);
    if (stage_ms) {
      DPST_CUDA(cudaEventSynchronize(ev[7]));
      const int from[8] = {0, 1, 2, 3, 4, 5, 6, 0}, to[8] = {1, 2, 3, 4, 5, 6, 7, 7};
      for (int k = 0; k < 8; ++k) DPST_CUDA(cudaEventElapsedTime(&stage_ms[k], ev[from[k]], ev[to[k]]));
    }
  }

  // per-wavenumber solve (+ k = 0) on the spectrum sp, in place
  void bvp_stage(CR *sp, cudaStream_t s) {
    if (!use_static_scratch && dfsolve) {
      DPST_CUDA(launch_bvp_df<R>(ks, (R *)sp, corr.as<double2>(), bvp_df_scratch.as<float2>(), bvp_df_grid,
                                 df_variant, s));
      DPST_CUDA(launch_bvp_k0<R>(ks, (R *)sp, s));
    } else if (!use_static_scratch) {
      DPST_CUDA(launch_bvp<R>(ks, (R *)sp, corr.as<double2>(), bvp_scratch.as<double>(), bvp_grid, s));
    } else {
      bool too_big = false;
      cudaError_t e = launch_bvp_noalloc<R>(ks, (R *)sp, corr.as<double2>(), bvp_grid, s, &too_big);
      if (too_big)
        throw Error(DPST_ERR_UNSUPPORTED,
                    "dpst_mdot_noalloc: one CTA of the solve needs nz*192 = " + std::to_string(nz * 192) +
                        " doubles of scratch, more than the static array's " +
                        std::to_string(noalloc_scratch_bytes() / sizeof(double)));
      DPST_CUDA(e);
    }
  }

  // x-y transforms of `planes` grid planes (3 nz for one grid): the library's
  // row and column passes, or the cuFFT plan given (made for that many planes)
  void exec_fwd(R *gr, CR *sp, cudaStream_t s, int64_t planes = 0, cufftHandle plan = 0) {
    if (planes == 0) planes = 3 * (int64_t)nz;
    if (plan == 0) plan = plan_f;
    if constexpr (sizeof(R) == 8) {
      if (ownfft_d) {
        DPST_CUDA(fft_rows_df(false, reinterpret_cast<const double *>(gr), reinterpret_cast<double2 *>(sp), nullptr,
                              nullptr, nx, planes * ny, twxd.as<float4>(), s));
        DPST_CUDA(fft_cols_df(false, reinterpret_cast<double2 *>(sp), ny, nxh, planes, twyd.as<float4>(), s));
        return;
      }
    }
    if (ownfft && xycl) {
      DPST_CUDA(fft_xy_cluster(false, reinterpret_cast<const float *>(gr), reinterpret_cast<float2 *>(sp), nullptr, nx,
                               ny, planes, twx.as<float2>(), twy.as<float2>(), xycl_err.as<int>(), xycl_grid, s));
      return;
    }
    if (ownfft && xyfused && planes <= xy_planes) {
      DPST_CUDA(fft_xy_fused(false, reinterpret_cast<const float *>(gr), reinterpret_cast<float2 *>(sp), nullptr, nx,
                             ny, planes, twx.as<float2>(), twy.as<float2>(), xyctr.as<int>(), xy_grid, xy_lag, s));
      return;
    }
    if (ownfft) {
      DPST_CUDA(fft_rows(false, reinterpret_cast<const float *>(gr), reinterpret_cast<float2 *>(sp), nullptr,
                         nullptr, nx, planes * ny, twx.as<float2>(), s));
      DPST_CUDA(fft_cols(false, reinterpret_cast<float2 *>(sp), ny, nxh, planes, twy.as<float2>(), s));
      return;
    }
    DPST_CUFFT(cufftSetStream(plan, s));
    if (sizeof(R) == 8)
      DPST_CUFFT(cufftExecD2Z(plan, (cufftDoubleReal *)gr, (cufftDoubleComplex *)sp));
    else
      DPST_CUFFT(cufftExecR2C(plan, (cufftReal *)gr, (cufftComplex *)sp));
  }
  void exec_inv(CR *sp, R *gr, cudaStream_t s, int64_t planes = 0, cufftHandle plan = 0) {
    if (planes == 0) planes = 3 * (int64_t)nz;
    if (plan == 0) plan = plan_b;
    if constexpr (sizeof(R) == 8) {
      if (ownfft_d) {
        DPST_CUDA(fft_cols_df(true, reinterpret_cast<double2 *>(sp), ny, nxh, planes, twyd.as<float4>(), s));
        DPST_CUDA(fft_rows_df(true, nullptr, nullptr, reinterpret_cast<const double2 *>(sp),
                              reinterpret_cast<double *>(gr), nx, planes * ny, twxd.as<float4>(), s));
        return;
      }
    }
    if (ownfft && xycl) {
      DPST_CUDA(fft_xy_cluster(true, nullptr, reinterpret_cast<float2 *>(sp), reinterpret_cast<float *>(gr), nx, ny,
                               planes, twx.as<float2>(), twy.as<float2>(), xycl_err.as<int>(), xycl_grid, s));
      return;
    }
    if (ownfft && xyfused && planes <= xy_planes) {
      DPST_CUDA(fft_xy_fused(true, nullptr, reinterpret_cast<float2 *>(sp), reinterpret_cast<float *>(gr), nx, ny,
                             planes, twx.as<float2>(), twy.as<float2>(), xyctr.as<int>(), xy_grid, xy_lag, s));
      return;
    }
    if (ownfft) {
      DPST_CUDA(fft_cols(true, reinterpret_cast<float2 *>(sp), ny, nxh, planes, twy.as<float2>(), s));
      DPST_CUDA(fft_rows(true, nullptr, nullptr, reinterpret_cast<const float2 *>(sp), reinterpret_cast<float *>(gr),
                         nx, planes * ny, twx.as<float2>(), s));
      return;
    }
    DPST_CUFFT(cufftSetStream(plan, s));
    if (sizeof(R) == 8)
      DPST_CUFFT(cufftExecZ2D(plan, (cufftDoubleComplex *)sp, (cufftDoubleReal *)gr));
    else
      DPST_CUFFT(cufftExecC2R(plan, (cufftComplex *)sp, (cufftReal *)gr));
  }

  // interpolate V (and, with W, the angular velocities) from the grid gr with
  // the ghost layers gm, gd
  template <typename RF>
  void interp_from(const R *gr, const Ghosts<R> &gm, const Ghosts<R> &gd, bool torque, RF *V, RF *W,
                   cudaStream_t s) {
    if (p.has_torque && W != nullptr) {
      // without torques the reference's torque grid still holds the last
      // z-derivative spread; with T = NULL it is zero
      Ghosts<R> gz = gd;
      if (!torque) { gz.top = nullptr; gz.bot = nullptr; }
      if (fused) {
        launch_interp_fused<R, RF>(gr, N, km.d, kd.d, g, stm, std_, gm, gz, V, W, s, perm.as<int>());
      } else {
        launch_interp<R, RF>(false, gr, N, km.d, g, stm, gm, V, s, perm.as<int>());
        launch_interp<R, RF>(true, gr, N, kd.d, g, std_, gz, W, s, perm.as<int>());
      }
    } else {
      launch_interp<R, RF>(false, gr, N, km.d, g, stm, gm, V, s, perm.as<int>());
    }
    DPST_CUDA(cudaGetLastError());
  }

  // ---- multi-RHS Mdot (dpst_mdot_multi) -------------------------------------
  // K force (and torque) columns at the same positions.  Per column: the spread
  // into its slice of K-column grid and ghost-layer buffers, the z transforms,
  // the interpolation; across columns: one cuFFT execution per direction over
  // the K x 3 nz planes and one solve over the K nk wavenumbers (the batched
  // solve kernels with one table entry per column, sharing the factors).
  // Buffers are sized on the first call with a given K (a larger K replaces
  // them).
  int multi_k = 0;
  DevBuf gridK, specK, corrK, corrfK, ghostK[4], sysK, mprefK, bvpK_scratch;
  int64_t bvpK_grid = 0;
  cufftHandle planK_f = 0, planK_b = 0;

  void ensure_multi(int K) {
    if (K <= multi_k) return;
    if (planK_f) cufftDestroy(planK_f);
    if (planK_b) cufftDestroy(planK_b);
    planK_f = planK_b = 0;
    multi_k = 0;
    gridK.alloc(grid.bytes * K);
    specK.alloc(spec.bytes * K);
    if (corr.p) corrK.alloc(corr.bytes * K);
    if (corrf.p) corrfK.alloc(corrf.bytes * K);
    int n2[2] = {ny, nx};
    int inem[2] = {ny, nx}, onem[2] = {ny, nxh};
    const int batch = 3 * nz * K;
    DPST_CUFFT(cufftPlanMany(&planK_f, 2, n2, inem, 1, ny * nx, onem, 1, (int)nk,
                             sizeof(R) == 8 ? CUFFT_D2Z : CUFFT_R2C, batch));
    DPST_CUFFT(cufftPlanMany(&planK_b, 2, n2, onem, 1, (int)nk, inem, 1, ny * nx,
                             sizeof(R) == 8 ? CUFFT_Z2D : CUFFT_C2R, batch));
    std::vector<SysK<R>> sk(K);
    std::vector<int64_t> mp(K + 1, 0);
    for (int k = 0; k < K; ++k) {
      sk[k].ks = ks;
      sk[k].ks.corrf = corrf.p ? corrfK.as<float2>() + (size_t)k * 16 * nk : nullptr;
      sk[k].spec = reinterpret_cast<R *>(specK.as<CR>() + (size_t)k * 3 * nz * nk);
      sk[k].corr = corr.p ? corrK.as<double2>() + (size_t)k * 16 * nk : nullptr;
      mp[k + 1] = mp[k] + nk;
    }
    upload(sysK, sk);
    upload(mprefK, mp);
    size_t bytes = 0;
    if (dfsolve) {
      DPST_CUDA(bvp_df_plan_b(ks, (int64_t)K * nk, nsm, &bvpK_grid, &bytes));
    } else {
      DPST_CUDA(bvp_plan_b<R>(nz, (int64_t)K * nk, nsm, &bvpK_grid, &bytes));
    }
    bvpK_scratch.alloc(bytes);
    if (xy_planes > 0) grow_xy_counters(3 * (int64_t)nz * K);
    DPST_CUDA(cudaDeviceSynchronize());
    multi_k = K;
  }

  // column k's ghost layers: slices of K-column buffers shaped like the
  // single-column ones (their sizes follow the current positions)
  Ghosts<R> ghosts_of(const Ghosts<R> &g1, const KernelDesc &d, DevBuf *b, int k, int K) {
    Ghosts<R> gk = g1;
    const size_t lev = (size_t)d.nyeff * d.nxeff * 3;
    if (g1.top) {
      if (b[0].bytes < sizeof(R) * lev * g1.ntop * K) b[0].alloc(sizeof(R) * lev * g1.ntop * K);
      gk.top = b[0].as<R>() + (size_t)k * lev * g1.ntop;
    }
    if (g1.bot) {
      if (b[1].bytes < sizeof(R) * lev * g1.nbot * K) b[1].alloc(sizeof(R) * lev * g1.nbot * K);
      gk.bot = b[1].as<R>() + (size_t)k * lev * g1.nbot;
    }
    return gk;
  }

  template <typename RF>
  void run_multi(int K, const RF *F, const RF *T, RF *V, RF *W, cudaStream_t s) {
    ensure_multi(K);
    const bool torque = p.has_torque && T != nullptr;
    const size_t col = 3 * (size_t)N;
    const size_t gcol = grid.bytes / sizeof(R), scol = 3 * (size_t)nz * nk;
    R *gK = gridK.as<R>();
    CR *sK = specK.as<CR>();
    std::vector<Ghosts<R>> gm(K), gd(K);
    for (int k = 0; k < K; ++k) {
      gm[k] = ghosts_of(ghm, km.d, ghostK, k, K);
      gd[k] = p.has_torque ? ghosts_of(ghd, kd.d, ghostK + 2, k, K) : ghd;
      spread_into<RF>(F + k * col, torque ? T + k * col : nullptr, gK + k * gcol, gm[k], gd[k], s);
    }
    exec_fwd(gK, sK, s, 3 * (int64_t)nz * K, planK_f);
    EpiArgs ef;
    memset(&ef, 0, sizeof(ef));
    ef.inverse = 0;
    ef.scale = 1.0;
    ef.ks = ks;
    for (int k = 0; k < K; ++k) DPST_CUDA(zgemm((R *)(sK + k * scol), Tf.as<R>(), ef, false, s));
    if (dfsolve) {
      // the K columns' modes interleaved wavenumber-major (shared factor reads)
      DPST_CUDA(launch_bvp_df_cols<R>(ks, reinterpret_cast<R *>(sK), 2 * (int64_t)scol,
                                      corr.p ? corrK.as<double2>() : nullptr,
                                      corrf.p ? corrfK.as<float2>() : nullptr, 16 * (int64_t)nk, K,
                                      bvpK_scratch.as<float2>(), bvpK_grid, df_variant, s));
      DPST_CUDA(launch_bvp_k0_b<R>(sysK.as<SysK<R>>(), K, s));
    } else {
      DPST_CUDA(launch_bvp_b<R>(sysK.as<SysK<R>>(), K, mprefK.as<int64_t>(), (int64_t)K * nk, nz,
                                bvpK_scratch.as<double>(), bvpK_grid, s));
    }
    for (int k = 0; k < K; ++k) {
      EpiArgs eb = ef;
      eb.inverse = 1;
      eb.scale = 1.0 / ((double)nx * (double)ny);
      epi_corr(eb);
      if (eb.corr) eb.corr = corrK.as<double2>() + (size_t)k * 16 * nk;
      if (eb.corrf) eb.corrf = corrfK.as<float2>() + (size_t)k * 16 * nk;
      DPST_CUDA(zgemm((R *)(sK + k * scol), Ti.as<R>(), eb, true, s));
    }
    exec_inv(sK, gK, s, 3 * (int64_t)nz * K, planK_b);
    for (int k = 0; k < K; ++k)
      interp_from<RF>(gK + k * gcol, gm[k], gd[k], torque, V + k * col, W ? W + k * col : nullptr, s);
  }

  void mdot_multi(int K, const void *F, const void *T, void *V, void *W, int dtype, cudaStream_t s) override {
    if (!positioned) throw Error(DPST_ERR_NOT_READY, "positions have not been set");
    if (K < 1) throw Error(DPST_ERR_INVALID_ARG, "K must be at least 1");
    if (N == 0) return;
    if (F == nullptr || V == nullptr) throw Error(DPST_ERR_INVALID_ARG, "F and V must not be NULL");
    if (reg) {  // one Mdot per column
      if (dtype != DPST_F64 && dtype != DPST_F32)
        throw Error(DPST_ERR_INVALID_ARG, "dtype must be DPST_F64 or DPST_F32");
      const size_t col = 3 * (size_t)N * (dtype == DPST_F64 ? 8 : 4);
      for (int k = 0; k < K; ++k)
        mdot((const char *)F + k * col, T ? (const char *)T + k * col : nullptr, (char *)V + k * col,
             W ? (char *)W + k * col : nullptr, dtype, s);
      return;
    }
    if (dtype == DPST_F64)
      run_multi<double>(K, (const double *)F, (const double *)T, (double *)V, (double *)W, s);
    else if (dtype == DPST_F32)
      run_multi<float>(K, (const float *)F, (const float *)T, (float *)V, (float *)W, s);
    else
      throw Error(DPST_ERR_INVALID_ARG, "dtype must be DPST_F64 or DPST_F32");
  }

  // ---- backward pass -------------------------------------------------------
  // Buffers are allocated on the first backward call: the adjoint grid, the
  // adjoint solve's scratch, the transposed DCT matrices, the position
  // derivatives of the stencils and the adjoint ghost layers.
  DevBuf grid2, adj_scratch, TfTn, TiT;
  int64_t adj_grid = 0;
  DevBuf gs_m[4], gs_d[8];
  GradStencils<R> gsm, gsd;
  DevBuf gha_m[2], gha_d[2];
  Ghosts<R> gham, ghad;
  bool grad_ready = false;

  // The double-float adjoint's kernel variant, timed like the forward's on
  // the spectrum buffer (FP32 spectra; DPSTOKES_GB300_SOLVE_VARIANT fixes it)
  int adj_variant = 1;
  float adj_ms[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  void tune_adjoint() {
    if (sizeof(R) != 4) return;
    const char *env = getenv("DPSTOKES_GB300_SOLVE_VARIANT");
    if (env && *env) {
      adj_variant = atoi(env);
      return;
    }
    cudaEvent_t a, b;
    DPST_CUDA(cudaEventCreate(&a));
    DPST_CUDA(cudaEventCreate(&b));
    float best = 0.0f;
    for (int v = 0; v < bvp_df_variants(); ++v) {
      auto run = [&] {
        DPST_CUDA(launch_adj_df<R>(ks, spec.as<R>(), corr.as<double2>(), adj_scratch.as<float2>(), adj_grid, v, 0));
      };
      run();
      DPST_CUDA(cudaEventRecord(a, 0));
      for (int rep = 0; rep < 3; ++rep) run();
      DPST_CUDA(cudaEventRecord(b, 0));
      DPST_CUDA(cudaEventSynchronize(b));
      DPST_CUDA(cudaEventElapsedTime(&adj_ms[v], a, b));
      adj_ms[v] /= 3.0f;
      if (v == 0 || adj_ms[v] < best) {
        best = adj_ms[v];
        adj_variant = v;
      }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }

  void ensure_grad() {
    if (!grad_ready) {
      grid2.alloc(grid.bytes);
      size_t bytes = 0;
      if (dfsolve) {
        DPST_CUDA(bvp_adj_df_plan(ks, nsm, &adj_grid, &bytes));
      } else {
        DPST_CUDA(adj_plan<R>(ks, nsm, &adj_grid, &bytes));
      }
      adj_scratch.alloc(bytes);
      if (dfsolve) tune_adjoint();
      std::vector<double> tf, ti;
      dct_matrices(nz, tf, ti);
      const double sc = 1.0 / ((double)nx * (double)ny);
      std::vector<R> tft((size_t)nz * nz), tit((size_t)nz * nz);
      for (int r = 0; r < nz; ++r)
        for (int c = 0; c < nz; ++c) {
          tft[(size_t)r * nz + c] = (R)(tf[(size_t)c * nz + r] * sc);
          tit[(size_t)r * nz + c] = (R)ti[(size_t)c * nz + r];
        }
      upload(TfTn, tft);
      upload(TiT, tit);
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
    // adjoint ghost layers mirror the forward's (which depend on positions)
    auto mirror = [&](const Ghosts<R> &f, const KernelDesc &d, DevBuf *b, Ghosts<R> &a) {
      const size_t lev = sizeof(R) * (size_t)d.nyeff * d.nxeff * 3;
      a = f;
      if (f.top) {
        if (b[0].bytes < lev * f.ntop) b[0].alloc(lev * f.ntop);
        a.top = b[0].as<R>();
      }
      if (f.bot) {
        if (b[1].bytes < lev * f.nbot) b[1].alloc(lev * f.nbot);
        a.bot = b[1].as<R>();
      }
    };
    mirror(ghm, km.d, gha_m, gham);
    if (p.has_torque) mirror(ghd, kd.d, gha_d, ghad);
    else memset(&ghad, 0, sizeof(ghad));
  }

  // adjoint grid -> psi = L^T (adjoint grid), in place in grid2
  void adjoint_solve_stage(cudaStream_t s) {
    R *g2 = grid2.as<R>();
    CR *sp = spec.as<CR>();
    exec_fwd(g2, sp, s);
    if (p.mode != DPST_MODE_NOWALL) DPST_CUDA(launch_corr_adj<R>(ks, (const R *)sp, corr.as<double2>(), s));
    EpiArgs e;
    memset(&e, 0, sizeof(e));
    e.inverse = 0;
    e.scale = 1.0;
    e.ks = ks;
    DPST_CUDA(zgemm((R *)sp, TiT.as<R>(), e, false, s));
    if (dfsolve) {
      DPST_CUDA(launch_adj_df<R>(ks, (R *)sp, corr.as<double2>(), adj_scratch.as<float2>(), adj_grid, adj_variant,
                                 s));
      DPST_CUDA(launch_adj_k0<R>(ks, (R *)sp, s));
    } else {
      DPST_CUDA(launch_adj_solve<R>(ks, (R *)sp, corr.as<double2>(), adj_scratch.as<double>(), adj_grid, s));
    }
    DPST_CUDA(zgemm((R *)sp, TfTn.as<R>(), e, true, s));
    exec_inv(sp, g2, s);
  }

  template <typename RF>
  void run_backward(const RF *F, const RF *T, const RF *gV, const RF *gW, RF *gF, RF *gT, RF *gX,
                    cudaStream_t s) {
    const bool torque = p.has_torque && T != nullptr;
    const bool want_x = gX != nullptr;
    ensure_grad();
    R *gr = grid.as<R>(), *g2 = grid2.as<R>();
    Ghosts<R> none;
    memset(&none, 0, sizeof(none));
    // the dipole interpolation reads ghost layers only when torques were spread
    const Ghosts<R> &ghd_u = torque ? ghd : none;
    const Ghosts<R> &ghd_a = torque ? ghad : none;
    if (want_x) {
      launch_locate_grad<R>(false, pos64.as<double>(), N, km.d, zext.as<double>(), wext.as<double>(), g, stm,
                            gsm, s);
      if (p.has_torque)
        launch_locate_grad<R>(true, pos64.as<double>(), N, kd.d, zext.as<double>(), wext.as<double>(), g, std_,
                              gsd, s);
      // velocity grid and ghost layers of the forward, recomputed unless the
      // handle still holds that forward's
      if (!reuse_forward) {
        spread_stage<RF>(F, T, s);
        solve_stage(s);
      }
    }
    // adjoint source J^T (gV, gW) on grid2 and the adjoint ghost layers
    DPST_CUDA(cudaMemsetAsync(g2, 0, grid2.bytes, s));
    for (Ghosts<R> *gh : {&gham, &ghad}) {
      const KernelDesc &d = (gh == &gham) ? km.d : kd.d;
      const size_t lev = (size_t)d.nyeff * d.nxeff * 3 * sizeof(R);
      if (gh->top) DPST_CUDA(cudaMemsetAsync(gh->top, 0, lev * gh->ntop, s));
      if (gh->bot) DPST_CUDA(cudaMemsetAsync(gh->bot, 0, lev * gh->nbot, s));
    }
    Stencils<R> sw = stm;
    sw.phz = stm.phzw;  // the interpolation's weights
    launch_spread<R, RF>(false, gV, N, km.d, g, sw, g2, gham, s, perm.as<int>());
    if (gW) launch_adj_spread_dip<R, RF>(gW, N, kd.d, g, std_, g2, ghd_a, s);
    launch_ghost_fold_t<R>(gham.top, gham.ntop, nx, ny, km.d, s);
    launch_ghost_fold_t<R>(gham.bot, gham.nbot, nx, ny, km.d, s);
    if (torque) {
      launch_ghost_fold_t<R>(ghad.top, ghad.ntop, nx, ny, kd.d, s);
      launch_ghost_fold_t<R>(ghad.bot, ghad.nbot, nx, ny, kd.d, s);
    }
    DPST_CUDA(cudaGetLastError());
    adjoint_solve_stage(s);
    // gathers: S^T psi and the position gradient
    if (gF || want_x)
      launch_gather_mono<R, RF>(want_x ? gr : nullptr, g2, N, km.d, g, stm, gsm, ghm, gham, F, gV, gF, gX, s);
    if (p.has_torque && (gT || (want_x && (torque || gW))))
      launch_gather_dip<R, RF>(want_x ? gr : nullptr, g2, N, kd.d, g, std_, gsd, ghd_u, ghd_a,
                               torque ? T : nullptr, gW, gT, gX, s);
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
    if (gW != nullptr && !p.has_torque)
      throw Error(DPST_ERR_INVALID_ARG, "gW needs an operator created with torques");
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

  void info(dpst_info *o) const override {
    memset(o, 0, sizeof(*o));
    o->nxh = nxh;
    o->n_modes = (int)nk;
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
    // spread (mono [+ dip]), ghost folds (2 kernels per buffer in use),
    // forward z GEMM, BVP pairs + k=0, inverse z GEMM, interp (mono [+ dip])
    int nbuf = (ghm.top != nullptr) + (ghm.bot != nullptr) + (ghd.top != nullptr) + (ghd.bot != nullptr);
    o->ghost_layers_in_use = nbuf;
    o->ztransform = ztc[0];
    o->ztransform_ms[0] = ztc_ms[0][0];
    o->ztransform_ms[1] = ztc_ms[0][1];
    o->ztransform_inverse = ztc[1];
    o->ztransform_inverse_ms[0] = ztc_ms[1][0];
    o->ztransform_inverse_ms[1] = ztc_ms[1][1];
    const int particle_passes = (p.has_torque && !fused) ? 2 : 1;
    o->kernels_per_mdot = particle_passes + 2 * nbuf + 1 + 2 + 1 + particle_passes;
    // regular-kernel torques: + the torques' forward z transform and curl, the
    // vorticity's forward z transform, curl and inverse z transform
    if (reg) o->kernels_per_mdot += (p.mode == DPST_MODE_NOWALL) ? 4 : 5;
    o->fused_particle_passes = fused ? 1 : 0;
    o->solve_arith = dfsolve ? DPST_SOLVE_DF64 : DPST_SOLVE_FP64;
    o->solve_variant = dfsolve ? df_variant : 0;
    o->xy_transform = ownfft ? (xycl ? 4 : xyfused ? 2 : 1) : (ownfft_d ? 3 : 0);
    o->xy_cluster_ms = xycl_ms;
    o->spread_tiles = (tile_spread && p.has_torque) ? 1 : 0;
    o->xy_ms[0] = sizeof(R) == 8 ? xyd_ms[0] : xy_ms[0];
    o->xy_ms[1] = sizeof(R) == 8 ? xyd_ms[1] : xy_ms[1];
    o->ztransform_tma_ms[0] = ztm_ms[0];
    o->ztransform_tma_ms[1] = ztm_ms[1];
    for (int d = 0; d < 2; ++d) {
      o->ztransform_tma_variant[d] = ztm_var[d];
      for (int v = 0; v < 3; ++v) o->ztransform_tma_variant_ms[3 * d + v] = ztm_vms[d][v];
    }
    if (ownfft || ownfft_d) o->kernels_per_mdot += (xyfused || xycl ? 2 : 4) * (reg && p.has_torque ? 2 : 1);
    if (sizeof(R) == 4 && ztc[1] && p.mode != DPST_MODE_NOWALL) o->kernels_per_mdot += 1;  // correction pass
    for (int v = 0; v < 4; ++v) o->solve_ms[v] = df_ms[v];
    int64_t b = 0;
    const DevBuf *all[] = {&bvp_scratch, &grid, &spec, &corr, &zext, &wext, &kvx, &kvy, &zn, &bands, &bcrows,
                           &k0rows, &Tf, &Ti, &fac_m, &fac_i, &fac_d, &fac_a0, &fac_a1, &fac_c0, &fac_c1, &fac_pm, &fac_pb, &fac_pa,
                           &fac_g, &pos64, &flags, &dphzw_buf, &ord_count, &ord_start, &perm,
                           &corrf, &cmode, &znf, &gridT, &specT, &df_mf, &df_bk, &df_ab, &df_gi, &df_km,
                           &df_dx, &df_dy, &bvp_df_scratch, &twx, &twy};
    for (const DevBuf *d : all) b += d->bytes;
    for (int i = 0; i < 8; ++i) b += st_m[i].bytes + st_d[i].bytes;
    for (int i = 0; i < 2; ++i) b += gh_m[i].bytes + gh_d[i].bytes;
    o->device_bytes = b;
  }
};

// positions -> FP64 [N][3] with z relative to zmin
template <typename RP>
__global__ void k_prep_pos(const RP *pos, int64_t N, double zmin, double *out) {
  int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= N) return;
  out[3 * p] = (double)pos[3 * p];
  out[3 * p + 1] = (double)pos[3 * p + 1];
  out[3 * p + 2] = (double)pos[3 * p + 2] - zmin;
}

void launch_prep_positions(const void *pos, int dtype, int64_t N, double zmin, double *out, cudaStream_t s) {
  int bs = 256;
  int64_t nb = (N + bs - 1) / bs;
  if (N == 0) return;
  if (dtype == DPST_F64) k_prep_pos<double><<<nb, bs, 0, s>>>((const double *)pos, N, zmin, out);
  else if (dtype == DPST_F32) k_prep_pos<float><<<nb, bs, 0, s>>>((const float *)pos, N, zmin, out);
  else throw Error(DPST_ERR_INVALID_ARG, "dtype must be DPST_F64 or DPST_F32");
  DPST_CUDA(cudaGetLastError());
}

template <typename R>
void Engine<R>::convert_positions(const void *pos, int dtype, cudaStream_t s) {
  launch_prep_positions(pos, dtype, N, p.zmin, pos64.as<double>(), s);
}



}  // namespace dpst

struct dpst_engine {
  std::unique_ptr<dpst::EngineBase> e;
  // device staging for the host-array entry points
  void *dpos = nullptr, *dF = nullptr, *dT = nullptr, *dV = nullptr, *dW = nullptr;
  ~dpst_engine() {
    for (void *q : {dpos, dF, dT, dV, dW})
      if (q) cudaFree(q);
  }
};

using dpst::Error;

using dpst::guarded;

extern "C" {

const char *dpst_version(void) { return "dpstokes_gb300 0.1"; }

const char *dpst_last_error(void) { return dpst::g_last_error.c_str(); }

int dpst_create(const dpst_params *p, int64_t n_particles, int device, dpst_handle *out) {
  return guarded([&] {
    if (!out) throw Error(DPST_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    dpst::validate(p, n_particles, true);
    std::unique_ptr<dpst_engine> h(new dpst_engine());
    if (p->mode == DPST_MODE_PERIODIC) h->e.reset(dpst::make_engine_tp(*p, n_particles, device));
    else if (p->precision == DPST_PREC_FP64) h->e.reset(new dpst::Engine<double>(*p, n_particles, device));
    else h->e.reset(new dpst::Engine<float>(*p, n_particles, device));
    *out = h.release();
  });
}

int dpst_destroy(dpst_handle h) {
  return guarded([&] { delete h; });
}

// Forward bookkeeping (EngineBase::serial, grid_serial): a call that moves
// the particles or overwrites the velocity grid with anything but a
// single-column Mdot's result forgets the held grid; a single-column Mdot
// records itself as the holder once it has completed its launches.
static void grid_forget(dpst::EngineBase *e) {
  ++e->serial;
  e->grid_serial = 0;
}
static void grid_hold(dpst::EngineBase *e) { e->grid_serial = ++e->serial; }

int dpst_set_positions(dpst_handle h, const void *pos, int dtype, void *stream) {
  return guarded([&] {
    if (!h) throw Error(DPST_ERR_INVALID_ARG, "handle is NULL");
    DPST_CUDA(cudaSetDevice(h->e->device));
    grid_forget(h->e.get());
    h->e->set_positions(pos, dtype, (cudaStream_t)stream);
  });
}

int dpst_mdot(dpst_handle h, const void *F, const void *T, void *V, void *W, int dtype, void *stream) {
  return guarded([&] {
    if (!h) throw Error(DPST_ERR_INVALID_ARG, "handle is NULL");
    DPST_CUDA(cudaSetDevice(h->e->device));
    grid_forget(h->e.get());
    h->e->mdot(F, T, V, W, dtype, (cudaStream_t)stream);
    grid_hold(h->e.get());
  });
}

int dpst_forward_serial(dpst_handle h, uint64_t *out) {
  return guarded([&] {
    if (!h || !out) throw Error(DPST_ERR_INVALID_ARG, "NULL argument");
    *out = h->e->grid_serial;
  });
}

int dpst_mdot_multi(dpst_handle h, int K, const void *F, const void *T, void *V, void *W, int dtype,
                    void *stream) {
  return guarded([&] {
    if (!h) throw Error(DPST_ERR_INVALID_ARG, "handle is NULL");
    DPST_CUDA(cudaSetDevice(h->e->device));
    grid_forget(h->e.get());
    h->e->mdot_multi(K, F, T, V, W, dtype, (cudaStream_t)stream);
  });
}

static size_t elem_size(int dtype) {
  if (dtype == DPST_F64) return 8;
  if (dtype == DPST_F32) return 4;
  throw Error(DPST_ERR_INVALID_ARG, "dtype must be DPST_F64 or DPST_F32");
}

int dpst_set_positions_host(dpst_handle h, const void *pos, int dtype, void *stream) {
  return guarded([&] {
    if (!h) throw Error(DPST_ERR_INVALID_ARG, "handle is NULL");
    if (!pos) throw Error(DPST_ERR_INVALID_ARG, "positions pointer is NULL");
    DPST_CUDA(cudaSetDevice(h->e->device));
    const size_t bytes = 3 * (size_t)h->e->N * 8;
    if (!h->dpos && bytes) DPST_CUDA(cudaMalloc(&h->dpos, bytes));
    cudaStream_t s = (cudaStream_t)stream;
    const size_t b = 3 * (size_t)h->e->N * elem_size(dtype);
    if (b) DPST_CUDA(cudaMemcpyAsync(h->dpos, pos, b, cudaMemcpyHostToDevice, s));
    grid_forget(h->e.get());
    h->e->set_positions(h->dpos, dtype, s);
  });
}

int dpst_mdot_host(dpst_handle h, const void *F, const void *T, void *V, void *W, int dtype, void *stream) {
  return guarded([&] {
    if (!h) throw Error(DPST_ERR_INVALID_ARG, "handle is NULL");
    if (!F || !V) throw Error(DPST_ERR_INVALID_ARG, "F and V must not be NULL");
    DPST_CUDA(cudaSetDevice(h->e->device));
    const size_t b = 3 * (size_t)h->e->N * elem_size(dtype);
    const size_t cap = 3 * (size_t)h->e->N * 8;
    cudaStream_t s = (cudaStream_t)stream;
    if (cap) {
      for (void **q : {&h->dF, &h->dT, &h->dV, &h->dW})
        if (!*q) DPST_CUDA(cudaMalloc(q, cap));
      DPST_CUDA(cudaMemcpyAsync(h->dF, F, b, cudaMemcpyHostToDevice, s));
      if (T) DPST_CUDA(cudaMemcpyAsync(h->dT, T, b, cudaMemcpyHostToDevice, s));
    }
    grid_forget(h->e.get());
    h->e->mdot(h->dF, T ? h->dT : nullptr, h->dV, W ? h->dW : nullptr, dtype, s);
    grid_hold(h->e.get());
    if (cap) {
      DPST_CUDA(cudaMemcpyAsync(V, h->dV, b, cudaMemcpyDeviceToHost, s));
      if (W) DPST_CUDA(cudaMemcpyAsync(W, h->dW, b, cudaMemcpyDeviceToHost, s));
    }
    DPST_CUDA(cudaStreamSynchronize(s));
  });
}

int dpst_spread_grid(dpst_handle h, const void *F, const void *T, int dtype, void *grid_out, void *stream) {
  return guarded([&] {
    if (!h) throw Error(DPST_ERR_INVALID_ARG, "handle is NULL");
    DPST_CUDA(cudaSetDevice(h->e->device));
    grid_forget(h->e.get());
    h->e->spread_grid(F, T, dtype, grid_out, (cudaStream_t)stream);
  });
}

int dpst_velocity_grid(dpst_handle h, void *grid_out, void *stream) {
  return guarded([&] {
    if (!h) throw Error(DPST_ERR_INVALID_ARG, "handle is NULL");
    DPST_CUDA(cudaSetDevice(h->e->device));
    h->e->velocity_grid(grid_out, (cudaStream_t)stream);
  });
}

int dpst_mdot_timed(dpst_handle h, const void *F, const void *T, void *V, void *W, int dtype, void *stream,
                    float *stage_ms) {
  return guarded([&] {
    if (!h || !stage_ms) throw Error(DPST_ERR_INVALID_ARG, "NULL argument");
    DPST_CUDA(cudaSetDevice(h->e->device));
    h->e->stage_ms = stage_ms;
    grid_forget(h->e.get());
    try {
      h->e->mdot(F, T, V, W, dtype, (cudaStream_t)stream);
    } catch (...) {
      h->e->stage_ms = nullptr;
      throw;
    }
    h->e->stage_ms = nullptr;
    grid_hold(h->e.get());
  });
}

int dpst_mdot_noalloc(dpst_handle h, const void *F, const void *T, void *V, void *W, int dtype, void *stream) {
  return guarded([&] {
    if (!h) throw Error(DPST_ERR_INVALID_ARG, "handle is NULL");
    DPST_CUDA(cudaSetDevice(h->e->device));
    h->e->use_static_scratch = true;
    grid_forget(h->e.get());
    try {
      h->e->mdot(F, T, V, W, dtype, (cudaStream_t)stream);
    } catch (...) {
      h->e->use_static_scratch = false;
      throw;
    }
    h->e->use_static_scratch = false;
    grid_hold(h->e.get());
  });
}

int dpst_mdot_backward(dpst_handle h, const void *F, const void *T, const void *gV, const void *gW, void *gF,
                       void *gT, void *gX, int dtype, void *stream) {
  return guarded([&] {
    if (!h) throw Error(DPST_ERR_INVALID_ARG, "handle is NULL");
    DPST_CUDA(cudaSetDevice(h->e->device));
    grid_forget(h->e.get());  // a position gradient recomputes the velocity grid from these F, T
    h->e->backward(F, T, gV, gW, gF, gT, gX, dtype, (cudaStream_t)stream);
  });
}

int dpst_mdot_backward_saved(dpst_handle h, uint64_t forward_serial, const void *F, const void *T, const void *gV,
                             const void *gW, void *gF, void *gT, void *gX, int dtype, void *stream, int *reused) {
  return guarded([&] {
    if (!h) throw Error(DPST_ERR_INVALID_ARG, "handle is NULL");
    DPST_CUDA(cudaSetDevice(h->e->device));
    const bool reuse = forward_serial != 0 && forward_serial == h->e->grid_serial;
    if (reused) *reused = reuse ? 1 : 0;
    if (!reuse) grid_forget(h->e.get());
    h->e->reuse_forward = reuse;
    try {
      h->e->backward(F, T, gV, gW, gF, gT, gX, dtype, (cudaStream_t)stream);
    } catch (...) {
      h->e->reuse_forward = false;
      grid_forget(h->e.get());
      throw;
    }
    h->e->reuse_forward = false;
  });
}

int dpst_get_info(dpst_handle h, dpst_info *out) {
  return guarded([&] {
    if (!h || !out) throw Error(DPST_ERR_INVALID_ARG, "NULL argument");
    h->e->info(out);
  });
}

int dpst_xy_transform(int nx, int ny, int64_t planes, void *in, void *out, int inverse, int form, int device,
                      void *stream) {
  return guarded([&] {
    if (!in || !out || planes < 1) throw Error(DPST_ERR_INVALID_ARG, "NULL argument or no planes");
    if (form != 0 && form != 1 && form != 2)
      throw Error(DPST_ERR_INVALID_ARG, "form must be 0 (two passes), 1 (one launch) or 2 (clusters)");
    if (!dpst::own_fft_supported(nx, ny))
      throw Error(DPST_ERR_UNSUPPORTED, "the library's x-y transforms take powers of two, 64 <= nx <= 2048, "
                                        "32 <= ny <= 1024");
    if (form == 1 && !dpst::fft_xy_fused_supported(nx, ny))
      throw Error(DPST_ERR_UNSUPPORTED, "the one-launch x-y transform takes nx = ny in 128, 256, 512, 1024");
    if (form == 2 && !dpst::fft_xy_cluster_supported(nx, ny))
      throw Error(DPST_ERR_UNSUPPORTED, "the cluster x-y transform takes nx = ny in 256, 512");
    DPST_CUDA(cudaSetDevice(device));
    cudaStream_t s = (cudaStream_t)stream;
    dpst::DevBuf twx, twy;
    dpst::upload(twx, dpst::fft_twiddles(nx));
    dpst::upload(twy, dpst::fft_twiddles(ny));
    DPST_CUDA(dpst::fft_setup(nx, ny));
    const int nxh = nx / 2 + 1;
    if (form == 2) {
      int grid = 0;
      DPST_CUDA(dpst::fft_xy_cluster_setup(nx, ny, &grid));
      if (grid <= 0) throw Error(DPST_ERR_UNSUPPORTED, "the cluster x-y transform cannot be resident on this device");
      dpst::DevBuf err;
      err.alloc(sizeof(int));
      DPST_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
      if (!inverse)
        DPST_CUDA(dpst::fft_xy_cluster(false, (const float *)in, (float2 *)out, nullptr, nx, ny, planes,
                                       twx.as<float2>(), twy.as<float2>(), err.as<int>(), grid, s));
      else
        DPST_CUDA(dpst::fft_xy_cluster(true, nullptr, (float2 *)in, (float *)out, nx, ny, planes, twx.as<float2>(),
                                       twy.as<float2>(), err.as<int>(), grid, s));
      int word = 0;
      DPST_CUDA(cudaMemcpyAsync(&word, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
      DPST_CUDA(cudaStreamSynchronize(s));
      if (word != 0) throw Error(DPST_ERR_CUDA, "cluster x-y transform: a wait gave up");
      return;
    }
    if (form == 1) {
      int grid = 0;
      DPST_CUDA(dpst::fft_xy_setup(nx, ny, &grid));
      dpst::DevBuf ctr;
      ctr.alloc(sizeof(int) * dpst::fft_xy_counter_ints(planes));
      DPST_CUDA(cudaMemsetAsync(ctr.p, 0, sizeof(int) * dpst::fft_xy_counter_ints(planes), s));
      const int lag = dpst::xy_lag_setting();
      if (!inverse)
        DPST_CUDA(dpst::fft_xy_fused(false, (const float *)in, (float2 *)out, nullptr, nx, ny, planes,
                                     twx.as<float2>(), twy.as<float2>(), ctr.as<int>(), grid, lag, s));
      else
        DPST_CUDA(dpst::fft_xy_fused(true, nullptr, (float2 *)in, (float *)out, nx, ny, planes, twx.as<float2>(),
                                     twy.as<float2>(), ctr.as<int>(), grid, lag, s));
      int word[2] = {0, 0};
      DPST_CUDA(cudaMemcpyAsync(word, ctr.as<int>() + 1, sizeof(word), cudaMemcpyDeviceToHost, s));
      DPST_CUDA(cudaStreamSynchronize(s));
      if (word[1] != 0) throw Error(DPST_ERR_CUDA, "one-launch x-y transform: a wait gave up");
      if (word[0] != 0) throw Error(DPST_ERR_CUDA, "one-launch x-y transform: counters not reset");
      return;
    }
    if (!inverse) {
      DPST_CUDA(dpst::fft_rows(false, (const float *)in, (float2 *)out, nullptr, nullptr, nx, planes * ny,
                               twx.as<float2>(), s));
      DPST_CUDA(dpst::fft_cols(false, (float2 *)out, ny, nxh, planes, twy.as<float2>(), s));
    } else {
      DPST_CUDA(dpst::fft_cols(true, (float2 *)in, ny, nxh, planes, twy.as<float2>(), s));
      DPST_CUDA(dpst::fft_rows(true, nullptr, nullptr, (const float2 *)in, (float *)out, nx, planes * ny,
                               twx.as<float2>(), s));
    }
    DPST_CUDA(cudaStreamSynchronize(s));
  });
}

}  // extern "C"
