// Declarations shared by the host engines (dpst_engine.cu: the doubly
// periodic geometries, dpst_tp.cu: the triply periodic mode): the engine
// interface behind the C ABI and the launchers of the particle kernels
// (dpst_particles.cu).
#pragma once
#include <cuda_runtime.h>

#include "../../include/dpstokes_gb300.h"
#include "dpst_internal.cuh"

namespace dpst {

// One operator handle: the C ABI entry points call these.
struct EngineBase {
  virtual ~EngineBase() {}
  virtual void set_positions(const void *pos, int dtype, cudaStream_t s) = 0;
  virtual void mdot(const void *F, const void *T, void *V, void *W, int dtype, cudaStream_t s) = 0;
  virtual void mdot_multi(int K, const void *F, const void *T, void *V, void *W, int dtype, cudaStream_t s) = 0;
  bool use_static_scratch = false;  // set by dpst_mdot_noalloc for one call
  virtual void info(dpst_info *o) const = 0;
  virtual void spread_grid(const void *F, const void *T, int dtype, void *out, cudaStream_t s) = 0;
  virtual void velocity_grid(void *out, cudaStream_t s) = 0;
  virtual void backward(const void *F, const void *T, const void *gV, const void *gW, void *gF, void *gT,
                        void *gX, int dtype, cudaStream_t s) = 0;
  float *stage_ms = nullptr;  // set by dpst_mdot_timed for one call
  // Forward bookkeeping for dpst_mdot_backward_saved: `serial` counts the
  // calls that change positions or the velocity grid; `grid_serial` is the
  // serial of the single-column Mdot whose velocity grid (and open-end ghost
  // layers) the handle still holds, 0 if none; `reuse_forward` is set for
  // one backward call that takes that grid instead of recomputing it.
  uint64_t serial = 0, grid_serial = 0;
  bool reuse_forward = false;
  int device = 0;
  int64_t N = 0;
  dpst_params p;
};

// triply periodic operator (dpst_tp.cu)
EngineBase *make_engine_tp(const dpst_params &p, int64_t n, int device);

// positions (FP64 or FP32, [N][3]) -> FP64 [N][3] with z relative to zmin
void launch_prep_positions(const void *pos, int dtype, int64_t N, double zmin, double *out, cudaStream_t s);

template <typename R>
void launch_locate(bool dipole, const double *pos, int64_t N, const KernelDesc &kd, const double *zext,
                   const double *wext, const GridArgs &g, const Stencils<R> &st, int *err, int *reach,
                   cudaStream_t s);
template <typename R, typename RF>
void launch_spread(bool dipole, const RF *FT, int64_t N, const KernelDesc &kd, const GridArgs &g,
                   const Stencils<R> &st, R *grid, const Ghosts<R> &gh, cudaStream_t s, const int *perm = nullptr);
template <typename R>
void launch_tile_order(int64_t N, const GridArgs &g, const Stencils<R> &st, int *count, int *start, int *perm,
                       cudaStream_t s);
size_t tile_order_tiles(int nx, int ny);
bool fused_supports(const KernelDesc &km, const KernelDesc &kd);
template <typename R, typename RF>
void launch_spread_fused(const RF *F, const RF *T, int64_t N, const KernelDesc &km, const KernelDesc &kd,
                         const GridArgs &g, const Stencils<R> &sm, const Stencils<R> &sd, R *grid,
                         const Ghosts<R> &ghm, const Ghosts<R> &ghd, cudaStream_t s, const int *perm);
template <typename R, typename RV>
void launch_interp_fused(const R *grid, int64_t N, const KernelDesc &km, const KernelDesc &kd, const GridArgs &g,
                         const Stencils<R> &sm, const Stencils<R> &sd, const Ghosts<R> &ghm,
                         const Ghosts<R> &ghd, RV *V, RV *W, cudaStream_t s, const int *perm);
template <typename R>
void launch_ghost_fold(R *buf, int levels, int nx, int ny, const KernelDesc &kd, cudaStream_t s);
template <typename R, typename RV>
void launch_interp(bool dipole, const R *grid, int64_t N, const KernelDesc &kd, const GridArgs &g,
                   const Stencils<R> &st, const Ghosts<R> &gh, RV *out, cudaStream_t s, const int *perm = nullptr);

}  // namespace dpst
