/*
 * dpstokes_gb300.h -- C ABI of the GB300 doubly periodic Stokes mobility
 * operator (libdpstokes_gb300.so).
 *
 * Computes [V; W] = M [F; T] for N blobs with exponential-of-semicircle (ES)
 * kernels in a domain periodic in x, y and open (no wall), bounded below by a
 * no-slip wall, or bounded by two no-slip walls in z, or periodic in z too
 * (triply periodic).  Forces F, torques T, linear velocities V and angular
 * velocities W are [N][3] arrays.
 *
 * Drop-in boundary.  Each entry point replaces one call of the reference's
 * interface for this path (paths are within stochasticHydroTools/
 * DoublyPeriodicStokes):
 *   dpst_create        <- DPStokesGlue::initialize(PyParameters, int)
 *                         (source/gpu/python_wrapper/uammd_interface.h:44-52,
 *                          uammd_wrapper.cu:182-184) and, on the CPU path,
 *                         FCM.Initialize (source/cpu/python/FCM.py:149-268)
 *   dpst_destroy       <- DPStokesGlue::clear (uammd_interface.h:54-56,
 *                         uammd_wrapper.cu:188-191) / FCM.Clean (FCM.py:443)
 *   dpst_set_positions <- DPStokesGlue::setPositions(const real*)
 *                         (uammd_interface.h:58, uammd_wrapper.cu:136-143) /
 *                         FCM.SetPositions (FCM.py:270-332)
 *   dpst_mdot          <- DPStokesGlue::Mdot(F, T|nullptr, MF, MT)
 *                         (uammd_interface.h:60-63, uammd_wrapper.cu:146-170) /
 *                         FCM.Mdot (FCM.py:334-441)
 *   dpst_*_host        <- the same calls with host arrays, copied in and out on
 *                         every call as the reference glue does
 *                         (uammd_wrapper.cu:139-169)
 *   dpst_spread_grid,  <- the reference's grid accessors GetData / CopyData
 *   dpst_velocity_grid    (source/cpu/wrapper/GridWrapper.cpp:66-67), used by
 *                         FCM.Mdot to hand the spread grid to the transform and
 *                         the velocity grid to the interpolation (FCM.py:356,406)
 *   dpst_mdot_timed    <- the stage-timed Mdot of the reference's benchmark
 *                         (source/cpu/examples/mobility_bench.py:311-442)
 *   dpst_last_error    <- replaces the C++ exceptions / exit(1) of the
 *                         reference (uammd_wrapper.cu:106,208-211,
 *                         source/cpu/include/exceptions.h:30-34)
 *
 * Conventions
 *   - Every function returns DPST_OK (0) or an error code; on error
 *     dpst_last_error() returns a message (thread-local).  Nothing throws.
 *   - Device pointers are CUDA device addresses on the handle's device;
 *     `stream` is a cudaStream_t (NULL = legacy default stream).  Device
 *     entry points are asynchronous with respect to the host except
 *     dpst_set_positions, which synchronises the stream once to report
 *     out-of-domain particles.
 *   - A handle is not thread-safe; separate handles are independent.
 *   - Positions: x in [0, Lx], y in [0, Ly] (periodic), z in [zmin, zmax].
 *   - Kernel: phi(r) = exp(beta (sqrt(1 - r^2/alpha^2) - 1)) per axis, with w
 *     grid points under it (alpha in physical units; the reference's
 *     UseCbeta convention gives alpha = w h / 2).  The dipole kernel
 *     (w_d, beta_d, alpha_d) spreads torques through the curl and
 *     interpolates the vorticity with kernel derivatives, as the reference
 *     CPU path does by default; torque_kernel = DPST_TORQUE_REG selects its
 *     regular-kernel coupling with spectral curls instead.
 */
#ifndef DPSTOKES_GB300_H
#define DPSTOKES_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* return codes */
#define DPST_OK 0
#define DPST_ERR_INVALID_ARG 1   /* bad parameter or pointer */
#define DPST_ERR_NOT_READY 2     /* positions not set */
#define DPST_ERR_OUT_OF_DOMAIN 3 /* a particle lies outside the unit cell */
#define DPST_ERR_CUDA 4          /* CUDA / cuFFT failure */
#define DPST_ERR_UNSUPPORTED 5   /* configuration the reference cannot run either */
#define DPST_ERR_ALLOC 6         /* device or host allocation failed */

/* geometry: reference domType DP / DPBW / DPSC / TP (FCM.py:211-229) */
#define DPST_MODE_NOWALL 0
#define DPST_MODE_BOTTOM 1
#define DPST_MODE_SLIT 2
#define DPST_MODE_PERIODIC 3 /* triply periodic: nz uniform points on the periodic
                                [zmin, zmax); the reference GPU module's mode
                                'periodic' (uammd_wrapper.cu:122-126) and CPU
                                domType 'TP' (TPTools.cpp:6-46).  dpst_create only
                                (no batched systems); multi-column Mdot runs column
                                by column */

/* arithmetic of the operator */
#define DPST_PREC_FP64 0  /* every stage in FP64: the drop-in for the reference */
#define DPST_PREC_MIXED 1 /* FP32 spread/FFT/interp, FP32 z transform, FP64 BVP
                             (PERIODIC: FP32 throughout; its solve is elementwise) */

/* torque coupling (has_torque) */
#define DPST_TORQUE_DERIV 0 /* derivative ES kernels spread the torque curl and interpolate the
                               velocity gradient: the reference's default (FCM.py:362-371,
                               411-426; useRegKernel = False) */
#define DPST_TORQUE_REG 1   /* regular ES kernel of the dipole's (w, beta, alpha) for torques and
                               angular velocities, curls taken spectrally (FCM.py:372-396,
                               427-439; useRegKernel = True).  dpst_create only: no batched
                               systems, no backward */

/* arithmetic of the per-wavenumber solve (dpst_params.solve_arith) */
#define DPST_SOLVE_DEFAULT 0 /* FP64 for DPST_PREC_FP64, double-float for DPST_PREC_MIXED */
#define DPST_SOLVE_FP64 1    /* FP64 on the FP64 pipe */
#define DPST_SOLVE_DF64 2    /* double-float: pairs of FP32 (about 48 significant bits, FP32's
                                exponent range) on the FP32 pipe, the same algorithm and factors
                                as the FP64 solve; the slit channel's wall-correction
                                coefficients stay FP64.  Open and wall geometries, single
                                handles, batched systems and multi-column Mdot; the triply
                                periodic mode has no such solve and dpst_mdot_noalloc runs
                                the FP64 one */

/* element type of the particle arrays passed to mdot */
#define DPST_F64 0
#define DPST_F32 1

typedef struct dpst_params {
  int mode;          /* DPST_MODE_* */
  int nx, ny, nz;    /* grid: nx*ny Fourier modes, nz Chebyshev points (PERIODIC:
                        nz uniform points, hz = (zmax - zmin) / nz) */
  double Lx, Ly;     /* periodic box */
  double zmin, zmax; /* Chebyshev interval; walls sit at zmin (bottom) / zmax (slit top);
                        PERIODIC: the periodic z box */
  double viscosity;
  int w;             /* monopole kernel: points per axis */
  double beta;       /* monopole ES beta (the reference's beta_hat * w) */
  double alpha;      /* monopole ES half width, physical units */
  int has_torque;    /* 1: torques in, angular velocities out */
  int w_d;           /* dipole kernel (used when has_torque) */
  double beta_d;
  double alpha_d;
  int precision;     /* DPST_PREC_* */
  int torque_kernel; /* DPST_TORQUE_* (0 when the initialiser stops before it) */
  int solve_arith;   /* DPST_SOLVE_* (0 when the initialiser stops before it) */
} dpst_params;

typedef struct dpst_info {
  int nxh;              /* nx/2 + 1 half-spectrum columns */
  int n_modes;          /* ny * nxh wavenumbers solved per Mdot */
  int nzeff_m, nzeff_d; /* extended z grid sizes (monopole, dipole) */
  int ghost_m, ghost_d; /* ghost layers per z end */
  int wz_max_m, wz_max_d;
  double thr_m, thr_d;  /* kernel truncation thresholds */
  double norm_m, norm_d;/* 1-D kernel integrals */
  int64_t device_bytes; /* device memory held by the handle */
  int64_t n_particles;
  int kernels_per_mdot; /* kernels of this library one dpst_mdot launches (with T
                           and W given); cuFFT kernels and memsets not counted */
  int ghost_layers_in_use; /* open-end ghost buffers the current positions need */
  int ztransform;          /* z-transform kernel chosen at creation for the forward
                              transform (and the backward's adjoint transforms): 0
                              FP32/FP64 SIMT (even/odd folded), 1 tcgen05 split-TF32
                              (mixed only), 2 double-float SIMT (FP64 operator), 3
                              tcgen05 split-TF32 fed by TMA (mixed, 32 <= nz <= 128,
                              an even number of modes) */
  float ztransform_ms[2];  /* creation-time timings of one transform: SIMT and the
                              alternative (tcgen05 with register-staged operands for
                              the mixed operator, double-float for the FP64 one); 0 if
                              not timed */
  int fused_particle_passes; /* 1: torques spread and interpolate in the same pass as
                                the forces (the dipole kernel's stencil columns and z
                                ghost extension equal the monopole's and its threshold
                                is not larger); 0: separate monopole / dipole passes */
  int ztransform_inverse;          /* kernel of the inverse z transform (with the wall-
                                      correction), chosen separately: 0 / 1 / 2 / 3 */
  float ztransform_inverse_ms[2];  /* its creation-time timings, as ztransform_ms */
  int z_fused;                     /* triply periodic: 1 when the z transform and the solve
                                      run in one kernel after 2-D x-y transforms (nz = 16,
                                      32, 64), 0 with cuFFT's 3-D transforms */
  int solve_arith;                 /* arithmetic of the per-wavenumber solve dpst_mdot runs:
                                      DPST_SOLVE_FP64 or DPST_SOLVE_DF64 (triply periodic: 0) */
  int solve_variant;               /* DPST_SOLVE_DF64 in the mixed operator: the kernel variant
                                      (prefetch depths, warps per SM) chosen at creation */
  float solve_ms[4];               /* its creation-time timings per variant (0 if not timed) */
  int xy_transform;                /* x-y transforms: the library's own in the mixed operator
                                      with power-of-two nx and ny, 1 as two passes (rows,
                                      columns), 2 as one launch of both passes (nx = ny in
                                      128, 256, 512, 1024, when faster at creation); 3 the
                                      FP64 operator's own double-float two passes (powers of
                                      two, nx <= 1024, ny <= 512, when faster than cuFFT);
                                      4 one launch of thread-block clusters, each plane held
                                      in the shared memory of 8 CTAs (nx = ny in 256, 512,
                                      when faster at creation); 0 cuFFT.
                                      DPSTOKES_GB300_XY_FFT=cufft | twopass | fused |
                                      cluster | own forces one */
  float xy_ms[2];                  /* creation-time timings of a forward + inverse pair:
                                      mixed: two-pass, one-launch; FP64: cuFFT, own
                                      double-float (0 if not timed) */
  int spread_tiles;                /* 1: the spread of forces and torques writes the grid once
                                      per 8 x 8-column tile from shared memory (mixed operator,
                                      fused kernel pair, DPSTOKES_GB300_SPREAD=tiles); 0: the grid
                                      is cleared and the contributions added with atomics (default,
                                      faster on the measured configurations) */
  float ztransform_tma_ms[2];      /* creation-time timings of the TMA-fed tcgen05 z transform,
                                      forward and inverse, its fastest variant (0 if not timed) */
  int ztransform_tma_variant[2];   /* that variant per direction: 0, 1, 2 = (TMA ring stages,
                                      converted operand stages) (6, 2), (4, 3), (7, 2) */
  float ztransform_tma_variant_ms[6]; /* every variant's timing, [direction][variant] */
  float xy_cluster_ms;             /* creation-time timing of the cluster form's forward +
                                      inverse pair (0 if not timed) */
} dpst_info;

typedef struct dpst_engine *dpst_handle;

/* Create an operator for n_particles on CUDA device `device`.  Plans FFTs,
 * precomputes the per-wavenumber BVP factors and allocates all buffers. */
int dpst_create(const dpst_params *p, int64_t n_particles, int device, dpst_handle *out);

/* Release everything the handle owns.  NULL is accepted. */
int dpst_destroy(dpst_handle h);

/* Positions: device array [N][3] of `dtype` (DPST_F64 or DPST_F32). */
int dpst_set_positions(dpst_handle h, const void *pos, int dtype, void *stream);

/* V = M_FF F + M_FT T, W = M_TF F + M_TT T.  F, V: device [N][3]; T, W
 * device [N][3] or NULL (no torques in / no angular velocities out).  All
 * four arrays have element type `dtype`. */
int dpst_mdot(dpst_handle h, const void *F, const void *T, void *V, void *W, int dtype,
              void *stream);

/* Multi-RHS Mdot: K force (and torque) columns at the current positions, as the
 * reference's mobility-matrix and Lanczos drivers apply M (mobility_matrix.py:5-48,
 * a loop of FCMJoint.Mdot calls there).  F, V: device [K][N][3]; T, W: device
 * [K][N][3] or NULL.  Column k equals dpst_mdot on column k (up to the order of
 * the spreading's atomic sums).  The K columns share the stencils and the
 * per-wavenumber factors; the x-y FFTs and the solve run once over all K.
 * Buffers for K columns are allocated on the first call with that K (or a
 * larger one). */
int dpst_mdot_multi(dpst_handle h, int K, const void *F, const void *T, void *V, void *W, int dtype,
                    void *stream);

/* Host-array variants: copy in, run, copy out, synchronise. */
int dpst_set_positions_host(dpst_handle h, const void *pos, int dtype, void *stream);
int dpst_mdot_host(dpst_handle h, const void *F, const void *T, void *V, void *W, int dtype,
                   void *stream);

/* Diagnostics.
 * dpst_spread_grid: run only the spreading stage (forces and, with T, the
 *   torque curl, with the boundary fold) and copy the resulting grid to the
 *   device buffer grid_out, layout [3][nz][ny][nx] (z index 0 at zmax; in the
 *   triply periodic mode z index 0 at zmin), element type double for
 *   DPST_PREC_FP64 and float for DPST_PREC_MIXED.  With DPST_TORQUE_REG the
 *   grid holds the forces only (the torque curl is added in wavenumber space).
 * dpst_velocity_grid: copy the fluid velocity on the grid from the last Mdot
 *   (same layout and type) to grid_out.
 * dpst_mdot_timed: dpst_mdot that also records CUDA events between stages and
 *   synchronises; stage_ms[0..7] receive the milliseconds of: zero + spread,
 *   forward x-y FFT, forward z transform, per-wavenumber solve, inverse z
 *   transform (+ wall correction), inverse x-y FFT, interpolation, total (in
 *   the triply periodic mode the transforms are 3-D, or 2-D with the z
 *   transform inside the solve, and the z-transform entries are ~0). */
int dpst_spread_grid(dpst_handle h, const void *F, const void *T, int dtype, void *grid_out,
                     void *stream);
int dpst_velocity_grid(dpst_handle h, void *grid_out, void *stream);
int dpst_mdot_timed(dpst_handle h, const void *F, const void *T, void *V, void *W, int dtype,
                    void *stream, float *stage_ms);

/* Allocation-free Mdot.  No counterpart in the reference.
 * For callers that cannot allocate device memory when they call the
 * operator: a host application whose own memory pool has already reserved
 * the device (a cudaMalloc from the library would fail, or take memory the
 * pool counts on), or a time-critical loop that must not pay for cudaMalloc /
 * cudaFree and the device-wide synchronisation cudaFree implies.  Same
 * arguments and results as dpst_mdot; the call
 * allocates nothing (no cudaMalloc / cudaFree, no allocating library
 * routine): the per-wavenumber solve takes its scratch from a 4 MiB static
 * device array compiled into the library (held by every GPU that loads it
 * until the process exits) instead of memory owned by the handle, and runs
 * on as many CTAs as that array holds.  Limits and rules:
 *   - grids needing more than 4 MiB of solve scratch per CTA (nz x 192
 *     doubles) are rejected with DPST_ERR_UNSUPPORTED; every nz the library
 *     accepts (<= 128) fits;
 *   - the first call on a device looks up the array's device address with
 *     that device current; make that first call before any stream capture
 *     (later calls look it up again whenever their stream is not capturing);
 *   - all calls share the one array: calls that overlap on the GPU (other
 *     streams, handles or threads) race on it and must be serialised. */
int dpst_mdot_noalloc(dpst_handle h, const void *F, const void *T, void *V, void *W, int dtype,
                      void *stream);

/* Backward pass (vector-Jacobian product) of dpst_mdot at the current
 * positions.  No counterpart in the reference, which has no derivatives;
 * it differentiates the same discrete operator dpst_mdot applies.
 * For a scalar loss l with dl/dV = gV and dl/dW = gW it writes
 *   gF = dl/dF = M_VF^T gV + M_WF^T gW,   gT = dl/dT = M_VT^T gV + M_WT^T gW,
 *   gX = dl/dX (position gradient; the ES-kernel derivatives enter through
 *        the spreading and the interpolation weights),
 * all [N][3] device arrays of `dtype` on the handle's device.
 *   - F, T: the forward call's forces and torques.  T = NULL means the
 *     forward had no torques (which also changes which ghost layers the
 *     vorticity reads).  F is needed only for gX.
 *   - gV is required; gW may be NULL (zero) and is accepted only by handles
 *     created with torques.
 *   - gF, gT, gX may each be NULL (not computed); gT needs T.
 * The velocity grid of the forward is recomputed (spread + solve), not kept
 * from dpst_mdot (dpst_mdot_backward_saved below takes it when the handle
 * still holds it).  Offsets the forward clamps to the kernel threshold and
 * the stencil's discrete choices (nearest node, z window) have zero
 * derivative; dl/dX is the gradient of the operator between those events.
 * Buffers for the backward pass are allocated on its first call.
 * Mode PERIODIC: the same outputs (its grid-to-grid map is self-adjoint, so
 * the adjoint solve is the forward one).  torque_kernel = DPST_TORQUE_REG
 * returns DPST_ERR_UNSUPPORTED. */
int dpst_mdot_backward(dpst_handle h, const void *F, const void *T, const void *gV, const void *gW,
                       void *gF, void *gT, void *gX, int dtype, void *stream);

/* The serial of the single-column Mdot (dpst_mdot, _host, _timed, _noalloc)
 * whose velocity grid the handle still holds, 0 if none: every position
 * update, multi-column Mdot, dpst_spread_grid and recomputing backward call
 * forgets it.  Read it right after the forward call. */
int dpst_forward_serial(dpst_handle h, uint64_t *out);

/* dpst_mdot_backward after a known forward: when forward_serial is the
 * value dpst_forward_serial gave right after the Mdot whose F, T these are,
 * and the handle still holds that Mdot's velocity grid (no position update
 * or other grid-writing call since), the position gradient takes that grid
 * and its open-end ghost layers instead of recomputing them (the spread and
 * the solve of the forward are skipped); otherwise it recomputes them, as
 * dpst_mdot_backward does.  *reused (may be NULL) tells which.  The caller
 * guarantees that F and T are unchanged since that Mdot (autograd's saved
 * tensors do). */
int dpst_mdot_backward_saved(dpst_handle h, uint64_t forward_serial, const void *F, const void *T,
                             const void *gV, const void *gW, void *gF, void *gT, void *gX, int dtype,
                             void *stream, int *reused);

/* ---- Batched systems (no counterpart in the reference, which runs one
 * system per FCM / DPStokes instance) ------------------------------------
 * Many independent systems -- uneven particle counts, box sizes and grids --
 * in one pipeline: one launch per stage over all systems (one cuFFT plan
 * pair per distinct (nx, ny)), captured into a CUDA graph on the first
 * dpst_batched_mdot of each (dtype, torques, vorticity) combination and
 * replayed afterwards.  Each system's V, W equal what dpst_mdot gives for it
 * alone.  The systems must share nz, zmin, zmax, mode, viscosity, precision
 * and has_torque; everything else (nx, ny, Lx, Ly, kernels, particle count)
 * is per system.  Arrays are the systems' [N_s][3] arrays concatenated in
 * the order of `params`, on the handle's device. */
typedef struct dpst_batch_engine *dpst_batch;

typedef struct {
  int n_systems;
  int n_size_classes;   /* distinct (nx, ny): one cuFFT plan pair each */
  int64_t n_particles;  /* sum of N_s */
  int64_t n_modes;      /* sum of ny (nx/2 + 1) */
  int kernels_per_mdot; /* kernels of this library in one batched Mdot (cuFFT excluded) */
  int fft_plans;
  int64_t device_bytes;
  int ztransform, ztransform_inverse; /* z transforms over all systems: 1 tcgen05, 3 tcgen05 fed by
                                         TMA (every system's own tensor maps), 0 SIMT (chosen at
                                         creation by timing, mixed operator; DPSTOKES_GB300_ZTRANSFORM
                                         forces one) */
  float ztransform_ms[2];             /* creation-time timings, forward: SIMT, tcgen05 */
  float ztransform_inverse_ms[2];     /* inverse (with the wall correction): SIMT, tcgen05 */
  float ztransform_tma_ms[2];         /* the TMA-fed form's: forward, inverse (0 if not timed) */
} dpst_batch_info;

int dpst_batched_create(const dpst_params *params, const int64_t *n_particles, int n_systems, int device,
                        dpst_batch *out);
int dpst_batched_destroy(dpst_batch b);
int dpst_batched_set_positions(dpst_batch b, const void *pos, int dtype, void *stream);
int dpst_batched_mdot(dpst_batch b, const void *F, const void *T, void *V, void *W, int dtype, void *stream);
int dpst_batched_get_info(dpst_batch b, dpst_batch_info *out);

/* Sizes and derived constants of a handle. */
int dpst_get_info(dpst_handle h, dpst_info *out);

/* Diagnostic: the mixed operator's own x-y transform on `planes` FP32 planes,
 * unnormalised, as the operator applies it (no counterpart in the reference;
 * it stands for the x-y part of Transform.cpp:215-304).  Forward
 * (inverse = 0): in = real [planes][ny][nx], out = complex
 * [planes][ny][nx/2 + 1] (cuFFT's R2C layout).  Inverse: in = the complex
 * half spectrum, which is overwritten, out = real [planes][ny][nx], the
 * imaginary parts of the kx = 0 and Nyquist columns after the y pass being
 * dropped as a complex-to-real transform does.  Powers of two, 64 <= nx <=
 * 2048, 32 <= ny <= 1024.  form 0: two launches (rows, columns); form 1:
 * one persistent launch of both passes (nx = ny in 128, 256, 512, 1024,
 * else DPST_ERR_UNSUPPORTED), whose bounded waits report DPST_ERR_CUDA if
 * one gave up; form 2: one launch of 8-CTA thread-block clusters, a plane
 * held in a cluster's shared memory (nx = ny in 256, 512, else
 * DPST_ERR_UNSUPPORTED; a bounded wait that gave up reports DPST_ERR_CUDA).
 * Allocates its tables and synchronises the stream. */
int dpst_xy_transform(int nx, int ny, int64_t planes, void *in, void *out, int inverse, int form, int device,
                      void *stream);

/* Last error message of the calling thread ("" if none). */
const char *dpst_last_error(void);

/* Library version string. */
const char *dpst_version(void);

#ifdef __cplusplus
}
#endif

#endif /* DPSTOKES_GB300_H */
