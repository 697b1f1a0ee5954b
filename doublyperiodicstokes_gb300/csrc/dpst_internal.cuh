// Internal types shared by the kernels (dpst_kernels.cu, dpst_kspace.cu) and
// the engine / C ABI (dpst_engine.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace dpst {

// One ES kernel (monopole or dipole) as laid out on the grid.  Mirrors the
// ParticleList/Grid state of the reference for one particle type
// (ParticleList.cpp:211-276 normalisation and threshold, :394-451 extended z
// grid, Grid.h Nxeff/Nyeff).
struct KernelDesc {
  int wx, wy;         // stencil widths = round(2 thr / h)
  int evenx, eveny;   // 1 for even widths (stencil start offset)
  int nxeff, nyeff;   // extended x-y sizes of the reference grid (ghost buffers)
  int lend, bend;     // x / y ghost widths
  int nzeff, dend;    // extended z grid size, ghost layers per end
  int wz_max;         // upper bound of the z window length
  int zext_off;       // offset of this kernel's extended z grid in the tables
  int unif_z;         // 1: uniform periodic z grid (triply periodic mode); the
                      // window is wz_max points around the nearest node
  int evenz;          // uniform z: 1 for an even z width
  double hz;          // uniform z: grid spacing
  double beta, alpha, alpha2, thr, inv_norm3, norm;
  double inv_alpha2;  // 1 / alpha2
};

// Boundary handling of the z ends for one BC set (reference BCs / BCst_z,
// FCM.py:215-248): an active end folds ghost data back with sign s and
// multiplies the boundary node by (1+s) (BoundaryConditions.h:284-341,
// 650-729); an inactive end ('none') drops spread data and leaves ghost
// layers untouched.
struct ZEnds {
  int top_active, bot_active;  // top = z max (extended index 0)
  double s_top, s_bot;
  int periodic;                // triply periodic: z wraps like x and y
};

// Everything a particle kernel needs (passed by value).
struct GridArgs {
  int nx, ny, nz;
  double hx, hy, Lx, Ly, Lz;
  ZEnds bcA;  // BCs  : forces, x/y torque derivatives
  ZEnds bcB;  // BCst : z torque derivative
};

// Per-particle stencil data for one kernel type, structure of arrays.
template <typename R>
struct Stencils {
  int4 *cell;   // (xclose, yclose, indl, wz)
  R *phx;       // [N][wx]  phi(x offsets)
  R *phy;       // [N][wy]
  R *phz;       // [N][wz_max] phi(z offsets) / norm^3
  R *phzw;      // [N][wz_max] phz * hx * hy * w_cc(z)  (interpolation weights)
  R *dphx;      // dipole only: derivative kernels
  R *dphy;
  R *dphz;
  R *dphzw;
};

// Derivatives of the stencil factors with respect to the particle's own
// coordinate, for the position gradient of the backward pass.  Same shapes as
// the matching Stencils arrays; zero where the forward clamped the offset.
template <typename R>
struct GradStencils {
  R *gx, *gy;     // d phx / d x, d phy / d y
  R *gz, *gzw;    // d phz / d z, d phzw / d z
  R *gdx, *gdy;   // dipole kernel: d dphx / d x, d dphy / d y
  R *gdz, *gdzw;  // dipole kernel: d dphz / d z, d dphzw / d z
};

// Ghost-layer buffers for open z ends: the reference leaves spread data in
// the extended grid's ghost layers at 'none' ends and the next interpolation
// reads it back (Grid::zeroExtGrid only before a spread, Ghostify copies only
// active ends).  Layout [level][nyeff][nxeff][3]; top levels are extended
// indices [0, dend), bottom levels [dend+nz, nzeff).
template <typename R>
struct Ghosts {
  R *top;     // nullptr if no particle reaches the top ghost layers
  R *bot;
  int ntop;   // number of levels stored (from the layer nearest the node)
  int nbot;
};

// One system of a batch (dpst_batched_*) as the particle kernels see it.
// Particles of system s are [pbase, pbase + n) of the concatenated arrays;
// its stencils, grid and ghost layers are its own slices.
template <typename R>
struct SysP {
  KernelDesc km, kd;  // monopole / dipole kernel
  GridArgs g;
  Stencils<R> stm, std_;
  Ghosts<R> ghm, ghd;
  R *grid;  // [3][nz][ny][nx]
  int64_t pbase, n;
};

// A ghost-layer buffer of one system, for the batched fold.
template <typename R>
struct FoldJob {
  R *buf;
  int levels, nx, ny;
  KernelDesc kd;
};

// Arguments of the wavenumber-space kernels (dpst_kspace.cu).
struct KsArgs {
  int nx, ny, nz, nxh;
  int64_t nk;
  double H, eta, Lz;
  int mode;  // 0 open, 1 bottom wall, 2 slit
  const double *kvx, *kvy;  // wavenumber tables, length nx / ny (reference ordering)
  const double *zn;         // Chebyshev nodes in [0, Lz], descending (zn[0] = Lz)
  // SIMat / FIMat bands (H-scaled), per row m
  const double *s0, *sp2, *sm2, *fm1, *fp1;
  double se0, se1, fe;
  // BC rows (length nz + 2 each) of the reference (Solvers.py:603-643)
  const double *bcr1, *bcr2, *bcl1, *bcl2;
  // per-mode factors as computed, [index][nk] (k_bvp_factors' working arrays)
  double *mfac, *invb, *dp2, *ab0, *ab1, *c0, *c1, *ginv;
  // packed factors read by the solve (k_bvp_pack):
  //   mf [nz][nk]     forward-sweep multipliers (rows 0, 1 are zero)
  //   bk [nz][nk][4]  back-sweep row data {1/beta_{j+1}, dp2_j, C0_j, C1_j}
  //                   (dp2 zero on the last two rows)
  //   ab [nz][nk]     border column of A^{-1}B: column 0 on even rows, column 1
  //                   on odd rows (A couples j with j +- 2 only, so each column
  //                   vanishes exactly on the other parity)
  double *mf, *bk, *ab;
  // k = 0 velocity correction: C rows (length nz) and Gi row-major
  const double *k0c0, *k0c1;
  double k0gi[4];
  // FP32 copy of the wall-correction coefficients [nk][16], written by the
  // solve beside the FP64 ones for the mixed operator's epilogue (nullptr:
  // not wanted)
  float2 *corrf;
  // per-wavenumber data of the double-float solve k_bvp_df, as hi, lo FP32
  // pairs (nullptr when the handle does not use it):
  //   kap2 [nz][nk]  kappa_j = K^2 / beta_{j+1} (K^2 times the reciprocal pivot
  //                  of row j); the sweeps run on K^2-scaled unknowns, so this
  //                  is the only per-row factor besides A^{-1}B
  //   ab2 [nz][nk]   as ab
  //   gi2 [4][nk]    as ginv
  //   km2 [nk]       {K^2, 1/K^2}; km3 [nk] {H^2 K, 1/(2K)} (zero for k = 0)
  //   dx2 [nxh], dy2 [ny]  the derivative wavenumbers Dx, Dy (kx, ky with the
  //                  Nyquist entries of even sizes zeroed)
  float2 *kap2, *ab2, *gi2, *dx2, *dy2;
  float4 *km2, *km3;
};

// Epilogue of the z-transform GEMM.
struct EpiArgs {
  int inverse;
  double scale;  // 1/(nx ny) for the inverse
  const double2 *corr;
  // FP32 form of the correction for the mixed operator (all nullptr: use
  // corr): the solve's FP32 coefficients [nk][16], per mode {k, kx, ky,
  // Hermitian ? 1 : 0} and {kx', ky', 0, 0} of the partner index, the nodes
  // in FP32 and 1 / (2 eta)
  const float2 *corrf;
  const float4 *cmode;
  const float *znf;
  float fac;
  KsArgs ks;
};

// One system of a batch as the wavenumber-space kernels see it.
template <typename R>
struct SysK {
  KsArgs ks;
  R *spec;        // [3][nz][nk] complex
  double2 *corr;  // [nk][16] wall-correction coefficients (walls only)
};

// Segment of the batched z transform: one system's spectrum.
template <typename R>
struct ZSeg {
  R *spec;
  int64_t ncols;  // 2 nk real columns per row
  EpiArgs e;
};

// Batched work items: item x of [0, prefix[S]) belongs to entry s with
// prefix[s] <= x < prefix[s+1] (entries with no items are skipped).
static __device__ __forceinline__ int find_sys(const int64_t *__restrict__ prefix, int S, int64_t x) {
  int lo = 0, hi = S;  // prefix[lo] <= x < prefix[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(prefix + mid) <= x) lo = mid;
    else hi = mid;
  }
  return lo;
}

}  // namespace dpst
