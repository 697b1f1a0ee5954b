// Particle-side kernels: stencil setup, spreading (forces and the torque
// curl) and interpolation (velocities and velocity gradients), with the
// reference's ghost fold / ghost copy semantics applied through index maps
// instead of an extended grid.
//
// Reference behaviour restated (source/cpu of stochasticHydroTools/
// DoublyPeriodicStokes):
//   stencil            ParticleList.cpp:394-526 (xclose, clamped offsets,
//                      z window by lower_bound on the descending extended grid)
//   kernel             ESKernels.h:8-46 (separable: the product of three 1-D
//                      factors equals exp of the summed exponents)
//   spread / interp    SpreadInterp.cpp:302-600, SpreadInterp.h:100-212
//   ghost fold / copy  BoundaryConditions.h:22-731
//   torque curl        SpreadInterpWrapper.cpp:66-107, FCM.py:362-371,411-426
#include "dpst_internal.cuh"
#include "dpst_pdev.cuh"

namespace dpst {

// ---------------------------------------------------------------------------
// Stencil setup: one thread per particle.  pos is [N][3] with z already
// relative to zmin.  Offsets are computed in FP64 exactly as the reference
// does (same operation order) and clamped to +thr when outside [-thr, thr].
// err bit 1: particle outside the unit cell; bit 2: z window longer than the
// allocated stride.  reach[0] = min indl, reach[1] = max indr (extended z).
// ---------------------------------------------------------------------------
template <typename R, bool DIPOLE>
static __device__ __forceinline__ void locate_item(int64_t p, const double *__restrict__ pos, const KernelDesc &kd,
                                                   const double *__restrict__ zext,
                                                   const double *__restrict__ wext, const GridArgs &g,
                                                   const Stencils<R> &st, int *err, int *reach) {
  double x = pos[3 * p], y = pos[3 * p + 1], z = pos[3 * p + 2];
  if (!(x >= 0.0 && x <= g.Lx && y >= 0.0 && y <= g.Ly && z >= 0.0 && z <= g.Lz)) {
    atomicOr(err, 1);
    st.cell[p] = make_int4(0, 0, 0, 0);
    return;
  }
  const double thr = kd.thr;
  int xclose = (int)(x / g.hx);
  int yclose = (int)(y / g.hy);
  if ((kd.wx & 1) && (x / g.hx - xclose > 0.5)) xclose += 1;
  if ((kd.wy & 1) && (y / g.hy - yclose > 0.5)) yclose += 1;
  for (int i = 0; i < kd.wx; ++i) {
    double o = ((double)xclose + i - kd.wx / 2 + kd.evenx) * g.hx - x;
    if (o > thr || o < -thr) o = thr;
    st.phx[p * kd.wx + i] = es1r<R>(o, kd);
    if (DIPOLE) st.dphx[p * kd.wx + i] = des1r<R>(o, kd);
  }
  for (int j = 0; j < kd.wy; ++j) {
    double o = ((double)yclose + j - kd.wy / 2 + kd.eveny) * g.hy - y;
    if (thr < o || o < -thr) o = thr;
    st.phy[p * kd.wy + j] = es1r<R>(o, kd);
    if (DIPOLE) st.dphy[p * kd.wy + j] = des1r<R>(o, kd);
  }
  if (kd.unif_z) {
    // uniform periodic z (ParticleList.cpp:285-366): the window is built like
    // the x and y windows; its first entry sits at extended index
    // zclose - wz/2 + evenz + dend; interpolation weight hx hy hz
    const int wz = kd.wz_max;
    int zclose = (int)(z / kd.hz);
    if ((wz & 1) && (z / kd.hz - zclose > 0.5)) zclose += 1;
    st.cell[p] = make_int4(xclose, yclose, zclose - wz / 2 + kd.evenz + kd.dend, wz);
    const double hxyz = g.hx * g.hy * kd.hz;
    for (int k = 0; k < wz; ++k) {
      double o = ((double)zclose + k - wz / 2 + kd.evenz) * kd.hz - z;
      if (thr < o || o < -thr) o = thr;
      const R v = es1r<R>(o, kd) * (R)kd.inv_norm3;
      st.phz[p * wz + k] = v;
      st.phzw[p * wz + k] = v * (R)hxyz;
      if (DIPOLE) {
        const R dv = des1r<R>(o, kd) * (R)kd.inv_norm3;
        st.dphz[p * wz + k] = dv;
        st.dphzw[p * wz + k] = dv * (R)hxyz;
      }
    }
    return;
  }
  // z window: zext is strictly descending; indl = #{zext > z + thr},
  // high = #{zext > z - thr}; indr = high - 1 unless zext[high] == z - thr.
  const double *ze = zext + kd.zext_off;
  const double *we = wext + kd.zext_off;
  const int n = kd.nzeff;
  auto count_greater = [&](double v) {
    int lo = 0, hi = n;  // first index with ze[idx] <= v
    while (lo < hi) {
      int mid = (lo + hi) >> 1;
      if (ze[mid] > v) lo = mid + 1; else hi = mid;
    }
    return lo;
  };
  int indl = count_greater(z + thr);
  int indr = count_greater(z - thr);
  if (indr == n) indr -= 1;
  else if (z - thr > ze[indr]) indr -= 1;
  int wz = indr - indl + 1;
  if (wz > kd.wz_max) {
    atomicOr(err, 2);
    st.cell[p] = make_int4(0, 0, 0, 0);
    return;
  }
  if (wz < 1) wz = 0;  // no node within the support: no z contributions
  st.cell[p] = make_int4(xclose, yclose, indl, wz);
  if (wz > 0) {
    atomicMin(&reach[0], indl);
    atomicMax(&reach[1], indr);
  }
  const double hxy = g.hx * g.hy;
  for (int k = 0; k < kd.wz_max; ++k) {
    R v = 0, dv = 0, wgt = 0;
    if (k < wz) {
      double o = ze[indl + k] - z;
      if (thr < o || o < -thr) o = thr;
      v = es1r<R>(o, kd) * (R)kd.inv_norm3;
      if (DIPOLE) dv = des1r<R>(o, kd) * (R)kd.inv_norm3;
      wgt = (R)(hxy * we[indl + k]);
    }
    st.phz[p * kd.wz_max + k] = v;
    st.phzw[p * kd.wz_max + k] = v * wgt;
    if (DIPOLE) {
      st.dphz[p * kd.wz_max + k] = dv;
      st.dphzw[p * kd.wz_max + k] = dv * wgt;
    }
  }
}

template <typename R, bool DIPOLE>
__global__ void k_locate(const double *__restrict__ pos, int64_t N, KernelDesc kd,
                         const double *__restrict__ zext, const double *__restrict__ wext,
                         GridArgs g, Stencils<R> st, int *err, int *reach) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= N) return;
  locate_item<R, DIPOLE>(p, pos, kd, zext, wext, g, st, err, reach);
}

// ---------------------------------------------------------------------------
// Monopole spread of forces: one thread per (particle, stencil column).
// grid layout [3][nz][ny][nx].
// ---------------------------------------------------------------------------
template <typename R, typename RF>
static __device__ __forceinline__ void spread_mono_item(int64_t p, int c, const RF *__restrict__ F,
                                                     const KernelDesc &kd, const GridArgs &g,
                                                     const Stencils<R> &st, R *__restrict__ grid,
                                                     const Ghosts<R> &gh) {
  int i = c % kd.wx, j = c / kd.wx;
  int4 cl = st.cell[p];
  if (cl.w == 0) return;
  const int ox = cl.x + i - kd.wx / 2 + kd.evenx;
  const int oy = cl.y + j - kd.wy / 2 + kd.eveny;
  const int px = wrapi(ox, g.nx), py = wrapi(oy, g.ny);
  const int ie = ox + kd.lend, je = oy + kd.bend;  // extended-grid column
  const R f0 = (R)F[3 * p], f1 = (R)F[3 * p + 1], f2 = (R)F[3 * p + 2];
  const R cxy = st.phx[p * kd.wx + i] * st.phy[p * kd.wy + j];
  const int64_t plane = (int64_t)g.nx * g.ny, comp = plane * g.nz;
  const int64_t col = (int64_t)py * g.nx + px;
  for (int k = 0; k < cl.w; ++k) {
    const R v = cxy * st.phz[p * kd.wz_max + k];
    ZMap zm = zmap(cl.z + k, kd.dend, g.nz, g.bcA);
    if (zm.m >= 0) {
      if (zm.wgt == 0.0) continue;
      const R a = v * (R)zm.wgt;
      R *dst = grid + zm.m * plane + col;
      atomic_add(dst, a * f0);
      atomic_add(dst + comp, a * f1);
      atomic_add(dst + 2 * comp, a * f2);
    } else {
      R *buf = (zm.m == -1) ? gh.top : gh.bot;
      if (buf == nullptr || ie < 0 || ie >= kd.nxeff || je < 0 || je >= kd.nyeff) continue;
      R *dst = buf + (((int64_t)zm.level * kd.nyeff + je) * kd.nxeff + ie) * 3;
      atomic_add(dst, v * f0);
      atomic_add(dst + 1, v * f1);
      atomic_add(dst + 2, v * f2);
    }
  }
}

// perm (optional): particles taken in this order (sorted by tile, so that
// neighbouring threads update nearby grid cells).
template <typename R, typename RF>
__global__ void k_spread_mono(const RF *__restrict__ F, int64_t N, KernelDesc kd, GridArgs g,
                            Stencils<R> st, R *__restrict__ grid, Ghosts<R> gh, const int *__restrict__ perm) {
  const int cols = kd.wx * kd.wy;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= N * cols) return;
  const int64_t q = t / cols;
  const int64_t p = perm ? (int64_t)perm[q] : q;
  spread_mono_item<R, RF>(p, (int)(t - q * cols), F, kd, g, st, grid, gh);
}

// ---------------------------------------------------------------------------
// Dipole spread of the torque curl, f += 1/2 curl(T delta) with derivative
// kernels: x and y derivative spreads use BC set A, the z derivative spread
// BC set B (FCM.py:362-371).  Ghost layers at inactive ends of set B keep the
// raw z-derivative spread (the last spread the reference does on its torque
// grid before interpolating).
// ---------------------------------------------------------------------------
template <typename R, typename RF>
static __device__ __forceinline__ void spread_dip_item(int64_t p, int c, const RF *__restrict__ T,
                                                     const KernelDesc &kd, const GridArgs &g,
                                                     const Stencils<R> &st, R *__restrict__ grid,
                                                     const Ghosts<R> &gh) {
  int i = c % kd.wx, j = c / kd.wx;
  int4 cl = st.cell[p];
  if (cl.w == 0) return;
  const int ox = cl.x + i - kd.wx / 2 + kd.evenx;
  const int oy = cl.y + j - kd.wy / 2 + kd.eveny;
  const int px = wrapi(ox, g.nx), py = wrapi(oy, g.ny);
  const int ie = ox + kd.lend, je = oy + kd.bend;
  const R tx = (R)T[3 * p], ty = (R)T[3 * p + 1], tz = (R)T[3 * p + 2];
  const R fx = st.phx[p * kd.wx + i], fy = st.phy[p * kd.wy + j];
  const R dfx = st.dphx[p * kd.wx + i], dfy = st.dphy[p * kd.wy + j];
  const R axy = dfx * fy, bxy = fx * dfy, cxy = fx * fy;
  const int64_t plane = (int64_t)g.nx * g.ny, comp = plane * g.nz;
  const int64_t col = (int64_t)py * g.nx + px;
  const R half = (R)0.5;
  for (int k = 0; k < cl.w; ++k) {
    const R phz = st.phz[p * kd.wz_max + k];
    const R ax = axy * phz;                          // d/dx kernel
    const R ay = bxy * phz;                          // d/dy kernel
    const R az = cxy * st.dphz[p * kd.wz_max + k];   // d/dz kernel
    const int kk = cl.z + k;
    ZMap a = zmap(kk, kd.dend, g.nz, g.bcA);
    ZMap b = zmap(kk, kd.dend, g.nz, g.bcB);
    if (a.m >= 0 && a.wgt != 0.0) {
      R *dst = grid + a.m * plane + col;
      const R wa = (R)a.wgt * half;
      atomic_add(dst, wa * (ay * tz));                   // addDy: fx += 1/2 Sy[Tz]
      atomic_add(dst + comp, -wa * (ax * tz));           // addDx: fy -= 1/2 Sx[Tz]
      atomic_add(dst + 2 * comp, wa * (ax * ty - ay * tx));  // fz += 1/2 Sx[Ty] - 1/2 Sy[Tx]
    }
    if (b.m >= 0) {
      if (b.wgt != 0.0) {
        R *dst = grid + b.m * plane + col;
        const R wb = (R)b.wgt * half;
        atomic_add(dst, -wb * (az * ty));       // addDz: fx -= 1/2 Sz[Ty]
        atomic_add(dst + comp, wb * (az * tx)); // fy += 1/2 Sz[Tx]
      }
    } else {
      R *buf = (b.m == -1) ? gh.top : gh.bot;
      if (buf == nullptr || ie < 0 || ie >= kd.nxeff || je < 0 || je >= kd.nyeff) continue;
      R *dst = buf + (((int64_t)b.level * kd.nyeff + je) * kd.nxeff + ie) * 3;
      atomic_add(dst, az * tx);
      atomic_add(dst + 1, az * ty);
      atomic_add(dst + 2, az * tz);
    }
  }
}

// perm (optional): particles taken in this order (sorted by tile, so that
// neighbouring threads update nearby grid cells).
template <typename R, typename RF>
__global__ void k_spread_dip(const RF *__restrict__ T, int64_t N, KernelDesc kd, GridArgs g,
                            Stencils<R> st, R *__restrict__ grid, Ghosts<R> gh, const int *__restrict__ perm) {
  const int cols = kd.wx * kd.wy;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= N * cols) return;
  const int64_t q = t / cols;
  const int64_t p = perm ? (int64_t)perm[q] : q;
  spread_dip_item<R, RF>(p, (int)(t - q * cols), T, kd, g, st, grid, gh);
}

// ---------------------------------------------------------------------------
// Fused monopole + dipole spread, for kernel pairs that share the x-y stencil
// columns and the extended z grid and whose dipole threshold is at most the
// monopole's (fused_supports): every dipole z window is then a sub-range of
// the same particle's monopole window, so one pass over the monopole window
// adds both contributions with one atomic per grid value (the separate
// passes take three for the forces and five for the torque curl).
// ---------------------------------------------------------------------------
template <typename R, typename RF>
static __device__ __forceinline__ void spread_fused_item(int64_t p, int c, const RF *__restrict__ F,
                                                         const RF *__restrict__ T, const KernelDesc &km,
                                                         const KernelDesc &kd, const GridArgs &g,
                                                         const Stencils<R> &sm, const Stencils<R> &sd,
                                                         R *__restrict__ grid, const Ghosts<R> &ghm,
                                                         const Ghosts<R> &ghd) {
  const int i = c % km.wx, j = c / km.wx;
  const int4 cm = sm.cell[p];
  if (cm.w == 0) return;
  const int4 cd = sd.cell[p];
  const int ox = cm.x + i - km.wx / 2 + km.evenx;
  const int oy = cm.y + j - km.wy / 2 + km.eveny;
  const int px = wrapi(ox, g.nx), py = wrapi(oy, g.ny);
  const int ie = ox + km.lend, je = oy + km.bend;
  const R f0 = (R)F[3 * p], f1 = (R)F[3 * p + 1], f2 = (R)F[3 * p + 2];
  const R tx = (R)T[3 * p], ty = (R)T[3 * p + 1], tz = (R)T[3 * p + 2];
  const R cm_xy = sm.phx[p * km.wx + i] * sm.phy[p * km.wy + j];
  const R fx = sd.phx[p * kd.wx + i], fy = sd.phy[p * kd.wy + j];
  const R dfx = sd.dphx[p * kd.wx + i], dfy = sd.dphy[p * kd.wy + j];
  const R axy = dfx * fy, bxy = fx * dfy, cxy = fx * fy;
  const int64_t plane = (int64_t)g.nx * g.ny, comp = plane * g.nz;
  const int64_t col = (int64_t)py * g.nx + px;
  const R half = (R)0.5;
  const int m0 = cm.z - km.dend;  // interior node of the window's first entry
  if (m0 >= 1 && m0 + cm.w <= g.nz - 1) {
    // every node of the window is an interior node of weight 1 under both
    // BC sets (zmap): one base pointer, the dipole's sub-range known upfront
    const int dk = cm.z - cd.z;
    const int k0 = max(-dk, 0), k1 = min(cd.w - dk, cm.w);
    const R *__restrict__ pz = sm.phz + p * km.wz_max;
    const R *__restrict__ pzd = sd.phz + p * kd.wz_max + dk;
    const R *__restrict__ dpzd = sd.dphz + p * kd.wz_max + dk;
    R *dst = grid + (int64_t)m0 * plane + col;
    for (int k = 0; k < cm.w; ++k, dst += plane) {
      const R v = cm_xy * pz[k];
      R gx = v * f0, gy = v * f1, gz = v * f2;
      if (k >= k0 && k < k1) {
        const R phz = pzd[k];
        const R ax = axy * phz, ay = bxy * phz, az = cxy * dpzd[k];
        gx += half * (ay * tz) + (-half) * (az * ty);
        gy += -half * (ax * tz) + half * (az * tx);
        gz += half * (ax * ty - ay * tx);
      }
      atomic_add(dst, gx);
      atomic_add(dst + comp, gy);
      atomic_add(dst + 2 * comp, gz);
    }
    return;
  }
  for (int k = 0; k < cm.w; ++k) {
    const int kk = cm.z + k;
    const R v = cm_xy * sm.phz[p * km.wz_max + k];
    const int kq = kk - cd.z;  // the dipole window's index of this node
    const bool dip = kq >= 0 && kq < cd.w;
    ZMap a = zmap(kk, km.dend, g.nz, g.bcA);
    // set A: the forces and the x, y derivative spreads of the curl
    R gx = 0, gy = 0, gz = 0;
    if (a.m >= 0) {
      if (a.wgt != 0.0) {
        const R am = v * (R)a.wgt;
        gx = am * f0;
        gy = am * f1;
        gz = am * f2;
      }
    } else {
      R *buf = (a.m == -1) ? ghm.top : ghm.bot;
      if (buf != nullptr && ie >= 0 && ie < km.nxeff && je >= 0 && je < km.nyeff) {
        R *dst = buf + (((int64_t)a.level * km.nyeff + je) * km.nxeff + ie) * 3;
        atomic_add(dst, v * f0);
        atomic_add(dst + 1, v * f1);
        atomic_add(dst + 2, v * f2);
      }
    }
    R bx = 0, by = 0;
    ZMap b;
    b.m = a.m;
    if (dip) {
      const R phz = sd.phz[p * kd.wz_max + kq];
      const R ax = axy * phz, ay = bxy * phz;
      const R az = cxy * sd.dphz[p * kd.wz_max + kq];
      if (a.m >= 0 && a.wgt != 0.0) {
        const R wa = (R)a.wgt * half;
        gx += wa * (ay * tz);
        gy += -wa * (ax * tz);
        gz += wa * (ax * ty - ay * tx);
      }
      b = zmap(kk, kd.dend, g.nz, g.bcB);
      if (b.m >= 0) {
        if (b.wgt != 0.0) {
          const R wb = (R)b.wgt * half;
          bx = -wb * (az * ty);
          by = wb * (az * tx);
        }
      } else {
        R *buf = (b.m == -1) ? ghd.top : ghd.bot;
        if (buf != nullptr && ie >= 0 && ie < kd.nxeff && je >= 0 && je < kd.nyeff) {
          R *dst = buf + (((int64_t)b.level * kd.nyeff + je) * kd.nxeff + ie) * 3;
          atomic_add(dst, az * tx);
          atomic_add(dst + 1, az * ty);
          atomic_add(dst + 2, az * tz);
        }
      }
    }
    if (a.m >= 0 && a.wgt != 0.0) {
      R *dst = grid + a.m * plane + col;
      if (dip && b.m == a.m) {  // set B lands on the same node: one atomic each
        gx += bx;
        gy += by;
        bx = 0;
        by = 0;
      }
      atomic_add(dst, gx);
      atomic_add(dst + comp, gy);
      atomic_add(dst + 2 * comp, gz);
    }
    if (dip && b.m >= 0 && (bx != (R)0 || by != (R)0)) {
      R *dst = grid + b.m * plane + col;
      atomic_add(dst, bx);
      atomic_add(dst + comp, by);
    }
  }
}

template <typename R, typename RF>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 4 : 1) k_spread_fused(const RF *__restrict__ F, const RF *__restrict__ T, int64_t N, KernelDesc km,
                               KernelDesc kd, GridArgs g, Stencils<R> sm, Stencils<R> sd, R *__restrict__ grid,
                               Ghosts<R> ghm, Ghosts<R> ghd, const int *__restrict__ perm) {
  const int cols = km.wx * km.wy;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= N * cols) return;
  const int64_t q = t / cols;
  const int64_t p = perm ? (int64_t)perm[q] : q;
  spread_fused_item<R, RF>(p, (int)(t - q * cols), F, T, km, kd, g, sm, sd, grid, ghm, ghd);
}

// ---------------------------------------------------------------------------
// Tile-owner spread (mixed operator, fused kernel pair): one CTA per
// ORDER_TILE x ORDER_TILE tile of grid columns holds the tile's whole grid
// block [3][nz][8][8] in shared memory, gathers the contributions of the
// particles of the 3 x 3 neighbouring tiles (every stencil reaching the tile
// starts there: wx, wy <= 14) to its own cells with shared-memory atomics,
// and writes the block once with plain stores.  Every grid value is written
// exactly once, zeros included, so the grid needs no clearing and HBM sees
// no atomics.  Particles whose window is not interior under both BC sets
// (spread_fused_item's general path: folds, ghost layers) are skipped here
// and spread afterwards from their list by k_spread_fused.
// ---------------------------------------------------------------------------
constexpr int ORDER_TILE = 8;  // columns per side of the particle-order tile (k_tile_order)
constexpr int TILE_SPREAD_THREADS = 256;

template <typename R, typename RF>
void launch_spread_fused(const RF *F, const RF *T, int64_t N, const KernelDesc &km, const KernelDesc &kd,
                         const GridArgs &g, const Stencils<R> &sm, const Stencils<R> &sd, R *grid,
                         const Ghosts<R> &ghm, const Ghosts<R> &ghd, cudaStream_t s, const int *perm);

static __device__ __forceinline__ bool fused_interior(const int4 &cm, int dend, int nz) {
  const int m0 = cm.z - dend;
  return cm.w == 0 || (m0 >= 1 && m0 + cm.w <= nz - 1);
}

template <typename RF>
__global__ void __launch_bounds__(TILE_SPREAD_THREADS, 2)
    k_spread_tiles(const RF *__restrict__ F, const RF *__restrict__ T, KernelDesc km, KernelDesc kd, GridArgs g,
                   Stencils<float> sm, Stencils<float> sd, float *__restrict__ grid, const int *__restrict__ perm,
                   const int *__restrict__ tstart, int ntx, int nty) {
  extern __shared__ float tb[];  // [3][nz][ORDER_TILE][ORDER_TILE]
  __shared__ int list[TILE_SPREAD_THREADS];
  __shared__ int nlist, rng[10];
  constexpr int TT = ORDER_TILE * ORDER_TILE;
  const int nz = g.nz;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = TILE_SPREAD_THREADS / 32;
  const int bx = blockIdx.x % ntx, by = blockIdx.x / ntx;
  const int x0 = bx * ORDER_TILE, y0 = by * ORDER_TILE;
  const int cells = 3 * nz * TT;
  for (int i = tid; i < cells; i += TILE_SPREAD_THREADS) tb[i] = 0.0f;
  // the candidates: the particles of the 3 x 3 neighbouring tiles, as one
  // range [0, rng[9]) with the tiles' offsets in rng
  if (tid == 0) {
    int acc = 0;
    for (int nb = 0; nb < 9; ++nb) {
      const int t = wrapi(by + nb / 3 - 1, nty) * ntx + wrapi(bx + nb % 3 - 1, ntx);
      rng[nb] = acc;
      acc += tstart[t + 1] - tstart[t];
    }
    rng[9] = acc;
  }
  __syncthreads();
  const int ncand = rng[9];
  const float half = 0.5f;
  const int comp = nz * TT;
  for (int c0 = 0; c0 < ncand; c0 += TILE_SPREAD_THREADS) {
    // one candidate per thread: keep the interior particles whose stencil
    // reaches this tile
    if (tid == 0) nlist = 0;
    __syncthreads();
    const int c = c0 + tid;
    if (c < ncand) {
      int nb = 0;
      while (c >= rng[nb + 1]) ++nb;
      const int t = wrapi(by + nb / 3 - 1, nty) * ntx + wrapi(bx + nb % 3 - 1, ntx);
      const int p = perm[tstart[t] + c - rng[nb]];
      const int4 cm = sm.cell[p];
      if (cm.w > 0 && fused_interior(cm, km.dend, nz)) {
        const int sx = wrapi(cm.x - km.wx / 2 + km.evenx - x0, g.nx), sy = wrapi(cm.y - km.wy / 2 + km.eveny - y0, g.ny);
        // the stencil's first column relative to the tile, modulo nx: it
        // reaches the tile when it starts inside or ends past the tile's start
        const bool hx = sx < ORDER_TILE || sx + km.wx > g.nx;
        const bool hy = sy < ORDER_TILE || sy + km.wy > g.ny;
        if (hx && hy) list[atomicAdd(&nlist, 1)] = p;
      }
    }
    __syncthreads();
    const int nl = nlist;
    for (int e = warp; e < nl; e += nw) {
      const int p = list[e];
      const int4 cm = sm.cell[p];
      const int4 cd = sd.cell[p];
      const int dk = cm.z - cd.z;
      const int k0 = max(-dk, 0), k1 = min(cd.w - dk, cm.w);
      const int m0 = cm.z - km.dend;
      // the stencil's columns inside the tile: i in [i0, i1), j in [j0, j1)
      int sx = cm.x - km.wx / 2 + km.evenx - x0, sy = cm.y - km.wy / 2 + km.eveny - y0;
      sx = wrapi(sx, g.nx);
      sy = wrapi(sy, g.ny);
      if (sx >= ORDER_TILE) sx -= g.nx;  // started left of the tile (wrapped)
      if (sy >= ORDER_TILE) sy -= g.ny;
      const int i0 = max(0, -sx), i1 = min(km.wx, ORDER_TILE - sx);
      const int j0 = max(0, -sy), j1 = min(km.wy, ORDER_TILE - sy);
      const int ni = i1 - i0, nj = j1 - j0;
      if (ni <= 0 || nj <= 0) continue;
      // the particle's factors in lanes: lane l holds entry l of each table
      const float lphx = lane < km.wx ? sm.phx[p * km.wx + lane] : 0.0f;
      const float lphy = lane < km.wy ? sm.phy[p * km.wy + lane] : 0.0f;
      const float lfx = lane < kd.wx ? sd.phx[p * kd.wx + lane] : 0.0f;
      const float lfy = lane < kd.wy ? sd.phy[p * kd.wy + lane] : 0.0f;
      const float ldfx = lane < kd.wx ? sd.dphx[p * kd.wx + lane] : 0.0f;
      const float ldfy = lane < kd.wy ? sd.dphy[p * kd.wy + lane] : 0.0f;
      // z factors of window entries lane and lane + 32
      float lpz[2], lpzd[2], ldpzd[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int kk = lane + 32 * h;
        lpz[h] = kk < cm.w ? sm.phz[p * km.wz_max + kk] : 0.0f;
        const bool dz = kk >= k0 && kk < k1;
        lpzd[h] = dz ? sd.phz[p * kd.wz_max + dk + kk] : 0.0f;
        ldpzd[h] = dz ? sd.dphz[p * kd.wz_max + dk + kk] : 0.0f;
      }
      const float f0 = (float)F[3 * p], f1 = (float)F[3 * p + 1], f2 = (float)F[3 * p + 2];
      const float tx_ = (float)T[3 * p], ty_ = (float)T[3 * p + 1], tz_ = (float)T[3 * p + 2];
      const int items = ni * nj * cm.w;
      for (int b = 0; b < items; b += 32) {
        const int it = b + lane;
        const bool live = it < items;
        const int k = live ? it / (ni * nj) : 0;
        const int r = live ? it - k * (ni * nj) : 0;
        const int jj = r / ni, ii = r - jj * ni;
        const int i = i0 + ii, j = j0 + jj;
        const float px = __shfl_sync(0xffffffffu, lphx, i), py = __shfl_sync(0xffffffffu, lphy, j);
        const float fx = __shfl_sync(0xffffffffu, lfx, i), fy = __shfl_sync(0xffffffffu, lfy, j);
        const float dfx = __shfl_sync(0xffffffffu, ldfx, i), dfy = __shfl_sync(0xffffffffu, ldfy, j);
        const int kh = k >> 5;
        const float pz0 = __shfl_sync(0xffffffffu, lpz[0], k), pz1 = __shfl_sync(0xffffffffu, lpz[1], k);
        const float pd0 = __shfl_sync(0xffffffffu, lpzd[0], k), pd1 = __shfl_sync(0xffffffffu, lpzd[1], k);
        const float dd0 = __shfl_sync(0xffffffffu, ldpzd[0], k), dd1 = __shfl_sync(0xffffffffu, ldpzd[1], k);
        const float pz = kh ? pz1 : pz0, phz = kh ? pd1 : pd0, dphz = kh ? dd1 : dd0;
        if (!live) continue;
        const float v = (px * py) * pz;
        float gx = v * f0, gy = v * f1, gz = v * f2;
        if (k >= k0 && k < k1) {
          const float ax = (dfx * fy) * phz, ay = (fx * dfy) * phz, az = (fx * fy) * dphz;
          gx += half * (ay * tz_) + (-half) * (az * ty_);
          gy += -half * (ax * tz_) + half * (az * tx_);
          gz += half * (ax * ty_ - ay * tx_);
        }
        float *dst = tb + ((m0 + k) * ORDER_TILE + sy + j) * ORDER_TILE + sx + i;
        atomicAdd(dst, gx);
        atomicAdd(dst + comp, gy);
        atomicAdd(dst + 2 * comp, gz);
      }
    }
    __syncthreads();
  }
  // the block to the grid: rows of ORDER_TILE values, two float4 per row
  const int64_t plane = (int64_t)g.nx * g.ny;
  const int rows = 3 * nz * ORDER_TILE;
  const bool full = x0 + ORDER_TILE <= g.nx && y0 + ORDER_TILE <= g.ny && (g.nx & 3) == 0;
  for (int r2 = tid; r2 < 2 * rows; r2 += TILE_SPREAD_THREADS) {
    const int r = r2 >> 1, h = r2 & 1;
    const int yl = r % ORDER_TILE, dm = r / ORDER_TILE;  // dm = d nz + m
    const int y = y0 + yl;
    const float *src = tb + r * ORDER_TILE + 4 * h;
    float *dst = grid + (int64_t)dm * plane + (int64_t)y * g.nx + x0 + 4 * h;
    if (full) {
      *reinterpret_cast<float4 *>(dst) = make_float4(src[0], src[1], src[2], src[3]);
    } else if (y < g.ny) {
      for (int e = 0; e < 4; ++e)
        if (x0 + 4 * h + e < g.nx) dst[e] = src[e];
    }
  }
}

// Particles whose fused window is not interior: list[0..count) (count at *count).
template <typename R>
__global__ void k_edge_list(int64_t N, Stencils<R> sm, int dend, int nz, int *count, int *list) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= N) return;
  if (!fused_interior(sm.cell[p], dend, nz)) list[atomicAdd(count, 1)] = (int)p;
}

template <typename R>
void launch_edge_list(int64_t N, const Stencils<R> &sm, const KernelDesc &km, int nz, int *count, int *list,
                      cudaStream_t s) {
  if (N == 0) return;
  k_edge_list<R><<<(unsigned)((N + 255) / 256), 256, 0, s>>>(N, sm, km.dend, nz, count, list);
}

// nz <= 128: the block fits in shared memory; wx, wy <= 14: stencils reach
// one tile at most; z windows of at most 64 nodes (two per lane); more than
// two tiles per axis: the 3 x 3 neighbourhood holds nine distinct tiles.
bool tile_spread_supported(const KernelDesc &km, const KernelDesc &kd, int nx, int ny, int nz) {
  return nz <= 128 && km.wx <= 14 && km.wy <= 14 && km.wz_max <= 64 && kd.wz_max <= 64 &&
         nx > 2 * ORDER_TILE && ny > 2 * ORDER_TILE;
}

size_t tile_spread_smem(int nz) { return sizeof(float) * 3 * (size_t)nz * ORDER_TILE * ORDER_TILE; }

cudaError_t tile_spread_setup(int nz) {
  cudaError_t e = cudaFuncSetAttribute(k_spread_tiles<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)tile_spread_smem(nz));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_spread_tiles<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)tile_spread_smem(nz));
  return e;
}

// The whole grid written by the tiles (no clearing needed); then the edge
// particles' contributions added with atomics (ghost layers, folds).
template <typename RF>
void launch_spread_tiles(const RF *F, const RF *T, const KernelDesc &km, const KernelDesc &kd, const GridArgs &g,
                         const Stencils<float> &sm, const Stencils<float> &sd, float *grid, const Ghosts<float> &ghm,
                         const Ghosts<float> &ghd, const int *perm, const int *tstart, const int *edge,
                         int64_t n_edge, cudaStream_t s) {
  const int ntx = (g.nx + ORDER_TILE - 1) / ORDER_TILE, nty = (g.ny + ORDER_TILE - 1) / ORDER_TILE;
  k_spread_tiles<RF><<<(unsigned)(ntx * nty), TILE_SPREAD_THREADS, tile_spread_smem(g.nz), s>>>(
      F, T, km, kd, g, sm, sd, grid, perm, tstart, ntx, nty);
  if (n_edge > 0) launch_spread_fused<float, RF>(F, T, n_edge, km, kd, g, sm, sd, grid, ghm, ghd, s, edge);
}

// ---------------------------------------------------------------------------
// Periodic x then y fold of the ghost-layer buffers, applied to every stored
// level exactly as the reference folds its whole extended grid
// (BoundaryConditions.h:43-84 then 143-184): x ghosts are added into the
// interior x range for every row (y ghosts included); then y ghost rows are
// added into interior rows for every column (x ghosts included).  Ghost
// cells themselves keep their raw values.
// ---------------------------------------------------------------------------
template <typename R>
static __device__ __forceinline__ void ghost_fold_x_item(int64_t t, R *buf, int levels, int nx,
                                                         const KernelDesc &kd) {
  int64_t per = (int64_t)kd.nyeff * kd.lend * 3;
  if (t >= levels * per * 2) return;
  int side = (int)(t / (levels * per));
  int64_t r = t - side * levels * per;
  int d = (int)(r % 3);
  int64_t q = r / 3;
  int i = (int)(q % kd.lend);
  int64_t q2 = q / kd.lend;
  int j = (int)(q2 % kd.nyeff);
  int l = (int)(q2 / kd.nyeff);
  R *row = buf + ((int64_t)l * kd.nyeff + j) * kd.nxeff * 3;
  int rbeg = kd.nxeff - kd.lend;
  if (side == 0) row[(i + nx) * 3 + d] += row[i * 3 + d];
  else row[(rbeg + i - nx) * 3 + d] += row[(rbeg + i) * 3 + d];
}

template <typename R>
__global__ void k_ghost_fold_x(R *buf, int levels, int nx, KernelDesc kd) {
  ghost_fold_x_item<R>(blockIdx.x * (int64_t)blockDim.x + threadIdx.x, buf, levels, nx, kd);
}

template <typename R>
static __device__ __forceinline__ void ghost_fold_y_item(int64_t t, R *buf, int levels, int ny,
                                                         const KernelDesc &kd) {
  int64_t per = (int64_t)kd.bend * kd.nxeff * 3;
  if (t >= levels * per * 2) return;
  int side = (int)(t / (levels * per));
  int64_t r = t - side * levels * per;
  int d = (int)(r % 3);
  int64_t q = r / 3;
  int i = (int)(q % kd.nxeff);
  int64_t q2 = q / kd.nxeff;
  int j = (int)(q2 % kd.bend);
  int l = (int)(q2 / kd.bend);
  R *lev = buf + (int64_t)l * kd.nyeff * kd.nxeff * 3;
  int tbeg = kd.nyeff - kd.bend;
  if (side == 0) lev[((int64_t)(j + ny) * kd.nxeff + i) * 3 + d] += lev[((int64_t)j * kd.nxeff + i) * 3 + d];
  else lev[((int64_t)(tbeg + j - ny) * kd.nxeff + i) * 3 + d] +=
      lev[((int64_t)(tbeg + j) * kd.nxeff + i) * 3 + d];
}

template <typename R>
__global__ void k_ghost_fold_y(R *buf, int levels, int ny, KernelDesc kd) {
  ghost_fold_y_item<R>(blockIdx.x * (int64_t)blockDim.x + threadIdx.x, buf, levels, ny, kd);
}

// ---------------------------------------------------------------------------
// Monopole interpolation: one warp per particle, V = sum u * phi * hx hy w_cc.
// ---------------------------------------------------------------------------
template <typename R, typename RV>
static __device__ __forceinline__ void interp_mono_item(int64_t p, int lane, const R *__restrict__ grid,
                                                     const KernelDesc &kd, const GridArgs &g,
                                                     const Stencils<R> &st, const Ghosts<R> &gh,
                                                     RV *__restrict__ V) {
  int4 cl = st.cell[p];
  R s0 = 0, s1 = 0, s2 = 0;
  if (cl.w > 0) {
    const int cols = kd.wx * kd.wy;
    const int tot = cols * cl.w;
    const int64_t plane = (int64_t)g.nx * g.ny, comp = plane * g.nz;
    for (int t = lane; t < tot; t += 32) {
      int k = t / cols;
      int c = t - k * cols;
      int i = c % kd.wx, j = c / kd.wx;
      const int ox = cl.x + i - kd.wx / 2 + kd.evenx;
      const int oy = cl.y + j - kd.wy / 2 + kd.eveny;
      const int64_t col = (int64_t)wrapi(oy, g.ny) * g.nx + wrapi(ox, g.nx);
      ZMap zm = zmap(cl.z + k, kd.dend, g.nz, g.bcA);
      R u[3];
      grid_value3(grid, zm, col, plane, comp, gh, kd, ox + kd.lend, oy + kd.bend, u);
      const R wgt = st.phx[p * kd.wx + i] * st.phy[p * kd.wy + j] * st.phzw[p * kd.wz_max + k];
      s0 += u[0] * wgt;
      s1 += u[1] * wgt;
      s2 += u[2] * wgt;
    }
  }
  s0 = warp_sum(s0);
  s1 = warp_sum(s1);
  s2 = warp_sum(s2);
  if (lane == 0) {
    V[3 * p] = (RV)s0;
    V[3 * p + 1] = (RV)s1;
    V[3 * p + 2] = (RV)s2;
  }
}

// perm (optional): the order in which warps take particles (sorted by tile,
// for locality of the grid reads).
template <typename R, typename RV>
__global__ void k_interp_mono(const R *__restrict__ grid, int64_t N, KernelDesc kd, GridArgs g,
                            Stencils<R> st, Ghosts<R> gh, RV *__restrict__ V, const int *__restrict__ perm) {
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (w >= N) return;
  const int64_t p = perm ? (int64_t)perm[w] : w;
  interp_mono_item<R, RV>(p, threadIdx.x & 31, grid, kd, g, st, gh, V);
}

// ---------------------------------------------------------------------------
// Dipole interpolation of the velocity gradient with derivative kernels and
// W = -1/2 curl v (FCM.py:411-426): d/dx, d/dy use BC set A, d/dz set B.
// ---------------------------------------------------------------------------
template <typename R, typename RV>
static __device__ __forceinline__ void interp_dip_item(int64_t p, int lane, const R *__restrict__ grid,
                                                     const KernelDesc &kd, const GridArgs &g,
                                                     const Stencils<R> &st, const Ghosts<R> &gh,
                                                     RV *__restrict__ W) {
  int4 cl = st.cell[p];
  // gradient terms needed for the curl
  R dyvz = 0, dzvy = 0, dzvx = 0, dxvz = 0, dxvy = 0, dyvx = 0;
  if (cl.w > 0) {
    const int cols = kd.wx * kd.wy;
    const int tot = cols * cl.w;
    const int64_t plane = (int64_t)g.nx * g.ny, comp = plane * g.nz;
    for (int t = lane; t < tot; t += 32) {
      int k = t / cols;
      int c = t - k * cols;
      int i = c % kd.wx, j = c / kd.wx;
      const int ox = cl.x + i - kd.wx / 2 + kd.evenx;
      const int oy = cl.y + j - kd.wy / 2 + kd.eveny;
      const int64_t col = (int64_t)wrapi(oy, g.ny) * g.nx + wrapi(ox, g.nx);
      const int kk = cl.z + k;
      ZMap za = zmap(kk, kd.dend, g.nz, g.bcA);
      ZMap zb = zmap(kk, kd.dend, g.nz, g.bcB);
      R ua[3], ub[3];
      grid_value3(grid, za, col, plane, comp, gh, kd, ox + kd.lend, oy + kd.bend, ua);
      grid_value3(grid, zb, col, plane, comp, gh, kd, ox + kd.lend, oy + kd.bend, ub);
      const R fx = st.phx[p * kd.wx + i], fy = st.phy[p * kd.wy + j];
      const R dfx = st.dphx[p * kd.wx + i], dfy = st.dphy[p * kd.wy + j];
      const R zw = st.phzw[p * kd.wz_max + k], dzw = st.dphzw[p * kd.wz_max + k];
      const R wx = dfx * fy * zw, wy = fx * dfy * zw, wz = fx * fy * dzw;
      dxvy += ua[1] * wx;
      dxvz += ua[2] * wx;
      dyvx += ua[0] * wy;
      dyvz += ua[2] * wy;
      dzvx += ub[0] * wz;
      dzvy += ub[1] * wz;
    }
  }
  dyvz = warp_sum(dyvz);
  dzvy = warp_sum(dzvy);
  dzvx = warp_sum(dzvx);
  dxvz = warp_sum(dxvz);
  dxvy = warp_sum(dxvy);
  dyvx = warp_sum(dyvx);
  if (lane == 0) {
    W[3 * p] = (RV)(-(R)0.5 * (dyvz - dzvy));
    W[3 * p + 1] = (RV)(-(R)0.5 * (dzvx - dxvz));
    W[3 * p + 2] = (RV)(-(R)0.5 * (dxvy - dyvx));
  }
}

// perm (optional): the order in which warps take particles (sorted by tile,
// for locality of the grid reads).
template <typename R, typename RV>
__global__ void k_interp_dip(const R *__restrict__ grid, int64_t N, KernelDesc kd, GridArgs g,
                            Stencils<R> st, Ghosts<R> gh, RV *__restrict__ W, const int *__restrict__ perm) {
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (w >= N) return;
  const int64_t p = perm ? (int64_t)perm[w] : w;
  interp_dip_item<R, RV>(p, threadIdx.x & 31, grid, kd, g, st, gh, W);
}

// ---------------------------------------------------------------------------
// Fused monopole + dipole interpolation (kernel pairs as for the fused
// spread): one warp per particle walks the monopole window once; an interior
// grid value read for the monopole also serves the dipole's set-A (and, when
// set B maps the node identically, set-B) derivatives.
// ---------------------------------------------------------------------------
template <typename R, typename RV>
static __device__ __forceinline__ void interp_fused_item(int64_t p, int lane, const R *__restrict__ grid,
                                                         const KernelDesc &km, const KernelDesc &kd,
                                                         const GridArgs &g, const Stencils<R> &sm,
                                                         const Stencils<R> &sd, const Ghosts<R> &ghm,
                                                         const Ghosts<R> &ghd, RV *__restrict__ V,
                                                         RV *__restrict__ W) {
  const int4 cm = sm.cell[p];
  const int4 cd = sd.cell[p];
  R s0 = 0, s1 = 0, s2 = 0;
  R dyvz = 0, dzvy = 0, dzvx = 0, dxvz = 0, dxvy = 0, dyvx = 0;
  if (cm.w > 0) {
    const int cols = km.wx * km.wy;
    const int tot = cols * cm.w;
    const int64_t plane = (int64_t)g.nx * g.ny, comp = plane * g.nz;
    for (int t = lane; t < tot; t += 32) {
      const int k = t / cols;
      const int c = t - k * cols;
      const int i = c % km.wx, j = c / km.wx;
      const int ox = cm.x + i - km.wx / 2 + km.evenx;
      const int oy = cm.y + j - km.wy / 2 + km.eveny;
      const int64_t col = (int64_t)wrapi(oy, g.ny) * g.nx + wrapi(ox, g.nx);
      const int kk = cm.z + k;
      const ZMap za = zmap(kk, km.dend, g.nz, g.bcA);
      R u[3];
      grid_value3(grid, za, col, plane, comp, ghm, km, ox + km.lend, oy + km.bend, u);
      const R wgt = sm.phx[p * km.wx + i] * sm.phy[p * km.wy + j] * sm.phzw[p * km.wz_max + k];
      s0 += u[0] * wgt;
      s1 += u[1] * wgt;
      s2 += u[2] * wgt;
      const int kq = kk - cd.z;
      if (kq >= 0 && kq < cd.w) {
        const ZMap zb = zmap(kk, kd.dend, g.nz, g.bcB);
        R ua[3], ub[3];
        if (za.m >= 0) {
          ua[0] = u[0];
          ua[1] = u[1];
          ua[2] = u[2];
        } else {
          grid_value3(grid, za, col, plane, comp, ghd, kd, ox + kd.lend, oy + kd.bend, ua);
        }
        if (zb.m >= 0 && zb.m == za.m && zb.wgt == za.wgt) {
          ub[0] = u[0];
          ub[1] = u[1];
        } else {
          grid_value3(grid, zb, col, plane, comp, ghd, kd, ox + kd.lend, oy + kd.bend, ub);
        }
        const R fx = sd.phx[p * kd.wx + i], fy = sd.phy[p * kd.wy + j];
        const R dfx = sd.dphx[p * kd.wx + i], dfy = sd.dphy[p * kd.wy + j];
        const R zw = sd.phzw[p * kd.wz_max + kq], dzw = sd.dphzw[p * kd.wz_max + kq];
        const R wx = dfx * fy * zw, wy = fx * dfy * zw, wz = fx * fy * dzw;
        dxvy += ua[1] * wx;
        dxvz += ua[2] * wx;
        dyvx += ua[0] * wy;
        dyvz += ua[2] * wy;
        dzvx += ub[0] * wz;
        dzvy += ub[1] * wz;
      }
    }
  }
  s0 = warp_sum(s0);
  s1 = warp_sum(s1);
  s2 = warp_sum(s2);
  dyvz = warp_sum(dyvz);
  dzvy = warp_sum(dzvy);
  dzvx = warp_sum(dzvx);
  dxvz = warp_sum(dxvz);
  dxvy = warp_sum(dxvy);
  dyvx = warp_sum(dyvx);
  if (lane == 0) {
    V[3 * p] = (RV)s0;
    V[3 * p + 1] = (RV)s1;
    V[3 * p + 2] = (RV)s2;
    W[3 * p] = (RV)(-(R)0.5 * (dyvz - dzvy));
    W[3 * p + 1] = (RV)(-(R)0.5 * (dzvx - dxvz));
    W[3 * p + 2] = (RV)(-(R)0.5 * (dxvy - dyvx));
  }
}

// Interior fast path of the fused interpolation (every window node an
// interior node of weight 1 under both BC sets, at most INTERP_TAB_COLS
// stencil columns): the warp first tabulates, per stencil column, the wrapped
// grid column and the x-y weights of both kernels in shared memory, then
// walks the (z level, column) cells with an incremental index, so that the
// per-cell work is three grid loads and the weighted sums.
constexpr int INTERP_TAB_COLS = 64;
constexpr int INTERP_WARPS = 8;

template <typename R>
struct InterpTab {
  int col[INTERP_TAB_COLS];
  R wm[INTERP_TAB_COLS], wdx[INTERP_TAB_COLS], wdy[INTERP_TAB_COLS], wdz[INTERP_TAB_COLS];
};

template <typename R, typename RV>
static __device__ __forceinline__ void interp_fused_interior(int64_t p, int lane, const R *__restrict__ grid,
                                                             const KernelDesc &km, const KernelDesc &kd,
                                                             const GridArgs &g, const Stencils<R> &sm,
                                                             const Stencils<R> &sd, int4 cm, int4 cd,
                                                             InterpTab<R> &tb, RV *__restrict__ V,
                                                             RV *__restrict__ W) {
  const int cols = km.wx * km.wy;
  for (int c = lane; c < cols; c += 32) {
    const int i = c % km.wx, j = c / km.wx;
    const int ox = cm.x + i - km.wx / 2 + km.evenx;
    const int oy = cm.y + j - km.wy / 2 + km.eveny;
    tb.col[c] = wrapi(oy, g.ny) * g.nx + wrapi(ox, g.nx);
    tb.wm[c] = sm.phx[p * km.wx + i] * sm.phy[p * km.wy + j];
    const R fx = sd.phx[p * kd.wx + i], fy = sd.phy[p * kd.wy + j];
    tb.wdx[c] = sd.dphx[p * kd.wx + i] * fy;
    tb.wdy[c] = fx * sd.dphy[p * kd.wy + j];
    tb.wdz[c] = fx * fy;
  }
  __syncwarp();
  const int64_t plane = (int64_t)g.nx * g.ny, comp = plane * g.nz;
  const R *__restrict__ base = grid + (int64_t)(cm.z - km.dend) * plane;
  const R *__restrict__ zwm = sm.phzw + p * km.wz_max;
  const int dk = cm.z - cd.z;
  const R *__restrict__ zwd = sd.phzw + p * kd.wz_max + dk;
  const R *__restrict__ dzwd = sd.dphzw + p * kd.wz_max + dk;
  const int k0 = max(-dk, 0), k1 = min(cd.w - dk, cm.w);
  R s0 = 0, s1 = 0, s2 = 0;
  R dyvz = 0, dzvy = 0, dzvx = 0, dxvz = 0, dxvy = 0, dyvx = 0;
  const int tot = cols * cm.w;
  int k = lane / cols, c = lane - k * cols;
  for (int t = lane; t < tot; t += 32) {
    const R *src = base + (int64_t)k * plane + tb.col[c];
    const R u0 = src[0], u1 = src[comp], u2 = src[2 * comp];
    const R wgt = tb.wm[c] * zwm[k];
    s0 += u0 * wgt;
    s1 += u1 * wgt;
    s2 += u2 * wgt;
    if (k >= k0 && k < k1) {
      const R zw = zwd[k];
      const R wx = tb.wdx[c] * zw, wy = tb.wdy[c] * zw, wz = tb.wdz[c] * dzwd[k];
      dxvy += u1 * wx;
      dxvz += u2 * wx;
      dyvx += u0 * wy;
      dyvz += u2 * wy;
      dzvx += u0 * wz;
      dzvy += u1 * wz;
    }
    c += 32;
    while (c >= cols) {
      c -= cols;
      ++k;
    }
  }
  s0 = warp_sum(s0);
  s1 = warp_sum(s1);
  s2 = warp_sum(s2);
  dyvz = warp_sum(dyvz);
  dzvy = warp_sum(dzvy);
  dzvx = warp_sum(dzvx);
  dxvz = warp_sum(dxvz);
  dxvy = warp_sum(dxvy);
  dyvx = warp_sum(dyvx);
  if (lane == 0) {
    V[3 * p] = (RV)s0;
    V[3 * p + 1] = (RV)s1;
    V[3 * p + 2] = (RV)s2;
    W[3 * p] = (RV)(-(R)0.5 * (dyvz - dzvy));
    W[3 * p + 1] = (RV)(-(R)0.5 * (dzvx - dxvz));
    W[3 * p + 2] = (RV)(-(R)0.5 * (dxvy - dyvx));
  }
}

template <typename R, typename RV>
__global__ void __launch_bounds__(32 * INTERP_WARPS, sizeof(R) == 4 ? 4 : 1) k_interp_fused(const R *__restrict__ grid, int64_t N, KernelDesc km,
                                                                    KernelDesc kd, GridArgs g, Stencils<R> sm,
                                                                    Stencils<R> sd, Ghosts<R> ghm, Ghosts<R> ghd,
                                                                    RV *__restrict__ V, RV *__restrict__ W,
                                                                    const int *__restrict__ perm) {
  __shared__ InterpTab<R> tabs[INTERP_WARPS];
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (w >= N) return;
  const int64_t p = perm ? (int64_t)perm[w] : w;
  const int lane = threadIdx.x & 31;
  const int4 cm = sm.cell[p];
  const int m0 = cm.z - km.dend;
  if (cm.w > 0 && km.wx * km.wy <= INTERP_TAB_COLS && m0 >= 1 && m0 + cm.w <= g.nz - 1) {
    interp_fused_interior<R, RV>(p, lane, grid, km, kd, g, sm, sd, cm, sd.cell[p], tabs[threadIdx.x >> 5], V, W);
  } else {
    interp_fused_item<R, RV>(p, lane, grid, km, kd, g, sm, sd, ghm, ghd, V, W);
  }
}

// ---------------------------------------------------------------------------
// Batched systems (dpst_batched_*): one launch over the particles (or
// particle-columns, or ghost cells) of every system.  prefix[s] is the first
// work item of system s (prefix[S] = total); an item finds its system by
// binary search and runs the single-system item with that system's tables.
// ---------------------------------------------------------------------------
template <typename R, bool DIPOLE>
__global__ void k_locate_b(const double *__restrict__ pos, const SysP<R> *__restrict__ sys,
                           const int64_t *__restrict__ pprefix, int S, const double *__restrict__ zext,
                           const double *__restrict__ wext, int *err, int *reach) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= __ldg(pprefix + S)) return;
  const int s = find_sys(pprefix, S, t);
  const SysP<R> &y = sys[s];
  locate_item<R, DIPOLE>(t - y.pbase, pos + 3 * y.pbase, DIPOLE ? y.kd : y.km, zext, wext, y.g,
                         DIPOLE ? y.std_ : y.stm, err, reach + 2 * s);
}

template <typename R, typename RF, bool DIP>
__global__ void k_spread_b(const RF *__restrict__ FT, const SysP<R> *__restrict__ sys,
                           const int64_t *__restrict__ iprefix, int S) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= __ldg(iprefix + S)) return;
  const int s = find_sys(iprefix, S, t);
  const SysP<R> &y = sys[s];
  const int cols = DIP ? y.kd.wx * y.kd.wy : y.km.wx * y.km.wy;
  const int64_t loc = t - __ldg(iprefix + s);
  const int64_t p = loc / cols;
  const int c = (int)(loc - p * cols);
  if (DIP) spread_dip_item<R, RF>(p, c, FT + 3 * y.pbase, y.kd, y.g, y.std_, y.grid, y.ghd);
  else spread_mono_item<R, RF>(p, c, FT + 3 * y.pbase, y.km, y.g, y.stm, y.grid, y.ghm);
}

template <typename R, bool YAXIS>
__global__ void k_ghost_fold_b(const FoldJob<R> *__restrict__ jobs, const int64_t *__restrict__ jprefix, int J) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= __ldg(jprefix + J)) return;
  const int j = find_sys(jprefix, J, t);
  const FoldJob<R> &f = jobs[j];
  const int64_t loc = t - __ldg(jprefix + j);
  if (YAXIS) ghost_fold_y_item<R>(loc, f.buf, f.levels, f.ny, f.kd);
  else ghost_fold_x_item<R>(loc, f.buf, f.levels, f.nx, f.kd);
}

// One warp per particle of the concatenated arrays.  dip_ghosts = false
// reads no ghost layers in the vorticity (the forward had no torques).
template <typename R, typename RV, bool DIP>
__global__ void k_interp_b(const SysP<R> *__restrict__ sys, const int64_t *__restrict__ pprefix, int S,
                           RV *__restrict__ out, int dip_ghosts) {
  const int64_t p = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (p >= __ldg(pprefix + S)) return;
  const int s = find_sys(pprefix, S, p);
  const SysP<R> &y = sys[s];
  if (DIP) {
    Ghosts<R> gz = y.ghd;
    if (!dip_ghosts) gz.top = gz.bot = nullptr;
    interp_dip_item<R, RV>(p - y.pbase, threadIdx.x & 31, y.grid, y.kd, y.g, y.std_, gz, out + 3 * y.pbase);
  } else {
    interp_mono_item<R, RV>(p - y.pbase, threadIdx.x & 31, y.grid, y.km, y.g, y.stm, y.ghm, out + 3 * y.pbase);
  }
}

template <typename R>
void launch_locate_b(bool dipole, const double *pos, int64_t total, const SysP<R> *sys, const int64_t *pprefix,
                     int S, const double *zext, const double *wext, int *err, int *reach, cudaStream_t s) {
  if (total == 0) return;
  const int bs = 128;
  const int64_t nb = (total + bs - 1) / bs;
  if (dipole) k_locate_b<R, true><<<nb, bs, 0, s>>>(pos, sys, pprefix, S, zext, wext, err, reach);
  else k_locate_b<R, false><<<nb, bs, 0, s>>>(pos, sys, pprefix, S, zext, wext, err, reach);
}

template <typename R, typename RF>
void launch_spread_b(bool dipole, const RF *FT, int64_t items, const SysP<R> *sys, const int64_t *iprefix, int S,
                     cudaStream_t s) {
  if (items == 0) return;
  const int bs = 256;
  const int64_t nb = (items + bs - 1) / bs;
  if (dipole) k_spread_b<R, RF, true><<<nb, bs, 0, s>>>(FT, sys, iprefix, S);
  else k_spread_b<R, RF, false><<<nb, bs, 0, s>>>(FT, sys, iprefix, S);
}

template <typename R>
void launch_ghost_fold_b(bool yaxis, const FoldJob<R> *jobs, const int64_t *jprefix, int J, int64_t items,
                         cudaStream_t s) {
  if (items == 0 || J == 0) return;
  const int bs = 256;
  const int64_t nb = (items + bs - 1) / bs;
  if (yaxis) k_ghost_fold_b<R, true><<<nb, bs, 0, s>>>(jobs, jprefix, J);
  else k_ghost_fold_b<R, false><<<nb, bs, 0, s>>>(jobs, jprefix, J);
}

template <typename R, typename RV>
void launch_interp_b(bool dipole, int64_t total, const SysP<R> *sys, const int64_t *pprefix, int S, RV *out,
                     bool dip_ghosts, cudaStream_t s) {
  if (total == 0) return;
  const int bs = 256;
  const int64_t nb = (total * 32 + bs - 1) / bs;
  if (dipole) k_interp_b<R, RV, true><<<nb, bs, 0, s>>>(sys, pprefix, S, out, dip_ghosts ? 1 : 0);
  else k_interp_b<R, RV, false><<<nb, bs, 0, s>>>(sys, pprefix, S, out, 0);
}

#define DPST_BATCH_INST(R, RF)                                                                          \
  template void launch_spread_b<R, RF>(bool, const RF *, int64_t, const SysP<R> *, const int64_t *, int, \
                                       cudaStream_t);                                                   \
  template void launch_interp_b<R, RF>(bool, int64_t, const SysP<R> *, const int64_t *, int, RF *, bool,  \
                                       cudaStream_t);
DPST_BATCH_INST(float, float)
DPST_BATCH_INST(float, double)
DPST_BATCH_INST(double, float)
DPST_BATCH_INST(double, double)
template void launch_locate_b<float>(bool, const double *, int64_t, const SysP<float> *, const int64_t *, int,
                                     const double *, const double *, int *, int *, cudaStream_t);
template void launch_locate_b<double>(bool, const double *, int64_t, const SysP<double> *, const int64_t *, int,
                                      const double *, const double *, int *, int *, cudaStream_t);
template void launch_ghost_fold_b<float>(bool, const FoldJob<float> *, const int64_t *, int, int64_t, cudaStream_t);
template void launch_ghost_fold_b<double>(bool, const FoldJob<double> *, const int64_t *, int, int64_t,
                                          cudaStream_t);

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
template <typename R>
void launch_locate(bool dipole, const double *pos, int64_t N, const KernelDesc &kd,
                   const double *zext, const double *wext, const GridArgs &g, const Stencils<R> &st,
                   int *err, int *reach, cudaStream_t s) {
  if (N == 0) return;
  int bs = 128;
  int64_t nb = (N + bs - 1) / bs;
  if (dipole) k_locate<R, true><<<nb, bs, 0, s>>>(pos, N, kd, zext, wext, g, st, err, reach);
  else k_locate<R, false><<<nb, bs, 0, s>>>(pos, N, kd, zext, wext, g, st, err, reach);
}

template <typename R, typename RF>
void launch_spread(bool dipole, const RF *FT, int64_t N, const KernelDesc &kd, const GridArgs &g,
                   const Stencils<R> &st, R *grid, const Ghosts<R> &gh, cudaStream_t s, const int *perm) {
  int64_t tot = N * kd.wx * kd.wy;
  if (tot == 0) return;
  int bs = 256;
  int64_t nb = (tot + bs - 1) / bs;
  if (dipole) k_spread_dip<R, RF><<<nb, bs, 0, s>>>(FT, N, kd, g, st, grid, gh, perm);
  else k_spread_mono<R, RF><<<nb, bs, 0, s>>>(FT, N, kd, g, st, grid, gh, perm);
}

// ---------------------------------------------------------------------------
// Particle order by grid tile (once per set of positions): a counting sort of
// the particles by the ORDER_TILE x ORDER_TILE column tile of their cell, so
// that the spread's and the interpolation's neighbouring threads touch
// neighbouring grid cells.  count holds ntiles ints, start ntiles + 1.
// ---------------------------------------------------------------------------

template <typename R, bool FILL>
__global__ void k_tile_order(int64_t N, GridArgs g, Stencils<R> st, int ntx, int *count, const int *start,
                             int *perm) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= N) return;
  const int4 cl = st.cell[p];
  const int t = (wrapi(cl.y, g.ny) / ORDER_TILE) * ntx + wrapi(cl.x, g.nx) / ORDER_TILE;
  const int pos = atomicAdd(&count[t], 1);
  if (FILL) perm[start[t] + pos] = (int)p;
}

// Exclusive prefix sum of n counts in one CTA of 1024 threads: start[0..n].
__global__ void __launch_bounds__(1024) k_scan_counts(const int *__restrict__ count, int n, int *__restrict__ start) {
  __shared__ int part[1024];
  const int tid = threadIdx.x, chunk = (n + 1023) / 1024;
  const int b = tid * chunk, e = min(b + chunk, n);
  int sum = 0;
  for (int i = b; i < e; ++i) sum += count[i];
  part[tid] = sum;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const int v = (tid >= o) ? part[tid - o] : 0;
    __syncthreads();
    part[tid] += v;
    __syncthreads();
  }
  int run = part[tid] - sum;
  for (int i = b; i < e; ++i) {
    start[i] = run;
    run += count[i];
  }
  if (tid == 1023) start[n] = part[1023];
}

template <typename R>
void launch_tile_order(int64_t N, const GridArgs &g, const Stencils<R> &st, int *count, int *start, int *perm,
                       cudaStream_t s) {
  if (N == 0) return;
  const int ntx = (g.nx + ORDER_TILE - 1) / ORDER_TILE, nty = (g.ny + ORDER_TILE - 1) / ORDER_TILE;
  const int ntiles = ntx * nty;
  const int bs = 256;
  const int64_t nb = (N + bs - 1) / bs;
  cudaMemsetAsync(count, 0, sizeof(int) * ntiles, s);
  k_tile_order<R, false><<<nb, bs, 0, s>>>(N, g, st, ntx, count, nullptr, nullptr);
  k_scan_counts<<<1, 1024, 0, s>>>(count, ntiles, start);
  cudaMemsetAsync(count, 0, sizeof(int) * ntiles, s);
  k_tile_order<R, true><<<nb, bs, 0, s>>>(N, g, st, ntx, count, start, perm);
}

size_t tile_order_tiles(int nx, int ny) {
  return (size_t)((nx + ORDER_TILE - 1) / ORDER_TILE) * ((ny + ORDER_TILE - 1) / ORDER_TILE);
}

template <typename R>
void launch_ghost_fold(R *buf, int levels, int nx, int ny, const KernelDesc &kd, cudaStream_t s) {
  if (buf == nullptr || levels <= 0) return;
  int bs = 256;
  int64_t tx = (int64_t)levels * kd.nyeff * kd.lend * 3 * 2;
  if (tx > 0) k_ghost_fold_x<R><<<(tx + bs - 1) / bs, bs, 0, s>>>(buf, levels, nx, kd);
  int64_t ty = (int64_t)levels * kd.bend * kd.nxeff * 3 * 2;
  if (ty > 0) k_ghost_fold_y<R><<<(ty + bs - 1) / bs, bs, 0, s>>>(buf, levels, ny, kd);
}

// The fused spread / interpolation apply to a monopole / dipole kernel pair
// with the same x-y stencil columns and extended z grid and a dipole
// threshold no larger than the monopole's (on a uniform periodic z grid: the
// same z width, so that both windows start at the same node).
bool fused_supports(const KernelDesc &km, const KernelDesc &kd) {
  return km.wx == kd.wx && km.wy == kd.wy && km.evenx == kd.evenx && km.eveny == kd.eveny &&
         km.nxeff == kd.nxeff && km.nyeff == kd.nyeff && km.lend == kd.lend && km.bend == kd.bend &&
         km.nzeff == kd.nzeff && km.dend == kd.dend && kd.thr <= km.thr && km.unif_z == kd.unif_z &&
         (!km.unif_z || (km.wz_max == kd.wz_max && km.evenz == kd.evenz));
}

template <typename R, typename RF>
void launch_spread_fused(const RF *F, const RF *T, int64_t N, const KernelDesc &km, const KernelDesc &kd,
                         const GridArgs &g, const Stencils<R> &sm, const Stencils<R> &sd, R *grid,
                         const Ghosts<R> &ghm, const Ghosts<R> &ghd, cudaStream_t s, const int *perm) {
  const int64_t tot = N * km.wx * km.wy;
  if (tot == 0) return;
  const int bs = 256;
  k_spread_fused<R, RF><<<(tot + bs - 1) / bs, bs, 0, s>>>(F, T, N, km, kd, g, sm, sd, grid, ghm, ghd, perm);
}

template <typename R, typename RV>
void launch_interp_fused(const R *grid, int64_t N, const KernelDesc &km, const KernelDesc &kd, const GridArgs &g,
                         const Stencils<R> &sm, const Stencils<R> &sd, const Ghosts<R> &ghm,
                         const Ghosts<R> &ghd, RV *V, RV *W, cudaStream_t s, const int *perm) {
  if (N == 0) return;
  const int bs = 32 * INTERP_WARPS;
  k_interp_fused<R, RV><<<(N * 32 + bs - 1) / bs, bs, 0, s>>>(grid, N, km, kd, g, sm, sd, ghm, ghd, V, W, perm);
}

template <typename R, typename RV>
void launch_interp(bool dipole, const R *grid, int64_t N, const KernelDesc &kd, const GridArgs &g,
                   const Stencils<R> &st, const Ghosts<R> &gh, RV *out, cudaStream_t s, const int *perm) {
  if (N == 0) return;
  int bs = 256;
  int64_t nb = (N * 32 + bs - 1) / bs;
  if (dipole) k_interp_dip<R, RV><<<nb, bs, 0, s>>>(grid, N, kd, g, st, gh, out, perm);
  else k_interp_mono<R, RV><<<nb, bs, 0, s>>>(grid, N, kd, g, st, gh, out, perm);
}

#define DPST_INST(R)                                                                           \
  template void launch_locate<R>(bool, const double *, int64_t, const KernelDesc &,             \
                                 const double *, const double *, const GridArgs &,              \
                                 const Stencils<R> &, int *, int *, cudaStream_t);              \
  template void launch_ghost_fold<R>(R *, int, int, int, const KernelDesc &, cudaStream_t);     \
  template void launch_spread<R, float>(bool, const float *, int64_t, const KernelDesc &,      \
                                        const GridArgs &, const Stencils<R> &, R *,            \
                                        const Ghosts<R> &, cudaStream_t, const int *);         \
  template void launch_spread<R, double>(bool, const double *, int64_t, const KernelDesc &,    \
                                         const GridArgs &, const Stencils<R> &, R *,           \
                                         const Ghosts<R> &, cudaStream_t, const int *);        \
  template void launch_interp<R, float>(bool, const R *, int64_t, const KernelDesc &,          \
                                        const GridArgs &, const Stencils<R> &,                 \
                                        const Ghosts<R> &, float *, cudaStream_t, const int *);\
  template void launch_interp<R, double>(bool, const R *, int64_t, const KernelDesc &,         \
                                         const GridArgs &, const Stencils<R> &,                \
                                         const Ghosts<R> &, double *, cudaStream_t, const int *);\
  template void launch_tile_order<R>(int64_t, const GridArgs &, const Stencils<R> &, int *, int *, \
                                     int *, cudaStream_t);\
  template void launch_spread_fused<R, float>(const float *, const float *, int64_t, const KernelDesc &,   \
                                              const KernelDesc &, const GridArgs &, const Stencils<R> &,  \
                                              const Stencils<R> &, R *, const Ghosts<R> &,                \
                                              const Ghosts<R> &, cudaStream_t, const int *);              \
  template void launch_spread_fused<R, double>(const double *, const double *, int64_t,                   \
                                               const KernelDesc &, const KernelDesc &, const GridArgs &,  \
                                               const Stencils<R> &, const Stencils<R> &, R *,             \
                                               const Ghosts<R> &, const Ghosts<R> &, cudaStream_t,        \
                                               const int *);                                               \
  template void launch_interp_fused<R, float>(const R *, int64_t, const KernelDesc &, const KernelDesc &,  \
                                              const GridArgs &, const Stencils<R> &, const Stencils<R> &, \
                                              const Ghosts<R> &, const Ghosts<R> &, float *, float *,     \
                                              cudaStream_t, const int *);                                 \
  template void launch_interp_fused<R, double>(const R *, int64_t, const KernelDesc &, const KernelDesc &, \
                                               const GridArgs &, const Stencils<R> &, const Stencils<R> &,\
                                               const Ghosts<R> &, const Ghosts<R> &, double *, double *,  \
                                               cudaStream_t, const int *);

DPST_INST(float)
DPST_INST(double)

template void launch_spread_tiles<float>(const float *, const float *, const KernelDesc &, const KernelDesc &,
                                         const GridArgs &, const Stencils<float> &, const Stencils<float> &, float *,
                                         const Ghosts<float> &, const Ghosts<float> &, const int *, const int *,
                                         const int *, int64_t, cudaStream_t);
template void launch_spread_tiles<double>(const double *, const double *, const KernelDesc &, const KernelDesc &,
                                          const GridArgs &, const Stencils<float> &, const Stencils<float> &,
                                          float *, const Ghosts<float> &, const Ghosts<float> &, const int *,
                                          const int *, const int *, int64_t, cudaStream_t);
template void launch_edge_list<float>(int64_t, const Stencils<float> &, const KernelDesc &, int, int *, int *,
                                      cudaStream_t);
template void launch_edge_list<double>(int64_t, const Stencils<double> &, const KernelDesc &, int, int *, int *,
                                       cudaStream_t);

}  // namespace dpst
