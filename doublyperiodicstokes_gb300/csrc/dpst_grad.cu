// Particle-side kernels of the backward pass of Mdot.
//
// The operator is V = J(X) u with u = L S(X) F (plus the open-end ghost
// path V += J_h(X) P S_h(X) F, P the x-y ghost fold), and likewise W with
// the dipole kernels.  For a loss l = <gV, V> + <gW, W>:
//   dl/dF = S^T psi (+ S_h^T P^T J_h^T gV),  psi = L^T J^T (gV, gW),
//   dl/dX_p = sum over p's stencil of (d interp weight / dX_p) (g_p . u)
//           + (d spread weight / dX_p) (F_p . psi)   (and the ghost terms).
// This file holds
//   k_locate_grad      position derivatives of the 1-D stencil factors
//   k_adj_spread_dip   J_dip^T gW (the transpose of the curl interpolation)
//                      onto the adjoint grid (J_mono^T gV is the forward's
//                      spread kernel with interpolation weights)
//   k_ghost_fold_*_t   P^T on the adjoint ghost layers
//   k_gather_mono/dip  S^T psi (dl/dF, dl/dT) and dl/dX, one warp per
//                      particle, reading the velocity grid u (recomputed by
//                      the caller) and the adjoint grid psi
// The forward counterparts are in dpst_particles.cu (same index maps and
// the same ghost rules, BoundaryConditions.h:22-731).
#include "dpst_internal.cuh"
#include "dpst_pdev.cuh"

namespace dpst {

// ---------------------------------------------------------------------------
// Position derivatives of the stencil factors, one thread per (particle,
// stencil entry): entries [0, wx) are x factors, [wx, wx + wy) y factors,
// then wz_max z factors; at the stencil k_locate chose (st.cell), with its
// offsets and clamping.
// ---------------------------------------------------------------------------
// FP64 for the FP64 operator, FP32 transcendentals for the mixed one.
template <typename R>
static __device__ __forceinline__ void pos_derivs(double o, const KernelDesc &kd, double &g1, double &g2) {
  if constexpr (sizeof(R) == 8) {
    es_pos_derivs(o, kd.beta, kd.alpha2, g1, g2);
  } else {
    float f1, f2;
    es_pos_derivs_f(o, kd.beta, kd.alpha2, kd.inv_alpha2, f1, f2);
    g1 = f1;
    g2 = f2;
  }
}

template <typename R, bool DIPOLE>
__global__ void k_locate_grad(const double *__restrict__ pos, int64_t N, KernelDesc kd,
                              const double *__restrict__ zext, const double *__restrict__ wext, GridArgs g,
                              Stencils<R> st, GradStencils<R> gs) {
  const int E = kd.wx + kd.wy + kd.wz_max;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= N * E) return;
  const int64_t p = t / E;
  const int e = (int)(t - p * E);
  const int4 cl = st.cell[p];
  const double thr = kd.thr;
  double g1 = 0.0, g2 = 0.0;
  if (e < kd.wx) {
    const double o = ((double)cl.x + e - kd.wx / 2 + kd.evenx) * g.hx - pos[3 * p];
    if (!(o > thr || o < -thr)) pos_derivs<R>(o, kd, g1, g2);
    gs.gx[p * kd.wx + e] = (R)g1;
    if (DIPOLE) gs.gdx[p * kd.wx + e] = (R)g2;
  } else if (e < kd.wx + kd.wy) {
    const int j = e - kd.wx;
    const double o = ((double)cl.y + j - kd.wy / 2 + kd.eveny) * g.hy - pos[3 * p + 1];
    if (!(thr < o || o < -thr)) pos_derivs<R>(o, kd, g1, g2);
    gs.gy[p * kd.wy + j] = (R)g1;
    if (DIPOLE) gs.gdy[p * kd.wy + j] = (R)g2;
  } else if (kd.unif_z) {  // uniform periodic z: the window of locate_item's uniform branch
    const int k = e - kd.wx - kd.wy;
    const int wz = kd.wz_max;
    const int zclose = cl.z - kd.dend + wz / 2 - kd.evenz;
    const double o = ((double)zclose + k - wz / 2 + kd.evenz) * kd.hz - pos[3 * p + 2];
    if (!(thr < o || o < -thr)) pos_derivs<R>(o, kd, g1, g2);
    g1 *= kd.inv_norm3;
    g2 *= kd.inv_norm3;
    const double wgt = g.hx * g.hy * kd.hz;
    gs.gz[p * kd.wz_max + k] = (R)g1;
    gs.gzw[p * kd.wz_max + k] = (R)(g1 * wgt);
    if (DIPOLE) {
      gs.gdz[p * kd.wz_max + k] = (R)g2;
      gs.gdzw[p * kd.wz_max + k] = (R)(g2 * wgt);
    }
  } else {
    const int k = e - kd.wx - kd.wy;
    double wgt = 0.0;
    if (k < cl.w) {
      const double o = zext[kd.zext_off + cl.z + k] - pos[3 * p + 2];
      if (!(thr < o || o < -thr)) pos_derivs<R>(o, kd, g1, g2);
      g1 *= kd.inv_norm3;
      g2 *= kd.inv_norm3;
      wgt = g.hx * g.hy * wext[kd.zext_off + cl.z + k];
    }
    gs.gz[p * kd.wz_max + k] = (R)g1;
    gs.gzw[p * kd.wz_max + k] = (R)(g1 * wgt);
    if (DIPOLE) {
      gs.gdz[p * kd.wz_max + k] = (R)g2;
      gs.gdzw[p * kd.wz_max + k] = (R)(g2 * wgt);
    }
  }
}

template <typename R>
static __device__ __forceinline__ R *ghost_cell(const Ghosts<R> &gh, const ZMap &zm, const KernelDesc &kd, int ie,
                                                int je) {
  R *buf = (zm.m == -1) ? gh.top : gh.bot;
  if (buf == nullptr || ie < 0 || ie >= kd.nxeff || je < 0 || je >= kd.nyeff) return nullptr;
  return buf + (((int64_t)zm.level * kd.nyeff + je) * kd.nxeff + ie) * 3;
}

// ---------------------------------------------------------------------------
// Transpose of the dipole interpolation W = -1/2 curl v (k_interp_dip):
// for a = gW_p and weights wx = dphx phy phzw, wy = phx dphy phzw,
// wz = phx phy dphzw, the adjoint of the bcA-mapped value is
// 1/2 (wy a2, -wx a2, wx a1 - wy a0) and of the bcB-mapped value
// 1/2 (-wz a1, wz a0, 0); interior layers take the map's weight, ghost
// layers (read raw by the forward) take them unweighted.  One thread per
// (particle, stencil column).
// ---------------------------------------------------------------------------
template <typename R, typename RG>
__global__ void k_adj_spread_dip(const RG *__restrict__ gW, int64_t N, KernelDesc kd, GridArgs g,
                                 Stencils<R> st, R *__restrict__ grid, Ghosts<R> gh) {
  const int cols = kd.wx * kd.wy;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= N * cols) return;
  const int64_t p = t / cols;
  const int c = (int)(t - p * cols);
  const int i = c % kd.wx, j = c / kd.wx;
  const int4 cl = st.cell[p];
  if (cl.w == 0) return;
  const int ox = cl.x + i - kd.wx / 2 + kd.evenx;
  const int oy = cl.y + j - kd.wy / 2 + kd.eveny;
  const int64_t col = (int64_t)wrapi(oy, g.ny) * g.nx + wrapi(ox, g.nx);
  const int ie = ox + kd.lend, je = oy + kd.bend;
  const R a0 = (R)gW[3 * p], a1 = (R)gW[3 * p + 1], a2 = (R)gW[3 * p + 2];
  const R fx = st.phx[p * kd.wx + i], fy = st.phy[p * kd.wy + j];
  const R dfx = st.dphx[p * kd.wx + i], dfy = st.dphy[p * kd.wy + j];
  const int64_t plane = (int64_t)g.nx * g.ny, comp = plane * g.nz;
  const R half = (R)0.5;
  for (int k = 0; k < cl.w; ++k) {
    const R zw = st.phzw[p * kd.wz_max + k], dzw = st.dphzw[p * kd.wz_max + k];
    const R wx = dfx * fy * zw, wy = fx * dfy * zw, wz = fx * fy * dzw;
    const R A0 = half * (wy * a2), A1 = -half * (wx * a2), A2 = half * (wx * a1 - wy * a0);
    const R B0 = -half * (wz * a1), B1 = half * (wz * a0);
    const int kk = cl.z + k;
    const ZMap za = zmap(kk, kd.dend, g.nz, g.bcA);
    const ZMap zb = zmap(kk, kd.dend, g.nz, g.bcB);
    if (za.m >= 0) {
      if (za.wgt != 0.0) {
        R *dst = grid + za.m * plane + col;
        const R w = (R)za.wgt;
        atomic_add(dst, w * A0);
        atomic_add(dst + comp, w * A1);
        atomic_add(dst + 2 * comp, w * A2);
      }
    } else if (R *dst = ghost_cell(gh, za, kd, ie, je)) {
      atomic_add(dst, A0);
      atomic_add(dst + 1, A1);
      atomic_add(dst + 2, A2);
    }
    if (zb.m >= 0) {
      if (zb.wgt != 0.0) {
        R *dst = grid + zb.m * plane + col;
        const R w = (R)zb.wgt;
        atomic_add(dst, w * B0);
        atomic_add(dst + comp, w * B1);
      }
    } else if (R *dst = ghost_cell(gh, zb, kd, ie, je)) {
      atomic_add(dst, B0);
      atomic_add(dst + 1, B1);
    }
  }
}

// ---------------------------------------------------------------------------
// Transpose of the ghost-layer fold (k_ghost_fold_x / _y): the forward adds
// ghost cells into interior cells (x fold on every row, then y fold on every
// column); the transpose adds interior cells into the ghost cells, y first.
// Sources (interior) and destinations (ghost cells) never overlap.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_ghost_fold_x_t(R *buf, int levels, int nx, KernelDesc kd) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t per = (int64_t)kd.nyeff * kd.lend * 3;
  if (t >= levels * per * 2) return;
  const int side = (int)(t / (levels * per));
  const int64_t r = t - side * levels * per;
  const int d = (int)(r % 3);
  const int64_t q = r / 3;
  const int i = (int)(q % kd.lend);
  const int64_t q2 = q / kd.lend;
  const int j = (int)(q2 % kd.nyeff);
  const int l = (int)(q2 / kd.nyeff);
  R *row = buf + ((int64_t)l * kd.nyeff + j) * kd.nxeff * 3;
  const int rbeg = kd.nxeff - kd.lend;
  if (side == 0) row[i * 3 + d] += row[(i + nx) * 3 + d];
  else row[(rbeg + i) * 3 + d] += row[(rbeg + i - nx) * 3 + d];
}

template <typename R>
__global__ void k_ghost_fold_y_t(R *buf, int levels, int ny, KernelDesc kd) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t per = (int64_t)kd.bend * kd.nxeff * 3;
  if (t >= levels * per * 2) return;
  const int side = (int)(t / (levels * per));
  const int64_t r = t - side * levels * per;
  const int d = (int)(r % 3);
  const int64_t q = r / 3;
  const int i = (int)(q % kd.nxeff);
  const int64_t q2 = q / kd.nxeff;
  const int j = (int)(q2 % kd.bend);
  const int l = (int)(q2 / kd.bend);
  R *lev = buf + (int64_t)l * kd.nyeff * kd.nxeff * 3;
  const int tbeg = kd.nyeff - kd.bend;
  if (side == 0) lev[((int64_t)j * kd.nxeff + i) * 3 + d] += lev[((int64_t)(j + ny) * kd.nxeff + i) * 3 + d];
  else lev[((int64_t)(tbeg + j) * kd.nxeff + i) * 3 + d] += lev[((int64_t)(tbeg + j - ny) * kd.nxeff + i) * 3 + d];
}

// A lane's walk over a particle's stencil items t = lane, lane + 32, ...
// (t = (k wy + j) wx + i: column (i, j), window level k) without a division
// per item: two divisions up front, then steps of 32 = qa wx + ra.
struct StencilWalk {
  int i, j, k, qa, ra;
  __device__ __forceinline__ StencilWalk(int lane, int wx, int wy) {
    const int cols = wx * wy;
    k = lane / cols;
    const int c = lane - k * cols;
    j = c / wx;
    i = c - j * wx;
    qa = 32 / wx;
    ra = 32 - qa * wx;
  }
  __device__ __forceinline__ void next(int wx, int wy) {
    i += ra;
    j += qa;
    if (i >= wx) {
      i -= wx;
      ++j;
    }
    while (j >= wy) {
      j -= wy;
      ++k;
    }
  }
};

// ---------------------------------------------------------------------------
// Monopole gather: dl/dF_p = sum phx phy phz psi (S^T, ghost layers from the
// adjoint ghost buffers) and, with gX, the position gradient
//   dl/dX_p += sum d(phx phy phzw)/dX (gV_p . u) + d(phx phy phz)/dX (F_p . psi).
// One warp per particle; u is not read without gX.
// ---------------------------------------------------------------------------
template <typename R, typename RF>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 4 : 2) k_gather_mono(const R *__restrict__ u, const R *__restrict__ psi, int64_t N, KernelDesc kd,
                              GridArgs g, Stencils<R> st, GradStencils<R> gs, Ghosts<R> ghu, Ghosts<R> ghp,
                              const RF *__restrict__ F, const RF *__restrict__ gV, RF *__restrict__ gF,
                              RF *__restrict__ gX) {
  const int64_t p = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (p >= N) return;
  const int4 cl = st.cell[p];
  const bool want_x = gX != nullptr;
  R f0 = 0, f1 = 0, f2 = 0, v0 = 0, v1 = 0, v2 = 0;
  if (want_x) {
    f0 = (R)F[3 * p];
    f1 = (R)F[3 * p + 1];
    f2 = (R)F[3 * p + 2];
    v0 = (R)gV[3 * p];
    v1 = (R)gV[3 * p + 1];
    v2 = (R)gV[3 * p + 2];
  }
  R s0 = 0, s1 = 0, s2 = 0, x0 = 0, x1 = 0, x2 = 0;
  if (cl.w > 0) {
    const int64_t plane = (int64_t)g.nx * g.ny, comp = plane * g.nz;
    StencilWalk sw(lane, kd.wx, kd.wy);
    for (; sw.k < cl.w; sw.next(kd.wx, kd.wy)) {
      const int i = sw.i, j = sw.j, k = sw.k;
      const int ox = cl.x + i - kd.wx / 2 + kd.evenx;
      const int oy = cl.y + j - kd.wy / 2 + kd.eveny;
      const int64_t col = (int64_t)wrapi(oy, g.ny) * g.nx + wrapi(ox, g.nx);
      const ZMap zm = zmap(cl.z + k, kd.dend, g.nz, g.bcA);
      R ps[3];
      grid_value3(psi, zm, col, plane, comp, ghp, kd, ox + kd.lend, oy + kd.bend, ps);
      const R fx = st.phx[p * kd.wx + i], fy = st.phy[p * kd.wy + j];
      const R fz = st.phz[p * kd.wz_max + k];
      const R w = fx * fy * fz;
      s0 += w * ps[0];
      s1 += w * ps[1];
      s2 += w * ps[2];
      if (want_x) {
        R uu[3];
        grid_value3(u, zm, col, plane, comp, ghu, kd, ox + kd.lend, oy + kd.bend, uu);
        const R a = v0 * uu[0] + v1 * uu[1] + v2 * uu[2];  // gV . u
        const R b = f0 * ps[0] + f1 * ps[1] + f2 * ps[2];  // F . psi
        const R fzw = st.phzw[p * kd.wz_max + k];
        const R gfx = gs.gx[p * kd.wx + i], gfy = gs.gy[p * kd.wy + j];
        const R gfz = gs.gz[p * kd.wz_max + k], gfzw = gs.gzw[p * kd.wz_max + k];
        const R zab = fzw * a + fz * b;
        x0 += gfx * fy * zab;
        x1 += fx * gfy * zab;
        x2 += fx * fy * (gfzw * a + gfz * b);
      }
    }
  }
  s0 = warp_sum(s0);
  s1 = warp_sum(s1);
  s2 = warp_sum(s2);
  if (want_x) {
    x0 = warp_sum(x0);
    x1 = warp_sum(x1);
    x2 = warp_sum(x2);
  }
  if (lane == 0) {
    if (gF) {
      gF[3 * p] = (RF)s0;
      gF[3 * p + 1] = (RF)s1;
      gF[3 * p + 2] = (RF)s2;
    }
    if (want_x) {
      gX[3 * p] = (RF)x0;
      gX[3 * p + 1] = (RF)x1;
      gX[3 * p + 2] = (RF)x2;
    }
  }
}

// ---------------------------------------------------------------------------
// Dipole gather.  Forward pieces (k_spread_dip, k_interp_dip) with
// ax = dphx phy phz, ay = phx dphy phz, az = phx phy dphz (spread) and
// wx, wy, wz the same with phzw / dphzw (interpolation):
//   spread  l_s = 1/2 sum (ax Pa + ay Pb + az Pc) + sum az (T . psi_ghost),
//           Pa = ty Ua2 - tz Ua1, Pb = tz Ua0 - tx Ua2, Pc = tx Ub1 - ty Ub0
//           (Ua, Ub: psi under the bcA / bcB maps, interior layers only)
//   interp  l_i = -1/2 sum (wx Qa + wy Qb + wz Qc),
//           Qa = a2 ua1 - a1 ua2, Qb = a0 ua2 - a2 ua0, Qc = a1 ub0 - a0 ub1
//           (a = gW_p; ua, ub: u under the bcA / bcB maps with ghost reads)
// dl/dT_p = d l_s / dT; dl/dX_p gets d(l_s + l_i)/dX with each factor's
// position derivative; it is added to gX (the monopole gather writes it
// first).
// ---------------------------------------------------------------------------
template <typename R, typename RF>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 3 : 2) k_gather_dip(const R *__restrict__ u, const R *__restrict__ psi, int64_t N, KernelDesc kd,
                             GridArgs g, Stencils<R> st, GradStencils<R> gs, Ghosts<R> ghu, Ghosts<R> ghp,
                             const RF *__restrict__ T, const RF *__restrict__ gW, RF *__restrict__ gT,
                             RF *__restrict__ gX) {
  const int64_t p = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (p >= N) return;
  const int4 cl = st.cell[p];
  const bool want_x = gX != nullptr;
  const bool xs = want_x && T != nullptr;   // spread part of dl/dX
  const bool xi = want_x && gW != nullptr;  // interpolation part of dl/dX
  R tx = 0, ty = 0, tz = 0, a0 = 0, a1 = 0, a2 = 0;
  if (T) {
    tx = (R)T[3 * p];
    ty = (R)T[3 * p + 1];
    tz = (R)T[3 * p + 2];
  }
  if (gW) {
    a0 = (R)gW[3 * p];
    a1 = (R)gW[3 * p + 1];
    a2 = (R)gW[3 * p + 2];
  }
  const R half = (R)0.5;
  R s0 = 0, s1 = 0, s2 = 0, x0 = 0, x1 = 0, x2 = 0;
  if (cl.w > 0) {
    const int64_t plane = (int64_t)g.nx * g.ny, comp = plane * g.nz;
    StencilWalk sw(lane, kd.wx, kd.wy);
    for (; sw.k < cl.w; sw.next(kd.wx, kd.wy)) {
      const int i = sw.i, j = sw.j, k = sw.k;
      const int ox = cl.x + i - kd.wx / 2 + kd.evenx;
      const int oy = cl.y + j - kd.wy / 2 + kd.eveny;
      const int ie = ox + kd.lend, je = oy + kd.bend;
      const int64_t col = (int64_t)wrapi(oy, g.ny) * g.nx + wrapi(ox, g.nx);
      const int kk = cl.z + k;
      const ZMap za = zmap(kk, kd.dend, g.nz, g.bcA);
      const ZMap zb = zmap(kk, kd.dend, g.nz, g.bcB);
      const R fx = st.phx[p * kd.wx + i], fy = st.phy[p * kd.wy + j];
      const R dfx = st.dphx[p * kd.wx + i], dfy = st.dphy[p * kd.wy + j];
      const R phz = st.phz[p * kd.wz_max + k], dphz = st.dphz[p * kd.wz_max + k];
      // psi as the spread's transpose reads it
      R Ua[3] = {0, 0, 0}, Ub[3] = {0, 0, 0}, Ph[3] = {0, 0, 0};
      if (za.m >= 0) grid_value3(psi, za, col, plane, comp, ghp, kd, ie, je, Ua);
      if (zb.m >= 0) grid_value3(psi, zb, col, plane, comp, ghp, kd, ie, je, Ub);
      else if (const R *src = ghost_cell(ghp, zb, kd, ie, je)) {
        Ph[0] = src[0];
        Ph[1] = src[1];
        Ph[2] = src[2];
      }
      const R ax = dfx * fy * phz, ay = fx * dfy * phz, az = fx * fy * dphz;
      if (gT) {
        s0 += half * (az * Ub[1] - ay * Ua[2]) + az * Ph[0];
        s1 += half * (ax * Ua[2] - az * Ub[0]) + az * Ph[1];
        s2 += half * (ay * Ua[0] - ax * Ua[1]) + az * Ph[2];
      }
      if (!want_x) continue;
      const R gfx = gs.gx[p * kd.wx + i], gfy = gs.gy[p * kd.wy + j];
      const R gdfx = gs.gdx[p * kd.wx + i], gdfy = gs.gdy[p * kd.wy + j];
      if (xs) {
        const R Pa = half * (ty * Ua[2] - tz * Ua[1]);
        const R Pb = half * (tz * Ua[0] - tx * Ua[2]);
        const R Pc = half * (tx * Ub[1] - ty * Ub[0]) + (tx * Ph[0] + ty * Ph[1] + tz * Ph[2]);
        const R gphz = gs.gz[p * kd.wz_max + k], gdphz = gs.gdz[p * kd.wz_max + k];
        x0 += gdfx * fy * phz * Pa + gfx * dfy * phz * Pb + gfx * fy * dphz * Pc;
        x1 += dfx * gfy * phz * Pa + fx * gdfy * phz * Pb + fx * gfy * dphz * Pc;
        x2 += dfx * fy * gphz * Pa + fx * dfy * gphz * Pb + fx * fy * gdphz * Pc;
      }
      if (xi) {
        R ua[3], ub[3];
        grid_value3(u, za, col, plane, comp, ghu, kd, ie, je, ua);
        grid_value3(u, zb, col, plane, comp, ghu, kd, ie, je, ub);
        const R Qa = -half * (a2 * ua[1] - a1 * ua[2]);
        const R Qb = -half * (a0 * ua[2] - a2 * ua[0]);
        const R Qc = -half * (a1 * ub[0] - a0 * ub[1]);
        const R zw = st.phzw[p * kd.wz_max + k], dzw = st.dphzw[p * kd.wz_max + k];
        const R gzw = gs.gzw[p * kd.wz_max + k], gdzw = gs.gdzw[p * kd.wz_max + k];
        x0 += gdfx * fy * zw * Qa + gfx * dfy * zw * Qb + gfx * fy * dzw * Qc;
        x1 += dfx * gfy * zw * Qa + fx * gdfy * zw * Qb + fx * gfy * dzw * Qc;
        x2 += dfx * fy * gzw * Qa + fx * dfy * gzw * Qb + fx * fy * gdzw * Qc;
      }
    }
  }
  if (gT) {
    s0 = warp_sum(s0);
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
  }
  if (want_x) {
    x0 = warp_sum(x0);
    x1 = warp_sum(x1);
    x2 = warp_sum(x2);
  }
  if (lane == 0) {
    if (gT) {
      gT[3 * p] = (RF)s0;
      gT[3 * p + 1] = (RF)s1;
      gT[3 * p + 2] = (RF)s2;
    }
    if (want_x) {
      gX[3 * p] = (RF)((R)gX[3 * p] + x0);
      gX[3 * p + 1] = (RF)((R)gX[3 * p + 1] + x1);
      gX[3 * p + 2] = (RF)((R)gX[3 * p + 2] + x2);
    }
  }
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
template <typename R>
void launch_locate_grad(bool dipole, const double *pos, int64_t N, const KernelDesc &kd, const double *zext,
                        const double *wext, const GridArgs &g, const Stencils<R> &st, const GradStencils<R> &gs,
                        cudaStream_t s) {
  if (N == 0) return;
  const int bs = 256;
  const int64_t nb = (N * (kd.wx + kd.wy + kd.wz_max) + bs - 1) / bs;
  if (dipole) k_locate_grad<R, true><<<nb, bs, 0, s>>>(pos, N, kd, zext, wext, g, st, gs);
  else k_locate_grad<R, false><<<nb, bs, 0, s>>>(pos, N, kd, zext, wext, g, st, gs);
}

template <typename R, typename RG>
void launch_adj_spread_dip(const RG *gW, int64_t N, const KernelDesc &kd, const GridArgs &g, const Stencils<R> &st,
                           R *grid, const Ghosts<R> &gh, cudaStream_t s) {
  const int64_t tot = N * kd.wx * kd.wy;
  if (tot == 0) return;
  const int bs = 256;
  k_adj_spread_dip<R, RG><<<(tot + bs - 1) / bs, bs, 0, s>>>(gW, N, kd, g, st, grid, gh);
}

template <typename R>
void launch_ghost_fold_t(R *buf, int levels, int nx, int ny, const KernelDesc &kd, cudaStream_t s) {
  if (buf == nullptr || levels <= 0) return;
  const int bs = 256;
  const int64_t ty = (int64_t)levels * kd.bend * kd.nxeff * 3 * 2;
  if (ty > 0) k_ghost_fold_y_t<R><<<(ty + bs - 1) / bs, bs, 0, s>>>(buf, levels, ny, kd);
  const int64_t tx = (int64_t)levels * kd.nyeff * kd.lend * 3 * 2;
  if (tx > 0) k_ghost_fold_x_t<R><<<(tx + bs - 1) / bs, bs, 0, s>>>(buf, levels, nx, kd);
}

template <typename R, typename RF>
void launch_gather_mono(const R *u, const R *psi, int64_t N, const KernelDesc &kd, const GridArgs &g,
                        const Stencils<R> &st, const GradStencils<R> &gs, const Ghosts<R> &ghu,
                        const Ghosts<R> &ghp, const RF *F, const RF *gV, RF *gF, RF *gX, cudaStream_t s) {
  if (N == 0) return;
  const int bs = 256;
  const int64_t nb = (N * 32 + bs - 1) / bs;
  k_gather_mono<R, RF><<<nb, bs, 0, s>>>(u, psi, N, kd, g, st, gs, ghu, ghp, F, gV, gF, gX);
}

template <typename R, typename RF>
void launch_gather_dip(const R *u, const R *psi, int64_t N, const KernelDesc &kd, const GridArgs &g,
                       const Stencils<R> &st, const GradStencils<R> &gs, const Ghosts<R> &ghu,
                       const Ghosts<R> &ghp, const RF *T, const RF *gW, RF *gT, RF *gX, cudaStream_t s) {
  if (N == 0) return;
  const int bs = 256;
  const int64_t nb = (N * 32 + bs - 1) / bs;
  k_gather_dip<R, RF><<<nb, bs, 0, s>>>(u, psi, N, kd, g, st, gs, ghu, ghp, T, gW, gT, gX);
}

#define DPST_GRAD_INST(R, RF)                                                                            \
  template void launch_adj_spread_dip<R, RF>(const RF *, int64_t, const KernelDesc &, const GridArgs &,   \
                                             const Stencils<R> &, R *, const Ghosts<R> &, cudaStream_t); \
  template void launch_gather_mono<R, RF>(const R *, const R *, int64_t, const KernelDesc &,             \
                                          const GridArgs &, const Stencils<R> &, const GradStencils<R> &, \
                                          const Ghosts<R> &, const Ghosts<R> &, const RF *, const RF *,  \
                                          RF *, RF *, cudaStream_t);                                      \
  template void launch_gather_dip<R, RF>(const R *, const R *, int64_t, const KernelDesc &,              \
                                         const GridArgs &, const Stencils<R> &, const GradStencils<R> &,  \
                                         const Ghosts<R> &, const Ghosts<R> &, const RF *, const RF *,   \
                                         RF *, RF *, cudaStream_t);

DPST_GRAD_INST(float, float)
DPST_GRAD_INST(float, double)
DPST_GRAD_INST(double, float)
DPST_GRAD_INST(double, double)

template void launch_locate_grad<float>(bool, const double *, int64_t, const KernelDesc &, const double *,
                                        const double *, const GridArgs &, const Stencils<float> &,
                                        const GradStencils<float> &, cudaStream_t);
template void launch_locate_grad<double>(bool, const double *, int64_t, const KernelDesc &, const double *,
                                         const double *, const GridArgs &, const Stencils<double> &,
                                         const GradStencils<double> &, cudaStream_t);
template void launch_ghost_fold_t<float>(float *, int, int, int, const KernelDesc &, cudaStream_t);
template void launch_ghost_fold_t<double>(double *, int, int, int, const KernelDesc &, cudaStream_t);

}  // namespace dpst
