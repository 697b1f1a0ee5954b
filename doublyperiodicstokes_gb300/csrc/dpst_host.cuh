// Host-side helpers shared by the single-system engine (dpst_engine.cu) and
// the batched engine (dpst_batch.cu): errors, device buffers, and the set-up
// arithmetic restated from the reference (Clenshaw-Curtis grids and weights,
// kernel normalisation and truncation threshold, extended z grid, DCT-I
// matrices, integration bands, BC rows, k = 0 rows).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/dpstokes_gb300.h"
#include "dpst_internal.cuh"

namespace dpst {

// ---- errors -----------------------------------------------------------------
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};
#define DPST_CUDA(call)                                                                          \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess)                                                                       \
      throw Error(e_ == cudaErrorMemoryAllocation ? DPST_ERR_ALLOC : DPST_ERR_CUDA,              \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                          \
  } while (0)
#define DPST_CUFFT(call)                                                                         \
  do {                                                                                           \
    cufftResult r_ = (call);                                                                     \
    if (r_ != CUFFT_SUCCESS)                                                                     \
      throw Error(r_ == CUFFT_ALLOC_FAILED ? DPST_ERR_ALLOC : DPST_ERR_CUDA,                     \
                  std::string(#call) + ": cuFFT error " + std::to_string((int)r_));            \
  } while (0)

extern thread_local std::string g_last_error;  // defined in dpst_engine.cu

// ---- device memory owned by the engine ---------------------------------------
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void alloc(size_t b) {
    release();
    if (b == 0) return;
    DPST_CUDA(cudaMalloc(&p, b));
    bytes = b;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <typename T>
  T *as() const { return reinterpret_cast<T *>(p); }
};

template <typename T>
static void upload(DevBuf &b, const std::vector<T> &v) {
  b.alloc(v.size() * sizeof(T));
  if (!v.empty()) DPST_CUDA(cudaMemcpy(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
}

// ---- host-side set-up arithmetic ----------------------------------------------
// Clenshaw-Curtis nodes and weights (Chebyshev.py:4-38 for the z grid,
// Quadrature.cpp:11-46 for the kernel normalisation; same arithmetic).
static void clencurt(int Np1, double a, double b, std::vector<double> &x, std::vector<double> &w) {
  const int N = Np1 - 1;
  const double H = (b - a) / 2.0, bpad2 = (b + a) / 2.0;
  x.assign(Np1, 0.0);
  w.assign(Np1, 0.0);
  for (int i = 0; i < Np1; ++i) x[i] = H * std::cos(M_PI * i / N) + bpad2;
  double w1;
  int end;
  if (N % 2) { w1 = H / (N * N); end = (N - 1) / 2 + 1; }
  else { w1 = H / (N * N - 1.0); end = N / 2; }
  w[0] = w1;
  w[N] = w1;
  std::vector<double> v(N > 1 ? N - 1 : 0, 1.0);
  for (int k = 1; k < end; ++k)
    for (int ii = 1; ii < N; ++ii) v[ii - 1] -= 2 * std::cos(2.0 * k * M_PI * ii / N) / (4.0 * k * k - 1.0);
  if (N % 2 == 0)
    for (int ii = 1; ii < N; ++ii) v[ii - 1] -= std::cos(N * M_PI * ii / N) / (N * N - 1.0);
  for (int ii = 1; ii < N; ++ii) w[ii] = 2 * H * v[ii - 1] / N;
}

static double es_norm(double beta, double alpha) {
  std::vector<double> x, w;
  clencurt(1000, -alpha, alpha, x, w);
  double s = 0.0;
  for (int j = 0; j < 1000; ++j) s += std::exp(beta * (std::sqrt(1 - x[j] * x[j] / (alpha * alpha)) - 1)) * w[j];
  return s;
}

// ParticleList.cpp:260-265 (complex principal branches)
static double dipole_threshold(double bw, double alpha) {
  typedef std::complex<double> C;
  C s = std::sqrt(C(-12 * bw * bw + 81, 0.0));
  C z = (C(8 * bw * bw, 0.0) + 12.0 * s - 108.0) * bw;
  C t = 6.0 * std::pow(z, 1.0 / 3.0) / bw + 24.0 * bw * std::pow(z, -1.0 / 3.0) + 12.0;
  return (std::sqrt(t) * alpha / 6.0).real();
}

static int cround(double v) { return (int)std::floor(v + 0.5); }

struct KernelHost {
  KernelDesc d;
  std::vector<double> zext, wext;
};

// Extended z grid for one kernel (ParticleList.cpp:419-451).
static KernelHost make_kernel(int w, double beta, double alpha, bool dipole, double hx, double hy, int nx,
                              int ny, const std::vector<double> &zG, const std::vector<double> &zW,
                              const char *what) {
  KernelHost k;
  KernelDesc &d = k.d;
  memset(&d, 0, sizeof(d));
  if (!(alpha > 0) || !(beta > 0) || w < 1)
    throw Error(DPST_ERR_INVALID_ARG, std::string(what) + ": w, beta and alpha must be positive");
  d.beta = beta;
  d.alpha = alpha;
  d.alpha2 = alpha * alpha;
  d.inv_alpha2 = 1.0 / d.alpha2;
  d.norm = es_norm(beta, alpha);
  d.inv_norm3 = 1.0 / (d.norm * d.norm * d.norm);
  d.thr = dipole ? dipole_threshold(beta, alpha) : alpha;
  if (!(d.thr > 0) || !(d.thr <= alpha))
    throw Error(DPST_ERR_INVALID_ARG, std::string(what) + ": kernel threshold is not in (0, alpha]");
  d.wx = cround(2 * d.thr / hx);
  d.wy = cround(2 * d.thr / hy);
  if (d.wx < 1 || d.wy < 1 || d.wx > nx || d.wy > ny)
    throw Error(DPST_ERR_INVALID_ARG, std::string(what) + ": kernel support does not fit the grid");
  d.evenx = 1 - (d.wx % 2);
  d.eveny = 1 - (d.wy % 2);
  d.nxeff = nx + d.wx + (d.wx % 2);
  d.nyeff = ny + d.wy + (d.wy % 2);
  d.lend = (d.nxeff - nx) / 2;
  d.bend = (d.nyeff - ny) / 2;
  const int nz = (int)zG.size();
  int up = 0, down = 0;
  for (int i = 1; i < nz && zG[0] - zG[i] <= d.thr; ++i) up++;
  for (int i = nz - 2; i >= 0 && zG[i] - zG[nz - 1] <= d.thr; --i) down++;
  if (up != down)
    throw Error(DPST_ERR_UNSUPPORTED,
                std::string(what) + ": a Chebyshev node lies exactly at the kernel threshold from one wall "
                "but not the other (asymmetric ghost extension; the reference overruns its grid here)");
  if (up >= nz - 1)
    throw Error(DPST_ERR_INVALID_ARG, std::string(what) + ": kernel wider than the z domain");
  d.dend = up;
  d.nzeff = nz + up + down;
  k.zext.assign(d.nzeff, 0.0);
  k.wext.assign(d.nzeff, 0.0);
  for (int i = up; i < d.nzeff - down; ++i) {
    k.zext[i] = zG[i - up];
    k.wext[i] = zW[i - up];
  }
  int j = 0;
  for (int i = up; i > 0; --i, ++j) {
    k.zext[j] = 2.0 * zG[0] - zG[i];
    k.wext[j] = zW[i];
  }
  j = d.nzeff - down;
  for (int i = nz - 2; i > nz - 2 - down; --i, ++j) {
    k.zext[j] = -1.0 * zG[i];
    k.wext[j] = zW[i];
  }
  // longest possible window: points within a closed interval of length 2 thr
  int wmax = 1;
  for (int a = 0; a < d.nzeff; ++a) {
    int c = 0;
    for (int b = a; b < d.nzeff && k.zext[a] - k.zext[b] <= 2 * d.thr * (1 + 1e-12); ++b) c++;
    wmax = std::max(wmax, c);
  }
  d.wz_max = wmax + 1;
  return k;
}

// Kernel on a uniform periodic z grid (triply periodic mode): widths
// round(2 thr / h) on every axis and extended sizes n + w + (w mod 2)
// (ParticleList.cpp:285-310).  No extended z tables.
static KernelHost make_kernel_tp(int w, double beta, double alpha, bool dipole, double hx, double hy, double hz,
                                 int nx, int ny, int nz, const char *what) {
  KernelHost k;
  KernelDesc &d = k.d;
  memset(&d, 0, sizeof(d));
  if (!(alpha > 0) || !(beta > 0) || w < 1)
    throw Error(DPST_ERR_INVALID_ARG, std::string(what) + ": w, beta and alpha must be positive");
  d.beta = beta;
  d.alpha = alpha;
  d.alpha2 = alpha * alpha;
  d.inv_alpha2 = 1.0 / d.alpha2;
  d.norm = es_norm(beta, alpha);
  d.inv_norm3 = 1.0 / (d.norm * d.norm * d.norm);
  d.thr = dipole ? dipole_threshold(beta, alpha) : alpha;
  if (!(d.thr > 0) || !(d.thr <= alpha))
    throw Error(DPST_ERR_INVALID_ARG, std::string(what) + ": kernel threshold is not in (0, alpha]");
  d.wx = cround(2 * d.thr / hx);
  d.wy = cround(2 * d.thr / hy);
  const int wz = cround(2 * d.thr / hz);
  if (d.wx < 1 || d.wy < 1 || wz < 1 || d.wx > nx || d.wy > ny || wz > nz)
    throw Error(DPST_ERR_INVALID_ARG, std::string(what) + ": kernel support does not fit the grid");
  d.evenx = 1 - (d.wx % 2);
  d.eveny = 1 - (d.wy % 2);
  d.evenz = 1 - (wz % 2);
  d.nxeff = nx + d.wx + (d.wx % 2);
  d.nyeff = ny + d.wy + (d.wy % 2);
  d.nzeff = nz + wz + (wz % 2);
  d.lend = (d.nxeff - nx) / 2;
  d.bend = (d.nyeff - ny) / 2;
  d.dend = (d.nzeff - nz) / 2;
  d.wz_max = wz;
  d.unif_z = 1;
  d.hz = hz;
  return k;
}

// DCT-I matrices (Transform.cpp:107-304): tf[j][m] gives Chebyshev
// coefficient j from node values m, ti[m][j] node value m from coefficient j.
static void dct_matrices(int nz, std::vector<double> &tf, std::vector<double> &ti) {
  tf.assign((size_t)nz * nz, 0.0);
  ti.assign((size_t)nz * nz, 0.0);
  const int Nm = nz - 1, Nu = 2 * Nm;
  for (int j = 0; j < nz; ++j)
    for (int m = 0; m < nz; ++m) {
      int r = (int)(((int64_t)j * m) % Nu);
      double c = std::cos(M_PI * (double)r / (double)Nm);
      double wj = (j == 0 || j == Nm) ? 1.0 : 2.0, vm = (m == 0 || m == Nm) ? 1.0 : 2.0;
      tf[(size_t)j * nz + m] = wj * vm * c / Nu;
      ti[(size_t)m * nz + j] = c;
    }
}

// z-direction tables shared by every wavenumber (and by every system of a
// batch with the same nz, Lz and geometry): integration-matrix bands
// (Chebyshev.py:119-160, H-scaled), BC rows (Solvers.py:603-643), k = 0
// correction rows and Gi (Solvers.py:499-504, 582-587).
struct ZTables {
  std::vector<double> bands;   // 5 nz: s0, sp2, sm2, fm1, fp1
  std::vector<double> bcrows;  // 4 (nz + 2): R1, R2, L1, L2
  std::vector<double> k0rows;  // 2 nz
  double k0gi[4];
};

static ZTables make_ztables(int nz, double H, int mode) {
  // integration matrix bands (Chebyshev.py:119-160), H-scaled
  std::vector<double> bandv(5 * nz, 0.0);
  double *s0 = &bandv[0], *sp2 = &bandv[nz], *sm2 = &bandv[2 * nz], *fm1 = &bandv[3 * nz],
         *fp1 = &bandv[4 * nz];
  const double H2 = H * H;
  for (int r = 0; r < nz; ++r) {
    double c0v, cp2v;
    if (r == 0) { c0v = 0; cp2v = 0; }
    else if (r == 1) { c0v = -0.125; cp2v = 0.125; }
    else if (r == 2) { c0v = -1. / 8. - 1. / 24.; cp2v = 1. / 24.; }
    else {
      double jj = r;
      c0v = -1 / (2 * jj * (2 * jj - 2)) - 1 / (2 * jj * (2 * jj + 2)) * (r < nz - 1 ? 1.0 : 0.0);
      cp2v = 1 / (2 * jj * (2 * jj + 2)) * (r < nz - 2 ? 1.0 : 0.0);
    }
    s0[r] = H2 * c0v;
    sp2[r] = H2 * cp2v;
    if (r >= 2) {
      double cm2v = (r == 2) ? 0.25 : 1 / (2.0 * r * (2.0 * r - 2));
      sm2[r] = H2 * cm2v;
    }
    if (r >= 1) fm1[r] = H * ((r == 1) ? 1.0 : 1 / (2.0 * r));
    double cp1v = (r == 0) ? 0.0 : (r == 1) ? -0.5 : -1 / (2.0 * r) * (r < nz - 1 ? 1.0 : 0.0);
    fp1[r] = H * cp1v;
  }
  // BC rows (Solvers.py:603-643)
  const int N2 = nz + 2;
  std::vector<double> bc(4 * N2, 0.0);
  double *R1 = &bc[0], *R2 = &bc[N2], *L1 = &bc[2 * N2], *L2 = &bc[3 * N2];
  {
    const int Nn = nz;
    R1[Nn + 1] = 1; R2[Nn] = 1; R1[0] = 1; R1[2] = -1.0 / 2;
    R2[Nn + 1] += 1; R2[1] = -1.0 / 8; R2[3] = 1.0 / 8;
    R1[1] += 1.0 / 4; R1[3] -= 1.0 / 4; R2[0] += 1.0 / 4; R2[2] -= (1.0 / 8 + 1.0 / 24);
    R2[4] += 1.0 / 24;
    L1[Nn + 1] = 1; L2[Nn] = -1; L1[0] = -1; L1[2] = 1.0 / 2;
    L2[Nn + 1] += 1; L2[1] = -1.0 / 8; L2[3] = 1.0 / 8;
    L1[1] += 1.0 / 4; L1[3] -= 1.0 / 4; L2[0] -= 1.0 / 4; L2[2] += 1.0 / 8 + 1.0 / 24;
    L2[4] -= 1.0 / 24;
    for (int jj = 3; jj < Nn; ++jj) {
      double sg = (jj % 2) ? -1.0 : 1.0;
      double a1 = 1.0 / (2 * jj), b1 = 1.0 / (2 * jj) * 1.0 / (2 * jj - 2), c1 = 1.0 / (2 * jj) * 1.0 / (2 * jj + 2);
      R1[jj - 1] += a1;
      L1[jj - 1] += sg / (2 * jj);
      if (jj < Nn - 1) { R1[jj + 1] -= a1; L1[jj + 1] -= sg / (2 * jj); }
      R2[jj - 2] += b1;
      L2[jj - 2] -= b1 * sg;
      if (jj < Nn - 2) { R2[jj + 2] += c1; L2[jj + 2] -= c1 * sg; }
      double m = b1 + (jj < Nn - 1 ? c1 : 0.0);
      R2[jj] -= m;
      L2[jj] += m * sg;
    }
  }
  // k = 0 velocity correction rows and Gi (Solvers.py:499-504, 582-587)
  std::vector<double> k0r(2 * nz, 0.0);
  double k0gi[4] = {0, 0, 0, 0};
  if (mode != DPST_MODE_NOWALL) {
    const double *top = (mode == DPST_MODE_BOTTOM) ? R1 : R2;
    for (int j = 0; j < nz; ++j) { k0r[j] = top[j]; k0r[nz + j] = L2[j]; }
    double D00 = -top[nz], D01 = -top[nz + 1], D10 = -L2[nz], D11 = -L2[nz + 1];
    double det = 1.0 / (D00 * D11 - D01 * D10);
    k0gi[0] = det * D11; k0gi[1] = det * -D01; k0gi[2] = det * -D10; k0gi[3] = det * D00;
  }
  ZTables zt;
  zt.bands = bandv;
  zt.bcrows = bc;
  zt.k0rows = k0r;
  for (int q = 0; q < 4; ++q) zt.k0gi[q] = k0gi[q];
  return zt;
}

// Boundary-condition sets of a geometry (FCM.py:215-248): set A for forces
// and the x/y torque derivatives, set B for the z torque derivative.  The
// triply periodic mode wraps z instead (its BCs are all 'none' and unused).
static void bc_sets(int mode, GridArgs &g) {
  memset(&g.bcA, 0, sizeof(g.bcA));
  memset(&g.bcB, 0, sizeof(g.bcB));
  if (mode == DPST_MODE_PERIODIC) {
    g.bcA.periodic = g.bcB.periodic = 1;
  } else if (mode == DPST_MODE_BOTTOM) {
    g.bcA.bot_active = 1; g.bcA.s_bot = -1.0;
    g.bcB.bot_active = 1; g.bcB.s_bot = 1.0;
  } else if (mode == DPST_MODE_SLIT) {
    g.bcA.bot_active = g.bcA.top_active = 1; g.bcA.s_bot = g.bcA.s_top = -1.0;
    g.bcB.bot_active = g.bcB.top_active = 1; g.bcB.s_bot = g.bcB.s_top = 1.0;
  }
}

// Wavenumbers in FFT order (Solvers.py:292-297).
static std::vector<double> wavenumbers(int n, double L) {
  std::vector<double> k(n);
  for (int i = 0; i < n; ++i) {
    const int m = (i <= n / 2) ? i : i - n;
    k[i] = 2 * M_PI * (double)m / L;
  }
  return k;
}

// Parameter checks of dpst_create (shared by the batched engine).
// periodic_ok: the caller (dpst_create) runs the triply periodic mode and the
// regular-kernel torque coupling; the batched engine does not.
static void validate(const dpst_params *p, int64_t n, bool periodic_ok = false) {
  if (!p) throw Error(DPST_ERR_INVALID_ARG, "params is NULL");
  if (n < 0) throw Error(DPST_ERR_INVALID_ARG, "n_particles < 0");
  if (p->mode == DPST_MODE_PERIODIC && !periodic_ok)
    throw Error(DPST_ERR_UNSUPPORTED, "mode PERIODIC is available through dpst_create only");
  if (p->mode < 0 || p->mode > 3)
    throw Error(DPST_ERR_INVALID_ARG, "mode must be NOWALL, BOTTOM, SLIT or PERIODIC");
  if (p->nx < 4 || p->ny < 4) throw Error(DPST_ERR_INVALID_ARG, "nx and ny must be >= 4");
  if (p->mode == DPST_MODE_PERIODIC) {
    if (p->nz < 4) throw Error(DPST_ERR_INVALID_ARG, "nz must be >= 4");
    if ((int64_t)p->nz * p->ny * p->nx > INT_MAX || (int64_t)p->nz * p->ny * (p->nx / 2 + 1) * 3 > INT_MAX)
      throw Error(DPST_ERR_UNSUPPORTED, "grid too large for one FFT plan");
  } else {
    if (p->nz < 5) throw Error(DPST_ERR_INVALID_ARG, "nz must be >= 5");
    if (p->nz > 128) throw Error(DPST_ERR_UNSUPPORTED, "nz > 128 is not supported yet");
    if ((int64_t)p->ny * (p->nx / 2 + 1) * 3 * p->nz > INT_MAX)
      throw Error(DPST_ERR_UNSUPPORTED, "grid too large for one FFT plan");
  }
  if (!(p->Lx > 0) || !(p->Ly > 0)) throw Error(DPST_ERR_INVALID_ARG, "Lx and Ly must be positive");
  if (!(p->zmax > p->zmin)) throw Error(DPST_ERR_INVALID_ARG, "zmax must exceed zmin");
  if (!(p->viscosity > 0)) throw Error(DPST_ERR_INVALID_ARG, "viscosity must be positive");
  if (p->precision != DPST_PREC_FP64 && p->precision != DPST_PREC_MIXED)
    throw Error(DPST_ERR_INVALID_ARG, "precision must be DPST_PREC_FP64 or DPST_PREC_MIXED");
  if (p->torque_kernel != DPST_TORQUE_DERIV && p->torque_kernel != DPST_TORQUE_REG)
    throw Error(DPST_ERR_INVALID_ARG, "torque_kernel must be DPST_TORQUE_DERIV or DPST_TORQUE_REG");
  if (p->solve_arith != DPST_SOLVE_DEFAULT && p->solve_arith != DPST_SOLVE_FP64 && p->solve_arith != DPST_SOLVE_DF64)
    throw Error(DPST_ERR_INVALID_ARG, "solve_arith must be DPST_SOLVE_DEFAULT, DPST_SOLVE_FP64 or DPST_SOLVE_DF64");
  if (p->torque_kernel == DPST_TORQUE_REG && !periodic_ok)
    throw Error(DPST_ERR_UNSUPPORTED, "torque_kernel DPST_TORQUE_REG is available through dpst_create only");
}

// Runs fn and turns exceptions into the C ABI's return codes and message.
template <typename Fn>
static int guarded(Fn &&fn) {
  try {
    fn();
    g_last_error.clear();
    return DPST_OK;
  } catch (const Error &e) {
    g_last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc &) {
    g_last_error = "host allocation failed";
    return DPST_ERR_ALLOC;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return DPST_ERR_CUDA;
  } catch (...) {
    g_last_error = "unknown error";
    return DPST_ERR_CUDA;
  }
}

}  // namespace dpst
