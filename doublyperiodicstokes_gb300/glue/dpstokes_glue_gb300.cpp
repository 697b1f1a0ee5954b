// DPStokesGlue on libdpstokes_gb300.so.
//
// The reference builds its Python module `uammd` from
// source/gpu/python_wrapper/uammd_python.cpp (pybind11) over the class
// DPStokesGlue declared in source/gpu/python_wrapper/uammd_interface.h:44-65
// and implemented on UAMMD in uammd_wrapper.cu:90-221.  This file implements
// the same class and uammd_wrapper::getPrecision on the GB300 operator's C
// ABI, so the reference's uammd_python.cpp compiles and links unchanged
// against it:
//
//   g++ -O2 -std=c++14 -shared -fPIC [-DDOUBLE_PRECISION] \
//       -I<reference>/source/gpu/python_wrapper -I<this repo>/include \
//       $(python3 -m pybind11 --includes) \
//       <reference>/source/gpu/python_wrapper/uammd_python.cpp dpstokes_glue_gb300.cpp \
//       -L<this repo>/doublyperiodicstokes_gb300/lib -ldpstokes_gb300 \
//       -Wl,-rpath,<this repo>/doublyperiodicstokes_gb300/lib \
//       -o uammd$(python3-config --extension-suffix)
//
// Semantics kept from the reference glue: host arrays in and out on every call
// (uammd_wrapper.cu:136-170), std::runtime_error on misuse
// (uammd_wrapper.cu:106, 208-211), an unknown mode string meaning 'none'
// (uammd_wrapper.cu:55-66), `real` = float unless DOUBLE_PRECISION
// (uammd_interface.h:9-13).  Differences: alpha and alpha_d are taken in grid
// units (as FCMJoint passes them, common_interface_wrapper.py:89-96) and
// scaled by h = Lx/nx; (zmin, zmax) are used at face value (no zOrigin shift);
// 'periodic' (triply periodic FCM) is not provided and throws; with
// DOUBLE_PRECISION the FP64 operator runs, otherwise the mixed one.
#include <memory>
#include <stdexcept>
#include <string>

#include "uammd_interface.h"   // the reference's header (declares DPStokesGlue)
#include "dpstokes_gb300.h"    // this project's C ABI

class DPStokesUAMMD {
 public:
  dpst_handle h = nullptr;
  ~DPStokesUAMMD() {
    if (h) dpst_destroy(h);
  }
};

namespace uammd_wrapper {
std::string getPrecision() { return sizeof(real) == sizeof(double) ? "double" : "single"; }
}  // namespace uammd_wrapper

namespace {
void check(int code) {
  if (code != DPST_OK) throw std::runtime_error(dpst_last_error());
}
int dtype() { return sizeof(real) == sizeof(double) ? DPST_F64 : DPST_F32; }
}  // namespace

void DPStokesGlue::initialize(PyParameters par, int numberParticles) {
  dpstokes.reset();
  if (par.nx <= 0 || par.ny <= 0 || par.nz <= 0) throw std::runtime_error("nx, ny and nz must be given");
  dpst_params p{};
  p.mode = par.mode == "bottom"     ? DPST_MODE_BOTTOM
           : par.mode == "slit"     ? DPST_MODE_SLIT
           : par.mode == "periodic" ? DPST_MODE_PERIODIC
                                    : DPST_MODE_NOWALL;
  p.nx = par.nx;
  p.ny = par.ny;
  p.nz = par.nz;
  p.Lx = par.Lx;
  p.Ly = par.Ly;
  p.zmin = par.zmin;
  p.zmax = par.zmax;
  p.viscosity = par.viscosity;
  const double h = (double)par.Lx / par.nx;
  p.w = (int)(par.w + 0.5);
  p.beta = par.beta;
  p.alpha = par.alpha * h;
  p.has_torque = (par.w_d > 0 && par.alpha_d > 0 && par.beta_d > 0) ? 1 : 0;
  p.w_d = p.has_torque ? (int)(par.w_d + 0.5) : 6;
  p.beta_d = p.has_torque ? par.beta_d : 1.0;
  p.alpha_d = p.has_torque ? par.alpha_d * h : 1.0;
  p.precision = sizeof(real) == sizeof(double) ? DPST_PREC_FP64 : DPST_PREC_MIXED;
  auto d = std::make_shared<DPStokesUAMMD>();
  check(dpst_create(&p, numberParticles, 0, &d->h));
  dpstokes = d;
}

void DPStokesGlue::clear() { dpstokes.reset(); }

void DPStokesGlue::setPositions(const real *h_pos) {
  throwIfInvalid();
  check(dpst_set_positions_host(dpstokes->h, h_pos, dtype(), nullptr));
}

void DPStokesGlue::Mdot(const real *h_forces, const real *h_torques, real *h_MF, real *h_MT) {
  throwIfInvalid();
  check(dpst_mdot_host(dpstokes->h, h_forces, h_torques, h_MF, h_torques ? h_MT : nullptr, dtype(), nullptr));
}

void DPStokesGlue::throwIfInvalid() {
  if (!dpstokes) throw std::runtime_error("DPStokes is not initialized. Call Initialize first");
}
