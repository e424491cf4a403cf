// cholla_dropin.cpp -- link-time replacement of Cholla's VL integrator entry points.
//
// A Cholla build adds this file (and links libchollagb) in place of the objects of
// src/integrators/VL_3D_cuda.cu, VL_2D_cuda.cu and VL_1D_cuda.cu.  The functions below have the exact
// C++ signatures the rest of Cholla calls (src/integrators/VL_3D_cuda.h:9-13, VL_2D_cuda.h:9-12, VL_1D_cuda.h,
// src/hydro/hydro_cuda.h:69-70, 90), so Grid3D::Execute_Hydro_Integrator, Calc_Inverse_Timestep
// and Update_Hydro_Grid need no change.  The compile-time scheme macros of the Cholla build
// (builds/make.type.*) and its global adiabatic index `gama` become the library's run-time
// scheme on first use.  Like the reference, the shim aborts the process on an error.
//
// Build inside Cholla:   CXXFLAGS += -I<cholla_gb300>/include ; LIBS += -L<lib dir> -lchollagb
#include <cstdio>
#include <cstdlib>

#include "cholla_gb300.h"

#ifndef CHOLLA_DROPIN_REAL
typedef double Real;  // PRECISION=2 (src/global/global.h:18-22); the library is FP64-state only
#endif

extern Real gama;  // src/global/global.h:147

namespace
{
bool configured = false;

void check(int rc, const char *where)
{
  if (rc != CGB_OK) {
    std::fprintf(stderr, "libchollagb: %s failed (%d): %s\n", where, rc, cgb_last_error());
    std::exit(rc);  // the reference's GPU_Error_Check -> chexit (src/utils/gpu.hpp:139-155)
  }
}

void configure()
{
  if (configured) return;
  cgb_scheme s{};
#if defined(PPMC)
  s.reconstruction = CGB_PPMC;
#elif defined(PLMC)
  s.reconstruction = CGB_PLMC;
#elif defined(PPMP)
  s.reconstruction = CGB_PPMP;
#elif defined(PLMP)
  s.reconstruction = CGB_PLMP;
#else
  s.reconstruction = CGB_PCM;
#endif
#if defined(HLLD)
  s.riemann_solver = CGB_HLLD;
#elif defined(ROE)
  s.riemann_solver = CGB_ROE;
#elif defined(HLL)
  s.riemann_solver = CGB_HLL;
#elif defined(EXACT)
  s.riemann_solver = CGB_EXACT;
#else
  s.riemann_solver = CGB_HLLC;
#endif
#ifdef DE
  s.dual_energy = 1;
#endif
#ifdef MHD
  s.mhd = 1;
#endif
#ifdef SCALAR
  s.n_scalars = NSCALARS;
#endif
#ifdef DENSITY_FLOOR
  s.density_floor = 1;
#endif
#ifdef TEMPERATURE_FLOOR
  s.temperature_floor = 1;
#endif
#ifdef CHOLLA_GB300_MIXED
  s.precision = CGB_MIXED;
#elif defined(CHOLLA_GB300_FP64_FAST)
  s.precision = CGB_FP64_FAST;
#else
  s.precision = CGB_FP64;
#endif
  s.gamma   = gama;
  s.U_floor = 0.0;
  check(cgb_set_scheme(&s), "cgb_set_scheme");
  configured = true;
}
}  // namespace

void VL_Algorithm_3D_CUDA(Real *d_conserved, Real *d_grav_potential, int nx, int ny, int nz, int x_off, int y_off,
                          int z_off, int n_ghost, Real dx, Real dy, Real dz, Real xbound, Real ybound, Real zbound,
                          Real dt, int n_fields, int custom_grav, Real density_floor, Real *host_grav_potential)
{
  configure();
  check(cgb_vl_algorithm_3d(d_conserved, d_grav_potential, nx, ny, nz, x_off, y_off, z_off, n_ghost, dx, dy, dz,
                            xbound, ybound, zbound, dt, n_fields, custom_grav, density_floor, host_grav_potential),
        "VL_Algorithm_3D_CUDA");
}

void Free_Memory_VL_3D() { check(cgb_free_memory_vl_3d(), "Free_Memory_VL_3D"); }

void VL_Algorithm_1D_CUDA(Real *d_conserved, int nx, int x_off, int n_ghost, Real dx, Real xbound, Real dt,
                          int n_fields, int custom_grav)
{
  configure();
  check(cgb_vl_algorithm_1d(d_conserved, nx, x_off, n_ghost, dx, xbound, dt, n_fields, custom_grav),
        "VL_Algorithm_1D_CUDA");
}

void Free_Memory_VL_1D() { check(cgb_free_memory_vl_3d(), "Free_Memory_VL_1D"); }

void VL_Algorithm_2D_CUDA(Real *d_conserved, int nx, int ny, int x_off, int y_off, int n_ghost, Real dx, Real dy,
                          Real xbound, Real ybound, Real dt, int n_fields, int custom_grav)
{
  configure();
  check(cgb_vl_algorithm_2d(d_conserved, nx, ny, x_off, y_off, n_ghost, dx, dy, xbound, ybound, dt, n_fields,
                            custom_grav),
        "VL_Algorithm_2D_CUDA");
}

void Free_Memory_VL_2D() { check(cgb_free_memory_vl_3d(), "Free_Memory_VL_2D"); }

// Calc_dt_GPU and Apply_Temperature_Floor are defined in src/hydro/hydro_cuda.cu next to
// kernels other files still use; build these replacements only once those two definitions
// are taken out of that file (-DCHOLLA_DROPIN_DT, -DCHOLLA_DROPIN_TFLOOR).
#ifdef CHOLLA_DROPIN_DT
Real Calc_dt_GPU(Real *dev_conserved, int nx, int ny, int nz, int n_ghost, int n_fields, Real dx, Real dy, Real dz,
                 Real gamma)
{
  configure();
  double max_dti = 0.0;
  check(cgb_calc_dt_gpu(dev_conserved, nx, ny, nz, n_ghost, n_fields, dx, dy, dz, gamma, &max_dti), "Calc_dt_GPU");
  return max_dti;
}
#endif

#ifdef CHOLLA_DROPIN_TFLOOR
void Apply_Temperature_Floor(Real *dev_conserved, int nx, int ny, int nz, int n_ghost, int n_fields, Real U_floor)
{
  configure();
  check(cgb_apply_temperature_floor(dev_conserved, nx, ny, nz, n_ghost, n_fields, U_floor),
        "Apply_Temperature_Floor");
}
#endif
