/*
 * ref_host.cpp -- the reference's own VL integrators and kernels, compiled unchanged from the
 * cholla source tree as host C++ (oracle/ref_host_shim.h) and exported through a C ABI.
 *
 * TEST INFRASTRUCTURE ONLY: a second oracle that runs the reference itself on the CPU, used by
 * tests/ to pin the FP64 restatement (cholla_oracle.cpp) bit for bit.  One shared library per
 * scheme (the reference's make.type macros), built by oracle/build_ref_host.sh into
 * oracle/_ref/host/ from the sources under the reference tree (-I <cholla>/src).  Nothing in the
 * product links or loads it, and it is not built where the reference tree is absent.
 *
 * Entry points (each returns 0, or -1 after the reference called chexit):
 *   refh_vl3d  VL_Algorithm_3D_CUDA   (src/integrators/VL_3D_cuda.cu:38)
 *   refh_vl2d  VL_Algorithm_2D_CUDA   (src/integrators/VL_2D_cuda.cu:25)
 *   refh_vl1d  VL_Algorithm_1D_CUDA   (src/integrators/VL_1D_cuda.cu:30)
 *   refh_plmp / refh_ppmp  PLMP_cuda / PPMP_cuda, one direction (reconstruction/plmp_cuda.cu:21,
 *              ppmp_cuda.cu:28), writing the interface arrays the caller passes
 *   refh_riemann  one launch of the HLLC, Roe, HLL or exact flux kernel along a direction
 *   refh_set_ghost_cells  SetGhostCells, the ghost fill of one face (grid/cuda_boundaries.cu:151)
 *   refh_temperature_floor  Apply_Temperature_Floor (hydro/hydro_cuda.cu:1103)
 *   refh_scheme  which of the make.type macros this library was compiled with
 * The library built with the exact solver has no integrator entry points: the reference's VL
 * integrators do not compile with it (VL_3D_cuda.cu:149).
 * The state is updated in place in the reference's field-major layout.  The integrators keep
 * their scratch in file-scope globals that are allocated on the first call and never resized
 * (VL_3D_cuda.cu:58-133); each entry point here releases them after the step, so successive
 * calls may pass another state array.  Launch sizes are function-local statics fixed by the
 * first call (VL_3D_cuda.cu:141 and beside each launch), so one loaded instance of a library
 * serves one grid shape: oracle/ref_host.py loads a private copy per shape.
 */
#include "global/global.h"

Real gama;  // the reference's adiabatic index global (global.h:147), an argument here

[[noreturn]] void chexit(int code) { throw std::runtime_error("chexit " + std::to_string(code)); }

#include "global/global_cuda.cu"
#include "grid/cuda_boundaries.cu"
#include "hydro/hydro_cuda.cu"
#ifndef EXACT  // the integrators do not compile with the exact solver (VL_3D_cuda.cu:149)
  #include "integrators/VL_1D_cuda.cu"
  #include "integrators/VL_2D_cuda.cu"
  #include "integrators/VL_3D_cuda.cu"
#else
  #include "riemann_solvers/exact_cuda.cu"
#endif
#include "reconstruction/pcm_cuda.cu"
#include "reconstruction/plmc_cuda.cu"
#include "reconstruction/plmp_cuda.cu"
#include "reconstruction/ppmc_cuda.cu"
#include "reconstruction/ppmp_cuda.cu"
#include "riemann_solvers/hll_cuda.cu"
#include "riemann_solvers/hllc_cuda.cu"
#include "riemann_solvers/roe_cuda.cu"
#ifdef MHD
  #include "mhd/ct_electric_fields.cu"
  #include "mhd/magnetic_update.cu"
  #include "riemann_solvers/hlld_cuda.cu"
  #include "utils/mhd_utilities.cu"
#endif

namespace
{
// Frees the integrators' file-scope scratch and clears the flag that guards its allocation.
void release_scratch()
{
  Real **arrays[] = {&dev_conserved_half, &Q_Lx, &Q_Rx, &Q_Ly, &Q_Ry, &Q_Lz, &Q_Rz, &F_x, &F_y, &F_z, &ctElectricFields};
  for (Real **a : arrays) {
    std::free(*a);
    *a = nullptr;
  }
  dev_conserved    = nullptr;
  memory_allocated = false;
}

template <class F>
int guarded(F f)
{
  release_scratch();
  int rc = 0;
  try {
    f();
  } catch (const std::exception &) {
    rc = -1;
  }
  release_scratch();
  return rc;
}

int launch_blocks(int n_cells) { return (n_cells + TPB - 1) / TPB; }
}  // namespace

extern "C" {

#ifndef EXACT
int refh_vl3d(double *U, int nx, int ny, int nz, int n_ghost, double dx, double dy, double dz, double dt, int n_fields,
              double gamma, double density_floor)
{
  gama = gamma;
  return guarded([&] {
    VL_Algorithm_3D_CUDA(U, nullptr, nx, ny, nz, 0, 0, 0, n_ghost, dx, dy, dz, 0.0, 0.0, 0.0, dt, n_fields, 0,
                         density_floor, nullptr);
  });
}

int refh_vl2d(double *U, int nx, int ny, int n_ghost, double dx, double dy, double dt, int n_fields, double gamma)
{
  gama = gamma;
  return guarded([&] { VL_Algorithm_2D_CUDA(U, nx, ny, 0, 0, n_ghost, dx, dy, 0.0, 0.0, dt, n_fields, 0); });
}

int refh_vl1d(double *U, int nx, int n_ghost, double dx, double dt, int n_fields, double gamma)
{
  gama = gamma;
  return guarded([&] { VL_Algorithm_1D_CUDA(U, nx, 0, n_ghost, dx, 0.0, dt, n_fields, 0); });
}
#endif

// One launch of a Riemann solver kernel over the whole grid along dir: 0 HLLC
// (hllc_cuda.cu:19), 1 Roe (roe_cuda.cu:19), 3 HLL (hll_cuda.cu:19), 4 exact (exact_cuda.cu:20,
// in the library built with EXACT only).  Returns -2 for a solver this library lacks.
int refh_riemann(int solver, double *QL, double *QR, double *F, int nx, int ny, int nz, int n_ghost, double gamma,
                 int dir, int n_fields)
{
  auto run = [&](auto kernel) {
    return guarded([&] {
      hipLaunchKernelGGL(kernel, launch_blocks(nx * ny * nz), TPB, 0, 0, QL, QR, F, nx, ny, nz, n_ghost, gamma, dir,
                         n_fields);
    });
  };
  switch (solver) {
    case 0:
      return run(Calculate_HLLC_Fluxes_CUDA);
    case 1:
      return run(Calculate_Roe_Fluxes_CUDA);
    case 3:
      return run(Calculate_HLL_Fluxes_CUDA);
#ifdef EXACT
    case 4:
      return run(Calculate_Exact_Fluxes_CUDA);
#endif
    default:
      return -2;
  }
}

int refh_plmp(double *U, double *QL, double *QR, int nx, int ny, int nz, int n_ghost, double dx, double dt,
              double gamma, int dir, int n_fields)
{
  return guarded([&] {
    hipLaunchKernelGGL(PLMP_cuda, launch_blocks(nx * ny * nz), TPB, 0, 0, U, QL, QR, nx, ny, nz, n_ghost, dx, dt, gamma,
                       dir, n_fields);
  });
}

int refh_ppmp(double *U, double *QL, double *QR, int nx, int ny, int nz, int n_ghost, double dx, double dt,
              double gamma, int dir, int n_fields)
{
#ifdef PPMP
  return guarded([&] {
    hipLaunchKernelGGL(PPMP_cuda, launch_blocks(nx * ny * nz), TPB, 0, 0, U, QL, QR, nx, ny, nz, n_ghost, dx, dt, gamma,
                       dir, n_fields);
  });
#else
  (void)U, (void)QL, (void)QR, (void)nx, (void)ny, (void)nz, (void)n_ghost, (void)dx, (void)dt, (void)gamma, (void)dir,
      (void)n_fields;
  return -2;  // PPMP_cuda is compiled only with the PPMP macro (ppmp_cuda.cu:4)
#endif
}

// SetGhostCells (grid/cuda_boundaries.cu:151-159) for one face dir over the ghost slab of
// isize x jsize x ksize cells starting at (imin, jmin, kmin), the extents the reference's
// Grid3D::Set_Boundary_Extents gives (grid/boundary_conditions.cpp:419-493).
int refh_set_ghost_cells(double *U, int nx, int ny, int nz, int n_fields, int n_ghost, const int *flags, int isize,
                         int jsize, int ksize, int imin, int jmin, int kmin, int dir)
{
  int f[6] = {flags[0], flags[1], flags[2], flags[3], flags[4], flags[5]};
  return guarded(
      [&] { SetGhostCells(U, nx, ny, nz, n_fields, nx * ny * nz, n_ghost, f, isize, jsize, ksize, imin, jmin, kmin, dir); });
}

// Apply_Temperature_Floor (hydro/hydro_cuda.cu:1103-1153): the internal-energy floor U_floor.
int refh_temperature_floor(double *U, int nx, int ny, int nz, int n_ghost, int n_fields, double U_floor)
{
  return guarded([&] { Apply_Temperature_Floor(U, nx, ny, nz, n_ghost, n_fields, U_floor); });
}

// Bit mask of the scheme macros: 1 DE, 2 MHD, 4 density floor, 8 scalar; the reconstruction
// (0 PCM, 1 PLMC, 2 PPMC, 3 PLMP, 4 PPMP) in bits 8-11 and the solver (0 HLLC, 1 Roe, 2 HLLD,
// 3 HLL, 4 exact) in bits 12-15.
int refh_scheme(void)
{
  int m = 0;
#ifdef DE
  m |= 1;
#endif
#ifdef MHD
  m |= 2;
#endif
#ifdef DENSITY_FLOOR
  m |= 4;
#endif
#ifdef SCALAR
  m |= 8;
#endif
#if defined(PLMC)
  m |= 1 << 8;
#elif defined(PPMC)
  m |= 2 << 8;
#elif defined(PLMP)
  m |= 3 << 8;
#elif defined(PPMP)
  m |= 4 << 8;
#endif
#if defined(ROE)
  m |= 1 << 12;
#elif defined(HLLD)
  m |= 2 << 12;
#elif defined(HLL)
  m |= 3 << 12;
#elif defined(EXACT)
  m |= 4 << 12;
#endif
  return m;
}

}  // extern "C"
