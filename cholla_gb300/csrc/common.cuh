// common.cuh -- shared types for the GB300 VL hydro/MHD step.
//
// State layout (the reference's, src/grid/grid_enum.h:18-111): field-major doubles
//   U[f * n_cells + x + y*nx + z*nx*ny], fields d, mx, my, mz, E, [scalars], [Bx, By, Bz], [GasEnergy].
// Magnetic fields are face-centred at the +1/2 face of their cell.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace cgb
{

constexpr double TINY  = 1.0e-20;  // src/global/global.h:25
constexpr double ETA_1 = 0.001;    // src/global/global.h:62-73 (non-cosmology)
constexpr double ETA_2 = 0.035;
constexpr int NS_MAX   = 2;        // passive scalars supported by the fused kernels
constexpr int NQ_MAX   = 5 + NS_MAX + 1;

// Bits of the per-box device status word (collected with atomicOr by the kernels; read by the
// host through cgb_check_status / cgb_box_check_status / cgb_batch_job_status).
constexpr int STATUS_NEG_DENSITY = 1;  // a real cell's update gave density <= 0 (repaired by averaging)
constexpr int STATUS_NONFINITE   = 2;  // a real cell holds non-finite density or energy, or density <= 0 after repair
// (bit 4, STATUS_TMA_TIMEOUT in tma.cuh: a bounded wait for a TMA copy ran out and a tile was left undone)

// x is NaN or +-infinity (exponent bits all ones), tested on the integer pipe
__device__ __forceinline__ bool not_finite(double x) { return (__double2hiint(x) & 0x7ff00000) == 0x7ff00000; }
// a density or energy pair that makes the cell unusable: density not a finite positive number, or
// non-finite total energy (the conditions of the reference's "Thread crashed" report,
// hydro_cuda.cu:381-389, with the floors' negative-energy case left to the floors)
__device__ __forceinline__ bool bad_cell(double d, double E)
{
  return __double_as_longlong(d) <= 0 || not_finite(d) || not_finite(E);
}

// Device allocations of the library go through these (alloc.cu), so that a test can make the
// n-th one fail on the host (cgb_debug_fail_alloc) without touching the GPU.
cudaError_t dev_malloc(void **p, size_t bytes);
cudaError_t dev_malloc_pool_async(void **p, size_t bytes, cudaMemPool_t pool, cudaStream_t s);

// the values of the C ABI's CGB_PCM .. CGB_PPMP and CGB_HLLC .. CGB_EXACT
enum Recon { RECON_PCM = 0, RECON_PLMC = 1, RECON_PPMC = 2, RECON_PLMP = 3, RECON_PPMP = 4 };
enum Solver { SOLVER_HLLC = 0, SOLVER_ROE = 1, SOLVER_HLLD = 2, SOLVER_HLL = 3, SOLVER_EXACT = 4 };

// Everything a kernel needs to know about one padded box.  Passed by value.
struct Box {
  int nx, ny, nz;   // padded extents
  int ng;           // ghost layers
  int nf;           // fields in the state array
  int ns;           // passive scalars (fields 5 .. 5+ns-1)
  int de;           // dual energy: GasEnergy is field nf-1
  int mhd;          // face-centred B at fields 5+ns .. 7+ns
  int floor_on;     // DENSITY_FLOOR behaviour
  long long n;      // nx*ny*nz
  double gamma;
  double dx, dy, dz;
  double density_floor;
  // used by the fast / mixed forms only, set on the host by with_inverses(): 1/dx, 1/dy, 1/dz
  // and 1/(gamma - 1), so that no kernel thread divides by them
  double idx, idy, idz, ig1;
  // binary32 roundings of gamma, gamma - 1 and 1/(gamma - 1) for the mixed form, also set by
  // with_inverses() (a per-thread conversion would issue on the FP64 pipe)
  float gf, gm1f, ig1f;
  __host__ __device__ long long id(int x, int y, int z) const
  {
    return (long long)x + (long long)y * nx + (long long)z * nx * ny;
  }
  __host__ __device__ int fGE() const { return nf - 1; }
  __host__ __device__ int fB() const { return 5 + ns; }
  // number of fields carried by reconstruction / Riemann: d, m(3), E, scalars, [ge]
  __host__ __device__ int nq() const { return 5 + ns + (de ? 1 : 0); }
};

inline Box with_inverses(Box b)
{
  b.idx = 1.0 / b.dx, b.idy = 1.0 / b.dy, b.idz = 1.0 / b.dz, b.ig1 = 1.0 / (b.gamma - 1.0);
  b.gf = (float)b.gamma, b.gm1f = (float)(b.gamma - 1.0), b.ig1f = (float)b.ig1;
  return b;
}

// Device scratch of one box, owned by the library (allocated once per box shape).
struct Scratch {
  double *Uh;      // half-step state, nf fields
  double *GEp;     // GasEnergy after the pdV partial update (DE)
  double *Epre;    // total energy after the full update, before the DE sync (DE)
  double *emf;     // 3 edge-EMF fields (MHD)
  double *Fx, *Fy, *Fz;  // face fluxes (MHD path only)
  void *W;               // half-step primitives of the fast / mixed paths (nq fields, 8 bytes each)
  unsigned long long *dti;  // encoded max inverse time step (one per box)
  int *status;              // device status word (bad cells seen, ...)
  double *mhd;              // MHD step: U½, 6 interface-state and 3 flux arrays, EMFs (mhd_scratch_doubles)
};

}  // namespace cgb
