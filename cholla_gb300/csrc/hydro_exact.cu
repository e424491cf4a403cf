// hydro_exact.cu -- the exact FP64 VL hydro step (PCM / PLMC / PPMC / PLMP / PPMP x HLLC / Roe /
// HLL / exact, dual energy, floors): run-time dispatch over the per-solver predictor + corrector
// (hydro_exact_step.cuh, one translation unit per solver), then the finalize pass.
//
// Built with -fmad=false: every kernel keeps the reference's operation order, so the result
// equals the reference's FP64 build bit for bit.
//
//   finalize   Uⁿ⁺¹          dual-energy selection + sync, temperature floor and the CFL
//                            reduction on the new state (hydro_cuda.cu:949-1099, 1117-1153, 514-597)
//
// Interface states and fluxes never leave the SM.
#include <cfloat>

#include "common.cuh"
#include "hydro_math.cuh"
#include "kernels.h"

namespace cgb
{

// hydro_exact_<solver>.cu
cudaError_t exact_step_hllc(const Box &b, int recon, double *U, const Scratch &sc, double dt, const double *dtp,
                            cudaStream_t s, cudaEvent_t *marks);
cudaError_t exact_step_roe(const Box &b, int recon, double *U, const Scratch &sc, double dt, const double *dtp,
                           cudaStream_t s, cudaEvent_t *marks);
cudaError_t exact_step_hll(const Box &b, int recon, double *U, const Scratch &sc, double dt, const double *dtp,
                           cudaStream_t s, cudaEvent_t *marks);
cudaError_t exact_step_exact(const Box &b, int recon, double *U, const Scratch &sc, double dt, const double *dtp,
                             cudaStream_t s, cudaEvent_t *marks);

namespace
{
// ------------------------------------------------------------------------------------------
// finalize: negative-density average, DE select + sync, temperature floor, CFL reduction
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ double hydro_inverse_crossing_time(double E, double d, double d_inv, double vx, double vy,
                                                              double vz, double dx, double dy, double dz,
                                                              double gamma)
{
  // hydro_cuda.cu:404-419 hydroInverseCrossingTime
  double const P  = (E - 0.5 * d * (vx * vx + vy * vy + vz * vz)) * (gamma - 1.0);
  double const cs = sqrt(d_inv * gamma * P);
  double m        = fmax((fabs(vx) + cs) / dx, (fabs(vy) + cs) / dy);
  m               = fmax(m, (fabs(vz) + cs) / dz);
  m               = fmax(m, 0.0);
  return m;
}

// hydro_cuda.cu:473-512 Calc_dt_2D: the pressure floored at TINY, the larger of the two crossing rates
__device__ __forceinline__ double hydro_inverse_crossing_time_2d(double E, double d, double d_inv, double vx,
                                                                 double vy, double vz, double dx, double dy,
                                                                 double gamma)
{
  double P = (E - 0.5 * d * (vx * vx + vy * vy + vz * vz)) * (gamma - 1.0);
  P        = fmax(P, TINY);
  double const cs = sqrt(d_inv * gamma * P);
  return fmax(-DBL_MAX, fmax((fabs(vx) + cs) / dx, (fabs(vy) + cs) / dy));
}

__device__ __forceinline__ void block_max_to(double v, unsigned long long *dst)
{
  // values are >= 0 (or -DBL_MAX for threads without a cell): compare as ordered bit patterns
  __shared__ double red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    int const nw = (blockDim.x + 31) >> 5;
    v            = (lane < nw) ? red[lane] : -1.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    if (lane == 0 && v >= 0.0) atomicMax(dst, (unsigned long long)__double_as_longlong(v));
  }
}

__global__ void __launch_bounds__(256) k_finalize(Box b, double *__restrict__ U, const double *__restrict__ Epre,
                                                  unsigned long long *__restrict__ dti, int *__restrict__ status,
                                                  double U_floor, int temp_floor, int do_dt)
{
  int const ng = b.ng;
  bool const one_d = (b.ny == 1 && b.nz == 1), two_d = (b.nz == 1 && b.ny > 1);
  int const rx = b.nx - 2 * ng, ry = one_d ? 1 : b.ny - 2 * ng, rz = b.nz == 1 ? 1 : b.nz - 2 * ng;
  long long const nreal = (long long)rx * ry * rz;
  long long const r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double m = -1.0;
  if (r < nreal) {
    int const x = (int)(r % rx) + ng;
    int const y = one_d ? 0 : (int)((r / rx) % ry) + ng;
    int const z = b.nz == 1 ? 0 : (int)(r / ((long long)rx * ry)) + ng;
    long long const n = b.n, id = b.id(x, y, z);
    double const d = U[id], d_inv = 1.0 / d;
    double const vx = U[n + id] * d_inv, vy = U[2 * n + id] * d_inv, vz = U[3 * n + id] * d_inv;
    double E = U[4 * n + id];
    if (b.de) {
      // hydro_cuda.cu:949-1016 Select_Internal_Energy_3D, then :1070-1099 Sync_Energies_3D
      long long const fge = (long long)(b.nf - 1) * n;
      double Emax;
      if (one_d) {
        int const imo = max(x - 1, ng), ipo = min(x + 1, b.nx - ng - 1);
        Emax = fmax(Epre[imo], E);
        Emax = fmax(Emax, Epre[ipo]);
      } else if (two_d) {  // hydro_cuda.cu:880-933 Select_Internal_Energy_2D
        Emax = fmax(Epre[b.id(max(x - 1, ng), y, 0)], E);
        Emax = fmax(Emax, Epre[b.id(min(x + 1, b.nx - ng - 1), y, 0)]);
        Emax = fmax(Emax, Epre[b.id(x, max(y - 1, ng), 0)]);
        Emax = fmax(Emax, Epre[b.id(x, min(y + 1, b.ny - ng - 1), 0)]);
      } else {
        Emax = fmax(Epre[b.id(max(x - 1, ng), y, z)], E);
        Emax = fmax(Emax, Epre[b.id(min(x + 1, b.nx - ng - 1), y, z)]);
        Emax = fmax(Emax, Epre[b.id(x, max(y - 1, ng), z)]);
        Emax = fmax(Emax, Epre[b.id(x, min(y + 1, b.ny - ng - 1), z)]);
        Emax = fmax(Emax, Epre[b.id(x, y, max(z - 1, ng))]);
        Emax = fmax(Emax, Epre[b.id(x, y, min(z + 1, b.nz - ng - 1))]);
      }
      double const U_adv   = U[fge + id];
      double const U_total = E - 0.5 * d * (vx * vx + vy * vy + vz * vz);
      double Ui            = ((U_total / E > ETA_1) or (U_total / Emax > ETA_2)) ? U_total : U_adv;
      Ui                   = fmax(Ui, TINY);
      U[fge + id]          = Ui;
      E                    = 0.5 * d * (vx * vx + vy * vy + vz * vz) + Ui;
      U[4 * n + id]        = E;
    }
    if (temp_floor) {
      // hydro_cuda.cu:1117-1153 Temperature_Floor_Kernel
      double const Ekin = 0.5 * d * (vx * vx + vy * vy + vz * vz);
      double Ui         = (E - Ekin) / d;
      if (Ui < U_floor) {
        E             = Ekin + d * U_floor;
        U[4 * n + id] = E;
      }
      if (b.de) {
        long long const fge = (long long)(b.nf - 1) * n;
        Ui                  = U[fge + id] / d;
        if (Ui < U_floor) U[fge + id] = d * U_floor;
      }
    }
    if (bad_cell(d, E)) atomicOr(status, STATUS_NONFINITE);
    if (do_dt) {
      if (one_d) {
        // hydro_cuda.cu:437-471 Calc_dt_1D
        double P = (E - 0.5 * d * (vx * vx + vy * vy + vz * vz)) * (b.gamma - 1.0);
        P        = fmax(P, TINY);
        double const cs = sqrt(d_inv * b.gamma * P);
        m               = fmax(-1.0, (fabs(vx) + cs) / b.dx);
      } else if (two_d) {
        m = hydro_inverse_crossing_time_2d(E, d, d_inv, vx, vy, vz, b.dx, b.dy, b.gamma);
      } else {
        m = hydro_inverse_crossing_time(E, d, d_inv, vx, vy, vz, b.dx, b.dy, b.dz, b.gamma);
      }
    }
  }
  if (do_dt) block_max_to(m, dti);
}

// Average_Cell_Single_Field for cells the corrector found with negative density
__global__ void k_negative_density_average(Box b, double *__restrict__ U)
{
  int const ng = b.ng;
  int const rx = b.nx - 2 * ng, ry = b.ny - 2 * ng, rz = b.nz - 2 * ng;
  long long const nreal = (long long)rx * ry * rz;
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < nreal;
       r += (long long)gridDim.x * blockDim.x) {
    int const x = (int)(r % rx) + ng, y = (int)((r / rx) % ry) + ng, z = (int)(r / ((long long)rx * ry)) + ng;
    long long const id = b.id(x, y, z);
    if (U[id] < b.density_floor && !(U[id] > 0)) {
      U[id] = (U[b.id(x - 1, y, z)] + U[b.id(x + 1, y, z)] + U[b.id(x, y - 1, z)] + U[b.id(x, y + 1, z)] +
               U[b.id(x, y, z - 1)] + U[b.id(x, y, z + 1)]) /
              6;
    }
  }
}

// standalone CFL reduction over the real cells (hydro_cuda.cu:514-597 Calc_dt_3D / Calc_dt_1D)
__global__ void __launch_bounds__(256) k_calc_dt(Box b, const double *__restrict__ U, unsigned long long *__restrict__ dti)
{
  int const ng = b.ng;
  bool const one_d = (b.ny == 1 && b.nz == 1), two_d = (b.nz == 1 && b.ny > 1);
  int const rx = b.nx - 2 * ng, ry = one_d ? 1 : b.ny - 2 * ng, rz = b.nz == 1 ? 1 : b.nz - 2 * ng;
  long long const nreal = (long long)rx * ry * rz;
  double m = -1.0;
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < nreal;
       r += (long long)gridDim.x * blockDim.x) {
    int const x = (int)(r % rx) + ng;
    int const y = one_d ? 0 : (int)((r / rx) % ry) + ng;
    int const z = b.nz == 1 ? 0 : (int)(r / ((long long)rx * ry)) + ng;
    long long const n = b.n, id = b.id(x, y, z);
    double const d = U[id], d_inv = 1.0 / d;
    double const vx = U[n + id] * d_inv, vy = U[2 * n + id] * d_inv, vz = U[3 * n + id] * d_inv;
    double const E = U[4 * n + id];
    if (one_d) {
      double P = (E - 0.5 * d * (vx * vx + vy * vy + vz * vz)) * (b.gamma - 1.0);
      P        = fmax(P, TINY);
      double const cs = sqrt(d_inv * b.gamma * P);
      m               = fmax(m, (fabs(vx) + cs) / b.dx);
    } else if (two_d) {
      m = fmax(m, hydro_inverse_crossing_time_2d(E, d, d_inv, vx, vy, vz, b.dx, b.dy, b.gamma));
    } else {
      m = fmax(m, hydro_inverse_crossing_time(E, d, d_inv, vx, vy, vz, b.dx, b.dy, b.dz, b.gamma));
    }
  }
  block_max_to(m, dti);
}

__global__ void k_temperature_floor(Box b, double *__restrict__ U, double U_floor)
{
  int const ng = b.ng;
  bool const one_d = (b.ny == 1 && b.nz == 1);
  int const rx = b.nx - 2 * ng, ry = one_d ? 1 : b.ny - 2 * ng, rz = one_d ? 1 : b.nz - 2 * ng;
  long long const nreal = (long long)rx * ry * rz;
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < nreal;
       r += (long long)gridDim.x * blockDim.x) {
    int const x = (int)(r % rx) + ng;
    int const y = one_d ? 0 : (int)((r / rx) % ry) + ng;
    int const z = one_d ? 0 : (int)(r / ((long long)rx * ry)) + ng;
    long long const n = b.n, id = b.id(x, y, z);
    double const d = U[id], d_inv = 1.0 / d;
    double const vx = U[n + id] * d_inv, vy = U[2 * n + id] * d_inv, vz = U[3 * n + id] * d_inv;
    double const E    = U[4 * n + id];
    double const Ekin = 0.5 * d * (vx * vx + vy * vy + vz * vz);
    double Ui         = (E - Ekin) / d;
    if (Ui < U_floor) U[4 * n + id] = Ekin + d * U_floor;
    if (b.de) {
      long long const fge = (long long)(b.nf - 1) * n;
      Ui                  = U[fge + id] / d;
      if (Ui < U_floor) U[fge + id] = d * U_floor;
    }
  }
}

}  // namespace

cudaError_t hydro_exact_step(const Box &b, int recon, int solver, double *U, const Scratch &sc, double dt,
                             const double *dt_dev, double U_floor, int temp_floor, int do_dt, cudaStream_t s,
                             cudaEvent_t *marks)
{
  bool const one_d = (b.ny == 1 && b.nz == 1), two_d = (b.nz == 1 && b.ny > 1);
  if (b.nz < 2 * b.ng + 1) temp_floor = 0;  // the reference's temperature floor acts in 3D only
  cudaError_t e;
  if (two_d) {
    e = hydro_2d_step(b, recon, solver, U, sc, dt, dt_dev, s);
  } else {
    switch (solver) {
    case SOLVER_ROE: e = exact_step_roe(b, recon, U, sc, dt, dt_dev, s, marks); break;
    case SOLVER_HLL: e = exact_step_hll(b, recon, U, sc, dt, dt_dev, s, marks); break;
    case SOLVER_EXACT: e = exact_step_exact(b, recon, U, sc, dt, dt_dev, s, marks); break;
    default: e = exact_step_hllc(b, recon, U, sc, dt, dt_dev, s, marks); break;
    }
  }
  if (e != cudaSuccess) return e;
  if (b.floor_on && !one_d && !two_d) {
    k_negative_density_average<<<152 * 4, 256, 0, s>>>(b, U);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  if (b.de || temp_floor || do_dt) {
    if (do_dt) {
      e = cudaMemsetAsync(sc.dti, 0, sizeof(unsigned long long), s);
      if (e != cudaSuccess) return e;
    }
    int const ng = b.ng;
    long long const nreal =
        (long long)(b.nx - 2 * ng) * (one_d ? 1 : b.ny - 2 * ng) * (b.nz == 1 ? 1 : b.nz - 2 * ng);
    k_finalize<<<(unsigned)((nreal + 255) / 256), 256, 0, s>>>(b, U, sc.Epre, sc.dti, sc.status, U_floor, temp_floor,
                                                               do_dt);
    e = cudaGetLastError();
  }
  if (marks) cudaEventRecord(marks[3], s);
  return e;
}

// dt = C_cfl / max_dti, clamped to t_end (main.cpp:258-261, grid3D.cpp:397); t advances by dt.
__global__ void k_cfl_dt(const unsigned long long *__restrict__ dti, double *__restrict__ dt_t, double c_cfl,
                         double t_end)
{
  double const m  = __longlong_as_double((long long)*dti);
  double dt       = c_cfl / m;
  double const t  = dt_t[1];
  if (t_end > 0.0 && t + dt > t_end) dt = t_end - t;
  dt_t[0] = dt;
  dt_t[1] = t + dt;
}

cudaError_t cfl_dt(const unsigned long long *dti, double *dt_t, double c_cfl, double t_end, cudaStream_t s)
{
  k_cfl_dt<<<1, 1, 0, s>>>(dti, dt_t, c_cfl, t_end);
  return cudaGetLastError();
}

cudaError_t hydro_calc_dt(const Box &b, const double *U, unsigned long long *dti, cudaStream_t s)
{
  cudaError_t e = cudaMemsetAsync(dti, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  k_calc_dt<<<152 * 8, 256, 0, s>>>(b, U, dti);
  return cudaGetLastError();
}

cudaError_t negative_density_average(const Box &b, double *U, cudaStream_t s)
{
  k_negative_density_average<<<152 * 4, 256, 0, s>>>(b, U);
  return cudaGetLastError();
}

// Temperature_Floor_Kernel acts on cells whose x, y and z all lie in the real range
// (hydro_cuda.cu:1130-1131), so on a 1D or 2D box (extent 1 in z) it changes nothing; neither does this.
cudaError_t hydro_temperature_floor(const Box &b, double *U, double U_floor, cudaStream_t s)
{
  if (b.nz < 2 * b.ng + 1) return cudaSuccess;
  k_temperature_floor<<<152 * 8, 256, 0, s>>>(b, U, U_floor);
  return cudaGetLastError();
}

}  // namespace cgb