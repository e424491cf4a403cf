// kernels.h -- host-side entry points of the CUDA kernels (internal to libchollagb).
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace cgb
{
// FP64 hydro VL step in the reference's operation order (hydro_exact.cu).  Runs the
// predictor, the corrector and the finalize pass (DE select/sync, temperature floor when
// temp_floor != 0, and the CFL reduction into sc.dti when do_dt != 0).
// dt_dev != nullptr: the kernels read the time step from device memory (engine path).
// marks != nullptr: four events recorded before the predictor, after it, after the
// corrector and after the finalize pass (per-kernel timing).
cudaError_t hydro_exact_step(const Box &b, int recon, int solver, double *U, const Scratch &sc, double dt,
                             const double *dt_dev, double U_floor, int temp_floor, int do_dt, cudaStream_t s,
                             cudaEvent_t *marks = nullptr);
// dt_t[0] = C_cfl / max_dti (clamped so that t does not pass t_end when t_end > 0), dt_t[1] += dt_t[0]
cudaError_t cfl_dt(const unsigned long long *dti, double *dt_t, double c_cfl, double t_end, cudaStream_t s);
// Fast FP64 (mixed = 0) or mixed-precision (mixed = 1) step (hydro_fast.cu).  sc.W holds the
// primitives of Uⁿ and of U½: 2 * (nf + 1) fields of 8 bytes cover both element types.
cudaError_t hydro_fast_step(const Box &b, int recon, int solver, int mixed, double *U, const Scratch &sc, void *W,
                            double dt, const double *dt_dev, double U_floor, int temp_floor, int do_dt,
                            cudaStream_t s, cudaEvent_t *marks = nullptr);
// Average_Cell_Single_Field of the density for real cells left with negative density
cudaError_t negative_density_average(const Box &b, double *U, cudaStream_t s);
cudaError_t hydro_calc_dt(const Box &b, const double *U, unsigned long long *dti, cudaStream_t s);
cudaError_t hydro_temperature_floor(const Box &b, double *U, double U_floor, cudaStream_t s);

// MHD (mhd_exact.cu): the VL step with HLLD and constrained transport, FP64 in the reference's
// operation order.  scratch holds mhd_scratch_doubles(b) doubles and must start zeroed.
size_t mhd_scratch_doubles(const Box &b);
// dt_dev != null: dt is read on the device (the box engine keeps it there)
cudaError_t mhd_exact_step(const Box &b, int recon, double *U, double *scratch, double dt, const double *dt_dev,
                           cudaStream_t s);
// max inverse crossing time with the fast magnetosonic speed into *dti (cleared first)
cudaError_t mhd_calc_dt(const Box &b, const double *U, unsigned long long *dti, cudaStream_t s);
// max |div B| over the real cells into *out (as the bits of a non-negative double; cleared first)
cudaError_t mhd_max_divb(const Box &b, const double *U, unsigned long long *out, cudaStream_t s);

// dispatch on the arithmetic: 0 = FP64 in the reference's order, 1 = mixed, 2 = fast FP64
inline cudaError_t hydro_step(const Box &b, int recon, int solver, int precision, double *U, const Scratch &sc,
                              double dt, const double *dt_dev, double U_floor, int temp_floor, int do_dt,
                              cudaStream_t s, cudaEvent_t *marks = nullptr)
{
  if (precision == 0)
    return hydro_exact_step(b, recon, solver, U, sc, dt, dt_dev, U_floor, temp_floor, do_dt, s, marks);
  return hydro_fast_step(b, recon, solver, precision == 1 ? 1 : 0, U, sc, sc.W, dt, dt_dev, U_floor, temp_floor,
                         do_dt, s, marks);
}

// ghost-cell fill of all six faces in one launch (boundaries.cu)
cudaError_t set_boundaries(const Box &b, double *U, const int flags[6], cudaStream_t s);
}  // namespace cgb
