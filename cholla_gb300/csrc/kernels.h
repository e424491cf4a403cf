// kernels.h -- host-side entry points of the CUDA kernels (internal to libchollagb).
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace cgb
{
// FP64 hydro VL step in the reference's operation order (hydro_exact.cu).  Runs the
// predictor, the corrector and the finalize pass (DE select/sync, temperature floor when
// temp_floor != 0, and the CFL reduction into sc.dti when do_dt != 0).
cudaError_t hydro_exact_step(const Box &b, int recon, int solver, double *U, const Scratch &sc, double dt,
                             double U_floor, int temp_floor, int do_dt, cudaStream_t s);
cudaError_t hydro_calc_dt(const Box &b, const double *U, unsigned long long *dti, cudaStream_t s);
cudaError_t hydro_temperature_floor(const Box &b, double *U, double U_floor, cudaStream_t s);

// ghost-cell fill of all six faces in one launch (boundaries.cu)
cudaError_t set_boundaries(const Box &b, double *U, const int flags[6], cudaStream_t s);
}  // namespace cgb
