// hydro_exact_roe.cu -- the exact FP64 predictor + corrector with the ROE Riemann solver
// (instantiated here alone; the kernels are in hydro_exact_step.cuh).  Built with -fmad=false.
#include "hydro_exact_step.cuh"

namespace cgb
{
cudaError_t exact_step_roe(const Box &b, int recon, double *U, const Scratch &sc, double dt, const double *dtp,
                  cudaStream_t s, cudaEvent_t *marks)
{
  return exact_solver_step<SOLVER_ROE>(b, recon, U, sc, dt, dtp, s, marks);
}
}  // namespace cgb
