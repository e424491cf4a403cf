// hydro_fast_exact.cu -- the fast forms' predictor and corrector sweeps with the exact Riemann
// solver (exact_cuda.cu), for single boxes, 1D boxes and batch chunks, in fast FP64 and mixed
// precision (the star state is solved in FP64 in both).
#include "hydro_fast_body.cuh"

namespace cgb
{
cudaError_t fast_solver_exact(const Box &b, int recon, int mixed, double *U, const Scratch &sc, double dt,
                              const double *dtp, cudaStream_t s, cudaEvent_t *marks)
{
  return fast_solver<SOLVER_EXACT>(b, recon, mixed, U, sc, dt, dtp, s, marks);
}

cudaError_t batch_solver_exact(const BatchChunk &C, int recon, int mixed, int set, int nsl, cudaStream_t s)
{
  return batch_solver<SOLVER_EXACT>(C, recon, mixed, set, nsl, s);
}
}  // namespace cgb
