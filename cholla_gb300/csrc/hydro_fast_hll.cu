// hydro_fast_hll.cu -- the fast forms' predictor and corrector sweeps with the HLL Riemann solver
// (hll_cuda.cu), for 3D boxes and batch chunks, in fast FP64 and mixed precision.
#include "hydro_fast_body.cuh"

namespace cgb
{
cudaError_t fast_solver_hll(const Box &b, int recon, int mixed, double *U, const Scratch &sc, double dt,
                            const double *dtp, cudaStream_t s, cudaEvent_t *marks)
{
  return fast_solver<SOLVER_HLL>(b, recon, mixed, U, sc, dt, dtp, s, marks);
}

cudaError_t batch_solver_hll(const BatchChunk &C, int recon, int mixed, int set, int nsl, cudaStream_t s)
{
  return batch_solver<SOLVER_HLL>(C, recon, mixed, set, nsl, s);
}
}  // namespace cgb
