// hydro_fast_hllc.cu -- the fast forms' predictor and corrector sweeps with the HLLC Riemann solver
// (hllc_cuda.cu), for single boxes and batch chunks, in fast FP64 and mixed precision.
#include "hydro_fast_body.cuh"

namespace cgb
{
cudaError_t fast_solver_hllc(const Box &b, int recon, int mixed, double *U, const Scratch &sc, double dt,
                             const double *dtp, cudaStream_t s, cudaEvent_t *marks)
{
  return fast_solver<SOLVER_HLLC>(b, recon, mixed, U, sc, dt, dtp, s, marks);
}

cudaError_t batch_solver_hllc(const BatchChunk &C, int recon, int mixed, int set, int nsl, cudaStream_t s)
{
  return batch_solver<SOLVER_HLLC>(C, recon, mixed, set, nsl, s);
}
}  // namespace cgb
