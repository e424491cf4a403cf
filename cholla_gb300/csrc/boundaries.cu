// boundaries.cu -- ghost-cell fill for one padded box (single GPU, no MPI faces): one launch
// over every cell, the ghost cells taking their mapped real cell (ghost.cuh).
#include "common.cuh"
#include "ghost.cuh"
#include "kernels.h"

namespace cgb
{
namespace
{
__global__ void k_ghost(Box b, double *__restrict__ U, Flags fl)
{
  for (long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x; id < b.n;
       id += (long long)gridDim.x * blockDim.x)
    ghost_cell(b, U, fl, id);
}
}  // namespace

cudaError_t set_boundaries(const Box &b, double *U, const int flags[6], cudaStream_t s)
{
  Flags const fl = ghost_flags(b, flags);
  long long blocks = (b.n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_ghost<<<(unsigned)blocks, 256, 0, s>>>(b, U, fl);
  return cudaGetLastError();
}
}  // namespace cgb
