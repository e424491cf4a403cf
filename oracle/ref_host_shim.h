/*
 * ref_host_shim.h -- force-included (g++ -include) ahead of the reference's own CUDA sources so
 * that they compile, unchanged, as host C++ and run on the CPU.
 *
 * TEST INFRASTRUCTURE ONLY: the reference's kernels executed on the host are a second oracle.
 * They pin the FP64 restatement in cholla_oracle.cpp on the CPU, bit for bit, for every scheme
 * option the reference's VL integrators compile with, without a GPU.  Nothing in the product
 * links or loads them.
 *
 * How a kernel runs here: the reference launches every VL-path kernel through the macro
 * hipLaunchKernelGGL (src/utils/gpu.hpp:124).  After gpu.hpp is processed this header redefines
 * that macro to call the kernel body once per (block, thread) index with threadIdx / blockIdx /
 * blockDim / gridDim set as thread-local variables.  Blocks run in parallel on OpenMP threads.
 * This is exact for the VL-path kernels: every one of them is a per-thread map with no shared
 * memory, no barrier and no atomic, and within a kernel no thread reads what another writes.
 * The device-side reductions (Calc_dt, temperature floor) use shared memory and warp shuffles; they
 * are compiled but never launched here, and their intrinsics abort if reached.
 *
 * Device memory is host memory: cudaMalloc / cudaMemset / cudaFree / cudaMemcpy become calloc /
 * memset / free / memcpy.  The sources are compiled with -ffp-contract=off, the host counterpart
 * of the reference build's -fmad=false; division and sqrt are correctly rounded on both sides.
 */
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <stdexcept>

#define __launch_bounds__(...)

static constexpr int warpSize = 32;
// integer min / max as CUDA's device library declares them (hydro_cuda.cu clamps indices with them)
inline int max(int a, int b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
// CUDA's reciprocal square root and reciprocal hypotenuse (used by the MHD characteristic
// projection, reconstruction.h:342,387), defined here from their mathematical meaning as a
// correctly rounded sqrt / hypot followed by a division: the same substitution the FP64
// restatement makes, so the two agree bit for bit; both may differ from the GPU in the last bit.
inline double rsqrt(double x) { return 1.0 / std::sqrt(x); }
inline double rhypot(double a, double b) { return 1.0 / std::hypot(a, b); }
// shared-memory reductions are not launched on the host
inline void __syncthreads() { std::abort(); }
template <class T>
T atomicMax(T *, T)
{
  std::abort();
}
template <class T>
T atomicMin(T *, T)
{
  std::abort();
}
template <class T>
T __shfl_down_sync(unsigned, T, int)
{
  std::abort();
}

static thread_local uint3 threadIdx, blockIdx;
static thread_local dim3 blockDim, gridDim;

// ---- the runtime calls the VL integrators make, on host memory ----
inline cudaError_t refh_malloc(void **p, size_t n)
{
  *p = std::calloc(n ? n : 1, 1);
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
inline cudaError_t refh_free(void *p)
{
  std::free(p);
  return cudaSuccess;
}
inline cudaError_t refh_memset(void *p, int v, size_t n)
{
  std::memset(p, v, n);
  return cudaSuccess;
}
inline cudaError_t refh_memcpy(void *d, const void *s, size_t n)
{
  std::memcpy(d, s, n);
  return cudaSuccess;
}
template <class K>
cudaError_t refh_occupancy(int *grid, int *block, K)
{
  *grid  = 0;
  *block = 256;
  return cudaSuccess;
}
#define cudaMalloc(P, N)                                  refh_malloc((void **)(P), (N))
#define cudaFree(P)                                       refh_free((void *)(P))
#define cudaMemset(P, V, N)                               refh_memset((P), (V), (N))
#define cudaMemcpy(D, S, N, K)                            refh_memcpy((D), (S), (N))
#define cudaDeviceSynchronize()                           cudaSuccess
#define cudaPeekAtLastError()                             cudaSuccess
#define cudaGetLastError()                                cudaSuccess
#define cudaGetErrorString(E)                             "host emulation"
#define cudaOccupancyMaxPotentialBlockSize(G, B, K, ...)  refh_occupancy((G), (B), (K))

#include "utils/gpu.hpp"

// ---- kernel launches: every (block, thread) index in turn; blocks in parallel ----
#undef hipLaunchKernelGGL
template <class K>
void refh_launch(dim3 g, dim3 b, const K &k)
{
  long const nb = (long)g.x * g.y * g.z;
#pragma omp parallel for schedule(dynamic, 8)
  for (long bi = 0; bi < nb; bi++) {
    gridDim    = g;
    blockDim   = b;
    blockIdx.x = (unsigned)(bi % g.x);
    blockIdx.y = (unsigned)((bi / g.x) % g.y);
    blockIdx.z = (unsigned)(bi / ((long)g.x * g.y));
    for (unsigned tz = 0; tz < b.z; tz++)
      for (unsigned ty = 0; ty < b.y; ty++)
        for (unsigned tx = 0; tx < b.x; tx++) {
          threadIdx.x = tx, threadIdx.y = ty, threadIdx.z = tz;
          k();
        }
  }
}
#define hipLaunchKernelGGL(F, G, B, M, S, ...) refh_launch(dim3(G), dim3(B), [&]() { F(__VA_ARGS__); })
