// selftest.cu -- device self-checks of arithmetic helpers that replace hardware instructions:
// the integer-pipe binary64 <-> binary32 conversions of hydro_fast.cuh against the hardware
// conversions, bit for bit (a NaN only has to stay a NaN); the fast FP64 reciprocal and square
// root against CUDA's correctly rounded ones; the FP64 pipe's FMA rate.
#include <cuda_runtime.h>

#include "../../include/cholla_gb300.h"
#include "hydro_fast.cuh"
#include "kernels.h"
#include "tma.cuh"

namespace
{
// mismatches: [0] narrowing (to_f32 vs (float)), [1] widening (to_f64 vs (double)); each input
// bit pattern is also read as the binary32 of its low word for the widening check; two NaNs match
__global__ void k_check_conversions(const double *__restrict__ x, long long n, unsigned long long *__restrict__ bad)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double const v = x[i];
    float const a = cgb::hf::to_f32(v), b = (float)v;
    if (__float_as_uint(a) != __float_as_uint(b) && !(isnan(a) && isnan(b))) atomicAdd(&bad[0], 1ULL);
    float const f = __uint_as_float((unsigned)__double2loint(v));
    double const c = cgb::hf::to_f64(f), d = (double)f;
    if (__double_as_longlong(c) != __double_as_longlong(d) && !(isnan(c) && isnan(d))) atomicAdd(&bad[1], 1ULL);
  }
}

// out[0 n + i] = rcp(x), out[1 n + i] = CUDA's correctly rounded 1 / x, out[2 n + i] = sqrtT(|x|),
// out[3 n + i] = CUDA's correctly rounded sqrt(|x|)
__global__ void k_fast_math(const double *__restrict__ x, long long n, double *__restrict__ out)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double const v = x[i], a = fabs(v);
    out[i]         = cgb::hf::rcp(v);
    out[n + i]     = __drcp_rn(v);
    out[2 * n + i] = cgb::hf::sqrtT(a);
    out[3 * n + i] = __dsqrt_rn(a);
  }
}

// FP64-pipe throughput: each thread runs 8 independent chains of `iters` FP64 fused multiply-adds
// (enough independent work per warp to keep the pipe issuing), writing one sum so nothing is
// removed as dead code
__global__ void k_fp64_rate(double *__restrict__ out, int iters, double a, double b)
{
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; k++) x[k] = (double)(threadIdx.x + k) * 1e-3;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = fma(x[k], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += x[k];
  if (s == 1.2345e300) out[blockIdx.x] = s;  // never true for these inputs; keeps the chains live
}

// an mbarrier that expects 16 bytes which no copy delivers: every thread's bounded wait runs out
__global__ void k_tma_timeout(int *__restrict__ status, unsigned limit)
{
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    cgb::mbar_init(&bar, 1);
    cgb::fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) cgb::mbar_arrive_expect_tx(&bar, 16);
  bool const ok = __syncthreads_and(cgb::mbar_wait(&bar, 0, limit));
  if (!ok && threadIdx.x == 0) atomicOr(status, cgb::STATUS_TMA_TIMEOUT);
}
}  // namespace

extern "C" int cgb_selftest_tma_timeout(int *d_status, unsigned limit, void *stream)
{
  if (!d_status) return CGB_ERR_ARGS;
  cudaStream_t const s = (cudaStream_t)stream;
  k_tma_timeout<<<1, 64, 0, s>>>(d_status, limit);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? CGB_OK : CGB_ERR_CUDA;
}

// FP64 fused multiply-adds per second of the whole GPU, measured with events on `stream`
extern "C" int cgb_selftest_fp64_rate(int iters, double *fma_per_s, void *stream)
{
  if (!fma_per_s || iters <= 0) return CGB_ERR_ARGS;
  cudaStream_t const s = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  unsigned const blocks = (unsigned)sms * 8u, threads = 256u;
  double *d            = nullptr;
  cudaEvent_t ev[2]    = {nullptr, nullptr};
  if (e == cudaSuccess) e = cudaMallocAsync((void **)&d, blocks * sizeof(double), s);
  if (e == cudaSuccess) e = cudaEventCreate(&ev[0]);
  if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
  float ms = 0.f;
  if (e == cudaSuccess) {
    k_fp64_rate<<<blocks, threads, 0, s>>>(d, iters / 8 + 1, 0.999999, 1e-7);  // warm-up
    cudaEventRecord(ev[0], s);
    k_fp64_rate<<<blocks, threads, 0, s>>>(d, iters, 0.999999, 1e-7);
    cudaEventRecord(ev[1], s);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev[0], ev[1]);
  }
  if (d) cudaFreeAsync(d, s);
  if (ev[0]) cudaEventDestroy(ev[0]);
  if (ev[1]) cudaEventDestroy(ev[1]);
  if (e != cudaSuccess || !(ms > 0.f)) return CGB_ERR_CUDA;
  *fma_per_s = (double)blocks * threads * 8.0 * iters / (ms * 1e-3);
  return CGB_OK;
}

extern "C" int cgb_set_tma(int enable)
{
  cgb::set_sweep_tma(enable);
  return CGB_OK;
}

extern "C" int cgb_selftest_fast_math(const double *d_values, long long n, double *d_out, void *stream)
{
  if (!d_values || !d_out || n < 0) return CGB_ERR_ARGS;
  cudaStream_t const s = (cudaStream_t)stream;
  if (n > 0) k_fast_math<<<1024, 256, 0, s>>>(d_values, n, d_out);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? CGB_OK : CGB_ERR_CUDA;
}

extern "C" int cgb_selftest_conversions(const double *d_values, long long n, unsigned long long *mismatches,
                                        void *stream)
{
  if (!d_values || n < 0 || !mismatches) return CGB_ERR_ARGS;
  cudaStream_t const s  = (cudaStream_t)stream;
  unsigned long long *d = nullptr;
  cudaError_t e         = cudaMallocAsync((void **)&d, 2 * sizeof(unsigned long long), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d, 0, 2 * sizeof(unsigned long long), s);
  if (e == cudaSuccess && n > 0) {
    k_check_conversions<<<1024, 256, 0, s>>>(d_values, n, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(mismatches, d, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (d) cudaFreeAsync(d, s);
  return e == cudaSuccess ? CGB_OK : CGB_ERR_CUDA;
}
