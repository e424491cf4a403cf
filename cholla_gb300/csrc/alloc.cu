// alloc.cu -- the library's device allocations, with a host-side failure injector.
//
// Every cudaMalloc / stream-ordered pool allocation of the library goes through dev_malloc /
// dev_malloc_pool_async.  cgb_debug_fail_alloc(n) makes the n-th allocation from then on report
// cudaErrorMemoryAllocation without calling CUDA, so the tests can check that each entry point
// turns an allocation failure into CGB_ERR_NOMEM and leaves the library usable.  The failure is
// made on the host: nothing runs on (or faults) the GPU.
#include <cuda_runtime.h>

#include <atomic>

#include "../../include/cholla_gb300.h"
#include "common.cuh"

namespace
{
std::atomic<int> g_fail_countdown{0};  // 0: off; k > 0: the k-th next allocation fails

bool injected_failure()
{
  int k = g_fail_countdown.load();
  while (k > 0) {
    if (g_fail_countdown.compare_exchange_weak(k, k - 1)) return k == 1;
  }
  return false;
}
}  // namespace

namespace cgb
{
cudaError_t dev_malloc(void **p, size_t bytes)
{
  if (injected_failure()) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMalloc(p, bytes);
}

cudaError_t dev_malloc_pool_async(void **p, size_t bytes, cudaMemPool_t pool, cudaStream_t s)
{
  if (injected_failure()) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMallocFromPoolAsync(p, bytes, pool, s);
}
}  // namespace cgb

extern "C" int cgb_debug_fail_alloc(int n)
{
  if (n < 0) return CGB_ERR_ARGS;
  g_fail_countdown.store(n);
  return CGB_OK;
}
