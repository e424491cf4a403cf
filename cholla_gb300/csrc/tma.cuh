// tma.cuh -- Tensor Memory Accelerator staging for the sweep tiles (sm_100 family).
//
// A field-major state array of one element type (the fast forms' primitives, float or double) is
// described to the TMA unit as a 4D tensor (x, y, z, slot), x contiguous.  A block copies the box of
// one slot it needs into shared memory with one cp.async.bulk.tensor instruction issued by one
// thread; completion is counted in bytes by an mbarrier that every thread waits on.  Boxes that
// reach outside the tensor are filled with zeros by the hardware.
//
// Waits are bounded: a block whose threads poll the mbarrier kTmaSpinLimit times without seeing
// the phase complete records status bit STATUS_TMA_TIMEOUT, waits once more (bounded) for the copies
// it issued, and leaves its tile undone; the host reports CGB_ERR_TIMEOUT.  Nothing spins forever.
#pragma once
#include <cuda.h>  // CUtensorMap and the encode function's type (the function itself comes from the runtime)
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace cgb
{
constexpr int STATUS_TMA_TIMEOUT = 4;        // a bounded wait for a TMA copy ran out
constexpr unsigned kTmaSpinLimit = 1u << 22;  // polls (each a try_wait with the hardware's own time slice)

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// make the initialised mbarrier visible to the async (TMA) proxy
__device__ __forceinline__ void fence_mbar_init()
{
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// order this thread's earlier generic-proxy shared-memory accesses before later async-proxy ones
// (the buffer a TMA copy overwrites was read by ordinary loads in the previous tile)
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// wait until the mbarrier's phase `parity` has completed; false if `limit` polls ran out
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, unsigned limit = kTmaSpinLimit)
{
  unsigned const a = smem_u32(bar);
  for (unsigned i = 0; i < limit; i++) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// one 4D tiled copy global -> shared of the box at (x, y, z, w), completing on `bar`
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y, int z,
                                            int w)
{
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(smem_u32(dst)),
      "l"((unsigned long long)map), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_u32(bar))
      : "memory");
}

// Host: encode the 4D tensor map of a [nslot][nz][ny][nx] array of elem_bytes-wide elements with a
// box of (bx, by, bz, 1).  False when the array cannot be described (the strides must be multiples
// of 16 bytes and the base 16-byte aligned) or the encode call is unavailable.
bool tma_encode_4d(CUtensorMap *map, const void *base, int elem_bytes, long long nx, long long ny, long long nz,
                   long long nslot, int bx, int by, int bz);
}  // namespace cgb
