// tma.cu -- host side of the TMA staging: tensor-map encoding through the runtime's driver entry
// point (the library links only the CUDA runtime).
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "tma.cuh"

namespace cgb
{
namespace
{
using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                              const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeFn encode_fn()
{
  static EncodeFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeFn>(p);
    else
      cudaGetLastError();
  });
  return fn;
}
}  // namespace

bool tma_encode_4d(CUtensorMap *map, const void *base, int elem_bytes, long long nx, long long ny, long long nz,
                   long long nslot, int bx, int by, int bz)
{
  EncodeFn const fn = encode_fn();
  if (!fn || (elem_bytes != 4 && elem_bytes != 8)) return false;
  unsigned long long const e = (unsigned long long)elem_bytes;
  cuuint64_t const dims[4]    = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz, (cuuint64_t)nslot};
  cuuint64_t const strides[3] = {nx * e, nx * ny * e, nx * ny * nz * e};  // bytes, dimensions 1 .. 3
  if (((unsigned long long)(uintptr_t)base & 15ULL) || (strides[0] & 15) || (strides[1] & 15) || (strides[2] & 15))
    return false;
  if ((bx * e) % 16 || bx > 256 || by > 256 || bz > 256) return false;
  cuuint32_t const box[4]  = {(cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz, 1};
  cuuint32_t const estr[4] = {1, 1, 1, 1};
  CUresult const r = fn(map, elem_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4,
                        const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}
}  // namespace cgb
