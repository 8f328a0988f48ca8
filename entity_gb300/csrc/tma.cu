// Host side of the TMA field-window loads: the tensor-map encoder, reached
// through the runtime's driver entry-point query so that the library links
// against the CUDA runtime only.
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "tma.cuh"

namespace pic {

namespace {

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encoder() {
  static std::once_flag once;
  static EncodeTiledFn  fn = nullptr;
  std::call_once(once, [] {
    void*                           p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

}  // namespace

bool tma_enabled() {
  const char* v = std::getenv("ENTITY_PIC_NO_TMA");
  return !(v && std::strcmp(v, "1") == 0);
}

bool encode_field_map(CUtensorMap* map, const void* base, int real_bytes, int rank,
                      const int64_t* dims, const int64_t* strides, const int* box) {
  if (rank < 1 || rank > 5 || (real_bytes != 4 && real_bytes != 8)) return false;
  if (reinterpret_cast<uintptr_t>(base) % 16 != 0) return false;
  if ((box[0] * real_bytes) % 16 != 0) return false;
  cuuint64_t gdim[5], gstride[4];
  cuuint32_t bdim[5], estride[5];
  for (int d = 0; d < rank; ++d) {
    if (dims[d] < 1 || dims[d] > (int64_t(1) << 32)) return false;
    if (box[d] < 1 || box[d] > 256) return false;
    gdim[d]    = (cuuint64_t)dims[d];
    bdim[d]    = (cuuint32_t)box[d];
    estride[d] = 1;
  }
  for (int d = 1; d < rank; ++d) {
    const int64_t b = strides[d - 1] * real_bytes;
    if (b <= 0 || b % 16 != 0 || b >= (int64_t(1) << 40)) return false;
    gstride[d - 1] = (cuuint64_t)b;
  }
  const EncodeTiledFn fn = encoder();
  if (!fn) return false;
  const CUresult r =
      fn(map, real_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
         (cuuint32_t)rank, const_cast<void*>(base), gdim, gstride, bdim, estride,
         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace pic
