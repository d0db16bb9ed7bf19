// Tensor maps for the TMA-staged passes: the driver's cuTensorMapEncodeTiled,
// taken once through the runtime's driver entry-point query (no link
// against the driver library), and one encoding call with the settings
// every staged pass uses (no interleave, no swizzle, 128-byte L2 promotion,
// zero fill outside the tensor).
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <mutex>

namespace lfg {

inline PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// rank <= 5; strides[rank - 1] in bytes (multiples of 16); unit element strides
inline bool encode_tensor_map(CUtensorMap* m, void* base, int rank, const cuuint64_t* dims,
                              const cuuint64_t* strides, const cuuint32_t* box,
                              CUtensorMapDataType type = CU_TENSOR_MAP_DATA_TYPE_INT32) {
  auto fn = tensor_map_encoder();
  if (!fn) return false;
  const cuuint32_t es[5] = {1, 1, 1, 1, 1};
  return fn(m, type, rank, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace lfg
