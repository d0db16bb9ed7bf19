// Launcher of the push/relabel pool kernel (instantiated in lf_pool_pr32.cu
// and lf_pool_pr64.cu).
#pragma once

#include "lf_pool_runner.h"
#include "lf_pool_tile.cuh"

namespace lfg {

// kernel-size pairs compiled: every generated size alone, plus the 2-d mix of
// 4- and 8-connected lattices
#define LF_POOL_PR_LIST(X) \
  X(4, 4) X(6, 6) X(8, 8) X(12, 12) X(16, 16) X(18, 18) X(20, 20) X(24, 24) X(26, 26) \
  X(28, 28) X(32, 32) X(36, 36) X(40, 40) X(48, 48) X(4, 8)

template <typename T>
cudaError_t launch_pool_pr(const PoolPR<T>& p, int KA, int KB, int threads, size_t smem,
                           bool single, int grid, cudaStream_t s) {
#define X(A, B)                                                                            \
  if (KA == A && KB == B) {                                                                \
    static bool attr = false;                                                              \
    if (!attr) {                                                                           \
      cudaFuncSetAttribute(k_pool_pr<T, A, B, true>,                                       \
                           cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);       \
      cudaFuncSetAttribute(k_pool_pr<T, A, B, false>,                                      \
                           cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);       \
      cudaFuncSetAttribute(k_pool_pr<T, A, B, true>,                                       \
                           cudaFuncAttributePreferredSharedMemoryCarveout, 100);           \
      cudaFuncSetAttribute(k_pool_pr<T, A, B, false>,                                      \
                           cudaFuncAttributePreferredSharedMemoryCarveout, 100);           \
      attr = true;                                                                         \
    }                                                                                      \
    if (single) k_pool_pr<T, A, B, true><<<grid, threads, smem, s>>>(p);                   \
    else k_pool_pr<T, A, B, false><<<grid, threads, smem, s>>>(p);                         \
    return cudaGetLastError();                                                             \
  }
  LF_POOL_PR_LIST(X)
#undef X
  return cudaErrorInvalidValue;
}

}  // namespace lfg
