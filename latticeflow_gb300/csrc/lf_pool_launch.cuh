// Launcher of the push/relabel pool kernel (instantiated in lf_pool_pr32.cu
// and lf_pool_pr64.cu).
#pragma once

#include "lf_pool_runner.h"
#include <algorithm>

#include "lf_pool_tile.cuh"

namespace lfg {

// kernel-size pairs compiled: every generated size alone, plus the 2-d mix of
// 4- and 8-connected lattices
#define LF_POOL_PR_LIST(X) \
  X(4, 4) X(6, 6) X(8, 8) X(12, 12) X(16, 16) X(18, 18) X(20, 20) X(24, 24) X(26, 26) \
  X(28, 28) X(32, 32) X(36, 36) X(40, 40) X(48, 48) X(4, 8)

// Blocks that fit on the device at once for this kernel and shape (the grid
// of a pass; its blocks stride over the queued tiles).
template <class Kern>
inline int occupancy_grid(Kern kernel, int threads, size_t smem) {
  int dev = 0, sms = 1, per = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem) != cudaSuccess || per < 1)
    per = 1;
  return per * sms;
}

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
    static int cap_t = 0, cap_f = 0;                                                       \
    static size_t cap_smem = 0;                                                            \
    if (!cap_t || cap_smem != smem) {                                                      \
      cap_t = occupancy_grid(k_pool_pr<T, A, B, true>, threads, smem);                     \
      cap_f = occupancy_grid(k_pool_pr<T, A, B, false>, threads, smem);                    \
      cap_smem = smem;                                                                     \
    }                                                                                      \
    if (single) k_pool_pr<T, A, B, true><<<std::min(grid, cap_t), threads, smem, s>>>(p);  \
    else k_pool_pr<T, A, B, false><<<std::min(grid, cap_f), threads, smem, s>>>(p);        \
    return cudaGetLastError();                                                             \
  }
  LF_POOL_PR_LIST(X)
#undef X
  return cudaErrorInvalidValue;
}

}  // namespace lfg
