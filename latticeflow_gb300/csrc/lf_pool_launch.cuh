// Launcher of the push/relabel pool kernel (instantiated in lf_pool_pr32.cu
// and lf_pool_pr64.cu).
#pragma once

#include "lf_pool_runner.h"
#include <algorithm>
#include <mutex>
#include <type_traits>

#include "lf_pool_tile.cuh"

namespace lfg {

// kernel-size pairs compiled: every generated size alone (1-d, 2-d, 3-d),
// plus the 2-d mix of 4- and 8-connected lattices
#define LF_POOL_PR_LIST(X) \
  X(2, 2) X(4, 4) X(6, 6) X(8, 8) X(10, 10) X(12, 12) X(14, 14) X(16, 16) X(18, 18) \
  X(20, 20) X(24, 24) X(26, 26) X(28, 28) X(32, 32) X(36, 36) X(40, 40) X(48, 48) X(4, 8)

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

template <typename T, int A, int B, bool S>
inline auto pr_kernel() {
  if constexpr (std::is_same<T, int>::value && B <= 8) return k_pool_pr<A, B, S>;
  else return k_pool_pr_wide<T, A, B, S>;
}

template <typename T>
cudaError_t launch_pool_pr(const PoolPR<T>& p, int KA, int KB, int threads, size_t smem,
                           bool single, int grid, cudaStream_t s) {
  // launches come from several host threads (server workers, TV batches)
  static std::mutex mu;
#define X(A, B)                                                                            \
  if (KA == A && KB == B) {                                                                \
    auto kt = pr_kernel<T, A, B, true>();                                                  \
    auto kf = pr_kernel<T, A, B, false>();                                                 \
    static bool attr = false;                                                              \
    static int cap_t = 0, cap_f = 0;                                                       \
    static size_t cap_smem = 0;                                                            \
    int ct, cf;                                                                            \
    {                                                                                      \
      std::lock_guard<std::mutex> lk(mu);                                                  \
      if (!attr) {                                                                         \
        cudaFuncSetAttribute(kt, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024); \
        cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024); \
        cudaFuncSetAttribute(kt, cudaFuncAttributePreferredSharedMemoryCarveout, 100);     \
        cudaFuncSetAttribute(kf, cudaFuncAttributePreferredSharedMemoryCarveout, 100);     \
        attr = true;                                                                       \
      }                                                                                    \
      if (!cap_t || cap_smem != smem) {                                                    \
        cap_t = occupancy_grid(kt, threads, smem);                                         \
        cap_f = occupancy_grid(kf, threads, smem);                                         \
        cap_smem = smem;                                                                   \
      }                                                                                    \
      ct = cap_t;                                                                          \
      cf = cap_f;                                                                          \
    }                                                                                      \
    if (single) kt<<<std::min(grid, ct), threads, smem, s>>>(p);                           \
    else kf<<<std::min(grid, cf), threads, smem, s>>>(p);                                  \
    return cudaGetLastError();                                                             \
  }
  LF_POOL_PR_LIST(X)
#undef X
  return cudaErrorInvalidValue;
}

}  // namespace lfg
