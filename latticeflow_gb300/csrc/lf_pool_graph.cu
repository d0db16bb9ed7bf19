// Launchers of the residual-graph passes (BFS relabel, forward closure).
#include <mutex>

#include "lf_pool_graph.cuh"

namespace lfg {

// launches come from several host threads (server workers, TV batches)
static std::mutex mu;

cudaError_t launch_pool_bfs(const PoolBFS& p, int KA, int KB, bool single, int grid,
                                   int threads, size_t smem, cudaStream_t s) {
#define X(A, B)                                                                 \
  if (KA == A && KB == B) {                                                     \
    static int cap_t = 0, cap_f = 0;                                            \
    static size_t cap_smem = 0;                                                 \
    int ct, cf;                                                                 \
    {                                                                           \
    std::lock_guard<std::mutex> lk(mu);                                         \
    if (!cap_t || cap_smem != smem) {                                           \
      cap_t = occupancy_grid(k_pool_bfs<A, B, true>, threads, smem);            \
      cap_f = occupancy_grid(k_pool_bfs<A, B, false>, threads, smem);           \
      cap_smem = smem;                                                          \
    }                                                                           \
    ct = cap_t;                                                                 \
    cf = cap_f;                                                                 \
    }                                                                           \
    if (single) k_pool_bfs<A, B, true><<<std::min(grid, ct), threads, smem, s>>>(p); \
    else k_pool_bfs<A, B, false><<<std::min(grid, cf), threads, smem, s>>>(p);       \
    return cudaGetLastError();                                                  \
  }
  LF_POOL_PR_LIST(X)
#undef X
  return cudaErrorInvalidValue;
}

cudaError_t launch_pool_reach(const PoolReach& p, int KA, int KB, bool single, int grid,
                                     int threads, size_t smem, cudaStream_t s) {
#define X(A, B)                                                                 \
  if (KA == A && KB == B) {                                                     \
    static int cap_t = 0, cap_f = 0;                                            \
    static size_t cap_smem = 0;                                                 \
    int ct, cf;                                                                 \
    {                                                                           \
    std::lock_guard<std::mutex> lk(mu);                                         \
    if (!cap_t || cap_smem != smem) {                                           \
      cap_t = occupancy_grid(k_pool_reach<A, B, true>, threads, smem);          \
      cap_f = occupancy_grid(k_pool_reach<A, B, false>, threads, smem);         \
      cap_smem = smem;                                                          \
    }                                                                           \
    ct = cap_t;                                                                 \
    cf = cap_f;                                                                 \
    }                                                                           \
    if (single) k_pool_reach<A, B, true><<<std::min(grid, ct), threads, smem, s>>>(p); \
    else k_pool_reach<A, B, false><<<std::min(grid, cf), threads, smem, s>>>(p);       \
    return cudaGetLastError();                                                  \
  }
  LF_POOL_PR_LIST(X)
#undef X
  return cudaErrorInvalidValue;
}

}  // namespace lfg
