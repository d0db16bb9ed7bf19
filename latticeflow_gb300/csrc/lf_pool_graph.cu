// Launchers of the residual-graph passes (BFS relabel, forward closure).
#include "lf_pool_graph.cuh"

namespace lfg {

cudaError_t launch_pool_bfs(const PoolBFS& p, int KA, int KB, bool single, int grid,
                                   int threads, size_t smem, cudaStream_t s) {
#define X(A, B)                                                                 \
  if (KA == A && KB == B) {                                                     \
    if (single) k_pool_bfs<A, B, true><<<grid, threads, smem, s>>>(p);          \
    else k_pool_bfs<A, B, false><<<grid, threads, smem, s>>>(p);                \
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
    if (single) k_pool_reach<A, B, true><<<grid, threads, smem, s>>>(p);        \
    else k_pool_reach<A, B, false><<<grid, threads, smem, s>>>(p);              \
    return cudaGetLastError();                                                  \
  }
  LF_POOL_PR_LIST(X)
#undef X
  return cudaErrorInvalidValue;
}

}  // namespace lfg
