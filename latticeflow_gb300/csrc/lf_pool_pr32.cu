// Instantiation of the push/relabel pool kernels for int capacities.
#include "lf_pool_launch.cuh"

namespace lfg {
template cudaError_t launch_pool_pr<int>(const PoolPR<int>&, int, int, int, size_t, bool, int, cudaStream_t);
}  // namespace lfg
