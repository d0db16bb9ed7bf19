// Instantiation of the push/relabel pool kernels for long long capacities.
#include "lf_pool_launch.cuh"

namespace lfg {
template cudaError_t launch_pool_pr<long long>(const PoolPR<long long>&, int, int, int, size_t, bool, int, cudaStream_t);
}  // namespace lfg
