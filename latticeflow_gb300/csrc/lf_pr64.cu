// Instantiation of the tile push/relabel kernels for long long capacities.
#include "lf_pr_tile.cuh"

namespace lfg {
template cudaError_t launch_pr_tile<long long>(const PRParams<long long>&, cudaStream_t);
}  // namespace lfg
