// Instantiation of the tile push/relabel kernels for int capacities.
#include "lf_pr_tile.cuh"

namespace lfg {
template cudaError_t launch_pr_tile<int>(const PRParams<int>&, cudaStream_t);
}  // namespace lfg
