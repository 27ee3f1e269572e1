// Instantiations of the cell-pair map kernel for batches of independent systems (self pairs;
// neighbour lists, scalar reductions and forces; exact and split forms; 2D and 3D).
#include "clm_pairs_kernel.cuh"

namespace clm {
namespace pk {

cudaError_t launch_pairs_batch(const LaunchSel& s, int& grid, cudaStream_t st, const PairArgs<float>& A) {
  return launch_batch_t<float>(s, grid, st, A);
}

cudaError_t launch_pairs_batch(const LaunchSel& s, int& grid, cudaStream_t st, const PairArgs<double>& A) {
  return launch_batch_t<double>(s, grid, st, A);
}

}  // namespace pk
}  // namespace clm
