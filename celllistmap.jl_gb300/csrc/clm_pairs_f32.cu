// Instantiations of the cell-pair map kernel for float positions: every operator kind, self and cross
// pairs, exact and split forms, 2D and 3D.
#include "clm_pairs_kernel.cuh"

namespace clm {
namespace pk {

cudaError_t launch_pairs_plain(const LaunchSel& s, int& grid, cudaStream_t st, const PairArgs<float>& A) {
  return launch_plain_t<float>(s, grid, st, A);
}

int pairs_blocks_per_sm(const LaunchSel& s, const PairArgs<float>*) { return occupancy_t<float>(s); }

}  // namespace pk
}  // namespace clm
