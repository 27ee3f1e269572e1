// Instantiations of the cell-pair map kernel for double positions: every operator kind, self and cross
// pairs, exact and split forms, 2D and 3D.
#include "clm_pairs_kernel.cuh"

namespace clm {
namespace pk {

cudaError_t launch_pairs_plain(const LaunchSel& s, int& grid, cudaStream_t st, const PairArgs<double>& A) {
  return launch_plain_t<double>(s, grid, st, A);
}

int pairs_blocks_per_sm(const LaunchSel& s, const PairArgs<double>*) { return occupancy_t<double>(s); }

}  // namespace pk
}  // namespace clm
