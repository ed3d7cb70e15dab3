// Grouped launches of reconstruction passes A and B (projection): one launch
// for up to kMaxItems holograms of one transform shape, grid z = item, grid y
// = the largest item's slice groups (ph_passes.cuh, GROUPED forms).
#include "ph_launch.cuh"

namespace ph {

cudaError_t launch_recon_a_group(int n, const ReconAGrouped &b, cudaStream_t s) {
    int gy = 1;
    for (int i = 0; i < b.nitems; ++i) gy = std::max(gy, (b.item_nb(i) + b.item_group(i) - 1) / b.item_group(i));
    return launch_len<true>(n, b, b.nx, gy, s, b.nitems);
}

cudaError_t launch_recon_b_group(int n, const ReconB<EPI_PROJ, true> &b, cudaStream_t s) {
    int gy = 1;
    for (int i = 0; i < b.nitems; ++i) gy = std::max(gy, (b.item_nb(i) + b.item_group(i) - 1) / b.item_group(i));
    return launch_len<false>(n, b, b.rows, gy, s, b.nitems);
}

}  // namespace ph
