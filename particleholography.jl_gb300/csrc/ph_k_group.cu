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

bool recon_a_group_tstore(int n) { return n == 256 || n == 512 || n == 1024 || n == 2048; }

cudaError_t launch_recon_a_group_tstore(int n, const ReconAGroupedTStore &b, const CUtensorMap &tm, cudaStream_t s) {
    int gy = 1;
    for (int i = 0; i < b.nitems; ++i) gy = std::max(gy, (b.item_nb(i) + b.item_group(i) - 1) / b.item_group(i));
    switch (n) {
        case 256: return launch_one_tm<256, true>(b, tm, b.nx, gy, s, b.nitems);
        case 512: return launch_one_tm<512, true>(b, tm, b.nx, gy, s, b.nitems);
        case 1024: return launch_one_tm<1024, true>(b, tm, b.nx, gy, s, b.nitems);
        case 2048: return launch_one_tm<2048, true>(b, tm, b.nx, gy, s, b.nitems);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_recon_b_group(int n, const ReconB<EPI_PROJ, true> &b, cudaStream_t s) {
    int gy = 1;
    for (int i = 0; i < b.nitems; ++i) gy = std::max(gy, (b.item_nb(i) + b.item_group(i) - 1) / b.item_group(i));
    return launch_len<false>(n, b, b.rows, gy, s, b.nitems);
}

}  // namespace ph
