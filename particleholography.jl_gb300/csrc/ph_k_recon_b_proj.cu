// Reconstruction pass B with the EPI_PROJ epilogue (one translation unit per
// epilogue so the build compiles them in parallel).
#include "ph_launch.cuh"

namespace ph {

cudaError_t launch_recon_b(int n, const ReconB<EPI_PROJ> &b, cudaStream_t s) {
    int groups = (b.nbatch + b.group - 1) / b.group;
    for (int i = 0; b.nitems > 1 && i < b.nitems; ++i)
        groups = std::max(groups, (b.nb_items[i] + b.group_items[i] - 1) / b.group_items[i]);
    return launch_len<false>(n, b, b.rows, groups, s, b.nitems);
}

}  // namespace ph
