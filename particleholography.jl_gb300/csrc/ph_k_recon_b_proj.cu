// Reconstruction pass B with the EPI_PROJ epilogue (one translation unit per
// epilogue so the build compiles them in parallel).
#include "ph_launch.cuh"

namespace ph {

cudaError_t launch_recon_b(int n, const ReconB<EPI_PROJ> &b, cudaStream_t s) {
    const int groups = (b.nbatch + b.group - 1) / b.group;
    return launch_len<false>(n, b, b.rows, groups, s);
}

}  // namespace ph
