// Reconstruction pass B: inverse FFT along kx with the projection / volume epilogues.
#include "ph_launch.cuh"

namespace ph {

template <int EPI>
static cudaError_t launch_b(int n, const ReconB<EPI> &b, cudaStream_t s) {
    const int groups = (b.nbatch + b.group - 1) / b.group;
    return launch_len<false>(n, b, b.rows, groups, s);
}

cudaError_t launch_recon_b(int n, const ReconB<EPI_PROJ> &b, cudaStream_t s) { return launch_b(n, b, s); }
cudaError_t launch_recon_b(int n, const ReconB<EPI_VOL> &b, cudaStream_t s) { return launch_b(n, b, s); }
cudaError_t launch_recon_b(int n, const ReconB<EPI_CVOL> &b, cudaStream_t s) { return launch_b(n, b, s); }

}  // namespace ph
