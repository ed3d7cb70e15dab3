// Reconstruction pass A: per-slice transfer + inverse FFT along ky, transposed store.
#include "ph_launch.cuh"

namespace ph {

cudaError_t launch_recon_a(int n, const ReconA &b, int nbatch, cudaStream_t s) {
    return launch_len<true>(n, b, b.nx, (nbatch + b.group - 1) / b.group, s);
}

}  // namespace ph
