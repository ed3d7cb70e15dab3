// Gerchberg-Saxton / propagation column pass (forward FFT, transfer, inverse FFT).
#include "ph_launch.cuh"

namespace ph {

cudaError_t launch_gs_col(int n, const GsCol &b, cudaStream_t s) {
    return launch_len<true>(n, b, b.nx, 1, s);
}

}  // namespace ph
