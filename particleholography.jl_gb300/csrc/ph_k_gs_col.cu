// Gerchberg-Saxton / propagation column pass (forward FFT, transfer, inverse FFT).
#include "ph_launch.cuh"

namespace ph {

cudaError_t launch_gs_col(int n, const GsCol &b, cudaStream_t s) {
    return launch_len<true>(n, b, b.nx, 1, s);
}

cudaError_t launch_gs_col_t(int n, const GsColT &b, cudaStream_t s) {
    return launch_staged_len<true>(n, b, b.nx, s);
}

bool gs_col_staged(int n) { return staged_len<GsColT>(n); }

}  // namespace ph
