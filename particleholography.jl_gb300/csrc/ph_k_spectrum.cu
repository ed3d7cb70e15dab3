// Spectrum-state column pass.
#include "ph_launch.cuh"

namespace ph {

cudaError_t launch_spectrum(int n, const SpectrumCols &b, cudaStream_t s) {
    return launch_len<true>(n, b, b.nx, 1, s, b.nitems);
}

}  // namespace ph
