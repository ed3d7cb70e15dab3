// Spectrum-state column pass.
#include "ph_launch.cuh"

namespace ph {

cudaError_t launch_spectrum(int n, const SpectrumCols &b, cudaStream_t s) {
    return launch_len<true>(n, b, b.nx, 1, s, b.nitems);
}

int spectrum_staged_rows(int n) {
    switch (n) {
#define PH_SPEC_ROWS(N) case N: return SpectrumColsT::staged<N>() ? Shape<N>::ROWS : 0;
        PH_SPEC_ROWS(512) PH_SPEC_ROWS(1024) PH_SPEC_ROWS(2048)
#undef PH_SPEC_ROWS
    }
    return 0;
}

cudaError_t launch_spectrum_staged(int n, const SpectrumColsT &b, const CUtensorMap &tm_hf, const CUtensorMap &tm_hdz,
                                   cudaStream_t s) {
    switch (n) {
#define PH_SPEC_CASE(N) \
    case N:         \
        if constexpr (SpectrumColsT::staged<N>()) return launch_one_tm2<N, true>(b, tm_hf, tm_hdz, b.nx, s); \
        break;
        PH_SPEC_CASE(512) PH_SPEC_CASE(1024) PH_SPEC_CASE(2048)
#undef PH_SPEC_CASE
    }
    return cudaErrorInvalidValue;
}

}  // namespace ph
