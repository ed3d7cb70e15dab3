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

// The tensor-map store at the lengths whose blocks hold 4 or 8 rows (2048, 1024).
bool gs_tstore_len(int n) { return n == 2048 || n == 1024; }

int gs_rows(int n) {
    switch (n) {
        case 1024: return Shape<1024>::ROWS;
        case 2048: return Shape<2048>::ROWS;
    }
    return 0;
}

cudaError_t launch_gs_col_ts(int n, const GsColT &b, const CUtensorMap &tm, cudaStream_t s) {
    GsColTS ts{};
    static_cast<GsColT &>(ts) = b;
    static_assert(GsColT::staged<1024>() && GsColT::staged<2048>() && gs_tstore_ok<1024>() && gs_tstore_ok<2048>(),
                  "tensor-map GS column pass at 1024 and 2048");
    switch (n) {
        case 1024: return launch_one_tm<1024, true>(ts, tm, b.nx, 1, s);
        case 2048: return launch_one_tm<2048, true>(ts, tm, b.nx, 1, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace ph
