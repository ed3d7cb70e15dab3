// Gerchberg-Saxton / propagation row passes.
#include "ph_launch.cuh"

namespace ph {

cudaError_t launch_gs_row(int n, const GsRow<ROW_MID> &b, cudaStream_t s) {
    return launch_len<true>(n, b, b.nrows, 1, s);
}
cudaError_t launch_gs_row(int n, const GsRow<ROW_FINAL> &b, cudaStream_t s) {
    return launch_len<false>(n, b, b.nrows, 1, s);
}
cudaError_t launch_gs_row(int n, const GsRow<ROW_INV> &b, cudaStream_t s) {
    return launch_len<false>(n, b, b.nrows, 1, s);
}

cudaError_t launch_gs_row_t(int n, const GsRowMidT &b, cudaStream_t s) {
    if (b.resid == nullptr) return launch_staged_len<true>(n, b, b.nrows, s);
    GsRowMidTResid br{};
    static_cast<GsRowMidT &>(br) = b;
    return launch_staged_len<true>(n, br, b.nrows, s);
}

bool gs_row_staged(int n) { return staged_len<GsRowMidT>(n); }

}  // namespace ph
