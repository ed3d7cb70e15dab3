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

cudaError_t launch_gs_row_final_t(int n, const GsRowMidT &b, cudaStream_t s) {
    GsRowFinalT f{};
    static_cast<GsRowMidT &>(f) = b;
    return launch_staged_len<true>(n, f, b.nrows, s);
}

template <bool RESID>
cudaError_t launch_gs_row_ts_form(int n, const GsRowMidT &b, const CUtensorMap &tm, cudaStream_t s) {
    GsRowMidTS<RESID> ts{};
    static_cast<GsRowMidT &>(ts) = b;
    static_assert(GsRowMidT::staged<1024>() && GsRowMidT::staged<2048>() && gs_tstore_ok<1024>() &&
                      gs_tstore_ok<2048>(),
                  "tensor-map GS row pass at 1024 and 2048");
    switch (n) {
        case 1024: return launch_one_tm<1024, true>(ts, tm, b.nrows, 1, s);
        case 2048: return launch_one_tm<2048, true>(ts, tm, b.nrows, 1, s);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_gs_row_ts(int n, const GsRowMidT &b, const CUtensorMap &tm, cudaStream_t s) {
    return b.resid == nullptr ? launch_gs_row_ts_form<false>(n, b, tm, s) : launch_gs_row_ts_form<true>(n, b, tm, s);
}

}  // namespace ph
