// Forward row passes (transposed store).
#include "ph_launch.cuh"

namespace ph {

cudaError_t launch_fwd_rows(int n, const FwdRowsT<FWD_COMPLEX> &b, cudaStream_t s) {
    return launch_len<true>(n, b, b.nrows, 1, s, b.nitems);
}
cudaError_t launch_fwd_rows(int n, const FwdRowsT<FWD_SQRT_REAL> &b, cudaStream_t s) {
    return launch_len<true>(n, b, b.nrows, 1, s, b.nitems);
}
cudaError_t launch_fwd_rows(int n, const FwdRowsT<FWD_PADDED> &b, cudaStream_t s) {
    return launch_len<true>(n, b, b.nrows, 1, s);
}

}  // namespace ph
