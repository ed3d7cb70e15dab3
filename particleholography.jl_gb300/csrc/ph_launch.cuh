// ph_launch.cuh -- runtime dispatch from a transform length to the pass kernel
// compiled for it, and the launch helpers the entry points call.
#pragma once

#include <algorithm>

#include "ph_passes.cuh"

namespace ph {

// Every supported transform length: 2^a (1..8192) and 3 * 2^a (3..6144).
#define PH_FOR_EACH_N(X)                                                                                  \
    X(1) X(2) X(4) X(8) X(16) X(32) X(64) X(128) X(256) X(512) X(1024) X(2048) X(4096) X(8192) X(3) X(6) \
        X(12) X(24) X(48) X(96) X(192) X(384) X(768) X(1536) X(3072) X(6144)

inline bool supported_len(int n) {
    if (n < 1) return false;
    if ((n & (n - 1)) == 0) return n <= 8192;
    return n % 3 == 0 && ((n / 3) & (n / 3 - 1)) == 0 && n <= 6144;
}

// Rows per CTA of the pass compiled for length n.
inline int rows_per_cta(int n) {
    switch (n) {
#define PH_ROWS_CASE(N) case N: return Shape<N>::ROWS;
        PH_FOR_EACH_N(PH_ROWS_CASE)
#undef PH_ROWS_CASE
    }
    return 0;
}

template <int N, bool ROW_FAST, class Body>
cudaError_t launch_one(const Body &body, int nrows, int grid_y, cudaStream_t s, int grid_z = 1) {
    static_assert(Body::EPT == PassBase::EPT, "the twiddle table is laid out for the common plan");
    auto kern = k_pass<N, ROW_FAST, Body>;
    constexpr size_t smem = Body::template smem<N, ROW_FAST>();
    static_assert(smem <= kSmemMax, "pass needs more shared memory than a CTA has");
    if constexpr (smem > 48 * 1024) {
        // Per-device opt-in to more than 48 KB of dynamic shared memory.
        static unsigned long long done_mask = 0;
        int dev = 0;
        cudaGetDevice(&dev);
        const unsigned long long bit = 1ull << (dev & 63);
        if (!(__atomic_load_n(&done_mask, __ATOMIC_ACQUIRE) & bit)) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e != cudaSuccess) return e;
            __atomic_fetch_or(&done_mask, bit, __ATOMIC_ACQ_REL);
        }
    }
    using S = Shape<N, Body::EPT, Body::TT>;
    int gx = (nrows + S::ROWS - 1) / S::ROWS;
    if constexpr (Body::template persistent<N>()) {
        // one CTA per resident slot (per device: the occupancy of this kernel x SMs)
        static int slots[64] = {};
        int dev = 0;
        cudaGetDevice(&dev);
        int c = __atomic_load_n(&slots[dev & 63], __ATOMIC_ACQUIRE);
        if (c == 0) {
            int per_sm = 0, sms = 0;
            cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, S::THREADS, smem);
            if (e != cudaSuccess) return e;
            e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return e;
            c = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
            __atomic_store_n(&slots[dev & 63], c, __ATOMIC_RELEASE);
        }
        gx = gx < c ? gx : c;
    }
    if (gx == 0) return cudaSuccess;
    constexpr int CS = Body::template cluster<N>();
    if constexpr (CS > 1) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((gx + CS - 1) / CS * CS, grid_y, grid_z);
        cfg.blockDim = dim3(S::THREADS);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = CS;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, kern, body);
    }
    if constexpr (Body::template pdl<N>()) {
        // programmatic dependent launch: the grid may start while the previous
        // kernel on the stream finishes (the body waits before touching its data)
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(gx, grid_y, grid_z);
        cfg.blockDim = dim3(S::THREADS);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, kern, body);
    }
    dim3 grid(gx, grid_y, grid_z);
    kern<<<grid, S::THREADS, smem, s>>>(body);
    return cudaGetLastError();
}

// A launch of k_pass_tm: the body and a tensor map (clusters of
// Body::cluster<N>() CTAs, persistent grids and programmatic dependents as in
// launch_one).
template <int N, bool ROW_FAST, class Body>
cudaError_t launch_one_tm(const Body &body, const CUtensorMap &tm, int nrows, int grid_y, cudaStream_t s,
                          int grid_z = 1) {
    auto kern = k_pass_tm<N, ROW_FAST, Body>;
    constexpr size_t smem = Body::template smem<N, ROW_FAST>();
    static_assert(smem <= kSmemMax, "pass needs more shared memory than a CTA has");
    if constexpr (smem > 48 * 1024) {
        static unsigned long long done_mask = 0;
        int dev = 0;
        cudaGetDevice(&dev);
        const unsigned long long bit = 1ull << (dev & 63);
        if (!(__atomic_load_n(&done_mask, __ATOMIC_ACQUIRE) & bit)) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e != cudaSuccess) return e;
            __atomic_fetch_or(&done_mask, bit, __ATOMIC_ACQ_REL);
        }
    }
    using S = Shape<N, Body::EPT, Body::TT>;
    int gx = (nrows + S::ROWS - 1) / S::ROWS;
    if constexpr (Body::template persistent<N>()) {
        static int slots[64] = {};
        int dev = 0;
        cudaGetDevice(&dev);
        int c = __atomic_load_n(&slots[dev & 63], __ATOMIC_ACQUIRE);
        if (c == 0) {
            int per_sm = 0, sms = 0;
            cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, S::THREADS, smem);
            if (e != cudaSuccess) return e;
            e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return e;
            c = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
            __atomic_store_n(&slots[dev & 63], c, __ATOMIC_RELEASE);
        }
        gx = gx < c ? gx : c;
    }
    if (gx == 0) return cudaSuccess;
    constexpr int CS = Body::template cluster<N>();
    static_assert(CS == 1 || !Body::template pdl<N>(), "cluster or programmatic-dependent launch, not both");
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((gx + CS - 1) / CS * CS, grid_y, grid_z);
    cfg.blockDim = dim3(S::THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    if constexpr (CS > 1) {
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = CS;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
    } else if constexpr (Body::template pdl<N>()) {
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
    }
    return cudaLaunchKernelEx(&cfg, kern, body, tm);
}

// A plain launch of k_pass_tm2 (two tensor maps), one grid row.
template <int N, bool ROW_FAST, class Body>
cudaError_t launch_one_tm2(const Body &body, const CUtensorMap &tm0, const CUtensorMap &tm1, int nrows,
                           cudaStream_t s) {
    auto kern = k_pass_tm2<N, ROW_FAST, Body>;
    constexpr size_t smem = Body::template smem<N, ROW_FAST>();
    static_assert(smem <= kSmemMax, "pass needs more shared memory than a CTA has");
    if constexpr (smem > 48 * 1024) {
        static unsigned long long done_mask = 0;
        int dev = 0;
        cudaGetDevice(&dev);
        const unsigned long long bit = 1ull << (dev & 63);
        if (!(__atomic_load_n(&done_mask, __ATOMIC_ACQUIRE) & bit)) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
            if (e != cudaSuccess) return e;
            __atomic_fetch_or(&done_mask, bit, __ATOMIC_ACQ_REL);
        }
    }
    using S = Shape<N, Body::EPT, Body::TT>;
    const int gx = (nrows + S::ROWS - 1) / S::ROWS;
    if (gx == 0) return cudaSuccess;
    kern<<<gx, S::THREADS, smem, s>>>(body, tm0, tm1);
    return cudaGetLastError();
}

// Launch of a pass that exists only for the lengths where Body::staged<N>() holds.
template <bool ROW_FAST, class Body>
cudaError_t launch_staged_len(int n, const Body &body, int nrows, cudaStream_t s) {
    switch (n) {
#define PH_STAGED_CASE(N)                                                             \
    case N:                                                                          \
        if constexpr (Body::template staged<N>()) return launch_one<N, ROW_FAST>(body, nrows, 1, s); \
        else return cudaErrorInvalidValue;
        PH_FOR_EACH_N(PH_STAGED_CASE)
#undef PH_STAGED_CASE
    }
    return cudaErrorInvalidValue;
}

template <class Body>
bool staged_len(int n) {
    switch (n) {
#define PH_STAGED_Q(N) case N: return Body::template staged<N>();
        PH_FOR_EACH_N(PH_STAGED_Q)
#undef PH_STAGED_Q
    }
    return false;
}

template <bool ROW_FAST, class Body>
cudaError_t launch_len(int n, const Body &body, int nrows, int grid_y, cudaStream_t s, int grid_z = 1) {
    switch (n) {
#define PH_LAUNCH_CASE(N) case N: return launch_one<N, ROW_FAST>(body, nrows, grid_y, s, grid_z);
        PH_FOR_EACH_N(PH_LAUNCH_CASE)
#undef PH_LAUNCH_CASE
    }
    return cudaErrorInvalidValue;
}

// ---- launchers, one translation unit each (compiled in parallel)

// (grouped launches: grid z = b.nitems; pass A / pass B grid y = the largest item's slice groups)
cudaError_t launch_fwd_rows(int n, const FwdRowsT<FWD_COMPLEX> &b, cudaStream_t s);
cudaError_t launch_fwd_rows(int n, const FwdRowsT<FWD_SQRT_REAL> &b, cudaStream_t s);
cudaError_t launch_fwd_rows(int n, const FwdRowsT<FWD_PADDED> &b, cudaStream_t s);
cudaError_t launch_spectrum(int n, const SpectrumCols &b, cudaStream_t s);
// The spectrum pass with staged transfers (lengths 512 .. 2048; spectrum_staged_rows
// gives the rows per CTA, 0 elsewhere); tm_hf, tm_hdz: the centred transfers
// as [n_slow][n_fast] 8-byte elements, boxes of rows x 256.
int spectrum_staged_rows(int n);
cudaError_t launch_spectrum_staged(int n, const SpectrumColsT &b, const CUtensorMap &tm_hf, const CUtensorMap &tm_hdz,
                                   cudaStream_t s);
cudaError_t launch_recon_a(int n, const ReconA &b, int nbatch, cudaStream_t s);
// Pass A with the tensor-map transposed store (lengths where recon_a_tstore holds;
// tm: T as [nbatch][ny_out = n][nx] 8-byte elements, boxes of 4 x 256 x 1).
bool recon_a_tstore(int n);
int recon_a_tstore_box(int n);   // kx per box (rows per CTA x CTAs per cluster)
cudaError_t launch_recon_a_tstore(int n, const ReconATStore &b, const CUtensorMap &tm, int nbatch, cudaStream_t s);
cudaError_t launch_recon_a_group(int n, const ReconAGrouped &b, cudaStream_t s);
// The grouped form with the tensor-map store, at the lengths where
// recon_a_tstore holds with one CTA per box (256 .. 2048); tm: the items' T
// slots as (kx, y, slice, item), boxes of recon_a_tstore_box(n) kx x 256 y.
bool recon_a_group_tstore(int n);
cudaError_t launch_recon_a_group_tstore(int n, const ReconAGroupedTStore &b, const CUtensorMap &tm, cudaStream_t s);
// The persistent GS passes with the tensor-map store (lengths where
// gs_tstore_len holds; tm: dst as a 2-D tensor of 8-byte elements, inner
// dimension the rows' index, boxes of rows-per-block x 256).
bool gs_tstore_len(int n);
int gs_rows(int n);   // rows per block of the persistent GS passes
cudaError_t launch_gs_col_ts(int n, const GsColT &b, const CUtensorMap &tm, cudaStream_t s);
cudaError_t launch_gs_row_ts(int n, const GsRowMidT &b, const CUtensorMap &tm, cudaStream_t s);
cudaError_t launch_recon_b_group(int n, const ReconB<EPI_PROJ, true> &b, cudaStream_t s);
int recon_a_rows(int n);   // rows per pass A CTA for transform length n
bool recon_a_chain(int n, bool tstore = false);   // whether pass A at length n (in the tensor-map
                                                  // store form) advances X by the product chain
cudaError_t launch_recon_b(int n, const ReconB<EPI_PROJ> &b, cudaStream_t s);
cudaError_t launch_recon_b(int n, const ReconB<EPI_VOL> &b, cudaStream_t s);
cudaError_t launch_recon_b(int n, const ReconB<EPI_CVOL> &b, cudaStream_t s);
cudaError_t launch_recon_b(int n, const ReconB<EPI_SUB> &b, cudaStream_t s);
cudaError_t launch_gs_row(int n, const GsRow<ROW_MID> &b, cudaStream_t s);
cudaError_t launch_gs_row(int n, const GsRow<ROW_FINAL> &b, cudaStream_t s);
cudaError_t launch_gs_row(int n, const GsRow<ROW_INV> &b, cudaStream_t s);
cudaError_t launch_gs_col(int n, const GsCol &b, cudaStream_t s);
// Persistent staged GS passes (row lengths where gs_row_staged / gs_col_staged hold).
bool gs_row_staged(int n);
bool gs_col_staged(int n);
cudaError_t launch_gs_row_t(int n, const GsRowMidT &b, cudaStream_t s);
// The last plane-1 pass (dst = [ny][nx], natural order), persistent.
cudaError_t launch_gs_row_final_t(int n, const GsRowMidT &b, cudaStream_t s);
cudaError_t launch_gs_col_t(int n, const GsColT &b, cudaStream_t s);
// Split-precision tensor-core pass B (ph_pass_tc.cuh) for the projection.
struct ReconBTc;
bool recon_b_tc_supported(int n, int form);
size_t recon_b_tc_table_bytes(int n, int form);
int recon_b_tc_rows(int n, int form);
void recon_b_tc_build_table(int n, int form, unsigned char *img);
cudaError_t launch_recon_b_tc(int n, int form, const ReconBTc &p, cudaStream_t s);

}  // namespace ph
