// ph_noalloc.cu -- a component count that allocates no device memory.
//
// Some callers of this library cannot call cudaMalloc: real-time acquisition
// loops that forbid allocation once the camera is running, and hosts that only
// lend the library buffers they registered up front.  For them, ph_ccl_count_noalloc
// gives the same count as count_labels / ph_ccl_roots without a context and
// without any allocation: its scratch -- the per-block root counts of the scan
// -- is a fixed device array compiled into this library.
//
// That array is file-scope `__device__` storage, so every GPU that loads the
// library holds it (256 KiB) until the process exits.  Host code may not use
// the array's name as a device address (on the host it names a stand-in), so
// the first call on each device looks its address up with
// cudaGetSymbolAddress, with that device current, and caches it.  That first
// call should therefore come before any stream capture, and calls must not
// cross a cudaDeviceReset (which would leave the cached address stale).  All calls share the
// one array: two calls whose work overlaps on the GPU (different streams, no
// ordering between them) race on it and may return wrong counts.
#include "phgb300.h"

#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

namespace ph {
cudaError_t roots_count_launch(const uint32_t *lab, int64_t n, int64_t slice_n, unsigned *counts,
                               unsigned long long *total, cudaStream_t s, int64_t *launches);
int64_t roots_blocks(int64_t n);
}  // namespace ph

// The fixed scratch: one count per scan block of 4096 labels, for up to 2^28
// labels per call (65,536 counts, 256 KiB).
static constexpr int64_t kMaxLabels = int64_t(1) << 28;
static constexpr int64_t kMaxBlocks = int64_t(1) << 16;
static __device__ __align__(256) unsigned g_block_counts[kMaxBlocks];

namespace {

std::mutex g_mu;
unsigned *g_scratch[64] = {};   // per-device address of g_block_counts
thread_local char g_err[256] = "";

int fail(int32_t status, const char *msg) {
    snprintf(g_err, sizeof g_err, "%s", msg);
    return status;
}

}  // namespace

extern "C" const char *ph_noalloc_last_error(void) { return g_err; }

extern "C" int32_t ph_ccl_count_noalloc(int64_t *count, const uint32_t *labels, int64_t n, void *stream) {
    if (count == nullptr || (labels == nullptr && n > 0)) return fail(PH_ERR_INVALID, "count and labels must not be NULL");
    if (n < 0) return fail(PH_ERR_SIZE, "negative label count");
    if (n > kMaxLabels || ph::roots_blocks(n) > kMaxBlocks) {
        char m[160];
        snprintf(m, sizeof m, "%lld labels exceed the fixed scratch of ph_ccl_count_noalloc (at most %lld)",
                 (long long)n, (long long)kMaxLabels);
        return fail(PH_ERR_TOO_LARGE, m);
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return fail(PH_ERR_CUDA, "no current CUDA device");
    }
    unsigned *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (g_scratch[dev] == nullptr) {
            void *p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_block_counts);
            if (e != cudaSuccess) {
                cudaGetLastError();
                return fail(PH_ERR_CUDA, cudaGetErrorString(e));
            }
            g_scratch[dev] = static_cast<unsigned *>(p);
        }
        scratch = g_scratch[dev];
    }
    if (n == 0) {
        const cudaError_t e = cudaMemsetAsync(count, 0, sizeof(int64_t), s);
        return e == cudaSuccess ? PH_OK : fail(PH_ERR_CUDA, cudaGetErrorString(e));
    }
    // Every block count the scan reads is written first by the count kernel, so
    // nothing left over from an earlier call is read.
    int64_t launches = 0;
    const cudaError_t e = ph::roots_count_launch(labels, n, n, scratch, reinterpret_cast<unsigned long long *>(count),
                                                 s, &launches);
    return e == cudaSuccess ? PH_OK : fail(PH_ERR_CUDA, cudaGetErrorString(e));
}
