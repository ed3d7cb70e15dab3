// ph_api.cu -- the extern "C" entry points of libphgb300.so (declared in
// include/phgb300.h): context management, the small setup kernels (transfer
// functions, Gabor wavefront, padding, twiddles) and the orchestration of the
// pass kernels for reconstruction, Gerchberg-Saxton and propagation.
#include "phgb300.h"

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <cmath>
#include <map>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ph_ctx.h"
#include "ph_launch.cuh"
#include "ph_pass_tc.cuh"

// The serving runtime: work slots (one CUDA stream each), a scratch pool
// sub-allocated per request under the server's HBM budget, the queue of
// requests waiting for a slot and memory, and the transfer-function cache.
struct ph_server;
struct ph_serve_ticket {
    int64_t id = 0;
    ph_serve_request req{};
    ph_server *srv = nullptr;
    std::atomic<int> done{0};
    double t_submit = 0.0, t_admit = 0.0, t_done = 0.0;   // seconds, steady clock
    cudaEvent_t submitted = nullptr;   // on the caller's stream at submission: the inputs are written
    cudaEvent_t ev = nullptr;          // on the slot's stream after the completion callback
    int slot = -1;                     // -1 while queued
    size_t off = 0, bytes = 0;         // the request's block of the pool (0 for a group's other members)
    bool harvested = false;            // its slot and block have been given back
    std::vector<ph_serve_ticket *> members;   // a group's leader: the other requests sharing its launches
};

struct ph_serve_tf {
    float2 *buf = nullptr;
    cudaEvent_t ready = nullptr;      // the build finished
    cudaEvent_t last_use = nullptr;   // the last request that read it finished
    uint64_t stamp = 0;               // LRU order
};

struct ph_server {
    ph_ctx *ctx = nullptr;
    std::mutex mu;                         // queue, pool, slots, tickets, cache
    int lanes = 1;
    int max_nx = 0, max_ny = 0, max_slices = 0;
    size_t pool_bytes = 0, used = 0, peak = 0;
    void *pool = nullptr;
    std::map<size_t, size_t> free_blocks;  // offset -> bytes, coalesced
    std::vector<cudaStream_t> streams;
    std::vector<ph_serve_ticket *> slot_job;   // nullptr = free
    std::deque<ph_serve_ticket *> pending;     // FIFO, admitted from the front
    std::mutex cmu;                            // completions, written by host callbacks
    std::vector<ph_serve_ticket *> completed;
    std::map<std::tuple<int, int, double, double, double>, ph_serve_tf> tfs;
    int tf_cap = 16;
    uint64_t clock = 0;
    int64_t next_ticket = 1;
    std::unordered_map<int64_t, ph_serve_ticket *> tickets;
    std::vector<cudaEvent_t> event_pool;
    int64_t admitted_total = 0, waited_total = 0;   // requests admitted; of them, ones that had to queue
    int64_t grouped_total = 0;                        // requests admitted in shared launches
};

// A planned batch of reconstructions: its items, lanes, own scratch and the
// recorded graph.
struct ph_batch {
    ph_ctx *ctx = nullptr;
    std::vector<ph_recon_item> items;
    std::vector<int> lane_of;
    int lanes = 1;
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    cudaGraphExec_t exec = nullptr;
    int64_t kernels = 0;
};

namespace ph {
cudaError_t ccl_launch(const void *img, bool is_bool, uint32_t *lab, int64_t rows, int64_t cols, int64_t slice_rows,
                       int64_t limit, int *err, cudaStream_t s, int64_t *launches);
int64_t roots_blocks(int64_t n);
cudaError_t roots_count_launch(const uint32_t *lab, int64_t n, int64_t slice_n, unsigned *counts,
                               unsigned long long *total, cudaStream_t s, int64_t *launches);
cudaError_t roots_write_launch(const uint32_t *lab, int64_t n, int64_t slice_n, const unsigned *offsets,
                               long long *out, int64_t cap, unsigned *rank, cudaStream_t s, int64_t *launches);
cudaError_t boxes_launch(const uint32_t *lab, int64_t rows, int64_t cols, int64_t slice_rows, const unsigned *rank,
                         int *boxes, int64_t count, cudaStream_t s, int64_t *launches);
cudaError_t synth_fill_one(float2 *psi, size_t n, cudaStream_t s);
cudaError_t synth_disc(float2 *psi, int nx, int ny, double cx, double cy, double diam, double dx, cudaStream_t s);
cudaError_t synth_finish(const float2 *psi, float *out, size_t n, const float *noise, float *mm, cudaStream_t s);
}  // namespace ph

using namespace ph;

namespace {

constexpr int kVersion = 100;
constexpr size_t kAlign = 256;
constexpr int kMaxGraphs = 32;

// ---------------------------------------------------------------- setup kernels

__device__ __forceinline__ float2 twiddle_fp64(int i, int n) {   // W_n^i rounded from FP64
    double s, c;
    sincospi(-2.0 * (double)i / (double)n, &s, &c);
    return make_float2((float)c, (float)s);
}

// w_j = (cos, sin)(2 pi j / n) in FP64, stored as FP32 pairs (cos hi, cos lo, sin hi, sin lo).
__global__ void k_phase_table(float4 *tab, int n) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double s, c;
    sincospi(2.0 * (double)j / (double)n, &s, &c);
    const float ch = (float)c, sh = (float)s;
    tab[j] = make_float4(ch, (float)(c - (double)ch), sh, (float)(s - (double)sh));
}

__global__ void k_twiddle(float2 *tw, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    tw[i] = twiddle_fp64(i, n);
}

// The stage blocks of the table (layout in ph_fft.cuh): entry [r-1][k] of the
// block of a stage with radix R and span NS is W_n^(r k n / (NS R)).
__global__ void k_twiddle_stage(float2 *blk, int n, int radix, int ns) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (radix - 1) * ns) return;
    const int r = e / ns + 1, k = e % ns;
    blk[e] = twiddle_fp64(r * k * (n / (ns * radix)), n);
}

// holofunc.jl:8-15 with the reference's Float64 operation order; the
// intrinsics keep the compiler from contracting into fma.
__device__ __forceinline__ double sqr_term(int i1, int n, double wavlen, double dx) {
    const double a = __dsub_rn(__dsub_rn((double)i1, (double)n / 2.0), 1.0);
    const double t = __ddiv_rn(__ddiv_rn(__dmul_rn(a, wavlen), (double)n), dx);
    return __dmul_rn(t, t);
}

__global__ void k_transfer_sqrt(float *out, int nx, int ny, double wavlen, double dx) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= nx || y >= ny) return;
    const double v = __dsub_rn(__dsub_rn(1.0, sqr_term(x + 1, nx, wavlen, dx)), sqr_term(y + 1, ny, wavlen, dx));
    out[(size_t)y * nx + x] = __double2float_rn(v);
}

// holofunc.jl:38-45: exp(i * c * sqrt(Float32 d)), c = 2 pi z0 / lambda (FP64).
__global__ void k_transfer(float2 *out, const float *d_sqr, size_t n, double c) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float s = sqrtf(d_sqr[i]);
    const double phase = __dmul_rn(c, (double)s);
    double sn, cs;
    sincos(phase, &sn, &cs);
    out[i] = make_float2(__double2float_rn(cs), __double2float_rn(sn));
}

// Exact physics: the square-root term in FP64, evanescent waves set to 0.
__global__ void k_transfer_fp64(float2 *out, int nx, int ny, double c, double wavlen, double dx) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= nx || y >= ny) return;
    const double s = 1.0 - sqr_term(x + 1, nx, wavlen, dx) - sqr_term(y + 1, ny, wavlen, dx);
    float2 v = make_float2(0.f, 0.f);
    if (s >= 0.0) {
        double sn, cs;
        sincos(c * sqrt(s), &sn, &cs);
        v = make_float2((float)cs, (float)sn);
    }
    out[(size_t)y * nx + x] = v;
}

__global__ void k_gabor(float2 *out, const float *holo, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = make_float2(sqrtf(holo[i]), 0.f);
}

// Sum of a complex array in FP64 -> acc[0..1] (acc zeroed by the caller).
__global__ void k_sum_c64(const float2 *in, size_t n, double *acc) {
    double sx = 0.0, sy = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float2 v = in[i];
        sx += v.x;
        sy += v.y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sy += __shfl_xor_sync(0xffffffffu, sy, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(acc, sx);
        atomicAdd(acc + 1, sy);
    }
}

__global__ void k_mean_finish(const double *acc, double n, float2 *mean) {
    *mean = make_float2((float)(acc[0] / n), (float)(acc[1] / n));
}

// cu_2d_pad (holofunc.jl:139-149): out (2n)^2 filled with the mean, `in` at offset off.
__global__ void k_pad_fill(float2 *out, const float2 *in, const float2 *mean, int nin_x, int nin_y, int nout,
                           int off) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= nout || y >= nout) return;
    const int xi = x - off, yi = y - off;
    float2 v = *mean;
    if (xi >= 0 && xi < nin_x && yi >= 0 && yi < nin_y) v = in[(size_t)yi * nin_x + xi];
    out[(size_t)y * nout + x] = v;
}

// ---- preprocessing (utils.jl)

// Per-pixel most frequent UInt8 value over `count` images (utils.jl:279-317):
// each thread owns one pixel and its 256 vote counters in shared memory
// ([bin][thread], so a warp's counters sit on distinct banks); the first
// maximum wins, as the reference's argmax loop.
constexpr int kModeThreads = 64;
__global__ void __launch_bounds__(kModeThreads)
    k_background_mode(double *out, const uint8_t *__restrict__ images, int64_t count, int64_t npix) {
    __shared__ uint16_t hist[256][kModeThreads];
    const int t = threadIdx.x;
    const int64_t p = (int64_t)blockIdx.x * kModeThreads + t;
    for (int b = 0; b < 256; ++b) hist[b][t] = 0;
    if (p >= npix) return;
    int64_t i = 0;
    for (; i + 4 <= count; i += 4) {   // four independent loads in flight
        const uint8_t v0 = images[(i + 0) * npix + p], v1 = images[(i + 1) * npix + p];
        const uint8_t v2 = images[(i + 2) * npix + p], v3 = images[(i + 3) * npix + p];
        ++hist[v0][t];
        ++hist[v1][t];
        ++hist[v2][t];
        ++hist[v3][t];
    }
    for (; i < count; ++i) ++hist[images[i * npix + p]][t];
    int best = 0;
    uint16_t bc = hist[0][t];
    for (int b = 1; b < 256; ++b) {
        const uint16_t c = hist[b][t];
        if (c > bc) { bc = c; best = b; }
    }
    out[p] = (double)best / 255.0;
}

// make_background(...; mode=:mean) (utils.jl:212-218): sum over the images of
// Float64(Float32(q / 255)), in image order, over the count.
__global__ void k_background_mean(double *out, const uint8_t *__restrict__ images, int64_t count, int64_t npix) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    double acc = 0.0;
    for (int64_t i = 0; i < count; ++i) acc += (double)__fdiv_rn((float)images[i * npix + p], 255.0f);
    out[p] = acc / (double)count;
}

__global__ void k_sqrt_f32(float *out, const float *in, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = sqrtf(in[i]);
}

__global__ void k_sum_f32(const float *in, size_t n, double *acc) {
    double sx = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        sx += in[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sx += __shfl_xor_sync(0xffffffffu, sx, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(acc, sx);
}

// pad_with_mean (utils.jl:319-325): padsize^2 of mean(img), the image at fast /
// slow offsets off_f / off_s.
__global__ void k_pad_mean_fill(float *out, const float *in, const double *acc, double n, int nin_f, int nin_s,
                                int pad, int off_f, int off_s) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= pad || y >= pad) return;
    const int xi = x - off_f, yi = y - off_s;
    float v = (float)(acc[0] / n);
    if (xi >= 0 && xi < nin_f && yi >= 0 && yi < nin_s) v = in[(size_t)yi * nin_f + xi];
    out[(size_t)y * pad + x] = v;
}

// Device ingest of an 8-bit camera frame: load_gray2float (utils.jl:23-25,
// level / 255 as Float32) of the frame stored row-major [row][col] (pitch
// bytes, `channels` interleaved equal channels, the first read; rows bottom-up
// when flip), written in the library's layout out[col][row] (the Julia buffer
// of the image: its first index, the row, is contiguous), then the background
// removal of the preprocessing docs, img .- bkg .+ offset in FP64 stored as
// Float32.  With acc, the FP64 sum of the result is accumulated (for
// pad_with_mean).  32 x 32 tiles transposed through shared memory.
__global__ void k_ingest_u8(float *out, const uint8_t *frame, int rows, int cols, int pitch, int channels, int flip,
                            const double *bkg, double offset, double *acc) {
    __shared__ float tile[32][33];
    const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;   // image row / column of the tile
    const int tx = threadIdx.x, ty = threadIdx.y;           // block (32, 8)
    for (int r = ty; r < 32; r += 8) {                      // read along columns of image row i0 + r
        const int i = i0 + r, j = j0 + tx;
        float v = 0.0f;
        if (i < rows && j < cols) {
            const int src_row = flip ? rows - 1 - i : i;
            v = (float)frame[(size_t)src_row * pitch + (size_t)j * channels] / 255.0f;
        }
        tile[tx][r] = v;                                    // [column][row]
    }
    __syncthreads();
    double sx = 0.0;
    for (int c = ty; c < 32; c += 8) {                      // write along rows of column j0 + c
        const int j = j0 + c, i = i0 + tx;
        if (i < rows && j < cols) {
            float v = tile[c][tx];
            const size_t o = (size_t)j * rows + i;
            if (bkg != nullptr) v = (float)((double)v - bkg[o] + offset);
            out[o] = v;
            sx += v;
        }
    }
    if (acc != nullptr) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sx += __shfl_xor_sync(0xffffffffu, sx, o);
        if (tx == 0) atomicAdd(acc, sx);
    }
}

__global__ void k_proj_finish(const unsigned long long *p64, float *proj, int32_t *argmin, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long p = p64[i];
    if (proj) proj[i] = __uint_as_float((unsigned)(p >> 32));
    if (argmin) argmin[i] = (int32_t)(unsigned)(p & 0xffffffffu);
}

// The identity of the packed-minimum merge: INT64_MAX (float bits 0x7fffffff,
// slice 0xffffffff).  Every packed word of a finite or NaN intensity orders
// below it, unsigned and signed alike (a non-negative float's sign bit is 0),
// so shards merged by any backend's int64 MIN never pick it over a real word.
constexpr unsigned long long kPackedEmpty = 0x7fffffffffffffffull;

__global__ void k_fill_u64(unsigned long long *p, size_t n, unsigned long long v) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        p[i] = v;
}

__global__ void k_binarize_le(uint8_t *out, const float *in, size_t n, float thr) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[i] <= thr ? 1 : 0;
}

// frequency_filters.jl:5-15: row i (slow) is the reference's x, column j its y.
__global__ void k_lpf_rect(float *out, int n, double maxi) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= n || j >= n) return;
    const double a = (double)(i + 1) - n / 2.0 + 1.0;
    const double b = (double)(j + 1) - n / 2.0;
    out[(size_t)i * n + j] = (__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)) >= __dmul_rn(maxi, maxi)) ? 0.0f : 1.0f;
}

// frequency_filters.jl:40-50.
__global__ void k_lpf_super_gaussian(float *out, int n, double pitch, double sigma) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= n || j >= n) return;
    const double tx = ((double)(i + 1) - n / 2.0 + 1.0) / n / pitch / sigma;
    const double ty = ((double)(j + 1) - n / 2.0 + 1.0) / n / pitch / sigma;
    const double r2 = tx * tx + ty * ty;
    out[(size_t)i * n + j] = (float)exp(-0.5 * (r2 * r2 * r2));
}

// frequency_filters.jl:33: 1/wavlen * imglen^2 * pitch^2 / sqrt(4 d^2 + imglen^2 pitch^2), same order.
double lpf_maxi(double prop_dist, double wavlen, int imglen, double pitch) {
    const double n2 = (double)((long long)imglen * imglen), p2 = pitch * pitch;
    return (1.0 / wavlen) * n2 * p2 / sqrt(4.0 * (prop_dist * prop_dist) + n2 * p2);
}

__global__ void k_resid_finish(const double *acc, double *out) {
    *out = acc[1] > 0.0 ? sqrt(acc[0] / acc[1]) : 0.0;
}

// ht[kx][ky] = scale * h[shift(ky)][shift(kx)]: a centred [ny][nx] transfer
// rearranged to the [kx][ky] rows the staged column pass multiplies by
// (32 x 32 tiles through shared memory, both sides coalesced).
__global__ void k_transfer_rows(float2 *ht, const float2 *h, int nx, int ny, float scale) {
    __shared__ float2 tile[32][33];
    const int kx0 = blockIdx.x * 32, ky0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int ky = ky0 + i, kx = kx0 + threadIdx.x;
        if (ky < ny && kx < nx) tile[i][threadIdx.x] = h[(size_t)shift_idx(ky, ny) * nx + shift_idx(kx, nx)];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int kx = kx0 + i, ky = ky0 + threadIdx.x;
        if (kx < nx && ky < ny) {
            const float2 v = tile[threadIdx.x][i];
            ht[(size_t)kx * ny + ky] = make_float2(v.x * scale, v.y * scale);
        }
    }
}

// ---------------------------------------------------------------- call plumbing

void set_err(ph_ctx *ctx, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    ctx->err = buf;
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && prev != cur) cudaSetDevice(prev);
    }
};

int cuda_status(ph_ctx *ctx, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return PH_OK;
    set_err(ctx, "%s: %s", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? PH_ERR_OOM : PH_ERR_CUDA;
}

#define PH_TRY(expr)                                     \
    do {                                                 \
        int _st = (expr);                                \
        if (_st != PH_OK) return _st;                    \
    } while (0)

#define PH_CUDA(call, what)                                  \
    do {                                                     \
        cudaError_t _e = (call);                             \
        if (_e != cudaSuccess) return cuda_status(ctx, _e, what); \
    } while (0)

bool capturing(cudaStream_t s) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &st) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return st != cudaStreamCaptureStatusNone;
}

// Orders this call after the previous call of the context when it ran on a
// different stream (the scratch arena is shared by all calls).
int begin_call(ph_ctx *ctx, cudaStream_t s) {
    if (ctx->has_last && ctx->last_stream != s && !capturing(s)) {
        PH_CUDA(cudaStreamWaitEvent(s, ctx->done, 0), "cudaStreamWaitEvent");
    }
    return PH_OK;
}

int end_call(ph_ctx *ctx, cudaStream_t s) {
    if (capturing(s)) return PH_OK;
    PH_CUDA(cudaEventRecord(ctx->done, s), "cudaEventRecord");
    ctx->last_stream = s;
    ctx->has_last = true;
    return PH_OK;
}

// Grows the scratch arena to at least `bytes`.  Growth waits for all earlier
// work of the context (the old arena may still be in use) before freeing.
int ensure_scratch(ph_ctx *ctx, size_t bytes, cudaStream_t s) {
    if (bytes <= ctx->scratch_bytes) return PH_OK;
    if (ctx->budget && bytes > ctx->budget) {
        set_err(ctx, "scratch of %zu bytes exceeds the context's HBM budget of %zu bytes", bytes, ctx->budget);
        return PH_ERR_OOM;
    }
    if (capturing(s)) {
        set_err(ctx, "scratch must grow to %zu bytes during a stream capture; call ph_reserve first", bytes);
        return PH_ERR_OOM;
    }
    if (ctx->scratch) {
        PH_CUDA(cudaStreamSynchronize(s), "cudaStreamSynchronize");
        if (ctx->has_last) PH_CUDA(cudaEventSynchronize(ctx->done), "cudaEventSynchronize");
        // Cached graphs reference the old arena.
        for (auto &g : ctx->graphs) cudaGraphExecDestroy(g.exec);
        ctx->graphs.clear();
        cudaFree(ctx->scratch);
        ctx->scratch = nullptr;
        ctx->scratch_bytes = 0;
    }
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_err(ctx, "cudaMalloc of %zu bytes of scratch failed: %s", bytes, cudaGetErrorString(e));
        return PH_ERR_OOM;
    }
    ctx->scratch = p;
    ctx->scratch_bytes = bytes;
    return PH_OK;
}

struct Arena {
    size_t off = 0;
    template <class T>
    size_t take(size_t count) {
        const size_t o = (off + kAlign - 1) / kAlign * kAlign;
        off = o + count * sizeof(T);
        return o;
    }
};

template <class T>
T *at(ph_ctx *ctx, size_t off) {
    return reinterpret_cast<T *>(static_cast<char *>(ctx->scratch) + off);
}

int get_twiddles(ph_ctx *ctx, int n, cudaStream_t s, const float2 **out) {
    auto it = ctx->tw.find(n);
    if (it != ctx->tw.end()) {
        *out = it->second;
        return PH_OK;
    }
    if (capturing(s)) {
        set_err(ctx, "twiddle table for length %d must be created outside a stream capture; call ph_reserve first", n);
        return PH_ERR_INVALID;
    }
    float2 *p = nullptr;
    const int e = engine_e(n, PassBase::EPT);
    PH_CUDA(cudaMalloc(&p, sizeof(float2) * (size_t)plan_tw_size(n, e)), "cudaMalloc(twiddles)");
    k_twiddle<<<(n + 255) / 256, 256, 0, s>>>(p, n);
    ctx->launches++;
    PH_CUDA(cudaGetLastError(), "k_twiddle");
    for (int st = 1; st < plan_nstages(n, e); ++st) {
        const int r = plan_radix(n, e, st), ns = plan_ns(n, e, st);
        const int cnt = (r - 1) * ns;
        k_twiddle_stage<<<(cnt + 255) / 256, 256, 0, s>>>(p + plan_tw_offset(n, e, st), n, r, ns);
        ctx->launches++;
        PH_CUDA(cudaGetLastError(), "k_twiddle_stage");
    }
    ctx->tw[n] = p;
    *out = p;
    return PH_OK;
}

// The tables of the tensor-core pass for (n, form), built on the host in FP64
// once per context and kept on the device.
int get_tc_table(ph_ctx *ctx, int n, int form, cudaStream_t s, const unsigned char **out) {
    const int key = 8 * n + form;
    auto it = ctx->tc_tables.find(key);
    if (it != ctx->tc_tables.end()) {
        *out = static_cast<const unsigned char *>(it->second);
        return PH_OK;
    }
    if (capturing(s)) {
        set_err(ctx, "tensor-core tables for length %d must be created outside a stream capture; call ph_reserve first",
                n);
        return PH_ERR_INVALID;
    }
    const size_t bytes = recon_b_tc_table_bytes(n, form);
    std::vector<unsigned char> img(bytes);
    recon_b_tc_build_table(n, form, img.data());
    void *p = nullptr;
    PH_CUDA(cudaMalloc(&p, bytes), "cudaMalloc(tensor-core tables)");
    const cudaError_t e = cudaMemcpyAsync(p, img.data(), bytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) cudaStreamSynchronize(s);   // the host image goes out of scope
    if (e != cudaSuccess) {
        cudaFree(p);
        return cuda_status(ctx, e, "cudaMemcpyAsync(tensor-core tables)");
    }
    ctx->tc_tables[key] = p;
    *out = static_cast<const unsigned char *>(p);
    return PH_OK;
}

int check_len(ph_ctx *ctx, int nx, int ny) {
    if (nx <= 0 || ny <= 0) {
        set_err(ctx, "array sizes must be positive. Got (%d, %d).", nx, ny);
        return PH_ERR_SIZE;
    }
    if (!supported_len(nx) || !supported_len(ny)) {
        set_err(ctx,
                "FFT length (%d, %d) is not supported: each axis must be 2^a up to 8192 or 3*2^a up to 6144.", nx,
                ny);
        return PH_ERR_UNSUPPORTED;
    }
    return PH_OK;
}

int launched(ph_ctx *ctx, cudaError_t e, const char *what, int count = 1) {
    ctx->launches += count;
    return cuda_status(ctx, e, what);
}

dim3 grid2d(int nx, int ny, dim3 b) { return dim3((nx + b.x - 1) / b.x, (ny + b.y - 1) / b.y); }

// ---------------------------------------------------------------- profiler

cudaEvent_t prof_event(ph_ctx *ctx) {
    if (!ctx->prof_pool.empty()) {
        cudaEvent_t e = ctx->prof_pool.back();
        ctx->prof_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return e;
}

// Brackets one pass launch with CUDA events on the caller's stream when
// PH_OPT_PROFILE is on (never inside a stream capture).
struct ProfScope {
    ph_ctx *ctx;
    cudaStream_t s;
    const char *name;
    cudaEvent_t a = nullptr, b = nullptr;
    ProfScope(ph_ctx *c, cudaStream_t st, const char *n) : ctx(c), s(st), name(n) {
        if (ctx->opt_profile && !capturing(s)) {
            a = prof_event(ctx);
            b = prof_event(ctx);
            if (a && b) cudaEventRecord(a, s);
        }
    }
    ~ProfScope() {
        if (a && b) {
            cudaEventRecord(b, s);
            ctx->prof.push_back({name, a, b});
        }
    }
};

template <class F>
int pass(ph_ctx *ctx, cudaStream_t s, const char *name, F &&launch, int count = 1) {
    ProfScope p(ctx, s, name);
    return launched(ctx, launch(), name, count);
}

// ---------------------------------------------------------------- graph replay

// Runs `issue(stream)` (a fixed sequence of launches whose parameters are all
// captured by `key`) as a cached CUDA graph: recorded once on the context's
// private capture stream, then launched on `s`.  Profiling, an ongoing capture
// of `s` by the caller, or PH_OPT_USE_GRAPHS = 0 issue the launches directly.
template <class F>
int run_graph(ph_ctx *ctx, cudaStream_t s, const char *key, F &&issue) {
    if (!ctx->opt_use_graphs || ctx->opt_profile || capturing(s)) return issue(s);
    for (auto it = ctx->graphs.begin(); it != ctx->graphs.end(); ++it) {
        if (it->key == key) {
            ctx->graphs.splice(ctx->graphs.begin(), ctx->graphs, it);
            PH_CUDA(cudaGraphLaunch(ctx->graphs.front().exec, s), "cudaGraphLaunch");
            ctx->launches += ctx->graphs.front().kernels;
            return PH_OK;
        }
    }
    const int64_t l0 = ctx->launches.load();
    cudaStream_t cs = ctx->capture_stream;
    PH_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    const int st = issue(cs);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(cs, &g);
    const int64_t kernels = ctx->launches.load() - l0;
    ctx->launches = l0;
    if (st != PH_OK || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        if (st != PH_OK) return st;
        return cuda_status(ctx, e, "cudaStreamEndCapture");
    }
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ei = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) return cuda_status(ctx, ei, "cudaGraphInstantiate");
    ctx->graphs.push_front({key, exec, kernels});
    while ((int)ctx->graphs.size() > kMaxGraphs) {
        cudaGraphExecDestroy(ctx->graphs.back().exec);
        ctx->graphs.pop_back();
    }
    PH_CUDA(cudaGraphLaunch(exec, s), "cudaGraphLaunch");
    ctx->launches += kernels;
    return PH_OK;
}

// ---------------------------------------------------------------- reconstruction plumbing

struct Spectrum {
    float4 *state;
    const float2 *tw_x, *tw_y;
};

// cuTensorMapEncodeTiled, looked up through the runtime's driver entry point
// (the library does not link the driver library); null if unavailable.
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
    static const EncodeTiledFn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

// Tensor map of a centred transfer [ny][nx] (8-byte elements) for the staged
// spectrum pass: boxes of `rows` columns x 256 rows.
bool tf_load_map(CUtensorMap *tm, const float2 *h, int nx, int ny, int rows) {
    const EncodeTiledFn enc = encode_tiled();
    if (enc == nullptr || ((uintptr_t)h & 15) != 0 || nx % 2 != 0 || rows < 2 || rows > 32) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)nx, (cuuint64_t)ny};
    const cuuint64_t strides[1] = {(cuuint64_t)nx * 8};
    const cuuint32_t box[2] = {(cuuint32_t)rows, 256};
    const cuuint32_t estr[2] = {1, 1};
    return enc(tm, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, const_cast<float2 *>(h), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Forward FFT of the (optionally mean-padded) wavefront and the spectrum state.
// nx, ny: transform size; a1: scratch [nx][ny] complex.  With `holo` (and wf
// NULL) the wavefront is sqrt(holo) + 0i, formed in the first FFT stage.
int issue_spectrum(ph_ctx *ctx, const float2 *wf, const float2 *hf, const float2 *hdz, int nx, int ny,
                   bool padded, int nin_x, int nin_y, float2 *a1, float4 *state, const float2 *tw_x,
                   const float2 *tw_y, double *acc, float2 *mean, cudaStream_t s, const float *holo = nullptr,
                   const float *lpf = nullptr) {
    if (holo != nullptr) {
        FwdRowsT<FWD_SQRT_REAL> f{};
        f.src_real = holo;
        f.dst = a1;
        f.tw = tw_x;
        f.nrows = ny;
        PH_TRY(pass(ctx, s, "fwd_rows", [&] { return launch_fwd_rows(nx, f, s); }));
    } else if (padded) {
        PH_CUDA(cudaMemsetAsync(acc, 0, 2 * sizeof(double), s), "cudaMemsetAsync");
        k_sum_c64<<<256, 256, 0, s>>>(wf, (size_t)nin_x * nin_y, acc);
        k_mean_finish<<<1, 1, 0, s>>>(acc, (double)nin_x * nin_y, mean);
        PH_TRY(launched(ctx, cudaGetLastError(), "mean", 2));
        FwdRowsT<FWD_PADDED> f{};
        f.src = wf;
        f.dst = a1;
        f.tw = tw_x;
        f.pad_mean = mean;
        f.nrows = ny;
        f.nx_in = nin_x;
        f.ny_in = nin_y;
        f.pad_off = nx / 4;
        PH_TRY(pass(ctx, s, "fwd_rows",[&] { return launch_fwd_rows(nx, f, s); }));
    } else {
        FwdRowsT<FWD_COMPLEX> f{};
        f.src = wf;
        f.dst = a1;
        f.tw = tw_x;
        f.nrows = ny;
        PH_TRY(pass(ctx, s, "fwd_rows",[&] { return launch_fwd_rows(nx, f, s); }));
    }
    SpectrumCols c{};
    c.a1 = a1;
    c.hf = hf;
    c.hdz = hdz;
    c.lpf = lpf;
    c.ptab = ctx->phase_tab;
    c.state = state;
    c.tw = tw_y;
    c.nx = nx;
    c.ny = ny;
    c.scale = (float)(1.0 / ((double)nx * (double)ny));
    // the transfers staged by tensor-map boxes where the lengths allow it
    const int rows = spectrum_staged_rows(ny);
    CUtensorMap tm_hf, tm_hdz;
    if (lpf == nullptr && rows > 0 && nx % (2 * rows) == 0 &&
        tf_load_map(&tm_hf, hf, nx, ny, rows) && tf_load_map(&tm_hdz, hdz, nx, ny, rows)) {
        SpectrumColsT ct{};
        static_cast<SpectrumCols &>(ct) = c;
        ct.err = static_cast<int *>(ctx->small);
        PH_TRY(pass(ctx, s, "spectrum", [&] { return launch_spectrum_staged(ny, ct, tm_hf, tm_hdz, s); }));
        return PH_OK;
    }
    PH_TRY(pass(ctx, s, "spectrum", [&] { return launch_spectrum(ny, c, s); }));
    return PH_OK;
}

// Slices per reconstruction batch.  A single call takes up to 8 GiB of slice
// intermediates (fewer, larger pass launches: 8 GiB measured 2 % faster per
// 2048^2 x 512 frame than 2 GiB), or half the context's HBM budget; the lanes
// of batches and servers, which hold scratch side by side, take 2 GiB each.
// Slice intermediate T per call: 16 GiB holds a 2048^2 x 512 frame in one
// batch (one pass A and one pass B launch, one last-wave tail each): 1.8 %
// faster per frame than two 8 GiB batches, which were 2 % faster than 2 GiB.
constexpr size_t kBatchBytes = size_t(16) << 30;
constexpr size_t kLaneBatchBytes = size_t(2) << 30;

// The autotuner's knobs for a transform shape, or null.
const ph_tuning *tuning_of(const ph_ctx *ctx, int nx, int ny) {
    auto it = ctx->tuned.find({nx, ny});
    return it == ctx->tuned.end() ? nullptr : &it->second;
}

// The form of the projection's row pass for this shape: the caller's choice,
// or under PH_FORM_TUNED the tuner's (FP32 where it chose none or the length
// has no tensor-core plan).
int effective_form(const ph_ctx *ctx, int nx, int ny) {
    int f = (int)ctx->opt_form;
    if (f == PH_FORM_TUNED) {
        const ph_tuning *tu = tuning_of(ctx, nx, ny);
        f = tu ? tu->form : PH_FORM_FP32;
    }
    return (f != PH_FORM_FP32 && recon_b_tc_supported(nx, f)) ? f : PH_FORM_FP32;
}

int slice_batch(ph_ctx *ctx, int nx, int ny, int slices, size_t target = kBatchBytes) {
    if (ctx->opt_slice_batch > 0) return (int)std::min<int64_t>(ctx->opt_slice_batch, slices);
    if (const ph_tuning *tu = tuning_of(ctx, nx, ny); tu && tu->batch_slices > 0) {
        const size_t fit = std::max<size_t>(1, target / ((size_t)nx * ny * sizeof(float2)));
        return (int)std::min<size_t>({(size_t)tu->batch_slices, fit, (size_t)std::max(slices, 1)});
    }
    const size_t slice_bytes = (size_t)nx * ny * sizeof(float2);
    if (ctx->budget) target = std::min(target, ctx->budget / 2);
    // clamped in size_t: a tiny slice would overflow an int count
    const size_t b = std::max<size_t>(1, target / slice_bytes);
    return (int)std::min<size_t>(b, (size_t)std::max(slices, 1));
}

struct ReconLayout {
    size_t a1, state, p64, t, acc, mean, total;
    int batch;
};

ReconLayout recon_layout(ph_ctx *ctx, int nx, int ny, int ny_out, int nx_out, int slices,
                         size_t target = kBatchBytes) {
    ReconLayout L{};
    L.batch = slice_batch(ctx, nx, ny, slices, target);
    Arena a;
    L.state = a.take<float4>((size_t)nx * ny);
    L.p64 = a.take<unsigned long long>((size_t)nx_out * ny_out);
    const size_t t_elems = std::max((size_t)L.batch * ny_out * nx, (size_t)nx * ny);   // a1 aliases t
    L.t = a.take<float2>(t_elems);
    L.a1 = L.t;
    L.acc = a.take<double>(4);
    L.mean = a.take<float2>(1);
    L.total = a.off;
    return L;
}

enum ReconKind { RK_PROJ, RK_VOL, RK_CVOL, RK_PADDED, RK_SUB };

// Device tables of a sub-volume reconstruction (pass B's EPI_SUB epilogue).
struct SubArgs {
    const int *row_ptr, *row_box;
    const SubBox *boxes;
};

int issue_recon_slices(ph_ctx *ctx, ReconKind kind, float *proj, int32_t *argmin, void *vol, int vol_dtype, int nx,
                       int ny, int nx_out, int ny_out, int x0, int y0, int slices, int batch, float4 *state, float2 *t,
                       unsigned long long *p64, const float2 *tw_x, const float2 *tw_y, bool want_proj,
                       cudaStream_t s, float threshold = 0.0f, int first = 0, const SubArgs *sub = nullptr);

// Shared driver of every reconstruction entry point.
//
// With `packed` (RK_PROJ only) the minimum of slices [first, first + slices)
// is merged into the caller's packed words (float bits << 32 | global slice)
// instead of the context's scratch, which `accumulate` = false first fills with
// the merge identity; no projection is unpacked.
int reconstruct(ph_ctx *ctx, ReconKind kind, float *proj, int32_t *argmin, void *vol, int vol_dtype,
                const float2 *wf, const float2 *hf, const float2 *hdz, int nin_x, int nin_y, int slices,
                cudaStream_t s, const float *lpf = nullptr, float threshold = 0.0f,
                unsigned long long *packed = nullptr, bool accumulate = false, int first = 0) {
    const bool padded = kind == RK_PADDED;
    const int nx = padded ? 2 * nin_x : nin_x;
    const int ny = padded ? 2 * nin_y : nin_y;
    PH_TRY(check_len(ctx, nx, ny));
    const int nx_out = nin_x, ny_out = nin_y;
    const int x0 = padded ? nin_x / 2 : 0;
    const int y0 = padded ? nin_y / 2 : 0;
    ReconLayout L = recon_layout(ctx, nx, ny, ny_out, nx_out, slices);
    PH_TRY(ensure_scratch(ctx, L.total, s));
    const float2 *tw_x = nullptr, *tw_y = nullptr;
    PH_TRY(get_twiddles(ctx, nx, s, &tw_x));
    PH_TRY(get_twiddles(ctx, ny, s, &tw_y));
    float4 *state = at<float4>(ctx, L.state);
    auto *p64 = packed != nullptr ? packed : at<unsigned long long>(ctx, L.p64);
    float2 *t = at<float2>(ctx, L.t);
    const bool want_proj = (kind == RK_PROJ) || proj != nullptr || argmin != nullptr;
    if (kind == RK_PROJ && effective_form(ctx, nx, ny) != PH_FORM_FP32) {
        const unsigned char *tab = nullptr;
        PH_TRY(get_tc_table(ctx, nx, effective_form(ctx, nx, ny), s, &tab));
    }
    const ph_tuning *tu = tuning_of(ctx, nx, ny);
    char key[512];
    uint32_t thr_bits = 0;
    memcpy(&thr_bits, &threshold, sizeof thr_bits);
    snprintf(key, sizeof key, "recon|%d|%d|%d|%d|%d|%d|%p|%p|%p|%p|%p|%p|%p|%d|%p|%08x|%p|%d|%d|%d", (int)kind, nin_x,
             nin_y, slices, L.batch, vol_dtype, (void *)proj, (void *)argmin, vol, (const void *)wf, (const void *)hf,
             (const void *)hdz, ctx->scratch, (int)ctx->opt_loop_limit, (const void *)lpf, thr_bits, (void *)packed,
             (int)accumulate, first, effective_form(ctx, nx, ny) * 1000 + (tu ? tu->group_cap : 0));
    return run_graph(ctx, s, key, [&](cudaStream_t s) -> int {
        PH_TRY(issue_spectrum(ctx, wf, hf, hdz, nx, ny, padded, nin_x, nin_y, at<float2>(ctx, L.a1), state, tw_x,
                              tw_y, at<double>(ctx, L.acc), at<float2>(ctx, L.mean), s, nullptr, lpf));
        const size_t npix = (size_t)nx_out * ny_out;
        if (packed != nullptr) {
            if (!accumulate) {
                k_fill_u64<<<(unsigned)std::min<size_t>((npix + 255) / 256, 4096), 256, 0, s>>>(p64, npix,
                                                                                               kPackedEmpty);
                PH_TRY(launched(ctx, cudaGetLastError(), "packed fill"));
            }
        } else if (want_proj) {
            PH_CUDA(cudaMemsetAsync(p64, 0xff, sizeof(unsigned long long) * npix, s), "memset");
        }
        return issue_recon_slices(ctx, kind, proj, argmin, vol, vol_dtype, nx, ny, nx_out, ny_out, x0, y0, slices,
                                  L.batch, state, t, p64, tw_x, tw_y, want_proj && packed == nullptr, s, threshold,
                                  first);
    });
}

// Slices one pass A / pass B CTA transforms: up to 32, fewer when the batch
// would then leave pass A with less than about four CTAs per SM.  Where pass A
// runs the product chain, up to 64 (half the chain starts, each an accurate
// sin/cos per value) as long as pass A keeps at least 16 waves of CTAs: 1.2 %
// faster per 2048^2 x 512 frame.  (A 64 cap without the wave condition made
// 1024^2 x 256 frames 7 % slower: 5 waves, the last one nearly empty.)
int recon_group(int nbatch, int nx_rows_a, bool chain, int cap_override = 0) {
    if (cap_override > 0) return std::max(1, std::min(cap_override, nbatch));
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 1;
    const int blocks = std::max(1, nx_rows_a);
    const int groups = std::max(1, (4 * sms + blocks - 1) / blocks);
    int cap = 32;
    if (chain) {
        const int g = std::max(1, std::min(64, nbatch / groups));
        const long long ctas = (long long)blocks * ((nbatch + g - 1) / g);
        if (g > 32 && ctas >= 16LL * sms) cap = 64;
    }
    return std::max(1, std::min(cap, nbatch / groups));
}

// Tensor map of the slice intermediate T = [nb][ny_out][nx] float2 (8-byte
// elements) for pass A's tiled store: boxes of box_kx kx x 256 y x 1 slice.
bool t_store_map(CUtensorMap *tm, float2 *t, int nx, int ny_out, int nb, int box_kx) {
    const EncodeTiledFn enc = encode_tiled();
    if (enc == nullptr || ((uintptr_t)t & 15) != 0 || nx % 4 != 0 || box_kx < 4 || box_kx > 32) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny_out, (cuuint64_t)nb};
    const cuuint64_t strides[2] = {(cuuint64_t)nx * 8, (cuuint64_t)nx * ny_out * 8};
    const cuuint32_t box[3] = {(cuuint32_t)box_kx, (cuuint32_t)ReconATStore::kBoxY, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return enc(tm, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, t, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Tensor map of a [outer][inner] float2 array for the persistent GS passes'
// tiled store: boxes of `rows` (along inner) x kGsBox (along outer).
bool gs_store_map(CUtensorMap *tm, float2 *p, int inner, int outer, int rows) {
    const EncodeTiledFn enc = encode_tiled();
    if (enc == nullptr || ((uintptr_t)p & 15) != 0 || inner % 4 != 0 || rows <= 0) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
    const cuuint64_t strides[1] = {(cuuint64_t)inner * 8};
    const cuuint32_t box[2] = {(cuuint32_t)rows, (cuuint32_t)kGsBox};
    const cuuint32_t estr[2] = {1, 1};
    return enc(tm, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, p, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Tensor map of the T slots of a grouped launch: item i's T = [nb][ny][nx]
// float2 at t + i * item_bytes; boxes of box_kx kx x 256 y x 1 slice x 1 item.
bool t_store_map_items(CUtensorMap *tm, float2 *t, int nx, int ny, int nb, int nitems, size_t item_bytes,
                       int box_kx) {
    const EncodeTiledFn enc = encode_tiled();
    if (enc == nullptr || ((uintptr_t)t & 15) != 0 || nx % 4 != 0 || box_kx < 4 || box_kx > 32 ||
        item_bytes % 16 != 0)
        return false;
    const cuuint64_t dims[4] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nb, (cuuint64_t)nitems};
    const cuuint64_t strides[3] = {(cuuint64_t)nx * 8, (cuuint64_t)nx * ny * 8, (cuuint64_t)item_bytes};
    const cuuint32_t box[4] = {(cuuint32_t)box_kx, (cuuint32_t)ReconATStore::kBoxY, 1, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    return enc(tm, CU_TENSOR_MAP_DATA_TYPE_UINT64, 4, t, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The slice loop of a reconstruction: pass A and pass B per batch, then the
// projection unpacking.
int issue_recon_slices(ph_ctx *ctx, ReconKind kind, float *proj, int32_t *argmin, void *vol, int vol_dtype, int nx,
                       int ny, int nx_out, int ny_out, int x0, int y0, int slices, int batch, float4 *state, float2 *t,
                       unsigned long long *p64, const float2 *tw_x, const float2 *tw_y, bool want_proj,
                       cudaStream_t s, float threshold, int first, const SubArgs *sub) {
    ReconLayout L{};
    L.batch = batch;
    const int row_blocks_a = (nx + recon_a_rows(ny) - 1) / recon_a_rows(ny);
    for (int k0 = first; k0 < first + slices; k0 += L.batch) {
        const int nb = std::min(L.batch, first + slices - k0);
        const ph_tuning *tu = tuning_of(ctx, nx, ny);
        const bool ts_shape = recon_a_tstore(ny) && y0 == 0 && ny_out == ny;   // the tensor-map store form
        const int group = recon_group(nb, row_blocks_a, recon_a_chain(ny, ts_shape), tu ? tu->group_cap : 0);
        const auto fill_a = [&](auto &a) {
            a.state = state;
            a.t = t;
            a.tw = tw_y;
            a.nx = nx;
            a.ny_out = ny_out;
            a.y0 = y0;
            a.k0 = k0;
            a.nbatch = nb;
            a.group = group;
            a.err = static_cast<int *>(ctx->small);
        };
        CUtensorMap tm;
        if (ts_shape && t_store_map(&tm, t, nx, ny_out, nb, recon_a_tstore_box(ny))) {
            ReconATStore a{};
            fill_a(a);
            PH_TRY(pass(ctx, s, "recon_a", [&] { return launch_recon_a_tstore(ny, a, tm, nb, s); }));
        } else {
            ReconA a{};
            fill_a(a);
            PH_TRY(pass(ctx, s, "recon_a", [&] { return launch_recon_a(ny, a, nb, s); }));
        }
        if (kind == RK_PROJ && effective_form(ctx, nx, ny) != PH_FORM_FP32) {
            const int form = effective_form(ctx, nx, ny);
            ReconBTc b{};
            PH_TRY(get_tc_table(ctx, nx, form, s, &b.table));
            b.t = t; b.proj64 = p64; b.rows = ny_out; b.k0 = k0; b.nbatch = nb; b.group = group;
            b.err = static_cast<int *>(ctx->small);
            PH_TRY(pass(ctx, s, "recon_b_tc", [&] { return launch_recon_b_tc(nx, form, b, s); }));
        } else if (kind == RK_PROJ) {
            ReconB<EPI_PROJ> b{};
            b.t = t; b.tw = tw_x; b.proj64 = p64; b.rows = ny_out; b.nx_out = nx_out; b.x0 = 0;
            b.k0 = k0; b.nbatch = nb; b.group = group; b.vol_slice_stride = (long long)nx_out * ny_out;
            b.err = static_cast<int *>(ctx->small);
            PH_TRY(pass(ctx, s, "recon_b",[&] { return launch_recon_b(nx, b, s); }));
        } else if (kind == RK_SUB) {
            ReconB<EPI_SUB> b{};
            b.t = t; b.tw = tw_x; b.vol = vol; b.rows = ny_out; b.nx_out = nx_out; b.x0 = 0;
            b.k0 = k0; b.nbatch = nb; b.group = group;
            b.row_ptr = sub->row_ptr; b.row_box = sub->row_box; b.boxes = sub->boxes;
            b.err = static_cast<int *>(ctx->small);
            PH_TRY(pass(ctx, s, "recon_b",[&] { return launch_recon_b(nx, b, s); }));
        } else if (kind == RK_CVOL) {
            ReconB<EPI_CVOL> b{};
            b.t = t; b.tw = tw_x; b.vol = vol; b.rows = ny_out; b.nx_out = nx_out; b.x0 = 0;
            b.k0 = k0; b.nbatch = nb; b.group = group; b.vol_slice_stride = (long long)nx_out * ny_out;
            b.err = static_cast<int *>(ctx->small);
            PH_TRY(pass(ctx, s, "recon_b",[&] { return launch_recon_b(nx, b, s); }));
        } else {
            ReconB<EPI_VOL> b{};
            b.t = t; b.tw = tw_x; b.vol = vol; b.vol_dtype = vol_dtype; b.proj64 = want_proj ? p64 : nullptr;
            b.threshold = threshold;
            b.rows = ny_out; b.nx_out = nx_out; b.x0 = x0;
            b.k0 = k0; b.nbatch = nb; b.group = group; b.vol_slice_stride = (long long)nx_out * ny_out;
            b.err = static_cast<int *>(ctx->small);
            PH_TRY(pass(ctx, s, "recon_b",[&] { return launch_recon_b(nx, b, s); }));
        }
    }
    if (want_proj && (proj != nullptr || argmin != nullptr)) {
        const size_t n = (size_t)nx_out * ny_out;
        k_proj_finish<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(p64, proj, argmin, n);
        PH_TRY(launched(ctx, cudaGetLastError(), "projection finish"));
    }
    return PH_OK;
}

// ---------------------------------------------------------------- propagation plumbing

// out = IFFT2( FFT2(in) .* H(centred) ) with H = transfer (or real mask).
int issue_propagate(ph_ctx *ctx, float2 *out, const float2 *in, const float2 *h, const float *mask, int nx, int ny,
                    float2 *bufa, float2 *bufb, const float2 *tw_x, const float2 *tw_y, cudaStream_t s) {
    FwdRowsT<FWD_COMPLEX> f{};
    f.src = in;
    f.dst = bufa;
    f.tw = tw_x;
    f.nrows = ny;
    PH_TRY(pass(ctx, s, "fwd_rows",[&] { return launch_fwd_rows(nx, f, s); }));
    GsCol c{};
    c.src = bufa;
    c.h = h;
    c.mask = mask;
    c.dst = bufb;
    c.tw = tw_y;
    c.nx = nx;
    c.scale = (float)(1.0 / ((double)nx * (double)ny));
    PH_TRY(pass(ctx, s, "gs_col",[&] { return launch_gs_col(ny, c, s); }));
    GsRow<ROW_INV> r{};
    r.src = bufb;
    r.dst = out;
    r.tw = tw_x;
    r.nrows = ny;
    PH_TRY(pass(ctx, s, "inv_rows",[&] { return launch_gs_row(nx, r, s); }));
    return PH_OK;
}

// ---------------------------------------------------------------- batches

// ---------------------------------------------------------------- serving

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

void CUDART_CB serve_done(void *p) {   // host callback: no CUDA calls here
    auto *t = static_cast<ph_serve_ticket *>(p);
    const double now = now_s();
    t->t_done = now;
    for (auto *m : t->members) m->t_done = now;
    std::lock_guard<std::mutex> lk(t->srv->cmu);   // held briefly, never around a CUDA call
    t->done.store(1, std::memory_order_release);
    t->srv->completed.push_back(t);
    for (auto *m : t->members) {
        m->done.store(1, std::memory_order_release);
        t->srv->completed.push_back(m);
    }
}

cudaEvent_t serve_event(ph_server *srv) {
    if (!srv->event_pool.empty()) {
        cudaEvent_t e = srv->event_pool.back();
        srv->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return e;
}

// The transfer function H(-z) of a request's grid, built on stream `ls` (the
// reference's Float32 square-root term, then its FP64-phase exponential) or
// taken from the cache; `ls` is ordered after its build.
int serve_transfer(ph_server *srv, cudaStream_t ls, float *dsqr, int nx, int ny, double z, double wavlen,
                   double dx, const float2 **out, ph_serve_tf **entry) {
    ph_ctx *ctx = srv->ctx;
    const auto key = std::make_tuple(nx, ny, z, wavlen, dx);
    auto it = srv->tfs.find(key);
    if (it == srv->tfs.end()) {
        if ((int)srv->tfs.size() >= srv->tf_cap) {   // evict the least recently used entry
            auto victim = srv->tfs.begin();
            for (auto jt = srv->tfs.begin(); jt != srv->tfs.end(); ++jt)
                if (jt->second.stamp < victim->second.stamp) victim = jt;
            // requests on any lane may still read it: let every lane drain first (evictions are rare)
            for (auto x : srv->streams) PH_CUDA(cudaStreamSynchronize(x), "cudaStreamSynchronize");
            cudaFree(victim->second.buf);
            cudaEventDestroy(victim->second.ready);
            cudaEventDestroy(victim->second.last_use);
            srv->tfs.erase(victim);
        }
        ph_serve_tf e{};
        PH_CUDA(cudaMalloc(&e.buf, sizeof(float2) * (size_t)nx * ny), "cudaMalloc(transfer)");
        if (cudaEventCreateWithFlags(&e.ready, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&e.last_use, cudaEventDisableTiming) != cudaSuccess) {
            cudaFree(e.buf);
            return cuda_status(ctx, cudaGetLastError(), "cudaEventCreate");
        }
        dim3 b(32, 8);
        k_transfer_sqrt<<<grid2d(nx, ny, b), b, 0, ls>>>(dsqr, nx, ny, wavlen, dx);
        const size_t n = (size_t)nx * ny;
        k_transfer<<<(unsigned)((n + 255) / 256), 256, 0, ls>>>(e.buf, dsqr, n, (2.0 * M_PI * (-z)) / wavlen);
        PH_TRY(launched(ctx, cudaGetLastError(), "serve transfer", 2));
        PH_CUDA(cudaEventRecord(e.ready, ls), "cudaEventRecord");
        it = srv->tfs.emplace(key, e).first;
    } else {
        PH_CUDA(cudaStreamWaitEvent(ls, it->second.ready, 0), "cudaStreamWaitEvent");
    }
    it->second.stamp = ++srv->clock;
    *out = it->second.buf;
    *entry = &it->second;
    return PH_OK;
}

// Longest-processing-time assignment of items (work = pixels x slices) to lanes.
// A group of batch items of one transform shape and input kind, issued as one
// launch of each pass (grid z = item): the forward rows, the spectrum, and per
// slice batch pass A and pass B, then each item's projection.  Items sit in
// consecutive scratch slots of `item_bytes` from `base`.  Every item gets the
// slice batches and slice groups of a single ph_reconst_xyproj call over its
// own slices, so its results equal that call's exactly.
size_t group_item_bytes(ph_ctx *ctx, int nx, int ny, int max_slices) {
    const ReconLayout L = recon_layout(ctx, nx, ny, ny, nx, max_slices, kLaneBatchBytes);
    return (L.total + kAlign - 1) / kAlign * kAlign;
}

int issue_recon_group(ph_ctx *ctx, const std::vector<const ph_recon_item *> &its, char *base, cudaStream_t s) {
    const int G = (int)its.size();
    const int nx = its[0]->n_fast, ny = its[0]->n_slow;
    int smax = 0;
    for (auto *it : its) smax = std::max(smax, (int)it->slices);
    const ReconLayout L = recon_layout(ctx, nx, ny, ny, nx, smax, kLaneBatchBytes);
    const size_t ib = group_item_bytes(ctx, nx, ny, smax);
    auto slot = [&](int i, size_t off) { return base + (size_t)i * ib + off; };
    const float2 *tw_x = ctx->tw[nx], *tw_y = ctx->tw[ny];
    // forward rows (the wavefront sqrt(I) formed in the first stage for hologram items)
    if (its[0]->hologram != nullptr) {
        FwdRowsT<FWD_SQRT_REAL> f{};
        f.src_real = its[0]->hologram;
        for (int i = 0; i < G; ++i) f.src_real_items[i] = its[i]->hologram;
        f.dst = reinterpret_cast<float2 *>(slot(0, L.a1));
        f.dst_stride = ib / sizeof(float2);
        f.tw = tw_x;
        f.nrows = ny;
        f.nitems = G;
        PH_TRY(pass(ctx, s, "fwd_rows", [&] { return launch_fwd_rows(nx, f, s); }));
    } else {
        FwdRowsT<FWD_COMPLEX> f{};
        f.src = static_cast<const float2 *>(its[0]->wavefront);
        for (int i = 0; i < G; ++i) f.src_items[i] = static_cast<const float2 *>(its[i]->wavefront);
        f.dst = reinterpret_cast<float2 *>(slot(0, L.a1));
        f.dst_stride = ib / sizeof(float2);
        f.tw = tw_x;
        f.nrows = ny;
        f.nitems = G;
        PH_TRY(pass(ctx, s, "fwd_rows", [&] { return launch_fwd_rows(nx, f, s); }));
    }
    SpectrumCols c{};
    c.a1 = reinterpret_cast<const float2 *>(slot(0, L.a1));
    c.hf = static_cast<const float2 *>(its[0]->tf_front);
    c.hdz = static_cast<const float2 *>(its[0]->tf_dz);
    for (int i = 0; i < G; ++i) {
        c.hf_items[i] = static_cast<const float2 *>(its[i]->tf_front);
        c.hdz_items[i] = static_cast<const float2 *>(its[i]->tf_dz);
    }
    c.lpf = nullptr;
    c.ptab = ctx->phase_tab;
    c.state = reinterpret_cast<float4 *>(slot(0, L.state));
    c.a1_stride = ib / sizeof(float2);
    c.state_stride = ib / sizeof(float4);
    c.tw = tw_y;
    c.nx = nx;
    c.ny = ny;
    c.scale = (float)(1.0 / ((double)nx * (double)ny));
    c.nitems = G;
    PH_TRY(pass(ctx, s, "spectrum", [&] { return launch_spectrum(ny, c, s); }));
    const size_t npix = (size_t)nx * ny;
    for (int i = 0; i < G; ++i)
        PH_CUDA(cudaMemsetAsync(slot(i, L.p64), 0xff, sizeof(unsigned long long) * npix, s), "cudaMemsetAsync");
    const int row_blocks_a = (nx + recon_a_rows(ny) - 1) / recon_a_rows(ny);
    const ph_tuning *tu = tuning_of(ctx, nx, ny);
    for (int k0 = 0; k0 < smax; k0 += L.batch) {
        ReconAGrouped a{};
        ReconB<EPI_PROJ, true> b{};
        for (int i = 0; i < G; ++i) {
            const int nb = std::max(0, std::min(L.batch, (int)its[i]->slices - k0));
            const int grp = nb > 0 ? recon_group(nb, row_blocks_a, recon_a_chain(ny), tu ? tu->group_cap : 0) : 1;
            a.set_item(i, nb, grp);
            b.set_item(i, nb, grp);
        }
        a.state = reinterpret_cast<const float4 *>(slot(0, L.state));
        a.t = reinterpret_cast<float2 *>(slot(0, L.t));
        a.item_state_stride = ib / sizeof(float4);
        a.item_t_stride = ib / sizeof(float2);
        a.tw = tw_y;
        a.nx = nx;
        a.ny_out = ny;
        a.y0 = 0;
        a.k0 = k0;
        a.nbatch = a.item_nb(0);   // item 0 has the most slices
        a.group = a.item_group(0);
        a.nitems = G;
        a.err = static_cast<int *>(ctx->small);
        CUtensorMap tm;
        if (recon_a_group_tstore(ny) &&
            t_store_map_items(&tm, a.t, nx, ny, L.batch, G, ib, recon_a_tstore_box(ny))) {
            ReconAGroupedTStore at{};
            static_cast<ReconItems &>(at) = static_cast<const ReconItems &>(a);
            at.state = a.state;
            at.t = a.t;
            at.tw = a.tw;
            at.err = a.err;
            at.nx = a.nx;
            at.ny_out = a.ny_out;
            at.y0 = a.y0;
            at.k0 = a.k0;
            at.nbatch = a.nbatch;
            at.group = a.group;
            PH_TRY(pass(ctx, s, "recon_a", [&] { return launch_recon_a_group_tstore(ny, at, tm, s); }));
        } else {
            PH_TRY(pass(ctx, s, "recon_a", [&] { return launch_recon_a_group(ny, a, s); }));
        }
        b.t = reinterpret_cast<const float2 *>(slot(0, L.t));
        b.tw = tw_x;
        b.proj64 = reinterpret_cast<unsigned long long *>(slot(0, L.p64));
        b.item_t_stride = ib / sizeof(float2);
        b.p64_stride = ib / sizeof(unsigned long long);
        b.rows = ny;
        b.nx_out = nx;
        b.x0 = 0;
        b.k0 = k0;
        b.nbatch = b.item_nb(0);
        b.group = b.item_group(0);
        b.vol_slice_stride = (long long)npix;
        b.nitems = G;
        b.err = static_cast<int *>(ctx->small);
        PH_TRY(pass(ctx, s, "recon_b", [&] { return launch_recon_b_group(nx, b, s); }));
    }
    for (int i = 0; i < G; ++i) {
        k_proj_finish<<<(unsigned)((npix + 255) / 256), 256, 0, s>>>(
            reinterpret_cast<const unsigned long long *>(slot(i, L.p64)), its[i]->proj, its[i]->argmin, npix);
        PH_TRY(launched(ctx, cudaGetLastError(), "projection finish"));
    }
    return PH_OK;
}

}  // namespace

// ====================================================================== C ABI

// An NVTX range named after the entry point spans every call (visible in
// Nsight timelines; a no-op without a tool attached).
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};

#define PH_ENTER(ctx, stream)                             \
    NvtxRange _nvtx(__func__);                            \
    if ((ctx) == nullptr) return PH_ERR_INVALID;          \
    std::lock_guard<std::mutex> _lk((ctx)->mu);           \
    DeviceGuard _dg((ctx)->device);                       \
    cudaStream_t s = static_cast<cudaStream_t>(stream);   \
    PH_TRY(begin_call((ctx), s))

#define PH_LEAVE(ctx) return end_call((ctx), s)

#define PH_NONNULL(p, name)                                           \
    do {                                                              \
        if ((p) == nullptr) {                                         \
            set_err(ctx, "%s must not be NULL", name);                \
            return PH_ERR_INVALID;                                    \
        }                                                             \
    } while (0)

extern "C" {

int32_t ph_version(void) { return kVersion; }

int32_t ph_create(int32_t device, size_t hbm_budget_bytes, ph_ctx **out) {
    if (out == nullptr) return PH_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return PH_ERR_CUDA;
    }
    ph_ctx *ctx = new ph_ctx();
    ctx->device = device;
    ctx->budget = hbm_budget_bytes;
    DeviceGuard g(device);
    if (cudaEventCreateWithFlags(&ctx->done, cudaEventDisableTiming) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->capture_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&ctx->small, 256) != cudaSuccess || cudaMemset(ctx->small, 0, 256) != cudaSuccess ||
        cudaMalloc(&ctx->phase_tab, sizeof(float4) * kPhaseTable) != cudaSuccess) {
        cudaGetLastError();
        ph_destroy(ctx);
        return PH_ERR_CUDA;
    }
    k_phase_table<<<(kPhaseTable + 255) / 256, 256>>>(ctx->phase_tab, kPhaseTable);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) {
        cudaGetLastError();
        ph_destroy(ctx);
        return PH_ERR_CUDA;
    }
    *out = ctx;
    return PH_OK;
}

void ph_destroy(ph_ctx *ctx) {
    if (ctx == nullptr) return;
    {
        DeviceGuard g(ctx->device);
        cudaDeviceSynchronize();
        for (auto &gr : ctx->graphs) cudaGraphExecDestroy(gr.exec);
        for (auto &r : ctx->prof) {
            cudaEventDestroy(r.start);
            cudaEventDestroy(r.stop);
        }
        for (auto e : ctx->prof_pool) cudaEventDestroy(e);
        for (auto &kv : ctx->tw) cudaFree(kv.second);
        for (auto &kv : ctx->tc_tables) cudaFree(kv.second);
        if (ctx->scratch) cudaFree(ctx->scratch);
        if (ctx->small) cudaFree(ctx->small);
        if (ctx->phase_tab) cudaFree(ctx->phase_tab);
        if (ctx->done) cudaEventDestroy(ctx->done);
        if (ctx->capture_stream) cudaStreamDestroy(ctx->capture_stream);
        cudaGetLastError();
    }
    delete ctx;
}

const char *ph_last_error(const ph_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int32_t ph_set_option(ph_ctx *ctx, int32_t option, int64_t value) {
    if (ctx == nullptr) return PH_ERR_INVALID;
    std::lock_guard<std::mutex> lk(ctx->mu);
    switch (option) {
        case PH_OPT_SLICE_BATCH: ctx->opt_slice_batch = value; return PH_OK;
        case PH_OPT_USE_GRAPHS: ctx->opt_use_graphs = value; return PH_OK;
        case PH_OPT_LOOP_LIMIT:
            if (value < 1) return PH_ERR_INVALID;
            ctx->opt_loop_limit = value;
            return PH_OK;
        case PH_OPT_PROFILE: ctx->opt_profile = value; return PH_OK;
        case PH_OPT_FORM:
            if (value < PH_FORM_FP32 || value > PH_FORM_TUNED) break;
            ctx->opt_form = value;
            return PH_OK;
    }
    set_err(ctx, "unknown option %d", option);
    return PH_ERR_INVALID;
}

int64_t ph_profile_report(ph_ctx *ctx, char *buf, int64_t cap) {
    if (ctx == nullptr) return -1;
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    std::vector<std::pair<std::string, std::pair<int64_t, double>>> agg;
    for (auto &r : ctx->prof) {
        float ms = 0.f;
        if (cudaEventSynchronize(r.stop) == cudaSuccess && cudaEventElapsedTime(&ms, r.start, r.stop) == cudaSuccess) {
            auto it = std::find_if(agg.begin(), agg.end(), [&](auto &e) { return e.first == r.name; });
            if (it == agg.end()) {
                agg.push_back({r.name, {1, (double)ms}});
            } else {
                it->second.first += 1;
                it->second.second += ms;
            }
        }
        cudaGetLastError();
        ctx->prof_pool.push_back(r.start);
        ctx->prof_pool.push_back(r.stop);
    }
    ctx->prof.clear();
    std::string out;
    char line[256];
    for (auto &e : agg) {
        snprintf(line, sizeof line, "%s,%lld,%.6f\n", e.first.c_str(), (long long)e.second.first, e.second.second);
        out += line;
    }
    if (buf && cap > 0) {
        const size_t n = std::min<size_t>(out.size(), (size_t)cap - 1);
        memcpy(buf, out.data(), n);
        buf[n] = '\0';
    }
    return (int64_t)out.size() + 1;
}

size_t ph_scratch_bytes(const ph_ctx *ctx) { return ctx ? ctx->scratch_bytes : 0; }
int64_t ph_kernel_launches(const ph_ctx *ctx) { return ctx ? ctx->launches.load() : 0; }

int32_t ph_reserve(ph_ctx *ctx, int32_t n_fast, int32_t n_slow, int32_t slices, void *stream) {
    PH_ENTER(ctx, stream);
    PH_TRY(check_len(ctx, n_fast, n_slow));
    ReconLayout L = recon_layout(ctx, n_fast, n_slow, n_slow, n_fast, std::max(1, (int)slices));
    const size_t gs = 2 * sizeof(float2) * (size_t)n_fast * n_slow + 2 * kAlign;
    PH_TRY(ensure_scratch(ctx, std::max(L.total, gs), s));
    const float2 *tw = nullptr;
    PH_TRY(get_twiddles(ctx, n_fast, s, &tw));
    PH_TRY(get_twiddles(ctx, n_slow, s, &tw));
    PH_LEAVE(ctx);
}

int32_t ph_transfer_sqrt(ph_ctx *ctx, float *out, int32_t n_fast, int32_t n_slow, double wavlen, double dx,
                         void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(out, "out");
    if (n_fast <= 0 || n_slow <= 0) { set_err(ctx, "sizes must be positive"); return PH_ERR_SIZE; }
    dim3 b(32, 8);
    k_transfer_sqrt<<<grid2d(n_fast, n_slow, b), b, 0, s>>>(out, n_fast, n_slow, wavlen, dx);
    PH_TRY(launched(ctx, cudaGetLastError(), "transfer_sqrt"));
    PH_LEAVE(ctx);
}

int32_t ph_transfer(ph_ctx *ctx, void *out, const float *d_sqr, int32_t n_fast, int32_t n_slow, double z0,
                    double wavlen, void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(out, "out");
    PH_NONNULL(d_sqr, "d_sqr");
    if (n_fast <= 0 || n_slow <= 0) { set_err(ctx, "sizes must be positive"); return PH_ERR_SIZE; }
    const size_t n = (size_t)n_fast * n_slow;
    const double c = (2.0 * M_PI * z0) / wavlen;
    k_transfer<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(static_cast<float2 *>(out), d_sqr, n, c);
    PH_TRY(launched(ctx, cudaGetLastError(), "transfer"));
    PH_LEAVE(ctx);
}

int32_t ph_transfer_fp64(ph_ctx *ctx, void *out, int32_t n_fast, int32_t n_slow, double z, double wavlen, double dx,
                         void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(out, "out");
    if (n_fast <= 0 || n_slow <= 0) { set_err(ctx, "sizes must be positive"); return PH_ERR_SIZE; }
    dim3 b(32, 8);
    const double c = (2.0 * M_PI * z) / wavlen;
    k_transfer_fp64<<<grid2d(n_fast, n_slow, b), b, 0, s>>>(static_cast<float2 *>(out), n_fast, n_slow, c, wavlen,
                                                          dx);
    PH_TRY(launched(ctx, cudaGetLastError(), "transfer_fp64"));
    PH_LEAVE(ctx);
}

int32_t ph_gabor_wavefront(ph_ctx *ctx, void *out, const float *holo, int32_t n_fast, int32_t n_slow,
                           void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(out, "out");
    PH_NONNULL(holo, "holo");
    if (n_fast <= 0 || n_slow <= 0) { set_err(ctx, "sizes must be positive"); return PH_ERR_SIZE; }
    const size_t n = (size_t)n_fast * n_slow;
    k_gabor<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(static_cast<float2 *>(out), holo, n);
    PH_TRY(launched(ctx, cudaGetLastError(), "gabor"));
    PH_LEAVE(ctx);
}

int32_t ph_pad2d(ph_ctx *ctx, void *out, const void *in, int32_t n_fast, int32_t n_slow, void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(out, "out");
    PH_NONNULL(in, "in");
    if (n_fast <= 0 || n_slow <= 0 || n_fast != n_slow) {
        set_err(ctx, "cu_2d_pad needs a square input. Got (%d, %d).", n_fast, n_slow);
        return PH_ERR_SIZE;
    }
    PH_TRY(ensure_scratch(ctx, 2 * kAlign, s));
    double *acc = at<double>(ctx, 0);
    float2 *mean = at<float2>(ctx, kAlign);
    PH_CUDA(cudaMemsetAsync(acc, 0, 2 * sizeof(double), s), "cudaMemsetAsync");
    const size_t n = (size_t)n_fast * n_slow;
    k_sum_c64<<<256, 256, 0, s>>>(static_cast<const float2 *>(in), n, acc);
    k_mean_finish<<<1, 1, 0, s>>>(acc, (double)n, mean);
    const int nout = 2 * n_fast;
    dim3 b(32, 8);
    k_pad_fill<<<grid2d(nout, nout, b), b, 0, s>>>(static_cast<float2 *>(out), static_cast<const float2 *>(in), mean,
                                                  n_fast, n_slow, nout, nout / 4);
    PH_TRY(launched(ctx, cudaGetLastError(), "pad2d", 3));
    PH_LEAVE(ctx);
}

int32_t ph_phase_retrieval(ph_ctx *ctx, void *out, const float *holo1, const float *holo2, const void *transfer,
                           const void *invtransfer, int32_t n_fast, int32_t n_slow, int32_t priter, double *residual,
                           void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(out, "out");
    PH_NONNULL(holo1, "holo1");
    PH_NONNULL(holo2, "holo2");
    PH_NONNULL(transfer, "transfer");
    PH_NONNULL(invtransfer, "invtransfer");
    PH_TRY(check_len(ctx, n_fast, n_slow));
    if (priter < 0) { set_err(ctx, "priter must be >= 0"); return PH_ERR_INVALID; }
    const int nx = n_fast, ny = n_slow;
    const size_t n = (size_t)nx * ny;
    float2 *o = static_cast<float2 *>(out);
    double *acc = reinterpret_cast<double *>(static_cast<char *>(ctx->small) + 64);
    if (priter == 0) {   // light1 = sqrt(I1) + 0im
        k_gabor<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(o, holo1, n);
        PH_TRY(launched(ctx, cudaGetLastError(), "gabor"));
        if (residual) PH_CUDA(cudaMemsetAsync(residual, 0, sizeof(double), s), "memset");
        PH_LEAVE(ctx);
    }
    // The staged persistent passes take the transfers as [kx][ky] rows.
    const bool staged = gs_row_staged(nx) && gs_col_staged(ny);
    Arena a;
    const size_t oa = a.take<float2>(n), ob = a.take<float2>(n);
    const size_t oh = staged ? a.take<float2>(n) : 0, ohi = staged ? a.take<float2>(n) : 0;
    const size_t oa1 = staged ? a.take<float>(n) : 0, oa2 = staged ? a.take<float>(n) : 0;
    PH_TRY(ensure_scratch(ctx, a.off, s));
    float2 *bufa = at<float2>(ctx, oa), *bufb = at<float2>(ctx, ob);
    float2 *ht = staged ? at<float2>(ctx, oh) : nullptr, *hti = staged ? at<float2>(ctx, ohi) : nullptr;
    float *amp1 = staged ? at<float>(ctx, oa1) : nullptr, *amp2 = staged ? at<float>(ctx, oa2) : nullptr;
    int *err = static_cast<int *>(ctx->small);
    const float2 *tw_x = nullptr, *tw_y = nullptr;
    PH_TRY(get_twiddles(ctx, nx, s, &tw_x));
    PH_TRY(get_twiddles(ctx, ny, s, &tw_y));
    char key[512];
    snprintf(key, sizeof key, "gs|%d|%d|%d|%p|%p|%p|%p|%p|%p|%p", nx, ny, priter, out, (const void *)holo1,
             (const void *)holo2, transfer, invtransfer, (void *)residual, ctx->scratch);
    PH_TRY(run_graph(ctx, s, key, [&](cudaStream_t s) -> int {
    if (residual) PH_CUDA(cudaMemsetAsync(acc, 0, 2 * sizeof(double), s), "memset");
    const float scale = (float)(1.0 / ((double)nx * (double)ny));
    if (staged) {
        dim3 tb(32, 8), tg((nx + 31) / 32, (ny + 31) / 32);
        k_transfer_rows<<<tg, tb, 0, s>>>(ht, static_cast<const float2 *>(transfer), nx, ny, scale);
        k_transfer_rows<<<tg, tb, 0, s>>>(hti, static_cast<const float2 *>(invtransfer), nx, ny, scale);
        // the amplitudes sqrt(I1), sqrt(I2) once per call, as the row passes would form them
        k_sqrt_f32<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(amp1, holo1, n);
        k_sqrt_f32<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(amp2, holo2, n);
        PH_TRY(launched(ctx, cudaGetLastError(), "transfer rows and amplitudes", 4));
    }

    FwdRowsT<FWD_SQRT_REAL> f{};
    f.src_real = holo1;
    f.dst = bufa;
    f.tw = tw_x;
    f.nrows = ny;
    PH_TRY(pass(ctx, s, "fwd_rows",[&] { return launch_fwd_rows(nx, f, s); }));
    // The staged passes store through tensor maps where their blocks allow it:
    // the column pass writes bufb = [ny][nx], the row pass bufa = [nx][ny].
    CUtensorMap tm_col, tm_row;
    const bool ts_col = staged && gs_tstore_len(ny) && gs_store_map(&tm_col, bufb, nx, ny, gs_rows(ny));
    const bool ts_row = staged && gs_tstore_len(nx) && gs_store_map(&tm_row, bufa, ny, nx, gs_rows(nx));
    const auto col = [&](const GsColT &c) {
        return ts_col ? launch_gs_col_ts(ny, c, tm_col, s) : launch_gs_col_t(ny, c, s);
    };
    const auto row = [&](const GsRowMidT &r) {
        return ts_row ? launch_gs_row_ts(nx, r, tm_row, s) : launch_gs_row_t(nx, r, s);
    };
    for (int it = 0; it < priter && staged; ++it) {
        const bool last = it == priter - 1;
        GsColT c{};
        c.src = bufa; c.ht = ht; c.dst = bufb; c.tw = tw_y; c.err = err; c.nx = nx;
        PH_TRY(pass(ctx, s, "gs_col",[&] { return col(c); }));
        GsRowMidT r2{};
        r2.src = bufb; r2.holo = amp2; r2.dst = bufa; r2.tw = tw_x; r2.err = err; r2.nrows = ny;
        r2.resid = (last && residual) ? acc : nullptr;
        PH_TRY(pass(ctx, s, "gs_row_mid",[&] { return row(r2); }));
        c.src = bufa; c.ht = hti; c.dst = bufb;
        PH_TRY(pass(ctx, s, "gs_col",[&] { return col(c); }));
        if (!last) {
            GsRowMidT r1{};
            r1.src = bufb; r1.holo = amp1; r1.dst = bufa; r1.tw = tw_x; r1.err = err; r1.nrows = ny;
            PH_TRY(pass(ctx, s, "gs_row_mid",[&] { return row(r1); }));
        } else {
            GsRowMidT r1{};   // the persistent pass in its final form: natural store into the output
            r1.src = bufb; r1.holo = amp1; r1.dst = o; r1.tw = tw_x; r1.err = err; r1.nrows = ny;
            PH_TRY(pass(ctx, s, "gs_row_final",[&] { return launch_gs_row_final_t(nx, r1, s); }));
        }
    }
    for (int it = 0; it < priter && !staged; ++it) {
        const bool last = it == priter - 1;
        GsCol c{};
        c.src = bufa; c.h = static_cast<const float2 *>(transfer); c.dst = bufb; c.tw = tw_y; c.nx = nx;
        c.scale = scale;
        PH_TRY(pass(ctx, s, "gs_col",[&] { return launch_gs_col(ny, c, s); }));
        GsRow<ROW_MID> r2{};
        r2.src = bufb; r2.holo = holo2; r2.dst = bufa; r2.tw = tw_x; r2.nrows = ny;
        r2.resid = (last && residual) ? acc : nullptr;
        PH_TRY(pass(ctx, s, "gs_row_mid",[&] { return launch_gs_row(nx, r2, s); }));
        c.src = bufa; c.h = static_cast<const float2 *>(invtransfer); c.dst = bufb;
        PH_TRY(pass(ctx, s, "gs_col",[&] { return launch_gs_col(ny, c, s); }));
        if (!last) {
            GsRow<ROW_MID> r1{};
            r1.src = bufb; r1.holo = holo1; r1.dst = bufa; r1.tw = tw_x; r1.nrows = ny;
            PH_TRY(pass(ctx, s, "gs_row_mid",[&] { return launch_gs_row(nx, r1, s); }));
        } else {
            GsRow<ROW_FINAL> r1{};
            r1.src = bufb; r1.holo = holo1; r1.dst = o; r1.tw = tw_x; r1.nrows = ny;
            PH_TRY(pass(ctx, s, "gs_row_final",[&] { return launch_gs_row(nx, r1, s); }));
        }
    }
    if (residual) {
        k_resid_finish<<<1, 1, 0, s>>>(acc, residual);
        PH_TRY(launched(ctx, cudaGetLastError(), "GS residual"));
    }
    return PH_OK;
    }));
    PH_LEAVE(ctx);
}

int32_t ph_asm_prop(ph_ctx *ctx, void *out, const void *in, const float *d_sqr, double zprop, int32_t n_fast,
                    int32_t n_slow, double wavlen, void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(out, "out");
    PH_NONNULL(in, "in");
    PH_NONNULL(d_sqr, "d_sqr");
    PH_TRY(check_len(ctx, n_fast, n_slow));
    const int nx = n_fast, ny = n_slow;
    const size_t n = (size_t)nx * ny;
    Arena a;
    const size_t oh = a.take<float2>(n), oa = a.take<float2>(n), ob = a.take<float2>(n);
    PH_TRY(ensure_scratch(ctx, a.off, s));
    const float2 *tw_x = nullptr, *tw_y = nullptr;
    PH_TRY(get_twiddles(ctx, nx, s, &tw_x));
    PH_TRY(get_twiddles(ctx, ny, s, &tw_y));
    float2 *h = at<float2>(ctx, oh);
    const double c = (2.0 * M_PI * zprop) / wavlen;
    k_transfer<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(h, d_sqr, n, c);
    PH_TRY(launched(ctx, cudaGetLastError(), "transfer"));
    PH_TRY(issue_propagate(ctx, static_cast<float2 *>(out), static_cast<const float2 *>(in), h, nullptr, nx, ny,
                           at<float2>(ctx, oa), at<float2>(ctx, ob), tw_x, tw_y, s));
    PH_LEAVE(ctx);
}

static int propagate_common(ph_ctx *ctx, void *out, const void *in, const float2 *tf, const float *mask, int nx,
                            int ny, cudaStream_t s) {
    PH_TRY(check_len(ctx, nx, ny));
    const size_t n = (size_t)nx * ny;
    Arena a;
    const size_t oa = a.take<float2>(n), ob = a.take<float2>(n);
    PH_TRY(ensure_scratch(ctx, a.off, s));
    const float2 *tw_x = nullptr, *tw_y = nullptr;
    PH_TRY(get_twiddles(ctx, nx, s, &tw_x));
    PH_TRY(get_twiddles(ctx, ny, s, &tw_y));
    return issue_propagate(ctx, static_cast<float2 *>(out), static_cast<const float2 *>(in), tf, mask, nx, ny,
                           at<float2>(ctx, oa), at<float2>(ctx, ob), tw_x, tw_y, s);
}

int32_t ph_propagate(ph_ctx *ctx, void *out, const void *in, const void *tf, int32_t n_fast, int32_t n_slow,
                     void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(out, "out");
    PH_NONNULL(in, "in");
    PH_NONNULL(tf, "tf");
    PH_TRY(propagate_common(ctx, out, in, static_cast<const float2 *>(tf), nullptr, n_fast, n_slow, s));
    PH_LEAVE(ctx);
}

int32_t ph_apply_lpf(ph_ctx *ctx, void *out, const void *in, const float *lpf, int32_t n_fast, int32_t n_slow,
                     void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(out, "out");
    PH_NONNULL(in, "in");
    PH_NONNULL(lpf, "lpf");
    PH_TRY(propagate_common(ctx, out, in, nullptr, lpf, n_fast, n_slow, s));
    PH_LEAVE(ctx);
}

int32_t ph_synth_hologram(ph_ctx *ctx, float *out, int32_t n_fast, int32_t n_slow, const double *discs_host,
                          int32_t count, double wavlen, double dx, double z_sensor, const float *noise,
                          void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(out, "out");
    if (count > 0) PH_NONNULL(discs_host, "discs");
    if (count < 0) { set_err(ctx, "negative disc count"); return PH_ERR_INVALID; }
    PH_TRY(check_len(ctx, n_fast, n_slow));
    const int nx = n_fast, ny = n_slow;
    const size_t n = (size_t)nx * ny;
    Arena a;
    const size_t opsi = a.take<float2>(n), oh = a.take<float2>(n), oa = a.take<float2>(n), ob = a.take<float2>(n);
    const size_t omm = a.take<float>(2);
    PH_TRY(ensure_scratch(ctx, a.off, s));
    const float2 *tw_x = nullptr, *tw_y = nullptr;
    PH_TRY(get_twiddles(ctx, nx, s, &tw_x));
    PH_TRY(get_twiddles(ctx, ny, s, &tw_y));
    float2 *psi = at<float2>(ctx, opsi), *h = at<float2>(ctx, oh);
    // farthest disc first (stable on ties)
    std::vector<int> order(count);
    for (int i = 0; i < count; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int p, int q) { return discs_host[4 * p + 3] > discs_host[4 * q + 3]; });
    PH_TRY(launched(ctx, synth_fill_one(psi, n, s), "synth fill"));
    dim3 b(32, 8);
    auto propagate_by = [&](double z) -> int {
        const double c = (2.0 * M_PI * z) / wavlen;
        k_transfer_fp64<<<grid2d(nx, ny, b), b, 0, s>>>(h, nx, ny, c, wavlen, dx);
        PH_TRY(launched(ctx, cudaGetLastError(), "synth transfer"));
        return issue_propagate(ctx, psi, psi, h, nullptr, nx, ny, at<float2>(ctx, oa), at<float2>(ctx, ob), tw_x,
                               tw_y, s);
    };
    double zc = count > 0 ? discs_host[4 * order[0] + 3] : z_sensor;
    for (int k = 0; k < count; ++k) {
        const double *d = discs_host + 4 * order[k];
        if (d[3] != zc) {
            PH_TRY(propagate_by(zc - d[3]));
            zc = d[3];
        }
        PH_TRY(launched(ctx, synth_disc(psi, nx, ny, d[0], d[1], d[2], dx, s), "synth disc"));
    }
    PH_TRY(propagate_by(zc - z_sensor));
    PH_TRY(launched(ctx, synth_finish(psi, out, n, noise, at<float>(ctx, omm), s), "synth finish", 3));
    PH_LEAVE(ctx);
}

int32_t ph_reconst_xyproj(ph_ctx *ctx, float *proj, int32_t *argmin, const void *wf, const void *tf_front,
                          const void *tf_dz, int32_t n_fast, int32_t n_slow, int32_t slices, void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(wf, "wavefront");
    PH_NONNULL(tf_front, "transfer_front");
    PH_NONNULL(tf_dz, "transfer_dz");
    if (proj == nullptr && argmin == nullptr) { set_err(ctx, "proj and argmin are both NULL"); return PH_ERR_INVALID; }
    if (slices < 1) { set_err(ctx, "slices must be >= 1. Got %d.", slices); return PH_ERR_SIZE; }
    PH_TRY(reconstruct(ctx, RK_PROJ, proj, argmin, nullptr, PH_F32, static_cast<const float2 *>(wf),
                       static_cast<const float2 *>(tf_front), static_cast<const float2 *>(tf_dz), n_fast, n_slow,
                       slices, s));
    PH_LEAVE(ctx);
}

// ---- autotuner: the reconstruction knobs per (n_fast, n_slow, device), timed once, cached as JSON
namespace {

// The cache file: {"<device>": {"<n_fast>x<n_slow>": {"slices": S, "form": F,
// "group_cap": G, "batch_slices": B, "ms": T}, ...}, ...}.  A small reader for
// exactly this shape (objects, strings, numbers).
struct JsonTune {
    std::map<std::string, std::map<std::string, std::map<std::string, double>>> dev;
};

void skip_ws(const std::string &t, size_t &i) {
    while (i < t.size() && (t[i] == ' ' || t[i] == '\n' || t[i] == '\r' || t[i] == '\t' || t[i] == ',')) ++i;
}
bool read_str(const std::string &t, size_t &i, std::string &out) {
    skip_ws(t, i);
    if (i >= t.size() || t[i] != '"') return false;
    const size_t j = t.find('"', i + 1);
    if (j == std::string::npos) return false;
    out = t.substr(i + 1, j - i - 1);
    i = j + 1;
    skip_ws(t, i);
    if (i >= t.size() || t[i] != ':') return false;
    ++i;
    return true;
}
bool expect(const std::string &t, size_t &i, char c) {
    skip_ws(t, i);
    if (i >= t.size() || t[i] != c) return false;
    ++i;
    return true;
}
bool peek(const std::string &t, size_t &i, char c) {
    skip_ws(t, i);
    return i < t.size() && t[i] == c;
}

bool parse_tune(const std::string &t, JsonTune &out) {
    size_t i = 0;
    if (!expect(t, i, '{')) return false;
    while (!peek(t, i, '}')) {
        std::string dname;
        if (!read_str(t, i, dname) || !expect(t, i, '{')) return false;
        while (!peek(t, i, '}')) {
            std::string shape;
            if (!read_str(t, i, shape) || !expect(t, i, '{')) return false;
            while (!peek(t, i, '}')) {
                std::string key;
                if (!read_str(t, i, key)) return false;
                skip_ws(t, i);
                char *end = nullptr;
                const double v = strtod(t.c_str() + i, &end);
                if (end == t.c_str() + i) return false;
                i = end - t.c_str();
                out.dev[dname][shape][key] = v;
            }
            ++i;
        }
        ++i;
    }
    return true;
}

std::string dump_tune(const JsonTune &j) {
    std::string o = "{\n";
    bool first_d = true;
    for (auto &d : j.dev) {
        o += (first_d ? "" : ",\n");
        first_d = false;
        o += " \"" + d.first + "\": {\n";
        bool first_s = true;
        for (auto &sh : d.second) {
            o += (first_s ? "" : ",\n");
            first_s = false;
            o += "  \"" + sh.first + "\": {";
            bool first_k = true;
            for (auto &kv : sh.second) {
                char num[64];
                snprintf(num, sizeof num, "%.9g", kv.second);
                o += (first_k ? "" : ", ");
                first_k = false;
                o += "\"" + kv.first + "\": " + num;
            }
            o += "}";
        }
        o += "\n }";
    }
    return o + "\n}\n";
}

std::string read_file(const char *path) {
    std::string t;
    if (FILE *f = fopen(path, "rb")) {
        char buf[4096];
        size_t n;
        while ((n = fread(buf, 1, sizeof buf, f)) > 0) t.append(buf, n);
        fclose(f);
    }
    return t;
}

}  // namespace

int32_t ph_autotune(ph_ctx *ctx, int32_t n_fast, int32_t n_slow, int32_t slices, int32_t allow_forms,
                    const char *cache_path, int32_t *choice, double *ms_out, void *stream) {
    PH_ENTER(ctx, stream);
    PH_TRY(check_len(ctx, n_fast, n_slow));
    if (slices < 1) { set_err(ctx, "slices must be >= 1. Got %d.", slices); return PH_ERR_SIZE; }
    if (capturing(s)) { set_err(ctx, "ph_autotune times launches and cannot run inside a stream capture"); return PH_ERR_INVALID; }
    cudaDeviceProp prop{};
    PH_CUDA(cudaGetDeviceProperties(&prop, ctx->device), "cudaGetDeviceProperties");
    std::string dname = prop.name;
    for (auto &c : dname) if (c == '"' || c == '\\') c = '_';
    char shape[64];
    snprintf(shape, sizeof shape, "%dx%d", n_fast, n_slow);
    JsonTune cache;
    if (cache_path != nullptr) {
        const std::string text = read_file(cache_path);
        if (!text.empty() && !parse_tune(text, cache)) cache.dev.clear();   // unreadable: retune and rewrite
    }
    auto report = [&](const ph_tuning &tu) {
        if (choice) { choice[0] = tu.form; choice[1] = tu.group_cap; choice[2] = tu.batch_slices; }
        if (ms_out) *ms_out = tu.ms;
    };
    auto dit = cache.dev.find(dname);
    if (dit != cache.dev.end()) {
        auto sit = dit->second.find(shape);
        if (sit != dit->second.end() && (int)sit->second["slices"] == slices &&
            (allow_forms || (int)sit->second["form"] == PH_FORM_FP32)) {
            ph_tuning tu;
            tu.form = (int)sit->second["form"];
            tu.group_cap = (int)sit->second["group_cap"];
            tu.batch_slices = (int)sit->second["batch_slices"];
            tu.slices = slices;
            tu.ms = sit->second["ms"];
            ctx->tuned[{n_fast, n_slow}] = tu;
            report(tu);
            PH_LEAVE(ctx);
        }
    }
    // timing inputs: unit-modulus transfer functions of the reference's form, and one as the wavefront
    const size_t n = (size_t)n_fast * n_slow;
    float2 *buf = nullptr;
    float *dsqr = nullptr, *proj = nullptr;
    int32_t *arg = nullptr;
    PH_CUDA(cudaMalloc(&buf, 3 * n * sizeof(float2)), "cudaMalloc(tuning inputs)");
    auto cleanup = [&]() {
        cudaFree(buf);
        if (dsqr) cudaFree(dsqr);
        if (proj) cudaFree(proj);
        if (arg) cudaFree(arg);
    };
    if (cudaMalloc(&dsqr, n * sizeof(float)) != cudaSuccess || cudaMalloc(&proj, n * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&arg, n * sizeof(int32_t)) != cudaSuccess) {
        cleanup();
        return cuda_status(ctx, cudaGetLastError(), "cudaMalloc(tuning outputs)");
    }
    float2 *wf = buf, *hf = buf + n, *hdz = buf + 2 * n;
    dim3 b2(32, 8);
    k_transfer_sqrt<<<grid2d(n_fast, n_slow, b2), b2, 0, s>>>(dsqr, n_fast, n_slow, 0.6328, 10.0);
    k_transfer<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(wf, dsqr, n, (2.0 * M_PI * 3000.0) / 0.6328);
    k_transfer<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(hf, dsqr, n, (2.0 * M_PI * -1000.0) / 0.6328);
    k_transfer<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(hdz, dsqr, n, (2.0 * M_PI * -200.0) / 0.6328);
    if (cudaGetLastError() != cudaSuccess) { cleanup(); return cuda_status(ctx, cudaErrorLaunchFailure, "tuning inputs"); }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int64_t saved_graphs = ctx->opt_use_graphs, saved_form = ctx->opt_form;
    const auto saved_entry = ctx->tuned.find({n_fast, n_slow});
    const bool had_entry = saved_entry != ctx->tuned.end();
    const ph_tuning saved_tu = had_entry ? saved_entry->second : ph_tuning{};
    ctx->opt_use_graphs = 0;
    ctx->opt_form = PH_FORM_TUNED;
    // candidates: slices per CTA, batch of intermediates (all / 64 slices), row-pass form
    std::vector<int> forms = {PH_FORM_FP32};
    if (allow_forms)
        for (int f : {PH_FORM_BF16X3, PH_FORM_FP16X3})
            if (recon_b_tc_supported(n_fast, f)) forms.push_back(f);
    ph_tuning best;
    best.ms = 1e300;
    int st = PH_OK;
    for (int form : forms) {
        for (int cap : {0, 16, 32, 64}) {
            for (int bs : {0, 64}) {
                if (bs > 0 && bs >= slices) continue;
                ph_tuning tu;
                tu.form = form;
                tu.group_cap = cap;
                tu.batch_slices = bs;
                tu.slices = slices;
                ctx->tuned[{n_fast, n_slow}] = tu;
                float best_ms = 1e30f;
                for (int rep = 0; rep < 3 && st == PH_OK; ++rep) {   // the first run also builds the tables
                    cudaEventRecord(e0, s);
                    st = reconstruct(ctx, RK_PROJ, proj, arg, nullptr, PH_F32, wf, hf, hdz, n_fast, n_slow, slices, s);
                    cudaEventRecord(e1, s);
                    if (st != PH_OK) break;
                    if (cudaEventSynchronize(e1) != cudaSuccess) { st = PH_ERR_CUDA; break; }
                    float ms = 0.0f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (rep > 0) best_ms = std::min(best_ms, ms);
                }
                if (st != PH_OK) break;
                if (best_ms < best.ms) {
                    best = tu;
                    best.ms = best_ms;
                }
            }
            if (st != PH_OK) break;
        }
        if (st != PH_OK) break;
    }
    ctx->opt_use_graphs = saved_graphs;
    ctx->opt_form = saved_form;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cleanup();
    if (st != PH_OK) {
        if (had_entry) ctx->tuned[{n_fast, n_slow}] = saved_tu;
        else ctx->tuned.erase({n_fast, n_slow});
        return st;
    }
    ctx->tuned[{n_fast, n_slow}] = best;
    report(best);
    if (cache_path != nullptr) {
        auto &e = cache.dev[dname][shape];
        e.clear();
        e["slices"] = slices;
        e["form"] = best.form;
        e["group_cap"] = best.group_cap;
        e["batch_slices"] = best.batch_slices;
        e["ms"] = best.ms;
        const std::string tmp = std::string(cache_path) + ".tmp";
        FILE *f = fopen(tmp.c_str(), "wb");
        const std::string text = dump_tune(cache);
        if (f == nullptr || fwrite(text.data(), 1, text.size(), f) != text.size()) {
            if (f) fclose(f);
            set_err(ctx, "could not write the tuning cache %s", cache_path);
            return PH_ERR_INVALID;
        }
        fclose(f);
        if (rename(tmp.c_str(), cache_path) != 0) {
            set_err(ctx, "could not replace the tuning cache %s", cache_path);
            return PH_ERR_INVALID;
        }
    }
    PH_LEAVE(ctx);
}

int32_t ph_reconst_xyproj_range(ph_ctx *ctx, int64_t *packed, const void *wf, const void *tf_front,
                                const void *tf_dz, int32_t n_fast, int32_t n_slow, int32_t k0, int32_t k1,
                                int32_t accumulate, void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(packed, "packed");
    PH_NONNULL(wf, "wavefront");
    PH_NONNULL(tf_front, "transfer_front");
    PH_NONNULL(tf_dz, "transfer_dz");
    if (k0 < 0 || k1 < k0) { set_err(ctx, "slice range [%d, %d) is invalid", k0, k1); return PH_ERR_SIZE; }
    auto *p = reinterpret_cast<unsigned long long *>(packed);
    if (k1 == k0) {
        // an empty shard contributes the merge identity
        PH_TRY(check_len(ctx, n_fast, n_slow));
        if (!accumulate) {
            const size_t npix = (size_t)n_fast * n_slow;
            k_fill_u64<<<(unsigned)std::min<size_t>((npix + 255) / 256, 4096), 256, 0, s>>>(p, npix, kPackedEmpty);
            PH_TRY(launched(ctx, cudaGetLastError(), "packed fill"));
        }
        PH_LEAVE(ctx);
    }
    PH_TRY(reconstruct(ctx, RK_PROJ, nullptr, nullptr, nullptr, PH_F32, static_cast<const float2 *>(wf),
                       static_cast<const float2 *>(tf_front), static_cast<const float2 *>(tf_dz), n_fast, n_slow,
                       k1 - k0, s, nullptr, 0.0f, p, accumulate != 0, k0));
    PH_LEAVE(ctx);
}

int32_t ph_unpack_projection(ph_ctx *ctx, float *proj, int32_t *argmin, const int64_t *packed, int32_t n_fast,
                             int32_t n_slow, void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(packed, "packed");
    if (proj == nullptr && argmin == nullptr) { set_err(ctx, "proj and argmin are both NULL"); return PH_ERR_INVALID; }
    if (n_fast < 1 || n_slow < 1) { set_err(ctx, "size %d x %d is invalid", n_fast, n_slow); return PH_ERR_SIZE; }
    const size_t n = (size_t)n_fast * n_slow;
    k_proj_finish<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(reinterpret_cast<const unsigned long long *>(packed),
                                                                proj, argmin, n);
    PH_TRY(launched(ctx, cudaGetLastError(), "projection unpack"));
    PH_LEAVE(ctx);
}

int32_t ph_batch_plan(ph_ctx *ctx, const ph_recon_item *items, int32_t count, int32_t lanes, ph_batch **out) {
    PH_ENTER(ctx, nullptr);
    PH_NONNULL(out, "out");
    *out = nullptr;
    if (count < 0 || (count > 0 && items == nullptr)) { set_err(ctx, "items must hold count >= 0 records"); return PH_ERR_INVALID; }
    if (lanes < 1 || lanes > 16) { set_err(ctx, "lanes must be in 1..16. Got %d.", lanes); return PH_ERR_INVALID; }
    for (int i = 0; i < count; ++i) {
        const ph_recon_item &it = items[i];
        if (it.hologram == nullptr && it.wavefront == nullptr) {
            set_err(ctx, "item %d: hologram and wavefront are both NULL", i);
            return PH_ERR_INVALID;
        }
        if (it.tf_front == nullptr || it.tf_dz == nullptr) { set_err(ctx, "item %d: transfer functions must not be NULL", i); return PH_ERR_INVALID; }
        if (it.proj == nullptr && it.argmin == nullptr) { set_err(ctx, "item %d: proj and argmin are both NULL", i); return PH_ERR_INVALID; }
        if (it.slices < 1) { set_err(ctx, "item %d: slices must be >= 1. Got %d.", i, it.slices); return PH_ERR_SIZE; }
        PH_TRY(check_len(ctx, it.n_fast, it.n_slow));
    }
    // Groups: items of one transform shape and input kind, most slices first,
    // up to kMaxItems per group and kGroupBytes of scratch, share one launch
    // of each pass.  Only items whose own pass A launch is small (under 4
    // waves of CTAs) are grouped: a large item fills the GPU alone, and the
    // grouped pass B runs fewer CTAs per SM.  (A shape whose projection runs a
    // tensor-core row pass keeps one item per group: that pass has no grouped
    // form.)
    constexpr size_t kGroupBytes = size_t(8) << 30;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess || sms <= 0) sms = 1;
    auto small_item = [&](const ph_recon_item &it) {
        const int rows_a = recon_a_rows(it.n_slow);
        const long long blocks = (it.n_fast + rows_a - 1) / rows_a;
        const int nb = std::min(it.slices, slice_batch(ctx, it.n_fast, it.n_slow, it.slices, kLaneBatchBytes));
        const int grp = recon_group(nb, (int)blocks, recon_a_chain(it.n_slow));
        return blocks * ((nb + grp - 1) / grp) < 4LL * sms;
    };
    std::map<std::tuple<int, int, int>, std::vector<int>> classes;
    for (int i = 0; i < count; ++i)
        classes[{items[i].n_fast, items[i].n_slow, items[i].hologram != nullptr ? 1 : 0}].push_back(i);
    std::vector<std::vector<int>> groups;
    for (auto &kv : classes) {
        auto &v = kv.second;
        std::stable_sort(v.begin(), v.end(), [&](int a, int c) { return items[a].slices > items[c].slices; });
        const int nx = std::get<0>(kv.first), ny = std::get<1>(kv.first);
        const bool tc = effective_form(ctx, nx, ny) != PH_FORM_FP32;
        for (size_t k = 0; k < v.size();) {
            const size_t ib = group_item_bytes(ctx, nx, ny, items[v[k]].slices);
            const bool alone = tc || !small_item(items[v[k]]);
            const size_t gmax = alone ? 1 : std::max<size_t>(1, std::min<size_t>(kMaxItems, kGroupBytes / ib));
            const size_t n = std::min(gmax, v.size() - k);
            groups.emplace_back(v.begin() + k, v.begin() + k + n);
            k += n;
        }
    }
    const int ngroups = (int)groups.size();
    lanes = std::max(1, std::min(lanes, std::max(ngroups, 1)));
    auto *b = new ph_batch();
    b->ctx = ctx;
    b->items.assign(items, items + count);
    b->lanes = lanes;
    // longest-processing-time assignment of the groups to lanes (work = pixels x slices)
    std::vector<int> group_lane(ngroups, 0), gorder(ngroups);
    {
        auto work = [&](int g) {
            double w = 0.0;
            for (int i : groups[g]) w += (double)items[i].n_fast * items[i].n_slow * items[i].slices;
            return w;
        };
        for (int g = 0; g < ngroups; ++g) gorder[g] = g;
        std::stable_sort(gorder.begin(), gorder.end(), [&](int a, int c) { return work(a) > work(c); });
        std::vector<double> load(lanes, 0.0);
        for (int g : gorder) {
            const int l = (int)(std::min_element(load.begin(), load.end()) - load.begin());
            group_lane[g] = l;
            load[l] += work(g);
        }
    }
    b->lane_of.assign(count, 0);
    for (int g = 0; g < ngroups; ++g)
        for (int i : groups[g]) b->lane_of[i] = group_lane[g];
    // per-lane scratch: the largest group among the lane's groups
    auto group_bytes = [&](int g) {
        const ph_recon_item &f = items[groups[g][0]];
        return groups[g].size() * group_item_bytes(ctx, f.n_fast, f.n_slow, f.slices);
    };
    std::vector<size_t> lane_bytes(lanes, 0), lane_off(lanes, 0);
    for (int g = 0; g < ngroups; ++g) lane_bytes[group_lane[g]] = std::max(lane_bytes[group_lane[g]], group_bytes(g));
    size_t total = 0;
    for (int l = 0; l < lanes; ++l) {
        lane_off[l] = total;
        total += (lane_bytes[l] + kAlign - 1) / kAlign * kAlign;
    }
    int st = PH_OK;
    std::vector<cudaStream_t> ls(lanes, nullptr);
    std::vector<cudaEvent_t> join(lanes, nullptr);
    cudaEvent_t fork = nullptr;
    auto fail = [&](int code) {
        for (auto x : ls) if (x) cudaStreamDestroy(x);
        for (auto e : join) if (e) cudaEventDestroy(e);
        if (fork) cudaEventDestroy(fork);
        if (b->scratch) cudaFree(b->scratch);
        delete b;
        cudaGetLastError();
        return code;
    };
    if (ctx->budget && total + ctx->scratch_bytes > ctx->budget) {
        set_err(ctx, "batch scratch of %zu bytes exceeds the context's HBM budget of %zu bytes", total, ctx->budget);
        return fail(PH_ERR_OOM);
    }
    if (total > 0 && cudaMalloc(&b->scratch, total) != cudaSuccess) {
        set_err(ctx, "cudaMalloc of %zu bytes of batch scratch failed", total);
        return fail(PH_ERR_OOM);
    }
    b->scratch_bytes = total;
    for (int i = 0; i < count; ++i) {   // twiddle tables exist before the capture
        const float2 *tw = nullptr;
        if ((st = get_twiddles(ctx, items[i].n_fast, nullptr, &tw)) != PH_OK) return fail(st);
        if ((st = get_twiddles(ctx, items[i].n_slow, nullptr, &tw)) != PH_OK) return fail(st);
    }
    for (int l = 0; l < lanes; ++l) {
        if (cudaStreamCreateWithFlags(&ls[l], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&join[l], cudaEventDisableTiming) != cudaSuccess) {
            set_err(ctx, "could not create the batch lanes");
            return fail(PH_ERR_CUDA);
        }
    }
    if (cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess) return fail(PH_ERR_CUDA);
    // record: capture stream -> fork to the lanes -> each lane's items in turn -> join
    cudaStream_t cs = ctx->capture_stream;
    const int64_t l0 = ctx->launches.load();
    if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return fail(PH_ERR_CUDA);
    cudaEventRecord(fork, cs);
    for (int l = 0; l < lanes && st == PH_OK; ++l) {
        cudaStreamWaitEvent(ls[l], fork, 0);
        char *base = static_cast<char *>(b->scratch) + lane_off[l];
        for (int g = 0; g < ngroups && st == PH_OK; ++g) {
            if (group_lane[g] != l) continue;
            if (groups[g].size() > 1) {
                std::vector<const ph_recon_item *> its;
                for (int i : groups[g]) its.push_back(&items[i]);
                st = issue_recon_group(ctx, its, base, ls[l]);
                continue;
            }
            const ph_recon_item &it = items[groups[g][0]];
            const int nx = it.n_fast, ny = it.n_slow;
            const ReconLayout L = recon_layout(ctx, nx, ny, ny, nx, it.slices, kLaneBatchBytes);
            const float2 *tw_x = ctx->tw[nx], *tw_y = ctx->tw[ny];
            auto *state = reinterpret_cast<float4 *>(base + L.state);
            auto *p64 = reinterpret_cast<unsigned long long *>(base + L.p64);
            auto *t = reinterpret_cast<float2 *>(base + L.t);
            st = issue_spectrum(ctx, static_cast<const float2 *>(it.wavefront), static_cast<const float2 *>(it.tf_front),
                                static_cast<const float2 *>(it.tf_dz), nx, ny, false, nx, ny,
                                reinterpret_cast<float2 *>(base + L.a1), state, tw_x, tw_y,
                                reinterpret_cast<double *>(base + L.acc), reinterpret_cast<float2 *>(base + L.mean),
                                ls[l], it.hologram);
            if (st != PH_OK) break;
            if (cudaMemsetAsync(p64, 0xff, sizeof(unsigned long long) * nx * ny, ls[l]) != cudaSuccess) {
                st = PH_ERR_CUDA;
                break;
            }
            st = issue_recon_slices(ctx, RK_PROJ, it.proj, it.argmin, nullptr, PH_F32, nx, ny, nx, ny, 0, 0,
                                    it.slices, L.batch, state, t, p64, tw_x, tw_y, true, ls[l]);
        }
        cudaEventRecord(join[l], ls[l]);
        cudaStreamWaitEvent(cs, join[l], 0);
    }
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(cs, &g);
    b->kernels = ctx->launches.load() - l0;
    ctx->launches = l0;
    if (st != PH_OK || ec != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        if (st == PH_OK) st = cuda_status(ctx, ec, "cudaStreamEndCapture");
        return fail(st);
    }
    const cudaError_t ei = cudaGraphInstantiate(&b->exec, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
        st = cuda_status(ctx, ei, "cudaGraphInstantiate");
        return fail(st);
    }
    for (auto x : ls) cudaStreamDestroy(x);
    for (auto e : join) cudaEventDestroy(e);
    cudaEventDestroy(fork);
    *out = b;
    PH_LEAVE(ctx);
}

int32_t ph_batch_run(ph_batch *batch, void *stream) {
    if (batch == nullptr) return PH_ERR_INVALID;
    ph_ctx *ctx = batch->ctx;
    PH_ENTER(ctx, stream);
    if (batch->exec) {
        PH_CUDA(cudaGraphLaunch(batch->exec, s), "cudaGraphLaunch");
        ctx->launches += batch->kernels;
    }
    PH_LEAVE(ctx);
}

size_t ph_batch_scratch_bytes(const ph_batch *batch) { return batch ? batch->scratch_bytes : 0; }

void ph_batch_destroy(ph_batch *batch) {
    if (batch == nullptr) return;
    {
        std::lock_guard<std::mutex> lk(batch->ctx->mu);
        DeviceGuard g(batch->ctx->device);
        cudaDeviceSynchronize();
        if (batch->exec) cudaGraphExecDestroy(batch->exec);
        if (batch->scratch) cudaFree(batch->scratch);
        cudaGetLastError();
    }
    delete batch;
}

// ---- serving: a block of the pool per request, admitted in arrival order
namespace {

// Bytes of one request's block: the reconstruction scratch (slice batches of
// at most kLaneBatchBytes), the hologram made by the device ingest, the
// transfer builder's square-root plane and the ingest's sum.
size_t serve_request_bytes(ph_ctx *ctx, int nx, int ny, int slices, ReconLayout *out = nullptr) {
    const ReconLayout L = recon_layout(ctx, nx, ny, ny, nx, slices, kLaneBatchBytes);
    if (out) *out = L;
    const size_t plane = ((size_t)nx * ny * sizeof(float) + kAlign - 1) / kAlign * kAlign;
    return (L.total + kAlign - 1) / kAlign * kAlign + 2 * plane + kAlign;
}

bool pool_alloc(ph_server *srv, size_t bytes, size_t *off) {
    for (auto it = srv->free_blocks.begin(); it != srv->free_blocks.end(); ++it) {
        if (it->second >= bytes) {
            *off = it->first;
            const size_t rest = it->second - bytes;
            const size_t next = it->first + bytes;
            srv->free_blocks.erase(it);
            if (rest) srv->free_blocks[next] = rest;
            srv->used += bytes;
            srv->peak = std::max(srv->peak, srv->used);
            return true;
        }
    }
    return false;
}

void pool_free(ph_server *srv, size_t off, size_t bytes) {
    srv->used -= bytes;
    auto it = srv->free_blocks.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != srv->free_blocks.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        srv->free_blocks.erase(nx);
    }
    if (it != srv->free_blocks.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            srv->free_blocks.erase(it);
        }
    }
}

// Gives back the slot and block of every request whose completion callback has run.
void serve_harvest(ph_server *srv) {
    std::vector<ph_serve_ticket *> done;
    {
        std::lock_guard<std::mutex> lk(srv->cmu);
        done.swap(srv->completed);
    }
    for (auto *t : done) {
        if (t->harvested) continue;
        if (t->bytes > 0) pool_free(srv, t->off, t->bytes);
        if (srv->slot_job[t->slot] == t) srv->slot_job[t->slot] = nullptr;
        t->harvested = true;
    }
}

// Same-shape requests with the same optics: one group, one launch of each pass.
bool serve_same_group(const ph_serve_request &a, const ph_serve_request &b) {
    return a.frame == nullptr && b.frame == nullptr && a.n_fast == b.n_fast && a.n_slow == b.n_slow &&
           a.slices == b.slices && a.z0 == b.z0 && a.dz == b.dz && a.wavlen == b.wavlen && a.dx == b.dx;
}

// Bytes of a group of g requests' block: their reconstruction slots and the
// transfer builder's plane.
size_t serve_group_bytes(ph_ctx *ctx, int nx, int ny, int slices, int g) {
    const size_t plane = ((size_t)nx * ny * sizeof(float) + kAlign - 1) / kAlign * kAlign;
    return (size_t)g * group_item_bytes(ctx, nx, ny, slices) + plane + kAlign;
}

// Issues an admitted group (leader + members) on the leader's slot.
int serve_issue_group(ph_server *srv, ph_serve_ticket *lead) {
    ph_ctx *ctx = srv->ctx;
    const ph_serve_request &rq = lead->req;
    const int nx = rq.n_fast, ny = rq.n_slow;
    cudaStream_t ls = srv->streams[lead->slot];
    std::vector<ph_serve_ticket *> all{lead};
    all.insert(all.end(), lead->members.begin(), lead->members.end());
    for (auto *m : all) PH_CUDA(cudaStreamWaitEvent(ls, m->submitted, 0), "cudaStreamWaitEvent");
    char *base = static_cast<char *>(srv->pool) + lead->off;
    float *dsqr = reinterpret_cast<float *>(base + all.size() * group_item_bytes(ctx, nx, ny, rq.slices));
    for (int n : {nx, ny}) {
        if (ctx->tw.find(n) == ctx->tw.end()) {
            const float2 *tw = nullptr;
            PH_TRY(get_twiddles(ctx, n, ls, &tw));
            PH_CUDA(cudaStreamSynchronize(ls), "cudaStreamSynchronize");
        }
    }
    const float2 *hf = nullptr, *hdz = nullptr;
    ph_serve_tf *ef = nullptr, *ed = nullptr;
    PH_TRY(serve_transfer(srv, ls, dsqr, nx, ny, rq.z0, rq.wavlen, rq.dx, &hf, &ef));
    PH_TRY(serve_transfer(srv, ls, dsqr, nx, ny, rq.dz, rq.wavlen, rq.dx, &hdz, &ed));
    std::vector<ph_recon_item> items(all.size());
    std::vector<const ph_recon_item *> its;
    for (size_t i = 0; i < all.size(); ++i) {
        const ph_serve_request &r = all[i]->req;
        items[i] = ph_recon_item{r.hologram, nullptr, hf, hdz, r.proj, r.argmin, nx, ny, r.slices};
        its.push_back(&items[i]);
    }
    PH_TRY(issue_recon_group(ctx, its, base, ls));
    cudaEventRecord(ef->last_use, ls);
    cudaEventRecord(ed->last_use, ls);
    PH_CUDA(cudaLaunchHostFunc(ls, serve_done, lead), "cudaLaunchHostFunc");
    for (auto *m : all) PH_CUDA(cudaEventRecord(m->ev, ls), "cudaEventRecord");
    return PH_OK;
}

// Issues one admitted request on its slot's stream.
int serve_issue(ph_server *srv, ph_serve_ticket *t) {
    ph_ctx *ctx = srv->ctx;
    const ph_serve_request *req = &t->req;
    const int nx = req->n_fast, ny = req->n_slow;
    cudaStream_t ls = srv->streams[t->slot];
    PH_CUDA(cudaStreamWaitEvent(ls, t->submitted, 0), "cudaStreamWaitEvent");
    ReconLayout L{};
    serve_request_bytes(ctx, nx, ny, req->slices, &L);
    char *base = static_cast<char *>(srv->pool) + t->off;
    const size_t plane = ((size_t)nx * ny * sizeof(float) + kAlign - 1) / kAlign * kAlign;
    const size_t recon_end = (L.total + kAlign - 1) / kAlign * kAlign;
    float *holo_buf = reinterpret_cast<float *>(base + recon_end);
    float *dsqr = reinterpret_cast<float *>(base + recon_end + plane);
    double *acc = reinterpret_cast<double *>(base + recon_end + 2 * plane);
    for (int n : {nx, ny}) {   // a new twiddle table is complete before any slot reads it
        if (ctx->tw.find(n) == ctx->tw.end()) {
            const float2 *tw = nullptr;
            PH_TRY(get_twiddles(ctx, n, ls, &tw));
            PH_CUDA(cudaStreamSynchronize(ls), "cudaStreamSynchronize");
        }
    }
    const float2 *tw_x = ctx->tw[nx], *tw_y = ctx->tw[ny];
    const float2 *hf = nullptr, *hdz = nullptr;
    ph_serve_tf *ef = nullptr, *ed = nullptr;
    PH_TRY(serve_transfer(srv, ls, dsqr, nx, ny, req->z0, req->wavlen, req->dx, &hf, &ef));
    PH_TRY(serve_transfer(srv, ls, dsqr, nx, ny, req->dz, req->wavlen, req->dx, &hdz, &ed));
    const float *holo = req->hologram;
    if (req->frame != nullptr) {   // device ingest: decode, background, mean padding
        const int fr = req->frame_n_fast, fc = req->frame_n_slow;
        const bool pad = fr != nx || fc != ny;
        float *img = pad ? reinterpret_cast<float *>(base + L.t) : holo_buf;   // T is free until the passes
        PH_CUDA(cudaMemsetAsync(acc, 0, sizeof(double), ls), "cudaMemsetAsync");
        dim3 b(32, 8), g((fr + 31) / 32, (fc + 31) / 32);
        k_ingest_u8<<<g, b, 0, ls>>>(img, req->frame, fr, fc, req->frame_pitch, req->frame_channels, req->frame_flip,
                                     req->background, req->background_offset, pad ? acc : nullptr);
        PH_TRY(launched(ctx, cudaGetLastError(), "ingest"));
        if (pad) {
            dim3 bp(32, 8);
            k_pad_mean_fill<<<grid2d(nx, ny, bp), bp, 0, ls>>>(holo_buf, img, acc, (double)fr * fc, fr, fc, nx,
                                                               nx / 2 - fr / 2, ny / 2 - fc / 2);
            PH_TRY(launched(ctx, cudaGetLastError(), "ingest padding"));
        }
        holo = holo_buf;
    }
    auto *state = reinterpret_cast<float4 *>(base + L.state);
    auto *p64 = reinterpret_cast<unsigned long long *>(base + L.p64);
    PH_TRY(issue_spectrum(ctx, nullptr, hf, hdz, nx, ny, false, nx, ny, reinterpret_cast<float2 *>(base + L.a1), state,
                          tw_x, tw_y, reinterpret_cast<double *>(base + L.acc), reinterpret_cast<float2 *>(base + L.mean),
                          ls, holo));
    PH_CUDA(cudaMemsetAsync(p64, 0xff, sizeof(unsigned long long) * nx * ny, ls), "cudaMemsetAsync");
    PH_TRY(issue_recon_slices(ctx, RK_PROJ, req->proj, req->argmin, nullptr, PH_F32, nx, ny, nx, ny, 0, 0,
                              req->slices, L.batch, state, reinterpret_cast<float2 *>(base + L.t), p64, tw_x, tw_y,
                              true, ls));
    cudaEventRecord(ef->last_use, ls);
    cudaEventRecord(ed->last_use, ls);
    PH_CUDA(cudaLaunchHostFunc(ls, serve_done, t), "cudaLaunchHostFunc");
    PH_CUDA(cudaEventRecord(t->ev, ls), "cudaEventRecord");
    return PH_OK;
}

// Harvests completions, then admits queued requests in arrival order while a
// slot is free and the pool holds the next request's block.  The caller holds
// srv->mu and ctx->mu.
int serve_dispatch(ph_server *srv) {
    serve_harvest(srv);
    while (!srv->pending.empty()) {
        ph_serve_ticket *t = srv->pending.front();
        int slot = -1;
        for (int l = 0; l < srv->lanes; ++l)
            if (srv->slot_job[l] == nullptr) { slot = l; break; }
        if (slot < 0) return PH_OK;
        // Requests of the same shape and optics queued right behind it share its
        // launches (their projection runs the FP32 row pass, which has a grouped form).
        int g = 1;
        while (g < (int)srv->pending.size() && g < kMaxItems && serve_same_group(t->req, srv->pending[g]->req)) ++g;
        if (g > 1 && effective_form(srv->ctx, t->req.n_fast, t->req.n_slow) != PH_FORM_FP32) g = 1;
        size_t off = 0;
        while (g > 1) {
            const size_t gb = serve_group_bytes(srv->ctx, t->req.n_fast, t->req.n_slow, t->req.slices, g);
            if (gb <= srv->pool_bytes && pool_alloc(srv, gb, &off)) {
                t->bytes = gb;
                break;
            }
            --g;
        }
        if (g > 1) {
            srv->pending.pop_front();
            t->members.clear();
            for (int i = 1; i < g; ++i) {
                ph_serve_ticket *m = srv->pending.front();
                srv->pending.pop_front();
                m->slot = slot;
                m->off = off;
                m->bytes = 0;
                m->t_admit = now_s();
                t->members.push_back(m);
            }
            t->slot = slot;
            t->off = off;
            t->t_admit = now_s();
            srv->slot_job[slot] = t;
            srv->admitted_total += g;
            srv->grouped_total += g;
            const int st = serve_issue_group(srv, t);
            if (st != PH_OK) {
                pool_free(srv, t->off, t->bytes);
                srv->slot_job[slot] = nullptr;
                for (auto *m : t->members) {
                    m->harvested = true;
                    m->done.store(-1, std::memory_order_release);
                }
                t->members.clear();
                t->harvested = true;
                t->done.store(-1, std::memory_order_release);
                return st;
            }
            continue;
        }
        if (!pool_alloc(srv, t->bytes, &off)) return PH_OK;   // waits for memory to free up
        srv->pending.pop_front();
        t->slot = slot;
        t->off = off;
        t->t_admit = now_s();
        srv->slot_job[slot] = t;
        ++srv->admitted_total;
        const int st = serve_issue(srv, t);
        if (st != PH_OK) {
            // the request failed to issue: give its block and slot back and report it
            pool_free(srv, t->off, t->bytes);
            srv->slot_job[slot] = nullptr;
            t->harvested = true;
            t->done.store(-1, std::memory_order_release);
            return st;
        }
    }
    return PH_OK;
}

}  // namespace

int32_t ph_serve_create(ph_ctx *ctx, int32_t lanes, int32_t max_n_fast, int32_t max_n_slow, int32_t max_slices,
                        int32_t tf_cache_entries, size_t scratch_budget_bytes, ph_server **out) {
    PH_ENTER(ctx, nullptr);
    PH_NONNULL(out, "out");
    *out = nullptr;
    if (lanes < 1 || lanes > 16) { set_err(ctx, "lanes must be in 1..16. Got %d.", lanes); return PH_ERR_INVALID; }
    if (max_slices < 1) { set_err(ctx, "max_slices must be >= 1. Got %d.", max_slices); return PH_ERR_SIZE; }
    if (tf_cache_entries < 2) { set_err(ctx, "the transfer cache needs at least 2 entries"); return PH_ERR_INVALID; }
    PH_TRY(check_len(ctx, max_n_fast, max_n_slow));
    const size_t largest = serve_request_bytes(ctx, max_n_fast, max_n_slow, max_slices);
    const size_t total = scratch_budget_bytes ? scratch_budget_bytes : largest * lanes;
    if (total < largest) {
        set_err(ctx, "a scratch budget of %zu bytes holds no request of the largest size (%zu bytes)", total, largest);
        return PH_ERR_OOM;
    }
    if (ctx->budget && total + ctx->scratch_bytes > ctx->budget) {
        set_err(ctx, "server scratch of %zu bytes exceeds the context's HBM budget of %zu bytes", total, ctx->budget);
        return PH_ERR_OOM;
    }
    auto *srv = new ph_server();
    srv->ctx = ctx;
    srv->lanes = lanes;
    srv->max_nx = max_n_fast;
    srv->max_ny = max_n_slow;
    srv->max_slices = max_slices;
    srv->tf_cap = tf_cache_entries;
    srv->pool_bytes = total;
    auto fail = [&](int code) {
        for (auto x : srv->streams) if (x) cudaStreamDestroy(x);
        if (srv->pool) cudaFree(srv->pool);
        delete srv;
        cudaGetLastError();
        return code;
    };
    if (cudaMalloc(&srv->pool, total) != cudaSuccess) {
        set_err(ctx, "cudaMalloc of %zu bytes of server scratch failed", total);
        return fail(PH_ERR_OOM);
    }
    srv->free_blocks[0] = total;
    srv->streams.assign(lanes, nullptr);
    srv->slot_job.assign(lanes, nullptr);
    for (int l = 0; l < lanes; ++l) {
        if (cudaStreamCreateWithFlags(&srv->streams[l], cudaStreamNonBlocking) != cudaSuccess) {
            set_err(ctx, "could not create the server's streams");
            return fail(PH_ERR_CUDA);
        }
    }
    *out = srv;
    PH_LEAVE(ctx);
}

int32_t ph_serve_submit(ph_server *srv, const ph_serve_request *req, int64_t *ticket, void *stream) {
    if (srv == nullptr || req == nullptr || ticket == nullptr) return PH_ERR_INVALID;
    ph_ctx *ctx = srv->ctx;
    std::lock_guard<std::mutex> slk(srv->mu);
    std::lock_guard<std::mutex> clk(ctx->mu);
    DeviceGuard dg(ctx->device);
    const int nx = req->n_fast, ny = req->n_slow;
    if (req->frame == nullptr) PH_NONNULL(req->hologram, "hologram");
    if (req->proj == nullptr && req->argmin == nullptr) { set_err(ctx, "proj and argmin are both NULL"); return PH_ERR_INVALID; }
    if (req->slices < 1) { set_err(ctx, "slices must be >= 1. Got %d.", req->slices); return PH_ERR_SIZE; }
    PH_TRY(check_len(ctx, nx, ny));
    if (req->frame != nullptr) {
        const int fr = req->frame_n_fast, fc = req->frame_n_slow;
        if (fr < 1 || fc < 1 || fr > nx || fc > ny || (req->frame_channels != 1 && req->frame_channels != 3) ||
            req->frame_pitch < fc * req->frame_channels) {
            set_err(ctx, "frame %d x %d (pitch %d, %d channels) does not fit the request %d x %d", fr, fc,
                    req->frame_pitch, req->frame_channels, nx, ny);
            return PH_ERR_SIZE;
        }
    }
    if ((size_t)nx * ny > (size_t)srv->max_nx * srv->max_ny || req->slices > srv->max_slices) {
        set_err(ctx, "request %d x %d x %d exceeds the server's maximum %d x %d x %d", nx, ny, req->slices,
                srv->max_nx, srv->max_ny, srv->max_slices);
        return PH_ERR_SIZE;
    }
    auto *t = new ph_serve_ticket();
    t->req = *req;
    t->srv = srv;
    t->bytes = serve_request_bytes(ctx, nx, ny, req->slices);
    if (t->bytes > srv->pool_bytes) {
        delete t;
        set_err(ctx, "request needs %zu bytes of scratch; the server holds %zu", t->bytes, srv->pool_bytes);
        return PH_ERR_SIZE;
    }
    t->submitted = serve_event(srv);
    t->ev = serve_event(srv);
    if (t->submitted == nullptr || t->ev == nullptr) {
        if (t->submitted) srv->event_pool.push_back(t->submitted);
        if (t->ev) srv->event_pool.push_back(t->ev);
        delete t;
        set_err(ctx, "cudaEventCreate failed");
        return PH_ERR_CUDA;
    }
    t->t_submit = now_s();
    // the request runs after the work already queued on the caller's stream (which wrote its inputs)
    PH_CUDA(cudaEventRecord(t->submitted, static_cast<cudaStream_t>(stream)), "cudaEventRecord");
    t->id = srv->next_ticket++;
    srv->tickets[t->id] = t;
    srv->pending.push_back(t);
    *ticket = t->id;
    const int st = serve_dispatch(srv);
    if (t->slot < 0 && t->done.load() == 0) ++srv->waited_total;   // queued for a slot or for memory
    return st;
}

int32_t ph_serve_poll(ph_server *srv, int64_t ticket, int32_t wait, double *latency_ms) {
    if (srv == nullptr) return PH_ERR_INVALID;
    ph_ctx *ctx = srv->ctx;
    std::unique_lock<std::mutex> lk(srv->mu);
    auto it = srv->tickets.find(ticket);
    if (it == srv->tickets.end()) {
        std::lock_guard<std::mutex> clk(ctx->mu);
        set_err(ctx, "unknown ticket %lld", (long long)ticket);
        return PH_ERR_INVALID;
    }
    ph_serve_ticket *t = it->second;
    for (;;) {
        {
            std::lock_guard<std::mutex> clk(ctx->mu);
            DeviceGuard dg(ctx->device);
            PH_TRY(serve_dispatch(srv));
        }
        if (t->done.load(std::memory_order_acquire) != 0) break;
        if (!wait) return PH_PENDING;
        // wait for this request if it runs, else for the oldest running one (which frees a slot and memory)
        cudaEvent_t ev = nullptr;
        if (t->slot >= 0) {
            ev = t->ev;
        } else {
            double oldest = 1e300;
            for (auto *j : srv->slot_job)
                if (j != nullptr && j->t_admit < oldest) { oldest = j->t_admit; ev = j->ev; }
        }
        if (ev == nullptr) {
            std::lock_guard<std::mutex> clk(ctx->mu);
            set_err(ctx, "ticket %lld is queued but no request runs", (long long)ticket);
            return PH_ERR_INVALID;
        }
        lk.unlock();
        cudaError_t e;
        {
            DeviceGuard dg(ctx->device);
            e = cudaEventSynchronize(ev);   // recorded after the completion callback
        }
        lk.lock();
        if (e != cudaSuccess) {
            std::lock_guard<std::mutex> clk(ctx->mu);
            return cuda_status(ctx, e, "cudaEventSynchronize");
        }
    }
    const int outcome = t->done.load(std::memory_order_acquire);
    if (latency_ms) *latency_ms = (t->t_done - t->t_submit) * 1e3;
    srv->event_pool.push_back(t->ev);
    srv->event_pool.push_back(t->submitted);
    srv->tickets.erase(ticket);
    delete t;
    if (outcome < 0) {
        std::lock_guard<std::mutex> clk(ctx->mu);
        set_err(ctx, "request %lld could not be issued", (long long)ticket);
        return PH_ERR_CUDA;
    }
    return PH_OK;
}

int32_t ph_serve_stats(ph_server *srv, int64_t *queued, int64_t *running, size_t *bytes_in_use, size_t *bytes_peak,
                       int64_t *waited, int64_t *grouped) {
    if (srv == nullptr) return PH_ERR_INVALID;
    std::lock_guard<std::mutex> lk(srv->mu);
    {
        std::lock_guard<std::mutex> clk(srv->ctx->mu);
        DeviceGuard dg(srv->ctx->device);
        PH_TRY(serve_dispatch(srv));
    }
    int64_t run = 0;
    for (auto *j : srv->slot_job) run += j != nullptr;
    if (queued) *queued = (int64_t)srv->pending.size();
    if (running) *running = run;
    if (bytes_in_use) *bytes_in_use = srv->used;
    if (bytes_peak) *bytes_peak = srv->peak;
    if (waited) *waited = srv->waited_total;
    if (grouped) *grouped = srv->grouped_total;
    return PH_OK;
}

void ph_serve_destroy(ph_server *srv) {
    if (srv == nullptr) return;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        DeviceGuard dg(srv->ctx->device);
        // every queued request is admitted and finished before the memory goes
        for (;;) {
            int st;
            {
                std::lock_guard<std::mutex> clk(srv->ctx->mu);
                st = serve_dispatch(srv);
            }
            for (auto x : srv->streams) cudaStreamSynchronize(x);   // (the completion callbacks have run)
            if (st != PH_OK || srv->pending.empty()) break;
        }
        for (auto &kv : srv->tickets) {
            srv->event_pool.push_back(kv.second->ev);
            srv->event_pool.push_back(kv.second->submitted);
            delete kv.second;
        }
        for (auto e : srv->event_pool) cudaEventDestroy(e);
        for (auto &kv : srv->tfs) {
            cudaFree(kv.second.buf);
            cudaEventDestroy(kv.second.ready);
            cudaEventDestroy(kv.second.last_use);
        }
        for (auto x : srv->streams) cudaStreamDestroy(x);
        if (srv->pool) cudaFree(srv->pool);
        cudaGetLastError();
    }
    delete srv;
}

int32_t ph_reconst_xyproj_lpf(ph_ctx *ctx, float *proj, int32_t *argmin, const void *wf, const void *tf_front,
                              const void *tf_dz, const float *lpf, int32_t n_fast, int32_t n_slow, int32_t slices,
                              void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(wf, "wavefront");
    PH_NONNULL(tf_front, "transfer_front");
    PH_NONNULL(tf_dz, "transfer_dz");
    PH_NONNULL(lpf, "lpf");
    if (proj == nullptr && argmin == nullptr) { set_err(ctx, "proj and argmin are both NULL"); return PH_ERR_INVALID; }
    if (slices < 1) { set_err(ctx, "slices must be >= 1. Got %d.", slices); return PH_ERR_SIZE; }
    PH_TRY(reconstruct(ctx, RK_PROJ, proj, argmin, nullptr, PH_F32, static_cast<const float2 *>(wf),
                       static_cast<const float2 *>(tf_front), static_cast<const float2 *>(tf_dz), n_fast, n_slow,
                       slices, s, lpf));
    PH_LEAVE(ctx);
}

int32_t ph_reconst_vol(ph_ctx *ctx, void *vol, int32_t vol_dtype, float *proj, const void *wf, const void *tf_front,
                       const void *tf_dz, int32_t n_fast, int32_t n_slow, int32_t slices, void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(vol, "vol");
    PH_NONNULL(wf, "wavefront");
    PH_NONNULL(tf_front, "transfer_front");
    PH_NONNULL(tf_dz, "transfer_dz");
    if (slices < 1) { set_err(ctx, "slices must be >= 1. Got %d.", slices); return PH_ERR_SIZE; }
    if (vol_dtype < PH_N0F8 || vol_dtype > PH_C64) {
        set_err(ctx, "return_type must be Subtype of AbstractFloat or N0f8. Got dtype code %d", vol_dtype);
        return PH_ERR_DTYPE;
    }
    if (vol_dtype == PH_C64 && proj != nullptr) {
        set_err(ctx, "a complex volume has no xy projection");
        return PH_ERR_INVALID;
    }
    PH_TRY(reconstruct(ctx, vol_dtype == PH_C64 ? RK_CVOL : RK_VOL, proj, nullptr, vol, vol_dtype,
                       static_cast<const float2 *>(wf), static_cast<const float2 *>(tf_front),
                       static_cast<const float2 *>(tf_dz), n_fast, n_slow, slices, s));
    PH_LEAVE(ctx);
}

int32_t ph_reconst_subvolumes(ph_ctx *ctx, uint8_t *out, int64_t *offsets_host, const int64_t *boxes_host,
                              int32_t count, const void *wf, const void *tf_front, const void *tf_dz, int32_t n_fast,
                              int32_t n_slow, int32_t slices, void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(offsets_host, "offsets");
    if (count < 0 || (count > 0 && boxes_host == nullptr)) { set_err(ctx, "boxes must hold count >= 0 records"); return PH_ERR_INVALID; }
    if (slices < 1) { set_err(ctx, "slices must be >= 1. Got %d.", slices); return PH_ERR_SIZE; }
    PH_TRY(check_len(ctx, n_fast, n_slow));
    std::vector<SubBox> bx((size_t)count);
    int64_t off = 0;
    int zlo = slices, zhi = -1;
    for (int i = 0; i < count; ++i) {
        const int64_t *v = boxes_host + 6 * (size_t)i;   // x_min y_min z_min x_max y_max z_max (x slow, y fast)
        if (!(1 <= v[0] && v[0] <= v[3] && v[3] <= n_slow && 1 <= v[1] && v[1] <= v[4] && v[4] <= n_fast &&
              1 <= v[2] && v[2] <= v[5] && v[5] <= slices)) {
            set_err(ctx, "box %d (%lld, %lld, %lld, %lld, %lld, %lld) lies outside the (%d, %d, %d) volume", i,
                    (long long)v[0], (long long)v[1], (long long)v[2], (long long)v[3], (long long)v[4],
                    (long long)v[5], n_fast, n_slow, slices);
            return PH_ERR_SIZE;
        }
        SubBox &b = bx[i];
        b.fx0 = (int)v[1] - 1; b.fx1 = (int)v[4] - 1;
        b.sy0 = (int)v[0] - 1; b.sy1 = (int)v[3] - 1;
        b.z0 = (int)v[2] - 1; b.z1 = (int)v[5] - 1;
        b.nxb = b.fx1 - b.fx0 + 1;
        b.nyb = b.sy1 - b.sy0 + 1;
        b.off = off;
        offsets_host[i] = off;
        off += (int64_t)b.nxb * b.nyb * (b.z1 - b.z0 + 1);
        zlo = std::min(zlo, b.z0);
        zhi = std::max(zhi, b.z1);
    }
    offsets_host[count] = off;
    if (out == nullptr || count == 0) PH_LEAVE(ctx);
    PH_NONNULL(wf, "wavefront");
    PH_NONNULL(tf_front, "transfer_front");
    PH_NONNULL(tf_dz, "transfer_dz");
    // boxes of each slow row (CSR)
    std::vector<int> row_ptr((size_t)n_slow + 1, 0), row_box;
    for (const SubBox &b : bx)
        for (int y = b.sy0; y <= b.sy1; ++y) ++row_ptr[y + 1];
    for (int y = 0; y < n_slow; ++y) row_ptr[y + 1] += row_ptr[y];
    row_box.resize((size_t)row_ptr[n_slow]);
    {
        std::vector<int> fill(row_ptr.begin(), row_ptr.end() - 1);
        for (int i = 0; i < count; ++i)
            for (int y = bx[i].sy0; y <= bx[i].sy1; ++y) row_box[fill[y]++] = i;
    }
    const int nz = zhi - zlo + 1;
    const int nx = n_fast, ny = n_slow;
    ReconLayout L = recon_layout(ctx, nx, ny, ny, nx, nz);
    Arena a;
    a.off = L.total;
    const size_t o_rp = a.take<int>(row_ptr.size()), o_rb = a.take<int>(std::max<size_t>(row_box.size(), 1)),
                 o_bx = a.take<SubBox>(bx.size());
    PH_TRY(ensure_scratch(ctx, a.off, s));
    PH_CUDA(cudaMemcpyAsync(at<int>(ctx, o_rp), row_ptr.data(), row_ptr.size() * sizeof(int), cudaMemcpyHostToDevice, s),
            "cudaMemcpyAsync");
    if (!row_box.empty())
        PH_CUDA(cudaMemcpyAsync(at<int>(ctx, o_rb), row_box.data(), row_box.size() * sizeof(int),
                                cudaMemcpyHostToDevice, s), "cudaMemcpyAsync");
    PH_CUDA(cudaMemcpyAsync(at<SubBox>(ctx, o_bx), bx.data(), bx.size() * sizeof(SubBox), cudaMemcpyHostToDevice, s),
            "cudaMemcpyAsync");
    const float2 *tw_x = nullptr, *tw_y = nullptr;
    PH_TRY(get_twiddles(ctx, nx, s, &tw_x));
    PH_TRY(get_twiddles(ctx, ny, s, &tw_y));
    float4 *state = at<float4>(ctx, L.state);
    PH_TRY(issue_spectrum(ctx, static_cast<const float2 *>(wf), static_cast<const float2 *>(tf_front),
                          static_cast<const float2 *>(tf_dz), nx, ny, false, nx, ny, at<float2>(ctx, L.a1), state, tw_x,
                          tw_y, at<double>(ctx, L.acc), at<float2>(ctx, L.mean), s));
    const SubArgs sub{at<int>(ctx, o_rp), at<int>(ctx, o_rb), at<SubBox>(ctx, o_bx)};
    PH_TRY(issue_recon_slices(ctx, RK_SUB, nullptr, nullptr, out, PH_N0F8, nx, ny, nx, ny, 0, 0, nz, L.batch, state,
                              at<float2>(ctx, L.t), at<unsigned long long>(ctx, L.p64), tw_x, tw_y, false, s, 0.0f,
                              zlo, &sub));
    PH_LEAVE(ctx);
}

int32_t ph_reconst_binary_vol(ph_ctx *ctx, uint8_t *vol, float threshold, float *proj, const void *wf,
                              const void *tf_front, const void *tf_dz, int32_t n_fast, int32_t n_slow, int32_t slices,
                              void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(vol, "vol");
    PH_NONNULL(wf, "wavefront");
    PH_NONNULL(tf_front, "transfer_front");
    PH_NONNULL(tf_dz, "transfer_dz");
    if (slices < 1) { set_err(ctx, "slices must be >= 1. Got %d.", slices); return PH_ERR_SIZE; }
    PH_TRY(reconstruct(ctx, RK_VOL, proj, nullptr, vol, PH_BOOL, static_cast<const float2 *>(wf),
                       static_cast<const float2 *>(tf_front), static_cast<const float2 *>(tf_dz), n_fast, n_slow,
                       slices, s, nullptr, threshold));
    PH_LEAVE(ctx);
}

int32_t ph_background_mode(ph_ctx *ctx, double *out, const uint8_t *images, int64_t count, int32_t n_fast,
                           int32_t n_slow, void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(out, "out");
    PH_NONNULL(images, "images");
    if (count < 1 || n_fast < 1 || n_slow < 1) { set_err(ctx, "need at least one image of positive size"); return PH_ERR_SIZE; }
    if (count > 65535) { set_err(ctx, "at most 65535 images per call. Got %lld.", (long long)count); return PH_ERR_TOO_LARGE; }
    const int64_t npix = (int64_t)n_fast * n_slow;
    k_background_mode<<<(unsigned)((npix + kModeThreads - 1) / kModeThreads), kModeThreads, 0, s>>>(out, images, count,
                                                                                                    npix);
    PH_TRY(launched(ctx, cudaGetLastError(), "background mode"));
    PH_LEAVE(ctx);
}

int32_t ph_background_mean(ph_ctx *ctx, double *out, const uint8_t *images, int64_t count, int32_t n_fast,
                           int32_t n_slow, void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(out, "out");
    PH_NONNULL(images, "images");
    if (count < 1 || n_fast < 1 || n_slow < 1) { set_err(ctx, "need at least one image of positive size"); return PH_ERR_SIZE; }
    const int64_t npix = (int64_t)n_fast * n_slow;
    k_background_mean<<<(unsigned)((npix + 255) / 256), 256, 0, s>>>(out, images, count, npix);
    PH_TRY(launched(ctx, cudaGetLastError(), "background mean"));
    PH_LEAVE(ctx);
}

int32_t ph_pad_with_mean(ph_ctx *ctx, float *out, const float *img, int32_t n_fast, int32_t n_slow, int32_t padsize,
                         void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(out, "out");
    PH_NONNULL(img, "img");
    if (!(padsize > n_fast && padsize > n_slow) || n_fast < 1 || n_slow < 1) {
        set_err(ctx, "Padsize should be larger than the image size. padsize: %d, img size: (%d, %d)", padsize, n_fast,
                n_slow);
        return PH_ERR_SIZE;
    }
    double *acc = reinterpret_cast<double *>(static_cast<char *>(ctx->small) + 64);
    PH_CUDA(cudaMemsetAsync(acc, 0, sizeof(double), s), "cudaMemsetAsync");
    const size_t n = (size_t)n_fast * n_slow;
    k_sum_f32<<<256, 256, 0, s>>>(img, n, acc);
    dim3 b(32, 8);
    k_pad_mean_fill<<<grid2d(padsize, padsize, b), b, 0, s>>>(out, img, acc, (double)n, n_fast, n_slow, padsize,
                                                             padsize / 2 - n_fast / 2, padsize / 2 - n_slow / 2);
    PH_TRY(launched(ctx, cudaGetLastError(), "pad with mean", 2));
    PH_LEAVE(ctx);
}

int32_t ph_reconst_vol_padded(ph_ctx *ctx, uint8_t *vol, float *proj, const void *wf, const void *tf_front,
                              const void *tf_dz, int32_t n_fast, int32_t n_slow, int32_t slices, int32_t return_dtype,
                              void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(vol, "vol");
    PH_NONNULL(wf, "wavefront");
    PH_NONNULL(tf_front, "transfer_front");
    PH_NONNULL(tf_dz, "transfer_dz");
    if (slices < 1) { set_err(ctx, "slices must be >= 1. Got %d.", slices); return PH_ERR_SIZE; }
    if (return_dtype < PH_N0F8 || return_dtype > PH_F64) {
        set_err(ctx, "return_type must be Subtype of AbstractFloat or N0f8. Got dtype code %d", return_dtype);
        return PH_ERR_DTYPE;
    }
    if (n_fast != n_slow || (n_fast & 1)) {
        set_err(ctx, "the padded reconstruction needs a square input of even size. Got (%d, %d).", n_fast, n_slow);
        return PH_ERR_SIZE;
    }
    PH_TRY(reconstruct(ctx, RK_PADDED, proj, nullptr, vol, PH_N0F8, static_cast<const float2 *>(wf),
                       static_cast<const float2 *>(tf_front), static_cast<const float2 *>(tf_dz), n_fast, n_slow,
                       slices, s));
    PH_LEAVE(ctx);
}

int32_t ph_lpf_rectangle(ph_ctx *ctx, float *out, int32_t imglen, double prop_dist, double wavlen, double pitch,
                         void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(out, "out");
    if (imglen <= 0) { set_err(ctx, "imglen must be positive"); return PH_ERR_SIZE; }
    dim3 b(32, 8);
    k_lpf_rect<<<grid2d(imglen, imglen, b), b, 0, s>>>(out, imglen, lpf_maxi(prop_dist, wavlen, imglen, pitch));
    PH_TRY(launched(ctx, cudaGetLastError(), "rectangle filter"));
    PH_LEAVE(ctx);
}

int32_t ph_lpf_super_gaussian(ph_ctx *ctx, float *out, int32_t imglen, double prop_dist, double wavlen, double pitch,
                              void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(out, "out");
    if (imglen <= 0) { set_err(ctx, "imglen must be positive"); return PH_ERR_SIZE; }
    const double maxi = lpf_maxi(prop_dist, wavlen, imglen, pitch);
    const double sigma = maxi / (imglen * pitch) / pow(2.0 * log(2.0), 1.0 / 6.0);
    dim3 b(32, 8);
    k_lpf_super_gaussian<<<grid2d(imglen, imglen, b), b, 0, s>>>(out, imglen, pitch, sigma);
    PH_TRY(launched(ctx, cudaGetLastError(), "super-Gaussian filter"));
    PH_LEAVE(ctx);
}

int32_t ph_binarize_le(ph_ctx *ctx, uint8_t *out, const float *in, int64_t n, float threshold, void *stream) {
    PH_ENTER(ctx, stream);
    PH_NONNULL(out, "out");
    PH_NONNULL(in, "in");
    if (n < 0) { set_err(ctx, "negative size"); return PH_ERR_SIZE; }
    if (n > 0) {
        PH_TRY(pass(ctx, s, "binarize", [&] {
            k_binarize_le<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(out, in, (size_t)n, threshold);
            return cudaGetLastError();
        }));
    }
    PH_LEAVE(ctx);
}

static int ccl_common(ph_ctx *ctx, uint32_t *labels, const void *img, int32_t img_dtype, int64_t rows, int64_t cols,
                      int64_t slice_rows, cudaStream_t s) {
    PH_NONNULL(labels, "labels");
    PH_NONNULL(img, "img");
    if (rows < 0 || cols < 0) { set_err(ctx, "negative size"); return PH_ERR_SIZE; }
    if ((unsigned long long)rows * (unsigned long long)cols > 4294967295ull) {
        set_err(ctx, "Image is too large. Maximum length is 2^32-1.");
        return PH_ERR_TOO_LARGE;
    }
    if (img_dtype != PH_F32 && img_dtype != PH_BOOL) {
        set_err(ctx, "labeling input must be Float32 or Bool. Got dtype code %d", img_dtype);
        return PH_ERR_DTYPE;
    }
    int64_t nl = 0;
    PH_TRY(pass(ctx, s, "ccl", [&] {
        return ccl_launch(img, img_dtype == PH_BOOL, labels, rows, cols, slice_rows, ctx->opt_loop_limit,
                          static_cast<int *>(ctx->small), s, &nl);
    }, 0));
    ctx->launches += nl;
    return PH_OK;
}

int32_t ph_ccl(ph_ctx *ctx, uint32_t *labels, const void *img, int32_t img_dtype, int64_t rows, int64_t cols,
               void *stream) {
    PH_ENTER(ctx, stream);
    PH_TRY(ccl_common(ctx, labels, img, img_dtype, rows, cols, rows, s));
    PH_LEAVE(ctx);
}

int32_t ph_ccl_batch(ph_ctx *ctx, uint32_t *labels, const void *img, int32_t img_dtype, int64_t slices, int64_t rows,
                     int64_t cols, void *stream) {
    PH_ENTER(ctx, stream);
    if (slices < 0) { set_err(ctx, "negative size"); return PH_ERR_SIZE; }
    PH_TRY(ccl_common(ctx, labels, img, img_dtype, slices * rows, cols, rows, s));
    PH_LEAVE(ctx);
}

// Roots (and optionally their bounding boxes) of labels holding `slices`
// images of rows x cols; out_host gets `per` int64 per root.  Synchronises.
static int roots_common(ph_ctx *ctx, const uint32_t *labels, int64_t slices, int64_t rows, int64_t cols, bool boxes,
                        int64_t *out_host, int64_t capacity, int64_t *count_host, cudaStream_t s) {
    PH_NONNULL(labels, "labels");
    PH_NONNULL(count_host, "count");
    if (capacity > 0) PH_NONNULL(out_host, "output");
    if (slices < 0 || rows < 0 || cols < 0) { set_err(ctx, "negative size"); return PH_ERR_SIZE; }
    *count_host = 0;
    const int64_t n = slices * rows * cols, slice_n = rows * cols;
    if (n == 0) return PH_OK;
    const int64_t nb = roots_blocks(n);
    int64_t nl = 0;
    auto layout = [&](int64_t want, size_t *oc, size_t *ot, size_t *orr, size_t *orank, size_t *obox) {
        Arena a;
        *oc = a.take<unsigned>(nb);
        *ot = a.take<unsigned long long>(1);
        *orr = a.take<long long>((size_t)std::max<int64_t>(want, 1));
        *orank = boxes ? a.take<unsigned>((size_t)n) : 0;
        *obox = boxes ? a.take<int>((size_t)std::max<int64_t>(want, 1) * 4) : 0;
        return a.off;
    };
    size_t oc, ot, orr, orank, obox;
    PH_TRY(ensure_scratch(ctx, layout(0, &oc, &ot, &orr, &orank, &obox), s));
    PH_TRY(cuda_status(ctx, roots_count_launch(labels, n, slice_n, at<unsigned>(ctx, oc),
                                               at<unsigned long long>(ctx, ot), s, &nl), "root count"));
    unsigned long long total = 0;
    int flag = 0;
    PH_CUDA(cudaMemcpyAsync(&total, at<unsigned long long>(ctx, ot), sizeof total, cudaMemcpyDeviceToHost, s),
            "copy count");
    PH_CUDA(cudaMemcpyAsync(&flag, ctx->small, sizeof flag, cudaMemcpyDeviceToHost, s), "copy flag");
    PH_CUDA(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    ctx->launches += nl;
    nl = 0;
    if (flag) {
        cudaMemsetAsync(ctx->small, 0, sizeof(int), s);
        set_err(ctx, "a labeling loop reached its iteration limit; labels are incomplete");
        return PH_ERR_TIMEOUT;
    }
    *count_host = (int64_t)total;
    const int64_t want = std::min<int64_t>((int64_t)total, capacity);
    if (want <= 0) return PH_OK;
    const size_t need = layout(boxes ? (int64_t)total : want, &oc, &ot, &orr, &orank, &obox);
    if (need > ctx->scratch_bytes) {   // growing discards the offsets: count again
        PH_TRY(ensure_scratch(ctx, need, s));
        PH_TRY(cuda_status(ctx, roots_count_launch(labels, n, slice_n, at<unsigned>(ctx, oc),
                                                   at<unsigned long long>(ctx, ot), s, &nl), "root count"));
    }
    PH_TRY(cuda_status(ctx, roots_write_launch(labels, n, slice_n, at<unsigned>(ctx, oc), at<long long>(ctx, orr),
                                               want, boxes ? at<unsigned>(ctx, orank) : nullptr, s, &nl),
                       "root write"));
    if (!boxes) {
        PH_CUDA(cudaMemcpyAsync(out_host, at<long long>(ctx, orr), sizeof(long long) * want, cudaMemcpyDeviceToHost,
                                s), "copy roots");
        PH_CUDA(cudaStreamSynchronize(s), "cudaStreamSynchronize");
        ctx->launches += nl;
        return PH_OK;
    }
    PH_TRY(cuda_status(ctx, boxes_launch(labels, slices * rows, cols, rows, at<unsigned>(ctx, orank),
                                         at<int>(ctx, obox), (int64_t)total, s, &nl), "boxes"));
    std::vector<long long> roots((size_t)want);
    std::vector<int> bx((size_t)want * 4);
    PH_CUDA(cudaMemcpyAsync(roots.data(), at<long long>(ctx, orr), sizeof(long long) * want, cudaMemcpyDeviceToHost,
                            s), "copy roots");
    PH_CUDA(cudaMemcpyAsync(bx.data(), at<int>(ctx, obox), sizeof(int) * 4 * want, cudaMemcpyDeviceToHost, s),
            "copy boxes");
    PH_CUDA(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    for (int64_t r = 0; r < want; ++r) {   // (root, x_min, y_min, x_max, y_max), 1-based; x = slow axis
        out_host[5 * r + 0] = roots[r];
        out_host[5 * r + 1] = bx[4 * r + 0] + 1;
        out_host[5 * r + 2] = bx[4 * r + 1] + 1;
        out_host[5 * r + 3] = bx[4 * r + 2] + 1;
        out_host[5 * r + 4] = bx[4 * r + 3] + 1;
    }
    ctx->launches += nl;
    return PH_OK;
}

int32_t ph_ccl_roots(ph_ctx *ctx, int64_t *roots_host, int64_t capacity, int64_t *count_host, const uint32_t *labels,
                     int64_t n, void *stream) {
    PH_ENTER(ctx, stream);
    PH_TRY(roots_common(ctx, labels, 1, 1, n, false, roots_host, capacity, count_host, s));
    PH_LEAVE(ctx);
}

int32_t ph_ccl_boxes(ph_ctx *ctx, int64_t *boxes_host, int64_t capacity, int64_t *count_host, const uint32_t *labels,
                     int64_t slices, int64_t rows, int64_t cols, void *stream) {
    PH_ENTER(ctx, stream);
    PH_TRY(roots_common(ctx, labels, slices, rows, cols, true, boxes_host, capacity, count_host, s));
    PH_LEAVE(ctx);
}

}  // extern "C"
