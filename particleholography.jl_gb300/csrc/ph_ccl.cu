// ph_ccl.cu -- connected-component labeling of equal-valued 8-connected
// regions (the semantics of ParticleHolography.jl src/ccl.jl:186-211) by
// lock-free union-find, plus the root compaction behind count_labels /
// cu_find_valid_labels (ccl.jl:213-238) and device-side bounding rectangles.
//
// Union-find after the published ECL-CC scheme (Jaiganesh & Burtscher, HPDC
// 2018): every parent array satisfies L[i] <= i and i is a root iff L[i] == i;
// parents start at the smallest equal-valued earlier neighbour; hooking links
// the larger of two roots to the smaller with compare-and-swap; finds shorten
// the path they walk (pointer jumping).  The root of a tree is therefore the
// minimum linear index of its component, and the final label (root + 1) is the
// reference's.  Every loop is bounded by an iteration limit that raises the
// context's error flag instead of running on.
#include <cstdint>
#include <cuda_runtime.h>

namespace ph {

constexpr int kCclBlockX = 32;
constexpr int kCclBlockY = 8;

template <class T>
__device__ __forceinline__ bool ccl_fg(T v);
template <>
__device__ __forceinline__ bool ccl_fg<float>(float v) { return v > 0.0f; }
template <>
__device__ __forceinline__ bool ccl_fg<uint8_t>(uint8_t v) { return v != 0; }

// Equality of pixel values: Float32 compares the values, Bool its truth.
__device__ __forceinline__ bool ccl_eq(float a, float b) { return a == b; }
__device__ __forceinline__ bool ccl_eq(uint8_t a, uint8_t b) { return (a != 0) == (b != 0); }

// Root of x, shortening the walked path on the way (benign races: every
// value written is an ancestor of the slot it is written to).
__device__ __forceinline__ uint32_t ccl_find(uint32_t *lab, uint32_t x, int64_t limit, int *err) {
    uint32_t cur = __ldcg(lab + x);
    if (cur == x) return x;
    uint32_t prev = x;
    int64_t it = 0;
    uint32_t next;
    while (cur > (next = __ldcg(lab + cur))) {
        lab[prev] = next;
        prev = cur;
        cur = next;
        if (++it > limit) { atomicExch(err, 1); break; }
    }
    return cur;
}

// Root of x without writing anything: the flatten pass may not shorten other
// pixels' paths, or a shortcut written after that pixel's own final root would
// leave a non-root label behind.
__device__ __forceinline__ uint32_t ccl_root(const uint32_t *lab, uint32_t x, int64_t limit, int *err) {
    uint32_t cur = __ldcg(lab + x), next;
    int64_t it = 0;
    while (cur > (next = __ldcg(lab + cur))) {
        cur = next;
        if (++it > limit) { atomicExch(err, 1); break; }
    }
    return cur;
}

// Links the trees of a and b (the larger root under the smaller).
__device__ __forceinline__ void ccl_hook(uint32_t *lab, uint32_t a, uint32_t b, int64_t limit, int *err) {
    uint32_t ra = ccl_find(lab, a, limit, err);
    uint32_t rb = ccl_find(lab, b, limit, err);
    int64_t it = 0;
    while (ra != rb) {
        if (ra < rb) { uint32_t t = ra; ra = rb; rb = t; }
        // ra > rb: make ra point to rb if ra is still a root
        const uint32_t ret = atomicCAS(lab + ra, ra, rb);
        if (ret == ra) return;
        ra = ret;   // ra gained a parent meanwhile: continue from it
        if (++it > limit) { atomicExch(err, 1); return; }
    }
}

// ---- tile-local phase: one CTA labels a 32 x 32 tile in shared memory

constexpr int kTile = 32;

// Local root of tile pixel x (parents in shared memory), shortening the path.
__device__ __forceinline__ int ccl_lfind(volatile int *p, int x, int64_t limit, int *err) {
    int cur = p[x];
    if (cur == x) return x;
    int prev = x, next;
    int64_t it = 0;
    while (cur > (next = p[cur])) {
        p[prev] = next;
        prev = cur;
        cur = next;
        if (++it > limit) { atomicExch(err, 1); break; }
    }
    return cur;
}

__device__ __forceinline__ int ccl_lroot(volatile int *p, int x, int64_t limit, int *err) {
    int cur = p[x], next;
    int64_t it = 0;
    while (cur > (next = p[cur])) {
        cur = next;
        if (++it > limit) { atomicExch(err, 1); break; }
    }
    return cur;
}

__device__ __forceinline__ void ccl_lhook(int *p, int a, int b, int64_t limit, int *err) {
    int ra = ccl_lfind(p, a, limit, err), rb = ccl_lfind(p, b, limit, err);
    int64_t it = 0;
    while (ra != rb) {
        if (ra < rb) { const int t = ra; ra = rb; rb = t; }
        const int ret = atomicCAS(p + ra, ra, rb);
        if (ret == ra) return;
        ra = ret;
        if (++it > limit) { atomicExch(err, 1); return; }
    }
}

// Labels each 32 x 32 tile on its own: parents start at the smallest
// equal-valued earlier neighbour inside the tile, the tile's W/NW/N/NE pairs
// are hooked in shared memory, and every pixel leaves the global index of its
// tile-local root.  Inside a tile, row-major tile order is global linear
// order, so a local root is the minimum global index of its local component
// and the global parents keep L[i] <= i.  Grid: (row tiles, column tiles),
// block (32, 8), 4 rows per thread.
template <class T>
__global__ void __launch_bounds__(kCclBlockX * kCclBlockY)
    k_ccl_local(const T *__restrict__ img, uint32_t *lab, int64_t rows, int64_t cols, int64_t slice_rows,
                int64_t limit, int *err) {
    __shared__ T sv[kTile][kTile];
    __shared__ int sp[kTile * kTile];
    const int64_t ty0 = (int64_t)blockIdx.x * kTile, tx0 = (int64_t)blockIdx.y * kTile;
    const int lx = threadIdx.x;
    constexpr int K = kTile / kCclBlockY;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int ly = threadIdx.y + k * kCclBlockY;
        const int64_t y = ty0 + ly, x = tx0 + lx;
        sv[ly][lx] = (y < rows && x < cols) ? img[y * cols + x] : T(0);   // outside: background
    }
    __syncthreads();
    // A tile of one foreground value, inside the image and one slice, is one
    // component whose root is its first pixel: label it without hooking (in a
    // projection thresholded into near-total foreground every tile is one,
    // and the shared-memory hooks of its 1024 pixels all meet at one root).
    {
        const T v0 = sv[0][0];
        bool same = ccl_fg<T>(v0) && ty0 + kTile <= rows && tx0 + kTile <= cols &&
                    (ty0 % slice_rows) + kTile <= slice_rows;
#pragma unroll
        for (int k = 0; k < K; ++k) same = same && ccl_eq(sv[threadIdx.y + k * kCclBlockY][lx], v0);
        if (__syncthreads_and(same)) {
            const uint32_t root = (uint32_t)(ty0 * cols + tx0);
#pragma unroll
            for (int k = 0; k < K; ++k) lab[(ty0 + threadIdx.y + k * kCclBlockY) * cols + tx0 + lx] = root;
            return;
        }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int ly = threadIdx.y + k * kCclBlockY;
        const int l = ly * kTile + lx;
        const T v = sv[ly][lx];
        int p = l;
        if (ccl_fg<T>(v)) {
            if (lx > 0 && ccl_eq(sv[ly][lx - 1], v)) p = l - 1;
            if (ly > 0 && (ty0 + ly) % slice_rows != 0) {
                if (lx + 1 < kTile && ccl_eq(sv[ly - 1][lx + 1], v)) p = l - kTile + 1;
                if (ccl_eq(sv[ly - 1][lx], v)) p = l - kTile;
                if (lx > 0 && ccl_eq(sv[ly - 1][lx - 1], v)) p = l - kTile - 1;
            }
        }
        sp[l] = p;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int ly = threadIdx.y + k * kCclBlockY;
        const int l = ly * kTile + lx;
        const T v = sv[ly][lx];
        if (!ccl_fg<T>(v)) continue;
        if (lx > 0 && ccl_eq(sv[ly][lx - 1], v)) ccl_lhook(sp, l, l - 1, limit, err);
        if (ly > 0 && (ty0 + ly) % slice_rows != 0) {
            if (lx > 0 && ccl_eq(sv[ly - 1][lx - 1], v)) ccl_lhook(sp, l, l - kTile - 1, limit, err);
            if (ccl_eq(sv[ly - 1][lx], v)) ccl_lhook(sp, l, l - kTile, limit, err);
            if (lx + 1 < kTile && ccl_eq(sv[ly - 1][lx + 1], v)) ccl_lhook(sp, l, l - kTile + 1, limit, err);
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int ly = threadIdx.y + k * kCclBlockY;
        const int64_t y = ty0 + ly, x = tx0 + lx;
        if (y >= rows || x >= cols) continue;
        const int l = ly * kTile + lx;
        const int r = ccl_fg<T>(sv[ly][lx]) ? ccl_lroot(sp, l, limit, err) : l;
        lab[y * cols + x] = (uint32_t)((ty0 + r / kTile) * cols + tx0 + r % kTile);
    }
}

// ---- merge across tile borders: the pairs whose earlier neighbour lies in
// another tile (W, NW of the left column; NW, N, NE of the top row; NE of the
// right column) are hooked in the global parents.  Grid: (row tiles, column
// tiles), 128 threads, 94 border pixels per tile.  Within a warp, pairs whose
// current parents are the same two nodes link the same two trees, so one lane
// of each such set hooks (between tiles of one value, as in a near-total
// foreground, one hook per neighbour tile instead of one per border pixel).
__device__ __forceinline__ void ccl_hook_dedup(uint32_t *lab, bool cond, uint32_t a, uint32_t b, int64_t limit,
                                               int *err) {
    const unsigned act = __ballot_sync(0xffffffffu, cond);
    if (cond) {
        const unsigned long long key = ((unsigned long long)__ldcg(lab + a) << 32) | __ldcg(lab + b);
        const unsigned peers = __match_any_sync(act, key);
        if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) ccl_hook(lab, a, b, limit, err);
    }
}

template <class T>
__global__ void k_ccl_border(const T *__restrict__ img, uint32_t *lab, int64_t rows, int64_t cols, int64_t slice_rows,
                             int64_t limit, int *err) {
    const int t = threadIdx.x;
    int ly = 0, lx = 0;
    bool on = true;   // every thread takes part in the warp votes below
    if (t < kTile) { ly = 0; lx = t; }
    else if (t < 2 * kTile - 1) { ly = t - (kTile - 1); lx = 0; }
    else if (t < 3 * kTile - 2) { ly = t - (2 * kTile - 2); lx = kTile - 1; }
    else on = false;
    const int64_t y = (int64_t)blockIdx.x * kTile + ly, x = (int64_t)blockIdx.y * kTile + lx;
    on = on && y < rows && x < cols;
    const int64_t i = on ? y * cols + x : 0;
    const T v = on ? img[i] : T(0);
    on = on && ccl_fg<T>(v);
    const bool up = on && y % slice_rows != 0;
    const int64_t u = i - cols;
    ccl_hook_dedup(lab, on && lx == 0 && x > 0 && ccl_eq(img[i - 1], v), (uint32_t)i, (uint32_t)(i - 1), limit, err);
    ccl_hook_dedup(lab, up && (lx == 0 || ly == 0) && x > 0 && ccl_eq(img[u - 1], v), (uint32_t)i, (uint32_t)(u - 1),
                   limit, err);
    ccl_hook_dedup(lab, up && ly == 0 && ccl_eq(img[u], v), (uint32_t)i, (uint32_t)u, limit, err);
    ccl_hook_dedup(lab, up && (ly == 0 || lx == kTile - 1) && x + 1 < cols && ccl_eq(img[u + 1], v), (uint32_t)i,
                   (uint32_t)(u + 1), limit, err);
}

template <class T>
__global__ void k_ccl_compress(const T *__restrict__ img, uint32_t *lab, int64_t n, int64_t limit, int *err) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (ccl_fg<T>(img[i])) lab[i] = ccl_root(lab, (uint32_t)i, limit, err);
}

// Final labels: 1 + the root's index within its own image, 0 for background.
template <class T>
__global__ void k_ccl_background(const T *__restrict__ img, uint32_t *lab, int64_t n, int64_t slice_n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t base = (uint32_t)((i / slice_n) * slice_n);
    lab[i] = ccl_fg<T>(img[i]) ? lab[i] - base + 1u : 0u;
}

template <class T>
static cudaError_t ccl_run(const T *img, uint32_t *lab, int64_t rows, int64_t cols, int64_t slice_rows, int64_t limit,
                           int *err, cudaStream_t s, int64_t *launches) {
    const int64_t n = rows * cols;
    const int tpb = 256;
    const unsigned g1 = (unsigned)((n + tpb - 1) / tpb);
    dim3 b2(kCclBlockX, kCclBlockY);
    dim3 gt((unsigned)((rows + kTile - 1) / kTile), (unsigned)((cols + kTile - 1) / kTile));
    k_ccl_local<T><<<gt, b2, 0, s>>>(img, lab, rows, cols, slice_rows, limit, err);
    k_ccl_border<T><<<gt, 128, 0, s>>>(img, lab, rows, cols, slice_rows, limit, err);
    k_ccl_compress<T><<<g1, tpb, 0, s>>>(img, lab, n, limit, err);
    k_ccl_background<T><<<g1, tpb, 0, s>>>(img, lab, n, slice_rows * cols);
    *launches += 4;
    return cudaGetLastError();
}

// Labels `rows x cols` pixels; with slice_rows < rows, every slice_rows rows
// form an independent image (a batch of slices labelled in one launch set).
cudaError_t ccl_launch(const void *img, bool is_bool, uint32_t *lab, int64_t rows, int64_t cols, int64_t slice_rows,
                       int64_t limit, int *err, cudaStream_t s, int64_t *launches) {
    if (rows <= 0 || cols <= 0) return cudaSuccess;
    if (slice_rows <= 0 || slice_rows > rows) slice_rows = rows;
    if (is_bool)
        return ccl_run<uint8_t>(static_cast<const uint8_t *>(img), lab, rows, cols, slice_rows, limit, err, s,
                                launches);
    return ccl_run<float>(static_cast<const float *>(img), lab, rows, cols, slice_rows, limit, err, s, launches);
}

// ---------------------------------------------------------------- bounding rectangles

// boxes[4 r .. 4 r + 3] = (min slow, min fast, max slow, max fast) over the pixels of root r (0-based).
__global__ void k_boxes(const uint32_t *__restrict__ lab, int64_t rows, int64_t cols, int64_t slice_rows,
                        const unsigned *rank, int *boxes) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * cols) return;
    const uint32_t l = lab[i];
    if (l == 0) return;
    const int64_t slice_n = slice_rows * cols;
    const int64_t base = (i / slice_n) * slice_n;
    const unsigned r = rank[base + l - 1];
    const int64_t li = i - base;
    const int slow = (int)(li / cols), fast = (int)(li % cols);
    atomicMin(boxes + 4 * r + 0, slow);
    atomicMin(boxes + 4 * r + 1, fast);
    atomicMax(boxes + 4 * r + 2, slow);
    atomicMax(boxes + 4 * r + 3, fast);
}

__global__ void k_boxes_init(int *boxes, int64_t count) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    boxes[4 * i + 0] = 0x7fffffff;
    boxes[4 * i + 1] = 0x7fffffff;
    boxes[4 * i + 2] = -1;
    boxes[4 * i + 3] = -1;
}

// ---------------------------------------------------------------- root compaction

constexpr int kRootThreads = 256;
constexpr int kRootItems = 16;                       // per thread
constexpr int kRootTile = kRootThreads * kRootItems; // elements per block

// A root carries its own index (within its image of slice_n pixels) plus one.
__device__ __forceinline__ bool is_root(const uint32_t *lab, int64_t i, int64_t slice_n) {
    return lab[i] == (uint32_t)(i % slice_n + 1);
}

__global__ void k_roots_count(const uint32_t *__restrict__ lab, int64_t n, int64_t slice_n, unsigned *counts) {
    __shared__ unsigned wsum[kRootThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kRootTile;
    unsigned c = 0;
#pragma unroll
    for (int k = 0; k < kRootItems; ++k) {
        const int64_t i = base + (int64_t)k * kRootThreads + threadIdx.x;
        if (i < n && is_root(lab, i, slice_n)) ++c;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = 0;
        for (int w = 0; w < kRootThreads / 32; ++w) t += wsum[w];
        counts[blockIdx.x] = t;
    }
}

// Exclusive scan of `nb` block counts in place (one CTA); total -> *total.
__global__ void k_roots_scan(unsigned *counts, int64_t nb, unsigned long long *total) {
    __shared__ unsigned long long carry;
    __shared__ unsigned long long wsum[kRootThreads / 32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t off = 0; off < nb; off += kRootThreads) {
        const int64_t i = off + threadIdx.x;
        const unsigned long long v = i < nb ? counts[i] : 0ull;
        unsigned long long incl = v;
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += u;
        }
        if (lane == 31) wsum[w] = incl;
        __syncthreads();
        unsigned long long wpre = 0;
        for (int k = 0; k < w; ++k) wpre += wsum[k];
        const unsigned long long excl = carry + wpre + incl - v;
        if (i < nb) counts[i] = (unsigned)excl;
        __syncthreads();
        if (threadIdx.x == kRootThreads - 1) carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

// Writes the 1-based linear index of every root, in increasing order, and
// (rank non-null) rank[i] = the root's position in that order.
__global__ void k_roots_write(const uint32_t *__restrict__ lab, int64_t n, int64_t slice_n, const unsigned *offsets,
                              long long *out, int64_t cap, unsigned *rank) {
    __shared__ unsigned wsum[kRootThreads / 32];
    __shared__ unsigned running;
    const int64_t base = (int64_t)blockIdx.x * kRootTile;
    if (threadIdx.x == 0) running = offsets[blockIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int k = 0; k < kRootItems; ++k) {
        const int64_t i = base + (int64_t)k * kRootThreads + threadIdx.x;
        const bool f = i < n && is_root(lab, i, slice_n);
        const unsigned m = __ballot_sync(0xffffffffu, f);
        if (lane == 0) wsum[w] = __popc(m);
        __syncthreads();
        unsigned pre = running;
        for (int q = 0; q < w; ++q) pre += wsum[q];
        pre += __popc(m & ((1u << lane) - 1u));
        if (f && (int64_t)pre < cap && out) out[pre] = (long long)(i + 1);
        if (f && rank) rank[i] = pre;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned t = 0;
            for (int q = 0; q < kRootThreads / 32; ++q) t += wsum[q];
            running += t;
        }
        __syncthreads();
    }
}

int64_t roots_blocks(int64_t n) { return (n + kRootTile - 1) / kRootTile; }

cudaError_t roots_count_launch(const uint32_t *lab, int64_t n, int64_t slice_n, unsigned *counts,
                               unsigned long long *total, cudaStream_t s, int64_t *launches) {
    const int64_t nb = roots_blocks(n);
    k_roots_count<<<(unsigned)nb, kRootThreads, 0, s>>>(lab, n, slice_n, counts);
    k_roots_scan<<<1, kRootThreads, 0, s>>>(counts, nb, total);
    *launches += 2;
    return cudaGetLastError();
}

cudaError_t roots_write_launch(const uint32_t *lab, int64_t n, int64_t slice_n, const unsigned *offsets,
                               long long *out, int64_t cap, unsigned *rank, cudaStream_t s, int64_t *launches) {
    const int64_t nb = roots_blocks(n);
    k_roots_write<<<(unsigned)nb, kRootThreads, 0, s>>>(lab, n, slice_n, offsets, out, cap, rank);
    *launches += 1;
    return cudaGetLastError();
}

// Boxes of `count` roots whose ranks are in `rank` (see k_roots_write).
cudaError_t boxes_launch(const uint32_t *lab, int64_t rows, int64_t cols, int64_t slice_rows, const unsigned *rank,
                         int *boxes, int64_t count, cudaStream_t s, int64_t *launches) {
    if (count > 0) k_boxes_init<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(boxes, count);
    const int64_t n = rows * cols;
    k_boxes<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(lab, rows, cols, slice_rows, rank, boxes);
    *launches += 2;
    return cudaGetLastError();
}

}  // namespace ph
