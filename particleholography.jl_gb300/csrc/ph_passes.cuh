// ph_passes.cuh -- the pass kernels of the reconstruction, Gerchberg-Saxton and
// propagation paths.  Every pass reads whole rows (contiguous), transforms them
// with the row-FFT engine and writes either whole rows or, with the
// transposed store, columns of the output: two passes make one 2-D transform
// and the transpose between them costs nothing extra.
//
// Layouts (n_fast = nx, n_slow = ny):
//   image-domain arrays       [ny][nx]   (wavefront, holograms, projection, slices)
//   transfer functions        [ny][nx]   centred (fftshifted), as the caller builds them
//   after a forward row pass  [nx][ny]   (row = kx, along y)
//   spectrum state            [nx][ny]   float4 (re, im, phase-rate bits, |Hdz|-1)
//   slice intermediate T      [batch][ny][nx]
//
// The reconstruction passes stage their input rows in shared memory: pass A
// forms X at its first slice and Hdz from the spectrum-state rows once and
// advances X slice by slice; pass B double-buffers the rows of the next slice
// with bulk asynchronous copies (TMA, ph_tma.cuh) while it transforms the
// current one.
//
// Each pass chooses its elements per thread (EPT, the main radix), its CTA size
// (TT) and the resident threads per SM its register budget is sized for (RTS):
// more resident warps hide more latency where a pass is latency-bound.
#pragma once

#include <cuda_fp16.h>
#include <type_traits>
#include "ph_fft.cuh"
#include "ph_tma.cuh"

#ifndef PH_HT_EARLY
#define PH_HT_EARLY 1
#endif
#ifndef PH_RECONB_RTS
#define PH_RECONB_RTS 640
#endif
#ifndef PH_RECONA_CHAIN
#define PH_RECONA_CHAIN -1   // pass A product chain: -1 per length (chain<N>()), 0 never, 1 always
#endif

namespace ph {

// ---------------------------------------------------------------- launch shape

// Shape of a pass over rows of length N with (up to) EPT values per thread:
// E values per thread (3 * EPT/2 for N = 3 * 2^a), P threads per row, ROWS rows
// and THREADS = ROWS * P threads (512 for every large N) per CTA.
__host__ __device__ constexpr int engine_e(int n, int ept) {
    return cmin(n, plan_pow2(n) ? ept : 3 * (ept / 2));
}

template <int N, int EPT = 16, int TT = 512>
struct Shape {
    static constexpr bool POW2 = (N & (N - 1)) == 0;
    static constexpr int E = engine_e(N, EPT);
    static constexpr int P = N / E;
    static constexpr int ROWS = cmax(1, cmin(64, TT / P));
    static constexpr int THREADS = ROWS * P;
    template <bool ROW_FAST>
    static constexpr int stride() { return SmemRow<N, ROWS, P, ROW_FAST>::STRIDE; }
    template <bool ROW_FAST>
    static constexpr size_t smem_bytes() { return (size_t)ROWS * stride<ROW_FAST>() * 8; }
};

template <int N, int EPT, int TT, bool ROW_FAST>
struct ThreadMap {
    using S = Shape<N, EPT, TT>;
    __device__ __forceinline__ static int row(int t) { return ROW_FAST ? t % S::ROWS : t / S::P; }
    __device__ __forceinline__ static int j(int t) { return ROW_FAST ? t / S::ROWS : t % S::P; }
};

constexpr size_t kSmemMax = 227 * 1024;   // opt-in dynamic shared memory per CTA

// Defaults of a pass: radix-16 engine, 512-thread CTAs, registers for 512
// resident threads per SM (128 per thread), one padded exchange row per
// transformed row of shared memory.
struct PassBase {
    static constexpr int EPT = 16;
    static constexpr int TT = 512;    // target threads per CTA
    static constexpr int RTS = 512;   // resident threads per SM the register budget allows
    template <int N>
    static constexpr int rts() { return RTS; }
    template <int N, bool ROW_FAST>
    static constexpr size_t smem() { return Shape<N, EPT, TT>::template smem_bytes<ROW_FAST>(); }
    // Persistent passes loop over row blocks; their grid is the resident CTA count.
    template <int N>
    static constexpr bool persistent() { return false; }
    // CTAs per thread-block cluster (consecutive blockIdx.x).
    template <int N>
    static constexpr int cluster() { return 1; }
    // Launched as a programmatic dependent of the previous kernel on the stream
    // (the body calls grid_dependency_wait before it touches that kernel's data).
    template <int N>
    static constexpr bool pdl() { return false; }
};

// Programmatic dependent launch.  The wait blocks until the kernels this grid
// depends on have completed and their memory is visible; the trigger lets the
// next dependent grid be scheduled once every CTA of this one has issued it.
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dependents_launch() { asm volatile("griddepcontrol.launch_dependents;" :::); }

constexpr size_t round128(size_t b) { return (b + 127) / 128 * 128; }

// Whether the stage twiddles of a length-N, E-per-thread transform also fit in
// the shared memory of a pass that uses `used` bytes (the copy starts at
// round128(used)), and the bytes they add.
template <int N, int E>
constexpr bool tw_fits(size_t used) {
    return round128(used) + stage_tw_bytes<N, E>() <= kSmemMax;
}
template <int N, int E>
constexpr size_t tw_extra(size_t used) {
    return tw_fits<N, E>(used) ? round128(used) - used + stage_tw_bytes<N, E>() : 0;
}

// The pointer, hidden from the optimiser: loads through it are not hoisted
// out of the enclosing loop (which would pin the values in registers).
template <class T>
__device__ __forceinline__ T *opaque(T *p) {
    asm volatile("" : "+l"(p));
    return p;
}

template <int N, int EPT, int TT, bool ROW_FAST>
__device__ __forceinline__ float2 *xrow(unsigned char *base, int r) {
    return reinterpret_cast<float2 *>(base) + (size_t)r * Shape<N, EPT, TT>::template stride<ROW_FAST>();
}

// Register budget: rts<N>() resident threads per SM.
template <int N, class Body>
constexpr int min_blocks() {
    return cmax(1, Body::template rts<N>() / Shape<N, Body::EPT, Body::TT>::THREADS);
}

template <int N, bool ROW_FAST, class Body>
__global__ void __launch_bounds__(Shape<N, Body::EPT, Body::TT>::THREADS, min_blocks<N, Body>())
    k_pass(const Body body) {
    extern __shared__ __align__(128) unsigned char ph_smem[];
    const int t = threadIdx.x;
    const int r = ThreadMap<N, Body::EPT, Body::TT, ROW_FAST>::row(t);
    const int j = ThreadMap<N, Body::EPT, Body::TT, ROW_FAST>::j(t);
    body.template run<N, ROW_FAST>(ph_smem, r, j);
}

// A pass whose body also takes a tensor map.  The map is a __grid_constant__
// parameter of its own (the copy engine reads it where the kernel's
// parameters live); the body stays an ordinary parameter.
template <int N, bool ROW_FAST, class Body>
__global__ void __launch_bounds__(Shape<N, Body::EPT, Body::TT>::THREADS, min_blocks<N, Body>())
    k_pass_tm(const Body body, const __grid_constant__ CUtensorMap tm) {
    extern __shared__ __align__(128) unsigned char ph_smem[];
    const int t = threadIdx.x;
    const int r = ThreadMap<N, Body::EPT, Body::TT, ROW_FAST>::row(t);
    const int j = ThreadMap<N, Body::EPT, Body::TT, ROW_FAST>::j(t);
    body.template run<N, ROW_FAST>(ph_smem, r, j, &tm);
}

// A pass whose body takes two tensor maps.
template <int N, bool ROW_FAST, class Body>
__global__ void __launch_bounds__(Shape<N, Body::EPT, Body::TT>::THREADS, min_blocks<N, Body>())
    k_pass_tm2(const Body body, const __grid_constant__ CUtensorMap tm0, const __grid_constant__ CUtensorMap tm1) {
    extern __shared__ __align__(128) unsigned char ph_smem[];
    const int t = threadIdx.x;
    const int r = ThreadMap<N, Body::EPT, Body::TT, ROW_FAST>::row(t);
    const int j = ThreadMap<N, Body::EPT, Body::TT, ROW_FAST>::j(t);
    body.template run<N, ROW_FAST>(ph_smem, r, j, &tm0, &tm1);
}

__device__ __forceinline__ int shift_idx(int i, int n) {   // centred index of natural frequency i
    int s = i + (n >> 1);
    return s >= n ? s - n : s;
}

// ---------------------------------------------------------------- grouped launches

// A grouped launch runs one pass for up to kMaxItems holograms of the same
// transform shape at once: blockIdx.z is the item.  Each item has its own
// input and transfer functions (pointer tables in the pass's parameters), its
// own slot of the scratch (the pass's pointers plus z times a stride) and its
// own slice count within the batch and slices per CTA
// (its packed item word), so every item is computed exactly as a single call would.
// With nitems = 1 (every single call) the tables are unused.
constexpr int kMaxItems = 8;

// The item tables of a grouped pass A / pass B, a base class of the grouped
// instantiations only: the single-call kernels keep their parameters (and
// their register allocation) unchanged.
// Item z's slices in the batch and slices per CTA are packed into the 32-bit
// halves of four 64-bit words (nb | group << 16) and selected without indexing
// an array by blockIdx.z (which would copy the parameters to local memory).
struct NoItems {};
struct ReconItems {
    int nitems = 1;
    size_t item_state_stride = 0, item_t_stride = 0, p64_stride = 0;
    unsigned long long item_words[kMaxItems / 2] = {};
    __host__ void set_item(int z, int nb, int group) {
        const unsigned long long w = (unsigned long long)((uint32_t)nb | ((uint32_t)group << 16));
        item_words[z >> 1] = (item_words[z >> 1] & ~(0xFFFFFFFFull << ((z & 1) * 32))) | (w << ((z & 1) * 32));
    }
    __host__ __device__ int item_nb(int z) const { return (int)(word(z) & 0xFFFFu); }
    __host__ __device__ int item_group(int z) const { return (int)(word(z) >> 16); }
    __host__ __device__ uint32_t word(int z) const {
        const unsigned long long a = (z >> 1) == 0 ? item_words[0]
                                   : (z >> 1) == 1 ? item_words[1]
                                   : (z >> 1) == 2 ? item_words[2]
                                                   : item_words[3];
        return (uint32_t)(a >> ((z & 1) * 32));
    }
};
static_assert(kMaxItems == 8, "four packed words");

// ---------------------------------------------------------------- forward rows (transposed store)

enum FwdInput { FWD_COMPLEX = 0, FWD_SQRT_REAL = 1, FWD_PADDED = 2 };

// out[kx][y] = FFT_x(in[y][:])[kx].  FWD_SQRT_REAL: in = sqrtf(real[y][x]) + 0i.
// FWD_PADDED: the input is the virtual 2n x 2n mean-padded array of `src`
// (n = nx_in) with `src` at rows/cols [pad_off, pad_off + n).
template <int MODE>
struct FwdRowsT : PassBase {
    const float2 *src;
    const float *src_real;
    float2 *dst;
    const float2 *tw;
    const float2 *pad_mean;   // device scalar (FWD_PADDED)
    int nrows;                // rows of the (virtual) input = ny
    int nx_in, ny_in, pad_off;
    int nitems = 1;           // grouped launch: item z reads src_items / src_real_items[z], writes dst + z dst_stride
    size_t dst_stride = 0;
    const float2 *src_items[kMaxItems] = {};
    const float *src_real_items[kMaxItems] = {};

    template <int N, bool RF>
    __device__ __forceinline__ void run(unsigned char *smem, int r, int j) const {
        using S = Shape<N, EPT, TT>;
        const int z = blockIdx.z;
        const float2 *src = nitems > 1 ? src_items[z] : this->src;
        const float *src_real = nitems > 1 ? src_real_items[z] : this->src_real;
        float2 *dst = this->dst + (size_t)z * dst_stride;
        const int y = blockIdx.x * S::ROWS + r;
        const bool valid = y < nrows;
        float2 mean = make_float2(0.f, 0.f);
        if (MODE == FWD_PADDED) mean = *pad_mean;
        fft_row<N, S::E, false>(
            xrow<N, EPT, TT, RF>(smem, r), j, tw,
            [&](int, int x) -> float2 {
                if (!valid) return make_float2(0.f, 0.f);
                if constexpr (MODE == FWD_COMPLEX) {
                    return src[(size_t)y * N + x];
                } else if constexpr (MODE == FWD_SQRT_REAL) {
                    return make_float2(sqrtf(src_real[(size_t)y * N + x]), 0.f);
                } else {
                    const int yi = y - pad_off, xi = x - pad_off;
                    if (yi >= 0 && yi < ny_in && xi >= 0 && xi < nx_in) return src[(size_t)yi * nx_in + xi];
                    return mean;
                }
            },
            [&](int, int kx, float2 v) {
                if (valid) dst[(size_t)kx * nrows + y] = v;
            });
    }
};

// ---------------------------------------------------------------- spectrum state

// Phase of h as a 32-bit fixed-point fraction of a turn, to ~1e-10 rad: the
// nearest of 4096 table angles j / 4096 turns (FP32 atan2 picks it), the
// rotation z = h * conj(w_j), and the remaining angle |phi| <~ pi / 4096 by
// FP32 atan2, whose ~2 ulp relative error is then ~2e-10 rad.  tab holds w_j =
// (cos, sin)(2 pi j / 4096), each as an FP32 pair hi + lo (computed in FP64).
// z's real part is ~|h| and needs FP32 only; its imaginary part hy wx - hx wy
// cancels to ~|h| pi / 4096, so it is formed from error-free products (fma)
// of the hi words, an error-free difference, and the lo words' products: FP32
// arithmetic to the accuracy the FP64 form had, which GB300 runs at 1/64 of
// its FP32 rate (the FP64 form spent about half of the spectrum pass there).
constexpr int kPhaseTable = 4096;
__device__ __forceinline__ uint32_t phase_turns_u32(float2 h, const float4 *__restrict__ tab) {
    const float a0 = atan2f(h.y, h.x);
    const int i = __float2int_rn(a0 * ((float)kPhaseTable / 6.28318530717958647692f));
    const float4 w = __ldg(tab + (i & (kPhaseTable - 1)));   // (cos hi, cos lo, sin hi, sin lo)
    const float zx = __fmaf_rn(h.x, w.x, __fmul_rn(h.y, w.z));
    const float p1 = __fmul_rn(h.y, w.x), e1 = __fmaf_rn(h.y, w.x, -p1);   // hy wx_hi = p1 + e1 exactly
    const float p2 = __fmul_rn(h.x, w.z), e2 = __fmaf_rn(h.x, w.z, -p2);   // hx wy_hi = p2 + e2 exactly
    const float d = __fsub_rn(p1, p2);                                       // p1 - p2 = d + ed exactly
    const float bv = __fsub_rn(d, p1);
    const float ed = __fadd_rn(__fsub_rn(p1, __fsub_rn(d, bv)), __fsub_rn(-p2, bv));
    const float lo = __fmaf_rn(h.y, w.y, -__fmul_rn(h.x, w.w));             // the lo words
    const float zy = __fadd_rn(d, __fadd_rn(__fadd_rn(ed, __fsub_rn(e1, e2)), lo));
    const float phi = atan2f(zy, zx);
    return ((uint32_t)i << 20) + (uint32_t)__float2int_rn(phi * (4294967296.0f / 6.28318530717958647692f));
}

// log2 |h|.  |h|^2 - 1 from error-free products (fma) and an error-free sum
// of them (s - 1 is exact for s in [1/2, 2]), so that there is no cancellation
// error near |h| = 1, over |h| + 1, then log1pf.  h = 0 gives -1e30 rather
// than -inf, so that k log2|h| is 0 at k = 0 (|h|^0 = 1) and |h|^k underflows
// to 0 for every k >= 1.
__device__ __forceinline__ float log2_modulus(float2 h) {
    const float a = __fmul_rn(h.x, h.x), ea = __fmaf_rn(h.x, h.x, -a);
    const float b = __fmul_rn(h.y, h.y), eb = __fmaf_rn(h.y, h.y, -b);
    const float s = __fadd_rn(a, b);
    const float bv = __fsub_rn(s, a);
    const float es = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bv)), __fsub_rn(b, bv));
    const float v = __fadd_rn(__fsub_rn(s, 1.0f), __fadd_rn(es, __fadd_rn(ea, eb)));
    const float w = v / (sqrtf(fmaf(h.x, h.x, h.y * h.y)) + 1.0f);
    return fmaxf(log1pf(w) * 1.44269504088896340736f, -1e30f);
}

// Rows kx of the forward-row output, FFT along y, times the front transfer
// (and 1/(nx ny)), stored with the slice phase rate of the slice transfer:
// state[kx][ky] = (X0, turns(Hdz), log2 |Hdz|).
struct SpectrumCols : PassBase {
    const float2 *a1;        // [nx][ny]
    const float2 *hf, *hdz;  // centred [ny][nx]
    const float *lpf;        // centred [ny][nx] low-pass filter, or null
    const float4 *ptab;      // kPhaseTable unit vectors as FP32 pairs (phase_turns_u32)
    float4 *state;           // [nx][ny]
    const float2 *tw;
    int nx, ny;
    float scale;
    int nitems = 1;          // grouped launch: item z's transfers from the tables, a1 / state + z strides
    size_t a1_stride = 0, state_stride = 0;
    const float2 *hf_items[kMaxItems] = {};
    const float2 *hdz_items[kMaxItems] = {};

    template <int N, bool RF>
    __device__ __forceinline__ void run(unsigned char *smem, int r, int j) const {
        using S = Shape<N, EPT, TT>;
        const int z = blockIdx.z;
        const float2 *a1 = this->a1 + (size_t)z * a1_stride;
        float4 *state = this->state + (size_t)z * state_stride;
        const float2 *hf = nitems > 1 ? hf_items[z] : this->hf;
        const float2 *hdz = nitems > 1 ? hdz_items[z] : this->hdz;
        const int kx = blockIdx.x * S::ROWS + r;
        const bool valid = kx < nx;
        const int sx = valid ? shift_idx(kx, nx) : 0;
        fft_row<N, S::E, false>(
            xrow<N, EPT, TT, RF>(smem, r), j, tw,
            [&](int, int y) -> float2 { return valid ? a1[(size_t)kx * N + y] : make_float2(0.f, 0.f); },
            [&](int, int ky, float2 v) {
                if (!valid) return;
                const size_t c = (size_t)shift_idx(ky, N) * nx + sx;
                const float2 x0 = cscale(cmul(v, hf[c]), lpf != nullptr ? scale * lpf[c] : scale);
                const float2 d = hdz[c];
                state[(size_t)kx * N + ky] =
                    make_float4(x0.x, x0.y, __uint_as_float(phase_turns_u32(d, ptab)), log2_modulus(d));
            });
    }
};

// The spectrum pass with the transfers staged: the columns of the front and
// slice transfers that the CTA's ROWS rows kx need are loaded into shared
// memory as [ky][kx mod ROWS] by tensor-map boxes of ROWS x 256 (issued before
// the transform, so they overlap it; kx's centred column is one of ROWS
// consecutive ones, ky's centred row range of a box is contiguous because N/2
// is a multiple of 256).  The outputs then read them conflict-free instead of
// gathering ROWS-element pieces from ROWS different lines per warp load.  One
// item, no low-pass mask, N a multiple of 512 (so that N/2 is one of 256),
// nx a multiple of 2 ROWS.
struct SpectrumColsT : SpectrumCols {
    int *err;   // raised if the staging wait times out
    template <int N, bool RF>
    static constexpr size_t xbytes() { return round128(Shape<N, EPT, TT>::template smem_bytes<RF>()); }
    template <int N>
    static constexpr size_t tbytes() { return (size_t)N * Shape<N, EPT, TT>::ROWS * 8; }   // one staged transfer
    template <int N, bool RF>
    static constexpr size_t smem() { return xbytes<N, RF>() + 2 * tbytes<N>() + 16; }
    template <int N>
    static constexpr bool staged() {
        return N % 512 == 0 && Shape<N, EPT, TT>::ROWS >= 4 && Shape<N, EPT, TT>::ROWS <= 32 &&
               smem<N, true>() <= kSmemMax;
    }
    template <int N, bool RF>
    __device__ __forceinline__ void run(unsigned char *smem, int r, int j, const void *tm_hf,
                                        const void *tm_hdz) const {
        using S = Shape<N, EPT, TT>;
        constexpr int ROWS = S::ROWS;
        float2 *shf = reinterpret_cast<float2 *>(smem + xbytes<N, RF>());
        float2 *shdz = shf + (size_t)N * ROWS;
        uint64_t *bar = reinterpret_cast<uint64_t *>(smem + xbytes<N, RF>() + 2 * tbytes<N>());
        const int kx0 = blockIdx.x * ROWS;
        const int kx = kx0 + r;
        const bool valid = kx < nx;
        const int sx0 = shift_idx(kx0, nx);   // the centred columns of kx0 .. kx0 + ROWS - 1
        if (threadIdx.x == 0) {
            mbar_init(bar, 1);
            mbar_fence_init();
            mbar_arrive_expect_tx(bar, (uint32_t)(2 * tbytes<N>()));
#pragma unroll 1
            for (int q = 0; q < N / 256; ++q) {
                const int sy = shift_idx(q * 256, N);
                tma_load_2d(shf + (size_t)q * 256 * ROWS, tm_hf, sx0, sy, bar);
                tma_load_2d(shdz + (size_t)q * 256 * ROWS, tm_hdz, sx0, sy, bar);
            }
        }
        __syncthreads();   // the barrier is initialised before any thread waits on it
        bool ready = false;
        fft_row<N, S::E, false>(
            xrow<N, EPT, TT, RF>(smem, r), j, tw,
            [&](int, int y) -> float2 { return valid ? a1[(size_t)kx * N + y] : make_float2(0.f, 0.f); },
            [&](int, int ky, float2 v) {
                if (!ready) {   // (the first output: the boxes have landed)
                    mbar_wait(bar, 0, err);
                    ready = true;
                }
                if (!valid) return;
                const float2 x0 = cscale(cmul(v, shf[ky * ROWS + r]), scale);
                const float2 d = shdz[ky * ROWS + r];
                state[(size_t)kx * N + ky] =
                    make_float4(x0.x, x0.y, __uint_as_float(phase_turns_u32(d, ptab)), log2_modulus(d));
            });
    }
};

// ---------------------------------------------------------------- reconstruction pass A

// Slice k of rows kx: X_k = X0 * Hdz^k; inverse FFT along ky; transposed store
// T[b][y - y0][kx] for y in [y0, y0 + ny_out).  Hdz^k X0 evaluated directly
// from the state uses the phase rate times k in exact integer turn arithmetic
// and |Hdz|^k = 2^(k log2 |Hdz|).
//
// A CTA transforms `group` consecutive slices from rows staged in shared
// memory once (the staging forms are described at FORM_CHAIN .. FORM_NONE).
// Staged rows are spaced so that the accesses of one phase of lanes (ROWS rows
// x consecutive columns) fall on distinct banks.
//
// The transposed store writes 4 consecutive kx (one 32-byte sector) per y.
// Where a CTA holds fewer than 4 rows (N >= 4096), 4 / ROWS CTAs form a
// thread-block cluster: each leaves its transformed rows in shared memory,
// and after a cluster barrier each stores a 1 / (4 / ROWS) share of the y
// range for all 4 rows, reading its peers' rows through distributed shared
// memory.  (Stores of 2 consecutive kx, 16 bytes, ran 2-4x slower.)
template <bool GROUPED = false, bool TSTORE = false>   // GROUPED: the grouped-launch form (grid z = item)
struct ReconAT : PassBase, std::conditional_t<GROUPED, ReconItems, NoItems> {
    // 4 rows of 128 threads at N = 2048: one CTA per SM.  (One row per CTA in
    // clusters of 4, or two in clusters of 2, measured 65 % / 59 % slower.)
    static constexpr int TT = 512;
    template <int N>
    static constexpr int cluster() {
        return Shape<N, EPT, TT>::ROWS >= 4 ? 1 : 4 / Shape<N, EPT, TT>::ROWS;
    }
    const float4 *state;   // [nx][ny]
    float2 *t;             // [batch][ny_out][nx]
    const float2 *tw;
    int *err;              // raised if a bulk-copy wait times out
    int nx, ny_out, y0;
    int k0;                // global slice index of batch slot 0
    int nbatch, group;     // slices in the batch, slices per CTA

    // Staged forms, the first that fits the CTA's shared memory beside the
    // exchange rows:
    //  FORM_CHAIN: per row, X_k and Hdz as two float2 rows; every slice reads
    //    X_k and advances it in place, X_{k+1} = X_k Hdz (the reference's
    //    cumulative product).  The CTA computes X at its first slice directly
    //    from the state, so each product chain spans at most `group` slices.
    //  FORM_STATE: the state rows, staged by bulk copy; every slice evaluates
    //    Hdz^k from them.
    //  FORM_X0: only X0 (8 of the state's 16 bytes) staged; the phase rate
    //    and log2 |Hdz| come from L2 every slice.  (3 * 2^a lengths, whose
    //    24-value threads give a CTA 8 rows: their full state does not fit.)
    //  FORM_NONE: the whole state from L2 every slice.
    // The chain saves the per-voxel sin/cos; the direct forms move fewer
    // shared-memory bytes per voxel and need fewer registers.  Measured per
    // pass A launch, chain against the staged state: 2048 3.7 % and 512 2.7 %
    // faster; 4096 with the tensor-map store 1.5 % faster; 1024 18 % slower
    // (register spills; 6 % slower in the tensor-map store form, unspilled); 4096 with the pull store 6 % slower (its distributed
    // loads compete for shared-memory bandwidth); 256 22 % slower (slice groups
    // of 6 slices do not repay the chain's start).  Other lengths keep the
    // direct form.
    enum { FORM_NONE = 0, FORM_X0 = 1, FORM_STATE = 2, FORM_CHAIN = 3 };
    template <int N>
    static constexpr bool chain() {
        return PH_RECONA_CHAIN >= 0 ? PH_RECONA_CHAIN != 0 : (N == 2048 || N == 512 || (TSTORE && N == 4096));
    }
    template <int N, bool RF>
    static constexpr int rec_stride() {   // float2 between rows: conflict-free for the load pattern
        using S = Shape<N, EPT, TT>;
        return N + SmemRow<N, S::ROWS, S::P, RF>::JC % 16;
    }
    template <int N>
    static constexpr size_t state_stride() {   // bytes between staged state rows
        constexpr int R = Shape<N, EPT, TT>::ROWS;
        constexpr size_t dense = (size_t)N * 16;
        return (dense + 127) / 128 * 128 + (16 * (8 / (R < 8 ? R : 8))) % 128;
    }
    template <int N, bool RF>
    static constexpr size_t form_bytes(int f) {   // staged rows (+ the bulk-copy barrier of FORM_STATE)
        using S = Shape<N, EPT, TT>;
        return f == FORM_CHAIN ? round128((size_t)2 * S::ROWS * rec_stride<N, RF>() * 8)
             : f == FORM_STATE ? round128((size_t)S::ROWS * state_stride<N>() + 8)
             : f == FORM_X0    ? round128((size_t)S::ROWS * rec_stride<N, RF>() * 8)
                               : 0;
    }
    template <int N, bool RF>
    static constexpr bool fits(int f) {
        return form_bytes<N, RF>(f) + Shape<N, EPT, TT>::template smem_bytes<RF>() <= kSmemMax;
    }
    template <int N, bool RF>
    static constexpr int form() {
        return (chain<N>() && fits<N, RF>(FORM_CHAIN)) ? FORM_CHAIN
             : fits<N, RF>(FORM_STATE)                ? FORM_STATE
             : fits<N, RF>(FORM_X0)                   ? FORM_X0
                                                      : FORM_NONE;
    }
    template <int N, bool RF>
    static constexpr size_t stage_total() {
        return form_bytes<N, RF>(form<N, RF>());
    }
    template <int N, bool RF>
    static constexpr size_t smem() {
        return stage_total<N, RF>() + Shape<N, EPT, TT>::template smem_bytes<RF>();
    }
    // Hdz^k X0 from the state (re, im, phase-rate bits, log2 |Hdz|): the phase
    // k p in exact integer turn arithmetic, the modulus |Hdz|^k = 2^(k log2|Hdz|)
    // (exact for any transfer, unit or not).
    __device__ __forceinline__ static float2 direct(const float4 s, uint32_t k) {
        const int32_t tt = (int32_t)(k * __float_as_uint(s.z));
        const float ang = (float)tt * 1.46291807926715968e-9f;   // 2 pi / 2^32
        float sn, cs;
        __sincosf(ang, &sn, &cs);
        const float mag = exp2f((float)k * s.w);
        return cmul(make_float2(s.x, s.y), make_float2(cs * mag, sn * mag));
    }

    // TSTORE: the transposed store through a tensor map, in boxes of 4 kx x
    // 256 y (whole 32-byte sectors: boxes of 2 kx, 16-byte halves, measured
    // 2-5x slower).  The last stage writes the 4 rows of kx to shared memory
    // as [y][kx mod 4] (over the exchange rows, after a barrier) and one
    // thread stores the boxes: the LSU no longer carries 8 sectors of 8
    // different lines per warp store.
    //  - 4 rows or more per CTA (lengths 256 .. 2048: 8192 / N rows, boxes of
    //    that many kx): the CTA stages and stores all y.
    //  - 2 rows per CTA, clusters of 2: CTA c stages y in [c N/2, (c+1) N/2)
    //    of all 4 rows; each CTA writes its outputs into the owner's staging
    //    (distributed shared memory for the peer's half) between two cluster
    //    barriers (the owner's last-stage reads are done; the writes are
    //    complete), then each stores its half.
    // Full-size frames only (y0 = 0, ny_out = N, nx a multiple of 4).
    static constexpr int kBoxY = 256;
    template <int N>
    static constexpr bool tstore_ok() {
        constexpr int R = Shape<N, EPT, TT>::ROWS;
        return N % kBoxY == 0 && ((R >= 4 && R <= 32 && cluster<N>() == 1) || (R == 2 && cluster<N>() == 2 && (N / 2) % kBoxY == 0));
    }

    template <int N, bool RF>
    __device__ __forceinline__ void run(unsigned char *smem, int r, int j, const void *tmap = nullptr) const {
        using S = Shape<N, EPT, TT>;
        constexpr int ROWS = S::ROWS;
        constexpr int FORM = form<N, RF>();
        static_assert(!TSTORE || tstore_ok<N>(), "tensor-map store: 4..32 rows per CTA or 2 in a cluster of 2, N a multiple of 256");
        unsigned char *xbase = smem + stage_total<N, RF>();
        constexpr int CS = cluster<N>();
        // The CTAs of one row block (its `gridDim.y` slice groups) are consecutive
        // in launch order, so they run together and share its state rows in L2.
        // (In a cluster launch the members of a cluster must stay consecutive.)
        const int lin = blockIdx.y * gridDim.x + blockIdx.x;
        const int g = CS == 1 ? lin % gridDim.y : blockIdx.y;
        const int kx0 = (CS == 1 ? lin / gridDim.y : blockIdx.x) * ROWS;
        const int kx = kx0 + r;
        const bool valid = kx < nx;   // (CTAs that only pad a cluster hold no valid row)
        // (the single-call form never touches the item tables: indexing them by
        // blockIdx.z costs registers that the common path does not have)
        int group = this->group, b1max = nbatch;
        const float4 *state = this->state;
        float2 *t = this->t;
        if constexpr (GROUPED) {   // item z: its own slot of the scratch, slices and group
            const int z = (int)blockIdx.z;
            group = this->item_group(z);
            b1max = this->item_nb(z);
            state += (size_t)z * this->item_state_stride;
            t += (size_t)z * this->item_t_stride;
        }
        const int b0 = g * group;
        const int b1 = min(b0 + group, b1max);
        if (GROUPED && b0 >= b1) return;   // (an item with fewer slices; uniform over a cluster: shared z and g)
        const float4 *srow = state + (size_t)(valid ? kx : 0) * N;
        float2 *xs = nullptr, *hs = nullptr;
        if constexpr (FORM == FORM_CHAIN) {
            constexpr int XS = rec_stride<N, RF>();
            xs = reinterpret_cast<float2 *>(smem) + (size_t)r * XS;
            hs = reinterpret_cast<float2 *>(smem) + (size_t)(ROWS + r) * XS;
            const uint32_t kf = (uint32_t)(k0 + b0);
#pragma unroll
            for (int q = 0; q < S::E; ++q) {
                const int col = in_col<N, S::E>(j, q);   // the columns this thread's first stage reads
                float2 x = make_float2(0.0f, 0.0f), h = x;
                if (valid) {
                    const float4 st = srow[col];
                    x = direct(st, kf);
                    // Hdz itself: the accurate sin/cos, as its error grows along the chain
                    float sn, cs;
                    sincospif((float)(int32_t)__float_as_uint(st.z) * 4.656612873077392578125e-10f, &sn, &cs);
                    const float mag = exp2f(st.w);
                    h = make_float2(cs * mag, sn * mag);
                }
                xs[col] = x;
                hs[col] = h;
            }
        } else if constexpr (FORM == FORM_X0) {
            xs = reinterpret_cast<float2 *>(smem) + (size_t)r * rec_stride<N, RF>();
#pragma unroll
            for (int q = 0; q < S::E; ++q) {
                const int col = in_col<N, S::E>(j, q);   // the columns this thread's first stage reads
                xs[col] = valid ? *reinterpret_cast<const float2 *>(srow + col) : make_float2(0.0f, 0.0f);
            }
        } else if constexpr (FORM == FORM_STATE) {
            constexpr size_t SS = state_stride<N>();
            uint64_t *bar = reinterpret_cast<uint64_t *>(smem + ROWS * SS);
            if (threadIdx.x == 0) {
                mbar_init(bar, 1);
                mbar_fence_init();
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                const int nvalid = max(0, min(ROWS, nx - kx0));
                mbar_arrive_expect_tx(bar, (uint32_t)(nvalid * N * 16));
                for (int q = 0; q < nvalid; ++q)
                    bulk_g2s(smem + (size_t)q * SS, state + (size_t)(kx0 + q) * N, N * 16, bar);
            }
            mbar_wait(bar, 0, err);
            srow = reinterpret_cast<const float4 *>(smem + (size_t)r * SS);
        }
        float2 *xr = xrow<N, EPT, TT, RF>(xbase, r);
        if constexpr (CS > 1 && !TSTORE) cluster_arrive_relaxed();   // pairs with the first slice's wait
        for (int b = b0; b < b1; ++b) {
            const uint32_t k = (uint32_t)(k0 + b);
            float2 *tb = t + (size_t)b * ny_out * nx;
            auto load = [&](int, int ky) -> float2 {
                if constexpr (FORM == FORM_CHAIN) {
                    const float2 x = xs[ky];   // written by this thread only
                    xs[ky] = cmul(x, hs[ky]);
                    return x;
                } else if constexpr (FORM == FORM_X0) {
                    const float2 x0 = xs[ky];   // written by this thread only
                    const float2 pm = __ldg(reinterpret_cast<const float2 *>(srow + ky) + 1);
                    return direct(make_float4(x0.x, x0.y, pm.x, pm.y), k);
                } else {
                    return direct(srow[ky], k);
                }
            };
            if constexpr (TSTORE && CS == 2) {
                // stg: [y - rank N/2][4] for this CTA's half of y, over the exchange rows
                constexpr int YH = N / 2;
                constexpr int LAST_SYNC = 2 * (FftPlan<N, S::E>::NSTAGES - 1);   // the one before store()
                const uint32_t rank = cluster_ctarank();
                const uint32_t stg_own = smem_addr(xbase);
                const uint32_t stg_peer = map_to_rank(stg_own, rank ^ 1u);
                int nsync = 0;
                // First barrier: the previous slice's boxes have left the
                // staging.  Last: both CTAs have read their last stage's
                // inputs, so the staging (the peer's included) may be written.
                // Its arrival is relaxed: the butterfly has consumed every
                // value read, so the reads are complete (a release arrival
                // made `membar` the third stall of the capture).
                const auto sync = [&nsync]() {
                    const int i = nsync++;
                    if (i == 0 && threadIdx.x == 0) bulk_wait_read_all();
                    if (i == LAST_SYNC) {
                        cluster_arrive_relaxed();
                        cluster_wait();
                    } else {
                        __syncthreads();
                    }
                };
                fft_row_sync<N, S::E, true, false, true>(
                    xr, j, tw, load,
                    [&](int, int y, float2 v) {
                        const uint32_t owner = (uint32_t)(y / YH);
                        const uint32_t off = (uint32_t)((((y % YH) * 4) + (int)rank * ROWS + r) * 8);
                        if (owner == rank) {
                            st_shared_f2(stg_own + off, v);
                        } else {
                            st_cluster_f2(stg_peer + off, v);
                        }
                    },
                    sync);
                fence_proxy_async_cluster();   // the staging writes (local and remote), before the copy engine reads them
                cluster_sync();                // every write into this CTA's staging has landed
                if (threadIdx.x == 0) {
#pragma unroll 1
                    for (int q = 0; q < YH / kBoxY; ++q)
                        tma_store_3d(tmap, reinterpret_cast<const float2 *>(xbase) + (size_t)q * kBoxY * 4,
                                     kx0 - (int)rank * ROWS, (int)rank * YH + q * kBoxY, b);
                    bulk_commit();
                }
            } else if constexpr (TSTORE) {
                float2 *stg = reinterpret_cast<float2 *>(xbase);   // [y][ROWS], over the exchange rows
                int nsync = 0;
                // The first barrier of the transform precedes its first exchange
                // write: the previous slice's boxes must have left the staging.
                const auto sync = [&nsync]() {
                    if (nsync++ == 0 && threadIdx.x == 0) bulk_wait_read_all();
                    __syncthreads();
                };
                fft_row_sync<N, S::E, true, false, true>(
                    xr, j, tw, load, [&](int, int y, float2 v) { stg[y * ROWS + r] = v; }, sync);
                fence_proxy_async_smem();   // the staging writes, before the copy engine reads them
                if (threadIdx.x < 32) {
                    named_bar_sync(1, S::THREADS);
                    if (threadIdx.x == 0) {
#pragma unroll 1
                        for (int q = 0; q < N / kBoxY; ++q) {
                            if constexpr (GROUPED) {   // one map over the items' slots: (kx, y, slice, item)
                                tma_store_4d(tmap, stg + (size_t)q * kBoxY * ROWS, kx0, q * kBoxY, b,
                                             (int)blockIdx.z);
                            } else {
                                tma_store_3d(tmap, stg + (size_t)q * kBoxY * ROWS, kx0, q * kBoxY, b);
                            }
                        }
                        bulk_commit();
                    }
                } else {
                    named_bar_arrive(1, S::THREADS);
                }
            } else if constexpr (CS == 1) {
                fft_row<N, S::E, true>(xr, j, tw, load, [&](int, int y, float2 v) {
                    const int yo = y - y0;
                    // streaming store: T passes through L2 once
                    if (valid && yo >= 0 && yo < ny_out) __stcs(tb + (size_t)yo * nx + kx, v);
                });
            } else {
                // The first barrier of the transform (before its first exchange
                // write) waits for the cluster: the peers have read this CTA's
                // rows of the previous slice.  The last one (after the output
                // write) is the cluster barrier that follows.
                constexpr int LAST_SYNC = 2 * FftPlan<N, S::E>::NSTAGES - 1;
                int nsync = 0;
                const auto sync = [&nsync]() {
                    const int i = nsync++;
                    if (i == 0) cluster_wait();
                    else if (i != LAST_SYNC) __syncthreads();
                };
                fft_row_sync<N, S::E, true, true>(xr, j, tw, load, [](int, int, float2 v) -> float2 { return v; },
                                                  sync);
                cluster_sync();   // every CTA of the cluster holds its transformed rows
                constexpr int RS = S::template stride<RF>();
                constexpr int YS = N / CS;   // y range each CTA stores
                const uint32_t rank = cluster_ctarank();
                const int kxc = kx0 - (int)rank * ROWS;   // first of the cluster's 4 rows
                const uint32_t xsh = smem_addr(xbase);
#pragma unroll
                for (int i = 0; i < S::E; ++i) {
                    const int f = threadIdx.x + i * S::THREADS;
                    const int q = f & 3;
                    const int y = (int)rank * YS + (f >> 2);
                    const uint32_t a = xsh + (uint32_t)(((q % ROWS) * RS + spad(y)) * 8);
                    const float2 v = ld_cluster_f2(map_to_rank(a, (uint32_t)(q / ROWS)));
                    const int yo = y - y0;
                    if (kxc + q < nx && yo >= 0 && yo < ny_out) __stcs(tb + (size_t)yo * nx + kxc + q, v);
                }
                // This thread has read the cluster's rows of slice b: the stores
                // above consumed every loaded value, so the loads are complete
                // and the arrival orders nothing.  (A release arrival waited for
                // those global stores: 10 % slower at 4096.)
                cluster_arrive_relaxed();
            }
        }
        if constexpr (CS > 1 && !TSTORE) cluster_wait();   // no CTA leaves while a peer reads its rows
        if constexpr (TSTORE) {
            if (threadIdx.x == 0) bulk_wait_all();   // the shared memory outlives the last boxes' reads
        }
    }
};

using ReconA = ReconAT<false>;
using ReconATStore = ReconAT<false, true>;
using ReconAGrouped = ReconAT<true>;
using ReconAGroupedTStore = ReconAT<true, true>;

// ---------------------------------------------------------------- reconstruction pass B

enum Epilogue {
    EPI_PROJ = 0,      // running min / argmin -> packed atomicMin
    EPI_VOL = 1,       // clamp + convert -> vol (optionally the min of the stored values)
    EPI_CVOL = 2,      // complex slice -> vol
    EPI_SUB = 3        // N0f8 values inside given boxes -> their sub-volumes
};

// One sub-volume: fast range [fx0, fx1], slow range [sy0, sy1], slices
// [z0, z1] (0-based, inclusive), stored [z][slow][fast] at byte offset off.
struct SubBox {
    int fx0, fx1, sy0, sy1, z0, z1, nxb, nyb;
    long long off;
};

__device__ __forceinline__ float clamp01(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }

// Rows y of T, inverse FFT along kx, |u|^2 and the epilogue.  A CTA handles
// ROWS rows for `group` consecutive batch slots; with EPI_PROJ the running
// minimum stays in registers across them and is merged with one atomicMin of
// (float bits << 32 | slice) per pixel.  The rows of slice b+1 arrive in
// shared memory by bulk copy while slice b is transformed: two buffers, each
// first the bulk-copy target (dense rows) and then, after the first stage has
// read it, the exchange rows of that slice's transform.  CTAs are small (128
// threads: one row at N >= 2048) so that the barriers of the FFT stages span
// only the warps that exchange data, and RTS / 128 CTAs share an SM.
template <int EPI, bool GROUPED = false>   // GROUPED: the grouped-launch form (EPI_PROJ, grid z = item)
struct ReconB : PassBase, std::conditional_t<GROUPED, ReconItems, NoItems> {
    static constexpr int TT = 128;
    static constexpr int RTS = PH_RECONB_RTS;
    // 3 * 2^a lengths hold 24 values per thread and their running minima:
    // 168 registers, three CTAs per SM.  Per launch at 1536 and 3072 that is
    // 28 % faster than five CTAs at 96 registers (spilling ~480 bytes) and
    // 9-12 % faster than four at 128 (spilling ~150 bytes).
    template <int N>
    static constexpr int rts() { return plan_pow2(N) ? (GROUPED ? 512 : RTS) : 384; }   // (grouped: 128 registers, no spill)
    const float2 *t;                 // [batch][rows][nx]
    const float2 *tw;
    unsigned long long *proj64;      // [rows_out][nx_out] or null
    void *vol;                       // [S][rows_out][nx_out] or null
    int *err;                        // raised if a bulk-copy wait times out
    int vol_dtype;                   // PH_N0F8 .. PH_F64, or PH_BOOL: intensity <= threshold
    float threshold;
    const int *row_ptr;              // EPI_SUB: boxes of row y are row_box[row_ptr[y] .. row_ptr[y + 1])
    const int *row_box;
    const SubBox *boxes;
    int rows;                        // rows of T per slice
    int nx_out, x0;                  // stored columns [x0, x0 + nx_out)
    int k0, nbatch, group;
    long long vol_slice_stride;      // elements per stored slice

    // One buffer: the exchange rows (which also hold the dense bulk-copied rows).
    template <int N, bool RF>
    static constexpr size_t buf_bytes() {
        return (Shape<N, EPT, TT>::template smem_bytes<RF>() + 127) / 128 * 128;
    }
    // Staged when a row is a multiple of 16 bytes (bulk-copy granularity) and
    // two buffers fit the CTA's shared memory.
    template <int N, bool RF>
    static constexpr bool staged() {
        return N % 2 == 0 && 2 * buf_bytes<N, RF>() + 16 <= kSmemMax;
    }
    template <int N, bool RF>
    static constexpr size_t smem() {
        return staged<N, RF>() ? 2 * buf_bytes<N, RF>() + 16 : Shape<N, EPT, TT>::template smem_bytes<RF>();
    }

    template <int N, bool RF>
    __device__ __forceinline__ void run(unsigned char *smem, int r, int j) const {
        using S = Shape<N, EPT, TT>;
        constexpr int E = S::E;
        constexpr int ROWS = S::ROWS;
        constexpr size_t BB = buf_bytes<N, RF>();
        uint64_t *bars = reinterpret_cast<uint64_t *>(smem + 2 * BB);
        const int yb = blockIdx.x * ROWS;
        const int y = yb + r;
        const bool valid = y < rows;
        int group = this->group, b1max = nbatch;
        const float2 *t = this->t;
        unsigned long long *proj64 = this->proj64;
        if constexpr (GROUPED) {   // item z: its own slot of the scratch, slices and group
            const int z = (int)blockIdx.z;
            group = this->item_group(z);
            b1max = this->item_nb(z);
            t += (size_t)z * this->item_t_stride;
            proj64 += (size_t)z * this->p64_stride;
        }
        const int b0 = blockIdx.y * group;
        const int b1 = min(b0 + group, b1max);
        if (GROUPED && b0 >= b1) return;   // (an item with fewer slices)
        const int nvalid = min(ROWS, rows - yb);
        auto issue = [&](int b, int buf) {   // one thread: the rows of slice b into buffer buf
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(bars + buf, (uint32_t)(nvalid * N * 8));
            for (int q = 0; q < nvalid; ++q)
                bulk_g2s(smem + buf * BB + (size_t)q * N * 8, t + ((size_t)b * rows + yb + q) * N, N * 8, bars + buf);
        };
        if constexpr (staged<N, RF>()) {
            if (threadIdx.x == 0) {
                mbar_init(bars, 1);
                mbar_init(bars + 1, 1);
                mbar_fence_init();
            }
            __syncthreads();
            if (threadIdx.x == 0 && b0 < b1) issue(b0, 0);
        }
        uint32_t parity = 0;   // bit q: parity of the next completion of buffer q

        float minv[E];
        int mink[E];
#pragma unroll
        for (int s = 0; s < E; ++s) { minv[s] = __int_as_float(0x7f800000); mink[s] = 0; }
        const bool track_min = (EPI == EPI_PROJ) || (EPI == EPI_VOL && proj64 != nullptr);

        int sub_b = 0, sub_e = 0;   // EPI_SUB: this row's box list
        if constexpr (EPI == EPI_SUB) {
            if (valid) { sub_b = row_ptr[y]; sub_e = row_ptr[y + 1]; }
        }
        for (int b = b0; b < b1; ++b) {
            const int k = k0 + b;
            const int buf = (b - b0) & 1;
            const float2 *in;
            float2 *xr;
            if constexpr (staged<N, RF>()) {
                // every thread is done with the other buffer (slice b-1's last stage): refill it
                __syncthreads();
                if (threadIdx.x == 0 && b + 1 < b1) issue(b + 1, buf ^ 1);
                mbar_wait(bars + buf, (parity >> buf) & 1u, err);
                parity ^= 1u << buf;
                in = reinterpret_cast<const float2 *>(smem + buf * BB) + (size_t)r * N;
                xr = xrow<N, EPT, TT, RF>(smem + buf * BB, r);
            } else {
                in = t + ((size_t)b * rows + (valid ? y : 0)) * N;
                xr = xrow<N, EPT, TT, RF>(smem, r);
            }
            fft_row<N, E, true>(
                xr, j, tw, [&](int, int kx) -> float2 { return in[kx]; },
                [&](int slot, int x, float2 v) {
                    if constexpr (EPI == EPI_PROJ) {
                        const float i2 = fmaf(v.x, v.x, v.y * v.y);
                        if (i2 < minv[slot]) { minv[slot] = i2; mink[slot] = k; }
                    } else if constexpr (EPI == EPI_SUB) {
                        if (sub_b == sub_e) return;
                        const float i2 = clamp01(fmaf(v.x, v.x, v.y * v.y));
                        const uint8_t q = (uint8_t)__float2uint_rn(i2 * 255.0f);   // N0f8, as EPI_VOL
                        for (int i = sub_b; i < sub_e; ++i) {
                            const SubBox bx = boxes[row_box[i]];
                            if (k >= bx.z0 && k <= bx.z1 && x >= bx.fx0 && x <= bx.fx1)
                                reinterpret_cast<uint8_t *>(vol)[bx.off + ((long long)(k - bx.z0) * bx.nyb + (y - bx.sy0)) *
                                                                               bx.nxb + (x - bx.fx0)] = q;
                        }
                    } else {
                        const int xo = x - x0;
                        if (!valid || xo < 0 || xo >= nx_out) return;
                        const size_t o = (size_t)k * vol_slice_stride + (size_t)y * nx_out + xo;
                        if constexpr (EPI == EPI_CVOL) {
                            reinterpret_cast<float2 *>(vol)[o] = v;
                        } else {
                            const float i2 = clamp01(fmaf(v.x, v.x, v.y * v.y));
                            float stored;
                            switch (vol_dtype) {
                                case 0: {   // N0f8
                                    const unsigned q = __float2uint_rn(i2 * 255.0f);
                                    reinterpret_cast<uint8_t *>(vol)[o] = (uint8_t)q;
                                    stored = __fdiv_rn((float)q, 255.0f);
                                    break;
                                }
                                case 1: {
                                    const __half h = __float2half_rn(i2);
                                    reinterpret_cast<__half *>(vol)[o] = h;
                                    stored = __half2float(h);
                                    break;
                                }
                                case 3:
                                    reinterpret_cast<double *>(vol)[o] = (double)i2;
                                    stored = i2;
                                    break;
                                case 5:   // binary volume: the clamped Float32 intensity <= threshold
                                    reinterpret_cast<uint8_t *>(vol)[o] = i2 <= threshold ? 1 : 0;
                                    stored = i2;
                                    break;
                                default:
                                    reinterpret_cast<float *>(vol)[o] = i2;
                                    stored = i2;
                                    break;
                            }
                            if (track_min && stored < minv[slot]) { minv[slot] = stored; mink[slot] = k; }
                        }
                    }
                });
        }
        if (track_min && valid) {
#pragma unroll
            for (int s = 0; s < E; ++s) {
                const int x = out_col<N, E>(j, s);
                const int xo = x - x0;
                if (xo >= 0 && xo < nx_out && b1 > b0)
                    atomicMin(proj64 + (size_t)y * nx_out + xo, pack_min(minv[s], mink[s]));
            }
        }
    }
};

// ---------------------------------------------------------------- Gerchberg-Saxton / propagation

// Tensor-map stores of the persistent GS passes: boxes of ROWS x kGsBox,
// where a block holds 4 or 8 rows (whole 32-byte sectors or two) and the
// transform length is a multiple of kGsBox.
constexpr int kGsBox = 256;
template <int N>
constexpr bool gs_tstore_ok() {
    return (Shape<N>::ROWS == 4 || Shape<N>::ROWS == 8) && N % kGsBox == 0;
}

enum RowMode {
    ROW_MID = 0,      // inverse FFT -> amplitude replace -> forward FFT -> transposed store
    ROW_FINAL = 1,    // inverse FFT -> amplitude replace -> natural store
    ROW_INV = 2,      // inverse FFT -> natural store
};

// s / |u| where |u|^2 is not a normal, representable float: rhypotf (scaled);
// -1 for a zero field.  Out of line, so that the rare path takes no registers
// from the transforms around the common one.
static __device__ __noinline__ float amplitude_scale_slow(float2 u, float s) {
    if (u.x == 0.0f && u.y == 0.0f) return -1.0f;
    return rhypotf(u.x, u.y) * s;
}
// s u / |u|, and (s, 0) for u == 0 (angle(0) == 0).  1/|u| from the hardware
// reciprocal square root where |u|^2 is a normal, representable float (one
// test on the common path).
__device__ __forceinline__ float2 amplitude_replace(float2 u, float s) {
    const float n2 = fmaf(u.x, u.x, u.y * u.y);
    float k;
    if (__builtin_expect(n2 > 1e-36f && n2 < 1e36f, 1)) {
        k = rsqrtf(n2) * s;
    } else {
        k = amplitude_scale_slow(u, s);
        if (k < 0.0f) return make_float2(s, 0.0f);
    }
    return make_float2(u.x * k, u.y * k);
}

// Rows y of [y][kx] data (row length nx).
template <int MODE>
struct GsRow : PassBase {
    const float2 *src;       // [ny][nx]
    const float *holo;       // [ny][nx] intensity whose sqrt replaces the amplitude
    float2 *dst;             // MID: [nx][ny]; FINAL / INV: [ny][nx]
    const float2 *tw;
    double *resid;           // nullable: [0] += (|u| - s)^2, [1] += s^2
    int nrows;

    template <int N, bool RF>
    __device__ __forceinline__ void run(unsigned char *smem, int r, int j) const {
        using S = Shape<N, EPT, TT>;
        constexpr int E = S::E;
        float2 *srow = xrow<N, EPT, TT, RF>(smem, r);
        const int y = blockIdx.x * S::ROWS + r;
        const bool valid = y < nrows;
        const float2 *in = src + (size_t)(valid ? y : 0) * N;
        auto ld = [&](int, int x) -> float2 { return valid ? in[x] : make_float2(0.f, 0.f); };
        if constexpr (MODE == ROW_INV) {
            fft_row<N, E, true>(srow, j, tw, ld, [&](int, int x, float2 v) {
                if (valid) dst[(size_t)y * N + x] = v;
            });
        } else if constexpr (MODE == ROW_FINAL) {
            fft_row<N, E, true>(srow, j, tw, ld, [&](int, int x, float2 v) {
                if (valid) dst[(size_t)y * N + x] = amplitude_replace(v, sqrtf(holo[(size_t)y * N + x]));
            });
        } else {
            double acc0 = 0.0, acc1 = 0.0;
            // the amplitude replacement passes between the transforms in
            // registers (columns j + s P, as in GsRowMidT)
            float2 mid[E];
            fft_row<N, E, true>(srow, j, tw, ld, [&](int, int x, float2 v) {
                float2 w = make_float2(0.f, 0.f);
                if (valid) {
                    const float s = sqrtf(holo[(size_t)y * N + x]);
                    if (resid != nullptr) {
                        const double a = sqrt((double)v.x * v.x + (double)v.y * v.y) - (double)s;
                        acc0 += a * a;
                        acc1 += (double)s * s;
                    }
                    w = amplitude_replace(v, s);
                }
                mid[(x - j) / S::P] = w;
            });
            fft_row<N, E, false>(
                srow, j, tw, [&](int, int x) -> float2 { return mid[(x - j) / S::P]; },
                [&](int, int kx, float2 v) {
                    if (valid) dst[(size_t)kx * nrows + y] = v;
                });
            if (resid != nullptr) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    acc0 += __shfl_xor_sync(0xffffffffu, acc0, o);
                    acc1 += __shfl_xor_sync(0xffffffffu, acc1, o);
                }
                if ((threadIdx.x & 31) == 0) {
                    atomicAdd(resid, acc0);
                    atomicAdd(resid + 1, acc1);
                }
            }
        }
    }
};

// Rows kx of [kx][y] data (row length ny): forward FFT along y, times the
// centred transfer (and `scale`), inverse FFT along y, transposed store [y][kx].
// With `mask` (real, centred) instead of `h`, the multiplier is the mask.
struct GsCol : PassBase {
    const float2 *src;       // [nx][ny]
    const float2 *h;         // centred [ny][nx] (or null)
    const float *mask;       // centred [ny][nx] (or null)
    float2 *dst;             // [ny][nx]
    const float2 *tw;
    int nx;
    float scale;

    template <int N, bool RF>
    __device__ __forceinline__ void run(unsigned char *smem, int r, int j) const {
        using S = Shape<N, EPT, TT>;
        constexpr int E = S::E;
        float2 *srow = xrow<N, EPT, TT, RF>(smem, r);
        const int kx = blockIdx.x * S::ROWS + r;
        const bool valid = kx < nx;
        const int sx = valid ? shift_idx(kx, nx) : 0;
        const float2 *in = src + (size_t)(valid ? kx : 0) * N;
        // the product passes between the transforms in registers (this
        // thread's columns j + s P, as in GsColT)
        float2 mid[E];
        fft_row<N, E, false>(
            srow, j, tw, [&](int, int y) -> float2 { return valid ? in[y] : make_float2(0.f, 0.f); },
            [&](int, int ky, float2 v) {
                float2 w = make_float2(0.f, 0.f);
                if (valid) {
                    const size_t c = (size_t)shift_idx(ky, N) * nx + sx;
                    w = mask != nullptr ? cscale(v, mask[c] * scale) : cscale(cmul(v, h[c]), scale);
                }
                mid[(ky - j) / S::P] = w;
            });
        fft_row<N, E, true>(
            srow, j, tw, [&](int, int ky) -> float2 { return mid[(ky - j) / S::P]; },
            [&](int, int y, float2 v) {
                if (valid) dst[(size_t)y * nx + kx] = v;
            });
    }
};

// ---------------------------------------------------------------- staged Gerchberg-Saxton passes

// Row stride (elements) of a staged row of ROWS rows read rows-fastest across
// lanes: a multiple of 16 bytes, with consecutive rows 16/ROWS 8-byte words (or
// 32/ROWS 4-byte words) apart, so that the ROWS x (16/ROWS) lanes of an access
// phase fall on distinct banks.
template <int N, int ROWS, int ELEM>
constexpr int staged_stride() {
    return ELEM == 8 ? (N + 15) / 16 * 16 + (16 / ROWS) % 16 : (N + 31) / 32 * 32 + (32 / ROWS) % 32;
}

// Persistent form of the GS row pass with the transposed store (ROW_MID): each
// CTA walks row blocks rb = blockIdx.x, blockIdx.x + gridDim.x, ...; the field
// rows and hologram rows of the next block arrive by bulk copy into the second
// of two buffers while the current block is transformed.  A field buffer holds
// the dense rows at the exchange-row offsets, so the transform runs in place.
struct GsRowMidT : PassBase {
    const float2 *src;       // [ny][nx]
    const float *holo;       // [ny][nx] amplitudes sqrt(I), computed once per call
    float2 *dst;             // [nx][ny]
    const float2 *tw;
    double *resid;           // nullable: [0] += (|u| - s)^2, [1] += s^2
    int *err;                // raised if a bulk-copy wait times out
    int nrows;

    template <int N>
    using S = Shape<N, EPT, TT>;
    template <int N>
    static constexpr size_t fbytes() { return round128(S<N>::template smem_bytes<true>()); }
    template <int N>
    static constexpr size_t hbytes() { return round128((size_t)S<N>::ROWS * staged_stride<N, S<N>::ROWS, 4>() * 4); }
    template <int N>
    static constexpr size_t buf_bytes() { return fbytes<N>() + hbytes<N>(); }
    template <int N>
    static constexpr bool staged() {
        return S<N>::ROWS <= 8 && N % 4 == 0 && 2 * buf_bytes<N>() + 16 <= kSmemMax;
    }
    template <int N>
    static constexpr bool persistent() { return true; }
    template <int N>
    static constexpr bool pdl() { return true; }
    template <int N, bool RF>
    static constexpr size_t smem() { return 2 * buf_bytes<N>() + 16; }

    template <int N, bool RF>
    __device__ __forceinline__ void run(unsigned char *smem, int r, int j) const {
        run_blocks<N, RF, false, false>(smem, r, j, nullptr);
    }

    // The transposed store through a tensor map (gs_tstore_ok: 4 or 8 rows
    // per block, N a multiple of 256): the forward transform's outputs are
    // staged as [kx][y mod ROWS] over the block's field rows and one thread
    // stores them in boxes of ROWS y x 256 kx (whole 32-byte sectors), as in
    // pass A.  The buffer is refilled only after the copy engine has read it.
    // FINAL: the last plane-1 pass of a call: the inverse transform and the
    // amplitude replacement only, stored in natural order (dst = [ny][nx]).
    template <int N, bool RF, bool RESID, bool TS, bool FINAL = false>
    __device__ __forceinline__ void run_blocks(unsigned char *smem, int r, int j, const void *tmap) const {
        static_assert(RF, "rows-fastest launch");
        using SN = S<N>;
        constexpr int E = SN::E, ROWS = SN::ROWS;
        constexpr int FS = SN::template stride<true>();
        constexpr int HS = staged_stride<N, ROWS, 4>();
        constexpr size_t FB = fbytes<N>(), BUF = buf_bytes<N>();
        uint64_t *bars = reinterpret_cast<uint64_t *>(smem + 2 * BUF);
        const int nblocks = (nrows + ROWS - 1) / ROWS;
        auto issue = [&](int rb, int buf) {   // one thread: field and hologram rows of block rb
            const int yb = rb * ROWS, nv = min(ROWS, nrows - yb);
            unsigned char *base = smem + buf * BUF;
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(bars + buf, (uint32_t)(nv * N * 12));
            for (int q = 0; q < nv; ++q) {
                bulk_g2s(base + (size_t)q * FS * 8, src + (size_t)(yb + q) * N, N * 8, bars + buf);
                bulk_g2s(base + FB + (size_t)q * HS * 4, holo + (size_t)(yb + q) * N, N * 4, bars + buf);
            }
        };
        // every CTA of this persistent grid is resident: the next pass may be
        // scheduled onto the SMs this one leaves idle in its last round
        grid_dependents_launch();
        if (threadIdx.x == 0) {
            mbar_init(bars, 1);
            mbar_init(bars + 1, 1);
            mbar_fence_init();
        }
        __syncthreads();
        grid_dependency_wait();   // the previous pass wrote src and may still read dst
        if (threadIdx.x == 0 && (int)blockIdx.x < nblocks) issue(blockIdx.x, 0);
        uint32_t parity = 0;
        double acc0 = 0.0, acc1 = 0.0;
        int it = 0;
        for (int rb = blockIdx.x; rb < nblocks; rb += gridDim.x, ++it) {
            const int buf = it & 1;
            __syncthreads();   // every thread is done with the other buffer
            if (threadIdx.x == 0 && rb + (int)gridDim.x < nblocks) {
                if constexpr (TS) bulk_wait_read_all();   // the other buffer's staged outputs have left
                issue(rb + gridDim.x, buf ^ 1);
            }
            mbar_wait(bars + buf, (parity >> buf) & 1u, err);
            parity ^= 1u << buf;
            unsigned char *base = smem + buf * BUF;
            float2 *xr = reinterpret_cast<float2 *>(base) + (size_t)r * FS;
            const float *hr = reinterpret_cast<const float *>(base + FB) + (size_t)r * HS;
            const int y = rb * ROWS + r;
            const bool valid = y < nrows;
            const float2 *tw = opaque(this->tw);   // twiddles are re-read per block, not held in registers
            // The inverse transform's last stage leaves this thread the columns
            // j + s P (s < E), the very columns the forward transform's first
            // stage reads: the amplitude replacement passes between them in
            // registers.
            if constexpr (FINAL) {
                fft_row<N, E, true>(xr, j, tw, [&](int, int x) -> float2 { return xr[x]; },
                                    [&](int, int x, float2 v) {
                                        if (valid) dst[(size_t)y * N + x] = amplitude_replace(v, hr[x]);
                                    });
                continue;
            }
            float2 mid[E];
            fft_row<N, E, true>(xr, j, tw, [&](int, int x) -> float2 { return xr[x]; },
                                [&](int, int x, float2 v) {
                                    const float s = hr[x];
                                    if (RESID && valid) {
                                        const double a = sqrt((double)v.x * v.x + (double)v.y * v.y) - (double)s;
                                        acc0 += a * a;
                                        acc1 += (double)s * s;
                                    }
                                    mid[(x - j) / SN::P] = amplitude_replace(v, s);
                                });
            if constexpr (TS) {
                float2 *stg = reinterpret_cast<float2 *>(base);   // [kx][ROWS], over the field rows
                fft_row_sync<N, E, false, false, true>(
                    xr, j, tw, [&](int, int x) -> float2 { return mid[(x - j) / SN::P]; },
                    [&](int, int kx, float2 v) { stg[kx * ROWS + r] = v; }, CtaSync{});
                fence_proxy_async_smem();   // the staging writes, before the copy engine reads them
                if (threadIdx.x < 32) {
                    named_bar_sync(1, SN::THREADS);
                    if (threadIdx.x == 0) {
#pragma unroll 1
                        for (int q = 0; q < N / kGsBox; ++q)
                            tma_store_2d(tmap, stg + (size_t)q * kGsBox * ROWS, rb * ROWS, q * kGsBox);
                        bulk_commit();
                    }
                } else {
                    named_bar_arrive(1, SN::THREADS);
                }
            } else {
                fft_row<N, E, false>(xr, j, tw, [&](int, int x) -> float2 { return mid[(x - j) / SN::P]; },
                                     [&](int, int kx, float2 v) {
                                         if (valid) dst[(size_t)kx * nrows + y] = v;
                                     });
            }
        }
        if constexpr (TS) {
            if (threadIdx.x == 0) bulk_wait_all();   // the stores are complete before the grid is
        }
        if (RESID) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                acc0 += __shfl_xor_sync(0xffffffffu, acc0, o);
                acc1 += __shfl_xor_sync(0xffffffffu, acc1, o);
            }
            if ((threadIdx.x & 31) == 0) {
                atomicAdd(resid, acc0);
                atomicAdd(resid + 1, acc1);
            }
        }
    }
};

// The pass that also accumulates the GS residual (the last plane-2 pass of a
// call that asks for it): its own kernel, so that the FP64 accumulators do not
// enlarge the register budget of every other row pass.
struct GsRowMidTResid : GsRowMidT {
    template <int N, bool RF>
    __device__ __forceinline__ void run(unsigned char *smem, int r, int j) const {
        run_blocks<N, RF, true, false>(smem, r, j, nullptr);
    }
};
// The last plane-1 pass in the persistent form (natural store).
struct GsRowFinalT : GsRowMidT {
    template <int N, bool RF>
    __device__ __forceinline__ void run(unsigned char *smem, int r, int j) const {
        run_blocks<N, RF, false, false, true>(smem, r, j, nullptr);
    }
};
// The two forms with the tensor-map store (launched with the map of dst).
template <bool RESID>
struct GsRowMidTS : GsRowMidT {
    template <int N, bool RF>
    __device__ __forceinline__ void run(unsigned char *smem, int r, int j, const void *tmap) const {
        run_blocks<N, RF, RESID, true>(smem, r, j, tmap);
    }
};

// Persistent form of the GS column pass: rows kx of [kx][y] data, forward FFT
// along y, times ht[kx][ky] (the centred transfer rearranged to this layout,
// scale included), inverse FFT along y, transposed store [y][kx].  The field
// rows are double-buffered; the transfer rows of the next block are copied in
// once this block's multiply has read them.
struct GsColT : PassBase {
    static constexpr bool HT_EARLY = PH_HT_EARLY;
    const float2 *src;       // [nx][ny]
    const float2 *ht;        // [nx][ny]
    float2 *dst;             // [ny][nx]
    const float2 *tw;
    int *err;
    int nx;

    template <int N>
    using S = Shape<N, EPT, TT>;
    template <int N>
    static constexpr size_t fbytes() { return round128(S<N>::template smem_bytes<true>()); }
    template <int N>
    static constexpr size_t hbytes() { return round128((size_t)S<N>::ROWS * staged_stride<N, S<N>::ROWS, 8>() * 8); }
    template <int N>
    static constexpr bool staged() {
        return S<N>::ROWS <= 8 && N % 2 == 0 && 2 * fbytes<N>() + hbytes<N>() + 32 <= kSmemMax;
    }
    template <int N>
    static constexpr bool persistent() { return true; }
    template <int N>
    static constexpr bool pdl() { return true; }
    template <int N, bool RF>
    static constexpr size_t smem() {
        return 2 * fbytes<N>() + hbytes<N>() + 32 + tw_extra<N, S<N>::E>(2 * fbytes<N>() + hbytes<N>() + 32);
    }

    template <int N, bool RF>
    __device__ __forceinline__ void run(unsigned char *smem, int r, int j) const {
        run_impl<N, RF, false>(smem, r, j, nullptr);
    }

    // TS: the transposed store through a tensor map, as in GsRowMidT (the
    // inverse transform's outputs staged as [y][kx mod ROWS] over the block's
    // field rows, boxes of ROWS kx x 256 y).
    template <int N, bool RF, bool TS>
    __device__ __forceinline__ void run_impl(unsigned char *smem, int r, int j, const void *tmap) const {
        static_assert(RF, "rows-fastest launch");
        using SN = S<N>;
        constexpr int E = SN::E, ROWS = SN::ROWS;
        constexpr int FS = SN::template stride<true>();
        constexpr int HS = staged_stride<N, ROWS, 8>();
        constexpr size_t FB = fbytes<N>(), HB = hbytes<N>();
        unsigned char *hbase = smem + 2 * FB;
        uint64_t *bars = reinterpret_cast<uint64_t *>(hbase + HB);   // [0], [1] field buffers, [2] transfer
        // The stage twiddles in shared memory where they fit: 4.7 % faster at
        // 2048 than reading them through L1 (the row pass and pass A measured
        // slower with the same copy, so they read the table in global memory).
        constexpr size_t U = 2 * FB + HB + 32;
        constexpr bool TWS = tw_fits<N, E>(U);
        SmemTw<N> tws{nullptr};
        if constexpr (TWS) tws = stage_tw_to_smem<N, E>(reinterpret_cast<float2 *>(smem + round128(U)), tw);
        const int nblocks = (nx + ROWS - 1) / ROWS;
        auto issue_field = [&](int rb, int buf) {
            const int kb = rb * ROWS, nv = min(ROWS, nx - kb);
            unsigned char *base = smem + buf * FB;
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(bars + buf, (uint32_t)(nv * N * 8));
            for (int q = 0; q < nv; ++q)
                bulk_g2s(base + (size_t)q * FS * 8, src + (size_t)(kb + q) * N, N * 8, bars + buf);
        };
        auto issue_ht = [&](int rb) {
            const int kb = rb * ROWS, nv = min(ROWS, nx - kb);
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(bars + 2, (uint32_t)(nv * N * 8));
            for (int q = 0; q < nv; ++q)
                bulk_g2s(hbase + (size_t)q * HS * 8, ht + (size_t)(kb + q) * N, N * 8, bars + 2);
        };
        grid_dependents_launch();   // as in GsRowMidT
        if (threadIdx.x == 0) {
            mbar_init(bars, 1);
            mbar_init(bars + 1, 1);
            mbar_init(bars + 2, 1);
            mbar_fence_init();
        }
        __syncthreads();
        // the transfer rows come from an earlier kernel than the one this grid
        // depends on; the field rows (and the buffer written) only after it
        if (threadIdx.x == 0 && (int)blockIdx.x < nblocks) issue_ht(blockIdx.x);
        grid_dependency_wait();
        if (threadIdx.x == 0 && (int)blockIdx.x < nblocks) issue_field(blockIdx.x, 0);
        uint32_t parity = 0;   // bits 0, 1: field buffers; bit 2: transfer buffer
        int it = 0;
        for (int rb = blockIdx.x; rb < nblocks; rb += gridDim.x, ++it) {
            const int buf = it & 1;
            const int next = rb + gridDim.x;
            __syncthreads();   // every thread is done with the other field buffer
            if (threadIdx.x == 0 && next < nblocks) {
                if constexpr (TS) bulk_wait_read_all();   // the other buffer's staged outputs have left
                issue_field(next, buf ^ 1);
            }
            if (!HT_EARLY && threadIdx.x == 0 && it > 0) issue_ht(rb);
            mbar_wait(bars + buf, (parity >> buf) & 1u, err);
            parity ^= 1u << buf;
            mbar_wait(bars + 2, (parity >> 2) & 1u, err);
            parity ^= 4u;
            float2 *xr = reinterpret_cast<float2 *>(smem + buf * FB) + (size_t)r * FS;
            const float2 *hr = reinterpret_cast<const float2 *>(hbase) + (size_t)r * HS;
            const int kx = rb * ROWS + r;
            const bool valid = kx < nx;
            auto go = [&](const auto twv) {
                // The forward transform's last stage leaves this thread the columns
                // j + s P (s < E), the very columns the inverse transform's first
                // stage reads: the product with the transfer passes between them
                // in registers.
                float2 mid[E];
                fft_row<N, E, false>(xr, j, twv, [&](int, int y) -> float2 { return xr[y]; },
                                     [&](int, int ky, float2 v) { mid[(ky - j) / SN::P] = cmul(v, hr[ky]); });
                int nsync = 0;
                const auto sync = [&]() {
                    __syncthreads();
                    // first barrier of the inverse transform: every thread has read
                    // the transfer rows, so the next block's may come in
                    if (nsync++ == 0 && HT_EARLY && threadIdx.x == 0 && next < nblocks) issue_ht(next);
                };
                if constexpr (TS) {
                    float2 *stg = reinterpret_cast<float2 *>(smem + buf * FB);   // [y][ROWS], over the field rows
                    fft_row_sync<N, E, true, false, true>(
                        xr, j, twv, [&](int, int ky) -> float2 { return mid[(ky - j) / SN::P]; },
                        [&](int, int y, float2 v) { stg[y * ROWS + r] = v; }, sync);
                    fence_proxy_async_smem();   // the staging writes, before the copy engine reads them
                    if (threadIdx.x < 32) {
                        named_bar_sync(1, SN::THREADS);
                        if (threadIdx.x == 0) {
#pragma unroll 1
                            for (int q = 0; q < N / kGsBox; ++q)
                                tma_store_2d(tmap, stg + (size_t)q * kGsBox * ROWS, rb * ROWS, q * kGsBox);
                            bulk_commit();
                        }
                    } else {
                        named_bar_arrive(1, SN::THREADS);
                    }
                } else {
                    fft_row_sync<N, E, true>(xr, j, twv,
                                             [&](int, int ky) -> float2 { return mid[(ky - j) / SN::P]; },
                                             [&](int, int y, float2 v) {
                                                 if (valid) dst[(size_t)y * nx + kx] = v;
                                             },
                                             sync);
                }
            };
            if constexpr (TWS) go(tws);
            else go(opaque(this->tw));   // twiddles are re-read per block, not held in registers
        }
        if constexpr (TS) {
            if (threadIdx.x == 0) bulk_wait_all();   // the stores are complete before the grid is
        }
    }
};
struct GsColTS : GsColT {
    template <int N, bool RF>
    __device__ __forceinline__ void run(unsigned char *smem, int r, int j, const void *tmap) const {
        run_impl<N, RF, true>(smem, r, j, tmap);
    }
};

}  // namespace ph
