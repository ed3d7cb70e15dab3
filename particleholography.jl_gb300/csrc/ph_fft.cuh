// ph_fft.cuh -- the row-FFT engine every pass kernel is built from.
//
// A CTA transforms ROWS rows of length N at once.  Each row is handled by
// P = N/E threads; each thread keeps E complex values in registers and runs
// radix-E Stockham stages (radix LAST for the trailing stage when N is not a
// power of E).  Stages exchange data through one padded shared-memory row per
// transformed row.  The first stage reads its inputs through a caller-supplied
// `load(slot, col)` and the last stage hands its outputs to `store(slot, col,
// v)`, so the caller fuses its prologue (transfer multiply, padding, amplitude
// replacement ...) and epilogue (transposed store, |u|^2, min/argmin, clamp
// and convert ...) into the transform's first and last register stages.
//
// Stockham stage s (radix R, Ns = product of the earlier radices), butterfly b
// in [0, N/R):   inputs  x[b + r N/R]                     r = 0..R-1
//               twiddle  x_r *= W_{Ns R}^{r (b mod Ns)}
//               outputs  y[(b/Ns) Ns R + (b mod Ns) + r Ns]
// Thread j owns butterflies b = j + m P, m = 0..E/R-1.  In the first and last
// stage the thread's elements sit at columns b + r N/R (strided by P), which
// keeps global accesses coalesced across the threads of a row.
#pragma once

#include "ph_common.cuh"

namespace ph {

// Radix plan of a length-N transform with E values per thread.  N is a power
// of two (radix-E stages, then a smaller power-of-two radix) or three times a
// power of two (E = 3 E2: radix-E2 stages, a smaller power-of-two radix, and a
// final radix-3 stage, so every stage before the last has a power-of-two
// span).  Every radix divides E.  The plan is written as constexpr functions
// of (N, E) so that the host code laying out the twiddle table follows the
// same plan as the device engine.
__host__ __device__ constexpr bool plan_pow2(int n) { return (n & (n - 1)) == 0; }
__host__ __device__ constexpr int plan_r2(int n, int e) { return plan_pow2(n) ? e : e / 3; }
__host__ __device__ constexpr int plan_nfull(int n, int e) {
    return ilog2c(plan_r2(n, e)) == 0 ? 0 : ilog2c(plan_pow2(n) ? n : n / 3) / ilog2c(plan_r2(n, e));
}
__host__ __device__ constexpr int plan_last(int n, int e) {   // trailing power-of-two radix (1 = none)
    return 1 << (ilog2c(plan_pow2(n) ? n : n / 3) - plan_nfull(n, e) * ilog2c(plan_r2(n, e)));
}
__host__ __device__ constexpr int plan_nstages(int n, int e) {
    return plan_nfull(n, e) + (plan_last(n, e) > 1 ? 1 : 0) + (plan_pow2(n) ? 0 : 1);
}
__host__ __device__ constexpr int plan_radix(int n, int e, int s) {
    return s < plan_nfull(n, e) ? plan_r2(n, e) : ((plan_last(n, e) > 1 && s == plan_nfull(n, e)) ? plan_last(n, e) : 3);
}
__host__ __device__ constexpr int plan_ns(int n, int e, int s) {   // product of the radices before stage s
    int v = 1;
    for (int t = 0; t < s; ++t) v *= plan_radix(n, e, t);
    return v;
}
// Twiddle table layout: W_N^i for i in [0, N), then for every stage s >= 1 a
// block of (R - 1) x NS twiddles, entry [r - 1][k] = W_N^(r k N / (NS R)).  A
// stage's lanes (consecutive butterflies, consecutive k) read consecutive
// entries of one block row.
__host__ __device__ constexpr int plan_tw_offset(int n, int e, int s) {
    int off = n;
    for (int t = 1; t < s; ++t) off += (plan_radix(n, e, t) - 1) * plan_ns(n, e, t);
    return off;
}
__host__ __device__ constexpr int plan_tw_size(int n, int e) { return plan_tw_offset(n, e, plan_nstages(n, e)); }

template <int N, int E>
struct FftPlan {
    static constexpr bool POW2 = plan_pow2(N);
    static_assert(N >= 1 && (POW2 || ((N % 3) == 0 && ((N / 3) & (N / 3 - 1)) == 0)), "N must be 2^a or 3*2^a");
    static_assert(E >= 1 && E <= N && N % E == 0, "E must divide N");
    static constexpr int P = N / E;                       // threads per row
    static constexpr int NFULL = plan_nfull(N, E);
    static constexpr int LAST = plan_last(N, E);
    static constexpr int NSTAGES = plan_nstages(N, E);
    template <int S>
    __host__ __device__ static constexpr int radix() { return plan_radix(N, E, S); }
    template <int S>
    __host__ __device__ static constexpr int ns() { return plan_ns(N, E, S); }
    template <int S>
    __host__ __device__ static constexpr int tw_offset() { return plan_tw_offset(N, E, S); }
};

// Input q-th consumed by dft<R>: the split radices (R = P x Q, see dft_split)
// read inputs Q*n1 + n2 with n2 outer and n1 inner.
template <int R>
__host__ __device__ constexpr int dft_input_order(int q) {
    return R == 16 ? 4 * (q % 4) + q / 4
         : R == 8  ? 4 * (q % 2) + q / 2
         : R == 32 ? 8 * (q % 4) + q / 4
         : R == 64 ? 8 * (q % 8) + q / 8
                   : q;
}

// Shared-memory index of column i of a row: one pad element per 16 keeps the
// strided stage writes free of bank conflicts.
__device__ __forceinline__ int spad(int i) { return i + (i >> 4); }

// Row stride (in float2) of the shared buffer.  A half-warp of 8-byte accesses
// covers `rows` rows x `jc` consecutive columns (ROW_FAST: rows fastest; else
// columns fastest).  Offsetting each row by jc (mod 16) banks puts the rows of a
// half-warp on disjoint bank pairs.
template <int N, int ROWS, int P, bool ROW_FAST>
struct SmemRow {
    static constexpr int PADDED = N + (N >> 4);
    static constexpr int JC = ROW_FAST ? 16 / (ROWS < 16 ? ROWS : 16) : (P < 16 ? P : 16);
    static constexpr int STRIDE = ((PADDED + 15) / 16) * 16 + (JC % 16);
};

// Twiddle table entry i (layout above) for the forward transform, or its
// conjugate for the inverse.
template <bool INV>
__device__ __forceinline__ float2 load_tw(const float2 *__restrict__ tw, int i) {
    float2 w = __ldg(tw + i);
    if (INV) w.y = -w.y;
    return w;
}

// The stage blocks of the table (entries [B, size), B = N: all that the stages
// read) copied to shared memory; p[0] holds entry B.
template <int B>
struct SmemTw {
    const float2 *p;
};
template <bool INV, int B>
__device__ __forceinline__ float2 load_tw(const SmemTw<B> &tw, int i) {
    float2 w = tw.p[i - B];
    if (INV) w.y = -w.y;
    return w;
}
template <int N, int E>
constexpr size_t stage_tw_bytes() {
    return ((size_t)(plan_tw_size(N, E) - plan_tw_offset(N, E, 1)) * 8 + 127) / 128 * 128;
}
// Every thread of the CTA calls this; the copy is visible after the next CTA barrier.
template <int N, int E>
__device__ __forceinline__ SmemTw<N> stage_tw_to_smem(float2 *dst, const float2 *__restrict__ tw) {
    constexpr int B = plan_tw_offset(N, E, 1);
    constexpr int C = plan_tw_size(N, E) - B;
    for (int i = threadIdx.x; i < C; i += blockDim.x) dst[i] = __ldg(tw + B + i);
    return SmemTw<N>{dst};
}

// Value the OUT_SMEM variant writes to shared memory: the store callback's result.
template <bool OUT_SMEM, class Store>
__device__ __forceinline__ float2 smem_out_value(Store &store, int slot, int col, float2 v) {
    if constexpr (OUT_SMEM) {
        return store(slot, col, v);
    } else {
        return v;
    }
}

// Barriers of the engine: the whole CTA, or only the P threads (whole warps)
// that transform one row, with a named barrier per row.
struct CtaSync {
    __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
struct RowSync {
    int id;      // 1..15 (0 is the CTA barrier)
    int count;   // threads of the row, a multiple of 32
    __device__ __forceinline__ void operator()() const {
        asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
    }
};

// Runs one length-N transform per row.  Every thread that `sync` covers must
// call it.  `srow` is this thread's shared row.
//
//   tw:    the twiddle table (global pointer) or its stage blocks in shared memory (SmemTw)
//   Load:  float2 load(int slot, int col)   -- slot = m*R0 + r (compile-time after unrolling)
//   Store: void store(int slot, int col, float2 v)
//   OUT_SMEM: write the outputs to srow (after an internal barrier) and call
//             store() first so it may transform the value; ends with a barrier.
//             store() must then RETURN the value to write: float2 store(slot, col, v).
//   STORE_SYNC: (without OUT_SMEM) a barrier between the last stage's reads of
//             srow and the store() calls, which may then write shared memory
//             that other threads' last-stage inputs occupied.
template <int N, int E, bool INV, bool OUT_SMEM = false, bool STORE_SYNC = false, class Tw, class Load,
          class Store, class Sync>
__device__ __forceinline__ void fft_row_sync(float2 *__restrict__ srow, int j, const Tw tw, Load &&load,
                                             Store &&store, const Sync &sync) {
    using PL = FftPlan<N, E>;
    constexpr int P = PL::P;
    float2 v[E];

    if constexpr (PL::NSTAGES == 0) {
        // N == 1: identity transform.
        v[0] = load(0, 0);
        if constexpr (OUT_SMEM) {
            sync();
            srow[0] = store(0, 0, v[0]);
            sync();
        } else {
            store(0, 0, v[0]);
        }
        return;
    } else {
        static_for<PL::NSTAGES>([&](auto SI) {
            constexpr int S = decltype(SI)::value;
            constexpr int R = PL::template radix<S>();
            constexpr int NS = PL::template ns<S>();
            constexpr int M = E / R;              // butterflies per thread in this stage
            constexpr int STRIDE_IN = N / R;
            constexpr bool FIRST = (S == 0);
            constexpr bool LASTSTAGE = (S == PL::NSTAGES - 1);

            // ---- gather inputs, in the order the butterfly consumes them
#pragma unroll
            for (int m = 0; m < M; ++m) {
                const int b = j + m * P;
#pragma unroll
                for (int q = 0; q < R; ++q) {
                    const int r = dft_input_order<R>(q);
                    const int col = b + r * STRIDE_IN;
                    if constexpr (FIRST) {
                        v[m * R + r] = load(m * R + r, col);
                    } else {
                        v[m * R + r] = srow[spad(col)];
                    }
                }
            }
            // ---- twiddle + butterfly
#pragma unroll
            for (int m = 0; m < M; ++m) {
                const int b = j + m * P;
                float2 t[R];
#pragma unroll
                for (int r = 0; r < R; ++r) t[r] = v[m * R + r];
                if constexpr (NS > 1) {
                    const int k = b & (NS - 1);
                    constexpr int TOFF = PL::template tw_offset<S>();
#pragma unroll
                    for (int q = 0; q < R; ++q) {
                        const int r = dft_input_order<R>(q);
                        if (r > 0) t[r] = cmul(t[r], load_tw<INV>(tw, TOFF + (r - 1) * NS + k));
                    }
                }
                dft<R, INV>(t);
#pragma unroll
                for (int r = 0; r < R; ++r) v[m * R + r] = t[r];
            }
            // ---- scatter outputs
            if constexpr (LASTSTAGE && !OUT_SMEM) {
                if constexpr (STORE_SYNC) sync();
#pragma unroll
                for (int m = 0; m < M; ++m) {
                    const int b = j + m * P;   // last stage: (b / NS) == 0, out = b + r*NS
#pragma unroll
                    for (int r = 0; r < R; ++r) store(m * R + r, b + r * NS, v[m * R + r]);
                }
            } else {
                sync();   // every thread has read this stage's inputs
#pragma unroll
                for (int m = 0; m < M; ++m) {
                    const int b = j + m * P;
                    const int base = (b / NS) * NS * R + (b & (NS - 1));
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        const int col = base + r * NS;
                        if constexpr (LASTSTAGE) {
                            srow[spad(col)] = smem_out_value<OUT_SMEM>(store, m * R + r, col, v[m * R + r]);
                        } else {
                            srow[spad(col)] = v[m * R + r];
                        }
                    }
                }
                sync();
            }
        });
    }
}

// The transform with CTA-wide barriers.
template <int N, int E, bool INV, bool OUT_SMEM = false, class Tw, class Load, class Store>
__device__ __forceinline__ void fft_row(float2 *__restrict__ srow, int j, const Tw tw, Load &&load, Store &&store) {
    fft_row_sync<N, E, INV, OUT_SMEM>(srow, j, tw, load, store, CtaSync{});
}

// Column of output slot `slot` (= m*R + r of the last stage) for thread j.
template <int N, int E>
__device__ __forceinline__ int out_col(int j, int slot) {
    using PL = FftPlan<N, E>;
    if constexpr (PL::NSTAGES == 0) {
        return 0;
    } else {
        constexpr int R = PL::template radix<PL::NSTAGES - 1>();
        constexpr int NS = PL::template ns<PL::NSTAGES - 1>();
        const int m = slot / R, r = slot % R;
        return j + m * PL::P + r * NS;
    }
}

// Column of input slot `slot` (= m*R0 + r of the first stage) for thread j.
template <int N, int E>
__device__ __forceinline__ int in_col(int j, int slot) {
    using PL = FftPlan<N, E>;
    if constexpr (PL::NSTAGES == 0) {
        return 0;
    } else {
        constexpr int R = PL::template radix<0>();
        const int m = slot / R, r = slot % R;
        return j + m * PL::P + r * (N / R);
    }
}

}  // namespace ph
