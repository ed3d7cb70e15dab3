// ph_pass_tc.cuh -- the split-precision tensor-core form of reconstruction
// pass B: rows y of the slice intermediate T, inverse DFT along kx as two
// small complex DFT GEMMs on the 5th-generation tensor cores, |u|^2 and the
// running min / argmin per pixel.
//
// Length N = N1 N2 (N1, N2 in {32, 64}).  With n = n1 + N1 n2 and
// k = k2 + N2 k1 (W_m = exp(+2 pi i / m), the inverse transform):
//   GEMM 1   Y[n1][k2]  = sum_n2 x[n1 + N1 n2] W_N2^(n2 k2)      (DFT-N2 per n1)
//   twiddle  Y'[n1][k2] = Y[n1][k2] W_N^(n1 k2)                    (CUDA cores, FP32)
//   GEMM 3   X[k2 + N2 k1] = sum_n1 Y'[n1][k2] W_N1^(n1 k1)        (DFT-N1 per k2)
// Complex products are real GEMMs over interleaved (re, im): the data row
// (re, im, re, im ...) is the A operand, K-major, and the DFT matrix F becomes
// the real B operand [2k + c'][2n + c] = [[Fr, -Fi], [Fi, Fr]] so that
// D[m][2k] = Re(x F), D[m][2k + 1] = Im(x F).
//
// Split precision: every operand v is held as v_hi + v_lo (16-bit each, v_hi =
// round(v), v_lo = round(v - v_hi)) and a product is accumulated in FP32 from
// A_hi B_hi + A_lo B_hi + A_hi B_lo (TERMS = 3; A_lo B_lo is below FP32
// rounding) or from A_hi B_hi + A_lo B_hi (TERMS = 2: the matrix in one 16-bit
// word).  BF16 keeps FP32's exponent range; FP16 has 3 more significant bits
// per word and a tile is scaled by a power of two so that its largest value
// is at most 2^9 (GEMM 1 grows it by at most N2 sqrt 2 < 2^15.5, inside FP16).
//
// A CTA (384 threads, one per SM: 225 KB of shared memory at N = 2048) owns
// ROWS = 128 / N2 consecutive rows y and walks the slices of its group; one
// tile is those rows of one slice.  GEMM 1 takes 128 / N1 rows per MMA chain
// (HALVES chains per tile), GEMM 3 the whole tile.  Warp roles and the
// pipeline between them are described at k_recon_b_tc.
//
// Tables (built on the host in FP64, copied in one bulk copy per CTA): B1 and
// B3 as swizzled K-major tiles (hi, then lo when TERMS = 3), then the twiddles
// W_N^(n1 k2) as FP32 complex [k2][n1].
#pragma once

#include <cuda_fp16.h>
#include "ph_common.cuh"
#include "ph_tc.cuh"

namespace ph {

enum TcForm { TC_FP32 = 0, TC_BF16X3 = 1, TC_FP16X3 = 2, TC_FP16X2 = 3 };

__host__ __device__ constexpr bool tc_form_fp16(int form) { return form == TC_FP16X3 || form == TC_FP16X2; }
__host__ __device__ constexpr int tc_form_terms(int form) { return form == TC_FP16X2 ? 2 : 3; }

template <int N1_, int N2_, int FORM_>
struct TcPlan {
    static constexpr int N1 = N1_, N2 = N2_, N = N1 * N2, FORM = FORM_;
    static constexpr bool FP16 = tc_form_fp16(FORM);
    static constexpr int TERMS = tc_form_terms(FORM);
    static constexpr int BTERMS = TERMS == 3 ? 2 : 1;          // matrix words: hi (+ lo)
    static constexpr int K1 = 2 * N2, NN1 = 2 * N2;            // GEMM 1: K, N (real)
    static constexpr int K3 = 2 * N1, NN3 = 2 * N1;            // GEMM 3: K, N (real)
    static constexpr int ROWS1 = 128 / N1;                     // rows per GEMM 1 chain
    static constexpr int ROWS = 128 / N2;                      // rows per tile
    static constexpr int HALVES = ROWS / ROWS1;                // GEMM 1 chains per tile
    static constexpr int THREADS = 384;                      // 8 consumer + 4 producer warps
    // shared-memory layout (bytes; every tile on a 1024-byte boundary)
    static constexpr uint32_t B1_BYTES = tc::sw128_bytes(NN1, K1);
    static constexpr uint32_t B3_BYTES = tc::sw128_bytes(NN3, K3);
    static constexpr uint32_t A1_BYTES = tc::sw128_bytes(128, K1);   // one chain, one word
    static constexpr uint32_t A3_BYTES = tc::sw128_bytes(128, K3);
    static constexpr uint32_t TW_BYTES = (uint32_t)N * 8;
    static constexpr uint32_t OFF_B1 = 0;
    static constexpr uint32_t OFF_B3 = OFF_B1 + BTERMS * B1_BYTES;
    static constexpr uint32_t OFF_TW = OFF_B3 + BTERMS * B3_BYTES;
    static constexpr uint32_t TABLE_BYTES = OFF_TW + TW_BYTES;        // the global image
    static constexpr uint32_t OFF_A1 = (TABLE_BYTES + 1023) / 1024 * 1024;
    static constexpr uint32_t OFF_A3 = OFF_A1 + 2 * HALVES * A1_BYTES;  // hi, lo per chain
    static constexpr uint32_t OFF_BAR = OFF_A3 + 2 * A3_BYTES;
    static constexpr uint32_t SMEM = OFF_BAR + 256 + 1024;             // + alignment slack
    // two buffers each of D1 (HALVES x NN1 columns) and D3 (NN3 columns)
    static constexpr uint32_t D1_COLS = HALVES * NN1, D3_COLS = NN3;
    static constexpr uint32_t TMEM_COLS = 2 * (D1_COLS + D3_COLS) <= 256 ? 256 : 512;
    static_assert(2 * (D1_COLS + D3_COLS) <= TMEM_COLS, "tensor memory");
    static_assert(N1 % 32 == 0 && N2 % 32 == 0 && N1 <= 64 && N2 <= 64, "N1, N2 in {32, 64}");
    static_assert(SMEM <= 227 * 1024, "shared memory");
    // epilogue: each of the two warps on a lane quarter takes half of D3's columns
    static constexpr int PIX = N1 / 2;                                  // pixels per thread
};

struct ReconBTc {
    const float2 *t;                 // [batch][rows][n]
    const unsigned char *table;      // TcPlan::TABLE_BYTES, 16-byte aligned
    unsigned long long *proj64;      // [rows][n]
    int *err;
    int rows, k0, nbatch, group;
};

// 16-bit words of (x0, x1) in the form's type: hi and lo.
template <bool FP16>
__device__ __forceinline__ void split2(float x0, float x1, uint32_t &hi, uint32_t &lo) {
    if constexpr (FP16) {
        tc::split_f16x2(x0, x1, hi, lo);
    } else {
        tc::split_bf16x2(x0, x1, hi, lo);
    }
}

// Warp roles (384 threads): warps 0-7 are the consumers (8 warps, two per
// tensor-memory lane quarter), warps 8-11 the producers.  D1 and D3 each have
// two tensor-memory buffers (tile b uses buffer b & 1).
//   producers, tile b:  wait GEMM 1 (b-1) done (A1 free) -> load + split the
//                       rows of slice b into A1 -> barrier -> one thread waits
//                       until the consumers have read D1 buffer (b & 1) of
//                       tile b-2, issues GEMM 1 (b) into it
//   consumers, tile b:  wait GEMM 1 (b) done, and GEMM 3 (b-1) done (A3 free)
//                       -> twiddle + split D1 -> A3 -> release that D1 buffer
//                       -> barrier -> one thread issues GEMM 3 (b) -> reduce
//                       tile b-1 (|D3|^2 -> running minimum) while it runs
// so the global loads of tile b + 1 and the reduction of tile b - 1 overlap
// the tensor pipe.  Hand-offs are mbarriers: GEMM 1 completion (one barrier
// per D1 buffer: GEMM 1 (b + 1) may finish before the consumers wait for
// GEMM 1 (b)), GEMM 3 completion (tcgen05.commit), each D1 buffer released
// (256 consumer arrivals; one barrier per buffer) and, for the FP16 forms, the row scales of a tile (128
// producer arrivals; a ring of four barriers and scale slots, as the producers
// run at most two tiles ahead).  No waiter falls two phases behind a barrier.
// Every wait is bounded.
constexpr int kTcConsumers = 256, kTcProducers = 128;

template <class PL>
__global__ void __launch_bounds__(384, 1) k_recon_b_tc(const ReconBTc p) {
    constexpr int N = PL::N, N1 = PL::N1, N2 = PL::N2;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *smem =
        reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    // barriers: [0] tables, [1], [2] GEMM 1 done per D1 buffer, [3] GEMM 3 done, [4], [5] D1 buffer
    // released, [6..9] row scales
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + PL::OFF_BAR);
    constexpr int G1 = 1, G3 = 3, D1R = 4, SC = 6;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + 10);
    float *rmax = reinterpret_cast<float *>(bars + 11);         // [4 producer warps] per-warp row maxima
    float *rscale = rmax + 4;                                    // [4][ROWS] per-row scales (FP16 forms)
    const float2 *tw = reinterpret_cast<const float2 *>(smem + PL::OFF_TW);

    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const bool producer = warp >= 8;
    const int yb = blockIdx.x * PL::ROWS;
    const int b0 = blockIdx.y * p.group;
    const int b1 = min(b0 + p.group, p.nbatch);
    if (b0 >= b1) return;

    if (warp == 0) tc::tmem_alloc(tslot, PL::TMEM_COLS);
    if (t == 0) {
        mbar_init(bars + 0, 1);
        mbar_init(bars + G1, 1);
        mbar_init(bars + G1 + 1, 1);
        mbar_init(bars + G3, 1);
        mbar_init(bars + D1R, kTcConsumers);
        mbar_init(bars + D1R + 1, kTcConsumers);
        for (int q = 0; q < 4; ++q) mbar_init(bars + SC + q, kTcProducers);
        mbar_fence_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    auto d1 = [&](int b) { return tmem + (uint32_t)(b & 1) * PL::D1_COLS; };                       // tile b's D1
    auto d3 = [&](int b) { return tmem + 2 * PL::D1_COLS + (uint32_t)(b & 1) * PL::D3_COLS; };   // tile b's D3
    if (t == 0) {
        mbar_arrive_expect_tx(bars + 0, PL::TABLE_BYTES);
        for (uint32_t o = 0; o < PL::TABLE_BYTES; o += 65536u) {
            const uint32_t sz = PL::TABLE_BYTES - o < 65536u ? PL::TABLE_BYTES - o : 65536u;
            bulk_g2s(smem + o, p.table + o, sz, bars + 0);
        }
    }
    const volatile int *errv = p.err;
    mbar_wait(bars + 0, 0, p.err);                         // tables in shared memory

    if (producer) {
        // ---------------------------------------------------------- producers
        const int pt = t - kTcConsumers, pw = pt >> 5;
        const int m1 = pt;                                 // A1 row of every chain
        const int r1 = m1 / N1, n1 = m1 % N1;
        const uint32_t tile_bytes = (uint32_t)(min(PL::ROWS, p.rows - yb) * N * 8);
        uint32_t ph1 = 0, phd = 0;                         // parity bits per buffer
        for (int b = b0; b < b1; ++b) {
            if (b > b0) {                                  // GEMM 1 (b - 1) has read A1
                const int q = (b - 1) & 1;
                mbar_wait(bars + G1 + q, (ph1 >> q) & 1u, p.err);
                ph1 ^= 1u << q;
            }
            if (pt == 0 && b + 2 < b1) tc::prefetch_l2(p.t + ((size_t)(b + 2) * p.rows + yb) * N, tile_bytes);
#pragma unroll 1
            for (int h = 0; h < PL::HALVES; ++h) {
                const int row1 = h * PL::ROWS1 + r1;
                const bool valid = yb + row1 < p.rows;
                const float2 *src = p.t + ((size_t)b * p.rows + (valid ? yb + row1 : 0)) * N;
                float2 v[N2];
#pragma unroll
                for (int i = 0; i < N2; ++i) v[i] = valid ? __ldcs(src + n1 + N1 * i) : make_float2(0.f, 0.f);
                if constexpr (PL::FP16) {
                    // per-row power-of-two scale: the row's largest value at most 2^9
                    float mx = 0.0f;
#pragma unroll
                    for (int i = 0; i < N2; ++i) mx = fmaxf(mx, fmaxf(fabsf(v[i].x), fabsf(v[i].y)));
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
                    constexpr int WPR = N1 / 32;           // producer warps per row
                    if (WPR > 1) {
                        if (lane == 0) rmax[pw] = mx;
                        asm volatile("bar.sync 1, %0;" ::"r"(kTcProducers) : "memory");
                        mx = fmaxf(rmax[pw & ~1], rmax[pw | 1]);
                        asm volatile("bar.sync 1, %0;" ::"r"(kTcProducers) : "memory");
                    }
                    int e = 0;
                    frexpf(mx, &e);
                    const float sc = mx > 0.0f ? ldexpf(1.0f, 9 - e) : 1.0f;
                    if (n1 == 0) rscale[(b & 3) * PL::ROWS + row1] = sc;
#pragma unroll
                    for (int i = 0; i < N2; ++i) v[i] = make_float2(v[i].x * sc, v[i].y * sc);
                }
                unsigned char *ahi = smem + PL::OFF_A1 + (2 * h) * PL::A1_BYTES;
                unsigned char *alo = ahi + PL::A1_BYTES;
#pragma unroll
                for (int i = 0; i < N2; i += 4) {
                    uint4 hv, lv;
                    split2<PL::FP16>(v[i].x, v[i].y, hv.x, lv.x);
                    split2<PL::FP16>(v[i + 1].x, v[i + 1].y, hv.y, lv.y);
                    split2<PL::FP16>(v[i + 2].x, v[i + 2].y, hv.z, lv.z);
                    split2<PL::FP16>(v[i + 3].x, v[i + 3].y, hv.w, lv.w);
                    const uint32_t off = tc::sw128_offset(128, m1, 2 * i);
                    *reinterpret_cast<uint4 *>(ahi + off) = hv;
                    *reinterpret_cast<uint4 *>(alo + off) = lv;
                }
            }
            if constexpr (PL::FP16) mbar_arrive(bars + SC + (b & 3));  // this tile's row scales are written
            fence_proxy_async_smem();
            // every producer has written A1; stop together if any wait anywhere gave up
            const bool stop = bar_sync_or(1, kTcProducers, *errv != 0);
            if (stop) break;
            if (pt == 0) {
                if (b >= b0 + 2) {                         // the consumers have read this D1 buffer (tile b - 2)
                    const int q = b & 1;
                    mbar_wait(bars + D1R + q, (phd >> q) & 1u, p.err);
                    phd ^= 1u << q;
                }
                tc::fence_after_sync();
                constexpr uint32_t idesc = tc::idesc_f16(128, PL::NN1, !PL::FP16);
#pragma unroll
                for (int h = 0; h < PL::HALVES; ++h) {
                    const uint32_t ahi = smem_addr(smem + PL::OFF_A1 + (2 * h) * PL::A1_BYTES);
                    const uint32_t alo = ahi + PL::A1_BYTES;
                    const uint32_t bhi = smem_addr(smem + PL::OFF_B1);
                    const uint32_t blo = bhi + PL::B1_BYTES;
                    const uint32_t d = d1(b) + (uint32_t)(h * PL::NN1);
#pragma unroll
                    for (int s = 0; s < PL::K1 / 16; ++s) {
                        const uint32_t oa = (uint32_t)((s >> 2) * 128 * 128 + (s & 3) * 32);
                        const uint32_t ob = (uint32_t)((s >> 2) * PL::NN1 * 128 + (s & 3) * 32);
                        tc::mma_f16(d, tc::desc_sw128(ahi + oa), tc::desc_sw128(bhi + ob), idesc, s > 0);
                        tc::mma_f16(d, tc::desc_sw128(alo + oa), tc::desc_sw128(bhi + ob), idesc, true);
                        if constexpr (PL::TERMS == 3)
                            tc::mma_f16(d, tc::desc_sw128(ahi + oa), tc::desc_sw128(blo + ob), idesc, true);
                    }
                }
                tc::mma_commit(bars + G1 + (b & 1));
            }
        }
    } else {
        // ---------------------------------------------------------- consumers
        const int quarter = warp & 3;                      // tensor-memory lane quarter
        // twiddle + split: D1 lane m of chain h -> A3 rows N2 R + k2, K 2 n1 + c
        constexpr int WPQ1 = 2 / PL::HALVES;
        const int h1 = PL::HALVES == 2 ? (warp >> 2) : 0;
        const int m1 = quarter * 32 + lane;
        const int r1 = m1 / N1, n1 = m1 % N1;
        const int row1 = h1 * PL::ROWS1 + r1;
        constexpr int K2W = N2 / WPQ1;
        const int k2a = PL::HALVES == 2 ? 0 : (warp >> 2) * K2W;
        // reduction: D3 lane m3 = N2 R + k2, this warp's half of the columns
        const int m3 = quarter * 32 + lane;
        const int row3 = m3 / N2, k2e = m3 % N2;
        const int k1a = (warp >> 2) * PL::PIX;
        const bool valid3 = yb + row3 < p.rows;
        float minv[PL::PIX];
        int mink[PL::PIX];
#pragma unroll
        for (int i = 0; i < PL::PIX; ++i) { minv[i] = __int_as_float(0x7f800000); mink[i] = 0; }
        // |D3|^2 of tile b (in its buffer) into the running minimum
        auto reduce = [&](int b, float inv_s2) {
            const int k = p.k0 + b;
            const uint32_t taddr = d3(b) + (uint32_t)(2 * k1a) + ((uint32_t)(quarter * 32) << 16);
#pragma unroll
            for (int c = 0; c < PL::PIX; c += 16) {
                float v[32];
                tc::tmem_ld32(taddr + (uint32_t)(2 * c), v);
                tc::tmem_wait_ld();
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    float i2 = fmaf(v[2 * i], v[2 * i], v[2 * i + 1] * v[2 * i + 1]);
                    if constexpr (PL::FP16) i2 *= inv_s2;
                    if (i2 < minv[c + i]) { minv[c + i] = i2; mink[c + i] = k; }
                }
            }
        };
        uint32_t ph1 = 0, ph3 = 0, phs = 0;               // parity bits per barrier of a ring
        float inv_prev = 1.0f;                             // 1 / scale^2 of tile b - 1 (FP16 forms)
        bool stopped = false;
        for (int b = b0; b < b1; ++b) {
            mbar_wait(bars + G1 + (b & 1), (ph1 >> (b & 1)) & 1u, p.err);   // GEMM 1 (b) done: D1 (b) ready
            ph1 ^= 1u << (b & 1);
            float inv_s2 = 1.0f;
            if constexpr (PL::FP16) {
                mbar_wait(bars + SC + (b & 3), (phs >> (b & 3)) & 1u, p.err);
                phs ^= 1u << (b & 3);
                const float sc = rscale[(b & 3) * PL::ROWS + row3];
                inv_s2 = 1.0f / (sc * sc);
            }
            if (b > b0) {                                  // GEMM 3 (b - 1) done: A3 free, D3 (b - 1) ready
                mbar_wait(bars + G3, ph3, p.err);
                ph3 ^= 1u;
            }
            tc::fence_after_sync();
            {
                unsigned char *ahi = smem + PL::OFF_A3;
                unsigned char *alo = ahi + PL::A3_BYTES;
                const uint32_t taddr = d1(b) + (uint32_t)(h1 * PL::NN1) + ((uint32_t)(quarter * 32) << 16);
#pragma unroll
                for (int c = 0; c < K2W; c += 16) {        // 16 k2 = 32 columns per load
                    float v[32];
                    tc::tmem_ld32(taddr + (uint32_t)(2 * (k2a + c)), v);
                    tc::tmem_wait_ld();
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        const int k2 = k2a + c + i;
                        const float2 w = tw[k2 * N1 + n1];
                        const float2 y = cmul(make_float2(v[2 * i], v[2 * i + 1]), w);
                        uint32_t hw, lw;
                        split2<PL::FP16>(y.x, y.y, hw, lw);
                        const uint32_t off = tc::sw128_offset(128, N2 * row1 + k2, 2 * n1);
                        *reinterpret_cast<uint32_t *>(ahi + off) = hw;
                        *reinterpret_cast<uint32_t *>(alo + off) = lw;
                    }
                }
            }
            tc::fence_before_sync();
            mbar_arrive(bars + D1R + (b & 1));             // D1 buffer (b & 1) read: GEMM 1 (b + 2) may write it
            fence_proxy_async_smem();
            const bool stop = bar_sync_or(2, kTcConsumers, *errv != 0);   // a uniform decision
            tc::fence_after_sync();
            if (stop) {
                stopped = true;
                break;
            }
            if (t == 0) {
                constexpr uint32_t idesc = tc::idesc_f16(128, PL::NN3, !PL::FP16);
                const uint32_t ahi = smem_addr(smem + PL::OFF_A3);
                const uint32_t alo = ahi + PL::A3_BYTES;
                const uint32_t bhi = smem_addr(smem + PL::OFF_B3);
                const uint32_t blo = bhi + PL::B3_BYTES;
                const uint32_t d = d3(b);
#pragma unroll
                for (int s = 0; s < PL::K3 / 16; ++s) {
                    const uint32_t oa = (uint32_t)((s >> 2) * 128 * 128 + (s & 3) * 32);
                    const uint32_t ob = (uint32_t)((s >> 2) * PL::NN3 * 128 + (s & 3) * 32);
                    tc::mma_f16(d, tc::desc_sw128(ahi + oa), tc::desc_sw128(bhi + ob), idesc, s > 0);
                    tc::mma_f16(d, tc::desc_sw128(alo + oa), tc::desc_sw128(bhi + ob), idesc, true);
                    if constexpr (PL::TERMS == 3)
                        tc::mma_f16(d, tc::desc_sw128(ahi + oa), tc::desc_sw128(blo + ob), idesc, true);
                }
                tc::mma_commit(bars + G3);
            }
            if (b > b0) reduce(b - 1, inv_prev);           // while GEMM 3 (b) runs
            inv_prev = inv_s2;
            tc::fence_before_sync();
        }
        if (!stopped) {
            mbar_wait(bars + G3, ph3, p.err);              // GEMM 3 of the last tile
            tc::fence_after_sync();
            reduce(b1 - 1, inv_prev);
            tc::fence_before_sync();
        }
        if (valid3) {
            unsigned long long *out = p.proj64 + (size_t)(yb + row3) * N;
#pragma unroll
            for (int i = 0; i < PL::PIX; ++i) atomicMin(out + k2e + N2 * (k1a + i), pack_min(minv[i], mink[i]));
        }
    }
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, PL::TMEM_COLS);
}

}  // namespace ph
