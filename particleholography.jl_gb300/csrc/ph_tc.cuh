// ph_tc.cuh -- 5th-generation tensor cores (tcgen05) as inline PTX for sm_103a:
// tensor-memory allocation, shared-memory matrix descriptors, the MMA issue and
// its completion barrier, and tensor-memory loads.
//
// Operand layout used throughout: K-major tiles with the 128-byte swizzle.
// A tile of R rows (M or N) by K 16-bit elements is stored as K/64 blocks;
// block kb holds every row's elements [64 kb, 64 kb + 64) as one 128-byte line
// per row, 8 rows per 1024-byte swizzle atom, and within an atom the 16-byte
// chunk c of row r sits at chunk position c ^ (r mod 8).  Every block starts on
// a 1024-byte boundary.  The descriptor of one MMA's K step (16 elements, 32
// bytes) points at the block's base plus 32 bytes per step; the hardware
// applies the swizzle to the absolute address bits.
//
// Accumulators (FP32) live in tensor memory: for M = 128 and one CTA, row m of
// D is lane m and column n of D is column (base + n).  Warp w of the CTA reads
// lanes [32 (w mod 4), 32 (w mod 4) + 32).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include "ph_tma.cuh"

namespace ph {
namespace tc {

// ---------------------------------------------------------------- operand tiles

// Byte offset of element (row, k) in a K-major, 128-byte-swizzled tile of
// `rows` rows (rows a multiple of 8).
__host__ __device__ constexpr uint32_t sw128_offset(int rows, int row, int k) {
    return (uint32_t)((k >> 6) * rows * 128 + (row >> 3) * 1024 + (row & 7) * 128 +
                      ((((k & 63) >> 3) ^ (row & 7)) << 4) + ((k & 7) << 1));
}
// Bytes of such a tile.
__host__ __device__ constexpr uint32_t sw128_bytes(int rows, int k) { return (uint32_t)(rows * k * 2); }

// Shared-memory matrix descriptor (K-major, 128-byte swizzle): start address,
// stride between 8-row groups (1024 bytes), version 1, layout type 2.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);          // bits 0-13: start address >> 4
    d |= (uint64_t)(16u >> 4) << 16;                   // bits 16-29: leading byte offset (unused here)
    d |= (uint64_t)(1024u >> 4) << 32;                 // bits 32-45: stride byte offset
    d |= (uint64_t)1 << 46;                            // bits 46-47: descriptor version
    d |= (uint64_t)2 << 61;                            // bits 61-63: 128-byte swizzle
    return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, A and B both BF16
// (bf16 = true) or both FP16, both K-major, shape M x N.
__host__ __device__ constexpr uint32_t idesc_f16(int m, int n, bool bf16) {
    return (1u << 4)                                    // D format: F32
         | ((bf16 ? 1u : 0u) << 7)                      // A format
         | ((bf16 ? 1u : 0u) << 10)                     // B format
         | ((uint32_t)(n >> 3) << 17)                   // N >> 3
         | ((uint32_t)(m >> 4) << 24);                  // M >> 4
}

// ---------------------------------------------------------------- tensor memory

// One warp allocates `ncols` columns (a power of two, 32..512) and writes the
// base address to *slot (shared memory); the permit to allocate is given up
// at once, so that co-resident CTAs can allocate.
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
// The allocating warp frees the columns.
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ---------------------------------------------------------------- MMA

// D (tensor memory) = A B^T (+ D when accumulate): A [M][K], B [N][K] from
// shared-memory descriptors.  Issued by one thread.
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                        bool accumulate) {
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "setp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate ? 1u : 0u)
        : "memory");
}

// The barrier receives one arrival once every MMA this thread issued before
// has completed (its shared-memory reads and tensor-memory writes).
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_addr(bar))
                 : "memory");
}

// ---------------------------------------------------------------- tensor-memory loads

// 16 consecutive 32-bit columns of this thread's lane (32x32b shape): every
// thread of the warp calls it with the warp's lane-quarter base in taddr.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
// 32 consecutive columns in one load.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Asks the copy engine to bring [src, src + bytes) into L2 (no completion to
// wait for).  src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void prefetch_l2(const void *src, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// ---------------------------------------------------------------- split precision

// x ~ hi + lo with hi = bf16(x) and lo = bf16(x - hi): about 16 significant
// bits.  Returns the pairs packed for (x0, x1).
__device__ __forceinline__ void split_bf16x2(float x0, float x1, uint32_t &hi, uint32_t &lo) {
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(hi) : "f"(x1), "f"(x0));
    const float h0 = __uint_as_float(hi << 16);
    const float h1 = __uint_as_float(hi & 0xFFFF0000u);
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(lo) : "f"(x1 - h1), "f"(x0 - h0));
}
// The same with FP16 (11 significant bits each, about 22 together): the
// caller keeps x in FP16's range by a power-of-two scale.
__device__ __forceinline__ void split_f16x2(float x0, float x1, uint32_t &hi, uint32_t &lo) {
    asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(hi) : "f"(x1), "f"(x0));
    float h0, h1;
    asm("{\n.reg .f16 a, b;\nmov.b32 {a, b}, %2;\ncvt.f32.f16 %0, a;\ncvt.f32.f16 %1, b;\n}" : "=f"(h0), "=f"(h1)
        : "r"(hi));
    asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(lo) : "f"(x1 - h1), "f"(x0 - h0));
}

}  // namespace tc
}  // namespace ph
