// ph_tc_check.cu -- ph_tc_selftest: one tensor-core product D = A B^T through
// the same operand layout, descriptors, MMA issue, completion barrier and
// tensor-memory loads as the split-precision transform passes, so that a
// caller can check the tensor path of a device against a host product.
#include "phgb300.h"

#include <cuda_runtime.h>

#include "ph_tc.cuh"

namespace {

using namespace ph;

constexpr int kM = 128;

// One CTA of 128 threads: A [128][k], B [n][k] (BF16 or FP16 bits, row-major,
// K contiguous) into swizzled tiles, k/16 MMAs into tensor memory, D [128][n]
// (FP32) back to global memory.  n in {16, 32, ..., 256}, k a multiple of 64,
// n * k <= 128 * 128.
__global__ void __launch_bounds__(128, 1)
    k_tc_selftest(float *d, const uint16_t *a, const uint16_t *b, int n, int k, int fp16, int *err) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *smem = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                            ~uintptr_t(1023));
    unsigned char *ta = smem;                                   // 128 x k
    unsigned char *tb = smem + tc::sw128_bytes(kM, 128);        // n x k (room for 128 x 128)
    uint64_t *bar = reinterpret_cast<uint64_t *>(tb + tc::sw128_bytes(256, 64));
    uint32_t *slot = reinterpret_cast<uint32_t *>(bar + 1);
    const int t = threadIdx.x;
    const int warp = t >> 5;
    uint32_t ncols = 32;
    while ((int)ncols < n) ncols <<= 1;
    if (warp == 0) tc::tmem_alloc(slot, ncols);
    if (t == 0) {
        mbar_init(bar, 1);
        mbar_fence_init();
    }
    for (int i = t; i < kM * k; i += blockDim.x) {
        const int row = i / k, kk = i % k;
        *reinterpret_cast<uint16_t *>(ta + tc::sw128_offset(kM, row, kk)) = a[i];
    }
    for (int i = t; i < n * k; i += blockDim.x) {
        const int row = i / k, kk = i % k;
        *reinterpret_cast<uint16_t *>(tb + tc::sw128_offset(n, row, kk)) = b[i];
    }
    fence_proxy_async_smem();   // the operand writes, before the tensor core reads them
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *slot;
    if (t == 0) {
        const uint32_t idesc = tc::idesc_f16(kM, n, fp16 == 0);
        for (int s = 0; s < k / 16; ++s) {
            const uint32_t off_a = (uint32_t)((s >> 2) * kM * 128 + (s & 3) * 32);
            const uint32_t off_b = (uint32_t)((s >> 2) * n * 128 + (s & 3) * 32);
            tc::mma_f16(tmem, tc::desc_sw128(smem_addr(ta + off_a)), tc::desc_sw128(smem_addr(tb + off_b)), idesc,
                        s > 0);
        }
        tc::mma_commit(bar);
    }
    mbar_wait(bar, 0, err);
    tc::fence_after_sync();
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    const int row = t;   // warp w reads lanes 32w .. 32w + 31
    for (int c = 0; c < n; c += 16) {
        float v[16];
        tc::tmem_ld16(tmem + lane_base + (uint32_t)c, v);
        tc::tmem_wait_ld();
#pragma unroll
        for (int i = 0; i < 16; ++i) d[(size_t)row * n + c + i] = v[i];
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

}  // namespace

extern "C" int32_t ph_tc_selftest(float *d, const uint16_t *a, const uint16_t *b, int32_t n, int32_t k,
                                  int32_t fp16, int32_t *err, void *stream) {
    if (d == nullptr || a == nullptr || b == nullptr || err == nullptr) return PH_ERR_INVALID;
    if (n < 16 || n > 128 || n % 16 != 0 || k < 64 || k % 64 != 0 || n * k > 128 * 128 || k > 128)
        return PH_ERR_SIZE;
    const size_t smem = 1024 + tc::sw128_bytes(kM, 128) + tc::sw128_bytes(256, 64) + 64;
    cudaError_t e = cudaFuncSetAttribute(k_tc_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return PH_ERR_CUDA;
    k_tc_selftest<<<1, 128, smem, static_cast<cudaStream_t>(stream)>>>(d, a, b, n, k, fp16, err);
    return cudaGetLastError() == cudaSuccess ? PH_OK : PH_ERR_CUDA;
}
