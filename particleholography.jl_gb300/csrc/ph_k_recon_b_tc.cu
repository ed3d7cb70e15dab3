// ph_k_recon_b_tc.cu -- the split-precision tensor-core pass B (ph_pass_tc.cuh):
// host-built tables and the launcher.
#include "ph_pass_tc.cuh"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cmath>
#include <cstring>

namespace ph {

namespace {

// The plan of a supported length: N = N1 N2 with N1 >= N2 (GEMM 3, the
// N1-point DFT, has the larger K and N).  At 4096 (64 x 64) the operand tiles
// and tables of the three-product forms need 288 KB of shared memory, more
// than a CTA has: 4096 stays on the FP32 pass.
template <class F>
bool with_plan(int n, int form, F &&f) {
    switch (form) {
        case TC_BF16X3:
            if (n == 1024) return f(TcPlan<32, 32, TC_BF16X3>{}), true;
            if (n == 2048) return f(TcPlan<64, 32, TC_BF16X3>{}), true;
            return false;
        case TC_FP16X3:
            if (n == 1024) return f(TcPlan<32, 32, TC_FP16X3>{}), true;
            if (n == 2048) return f(TcPlan<64, 32, TC_FP16X3>{}), true;
            return false;
        case TC_FP16X2:
            if (n == 1024) return f(TcPlan<32, 32, TC_FP16X2>{}), true;
            if (n == 2048) return f(TcPlan<64, 32, TC_FP16X2>{}), true;
            return false;
    }
    return false;
}

// 16-bit word of v (nearest) in the form's type, and its value.
uint16_t to16(double v, bool fp16, double *back) {
    if (fp16) {
        const __half h = __float2half_rn((float)v);
        *back = (double)__half2float(h);
        uint16_t u;
        memcpy(&u, &h, 2);
        return u;
    }
    const __nv_bfloat16 h = __float2bfloat16_rn((float)v);
    *back = (double)__bfloat162float(h);
    uint16_t u;
    memcpy(&u, &h, 2);
    return u;
}

// The real form of the inverse M-point DFT matrix as a K-major swizzled tile
// [2k + c'][2n + c] (hi words at hi, lo words at lo when lo is not null).
void put_dft(unsigned char *hi, unsigned char *lo, int m, bool fp16) {
    const int rows = 2 * m;
    for (int k = 0; k < m; ++k) {
        for (int n = 0; n < m; ++n) {
            const long long j = ((long long)n * k) % m;
            const double a = 2.0 * 3.14159265358979323846 * (double)j / (double)m;
            const double c = std::cos(a), s = std::sin(a);
            const double e[2][2] = {{c, -s}, {s, c}};   // [c'][c]
            for (int co = 0; co < 2; ++co) {
                for (int ci = 0; ci < 2; ++ci) {
                    double hv = 0.0, lv = 0.0;
                    const uint16_t wh = to16(e[co][ci], fp16, &hv);
                    const uint16_t wl = to16(e[co][ci] - hv, fp16, &lv);
                    const uint32_t off = tc::sw128_offset(rows, 2 * k + co, 2 * n + ci);
                    memcpy(hi + off, &wh, 2);
                    if (lo != nullptr) memcpy(lo + off, &wl, 2);
                }
            }
        }
    }
}

}  // namespace

bool recon_b_tc_supported(int n, int form) {
    return with_plan(n, form, [](auto) {});
}

size_t recon_b_tc_table_bytes(int n, int form) {
    size_t b = 0;
    with_plan(n, form, [&](auto pl) { b = decltype(pl)::TABLE_BYTES; });
    return b;
}

int recon_b_tc_rows(int n, int form) {
    int r = 0;
    with_plan(n, form, [&](auto pl) { r = decltype(pl)::ROWS; });
    return r;
}

// Fills the table image (recon_b_tc_table_bytes bytes) in FP64: the two DFT
// matrices split into hi (+ lo) words and the twiddles W_N^(n1 k2) as FP32.
void recon_b_tc_build_table(int n, int form, unsigned char *img) {
    with_plan(n, form, [&](auto pl) {
        using PL = decltype(pl);
        memset(img, 0, PL::TABLE_BYTES);
        put_dft(img + PL::OFF_B1, PL::BTERMS == 2 ? img + PL::OFF_B1 + PL::B1_BYTES : nullptr, PL::N2, PL::FP16);
        put_dft(img + PL::OFF_B3, PL::BTERMS == 2 ? img + PL::OFF_B3 + PL::B3_BYTES : nullptr, PL::N1, PL::FP16);
        float *tw = reinterpret_cast<float *>(img + PL::OFF_TW);
        for (int k2 = 0; k2 < PL::N2; ++k2) {
            for (int n1 = 0; n1 < PL::N1; ++n1) {
                const long long j = ((long long)n1 * k2) % PL::N;
                const double a = 2.0 * 3.14159265358979323846 * (double)j / (double)PL::N;
                tw[2 * (k2 * PL::N1 + n1)] = (float)std::cos(a);
                tw[2 * (k2 * PL::N1 + n1) + 1] = (float)std::sin(a);
            }
        }
    });
}

cudaError_t launch_recon_b_tc(int n, int form, const ReconBTc &p, cudaStream_t s) {
    cudaError_t err = cudaErrorInvalidValue;
    with_plan(n, form, [&](auto pl) {
        using PL = decltype(pl);
        auto kern = k_recon_b_tc<PL>;
        static unsigned long long done_mask = 0;   // per-device opt-in to the shared memory
        int dev = 0;
        cudaGetDevice(&dev);
        const unsigned long long bit = 1ull << (dev & 63);
        if (!(__atomic_load_n(&done_mask, __ATOMIC_ACQUIRE) & bit)) {
            err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PL::SMEM);
            if (err != cudaSuccess) return;
            __atomic_fetch_or(&done_mask, bit, __ATOMIC_ACQ_REL);
        }
        const int gx = (p.rows + PL::ROWS - 1) / PL::ROWS;
        const int gy = (p.nbatch + p.group - 1) / p.group;
        if (gx == 0 || gy == 0) {
            err = cudaSuccess;
            return;
        }
        kern<<<dim3(gx, gy), PL::THREADS, PL::SMEM, s>>>(p);
        err = cudaGetLastError();
    });
    return err;
}

}  // namespace ph
