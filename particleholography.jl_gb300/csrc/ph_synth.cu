// ph_synth.cu -- kernels of the seeded synthetic-hologram generator: opaque
// disc masks, |psi|^2 with min/max reduction, normalisation plus noise.
// The propagation between disc planes uses the library's own FFT passes with
// FP64-phase transfer functions (see ph_synth_hologram in ph_api.cu).
#include <cstdint>
#include <cuda_runtime.h>

namespace ph {

// psi *= (1 - A): zero the pixels whose centre (ix dx, iy dx) lies in the disc.
__global__ void k_disc_mask(float2 *psi, int nx, int ny, double cx, double cy, double r, double dx, int x0, int y0,
                            int w, int h) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w * h) return;
    const int x = x0 + i % w, y = y0 + i / w;
    if (x < 0 || x >= nx || y < 0 || y >= ny) return;
    const double ddx = x * dx - cx, ddy = y * dx - cy;
    if (ddx * ddx + ddy * ddy <= r * r) psi[(size_t)y * nx + x] = make_float2(0.f, 0.f);
}

__global__ void k_fill_one(float2 *psi, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) psi[i] = make_float2(1.f, 0.f);
}

__device__ __forceinline__ void atomic_min_f(float *a, float v) {   // v >= 0
    atomicMin(reinterpret_cast<int *>(a), __float_as_int(v));
}
__device__ __forceinline__ void atomic_max_f(float *a, float v) {
    atomicMax(reinterpret_cast<int *>(a), __float_as_int(v));
}

// out = |psi|^2 and the running min / max (non-negative floats order like ints).
__global__ void k_intensity_minmax(const float2 *psi, float *out, size_t n, float *mm) {
    float lo = __int_as_float(0x7f800000), hi = 0.f;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float2 v = psi[i];
        const float in = v.x * v.x + v.y * v.y;
        out[i] = in;
        lo = fminf(lo, in);
        hi = fmaxf(hi, in);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomic_min_f(mm, lo);
        atomic_max_f(mm + 1, hi);
    }
}

__global__ void k_normalise_noise(float *out, const float *noise, size_t n, const float *mm) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float lo = mm[0], hi = mm[1];
    const float scale = hi > lo ? 1.0f / (hi - lo) : 0.0f;
    float v = (out[i] - lo) * scale;
    if (noise) v = fmaxf(v + noise[i], 0.0f);   // a sensor records no negative intensity
    out[i] = v;
}

cudaError_t synth_fill_one(float2 *psi, size_t n, cudaStream_t s) {
    k_fill_one<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(psi, n);
    return cudaGetLastError();
}

cudaError_t synth_disc(float2 *psi, int nx, int ny, double cx, double cy, double diam, double dx, cudaStream_t s) {
    const double r = diam / 2.0;
    const int x0 = (int)floor((cx - r) / dx) - 1, x1 = (int)ceil((cx + r) / dx) + 1;
    const int y0 = (int)floor((cy - r) / dx) - 1, y1 = (int)ceil((cy + r) / dx) + 1;
    const int w = x1 - x0 + 1, h = y1 - y0 + 1;
    if (w <= 0 || h <= 0) return cudaSuccess;
    k_disc_mask<<<(w * h + 255) / 256, 256, 0, s>>>(psi, nx, ny, cx, cy, r, dx, x0, y0, w, h);
    return cudaGetLastError();
}

__global__ void k_minmax_init(float *mm) {
    mm[0] = __int_as_float(0x7f800000);
    mm[1] = 0.0f;
}

cudaError_t synth_finish(const float2 *psi, float *out, size_t n, const float *noise, float *mm, cudaStream_t s) {
    k_minmax_init<<<1, 1, 0, s>>>(mm);
    k_intensity_minmax<<<256, 256, 0, s>>>(psi, out, n, mm);
    k_normalise_noise<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(out, noise, n, mm);
    return cudaGetLastError();
}

}  // namespace ph
