// ph_common.cuh -- shared device helpers: complex arithmetic, compile-time
// twiddle constants and small in-register DFTs.
#pragma once

#include <cstdint>
#include <utility>
#include <cuda_runtime.h>

namespace ph {

// ---------------------------------------------------------------- complex

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// Multiplication by -i (forward quarter turn) and +i.
__device__ __forceinline__ float2 mul_mi(float2 a) { return make_float2(a.y, -a.x); }
__device__ __forceinline__ float2 mul_pi(float2 a) { return make_float2(-a.y, a.x); }

// ---------------------------------------------------------------- compile-time loops

template <int... Is, class F>
__device__ __forceinline__ void static_for_impl(std::integer_sequence<int, Is...>, F &&f) {
    (f(std::integral_constant<int, Is>{}), ...);
}
template <int N, class F>
__device__ __forceinline__ void static_for(F &&f) {
    static_for_impl(std::make_integer_sequence<int, N>{}, f);
}

// ---------------------------------------------------------------- compile-time trig
// Taylor series evaluated by the compiler; used only to build constants.

constexpr double kTwoPi = 6.283185307179586476925286766559;

constexpr double cx_sin_small(double x) {   // |x| <= pi/4
    double x2 = x * x, t = x, s = x;
    for (int n = 1; n < 14; ++n) { t *= -x2 / double((2 * n) * (2 * n + 1)); s += t; }
    return s;
}
constexpr double cx_cos_small(double x) {
    double x2 = x * x, t = 1.0, s = 1.0;
    for (int n = 1; n < 14; ++n) { t *= -x2 / double((2 * n - 1) * (2 * n)); s += t; }
    return s;
}
// cos / sin of 2*pi*k/r with exact octant reduction on the integers.
constexpr double cx_cos_turn(long long k, long long r) {
    k %= r; if (k < 0) k += r;
    // angle = 2 pi k / r; reduce to [0, pi/4] using quarter-turn symmetries
    long long k8 = 8 * k;
    if (k8 <= r) return cx_cos_small(kTwoPi * double(k) / double(r));                 // [0, 45]
    if (k8 <= 2 * r) return cx_sin_small(kTwoPi * double(r - 4 * k) / double(4 * r)); // [45, 90]
    if (k8 <= 4 * r) return -cx_cos_turn(r - 2 * k, 2 * r);                              // (90, 180]
    return cx_cos_turn(r - k, r);                                                         // (180, 360)
}
constexpr double cx_sin_turn(long long k, long long r) {
    // sin(a) = cos(a - pi/2) = cos(2 pi (4k - r) / (4r))
    return cx_cos_turn(4 * k - r, 4 * r);
}

// W_R^K = exp(-2 pi i K / R) for the forward transform (conjugate for inverse).
template <int K, int R, bool INV>
struct Tw {
    static constexpr int k = ((K % R) + R) % R;
    static constexpr float c = float(cx_cos_turn(k, R));
    static constexpr float s = INV ? float(cx_sin_turn(k, R)) : -float(cx_sin_turn(k, R));
};

// v * W_R^K with the trivial cases folded.
template <int K, int R, bool INV>
__device__ __forceinline__ float2 twiddle_const(float2 v) {
    constexpr int k = ((K % R) + R) % R;
    if constexpr (k == 0) {
        return v;
    } else if constexpr (2 * k == R) {
        return make_float2(-v.x, -v.y);
    } else if constexpr (4 * k == R) {
        return INV ? mul_pi(v) : mul_mi(v);
    } else if constexpr (4 * k == 3 * R) {
        return INV ? mul_mi(v) : mul_pi(v);
    } else if constexpr ((8 * k) % R == 0) {
        // odd multiples of 45 degrees: (c + i s) with |c| = |s| = 1/sqrt(2)
        constexpr float h = 0.70710678118654752440f;
        constexpr float c = Tw<K, R, INV>::c;
        constexpr float s = Tw<K, R, INV>::s;
        constexpr float sc = c > 0 ? h : -h;
        constexpr float ss = s > 0 ? h : -h;
        // (x + i y)(sc + i ss) = (x sc - y ss) + i (x ss + y sc)
        if constexpr (sc == ss) {
            return make_float2((v.x - v.y) * sc, (v.x + v.y) * sc);
        } else {
            return make_float2((v.x + v.y) * sc, (v.y - v.x) * sc);
        }
    } else {
        constexpr float c = Tw<K, R, INV>::c;
        constexpr float s = Tw<K, R, INV>::s;
        return make_float2(fmaf(v.x, c, -v.y * s), fmaf(v.x, s, v.y * c));
    }
}

// ---------------------------------------------------------------- in-register DFTs
// dft<R, INV>(v): in place, natural-order input and output, unnormalised.

template <bool INV>
__device__ __forceinline__ void dft2(float2 &a, float2 &b) {
    float2 t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

template <bool INV>
__device__ __forceinline__ void dft4(float2 &a0, float2 &a1, float2 &a2, float2 &a3) {
    float2 s02 = cadd(a0, a2), d02 = csub(a0, a2);
    float2 s13 = cadd(a1, a3), d13 = csub(a1, a3);
    // forward: X1 = d02 - i d13, X3 = d02 + i d13
    float2 r = INV ? mul_pi(d13) : mul_mi(d13);
    a0 = cadd(s02, s13);
    a2 = csub(s02, s13);
    a1 = cadd(d02, r);
    a3 = csub(d02, r);
}

// Radix 3: X1,2 = a - (b + c)/2 -/+ i (sqrt(3)/2)(b - c) (forward; signs swap for inverse).
template <bool INV>
__device__ __forceinline__ void dft3(float2 &a, float2 &b, float2 &c) {
    constexpr float h = 0.86602540378443864676f;   // sqrt(3)/2
    const float2 s = cadd(b, c), d = csub(b, c);
    const float2 m = make_float2(fmaf(-0.5f, s.x, a.x), fmaf(-0.5f, s.y, a.y));
    const float2 r = INV ? make_float2(-h * d.y, h * d.x) : make_float2(h * d.y, -h * d.x);   // (+/-) i h d
    a = cadd(a, s);
    b = cadd(m, r);
    c = csub(m, r);
}

template <int R, bool INV>
__device__ __forceinline__ void dft(float2 (&v)[R]);

template <int P, int Q, bool INV>
__device__ __forceinline__ void dft_split(float2 (&v)[P * Q]) {
    // R = P*Q, n = Q*n1 + n2, k = k1 + P*k2.
    constexpr int R = P * Q;
    float2 y[Q][P];
#pragma unroll
    for (int n2 = 0; n2 < Q; ++n2) {
        float2 t[P];
#pragma unroll
        for (int n1 = 0; n1 < P; ++n1) t[n1] = v[Q * n1 + n2];
        dft<P, INV>(t);
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) y[n2][k1] = t[k1];
    }
    static_for<Q>([&](auto N2) {
        constexpr int n2 = decltype(N2)::value;
        static_for<P>([&](auto K1) {
            constexpr int k1 = decltype(K1)::value;
            y[n2][k1] = twiddle_const<n2 * k1, R, INV>(y[n2][k1]);
        });
    });
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) {
        float2 t[Q];
#pragma unroll
        for (int n2 = 0; n2 < Q; ++n2) t[n2] = y[n2][k1];
        dft<Q, INV>(t);
#pragma unroll
        for (int k2 = 0; k2 < Q; ++k2) v[k1 + P * k2] = t[k2];
    }
}

template <int R, bool INV>
__device__ __forceinline__ void dft(float2 (&v)[R]) {
    if constexpr (R == 1) {
    } else if constexpr (R == 2) {
        dft2<INV>(v[0], v[1]);
    } else if constexpr (R == 3) {
        dft3<INV>(v[0], v[1], v[2]);
    } else if constexpr (R == 4) {
        dft4<INV>(v[0], v[1], v[2], v[3]);
    } else if constexpr (R == 8) {
        dft_split<2, 4, INV>(v);
    } else if constexpr (R == 16) {
        dft_split<4, 4, INV>(v);
    } else if constexpr (R == 32) {
        dft_split<4, 8, INV>(v);
    } else if constexpr (R == 64) {
        dft_split<8, 8, INV>(v);
    } else {
        static_assert(R == 0, "unsupported radix");
    }
}

// ---------------------------------------------------------------- misc

__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }
__host__ __device__ constexpr int cmin(int a, int b) { return a < b ? a : b; }
__host__ __device__ constexpr int cmax(int a, int b) { return a > b ? a : b; }

// Float bits of a non-negative float, ordered like the float; NaN sorts last.
__device__ __forceinline__ uint64_t pack_min(float v, int k) {
    return (uint64_t(__float_as_uint(v)) << 32) | uint32_t(k);
}

}  // namespace ph
