// libm_f32.cuh — acosf, atanf and atan2f as the reference's C library evaluates them.
//
// The reference's servo and gear rows call glm::orientedAngle and glm::atan(y, x)
// (src/Joints/ServoJoint.cpp:52-54, src/Joints/GearJoint.cpp:16-29), i.e. the C
// library's acosf and atan2f.  glibc 2.39 evaluates both with the single-precision
// algorithms of fdlibm (Sun Microsystems, 1993): argument reduction to a few intervals
// and minimax polynomials in float.  Those results are not always correctly rounded
// (about 8% of acosf and 20% of atan2f results differ in the last bit from the
// correctly rounded value), so neither CUDA's functions nor a double-precision
// evaluation reproduces them.  The functions below restate the published algorithms,
// with their reductions, coefficients and float operation order, so that the joint rows
// round as the reference's do.  They need IEEE float division and square root and no
// fused multiply-add, which is how this library is compiled; tests/test_libm_f32.py
// compares them with the host's C library on many arguments.
#pragma once
#include <cstdint>
#include <cstring>
#include <cmath>

#ifndef __CUDACC__
#define PSX_HD inline
#else
#define PSX_HD __host__ __device__ __forceinline__
#endif

// glibc built for aarch64 lets the compiler fuse a product with the sum or difference
// that consumes it into one fused multiply-add (GCC's default on that target), and x86-64
// builds cannot; the results differ in the last bit for a few arguments in ten thousand.
// The places below are where that build fuses, found by comparing candidate forms with
// the aarch64 C library on millions of arguments: the polynomials' Horner steps, the
// sum of atanf's two partial polynomials and acosf's closing steps, not atanf's last
// subtractions.
// PSX_LIBM_FUSED (set when this library is built on an aarch64 host) selects the fused
// form at each place where that compiler fuses, so that the device matches the C library
// of the host it is built for.
#if defined(PSX_LIBM_FUSED)
#ifdef __CUDA_ARCH__
#define PSX_MAD(a, b, c) __fmaf_rn((a), (b), (c))
#else
#define PSX_MAD(a, b, c) std::fma((float)(a), (float)(b), (float)(c))
#endif
#else
#define PSX_MAD(a, b, c) ((a) * (b) + (c))
#endif

namespace psx {
namespace libm {

PSX_HD uint32_t bits(float x) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(x);
#else
    uint32_t u;
    std::memcpy(&u, &x, 4);
    return u;
#endif
}

PSX_HD float from_bits(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float x;
    std::memcpy(&x, &u, 4);
    return x;
#endif
}

PSX_HD float neg(float x) { return from_bits(bits(x) ^ 0x80000000u); }

// arctangent: |x| reduced against one of the breakpoints 1/2, 1, 3/2 and infinity, whose
// arctangents are kept as a float pair (high, low), then an odd polynomial of degree 23
// in the reduced argument, split into even and odd powers of x^4
PSX_HD float atanf(float x) {
    const float head[4] = {4.6364760399e-01f, 7.8539812565e-01f, 9.8279368877e-01f, 1.5707962513e+00f};
    const float tail[4] = {5.0121582440e-09f, 3.7748947079e-08f, 3.4473217170e-08f, 7.5497894159e-08f};
    const float c[11] = {3.3333334327e-01f, -2.0000000298e-01f, 1.4285714924e-01f, -1.1111110449e-01f,
                         9.0908870101e-02f, -7.6918758452e-02f, 6.6610731184e-02f, -5.8335702866e-02f,
                         4.9768779427e-02f, -3.6531571299e-02f, 1.6285819933e-02f};
    const uint32_t hx = bits(x), ix = hx & 0x7fffffffu;
    const bool negative = (hx >> 31) != 0;
    if (ix >= 0x4c000000u) {                       // |x| >= 2^25 (or not a number)
        if (ix > 0x7f800000u) return x + x;
        const float r = head[3] + tail[3];
        return negative ? neg(r) : r;
    }
    int k;
    if (ix < 0x3ee00000u) {                        // |x| < 7/16
        if (ix < 0x31000000u) return x;            // |x| < 2^-29: atan x = x in float
        k = -1;
    } else {
        x = std::fabs(x);
        if (ix < 0x3f980000u) {                    // |x| < 19/16
            if (ix < 0x3f300000u) { k = 0; x = PSX_MAD(2.0f, x, -1.0f) / (2.0f + x); }   // 7/16 <= |x| < 11/16
            else { k = 1; x = (x - 1.0f) / (x + 1.0f); }                           // 11/16 <= |x| < 19/16
        } else if (ix < 0x401c0000u) {             // 19/16 <= |x| < 39/16
            k = 2; x = (x - 1.5f) / PSX_MAD(1.5f, x, 1.0f);
        } else {                                   // 39/16 <= |x| < 2^25
            k = 3; x = -1.0f / x;
        }
    }
    const float z = x * x, w = z * z;
    const float t_odd = PSX_MAD(w, PSX_MAD(w, PSX_MAD(w, PSX_MAD(w, PSX_MAD(w, c[10], c[8]), c[6]), c[4]), c[2]), c[0]);
    const float t_even = PSX_MAD(w, PSX_MAD(w, PSX_MAD(w, PSX_MAD(w, c[9], c[7]), c[5]), c[3]), c[1]);
    const float sum = PSX_MAD(z, t_odd, w * t_even);   // odd + even powers: z t_odd + w t_even
    if (k < 0) return x - x * sum;
    const float r = head[k] - ((x * sum - tail[k]) - x);
    return negative ? neg(r) : r;
}

// two-argument arctangent: special values, then atan(|y / x|) placed in the quadrant of
// (x, y) with pi kept as a float pair; a quotient beyond 2^60 in either direction skips
// the division
PSX_HD float atan2f(float y, float x) {
    const float tiny = 1.0e-30f, pi_4 = 7.8539818525e-01f, pi_2 = 1.5707963705e+00f, pi = 3.1415927410e+00f,
                pi_tail = -8.7422776573e-08f;
    const uint32_t hx = bits(x), hy = bits(y), ix = hx & 0x7fffffffu, iy = hy & 0x7fffffffu;
    if (ix > 0x7f800000u || iy > 0x7f800000u) return x + y;
    if (hx == 0x3f800000u) return atanf(y);        // x = 1
    const int q = (int)((hy >> 31) & 1u) | (int)((hx >> 30) & 2u);   // bit 0: y < 0, bit 1: x < 0
    if (iy == 0) {
        if (q < 2) return y;
        return q == 2 ? pi + tiny : -pi - tiny;
    }
    if (ix == 0) return (hy >> 31) ? -pi_2 - tiny : pi_2 + tiny;
    if (ix == 0x7f800000u) {
        if (iy == 0x7f800000u) {
            switch (q) {
                case 0: return pi_4 + tiny;
                case 1: return -pi_4 - tiny;
                case 2: return 3.0f * pi_4 + tiny;
                default: return -3.0f * pi_4 - tiny;
            }
        }
        switch (q) {
            case 0: return 0.0f;
            case 1: return -0.0f;
            case 2: return pi + tiny;
            default: return -pi - tiny;
        }
    }
    if (iy == 0x7f800000u) return (hy >> 31) ? -pi_2 - tiny : pi_2 + tiny;
    const int e = ((int)iy - (int)ix) >> 23;
    float z;
    if (e > 60) z = pi_2 + 0.5f * pi_tail;
    else if ((hx >> 31) && e < -60) z = 0.0f;
    else z = atanf(std::fabs(y / x));
    switch (q) {
        case 0: return z;
        case 1: return neg(z);
        case 2: return pi - (z - pi_tail);
        default: return (z - pi_tail) - pi;
    }
}

// arccosine: |x| < 1/2 through asin's rational approximation around 0; |x| >= 1/2 through
// acos x = 2 asin(sqrt((1 - |x|) / 2)), with sqrt split into a 12-bit head and a
// correction for x > 1/2
PSX_HD float acosf(float x) {
    const float pi = 3.1415925026e+00f, pi_2_head = 1.5707962513e+00f, pi_2_tail = 7.5497894159e-08f;
    const float p0 = 1.6666667163e-01f, p1 = -3.2556581497e-01f, p2 = 2.0121252537e-01f, p3 = -4.0055535734e-02f,
                p4 = 7.9153501429e-04f, p5 = 3.4793309169e-05f;
    const float q1 = -2.4033949375e+00f, q2 = 2.0209457874e+00f, q3 = -6.8828397989e-01f, q4 = 7.7038154006e-02f;
    const uint32_t hx = bits(x), ix = hx & 0x7fffffffu;
    if (ix == 0x3f800000u) return (hx >> 31) ? pi + 2.0f * pi_2_tail : 0.0f;   // |x| = 1
    if (ix > 0x3f800000u) return (x - x) / (x - x);                           // |x| > 1: not a number
    if (ix < 0x3f000000u) {                                                   // |x| < 1/2
        if (ix <= 0x23000000u) return pi_2_head + pi_2_tail;
        const float z = x * x;
        const float p = z * PSX_MAD(z, PSX_MAD(z, PSX_MAD(z, PSX_MAD(z, PSX_MAD(z, p5, p4), p3), p2), p1), p0);
        const float q = PSX_MAD(z, PSX_MAD(z, PSX_MAD(z, PSX_MAD(z, q4, q3), q2), q1), 1.0f);
        const float r = p / q;
        return pi_2_head - (x - PSX_MAD(-x, r, pi_2_tail));
    }
    if (hx >> 31) {                                                           // x <= -1/2
        const float z = (1.0f + x) * 0.5f;
        const float p = z * PSX_MAD(z, PSX_MAD(z, PSX_MAD(z, PSX_MAD(z, PSX_MAD(z, p5, p4), p3), p2), p1), p0);
        const float q = PSX_MAD(z, PSX_MAD(z, PSX_MAD(z, PSX_MAD(z, q4, q3), q2), q1), 1.0f);
        const float s = std::sqrt(z);
        const float r = p / q;
        const float w = PSX_MAD(r, s, -pi_2_tail);
        return PSX_MAD(-2.0f, s + w, pi);
    }
    const float z = (1.0f - x) * 0.5f;                                        // x >= 1/2
    const float s = std::sqrt(z);
    const float head = from_bits(bits(s) & 0xfffff000u);
    const float corr = PSX_MAD(-head, head, z) / (s + head);
    const float p = z * PSX_MAD(z, PSX_MAD(z, PSX_MAD(z, PSX_MAD(z, PSX_MAD(z, p5, p4), p3), p2), p1), p0);
    const float q = PSX_MAD(z, PSX_MAD(z, PSX_MAD(z, PSX_MAD(z, q4, q3), q2), q1), 1.0f);
    const float r = p / q;
    const float w = PSX_MAD(r, s, corr);
    return 2.0f * (head + w);
}

}  // namespace libm
}  // namespace psx

#undef PSX_HD
#undef PSX_MAD
