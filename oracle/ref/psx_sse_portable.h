/*
 * Portable stand-in for the SSE intrinsics the Physecs reference uses, written
 * on GCC vector extensions so the reference compiles on aarch64 hosts.  Test
 * infrastructure only (oracle); never part of the physecs_gb300 product.
 *
 * Each function restates the documented lane semantics of the Intel intrinsic
 * of the same name (Intel Intrinsics Guide): IEEE single-precision lane
 * arithmetic, all-ones / all-zeros comparison masks, min/max returning the
 * second operand when either input is NaN, blends keyed on the mask sign bit.
 */
#pragma once
#include <cstring>
#include <cmath>
#include <cstdint>

typedef float __m128 __attribute__((vector_size(16), __may_alias__));
typedef long long __m128i __attribute__((vector_size(16), __may_alias__));
typedef int psx_v4si __attribute__((vector_size(16), __may_alias__));
typedef unsigned char psx_v16qu __attribute__((vector_size(16), __may_alias__));

#define _MM_SHUFFLE(z, y, x, w) (((z) << 6) | ((y) << 4) | ((x) << 2) | (w))

static inline __m128 _mm_setzero_ps() { return (__m128){0.f, 0.f, 0.f, 0.f}; }
static inline __m128 _mm_set1_ps(float a) { return (__m128){a, a, a, a}; }
static inline __m128 _mm_setr_ps(float a, float b, float c, float d) { return (__m128){a, b, c, d}; }
static inline __m128 _mm_add_ps(__m128 a, __m128 b) { return a + b; }
static inline __m128 _mm_sub_ps(__m128 a, __m128 b) { return a - b; }
static inline __m128 _mm_mul_ps(__m128 a, __m128 b) { return a * b; }
static inline __m128 _mm_div_ps(__m128 a, __m128 b) { return a / b; }
static inline __m128 _mm_sqrt_ps(__m128 a) {
    return (__m128){std::sqrt(a[0]), std::sqrt(a[1]), std::sqrt(a[2]), std::sqrt(a[3])};
}
static inline __m128 _mm_max_ps(__m128 a, __m128 b) {
    __m128 r;
    for (int i = 0; i < 4; ++i) r[i] = a[i] > b[i] ? a[i] : b[i];
    return r;
}
static inline __m128 _mm_min_ps(__m128 a, __m128 b) {
    __m128 r;
    for (int i = 0; i < 4; ++i) r[i] = a[i] < b[i] ? a[i] : b[i];
    return r;
}
static inline __m128 psx_mask_ps(psx_v4si m) { __m128 r; std::memcpy(&r, &m, 16); return r; }
static inline __m128 _mm_cmpneq_ps(__m128 a, __m128 b) {
    psx_v4si m;
    for (int i = 0; i < 4; ++i) m[i] = !(a[i] == b[i]) ? -1 : 0;
    return psx_mask_ps(m);
}
static inline __m128 _mm_cmplt_ps(__m128 a, __m128 b) {
    psx_v4si m;
    for (int i = 0; i < 4; ++i) m[i] = (a[i] < b[i]) ? -1 : 0;
    return psx_mask_ps(m);
}
static inline __m128 _mm_cmpgt_ps(__m128 a, __m128 b) {
    psx_v4si m;
    for (int i = 0; i < 4; ++i) m[i] = (a[i] > b[i]) ? -1 : 0;
    return psx_mask_ps(m);
}
static inline __m128 _mm_and_ps(__m128 a, __m128 b) {
    psx_v4si x, y; std::memcpy(&x, &a, 16); std::memcpy(&y, &b, 16);
    return psx_mask_ps(x & y);
}
static inline __m128 _mm_blendv_ps(__m128 a, __m128 b, __m128 mask) {
    psx_v4si m; std::memcpy(&m, &mask, 16);
    __m128 r;
    for (int i = 0; i < 4; ++i) r[i] = (m[i] < 0) ? b[i] : a[i];
    return r;
}
static inline __m128i _mm_castps_si128(__m128 a) { __m128i r; std::memcpy(&r, &a, 16); return r; }
static inline __m128 _mm_castsi128_ps(__m128i a) { __m128 r; std::memcpy(&r, &a, 16); return r; }
static inline __m128 _mm_shuffle_ps_fn(__m128 a, __m128 b, int imm) {
    return (__m128){a[imm & 3], a[(imm >> 2) & 3], b[(imm >> 4) & 3], b[(imm >> 6) & 3]};
}
#define _mm_shuffle_ps(a, b, imm) _mm_shuffle_ps_fn((a), (b), (imm))
static inline __m128 _mm_unpacklo_ps(__m128 a, __m128 b) { return (__m128){a[0], b[0], a[1], b[1]}; }
static inline __m128 _mm_unpackhi_ps(__m128 a, __m128 b) { return (__m128){a[2], b[2], a[3], b[3]}; }
static inline __m128 _mm_load_ps(const float* p) { __m128 r; std::memcpy(&r, p, 16); return r; }
static inline __m128 _mm_loadu_ps(const float* p) { __m128 r; std::memcpy(&r, p, 16); return r; }
static inline void _mm_store_ps(float* p, __m128 a) { std::memcpy(p, &a, 16); }
static inline void _mm_storeu_ps(float* p, __m128 a) { std::memcpy(p, &a, 16); }

static inline psx_v4si psx_i32(__m128i a) { psx_v4si r; std::memcpy(&r, &a, 16); return r; }
static inline __m128i psx_m128i(psx_v4si a) { __m128i r; std::memcpy(&r, &a, 16); return r; }
static inline __m128i _mm_setzero_si128() { return psx_m128i((psx_v4si){0, 0, 0, 0}); }
static inline __m128i _mm_set1_epi32(int a) { return psx_m128i((psx_v4si){a, a, a, a}); }
static inline __m128i _mm_setr_epi32(int a, int b, int c, int d) { return psx_m128i((psx_v4si){a, b, c, d}); }
static inline __m128i _mm_add_epi32(__m128i a, __m128i b) { return psx_m128i(psx_i32(a) + psx_i32(b)); }
static inline __m128i _mm_cmpgt_epi32(__m128i a, __m128i b) {
    psx_v4si x = psx_i32(a), y = psx_i32(b), r;
    for (int i = 0; i < 4; ++i) r[i] = x[i] > y[i] ? -1 : 0;
    return psx_m128i(r);
}
static inline __m128i _mm_and_si128(__m128i a, __m128i b) { return a & b; }
#define _mm_and_epi32(a, b) _mm_and_si128((a), (b))
static inline __m128i _mm_slli_si128_fn(__m128i a, int imm) {
    psx_v16qu x, r; std::memcpy(&x, &a, 16);
    for (int i = 0; i < 16; ++i) r[i] = (i - imm >= 0) ? x[i - imm] : 0;
    __m128i o; std::memcpy(&o, &r, 16); return o;
}
#define _mm_slli_si128(a, imm) _mm_slli_si128_fn((a), (imm))
static inline __m128i _mm_shuffle_epi32_fn(__m128i a, int imm) {
    psx_v4si x = psx_i32(a);
    return psx_m128i((psx_v4si){x[imm & 3], x[(imm >> 2) & 3], x[(imm >> 4) & 3], x[(imm >> 6) & 3]});
}
#define _mm_shuffle_epi32(a, imm) _mm_shuffle_epi32_fn((a), (imm))
static inline int _mm_movemask_ps(__m128 a) {
    psx_v4si m; std::memcpy(&m, &a, 16);
    int r = 0;
    for (int i = 0; i < 4; ++i) r |= (m[i] < 0 ? 1 : 0) << i;
    return r;
}
static inline int _mm_testz_si128(__m128i a, __m128i b) {
    __m128i c = a & b;
    return (c[0] == 0 && c[1] == 0) ? 1 : 0;
}
static inline __m128i _mm_blendv_epi8(__m128i a, __m128i b, __m128i mask) {
    psx_v16qu x, y, m, r;
    std::memcpy(&x, &a, 16); std::memcpy(&y, &b, 16); std::memcpy(&m, &mask, 16);
    for (int i = 0; i < 16; ++i) r[i] = (m[i] & 0x80) ? y[i] : x[i];
    __m128i o; std::memcpy(&o, &r, 16); return o;
}
static inline void _mm_storeu_epi32(void* p, __m128i a) { std::memcpy(p, &a, 16); }
static inline void _mm_pause() {}
