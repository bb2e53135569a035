/*
 * Force-included compatibility header for building the Physecs reference
 * (an MSVC-first code base) with g++ on Linux.  Test infrastructure only:
 * nothing in the physecs_gb300 package includes or links this file.
 *
 * It supplies the handful of MSVC-only spellings the reference uses
 * (src/Physecs.cpp:702 _BitScanForward, include/Physecs/Constraint1DContainer.h:142
 * _mm_and_epi32, src/GJK.h:96 _mm_storeu_epi32, include/Physecs/*.h
 * __forceinline).  Arithmetic is untouched: every float operation in the
 * reference still runs exactly as written.
 *
 * On aarch64 hosts (the GPU machine) an SSE emulation header built on GCC vector
 * extensions stands in for <immintrin.h>; see psx_sse_portable.h.
 */
#pragma once

#if (defined(__x86_64__) || defined(__i386__)) && !defined(PSX_SSE_PORTABLE)
#include <immintrin.h>
#else
#include "psx_sse_portable.h"
#endif

#include <cstdint>

#ifndef __forceinline
#define __forceinline inline __attribute__((always_inline))
#endif

static inline unsigned char _BitScanForward(unsigned long* index, unsigned long mask) {
    if (!mask) return 0;
    *index = (unsigned long)__builtin_ctzl(mask);
    return 1;
}

#if (defined(__x86_64__) || defined(__i386__)) && !defined(PSX_SSE_PORTABLE)
#ifndef _mm_and_epi32
#define _mm_and_epi32(a, b) _mm_and_si128((a), (b))
#endif
static inline void psx_storeu_epi32(void* p, __m128i v) { _mm_storeu_si128((__m128i*)p, v); }
#define _mm_storeu_epi32(p, v) psx_storeu_epi32((p), (v))
#endif
