// ordkey.cuh — order-preserving 64-bit keys for parallel min / max reductions that
// must pick the same value as a sequential left fold: among equal values (+0 and -0
// compare equal) the fold keeps the first one, so the key carries the element's index
// after the value and ties go to the lowest index.
#pragma once
#include <cuda_runtime.h>

namespace psx {

constexpr unsigned long long kKeyMinInit = ~0ull, kKeyMaxInit = 0ull;

// order-preserving key of a float, +0 and -0 equal
__device__ __forceinline__ unsigned ord_fkey(float v) {
    unsigned u = __float_as_uint(v == 0.f ? 0.f : v);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ unsigned long long key_min(float v, int idx) {
    return ((unsigned long long)ord_fkey(v) << 32) | (unsigned)idx;
}
__device__ __forceinline__ unsigned long long key_max(float v, int idx) {
    return ((unsigned long long)ord_fkey(v) << 32) | (0xffffffffu - (unsigned)idx);
}
__device__ __forceinline__ int key_min_index(unsigned long long k) { return (int)(unsigned)k; }
__device__ __forceinline__ int key_max_index(unsigned long long k) { return (int)(0xffffffffu - (unsigned)k); }

}  // namespace psx
