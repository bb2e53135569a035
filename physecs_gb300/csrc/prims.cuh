// prims.cuh — device-wide primitives: exclusive scan, LSD radix sort of 32-bit
// keys with 32-bit payloads, and a bounded grid barrier.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace psx {

// Exclusive prefix sum of n ints; writes the grand total to *total (device pointer).
// scratch must hold scan_scratch_ints(n) ints.
size_t scan_scratch_ints(int n);
void scan_exclusive(const int* in, int* out, int n, int* total, int* scratch, cudaStream_t s);
// Variant whose element count is read on the device from *n_dev (at most n_max elements).
void scan_exclusive_dev(const int* in, int* out, const int* n_dev, int n_max, int* total, int* scratch, cudaStream_t s);

// Stable LSD radix sort of (key, value) pairs over bits [0, bits).  The result ends
// up in (keys, vals); tmp buffers hold n elements each; hist needs radix_hist_ints(n).
// Returns the number of kernels queued.
size_t radix_hist_ints(int n);
int radix_sort_pairs(uint32_t* keys, int* vals, uint32_t* tmpk, int* tmpv, int n, int bits, int* hist, cudaStream_t s);

// Grid-wide barrier for cooperative launches.  Every block calls it; the wait is
// bounded: after ~0.5 s without progress the barrier records ERR_BARRIER_TIMEOUT in
// *err and lets the caller continue so the kernel always terminates.
struct GridBarrier {
    unsigned int* count;
    unsigned int* gen;
    int* err;
    __device__ __forceinline__ void sync() const {
        __syncthreads();
        if (threadIdx.x == 0) {
            volatile unsigned int* vgen = gen;
            unsigned int g = *vgen;
            __threadfence();
            unsigned int arrived = atomicAdd(count, 1u);
            if (arrived == gridDim.x - 1) {
                atomicExch(count, 0u);
                __threadfence();
                atomicAdd(gen, 1u);
            } else {
                long long spins = 0;
                while (*vgen == g) {
                    __nanosleep(64);
                    if (++spins > (1ll << 23)) { atomicOr(err, 1 << 5); break; }
                }
            }
            __threadfence();
        }
        __syncthreads();
    }
};

}  // namespace psx
