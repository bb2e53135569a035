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

// Bit of the device error word that a grid barrier whose wait ran out sets.
constexpr int kBarrierTimeoutBit = 1 << 5;
// Polls of a grid barrier's wait before it gives up (64 ns apart: about half a second).
constexpr long long kDefaultWaitPolls = 1ll << 23;

// Grid-wide barrier for cooperative launches.  Every block calls it.  The wait is
// bounded: a block that polls more than `limit` times records kBarrierTimeoutBit in
// *err.  A block that finds the bit set, because its own wait ran out or another
// block's did, leaves the kernel at once instead of arriving.  So no block runs past
// a barrier that the grid did not complete, and after a timeout every block ends
// within one more bounded wait.  A kernel that uses it must leave nothing behind that
// a later launch relies on besides *err; the barrier words themselves are reset
// before each launch.
struct GridBarrier {
    unsigned int* count;
    unsigned int* gen;
    int* err;
    long long limit;
    __device__ __forceinline__ void sync() const {
        __shared__ int leave;
        __syncthreads();
        if (threadIdx.x == 0) {
            volatile int* verr = err;
            volatile unsigned int* vgen = gen;
            int out = (*verr & kBarrierTimeoutBit) != 0;
            if (!out) {
                unsigned int g = *vgen;
                __threadfence();
                unsigned int arrived = atomicAdd(count, 1u);
                if (arrived == gridDim.x - 1) {
                    atomicExch(count, 0u);
                    __threadfence();
                    atomicAdd(gen, 1u);
                } else {
                    long long polls = 0;
                    while (*vgen == g) {
                        __nanosleep(64);
                        if (*verr & kBarrierTimeoutBit) { out = 1; break; }
                        if (++polls > limit) { atomicOr(err, kBarrierTimeoutBit); out = 1; break; }
                    }
                }
                __threadfence();
            }
            leave = out;
        }
        __syncthreads();
        // every thread of the block reads the same flag here, so the whole block leaves
        if (leave) asm volatile("exit;");
    }
};

}  // namespace psx
