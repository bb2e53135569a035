// prims.cu — exclusive scan and LSD radix sort (hand-written; no CUB).
#include "prims.cuh"

namespace psx {

namespace {
constexpr int kScanBlock = 1024;  // elements per block: 256 threads x 4

__device__ __forceinline__ int warp_incl_scan(int v) {
    const unsigned m = 0xffffffffu;
    int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(m, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// block-wide exclusive scan of one value per thread (256 threads); returns block total via *tot
__device__ __forceinline__ int block_excl_scan(int v, int* sh, int* tot) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int inc = warp_incl_scan(v);
    if (lane == 31) sh[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int s = (lane < (blockDim.x >> 5)) ? sh[lane] : 0;
        int si = warp_incl_scan(s);
        sh[lane] = si - s;
        if (lane == 31) sh[32] = si;
    }
    __syncthreads();
    int r = inc - v + sh[wid];
    if (tot) *tot = sh[32];
    __syncthreads();
    return r;
}

__global__ void k_scan_blocks(const int* in, int* out, int n, const int* n_dev, int* block_sums) {
    __shared__ int sh[33];
    if (n_dev) n = min(n, *n_dev);
    int base = blockIdx.x * kScanBlock + threadIdx.x * 4;
    int v[4], s = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) { v[k] = (base + k < n) ? in[base + k] : 0; s += v[k]; }
    int tot;
    int ex = block_excl_scan(s, sh, &tot);
#pragma unroll
    for (int k = 0; k < 4; ++k) { if (base + k < n) out[base + k] = ex; ex += v[k]; }
    if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

// single block scans the per-block sums (any count) in chunks of 1024
__global__ void k_scan_sums(int* sums, int nb, int* total) {
    __shared__ int sh[33];
    int carry = 0;
    for (int c = 0; c < nb; c += kScanBlock) {
        int base = c + threadIdx.x * 4;
        int v[4], s = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) { v[k] = (base + k < nb) ? sums[base + k] : 0; s += v[k]; }
        int tot;
        int ex = block_excl_scan(s, sh, &tot) + carry;
#pragma unroll
        for (int k = 0; k < 4; ++k) { if (base + k < nb) sums[base + k] = ex; ex += v[k]; }
        carry += tot;
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

__global__ void k_scan_add(int* out, int n, const int* n_dev, const int* sums) {
    if (n_dev) n = min(n, *n_dev);
    int add = sums[blockIdx.x];
    int base = blockIdx.x * kScanBlock + threadIdx.x * 4;
#pragma unroll
    for (int k = 0; k < 4; ++k) if (base + k < n) out[base + k] += add;
}
}  // namespace

size_t scan_scratch_ints(int n) { return (size_t)(n + kScanBlock - 1) / kScanBlock + 1; }

static void scan_impl(const int* in, int* out, int n, const int* n_dev, int* total, int* scratch, cudaStream_t s) {
    int nb = (n + kScanBlock - 1) / kScanBlock;
    if (nb == 0) nb = 1;
    k_scan_blocks<<<nb, 256, 0, s>>>(in, out, n, n_dev, scratch);
    k_scan_sums<<<1, 256, 0, s>>>(scratch, nb, total);
    k_scan_add<<<nb, 256, 0, s>>>(out, n, n_dev, scratch);
}

void scan_exclusive(const int* in, int* out, int n, int* total, int* scratch, cudaStream_t s) {
    scan_impl(in, out, n, nullptr, total, scratch, s);
}
void scan_exclusive_dev(const int* in, int* out, const int* n_dev, int n_max, int* total, int* scratch, cudaStream_t s) {
    scan_impl(in, out, n_max, n_dev, total, scratch, s);
}

// ---------------------------------------------------------------- radix sort
//
// One 8-bit digit per pass.  A tile of kTile keys is split into 8 contiguous
// warp chunks; per-warp digit counters make the ranking stable: a key's rank is
// (keys of the same digit in earlier tiles) + (in earlier warps of this tile) +
// (earlier in this warp's chunk), the last counted 32 keys at a time with
// __match_any_sync.
namespace {
constexpr int kTile = 4096;
constexpr int kRadixThreads = 256;
constexpr int kWarps = kRadixThreads / 32;
constexpr int kPerWarp = kTile / kWarps;  // 512 keys per warp

__global__ void k_radix_hist(const uint32_t* keys, int n, int shift, int* hist, int ntiles) {
    __shared__ int h[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    int base = blockIdx.x * kTile;
    for (int i = threadIdx.x; i < kTile; i += blockDim.x) {
        int k = base + i;
        if (k < n) atomicAdd(&h[(keys[k] >> shift) & 255], 1);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[d * ntiles + blockIdx.x] = h[d];
}

__global__ void k_radix_scatter(const uint32_t* keys, const int* vals, uint32_t* ok, int* ov, int n, int shift,
                                const int* offs, int ntiles) {
    __shared__ int wc[kWarps][256];   // per-warp running counters, then per-warp base offsets
    int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = lane; i < 256; i += 32) wc[wid][i] = 0;
    __syncwarp();
    int cbase = blockIdx.x * kTile + wid * kPerWarp;
    // pass 1: per-warp digit histogram
    for (int r = 0; r < kPerWarp; r += 32) {
        int k = cbase + r + lane;
        if (k < n) atomicAdd(&wc[wid][(keys[k] >> shift) & 255], 1);
    }
    __syncthreads();
    // exclusive scan across warps per digit, plus the global tile offset
    for (int d = threadIdx.x; d < 256; d += blockDim.x) {
        int run = offs[d * ntiles + blockIdx.x];
        for (int w = 0; w < kWarps; ++w) { int c = wc[w][d]; wc[w][d] = run; run += c; }
    }
    __syncthreads();
    // pass 2: stable scatter, 32 keys at a time
    for (int r = 0; r < kPerWarp; r += 32) {
        int k = cbase + r + lane;
        bool valid = k < n;
        uint32_t key = valid ? keys[k] : 0xffffffffu;
        int d = valid ? (int)((key >> shift) & 255) : 256 + lane;  // invalid lanes match nobody
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int rank = __popc(peers & ((1u << lane) - 1));
        int cnt = __popc(peers);
        int leader = __ffs(peers) - 1;
        int basev = 0;
        if (valid && lane == leader) basev = wc[wid][d];
        basev = __shfl_sync(0xffffffffu, basev, leader);
        if (valid) {
            int dst = basev + rank;
            ok[dst] = key;
            ov[dst] = vals[k];
        }
        __syncwarp();
        if (valid && lane == leader) wc[wid][d] = basev + cnt;
        __syncwarp();
    }
}
}  // namespace

size_t radix_hist_ints(int n) {
    int ntiles = (n + kTile - 1) / kTile;
    if (ntiles == 0) ntiles = 1;
    size_t h = (size_t)256 * ntiles;
    return 2 * h + scan_scratch_ints((int)h) + 1;
}

int radix_sort_pairs(uint32_t* keys, int* vals, uint32_t* tmpk, int* tmpv, int n, int bits, int* hist, cudaStream_t s) {
    if (n <= 0) return 0;
    int ntiles = (n + kTile - 1) / kTile;
    int h = 256 * ntiles;
    int* offs = hist + h;
    int* scratch = offs + h;
    uint32_t* ka = keys; int* va = vals;
    uint32_t* kb = tmpk; int* vb = tmpv;
    int passes = (bits + 7) / 8;
    for (int p = 0; p < passes; ++p) {
        int shift = 8 * p;
        k_radix_hist<<<ntiles, kRadixThreads, 0, s>>>(ka, n, shift, hist, ntiles);
        scan_exclusive(hist, offs, h, nullptr, scratch, s);
        k_radix_scatter<<<ntiles, kRadixThreads, 0, s>>>(ka, va, kb, vb, n, shift, offs, ntiles);
        uint32_t* tk = ka; ka = kb; kb = tk;
        int* tv = va; va = vb; vb = tv;
    }
    if (ka != keys) {
        cudaMemcpyAsync(keys, ka, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(vals, va, sizeof(int) * n, cudaMemcpyDeviceToDevice, s);
    }
    return passes * 5;
}

}  // namespace psx
