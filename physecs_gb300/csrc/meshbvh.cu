// meshbvh.cu — TriangleMesh's BVH (src/TriangleMesh.cpp:7-164) built on the device.
//
// The reference builds a binned-SAH tree (6 buckets per axis) by recursion: a node's
// best (axis, bucket) split partitions its triangle range in place with two pointers,
// the two children are appended to the node array, and the left subtree is built
// before the right one.  Contacts name triangles by their position in that order, so
// the device build reproduces the reference's layout exactly: the same triangle order,
// node ids, bounds (bit for bit) and leaf ranges.
//
//   * Top levels (nodes above kSmall triangles): level by level over chunks of kChunk
//     triangles.  Bucket bounds are reduced with 64-bit keys (value, position) so that,
//     among equal values (+0 / -0), the first triangle in the node's order wins, as in
//     the reference's left fold.  One thread per node picks the split by the
//     reference's own sequence of comparisons.
//   * The partition uses a closed form of the reference's two-pointer loop.  With k
//     triangles going left, the loop keeps left triangles of [0, k) in place, pairs
//     the t-th right triangle of [0, k) with the t-th left triangle of [k, n) counted
//     from the end (q_t), moves that right triangle to q_{t-1} - 1 (q_0 = n), the
//     left one to the right one's place, and every right triangle of [k, n) down by
//     one, except the one at k, which goes to q_r - 1.
//   * Nodes of at most kSmall triangles: one warp builds the whole subtree, in shared
//     memory.
//   * Node ids: the reference appends the children of its m-th split (in pre-order)
//     at 2m+1 and 2m+2.  A split node's pre-order rank among split nodes is its depth
//     plus the leaves before its range minus the right turns on its path (every node
//     of a left sibling subtree precedes it), so ids follow from one scan over leaf
//     starts once the tree is complete.
#include <algorithm>
#include <cfloat>
#include <vector>
#include "meshbvh.cuh"
#include "ordkey.cuh"
#include "prims.cuh"

namespace psx {
namespace {

constexpr int kBk = 6;              // TriangleMesh::numBuckets
constexpr int kBins = 3 * kBk;      // (axis, bucket)
constexpr int kKeys = kBins * 6;    // min xyz, max xyz per bin
constexpr int kSmall = 64;          // nodes up to this size: one warp builds the subtree
constexpr int kChunk = 512;         // triangles per block in the level kernels
constexpr int kThreads = 256;
constexpr int kPer = kChunk / kThreads;
constexpr int kWarpsSmall = 4;
constexpr unsigned long long kMinInit = kKeyMinInit, kMaxInit = kKeyMaxInit;

struct BNode {
    int start, count;       // positions, build-wide
    int mesh, depth;
    int rturns, parent;     // right turns on the path from the root; parent (-1: root)
    int side, leaf;         // 0 left / 1 right; 1 for a final leaf
    int rank, pad;          // split nodes: pre-order rank among the mesh's split nodes
    float bmin[3], bmax[3];
};

struct Slot {               // a node of the current level above kSmall triangles
    int node, chunk_base, nchunks, ok;
    int axis, split, k, r;
};

struct Build {
    const float4* verts;
    const int4* idx;
    const BuildMesh* meshes;
    int tri_lo, n_tris, node_cap;   // the build covers positions [tri_lo, n_tris)
    TriDev* tri;            // original order
    int* perm;              // position -> original triangle
    int* perm_tmp;
    unsigned char* lab;     // 1: goes left at this level's split
    int* rnk;               // rank of a front-right / back-left triangle within its node
    int* fr;                // at node start + t: position of the t-th front-right
    int* bl;                // at node start + t: position of the t-th back-left (ascending)
    BNode* nodes;
    int* n_nodes;
    int* small;             // nodes of 2..kSmall triangles
    int* n_small;
    int* mark;              // [n_tris] 1 where a leaf starts
    int* lb;                // exclusive scan of mark
    int* err;
};

struct Level {
    Slot* slots;
    int* n_slots;
    unsigned long long* keys;   // [slot][kKeys]
    int* cnt;                   // [slot][kBins]
    int* chunk_slot;
    int* chunk_k;
    int* n_chunks;
    int2* chunk_cnt;            // (front-right, back-left) per chunk
    int2* chunk_off;
    int slot_cap, chunk_cap;
};

__device__ __forceinline__ unsigned long long kmin(float v, int pos) { return key_min(v, pos); }
__device__ __forceinline__ unsigned long long kmax(float v, int pos) { return key_max(v, pos); }
__device__ __forceinline__ int kpos_min(unsigned long long k) { return key_min_index(k); }
__device__ __forceinline__ int kpos_max(unsigned long long k) { return key_max_index(k); }

__device__ __forceinline__ float comp(const TriDev& t, int c) {
    switch (c) {
        case 0: return t.bmin.x;
        case 1: return t.bmin.y;
        case 2: return t.bmin.z;
        case 3: return t.bmax.x;
        case 4: return t.bmax.y;
        default: return t.bmax.z;
    }
}
__device__ __forceinline__ float cen(const TriDev& t, int a) { return a == 0 ? t.centroid.x : (a == 1 ? t.centroid.y : t.centroid.z); }

// fillBuckets' bucket (src/TriangleMesh.cpp:31-32)
// (clamped below at 0 too: a centroid rounded below its node's minimum would give the
// reference a negative bucket, outside its array)
__device__ __forceinline__ int bucket_of(float c, float s, float len) {
    return max(0, min(kBk - 1, (int)((c - s) / len * kBk)));
}
// subdivide's partition test (src/TriangleMesh.cpp:116-117): the same expression unclamped
__device__ __forceinline__ bool goes_left(float c, float s, float len, int split) {
    return (int)((c - s) / len * kBk) < split;
}

// Bounds::area (src/Bounds.cpp:28-31)
__device__ __forceinline__ float area6(const float* b) {
    const float dx = b[3] - b[0], dy = b[4] - b[1], dz = b[5] - b[2];
    return 2 * (dx * dy + dy * dz + dz * dx);
}

// chooseSplit / evaluateSplit (src/TriangleMesh.cpp:42-99) across a warp, from decoded
// bins val[bin * 6 + c] and cnt[bin]: lane c < 15 evaluates candidate (axis c / 5, split c % 5 + 1)
// as evaluateSplit does; scanning the candidates in that order with the reference's
// strict "cost < bestCost" from FLT_MAX picks the same split as its sequential loop.
// Returns the pick (-1: no split; the same on every lane); lane `pick` holds its L, R,
// cl and cr.
__device__ int warp_choose(const float* val, const int* cnt, const float* nb, float* L, float* R, int& cl, int& cr) {
    const int lane = threadIdx.x & 31;
    bool valid = false;
    float cost = 0.f;
    cl = cr = 0;
    if (lane < 3 * (kBk - 1)) {
        const int a = lane / (kBk - 1), sp = lane % (kBk - 1) + 1;
        if (nb[3 + a] - nb[a]) {
            float l[6] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
            float r[6] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
            int nl = 0, nr = 0;
            for (int i = 0; i < kBk; ++i) {
                const float* v = val + (a * kBk + i) * 6;
                float* d = i < sp ? l : r;
                for (int c = 0; c < 3; ++c) { d[c] = fminG(d[c], v[c]); d[3 + c] = fmaxG(d[3 + c], v[3 + c]); }
                if (i < sp) nl += cnt[a * kBk + i]; else nr += cnt[a * kBk + i];
            }
            if (nl && nr) {
                valid = true;
                cost = nl * area6(l) + nr * area6(r);
                cl = nl; cr = nr;
                for (int c = 0; c < 6; ++c) { L[c] = l[c]; R[c] = r[c]; }
            }
        }
    }
    float best = FLT_MAX;
    int pick = -1;
    for (int c = 0; c < 3 * (kBk - 1); ++c) {
        const float cc = __shfl_sync(0xffffffffu, cost, c);
        const int vv = __shfl_sync(0xffffffffu, (int)valid, c);
        if (vv && cc < best) { best = cc; pick = c; }
    }
    return pick;
}

// new node record; returns its id (or -1 past capacity)
__device__ int new_node(const Build& B, int start, int count, int mesh, int depth, int rturns, int parent, int side,
                        const float* b) {
    const int id = atomicAdd(B.n_nodes, 1);
    if (id >= B.node_cap) { atomicOr(B.err, 1); return -1; }
    BNode n;
    n.start = start; n.count = count; n.mesh = mesh; n.depth = depth; n.rturns = rturns; n.parent = parent;
    n.side = side; n.leaf = count <= 1; n.rank = -1; n.pad = 0;
    for (int c = 0; c < 3; ++c) { n.bmin[c] = b[c]; n.bmax[c] = b[3 + c]; }
    B.nodes[id] = n;
    return id;
}

// a node above kSmall triangles joins the level: a slot, empty bins, its chunks
__device__ void add_slot(const Level& Lv, int node, int count, const Build& B) {
    const int s = atomicAdd(Lv.n_slots, 1);
    const int nch = (count + kChunk - 1) / kChunk;
    const int cb = atomicAdd(Lv.n_chunks, nch);
    if (s >= Lv.slot_cap || cb + nch > Lv.chunk_cap) {
        atomicOr(B.err, 2);
        for (int i = 0; i < nch && cb + i < Lv.chunk_cap; ++i) Lv.chunk_slot[cb + i] = -1;
        return;
    }
    Slot sl;
    sl.node = node; sl.chunk_base = cb; sl.nchunks = nch; sl.ok = 0;
    sl.axis = sl.split = sl.k = sl.r = 0;
    Lv.slots[s] = sl;
    for (int i = 0; i < kKeys; ++i) Lv.keys[(size_t)s * kKeys + i] = (i % 6) < 3 ? kMinInit : kMaxInit;
    for (int i = 0; i < kBins; ++i) Lv.cnt[(size_t)s * kBins + i] = 0;
    for (int i = 0; i < nch; ++i) { Lv.chunk_slot[cb + i] = s; Lv.chunk_k[cb + i] = i; }
}

__device__ void route_child(const Build& B, const Level& next, int id) {
    if (id < 0) return;
    const int count = B.nodes[id].count;
    if (count <= 1) return;
    if (count <= kSmall) {
        const int i = atomicAdd(B.n_small, 1);
        B.small[i] = id;   // at most one entry per node: n_small < node_cap
    } else {
        add_slot(next, id, count, B);
    }
}

// ---------------------------------------------------------------- triangles and roots

// TriangleMesh's constructor (src/TriangleMesh.cpp:144-160): bounds, normal, centroid
__global__ void k_tri_setup(Build B) {
    for (int t = B.tri_lo + blockIdx.x * blockDim.x + threadIdx.x; t < B.n_tris; t += gridDim.x * blockDim.x) {
        const int4 ix = B.idx[t];
        const int vb = ix.w;   // the mesh's first vertex
        const V3 a = ld3(B.verts[vb + ix.x]), b = ld3(B.verts[vb + ix.y]), c = ld3(B.verts[vb + ix.z]);
        TriDev d;
        d.idx = make_int4(ix.x, ix.y, ix.z, 0);
        d.bmin = st4(vmin(vmin(a, b), c));
        d.bmax = st4(vmax(vmax(a, b), c));
        d.normal = st4(normalize(cross(b - a, c - a)));
        d.centroid = st4((a + b + c) / 3.f);
        B.tri[t] = d;
        B.perm[t] = t;
    }
}

// updateNodeBounds of each root (src/TriangleMesh.cpp:7-14): keys per mesh, one chunk a block
__global__ void __launch_bounds__(kThreads) k_root_keys(Build B, const int2* chunks, int n_chunks,
                                                         unsigned long long* root_keys) {
    __shared__ unsigned long long sk[6];
    for (int c = blockIdx.x; c < n_chunks; c += gridDim.x) {
        const int m = chunks[c].x;
        const BuildMesh M = B.meshes[m];
        const int p0 = M.tri_start + chunks[c].y * kChunk, p1 = min(p0 + kChunk, M.tri_start + M.tri_count);
        if (threadIdx.x < 6) sk[threadIdx.x] = threadIdx.x < 3 ? kMinInit : kMaxInit;
        __syncthreads();
        unsigned long long k[6] = {kMinInit, kMinInit, kMinInit, kMaxInit, kMaxInit, kMaxInit};
        for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
            const TriDev& t = B.tri[p];
            for (int i = 0; i < 3; ++i) k[i] = min(k[i], kmin(comp(t, i), p));
            for (int i = 3; i < 6; ++i) k[i] = max(k[i], kmax(comp(t, i), p));
        }
        for (int o = 16; o; o >>= 1)
            for (int i = 0; i < 6; ++i) {
                const unsigned long long v = __shfl_xor_sync(0xffffffffu, k[i], o);
                k[i] = i < 3 ? min(k[i], v) : max(k[i], v);
            }
        if ((threadIdx.x & 31) == 0)
            for (int i = 0; i < 6; ++i) i < 3 ? atomicMin(&sk[i], k[i]) : atomicMax(&sk[i], k[i]);
        __syncthreads();
        if (threadIdx.x < 6) {
            const int i = threadIdx.x;
            i < 3 ? atomicMin(&root_keys[m * 6 + i], sk[i]) : atomicMax(&root_keys[m * 6 + i], sk[i]);
        }
        __syncthreads();
    }
}

// root nodes: ids 0 .. n_meshes-1
__global__ void k_roots(Build B, int n_meshes, const unsigned long long* root_keys, Level L0) {
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n_meshes; m += gridDim.x * blockDim.x) {
        const BuildMesh M = B.meshes[m];
        float b[6];
        for (int i = 0; i < 6; ++i) {
            const unsigned long long k = root_keys[m * 6 + i];
            b[i] = comp(B.tri[i < 3 ? kpos_min(k) : kpos_max(k)], i);
        }
        BNode n;
        n.start = M.tri_start; n.count = M.tri_count; n.mesh = m; n.depth = 0; n.rturns = 0; n.parent = -1;
        n.side = 0; n.leaf = M.tri_count <= 1; n.rank = -1; n.pad = 0;
        for (int c = 0; c < 3; ++c) { n.bmin[c] = b[c]; n.bmax[c] = b[3 + c]; }
        B.nodes[m] = n;
        if (M.tri_count <= 1) continue;
        if (M.tri_count <= kSmall) B.small[atomicAdd(B.n_small, 1)] = m;
        else add_slot(L0, m, M.tri_count, B);
    }
}

// ---------------------------------------------------------------- one level

// fillBuckets for every axis (src/TriangleMesh.cpp:16-40), one chunk a block.  A thread
// takes kPer consecutive triangles and folds runs that share a bucket before it
// touches shared memory.
__global__ void __launch_bounds__(kThreads) k_level_bins(Build B, Level Lv) {
    __shared__ unsigned long long sk[kKeys];
    __shared__ int sc[kBins];
    const int nc = min(*Lv.n_chunks, Lv.chunk_cap), ns = min(*Lv.n_slots, Lv.slot_cap);
    for (int c = blockIdx.x; c < nc; c += gridDim.x) {
        const int si = Lv.chunk_slot[c];
        if (si < 0 || si >= ns) continue;
        const Slot sl = Lv.slots[si];
        const BNode nd = B.nodes[sl.node];
        for (int i = threadIdx.x; i < kKeys; i += blockDim.x) sk[i] = (i % 6) < 3 ? kMinInit : kMaxInit;
        for (int i = threadIdx.x; i < kBins; i += blockDim.x) sc[i] = 0;
        __syncthreads();
        float s[3], len[3];
        for (int a = 0; a < 3; ++a) { s[a] = nd.bmin[a]; len[a] = nd.bmax[a] - nd.bmin[a]; }
        const int base = nd.start + Lv.chunk_k[c] * kChunk, end = nd.start + nd.count;
        int cur[3] = {-1, -1, -1}, n[3] = {0, 0, 0};
        unsigned long long k[3][6];
        auto flush = [&](int a) {
            if (!n[a]) return;
            unsigned long long* d = sk + (a * kBk + cur[a]) * 6;
            for (int i = 0; i < 3; ++i) atomicMin(&d[i], k[a][i]);
            for (int i = 3; i < 6; ++i) atomicMax(&d[i], k[a][i]);
            atomicAdd(&sc[a * kBk + cur[a]], n[a]);
        };
        for (int j = 0; j < kPer; ++j) {
            const int p = base + threadIdx.x * kPer + j;
            if (p >= end) break;
            const TriDev t = B.tri[B.perm[p]];
            unsigned long long kv[6];
            for (int i = 0; i < 3; ++i) kv[i] = kmin(comp(t, i), p);
            for (int i = 3; i < 6; ++i) kv[i] = kmax(comp(t, i), p);
            for (int a = 0; a < 3; ++a) {
                if (!len[a]) continue;
                const int bi = bucket_of(cen(t, a), s[a], len[a]);
                if (bi != cur[a]) {
                    flush(a);
                    cur[a] = bi; n[a] = 0;
                    for (int i = 0; i < 6; ++i) k[a][i] = i < 3 ? kMinInit : kMaxInit;
                }
                for (int i = 0; i < 3; ++i) k[a][i] = min(k[a][i], kv[i]);
                for (int i = 3; i < 6; ++i) k[a][i] = max(k[a][i], kv[i]);
                ++n[a];
            }
        }
        for (int a = 0; a < 3; ++a) flush(a);
        __syncthreads();
        const size_t so = (size_t)si;
        for (int i = threadIdx.x; i < kKeys; i += blockDim.x) {
            const unsigned long long v = sk[i];
            if ((i % 6) < 3) { if (v != kMinInit) atomicMin(&Lv.keys[so * kKeys + i], v); }
            else if (v != kMaxInit) atomicMax(&Lv.keys[so * kKeys + i], v);
        }
        for (int i = threadIdx.x; i < kBins; i += blockDim.x)
            if (sc[i]) atomicAdd(&Lv.cnt[so * kBins + i], sc[i]);
        __syncthreads();
    }
}

// chooseSplit for each node of the level, a warp per node; its children join the next
// level, the small list, or are leaves
constexpr int kChooseWarps = 4;
__global__ void __launch_bounds__(32 * kChooseWarps) k_level_choose(Build B, Level Lv, Level next) {
    __shared__ float sval[kChooseWarps][kKeys];
    __shared__ int scnt[kChooseWarps][kBins];
    const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ns = min(*Lv.n_slots, Lv.slot_cap);
    for (int s = blockIdx.x * kChooseWarps + wi; s < ns; s += gridDim.x * kChooseWarps) {
        Slot sl = Lv.slots[s];
        const BNode nd = B.nodes[sl.node];
        if (lane < kBins) scnt[wi][lane] = Lv.cnt[(size_t)s * kBins + lane];
        __syncwarp();
        for (int i = lane; i < kKeys; i += 32) {
            const int c = i % 6;
            if (!scnt[wi][i / 6]) { sval[wi][i] = c < 3 ? FLT_MAX : -FLT_MAX; continue; }
            const unsigned long long k = Lv.keys[(size_t)s * kKeys + i];
            sval[wi][i] = comp(B.tri[B.perm[c < 3 ? kpos_min(k) : kpos_max(k)]], c);
        }
        __syncwarp();
        const float nb[6] = {nd.bmin[0], nd.bmin[1], nd.bmin[2], nd.bmax[0], nd.bmax[1], nd.bmax[2]};
        float L[6], R[6];
        int cl, cr;
        const int pick = warp_choose(sval[wi], scnt[wi], nb, L, R, cl, cr);
        if (pick < 0) {
            if (lane == 0) B.nodes[sl.node].leaf = 1;
        } else if (lane == pick) {
            sl.ok = 1; sl.axis = pick / (kBk - 1); sl.split = pick % (kBk - 1) + 1; sl.k = cl;
            Lv.slots[s] = sl;
            const int l = new_node(B, nd.start, cl, nd.mesh, nd.depth + 1, nd.rturns, sl.node, 0, L);
            const int r = new_node(B, nd.start + cl, cr, nd.mesh, nd.depth + 1, nd.rturns + 1, sl.node, 1, R);
            route_child(B, next, l);
            route_child(B, next, r);
        }
        __syncwarp();
    }
}

// labels, then front-right / back-left counts of each chunk of a split node
__global__ void __launch_bounds__(kThreads) k_level_count(Build B, Level Lv) {
    __shared__ int s_fr, s_bl;
    const int nc = min(*Lv.n_chunks, Lv.chunk_cap), ns = min(*Lv.n_slots, Lv.slot_cap);
    for (int c = blockIdx.x; c < nc; c += gridDim.x) {
        const int si = Lv.chunk_slot[c];
        if (si < 0 || si >= ns) continue;
        const Slot sl = Lv.slots[si];
        if (!sl.ok) continue;
        const BNode nd = B.nodes[sl.node];
        if (threadIdx.x == 0) { s_fr = 0; s_bl = 0; }
        __syncthreads();
        const float s = nd.bmin[sl.axis], len = nd.bmax[sl.axis] - nd.bmin[sl.axis];
        const int base = nd.start + Lv.chunk_k[c] * kChunk, end = nd.start + nd.count;
        int fr = 0, bl = 0;
        for (int p = base + threadIdx.x; p < min(base + kChunk, end); p += blockDim.x) {
            const bool left = goes_left(cen(B.tri[B.perm[p]], sl.axis), s, len, sl.split);
            B.lab[p] = left;
            const bool front = p - nd.start < sl.k;
            fr += front && !left;
            bl += !front && left;
        }
        for (int o = 16; o; o >>= 1) { fr += __shfl_xor_sync(0xffffffffu, fr, o); bl += __shfl_xor_sync(0xffffffffu, bl, o); }
        if ((threadIdx.x & 31) == 0) { atomicAdd(&s_fr, fr); atomicAdd(&s_bl, bl); }
        __syncthreads();
        if (threadIdx.x == 0) Lv.chunk_cnt[c] = make_int2(s_fr, s_bl);
        __syncthreads();
    }
}

// per split node: chunk offsets in position order, and r
__global__ void k_level_scan(Level Lv, int* err) {
    const int ns = min(*Lv.n_slots, Lv.slot_cap);
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
        Slot sl = Lv.slots[s];
        if (!sl.ok) continue;
        int a = 0, b = 0;
        for (int i = 0; i < sl.nchunks; ++i) {
            const int2 v = Lv.chunk_cnt[sl.chunk_base + i];
            Lv.chunk_off[sl.chunk_base + i] = make_int2(a, b);
            a += v.x; b += v.y;
        }
        sl.r = a;
        if (a != b) { sl.ok = 0; atomicOr(err, 16); }   // cannot happen: both count the misplaced pairs
        Lv.slots[s] = sl;
    }
}

// block-wide exclusive scan of one int per thread
__device__ __forceinline__ int block_excl(int v, int* sh, int& total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < (int)(blockDim.x >> 5)) sh[lane] = t;
    }
    __syncthreads();
    total = sh[(blockDim.x >> 5) - 1];
    const int r = x - v + (w ? sh[w - 1] : 0);
    __syncthreads();
    return r;
}

// ranks: fr / bl hold positions (relative to the node) by rank
__global__ void __launch_bounds__(kThreads) k_level_rank(Build B, Level Lv) {
    __shared__ int sh[kThreads / 32];
    const int nc = min(*Lv.n_chunks, Lv.chunk_cap), ns = min(*Lv.n_slots, Lv.slot_cap);
    for (int c = blockIdx.x; c < nc; c += gridDim.x) {
        const int si = Lv.chunk_slot[c];
        if (si < 0 || si >= ns) continue;
        const Slot sl = Lv.slots[si];
        if (!sl.ok) continue;
        const BNode nd = B.nodes[sl.node];
        const int2 off = Lv.chunk_off[c];
        const int base = nd.start + Lv.chunk_k[c] * kChunk, end = min(base + kChunk, nd.start + nd.count);
        const int p0 = base + threadIdx.x * kPer;
        int nfr = 0, nbl = 0;
        for (int j = 0; j < kPer; ++j) {
            const int p = p0 + j;
            if (p >= end) break;
            const bool left = B.lab[p], front = p - nd.start < sl.k;
            nfr += front && !left;
            nbl += !front && left;
        }
        int tfr, tbl;
        int rfr = block_excl(nfr, sh, tfr) + off.x;
        int rbl = block_excl(nbl, sh, tbl) + off.y;
        for (int j = 0; j < kPer; ++j) {
            const int p = p0 + j;
            if (p >= end) break;
            const int x = p - nd.start;
            const bool left = B.lab[p], front = x < sl.k;
            if (front && !left) { B.fr[nd.start + rfr] = x; B.rnk[p] = rfr++; }
            else if (!front && left) { B.bl[nd.start + rbl] = x; B.rnk[p] = rbl++; }
        }
    }
}

// final positions (the reference's two-pointer partition, in closed form)
__global__ void __launch_bounds__(kThreads) k_level_scatter(Build B, Level Lv) {
    const int nc = min(*Lv.n_chunks, Lv.chunk_cap), ns = min(*Lv.n_slots, Lv.slot_cap);
    for (int c = blockIdx.x; c < nc; c += gridDim.x) {
        const int si = Lv.chunk_slot[c];
        if (si < 0 || si >= ns) continue;
        const Slot sl = Lv.slots[si];
        if (!sl.ok) continue;
        const BNode nd = B.nodes[sl.node];
        const int base = nd.start + Lv.chunk_k[c] * kChunk, end = min(base + kChunk, nd.start + nd.count);
        const int n = nd.count, k = sl.k, r = sl.r;
        for (int p = base + threadIdx.x; p < end; p += blockDim.x) {
            const int x = p - nd.start;
            const bool left = B.lab[p];
            int dest;
            if (x < k) {
                // a front-right of rank t (0-based) goes below the back-left of rank t-1 from the end
                dest = left ? x : (B.rnk[p] == 0 ? n : B.bl[nd.start + r - B.rnk[p]]) - 1;
            } else if (left) {
                // the back-left of rank u from the start is the (r-u)-th from the end
                dest = B.fr[nd.start + r - 1 - B.rnk[p]];
            } else {
                dest = x == k ? (r ? B.bl[nd.start] : n) - 1 : x - 1;
            }
            if (dest < 0 || dest >= n) { atomicOr(B.err, 32); continue; }
            B.perm_tmp[nd.start + dest] = B.perm[p];
        }
    }
}

__global__ void k_level_copy(Build B, Level Lv) {
    const int nc = min(*Lv.n_chunks, Lv.chunk_cap), ns = min(*Lv.n_slots, Lv.slot_cap);
    for (int c = blockIdx.x; c < nc; c += gridDim.x) {
        const int si = Lv.chunk_slot[c];
        if (si < 0 || si >= ns) continue;
        const Slot sl = Lv.slots[si];
        if (!sl.ok) continue;
        const BNode nd = B.nodes[sl.node];
        const int base = nd.start + Lv.chunk_k[c] * kChunk, end = min(base + kChunk, nd.start + nd.count);
        for (int p = base + threadIdx.x; p < end; p += blockDim.x) B.perm[p] = B.perm_tmp[p];
    }
}

// ---------------------------------------------------------------- small subtrees

struct WarpSmem {
    unsigned long long key[kKeys];
    int cnt[kBins];
    float val[kKeys];
    int fr[kSmall], bl[kSmall], stage[kSmall], stack[kSmall];
    int choice[6];   // ok, axis, split, cl, left id, right id
    float lr[12];
};

// One warp builds the subtree of a node of at most kSmall triangles (two per lane),
// depth first with a stack in shared memory.
__global__ void __launch_bounds__(32 * kWarpsSmall) k_small_subtrees(Build B) {
    __shared__ WarpSmem smem[kWarpsSmall];
    WarpSmem& S = smem[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * kWarpsSmall;
    const int n_small = *B.n_small;
    for (int w = blockIdx.x * kWarpsSmall + (threadIdx.x >> 5); w < n_small; w += warps) {
        if (lane == 0) S.stack[0] = B.small[w];
        int top = 1;
        __syncwarp();
        while (top > 0) {
            const int id = S.stack[--top];
            __syncwarp();
            const BNode nd = B.nodes[id];
            for (int i = lane; i < kKeys; i += 32) S.key[i] = (i % 6) < 3 ? kMinInit : kMaxInit;
            if (lane < kBins) S.cnt[lane] = 0;
            __syncwarp();
            float s[3], len[3];
            for (int a = 0; a < 3; ++a) { s[a] = nd.bmin[a]; len[a] = nd.bmax[a] - nd.bmin[a]; }
            int pos[2], orig[2];
            for (int j = 0; j < 2; ++j) {
                const int x = lane + 32 * j;
                pos[j] = nd.start + x;
                orig[j] = x < nd.count ? B.perm[pos[j]] : -1;
                if (orig[j] < 0) continue;
                const TriDev t = B.tri[orig[j]];
                for (int a = 0; a < 3; ++a) {
                    if (!len[a]) continue;
                    const int bi = bucket_of(cen(t, a), s[a], len[a]);
                    unsigned long long* k = S.key + (a * kBk + bi) * 6;
                    for (int i = 0; i < 3; ++i) atomicMin(&k[i], kmin(comp(t, i), pos[j]));
                    for (int i = 3; i < 6; ++i) atomicMax(&k[i], kmax(comp(t, i), pos[j]));
                    atomicAdd(&S.cnt[a * kBk + bi], 1);
                }
            }
            __syncwarp();
            for (int i = lane; i < kKeys; i += 32) {
                const int c = i % 6;
                if (!S.cnt[i / 6]) { S.val[i] = c < 3 ? FLT_MAX : -FLT_MAX; continue; }
                const unsigned long long k = S.key[i];
                S.val[i] = comp(B.tri[B.perm[c < 3 ? kpos_min(k) : kpos_max(k)]], c);
            }
            __syncwarp();
            {
                const float nb[6] = {nd.bmin[0], nd.bmin[1], nd.bmin[2], nd.bmax[0], nd.bmax[1], nd.bmax[2]};
                float L[6], R[6];
                int cl, cr;
                const int pick = warp_choose(S.val, S.cnt, nb, L, R, cl, cr);
                if (pick < 0) {
                    if (lane == 0) { S.choice[0] = 0; B.nodes[id].leaf = 1; }
                } else if (lane == pick) {
                    S.choice[0] = 1; S.choice[1] = pick / (kBk - 1); S.choice[2] = pick % (kBk - 1) + 1; S.choice[3] = cl;
                    for (int c = 0; c < 6; ++c) { S.lr[c] = L[c]; S.lr[6 + c] = R[c]; }
                }
            }
            __syncwarp();
            if (!S.choice[0]) continue;
            const int axis = S.choice[1], split = S.choice[2], k = S.choice[3];
            bool left[2], fr[2], bl[2];
            for (int j = 0; j < 2; ++j) {
                const int x = lane + 32 * j;
                left[j] = orig[j] >= 0 && goes_left(cen(B.tri[orig[j]], axis), s[axis], len[axis], split);
                fr[j] = orig[j] >= 0 && x < k && !left[j];
                bl[j] = orig[j] >= 0 && x >= k && left[j];
            }
            const unsigned below = (1u << lane) - 1u;
            const unsigned mfr0 = __ballot_sync(0xffffffffu, fr[0]), mfr1 = __ballot_sync(0xffffffffu, fr[1]);
            const unsigned mbl0 = __ballot_sync(0xffffffffu, bl[0]), mbl1 = __ballot_sync(0xffffffffu, bl[1]);
            int rk[2];
            rk[0] = fr[0] ? __popc(mfr0 & below) : __popc(mbl0 & below);
            rk[1] = fr[1] ? __popc(mfr0) + __popc(mfr1 & below) : __popc(mbl0) + __popc(mbl1 & below);
            const int r = __popc(mfr0) + __popc(mfr1);
            for (int j = 0; j < 2; ++j) {
                if (fr[j]) S.fr[rk[j]] = lane + 32 * j;
                if (bl[j]) S.bl[rk[j]] = lane + 32 * j;
            }
            __syncwarp();
            const int n = nd.count;
            for (int j = 0; j < 2; ++j) {
                if (orig[j] < 0) continue;
                const int x = lane + 32 * j;
                int dest;
                if (x < k) dest = left[j] ? x : (rk[j] == 0 ? n : S.bl[r - rk[j]]) - 1;
                else if (left[j]) dest = S.fr[r - 1 - rk[j]];
                else dest = x == k ? (r ? S.bl[0] : n) - 1 : x - 1;
                if (dest < 0 || dest >= n) { atomicOr(B.err, 32); continue; }
                S.stage[dest] = orig[j];
            }
            __syncwarp();
            for (int j = 0; j < 2; ++j) {
                const int x = lane + 32 * j;
                if (x < n) B.perm[nd.start + x] = S.stage[x];
            }
            if (lane == 0) {
                const int l = new_node(B, nd.start, k, nd.mesh, nd.depth + 1, nd.rturns, id, 0, S.lr);
                const int rr = new_node(B, nd.start + k, n - k, nd.mesh, nd.depth + 1, nd.rturns + 1, id, 1, S.lr + 6);
                S.choice[4] = l; S.choice[5] = rr;
            }
            __syncwarp();
            const int l = S.choice[4], rr = S.choice[5];
            // at most one stack entry per pending leaf: the stack never outgrows kSmall
            if (l >= 0 && k > 1 && top < kSmall) { if (lane == 0) S.stack[top] = l; ++top; }
            if (rr >= 0 && n - k > 1 && top < kSmall) { if (lane == 0) S.stack[top] = rr; ++top; }
            __syncwarp();
        }
    }
}

// ---------------------------------------------------------------- node ids and output

__global__ void k_leaf_marks(Build B) {
    const int n = min(*B.n_nodes, B.node_cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (B.nodes[i].leaf) B.mark[B.nodes[i].start] = 1;
}

__global__ void k_node_ranks(Build B) {
    const int n = min(*B.n_nodes, B.node_cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const BNode nd = B.nodes[i];
        if (nd.leaf) continue;
        const int ms = B.meshes[nd.mesh].tri_start;
        B.nodes[i].rank = nd.depth + (B.lb[nd.start] - B.lb[ms]) - nd.rturns;
    }
}

__global__ void k_emit_nodes(Build B, TriNodeDev* out) {
    const int n = min(*B.n_nodes, B.node_cap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const BNode nd = B.nodes[i];
        const BuildMesh M = B.meshes[nd.mesh];
        const int id = nd.parent < 0 ? 0 : 2 * B.nodes[nd.parent].rank + 1 + nd.side;
        if (id < 0 || id >= max(1, 2 * M.tri_count - 1)) { atomicOr(B.err, 64); continue; }
        TriNodeDev o;
        o.bmin = make_float4(nd.bmin[0], nd.bmin[1], nd.bmin[2], __int_as_float(nd.leaf ? nd.count : 0));
        o.bmax = make_float4(nd.bmax[0], nd.bmax[1], nd.bmax[2],
                             __int_as_float(nd.leaf ? nd.start - M.tri_start : 2 * nd.rank + 1));
        out[M.node_start + id] = o;
    }
}

// a mesh's node count: 2 leaves - 1
__global__ void k_mesh_node_counts(Build B, int n_meshes, int* mesh_nodes) {
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n_meshes; m += gridDim.x * blockDim.x) {
        const BuildMesh M = B.meshes[m];
        mesh_nodes[m] = 2 * (B.lb[M.tri_start + M.tri_count] - B.lb[M.tri_start]) - 1;
    }
}

__global__ void k_emit_tris(Build B, TriDev* out) {
    for (int p = B.tri_lo + blockIdx.x * blockDim.x + threadIdx.x; p < B.n_tris; p += gridDim.x * blockDim.x)
        out[p] = B.tri[B.perm[p]];
}

}  // namespace

// ---------------------------------------------------------------- host

struct MeshBuildScratch {
    std::vector<void*> ptrs;
    template <class T>
    cudaError_t get(T*& p, size_t n) {
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, std::max<size_t>(1, n) * sizeof(T));
        if (e == cudaSuccess) ptrs.push_back(q);
        p = (T*)q;
        return e;
    }
    ~MeshBuildScratch() { for (void* q : ptrs) cudaFree(q); }
};

cudaError_t build_mesh_bvhs(const float4* verts, const int4* idx, const std::vector<BuildMesh>& meshes, TriDev* tris_out,
                            TriNodeDev* nodes_out, std::vector<int>& node_counts, int* err_out, cudaStream_t st) {
    node_counts.assign(meshes.size(), 0);
    *err_out = 0;
    std::vector<BuildMesh> work;
    std::vector<int> work_of;
    for (size_t i = 0; i < meshes.size(); ++i)
        if (meshes[i].tri_count > 0) { work.push_back(meshes[i]); work_of.push_back((int)i); }
    // the meshes with triangles must tile one range of positions
    int tri_lo = 0, n_tris = 0;
    {
        std::vector<BuildMesh> srt = work;
        std::sort(srt.begin(), srt.end(), [](const BuildMesh& a, const BuildMesh& b) { return a.tri_start < b.tri_start; });
        if (!srt.empty()) tri_lo = srt[0].tri_start;
        n_tris = tri_lo;
        for (const BuildMesh& m : srt) {
            if (m.tri_start != n_tris) { *err_out = 8; return cudaSuccess; }
            n_tris += m.tri_count;
        }
    }
    // a mesh without triangles: one empty leaf (the reference's root over no triangle)
    for (size_t i = 0; i < meshes.size(); ++i) {
        if (meshes[i].tri_count > 0) continue;
        TriNodeDev e;   // triCount 0, index 0: both w words are zero bits
        e.bmin = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.f);
        e.bmax = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f);
        cudaError_t ce = cudaMemcpyAsync(nodes_out + meshes[i].node_start, &e, sizeof(e), cudaMemcpyHostToDevice, st);
        if (ce != cudaSuccess) return ce;
        node_counts[i] = 1;
    }
    if (work.empty()) return cudaStreamSynchronize(st);
    const int nm = (int)work.size();

#define MB_TRY(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return e_; } while (0)
    MeshBuildScratch S;
    Build B{};
    B.verts = verts;
    B.idx = idx;
    B.tri_lo = tri_lo;
    B.n_tris = n_tris;
    int total = 0;
    for (const BuildMesh& m : work) total += m.tri_count;
    B.node_cap = 2 * total + nm;
    BuildMesh* d_meshes;
    MB_TRY(S.get(d_meshes, nm));
    MB_TRY(cudaMemcpyAsync(d_meshes, work.data(), sizeof(BuildMesh) * nm, cudaMemcpyHostToDevice, st));
    B.meshes = d_meshes;
    MB_TRY(S.get(B.tri, n_tris));
    MB_TRY(S.get(B.perm, n_tris));
    MB_TRY(S.get(B.perm_tmp, n_tris));
    MB_TRY(S.get(B.lab, n_tris));
    MB_TRY(S.get(B.rnk, n_tris));
    MB_TRY(S.get(B.fr, n_tris));
    MB_TRY(S.get(B.bl, n_tris));
    MB_TRY(S.get(B.nodes, B.node_cap));
    MB_TRY(S.get(B.n_nodes, 1));
    MB_TRY(S.get(B.small, B.node_cap));
    MB_TRY(S.get(B.n_small, 1));
    MB_TRY(S.get(B.mark, n_tris + 1));
    MB_TRY(S.get(B.lb, n_tris + 1));
    MB_TRY(S.get(B.err, 1));
    int* d_total;
    MB_TRY(S.get(d_total, 1));
    int* scratch;
    MB_TRY(S.get(scratch, scan_scratch_ints(n_tris + 1)));
    MB_TRY(cudaMemsetAsync(B.n_nodes, 0, sizeof(int), st));
    MB_TRY(cudaMemsetAsync(B.n_small, 0, sizeof(int), st));
    MB_TRY(cudaMemsetAsync(B.err, 0, sizeof(int), st));
    MB_TRY(cudaMemsetAsync(B.mark, 0, sizeof(int) * (n_tris + 1), st));
    // root nodes take ids 0 .. nm-1
    MB_TRY(cudaMemcpyAsync(B.n_nodes, &nm, sizeof(int), cudaMemcpyHostToDevice, st));

    Level L[2];
    const int slot_cap = total / kSmall + nm + 1;
    const int chunk_cap = slot_cap + total / kChunk + 1;
    for (Level& v : L) {
        v.slot_cap = slot_cap;
        v.chunk_cap = chunk_cap;
        MB_TRY(S.get(v.slots, slot_cap));
        MB_TRY(S.get(v.n_slots, 1));
        MB_TRY(S.get(v.keys, (size_t)slot_cap * kKeys));
        MB_TRY(S.get(v.cnt, (size_t)slot_cap * kBins));
        MB_TRY(S.get(v.chunk_slot, chunk_cap));
        MB_TRY(S.get(v.chunk_k, chunk_cap));
        MB_TRY(S.get(v.n_chunks, 1));
        MB_TRY(S.get(v.chunk_cnt, chunk_cap));
        MB_TRY(S.get(v.chunk_off, chunk_cap));
        MB_TRY(cudaMemsetAsync(v.n_slots, 0, sizeof(int), st));
        MB_TRY(cudaMemsetAsync(v.n_chunks, 0, sizeof(int), st));
    }

    const int grid = 152 * 4;
    k_tri_setup<<<grid, 256, 0, st>>>(B);
    // roots: bounds over each mesh's triangles in their original order
    std::vector<int2> rc;
    for (int m = 0; m < nm; ++m)
        for (int c = 0; c * kChunk < work[m].tri_count; ++c) rc.push_back(make_int2(m, c));
    int2* d_rc;
    unsigned long long* d_rk;
    MB_TRY(S.get(d_rc, rc.size()));
    MB_TRY(S.get(d_rk, (size_t)nm * 6));
    MB_TRY(cudaMemcpyAsync(d_rc, rc.data(), sizeof(int2) * rc.size(), cudaMemcpyHostToDevice, st));
    {
        std::vector<unsigned long long> init((size_t)nm * 6);
        for (size_t i = 0; i < init.size(); ++i) init[i] = (i % 6) < 3 ? kMinInit : kMaxInit;
        MB_TRY(cudaMemcpyAsync(d_rk, init.data(), sizeof(unsigned long long) * init.size(), cudaMemcpyHostToDevice, st));
        k_root_keys<<<std::min<int>(grid, (int)rc.size()), kThreads, 0, st>>>(B, d_rc, (int)rc.size(), d_rk);
        k_roots<<<(nm + 127) / 128, 128, 0, st>>>(B, nm, d_rk, L[0]);
        MB_TRY(cudaStreamSynchronize(st));   // the host vectors above go out of scope
    }
    // top levels
    int* h_cnt = nullptr;
    MB_TRY(cudaMallocHost(&h_cnt, sizeof(int)));
    cudaError_t le = cudaSuccess;
    // every level lowers the largest remaining node by at least one triangle
    bool done = false;
    for (int lv = 0; lv <= total; ++lv) {
        Level& cur = L[lv & 1];
        Level& nxt = L[(lv + 1) & 1];
        cudaMemcpyAsync(h_cnt, cur.n_slots, sizeof(int), cudaMemcpyDeviceToHost, st);
        le = cudaStreamSynchronize(st);
        if (le != cudaSuccess) break;
        if (*h_cnt == 0) { done = true; break; }
        k_level_bins<<<grid, kThreads, 0, st>>>(B, cur);
        k_level_choose<<<(std::min(*h_cnt, slot_cap) + kChooseWarps - 1) / kChooseWarps, 32 * kChooseWarps, 0, st>>>(B, cur, nxt);
        k_level_count<<<grid, kThreads, 0, st>>>(B, cur);
        k_level_scan<<<(std::min(*h_cnt, slot_cap) + 127) / 128, 128, 0, st>>>(cur, B.err);
        k_level_rank<<<grid, kThreads, 0, st>>>(B, cur);
        k_level_scatter<<<grid, kThreads, 0, st>>>(B, cur);
        k_level_copy<<<grid, kThreads, 0, st>>>(B, cur);
        cudaMemsetAsync(cur.n_slots, 0, sizeof(int), st);
        cudaMemsetAsync(cur.n_chunks, 0, sizeof(int), st);
    }
    cudaFreeHost(h_cnt);
    MB_TRY(le);
    if (!done) { *err_out = 4; return cudaSuccess; }
    k_small_subtrees<<<grid * 2, 32 * kWarpsSmall, 0, st>>>(B);
    // node ids
    k_leaf_marks<<<grid, 256, 0, st>>>(B);
    scan_exclusive(B.mark, B.lb, n_tris + 1, d_total, scratch, st);
    k_node_ranks<<<grid, 256, 0, st>>>(B);
    int* d_mesh_nodes;
    MB_TRY(S.get(d_mesh_nodes, nm));
    k_emit_nodes<<<grid, 256, 0, st>>>(B, nodes_out);
    k_mesh_node_counts<<<(nm + 127) / 128, 128, 0, st>>>(B, nm, d_mesh_nodes);
    k_emit_tris<<<grid, 256, 0, st>>>(B, tris_out);
    std::vector<int> mn(nm);
    int err = 0;
    MB_TRY(cudaMemcpyAsync(mn.data(), d_mesh_nodes, sizeof(int) * nm, cudaMemcpyDeviceToHost, st));
    MB_TRY(cudaMemcpyAsync(&err, B.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    MB_TRY(cudaStreamSynchronize(st));
    MB_TRY(cudaGetLastError());
    for (int m = 0; m < nm; ++m) node_counts[work_of[m]] = mn[m];
    *err_out = err;
#undef MB_TRY
    return cudaSuccess;
}

}  // namespace psx

// ---------------------------------------------------------------- C ABI

#include <cmath>
#include "runtime.cuh"

namespace {

using namespace psx;
using namespace psx::rt;

psx_status check_vertices(const float* v, int n) {
    for (int i = 0; i < 3 * n; ++i)
        if (!std::isfinite(v[i])) return fail(PSX_ERR_INVALID_ARG, "triangle mesh: vertex not finite");
    return PSX_OK;
}

template <class T>
struct DevArr {
    T* p = nullptr;
    ~DevArr() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, std::max<size_t>(1, n) * sizeof(T)); }
};

}  // namespace

extern "C" {

PSX_API psx_status psx_trimesh_build(int32_t device, const float* vertices, int32_t n_vertices, const uint32_t* indices,
                                     int32_t n_indices, psx_trimesh_triangle* triangles, psx_trimesh_node* nodes,
                                     int32_t* n_nodes) {
    if (n_vertices < 0 || n_indices < 0 || (n_vertices && !vertices) || (n_indices && !indices) || !nodes || !n_nodes ||
        (n_indices >= 3 && !triangles))
        return fail(PSX_ERR_INVALID_ARG, "psx_trimesh_build: bad arguments");
    const int nt = n_indices / 3;
    for (int i = 0; i < 3 * nt; ++i)
        if (indices[i] >= (uint32_t)n_vertices) return fail(PSX_ERR_INVALID_ARG, "psx_trimesh_build: vertex index out of range");
    PSX_TRY(check_vertices(vertices, n_vertices));
    PSX_CUDA(cudaSetDevice(device));
    static_assert(sizeof(psx_trimesh_triangle) == sizeof(TriDev), "psx_trimesh_triangle layout");
    static_assert(sizeof(psx_trimesh_node) == sizeof(TriNodeDev), "psx_trimesh_node layout");
    std::vector<float4> v(n_vertices);
    for (int i = 0; i < n_vertices; ++i) v[i] = make_float4(vertices[3 * i], vertices[3 * i + 1], vertices[3 * i + 2], 0.f);
    std::vector<int4> ix(nt);
    for (int t = 0; t < nt; ++t) ix[t] = make_int4((int)indices[3 * t], (int)indices[3 * t + 1], (int)indices[3 * t + 2], 0);
    const int ncap = std::max(1, 2 * nt - 1);
    DevArr<float4> dv;
    DevArr<int4> di;
    DevArr<TriDev> dt;
    DevArr<TriNodeDev> dn;
    PSX_CUDA(dv.alloc(n_vertices));
    PSX_CUDA(di.alloc(nt));
    PSX_CUDA(dt.alloc(nt));
    PSX_CUDA(dn.alloc(ncap));
    cudaStream_t st;
    PSX_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamDestroy(s); } } guard{st};
    if (n_vertices) PSX_CUDA(cudaMemcpyAsync(dv.p, v.data(), sizeof(float4) * n_vertices, cudaMemcpyHostToDevice, st));
    if (nt) PSX_CUDA(cudaMemcpyAsync(di.p, ix.data(), sizeof(int4) * nt, cudaMemcpyHostToDevice, st));
    std::vector<int> counts;
    int err = 0;
    PSX_CUDA(build_mesh_bvhs(dv.p, di.p, {BuildMesh{0, nt, 0, 0}}, dt.p, dn.p, counts, &err, st));
    if (err) return fail(PSX_ERR_CAPACITY, "psx_trimesh_build: build capacity");
    if (nt) PSX_CUDA(cudaMemcpyAsync(triangles, dt.p, sizeof(TriDev) * nt, cudaMemcpyDeviceToHost, st));
    PSX_CUDA(cudaMemcpyAsync(nodes, dn.p, sizeof(TriNodeDev) * counts[0], cudaMemcpyDeviceToHost, st));
    PSX_CUDA(cudaStreamSynchronize(st));
    *n_nodes = counts[0];
    return PSX_OK;
}

PSX_API psx_status psx_world_update_trimesh(psx_world* W, int32_t scene, int32_t mesh, const float* vertices) {
    if (!W || scene < 0 || scene >= W->n_scenes || !vertices) return fail(PSX_ERR_INVALID_ARG, "psx_world_update_trimesh: bad arguments");
    const int m = W->h_scene_trimesh[scene] + mesh;
    if (mesh < 0 || m >= W->h_scene_trimesh[scene + 1]) return fail(PSX_ERR_INVALID_ARG, "psx_world_update_trimesh: mesh index");
    const TriMeshDev tm = W->h_trimesh[m];
    PSX_TRY(check_vertices(vertices, tm.vert_count));
    PSX_CUDA(cudaSetDevice(W->device));
    PSX_CUDA(cudaStreamSynchronize(W->stream));
    std::vector<float4> v(tm.vert_count);
    for (int i = 0; i < tm.vert_count; ++i) v[i] = make_float4(vertices[3 * i], vertices[3 * i + 1], vertices[3 * i + 2], 0.f);
    if (tm.vert_count)
        PSX_CUDA(cudaMemcpyAsync(W->w.tri_verts + tm.vert_start, v.data(), sizeof(float4) * tm.vert_count,
                                 cudaMemcpyHostToDevice, W->stream));
    std::vector<int> counts;
    int err = 0;
    PSX_CUDA(build_mesh_bvhs(W->w.tri_verts, W->w.tri_src, {BuildMesh{tm.tri_start, tm.tri_count, tm.vert_start, tm.node_start}},
                             W->w.tris, W->w.tri_nodes, counts, &err, W->stream));
    if (err) return fail(PSX_ERR_CAPACITY, "psx_world_update_trimesh: build capacity");
    for (int c = 0; c < (int)W->h_col_trimesh.size(); ++c)
        if (W->h_col_trimesh[c] == m) launch_aabb_range(W->w, c, c + 1, 0, W->stream);
    PSX_CUDA(cudaStreamSynchronize(W->stream));
    return PSX_OK;
}

}  // extern "C"
