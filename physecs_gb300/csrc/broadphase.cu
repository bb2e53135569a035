// broadphase.cu — collider bounds and the LBVH broadphase.
//
// Replaces the reference's sweep-and-prune (Physecs src/Physecs.cpp:119-173).  The
// pair SET is identical: a pair is reported iff both colliders have
// enableSimulation, they belong to different entities, at least one is dynamic, and
// their bounds overlap inclusively on all three axes — exactly the SAP conditions.
// Steps per frame: per-scene centroid bounds -> 30-bit Morton keys -> radix sort
// by (scene, Morton) -> Karras (2012) radix tree per scene segment -> bottom-up
// refit -> per-leaf traversal (count, scan, emit) writing canonical pairs
// (entity0 < entity1, src/Physecs.cpp:156-170), each leaf's pairs ordered by
// partner collider.
#include "frame.cuh"
#include "ordkey.cuh"
#include "narrow_convex.cuh"

namespace psx {

// ---------------------------------------------------------------- bounds

// getBounds (src/BoundsUtil.cpp:23-85) at the collider's world pose (src/Physecs.cpp:79-90).
// margin_mode 0: every collider, no margin (onRigidBodyCreate, src/Physecs.cpp:25-37);
// margin_mode 1: colliders of simulated dynamic bodies, +0.01 m (src/Physecs.cpp:555-559).
__global__ void k_aabb(World w, int c0, int c1, int margin_mode) {
    int c = c0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= c1) return;
    int4 ci = w.col_info[c];
    int4 bi = w.info[ci.x];
    bool simulated = (bi.y & BODY_DYN) && !(bi.y & BODY_KIN);
    if (margin_mode == 1 && !simulated) return;
    if (ci.y == G_TRIMESH) return;   // k_trimesh_bounds (no margin: a mesh never gets one)
    Q4 bq = ld4(w.quat[ci.x]);
    V3 bp = ld3(w.pos[ci.x]);
    V3 pos = bp + qrot(bq, ld3(w.col_pos[c]));
    Q4 ori = qmul(bq, ld4(w.col_quat[c]));
    float4 pr = w.col_params[c];
    GeomD g{ci.y, {pr.x, pr.y, pr.z}, ci.z};
    Bounds b;
    b = getBounds(w, pos, ori, g);
    if (margin_mode == 1) { b.max += v3s(0.01f); b.min -= v3s(0.01f); }
    w.aabb_min[c] = st4(b.min);
    w.aabb_max[c] = st4(b.max);
}

// getBoundsTriangleMesh (src/BoundsUtil.cpp:77-85) for the triangle-mesh colliders in
// [c0, c1): every vertex at the collider's world pose, in chunks of kMeshBoundsChunk
// vertices a block.  The reference folds the vertices in order; (value, index) keys
// reduced across the blocks give the same pick, and a last pass reads the picked
// vertices back.  trimesh_keys holds [6][n_trimesh_cols] keys: min x, y, z, max x, y, z.
__device__ __forceinline__ V3 mesh_vertex_world(const World& w, int c, const TriMeshDev& tm, int i, V3 pos, Q4 ori) {
    return pos + qrot(ori, ld3(w.tri_verts[tm.vert_start + i]));
}
__device__ __forceinline__ void collider_world_pose(const World& w, int c, V3& pos, Q4& ori) {
    const int4 ci = w.col_info[c];
    const Q4 bq = ld4(w.quat[ci.x]);
    pos = ld3(w.pos[ci.x]) + qrot(bq, ld3(w.col_pos[c]));
    ori = qmul(bq, ld4(w.col_quat[c]));
}

__global__ void __launch_bounds__(256) k_trimesh_bounds_part(World w, int c0, int c1) {
    __shared__ unsigned long long sk[6];
    const int2 ch = w.trimesh_chunks[blockIdx.x];   // (trimesh collider slot, chunk)
    const int c = w.trimesh_cols[ch.x];
    if (c < c0 || c >= c1) return;
    V3 pos;
    Q4 ori;
    collider_world_pose(w, c, pos, ori);
    const TriMeshDev tm = w.trimesh[w.col_info[c].z];
    if (threadIdx.x < 6) sk[threadIdx.x] = threadIdx.x < 3 ? kKeyMinInit : kKeyMaxInit;
    __syncthreads();
    unsigned long long k[6] = {kKeyMinInit, kKeyMinInit, kKeyMinInit, kKeyMaxInit, kKeyMaxInit, kKeyMaxInit};
    const int i1 = min(tm.vert_count, (ch.y + 1) * kMeshBoundsChunk);
    for (int i = ch.y * kMeshBoundsChunk + threadIdx.x; i < i1; i += blockDim.x) {
        const V3 t = mesh_vertex_world(w, c, tm, i, pos, ori);
        k[0] = min(k[0], key_min(t.x, i)); k[1] = min(k[1], key_min(t.y, i)); k[2] = min(k[2], key_min(t.z, i));
        k[3] = max(k[3], key_max(t.x, i)); k[4] = max(k[4], key_max(t.y, i)); k[5] = max(k[5], key_max(t.z, i));
    }
    for (int o = 16; o; o >>= 1)
        for (int j = 0; j < 6; ++j) {
            const unsigned long long v = __shfl_xor_sync(0xffffffffu, k[j], o);
            k[j] = j < 3 ? min(k[j], v) : max(k[j], v);
        }
    if ((threadIdx.x & 31) == 0)
        for (int j = 0; j < 6; ++j) j < 3 ? atomicMin(&sk[j], k[j]) : atomicMax(&sk[j], k[j]);
    __syncthreads();
    if (threadIdx.x < 6) {
        const int j = threadIdx.x;
        unsigned long long* d = &w.trimesh_keys[(size_t)j * w.n_trimesh_cols + ch.x];
        j < 3 ? atomicMin(d, sk[j]) : atomicMax(d, sk[j]);
    }
}

__global__ void k_trimesh_bounds_final(World w, int c0, int c1, int margin) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < w.n_trimesh_cols; t += gridDim.x * blockDim.x) {
        const int c = w.trimesh_cols[t];
        if (c < c0 || c >= c1) continue;
        V3 pos;
        Q4 ori;
        collider_world_pose(w, c, pos, ori);
        const TriMeshDev tm = w.trimesh[w.col_info[c].z];
        float b[6];
        for (int j = 0; j < 6; ++j) {
            if (!tm.vert_count) { b[j] = j < 3 ? FLT_MAX : -FLT_MAX; continue; }
            const unsigned long long k = w.trimesh_keys[(size_t)j * w.n_trimesh_cols + t];
            const V3 v = mesh_vertex_world(w, c, tm, j < 3 ? key_min_index(k) : key_max_index(k), pos, ori);
            b[j] = (j % 3) == 0 ? v.x : ((j % 3) == 1 ? v.y : v.z);
        }
        Bounds bb{{b[0], b[1], b[2]}, {b[3], b[4], b[5]}};
        if (margin) { bb.max += v3s(0.01f); bb.min -= v3s(0.01f); }
        w.aabb_min[c] = st4(bb.min);
        w.aabb_max[c] = st4(bb.max);
    }
}

// Registry deltas, one coalesced record per body (the host folded the batch in order):
// pose, velocity, the kinematic flag and the broadphase's dynamic flag of the body's
// colliders; a posed body's colliders get updateBounds' bounds with the margin
// (src/Physecs.cpp:51-54, 78-90, 753-770).  Triangle-mesh colliders are left to
// k_trimesh_bounds_*.
__global__ void k_apply_deltas(World w, const DeltaRec* d, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const DeltaRec e = d[i];
        const int b = e.body;
        int4 inf = w.info[b];
        if (e.mask & DELTA_POSE) {
            w.pos[b] = make_float4(e.pos[0], e.pos[1], e.pos[2], 0.f);
            w.quat[b] = make_float4(e.quat[0], e.quat[1], e.quat[2], e.quat[3]);
        }
        if ((e.mask & DELTA_VELOCITY) && inf.z >= 0) {
            w.vel[inf.z] = make_float4(e.vel[0], e.vel[1], e.vel[2], 0.f);
            w.ang[inf.z] = make_float4(e.ang[0], e.ang[1], e.ang[2], 0.f);
        }
        if (e.mask & DELTA_KINEMATIC) {
            inf.y = e.kinematic ? (inf.y | BODY_KIN) : (inf.y & ~BODY_KIN);
            w.info[b] = inf;
        }
        const bool sim = (inf.y & BODY_DYN) && !(inf.y & BODY_KIN);
        const Q4 bq = ld4(w.quat[b]);
        const V3 bp = ld3(w.pos[b]);
        for (int c = w.body_col[b]; c < w.body_col[b + 1]; ++c) {
            int4 ci = w.col_info[c];
            if (e.mask & DELTA_KINEMATIC) {
                ci.w = sim ? (ci.w | COL_DYNAMIC) : (ci.w & ~COL_DYNAMIC);
                w.col_info[c] = ci;
            }
            if (!(e.mask & DELTA_POSE) || ci.y == G_TRIMESH) continue;
            const V3 pos = bp + qrot(bq, ld3(w.col_pos[c]));
            const Q4 ori = qmul(bq, ld4(w.col_quat[c]));
            const float4 pr = w.col_params[c];
            const GeomD g{ci.y, {pr.x, pr.y, pr.z}, ci.z};
            Bounds bb = getBounds(w, pos, ori, g);
            bb.max += v3s(0.01f);
            bb.min -= v3s(0.01f);
            w.aabb_min[c] = st4(bb.min);
            w.aabb_max[c] = st4(bb.max);
        }
    }
}

// The joints of bodies whose kinematic flag changed: the simulated ends and the anchors
// relative to their centre of mass, as the reference takes them each frame
// (src/Physecs.cpp:335-345)
__global__ void k_joint_fix(World w, const int* js, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        JointDev& J = w.joints[js[i]];
        const int4 i0 = w.info[J.body0], i1 = w.info[J.body1];
        const bool s0 = (i0.y & BODY_DYN) && !(i0.y & BODY_KIN), s1 = (i1.y & BODY_DYN) && !(i1.y & BODY_KIN);
        J.b0 = s0 ? i0.z : -1;
        J.b1 = s1 ? i1.z : -1;
        const V3 a0 = ld3(J.a0p), a1 = ld3(J.a1p);
        J.r0 = st4(s0 ? a0 - ld3(w.com[i0.z]) : a0);
        J.r1 = st4(s1 ? a1 - ld3(w.com[i1.z]) : a1);
    }
}

// Body state between the caller's layout (pos, vel, ang_vel: 3 floats a body; every body,
// static ones reading as zero velocity) and the world's float4 arrays (velocities per
// dynamic body).  A null array is skipped.
__global__ void k_unpack_bodies(World w, const float* pos, const float* vel, const float* ang) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < w.n_bodies; b += gridDim.x * blockDim.x) {
        if (pos) w.pos[b] = make_float4(pos[3 * b], pos[3 * b + 1], pos[3 * b + 2], 0.f);
        const int d = w.info[b].z;
        if (d < 0) continue;
        if (vel) w.vel[d] = make_float4(vel[3 * b], vel[3 * b + 1], vel[3 * b + 2], 0.f);
        if (ang) w.ang[d] = make_float4(ang[3 * b], ang[3 * b + 1], ang[3 * b + 2], 0.f);
    }
}

__global__ void k_pack_bodies(World w, float* pos, float* vel, float* ang) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < w.n_bodies; b += gridDim.x * blockDim.x) {
        if (pos) { const float4 p = w.pos[b]; pos[3 * b] = p.x; pos[3 * b + 1] = p.y; pos[3 * b + 2] = p.z; }
        const int d = w.info[b].z;
        const float4 v = d >= 0 ? w.vel[d] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 a = d >= 0 ? w.ang[d] : make_float4(0.f, 0.f, 0.f, 0.f);
        if (vel) { vel[3 * b] = v.x; vel[3 * b + 1] = v.y; vel[3 * b + 2] = v.z; }
        if (ang) { ang[3 * b] = a.x; ang[3 * b + 1] = a.y; ang[3 * b + 2] = a.z; }
    }
}

int launch_unpack_bodies(const World& w, const float* pos, const float* vel, const float* ang, cudaStream_t s) {
    if (!w.n_bodies || !(pos || vel || ang)) return 0;
    k_unpack_bodies<<<std::min(152 * 8, (w.n_bodies + 255) / 256), 256, 0, s>>>(w, pos, vel, ang);
    return 1;
}

int launch_pack_bodies(const World& w, float* pos, float* vel, float* ang, cudaStream_t s) {
    if (!w.n_bodies || !(pos || vel || ang)) return 0;
    k_pack_bodies<<<std::min(152 * 8, (w.n_bodies + 255) / 256), 256, 0, s>>>(w, pos, vel, ang);
    return 1;
}

int launch_apply_deltas(const World& w, const DeltaRec* d, int n, const int* joints, int nj, cudaStream_t s) {
    int k = 0;
    if (n > 0) { k_apply_deltas<<<(n + 127) / 128, 128, 0, s>>>(w, d, n); ++k; }
    if (nj > 0) { k_joint_fix<<<(nj + 127) / 128, 128, 0, s>>>(w, joints, nj); ++k; }
    return k;
}

int launch_aabb(const World& w, int margin_mode, cudaStream_t s) {
    return launch_aabb_range(w, 0, w.n_colliders, margin_mode, s);
}

int launch_aabb_range(const World& w, int c0, int c1, int margin_mode, cudaStream_t s) {
    if (c1 <= c0) return 0;
    k_aabb<<<(c1 - c0 + 255) / 256, 256, 0, s>>>(w, c0, c1, margin_mode);
    if (margin_mode == 1) return 1;
    return 1 + launch_trimesh_bounds(w, c0, c1, false, s);
}

int launch_trimesh_bounds(const World& w, int c0, int c1, bool margin, cudaStream_t s) {
    if (!w.n_trimesh_cols || c1 <= c0) return 0;
    const size_t n3 = 3 * (size_t)w.n_trimesh_cols;
    cudaMemsetAsync(w.trimesh_keys, 0xff, n3 * sizeof(unsigned long long), s);
    cudaMemsetAsync(w.trimesh_keys + n3, 0, n3 * sizeof(unsigned long long), s);
    k_trimesh_bounds_part<<<w.n_trimesh_chunks, 256, 0, s>>>(w, c0, c1);
    k_trimesh_bounds_final<<<(w.n_trimesh_cols + 127) / 128, 128, 0, s>>>(w, c0, c1, margin ? 1 : 0);
    return 2;
}

// ---------------------------------------------------------------- Morton keys

__global__ void k_scene_bounds(World w, FrameBuf f) {
    int s = blockIdx.x;
    int cs = w.scene_col[s], ce = w.scene_col[s + 1];
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    float size_sum = 0.f;   // longest side of the colliders' bounds, summed
    int count = 0;
    for (int c = cs + threadIdx.x; c < ce; c += blockDim.x) {
        if (!(w.col_info[c].w & COL_ENABLE)) continue;   // disabled colliders never pair
        float4 a = w.aabb_min[c], b = w.aabb_max[c];
        float m[3] = {(a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f};
        for (int k = 0; k < 3; ++k) { lo[k] = fminf(lo[k], m[k]); hi[k] = fmaxf(hi[k], m[k]); }
        const float size = fmaxf(fmaxf(b.x - a.x, b.y - a.y), b.z - a.z);
        if (size < FLT_MAX) { size_sum += size; ++count; }
    }
    __shared__ float sh[7][32];
    __shared__ int shn[32];
    for (int k = 0; k < 3; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        size_sum += __shfl_xor_sync(0xffffffffu, size_sum, o);
        count += __shfl_xor_sync(0xffffffffu, count, o);
    }
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        for (int k = 0; k < 3; ++k) { sh[k][wid] = lo[k]; sh[3 + k][wid] = hi[k]; }
        sh[6][wid] = size_sum;
        shn[wid] = count;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < (int)(blockDim.x >> 5); ++q) {
            for (int k = 0; k < 3; ++k) { sh[k][0] = fminf(sh[k][0], sh[k][q]); sh[3 + k][0] = fmaxf(sh[3 + k][0], sh[3 + k][q]); }
            sh[6][0] += sh[6][q];
            shn[0] += shn[q];
        }
        // .w of the upper corner: the colliders' mean longest side
        f.scene_lo[s] = make_float4(sh[0][0], sh[1][0], sh[2][0], 0.f);
        f.scene_hi[s] = make_float4(sh[3][0], sh[4][0], sh[5][0], shn[0] ? sh[6][0] / (float)shn[0] : 0.f);
    }
}

__device__ __forceinline__ uint32_t expand_bits(uint32_t v, int bits) {
    // spread the low `bits` bits of v three positions apart
    uint32_t r = 0;
    for (int i = 0; i < bits; ++i) r |= ((v >> i) & 1u) << (3 * i);
    return r;
}

// 30-bit Morton code of the collider's bounds centre within its scene's bounds.  Bit 30
// marks a collider as large (its bounds' longest side at least a quarter of the longest
// side of the scene's centre bounds, or sixteen times the scene's mean: ground boxes,
// terrain, a ceiling over bodies that have scattered), bit 31 a disabled one, so that within a scene the
// ordinary colliders sort first, then the large ones, then those that never pair.  Every
// leaf looks for partners after itself, so a large collider is found from the small
// ones' leaves instead of walking the whole tree itself.  The code depends only on the
// collider's own scene, never on how many scenes share the world, so a scene gets the
// same order alone or in any batch.
__global__ void k_morton(World w, FrameBuf f) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= w.n_colliders) return;
    int4 ci = w.col_info[c];
    uint32_t code = 1u << 31;
    if (ci.w & COL_ENABLE) {
        int s = w.info[ci.x].w;
        float4 lo = f.scene_lo[s], hi = f.scene_hi[s];
        float4 a = w.aabb_min[c], b = w.aabb_max[c];
        const float scale = 1024.f;
        float m[3] = {(a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f};
        float l[3] = {lo.x, lo.y, lo.z}, h[3] = {hi.x, hi.y, hi.z};
        code = 0;
        for (int k = 0; k < 3; ++k) {
            float ext = h[k] - l[k];
            float u = ext > 0.f ? (m[k] - l[k]) / ext : 0.f;
            u = fminf(fmaxf(u, 0.f), 1.f);
            uint32_t q = (uint32_t)fminf(u * scale, scale - 1.f);
            code |= expand_bits(q, 10) << (2 - k);
        }
        float spread = fmaxf(fmaxf(h[0] - l[0], h[1] - l[1]), h[2] - l[2]);
        float size = fmaxf(fmaxf(b.x - a.x, b.y - a.y), b.z - a.z);
        if ((spread > 0.f && size >= 0.25f * spread) || (hi.w > 0.f && size >= 16.f * hi.w)) code |= 1u << 30;
    }
    f.mkey[c] = code;
    f.keys[c] = code;
    f.order[c] = c;
}

// after the Morton sort: scene index of each sorted leaf, for the stable scene pass
__global__ void k_scene_keys(World w, FrameBuf f) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= w.n_colliders) return;
    f.keys[p] = (uint32_t)w.info[w.col_info[f.order[p]].x].w;
}

// after the scene pass: the Morton code of each sorted leaf again, for the tree build
__global__ void k_gather_keys(World w, FrameBuf f) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= w.n_colliders) return;
    f.keys[p] = f.mkey[f.order[p]];
}

// ---------------------------------------------------------------- Karras radix tree

__device__ __forceinline__ int kdelta(const uint32_t* keys, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    uint32_t a = keys[i], b = keys[j];
    if (a == b) return 32 + __clz((uint32_t)(i ^ j));
    return __clz(a ^ b);
}

__device__ __forceinline__ int scene_of_position(const World& w, int p) {
    int lo = 0, hi = w.n_scenes;  // largest s with scene_col[s] <= p
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (w.scene_col[mid] <= p) lo = mid; else hi = mid;
    }
    return lo;
}

// one thread per sorted leaf position p; position p builds internal node (p - cs) of its scene
__global__ void k_karras(World w, FrameBuf f) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= w.n_colliders) return;
    int s = scene_of_position(w, p);
    int cs = w.scene_col[s], ce = w.scene_col[s + 1];
    int n = ce - cs;
    int i = p - cs;
    if (n < 2 || i >= n - 1) return;
    const uint32_t* keys = f.keys + cs;
    int ibase = cs - s;
    int d = (kdelta(keys, n, i, i + 1) - kdelta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = kdelta(keys, n, i, i - d);
    int lmax = 2;
    while (kdelta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (kdelta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = kdelta(keys, n, i, j);
    int sp = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (kdelta(keys, n, i, i + (sp + t) * d) > dnode) sp += t;
    } while (t > 1);
    int gamma = i + sp * d + min(d, 0);
    int lo = min(i, j), hi = max(i, j);
    int node = ibase + i;
    int left = (lo == gamma) ? ~(cs + gamma) : ibase + gamma;
    int right = (hi == gamma + 1) ? ~(cs + gamma + 1) : ibase + gamma + 1;
    f.bvh.left[node] = left;
    f.bvh.right[node] = right;
    f.bvh.first[node] = cs + lo;
    f.bvh.last[node] = cs + hi;
    f.bvh.visits[node] = 0;
    if (left >= 0) f.bvh.parent[left] = node; else f.bvh.leaf_parent[~left] = node;
    if (right >= 0) f.bvh.parent[right] = node; else f.bvh.leaf_parent[~right] = node;
    if (i == 0) f.bvh.parent[node] = -1;
}

// a disabled collider never pairs: it contributes empty bounds to its tree nodes, so a
// subtree holding only disabled colliders is pruned at its root
// ALL: every collider with its bounds (scene queries reach colliders that do not
// simulate, as the reference's query tree holds every collider); otherwise a collider
// with enableSimulation off gets empty bounds and pairs with nothing
template <bool ALL>
__device__ __forceinline__ void leaf_bounds(const World& w, int c, float4& mn, float4& mx) {
    if (ALL || (w.col_info[c].w & COL_ENABLE)) {
        mn = w.aabb_min[c];
        mx = w.aabb_max[c];
    } else {
        mn = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.f);
        mx = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f);
    }
}

template <bool ALL>
__global__ void k_refit(World w, FrameBuf f) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= w.n_colliders) return;
    int s = scene_of_position(w, p);
    int n = w.scene_col[s + 1] - w.scene_col[s];
    if (n < 2) return;
    int node = f.bvh.leaf_parent[p];
    while (node >= 0) {
        __threadfence();
        if (atomicAdd(&f.bvh.visits[node], 1) == 0) return;
        __threadfence();
        int L = f.bvh.left[node], R = f.bvh.right[node];
        float4 lmin, lmax, rmin, rmax;
        if (L < 0) leaf_bounds<ALL>(w, f.order[~L], lmin, lmax);
        else { lmin = __ldcg(&f.bvh.bmin[L]); lmax = __ldcg(&f.bvh.bmax[L]); }
        if (R < 0) leaf_bounds<ALL>(w, f.order[~R], rmin, rmax);
        else { rmin = __ldcg(&f.bvh.bmin[R]); rmax = __ldcg(&f.bvh.bmax[R]); }
        f.bvh.bmin[node] = make_float4(fminf(lmin.x, rmin.x), fminf(lmin.y, rmin.y), fminf(lmin.z, rmin.z), 0.f);
        f.bvh.bmax[node] = make_float4(fmaxf(lmax.x, rmax.x), fmaxf(lmax.y, rmax.y), fmaxf(lmax.z, rmax.z), 0.f);
        node = f.bvh.parent[node];
    }
}

// ---------------------------------------------------------------- traversal

// Inclusive overlap on all three axes (physecs::intersects, src/BoundsUtil.cpp:87-92),
// written as a conjunction so that bounds holding a NaN overlap nothing: for finite
// bounds the result is the reference's; a body whose state has become NaN is left
// without pairs instead of pairing with every collider of its scene.
__device__ __forceinline__ bool overlap_incl(float4 amin, float4 amax, float4 bmin, float4 bmax) {
    return amax.x >= bmin.x && amin.x <= bmax.x && amax.y >= bmin.y && amin.y <= bmax.y && amax.z >= bmin.z &&
           amin.z <= bmax.z;
}

// SAP filters of src/Physecs.cpp:138-147
__device__ __forceinline__ bool pair_ok(const World& w, int ca, int cb) {
    int4 a = w.col_info[ca], b = w.col_info[cb];
    if (!(a.w & COL_ENABLE) || !(b.w & COL_ENABLE)) return false;
    if (a.x == b.x) return false;
    if (!((a.w & COL_DYNAMIC) || (b.w & COL_DYNAMIC))) return false;
    return true;
}

// A warp takes 32 consecutive sorted leaves (Morton neighbours, so their bounds are
// usually close) and walks their scene's tree together: a node is entered when it may
// hold a partner of any lane, every lane reads the same node (one broadcast load), and
// the walk stays warp-uniform; when the leaves lie far apart, each lane walks alone.  Each lane tests only its own leaf p against the leaves q > p
// the walk reaches.  The walk is left-first depth-first, so each lane's partners come
// out in increasing sorted position: an order that depends only on the scene (its
// Morton codes), never on the tree's shape, the warp's other lanes or the batch.  A
// warp whose leaves belong to two scenes walks them one after the other.
//
// The pairs of a leaf go to pairs[leaf_off[p] + k] for its k-th partner, and leaf_off is
// the scan of the counts, so the walk runs before the scan (counting) and after it
// (placing).  Modes: kCount counts; kEmit places every pair; kCollect counts and keeps a
// leaf's first trav_k pairs in a per-leaf scratch, which k_pairs_place copies into place
// after the scan, so that one walk does both; kTail walks again only the leaves with more
// than trav_k pairs, to place the rest.
enum TraverseMode { kCount = 0, kEmit = 1, kCollect = 2, kTail = 3 };

__device__ __forceinline__ int2* trav_scratch(const FrameBuf& f) { return reinterpret_cast<int2*>(f.cat_list); }

// the count-th partner cb of leaf p (collider ca): the pair in entity order, placed or kept
template <int MODE>
__device__ __forceinline__ void place_pair(const World& w, const FrameBuf& f, int ca, int cb, int p, int out, int count) {
    if (MODE == kCount || (MODE == kTail && count < f.trav_k) || (MODE == kCollect && count >= f.trav_k)) return;
    const uint32_t ea = (uint32_t)w.info[w.col_info[ca].x].x, eb = (uint32_t)w.info[w.col_info[cb].x].x;
    const int2 pr = ea < eb ? make_int2(ca, cb) : make_int2(cb, ca);
    if (MODE == kCollect) {
        trav_scratch(f)[(size_t)p * f.trav_k + count] = pr;
    } else {
        const int slot = out + count;
        if (slot < f.pair_cap) f.pairs[slot] = pr;
    }
}

template <int MODE>
__global__ void __launch_bounds__(256) k_traverse(World w, FrameBuf f) {
    constexpr bool EMIT = MODE == kEmit || MODE == kTail;
    if (MODE == kTail && *f.trav_tail == 0) return;
    if (MODE == kCollect && blockIdx.x == 0 && threadIdx.x == 0) *f.trav_tail = 0;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int ca = 0, s = -1, root = 0;
    float4 qmin = make_float4(0.f, 0.f, 0.f, 0.f), qmax = qmin;
    bool want = false;
    if (p < w.n_colliders) {
        ca = f.order[p];
        s = w.info[w.col_info[ca].x].w;
        int cs = w.scene_col[s], n = w.scene_col[s + 1] - cs;
        bool active = !w.scene_active || w.scene_active[s];
        want = n >= 2 && active && (w.col_info[ca].w & COL_ENABLE);
        if (MODE == kTail) want = want && f.leaf_cnt[p] > f.trav_k;
        root = cs - s;   // root of this scene's tree
        qmin = w.aabb_min[ca];
        qmax = w.aabb_max[ca];
    }
    int count = 0;
    const int out = (EMIT && p < w.n_colliders) ? f.leaf_off[p] : 0;
    unsigned pending = __ballot_sync(~0u, want);
    while (pending) {
        const int leader = __ffs(pending) - 1;
        const int gs = __shfl_sync(~0u, s, leader);
        const int groot = __shfl_sync(~0u, root, leader);
        const bool mine = want && s == gs;
        pending &= ~__ballot_sync(~0u, mine);
        // The joint walk pays for the union of the lanes' bounds.  Leaves that are Morton
        // neighbours but far apart (scattered bodies, where the curve jumps) make that union
        // much larger than any lane's own bounds; each lane then walks alone.  Either walk
        // reaches each lane's partners in increasing sorted position, so the output is the
        // same.
        float ulo[3] = {qmin.x, qmin.y, qmin.z}, uhi[3] = {qmax.x, qmax.y, qmax.z};
        float own = fmaxf(fmaxf(qmax.x - qmin.x, qmax.y - qmin.y), qmax.z - qmin.z);
        if (!mine) {
            ulo[0] = ulo[1] = ulo[2] = FLT_MAX;
            uhi[0] = uhi[1] = uhi[2] = -FLT_MAX;
            own = 0.f;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                ulo[k] = fminf(ulo[k], __shfl_xor_sync(~0u, ulo[k], o));
                uhi[k] = fmaxf(uhi[k], __shfl_xor_sync(~0u, uhi[k], o));
            }
            own = fmaxf(own, __shfl_xor_sync(~0u, own, o));
        }
        const float spread = fmaxf(fmaxf(uhi[0] - ulo[0], uhi[1] - ulo[1]), uhi[2] - ulo[2]);
        int stack[64];
        int sp = 0;
        if (!(spread <= 8.f * own)) {   // scattered leaves (or a NaN bound): one walk per lane
            if (mine) stack[sp++] = groot;
            while (sp) {
                const int c = stack[--sp];
                if (c < 0) {
                    const int q = ~c;
                    if (q <= p) continue;
                    const int cb = f.order[q];
                    if (!overlap_incl(qmin, qmax, w.aabb_min[cb], w.aabb_max[cb])) continue;
                    if (!pair_ok(w, ca, cb)) continue;
                    place_pair<MODE>(w, f, ca, cb, p, out, count);
                    ++count;
                } else {
                    // the node's fields in one round of loads (c is a node of the lane's tree)
                    const int last = f.bvh.last[c], L = f.bvh.left[c], R = f.bvh.right[c];
                    const float4 bmn = f.bvh.bmin[c], bmx = f.bvh.bmax[c];
                    if (last > p && overlap_incl(qmin, qmax, bmn, bmx)) {
                        if (sp + 2 <= 64) {
                            stack[sp++] = R;
                            stack[sp++] = L;
                        } else {
                            atomicOr(w.err, ERR_STACK_CAPACITY);
                        }
                    }
                }
            }
            continue;
        }
        // the joint walk: the stack is the same in every lane
        stack[sp++] = groot;
        while (sp) {
            const int c = stack[--sp];
            if (c < 0) {
                const int q = ~c;
                if (!mine || q <= p) continue;
                const int cb = f.order[q];
                if (!overlap_incl(qmin, qmax, w.aabb_min[cb], w.aabb_max[cb])) continue;
                if (!pair_ok(w, ca, cb)) continue;
                place_pair<MODE>(w, f, ca, cb, p, out, count);
                ++count;
            } else {
                // the node's fields in one round of loads, children before the vote
                const int last = f.bvh.last[c], L = f.bvh.left[c], R = f.bvh.right[c];
                const float4 bmn = f.bvh.bmin[c], bmx = f.bvh.bmax[c];
                const bool go = mine && last > p && overlap_incl(qmin, qmax, bmn, bmx);
                if (!__any_sync(~0u, go)) continue;
                if (sp + 2 <= 64) {
                    stack[sp++] = R;
                    stack[sp++] = L;
                } else if (lane == 0) {
                    atomicOr(w.err, ERR_STACK_CAPACITY);
                }
            }
        }
    }
    if (!EMIT && p < w.n_colliders) f.leaf_cnt[p] = count;
}

// After the scan: each leaf's kept pairs (its first trav_k) copied to their places, a
// warp per 32 leaves so that the copies of one leaf are consecutive lanes' stores.
__global__ void __launch_bounds__(256) k_pairs_place(World w, FrameBuf f) {
    const int K = f.trav_k;
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    const int2* scratch = trav_scratch(f);
    bool tail = false;
    for (int base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; base < w.n_colliders; base += warps * 32) {
        const int p = base + lane;
        const int cnt = p < w.n_colliders ? f.leaf_cnt[p] : 0;
        const int off = p < w.n_colliders ? f.leaf_off[p] : 0;
        tail |= cnt > K;
        unsigned busy = __ballot_sync(~0u, cnt > 0);
        while (busy) {
            const int l = __ffs(busy) - 1;
            busy &= busy - 1;
            const int lc = min(__shfl_sync(~0u, cnt, l), K), lo = __shfl_sync(~0u, off, l);
            for (int r = lane; r < lc; r += 32)
                if (lo + r < f.pair_cap) f.pairs[lo + r] = scratch[(size_t)(base + l) * K + r];
        }
    }
    if (tail) *f.trav_tail = 1;
}

__global__ void k_pairs_check(FrameBuf f, int* err) {
    if (*f.n_pairs > f.pair_cap) { atomicOr(err, ERR_PAIR_CAPACITY); *f.n_pairs = f.pair_cap; }
}

// One block per scene sorts the scene's (Morton code, collider) pairs in shared memory
// with a bitonic network over 64-bit keys (code << 32 | collider), which orders equal
// codes by collider exactly like the stable radix sort.  A scene that is not running
// gets a constant code instead: its tree is never walked, only built and refitted.
__global__ void __launch_bounds__(256) k_scene_sort(World w, FrameBuf f, int pmax) {
    extern __shared__ unsigned long long sk[];
    const int s = blockIdx.x;
    const int cs = w.scene_col[s], n = w.scene_col[s + 1] - cs;
    if (n <= 0) return;
    if (w.scene_active && !w.scene_active[s]) {
        for (int i = threadIdx.x; i < n; i += blockDim.x) { f.order[cs + i] = cs + i; f.keys[cs + i] = 0u; }
        return;
    }
    int P = 1;
    while (P < n) P <<= 1;
    if (P > pmax) return;   // the launch sizes pmax for the largest scene
    for (int i = threadIdx.x; i < P; i += blockDim.x)
        sk[i] = i < n ? ((unsigned long long)f.mkey[cs + i] << 32) | (unsigned)(cs + i) : ~0ull;
    __syncthreads();
    for (int size = 2; size <= P; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = threadIdx.x; t < P / 2; t += blockDim.x) {
                int i = 2 * t - (t & (stride - 1));   // first of the pair
                int j = i + stride;
                bool up = (i & size) == 0;
                unsigned long long a = sk[i], b = sk[j];
                if ((a > b) == up) { sk[i] = b; sk[j] = a; }
            }
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        unsigned long long v = sk[i];
        f.order[cs + i] = (int)(unsigned)v;
        f.keys[cs + i] = (uint32_t)(v >> 32);
    }
}

// Each scene's LBVH over the colliders' current bounds: scene bounds, Morton codes, the
// per-scene sort, Karras' construction and the bottom-up refit.
int launch_bvh_build(const World& w, FrameBuf& f, int scene_bits, int scene_sort_pmax, bool all_leaves, cudaStream_t s) {
    int n = w.n_colliders;
    if (n == 0) return 0;
    int nb = (n + 255) / 256;
    k_scene_bounds<<<w.n_scenes, 256, 0, s>>>(w, f);
    k_morton<<<nb, 256, 0, s>>>(w, f);
    int k = 2;
    if (scene_sort_pmax > 0) {
        k_scene_sort<<<w.n_scenes, 256, scene_sort_pmax * sizeof(unsigned long long), s>>>(w, f, scene_sort_pmax);
        ++k;
    } else {
        // (scene, Morton) order as two stable LSD sorts: Morton first, then scene
        k += radix_sort_pairs(f.keys, f.order, f.keys_tmp, f.order_tmp, n, 32, f.radix_hist, s);
        if (scene_bits > 0) {
            k_scene_keys<<<nb, 256, 0, s>>>(w, f);
            k += 1 + radix_sort_pairs(f.keys, f.order, f.keys_tmp, f.order_tmp, n, scene_bits, f.radix_hist, s);
        }
        k_gather_keys<<<nb, 256, 0, s>>>(w, f);
        ++k;
    }
    k_karras<<<nb, 256, 0, s>>>(w, f);
    if (all_leaves) k_refit<true><<<nb, 256, 0, s>>>(w, f);
    else k_refit<false><<<nb, 256, 0, s>>>(w, f);
    return k + 2;
}

int launch_broadphase(const World& w, FrameBuf& f, int scene_bits, int scene_sort_pmax, cudaStream_t s) {
    int n = w.n_colliders;
    if (n == 0) return 0;
    int nb = (n + 255) / 256;
    int k = launch_bvh_build(w, f, scene_bits, scene_sort_pmax, false, s) - 2;
    if (f.trav_k > 0) {   // one walk, the kept pairs placed after the scan, a second walk only for long lists
        k_traverse<kCollect><<<nb, 256, 0, s>>>(w, f);
        scan_exclusive(f.leaf_cnt, f.leaf_off, n, f.n_pairs, f.scan_scratch, s);
        k_pairs_place<<<std::min(nb, 152 * 8), 256, 0, s>>>(w, f);
        k_traverse<kTail><<<nb, 256, 0, s>>>(w, f);
        ++k;
    } else {
        k_traverse<kCount><<<nb, 256, 0, s>>>(w, f);
        scan_exclusive(f.leaf_cnt, f.leaf_off, n, f.n_pairs, f.scan_scratch, s);
        k_traverse<kEmit><<<nb, 256, 0, s>>>(w, f);
    }
    k_pairs_check<<<1, 1, 0, s>>>(f, w.err);
    return k + 4 + 3 + 1;
}

}  // namespace psx
