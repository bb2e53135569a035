// narrowphase.cu — per-pair collision kernels.
//
// The pair list is split by kind so each kernel runs one code path: analytic
// pairs (sphere / capsule / box), convex-mesh pairs (GJK + EPA + face clipping)
// and triangle-mesh pairs (BVH midphase + per-triangle tests).  Every pair is one
// thread; every kernel writes its manifolds into per-pair slots, and a count /
// scan / compact pass produces the manifold list in pair order, so the output is
// deterministic.  Pair geometry follows src/Physecs.cpp:188-213: collider world
// pose = body pose composed with the collider's local pose.
#include "frame.cuh"
#include "narrow_tri.cuh"

namespace psx {

__device__ __forceinline__ void collider_pose(const World& w, int c, V3& pos, Q4& ori, GeomD& g) {
    int4 ci = w.col_info[c];
    Q4 bq = ld4(w.quat[ci.x]);
    pos = ld3(w.pos[ci.x]) + qrot(bq, ld3(w.col_pos[c]));
    ori = qmul(bq, ld4(w.col_quat[c]));
    float4 pr = w.col_params[c];
    g = GeomD{ci.y, {pr.x, pr.y, pr.z}, ci.z};
}

__device__ __forceinline__ void store_manifold(Manifold& out, const ManifoldL& m, int pair) {
    out.n = st4(m.normal);
    for (int k = 0; k < 4; ++k) {
        if (k < m.numPoints) { out.p0[k] = st4(m.points[k].p0); out.p1[k] = st4(m.points[k].p1); }
    }
    out.np = m.numPoints;
    out.tri = m.triangleIndex;
    out.pair = pair;
}

// pair category and trigger / joint filters (src/Physecs.cpp:200-209)
__global__ void k_classify(World w, FrameBuf f) {
    const int2* noncolliding = w.nc_pairs;
    int n_nc = w.n_nc;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    int np = *f.n_pairs;
    if (p >= f.pair_cap) return;
    int cat = 3;  // 3 = skipped
    if (p < np) {
        int2 pr = f.pairs[p];
        int4 a = w.col_info[pr.x], b = w.col_info[pr.y];
        bool trigger = (a.w & COL_TRIGGER) || (b.w & COL_TRIGGER);
        bool jointed = false;
        if (n_nc) {
            // sorted (body_lo, body_hi) list of jointed body pairs
            int lo = min(a.x, b.x), hi = max(a.x, b.x);
            int L = 0, R = n_nc;
            while (L < R) {
                int m = (L + R) >> 1;
                int2 v = noncolliding[m];
                if (v.x < lo || (v.x == lo && v.y < hi)) L = m + 1; else R = m;
            }
            jointed = L < n_nc && noncolliding[L].x == lo && noncolliding[L].y == hi;
        }
        if (!trigger && !jointed) {
            if (a.y == G_TRIMESH || b.y == G_TRIMESH) cat = 2;
            else if (a.y == G_CONVEX || b.y == G_CONVEX) cat = 1;
            else cat = 0;
        }
    }
    f.pair_cat[p] = cat;
    f.pair_nman[p] = 0;
}

__global__ void k_cat_flags(FrameBuf f, int cat) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= f.pair_cap) return;
    f.cat_flag[p] = (p < *f.n_pairs && f.pair_cat[p] == cat) ? 1 : 0;
}

__global__ void k_cat_scatter(FrameBuf f, int cat) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= f.pair_cap || p >= *f.n_pairs) return;
    if (f.pair_cat[p] == cat) f.cat_list[cat * f.pair_cap + f.cat_pos[cat][p]] = p;
}

// analytic pairs: sphere / capsule / box
__global__ void __launch_bounds__(128) k_narrow_analytic(World w, FrameBuf f) {
    int n = f.cat_count[0];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int p = f.cat_list[t];
        int2 pr = f.pairs[p];
        V3 pos0, pos1;
        Q4 or0, or1;
        GeomD g0, g1;
        collider_pose(w, pr.x, pos0, or0, g0);
        collider_pose(w, pr.y, pos1, or1, g1);
        ManifoldL m;
        bool hit = collideAnalytic(pos0, or0, g0, pos1, or1, g1, m, w.err);
        int cnt = (hit && m.numPoints) ? 1 : 0;
        if (cnt) store_manifold(f.man_pair[p], m, p);
        f.pair_nman[p] = cnt;
    }
}

// convex-mesh pairs: GJK + EPA + clipping
__global__ void __launch_bounds__(64) k_narrow_convex(World w, FrameBuf f) {
    int n = f.cat_count[1];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int p = f.cat_list[f.pair_cap + t];
        int2 pr = f.pairs[p];
        V3 pos0, pos1;
        Q4 or0, or1;
        GeomD g0, g1;
        collider_pose(w, pr.x, pos0, or0, g0);
        collider_pose(w, pr.y, pos1, or1, g1);
        ManifoldL m;
        Polytope poly;
        bool hit = collideConvex(w, pos0, or0, g0, pos1, or1, g1, m, poly, w.err);
        int cnt = (hit && m.numPoints) ? 1 : 0;
        if (cnt) store_manifold(f.man_pair[p], m, p);
        f.pair_nman[p] = cnt;
    }
}

// triangle-mesh pairs (src/Collision.cpp:897-907): the mesh may be either collider
__global__ void __launch_bounds__(64) k_narrow_tri(World w, FrameBuf f) {
    int n = f.cat_count[2];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int p = f.cat_list[2 * f.pair_cap + t];
        if (t >= f.tri_cap) { atomicOr(w.err, ERR_TRI_CAPACITY); f.pair_nman[p] = 0; continue; }
        f.pair_tslot[p] = t;
        int2 pr = f.pairs[p];
        V3 pos0, pos1;
        Q4 or0, or1;
        GeomD g0, g1;
        collider_pose(w, pr.x, pos0, or0, g0);
        collider_pose(w, pr.y, pos1, or1, g1);
        ManifoldL ms[kTriManifolds];
        TCI cand[kTriCandidates];
        Polytope poly;
        ManOut out{ms, 0, kTriManifolds, w.err};
        bool flip = g0.type == G_TRIMESH;
        if (flip) collideTriMesh(w, pos1, or1, g1, pos0, or0, g0.mesh, out, cand, poly);
        else collideTriMesh(w, pos0, or0, g0, pos1, or1, g1.mesh, out, cand, poly);
        int cnt = 0;
        for (int k = 0; k < out.n; ++k) {
            ManifoldL& m = ms[k];
            if (flip) flipM(m);
            if (!m.numPoints) continue;
            store_manifold(f.man_tri[t * kTriManifolds + cnt], m, p);
            ++cnt;
        }
        f.pair_nman[p] = cnt;
    }
}

int launch_narrowphase(const World& w, FrameBuf& f, cudaStream_t s) {
    int nb = (f.pair_cap + 255) / 256;
    k_classify<<<nb, 256, 0, s>>>(w, f);
    for (int c = 0; c < 3; ++c) {
        k_cat_flags<<<nb, 256, 0, s>>>(f, c);
        scan_exclusive(f.cat_flag, f.cat_pos[c], f.pair_cap, f.cat_count + c, f.scan_scratch, s);
        k_cat_scatter<<<nb, 256, 0, s>>>(f, c);
    }
    k_narrow_analytic<<<1216, 128, 0, s>>>(w, f);
    k_narrow_convex<<<1216, 64, 0, s>>>(w, f);
    k_narrow_tri<<<1216, 64, 0, s>>>(w, f);
    scan_exclusive_dev(f.pair_nman, f.pair_moff, f.n_pairs, f.pair_cap, f.n_man, f.scan_scratch, s);
    return 1 + 3 * 5 + 3 + 3;
}

}  // namespace psx
