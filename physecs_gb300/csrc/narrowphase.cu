// narrowphase.cu — per-pair collision kernels.
//
// The pair list is split by kind so each kernel runs one code path: analytic
// pairs (sphere / capsule / box), convex-mesh pairs (GJK + EPA + face clipping)
// and triangle-mesh pairs (BVH midphase + per-triangle tests).  Every pair is one
// thread; every kernel writes its manifolds into per-pair slots, and a count /
// scan / compact pass produces the manifold list in pair order, so the output is
// deterministic.  Pair geometry follows src/Physecs.cpp:188-213: collider world
// pose = body pose composed with the collider's local pose.
#include <algorithm>
#include "frame.cuh"
#include "narrow_tri.cuh"
#include "narrow_warp.cuh"
#include "narrow_epa_flat.cuh"

namespace psx {

__device__ __forceinline__ void store_manifold(Manifold& out, const ManifoldL& m, int pair) {
    out.n = st4(m.normal);
    for (int k = 0; k < 4; ++k) {
        if (k < m.numPoints) { out.p0[k] = st4(m.points[k].p0); out.p1[k] = st4(m.points[k].p1); }
    }
    out.np = m.numPoints;
    out.tri = m.triangleIndex;
    out.pair = pair;
}

// Pair category and the trigger / jointed-pair filters (src/Physecs.cpp:200-209), appended
// to the category lists with one atomic per warp and category.  A list's order decides
// only which thread handles which pair: every pair writes its own manifold slots.  The
// default contact filter makes every pair with a trigger collider a trigger pair, tested
// for overlap only and ahead of the jointed-pair filter (list 7, when the world keeps
// trigger sets).
__global__ void k_classify(World w, FrameBuf f) {
    const int2* noncolliding = w.nc_pairs;
    const int n_nc = w.n_nc;
    const int np = *f.n_pairs;
    const int lane = threadIdx.x & 31;
    for (int base = blockIdx.x * blockDim.x; base < np; base += gridDim.x * blockDim.x) {
        const int p = base + threadIdx.x;
        int cat = 3;  // 3 = skipped
        if (p < np) {
            int2 pr = f.pairs[p];
            int4 a = w.col_info[pr.x], b = w.col_info[pr.y];
            // the contact filter (src/Physecs.cpp:200): the default one, or the user's as a
            // table over the colliders' (isTrigger, data) classes
            bool trigger = w.filter_table ? w.filter_table[w.col_class[pr.x] * w.n_classes + w.col_class[pr.y]] != 0
                                          : ((a.w & COL_TRIGGER) || (b.w & COL_TRIGGER));
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
            f.pair_cat[p] = cat;
            if (trigger && f.trig_cap) cat = 7;
            f.pair_nman[p] = 0;
            // analytic pairs go to three lists by their boxes (none, one, two), so that a
            // warp's pairs take the same path (box-box SAT and clipping cost the most)
            if (cat == 0) {
                const int boxes = (a.y == G_BOX) + (b.y == G_BOX);
                cat = boxes == 0 ? 0 : (boxes == 1 ? 4 : 5);
            }
        }
        for (int c : {0, 1, 2, 4, 5, 7}) {
            unsigned m = __ballot_sync(0xffffffffu, cat == c);
            if (!m) continue;
            int first = 0;
            if (lane == __ffs(m) - 1) first = atomicAdd(&f.cat_count[c], __popc(m));
            first = __shfl_sync(0xffffffffu, first, __ffs(m) - 1);
            if (cat == c) f.cat_list[c * (size_t)f.pair_cap + first + __popc(m & ((1u << lane) - 1u))] = p;
        }
    }
}

// analytic pairs: sphere / capsule / box, one kernel per list (BOXES boxes in the pair:
// list 5 for two, 4 for one, 0 for none), so that each kernel holds only its routines
template <int BOXES>
__global__ void __launch_bounds__(256) k_narrow_analytic(World w, FrameBuf f) {
    constexpr int lst = BOXES == 2 ? 5 : (BOXES == 1 ? 4 : 0);
    const int n = f.cat_count[lst];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int p = f.cat_list[lst * (size_t)f.pair_cap + t];
        int2 pr = f.pairs[p];
        V3 pos0, pos1;
        Q4 or0, or1;
        GeomD g0, g1;
        collider_pose(w, pr.x, pos0, or0, g0);
        collider_pose(w, pr.y, pos1, or1, g1);
        ManifoldL m;
        bool hit = collideAnalyticT<BOXES>(pos0, or0, g0, pos1, or1, g1, m, w.err);
        int cnt = (hit && m.numPoints) ? 1 : 0;
        if (cnt) store_manifold(f.man_pair[p], m, p);
        f.pair_nman[p] = cnt;
    }
}

// convex-mesh pairs, part 1: GJK, then EPA for the pairs GJK finds overlapping.  The
// EPA normal and closest points (or "no contact") are staged in the pair's manifold slot.

__device__ __forceinline__ bool convex_pair_ordered(const World& w, int2 pr, V3& pos0, Q4& or0, GeomD& g0, V3& pos1,
                                                    Q4& or1, GeomD& g1) {
    collider_pose(w, pr.x, pos0, or0, g0);
    collider_pose(w, pr.y, pos1, or1, g1);
    // physecs::collision calls the (other, convex mesh) routine and flips the result
    // when only the first collider is the convex mesh (Collision.cpp:910-1016)
    bool swap = g1.type != G_CONVEX;
    if (swap) {
        V3 tp = pos0; pos0 = pos1; pos1 = tp;
        Q4 tq = or0; or0 = or1; or1 = tq;
        GeomD tg = g0; g0 = g1; g1 = tg;
    }
    return swap;
}

// GJK with one thread per pair.  Its simplex arithmetic is f64, and the FP64 pipe costs
// the same for a warp instruction whatever the number of lanes that use it, so 32 pairs
// per warp instruction is where GJK is cheapest; the support searches are f32.  Most
// pairs end here without contact (their bounds overlap, their shapes do not).  For an
// overlapping pair the final simplex is kept in the pair's manifold slot (the f32
// support points; each Minkowski vertex is their difference widened to f64, so it is
// rebuilt exactly) and the pair joins the list that EPA works through.
__global__ void __launch_bounds__(128, 4) k_convex_gjk(World w, FrameBuf f) {
    const int n = f.cat_count[1];
    const int lane = threadIdx.x & 31;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int p = f.cat_list[f.pair_cap + t];
        V3 pos0, pos1;
        Q4 or0, or1;
        GeomD g0, g1;
        convex_pair_ordered(w, f.pairs[p], pos0, or0, g0, pos1, or1, g1);
        Support a, b;
        convexOrderedSupports(w, pos0, or0, g0, pos1, or1, g1, a, b);
        GjkSimplex s;
        const bool hit = gjk(a, b, pos1 - pos0, s);
        Manifold& m = f.man_pair[p];
        if (hit) {
            m.np = 1;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                m.p0[i] = make_float4(s.v[i].sp0.x, s.v[i].sp0.y, s.v[i].sp0.z, 0.f);
                m.p1[i] = make_float4(s.v[i].sp1.x, s.v[i].sp1.y, s.v[i].sp1.z, 0.f);
            }
        } else {
            m.np = -1;
            m.n = make_float4(0.f, 0.f, 0.f, 0.f);
            m.p0[0] = m.n;
            m.p1[0] = m.n;
        }
        const unsigned act = __activemask();
        const unsigned hm = __ballot_sync(act, hit);
        int first = 0;
        if (hm) {
            const int leader = __ffs(hm) - 1;
            if (lane == leader) first = atomicAdd(&f.cat_count[3], __popc(hm));
            first = __shfl_sync(act, first, leader);
            if (hit) f.cat_list[3 * (size_t)f.pair_cap + first + __popc(hm & ((1u << lane) - 1u))] = t;
        }
    }
}

// Polytopes handed between the EPA passes: the lane-per-pair pass's (LaneSave, the first
// f.lane_saves of them a frame) and the grouped pass's (GroupSave, the first
// f.group_saves), each by its position in the list of pairs handed over.  Pairs past
// those counts start again from the simplex.  About 3.5 % of the overlapping pairs go on
// from the lane pass and a few in 10^4 from the grouped one.
using GroupSave = PolySave<SmallPoly::kV, SmallPoly::kF>;
__device__ __forceinline__ LaneSave* lane_saves(const FrameBuf& f) { return reinterpret_cast<LaneSave*>(f.epa_save); }
__device__ __forceinline__ GroupSave* group_saves(const FrameBuf& f) {
    return reinterpret_cast<GroupSave*>(f.epa_save + sizeof(LaneSave) * (size_t)f.lane_saves);
}
void epa_save_caps(int pair_cap, int& lane, int& group) {
    lane = std::min(32768, std::max(256, pair_cap / 16));
    group = std::min(1024, std::max(64, pair_cap / 1024));
}
size_t epa_save_bytes(int lane, int group) { return sizeof(LaneSave) * (size_t)lane + sizeof(GroupSave) * (size_t)group; }

// EPA for one overlapping pair, from the simplex GJK kept in its manifold slot or from a
// handed-over polytope (resume); the pair's normal and closest points replace the
// simplex there.  1: done; 0 / -1: the polytope outgrew P (kSpill) before / part way
// through a step, nothing was written.
template <int G, class PT, bool kSpill, class RS>
__device__ __forceinline__ int epa_pair(const World& w, FrameBuf& f, int t, PT& P, const Group<G>& g, const RS* resume) {
    const int p = f.cat_list[f.pair_cap + t];
    V3 pos0, pos1;
    Q4 or0, or1;
    GeomD g0, g1;
    convex_pair_ordered(w, f.pairs[p], pos0, or0, g0, pos1, or1, g1);
    Support a, b;
    convexOrderedSupports(w, pos0, or0, g0, pos1, or1, g1, a, b);
    Manifold& m = f.man_pair[p];
    GjkSimplex s;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const V3 sa = ld3(m.p0[i]), sb = ld3(m.p1[i]);
        s.v[i] = {d3(sa - sb), sa, sb};
    }
    V3 nrm, c0, c1;
    const int r = group_epa<G, PT, kSpill>(a, b, s, nrm, c0, c1, P, g, w.err, resume);   // ends with a group barrier
    if (r <= 0) return r;
    if (g.gl == 0) {
        m.n = st4(nrm);
        m.p0[0] = st4(c0);
        m.p1[0] = st4(c1);
    }
    return 1;
}

// EPA for the overlapping pairs of list `src`: a group of G lanes per pair (32 / G pairs
// per warp), WARPS warps per block, a SmallPoly (about 5.5 KB of dynamic shared memory)
// per group.  Pairs that outgrow it go to the overflow list for k_convex_epa_full.
template <int G, int WARPS>
__global__ void __launch_bounds__(32 * WARPS) k_convex_epa(World w, FrameBuf f, int src) {
    extern __shared__ __align__(16) unsigned char epa_smem[];
    constexpr int GPW = 32 / G;   // groups per warp
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const Group<G> g(lane);
    SmallPoly& P = reinterpret_cast<SmallPoly*>(epa_smem)[wid * GPW + lane / G];
    const int n = f.cat_count[src];
    for (int h = (blockIdx.x * WARPS + wid) * GPW + lane / G; h < n; h += gridDim.x * WARPS * GPW) {
        const int t = f.cat_list[src * (size_t)f.pair_cap + h];
        const LaneSave* rs = nullptr;
        if (src == 8 && h < f.lane_saves && lane_saves(f)[h].nv > 0) rs = &lane_saves(f)[h];
        const int r = epa_pair<G, SmallPoly, true>(w, f, t, P, g, rs);
        if (r <= 0) {   // on to the full polytope, with this one when it is whole
            int h6 = 0;
            if (g.gl == 0) {
                h6 = atomicAdd(&f.cat_count[6], 1);
                f.cat_list[6 * (size_t)f.pair_cap + h6] = t;
            }
            h6 = __shfl_sync(g.gm, h6, g.gb);
            if (h6 < f.group_saves) {
                if (r == 0) group_save<G>(P, group_saves(f)[h6], g);
                else if (g.gl == 0) group_saves(f)[h6].nv = 0;
            }
            g.sync();
        }
    }
}

// EPA for the overlapping pairs (list 3) with one lane per pair and the faces built by the
// whole warp (narrow_epa_flat.cuh).  Each warp takes pairs from a shared counter as its
// lanes free up; a pair whose polytope would outgrow the lane's room goes to list 8 for
// the grouped kernel.  One block of WARPS warps per SM: the polytopes take about 54 KB of
// shared memory a warp.
template <int WARPS>
__global__ void __launch_bounds__(32 * WARPS, 1) k_convex_epa_flat(World w, FrameBuf f) {
    extern __shared__ __align__(16) unsigned char epa_smem[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    FlatPoly& P = reinterpret_cast<FlatPoly*>(epa_smem)[wid];
    const int n = f.cat_count[3];
    const unsigned below = (1u << lane) - 1u;
    int t = -1;              // the lane's pair (index into list 1), -1 when it has none
    bool drained = false;    // no pair left for this lane
    int p = 0, nv = 0, nf = 0, nnew = 0;
    Support s0, s1;
    for (;;) {
        // lanes without a pair take the next ones
        const bool need = t < 0 && !drained;
        const unsigned needm = __ballot_sync(~0u, need);
        if (needm) {
            const int leader = __ffs(needm) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(&f.cat_count[9], __popc(needm));
            base = __shfl_sync(~0u, base, leader);
            if (need) {
                const int h = base + __popc(needm & below);
                if (h < n) {
                    t = f.cat_list[3 * (size_t)f.pair_cap + h];
                    p = f.cat_list[f.pair_cap + t];
                    V3 pos0, pos1;
                    Q4 or0, or1;
                    GeomD g0, g1;
                    convex_pair_ordered(w, f.pairs[p], pos0, or0, g0, pos1, or1, g1);
                    convexOrderedSupports(w, pos0, or0, g0, pos1, or1, g1, s0, s1);
                    const Manifold& m = f.man_pair[p];
                    GjkSimplex sx;
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const V3 sa = ld3(m.p0[i]), sb = ld3(m.p1[i]);
                        sx.v[i] = {d3(sa - sb), sa, sb};
                        fp_set_vertex(P, i, lane, sx.v[i]);
                    }
                    // EPA.h initial tetrahedron, wound so that every normal points outwards
                    const D3 n0 = cross(sx.v[0].pos - sx.v[1].pos, sx.v[2].pos - sx.v[1].pos);
                    const bool flip = dot(sx.v[3].pos - sx.v[0].pos, n0) < 0;
                    const unsigned char tri[4][3] = {{0, (unsigned char)(flip ? 1 : 2), (unsigned char)(flip ? 2 : 1)},
                                                     {3, (unsigned char)(flip ? 1 : 2), 0},
                                                     {3, (unsigned char)(flip ? 2 : 1), (unsigned char)(flip ? 1 : 2)},
                                                     {3, 0, (unsigned char)(flip ? 2 : 1)}};
#pragma unroll
                    for (int k = 0; k < 4; ++k) { P.t0[k][lane] = tri[k][0]; P.t1[k][lane] = tri[k][1]; P.t2[k][lane] = tri[k][2]; }
                    P.nbase[lane] = 0;
                    nv = 4;
                    nf = 0;
                    nnew = 4;
                } else {
                    drained = true;
                }
            }
        }
        if (!__ballot_sync(~0u, t >= 0)) break;
        // the step's new faces of every lane, built by all lanes
        int incl = t >= 0 ? nnew : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(~0u, incl, o);
            if (lane >= o) incl += y;
        }
        P.offs[lane + 1] = incl;
        if (lane == 0) P.offs[0] = 0;
        const int total = __shfl_sync(~0u, incl, 31);
        __syncwarp();
        for (int k = lane; k < total; k += 32) {
            int lo = 0, hi = 32;   // the slot s with offs[s] <= k < offs[s + 1]
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (P.offs[mid] <= k) lo = mid; else hi = mid;
            }
            const int m = k - P.offs[lo];
            fp_make_face(P, lo, P.nbase[lo] + m, P.t0[m][lo], P.t1[m][lo], P.t2[m][lo]);
        }
        __syncwarp();
        if (t >= 0) {
            nf = P.nbase[lane] + nnew;
            nnew = 0;
            // the closest face, by the reference's scan: the running minimum is a float
            // (compared as the double it widens to, kept beside it)
            float minDist = (float)DBL_MAX;
            double minWide = (double)minDist;
            int fi = 0;
            for (int k = 0; k < nf; ++k) {
                const double d = P.fd[k][lane];
                if (d < minWide) { minDist = (float)d; minWide = f64_of(minDist); fi = k; }
            }
            const D3 normal = fp_n(P, fi, lane);
            const GjkVertex v = mink(s0, s1, f3(normal));
            if (dot(v.pos, normal) - minWide < (double)0.00001f) {
                V3 cp0, cp1;
                fp_closest_points(P, lane, fi, cp0, cp1);
                Manifold& m = f.man_pair[p];
                m.n = st4(f3(normal));
                m.p0[0] = st4(cp0);
                m.p1[0] = st4(cp1);
                t = -1;
            } else {
                const int r = fp_insert(P, lane, nv, nf, nnew, v);
                if (r <= 0) {   // on to a longer pass, with this polytope when it is whole
                    const int h8 = atomicAdd(&f.cat_count[8], 1);
                    f.cat_list[8 * (size_t)f.pair_cap + h8] = t;
                    if (h8 < f.lane_saves) {
                        LaneSave& out = lane_saves(f)[h8];
                        if (r == 0) fp_save(P, lane, nv, nf, out);
                        else out.nv = 0;
                    }
                    t = -1;
                }
            }
        }
        __syncwarp();
    }
}

// EPA with the reference's full capacity, one warp and one WarpPoly (about 15 KB) per
// block, over list `lst`: the pairs whose polytope outgrew SmallPoly (6), or every
// overlapping pair (3) when the small pass is off.
__global__ void __launch_bounds__(32) k_convex_epa_full(World w, FrameBuf f, int lst) {
    extern __shared__ __align__(16) unsigned char epa_smem[];
    const Group<32> g(threadIdx.x);
    WarpPoly& P = *reinterpret_cast<WarpPoly*>(epa_smem);
    const int n = f.cat_count[lst];
    for (int h = blockIdx.x; h < n; h += gridDim.x) {
        const int t = f.cat_list[lst * (size_t)f.pair_cap + h];
        if (lst == 6 && h < f.group_saves && group_saves(f)[h].nv > 0)
            epa_pair<32, WarpPoly, false>(w, f, t, P, g, &group_saves(f)[h]);
        else if (lst == 8 && h < f.lane_saves && lane_saves(f)[h].nv > 0)
            epa_pair<32, WarpPoly, false>(w, f, t, P, g, &lane_saves(f)[h]);
        else
            epa_pair<32, WarpPoly, false>(w, f, t, P, g, (const GroupSave*)nullptr);
    }
}

// convex-mesh pairs, part 2: contact generation after EPA (face selection and
// clipping, Collision.cpp:352-887), one thread per pair.
__global__ void __launch_bounds__(256) k_convex_contacts(World w, FrameBuf f) {
    const int n = f.cat_count[1];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int p = f.cat_list[f.pair_cap + t];
        Manifold& m = f.man_pair[p];
        if (m.np < 0) { f.pair_nman[p] = 0; continue; }
        V3 pos0, pos1;
        Q4 or0, or1;
        GeomD g0, g1;
        bool swap = convex_pair_ordered(w, f.pairs[p], pos0, or0, g0, pos1, or1, g1);
        ManifoldL r;
        r.numPoints = 0;
        r.triangleIndex = -1;
        r.normal = ld3(m.n);
        r.points[0] = {ld3(m.p0[0]), ld3(m.p1[0])};
        convexOrderedContacts(w, pos0, or0, g0, pos1, or1, g1, r, w.err);
        if (swap) flipM(r);
        int cnt = r.numPoints ? 1 : 0;
        if (cnt) store_manifold(m, r, p);
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

// A kernel's shared memory attributes are per device: each function keeps, per device
// index, whether they were set there.
constexpr int kMaxDevices = 64;
static void set_smem_attrs(const void* fn, bool* done, int bytes) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxDevices || done[dev]) return;
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    done[dev] = true;
}

template <int G, int WARPS>
static void launch_convex_epa(const World& w, FrameBuf& f, int blocks_per_sm, int src, cudaStream_t s) {
    const int smem = (int)sizeof(SmallPoly) * WARPS * (32 / G);
    static bool done[kMaxDevices] = {};
    set_smem_attrs((const void*)k_convex_epa<G, WARPS>, done, smem);
    k_convex_epa<G, WARPS><<<152 * blocks_per_sm, 32 * WARPS, smem, s>>>(w, f, src);
}

constexpr int kFlatWarps = 4;
static void launch_convex_epa_flat(const World& w, FrameBuf& f, cudaStream_t s) {
    const int smem = (int)sizeof(FlatPoly) * kFlatWarps;
    static bool done[kMaxDevices] = {};
    set_smem_attrs((const void*)k_convex_epa_flat<kFlatWarps>, done, smem);
    k_convex_epa_flat<kFlatWarps><<<152, 32 * kFlatWarps, smem, s>>>(w, f);
}

// The convex kernels (bound by the FP64 pipe) run on the aux stream beside the analytic
// and triangle-mesh kernels (FP32, latency-bound); the categories write disjoint slots.
int launch_narrowphase(const World& w, FrameBuf& f, const StreamPair& sp, const NarrowShape& ns, cudaStream_t s) {
    cudaMemsetAsync(f.cat_count, 0, 10 * sizeof(int), s);
    k_classify<<<1216, 256, 0, s>>>(w, f);
    cudaEventRecord(sp.fork, s);
    cudaStreamWaitEvent(sp.aux, sp.fork, 0);
    k_convex_gjk<<<152 * ns.gjk_blocks_per_sm, 128, 0, sp.aux>>>(w, f);
    // epa_lanes 1: a lane per pair first; the pairs that outgrow it go to the grouped
    // kernel (16 lanes), or with epa_full_only straight to the full polytope.
    // (Generating the finished pairs' contacts on another stream beside the longer passes
    // was measured slower: it takes SMs from them.)
    const bool flat = ns.epa_lanes == 1;
    if (flat) launch_convex_epa_flat(w, f, sp.aux);
    if (!ns.epa_full_only) {
        const int src = flat ? 8 : 3;
        if (ns.epa_lanes == 8) launch_convex_epa<8, 1>(w, f, ns.convex_blocks_per_sm, src, sp.aux);
        else if (ns.epa_lanes == 16 || ns.epa_lanes == 1) launch_convex_epa<16, 1>(w, f, ns.convex_blocks_per_sm, src, sp.aux);
        else if (ns.convex_warps == 1) launch_convex_epa<32, 1>(w, f, ns.convex_blocks_per_sm, src, sp.aux);
        else if (ns.convex_warps == 2) launch_convex_epa<32, 2>(w, f, ns.convex_blocks_per_sm, src, sp.aux);
        else launch_convex_epa<32, 3>(w, f, ns.convex_blocks_per_sm, src, sp.aux);
    }
    {
        static bool done[kMaxDevices] = {};
        set_smem_attrs((const void*)k_convex_epa_full, done, (int)sizeof(WarpPoly));
        // the full pass alone: as many blocks as shared memory lets reside
        const int lst = ns.epa_full_only ? (flat ? 8 : 3) : 6;
        k_convex_epa_full<<<ns.epa_full_only && !flat ? 152 * 16 : 152 * 4, 32, sizeof(WarpPoly), sp.aux>>>(w, f, lst);
    }
    k_convex_contacts<<<1216 * 128 / ns.contacts_threads, ns.contacts_threads, 0, sp.aux>>>(w, f);
    cudaEventRecord(sp.join, sp.aux);
    // box-box pairs first: the longest
    k_narrow_analytic<2><<<152 * ns.analytic_blocks_per_sm, ns.analytic_threads, 0, s>>>(w, f);
    k_narrow_analytic<1><<<152 * ns.analytic_blocks_per_sm, ns.analytic_threads, 0, s>>>(w, f);
    k_narrow_analytic<0><<<152 * ns.analytic_blocks_per_sm, ns.analytic_threads, 0, s>>>(w, f);
    k_narrow_tri<<<1216, 64, 0, s>>>(w, f);
    const int kt = launch_triggers(w, f, s);
    cudaStreamWaitEvent(s, sp.join, 0);
    scan_exclusive_dev(f.pair_nman, f.pair_moff, f.n_pairs, f.pair_cap, f.n_man, f.scan_scratch, s);
    return 2 + 8 + 3 + kt + (flat ? 1 : 0) - (ns.epa_full_only ? 1 : 0);
}

}  // namespace psx
