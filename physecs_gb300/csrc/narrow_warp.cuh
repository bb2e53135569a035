// narrow_warp.cuh — EPA with a group of G lanes per convex pair (G = 8, 16 or 32).
//
// The arithmetic is exactly that of epa() in narrow_convex.cuh (EPA.h of the
// reference, f32 supports and an f64 polytope); only the loops over vertices and
// faces are spread across the group's lanes:
//   * support of a convex mesh: each lane scans every G-th vertex, and a group
//     reduction picks the same vertex as the reference's 4-lane SIMD scan
//     (largest dot; among equal dots the lowest vertex index modulo 4, then the
//     lowest index);
//   * EPA closest face: each lane measures every G-th face (distances compared as
//     ordered integers); the reductions below reproduce the sequential scan in
//     which the running minimum is kept as a float (EPA.h:52-60), including which
//     face wins among faces whose distances round to the same float;
//   * EPA visibility of the faces from the new vertex: one ballot per G faces, each
//     test settled in f32 when clear of its error bound;
//   * new faces on the horizon: one lane per horizon edge.
// The horizon edge list is built in the reference's order (faces from last to first,
// edges removed by swapping in the last edge), which fixes the order of the faces and
// so every later tie-break: the group searches the list together and its first lane
// edits it.  A pass can also go on from a polytope that an earlier pass handed over
// (PolySave) instead of starting from the GJK simplex.
//
// Why groups: the FP64 pipe charges a warp instruction the same whatever the
// number of lanes it carries, and one pair keeps only a handful of lanes busy (11
// faces on average, fewer new faces, one lane for the horizon).  With 32 / G pairs
// per warp, each f64 instruction serves up to 32 / G pairs.
//
// Every support point of the polytope is a float (held as float in shared
// memory, exactly); the Minkowski vertices, face normals and face distances are
// held as doubles so that the face loops convert and recompute nothing.  The full
// polytope of one pair takes about 15 KB of shared memory, the small one about 5.5 KB.
#pragma once
#include <math_constants.h>
#include "narrow_convex.cuh"

namespace psx {

// One pair's polytope with room for VC vertices, FC faces and EC horizon edges.
template <int VC, int FC, int EC>
struct PolyT {
    static constexpr int kV = VC, kF = FC, kE = EC;
    double nx[FC], ny[FC], nz[FC];
    double fd[FC];                                  // face distance dot(v[i0], n), fixed at creation
    long long fk[FC];                               // fd as an ordered integer (order_key)
    float ff[FC];                                   // fd rounded to float
    double px[VC], py[VC], pz[VC];                  // Minkowski vertex
    float ax[VC], ay[VC], az[VC];                   // support point on shape 0
    float bx[VC], by[VC], bz[VC];                   // support point on shape 1
    unsigned char i0[FC], i1[FC], i2[FC];
    unsigned char e0[EC], e1[EC];
    unsigned int vis[(FC + 31) / 32];               // face visibility bitset
    int nf, nv, ne, full;
};
// the reference's capacity (4 + 100 iterations)
using WarpPoly = PolyT<kEpaVerts, kEpaFaces, kEpaEdges>;
// room for 36 iterations in about a third of the space: most pairs need about five,
// and a pair that outgrows it is solved again with WarpPoly
using SmallPoly = PolyT<40, 76, 40>;

// A polytope handed from one EPA pass to the next, taken at the start of a step (before
// the step's closest face is chosen), so that the next pass goes on from that step
// instead of starting again from the simplex.  nv == 0: nothing handed over.  Vertices
// are floats (they hold floats exactly).
template <int VC, int FC>
struct PolySave {
    static constexpr int kV = VC, kF = FC;
    int nv, nf;
    float v[VC][9];                                 // Minkowski point, support on shape 0, on shape 1
    double n[FC][4];                                // normal and distance
    unsigned char idx[FC][3];
};

template <class PT>
__device__ __forceinline__ D3 wp_pos(const PT& P, int i) { return {P.px[i], P.py[i], P.pz[i]}; }
template <class PT>
__device__ __forceinline__ D3 wp_n(const PT& P, int f) { return {P.nx[f], P.ny[f], P.nz[f]}; }
template <class PT>
__device__ __forceinline__ void wp_set_vertex(PT& P, int i, const GjkVertex& v) {
    P.px[i] = v.pos.x; P.py[i] = v.pos.y; P.pz[i] = v.pos.z;
    P.ax[i] = v.sp0.x; P.ay[i] = v.sp0.y; P.az[i] = v.sp0.z;
    P.bx[i] = v.sp1.x; P.by[i] = v.sp1.y; P.bz[i] = v.sp1.z;
}
// EPA.h face construction: normal = normalize(cross(v0 - v1, v2 - v1)), left as is when degenerate
template <class PT>
__device__ __forceinline__ void wp_set_face(PT& P, int slot, int i0, int i1, int i2) {
    D3 n = cross(wp_pos(P, i0) - wp_pos(P, i1), wp_pos(P, i2) - wp_pos(P, i1));
    double len = length(n);
    if (len) n = n / len;
    P.nx[slot] = n.x; P.ny[slot] = n.y; P.nz[slot] = n.z;
    const double fd = dot(wp_pos(P, i0), n);
    P.fd[slot] = fd;
    P.fk[slot] = order_key(fd);
    P.ff[slot] = (float)fd;
    P.i0[slot] = (unsigned char)i0; P.i1[slot] = (unsigned char)i1; P.i2[slot] = (unsigned char)i2;
}

// Lanes of one group: gl = lane within the group, gb = the group's first lane of
// the warp, gm = the group's lanes as a warp mask.
template <int G>
struct Group {
    int gl, gb;
    unsigned gm;
    __device__ explicit Group(int lane)
        : gl(lane & (G - 1)), gb(lane & ~(G - 1)), gm(G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)))) {}
    __device__ __forceinline__ void sync() const { __syncwarp(gm); }
    // the group's bits of a ballot, lane gb first
    __device__ __forceinline__ unsigned ballot(bool v) const {
        unsigned b = __ballot_sync(gm, v);
        return G == 32 ? b : (b >> gb) & ((1u << G) - 1u);
    }
};

// Support of a convex mesh with the group's lanes splitting its vertices.
template <int G>
__device__ inline V3 group_support_convex(const Support& s, V3 dir, const Group<G>& g) {
    V3 d = s.scale * multiplyTranspose(s.basis, dir);
    float best = -FLT_MAX;
    int key = 0x7fffffff;   // (index & 3) << 24 | index: smaller wins among equal dots
    for (int i = g.gl; i < s.nverts; i += G) {
        float4 v = __ldg(&s.verts[i]);
        float dp = (v.x * d.x + v.y * d.y) + v.z * d.z;
        // a vertex that never beats -FLT_MAX leaves its class at the class's first index
        int k;
        if (dp > -FLT_MAX) k = ((i & 3) << 24) | i;
        else { dp = -FLT_MAX; k = ((i & 3) << 24) | (i & 3); }
        if (dp > best || (dp == best && k < key)) { best = dp; key = k; }
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        float ob = __shfl_xor_sync(g.gm, best, o, G);
        int ok = __shfl_xor_sync(g.gm, key, o, G);
        if (ob > best || (ob == best && ok < key)) { best = ob; key = ok; }
    }
    int mi = key & 0xffffff;
    return s.pos + mv(s.basis, s.scale * ld3(s.verts[mi]));
}

// Not inlined: EPA calls it from two places, and one copy of the support code keeps
// the kernel within the instruction cache.
template <int G>
__device__ __noinline__ GjkVertex group_mink(const Support& s0, const Support& s1, V3 dir, const Group<G> g) {
    V3 a = s0.kind == 3 ? group_support_convex<G>(s0, dir, g) : support(s0, dir);
    V3 b = s1.kind == 3 ? group_support_convex<G>(s1, -dir, g) : support(s1, -dir);
    return {d3(a - b), a, b};
}

template <int G>
__device__ __forceinline__ long long group_min_key(long long v, const Group<G>& g) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        const long long u = __shfl_xor_sync(g.gm, v, o, G);
        v = u < v ? u : v;
    }
    return v;
}

// EPA.h:10-186 for one group of G lanes.  Every lane of the group gets the same normal
// and points.  Capacity: with kSpill, a polytope that would outgrow P stops the walk and
// the call returns false (nothing is produced; the caller solves the pair again with a
// larger polytope); without, the capacity error is raised and the walk goes on
// truncated, as it can only with the reference's own 100-iteration room exhausted.
template <int G, class PT, bool kSpill, class RS>
__device__ inline int group_epa(const Support& s0, const Support& s1, const GjkSimplex& s, V3& nrm, V3& cp0, V3& cp1,
                                PT& P, const Group<G>& g, int* err, const RS* resume) {
    const int gl = g.gl;
    int it0 = 0;
    if (resume) {
        // the polytope of an earlier pass, as it stood at the start of step nv - 4
        static_assert(RS::kV <= PT::kV && RS::kF <= PT::kF, "a handed-over polytope fits");
        const int nv = resume->nv, nf = resume->nf;
        for (int i = gl; i < nv; i += G) {
            const float* q = resume->v[i];
            P.px[i] = f64_of(q[0]); P.py[i] = f64_of(q[1]); P.pz[i] = f64_of(q[2]);
            P.ax[i] = q[3]; P.ay[i] = q[4]; P.az[i] = q[5];
            P.bx[i] = q[6]; P.by[i] = q[7]; P.bz[i] = q[8];
        }
        for (int k = gl; k < nf; k += G) {
            const double* q = resume->n[k];
            P.nx[k] = q[0]; P.ny[k] = q[1]; P.nz[k] = q[2];
            P.fd[k] = q[3]; P.fk[k] = order_key(q[3]); P.ff[k] = (float)q[3];
            P.i0[k] = resume->idx[k][0]; P.i1[k] = resume->idx[k][1]; P.i2[k] = resume->idx[k][2];
        }
        if (gl == 0) { P.nv = nv; P.nf = nf; }
        it0 = nv - 4;
        g.sync();
    }
    if (!resume) {   // EPA.h initial tetrahedron from the simplex
        if (gl == 0) {
            for (int i = 0; i < 4; ++i) wp_set_vertex(P, i, s.v[i]);
            P.nv = 4;
        }
        g.sync();
        D3 n0 = cross(s.v[0].pos - s.v[1].pos, s.v[2].pos - s.v[1].pos);
        bool flip = dot(s.v[3].pos - s.v[0].pos, n0) < 0;
        if (gl < 4) {
            // EPA.h initial tetrahedron, wound so that every normal points outwards
            int t0, t1, t2;
            switch (gl) {
                case 0: t0 = 0; t1 = flip ? 1 : 2; t2 = flip ? 2 : 1; break;
                case 1: t0 = 3; t1 = flip ? 1 : 2; t2 = 0; break;
                case 2: t0 = 3; t1 = flip ? 2 : 1; t2 = flip ? 1 : 2; break;
                default: t0 = 3; t1 = 0; t2 = flip ? 2 : 1; break;
            }
            wp_set_face(P, gl, t0, t1, t2);
        }
        if (gl == 0) P.nf = 4;
        g.sync();
    }

    float minDist = 0;
    D3 normal = {0, 0, 0};
    int fi = 0;
    for (int it = it0; it < 100; ++it) {
        const int nf = P.nf;
        const int nslots = (nf + G - 1) / G;   // face slots in use (group-uniform)
        // smallest distance of this lane's faces (compared as ordered integers: the
        // FP64 pipe is the scarce one)
        long long kmin = LLONG_MAX;
        for (int j = 0; j < nslots; ++j) {
            int k = gl + G * j;
            if (k < nf) {
                const long long kk = P.fk[k];
                if (kk < kmin) kmin = kk;
            }
        }
        // Sequential rule: a face is taken when its distance is below the running
        // minimum, which is stored as a float.  The running minimum therefore ends
        // at M = float(smallest distance); the first face whose distance rounds to
        // M takes it, and after that every face with distance < M takes over.
        minDist = (float)DBL_MAX;
        kmin = group_min_key<G>(kmin, g);
        const long long kinf = order_key(CUDART_INF);
        if (kmin < kinf) {
            const float M = (float)key_value(kmin);
            const long long kM = order_key(f64_of(M));
            int first = 0x7fffffff, last = -1;
            for (int j = 0; j < nslots; ++j) {
                int k = gl + G * j;
                if (k < nf && k < first && P.ff[k] == M && P.fk[k] < kinf) first = k;
            }
            first = __reduce_min_sync(g.gm, first);
            for (int j = 0; j < nslots; ++j) {
                int k = gl + G * j;
                if (k < nf && k > first && P.fk[k] < kM) last = k;
            }
            last = __reduce_max_sync(g.gm, last);
            fi = last >= 0 ? last : first;
            normal = wp_n(P, fi);
            minDist = P.ff[fi];
        }
        GjkVertex v = group_mink<G>(s0, s1, f3(normal), g);
        if (dot(v.pos, normal) - minDist < (double)0.00001f) break;

        // ---- insert v (EPA.h:62-99)
        // no room for v: hand the polytope over as it stands (the next pass redoes this
        // step's search and support, with the same results)
        if (kSpill && P.nv >= PT::kV) return 0;
        // visibility of every current face, as a bitset over the face index
        const V3 vf = v.sp0 - v.sp1;   // v.pos exactly: it is this f32 difference, widened
        unsigned mine = 0;
        for (int j = 0; j < nslots; ++j) {
            int k = gl + G * j;
            if (k < nf && sees_face(wp_n(P, k), v.pos, vf, wp_pos(P, P.i0[k]))) mine |= 1u << j;
        }
        for (int j = 0; j < nslots; ++j) {
            unsigned m = g.ballot((mine >> j) & 1u);
            if (gl == 0) {
                const int bit = G * j;
                if ((bit & 31) == 0) P.vis[bit >> 5] = m;
                else P.vis[bit >> 5] |= m << (bit & 31);
            }
        }
        g.sync();
        {
            // The horizon in the reference's order: faces from last to first; each edge of a
            // visible face cancels the latest matching reversed edge of the list (the list's
            // last edge moves into its place) or is appended.  The group searches the list
            // together and its first lane edits it, so every lane follows the same counts.
            // Only the visible faces are visited, highest index first, by walking the set
            // bits of the bitset: a removal moves the current last face into the removed
            // slot, and that face has a higher index, so it has been looked at already and
            // the bits below stay valid.
            int ne = 0, n = nf;
            bool full = false;
            for (int word = (nf - 1) >> 5; word >= 0; --word)
            for (unsigned bits = P.vis[word]; bits; ) {
                const int bit = 31 - __clz(bits);
                bits &= ~(1u << bit);
                const int k = (word << 5) + bit;
                const int a[3] = {P.i0[k], P.i1[k], P.i2[k]}, b[3] = {P.i1[k], P.i2[k], P.i0[k]};
                bool found[3];
                for (int j = 0; j < 3; ++j) {
                    int hit = -1;
                    for (int m = gl; m < ne; m += G)
                        if (P.e0[m] == b[j] && P.e1[m] == a[j]) hit = m;
                    hit = __reduce_max_sync(g.gm, hit);
                    found[j] = hit >= 0;
                    if (found[j]) {
                        if (gl == 0) { P.e0[hit] = P.e0[ne - 1]; P.e1[hit] = P.e1[ne - 1]; }
                        --ne;
                        g.sync();
                    }
                }
                for (int j = 0; j < 3; ++j) {
                    if (found[j]) continue;
                    if (ne < PT::kE) {
                        if (gl == 0) { P.e0[ne] = (unsigned char)a[j]; P.e1[ne] = (unsigned char)b[j]; }
                        ++ne;
                    } else if (kSpill) {
                        full = true;
                    } else if (gl == 0) {
                        raise_err(err, ERR_EPA_CAPACITY);
                    }
                }
                // remove face k: the last face moves into its slot
                const int l = n - 1;
                if (gl == 0) {
                    P.nx[k] = P.nx[l]; P.ny[k] = P.ny[l]; P.nz[k] = P.nz[l]; P.fd[k] = P.fd[l];
                    P.fk[k] = P.fk[l]; P.ff[k] = P.ff[l];
                    P.i0[k] = P.i0[l]; P.i1[k] = P.i1[l]; P.i2[k] = P.i2[l];
                }
                --n;
                g.sync();
            }
            if (gl == 0) {
                if (kSpill && (P.nv >= PT::kV || n + ne > PT::kF)) {
                    full = true;
                } else if (P.nv >= PT::kV) {
                    raise_err(err, ERR_EPA_CAPACITY);
                    ne = 0;
                } else {
                    wp_set_vertex(P, P.nv, v);
                    P.nv = P.nv + 1;
                }
                P.ne = ne;
                P.nf = n;
                P.full = full;
            }
        }
        g.sync();
        if (kSpill && P.full) return -1;
        const int ne = P.ne, nbase = P.nf, vi = P.nv - 1;
        for (int m = gl; m < ne; m += G) {
            int slot = nbase + m;
            if (slot < PT::kF) wp_set_face(P, slot, vi, P.e0[m], P.e1[m]);
            else raise_err(err, ERR_EPA_CAPACITY);
        }
        g.sync();
        if (gl == 0) P.nf = min(nbase + ne, PT::kF);
        g.sync();
    }
    // closest points on the closest face (EPA.h:101-143); the projection adds the
    // face distance to every normal component, as the reference does
    const int f0 = P.i0[fi], f1 = P.i1[fi], f2 = P.i2[fi];
    D3 fn = wp_n(P, fi);
    D3 pa = wp_pos(P, f0), pb = wp_pos(P, f1), pc = wp_pos(P, f2);
    D3 proj = fn + P.fd[fi];
    V3 v0 = f3(pb - pa), v1 = f3(pc - pa), v2 = f3(proj - pa);
    double d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1), d20 = dot(v2, v0), d21 = dot(v2, v1);
    double denom = d00 * d11 - d01 * d01;
    double u, vv, ww;
    if (denom) {
        vv = (d20 * d11 - d21 * d01) / denom;
        ww = (d00 * d21 - d01 * d20) / denom;
        u = 1.0f - vv - ww;
    } else {
        ww = 0;
        if (d00) { vv = d20 / d00; u = 1.0f - vv; }
        else { vv = 0; u = 1.0; }
    }
    D3 a0 = {(double)P.ax[f0], (double)P.ay[f0], (double)P.az[f0]};   // f32 support points widened here
    D3 a1 = {(double)P.ax[f1], (double)P.ay[f1], (double)P.az[f1]};
    D3 a2 = {(double)P.ax[f2], (double)P.ay[f2], (double)P.az[f2]};
    D3 b0 = {(double)P.bx[f0], (double)P.by[f0], (double)P.bz[f0]};
    D3 b1 = {(double)P.bx[f1], (double)P.by[f1], (double)P.bz[f1]};
    D3 b2 = {(double)P.bx[f2], (double)P.by[f2], (double)P.bz[f2]};
    cp0 = f3(u * a0 + vv * a1 + ww * a2);
    cp1 = f3(u * b0 + vv * b1 + ww * b2);
    g.sync();
    nrm = f3(normal);
    return 1;
}

// The group's polytope into a save record (all lanes of the group take part).
template <int G, class PT, class RS>
__device__ inline void group_save(const PT& P, RS& out, const Group<G>& g) {
    const int nv = P.nv, nf = P.nf;
    if (nv > RS::kV || nf > RS::kF) {   // cannot happen for the sizes in use; start over then
        if (g.gl == 0) out.nv = 0;
        return;
    }
    for (int i = g.gl; i < nv; i += G) {
        float* q = out.v[i];
        q[0] = (float)P.px[i]; q[1] = (float)P.py[i]; q[2] = (float)P.pz[i];
        q[3] = P.ax[i]; q[4] = P.ay[i]; q[5] = P.az[i];
        q[6] = P.bx[i]; q[7] = P.by[i]; q[8] = P.bz[i];
    }
    for (int k = g.gl; k < nf; k += G) {
        double* q = out.n[k];
        q[0] = P.nx[k]; q[1] = P.ny[k]; q[2] = P.nz[k]; q[3] = P.fd[k];
        out.idx[k][0] = P.i0[k]; out.idx[k][1] = P.i1[k]; out.idx[k][2] = P.i2[k];
    }
    if (g.gl == 0) { out.nv = nv; out.nf = nf; }
}

}  // namespace psx
