// narrow_warp.cuh — GJK + EPA with one warp per convex pair.
//
// The arithmetic is exactly that of gjk()/epa() in narrow_convex.cuh (GJK.h /
// EPA.h of the reference, f32 supports and an f64 simplex and polytope); only
// the loops over vertices and faces are spread across the 32 lanes:
//   * support of a convex mesh: each lane scans every 32nd vertex, and a warp
//     reduction picks the same vertex as the reference's 4-lane SIMD scan
//     (largest dot; among equal dots the lowest vertex index modulo 4, then the
//     lowest index);
//   * EPA closest face: each lane measures every 32nd face; the reductions
//     below reproduce the sequential scan in which the running minimum is kept
//     as a float (EPA.h:52-60), including which face wins among faces whose
//     distances round to the same float;
//   * EPA visibility of the faces from the new vertex: one ballot per 32 faces;
//   * new faces on the horizon: one lane per horizon edge.
// The horizon edge list itself is built by lane 0 in the reference's order
// (faces from last to first, edges removed by swapping in the last edge), which
// fixes the order of the faces and so every later tie-break.
//
// Every support point of the polytope is a float (held as float in shared
// memory, exactly); the Minkowski vertices, face normals and face distances are
// held as doubles so that the face loops convert and recompute nothing.  The whole
// polytope of one pair takes about 12.5 KB of shared memory.
#pragma once
#include <math_constants.h>
#include "narrow_convex.cuh"

namespace psx {

constexpr int kFaceSlots = (kEpaFaces + 31) / 32;   // faces per lane

struct WarpPoly {
    double nx[kEpaFaces], ny[kEpaFaces], nz[kEpaFaces];
    double fd[kEpaFaces];                                   // face distance dot(v[i0], n), fixed at creation
    double px[kEpaVerts], py[kEpaVerts], pz[kEpaVerts];     // Minkowski vertex
    float ax[kEpaVerts], ay[kEpaVerts], az[kEpaVerts];      // support point on shape 0
    float bx[kEpaVerts], by[kEpaVerts], bz[kEpaVerts];      // support point on shape 1
    unsigned char i0[kEpaFaces], i1[kEpaFaces], i2[kEpaFaces];
    unsigned char e0[kEpaEdges], e1[kEpaEdges];
    unsigned int vis[kFaceSlots];
    int nf, nv, ne;
};

__device__ __forceinline__ D3 wp_pos(const WarpPoly& P, int i) { return {P.px[i], P.py[i], P.pz[i]}; }
__device__ __forceinline__ D3 wp_n(const WarpPoly& P, int f) { return {P.nx[f], P.ny[f], P.nz[f]}; }
__device__ __forceinline__ void wp_set_vertex(WarpPoly& P, int i, const GjkVertex& v) {
    P.px[i] = v.pos.x; P.py[i] = v.pos.y; P.pz[i] = v.pos.z;
    P.ax[i] = v.sp0.x; P.ay[i] = v.sp0.y; P.az[i] = v.sp0.z;
    P.bx[i] = v.sp1.x; P.by[i] = v.sp1.y; P.bz[i] = v.sp1.z;
}
// EPA.h face construction: normal = normalize(cross(v0 - v1, v2 - v1)), left as is when degenerate
__device__ __forceinline__ void wp_set_face(WarpPoly& P, int slot, int i0, int i1, int i2) {
    D3 n = cross(wp_pos(P, i0) - wp_pos(P, i1), wp_pos(P, i2) - wp_pos(P, i1));
    double len = length(n);
    if (len) n = n / len;
    P.nx[slot] = n.x; P.ny[slot] = n.y; P.nz[slot] = n.z;
    P.fd[slot] = dot(wp_pos(P, i0), n);
    P.i0[slot] = (unsigned char)i0; P.i1[slot] = (unsigned char)i1; P.i2[slot] = (unsigned char)i2;
}

// Support of a convex mesh with the lanes splitting its vertices.
__device__ inline V3 warp_support_convex(const Support& s, V3 dir, int lane) {
    V3 d = s.scale * multiplyTranspose(s.basis, dir);
    float best = -FLT_MAX;
    int key = 0x7fffffff;   // (index & 3) << 24 | index: smaller wins among equal dots
    for (int i = lane; i < s.nverts; i += 32) {
        float4 v = __ldg(&s.verts[i]);
        float dp = (v.x * d.x + v.y * d.y) + v.z * d.z;
        // a vertex that never beats -FLT_MAX leaves its class at the class's first index
        int k;
        if (dp > -FLT_MAX) k = ((i & 3) << 24) | i;
        else { dp = -FLT_MAX; k = ((i & 3) << 24) | (i & 3); }
        if (dp > best || (dp == best && k < key)) { best = dp; key = k; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        float ob = __shfl_xor_sync(0xffffffffu, best, o);
        int ok = __shfl_xor_sync(0xffffffffu, key, o);
        if (ob > best || (ob == best && ok < key)) { best = ob; key = ok; }
    }
    int mi = key & 0xffffff;
    return s.pos + mv(s.basis, s.scale * ld3(s.verts[mi]));
}

__device__ __forceinline__ V3 warp_support(const Support& s, V3 dir, int lane) {
    if (s.kind == 3) return warp_support_convex(s, dir, lane);
    return support(s, dir);
}

// Not inlined: GJK and EPA call it from a dozen places, and one copy of the
// support code keeps the kernel within the instruction cache.
__device__ __noinline__ GjkVertex warp_mink(const Support& s0, const Support& s1, V3 dir, int lane) {
    V3 a = warp_support(s0, dir, lane);
    V3 b = warp_support(s1, -dir, lane);
    return {d3(a - b), a, b};
}

// GJK.h containsOrigin with its three face tests on lanes 0-2 at once; the first face
// (in the reference's order) whose test holds gives the new direction, as in the
// sequential version.
__device__ inline bool warp_contains_origin(GjkSimplex& s, D3& dir, int& fi, int lane) {
    const int j = lane < 3 ? lane : 0;
    const int b = j == 0 ? 0 : (j == 1 ? 2 : 1), c = j == 0 ? 1 : (j == 1 ? 0 : 2), o = 2 - j;
    D3 n;
    bool hit = checkFace(s.v[3].pos, s.v[b].pos, s.v[c].pos, s.v[o].pos, n);
    unsigned m = __ballot_sync(0xffffffffu, hit && lane < 3);
    if (!m) { fi = 0; return true; }
    int w = __ffs(m) - 1;
    dir = {__shfl_sync(0xffffffffu, n.x, w), __shfl_sync(0xffffffffu, n.y, w), __shfl_sync(0xffffffffu, n.z, w)};
    fi = 2 - w;
    return false;
}

struct WarpMink {
    const Support& s0;
    const Support& s1;
    int lane;
    __device__ GjkVertex operator()(V3 dir) const { return warp_mink(s0, s1, dir, lane); }
    __device__ bool containsOrigin(GjkSimplex& s, D3& dir, int& fi) const { return warp_contains_origin(s, dir, fi, lane); }
};

__device__ __forceinline__ double warp_min_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// EPA.h:10-186 for one warp.  Every lane returns the same normal and points.
__device__ inline V3 warp_epa(const WarpMink& mk, const GjkSimplex& s, V3& cp0, V3& cp1, WarpPoly& P, int lane, int* err) {
    if (lane == 0) {
        for (int i = 0; i < 4; ++i) wp_set_vertex(P, i, s.v[i]);
        P.nv = 4;
    }
    __syncwarp();
    D3 n0 = cross(s.v[0].pos - s.v[1].pos, s.v[2].pos - s.v[1].pos);
    bool flip = dot(s.v[3].pos - s.v[0].pos, n0) < 0;
    if (lane < 4) {
        // EPA.h initial tetrahedron, wound so that every normal points outwards
        int t0, t1, t2;
        switch (lane) {
            case 0: t0 = 0; t1 = flip ? 1 : 2; t2 = flip ? 2 : 1; break;
            case 1: t0 = 3; t1 = flip ? 1 : 2; t2 = 0; break;
            case 2: t0 = 3; t1 = flip ? 2 : 1; t2 = flip ? 1 : 2; break;
            default: t0 = 3; t1 = 0; t2 = flip ? 2 : 1; break;
        }
        wp_set_face(P, lane, t0, t1, t2);
    }
    if (lane == 0) P.nf = 4;
    __syncwarp();

    float minDist = 0;
    D3 normal = {0, 0, 0};
    int fi = 0;
    for (int it = 0; it < 100; ++it) {
        const int nf = P.nf;
        const int nslots = (nf + 31) >> 5;   // face slots in use (warp-uniform)
        // distances of this lane's faces
        double dk[kFaceSlots];
        double dmin = CUDART_INF;
#pragma unroll
        for (int j = 0; j < kFaceSlots; ++j) {
            if (j >= nslots) break;
            int k = lane + 32 * j;
            dk[j] = CUDART_NAN;
            if (k < nf) {
                dk[j] = P.fd[k];
                if (dk[j] < dmin) dmin = dk[j];
            }
        }
        // Sequential rule: a face is taken when its distance is below the running
        // minimum, which is stored as a float.  The running minimum therefore ends
        // at M = float(smallest distance); the first face whose distance rounds to
        // M takes it, and after that every face with distance < M takes over.
        minDist = (float)DBL_MAX;
        double dstar = warp_min_d(dmin);
        if (dstar < CUDART_INF) {
            float M = (float)dstar;
            int first = 0x7fffffff, last = -1;
#pragma unroll
            for (int j = 0; j < kFaceSlots; ++j) {
                if (j >= nslots) break;
                int k = lane + 32 * j;
                if (k < nf && (float)dk[j] == M && dk[j] < CUDART_INF && k < first) first = k;
            }
            first = __reduce_min_sync(0xffffffffu, first);
#pragma unroll
            for (int j = 0; j < kFaceSlots; ++j) {
                if (j >= nslots) break;
                int k = lane + 32 * j;
                if (k < nf && k > first && dk[j] < (double)M) last = k;
            }
            last = __reduce_max_sync(0xffffffffu, last);
            fi = last >= 0 ? last : first;
            normal = wp_n(P, fi);
            minDist = (float)P.fd[fi];
        }
        GjkVertex v = mk(f3(normal));
        if (dot(v.pos, normal) - minDist < (double)0.00001f) break;

        // ---- insert v (EPA.h:62-99)
        // visibility of every current face
#pragma unroll
        for (int j = 0; j < kFaceSlots; ++j) {
            if (j >= nslots) break;
            int k = lane + 32 * j;
            bool vis = false;
            if (k < nf) vis = dot(wp_n(P, k), v.pos - wp_pos(P, P.i0[k])) > 0;
            unsigned m = __ballot_sync(0xffffffffu, vis);
            if (lane == 0) P.vis[j] = m;
        }
        __syncwarp();
        if (lane == 0) {
            int ne = 0, n = nf;
            for (int k = nf - 1; k >= 0; --k) {
                if (!((P.vis[k >> 5] >> (k & 31)) & 1u)) continue;
                int a[3] = {P.i0[k], P.i1[k], P.i2[k]}, b[3] = {P.i1[k], P.i2[k], P.i0[k]};
                bool found[3] = {false, false, false};
                for (int j = 0; j < 3; ++j) {
                    for (int m = ne - 1; m >= 0; --m) {
                        if (P.e0[m] == b[j] && P.e1[m] == a[j]) {
                            found[j] = true;
                            P.e0[m] = P.e0[ne - 1]; P.e1[m] = P.e1[ne - 1]; --ne;
                            break;
                        }
                    }
                }
                for (int j = 0; j < 3; ++j) {
                    if (found[j]) continue;
                    if (ne < kEpaEdges) { P.e0[ne] = (unsigned char)a[j]; P.e1[ne] = (unsigned char)b[j]; ++ne; }
                    else raise_err(err, ERR_EPA_CAPACITY);
                }
                // remove face k: the last face moves into its slot
                int l = n - 1;
                P.nx[k] = P.nx[l]; P.ny[k] = P.ny[l]; P.nz[k] = P.nz[l]; P.fd[k] = P.fd[l];
                P.i0[k] = P.i0[l]; P.i1[k] = P.i1[l]; P.i2[k] = P.i2[l];
                --n;
            }
            if (P.nv >= kEpaVerts) {
                raise_err(err, ERR_EPA_CAPACITY);
                ne = 0;
            } else {
                wp_set_vertex(P, P.nv, v);
                P.nv = P.nv + 1;
            }
            P.ne = ne;
            P.nf = n;
        }
        __syncwarp();
        const int ne = P.ne, nbase = P.nf, vi = P.nv - 1;
        for (int m = lane; m < ne; m += 32) {
            int slot = nbase + m;
            if (slot < kEpaFaces) wp_set_face(P, slot, vi, P.e0[m], P.e1[m]);
            else raise_err(err, ERR_EPA_CAPACITY);
        }
        __syncwarp();
        if (lane == 0) P.nf = min(nbase + ne, kEpaFaces);
        __syncwarp();
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
    __syncwarp();
    return f3(normal);
}

}  // namespace psx
