// narrow_epa_flat.cuh — EPA with one lane per convex pair and the warp's face
// construction spread over all of its lanes.
//
// The arithmetic is that of epa() in narrow_convex.cuh (EPA.h:10-186 of the reference:
// f32 supports, an f64 polytope), operation for operation; only the schedule differs.
//
// Why: the polytope's f64 work runs on the FP64 pipe, which charges a warp instruction
// the same whatever the number of lanes it carries.  Most of that work is face
// construction (a cross product, a square root, three divisions and a dot product per
// face), and one pair makes only a handful of faces per step.  Here each lane owns one
// pair and walks it with the reference's sequential steps (closest face, support,
// termination test, visibility, horizon, face removal), and the faces that the warp's
// pairs create in a step are pooled and built by all 32 lanes together, so the FP64
// pipe sees full warps.  A lane whose pair ends takes the next one at once; a new pair's
// four initial faces join the same pool.
//
// The polytope of a pair lives in shared memory with room for 16 vertices (12 steps;
// about 96.5% of the pairs need fewer).  A pair that would outgrow it is handed to the
// grouped EPA of narrow_warp.cuh with its polytope, which goes on from the same step;
// in the rare case that the room runs out part way through a step, the grouped pass
// starts again from the GJK simplex, still in the pair's manifold slot.
#pragma once
#include "narrow_warp.cuh"

namespace psx {

constexpr int kTV = 16;   // vertices: the GJK simplex and 12 insertions
constexpr int kTF = 28;   // faces: 2 kTV - 4, the most a closed polytope of kTV vertices has
constexpr int kTE = 24;   // horizon edges, and faces created in one step

// The polytopes of one warp's 32 pairs, slot-interleaved: element [k][slot].  A vertex
// is stored as floats: its Minkowski point is the difference of two f32 support points
// taken in f32 (GJK.h) and widened, so the float holds it exactly.
struct FlatPoly {
    double nx[kTF][32], ny[kTF][32], nz[kTF][32];
    double fd[kTF][32];                          // face distance dot(v[i0], n), fixed at creation
    float px[kTV][32], py[kTV][32], pz[kTV][32];   // Minkowski vertex
    float ax[kTV][32], ay[kTV][32], az[kTV][32];   // support point on shape 0
    float bx[kTV][32], by[kTV][32], bz[kTV][32];   // support point on shape 1
    unsigned char i0[kTF][32], i1[kTF][32], i2[kTF][32];
    unsigned char e0[kTE][32], e1[kTE][32];      // horizon edges being collected
    unsigned char t0[kTE][32], t1[kTE][32], t2[kTE][32];   // faces to create this step
    int nbase[32];                               // first face index the slot's new faces take
    int offs[33];                                // the pooled faces' slot boundaries
};

__device__ __forceinline__ D3 fp_pos(const FlatPoly& P, int i, int s) {
    return {f64_of(P.px[i][s]), f64_of(P.py[i][s]), f64_of(P.pz[i][s])};
}
__device__ __forceinline__ V3 fp_posf(const FlatPoly& P, int i, int s) { return {P.px[i][s], P.py[i][s], P.pz[i][s]}; }
__device__ __forceinline__ D3 fp_n(const FlatPoly& P, int k, int s) { return {P.nx[k][s], P.ny[k][s], P.nz[k][s]}; }
// the Minkowski point is stored as the f32 difference of the supports that made it
__device__ __forceinline__ void fp_set_vertex(FlatPoly& P, int i, int s, const GjkVertex& v) {
    const V3 d = v.sp0 - v.sp1;
    P.px[i][s] = d.x; P.py[i][s] = d.y; P.pz[i][s] = d.z;
    P.ax[i][s] = v.sp0.x; P.ay[i][s] = v.sp0.y; P.az[i][s] = v.sp0.z;
    P.bx[i][s] = v.sp1.x; P.by[i][s] = v.sp1.y; P.bz[i][s] = v.sp1.z;
}
// EPA.h face construction: normal = normalize(cross(v0 - v1, v2 - v1)), left as is when
// degenerate; the distance is dot(v0, normal)
__device__ __forceinline__ void fp_make_face(FlatPoly& P, int s, int k, int a, int b, int c) {
    const D3 pa = fp_pos(P, a, s), pb = fp_pos(P, b, s), pc = fp_pos(P, c, s);
    D3 n = cross(pa - pb, pc - pb);
    const double len = length(n);
    if (len) n = n / len;
    P.nx[k][s] = n.x; P.ny[k][s] = n.y; P.nz[k][s] = n.z;
    P.fd[k][s] = dot(pa, n);
    P.i0[k][s] = (unsigned char)a; P.i1[k][s] = (unsigned char)b; P.i2[k][s] = (unsigned char)c;
}

// the polytope handed to the grouped pass when a lane's pair outgrows its room
using LaneSave = PolySave<kTV, kTF>;

// One EPA step's polytope update for slot s (EPA.h:62-99): the faces that see v are
// removed (each replaced by the current last face), their boundary edges collected in the
// reference's order, v appended, and one new face per edge queued.  1: done; 0: no room
// for v, the polytope untouched (it can be handed over as it stands); -1: the polytope
// outgrew its room part way (the next pass starts again from the simplex).
__device__ __forceinline__ int fp_insert(FlatPoly& P, int s, int& nv, int& nf, int& nnew, const GjkVertex& v) {
    if (nv >= kTV) return 0;
    // visibility of every current face, as a bitset (faces are only ever swapped in from
    // the end, and a face swapped in has been looked at already)
    const V3 vf = v.sp0 - v.sp1;   // v.pos exactly
    unsigned vis = 0;
    for (int k = 0; k < nf; ++k) {
        const int i = P.i0[k][s];
        const D3 n = fp_n(P, k, s);
        int r = sees_face_f32(n, vf, fp_posf(P, i, s));
        if (r < 0) r = dot(n, v.pos - fp_pos(P, i, s)) > 0;
        if (r) vis |= 1u << k;
    }
    int ne = 0, n = nf;
    bool full = false;
    for (unsigned bits = vis; bits; ) {   // visible faces, highest index first
        const int k = 31 - __clz(bits);
        bits &= ~(1u << k);
        const int a[3] = {P.i0[k][s], P.i1[k][s], P.i2[k][s]};
        const int b[3] = {a[1], a[2], a[0]};
        bool found[3] = {false, false, false};
        for (int j = 0; j < 3; ++j) {
            for (int m = ne - 1; m >= 0; --m) {
                if (P.e0[m][s] == b[j] && P.e1[m][s] == a[j]) {
                    found[j] = true;
                    P.e0[m][s] = P.e0[ne - 1][s];
                    P.e1[m][s] = P.e1[ne - 1][s];
                    --ne;
                    break;
                }
            }
        }
        for (int j = 0; j < 3; ++j) {
            if (found[j]) continue;
            if (ne < kTE) { P.e0[ne][s] = (unsigned char)a[j]; P.e1[ne][s] = (unsigned char)b[j]; ++ne; }
            else full = true;
        }
        const int l = n - 1;   // face k is removed: the last face moves into its slot
        P.nx[k][s] = P.nx[l][s]; P.ny[k][s] = P.ny[l][s]; P.nz[k][s] = P.nz[l][s]; P.fd[k][s] = P.fd[l][s];
        P.i0[k][s] = P.i0[l][s]; P.i1[k][s] = P.i1[l][s]; P.i2[k][s] = P.i2[l][s];
        --n;
    }
    if (full || n + ne > kTF) return -1;
    fp_set_vertex(P, nv, s, v);
    const int vi = nv++;
    for (int m = 0; m < ne; ++m) {
        P.t0[m][s] = (unsigned char)vi; P.t1[m][s] = P.e0[m][s]; P.t2[m][s] = P.e1[m][s];
    }
    P.nbase[s] = n;
    nf = n;
    nnew = ne;
    return 1;
}

// Slot s's polytope (nv vertices, nf faces) into a save record.
__device__ __forceinline__ void fp_save(const FlatPoly& P, int s, int nv, int nf, LaneSave& out) {
    for (int i = 0; i < nv; ++i) {
        float* q = out.v[i];
        q[0] = P.px[i][s]; q[1] = P.py[i][s]; q[2] = P.pz[i][s];
        q[3] = P.ax[i][s]; q[4] = P.ay[i][s]; q[5] = P.az[i][s];
        q[6] = P.bx[i][s]; q[7] = P.by[i][s]; q[8] = P.bz[i][s];
    }
    for (int k = 0; k < nf; ++k) {
        double* q = out.n[k];
        q[0] = P.nx[k][s]; q[1] = P.ny[k][s]; q[2] = P.nz[k][s]; q[3] = P.fd[k][s];
        out.idx[k][0] = P.i0[k][s]; out.idx[k][1] = P.i1[k][s]; out.idx[k][2] = P.i2[k][s];
    }
    out.nv = nv;
    out.nf = nf;
}

// Closest points on the closest face (EPA.h:101-143); the projection adds the face
// distance to every normal component, as the reference does.
__device__ __forceinline__ void fp_closest_points(const FlatPoly& P, int s, int fi, V3& cp0, V3& cp1) {
    const int f0 = P.i0[fi][s], f1 = P.i1[fi][s], f2 = P.i2[fi][s];
    const D3 fn = fp_n(P, fi, s);
    const D3 pa = fp_pos(P, f0, s), pb = fp_pos(P, f1, s), pc = fp_pos(P, f2, s);
    const D3 proj = fn + P.fd[fi][s];
    const V3 v0 = f3(pb - pa), v1 = f3(pc - pa), v2 = f3(proj - pa);
    const double d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1), d20 = dot(v2, v0), d21 = dot(v2, v1);
    const double denom = d00 * d11 - d01 * d01;
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
    const D3 a0 = {f64_of(P.ax[f0][s]), f64_of(P.ay[f0][s]), f64_of(P.az[f0][s])};
    const D3 a1 = {f64_of(P.ax[f1][s]), f64_of(P.ay[f1][s]), f64_of(P.az[f1][s])};
    const D3 a2 = {f64_of(P.ax[f2][s]), f64_of(P.ay[f2][s]), f64_of(P.az[f2][s])};
    const D3 b0 = {f64_of(P.bx[f0][s]), f64_of(P.by[f0][s]), f64_of(P.bz[f0][s])};
    const D3 b1 = {f64_of(P.bx[f1][s]), f64_of(P.by[f1][s]), f64_of(P.bz[f1][s])};
    const D3 b2 = {f64_of(P.bx[f2][s]), f64_of(P.by[f2][s]), f64_of(P.bz[f2][s])};
    cp0 = f3(u * a0 + vv * a1 + ww * a2);
    cp1 = f3(u * b0 + vv * b1 + ww * b2);
}

}  // namespace psx
