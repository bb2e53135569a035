// narrow_convex.cuh — device pair tests for spheres, capsules, boxes and convex meshes.
//
// Restates Physecs src/Collision.cpp:54-1016 (analytic pairs, box-box SAT with
// face clipping, GJK + EPA with face clipping, the 4x4 dispatcher with flipped
// manifolds) and src/GJK.h / src/EPA.h including their mixed precision (float
// supports, double simplex and polytope).
#pragma once
#include <climits>
#include "narrow_util.cuh"

namespace psx {

struct GeomD {
    int type;
    float p[3];  // sphere {r}; capsule {halfHeight, r}; box {he}; convex {scale}
    int mesh;
};

__device__ __forceinline__ V3 gv(const GeomD& g) { return {g.p[0], g.p[1], g.p[2]}; }

// world pose and geometry of collider c: transform.position + transform.orientation *
// collider.position, transform.orientation * collider.orientation (src/Physecs.cpp:195-198)
__device__ __forceinline__ void collider_pose(const World& w, int c, V3& pos, Q4& ori, GeomD& g) {
    int4 ci = w.col_info[c];
    Q4 bq = ld4(w.quat[ci.x]);
    pos = ld3(w.pos[ci.x]) + qrot(bq, ld3(w.col_pos[c]));
    ori = qmul(bq, ld4(w.col_quat[c]));
    float4 pr = w.col_params[c];
    g = GeomD{ci.y, {pr.x, pr.y, pr.z}, ci.z};
}

// ---------------------------------------------------------------- bounds (BoundsUtil.cpp:23-85)

__device__ inline Bounds getBounds(const World& w, V3 pos, Q4 ori, const GeomD& g) {
    switch (g.type) {
        case G_SPHERE: return {pos - v3s(g.p[0]), pos + v3s(g.p[0])};
        case G_CAPSULE: {
            V3 p0 = pos + qrot(ori, {0, g.p[0], 0});
            V3 p1 = pos + qrot(ori, {0, -g.p[0], 0});
            return {vmin(p0, p1) - g.p[1], vmax(p0, p1) + g.p[1]};
        }
        case G_BOX: {
            M3 u = mat3_cast(ori);
            M3 a = m3cols(vabs(u.c[0]), vabs(u.c[1]), vabs(u.c[2]));
            V3 e = mv(a, gv(g));
            return {pos - e, pos + e};
        }
        case G_CONVEX: {
            const ConvexMeshDev cm = w.convex[g.mesh];
            V3 mn = v3s(FLT_MAX), mx = v3s(-FLT_MAX);
            V3 sc = gv(g);
            for (int i = 0; i < cm.vert_count_padded; ++i) {
                V3 t = pos + qrot(ori, sc * ld3(w.convex_verts[cm.vert_start + i]));
                mn = vmin(mn, t); mx = vmax(mx, t);
            }
            return {mn, mx};
        }
        default: {
            const TriMeshDev tm = w.trimesh[g.mesh];
            V3 mn = v3s(FLT_MAX), mx = v3s(-FLT_MAX);
            for (int i = 0; i < tm.vert_count; ++i) {
                V3 t = pos + qrot(ori, ld3(w.tri_verts[tm.vert_start + i]));
                mn = vmin(mn, t); mx = vmax(mx, t);
            }
            return {mn, mx};
        }
    }
}

// ---------------------------------------------------------------- supports (GJK.h:13-128)

struct Support {
    int kind;  // 0 sphere, 1 capsule, 2 box, 3 convex, 4 triangle
    V3 pos;
    float radius, halfHeight;
    V3 axis;
    M3 basis;
    V3 he;
    const float4* verts;
    int nverts;  // padded count
    V3 scale;
    V3 a, b, c;
};

__device__ inline V3 support(const Support& s, V3 dir) {
    switch (s.kind) {
        case 0: return s.pos + dir * s.radius;
        case 1: return s.pos + s.axis * signG(dot(dir, s.axis)) * s.halfHeight + dir * s.radius;
        case 2: {
            V3 r = s.pos;
            for (int i = 0; i < 3; ++i) r += signG(dot(dir, s.basis.c[i])) * s.basis.c[i] * at(s.he, i);
            return r;
        }
        case 3: {
            V3 d = s.scale * multiplyTranspose(s.basis, dir);
            float best[4];
            int bi[4];
            for (int l = 0; l < 4; ++l) { best[l] = -FLT_MAX; bi[l] = l; }
            for (int i = 0; i < s.nverts; i += 4) {
#pragma unroll
                for (int l = 0; l < 4; ++l) {
                    float4 v = __ldg(&s.verts[i + l]);
                    float dp = (v.x * d.x + v.y * d.y) + v.z * d.z;
                    if (dp > best[l]) bi[l] = i + l;
                    best[l] = (dp > best[l]) ? dp : best[l];
                }
            }
            int mi = bi[0];
            float mval = best[0];
            for (int l = 1; l < 4; ++l) if (best[l] > mval) { mval = best[l]; mi = bi[l]; }
            return s.pos + mv(s.basis, s.scale * ld3(s.verts[mi]));
        }
        default:
            if (dot(dir, s.a) > dot(dir, s.b)) return (dot(dir, s.a) > dot(dir, s.c)) ? s.a : s.c;
            return (dot(dir, s.b) > dot(dir, s.c)) ? s.b : s.c;
    }
}

// The simplex / polytope vertex (GJK.h): the f64 Minkowski point and the two f32 support
// points it came from (the reference widens them to f64 when it stores them; they are
// widened here where they are used, with identical values).
struct GjkVertex { D3 pos; V3 sp0, sp1; };
struct GjkSimplex { GjkVertex v[4]; };

__device__ inline GjkVertex mink(const Support& s0, const Support& s1, V3 dir) {
    V3 a = support(s0, dir);
    V3 b = support(s1, -dir);
    return {d3(a - b), a, b};
}
__device__ inline float sqrDistPointToLine(V3 p, V3 a, V3 b) {
    V3 r = p - a, d = b - a;
    V3 q = a + dot(r, d) / dot(d, d) * d;
    V3 pq = p - q;
    return dot(pq, pq);
}
__device__ inline float distPointToPlane(V3 p, V3 o, V3 n) { return fabsf(dot(p - o, n)); }
__device__ inline bool isZeroF(V3 v) { return (double)length2(v) < 1e-6; }
// The GJK routines are generic over the Minkowski-difference support `mk(dir)`, so
// that the thread-per-pair path (mink of two Supports) and the warp-per-pair path
// (lane-parallel support search) share one statement of the algorithm.
template <class MK>
__device__ inline bool checkDirection(MK& mk, D3 dir, GjkVertex& v) {
    dir = normalize(dir);
    v = mk(f3(dir));
    return dot(v.pos, dir) >= 0;
}
__device__ inline bool checkFace(D3 v0, D3 v1, D3 v2, D3 opp, D3& n) {
    n = cross(v1 - v0, v2 - v0);
    n = signD(dot(v0 - opp, n)) * n;
    return dot(n, -v0) > (double)0.00001f;
}
__device__ inline bool containsOrigin(GjkSimplex& s, D3& dir, int& fi) {
    fi = 2;
    if (checkFace(s.v[3].pos, s.v[0].pos, s.v[1].pos, s.v[fi].pos, dir)) return false;
    if (checkFace(s.v[3].pos, s.v[2].pos, s.v[0].pos, s.v[--fi].pos, dir)) return false;
    if (checkFace(s.v[3].pos, s.v[1].pos, s.v[2].pos, s.v[--fi].pos, dir)) return false;
    return true;
}
template <class MK>
__device__ inline void completeFromLine(MK& mk, GjkSimplex& s) {
    D3 dir = cross(s.v[0].pos - s.v[1].pos, D3{0, 1, 0});
    if (isZeroF(f3(dir))) dir = cross(s.v[0].pos - s.v[1].pos, D3{0, 0, 1});
    s.v[2] = mk(f3(normalize(dir)));
    if (sqrDistPointToLine(f3(s.v[2].pos), f3(s.v[0].pos), f3(s.v[1].pos)) < 0.00001f) s.v[2] = mk(f3(-dir));
    dir = normalize(cross(s.v[1].pos - s.v[0].pos, s.v[2].pos - s.v[0].pos));
    s.v[3] = mk(f3(dir));
    if (distPointToPlane(f3(s.v[3].pos), f3(s.v[0].pos), f3(dir)) < 0.0001f) s.v[3] = mk(f3(-dir));
}

// GJK.h:226-292
template <class MK>
__device__ inline bool gjkT(MK& mk, V3 startDir, GjkSimplex& s) {
    D3 dir = d3(normalize(startDir));
    s.v[0] = mk(f3(dir));
    if (isZeroF(f3(s.v[0].pos))) {
        dir = -dir;
        s.v[1] = mk(f3(dir));
        completeFromLine(mk, s);
        return true;
    }
    dir = -s.v[0].pos;
    if (!checkDirection(mk, dir, s.v[1])) return false;
    dir = cross(cross(s.v[0].pos - s.v[1].pos, -s.v[1].pos), s.v[0].pos - s.v[1].pos);
    if (isZeroF(f3(dir))) { completeFromLine(mk, s); return true; }
    if (!checkDirection(mk, dir, s.v[2])) return false;
    dir = cross(s.v[1].pos - s.v[0].pos, s.v[2].pos - s.v[0].pos);
    double sg = signD(dot(-s.v[0].pos, dir));
    if (!sg) {
        dir = normalize(dir);
        s.v[3] = mk(f3(dir));
        if (distPointToPlane(f3(s.v[3].pos), f3(s.v[0].pos), f3(dir)) < 0.0001f) s.v[3] = mk(f3(-dir));
        return true;
    }
    dir = sg * dir;
    if (!checkDirection(mk, dir, s.v[3])) return false;
    int fi;
    for (int i = 0; i < 100; ++i) {
        if (mk.containsOrigin(s, dir, fi)) return true;
        if (!checkDirection(mk, dir, s.v[fi])) return false;
        GjkVertex t = s.v[fi];
        s.v[fi] = s.v[3];
        s.v[3] = t;
    }
    return false;
}

struct PairMink {
    const Support& s0;
    const Support& s1;
    __device__ GjkVertex operator()(V3 dir) const { return mink(s0, s1, dir); }
    __device__ bool containsOrigin(GjkSimplex& s, D3& dir, int& fi) const { return psx::containsOrigin(s, dir, fi); }
};

__device__ inline bool gjk(const Support& s0, const Support& s1, V3 startDir, GjkSimplex& s) {
    PairMink mk{s0, s1};
    return gjkT(mk, startDir, s);
}

// ---- f32 shortcuts for f64 decisions
//
// The FP64 pipe is the narrowphase's bottleneck, and conversions between double and float
// run on it too.  These helpers move float data through integer operations and settle a
// sign test in f32 when the f32 value is clear of its error bound, falling back to the
// reference's f64 expression otherwise, so every decision is the reference's.

// float from a double by truncating the mantissa (exact when the double holds a float);
// ok is cleared when the value lies outside the normal float range (zero is exact)
__device__ __forceinline__ float f32_trunc(double x, bool& ok) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const unsigned sign = hi & 0x80000000u;
    if (((hi & 0x7fffffffu) | lo) == 0u) return __uint_as_float(sign);
    const int e = (int)((hi >> 20) & 0x7ffu) - 896;
    ok &= e >= 1 && e <= 254;
    return __uint_as_float(sign | ((unsigned)(e & 0xff) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29));
}
// the double holding float x (exact), from its bits
__device__ __forceinline__ double f64_of(float x) {
    const unsigned b = __float_as_uint(x);
    const unsigned e = (b >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) return (double)x;   // zero, subnormal, infinity, NaN
    const unsigned hi = (b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7fffffu) >> 3);
    return __hiloint2double((int)hi, (int)(b << 29));
}
// A double as an integer with the same order (for doubles that compare equal, the same
// integer: both zeros map to 0); a NaN maps above everything, so it is never below
// another distance, as in the f64 comparison.
__device__ __forceinline__ long long order_key(double x) {
    const long long b = __double_as_longlong(x);
    const long long mag = b & 0x7fffffffffffffffLL;
    if (mag == 0) return 0;
    if (mag > 0x7ff0000000000000LL) return LLONG_MAX;
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}
// the double of a key of a number (zero comes back as +0)
__device__ __forceinline__ double key_value(long long k) {
    return __longlong_as_double(k >= 0 ? k : (k ^ 0x7fffffffffffffffLL));
}
// dot(n, v - p) > 0 in f32 for v and p that are floats: 1 or 0 when the f32 value is
// further from zero than a bound on its distance from the f64 value (n truncated: 2^-23;
// v - p, the products and the two sums rounded: 2^-24 each; the f64 evaluation's own
// error is far below), -1 when undecided
__device__ __forceinline__ int sees_face_f32(D3 n, V3 vf, V3 pf) {
    bool ok = true;
    const float nx = f32_trunc(n.x, ok), ny = f32_trunc(n.y, ok), nz = f32_trunc(n.z, ok);
    if (!ok) return -1;
    const float dx = vf.x - pf.x, dy = vf.y - pf.y, dz = vf.z - pf.z;
    const float px = nx * dx, py = ny * dy, pz = nz * dz;
    const float sv = (px + py) + pz;
    const float bound = ((fabsf(px) + fabsf(py)) + fabsf(pz)) * 6.0e-7f;   // 10 * 2^-24 of the magnitudes
    if (sv > bound) return 1;
    if (sv < -bound) return 0;
    return -1;
}
// EPA.h:71: does the face (normal n, vertex p) see the new vertex v; v and p hold floats
__device__ __forceinline__ bool sees_face(D3 n, D3 v, V3 vf, D3 p) {
    bool ok = true;
    const V3 pf = {f32_trunc(p.x, ok), f32_trunc(p.y, ok), f32_trunc(p.z, ok)};
    const int r = ok ? sees_face_f32(n, vf, pf) : -1;
    if (r >= 0) return r != 0;
    return dot(n, v - p) > 0;
}

// EPA.h:10-186 with fixed capacities (104 vertices = 4 + 100 iterations)
constexpr int kEpaVerts = 104;
constexpr int kEpaFaces = 216;
constexpr int kEpaEdges = 96;
struct EpaFace { int i0, i1, i2; D3 n; };
struct Polytope {
    GjkVertex v[kEpaVerts];
    EpaFace f[kEpaFaces];
    int nv, nf;
};

__device__ inline void epaCreateFace(Polytope& p, int i0, int i1, int i2, int* err) {
    D3 n = cross(p.v[i0].pos - p.v[i1].pos, p.v[i2].pos - p.v[i1].pos);
    double len = length(n);
    if (len) n = n / len;
    if (p.nf < kEpaFaces) p.f[p.nf++] = {i0, i1, i2, n};
    else raise_err(err, ERR_EPA_CAPACITY);
}
__device__ __forceinline__ double epaDist(const Polytope& p, const EpaFace& f) { return dot(p.v[f.i0].pos, f.n); }

__device__ inline void epaInsert(Polytope& p, const GjkVertex& q, int* err) {
    int e0[kEpaEdges], e1[kEpaEdges];
    int ne = 0;
    for (int k = p.nf - 1; k >= 0; --k) {
        EpaFace fc = p.f[k];
        if (dot(fc.n, q.pos - p.v[fc.i0].pos) > 0) {
            int a[3] = {fc.i0, fc.i1, fc.i2}, b[3] = {fc.i1, fc.i2, fc.i0};
            bool found[3] = {false, false, false};
            for (int j = 0; j < 3; ++j) {
                for (int m = ne - 1; m >= 0; --m) {
                    if (e0[m] == b[j] && e1[m] == a[j]) {
                        found[j] = true;
                        e0[m] = e0[ne - 1]; e1[m] = e1[ne - 1]; --ne;
                        break;
                    }
                }
            }
            for (int j = 0; j < 3; ++j) {
                if (found[j]) continue;
                if (ne < kEpaEdges) { e0[ne] = a[j]; e1[ne] = b[j]; ++ne; }
                else raise_err(err, ERR_EPA_CAPACITY);
            }
            p.f[k] = p.f[p.nf - 1];
            --p.nf;
        }
    }
    if (p.nv >= kEpaVerts) { raise_err(err, ERR_EPA_CAPACITY); return; }
    int vi = p.nv;
    p.v[p.nv++] = q;
    for (int m = 0; m < ne; ++m) epaCreateFace(p, vi, e0[m], e1[m], err);
}

__device__ inline V3 epa(const Support& s0, const Support& s1, GjkSimplex& s, V3& cp0, V3& cp1, Polytope& p, int* err) {
    p.nv = 0; p.nf = 0;
    for (int i = 0; i < 4; ++i) p.v[p.nv++] = s.v[i];
    D3 n = cross(p.v[0].pos - p.v[1].pos, p.v[2].pos - p.v[1].pos);
    if (dot(p.v[3].pos - p.v[0].pos, n) < 0) {
        epaCreateFace(p, 0, 1, 2, err); epaCreateFace(p, 3, 1, 0, err); epaCreateFace(p, 3, 2, 1, err); epaCreateFace(p, 3, 0, 2, err);
    } else {
        epaCreateFace(p, 0, 2, 1, err); epaCreateFace(p, 3, 2, 0, err); epaCreateFace(p, 3, 1, 2, err); epaCreateFace(p, 3, 0, 1, err);
    }
    float minDist = 0;
    D3 normal = {0, 0, 0};
    int fi = 0;
    for (int it = 0; it < 100; ++it) {
        minDist = (float)DBL_MAX;
        for (int k = 0; k < p.nf; ++k) {
            double d = epaDist(p, p.f[k]);
            if (d < minDist) { minDist = (float)d; normal = p.f[k].n; fi = k; }
        }
        GjkVertex v = mink(s0, s1, f3(normal));
        if (dot(v.pos, normal) - minDist < (double)0.00001f) break;
        epaInsert(p, v, err);
    }
    // closest points on the closest face (EPA.h:101-143); the projection adds the
    // face distance to every normal component, as the reference does
    const EpaFace& fc = p.f[fi];
    const GjkVertex& a = p.v[fc.i0];
    const GjkVertex& b = p.v[fc.i1];
    const GjkVertex& c = p.v[fc.i2];
    D3 proj = fc.n + epaDist(p, fc);
    V3 v0 = f3(b.pos - a.pos), v1 = f3(c.pos - a.pos), v2 = f3(proj - a.pos);
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
    cp0 = f3(u * d3(a.sp0) + vv * d3(b.sp0) + ww * d3(c.sp0));
    cp1 = f3(u * d3(a.sp1) + vv * d3(b.sp1) + ww * d3(c.sp1));
    return f3(normal);
}

// ---------------------------------------------------------------- analytic pairs

__device__ inline bool sphereSphere(V3 pos0, float r0, V3 pos1, float r1, ManifoldL& res) {
    V3 d = pos1 - pos0;
    float rs = r0 + r1;
    if (dot(d, d) > rs * rs) return false;
    float len = length(d);
    res.normal = len ? d / len : V3{0, 1, 0};
    res.numPoints = 1;
    res.points[0] = {pos0 + res.normal * r0, pos1 - res.normal * r1};
    return true;
}

__device__ inline bool capsuleCapsule(V3 pos0, Q4 or0, float hh0, float r0, V3 pos1, Q4 or1, float hh1, float r1, ManifoldL& res) {
    V3 up = {0, 1, 0};
    V3 v0 = qrot(or0, up), v1 = qrot(or1, up);
    V3 a, b;
    closestPointsBetweenSegments(pos0, v0, -hh0, hh0, pos1, v1, -hh1, hh1, a, b);
    V3 d = b - a;
    float rs = r0 + r1;
    if (dot(d, d) > rs * rs) return false;
    float len = length(d);
    res.normal = len ? d / len : up;
    res.numPoints = 1;
    res.points[0] = {a + res.normal * r0, b - res.normal * r1};
    return true;
}

__device__ inline bool sphereCapsule(V3 pos0, float r0, V3 pos1, Q4 or1, float hh1, float r1, ManifoldL& res) {
    V3 up = {0, 1, 0};
    V3 dir = qrot(or1, up);
    V3 q = closestPointOnSegment(pos0, pos1, dir, -hh1, hh1);
    V3 v = q - pos0;
    float rs = r0 + r1;
    if (dot(v, v) > rs * rs) return false;
    float len = length(v);
    res.normal = len ? v / len : up;
    res.numPoints = 1;
    res.points[0] = {pos0 + res.normal * r0, q - res.normal * r1};
    return true;
}

__device__ inline bool sphereBox(V3 pos0, float r0, V3 pos1, Q4 or1, V3 he1, ManifoldL& res) {
    M3 u1 = mat3_cast(or1);
    V3 d = pos0 - pos1;
    d = {dot(d, u1.c[0]), dot(d, u1.c[1]), dot(d, u1.c[2])};
    V3 q = pos1 + mv(u1, vclamp(d, -he1, he1));
    V3 v = q - pos0;
    if (dot(v, v) > r0 * r0) return false;
    float len = length(v);
    if (len) {
        res.normal = v / len;
        res.numPoints = 1;
        res.points[0] = {pos0 + res.normal * r0, q};
    } else {
        float mn = FLT_MAX;
        int ax = 0;
        for (int i = 0; i < 3; i++) {
            float depth = at(he1, i) - fabsf(at(d, i));
            if (depth < mn) { mn = depth; ax = i; }
        }
        float sg = at(d, ax) ? signG(at(d, ax)) : 1.f;
        V3 bp = d;
        at(bp, ax) = sg * at(he1, ax);
        res.normal = -sg * u1.c[ax];
        res.numPoints = 1;
        res.points[0] = {pos0, pos1 + mv(u1, bp)};
    }
    return true;
}

__device__ inline void capsuleBoxContacts(V3 p0L, V3 p1L, float radius, V3 normal, V3 boxCenter, V3 he, const M3& basis, ManifoldL& res) {
    int boxAxis = 0;
    float boxAxisSign = 0, maxDot = 0;
    for (int i = 0; i < 3; ++i) {
        float d = dot(normal, basis.c[i]);
        float ad = fabsf(d);
        if (ad > maxDot) { maxDot = ad; boxAxis = i; boxAxisSign = d < 0 ? 1 : -1; }
    }
    int cx = (boxAxis + 1) % 3, cy = (boxAxis + 2) % 3;
    V2 l0 = {at(p0L, cx), at(p0L, cy)}, l1 = {at(p1L, cx), at(p1L, cy)};
    V2 clip[4] = {{at(he, cx), at(he, cy)}, {at(he, cx), -at(he, cy)}, {-at(he, cx), -at(he, cy)}, {-at(he, cx), at(he, cy)}};
    if (clipLine(l0, l1, clip, 4)) {
        float onAxis = boxAxisSign * at(he, boxAxis);
        V3 p0 = {0, 0, 0}, p1 = {0, 0, 0};
        float dX = at(p0L, cx) - at(p1L, cx), dY = at(p0L, cy) - at(p1L, cy);
        float aX = fabsf(dX), aY = fabsf(dY);
        if (aX > aY) {
            at(p0, boxAxis) = mixG(at(p0L, boxAxis), at(p1L, boxAxis), (at(p0L, cx) - l0.x) / dX);
            at(p1, boxAxis) = mixG(at(p1L, boxAxis), at(p0L, boxAxis), (at(p1L, cx) - l1.x) / -dX);
        } else if (aY > aX) {
            at(p0, boxAxis) = mixG(at(p0L, boxAxis), at(p1L, boxAxis), (at(p0L, cy) - l0.y) / dY);
            at(p1, boxAxis) = mixG(at(p1L, boxAxis), at(p0L, boxAxis), (at(p1L, cy) - l1.y) / -dY);
        } else {
            at(p0, boxAxis) = at(p0L, boxAxis);
            at(p1, boxAxis) = at(p1L, boxAxis);
        }
        at(p0, boxAxis) -= boxAxisSign * radius;
        at(p1, boxAxis) -= boxAxisSign * radius;
        int n = 0;
        if (fabsf(at(p0, boxAxis)) < at(he, boxAxis)) {
            at(p0, cx) = l0.x; at(p0, cy) = l0.y;
            V3 ob = p0; at(ob, boxAxis) = onAxis;
            res.points[n++] = {boxCenter + mv(basis, p0), boxCenter + mv(basis, ob)};
        }
        if (fabsf(at(p1, boxAxis)) < at(he, boxAxis)) {
            at(p1, cx) = l1.x; at(p1, cy) = l1.y;
            V3 ob = p1; at(ob, boxAxis) = onAxis;
            res.points[n++] = {boxCenter + mv(basis, p1), boxCenter + mv(basis, ob)};
        }
        res.numPoints = n;
    } else {
        res.numPoints = 0;
    }
}

__device__ inline bool capsuleBox(V3 pos0, Q4 or0, float hh0, float r0, V3 pos1, Q4 or1, V3 he1, ManifoldL& res) {
    M3 u1 = mat3_cast(or1);
    V3 p = pos0 - pos1;
    p = {dot(p, u1.c[0]), dot(p, u1.c[1]), dot(p, u1.c[2])};
    V3 dir = qrot(or0, {0, 1, 0});
    V3 dl = {dot(dir, u1.c[0]), dot(dir, u1.c[1]), dot(dir, u1.c[2])};
    float t = 0;
    V3 q = {0, 0, 0};
    float sq = sqrDistSegmentAABB(p, dl, -hh0, hh0, he1, t, q);
    if (sq >= r0 * r0) return false;
    V3 onSeg = pos0 + dir * t;
    V3 onBox = pos1 + mv(u1, q);
    V3 normal = onBox - onSeg;
    float nl = length(normal);
    if (nl) {
        res.normal = normal / nl;
    } else {
        V3 r, ar;
        for (int i = 0; i < 3; ++i) { at(r, i) = dot(dir, u1.c[i]); at(ar, i) = fabsf(at(r, i)); }
        float mx = -FLT_MAX;
        bool edge = false;
        int axis = 0;
        float ra, rb, l, d;
        for (int i = 0; i < 3; i++) {
            ra = hh0 * at(ar, i) + r0;
            rb = at(he1, i);
            l = fabsf(at(p, i));
            d = l - ra - rb;
            if (d > mx) { mx = d; edge = false; axis = i; }
        }
        const float edgeLimit = 0.999f;
        float edgeOffset = 0.1f;
        rb = he1.y * ar.z + he1.z * ar.y;
        l = fabsf(p.z * r.y - p.y * r.z);
        d = l - r0 - rb;
        if (ar.x < edgeLimit && d > mx + edgeOffset) { mx = d; edge = true; axis = 0; edgeOffset = 0; }
        rb = he1.x * ar.z + he1.z * ar.x;
        l = fabsf(p.x * r.z - p.z * r.x);
        d = l - r0 - rb;
        if (ar.y < edgeLimit && d > mx + edgeOffset) { mx = d; edge = true; axis = 1; edgeOffset = 0; }
        rb = he1.x * ar.y + he1.y * ar.x;
        l = fabsf(p.y * r.x - p.x * r.y);
        d = l - r0 - rb;
        if (ar.z < edgeLimit && d > mx + edgeOffset) { mx = d; edge = true; axis = 2; }
        V3 sep = edge ? cross(dir, u1.c[axis]) : u1.c[axis];
        res.normal = normalize(dot(sep, pos1 - pos0) > 0 ? sep : -sep);
    }
    capsuleBoxContacts(p - dl * hh0, p + dl * hh0, r0, res.normal, pos1, he1, u1, res);
    if (!res.numPoints) {
        res.numPoints = 1;
        res.points[0] = {onSeg + res.normal * r0, onBox};
    }
    return true;
}

// ---------------------------------------------------------------- box-box (Collision.cpp:54-350)

__device__ inline void boxBoxFaceContacts(const M3& uRef, V3 posRef, V3 heRef, const M3& uInc, V3 posInc, V3 heInc,
                                          int refAxis, ContactPoint* cp, int& np, int* err) {
    V3 axis = uRef.c[refAxis];
    float refSign = dot(axis, posInc - posRef) < 0 ? -1 : 1;
    float maxDot = 0;
    int incAxis = 0;
    float incSign = 1;
    for (int i = 0; i < 3; ++i) {
        float d = dot(-refSign * axis, uInc.c[i]);
        float ad = fabsf(d);
        if (ad > maxDot) { maxDot = ad; incAxis = i; incSign = d < 0 ? -1 : 1; }
    }
    int a1 = (incAxis + 1) % 3, a2 = (incAxis + 2) % 3;
    M3 inv = inverse(uRef);
    V3 incO = mv(inv, posInc + uInc.c[incAxis] * at(heInc, incAxis) * incSign - posRef);
    V3 e1 = uInc.c[a1] * at(heInc, a1), e2 = uInc.c[a2] * at(heInc, a2);
    V3 ne1 = -uInc.c[a1] * at(heInc, a1);
    V3 p0 = incO + mv(inv, e1 + e2);
    V3 p1 = incO + mv(inv, ne1 + e2);
    V3 p2 = incO + mv(inv, ne1 - e2);
    V3 p3 = incO + mv(inv, e1 - e2);
    int cx = (refAxis + 1) % 3, cy = (refAxis + 2) % 3;
    Poly poly;
    poly.n = 4;
    poly.p[0] = {at(p0, cx), at(p0, cy)};
    poly.p[1] = {at(p1, cx), at(p1, cy)};
    poly.p[2] = {at(p2, cx), at(p2, cy)};
    poly.p[3] = {at(p3, cx), at(p3, cy)};
    V2 clip[4] = {{at(heRef, cx), at(heRef, cy)}, {at(heRef, cx), -at(heRef, cy)},
                  {-at(heRef, cx), -at(heRef, cy)}, {-at(heRef, cx), at(heRef, cy)}};
    suthHodgClip(poly, clip, 4, err);
    V3 incN = mv(inv, uInc.c[incAxis]);
    contactsPolygonBoxFace(posRef, uRef, refAxis, (int)refSign, heRef, incO, incN, poly, cx, cy, cp, np);
}

__device__ inline bool boxBox(V3 pos0, Q4 or0, V3 he0, V3 pos1, Q4 or1, V3 he1, ManifoldL& res, int* err) {
    float edgeOffset = 0.1f;
    const float edgeLimit = 0.999f;
    bool edge = false;
    int fBox = 0, fAxis = 0, e0 = 0, e1 = 0;
    float mx = -FLT_MAX;
    M3 u0 = mat3_cast(or0), u1 = mat3_cast(or1);
    V3 t = pos1 - pos0;
    t = {dot(t, u0.c[0]), dot(t, u0.c[1]), dot(t, u0.c[2])};
    float r[3][3], ar[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) { r[i][j] = dot(u0.c[i], u1.c[j]); ar[i][j] = fabsf(r[i][j]); }
    float ra, rb, l, d;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        ra = at(he0, i);
        rb = he1.x * ar[i][0] + he1.y * ar[i][1] + he1.z * ar[i][2];
        l = fabsf(at(t, i));
        d = l - ra - rb;
        if (d > 0) return false;
        if (d > mx) { mx = d; edge = false; fBox = 0; fAxis = i; }
    }
#pragma unroll
    for (int i = 0; i < 3; i++) {
        ra = he0.x * ar[0][i] + he0.y * ar[1][i] + he0.z * ar[2][i];
        rb = at(he1, i);
        l = fabsf(t.x * r[0][i] + t.y * r[1][i] + t.z * r[2][i]);
        d = l - ra - rb;
        if (d > 0) return false;
        if (d > mx) { mx = d; edge = false; fBox = 1; fAxis = i; }
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const int i = k / 3, j = k % 3;
        switch (k) {
            case 0: ra = he0.y * ar[2][0] + he0.z * ar[1][0]; rb = he1.y * ar[0][2] + he1.z * ar[0][1]; l = fabsf(t.z * r[1][0] - t.y * r[2][0]); break;
            case 1: ra = he0.y * ar[2][1] + he0.z * ar[1][1]; rb = he1.x * ar[0][2] + he1.z * ar[0][0]; l = fabsf(t.z * r[1][1] - t.y * r[2][1]); break;
            case 2: ra = he0.y * ar[2][2] + he0.z * ar[1][2]; rb = he1.x * ar[0][1] + he1.y * ar[0][0]; l = fabsf(t.z * r[1][2] - t.y * r[2][2]); break;
            case 3: ra = he0.x * ar[2][0] + he0.z * ar[0][0]; rb = he1.y * ar[1][2] + he1.z * ar[1][1]; l = fabsf(t.x * r[2][0] - t.z * r[0][0]); break;
            case 4: ra = he0.x * ar[2][1] + he0.z * ar[0][1]; rb = he1.x * ar[1][2] + he1.z * ar[1][0]; l = fabsf(t.x * r[2][1] - t.z * r[0][1]); break;
            case 5: ra = he0.x * ar[2][2] + he0.z * ar[0][2]; rb = he1.x * ar[1][1] + he1.y * ar[1][0]; l = fabsf(t.x * r[2][2] - t.z * r[0][2]); break;
            case 6: ra = he0.x * ar[1][0] + he0.y * ar[0][0]; rb = he1.y * ar[2][2] + he1.z * ar[2][1]; l = fabsf(t.y * r[0][0] - t.x * r[1][0]); break;
            case 7: ra = he0.x * ar[1][1] + he0.y * ar[0][1]; rb = he1.x * ar[2][2] + he1.z * ar[2][0]; l = fabsf(t.y * r[0][1] - t.x * r[1][1]); break;
            default: ra = he0.x * ar[1][2] + he0.y * ar[0][2]; rb = he1.x * ar[2][1] + he1.y * ar[2][0]; l = fabsf(t.y * r[0][2] - t.x * r[1][2]); break;
        }
        d = l - ra - rb;
        if (d > 0) return false;
        if (ar[i][j] < edgeLimit && d > mx + edgeOffset) {
            mx = d; edge = true; e0 = i; e1 = j;
            if (k < 8) edgeOffset = 0;
        }
    }
    if (!edge) {
        V3 axis;
        ContactPoint cp[4];
        int np = 0;
        if (fBox) {
            axis = u1.c[fAxis];
            boxBoxFaceContacts(u1, pos1, he1, u0, pos0, he0, fAxis, cp, np, err);
            for (int i = 0; i < np; i++) res.points[i] = {cp[i].p1, cp[i].p0};
        } else {
            axis = u0.c[fAxis];
            boxBoxFaceContacts(u0, pos0, he0, u1, pos1, he1, fAxis, cp, np, err);
            for (int i = 0; i < np; i++) res.points[i] = cp[i];
        }
        res.numPoints = np;
        res.normal = dot(axis, pos1 - pos0) < 0 ? -axis : axis;
    } else {
        V3 axis = cross(u0.c[e0], u1.c[e1]);
        res.normal = normalize(dot(axis, pos1 - pos0) < 0 ? -axis : axis);
        V3 s0 = v3s(-1);
        at(s0, (e0 + 1) % 3) = dot(u0.c[(e0 + 1) % 3], res.normal) < 0 ? -1 : 1;
        at(s0, (e0 + 2) % 3) = dot(u0.c[(e0 + 2) % 3], res.normal) < 0 ? -1 : 1;
        V3 p0 = pos0 + s0.x * he0.x * u0.c[0] + s0.y * he0.y * u0.c[1] + s0.z * he0.z * u0.c[2];
        V3 s1 = v3s(-1);
        at(s1, (e1 + 1) % 3) = dot(u1.c[(e1 + 1) % 3], res.normal) > 0 ? -1 : 1;
        at(s1, (e1 + 2) % 3) = dot(u1.c[(e1 + 2) % 3], res.normal) > 0 ? -1 : 1;
        V3 p1 = pos1 + s1.x * he1.x * u1.c[0] + s1.y * he1.y * u1.c[1] + s1.z * he1.z * u1.c[2];
        res.numPoints = 1;
        V3 q0, q1;
        closestPointsBetweenSegments(p0, u0.c[e0], 0, at(he0, e0) * 2, p1, u1.c[e1], 0, at(he1, e1) * 2, q0, q1);
        res.points[0] = {q0, q1};
    }
    return true;
}

// ---------------------------------------------------------------- convex meshes (Collision.cpp:352-887)

struct ConvexView {
    const float4* verts;
    int nverts;
    int face_start, face_count;
};
__device__ __forceinline__ ConvexView convexView(const World& w, int mesh) {
    ConvexMeshDev cm = w.convex[mesh];
    return {w.convex_verts + cm.vert_start, cm.vert_count_padded, cm.face_start, cm.face_count};
}
__device__ __forceinline__ Support convexSupport(const World& w, V3 pos, Q4 ori, int mesh, V3 scale) {
    Support s;
    s.kind = 3; s.pos = pos; s.basis = mat3_cast(ori);
    ConvexMeshDev cm = w.convex[mesh];
    s.verts = w.convex_verts + cm.vert_start; s.nverts = cm.vert_count_padded; s.scale = scale;
    return s;
}
__device__ __forceinline__ V3 faceNormal(const World& w, int f) { return ld3(w.face_normal[f]); }
__device__ __forceinline__ V3 faceCentroid(const World& w, int f) { return ld3(w.face_centroid[f]); }

__device__ inline void convexConvexContacts(const World& w, V3 pos0, Q4 or0, int m0, V3 sc0, V3 pos1, Q4 or1, int m1, V3 sc1,
                                            V3 normal, ContactPoint* cp, int& np, int* err) {
    ConvexView A = convexView(w, m0), B = convexView(w, m1);
    int f0 = 0;
    float maxDot = 0;
    for (int i = 0; i < A.face_count; ++i) {
        float d = dot(normal, normalize(qrot(or0, faceNormal(w, A.face_start + i) / sc0)));
        if (d > maxDot) { maxDot = d; f0 = i; }
    }
    int f1 = 0;
    float minDot = 0;
    for (int i = 0; i < B.face_count; ++i) {
        float d = dot(normal, normalize(qrot(or1, faceNormal(w, B.face_start + i) / sc1)));
        if (d < minDot) { minDot = d; f1 = i; }
    }
    int F0 = A.face_start + f0, F1 = B.face_start + f1;
    M3 c0w = mat3_cast(or0);
    M3 wc0 = transpose(c0w);
    V3 refO = sc0 * faceCentroid(w, F0);
    int i0s = w.face_idx_start[F0], i0e = w.face_idx_start[F0 + 1];
    int i1s = w.face_idx_start[F1], i1e = w.face_idx_start[F1 + 1];
    V3 u0 = normalize(sc0 * ld3(A.verts[w.face_idx[i0s]]) - refO);
    V3 u1 = normalize(faceNormal(w, F0) / sc0);
    V3 u2 = cross(u0, u1);
    M3 c0r = transpose(m3cols(u0, u1, u2));
    M3 wr = mm(c0r, wc0);
    const int cx = 2, cy = 0;
    V2 clip[kMaxPoly];
    int nc = min(i0e - i0s, kMaxPoly);
    for (int i = 0; i < nc; ++i) {
        V3 v = mv(c0r, sc0 * ld3(A.verts[w.face_idx[i0s + i]]));
        clip[i] = {at(v, cx), at(v, cy)};
    }
    Poly poly;
    poly.n = min(i1e - i1s, kMaxPoly);
    for (int i = 0; i < poly.n; ++i) {
        V3 v = mv(wr, pos1 + qrot(or1, sc1 * ld3(B.verts[w.face_idx[i1s + i]])) - pos0);
        poly.p[i] = {at(v, cx), at(v, cy)};
    }
    suthHodgClip(poly, clip, nc, err);
    V3 incO = mv(wr, pos1 + qrot(or1, sc1 * faceCentroid(w, F1)) - pos0);
    V3 incN = mv(wr, qrot(or1, normalize(faceNormal(w, F1) / sc1)));
    M3 rw = transpose(wr);
    contactsPolygonPolygonFace(pos0, rw, refO, u1, incO, incN, poly, cx, cy, cp, np);
}

__device__ inline void capsuleConvexContacts(const World& w, V3 p0L, V3 p1L, float radius, V3 meshPos, const M3& c2w, int mesh,
                                             V3 sc, ManifoldL& res) {
    ConvexView C = convexView(w, mesh);
    int fi = 0;
    float minDot = 0;
    for (int i = 0; i < C.face_count; ++i) {
        float d = dot(res.normal, normalize(mv(c2w, faceNormal(w, C.face_start + i) / sc)));
        if (d < minDot) { minDot = d; fi = i; }
    }
    int F = C.face_start + fi;
    int is = w.face_idx_start[F], ie = w.face_idx_start[F + 1];
    V3 refO = sc * faceCentroid(w, F);
    V3 u0 = normalize(sc * ld3(C.verts[w.face_idx[is]]) - refO);
    V3 u1 = normalize(faceNormal(w, F) / sc);
    V3 u2 = cross(u0, u1);
    M3 c2r = transpose(m3cols(u0, u1, u2));
    const int fa = 1, cx = 2, cy = 0;
    V2 clip[kMaxPoly];
    int nc = min(ie - is, kMaxPoly);
    for (int i = 0; i < nc; ++i) {
        V3 v = mv(c2r, sc * ld3(C.verts[w.face_idx[is + i]]));
        clip[i] = {at(v, cx), at(v, cy)};
    }
    V3 p0R = mv(c2r, p0L), p1R = mv(c2r, p1L);
    V2 l0 = {at(p0R, cx), at(p0R, cy)}, l1 = {at(p1R, cx), at(p1R, cy)};
    if (clipLine(l0, l1, clip, nc)) {
        M3 r2w = mm(c2w, transpose(c2r));
        float dPlane = dot(refO, u1);
        V3 p0 = {0, 0, 0}, p1 = {0, 0, 0};
        float dX = at(p0R, cx) - at(p1R, cx), dY = at(p0R, cy) - at(p1R, cy);
        float aX = fabsf(dX), aY = fabsf(dY);
        if (aX && aX >= aY) {
            at(p0, fa) = mixG(at(p0R, fa), at(p1R, fa), (at(p0R, cx) - l0.x) / dX);
            at(p1, fa) = mixG(at(p1R, fa), at(p0R, fa), (at(p1R, cx) - l1.x) / -dX);
        } else if (aY > aX) {
            at(p0, fa) = mixG(at(p0R, fa), at(p1R, fa), (at(p0R, cy) - l0.y) / dY);
            at(p1, fa) = mixG(at(p1R, fa), at(p0R, fa), (at(p1R, cy) - l1.y) / -dY);
        } else {
            at(p0, fa) = at(p0R, fa);
            at(p1, fa) = at(p1R, fa);
        }
        at(p0, fa) -= radius;
        at(p1, fa) -= radius;
        int n = 0;
        if (at(p0, fa) < dPlane) {
            at(p0, cx) = l0.x; at(p0, cy) = l0.y;
            V3 of = p0; at(of, fa) = dPlane;
            res.points[n++] = {meshPos + mv(r2w, p0), meshPos + mv(r2w, of)};
        }
        if (at(p1, fa) < dPlane) {
            at(p1, cx) = l1.x; at(p1, cy) = l1.y;
            V3 of = p1; at(of, fa) = dPlane;
            res.points[n++] = {meshPos + mv(r2w, p1), meshPos + mv(r2w, of)};
        }
        res.numPoints = n;
    } else {
        res.numPoints = 0;
    }
}

__device__ inline void boxConvexContacts(const World& w, V3 boxC, const M3& basis, V3 he, V3 cPos, Q4 cOr, int mesh, V3 sc,
                                         V3 normal, ContactPoint* cp, int& np, int* err) {
    ConvexView C = convexView(w, mesh);
    int boxAxis = 0;
    float boxAxisSign = 0, maxDot = 0;
    for (int i = 0; i < 3; ++i) {
        float d = dot(normal, basis.c[i]);
        float ad = fabsf(d);
        if (ad > maxDot) { maxDot = ad; boxAxis = i; boxAxisSign = d < 0 ? -1 : 1; }
    }
    int fi = 0;
    float minDot = 0;
    for (int i = 0; i < C.face_count; ++i) {
        float d = dot(normal, normalize(qrot(cOr, faceNormal(w, C.face_start + i) / sc)));
        if (d < minDot) { minDot = d; fi = i; }
    }
    int F = C.face_start + fi;
    int is = w.face_idx_start[F], ie = w.face_idx_start[F + 1];
    int cx = (boxAxis + 1) % 3, cy = (boxAxis + 2) % 3;
    M3 w2b = transpose(basis);
    Poly poly;
    poly.n = min(ie - is, kMaxPoly);
    for (int i = 0; i < poly.n; ++i) {
        V3 v = mv(w2b, cPos + qrot(cOr, sc * ld3(C.verts[w.face_idx[is + i]])) - boxC);
        poly.p[i] = {at(v, cx), at(v, cy)};
    }
    V2 clip[4] = {{at(he, cx), at(he, cy)}, {at(he, cx), -at(he, cy)}, {-at(he, cx), -at(he, cy)}, {-at(he, cx), at(he, cy)}};
    suthHodgClip(poly, clip, 4, err);
    V3 incO = mv(w2b, cPos + qrot(cOr, sc * faceCentroid(w, F)) - boxC);
    V3 incN = normalize(mv(w2b, qrot(cOr, faceNormal(w, F) / sc)));
    contactsPolygonBoxFace(boxC, basis, boxAxis, (int)boxAxisSign, he, incO, incN, poly, cx, cy, cp, np);
}

__device__ __forceinline__ void flipM(ManifoldL& r) {
    r.normal = -r.normal;
    for (int i = 0; i < r.numPoints; ++i) r.points[i] = {r.points[i].p1, r.points[i].p0};
}

// The analytic part of physecs::collision (Collision.cpp:910-1016) for pairs without convex meshes.
__device__ inline bool collideAnalytic(V3 pos0, Q4 or0, const GeomD& g0, V3 pos1, Q4 or1, const GeomD& g1, ManifoldL& r, int* err) {
    r.numPoints = 0;
    r.triangleIndex = -1;
    switch (g0.type) {
        case G_SPHERE:
            switch (g1.type) {
                case G_SPHERE: return sphereSphere(pos0, g0.p[0], pos1, g1.p[0], r);
                case G_CAPSULE: return sphereCapsule(pos0, g0.p[0], pos1, or1, g1.p[0], g1.p[1], r);
                default: return sphereBox(pos0, g0.p[0], pos1, or1, gv(g1), r);
            }
        case G_CAPSULE:
            switch (g1.type) {
                case G_SPHERE: { bool h = sphereCapsule(pos1, g1.p[0], pos0, or0, g0.p[0], g0.p[1], r); flipM(r); return h; }
                case G_CAPSULE: return capsuleCapsule(pos0, or0, g0.p[0], g0.p[1], pos1, or1, g1.p[0], g1.p[1], r);
                default: return capsuleBox(pos0, or0, g0.p[0], g0.p[1], pos1, or1, gv(g1), r);
            }
        default:
            switch (g1.type) {
                case G_SPHERE: { bool h = sphereBox(pos1, g1.p[0], pos0, or0, gv(g0), r); flipM(r); return h; }
                case G_CAPSULE: { bool h = capsuleBox(pos1, or1, g1.p[0], g1.p[1], pos0, or0, gv(g0), r); flipM(r); return h; }
                default: return boxBox(pos0, or0, gv(g0), pos1, or1, gv(g1), r, err);
            }
    }
}

// collideAnalytic for pairs with BOXES boxes: each list's kernel holds only its own routines
template <int BOXES>
__device__ inline bool collideAnalyticT(V3 pos0, Q4 or0, const GeomD& g0, V3 pos1, Q4 or1, const GeomD& g1, ManifoldL& r, int* err) {
    r.numPoints = 0;
    r.triangleIndex = -1;
    if constexpr (BOXES == 2) {
        return boxBox(pos0, or0, gv(g0), pos1, or1, gv(g1), r, err);
    } else if constexpr (BOXES == 1) {
        if (g1.type == G_BOX) {
            if (g0.type == G_SPHERE) return sphereBox(pos0, g0.p[0], pos1, or1, gv(g1), r);
            return capsuleBox(pos0, or0, g0.p[0], g0.p[1], pos1, or1, gv(g1), r);
        }
        if (g1.type == G_SPHERE) { bool h = sphereBox(pos1, g1.p[0], pos0, or0, gv(g0), r); flipM(r); return h; }
        bool h = capsuleBox(pos1, or1, g1.p[0], g1.p[1], pos0, or0, gv(g0), r);
        flipM(r);
        return h;
    } else {
        if (g0.type == G_SPHERE) {
            if (g1.type == G_SPHERE) return sphereSphere(pos0, g0.p[0], pos1, g1.p[0], r);
            return sphereCapsule(pos0, g0.p[0], pos1, or1, g1.p[0], g1.p[1], r);
        }
        if (g1.type == G_SPHERE) { bool h = sphereCapsule(pos1, g1.p[0], pos0, or0, g0.p[0], g0.p[1], r); flipM(r); return h; }
        return capsuleCapsule(pos0, or0, g0.p[0], g0.p[1], pos1, or1, g1.p[0], g1.p[1], r);
    }
}

// convex-mesh pairs of physecs::collision (Collision.cpp:414-426, 488-499, 787-807, 873-887),
// in three parts: the two supports, GJK + EPA, and the contact generation that
// follows EPA.  g1 is always the convex mesh here.
__device__ inline void convexOrderedSupports(const World& w, V3 pos0, Q4 or0, const GeomD& g0, V3 pos1, Q4 or1,
                                             const GeomD& g1, Support& a, Support& b) {
    b = convexSupport(w, pos1, or1, g1.mesh, gv(g1));
    switch (g0.type) {
        case G_SPHERE: a.kind = 0; a.pos = pos0; a.radius = g0.p[0]; break;
        case G_CAPSULE: a.kind = 1; a.pos = pos0; a.axis = qrot(or0, {0, 1, 0}); a.halfHeight = g0.p[0]; a.radius = g0.p[1]; break;
        case G_BOX: a.kind = 2; a.pos = pos0; a.basis = mat3_cast(or0); a.he = gv(g0); break;
        default: a = convexSupport(w, pos0, or0, g0.mesh, gv(g0)); break;
    }
}

// r.normal and r.points[0] hold the EPA normal and closest points on entry.
__device__ inline void convexOrderedContacts(const World& w, V3 pos0, Q4 or0, const GeomD& g0, V3 pos1, Q4 or1,
                                             const GeomD& g1, ManifoldL& r, int* err) {
    switch (g0.type) {
        case G_SPHERE: r.numPoints = 1; break;
        case G_CAPSULE: {
            M3 c2w = mat3_cast(or1);
            M3 w2c = inverse(c2w);
            V3 p = mv(w2c, pos0 - pos1);
            V3 al = mv(w2c, qrot(or0, {0, 1, 0}));
            capsuleConvexContacts(w, p + al * g0.p[0], p - al * g0.p[0], g0.p[1], pos1, c2w, g1.mesh, gv(g1), r);
            if (!r.numPoints) r.numPoints = 1;
            break;
        }
        case G_BOX:
            boxConvexContacts(w, pos0, mat3_cast(or0), gv(g0), pos1, or1, g1.mesh, gv(g1), r.normal, r.points, r.numPoints, err);
            if (!r.numPoints) r.numPoints = 1;
            break;
        default:
            convexConvexContacts(w, pos0, or0, g0.mesh, gv(g0), pos1, or1, g1.mesh, gv(g1), r.normal, r.points, r.numPoints, err);
            if (!r.numPoints) r.numPoints = 1;
            break;
    }
}

__device__ inline bool collideConvexOrdered(const World& w, V3 pos0, Q4 or0, const GeomD& g0, V3 pos1, Q4 or1, const GeomD& g1,
                                            ManifoldL& r, Polytope& poly, int* err) {
    Support a, b;
    convexOrderedSupports(w, pos0, or0, g0, pos1, or1, g1, a, b);
    GjkSimplex s;
    if (!gjk(a, b, pos1 - pos0, s)) return false;
    r.normal = epa(a, b, s, r.points[0].p0, r.points[0].p1, poly, err);
    r.numPoints = 0;
    convexOrderedContacts(w, pos0, or0, g0, pos1, or1, g1, r, err);
    return true;
}

__device__ inline bool collideConvex(const World& w, V3 pos0, Q4 or0, const GeomD& g0, V3 pos1, Q4 or1, const GeomD& g1,
                                     ManifoldL& r, Polytope& poly, int* err) {
    r.numPoints = 0;
    r.triangleIndex = -1;
    if (g1.type == G_CONVEX) return collideConvexOrdered(w, pos0, or0, g0, pos1, or1, g1, r, poly, err);
    // convex mesh first: the reference calls the (other, convex) routine and flips the manifold
    bool h = collideConvexOrdered(w, pos1, or1, g1, pos0, or0, g0, r, poly, err);
    flipM(r);
    return h;
}

}  // namespace psx
