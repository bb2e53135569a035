// narrow_util.cuh — closest-point kernels, polygon clipping and manifold
// reduction used by the narrowphase kernels.
//
// Device restatement of Physecs src/GeomUtil.cpp:7-665, src/Clipping.cpp:9-71
// and src/ContactsUtil.cpp:9-204, floating-point operation for operation.
#pragma once
#include "types.cuh"

namespace psx {

enum { TF_FACE = 0, TF_EDGE = 1, TF_VERTEX = 2 };

struct ContactPoint { V3 p0, p1; };
struct ManifoldL {
    int numPoints;
    ContactPoint points[4];
    V3 normal;
    int triangleIndex;
};

struct Poly { V2 p[kMaxPoly]; int n; };

__device__ __forceinline__ void raise_err(int* err, int bit) { atomicOr(err, bit); }

// GeomUtil.cpp:7-12
__device__ inline V3 closestPointOnSegment(V3 point, V3 o, V3 d, float mn, float mx) {
    V3 r = o - point;
    float t = -dot(r, d);
    t = clampG(t, mn, mx);
    return o + t * d;
}

// GeomUtil.cpp:14-59
__device__ inline void closestPointsBetweenSegments(V3 o0, V3 d0, float min0, float max0, V3 o1, V3 d1, float min1,
                                                    float max1, V3& p0, V3& p1) {
    float v1v2 = dot(d0, d1);
    V3 r = o1 - o0;
    float rv1 = dot(r, d0), rv2 = dot(r, d1);
    float t1 = fabsf(v1v2) > 1.f - 0.0001f ? 0 : (rv1 * v1v2 - rv2) / (1.f - v1v2 * v1v2);
    float t0 = rv1 + t1 * v1v2;
    if (t0 < min0) { t0 = min0; p0 = o0 + t0 * d0; t1 = -dot(o1 - p0, d1); }
    else if (t0 > max0) { t0 = max0; p0 = o0 + t0 * d0; t1 = -dot(o1 - p0, d1); }
    else p0 = o0 + t0 * d0;
    if (t1 < min1) { t1 = min1; p1 = o1 + t1 * d1; t0 = -dot(o0 - p1, d0); t0 = clampG(t0, min0, max0); p0 = o0 + t0 * d0; }
    else if (t1 > max1) { t1 = max1; p1 = o1 + t1 * d1; t0 = -dot(o0 - p1, d0); t0 = clampG(t0, min0, max0); p0 = o0 + t0 * d0; }
    else p1 = o1 + t1 * d1;
}

// GeomUtil.cpp:61-127
__device__ inline void closestPointsBetweenSegmentsV(V3 o0, V3 v0, V3 o1, V3 v1, V3& p0, V3& p1) {
    float v0v0 = dot(v0, v0);
    if (v0v0 < 0.0001f) {
        float v1v1 = dot(v1, v1);
        if (v1v1 < 0.0001f) { p0 = o0; p1 = o1; return; }
        float t1 = -dot(o1 - o0, v1) / v1v1;
        p0 = o0; p1 = o1 + t1 * v1; return;
    }
    float v1v1 = dot(v1, v1);
    if (v1v1 < 0.0001f) {
        float t0 = -dot(o0 - o1, v0) / v0v0;
        p0 = o0 + t0 * v0; p1 = o1; return;
    }
    float v0v1 = dot(v0, v1);
    V3 r = o1 - o0;
    float rv0 = dot(r, v0), rv1 = dot(r, v1);
    float denom = v0v0 * v1v1 - v0v1 * v0v1;
    float t1 = fabsf(denom) < 0.0001f ? 0 : (rv0 * v0v1 - rv1 * v0v0) / denom;
    float t0 = (rv0 + t1 * v0v1) / v0v0;
    if (t0 < 0) { t0 = 0; p0 = o0 + t0 * v0; t1 = -dot(o1 - p0, v1) / v1v1; }
    else if (t0 > 1) { t0 = 1; p0 = o0 + t0 * v0; t1 = -dot(o1 - p0, v1) / v1v1; }
    else p0 = o0 + t0 * v0;
    if (t1 < 0) { t1 = 0; p1 = o1 + t1 * v1; t0 = -dot(o0 - p1, v0) / v0v0; t0 = clampG(t0, 0.f, 1.f); p0 = o0 + t0 * v0; }
    else if (t1 > 1) { t1 = 1; p1 = o1 + t1 * v1; t0 = -dot(o0 - p1, v0) / v0v0; t0 = clampG(t0, 0.f, 1.f); p0 = o0 + t0 * v0; }
    else p1 = o1 + t1 * v1;
}

// GeomUtil.cpp:129-169
__device__ inline float caseTwoZeros(V3 p, int axis, V3 he, float& t, V3& q) {
    float sq = 0;
    t = at(he, axis) - at(p, axis);
    at(q, axis) = at(p, axis) + t;
    int a1 = (axis + 1) % 3, a2 = (axis + 2) % 3;
    if (at(p, a1) > at(he, a1)) { float d = at(p, a1) - at(he, a1); sq += d * d; at(q, a1) = at(he, a1); }
    else if (at(p, a1) < -at(he, a1)) { float d = at(p, a1) + at(he, a1); sq += d * d; at(q, a1) = -at(he, a1); }
    else at(q, a1) = at(p, a1);
    if (at(p, a2) > at(he, a2)) { float d = at(p, a2) - at(he, a2); sq += d * d; at(q, a2) = at(he, a2); }
    else if (at(p, a2) < -at(he, a2)) { float d = at(p, a2) + at(he, a2); sq += d * d; at(q, a2) = -at(he, a2); }
    else at(q, a2) = at(p, a2);
    return sq;
}

// GeomUtil.cpp:171-235
__device__ inline float caseOneZero(V3 p, int z0, V3 dir, V3 he, float& t, V3& q) {
    float sq = 0;
    at(q, z0) = at(p, z0);
    V3 pm = p - he;
    int x = (z0 + 1) % 3, y = (z0 + 2) % 3;
    float prod0 = at(dir, y) * at(pm, x);
    float prod1 = at(dir, x) * at(pm, y);
    if (prod0 >= prod1) {
        at(q, x) = at(he, x);
        float eY = at(p, y) + at(he, y);
        float delta = prod0 - at(dir, x) * eY;
        if (delta >= 0) { sq += delta * delta; at(q, y) = -at(he, y); t = -(at(pm, x) * at(dir, x) + eY * at(dir, y)); }
        else { at(q, y) = at(p, y) - prod0 / at(dir, x); t = -at(pm, x) / at(dir, x); }
    } else {
        at(q, y) = at(he, y);
        float eX = at(p, x) + at(he, x);
        float delta = prod1 - at(dir, y) * eX;
        if (delta >= 0) { sq += delta * delta; at(q, x) = -at(he, x); t = -(eX * at(dir, x) + at(pm, y) * at(dir, y)); }
        else { at(q, x) = at(p, x) - prod1 / at(dir, y); t = -at(pm, y) / at(dir, y); }
    }
    if (at(p, z0) < -at(he, z0)) { float d = at(p, z0) + at(he, z0); sq += d * d; at(q, z0) = -at(he, z0); }
    else if (at(p, z0) > at(he, z0)) { float d = at(p, z0) - at(he, z0); sq += d * d; at(q, z0) = at(he, z0); }
    return sq;
}

// GeomUtil.cpp:237-370, including the region-5 expression exactly as the reference writes it
__device__ inline float sqrDistLineAABBFace(V3 p, V3 dir, V3 he, int x, V3 pm, float& t, V3& q) {
    q = p;
    t = 0;
    float sq = 0;
    int y = (x + 1) % 3, z = (y + 1) % 3;
    V3 pp = p + he;
    const float Dx = at(dir, x), Dy = at(dir, y), Dz = at(dir, z);
    const float PMx = at(pm, x), PMy = at(pm, y), PMz = at(pm, z);
    const float PPy = at(pp, y), PPz = at(pp, z);
    const float Py = at(p, y), Pz = at(p, z);
    const float Hx = at(he, x), Hy = at(he, y), Hz = at(he, z);
    if (Dx * PPy >= Dy * PMx) {
        if (Dx * PPz >= Dz * PMx) {
            at(q, x) = Hx;
            at(q, y) -= PMx * Dy / Dx;
            at(q, z) -= PMx * Dz / Dx;
            t = -PMx / Dx;
        } else {
            float sqrLen = Dx * Dx + Dz * Dz;
            float nY = Py - Dy * (Dx * PMx + Dz * PPz) / sqrLen;
            if (nY <= Hy) {
                float tmp = Py - nY;
                float delta = Dx * PMx + Dy * tmp + Dz * PPz;
                t = -delta;
                sq = PMx * PMx + tmp * tmp + PPz * PPz - delta * delta;
                at(q, x) = Hx; at(q, y) = nY; at(q, z) = -Hz;
            } else {
                float delta = Dx * PMx + Dy * PMy + Dz * PPz;
                t = -delta;
                sq = PMx * PMx + PMy + PMy + PPz * PPz - delta * delta;
                at(q, x) = Hx; at(q, y) = Hy; at(q, z) = -Hz;
            }
        }
    } else {
        if (Dx * PPz >= Dz * PMx) {
            float sqrLen = Dx * Dx + Dy * Dy;
            float nZ = Pz - Dz * (Dx * PMx + Dy * PPy) / sqrLen;
            if (nZ <= Hz) {
                float tmp = Pz - nZ;
                float delta = Dx * PMx + Dy * PPy + Dz * tmp;
                t = -delta;
                sq = PMx * PMx + PPy * PPy + tmp * tmp - delta * delta;
                at(q, x) = Hx; at(q, y) = -Hy; at(q, z) = nZ;
            } else {
                float delta = Dx * PMx + Dy * PPy + Dz * PMz;
                t = -delta;
                sq = PMx * PMx + PPy * PPy + PMz * PMz - delta * delta;
                at(q, x) = Hx; at(q, y) = -Hy; at(q, z) = Hz;
            }
        } else {
            float nY = Py - Dy * (Dx * PMx + Dz * PPz) / (Dx * Dx + Dz * Dz);
            if (nY >= -Hy) {
                if (nY <= Hy) {
                    float tmp = Py - nY;
                    float delta = Dx * PMx + Dy * tmp + Dz * PPz;
                    t = -delta;
                    sq = PMx * PMx + tmp * tmp + PPz * PPz - delta * delta;
                    at(q, x) = Hx; at(q, y) = nY; at(q, z) = -Hz;
                } else {
                    float delta = Dx * PMx + Dy * PMy + Dz * PPz;
                    t = -delta;
                    sq = PMx * PMx + PMy + PMy + PPz * PPz - delta * delta;
                    at(q, x) = Hx; at(q, y) = Hy; at(q, z) = -Hz;
                }
                return sq;
            }
            float nZ = Pz - Dz * (Dx * PMx + Dy * PPy) / (Dx * Dx + Dy * Dy);
            if (nZ >= -Hz) {
                if (nZ <= Hz) {
                    float tmp = Pz - nZ;
                    float delta = Dx * PMx + Dy * PPy + Dz * tmp;
                    t = -delta;
                    sq = PMx * PMx + PPy * PPy + tmp * tmp - delta * delta;
                    at(q, x) = Hx; at(q, y) = -Hy; at(q, z) = nZ;
                } else {
                    float delta = Dx * PMx + Dy * PPy + Dz * PMz;
                    t = -delta;
                    sq = PMx * PMx + PPy * PPy + PMz * PMz - delta * delta;
                    at(q, x) = Hx; at(q, y) = -Hy; at(q, z) = Hz;
                }
                return sq;
            }
            float delta = Dx * PMx + Dy * PPy + Dz * PPz;
            t = -delta;
            sq = PMx * PMx + PPy * PPy + PPz * PPz - delta * delta;
            at(q, x) = Hx; at(q, y) = -Hy; at(q, z) = -Hz;
        }
    }
    return sq;
}

// GeomUtil.cpp:372-399
__device__ inline float caseNoZeroes(V3 p, V3 dir, V3 he, float& t, V3& q) {
    V3 pm = p - he;
    float dxEy = dir.x * pm.y, dyEx = dir.y * pm.x;
    if (dyEx >= dxEy) {
        float dzEx = dir.z * pm.x, dxEz = dir.x * pm.z;
        return (dzEx >= dxEz) ? sqrDistLineAABBFace(p, dir, he, 0, pm, t, q) : sqrDistLineAABBFace(p, dir, he, 2, pm, t, q);
    }
    float dzEy = dir.z * pm.y, dyEz = dir.y * pm.z;
    return (dzEy >= dyEz) ? sqrDistLineAABBFace(p, dir, he, 1, pm, t, q) : sqrDistLineAABBFace(p, dir, he, 2, pm, t, q);
}

// GeomUtil.cpp:401-405
__device__ inline float sqrDistPointAABB(V3 p, V3 he, V3& q) {
    q = vclamp(p, -he, he);
    V3 d = p - q;
    return dot(d, d);
}

// GeomUtil.cpp:407-453
__device__ inline float sqrDistLineAABB(V3 p, V3 dir, V3 he, float& t, V3& q) {
    bool refl[3];
    for (int i = 0; i < 3; i++) {
        if (at(dir, i) < 0.0f) { at(p, i) = -at(p, i); at(dir, i) = -at(dir, i); refl[i] = true; }
        else refl[i] = false;
    }
    float sq;
    if (dir.x > 0) {
        if (dir.y > 0) sq = (dir.z > 0) ? caseNoZeroes(p, dir, he, t, q) : caseOneZero(p, 2, dir, he, t, q);
        else sq = (dir.z > 0) ? caseOneZero(p, 1, dir, he, t, q) : caseTwoZeros(p, 0, he, t, q);
    } else {
        if (dir.y > 0) sq = (dir.z > 0) ? caseOneZero(p, 0, dir, he, t, q) : caseTwoZeros(p, 1, he, t, q);
        else {
            if (dir.z > 0) sq = caseTwoZeros(p, 2, he, t, q);
            else { sq = sqrDistPointAABB(p, he, q); t = 0; }
        }
    }
    for (int i = 0; i < 3; i++) if (refl[i]) at(q, i) = -at(q, i);
    return sq;
}

// GeomUtil.cpp:455-467
__device__ inline float sqrDistSegmentAABB(V3 p, V3 dir, float mn, float mx, V3 he, float& t, V3& q) {
    float sq = sqrDistLineAABB(p, dir, he, t, q);
    if (t < mn) { t = mn; sq = sqrDistPointAABB(p + dir * t, he, q); }
    else if (t > mx) { t = mx; sq = sqrDistPointAABB(p + dir * t, he, q); }
    return sq;
}

// GeomUtil.cpp:469-538
__device__ inline float sqrDistPointTriangle(V3 p, V3 a, V3 b, V3 c, V3& q, int& feature, int& fi) {
    V3 ab = b - a, ac = c - a, ap = p - a;
    float d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0.f && d2 <= 0.f) { feature = TF_VERTEX; fi = 0; q = a; return distance2(p, q); }
    V3 bp = p - b;
    float d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0.f && d4 <= d3) { feature = TF_VERTEX; fi = 1; q = b; return distance2(p, q); }
    float vc = d1 * d4 - d3 * d2;
    if (vc <= 0 && d1 >= 0.f && d3 <= 0.f) { feature = TF_EDGE; fi = 2; q = a + d1 / (d1 - d3) * ab; return distance2(p, q); }
    V3 cp = p - c;
    float d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0.f && d5 <= d6) { feature = TF_VERTEX; fi = 2; q = c; return distance2(p, q); }
    float va = d3 * d6 - d5 * d4;
    if (va <= 0 && d4 >= d3 && d5 >= d6) { feature = TF_EDGE; fi = 0; q = b + (d4 - d3) / (d4 - d3 + d5 - d6) * (c - b); return distance2(p, q); }
    float vb = d5 * d2 - d1 * d6;
    if (vb <= 0 && d2 >= 0.f && d6 <= 0.f) { feature = TF_EDGE; fi = 1; q = c + d2 / (d2 - d6) * ac; return distance2(p, q); }
    feature = TF_FACE;
    float denom = va + vb + vc;
    float u = va / denom, v = vb / denom, w = 1 - u - v;
    q = u * a + v * b + w * c;
    return distance2(p, q);
}

// GeomUtil.cpp:540-581
__device__ inline float sqrDistLineSegment(V3 p, V3 dir, V3 a, V3 b, float& t, V3& q, int& vflag) {
    V3 ab = b - a;
    float v1v2 = dot(dir, ab), v2v2 = dot(ab, ab);
    V3 r = p - a;
    float rv1 = dot(r, dir), rv2 = dot(r, ab);
    float denom = (v1v2 * v1v2 - v2v2);
    if (fabsf(denom) <= 1e-6f) { q = a; t = -rv1; vflag = 0; V3 d = p + t * dir - a; return dot(d, d); }
    float s = (rv1 * v1v2 - rv2) / denom;
    if (s <= 0.f) { q = a; t = -rv1; vflag = 1; V3 d = p + t * dir - a; return dot(d, d); }
    if (s >= 1.f) { q = b; t = -dot(p - b, dir); vflag = 2; V3 d = p + t * dir - b; return dot(d, d); }
    q = a + s * ab;
    t = s * v1v2 - rv1;
    vflag = 0;
    V3 d = p + t * dir - q;
    return dot(d, d);
}

// GeomUtil.cpp:583-647
__device__ inline float sqrDistLineTriangle(V3 p, V3 dir, V3 a, V3 b, V3 c, float& t, V3& q, int& feature, int& fi) {
    V3 e0 = b - a, e1 = c - a;
    float det = determinant(m3cols(e0, e1, -dir));
    if (fabsf(det) > 1e-6f) {
        V3 diff = p - a;
        float invDet = 1 / det;
        float u = invDet * determinant(m3cols(diff, e1, -dir));
        float v = invDet * determinant(m3cols(e0, diff, -dir));
        float w = 1 - u - v;
        if (u >= 0.f && v >= 0.f && w >= 0.f) {
            t = invDet * determinant(m3cols(e0, e1, diff));
            q = a + u * e0 + v * e1;
            feature = TF_FACE;
            return 0;
        }
    }
    float t1;
    V3 q1;
    int vf, vf1;
    fi = 2;
    float dist = sqrDistLineSegment(p, dir, a, b, t, q, vf);
    float dist1 = sqrDistLineSegment(p, dir, b, c, t1, q1, vf1);
    if (dist1 < dist) { fi = 0; t = t1; q = q1; vf = vf1; dist = dist1; }
    dist1 = sqrDistLineSegment(p, dir, c, a, t1, q1, vf1);
    if (dist1 < dist) { fi = 1; t = t1; q = q1; vf = vf1; dist = dist1; }
    if (vf) { feature = TF_VERTEX; fi = (fi + vf) % 3; }
    else feature = TF_EDGE;
    return dist;
}

// GeomUtil.cpp:649-660
__device__ inline float sqrDistSegmentTriangle(V3 p, V3 dir, float mn, float mx, V3 a, V3 b, V3 c, float& t, V3& q,
                                               int& feature, int& fi) {
    float sq = sqrDistLineTriangle(p, dir, a, b, c, t, q, feature, fi);
    if (t < mn) { t = mn; sq = sqrDistPointTriangle(p + dir * t, a, b, c, q, feature, fi); }
    else if (t > mx) { t = mx; sq = sqrDistPointTriangle(p + dir * t, a, b, c, q, feature, fi); }
    return sq;
}

// GeomUtil.cpp:662-665
__device__ inline float distanceAABBPlane(V3 he, V3 n, float d) {
    float r = he.x * fabsf(n.x) + he.y * fabsf(n.y) + he.z * fabsf(n.z);
    return fabsf(d) - r;
}

// ---------------------------------------------------------------- clipping (Clipping.cpp)

__device__ __forceinline__ bool isInside(V2 p, V2 a, V2 b) { return (b.y - a.y) * (p.x - a.x) - (b.x - a.x) * (p.y - a.y) > 0; }

__device__ __forceinline__ V2 intersection(V2 a1, V2 b1, V2 a2, V2 b2) {
    V2 r1 = b1 - a1, r2 = b2 - a2;
    float t = det2(a1 - a2, r2) / det2(-r1, r2);
    return a1 + t * r1;
}

// Clipping.cpp:20-45, in place with a bounded output buffer
__device__ inline void clipEdge(Poly& poly, V2 a, V2 b, int* err) {
    V2 np[kMaxPoly];
    int nc = 0;
    int n = poly.n;
    for (int i = 0; i < n; ++i) {
        int j = (i + 1) % n;
        bool iin = isInside(poly.p[i], a, b), jin = isInside(poly.p[j], a, b);
        if (nc + 2 > kMaxPoly) { raise_err(err, ERR_POLY_CAPACITY); break; }
        if (iin && jin) np[nc++] = poly.p[j];
        else if (iin) np[nc++] = intersection(poly.p[i], poly.p[j], a, b);
        else if (jin) { np[nc++] = intersection(poly.p[i], poly.p[j], a, b); np[nc++] = poly.p[j]; }
    }
    poly.n = nc;
    for (int i = 0; i < nc; ++i) poly.p[i] = np[i];
}

__device__ inline void suthHodgClip(Poly& poly, const V2* clip, int nclip, int* err) {
    for (int i = 0; i < nclip; ++i) clipEdge(poly, clip[i], clip[(i + 1) % nclip], err);
}

// Clipping.cpp:54-71
__device__ inline bool clipLine(V2& p0, V2& p1, const V2* clip, int n) {
    for (int i = 0; i < n; ++i) {
        int j = (i + 1) % n;
        bool in0 = isInside(p0, clip[i], clip[j]), in1 = isInside(p1, clip[i], clip[j]);
        if (in0 && in1) continue;
        if (in0) p1 = intersection(p0, p1, clip[i], clip[j]);
        else if (in1) p0 = intersection(p0, p1, clip[i], clip[j]);
        else return false;
    }
    return true;
}

// ---------------------------------------------------------------- manifold reduction (ContactsUtil.cpp)

__device__ inline void reduce4(const V3* pts, int n, int cx, int cy, int& i1, int& i2, int& i3) {
    float maxDistance = 0; i1 = 0;
    for (int i = 0; i < n; ++i) {
        float d = distance2(pts[0], pts[i]);
        if (d > maxDistance) { maxDistance = d; i1 = i; }
    }
    float maxArea = 0; i2 = 0;
    for (int i = 0; i < n; ++i) {
        V3 ca = pts[0] - pts[i], cb = pts[i1] - pts[i];
        float area = det2({at(ca, cx), at(ca, cy)}, {at(cb, cx), at(cb, cy)});
        if (area > maxArea) { maxArea = area; i2 = i; }
    }
    float minArea = 0; i3 = 0;
    for (int i = 0; i < n; ++i) {
        V3 da = pts[0] - pts[i], db = pts[i1] - pts[i];
        float area = det2({at(da, cx), at(da, cy)}, {at(db, cx), at(db, cy)});
        if (area < minArea) { minArea = area; i3 = i; }
    }
}

// ContactsUtil.cpp:9-107
__device__ inline void contactsPolygonBoxFace(V3 boxCenter, const M3& basis, int boxAxis, int boxAxisSign, V3 he,
                                              V3 incO, V3 incN, const Poly& poly, int cx, int cy, ContactPoint* cp, int& np) {
    V3 pen[kMaxPoly];
    int n = 0;
    const float eps = 1e-4f;
    for (int k = 0; k < poly.n; ++k) {
        V3 p3 = {0, 0, 0};
        at(p3, cx) = poly.p[k].x;
        at(p3, cy) = poly.p[k].y;
        V3 dir = {0, 0, 0};
        at(dir, boxAxis) = (float)boxAxisSign;
        float distance = dot((incO - p3), incN) / dot(dir, incN);
        if (distance < at(he, boxAxis) + eps) {
            at(p3, boxAxis) = boxAxisSign * distance;
            pen[n++] = p3;
        }
    }
    auto emit = [&](int slot, int idx) {
        V3 a = pen[idx];
        at(a, boxAxis) = boxAxisSign * at(he, boxAxis);
        cp[slot] = {boxCenter + mv(basis, a), boxCenter + mv(basis, pen[idx])};
    };
    if (n > 4) {
        int i1, i2, i3;
        emit(0, 0);
        reduce4(pen, n, cx, cy, i1, i2, i3);
        emit(1, i1); emit(2, i2); emit(3, i3);
        np = 4;
    } else {
        for (int i = 0; i < n; ++i) emit(i, i);
        np = n;
    }
}

// ContactsUtil.cpp:109-204
__device__ inline void contactsPolygonPolygonFace(V3 refPos, const M3& r2w, V3 refO, V3 refN, V3 incO, V3 incN,
                                                  const Poly& poly, int cx, int cy, ContactPoint* cp, int& np) {
    V3 pen[kMaxPoly];
    int n = 0;
    const float eps = 1e-4f;
    float dRef = dot(refO, refN);
    for (int k = 0; k < poly.n; ++k) {
        V3 p3 = {poly.p[k].y, 0, poly.p[k].x};
        V3 dir = {0, 1, 0};
        float distance = dot((incO - p3), incN) / dot(dir, incN);
        if (distance < dRef + eps) {
            p3.y = distance;
            pen[n++] = p3;
        }
    }
    auto emit = [&](int slot, int idx) {
        V3 a = pen[idx];
        a.y = dRef;
        cp[slot] = {refPos + mv(r2w, a), refPos + mv(r2w, pen[idx])};
    };
    if (n > 4) {
        int i1, i2, i3;
        emit(0, 0);
        reduce4(pen, n, cx, cy, i1, i2, i3);
        emit(1, i1); emit(2, i2); emit(3, i3);
        np = 4;
    } else {
        for (int i = 0; i < n; ++i) emit(i, i);
        np = n;
    }
}

}  // namespace psx
