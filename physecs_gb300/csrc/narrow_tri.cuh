// narrow_tri.cuh — device triangle-mesh midphase and contacts.
//
// Restates Physecs src/TriangleMesh.cpp:166-192 (DFS overlap query, left child
// first) and src/CollisionTriangleMesh.cpp:44-956 (per-triangle tests, face
// contacts in reverse candidate order, then edge / vertex contacts by ascending
// distance with voided-vertex suppression).  The distance sort is a stable
// insertion sort, which is what libstdc++'s std::sort does for the 16 or fewer
// elements a body meets on one mesh in practice.
#pragma once
#include "narrow_convex.cuh"

namespace psx {

enum { BF_FACE = 0, BF_EDGE = 1, BF_UNKNOWN = 2 };
struct TCI {
    int tri;
    V3 normal, cpBody, cpTri;
    int feature, featureIndex;
    float distance;
    int boxFeature, boxAxis;
};

struct TriView {
    const float4* verts;
    const TriDev* tris;
    const TriNodeDev* nodes;
};

__device__ __forceinline__ V3 tv(const TriView& m, int i) { return ld3(m.verts[i]); }

__device__ __forceinline__ bool intersectsB(const Bounds& a, V3 bmin, V3 bmax) {
    if (a.max.x < bmin.x || a.min.x > bmax.x) return false;
    if (a.max.y < bmin.y || a.min.y > bmax.y) return false;
    if (a.max.z < bmin.z || a.min.z > bmax.z) return false;
    return true;
}

__device__ inline bool sphereTri(V3 pos0, float r0, V3 a, V3 b, V3 c, V3 n, TCI& o) {
    V3 u;
    int f, fi = 0;
    float sq = sqrDistPointTriangle(pos0, a, b, c, u, f, fi);
    if (sq > r0 * r0) return false;
    if (f == TF_FACE) o.normal = -n;
    else {
        V3 nn = u - pos0;
        float len = length(nn);
        if (len) { nn = nn / len; o.normal = nn; }
        else o.normal = -n;
    }
    o.cpBody = pos0 + o.normal * r0;
    o.cpTri = u;
    o.feature = f; o.featureIndex = fi; o.distance = sq;
    return true;
}

__device__ inline bool capsuleTri(V3 pos, Q4 ori, float hh, float r, V3 a, V3 b, V3 c, V3 n, TCI& o) {
    V3 dir = qrot(ori, {0, 1, 0});
    float t = 0;
    V3 u;
    int f, fi = 0;
    float sq = sqrDistSegmentTriangle(pos, dir, -hh, hh, a, b, c, t, u, f, fi);
    if (sq > r * r) return false;
    V3 onSeg = pos + dir * t;
    if (f == TF_FACE) o.normal = -n;
    else {
        V3 nn = u - onSeg;
        float len = length(nn);
        if (len) { nn = nn / len; o.normal = nn; }
        else o.normal = -n;
    }
    o.cpBody = onSeg + o.normal * r;
    o.cpTri = u;
    o.feature = f; o.featureIndex = fi; o.distance = sq;
    return true;
}

__device__ __forceinline__ float sepd(float a0, float a1, float rr) { return fmaxG(-fmaxG(a0, a1), fminG(a0, a1)) - rr; }

// CollisionTriangleMesh.cpp:221-456
__device__ inline bool boxTri(V3 pos, Q4 ori, V3 he, V3 a, V3 b, V3 c, V3 n, TCI& o) {
    float edgeOffset = 0.f;
    const float edgeLimit = 0.999f;
    M3 u = mat3_cast(ori);
    M3 invU = transpose(u);
    V3 v0 = mv(invU, a - pos), v1 = mv(invU, b - pos), v2 = mv(invU, c - pos);
    V3 f0 = v1 - v0, f1 = v2 - v1, f2 = v0 - v2;
    float fl[3] = {edgeLimit * length2(f0), edgeLimit * length2(f1), edgeLimit * length2(f2)};
    float mx = -FLT_MAX;
    float p0, p1, r, d;
#define PSX_EDGE_AXIS(FXX, LIM, TE, AX)                                                 \
    d = sepd(p0, p1, r);                                                                \
    if (d > 0) return false;                                                            \
    if ((FXX) < (LIM) && d > mx) {                                                      \
        mx = d; o.feature = TF_EDGE; o.featureIndex = (TE); o.distance = d;             \
        o.boxFeature = BF_EDGE; o.boxAxis = (AX); edgeOffset = 0.1f;                    \
    }
    p0 = v0.z * f0.y - v0.y * f0.z; p1 = v2.z * f0.y - v2.y * f0.z; r = he.y * fabsf(f0.z) + he.z * fabsf(f0.y);
    PSX_EDGE_AXIS(f0.x * f0.x, fl[0], 2, 0)
    p0 = v0.z * f1.y - v0.y * f1.z; p1 = v1.z * f1.y - v1.y * f1.z; r = he.y * fabsf(f1.z) + he.z * fabsf(f1.y);
    PSX_EDGE_AXIS(f1.x * f1.x, fl[1], 0, 0)
    p0 = v1.z * f2.y - v1.y * f2.z; p1 = v2.z * f2.y - v2.y * f2.z; r = he.y * fabsf(f2.z) + he.z * fabsf(f2.y);
    PSX_EDGE_AXIS(f2.x * f2.x, fl[2], 1, 0)
    p0 = v0.x * f0.z - v0.z * f0.x; p1 = v2.x * f0.z - v2.z * f0.x; r = he.x * fabsf(f0.z) + he.z * fabsf(f0.x);
    PSX_EDGE_AXIS(f0.y * f0.y, fl[0], 2, 1)
    p0 = v0.x * f1.z - v0.z * f1.x; p1 = v1.x * f1.z - v1.z * f1.x; r = he.x * fabsf(f1.z) + he.z * fabsf(f1.x);
    PSX_EDGE_AXIS(f1.y * f1.y, fl[1], 0, 1)
    p0 = v1.x * f2.z - v1.z * f2.x; p1 = v2.x * f2.z - v2.z * f2.x; r = he.x * fabsf(f2.z) + he.z * fabsf(f2.x);
    PSX_EDGE_AXIS(f2.y * f2.y, fl[2], 1, 1)
    p0 = v0.y * f0.x - v0.x * f0.y; p1 = v2.y * f0.x - v2.x * f0.y; r = he.x * fabsf(f0.y) + he.y * fabsf(f0.x);
    PSX_EDGE_AXIS(f0.z * f0.z, fl[0], 2, 2)
    p0 = v0.y * f1.x - v0.x * f1.y; p1 = v1.y * f1.x - v1.x * f1.y; r = he.x * fabsf(f1.y) + he.y * fabsf(f1.x);
    PSX_EDGE_AXIS(f1.z * f1.z, fl[1], 0, 2)
    p0 = v1.y * f2.x - v1.x * f2.y; p1 = v2.y * f2.x - v2.x * f2.y; r = he.x * fabsf(f2.y) + he.y * fabsf(f2.x);
    PSX_EDGE_AXIS(f2.z * f2.z, fl[2], 1, 2)
#undef PSX_EDGE_AXIS
    for (int i = 0; i < 3; ++i) {
        float a0 = at(v0, i), a1 = at(v1, i), a2 = at(v2, i), h = at(he, i);
        d = fmaxG(-fmaxG(fmaxG(a0, a1), a2), fminG(fminG(a0, a1), a2)) - h;
        if (d > 0) return false;
        if (d > mx - edgeOffset) {
            mx = d;
            bool i0 = fabsf(a0) < h, i1 = fabsf(a1) < h, i2 = fabsf(a2) < h;
            if (i0) {
                if (i1) {
                    if (i2) o.feature = TF_FACE;
                    else { o.feature = TF_EDGE; o.featureIndex = 2; }
                } else {
                    if (i2) { o.feature = TF_EDGE; o.featureIndex = 1; }
                    else { o.feature = TF_VERTEX; o.featureIndex = 0; }
                }
            } else {
                if (i1) {
                    if (i2) { o.feature = TF_EDGE; o.featureIndex = 0; }
                    else { o.feature = TF_VERTEX; o.featureIndex = 1; }
                } else { o.feature = TF_VERTEX; o.featureIndex = 2; }
            }
            o.boxFeature = BF_FACE; o.boxAxis = i;
            o.distance = d;
            edgeOffset = 0.f;
        }
    }
    V3 nl = mv(invU, n);
    d = distanceAABBPlane(he, nl, dot(nl, v0));
    if (d > 0) return false;
    if (d > mx - edgeOffset) { o.feature = TF_FACE; o.distance = d; o.boxFeature = BF_UNKNOWN; }
    return true;
}

// CollisionTriangleMesh.cpp:614-699
__device__ inline bool convexTri(const World& w, V3 pos, Q4 ori, int mesh, V3 sc, V3 a, V3 b, V3 c, V3 cen, TCI& o,
                                 Polytope& poly, int* err) {
    Support s0 = convexSupport(w, pos, ori, mesh, sc);
    Support s1; s1.kind = 4; s1.a = a; s1.b = b; s1.c = c;
    GjkSimplex s;
    if (!gjk(s0, s1, cen - pos, s)) return false;
    o.normal = epa(s0, s1, s, o.cpBody, o.cpTri, poly, err);
    o.distance = dot(o.cpTri - o.cpBody, o.normal);
    V3 v0 = b - a, v1 = c - a, v2 = o.cpTri - a;
    float d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1), d20 = dot(v2, v0), d21 = dot(v2, v1);
    float denom = d00 * d11 - d01 * d01;
    float u, v, ww;
    if (denom) {
        v = (d20 * d11 - d21 * d01) / denom;
        ww = (d00 * d21 - d01 * d20) / denom;
        u = 1.0f - v - ww;
    } else {
        ww = 0;
        if (d00) { v = d20 / d00; u = 1.0f - v; }
        else { v = 0; u = 1.0; }
    }
    float eps = 1e-4;
    if (u < eps) {
        if (v < eps) { o.feature = TF_VERTEX; o.featureIndex = 2; }
        else if (ww < eps) { o.feature = TF_VERTEX; o.featureIndex = 1; }
        else { o.feature = TF_EDGE; o.featureIndex = 0; }
    } else {
        if (v < eps) {
            if (ww < eps) { o.feature = TF_VERTEX; o.featureIndex = 0; }
            else { o.feature = TF_EDGE; o.featureIndex = 1; }
        } else if (ww < eps) {
            if (u < eps) { o.feature = TF_VERTEX; o.featureIndex = 0; }
            else { o.feature = TF_EDGE; o.featureIndex = 2; }
        } else o.feature = TF_FACE;
    }
    return true;
}

// ---------------------------------------------------------------- contact generators

struct ManOut {
    ManifoldL* m;
    int n, cap;
    int* err;
    __device__ ManifoldL* push() {
        if (n >= cap) { raise_err(err, ERR_TRI_CAPACITY); return nullptr; }
        ManifoldL* r = &m[n++];
        r->numPoints = 0; r->triangleIndex = -1;
        return r;
    }
};

__device__ inline void sphereTriContacts(V3 pos1, Q4 or1, const TCI& c, ManOut& out) {
    ManifoldL* mf = out.push();
    if (!mf) return;
    mf->normal = qrot(or1, c.normal);
    mf->numPoints = 1;
    mf->points[0] = {pos1 + qrot(or1, c.cpBody), pos1 + qrot(or1, c.cpTri)};
    mf->triangleIndex = c.tri;
}

__device__ inline void triFrame(const TriView& mesh, const TriDev& tri, bool normalizeN, V3& refO, V3& u1, M3& m2r, V2* clip) {
    refO = ld3(tri.centroid);
    V3 u0 = normalize(tv(mesh, tri.idx.x) - refO);
    u1 = normalizeN ? normalize(ld3(tri.normal)) : ld3(tri.normal);
    V3 u2 = cross(u0, u1);
    m2r = transpose(m3cols(u0, u1, u2));
    int id[3] = {tri.idx.x, tri.idx.y, tri.idx.z};
    for (int i = 0; i < 3; i++) {
        V3 v = mv(m2r, tv(mesh, id[i]));
        clip[3 - i - 1] = {v.z, v.x};
    }
}

__device__ inline void capsuleTriFace(V3 pos0, Q4 or0, float hh0, float r0, V3 pos1, Q4 or1, const TriView& mesh, const TCI& c,
                                      ManOut& out) {
    V3 dir = qrot(or0, {0, 1, 0});
    V3 p0l = pos0 - dir * hh0, p1l = pos0 + dir * hh0;
    const TriDev tri = mesh.tris[c.tri];
    V3 refO, u1;
    M3 m2r;
    V2 clip[3];
    triFrame(mesh, tri, true, refO, u1, m2r, clip);
    const int fa = 1, cx = 2, cy = 0;
    V3 p0R = mv(m2r, p0l), p1R = mv(m2r, p1l);
    V2 l0 = {at(p0R, cx), at(p0R, cy)}, l1 = {at(p1R, cx), at(p1R, cy)};
    if (!clipLine(l0, l1, clip, 3)) return;
    M3 m2w = mat3_cast(or1);
    M3 r2w = mm(m2w, transpose(m2r));
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
    at(p0, fa) -= r0;
    at(p1, fa) -= r0;
    ManifoldL* res = out.push();
    if (!res) return;
    int n = 0;
    res->triangleIndex = c.tri;
    res->normal = mv(m2w, c.normal);
    if (at(p0, fa) < dPlane) {
        at(p0, cx) = l0.x; at(p0, cy) = l0.y;
        V3 of = p0; at(of, fa) = dPlane;
        res->points[n++] = {pos1 + mv(r2w, p0), pos1 + mv(r2w, of)};
    }
    if (at(p1, fa) < dPlane) {
        at(p1, cx) = l1.x; at(p1, cy) = l1.y;
        V3 of = p1; at(of, fa) = dPlane;
        res->points[n++] = {pos1 + mv(r2w, p1), pos1 + mv(r2w, of)};
    }
    if (!n) {
        n = 1;
        res->points[0] = {pos1 + mv(m2w, c.cpBody), pos1 + mv(m2w, c.cpTri)};
    }
    res->numPoints = n;
}

__device__ inline void boxTriFace(V3 boxPos, Q4 boxOr, V3 he, V3 meshPos, Q4 meshOr, const TriView& mesh, const TCI& c,
                                  ManOut& out) {
    M3 bb = mat3_cast(boxOr);
    const TriDev tri = mesh.tris[c.tri];
    V3 tn = ld3(tri.normal);
    V3 refO, u1;
    M3 m2r;
    V2 clip[3];
    triFrame(mesh, tri, true, refO, u1, m2r, clip);
    const int cx = 2, cy = 0;
    int incAxis = 0;
    float incSign = 1;
    if (c.boxFeature == BF_FACE) {
        incAxis = c.boxAxis;
        incSign = dot(tn, bb.c[incAxis]) > 0 ? -1 : 1;
    } else {
        float maxDot = 0;
        for (int i = 0; i < 3; ++i) {
            float d = dot(tn, bb.c[i]);
            float ad = fabsf(d);
            if (ad > maxDot) { maxDot = ad; incAxis = i; incSign = d > 0 ? -1 : 1; }
        }
    }
    int a1 = (incAxis + 1) % 3, a2 = (incAxis + 2) % 3;
    V3 incO = mv(m2r, boxPos + bb.c[incAxis] * at(he, incAxis) * incSign);
    V3 e1 = bb.c[a1] * at(he, a1), e2 = bb.c[a2] * at(he, a2);
    V3 ne1 = -bb.c[a1] * at(he, a1);
    V3 q0 = incO + mv(m2r, e1 + e2), q1 = incO + mv(m2r, ne1 + e2), q2 = incO + mv(m2r, ne1 - e2), q3 = incO + mv(m2r, e1 - e2);
    Poly poly;
    poly.n = 4;
    poly.p[0] = {at(q0, cx), at(q0, cy)};
    poly.p[1] = {at(q1, cx), at(q1, cy)};
    poly.p[2] = {at(q2, cx), at(q2, cy)};
    poly.p[3] = {at(q3, cx), at(q3, cy)};
    suthHodgClip(poly, clip, 3, out.err);
    V3 incN = mv(m2r, bb.c[incAxis]);
    M3 m2w = mat3_cast(meshOr);
    M3 r2w = mm(m2w, transpose(m2r));
    ManifoldL* mf = out.push();
    if (!mf) return;
    mf->normal = -mv(m2w, tn);
    mf->triangleIndex = c.tri;
    contactsPolygonPolygonFace(meshPos, r2w, refO, u1, incO, incN, poly, cx, cy, mf->points, mf->numPoints);
    for (int i = 0; i < mf->numPoints; ++i) mf->points[i] = {mf->points[i].p1, mf->points[i].p0};
}

__device__ inline void boxFaceTri(V3 boxPos, Q4 boxOr, V3 he, V3 meshPos, Q4 meshOr, const TriView& mesh, const TCI& c,
                                  ManOut& out) {
    M3 bb = mat3_cast(boxOr);
    const TriDev tri = mesh.tris[c.tri];
    M3 m2b = transpose(bb);
    int ra = c.boxAxis;
    V3 cen = ld3(tri.centroid);
    float rs = dot(bb.c[ra], cen - boxPos) < 0 ? -1 : 1;
    int cx = (ra + 1) % 3, cy = (ra + 2) % 3;
    Poly poly;
    poly.n = 3;
    int id[3] = {tri.idx.x, tri.idx.y, tri.idx.z};
    for (int i = 0; i < 3; ++i) {
        V3 v = mv(m2b, tv(mesh, id[i]) - boxPos);
        poly.p[i] = {at(v, cx), at(v, cy)};
    }
    V2 clip[4] = {{at(he, cx), at(he, cy)}, {at(he, cx), -at(he, cy)}, {-at(he, cx), -at(he, cy)}, {-at(he, cx), at(he, cy)}};
    suthHodgClip(poly, clip, 4, out.err);
    V3 incO = mv(m2b, cen - boxPos);
    V3 incN = mv(m2b, ld3(tri.normal));
    M3 m2w = mat3_cast(meshOr);
    ManifoldL* mf = out.push();
    if (!mf) return;
    mf->normal = mv(m2w, rs * bb.c[ra]);
    mf->triangleIndex = c.tri;
    contactsPolygonBoxFace(boxPos, bb, ra, (int)rs, he, incO, incN, poly, cx, cy, mf->points, mf->numPoints);
    for (int i = 0; i < mf->numPoints; ++i) {
        mf->points[i].p0 = meshPos + mv(m2w, mf->points[i].p0);
        mf->points[i].p1 = meshPos + mv(m2w, mf->points[i].p1);
    }
}

__device__ inline void boxEdgeTriEdge(V3 boxPos, Q4 boxOr, V3 he, V3 meshPos, Q4 meshOr, const TriView& mesh, const TCI& c,
                                      ManOut& out) {
    M3 bb = mat3_cast(boxOr);
    const TriDev tri = mesh.tris[c.tri];
    int ba = c.boxAxis, te = c.featureIndex;
    int id[3] = {tri.idx.x, tri.idx.y, tri.idx.z};
    V3 ta = tv(mesh, id[(te + 1) % 3]);
    V3 tb = tv(mesh, id[(te + 2) % 3]);
    V3 tEdge = tb - ta;
    V3 axis = cross(bb.c[ba], tEdge);
    M3 m2w = mat3_cast(meshOr);
    ManifoldL* mf = out.push();
    if (!mf) return;
    mf->normal = mv(m2w, normalize(dot(axis, ld3(tri.centroid) - boxPos) < 0 ? -axis : axis));
    mf->numPoints = 1;
    mf->triangleIndex = c.tri;
    V3 sb = v3s(-1);
    at(sb, (ba + 1) % 3) = dot(bb.c[(ba + 1) % 3], mf->normal) < 0 ? -1 : 1;
    at(sb, (ba + 2) % 3) = dot(bb.c[(ba + 2) % 3], mf->normal) < 0 ? -1 : 1;
    V3 bA = boxPos + sb.x * he.x * bb.c[0] + sb.y * he.y * bb.c[1] + sb.z * he.z * bb.c[2];
    V3 bEdge = bb.c[ba] * at(he, ba) * 2.f;
    V3 p0, p1;
    closestPointsBetweenSegmentsV(bA, bEdge, ta, tEdge, p0, p1);
    mf->points[0] = {meshPos + mv(m2w, p0), meshPos + mv(m2w, p1)};
}

__device__ inline void convexTriFace(const World& w, V3 cPos, Q4 cOr, int cmesh, V3 sc, V3 meshPos, Q4 meshOr,
                                     const TriView& mesh, const TCI& c, ManOut& out) {
    const TriDev tri = mesh.tris[c.tri];
    V3 tn = ld3(tri.normal);
    V3 refO, u1;
    M3 m2r;
    V2 clip[3];
    triFrame(mesh, tri, false, refO, u1, m2r, clip);
    const int cx = 2, cy = 0;
    ConvexView C = convexView(w, cmesh);
    int fi = 0;
    float minDot = 0;
    for (int i = 0; i < C.face_count; ++i) {
        float d = dot(tn, normalize(qrot(cOr, faceNormal(w, C.face_start + i) / sc)));
        if (d < minDot) { minDot = d; fi = i; }
    }
    int F = C.face_start + fi;
    int is = w.face_idx_start[F], ie = w.face_idx_start[F + 1];
    Poly poly;
    poly.n = min(ie - is, kMaxPoly);
    for (int i = 0; i < poly.n; ++i) {
        V3 v = mv(m2r, cPos + qrot(cOr, sc * ld3(C.verts[w.face_idx[is + i]])));
        poly.p[i] = {at(v, cx), at(v, cy)};
    }
    suthHodgClip(poly, clip, 3, out.err);
    V3 incO = mv(m2r, cPos + qrot(cOr, sc * faceCentroid(w, F)));
    V3 incN = mv(m2r, qrot(cOr, normalize(faceNormal(w, F) / sc)));
    M3 m2w = mat3_cast(meshOr);
    M3 r2w = mm(m2w, transpose(m2r));
    ManifoldL* mf = out.push();
    if (!mf) return;
    mf->normal = -mv(m2w, tn);
    mf->triangleIndex = c.tri;
    contactsPolygonPolygonFace(meshPos, r2w, refO, u1, incO, incN, poly, cx, cy, mf->points, mf->numPoints);
    for (int i = 0; i < mf->numPoints; ++i) mf->points[i] = {mf->points[i].p1, mf->points[i].p0};
}

__device__ inline void convexFaceTri(const World& w, V3 cPos, Q4 cOr, int cmesh, V3 sc, V3 meshPos, Q4 meshOr,
                                     const TriView& mesh, const TCI& c, ManOut& out) {
    const TriDev tri = mesh.tris[c.tri];
    M3 c2m = mat3_cast(cOr);
    M3 m2c = transpose(c2m);
    ConvexView C = convexView(w, cmesh);
    int fi = 0;
    float maxDot = 0;
    for (int i = 0; i < C.face_count; ++i) {
        float d = dot(c.normal, normalize(qrot(cOr, faceNormal(w, C.face_start + i) / sc)));
        if (d > maxDot) { maxDot = d; fi = i; }
    }
    int F = C.face_start + fi;
    int is = w.face_idx_start[F], ie = w.face_idx_start[F + 1];
    V3 refO = sc * faceCentroid(w, F);
    V3 u0 = normalize(sc * ld3(C.verts[w.face_idx[is]]) - refO);
    V3 u1 = normalize(faceNormal(w, F) / sc);
    V3 u2 = cross(u0, u1);
    M3 c2r = transpose(m3cols(u0, u1, u2));
    M3 m2r = mm(c2r, m2c);
    const int cx = 2, cy = 0;
    V2 clip[kMaxPoly];
    int nc = min(ie - is, kMaxPoly);
    for (int i = 0; i < nc; ++i) {
        V3 v = mv(c2r, sc * ld3(C.verts[w.face_idx[is + i]]));
        clip[i] = {at(v, cx), at(v, cy)};
    }
    Poly poly;
    poly.n = 3;
    int id[3] = {tri.idx.x, tri.idx.y, tri.idx.z};
    for (int i = 0; i < 3; ++i) {
        V3 v = mv(m2r, tv(mesh, id[i]) - cPos);
        poly.p[i] = {at(v, cx), at(v, cy)};
    }
    suthHodgClip(poly, clip, nc, out.err);
    V3 incO = mv(m2r, ld3(tri.centroid) - cPos);
    V3 incN = mv(m2r, ld3(tri.normal));
    M3 m2w = mat3_cast(meshOr);
    M3 r2m = transpose(m2r);
    ManifoldL* mf = out.push();
    if (!mf) return;
    mf->triangleIndex = c.tri;
    contactsPolygonPolygonFace(cPos, r2m, refO, u1, incO, incN, poly, cx, cy, mf->points, mf->numPoints);
    if (mf->numPoints) {
        for (int i = 0; i < mf->numPoints; ++i) {
            mf->points[i].p0 = meshPos + mv(m2w, mf->points[i].p0);
            mf->points[i].p1 = meshPos + mv(m2w, mf->points[i].p1);
        }
        mf->normal = mv(mm(m2w, c2m), u1);
    } else {
        mf->normal = mv(m2w, c.normal);
        mf->numPoints = 1;
        mf->points[0] = {meshPos + mv(m2w, c.cpBody), meshPos + mv(m2w, c.cpTri)};
    }
}

__device__ __forceinline__ bool inSet(const uint32_t* s, int n, uint32_t v) {
    for (int i = 0; i < n; ++i) if (s[i] == v) return true;
    return false;
}

// collisionTriangleMesh (CollisionTriangleMesh.cpp:882-956): body (g0 at pos0/or0) against mesh at pos1/or1.
// Writes manifolds in the reference's emission order; returns whether any triangle was hit.
__device__ inline bool collideTriMesh(const World& w, V3 pos0, Q4 or0, const GeomD& g0, V3 pos1, Q4 or1, int meshId,
                                      ManOut& out, TCI* contacts, Polytope& epaPoly) {
    TriMeshDev tm = w.trimesh[meshId];
    TriView mesh{w.tri_verts + tm.vert_start, w.tris + tm.tri_start, w.tri_nodes + tm.node_start};
    Q4 inv1 = qinverse(or1);
    V3 lp = qrot(inv1, pos0 - pos1);
    Q4 lo = qmul(inv1, or0);
    Bounds lb = getBounds(w, lp, lo, g0);
    // midphase: depth-first BVH query, right child pushed first (TriangleMesh.cpp:166-192)
    int stack[64];
    int sp = 0;
    stack[sp++] = 0;
    int nc = 0;
    while (sp) {
        int ni = stack[--sp];
        TriNodeDev node = mesh.nodes[ni];
        if (!intersectsB(lb, ld3(node.bmin), ld3(node.bmax))) continue;
        int triCount = __float_as_int(node.bmin.w), index = __float_as_int(node.bmax.w);
        if (triCount) {
            for (int i = 0; i < triCount; ++i) {
                int ti = index + i;
                const TriDev tri = mesh.tris[ti];
                V3 a = tv(mesh, tri.idx.x), b = tv(mesh, tri.idx.y), c = tv(mesh, tri.idx.z);
                TCI ci;
                ci.boxFeature = BF_FACE; ci.boxAxis = 0; ci.featureIndex = 0; ci.feature = TF_FACE;
                bool hit = false;
                switch (g0.type) {
                    case G_SPHERE: hit = sphereTri(lp, g0.p[0], a, b, c, ld3(tri.normal), ci); break;
                    case G_CAPSULE: hit = capsuleTri(lp, lo, g0.p[0], g0.p[1], a, b, c, ld3(tri.normal), ci); break;
                    case G_BOX: hit = boxTri(lp, lo, gv(g0), a, b, c, ld3(tri.normal), ci); break;
                    case G_CONVEX: hit = convexTri(w, lp, lo, g0.mesh, gv(g0), a, b, c, ld3(tri.centroid), ci, epaPoly, out.err); break;
                    default: break;
                }
                if (hit) {
                    if (nc < kTriCandidates) { ci.tri = ti; contacts[nc++] = ci; }
                    else raise_err(out.err, ERR_TRI_CAPACITY);
                }
            }
        } else {
            if (sp + 2 > 64) { raise_err(out.err, ERR_STACK_CAPACITY); break; }
            stack[sp++] = index + 1;
            stack[sp++] = index;
        }
    }
    if (nc == 0) return false;
    uint32_t voided[3 * kTriCandidates];
    int nvoid = 0;
    V3 he = gv(g0);
    for (int i = nc - 1; i >= 0; i--) {
        TCI c = contacts[i];
        if (c.feature == TF_FACE) {
            const TriDev tri = mesh.tris[c.tri];
            uint32_t id[3] = {(uint32_t)tri.idx.x, (uint32_t)tri.idx.y, (uint32_t)tri.idx.z};
            for (int k = 0; k < 3; ++k) if (!inSet(voided, nvoid, id[k])) voided[nvoid++] = id[k];
            switch (g0.type) {
                case G_SPHERE: sphereTriContacts(pos1, or1, c, out); break;
                case G_CAPSULE: capsuleTriFace(lp, lo, g0.p[0], g0.p[1], pos1, or1, mesh, c, out); break;
                case G_BOX: boxTriFace(lp, lo, he, pos1, or1, mesh, c, out); break;
                case G_CONVEX: convexTriFace(w, lp, lo, g0.mesh, he, pos1, or1, mesh, c, out); break;
            }
            contacts[i] = contacts[nc - 1];
            contacts[nc - 1] = c;
            --nc;
        }
    }
    // stable insertion sort by distance
    for (int i = 1; i < nc; ++i) {
        TCI v = contacts[i];
        int j = i;
        while (j > 0 && v.distance < contacts[j - 1].distance) { contacts[j] = contacts[j - 1]; --j; }
        contacts[j] = v;
    }
    for (int i = 0; i < nc; ++i) {
        const TCI c = contacts[i];
        const TriDev tri = mesh.tris[c.tri];
        uint32_t id[3] = {(uint32_t)tri.idx.x, (uint32_t)tri.idx.y, (uint32_t)tri.idx.z};
        if (c.feature == TF_EDGE) {
            if (inSet(voided, nvoid, id[(c.featureIndex + 1) % 3]) && inSet(voided, nvoid, id[(c.featureIndex + 2) % 3])) continue;
            switch (g0.type) {
                case G_SPHERE: case G_CAPSULE: sphereTriContacts(pos1, or1, c, out); break;
                case G_BOX:
                    if (c.boxFeature == BF_FACE) boxFaceTri(lp, lo, he, pos1, or1, mesh, c, out);
                    else boxEdgeTriEdge(lp, lo, he, pos1, or1, mesh, c, out);
                    break;
                case G_CONVEX: convexFaceTri(w, lp, lo, g0.mesh, he, pos1, or1, mesh, c, out); break;
            }
        } else if (c.feature == TF_VERTEX) {
            if (inSet(voided, nvoid, id[c.featureIndex])) continue;
            switch (g0.type) {
                case G_SPHERE: case G_CAPSULE: sphereTriContacts(pos1, or1, c, out); break;
                case G_BOX: boxFaceTri(lp, lo, he, pos1, or1, mesh, c, out); break;
                case G_CONVEX: convexFaceTri(w, lp, lo, g0.mesh, he, pos1, or1, mesh, c, out); break;
            }
        }
        for (int k = 0; k < 3; ++k) if (!inSet(voided, nvoid, id[k])) voided[nvoid++] = id[k];
    }
    return true;
}

}  // namespace psx
