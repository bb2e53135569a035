/*
 * collide_tri.cpp — triangle-mesh BVH, midphase and contacts of the CPU oracle.
 * ORACLE (test infrastructure only; see omath.h).
 *
 * Restates src/TriangleMesh.cpp:7-192 (binned SAH build with 6 buckets, DFS
 * overlap query) and src/CollisionTriangleMesh.cpp:44-956 (per-triangle tests,
 * face contacts first in reverse order, then edge / vertex contacts sorted by
 * distance with voided-vertex suppression).
 */
#include "collide_util.h"
#include <algorithm>
#include <unordered_set>

namespace orc {

static Bounds bunion(const Bounds& a, const Bounds& b) {
    return {{fminG(a.min.x, b.min.x), fminG(a.min.y, b.min.y), fminG(a.min.z, b.min.z)},
            {fmaxG(a.max.x, b.max.x), fmaxG(a.max.y, b.max.y), fmaxG(a.max.z, b.max.z)}};
}
static float barea(const Bounds& b) {
    V3 d = b.max - b.min;
    return 2 * (d.x * d.y + d.y * d.z + d.z * d.x);
}
static bool intersects(const Bounds& a, const Bounds& b) {
    if (a.max.x < b.min.x || a.min.x > b.max.x) return false;
    if (a.max.y < b.min.y || a.min.y > b.max.y) return false;
    if (a.max.z < b.min.z || a.min.z > b.max.z) return false;
    return true;
}

namespace {
constexpr int kBuckets = 6;
struct Builder {
    TriangleMesh& m;
    void updateNodeBounds(int id) {
        Bounds b{v3s(FLT_MAX), v3s(-FLT_MAX)};
        TriNode& n = m.bvh[id];
        for (int i = 0; i < n.triCount; ++i) b = bunion(b, m.triangles[n.index + i].bounds);
        n.bounds = b;
    }
    bool fill(int id, int axis, Bounds* bb, int* bc) {
        TriNode& n = m.bvh[id];
        for (int i = 0; i < kBuckets; ++i) { bb[i] = {v3s(FLT_MAX), v3s(-FLT_MAX)}; bc[i] = 0; }
        float s = at(n.bounds.min, axis), e = at(n.bounds.max, axis);
        float len = e - s;
        if (!len) return false;
        for (int i = 0; i < n.triCount; ++i) {
            const Triangle& t = m.triangles[n.index + i];
            int bi = std::min(kBuckets - 1, (int)((at(t.centroid, axis) - s) / len * kBuckets));
            bb[bi] = bunion(bb[bi], t.bounds);
            bc[bi]++;
        }
        return true;
    }
    static bool evaluate(int split, const Bounds* bb, const int* bc, float& cost, Bounds& L, Bounds& R, int& cl, int& cr) {
        L = {v3s(FLT_MAX), v3s(-FLT_MAX)};
        R = {v3s(FLT_MAX), v3s(-FLT_MAX)};
        cl = cr = 0;
        for (int i = 0; i < kBuckets; ++i) {
            if (i < split) { L = bunion(L, bb[i]); cl += bc[i]; }
            else { R = bunion(R, bb[i]); cr += bc[i]; }
        }
        if (!cl || !cr) return false;
        cost = cl * barea(L) + cr * barea(R);
        return true;
    }
    bool choose(int id, int& axisOut, int& splitOut, Bounds& L, Bounds& R, int& cl, int& cr) {
        float best = FLT_MAX;
        for (int axis = 0; axis < 3; ++axis) {
            Bounds bb[kBuckets];
            int bc[kBuckets];
            if (!fill(id, axis, bb, bc)) continue;
            for (int i = 1; i < kBuckets; ++i) {
                float cost;
                Bounds l, r;
                int a = 0, b = 0;
                if (evaluate(i, bb, bc, cost, l, r, a, b) && cost < best) {
                    best = cost; axisOut = axis; splitOut = i; L = l; R = r; cl = a; cr = b;
                }
            }
        }
        return cl && cr;
    }
    void subdivide(int id) {
        int axis = 0, split = 0, cl = 0, cr = 0;
        Bounds L, R;
        if (!choose(id, axis, split, L, R, cl, cr)) return;
        TriNode n = m.bvh[id];
        float s = at(n.bounds.min, axis), e = at(n.bounds.max, axis);
        float len = e - s;
        int i = n.index, j = i + n.triCount - 1;
        while (i <= j) {
            int bi = (int)((at(m.triangles[i].centroid, axis) - s) / len * kBuckets);
            if (bi < split) ++i;
            else std::swap(m.triangles[i], m.triangles[j--]);
        }
        m.bvh.push_back({L, cl, n.index});
        m.bvh.push_back({R, cr, i});
        m.bvh[id].triCount = 0;
        m.bvh[id].index = (int)m.bvh.size() - 2;
        int left = m.bvh[id].index;
        subdivide(left);
        subdivide(left + 1);
    }
};
}  // namespace

// TriangleMesh.cpp:144-164
void TriangleMesh::build(const std::vector<V3>& verts, const std::vector<uint32_t>& idx) {
    vertices = verts;
    triangles.clear();
    for (size_t i = 0; i + 2 < idx.size(); i += 3) {
        uint32_t i0 = idx[i], i1 = idx[i + 1], i2 = idx[i + 2];
        V3 a = verts[i0], b = verts[i1], c = verts[i2];
        Triangle t;
        t.idx[0] = i0; t.idx[1] = i1; t.idx[2] = i2;
        t.bounds = {vmin(vmin(a, b), c), vmax(vmax(a, b), c)};
        t.normal = normalize(cross(b - a, c - a));
        t.centroid = (a + b + c) / 3.f;
        triangles.push_back(t);
    }
    bvh.clear();
    bvh.reserve(2 * triangles.size());
    bvh.push_back({{}, (int)triangles.size(), 0});
    Builder bld{*this};
    bld.updateNodeBounds(0);
    bld.subdivide(0);
}

// TriangleMesh.cpp:166-192
void TriangleMesh::overlap(const Bounds& b, std::vector<int>& out) const {
    out.clear();
    std::vector<int> stack;
    stack.push_back(0);
    while (!stack.empty()) {
        const TriNode& n = bvh[stack.back()];
        stack.pop_back();
        if (intersects(b, n.bounds)) {
            if (n.triCount) {
                for (int i = 0; i < n.triCount; ++i) out.push_back(n.index + i);
            } else {
                stack.push_back(n.index + 1);
                stack.push_back(n.index);
            }
        }
    }
}

// ---------------------------------------------------------------- per-triangle tests

namespace {
enum BoxFeature { BF_FACE = 0, BF_EDGE = 1, BF_UNKNOWN = 2 };
struct TCI {  // TriangleContactInfo, CollisionTriangleMesh.cpp:22-35
    int tri = 0;
    V3 normal{0, 0, 0}, cpBody{0, 0, 0}, cpTri{0, 0, 0};
    int feature = TF_FACE, featureIndex = 0;
    float distance = 0;
    int boxFeature = BF_FACE, boxAxis = 0;
};
}  // namespace

// CollisionTriangleMesh.cpp:44-71
static bool sphereTri(V3 pos0, float r0, V3 a, V3 b, V3 c, V3 n, TCI& o) {
    V3 u;
    int f, fi;
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

// CollisionTriangleMesh.cpp:85-119
static bool capsuleTri(V3 pos, Q4 ori, float hh, float r, V3 a, V3 b, V3 c, V3 n, TCI& o) {
    V3 dir = qrot(ori, {0, 1, 0});
    float t;
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

// CollisionTriangleMesh.cpp:221-456
static bool boxTri(V3 pos, Q4 ori, V3 he, V3 a, V3 b, V3 c, V3 n, TCI& o) {
    float edgeOffset = 0.f;
    const float edgeLimit = 0.999f;
    M3 u = mat3_cast(ori);
    M3 invU = transpose(u);
    V3 v0 = mv(invU, a - pos), v1 = mv(invU, b - pos), v2 = mv(invU, c - pos);
    V3 f0 = v1 - v0, f1 = v2 - v1, f2 = v0 - v2;
    float f0L = edgeLimit * length2(f0), f1L = edgeLimit * length2(f1), f2L = edgeLimit * length2(f2);
    float p0, p1, r, d;
    float mx = -FLT_MAX;
    auto edgeAxis = [&](float fxx, float lim, int triEdge, int axis) {
        // shared tail of the nine edge-edge axes
        if (fxx < lim && d > mx) {
            mx = d;
            o.feature = TF_EDGE; o.featureIndex = triEdge; o.distance = d;
            o.boxFeature = BF_EDGE; o.boxAxis = axis;
            edgeOffset = 0.1f;
        }
    };
    auto sepd = [](float a0, float a1, float rr) { return fmaxG(-fmaxG(a0, a1), fminG(a0, a1)) - rr; };
    // u0 x f0
    p0 = v0.z * f0.y - v0.y * f0.z; p1 = v2.z * f0.y - v2.y * f0.z; r = he.y * std::fabs(f0.z) + he.z * std::fabs(f0.y);
    d = sepd(p0, p1, r); if (d > 0) return false; edgeAxis(f0.x * f0.x, f0L, 2, 0);
    // u0 x f1
    p0 = v0.z * f1.y - v0.y * f1.z; p1 = v1.z * f1.y - v1.y * f1.z; r = he.y * std::fabs(f1.z) + he.z * std::fabs(f1.y);
    d = sepd(p0, p1, r); if (d > 0) return false; edgeAxis(f1.x * f1.x, f1L, 0, 0);
    // u0 x f2
    p0 = v1.z * f2.y - v1.y * f2.z; p1 = v2.z * f2.y - v2.y * f2.z; r = he.y * std::fabs(f2.z) + he.z * std::fabs(f2.y);
    d = sepd(p0, p1, r); if (d > 0) return false; edgeAxis(f2.x * f2.x, f2L, 1, 0);
    // u1 x f0
    p0 = v0.x * f0.z - v0.z * f0.x; p1 = v2.x * f0.z - v2.z * f0.x; r = he.x * std::fabs(f0.z) + he.z * std::fabs(f0.x);
    d = sepd(p0, p1, r); if (d > 0) return false; edgeAxis(f0.y * f0.y, f0L, 2, 1);
    // u1 x f1
    p0 = v0.x * f1.z - v0.z * f1.x; p1 = v1.x * f1.z - v1.z * f1.x; r = he.x * std::fabs(f1.z) + he.z * std::fabs(f1.x);
    d = sepd(p0, p1, r); if (d > 0) return false; edgeAxis(f1.y * f1.y, f1L, 0, 1);
    // u1 x f2
    p0 = v1.x * f2.z - v1.z * f2.x; p1 = v2.x * f2.z - v2.z * f2.x; r = he.x * std::fabs(f2.z) + he.z * std::fabs(f2.x);
    d = sepd(p0, p1, r); if (d > 0) return false; edgeAxis(f2.y * f2.y, f2L, 1, 1);
    // u2 x f0
    p0 = v0.y * f0.x - v0.x * f0.y; p1 = v2.y * f0.x - v2.x * f0.y; r = he.x * std::fabs(f0.y) + he.y * std::fabs(f0.x);
    d = sepd(p0, p1, r); if (d > 0) return false; edgeAxis(f0.z * f0.z, f0L, 2, 2);
    // u2 x f1
    p0 = v0.y * f1.x - v0.x * f1.y; p1 = v1.y * f1.x - v1.x * f1.y; r = he.x * std::fabs(f1.y) + he.y * std::fabs(f1.x);
    d = sepd(p0, p1, r); if (d > 0) return false; edgeAxis(f1.z * f1.z, f1L, 0, 2);
    // u2 x f2
    p0 = v1.y * f2.x - v1.x * f2.y; p1 = v2.y * f2.x - v2.x * f2.y; r = he.x * std::fabs(f2.y) + he.y * std::fabs(f2.x);
    d = sepd(p0, p1, r); if (d > 0) return false; edgeAxis(f2.z * f2.z, f2L, 1, 2);
    // box face normals
    for (int i = 0; i < 3; ++i) {
        float a0 = at(v0, i), a1 = at(v1, i), a2 = at(v2, i), h = at(he, i);
        d = fmaxG(-fmaxG(fmaxG(a0, a1), a2), fminG(fminG(a0, a1), a2)) - h;
        if (d > 0) return false;
        if (d > mx - edgeOffset) {
            mx = d;
            bool i0 = std::fabs(a0) < h, i1 = std::fabs(a1) < h, i2 = std::fabs(a2) < h;
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
    if (d > mx - edgeOffset) {
        o.feature = TF_FACE; o.distance = d; o.boxFeature = BF_UNKNOWN;
    }
    return true;
}

// CollisionTriangleMesh.cpp:614-699
static bool convexTri(V3 pos, Q4 ori, const ConvexMesh* m, V3 sc, V3 a, V3 b, V3 c, V3 cen, TCI& o) {
    Support s0; s0.kind = 3; s0.pos = pos; s0.basis = mat3_cast(ori); s0.mesh = m; s0.scale = sc;
    Support s1; s1.kind = 4; s1.a = a; s1.b = b; s1.c = c;
    GjkSimplex s;
    if (!gjk(s0, s1, cen - pos, s)) return false;
    o.normal = epa(s0, s1, s, o.cpBody, o.cpTri);
    o.distance = dot(o.cpTri - o.cpBody, o.normal);
    V3 v0 = b - a, v1 = c - a, v2 = o.cpTri - a;
    float d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1), d20 = dot(v2, v0), d21 = dot(v2, v1);
    float denom = d00 * d11 - d01 * d01;
    float u, v, w;
    if (denom) {
        v = (d20 * d11 - d21 * d01) / denom;
        w = (d00 * d21 - d01 * d20) / denom;
        u = 1.0f - v - w;
    } else {
        w = 0;
        if (d00) { v = d20 / d00; u = 1.0f - v; }
        else { v = 0; u = 1.0; }
    }
    float eps = 1e-4;
    if (u < eps) {
        if (v < eps) { o.feature = TF_VERTEX; o.featureIndex = 2; }
        else if (w < eps) { o.feature = TF_VERTEX; o.featureIndex = 1; }
        else { o.feature = TF_EDGE; o.featureIndex = 0; }
    } else {
        if (v < eps) {
            if (w < eps) { o.feature = TF_VERTEX; o.featureIndex = 0; }
            else { o.feature = TF_EDGE; o.featureIndex = 1; }
        } else if (w < eps) {
            if (u < eps) { o.feature = TF_VERTEX; o.featureIndex = 0; }
            else { o.feature = TF_EDGE; o.featureIndex = 2; }
        } else o.feature = TF_FACE;
    }
    return true;
}

// ---------------------------------------------------------------- contact generators

// CollisionTriangleMesh.cpp:73-81
static void sphereTriContacts(V3 pos1, Q4 or1, const TCI& c, std::vector<Manifold>& out) {
    Manifold mf;
    mf.normal = qrot(or1, c.normal);
    mf.numPoints = 1;
    mf.points[0] = {pos1 + qrot(or1, c.cpBody), pos1 + qrot(or1, c.cpTri)};
    mf.triangleIndex = c.tri;
    out.push_back(mf);
}

static void triFrame(const TriangleMesh* mesh, const Triangle& tri, bool normalizeN, V3& refO, V3& u1, M3& m2r, V2* clip) {
    refO = tri.centroid;
    V3 u0 = normalize(mesh->vertices[tri.idx[0]] - refO);
    u1 = normalizeN ? normalize(tri.normal) : tri.normal;
    V3 u2 = cross(u0, u1);
    m2r = transpose(m3cols(u0, u1, u2));
    for (int i = 0; i < 3; i++) {
        V3 v = mv(m2r, mesh->vertices[tri.idx[i]]);
        clip[3 - i - 1] = {v.z, v.x};
    }
}

// CollisionTriangleMesh.cpp:121-217
static void capsuleTriFace(V3 pos0, Q4 or0, float hh0, float r0, V3 pos1, Q4 or1, const TriangleMesh* mesh, const TCI& c,
                           std::vector<Manifold>& out) {
    V3 dir = qrot(or0, {0, 1, 0});
    V3 p0l = pos0 - dir * hh0, p1l = pos0 + dir * hh0;
    const Triangle& tri = mesh->triangles[c.tri];
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
    V3 p0{0, 0, 0}, p1{0, 0, 0};
    float dX = at(p0R, cx) - at(p1R, cx), dY = at(p0R, cy) - at(p1R, cy);
    float aX = std::fabs(dX), aY = std::fabs(dY);
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
    int n = 0;
    Manifold res;
    res.triangleIndex = c.tri;
    res.normal = mv(m2w, c.normal);
    if (at(p0, fa) < dPlane) {
        at(p0, cx) = l0.x; at(p0, cy) = l0.y;
        V3 of = p0; at(of, fa) = dPlane;
        res.points[n++] = {pos1 + mv(r2w, p0), pos1 + mv(r2w, of)};
    }
    if (at(p1, fa) < dPlane) {
        at(p1, cx) = l1.x; at(p1, cy) = l1.y;
        V3 of = p1; at(of, fa) = dPlane;
        res.points[n++] = {pos1 + mv(r2w, p1), pos1 + mv(r2w, of)};
    }
    if (!n) {
        n = 1;
        res.points[0] = {pos1 + mv(m2w, c.cpBody), pos1 + mv(m2w, c.cpTri)};
    }
    res.numPoints = n;
    out.push_back(res);
}

// CollisionTriangleMesh.cpp:458-530
static void boxTriFace(V3 boxPos, Q4 boxOr, V3 he, V3 meshPos, Q4 meshOr, const TriangleMesh* mesh, const TCI& c,
                       std::vector<Manifold>& out) {
    M3 bb = mat3_cast(boxOr);
    const Triangle& tri = mesh->triangles[c.tri];
    V3 refO, u1;
    M3 m2r;
    V2 clip[3];
    triFrame(mesh, tri, true, refO, u1, m2r, clip);
    const int cx = 2, cy = 0;
    int incAxis = 0;
    float incSign = 1;
    if (c.boxFeature == BF_FACE) {
        incAxis = c.boxAxis;
        incSign = dot(tri.normal, bb.c[incAxis]) > 0 ? -1 : 1;
    } else {
        float maxDot = 0;
        for (int i = 0; i < 3; ++i) {
            float d = dot(tri.normal, bb.c[i]);
            float ad = std::fabs(d);
            if (ad > maxDot) { maxDot = ad; incAxis = i; incSign = d > 0 ? -1 : 1; }
        }
    }
    int a1 = (incAxis + 1) % 3, a2 = (incAxis + 2) % 3;
    V3 incO = mv(m2r, boxPos + bb.c[incAxis] * at(he, incAxis) * incSign);
    V3 e1 = bb.c[a1] * at(he, a1), e2 = bb.c[a2] * at(he, a2);
    V3 ne1 = -bb.c[a1] * at(he, a1);
    V3 q0 = incO + mv(m2r, e1 + e2);
    V3 q1 = incO + mv(m2r, ne1 + e2);
    V3 q2 = incO + mv(m2r, ne1 - e2);
    V3 q3 = incO + mv(m2r, e1 - e2);
    Poly poly;
    poly.n = 4;
    poly.p[0] = {at(q0, cx), at(q0, cy)};
    poly.p[1] = {at(q1, cx), at(q1, cy)};
    poly.p[2] = {at(q2, cx), at(q2, cy)};
    poly.p[3] = {at(q3, cx), at(q3, cy)};
    suthHodgClip(poly, clip, 3);
    V3 incN = mv(m2r, bb.c[incAxis]);
    M3 m2w = mat3_cast(meshOr);
    M3 r2w = mm(m2w, transpose(m2r));
    Manifold mf;
    mf.normal = -mv(m2w, tri.normal);
    mf.triangleIndex = c.tri;
    generateContactsPolygonPolygonFace(meshPos, r2w, refO, u1, incO, incN, poly, cx, cy, mf.points, mf.numPoints);
    for (int i = 0; i < mf.numPoints; ++i) mf.points[i] = {mf.points[i].p1, mf.points[i].p0};
    out.push_back(mf);
}

// CollisionTriangleMesh.cpp:532-571
static void boxFaceTri(V3 boxPos, Q4 boxOr, V3 he, V3 meshPos, Q4 meshOr, const TriangleMesh* mesh, const TCI& c,
                       std::vector<Manifold>& out) {
    M3 bb = mat3_cast(boxOr);
    const Triangle& tri = mesh->triangles[c.tri];
    M3 m2b = transpose(bb);
    int ra = c.boxAxis;
    float rs = dot(bb.c[ra], tri.centroid - boxPos) < 0 ? -1 : 1;
    int cx = (ra + 1) % 3, cy = (ra + 2) % 3;
    Poly poly;
    poly.n = 3;
    for (int i = 0; i < 3; ++i) {
        V3 v = mv(m2b, mesh->vertices[tri.idx[i]] - boxPos);
        poly.p[i] = {at(v, cx), at(v, cy)};
    }
    V2 clip[4] = {{at(he, cx), at(he, cy)}, {at(he, cx), -at(he, cy)}, {-at(he, cx), -at(he, cy)}, {-at(he, cx), at(he, cy)}};
    suthHodgClip(poly, clip, 4);
    V3 incO = mv(m2b, tri.centroid - boxPos);
    V3 incN = mv(m2b, tri.normal);
    M3 m2w = mat3_cast(meshOr);
    Manifold mf;
    mf.normal = mv(m2w, rs * bb.c[ra]);
    mf.triangleIndex = c.tri;
    generateContactsPolygonBoxFace(boxPos, bb, ra, (int)rs, he, incO, incN, poly, cx, cy, mf.points, mf.numPoints);
    for (int i = 0; i < mf.numPoints; ++i) {
        mf.points[i].p0 = meshPos + mv(m2w, mf.points[i].p0);
        mf.points[i].p1 = meshPos + mv(m2w, mf.points[i].p1);
    }
    out.push_back(mf);
}

// CollisionTriangleMesh.cpp:573-601
static void boxEdgeTriEdge(V3 boxPos, Q4 boxOr, V3 he, V3 meshPos, Q4 meshOr, const TriangleMesh* mesh, const TCI& c,
                           std::vector<Manifold>& out) {
    M3 bb = mat3_cast(boxOr);
    const Triangle& tri = mesh->triangles[c.tri];
    int ba = c.boxAxis, te = c.featureIndex;
    V3 ta = mesh->vertices[tri.idx[(te + 1) % 3]];
    V3 tb = mesh->vertices[tri.idx[(te + 2) % 3]];
    V3 tEdge = tb - ta;
    V3 axis = cross(bb.c[ba], tEdge);
    M3 m2w = mat3_cast(meshOr);
    Manifold mf;
    mf.normal = mv(m2w, normalize(dot(axis, tri.centroid - boxPos) < 0 ? -axis : axis));
    mf.numPoints = 1;
    mf.triangleIndex = c.tri;
    V3 sb = v3s(-1);
    at(sb, (ba + 1) % 3) = dot(bb.c[(ba + 1) % 3], mf.normal) < 0 ? -1 : 1;
    at(sb, (ba + 2) % 3) = dot(bb.c[(ba + 2) % 3], mf.normal) < 0 ? -1 : 1;
    V3 bA = boxPos + sb.x * he.x * bb.c[0] + sb.y * he.y * bb.c[1] + sb.z * he.z * bb.c[2];
    V3 bEdge = bb.c[ba] * at(he, ba) * 2.f;
    V3 p0, p1;
    closestPointsBetweenSegmentsV(bA, bEdge, ta, tEdge, p0, p1);
    mf.points[0] = {meshPos + mv(m2w, p0), meshPos + mv(m2w, p1)};
    out.push_back(mf);
}

// CollisionTriangleMesh.cpp:701-755
static void convexTriFace(V3 cPos, Q4 cOr, const ConvexMesh* cm, V3 sc, V3 meshPos, Q4 meshOr, const TriangleMesh* mesh,
                          const TCI& c, std::vector<Manifold>& out) {
    const Triangle& tri = mesh->triangles[c.tri];
    V3 refO, u1;
    M3 m2r;
    V2 clip[3];
    triFrame(mesh, tri, false, refO, u1, m2r, clip);
    const int cx = 2, cy = 0;
    int fi = 0;
    float minDot = 0;
    for (int i = 0; i < (int)cm->faces.size(); ++i) {
        float d = dot(tri.normal, normalize(qrot(cOr, cm->faces[i].normal / sc)));
        if (d < minDot) { minDot = d; fi = i; }
    }
    const ConvexFace& F = cm->faces[fi];
    Poly poly;
    poly.n = (int)F.indices.size();
    for (int i = 0; i < poly.n; ++i) {
        V3 v = mv(m2r, cPos + qrot(cOr, sc * cm->buffer[F.indices[i]]));
        poly.p[i] = {at(v, cx), at(v, cy)};
    }
    suthHodgClip(poly, clip, 3);
    V3 incO = mv(m2r, cPos + qrot(cOr, sc * F.centroid));
    V3 incN = mv(m2r, qrot(cOr, normalize(F.normal / sc)));
    M3 m2w = mat3_cast(meshOr);
    M3 r2w = mm(m2w, transpose(m2r));
    Manifold mf;
    mf.normal = -mv(m2w, tri.normal);
    mf.triangleIndex = c.tri;
    generateContactsPolygonPolygonFace(meshPos, r2w, refO, u1, incO, incN, poly, cx, cy, mf.points, mf.numPoints);
    for (int i = 0; i < mf.numPoints; ++i) mf.points[i] = {mf.points[i].p1, mf.points[i].p0};
    out.push_back(mf);
}

// CollisionTriangleMesh.cpp:757-824
static void convexFaceTri(V3 cPos, Q4 cOr, const ConvexMesh* cm, V3 sc, V3 meshPos, Q4 meshOr, const TriangleMesh* mesh,
                          const TCI& c, std::vector<Manifold>& out) {
    const Triangle& tri = mesh->triangles[c.tri];
    M3 c2m = mat3_cast(cOr);
    M3 m2c = transpose(c2m);
    int fi = 0;
    float maxDot = 0;
    for (int i = 0; i < (int)cm->faces.size(); ++i) {
        float d = dot(c.normal, normalize(qrot(cOr, cm->faces[i].normal / sc)));
        if (d > maxDot) { maxDot = d; fi = i; }
    }
    const ConvexFace& F = cm->faces[fi];
    V3 refO = sc * F.centroid;
    V3 u0 = normalize(sc * cm->buffer[F.indices[0]] - refO);
    V3 u1 = normalize(F.normal / sc);
    V3 u2 = cross(u0, u1);
    M3 c2r = transpose(m3cols(u0, u1, u2));
    M3 m2r = mm(c2r, m2c);
    const int cx = 2, cy = 0;
    V2 clip[kMaxPoly];
    int nc = (int)F.indices.size();
    for (int i = 0; i < nc; ++i) {
        V3 v = mv(c2r, sc * cm->buffer[F.indices[i]]);
        clip[i] = {at(v, cx), at(v, cy)};
    }
    Poly poly;
    poly.n = 3;
    for (int i = 0; i < 3; ++i) {
        V3 v = mv(m2r, mesh->vertices[tri.idx[i]] - cPos);
        poly.p[i] = {at(v, cx), at(v, cy)};
    }
    suthHodgClip(poly, clip, nc);
    V3 incO = mv(m2r, tri.centroid - cPos);
    V3 incN = mv(m2r, tri.normal);
    M3 m2w = mat3_cast(meshOr);
    M3 r2m = transpose(m2r);
    Manifold mf;
    mf.triangleIndex = c.tri;
    generateContactsPolygonPolygonFace(cPos, r2m, refO, u1, incO, incN, poly, cx, cy, mf.points, mf.numPoints);
    if (mf.numPoints) {
        for (int i = 0; i < mf.numPoints; ++i) {
            mf.points[i].p0 = meshPos + mv(m2w, mf.points[i].p0);
            mf.points[i].p1 = meshPos + mv(m2w, mf.points[i].p1);
        }
        mf.normal = mv(mm(m2w, c2m), u1);
    } else {
        mf.normal = mv(m2w, c.normal);
        mf.numPoints = 1;
        mf.points[0] = {meshPos + mv(m2w, c.cpBody), meshPos + mv(m2w, c.cpTri)};
    }
    out.push_back(mf);
}

// ---------------------------------------------------------------- driver

// CollisionTriangleMesh.cpp:882-956
bool collisionTriangleMesh(V3 pos0, Q4 or0, const Geometry& g0, V3 pos1, Q4 or1, const TriangleMesh* mesh,
                           std::vector<Manifold>& out) {
    Q4 inv1 = qinverse(or1);
    V3 lp = qrot(inv1, pos0 - pos1);
    Q4 lo = qmul(inv1, or0);
    Bounds lb = getBounds(lp, lo, g0);
    static thread_local std::vector<int> cand;
    mesh->overlap(lb, cand);
    if (cand.empty()) return false;
    std::vector<TCI> contacts;
    contacts.reserve(cand.size());
    for (int ti : cand) {
        const Triangle& tri = mesh->triangles[ti];
        V3 a = mesh->vertices[tri.idx[0]], b = mesh->vertices[tri.idx[1]], c = mesh->vertices[tri.idx[2]];
        TCI ci;
        bool hit = false;
        switch (g0.type) {
            case SPHERE: hit = sphereTri(lp, g0.p[0], a, b, c, tri.normal, ci); break;
            case CAPSULE: hit = capsuleTri(lp, lo, g0.p[0], g0.p[1], a, b, c, tri.normal, ci); break;
            case BOX: hit = boxTri(lp, lo, {g0.p[0], g0.p[1], g0.p[2]}, a, b, c, tri.normal, ci); break;
            case CONVEX_MESH: hit = convexTri(lp, lo, g0.convex, {g0.p[0], g0.p[1], g0.p[2]}, a, b, c, tri.centroid, ci); break;
            default: break;
        }
        if (hit) { ci.tri = ti; contacts.push_back(ci); }
    }
    if (contacts.empty()) return false;
    std::unordered_set<uint32_t> voided;
    V3 he = {g0.p[0], g0.p[1], g0.p[2]};
    for (int i = (int)contacts.size() - 1; i >= 0; i--) {
        TCI& c = contacts[i];
        if (c.feature == TF_FACE) {
            const Triangle& tri = mesh->triangles[c.tri];
            voided.insert(tri.idx[0]); voided.insert(tri.idx[1]); voided.insert(tri.idx[2]);
            switch (g0.type) {
                case SPHERE: sphereTriContacts(pos1, or1, c, out); break;
                case CAPSULE: capsuleTriFace(lp, lo, g0.p[0], g0.p[1], pos1, or1, mesh, c, out); break;
                case BOX: boxTriFace(lp, lo, he, pos1, or1, mesh, c, out); break;
                case CONVEX_MESH: convexTriFace(lp, lo, g0.convex, he, pos1, or1, mesh, c, out); break;
            }
            std::swap(c, contacts.back());
            contacts.pop_back();
        }
    }
    std::sort(contacts.begin(), contacts.end(), [](const TCI& a, const TCI& b) { return a.distance < b.distance; });
    for (const TCI& c : contacts) {
        const Triangle& tri = mesh->triangles[c.tri];
        if (c.feature == TF_EDGE) {
            if (voided.count(tri.idx[(c.featureIndex + 1) % 3]) && voided.count(tri.idx[(c.featureIndex + 2) % 3])) continue;
            switch (g0.type) {
                case SPHERE: case CAPSULE: sphereTriContacts(pos1, or1, c, out); break;
                case BOX:
                    if (c.boxFeature == BF_FACE) boxFaceTri(lp, lo, he, pos1, or1, mesh, c, out);
                    else boxEdgeTriEdge(lp, lo, he, pos1, or1, mesh, c, out);
                    break;
                case CONVEX_MESH: convexFaceTri(lp, lo, g0.convex, he, pos1, or1, mesh, c, out); break;
            }
        } else if (c.feature == TF_VERTEX) {
            if (voided.count(tri.idx[c.featureIndex])) continue;
            switch (g0.type) {
                case SPHERE: case CAPSULE: sphereTriContacts(pos1, or1, c, out); break;
                case BOX: boxFaceTri(lp, lo, he, pos1, or1, mesh, c, out); break;
                case CONVEX_MESH: convexFaceTri(lp, lo, g0.convex, he, pos1, or1, mesh, c, out); break;
            }
        }
        voided.insert(tri.idx[0]); voided.insert(tri.idx[1]); voided.insert(tri.idx[2]);
    }
    return true;
}

}  // namespace orc
