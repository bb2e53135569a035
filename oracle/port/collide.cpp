/*
 * collide.cpp — narrowphase pair tests and bounds of the CPU oracle.
 * ORACLE (test infrastructure only; see omath.h).
 *
 * Restates src/Collision.cpp:54-1016 (sphere / capsule / box analytic tests,
 * box-box SAT with face clipping, GJK+EPA convex pairs with face clipping,
 * the 4x4 dispatcher with flipContacts) and src/BoundsUtil.cpp:23-107.
 */
#include "collide_util.h"

namespace orc {

bool collisionTriangleMesh(V3 pos0, Q4 or0, const Geometry& g0, V3 pos1, Q4 or1, const TriangleMesh* mesh,
                           std::vector<Manifold>& out);

// ---------------------------------------------------------------- bounds

Bounds getBounds(V3 pos, Q4 ori, const Geometry& g) {
    switch (g.type) {
        case SPHERE: return {pos - v3s(g.p[0]), pos + v3s(g.p[0])};
        case CAPSULE: {
            V3 p0 = pos + qrot(ori, {0, g.p[0], 0});
            V3 p1 = pos + qrot(ori, {0, -g.p[0], 0});
            return {vmin(p0, p1) - g.p[1], vmax(p0, p1) + g.p[1]};
        }
        case BOX: {
            M3 u = mat3_cast(ori);
            M3 a = m3cols(vabs(u.c[0]), vabs(u.c[1]), vabs(u.c[2]));
            V3 w = mv(a, {g.p[0], g.p[1], g.p[2]});
            return {pos - w, pos + w};
        }
        case CONVEX_MESH: {
            V3 mn = v3s(FLT_MAX), mx = v3s(-FLT_MAX);
            V3 sc = {g.p[0], g.p[1], g.p[2]};
            for (const V3& v : g.convex->buffer) {
                V3 t = pos + qrot(ori, sc * v);
                mn = vmin(mn, t); mx = vmax(mx, t);
            }
            return {mn, mx};
        }
        default: {
            V3 mn = v3s(FLT_MAX), mx = v3s(-FLT_MAX);
            for (const V3& v : g.tri->vertices) {
                V3 t = pos + qrot(ori, v);
                mn = vmin(mn, t); mx = vmax(mx, t);
            }
            return {mn, mx};
        }
    }
}

// ---------------------------------------------------------------- box-box

// Collision.cpp:54-107
static void boxBoxFaceContacts(const M3& uRef, V3 posRef, V3 heRef, const M3& uInc, V3 posInc, V3 heInc, int refAxis,
                               ContactPoint* cp, int& np) {
    V3 axis = uRef.c[refAxis];
    float refSign = dot(axis, posInc - posRef) < 0 ? -1 : 1;
    float maxDot = 0;
    int incAxis = 0;
    float incSign = 1;
    for (int i = 0; i < 3; ++i) {
        float d = dot(-refSign * axis, uInc.c[i]);
        float ad = std::fabs(d);
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
    suthHodgClip(poly, clip, 4);
    V3 incN = mv(inv, uInc.c[incAxis]);
    generateContactsPolygonBoxFace(posRef, uRef, refAxis, (int)refSign, heRef, incO, incN, poly, cx, cy, cp, np);
}

// Collision.cpp:135-350
static bool boxBox(V3 pos0, Q4 or0, V3 he0, V3 pos1, Q4 or1, V3 he1, Manifold& res) {
    float edgeOffset = 0.1f;
    const float edgeLimit = 0.999f;
    bool edge = false;
    int fBox = 0, fAxis = 0, e0 = 0, e1 = 0;
    float mx = -FLT_MAX;
    M3 u0 = mat3_cast(or0), u1 = mat3_cast(or1);
    V3 t = pos1 - pos0;
    t = {dot(t, u0.c[0]), dot(t, u0.c[1]), dot(t, u0.c[2])};
    float r[3][3], ar[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) { r[i][j] = dot(u0.c[i], u1.c[j]); ar[i][j] = std::fabs(r[i][j]); }
    float ra, rb, l, d;
    for (int i = 0; i < 3; i++) {
        ra = at(he0, i);
        rb = he1.x * ar[i][0] + he1.y * ar[i][1] + he1.z * ar[i][2];
        l = std::fabs(at(t, i));
        d = l - ra - rb;
        if (d > 0) return false;
        if (d > mx) { mx = d; edge = false; fBox = 0; fAxis = i; }
    }
    for (int i = 0; i < 3; i++) {
        ra = he0.x * ar[0][i] + he0.y * ar[1][i] + he0.z * ar[2][i];
        rb = at(he1, i);
        l = std::fabs(t.x * r[0][i] + t.y * r[1][i] + t.z * r[2][i]);
        d = l - ra - rb;
        if (d > 0) return false;
        if (d > mx) { mx = d; edge = false; fBox = 1; fAxis = i; }
    }
    // the nine edge-edge axes in the reference's order, with their exact ra/rb/l expressions
    struct EA { int i, j; };
    const EA order[9] = {{0, 0}, {0, 1}, {0, 2}, {1, 0}, {1, 1}, {1, 2}, {2, 0}, {2, 1}, {2, 2}};
    for (int k = 0; k < 9; ++k) {
        int i = order[k].i, j = order[k].j;
        int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
        // A_i x B_j: ra = a[i1]*|r[i2][j]| + a[i2]*|r[i1][j]|, rb = b[j1]*|r[i][j2]| + b[j2]*|r[i][j1]|,
        // l = |t[i2]*r[i1][j] - t[i1]*r[i2][j]|; written out to keep the reference's operand order.
        switch (k) {
            case 0: ra = he0.y * ar[2][0] + he0.z * ar[1][0]; rb = he1.y * ar[0][2] + he1.z * ar[0][1]; l = std::fabs(t.z * r[1][0] - t.y * r[2][0]); break;
            case 1: ra = he0.y * ar[2][1] + he0.z * ar[1][1]; rb = he1.x * ar[0][2] + he1.z * ar[0][0]; l = std::fabs(t.z * r[1][1] - t.y * r[2][1]); break;
            case 2: ra = he0.y * ar[2][2] + he0.z * ar[1][2]; rb = he1.x * ar[0][1] + he1.y * ar[0][0]; l = std::fabs(t.z * r[1][2] - t.y * r[2][2]); break;
            case 3: ra = he0.x * ar[2][0] + he0.z * ar[0][0]; rb = he1.y * ar[1][2] + he1.z * ar[1][1]; l = std::fabs(t.x * r[2][0] - t.z * r[0][0]); break;
            case 4: ra = he0.x * ar[2][1] + he0.z * ar[0][1]; rb = he1.x * ar[1][2] + he1.z * ar[1][0]; l = std::fabs(t.x * r[2][1] - t.z * r[0][1]); break;
            case 5: ra = he0.x * ar[2][2] + he0.z * ar[0][2]; rb = he1.x * ar[1][1] + he1.y * ar[1][0]; l = std::fabs(t.x * r[2][2] - t.z * r[0][2]); break;
            case 6: ra = he0.x * ar[1][0] + he0.y * ar[0][0]; rb = he1.y * ar[2][2] + he1.z * ar[2][1]; l = std::fabs(t.y * r[0][0] - t.x * r[1][0]); break;
            case 7: ra = he0.x * ar[1][1] + he0.y * ar[0][1]; rb = he1.x * ar[2][2] + he1.z * ar[2][0]; l = std::fabs(t.y * r[0][1] - t.x * r[1][1]); break;
            default: ra = he0.x * ar[1][2] + he0.y * ar[0][2]; rb = he1.x * ar[2][1] + he1.y * ar[2][0]; l = std::fabs(t.y * r[0][2] - t.x * r[1][2]); break;
        }
        (void)i1; (void)i2; (void)j1; (void)j2;
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
            boxBoxFaceContacts(u1, pos1, he1, u0, pos0, he0, fAxis, cp, np);
            for (int i = 0; i < np; i++) res.points[i] = {cp[i].p1, cp[i].p0};
        } else {
            axis = u0.c[fAxis];
            boxBoxFaceContacts(u0, pos0, he0, u1, pos1, he1, fAxis, cp, np);
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

// ---------------------------------------------------------------- spheres and capsules

// Collision.cpp:109-118
static bool sphereSphere(V3 pos0, float r0, V3 pos1, float r1, Manifold& res) {
    V3 d = pos1 - pos0;
    float rs = r0 + r1;
    if (dot(d, d) > rs * rs) return false;
    float len = length(d);
    res.normal = len ? d / len : V3{0, 1, 0};
    res.numPoints = 1;
    res.points[0] = {pos0 + res.normal * r0, pos1 - res.normal * r1};
    return true;
}

// Collision.cpp:120-133
static bool capsuleCapsule(V3 pos0, Q4 or0, float hh0, float r0, V3 pos1, Q4 or1, float hh1, float r1, Manifold& res) {
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

// Collision.cpp:428-440
static bool sphereCapsule(V3 pos0, float r0, V3 pos1, Q4 or1, float hh1, float r1, Manifold& res) {
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

// Collision.cpp:442-486
static bool sphereBox(V3 pos0, float r0, V3 pos1, Q4 or1, V3 he1, Manifold& res) {
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
            float depth = at(he1, i) - std::fabs(at(d, i));
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

// Collision.cpp:501-582
static void capsuleBoxContacts(V3 p0L, V3 p1L, float radius, V3 normal, V3 boxCenter, V3 he, const M3& basis, Manifold& res) {
    int boxAxis = 0;
    float boxAxisSign = 0, maxDot = 0;
    for (int i = 0; i < 3; ++i) {
        float d = dot(normal, basis.c[i]);
        float ad = std::fabs(d);
        if (ad > maxDot) { maxDot = ad; boxAxis = i; boxAxisSign = d < 0 ? 1 : -1; }
    }
    int cx = (boxAxis + 1) % 3, cy = (boxAxis + 2) % 3;
    V2 l0 = {at(p0L, cx), at(p0L, cy)}, l1 = {at(p1L, cx), at(p1L, cy)};
    V2 clip[4] = {{at(he, cx), at(he, cy)}, {at(he, cx), -at(he, cy)}, {-at(he, cx), -at(he, cy)}, {-at(he, cx), at(he, cy)}};
    if (clipLine(l0, l1, clip, 4)) {
        float onAxis = boxAxisSign * at(he, boxAxis);
        V3 p0{0, 0, 0}, p1{0, 0, 0};
        float dX = at(p0L, cx) - at(p1L, cx), dY = at(p0L, cy) - at(p1L, cy);
        float aX = std::fabs(dX), aY = std::fabs(dY);
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
        if (std::fabs(at(p0, boxAxis)) < at(he, boxAxis)) {
            at(p0, cx) = l0.x; at(p0, cy) = l0.y;
            V3 ob = p0; at(ob, boxAxis) = onAxis;
            res.points[n++] = {boxCenter + mv(basis, p0), boxCenter + mv(basis, ob)};
        }
        if (std::fabs(at(p1, boxAxis)) < at(he, boxAxis)) {
            at(p1, cx) = l1.x; at(p1, cy) = l1.y;
            V3 ob = p1; at(ob, boxAxis) = onAxis;
            res.points[n++] = {boxCenter + mv(basis, p1), boxCenter + mv(basis, ob)};
        }
        res.numPoints = n;
    } else {
        res.numPoints = 0;
    }
}

// Collision.cpp:584-692
static bool capsuleBox(V3 pos0, Q4 or0, float hh0, float r0, V3 pos1, Q4 or1, V3 he1, Manifold& res) {
    M3 u1 = mat3_cast(or1);
    V3 p = pos0 - pos1;
    p = {dot(p, u1.c[0]), dot(p, u1.c[1]), dot(p, u1.c[2])};
    V3 dir = qrot(or0, {0, 1, 0});
    V3 dl = {dot(dir, u1.c[0]), dot(dir, u1.c[1]), dot(dir, u1.c[2])};
    float t;
    V3 q{0, 0, 0};
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
        for (int i = 0; i < 3; ++i) { at(r, i) = dot(dir, u1.c[i]); at(ar, i) = std::fabs(at(r, i)); }
        float mx = -FLT_MAX;
        bool edge = false;
        int axis = 0;
        float ra, rb, l, d;
        for (int i = 0; i < 3; i++) {
            ra = hh0 * at(ar, i) + r0;
            rb = at(he1, i);
            l = std::fabs(at(p, i));
            d = l - ra - rb;
            if (d > mx) { mx = d; edge = false; axis = i; }
        }
        const float edgeLimit = 0.999f;
        float edgeOffset = 0.1f;
        rb = he1.y * ar.z + he1.z * ar.y;
        l = std::fabs(p.z * r.y - p.y * r.z);
        d = l - r0 - rb;
        if (ar.x < edgeLimit && d > mx + edgeOffset) { mx = d; edge = true; axis = 0; edgeOffset = 0; }
        rb = he1.x * ar.z + he1.z * ar.x;
        l = std::fabs(p.x * r.z - p.z * r.x);
        d = l - r0 - rb;
        if (ar.y < edgeLimit && d > mx + edgeOffset) { mx = d; edge = true; axis = 1; edgeOffset = 0; }
        rb = he1.x * ar.y + he1.y * ar.x;
        l = std::fabs(p.y * r.x - p.x * r.y);
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

// ---------------------------------------------------------------- convex meshes

static Support convexSupport(V3 pos, Q4 ori, const ConvexMesh* m, V3 scale) {
    Support s; s.kind = 3; s.pos = pos; s.basis = mat3_cast(ori); s.mesh = m; s.scale = scale;
    return s;
}

// Collision.cpp:352-412
static void convexConvexContacts(V3 pos0, Q4 or0, const ConvexMesh* m0, V3 sc0, V3 pos1, Q4 or1, const ConvexMesh* m1,
                                 V3 sc1, V3 normal, ContactPoint* cp, int& np) {
    int f0 = 0;
    float maxDot = 0;
    for (int i = 0; i < (int)m0->faces.size(); ++i) {
        float d = dot(normal, normalize(qrot(or0, m0->faces[i].normal / sc0)));
        if (d > maxDot) { maxDot = d; f0 = i; }
    }
    const ConvexFace& F0 = m0->faces[f0];
    int f1 = 0;
    float minDot = 0;
    for (int i = 0; i < (int)m1->faces.size(); ++i) {
        float d = dot(normal, normalize(qrot(or1, m1->faces[i].normal / sc1)));
        if (d < minDot) { minDot = d; f1 = i; }
    }
    const ConvexFace& F1 = m1->faces[f1];
    M3 c0w = mat3_cast(or0);
    M3 wc0 = transpose(c0w);
    V3 refO = sc0 * F0.centroid;
    V3 u0 = normalize(sc0 * m0->buffer[F0.indices[0]] - refO);
    V3 u1 = normalize(F0.normal / sc0);
    V3 u2 = cross(u0, u1);
    M3 c0r = transpose(m3cols(u0, u1, u2));
    M3 wr = mm(c0r, wc0);
    const int cx = 2, cy = 0;
    V2 clip[kMaxPoly];
    int nc = (int)F0.indices.size();
    for (int i = 0; i < nc; ++i) {
        V3 v = mv(c0r, sc0 * m0->buffer[F0.indices[i]]);
        clip[i] = {at(v, cx), at(v, cy)};
    }
    Poly poly;
    poly.n = (int)F1.indices.size();
    for (int i = 0; i < poly.n; ++i) {
        V3 v = mv(wr, pos1 + qrot(or1, sc1 * m1->buffer[F1.indices[i]]) - pos0);
        poly.p[i] = {at(v, cx), at(v, cy)};
    }
    suthHodgClip(poly, clip, nc);
    V3 incO = mv(wr, pos1 + qrot(or1, sc1 * F1.centroid) - pos0);
    V3 incN = mv(wr, qrot(or1, normalize(F1.normal / sc1)));
    M3 rw = transpose(wr);
    generateContactsPolygonPolygonFace(pos0, rw, refO, u1, incO, incN, poly, cx, cy, cp, np);
}

// Collision.cpp:414-426
static bool convexConvex(V3 pos0, Q4 or0, const ConvexMesh* m0, V3 sc0, V3 pos1, Q4 or1, const ConvexMesh* m1, V3 sc1, Manifold& res) {
    Support a = convexSupport(pos0, or0, m0, sc0), b = convexSupport(pos1, or1, m1, sc1);
    GjkSimplex s;
    if (!gjk(a, b, pos1 - pos0, s)) return false;
    res.normal = epa(a, b, s, res.points[0].p0, res.points[0].p1);
    convexConvexContacts(pos0, or0, m0, sc0, pos1, or1, m1, sc1, res.normal, res.points, res.numPoints);
    if (!res.numPoints) res.numPoints = 1;
    return true;
}

// Collision.cpp:488-499
static bool sphereConvex(V3 pos0, float r0, V3 pos1, Q4 or1, const ConvexMesh* m1, V3 sc1, Manifold& res) {
    Support a; a.kind = 0; a.pos = pos0; a.radius = r0;
    Support b = convexSupport(pos1, or1, m1, sc1);
    GjkSimplex s;
    if (!gjk(a, b, pos1 - pos0, s)) return false;
    res.normal = epa(a, b, s, res.points[0].p0, res.points[0].p1);
    res.numPoints = 1;
    return true;
}

// Collision.cpp:694-785
static void capsuleConvexContacts(V3 p0L, V3 p1L, float radius, V3 meshPos, const M3& c2w, const ConvexMesh* m, V3 sc, Manifold& res) {
    int fi = 0;
    float minDot = 0;
    for (int i = 0; i < (int)m->faces.size(); ++i) {
        float d = dot(res.normal, normalize(mv(c2w, m->faces[i].normal / sc)));
        if (d < minDot) { minDot = d; fi = i; }
    }
    const ConvexFace& F = m->faces[fi];
    V3 refO = sc * F.centroid;
    V3 u0 = normalize(sc * m->buffer[F.indices[0]] - refO);
    V3 u1 = normalize(F.normal / sc);
    V3 u2 = cross(u0, u1);
    M3 c2r = transpose(m3cols(u0, u1, u2));
    const int fa = 1, cx = 2, cy = 0;
    V2 clip[kMaxPoly];
    int nc = (int)F.indices.size();
    for (int i = 0; i < nc; ++i) {
        V3 v = mv(c2r, sc * m->buffer[F.indices[i]]);
        clip[i] = {at(v, cx), at(v, cy)};
    }
    V3 p0R = mv(c2r, p0L), p1R = mv(c2r, p1L);
    V2 l0 = {at(p0R, cx), at(p0R, cy)}, l1 = {at(p1R, cx), at(p1R, cy)};
    if (clipLine(l0, l1, clip, nc)) {
        M3 r2w = mm(c2w, transpose(c2r));
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

// Collision.cpp:787-807
static bool capsuleConvex(V3 pos0, Q4 or0, float hh0, float r0, V3 pos1, Q4 or1, const ConvexMesh* m1, V3 sc1, Manifold& res) {
    M3 c2w = mat3_cast(or1);
    V3 axis = qrot(or0, {0, 1, 0});
    Support a; a.kind = 1; a.pos = pos0; a.axis = axis; a.halfHeight = hh0; a.radius = r0;
    Support b; b.kind = 3; b.pos = pos1; b.basis = c2w; b.mesh = m1; b.scale = sc1;
    GjkSimplex s;
    if (!gjk(a, b, pos1 - pos0, s)) return false;
    res.normal = epa(a, b, s, res.points[0].p0, res.points[0].p1);
    M3 w2c = inverse(c2w);
    V3 p = mv(w2c, pos0 - pos1);
    V3 al = mv(w2c, axis);
    capsuleConvexContacts(p + al * hh0, p - al * hh0, r0, pos1, c2w, m1, sc1, res);
    if (!res.numPoints) res.numPoints = 1;
    return true;
}

// Collision.cpp:809-871
static void boxConvexContacts(V3 boxC, const M3& basis, V3 he, V3 cPos, Q4 cOr, const ConvexMesh* m, V3 sc, V3 normal,
                              ContactPoint* cp, int& np) {
    int boxAxis = 0;
    float boxAxisSign = 0, maxDot = 0;
    for (int i = 0; i < 3; ++i) {
        float d = dot(normal, basis.c[i]);
        float ad = std::fabs(d);
        if (ad > maxDot) { maxDot = ad; boxAxis = i; boxAxisSign = d < 0 ? -1 : 1; }
    }
    int fi = 0;
    float minDot = 0;
    for (int i = 0; i < (int)m->faces.size(); ++i) {
        float d = dot(normal, normalize(qrot(cOr, m->faces[i].normal / sc)));
        if (d < minDot) { minDot = d; fi = i; }
    }
    const ConvexFace& F = m->faces[fi];
    int cx = (boxAxis + 1) % 3, cy = (boxAxis + 2) % 3;
    M3 w2b = transpose(basis);
    Poly poly;
    poly.n = (int)F.indices.size();
    for (int i = 0; i < poly.n; ++i) {
        V3 v = mv(w2b, cPos + qrot(cOr, sc * m->buffer[F.indices[i]]) - boxC);
        poly.p[i] = {at(v, cx), at(v, cy)};
    }
    V2 clip[4] = {{at(he, cx), at(he, cy)}, {at(he, cx), -at(he, cy)}, {-at(he, cx), -at(he, cy)}, {-at(he, cx), at(he, cy)}};
    suthHodgClip(poly, clip, 4);
    V3 incO = mv(w2b, cPos + qrot(cOr, sc * F.centroid) - boxC);
    V3 incN = normalize(mv(w2b, qrot(cOr, F.normal / sc)));
    generateContactsPolygonBoxFace(boxC, basis, boxAxis, (int)boxAxisSign, he, incO, incN, poly, cx, cy, cp, np);
}

// Collision.cpp:873-887
static bool boxConvex(V3 pos0, Q4 or0, V3 he0, V3 pos1, Q4 or1, const ConvexMesh* m1, V3 sc1, Manifold& res) {
    M3 basis = mat3_cast(or0);
    Support a; a.kind = 2; a.pos = pos0; a.basis = basis; a.he = he0;
    Support b = convexSupport(pos1, or1, m1, sc1);
    GjkSimplex s;
    if (!gjk(a, b, pos1 - pos0, s)) return false;
    res.normal = epa(a, b, s, res.points[0].p0, res.points[0].p1);
    boxConvexContacts(pos0, basis, he0, pos1, or1, m1, sc1, res.normal, res.points, res.numPoints);
    if (!res.numPoints) res.numPoints = 1;
    return true;
}

// Collision.cpp:889-893
static void flip(Manifold& r) {
    r.normal = -r.normal;
    for (int i = 0; i < r.numPoints; ++i) r.points[i] = {r.points[i].p1, r.points[i].p0};
}

static V3 gv(const Geometry& g) { return {g.p[0], g.p[1], g.p[2]}; }

// Collision.cpp:895-1016
bool collision(V3 pos0, Q4 or0, const Geometry& g0, V3 pos1, Q4 or1, const Geometry& g1, std::vector<Manifold>& out) {
    if (g0.type == TRIANGLE_MESH) {
        size_t first = out.size();
        bool hit = collisionTriangleMesh(pos1, or1, g1, pos0, or0, g0.tri, out);
        for (size_t i = first; i < out.size(); ++i) flip(out[i]);
        return hit;
    }
    if (g1.type == TRIANGLE_MESH) return collisionTriangleMesh(pos0, or0, g0, pos1, or1, g1.tri, out);
    out.push_back(Manifold());
    Manifold& r = out.back();
    switch (g0.type) {
        case SPHERE:
            switch (g1.type) {
                case SPHERE: return sphereSphere(pos0, g0.p[0], pos1, g1.p[0], r);
                case CAPSULE: return sphereCapsule(pos0, g0.p[0], pos1, or1, g1.p[0], g1.p[1], r);
                case BOX: return sphereBox(pos0, g0.p[0], pos1, or1, gv(g1), r);
                default: return sphereConvex(pos0, g0.p[0], pos1, or1, g1.convex, gv(g1), r);
            }
        case CAPSULE:
            switch (g1.type) {
                case SPHERE: { bool h = sphereCapsule(pos1, g1.p[0], pos0, or0, g0.p[0], g0.p[1], r); flip(r); return h; }
                case CAPSULE: return capsuleCapsule(pos0, or0, g0.p[0], g0.p[1], pos1, or1, g1.p[0], g1.p[1], r);
                case BOX: return capsuleBox(pos0, or0, g0.p[0], g0.p[1], pos1, or1, gv(g1), r);
                default: return capsuleConvex(pos0, or0, g0.p[0], g0.p[1], pos1, or1, g1.convex, gv(g1), r);
            }
        case BOX:
            switch (g1.type) {
                case SPHERE: { bool h = sphereBox(pos1, g1.p[0], pos0, or0, gv(g0), r); flip(r); return h; }
                case CAPSULE: { bool h = capsuleBox(pos1, or1, g1.p[0], g1.p[1], pos0, or0, gv(g0), r); flip(r); return h; }
                case BOX: return boxBox(pos0, or0, gv(g0), pos1, or1, gv(g1), r);
                default: return boxConvex(pos0, or0, gv(g0), pos1, or1, g1.convex, gv(g1), r);
            }
        default:
            switch (g1.type) {
                case SPHERE: { bool h = sphereConvex(pos1, g1.p[0], pos0, or0, g0.convex, gv(g0), r); flip(r); return h; }
                case CAPSULE: { bool h = capsuleConvex(pos1, or1, g1.p[0], g1.p[1], pos0, or0, g0.convex, gv(g0), r); flip(r); return h; }
                case BOX: { bool h = boxConvex(pos1, or1, gv(g1), pos0, or0, g0.convex, gv(g0), r); flip(r); return h; }
                default: return convexConvex(pos0, or0, g0.convex, gv(g0), pos1, or1, g1.convex, gv(g1), r);
            }
    }
}

}  // namespace orc
