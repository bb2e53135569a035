/*
 * query.cpp — the CPU oracle's restatement of the scene queries: Scene::raycastClosest
 * (src/Physecs.cpp:571-626 with src/Raycast.cpp) and Scene::overlap
 * (src/Physecs.cpp:628-651 with src/Overlap.cpp).
 * ORACLE (test infrastructure only; see omath.h).
 *
 * The reference walks its own dynamic BVH; the result does not depend on the tree
 * (a box that rejects a ray or a shape rejects everything inside it), so the oracle
 * tests every broadphase entry with the same leaf box test and shape test.  Among ray
 * hits at exactly the same distance the collider with the lowest index wins (the
 * reference's choice follows its tree); overlap hits come in collider order.
 */
#include <algorithm>
#include <cmath>
#include "world.h"
#include "collide_util.h"

namespace orc {
namespace {

// intersectRayAABB (Raycast.cpp:5-29)
bool rayAABB(V3 o, V3 d, V3 mn, V3 mx, float& t) {
    float tMin = 0.f, tMax = FLT_MAX;
    for (int i = 0; i < 3; ++i) {
        if (std::fabs(at(d, i)) < 0.001f) {
            if (at(o, i) < at(mn, i) || at(o, i) > at(mx, i)) return false;
        } else {
            float ood = 1.f / at(d, i);
            float t1 = (at(mn, i) - at(o, i)) * ood;
            float t2 = (at(mx, i) - at(o, i)) * ood;
            if (t1 > t2) std::swap(t1, t2);
            if (t1 > tMin) tMin = t1;
            if (t2 < tMax) tMax = t2;
            if (tMin > tMax) return false;
        }
    }
    t = tMin;
    return true;
}

// intersectRaySphere (Raycast.cpp:31-45)
bool raySphere(V3 o, V3 d, V3 pos, float radius, float& t) {
    V3 m = o - pos;
    float b = dot(m, d);
    float c = dot(m, m) - radius * radius;
    if (c > 0.f && b > 0.f) return false;
    float discr = b * b - c;
    if (discr < 0.f) return false;
    t = -b - std::sqrt(discr);
    if (t < 0.f) t = 0.f;
    return true;
}

// intersectRayCapsule (Raycast.cpp:47-102)
bool rayCapsule(V3 o, V3 dir, V3 pos, Q4 ori, float hh, float radius, float& t) {
    Q4 inv = qinverse(ori);
    V3 p = qrot(inv, o - pos);
    V3 d = qrot(inv, dir);
    float pd = dot(p, d);
    float hdy = hh * d.y;
    float thpy = 2 * hh * p.y;
    float phr = dot(p, p) + hh * hh - radius * radius;
    float tMin = FLT_MAX;
    bool hit = false;
    float b = pd - hdy, c = phr - thpy, discr = b * b - c;
    if (discr >= 0.f) {
        t = -b - std::sqrt(discr);
        if (t < 0.f) t = 0.f;
        if ((p + t * d).y >= hh) { hit = true; tMin = t; }
    }
    float a = d.x * d.x + d.z * d.z;
    b = p.x * d.x + p.z * d.z;
    c = p.x * p.x + p.z * p.z - radius * radius;
    discr = b * b - a * c;
    if (discr >= 0.f) {
        t = (-b - std::sqrt(discr)) / a;
        if (t < 0.f) t = 0.f;
        float y = (p + t * d).y;
        if (-hh <= y && y < hh && t < tMin) { hit = true; tMin = t; }
    }
    b = pd + hdy;
    c = phr + thpy;
    discr = b * b - c;
    if (discr >= 0.f) {
        t = -b - std::sqrt(discr);
        if (t < 0.f) t = 0.f;
        if ((p + t * d).y < -hh && t < tMin) { hit = true; tMin = t; }
    }
    t = tMin;
    return hit;
}

// intersectRayBox (Raycast.cpp:104-109)
bool rayBox(V3 o, V3 dir, V3 pos, Q4 ori, V3 he, float& t) {
    Q4 inv = qinverse(ori);
    return rayAABB(qrot(inv, o - pos), qrot(inv, dir), -he, he, t);
}

// intersectRayConvexMesh (Raycast.cpp:111-140)
bool rayConvex(V3 o, V3 d, V3 pos, Q4 ori, const ConvexMesh& mesh, V3 scale, float& t) {
    float tMin = 0.f, tMax = FLT_MAX;
    const V3 invScale = v3s(1.f) / scale;
    for (const ConvexFace& face : mesh.faces) {
        V3 planeOrig = pos + qrot(ori, scale * face.centroid);
        V3 planeNormal = qrot(ori, invScale * face.normal);
        float denom = dot(d, planeNormal);
        float dist = dot(planeOrig - o, planeNormal);
        if (denom == 0.f) {
            if (dist > 0) return false;
        } else {
            t = dist / denom;
            if (denom < 0) {
                if (t > tMin) tMin = t;
            } else if (t < tMax) {
                tMax = t;
            }
            if (tMin > tMax) return false;
        }
    }
    t = tMin;
    return true;
}

// intersectRayGeometry (Raycast.cpp:142-151)
bool rayGeometry(V3 o, V3 d, V3 pos, Q4 ori, const Geometry& g, float& t) {
    switch (g.type) {
        case SPHERE: return raySphere(o, d, pos, g.p[0], t);
        case CAPSULE: return rayCapsule(o, d, pos, ori, g.p[0], g.p[1], t);
        case BOX: return rayBox(o, d, pos, ori, v3(g.p[0], g.p[1], g.p[2]), t);
        case CONVEX_MESH: return rayConvex(o, d, pos, ori, *g.convex, v3(g.p[0], g.p[1], g.p[2]), t);
        default: return false;
    }
}

// ---- Overlap.cpp

bool ovSphereSphere(V3 pos0, float r0, V3 pos1, float r1) {
    V3 d = pos1 - pos0;
    float rs = r0 + r1;
    return !(dot(d, d) > rs * rs);
}

bool ovCapsuleCapsule(V3 pos0, Q4 or0, float hh0, float r0, V3 pos1, Q4 or1, float hh1, float r1) {
    V3 p0, p1;
    closestPointsBetweenSegments(pos0, qrot(or0, v3(0, 1, 0)), -hh0, hh0, pos1, qrot(or1, v3(0, 1, 0)), -hh1, hh1, p0, p1);
    V3 d = p1 - p0;
    float rs = r0 + r1;
    return !(dot(d, d) > rs * rs);
}

bool ovBoxBox(V3 pos0, Q4 or0, V3 he0, V3 pos1, Q4 or1, V3 he1) {
    M3 u0 = mat3_cast(or0), u1 = mat3_cast(or1);
    V3 tv = pos1 - pos0;
    float t[3] = {dot(tv, u0.c[0]), dot(tv, u0.c[1]), dot(tv, u0.c[2])};
    float r[3][3], ar[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            r[i][j] = dot(u0.c[i], u1.c[j]);
            ar[i][j] = std::fabs(r[i][j]);
        }
    const float a[3] = {he0.x, he0.y, he0.z}, b[3] = {he1.x, he1.y, he1.z};
    float ra, rb, l, d;
    for (int i = 0; i < 3; i++) {
        ra = a[i];
        rb = b[0] * ar[i][0] + b[1] * ar[i][1] + b[2] * ar[i][2];
        l = std::fabs(t[i]);
        d = l - ra - rb;
        if (d > 0) return false;
    }
    for (int i = 0; i < 3; i++) {
        ra = a[0] * ar[0][i] + a[1] * ar[1][i] + a[2] * ar[2][i];
        rb = b[i];
        l = std::fabs(t[0] * r[0][i] + t[1] * r[1][i] + t[2] * r[2][i]);
        d = l - ra - rb;
        if (d > 0) return false;
    }
    // A_i x B_j for i, j in 0..2, in the reference's order
    for (int i = 0; i < 3; ++i) {
        const int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
        for (int j = 0; j < 3; ++j) {
            const int j1 = (j + 1) % 3, j2 = (j + 2) % 3;
            // the reference spells the nine axes out; with (i1, i2) and (j1, j2) the cyclic
            // successors, axis A_i x B_j has
            //   ra = a[lo(i1,i2)] * ar[hi][j] + a[hi(i1,i2)] * ar[lo][j]
            //   rb = b[lo(j1,j2)] * ar[i][hi] + b[hi(j1,j2)] * ar[i][lo]
            //   l  = |t[i2] * r[i1][j] - t[i1] * r[i2][j]|
            const int ia = i1 < i2 ? i1 : i2, ib = i1 < i2 ? i2 : i1;
            const int ja = j1 < j2 ? j1 : j2, jb = j1 < j2 ? j2 : j1;
            ra = a[ia] * ar[ib][j] + a[ib] * ar[ia][j];
            rb = b[ja] * ar[i][jb] + b[jb] * ar[i][ja];
            l = std::fabs(t[i2] * r[i1][j] - t[i1] * r[i2][j]);
            d = l - ra - rb;
            if (d > 0) return false;
        }
    }
    return true;
}

bool ovSphereCapsule(V3 pos0, float r0, V3 pos1, Q4 or1, float hh1, float r1) {
    V3 q = closestPointOnSegment(pos0, pos1, qrot(or1, v3(0, 1, 0)), -hh1, hh1);
    V3 v = q - pos0;
    float rs = r0 + r1;
    return !(dot(v, v) > rs * rs);
}

bool ovSphereBox(V3 pos0, float r0, V3 pos1, Q4 or1, V3 he1) {
    M3 u1 = mat3_cast(or1);
    V3 d = pos0 - pos1;
    d = v3(dot(d, u1.c[0]), dot(d, u1.c[1]), dot(d, u1.c[2]));
    V3 q = pos1 + mv(u1, vclamp(d, -he1, he1));
    V3 v = q - pos0;
    return !(dot(v, v) > r0 * r0);
}

bool ovCapsuleBox(V3 pos0, Q4 or0, float hh0, float r0, V3 pos1, Q4 or1, V3 he1) {
    M3 u1 = mat3_cast(or1);
    V3 p = pos0 - pos1;
    p = v3(dot(p, u1.c[0]), dot(p, u1.c[1]), dot(p, u1.c[2]));
    V3 dir = qrot(or0, v3(0, 1, 0));
    V3 dirLc = v3(dot(dir, u1.c[0]), dot(dir, u1.c[1]), dot(dir, u1.c[2]));
    float t;
    V3 q;
    return !(sqrDistSegmentAABB(p, dirLc, -hh0, hh0, he1, t, q) >= r0 * r0);
}

Support sphereSup(V3 pos, float r) { Support s; s.kind = 0; s.pos = pos; s.radius = r; return s; }
Support capsuleSup(V3 pos, Q4 ori, float hh, float r) {
    Support s; s.kind = 1; s.pos = pos; s.axis = qrot(ori, v3(0, 1, 0)); s.halfHeight = hh; s.radius = r; return s;
}
Support boxSup(V3 pos, Q4 ori, V3 he) { Support s; s.kind = 2; s.pos = pos; s.basis = mat3_cast(ori); s.he = he; return s; }
Support convexSup(V3 pos, Q4 ori, const Geometry& g) {
    Support s; s.kind = 3; s.pos = pos; s.basis = mat3_cast(ori); s.mesh = g.convex; s.scale = v3(g.p[0], g.p[1], g.p[2]); return s;
}
bool ovGjk(const Support& a, const Support& b, V3 dir) { GjkSimplex s; return gjk(a, b, dir, s); }

// physecs::overlap (Overlap.cpp:194-235), box / convex mesh with the mesh's support at
// the box's position as overlapBoxConvexMesh has it (Overlap.cpp:190)
bool overlapGeom(V3 pos0, Q4 or0, const Geometry& g0, V3 pos1, Q4 or1, const Geometry& g1) {
    const V3 e0 = v3(g0.p[0], g0.p[1], g0.p[2]), e1 = v3(g1.p[0], g1.p[1], g1.p[2]);
    if (g0.type > CONVEX_MESH || g1.type > CONVEX_MESH) return false;
    switch (g0.type) {
        case SPHERE:
            if (g1.type == SPHERE) return ovSphereSphere(pos0, g0.p[0], pos1, g1.p[0]);
            if (g1.type == CAPSULE) return ovSphereCapsule(pos0, g0.p[0], pos1, or1, g1.p[0], g1.p[1]);
            if (g1.type == BOX) return ovSphereBox(pos0, g0.p[0], pos1, or1, e1);
            return ovGjk(sphereSup(pos0, g0.p[0]), convexSup(pos1, or1, g1), pos1 - pos0);
        case CAPSULE:
            if (g1.type == SPHERE) return ovSphereCapsule(pos1, g1.p[0], pos0, or0, g0.p[0], g0.p[1]);
            if (g1.type == CAPSULE) return ovCapsuleCapsule(pos0, or0, g0.p[0], g0.p[1], pos1, or1, g1.p[0], g1.p[1]);
            if (g1.type == BOX) return ovCapsuleBox(pos0, or0, g0.p[0], g0.p[1], pos1, or1, e1);
            return ovGjk(capsuleSup(pos0, or0, g0.p[0], g0.p[1]), convexSup(pos1, or1, g1), pos1 - pos0);
        case BOX:
            if (g1.type == SPHERE) return ovSphereBox(pos1, g1.p[0], pos0, or0, e0);
            if (g1.type == CAPSULE) return ovCapsuleBox(pos1, or1, g1.p[0], g1.p[1], pos0, or0, e0);
            if (g1.type == BOX) return ovBoxBox(pos0, or0, e0, pos1, or1, e1);
            return ovGjk(boxSup(pos0, or0, e0), convexSup(pos0, or1, g1), pos1 - pos0);
        default:
            if (g1.type == SPHERE) return ovGjk(sphereSup(pos1, g1.p[0]), convexSup(pos0, or0, g0), pos0 - pos1);
            if (g1.type == CAPSULE) return ovGjk(capsuleSup(pos1, or1, g1.p[0], g1.p[1]), convexSup(pos0, or0, g0), pos0 - pos1);
            if (g1.type == BOX) return ovGjk(boxSup(pos1, or1, e1), convexSup(pos1, or0, g0), pos0 - pos1);
            return ovGjk(convexSup(pos0, or0, g0), convexSup(pos1, or1, g1), pos1 - pos0);
    }
}

bool boundsMeet(const Bounds& a, const Bounds& b) {
    return a.max.x >= b.min.x && a.min.x <= b.max.x && a.max.y >= b.min.y && a.min.y <= b.max.y && a.max.z >= b.min.z &&
           a.min.z <= b.max.z;
}

}  // namespace

int World::raycastClosest(V3 o, V3 d, float maxd, const uint8_t* accept, float& dist) const {
    int best = -1;
    float bestT = FLT_MAX;
    for (const BPEntry& e : bp) {
        const int c = bodies[e.body].cols[e.col];
        float t;
        if (!rayAABB(o, d, e.b.min, e.b.max, t) || t > maxd) continue;
        if (!rayGeometry(o, d, colPos(c), colQ(c), colliders[c].g, t) || t > maxd) continue;
        if (accept && !accept[e.body]) continue;
        if (t < bestT || (t == bestT && c < best)) { bestT = t; best = c; }
    }
    dist = bestT;
    return best;
}

void World::overlap(V3 pos, Q4 ori, const Geometry& g, int filter, std::vector<int>& out) const {
    const Bounds qb = getBounds(pos, ori, g);
    out.clear();
    for (const BPEntry& e : bp) {
        const int c = bodies[e.body].cols[e.col];
        if (!boundsMeet(qb, e.b)) continue;
        if (filter && !(colliders[c].data & filter)) continue;
        if (!overlapGeom(pos, ori, g, colPos(c), colQ(c), colliders[c].g)) continue;
        out.push_back(c);
    }
    std::sort(out.begin(), out.end());
}

// Scene::overlapWithMinTranslationalDistance (src/Physecs.cpp:653-688): the collision of
// every collider whose bounds meet the shape's (collider first), one record per manifold
// with points, its deepest point max(0, dot(p0 - p1, n))
bool World::overlapColliders(V3 pos0, Q4 or0, int c0, V3 pos1, Q4 or1, int c1) const {
    return overlapGeom(pos0, or0, colliders[c0].g, pos1, or1, colliders[c1].g);
}

// CharacterController::move (CharacterController.cpp:5-45).  Its step-up test calls
// Scene::raycastClosest without a filter, which never reports a hit (Physecs.cpp:580,
// 615), so the translation always stays as given; maxStepHeight is never read.  The hits
// of one iteration apply in the order (collider, triangle); the reference applies them in
// its query tree's order, which only changes the rounding of the summed moves.
int World::moveCharacter(int b, float height, float radius, float maxStepHeight, float slopeLimit, int iterations,
                         V3 translation) {
    (void)maxStepHeight;
    Body& B = bodies[b];
    const V3 up = qrot(B.q, v3(0, 1, 0));
    B.pos += translation;
    int flags = 0;
    Geometry g;
    g.type = CAPSULE;
    g.p[0] = height * 0.5f;
    g.p[1] = radius;
    g.p[2] = 0.f;
    std::vector<MtdHit> hits;
    for (int i = 0; i < iterations; ++i) {
        overlapMtd(B.pos + up * (height * 0.5f + radius), B.q, g, hits);
        std::stable_sort(hits.begin(), hits.end(), [](const MtdHit& x, const MtdHit& y) {
            return x.col < y.col || (x.col == y.col && x.tri < y.tri);
        });
        for (const MtdHit& h : hits) {
            const float d = dot(h.n, up);
            if (d > 0.001f) flags |= 1;
            else if (d < -0.001f) flags |= 4;
            else flags |= 2;
            if (d > slopeLimit) B.pos += up * h.mtd / d;
            else B.pos += h.n * h.mtd;
        }
    }
    updateBounds(b, true);   // registry.patch<TransformComponent> -> onRigidBodyMove
    return flags;
}

void World::overlapMtd(V3 pos, Q4 ori, const Geometry& g, std::vector<MtdHit>& out) const {
    const Bounds qb = getBounds(pos, ori, g);
    out.clear();
    for (const BPEntry& e : bp) {
        const int c = bodies[e.body].cols[e.col];
        if (!boundsMeet(qb, e.b)) continue;
        std::vector<Manifold> res;
        if (!collision(colPos(c), colQ(c), colliders[c].g, pos, ori, g, res)) continue;
        for (const Manifold& m : res) {
            if (!m.numPoints) continue;
            float mtd = 0;
            for (int i = 0; i < m.numPoints; ++i) {
                float dist = dot(m.points[i].p0 - m.points[i].p1, m.normal);
                if (dist > mtd) mtd = dist;
            }
            out.push_back({c, m.normal, mtd, m.triangleIndex});
        }
    }
}

}  // namespace orc
