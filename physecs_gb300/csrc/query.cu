// query.cu — batched scene queries against each scene's LBVH: the closest ray hit
// (Scene::raycastClosest, src/Physecs.cpp:571-626, with src/Raycast.cpp) and the
// colliders a shape overlaps (Scene::overlap, src/Physecs.cpp:628-651, with
// src/Overlap.cpp).  One thread per query; every query of a batch reads the same
// tree, built over the colliders' current bounds with every collider as a leaf (the
// reference's query tree holds every collider, whether it simulates or not).
//
// The tests restate the reference's arithmetic and its branch order.  Two places
// where the reference's result depends on its own tree's shape get a fixed rule
// here: among ray hits at exactly the same distance the collider with the lowest
// world index wins (the reference takes its right subtree's on a tie), and overlap
// hits are listed in tree order of this LBVH (the reference lists them in its tree's
// order; the set is the same).
#include "frame.cuh"
#include "narrow_convex.cuh"
#include "narrow_tri.cuh"

namespace psx {

// ---------------------------------------------------------------- rays (Raycast.cpp)

// intersectRayAABB (Raycast.cpp:5-29): slab test from t = 0; an axis the ray runs
// nearly parallel to (|d| < 0.001) rejects an origin outside its slab
__device__ inline bool rayAABB(V3 o, V3 d, V3 mn, V3 mx, float& t) {
    const float oc[3] = {o.x, o.y, o.z}, dc[3] = {d.x, d.y, d.z};
    const float lo[3] = {mn.x, mn.y, mn.z}, hi[3] = {mx.x, mx.y, mx.z};
    float tMin = 0.f, tMax = FLT_MAX;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        if (fabsf(dc[i]) < 0.001f) {
            if (oc[i] < lo[i] || oc[i] > hi[i]) return false;
        } else {
            const float ood = 1.f / dc[i];
            float t1 = (lo[i] - oc[i]) * ood;
            float t2 = (hi[i] - oc[i]) * ood;
            if (t1 > t2) { float tt = t1; t1 = t2; t2 = tt; }
            if (t1 > tMin) tMin = t1;
            if (t2 < tMax) tMax = t2;
            if (tMin > tMax) return false;
        }
    }
    t = tMin;
    return true;
}

// intersectRaySphere (Raycast.cpp:31-45)
__device__ inline bool raySphere(V3 o, V3 d, V3 pos, float radius, float& t) {
    V3 m = o - pos;
    float b = dot(m, d);
    float c = dot(m, m) - radius * radius;
    if (c > 0.f && b > 0.f) return false;
    float discr = b * b - c;
    if (discr < 0.f) return false;
    t = -b - sqrtf(discr);
    if (t < 0.f) t = 0.f;
    return true;
}

// intersectRayCapsule (Raycast.cpp:47-102): the two hemispheres and the cylinder,
// in the capsule's frame
__device__ inline bool rayCapsule(V3 o, V3 dir, V3 pos, Q4 ori, float hh, float radius, float& t) {
    Q4 inv = qinverse(ori);
    V3 p = qrot(inv, o - pos);
    V3 d = qrot(inv, dir);
    float pd = dot(p, d);
    float hdy = hh * d.y;
    float thpy = 2 * hh * p.y;
    float phr = dot(p, p) + hh * hh - radius * radius;
    float tMin = FLT_MAX;
    bool hit = false;
    float b, c, discr;
    b = pd - hdy;
    c = phr - thpy;
    discr = b * b - c;
    if (discr >= 0.f) {
        t = -b - sqrtf(discr);
        if (t < 0.f) t = 0.f;
        if ((p + t * d).y >= hh) { hit = true; tMin = t; }
    }
    float a = d.x * d.x + d.z * d.z;
    b = p.x * d.x + p.z * d.z;
    c = p.x * p.x + p.z * p.z - radius * radius;
    discr = b * b - a * c;
    if (discr >= 0.f) {
        t = (-b - sqrtf(discr)) / a;
        if (t < 0.f) t = 0.f;
        float y = (p + t * d).y;
        if (-hh <= y && y < hh && t < tMin) { hit = true; tMin = t; }
    }
    b = pd + hdy;
    c = phr + thpy;
    discr = b * b - c;
    if (discr >= 0.f) {
        t = -b - sqrtf(discr);
        if (t < 0.f) t = 0.f;
        if ((p + t * d).y < -hh && t < tMin) { hit = true; tMin = t; }
    }
    t = tMin;
    return hit;
}

// intersectRayBox (Raycast.cpp:104-109)
__device__ inline bool rayBox(V3 o, V3 dir, V3 pos, Q4 ori, V3 he, float& t) {
    Q4 inv = qinverse(ori);
    V3 p = qrot(inv, o - pos);
    V3 d = qrot(inv, dir);
    return rayAABB(p, d, -he, he, t);
}

// intersectRayConvexMesh (Raycast.cpp:111-140): clip the ray against every face plane
__device__ inline bool rayConvex(const World& w, V3 o, V3 d, V3 pos, Q4 ori, int mesh, V3 scale, float& t) {
    const ConvexMeshDev cm = w.convex[mesh];
    const V3 invScale = {1.f / scale.x, 1.f / scale.y, 1.f / scale.z};   // glm::vec3(1) / scale
    float tMin = 0.f, tMax = FLT_MAX;
    for (int i = 0; i < cm.face_count; ++i) {
        V3 planeOrig = pos + qrot(ori, scale * ld3(w.face_centroid[cm.face_start + i]));
        V3 planeNormal = qrot(ori, invScale * ld3(w.face_normal[cm.face_start + i]));
        float denom = dot(d, planeNormal);
        float dist = dot(planeOrig - o, planeNormal);
        if (denom == 0.f) {
            if (dist > 0) return false;
        } else {
            t = dist / denom;
            if (denom < 0) {
                if (t > tMin) tMin = t;
            } else {
                if (t < tMax) tMax = t;
            }
            if (tMin > tMax) return false;
        }
    }
    t = tMin;
    return true;
}

// intersectRayGeometry (Raycast.cpp:142-151): a triangle mesh is never hit
__device__ inline bool rayGeometry(const World& w, V3 o, V3 d, V3 pos, Q4 ori, const GeomD& g, float& t) {
    switch (g.type) {
        case G_SPHERE: return raySphere(o, d, pos, g.p[0], t);
        case G_CAPSULE: return rayCapsule(o, d, pos, ori, g.p[0], g.p[1], t);
        case G_BOX: return rayBox(o, d, pos, ori, gv(g), t);
        case G_CONVEX: return rayConvex(w, o, d, pos, ori, g.mesh, gv(g), t);
        default: return false;
    }
}

// ---------------------------------------------------------------- overlap (Overlap.cpp)

__device__ inline bool ovSphereSphere(V3 pos0, float r0, V3 pos1, float r1) {
    V3 d = pos1 - pos0;
    float rs = r0 + r1;
    return !(dot(d, d) > rs * rs);
}

__device__ inline bool ovCapsuleCapsule(V3 pos0, Q4 or0, float hh0, float r0, V3 pos1, Q4 or1, float hh1, float r1) {
    V3 v0 = qrot(or0, {0, 1, 0}), v1 = qrot(or1, {0, 1, 0});
    V3 p0, p1;
    closestPointsBetweenSegments(pos0, v0, -hh0, hh0, pos1, v1, -hh1, hh1, p0, p1);
    V3 d = p1 - p0;
    float rs = r0 + r1;
    return !(dot(d, d) > rs * rs);
}

// separating-axis test of two boxes (Overlap.cpp:37-144)
__device__ inline bool ovBoxBox(V3 pos0, Q4 or0, V3 he0, V3 pos1, Q4 or1, V3 he1) {
    const M3 u0 = mat3_cast(or0), u1 = mat3_cast(or1);
    V3 tv = pos1 - pos0;
    const float t[3] = {dot(tv, u0.c[0]), dot(tv, u0.c[1]), dot(tv, u0.c[2])};
    float r[3][3], ar[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            r[i][j] = dot(u0.c[i], u1.c[j]);
            ar[i][j] = fabsf(r[i][j]);
        }
    const float a[3] = {he0.x, he0.y, he0.z}, b[3] = {he1.x, he1.y, he1.z};
    float ra, rb, l, d;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        ra = a[i];
        rb = b[0] * ar[i][0] + b[1] * ar[i][1] + b[2] * ar[i][2];
        l = fabsf(t[i]);
        d = l - ra - rb;
        if (d > 0) return false;
    }
#pragma unroll
    for (int i = 0; i < 3; i++) {
        ra = a[0] * ar[0][i] + a[1] * ar[1][i] + a[2] * ar[2][i];
        rb = b[i];
        l = fabsf(t[0] * r[0][i] + t[1] * r[1][i] + t[2] * r[2][i]);
        d = l - ra - rb;
        if (d > 0) return false;
    }
    // the nine edge-edge axes, A_i x B_j, in the reference's order
    ra = a[1] * ar[2][0] + a[2] * ar[1][0]; rb = b[1] * ar[0][2] + b[2] * ar[0][1];
    l = fabsf(t[2] * r[1][0] - t[1] * r[2][0]); d = l - ra - rb; if (d > 0) return false;
    ra = a[1] * ar[2][1] + a[2] * ar[1][1]; rb = b[0] * ar[0][2] + b[2] * ar[0][0];
    l = fabsf(t[2] * r[1][1] - t[1] * r[2][1]); d = l - ra - rb; if (d > 0) return false;
    ra = a[1] * ar[2][2] + a[2] * ar[1][2]; rb = b[0] * ar[0][1] + b[1] * ar[0][0];
    l = fabsf(t[2] * r[1][2] - t[1] * r[2][2]); d = l - ra - rb; if (d > 0) return false;
    ra = a[0] * ar[2][0] + a[2] * ar[0][0]; rb = b[1] * ar[1][2] + b[2] * ar[1][1];
    l = fabsf(t[0] * r[2][0] - t[2] * r[0][0]); d = l - ra - rb; if (d > 0) return false;
    ra = a[0] * ar[2][1] + a[2] * ar[0][1]; rb = b[0] * ar[1][2] + b[2] * ar[1][0];
    l = fabsf(t[0] * r[2][1] - t[2] * r[0][1]); d = l - ra - rb; if (d > 0) return false;
    ra = a[0] * ar[2][2] + a[2] * ar[0][2]; rb = b[0] * ar[1][1] + b[1] * ar[1][0];
    l = fabsf(t[0] * r[2][2] - t[2] * r[0][2]); d = l - ra - rb; if (d > 0) return false;
    ra = a[0] * ar[1][0] + a[1] * ar[0][0]; rb = b[1] * ar[2][2] + b[2] * ar[2][1];
    l = fabsf(t[1] * r[0][0] - t[0] * r[1][0]); d = l - ra - rb; if (d > 0) return false;
    ra = a[0] * ar[1][1] + a[1] * ar[0][1]; rb = b[0] * ar[2][2] + b[2] * ar[2][0];
    l = fabsf(t[1] * r[0][1] - t[0] * r[1][1]); d = l - ra - rb; if (d > 0) return false;
    ra = a[0] * ar[1][2] + a[1] * ar[0][2]; rb = b[0] * ar[2][1] + b[1] * ar[2][0];
    l = fabsf(t[1] * r[0][2] - t[0] * r[1][2]); d = l - ra - rb; if (d > 0) return false;
    return true;
}

__device__ inline bool ovSphereCapsule(V3 pos0, float r0, V3 pos1, Q4 or1, float hh1, float r1) {
    V3 dir = qrot(or1, {0, 1, 0});
    V3 q = closestPointOnSegment(pos0, pos1, dir, -hh1, hh1);
    V3 v = q - pos0;
    float rs = r0 + r1;
    return !(dot(v, v) > rs * rs);
}

__device__ inline bool ovSphereBox(V3 pos0, float r0, V3 pos1, Q4 or1, V3 he1) {
    M3 u1 = mat3_cast(or1);
    V3 d = pos0 - pos1;
    d = {dot(d, u1.c[0]), dot(d, u1.c[1]), dot(d, u1.c[2])};
    V3 q = pos1 + mv(u1, vclamp(d, -he1, he1));
    V3 v = q - pos0;
    return !(dot(v, v) > r0 * r0);
}

__device__ inline bool ovCapsuleBox(V3 pos0, Q4 or0, float hh0, float r0, V3 pos1, Q4 or1, V3 he1) {
    M3 u1 = mat3_cast(or1);
    V3 p = pos0 - pos1;
    p = {dot(p, u1.c[0]), dot(p, u1.c[1]), dot(p, u1.c[2])};
    V3 dir = qrot(or0, {0, 1, 0});
    V3 dirLc = {dot(dir, u1.c[0]), dot(dir, u1.c[1]), dot(dir, u1.c[2])};
    float t;
    V3 q;
    float sqrDist = sqrDistSegmentAABB(p, dirLc, -hh0, hh0, he1, t, q);
    return !(sqrDist >= r0 * r0);
}

__device__ __forceinline__ Support sphereSupportOf(V3 pos, float r) {
    Support s;
    s.kind = 0; s.pos = pos; s.radius = r;
    return s;
}
__device__ __forceinline__ Support capsuleSupportOf(V3 pos, Q4 ori, float hh, float r) {
    Support s;
    s.kind = 1; s.pos = pos; s.axis = qrot(ori, {0, 1, 0}); s.halfHeight = hh; s.radius = r;
    return s;
}
__device__ __forceinline__ Support boxSupportOf(V3 pos, Q4 ori, V3 he) {
    Support s;
    s.kind = 2; s.pos = pos; s.basis = mat3_cast(ori); s.he = he;
    return s;
}
// GJK<A, B>::gjk(a, b, startDir) as an overlap test (Overlap.cpp:146-148, 160-162, 186-192)
__device__ __forceinline__ bool ovGjk(const Support& a, const Support& b, V3 startDir) {
    GjkSimplex s;
    return gjk(a, b, startDir, s);
}

// physecs::overlap (Overlap.cpp:194-235).  A pair with a triangle mesh falls through
// every case and is never reported.  The box / convex-mesh test places the mesh's
// support at the box's position, as overlapBoxConvexMesh does (Overlap.cpp:190).
__device__ inline bool overlapGeom(const World& w, V3 pos0, Q4 or0, const GeomD& g0, V3 pos1, Q4 or1, const GeomD& g1) {
    const int t0 = g0.type, t1 = g1.type;
    if (t0 > G_CONVEX || t1 > G_CONVEX) return false;
    if (t0 == G_SPHERE) {
        if (t1 == G_SPHERE) return ovSphereSphere(pos0, g0.p[0], pos1, g1.p[0]);
        if (t1 == G_CAPSULE) return ovSphereCapsule(pos0, g0.p[0], pos1, or1, g1.p[0], g1.p[1]);
        if (t1 == G_BOX) return ovSphereBox(pos0, g0.p[0], pos1, or1, gv(g1));
        return ovGjk(sphereSupportOf(pos0, g0.p[0]), convexSupport(w, pos1, or1, g1.mesh, gv(g1)), pos1 - pos0);
    }
    if (t0 == G_CAPSULE) {
        if (t1 == G_SPHERE) return ovSphereCapsule(pos1, g1.p[0], pos0, or0, g0.p[0], g0.p[1]);
        if (t1 == G_CAPSULE) return ovCapsuleCapsule(pos0, or0, g0.p[0], g0.p[1], pos1, or1, g1.p[0], g1.p[1]);
        if (t1 == G_BOX) return ovCapsuleBox(pos0, or0, g0.p[0], g0.p[1], pos1, or1, gv(g1));
        return ovGjk(capsuleSupportOf(pos0, or0, g0.p[0], g0.p[1]), convexSupport(w, pos1, or1, g1.mesh, gv(g1)), pos1 - pos0);
    }
    if (t0 == G_BOX) {
        if (t1 == G_SPHERE) return ovSphereBox(pos1, g1.p[0], pos0, or0, gv(g0));
        if (t1 == G_CAPSULE) return ovCapsuleBox(pos1, or1, g1.p[0], g1.p[1], pos0, or0, gv(g0));
        if (t1 == G_BOX) return ovBoxBox(pos0, or0, gv(g0), pos1, or1, gv(g1));
        return ovGjk(boxSupportOf(pos0, or0, gv(g0)), convexSupport(w, pos0, or1, g1.mesh, gv(g1)), pos1 - pos0);
    }
    // convex mesh first: the other shape's routine with the mesh second
    if (t1 == G_SPHERE) return ovGjk(sphereSupportOf(pos1, g1.p[0]), convexSupport(w, pos0, or0, g0.mesh, gv(g0)), pos0 - pos1);
    if (t1 == G_CAPSULE)
        return ovGjk(capsuleSupportOf(pos1, or1, g1.p[0], g1.p[1]), convexSupport(w, pos0, or0, g0.mesh, gv(g0)), pos0 - pos1);
    if (t1 == G_BOX) return ovGjk(boxSupportOf(pos1, or1, gv(g1)), convexSupport(w, pos1, or0, g0.mesh, gv(g0)), pos0 - pos1);
    return ovGjk(convexSupport(w, pos0, or0, g0.mesh, gv(g0)), convexSupport(w, pos1, or1, g1.mesh, gv(g1)), pos1 - pos0);
}

// ---------------------------------------------------------------- kernels

__device__ __forceinline__ bool boxes_meet(float4 amin, float4 amax, float4 bmin, float4 bmax) {
    return amax.x >= bmin.x && amin.x <= bmax.x && amax.y >= bmin.y && amin.y <= bmax.y && amax.z >= bmin.z &&
           amin.z <= bmax.z;
}
__device__ __forceinline__ V3 f3of(float4 v) { return {v.x, v.y, v.z}; }

// Closest accepted hit within max distance of each ray: the node and leaf box tests
// prune as the reference's do (a box entered beyond the max distance, or beyond the
// best hit so far, holds no better hit), then the collider's shape test decides.
__global__ void k_raycast(World w, FrameBuf f, const RayIn* rays, int n, const unsigned char* accept, RayOut* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const RayIn r = rays[i];
    const V3 o = {r.ox, r.oy, r.oz}, d = {r.dx, r.dy, r.dz};
    const int s = r.scene;
    const int cs = w.scene_col[s], nc = w.scene_col[s + 1] - cs;
    float best = FLT_MAX;
    int bestc = -1;
    float bestt = 0.f;
    auto leaf = [&](int q) {
        const int c = f.order[q];
        float t;
        if (!rayAABB(o, d, f3of(w.aabb_min[c]), f3of(w.aabb_max[c]), t) || t > r.maxd || t > best) return;
        V3 pos;
        Q4 ori;
        GeomD g;
        collider_pose(w, c, pos, ori, g);
        if (!rayGeometry(w, o, d, pos, ori, g, t) || t > r.maxd) return;
        if (accept && !accept[w.col_info[c].x]) return;
        if (t < best || (t == best && c < bestc)) { best = t; bestc = c; bestt = t; }
    };
    if (nc == 1) {
        leaf(cs);
    } else if (nc > 1) {
        int stack[64];
        int sp = 0;
        stack[sp++] = cs - s;   // root of this scene's tree
        while (sp) {
            const int c = stack[--sp];
            if (c < 0) { leaf(~c); continue; }
            float t;
            if (!rayAABB(o, d, f3of(f.bvh.bmin[c]), f3of(f.bvh.bmax[c]), t) || t > r.maxd || t > best) continue;
            if (sp + 2 > 64) { atomicOr(w.err, ERR_STACK_CAPACITY); continue; }
            stack[sp++] = f.bvh.right[c];
            stack[sp++] = f.bvh.left[c];
        }
    }
    out[i] = RayOut{bestc, bestt};
}

// Every collider whose bounds meet the query shape's bounds, whose data bits meet the
// filter (0: any) and whose shape overlaps the query's; up to cap hits a query.
__global__ void k_overlap(World w, FrameBuf f, const ShapeIn* qs, int n, int cap, int* counts, int* hits) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const ShapeIn qi = qs[i];
    const V3 pos = {qi.px, qi.py, qi.pz};
    const Q4 ori = {qi.qx, qi.qy, qi.qz, qi.qw};
    const GeomD g = GeomD{qi.type, {qi.p0, qi.p1, qi.p2}, qi.mesh};
    const Bounds b = getBounds(w, pos, ori, g);
    const float4 qmin = make_float4(b.min.x, b.min.y, b.min.z, 0.f), qmax = make_float4(b.max.x, b.max.y, b.max.z, 0.f);
    const int s = qi.scene;
    const int cs = w.scene_col[s], nc = w.scene_col[s + 1] - cs;
    int count = 0;
    auto leaf = [&](int q) {
        const int c = f.order[q];
        if (!boxes_meet(qmin, qmax, w.aabb_min[c], w.aabb_max[c])) return;
        if (qi.filter && !(__float_as_int(w.col_mat[c].w) & qi.filter)) return;
        V3 cp;
        Q4 co;
        GeomD cg;
        collider_pose(w, c, cp, co, cg);
        if (!overlapGeom(w, pos, ori, g, cp, co, cg)) return;
        if (count < cap) hits[(size_t)i * cap + count] = c;
        ++count;
    };
    if (nc == 1) {
        leaf(cs);
    } else if (nc > 1) {
        int stack[64];
        int sp = 0;
        stack[sp++] = cs - s;
        while (sp) {
            const int c = stack[--sp];
            if (c < 0) { leaf(~c); continue; }
            if (!boxes_meet(qmin, qmax, f.bvh.bmin[c], f.bvh.bmax[c])) continue;
            if (sp + 2 > 64) { atomicOr(w.err, ERR_STACK_CAPACITY); continue; }
            stack[sp++] = f.bvh.right[c];
            stack[sp++] = f.bvh.left[c];
        }
    }
    counts[i] = count;
}

// physecs::collision (Collision.cpp:895-1016) for one pair in one thread: the triangle-
// mesh routine (its manifolds flipped when the mesh is the first shape), the convex
// routine (GJK, EPA and face clipping, with the convex mesh second) or the analytic
// one.  Up to kTriManifolds manifolds go to ms; returns their number.
__device__ inline int collision_one(const World& w, V3 pos0, Q4 or0, GeomD g0, V3 pos1, Q4 or1, GeomD g1, ManifoldL* ms,
                                    TCI* cand, Polytope& poly, int* err) {
    if (g0.type == G_TRIMESH || g1.type == G_TRIMESH) {
        if (g0.type == G_TRIMESH && g1.type == G_TRIMESH) return 0;
        ManOut out{ms, 0, kTriManifolds, err};
        const bool flip = g0.type == G_TRIMESH;
        if (flip) collideTriMesh(w, pos1, or1, g1, pos0, or0, g0.mesh, out, cand, poly);
        else collideTriMesh(w, pos0, or0, g0, pos1, or1, g1.mesh, out, cand, poly);
        if (flip)
            for (int k = 0; k < out.n; ++k) flipM(ms[k]);
        return out.n;
    }
    if (g0.type == G_CONVEX || g1.type == G_CONVEX) {
        const bool swap = g1.type != G_CONVEX;
        if (swap) {
            V3 tp = pos0; pos0 = pos1; pos1 = tp;
            Q4 tq = or0; or0 = or1; or1 = tq;
            GeomD tg = g0; g0 = g1; g1 = tg;
        }
        Support a, b;
        convexOrderedSupports(w, pos0, or0, g0, pos1, or1, g1, a, b);
        GjkSimplex s;
        if (!gjk(a, b, pos1 - pos0, s)) return 0;
        ManifoldL& r = ms[0];
        r.numPoints = 0;
        r.triangleIndex = -1;
        V3 c0, c1;
        r.normal = epa(a, b, s, c0, c1, poly, err);
        r.points[0] = {c0, c1};
        convexOrderedContacts(w, pos0, or0, g0, pos1, or1, g1, r, err);
        if (swap) flipM(r);
        return 1;
    }
    return collideAnalytic(pos0, or0, g0, pos1, or1, g1, ms[0], err) ? 1 : 0;
}

// Scene::overlapWithMinTranslationalDistance (src/Physecs.cpp:653-688): every collider
// whose bounds meet the query shape's; for each manifold with points of the collision
// (collider first, shape second) its normal and the deepest point, max(0, max over the
// points of dot(p0 - p1, n)).  Up to cap records a query: {world collider, n xyz, mtd}.
// The MTD query of overlapWithMinTranslationalDistance: every collider of scene s whose
// bounds meet the shape's, collided with the collider first; fn(collider, manifold, mtd)
// for each manifold with points, mtd = max(0, deepest dot(p0 - p1, normal)).  The walk
// visits the scene's tree left first.
// self_body (>= 0): a body whose colliders are posed at self_pos instead of its stored
// position, while their bounds stay the stored ones (a character controller's entity,
// moved in the registry but not yet patched).
template <class F>
__device__ void for_each_mtd(const World& w, const FrameBuf& f, int s, V3 pos, Q4 ori, const GeomD& g, ManifoldL* ms,
                             TCI* cand, Polytope& poly, F&& fn, int self_body = -1, V3 self_pos = V3{0.f, 0.f, 0.f}) {
    const Bounds b = getBounds(w, pos, ori, g);
    const float4 qmin = make_float4(b.min.x, b.min.y, b.min.z, 0.f), qmax = make_float4(b.max.x, b.max.y, b.max.z, 0.f);
    const int cs = w.scene_col[s], nc = w.scene_col[s + 1] - cs;
    auto leaf = [&](int q) {
        const int c = f.order[q];
        if (!boxes_meet(qmin, qmax, w.aabb_min[c], w.aabb_max[c])) return;
        V3 cp;
        Q4 co;
        GeomD cg;
        collider_pose(w, c, cp, co, cg);
        if (w.col_info[c].x == self_body) cp = self_pos + qrot(ld4(w.quat[self_body]), ld3(w.col_pos[c]));
        const int nm = collision_one(w, cp, co, cg, pos, ori, g, ms, cand, poly, w.err);
        for (int k = 0; k < nm; ++k) {
            const ManifoldL& m = ms[k];
            if (!m.numPoints) continue;
            float mtd = 0.f;
            for (int p = 0; p < m.numPoints; ++p) {
                float dist = dot(m.points[p].p0 - m.points[p].p1, m.normal);
                if (dist > mtd) mtd = dist;
            }
            fn(c, m, mtd);
        }
    };
    if (nc == 1) {
        leaf(cs);
    } else if (nc > 1) {
        int stack[64];
        int sp = 0;
        stack[sp++] = cs - s;
        while (sp) {
            const int c = stack[--sp];
            if (c < 0) { leaf(~c); continue; }
            if (!boxes_meet(qmin, qmax, f.bvh.bmin[c], f.bvh.bmax[c])) continue;
            if (sp + 2 > 64) { atomicOr(w.err, ERR_STACK_CAPACITY); continue; }
            stack[sp++] = f.bvh.right[c];
            stack[sp++] = f.bvh.left[c];
        }
    }
}

__global__ void __launch_bounds__(64) k_overlap_mtd(World w, FrameBuf f, const ShapeIn* qs, int n, int cap, int* counts,
                                                    float4* hits, int* hit_col) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const ShapeIn qi = qs[i];
    const V3 pos = {qi.px, qi.py, qi.pz};
    const Q4 ori = {qi.qx, qi.qy, qi.qz, qi.qw};
    const GeomD g = GeomD{qi.type, {qi.p0, qi.p1, qi.p2}, qi.mesh};
    ManifoldL ms[kTriManifolds];
    TCI cand[kTriCandidates];
    Polytope poly;
    int count = 0;
    for_each_mtd(w, f, qi.scene, pos, ori, g, ms, cand, poly, [&](int c, const ManifoldL& m, float mtd) {
        if (count < cap) {
            hits[(size_t)i * cap + count] = make_float4(m.normal.x, m.normal.y, m.normal.z, mtd);
            hit_col[(size_t)i * cap + count] = c;
        }
        ++count;
    });
    counts[i] = count;
}

// CharacterController::move (src/CharacterController.cpp:5-45) for one controller a
// thread.  The reference's step-up test calls Scene::raycastClosest without a filter,
// which never reports a hit (src/Physecs.cpp:580, 615), so the translation stays as
// given.  Each iteration collects the capsule's MTD hits and applies them in the order
// (collider, triangle); the reference applies them in its tree's order, which only
// changes the rounding of the summed moves.  Controllers of one batch see each other
// at their poses before the batch: this kernel only reads the world and leaves each new
// pose in moved[i]; k_commit_characters writes them after every controller has moved.
// A controller's own colliders move with it, as the registry's transform does in the
// reference, while their bounds stay those before the move.
constexpr int kCharHits = 32;
__global__ void __launch_bounds__(64) k_move_characters(World w, FrameBuf f, const CharIn* cs, int n, unsigned char* flags_out,
                                                        float4* moved) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const CharIn ch = cs[i];
    const int b = ch.body;
    const Q4 q = ld4(w.quat[b]);
    V3 p = ld3(w.pos[b]);
    const V3 up = qrot(q, V3{0.f, 1.f, 0.f});
    p += V3{ch.tx, ch.ty, ch.tz};
    const GeomD g{G_CAPSULE, {ch.height * 0.5f, ch.radius, 0.f}, -1};
    ManifoldL ms[kTriManifolds];
    TCI cand[kTriCandidates];
    Polytope poly;
    int hc[kCharHits], ht[kCharHits];
    float4 hv[kCharHits];
    int flags = 0;
    for (int it = 0; it < ch.iterations; ++it) {
        int nh = 0;
        for_each_mtd(w, f, w.info[b].w, p + up * (ch.height * 0.5f + ch.radius), q, g, ms, cand, poly,
                     [&](int c, const ManifoldL& m, float mtd) {
                         if (nh == kCharHits) { flags |= 0x80; return; }
                         // insertion by (collider, triangle), stable
                         int k = nh++;
                         while (k > 0 && (hc[k - 1] > c || (hc[k - 1] == c && ht[k - 1] > m.triangleIndex))) {
                             hc[k] = hc[k - 1]; ht[k] = ht[k - 1]; hv[k] = hv[k - 1];
                             --k;
                         }
                         hc[k] = c; ht[k] = m.triangleIndex;
                         hv[k] = make_float4(m.normal.x, m.normal.y, m.normal.z, mtd);
                     }, b, p);
        for (int k = 0; k < nh; ++k) {
            const V3 nrm = ld3(hv[k]);
            const float mtd = hv[k].w;
            const float d = dot(nrm, up);
            flags |= d > 0.001f ? 1 : (d < -0.001f ? 4 : 2);
            if (d > ch.slope_limit) p += up * mtd / d;
            else p += nrm * mtd;
        }
    }
    moved[i] = st4(p);
    flags_out[i] = (unsigned char)flags;
}

// The moved controllers' poses into the world, then registry.patch<TransformComponent> ->
// updateBounds: their colliders' bounds with the margin.
__global__ void k_commit_characters(World w, const CharIn* cs, int n, const float4* moved) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int b = cs[i].body;
    const V3 p = ld3(moved[i]);
    const Q4 q = ld4(w.quat[b]);
    w.pos[b] = st4(p);
    for (int c = w.body_col[b]; c < w.body_col[b + 1]; ++c) {
        const int4 ci = w.col_info[c];
        if (ci.y == G_TRIMESH) continue;
        const V3 cp = p + qrot(q, ld3(w.col_pos[c]));
        const Q4 co = qmul(q, ld4(w.col_quat[c]));
        const float4 pr = w.col_params[c];
        Bounds bb = getBounds(w, cp, co, GeomD{ci.y, {pr.x, pr.y, pr.z}, ci.z});
        bb.max += v3s(0.01f);
        bb.min -= v3s(0.01f);
        w.aabb_min[c] = st4(bb.min);
        w.aabb_max[c] = st4(bb.max);
    }
}

int launch_move_characters(const World& w, FrameBuf& f, const CharIn* cs, int n, unsigned char* flags, float4* moved,
                           cudaStream_t s) {
    if (n <= 0) return 0;
    k_move_characters<<<(n + 63) / 64, 64, 0, s>>>(w, f, cs, n, flags, moved);
    k_commit_characters<<<(n + 127) / 128, 128, 0, s>>>(w, cs, n, moved);
    return 2;
}

int launch_overlap_mtd(const World& w, FrameBuf& f, const ShapeIn* qs, int n, int cap, int* counts, float4* hits,
                       int* hit_col, cudaStream_t s) {
    if (n <= 0) return 0;
    k_overlap_mtd<<<(n + 63) / 64, 64, 0, s>>>(w, f, qs, n, cap, counts, hits, hit_col);
    return 1;
}

int launch_raycast(const World& w, FrameBuf& f, const RayIn* rays, int n, const unsigned char* accept, RayOut* out,
                   cudaStream_t s) {
    if (n <= 0) return 0;
    k_raycast<<<(n + 127) / 128, 128, 0, s>>>(w, f, rays, n, accept, out);
    return 1;
}

int launch_overlap(const World& w, FrameBuf& f, const ShapeIn* qs, int n, int cap, int* counts, int* hits, cudaStream_t s) {
    if (n <= 0) return 0;
    k_overlap<<<(n + 127) / 128, 128, 0, s>>>(w, f, qs, n, cap, counts, hits);
    return 1;
}

// ---------------------------------------------------------------- trigger pairs
//
// Scene::simulate keeps the overlapping trigger pairs of a frame in a set, calls
// onTriggerEnter for the pairs new to it and onTriggerExit for the pairs gone from it,
// and swaps it with the last frame's (src/Physecs.cpp:200-207, 537-552).  Here the two
// sets are key lists with open-addressing tables for the lookups; each key keeps its
// table slot so that the last frame's table is emptied entry by entry, not swept.
// Events go to a log that the host drains.


// A table holds at most half its capacity, so every probe sequence meets an empty slot.
__device__ __forceinline__ bool trig_find(const unsigned long long* t, unsigned mask, unsigned long long key) {
    unsigned h = trig_hash(key) & mask;
    for (unsigned probe = 0; probe <= mask; ++probe, h = (h + 1) & mask) {
        const unsigned long long v = t[h];
        if (v == key) return true;
        if (v == kNoKey) return false;
    }
    return false;
}

__device__ __forceinline__ void trig_event(const FrameBuf& f, int frame, int kind, unsigned long long key) {
    const int i = atomicAdd(f.n_evt, 1);
    if (i < f.evt_cap) f.trig_evt[i] = make_int4(frame, kind, (int)(key >> 32), (int)(unsigned)key);
}

// Scene of a collider, and whether a scene placed into a server slot this frame: its
// pairs enter whatever the last frame's set holds (that set is the slot's last occupant's)
__device__ __forceinline__ int collider_scene(const World& w, int c) { return w.info[w.col_info[c].x].w; }
__device__ __forceinline__ bool scene_is_fresh(const World& w, int c) {
    return w.scene_fresh && w.scene_fresh[collider_scene(w, c)];
}

// physecs::overlap of every trigger pair at this frame's poses; a pair that overlaps
// joins this frame's set and, when the last frame's set lacks it, enters.
__global__ void __launch_bounds__(128) k_trigger_enter(World w, FrameBuf f) {
    const int cur = f.trig_state[0], frame = f.trig_state[3];
    const unsigned mask = (unsigned)f.trig_table_cap - 1u;
    const int n = f.cat_count[7];
    unsigned long long* tab = f.trig_table[cur];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int2 pr = f.pairs[f.cat_list[7 * (size_t)f.pair_cap + t]];
        V3 pos0, pos1;
        Q4 or0, or1;
        GeomD g0, g1;
        collider_pose(w, pr.x, pos0, or0, g0);
        collider_pose(w, pr.y, pos1, or1, g1);
        if (!overlapGeom(w, pos0, or0, g0, pos1, or1, g1)) continue;
        const unsigned long long key = ((unsigned long long)(unsigned)pr.x << 32) | (unsigned)pr.y;
        const int i = atomicAdd(&f.trig_state[1 + cur], 1);
        if (i >= f.trig_cap) { atomicOr(w.err, ERR_PAIR_CAPACITY); continue; }
        unsigned h = trig_hash(key) & mask;
        for (unsigned probe = 0; probe <= mask; ++probe, h = (h + 1) & mask)
            if (atomicCAS(&tab[h], kNoKey, key) == kNoKey) break;
        f.trig_keys[cur][i] = key;
        f.trig_slot[cur][i] = (int)h;
        if (scene_is_fresh(w, pr.x) || !trig_find(f.trig_table[cur ^ 1], mask, key)) trig_event(f, frame, 0, key);
    }
}

// The last frame's pairs missing from this frame's set exit; the last frame's table is
// emptied for the frame after.  In a server's world a pair whose slot is not running (its
// request has run all its frames) or has a new occupant leaves without an event.
__global__ void __launch_bounds__(128) k_trigger_exit(World w, FrameBuf f) {
    const int cur = f.trig_state[0], prev = cur ^ 1, frame = f.trig_state[3];
    const unsigned mask = (unsigned)f.trig_table_cap - 1u;
    const int n = min(f.trig_state[1 + prev], f.trig_cap);
    const unsigned long long* tab = f.trig_table[cur];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const unsigned long long key = f.trig_keys[prev][t];
        bool live = true;
        if (w.scene_active) {
            const int sc = collider_scene(w, (int)(key >> 32));
            live = w.scene_active[sc] && !(w.scene_fresh && w.scene_fresh[sc]);
        }
        if (live && !trig_find(tab, mask, key)) trig_event(f, frame, 1, key);
        f.trig_table[prev][f.trig_slot[prev][t]] = kNoKey;
    }
}

// This frame's set becomes the last frame's; the emptied one takes the next frame's pairs.
__global__ void k_trigger_swap(FrameBuf f) {
    const int prev = f.trig_state[0] ^ 1;
    f.trig_state[1 + prev] = 0;
    f.trig_state[0] = prev;
    f.trig_state[3] += 1;
}

int launch_triggers(const World& w, FrameBuf& f, cudaStream_t s) {
    if (!f.trig_cap) return 0;
    const int blocks = std::min(152 * 4, (f.trig_cap + 127) / 128);
    k_trigger_enter<<<blocks, 128, 0, s>>>(w, f);
    k_trigger_exit<<<blocks, 128, 0, s>>>(w, f);
    k_trigger_swap<<<1, 1, 0, s>>>(f);
    return 3;
}

}  // namespace psx

// ---------------------------------------------------------------- C ABI

#include <algorithm>
#include <tuple>
#include <vector>
#include "runtime.cuh"

namespace {

using namespace psx;
using namespace psx::rt;

// device staging of at least `bytes`, reused between calls
psx_status query_buffer(psx_world* W, size_t bytes, char** out) {
    if (W->qbuf_bytes < bytes) {
        if (W->qbuf) cudaFree(W->qbuf);
        W->qbuf = nullptr;
        W->qbuf_bytes = 0;
        PSX_CUDA(cudaMalloc(&W->qbuf, bytes));
        W->qbuf_bytes = bytes;
    }
    *out = static_cast<char*>(W->qbuf);
    return PSX_OK;
}

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// the device form of n overlap queries: scene-local convex meshes become world meshes
psx_status pack_shapes(psx_world* W, int n, const psx_overlap_query* queries, std::vector<ShapeIn>& in) {
    in.resize(n);
    for (int i = 0; i < n; ++i) {
        const psx_overlap_query& q = queries[i];
        if (q.scene < 0 || q.scene >= W->n_scenes) return fail(PSX_ERR_INVALID_ARG, "psx_world_overlap: scene index");
        if (q.type < PSX_SPHERE || q.type > PSX_TRIANGLE_MESH) return fail(PSX_ERR_INVALID_ARG, "psx_world_overlap: shape type");
        int mesh = -1;
        if (q.type == PSX_CONVEX_MESH) {
            const int m0 = W->h_scene_convex[q.scene], m1 = W->h_scene_convex[q.scene + 1];
            if (q.mesh < 0 || m0 + q.mesh >= m1) return fail(PSX_ERR_INVALID_ARG, "psx_world_overlap: convex mesh index");
            mesh = m0 + q.mesh;
        }
        // a triangle-mesh query overlaps nothing (Overlap.cpp:194-235); its count is set to 0
        // on the host, and the device tests it as a sphere of radius 0
        const bool tri = q.type == PSX_TRIANGLE_MESH;
        in[i] = ShapeIn{q.scene, q.pos[0], q.pos[1], q.pos[2], q.quat[0], q.quat[1], q.quat[2], q.quat[3],
                        tri ? PSX_SPHERE : q.type, tri ? 0.f : q.params[0], tri ? 0.f : q.params[1], tri ? 0.f : q.params[2],
                        mesh, q.filter};
    }
    return PSX_OK;
}

// the trees the queries walk: every scene's LBVH over the current bounds, every collider a leaf
void query_trees(psx_world* W) { launch_bvh_build(W->w, W->f, W->scene_bits, W->scene_sort_pmax, true, W->stream); }

}  // namespace

extern "C" {

PSX_API psx_status psx_world_raycast(psx_world* W, int32_t n, const psx_ray* rays, const uint8_t* accept, psx_ray_hit* hits) {
    if (!W || n < 0 || (n && (!rays || !hits))) return fail(PSX_ERR_INVALID_ARG, "psx_world_raycast: bad arguments");
    PSX_CUDA(cudaSetDevice(W->device));
    if (n == 0) return PSX_OK;
    static_assert(sizeof(psx_ray) == sizeof(RayIn), "psx_ray layout");
    for (int i = 0; i < n; ++i)
        if (rays[i].scene < 0 || rays[i].scene >= W->n_scenes) return fail(PSX_ERR_INVALID_ARG, "psx_world_raycast: scene index");
    const size_t nb = (size_t)W->w.n_bodies;
    const size_t in_b = align256(sizeof(RayIn) * n), acc_b = accept ? align256(nb) : 0, out_b = sizeof(RayOut) * n;
    char* buf = nullptr;
    PSX_TRY(query_buffer(W, in_b + acc_b + out_b, &buf));
    RayIn* d_in = reinterpret_cast<RayIn*>(buf);
    unsigned char* d_acc = accept ? reinterpret_cast<unsigned char*>(buf + in_b) : nullptr;
    RayOut* d_out = reinterpret_cast<RayOut*>(buf + in_b + acc_b);
    cudaStream_t st = W->stream;
    PSX_CUDA(cudaMemcpyAsync(d_in, rays, sizeof(RayIn) * n, cudaMemcpyHostToDevice, st));
    if (accept) PSX_CUDA(cudaMemcpyAsync(d_acc, accept, nb, cudaMemcpyHostToDevice, st));
    query_trees(W);
    launch_raycast(W->w, W->f, d_in, n, d_acc, d_out, st);
    std::vector<RayOut> res(n);
    PSX_CUDA(cudaMemcpyAsync(res.data(), d_out, sizeof(RayOut) * n, cudaMemcpyDeviceToHost, st));
    PSX_CUDA(cudaStreamSynchronize(st));
    PSX_TRY(check_err(W));
    for (int i = 0; i < n; ++i) {
        psx_ray_hit& h = hits[i];
        const int c = res[i].collider;
        if (c < 0) {
            h.body = -1; h.collider = -1; h.entity = 0; h.distance = 0.f;
            h.pos[0] = h.pos[1] = h.pos[2] = 0.f;
            continue;
        }
        const int b = W->h_col_body[c];
        h.body = b - W->h_scene_body[rays[i].scene];
        h.collider = W->h_col_local[c];
        h.entity = W->h_entity[b];
        h.distance = res[i].dist;
        // rayOrig + rayDir * distance (src/Physecs.cpp:624)
        for (int k = 0; k < 3; ++k) h.pos[k] = rays[i].origin[k] + rays[i].dir[k] * h.distance;
    }
    return PSX_OK;
}

PSX_API psx_status psx_world_overlap(psx_world* W, int32_t n, const psx_overlap_query* queries, int32_t cap,
                                     psx_overlap_hit* hits, int32_t* counts) {
    if (!W || n < 0 || cap < 0 || (n && (!queries || !counts || (cap && !hits))))
        return fail(PSX_ERR_INVALID_ARG, "psx_world_overlap: bad arguments");
    PSX_CUDA(cudaSetDevice(W->device));
    if (n == 0) return PSX_OK;
    std::vector<ShapeIn> in;
    PSX_TRY(pack_shapes(W, n, queries, in));
    const size_t in_b = align256(sizeof(ShapeIn) * n), cnt_b = align256(sizeof(int) * n), hit_b = sizeof(int) * (size_t)n * cap;
    char* buf = nullptr;
    PSX_TRY(query_buffer(W, in_b + cnt_b + hit_b, &buf));
    ShapeIn* d_in = reinterpret_cast<ShapeIn*>(buf);
    int* d_cnt = reinterpret_cast<int*>(buf + in_b);
    int* d_hit = reinterpret_cast<int*>(buf + in_b + cnt_b);
    cudaStream_t st = W->stream;
    PSX_CUDA(cudaMemcpyAsync(d_in, in.data(), sizeof(ShapeIn) * n, cudaMemcpyHostToDevice, st));
    query_trees(W);
    launch_overlap(W->w, W->f, d_in, n, cap, d_cnt, d_hit, st);
    std::vector<int> cnt(n), hit((size_t)n * cap);
    PSX_CUDA(cudaMemcpyAsync(cnt.data(), d_cnt, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
    if (hit_b) PSX_CUDA(cudaMemcpyAsync(hit.data(), d_hit, hit_b, cudaMemcpyDeviceToHost, st));
    PSX_CUDA(cudaStreamSynchronize(st));
    PSX_TRY(check_err(W));
    for (int i = 0; i < n; ++i) {
        counts[i] = queries[i].type == PSX_TRIANGLE_MESH ? 0 : cnt[i];
        const int m = std::min(counts[i], cap);
        for (int k = 0; k < m; ++k) {
            const int c = hit[(size_t)i * cap + k];
            const int b = W->h_col_body[c];
            psx_overlap_hit& h = hits[(size_t)i * cap + k];
            h.body = b - W->h_scene_body[queries[i].scene];
            h.collider = W->h_col_local[c];
            h.entity = W->h_entity[b];
        }
    }
    return PSX_OK;
}

PSX_API psx_status psx_world_overlap_mtd(psx_world* W, int32_t n, const psx_overlap_query* queries, int32_t cap,
                                         psx_overlap_mtd_hit* hits, int32_t* counts) {
    if (!W || n < 0 || cap < 0 || (n && (!queries || !counts || (cap && !hits))))
        return fail(PSX_ERR_INVALID_ARG, "psx_world_overlap_mtd: bad arguments");
    PSX_CUDA(cudaSetDevice(W->device));
    if (n == 0) return PSX_OK;
    std::vector<ShapeIn> in;
    PSX_TRY(pack_shapes(W, n, queries, in));
    const size_t in_b = align256(sizeof(ShapeIn) * n), cnt_b = align256(sizeof(int) * n);
    const size_t f4_b = align256(sizeof(float4) * (size_t)n * cap), col_b = sizeof(int) * (size_t)n * cap;
    char* buf = nullptr;
    PSX_TRY(query_buffer(W, in_b + cnt_b + f4_b + col_b, &buf));
    ShapeIn* d_in = reinterpret_cast<ShapeIn*>(buf);
    int* d_cnt = reinterpret_cast<int*>(buf + in_b);
    float4* d_f = reinterpret_cast<float4*>(buf + in_b + cnt_b);
    int* d_col = reinterpret_cast<int*>(buf + in_b + cnt_b + f4_b);
    cudaStream_t st = W->stream;
    PSX_CUDA(cudaMemcpyAsync(d_in, in.data(), sizeof(ShapeIn) * n, cudaMemcpyHostToDevice, st));
    query_trees(W);
    launch_overlap_mtd(W->w, W->f, d_in, n, cap, d_cnt, d_f, d_col, st);
    std::vector<int> cnt(n), col((size_t)n * cap);
    std::vector<float4> fv((size_t)n * cap);
    PSX_CUDA(cudaMemcpyAsync(cnt.data(), d_cnt, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
    if (cap) {
        PSX_CUDA(cudaMemcpyAsync(fv.data(), d_f, sizeof(float4) * (size_t)n * cap, cudaMemcpyDeviceToHost, st));
        PSX_CUDA(cudaMemcpyAsync(col.data(), d_col, col_b, cudaMemcpyDeviceToHost, st));
    }
    PSX_CUDA(cudaStreamSynchronize(st));
    PSX_TRY(check_err(W));
    for (int i = 0; i < n; ++i) {
        counts[i] = queries[i].type == PSX_TRIANGLE_MESH ? 0 : cnt[i];
        const int m = std::min(counts[i], cap);
        for (int k = 0; k < m; ++k) {
            const size_t j = (size_t)i * cap + k;
            const int c = col[j];
            const int b = W->h_col_body[c];
            psx_overlap_mtd_hit& h = hits[j];
            h.body = b - W->h_scene_body[queries[i].scene];
            h.collider = W->h_col_local[c];
            h.entity = W->h_entity[b];
            h.normal[0] = fv[j].x; h.normal[1] = fv[j].y; h.normal[2] = fv[j].z;
            h.mtd = fv[j].w;
        }
    }
    return PSX_OK;
}

PSX_API psx_status psx_world_move_characters(psx_world* W, int32_t n, const psx_character* chars, float dt,
                                             uint8_t* flags_out) {
    (void)dt;   // read by the reference only inside the step-up branch, which never runs
    if (!W || n < 0 || (n && (!chars || !flags_out))) return fail(PSX_ERR_INVALID_ARG, "psx_world_move_characters: bad arguments");
    PSX_CUDA(cudaSetDevice(W->device));
    if (n == 0) return PSX_OK;
    static_assert(sizeof(psx_character) == sizeof(CharIn), "psx_character layout");
    std::vector<CharIn> in(n);
    psx_status st = PSX_OK;
    for (int i = 0; i < n; ++i) {
        const psx_character& c = chars[i];
        if (c.scene < 0 || c.scene >= W->n_scenes || c.body < 0 ||
            c.body >= W->h_scene_body[c.scene + 1] - W->h_scene_body[c.scene] || c.num_iterations < 0 ||
            !(c.height >= 0.f) || !(c.radius >= 0.f)) {
            st = fail(PSX_ERR_INVALID_ARG, "psx_world_move_characters: record " + std::to_string(i));
            break;
        }
        const int b = W->h_scene_body[c.scene] + c.body;
        if (W->h_delta_slot[b] >= 0) {
            st = fail(PSX_ERR_INVALID_ARG, "psx_world_move_characters: one body twice in a batch");
            break;
        }
        W->h_delta_slot[b] = i;
        in[i] = CharIn{c.scene, b, c.height, c.radius, c.max_step_height, c.slope_limit, c.num_iterations,
                       c.translation[0], c.translation[1], c.translation[2]};
    }
    for (int i = 0; i < n; ++i)
        if (chars[i].scene >= 0 && chars[i].scene < W->n_scenes) {
            const int b = W->h_scene_body[chars[i].scene] + chars[i].body;
            if (b >= 0 && b < (int)W->h_delta_slot.size()) W->h_delta_slot[b] = -1;
        }
    if (st != PSX_OK) return st;
    const size_t in_b = align256(sizeof(CharIn) * n), fl_b = align256(n);
    char* buf = nullptr;
    PSX_TRY(query_buffer(W, in_b + fl_b + sizeof(float4) * n, &buf));
    CharIn* d_in = reinterpret_cast<CharIn*>(buf);
    unsigned char* d_fl = reinterpret_cast<unsigned char*>(buf + in_b);
    float4* d_moved = reinterpret_cast<float4*>(buf + in_b + fl_b);
    cudaStream_t s = W->stream;
    PSX_CUDA(cudaMemcpyAsync(d_in, in.data(), sizeof(CharIn) * n, cudaMemcpyHostToDevice, s));
    query_trees(W);
    W->launches += launch_move_characters(W->w, W->f, d_in, n, d_fl, d_moved, s);
    PSX_CUDA(cudaMemcpyAsync(flags_out, d_fl, n, cudaMemcpyDeviceToHost, s));
    PSX_CUDA(cudaStreamSynchronize(s));
    return check_err(W);
}

PSX_API psx_status psx_world_trigger_events(psx_world* W, psx_trigger_event* out, int32_t cap, int32_t* n_out,
                                            int64_t* n_lost) {
    if (!W || cap < 0 || (cap && !out) || !n_out) return fail(PSX_ERR_INVALID_ARG, "psx_world_trigger_events: bad arguments");
    PSX_CUDA(cudaSetDevice(W->device));
    const FrameBuf& f = W->f;
    std::vector<psx_trigger_event> due;   // exits of pairs a topology change removed, once their frame ran
    for (size_t i = 0; i < W->trig_vanished.size();) {
        if (W->trig_vanished[i].frame < W->frames_run) {
            due.push_back(W->trig_vanished[i]);
            W->trig_vanished.erase(W->trig_vanished.begin() + (long)i);
        } else {
            ++i;
        }
    }
    auto key = [](const psx_trigger_event& e) {
        return std::make_tuple(e.frame, e.kind, e.scene, e.body0, e.collider0, e.body1, e.collider1);
    };
    if (!f.trig_cap && !due.empty()) {
        std::sort(due.begin(), due.end(), [&](const psx_trigger_event& a, const psx_trigger_event& b) { return key(a) < key(b); });
        W->trig_pending.insert(W->trig_pending.end(), due.begin(), due.end());
    }
    if (f.trig_cap) {
        cudaStream_t st = W->stream;
        int n = 0;
        PSX_CUDA(cudaMemcpyAsync(&n, f.n_evt, sizeof(int), cudaMemcpyDeviceToHost, st));
        PSX_CUDA(cudaStreamSynchronize(st));
        if (n || !due.empty()) {
            const int kept = std::min(n, f.evt_cap);
            std::vector<int4> ev(kept);
            if (kept) PSX_CUDA(cudaMemcpyAsync(ev.data(), f.trig_evt, sizeof(int4) * kept, cudaMemcpyDeviceToHost, st));
            PSX_CUDA(cudaMemsetAsync(f.n_evt, 0, sizeof(int), st));
            PSX_CUDA(cudaStreamSynchronize(st));
            W->trig_lost += n - kept;
            std::vector<psx_trigger_event> batch(kept);
            for (int i = 0; i < kept; ++i) {
                const int c0 = ev[i].z, c1 = ev[i].w, b0 = W->h_col_body[c0], b1 = W->h_col_body[c1];
                const int sc = (int)(std::upper_bound(W->h_scene_body.begin(), W->h_scene_body.end(), b0) -
                                     W->h_scene_body.begin()) - 1;
                psx_trigger_event& e = batch[i];
                e.frame = ev[i].x;
                e.kind = ev[i].y;
                e.scene = sc;
                e.body0 = b0 - W->h_scene_body[sc];
                e.collider0 = W->h_col_local[c0];
                e.body1 = b1 - W->h_scene_body[sc];
                e.collider1 = W->h_col_local[c1];
                e.entity0 = W->h_entity[b0];
                e.entity1 = W->h_entity[b1];
            }
            batch.insert(batch.end(), due.begin(), due.end());
            std::sort(batch.begin(), batch.end(), [&](const psx_trigger_event& a, const psx_trigger_event& b) { return key(a) < key(b); });
            W->trig_pending.insert(W->trig_pending.end(), batch.begin(), batch.end());
        }
    }
    const int m = (int)std::min<size_t>((size_t)cap, W->trig_pending.size());
    std::copy(W->trig_pending.begin(), W->trig_pending.begin() + m, out);
    W->trig_pending.erase(W->trig_pending.begin(), W->trig_pending.begin() + m);
    *n_out = m;
    if (n_lost) { *n_lost = W->trig_lost; W->trig_lost = 0; }
    return PSX_OK;
}

}  // extern "C"
