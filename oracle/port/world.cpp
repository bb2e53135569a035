/*
 * world.cpp — the CPU oracle's restatement of physecs::Scene::simulate
 * (src/Physecs.cpp:112-561) with the reference's single-thread ordering.
 * ORACLE (test infrastructure only; see omath.h).
 *
 * Order of work per frame, as in the reference with numThreads = 0:
 *   SAP insertion sort on bounds.min.x and sweep         Physecs.cpp:119-173
 *   narrowphase over pairs from last to first            Physecs.cpp:181-317, ThreadPool.cpp:3-9
 *   joint rows per colour 0..8                           Physecs.cpp:320-355
 *   substeps: contact rows, joint rows, integrate         Physecs.cpp:363-531
 *             velocities, preSolve, iterations,
 *             integrate positions, relaxation, write-back
 *   cache swap and bounds update with 0.01 m margin      Physecs.cpp:553-559
 * Joint colours 0..7 use the 4-lane SIMD row arithmetic of src/Constraint1DW.cpp,
 * the overflow colour 8 the scalar arithmetic of src/Constraint1D.cpp.
 */
#include "world.h"
#include <algorithm>
#include <cmath>
#include <cstring>

namespace orc {

static V3 ld3(const float* p) { return {p[0], p[1], p[2]}; }
static Q4 ld4(const float* p) { return {p[0], p[1], p[2], p[3]}; }

V3 World::colPos(int c) const { const Body& b = bodies[colliders[c].body]; return b.pos + qrot(b.q, colliders[c].pos); }
Q4 World::colQ(int c) const { const Body& b = bodies[colliders[c].body]; return qmul(b.q, colliders[c].q); }

void World::init(const psx_scene_desc* d) {
    substeps = d->num_substeps; iterations = d->num_iterations; g = d->gravity;
    for (int m = 0; m < d->n_convex; ++m) {
        auto cm = std::make_unique<ConvexMesh>();
        for (int v = d->convex_vert_start[m]; v < d->convex_vert_start[m + 1]; ++v) cm->buffer.push_back(ld3(d->convex_verts + 3 * v));
        cm->count = (int)cm->buffer.size();
        int padded = (cm->count + 3) / 4 * 4;
        V3 last = cm->buffer.back();
        while ((int)cm->buffer.size() < padded) cm->buffer.push_back(last);
        for (int f = d->convex_face_start[m]; f < d->convex_face_start[m + 1]; ++f) {
            ConvexFace face;
            for (int k = d->face_index_start[f]; k < d->face_index_start[f + 1]; ++k) face.indices.push_back(d->face_indices[k]);
            face.normal = ld3(d->face_normal + 3 * f);
            face.centroid = ld3(d->face_centroid + 3 * f);
            cm->faces.push_back(face);
        }
        convex.push_back(std::move(cm));
    }
    for (int m = 0; m < d->n_trimesh; ++m) {
        std::vector<V3> verts;
        for (int v = d->tri_vert_start[m]; v < d->tri_vert_start[m + 1]; ++v) verts.push_back(ld3(d->tri_verts + 3 * v));
        std::vector<uint32_t> idx(d->tri_indices + d->tri_index_start[m], d->tri_indices + d->tri_index_start[m + 1]);
        auto tm = std::make_unique<TriangleMesh>();
        tm->build(verts, idx);
        tri.push_back(std::move(tm));
    }
    for (int b = 0; b < d->n_bodies; ++b) {
        Body B;
        B.entity = d->entity[b];
        B.hasDyn = (d->flags[b] & PSX_BODY_DYNAMIC) != 0;
        B.kinematic = (d->flags[b] & PSX_BODY_KINEMATIC) != 0;
        B.pos = ld3(d->pos + 3 * b);
        B.q = ld4(d->quat + 4 * b);
        if (B.hasDyn) {
            B.vel = ld3(d->vel + 3 * b);
            B.ang = ld3(d->ang_vel + 3 * b);
            B.invMass = d->inv_mass[b];
            B.com = ld3(d->com + 3 * b);
            for (int k = 0; k < 3; ++k) B.invI.c[k] = ld3(d->inv_inertia + 9 * b + 3 * k);
            B.dyn = (int)dynBodies.size();
            dynBodies.push_back(b);
        }
        for (int c = d->collider_start[b]; c < d->collider_start[b + 1]; ++c) B.cols.push_back(c);
        bodies.push_back(B);
    }
    for (int c = 0; c < d->n_colliders; ++c) {
        Collider C;
        int b = 0;
        while (!(d->collider_start[b] <= c && c < d->collider_start[b + 1])) ++b;
        C.body = b;
        C.local = c - d->collider_start[b];
        C.pos = ld3(d->col_pos + 3 * c);
        C.q = ld4(d->col_quat + 4 * c);
        C.g.type = d->col_type[c];
        for (int k = 0; k < 3; ++k) C.g.p[k] = d->col_params[4 * c + k];
        if (C.g.type == CONVEX_MESH) C.g.convex = convex[d->col_mesh[c]].get();
        if (C.g.type == TRIANGLE_MESH) C.g.tri = tri[d->col_mesh[c]].get();
        C.friction = d->col_material[3 * c];
        C.restitution = d->col_material[3 * c + 1];
        C.damping = d->col_material[3 * c + 2];
        C.trigger = d->col_is_trigger ? d->col_is_trigger[c] != 0 : false;
        C.enable = d->col_enable_sim ? d->col_enable_sim[c] != 0 : true;
        C.data = d->col_data ? d->col_data[c] : 0;
        colliders.push_back(C);
    }
    // onRigidBodyCreate (Physecs.cpp:25-37): creation bounds carry no margin
    for (int b = 0; b < (int)bodies.size(); ++b) {
        for (int k = 0; k < (int)bodies[b].cols.size(); ++k) {
            int c = bodies[b].cols[k];
            bp.push_back({bodies[b].entity, b, k, getBounds(colPos(c), colQ(c), colliders[c].g), colliders[c].enable,
                          bodies[b].simulated()});
        }
    }
    colorBits.assign(bodies.size(), 0);
    // registry.create() hands out ids 0, 1, ... at version 0 to a fresh registry
    for (const Body& B : bodies) entPacked.push_back(B.entity);
    entAlive = entPacked.size();
    for (int j = 0; j < d->n_joints; ++j)
        createJoint(d->joint_type[j], d->joint_body0[j], d->joint_body1[j], d->joint_frames + 14 * j,
                    d->joint_params + PSX_JOINT_PARAMS * j);
}

void World::updateBounds(int b, bool margin) {
    for (auto& e : bp) {
        if (e.body != b) continue;
        int c = bodies[b].cols[e.col];
        e.b = getBounds(colPos(c), colQ(c), colliders[c].g);
        if (margin) { e.b.max += v3s(0.01f); e.b.min -= v3s(0.01f); }
    }
}

// Scene::createJoint -> Scene::addJoint (Physecs.cpp:690-710): the pair stops colliding,
// the joint takes the lowest colour free on both bodies and goes last in that colour
int World::createJoint(int type, int b0, int b1, const float* f, const float* params) {
    Joint J;
    J.type = type;
    J.body0 = b0;
    J.body1 = b1;
    J.a0p = ld3(f); J.a0q = ld4(f + 3); J.a1p = ld3(f + 7); J.a1q = ld4(f + 10);
    std::memcpy(J.params, params, sizeof(J.params));
    if (J.type == PSX_JOINT_GEAR) J.persistent0 = J.persistent1 = J.virtual0 = J.virtual1 = 0;
    uint32_t e0 = bodies[b0].entity, e1 = bodies[b1].entity;
    nonColliding[e0 < e1 ? std::make_pair(e0, e1) : std::make_pair(e1, e0)] = 1;
    unsigned char u = colorBits[b0] | colorBits[b1];
    unsigned int inv = ~(unsigned int)u;
    int i = __builtin_ctz(inv);
    colorBits[b0] |= (unsigned char)(1u << i);
    colorBits[b1] |= (unsigned char)(1u << i);
    J.color = i;
    colors[i].push_back((int)joints.size());
    joints.push_back(J);
    return (int)joints.size() - 1;
}

// Scene::destroyJoint (Physecs.cpp:712-725): out of its colour (the others keep their
// order), the pair collides again, the colour is free again on both bodies
void World::destroyJoint(int j) {
    Joint& J = joints[j];
    auto& list = colors[J.color];
    auto it = std::find(list.begin(), list.end(), j);
    if (it == list.end()) return;
    list.erase(it);
    uint32_t e0 = bodies[J.body0].entity, e1 = bodies[J.body1].entity;
    nonColliding.erase(e0 < e1 ? std::make_pair(e0, e1) : std::make_pair(e1, e0));
    colorBits[J.body0] &= (unsigned char)~(1u << J.color);
    colorBits[J.body1] &= (unsigned char)~(1u << J.color);
}

// Scene::addCollider (Physecs.cpp:740-751): the entry goes last, with creation bounds
void World::addCollider(int b, const psx_scene_desc* d) {
    Body& B = bodies[b];
    Collider C;
    C.body = b;
    C.local = (int)B.cols.size();
    C.pos = ld3(d->col_pos);
    C.q = ld4(d->col_quat);
    C.g.type = d->col_type[0];
    for (int k = 0; k < 3; ++k) C.g.p[k] = d->col_params[k];
    if (C.g.type == CONVEX_MESH) C.g.convex = convex[d->col_mesh[0]].get();
    if (C.g.type == TRIANGLE_MESH) C.g.tri = tri[d->col_mesh[0]].get();
    C.friction = d->col_material[0];
    C.restitution = d->col_material[1];
    C.damping = d->col_material[2];
    C.trigger = d->col_is_trigger ? d->col_is_trigger[0] != 0 : false;
    C.enable = d->col_enable_sim ? d->col_enable_sim[0] != 0 : true;
    C.data = d->col_data ? d->col_data[0] : 0;
    const int c = (int)colliders.size();
    colliders.push_back(C);
    B.cols.push_back(c);
    bp.push_back({B.entity, b, C.local, getBounds(colPos(c), colQ(c), colliders[c].g), C.enable, B.simulated()});
}

// Scene::clearColliders (Physecs.cpp:727-738): each entry swapped with the last and popped
void World::clearColliders(int b) {
    Body& B = bodies[b];
    for (int k = 0; k < (int)B.cols.size(); ++k) {
        size_t id = 0;
        while (!(bp[id].body == b && bp[id].col == k)) ++id;
        bp[id] = bp.back();
        bp.pop_back();
    }
    B.cols.clear();
}

// EnTT 3.12: an entity's next version skips the reserved all-ones version
static uint32_t nextVersion(uint32_t e) {
    uint32_t v = (e >> 20) + 1;
    if (v == 0xfffu) v = 0;
    return (e & 0xfffffu) | (v << 20);
}

int World::createBody(const psx_scene_desc* d) {
    // registry.create(): the entity right past the live ones (the last destroyed), else a new id
    uint32_t e;
    if (entAlive < entPacked.size()) e = entPacked[entAlive];
    else { e = (uint32_t)entPacked.size(); entPacked.push_back(e); }
    ++entAlive;
    const int b = (int)bodies.size();
    Body B;
    B.entity = e;
    B.hasDyn = (d->flags[0] & PSX_BODY_DYNAMIC) != 0;
    B.kinematic = (d->flags[0] & PSX_BODY_KINEMATIC) != 0;
    B.pos = ld3(d->pos);
    B.q = ld4(d->quat);
    if (B.hasDyn) {
        B.vel = ld3(d->vel);
        B.ang = ld3(d->ang_vel);
        B.invMass = d->inv_mass[0];
        B.com = ld3(d->com);
        for (int k = 0; k < 3; ++k) B.invI.c[k] = ld3(d->inv_inertia + 3 * k);
    }
    for (int c = d->collider_start[0]; c < d->collider_start[1]; ++c) {
        Collider C;
        C.body = b;
        C.local = c - d->collider_start[0];
        B.cols.push_back((int)colliders.size());
        C.pos = ld3(d->col_pos + 3 * c);
        C.q = ld4(d->col_quat + 4 * c);
        C.g.type = d->col_type[c];
        for (int k = 0; k < 3; ++k) C.g.p[k] = d->col_params[4 * c + k];
        if (C.g.type == CONVEX_MESH) C.g.convex = convex[d->col_mesh[c]].get();
        if (C.g.type == TRIANGLE_MESH) C.g.tri = tri[d->col_mesh[c]].get();
        C.friction = d->col_material[3 * c];
        C.restitution = d->col_material[3 * c + 1];
        C.damping = d->col_material[3 * c + 2];
        C.trigger = d->col_is_trigger ? d->col_is_trigger[c] != 0 : false;
        C.enable = d->col_enable_sim ? d->col_enable_sim[c] != 0 : true;
        C.data = d->col_data ? d->col_data[c] : 0;
        colliders.push_back(C);
    }
    bodies.push_back(B);
    colorBits.push_back(0);
    // emplace<RigidBodyCollisionComponent>: onRigidBodyCreate appends the entries with
    // creation bounds (Physecs.cpp:25-37); emplace<RigidBodyDynamicComponent> then
    // appends to the dynamic storage and onDynamicCreate sets the entries' flag (:56-66)
    for (int k = 0; k < (int)B.cols.size(); ++k) {
        const int c = B.cols[k];
        bp.push_back({e, b, k, getBounds(colPos(c), colQ(c), colliders[c].g), colliders[c].enable, B.simulated()});
    }
    if (B.hasDyn) {
        bodies[b].dyn = (int)dynBodies.size();
        dynBodies.push_back(b);
    }
    return b;
}

void World::destroyBody(int b) {
    Body& B = bodies[b];
    // registry.destroy removes the components pool by pool, last created pool first:
    // RigidBodyDynamicComponent (onDynamicDelete, then swap-and-pop of the storage),
    // TransformComponent, RigidBodyCollisionComponent (onRigidBodyDelete, :39-49)
    if (B.hasDyn) {
        for (auto& e : bp) if (e.body == b) e.dynamic = false;
        const int i = B.dyn, last = dynBodies.back();
        dynBodies[i] = last;
        bodies[last].dyn = i;
        dynBodies.pop_back();
        B.dyn = -1;
        B.hasDyn = false;
    }
    for (int k = 0; k < (int)B.cols.size(); ++k) {
        size_t id = 0;
        while (!(bp[id].body == b && bp[id].col == k)) ++id;
        bp[id] = bp.back();
        bp.pop_back();
    }
    // the entity: version bumped, swapped just past the live ones
    size_t pos = 0;
    while (entPacked[pos] != B.entity) ++pos;
    entPacked[pos] = nextVersion(B.entity);
    if (pos != --entAlive) std::swap(entPacked[pos], entPacked[entAlive]);
    B.alive = false;
}

// registry.patch<TransformComponent> after a pose write: Scene::onRigidBodyMove ->
// updateBounds, with the margin (Physecs.cpp:51-54, 78-90)
void World::patchPose(int b, V3 p, Q4 q) {
    bodies[b].pos = p;
    bodies[b].q = q;
    updateBounds(b, true);
}

void World::setVelocity(int b, V3 v, V3 w) {
    bodies[b].vel = v;
    bodies[b].ang = w;
}

void World::setCanCollide(int b0, int b1, bool canCollide) {
    uint32_t e0 = bodies[b0].entity, e1 = bodies[b1].entity;
    std::pair<uint32_t, uint32_t> key = e0 < e1 ? std::make_pair(e0, e1) : std::make_pair(e1, e0);
    if (canCollide) nonColliding.erase(key);
    else nonColliding[key] = 1;
}

// Scene::setIsKinematic (Physecs.cpp:753-770)
void World::setIsKinematic(int b, bool kinematic) {
    Body& B = bodies[b];
    B.kinematic = kinematic;
    if (kinematic) { B.vel = {0, 0, 0}; B.ang = {0, 0, 0}; }
    for (auto& e : bp) if (e.body == b) e.dynamic = !kinematic;
}

// Physecs.cpp:119-173
void World::broadphase() {
    for (size_t i = 1; i < bp.size(); ++i) {
        BPEntry e = bp[i];
        size_t j = i;
        while (j > 0 && bp[j - 1].b.min.x > e.b.min.x) { bp[j] = bp[j - 1]; --j; }
        if (j < i) bp[j] = e;
    }
    pairs.clear();
    for (size_t i = 0; i + 1 < bp.size(); ++i) {
        const BPEntry& a = bp[i];
        if (!a.enable) continue;
        for (size_t j = i + 1; j < bp.size(); ++j) {
            const BPEntry& b = bp[j];
            if (!b.enable) continue;
            if (a.entity == b.entity) continue;
            if (!(a.dynamic || b.dynamic)) continue;
            if (a.b.max.x < b.b.min.x) break;
            if (a.b.max.y < b.b.min.y || a.b.min.y > b.b.max.y) continue;
            if (a.b.max.z < b.b.min.z || a.b.min.z > b.b.max.z) continue;
            if (a.entity < b.entity) { pairs.insert(pairs.end(), {a.body, a.col, b.body, b.col}); }
            else { pairs.insert(pairs.end(), {b.body, b.col, a.body, a.col}); }
        }
    }
}

// Physecs.cpp:181-317 with tasks in the order count-1 .. 0
void World::narrowphase() {
    contacts.clear();
    cacheTemp.clear();
    triggerCacheTemp.clear();
    int np = (int)pairs.size() / 4;
    std::vector<Manifold> buf;
    for (int idx = np - 1; idx >= 0; --idx) {
        int bA = pairs[4 * idx], cA = pairs[4 * idx + 1], bB = pairs[4 * idx + 2], cB = pairs[4 * idx + 3];
        const Body& B0 = bodies[bA];
        const Body& B1 = bodies[bB];
        int c0 = B0.cols[cA], c1 = B1.cols[cB];
        const Collider& C0 = colliders[c0];
        const Collider& C1 = colliders[c1];
        V3 pos0 = B0.pos + qrot(B0.q, C0.pos);
        Q4 or0 = qmul(B0.q, C0.q);
        V3 pos1 = B1.pos + qrot(B1.q, C1.pos);
        Q4 or1 = qmul(B1.q, C1.q);
        // the contact filter (the default one makes a pair with a trigger a TRIGGER pair): a
        // TRIGGER pair gets an overlap test, no contact, ahead of the jointed-pair filter
        // (Physecs.cpp:20-23, 200-207)
        const bool triggerPair = contactFilter ? contactFilter(C0.trigger, C0.data, C1.trigger, C1.data) == 1
                                               : (C0.trigger || C1.trigger);
        if (triggerPair) {
            if (overlapColliders(pos0, or0, c0, pos1, or1, c1)) triggerCacheTemp.insert({bA, cA, bB, cB});
            continue;
        }
        if (nonColliding.count({B0.entity, B1.entity})) continue;
        buf.clear();
        if (!collision(pos0, or0, C0.g, pos1, or1, C1.g, buf)) continue;
        V3 com0{0, 0, 0}, v0{0, 0, 0}, w0{0, 0, 0}, com1{0, 0, 0}, v1{0, 0, 0}, w1{0, 0, 0};
        if (B0.simulated()) { com0 = B0.pos + qrot(B0.q, B0.com); v0 = B0.vel; w0 = B0.ang; }
        if (B1.simulated()) { com1 = B1.pos + qrot(B1.q, B1.com); v1 = B1.vel; w1 = B1.ang; }
        int mi = 0;
        for (const Manifold& m : buf) {
            if (!m.numPoints) continue;
            V3 n = m.normal;
            CacheKey key{B0.entity, cA, B1.entity, cB, m.triangleIndex};
            auto it = cache.find(key);
            const CacheVal* prev = it != cache.end() ? &it->second : nullptr;
            CacheVal cur{};
            cur.np = m.numPoints;
            float friction = (C0.friction + C1.friction) * 0.5f;
            bool soft;
            float freq = 0, damp = 0, rest = 0;
            if (C0.damping || C1.damping) {
                soft = true;
                if (C0.damping && C1.damping) { freq = fminG(C0.restitution, C1.restitution); damp = fminG(C0.damping, C1.damping); }
                else if (C0.damping) { freq = C0.restitution; damp = C0.damping; }
                else { freq = C1.restitution; damp = C1.damping; }
                rest = 0;
            } else {
                soft = false;
                rest = (C0.restitution + C1.restitution) * 0.5f;
            }
            Contact cc{};
            cc.body0 = bA; cc.body1 = bB;
            cc.b0 = B0.simulated() ? B0.dyn : -1;
            cc.b1 = B1.simulated() ? B1.dyn : -1;
            cc.n = n; cc.friction = friction; cc.soft = soft; cc.frequency = freq; cc.damping = damp;
            cc.np = m.numPoints;
            cc.pair = idx; cc.manifold = mi++; cc.tri = m.triangleIndex;
            for (int k = 0; k < m.numPoints; ++k) {
                V3 r0 = m.points[k].p0 - com0;
                V3 r1 = m.points[k].p1 - com1;
                V3 rel = v1 + cross(w1, r1) - v0 - cross(w0, r0);
                float relN = dot(rel, n);
                r0 = qrot(qinverse(B0.q), r0);
                r1 = qrot(qinverse(B1.q), r1);
                float tv = 0;
                bool found = false;
                if (prev) {
                    for (int i = 0; i < prev->np; ++i) {
                        if ((double)distance(r0, prev->r0[i]) < 0.1) { found = true; tv = prev->tv[i]; break; }
                    }
                }
                if (!found) tv = -rest * relN;
                cur.r0[k] = r0; cur.tv[k] = tv;
                CPoint& p = cc.p[k];
                p = CPoint{};
                p.r0 = r0; p.r1 = r1; p.targetVelocity = tv;
            }
            cacheTemp[key] = cur;
            contacts.push_back(cc);
        }
    }
}

// ---------------------------------------------------------------- joint rows

static void rowP2P(std::vector<Row>& r, int& k, V3 p0, V3 p1, V3 r0, V3 r1) {  // JointsUtil.h:8-28
    V3 d = p1 - p0;
    r[k].linear = {1, 0, 0}; r[k].angular0 = {0, r0.z, -r0.y}; r[k].angular1 = {0, r1.z, -r1.y}; r[k].c = d.x; ++k;
    r[k].linear = {0, 1, 0}; r[k].angular0 = {-r0.z, 0, r0.x}; r[k].angular1 = {-r1.z, 0, r1.x}; r[k].c = d.y; ++k;
    r[k].linear = {0, 0, 1}; r[k].angular0 = {r0.y, -r0.x, 0}; r[k].angular1 = {r1.y, -r1.x, 0}; r[k].c = d.z; ++k;
}
static void rowAng(std::vector<Row>& r, int& k, V3 a, float c) {
    r[k].angular0 = a; r[k].angular1 = a; r[k].c = c; ++k;
}

static float angleDiff(float a0, float a1) {  // GearJoint.cpp:5-8
    const float pi = 3.14159265358979323846f, two_pi = 6.28318530717958647692f;
    float diff = fmodf(a1 - a0 + pi, two_pi) - pi;
    return diff < -pi ? diff + two_pi : diff;
}

// the makeConstraints of each joint type (src/Joints/*.cpp), writing rows in creation order
static void makeRows(Joint& J, V3 p0, V3 p1, V3 r0, V3 r1, const M3& u0, const M3& u1) {
    std::vector<Row>& r = J.rows;
    int k = 0;
    switch (J.type) {
        case PSX_JOINT_FIXED:
            rowP2P(r, k, p0, p1, r0, r1);
            rowAng(r, k, cross(u1.c[1], u0.c[0]), dot(u0.c[0], u1.c[1]));
            rowAng(r, k, cross(u1.c[2], u0.c[0]), dot(u0.c[0], u1.c[2]));
            rowAng(r, k, cross(u1.c[2], u0.c[1]), dot(u0.c[1], u1.c[2]));
            break;
        case PSX_JOINT_SPHERICAL:
            rowP2P(r, k, p0, p1, r0, r1);
            break;
        case PSX_JOINT_UNIVERSAL:
            rowP2P(r, k, p0, p1, r0, r1);
            rowAng(r, k, cross(u1.c[2], u0.c[2]), dot(u0.c[2], u1.c[2]));
            break;
        case PSX_JOINT_REVOLUTE:
            rowP2P(r, k, p0, p1, r0, r1);
            rowAng(r, k, cross(u1.c[1], u0.c[0]), dot(u0.c[0], u1.c[1]));
            rowAng(r, k, cross(u1.c[2], u0.c[0]), dot(u0.c[0], u1.c[2]));
            if (J.params[0] != 0.f) {
                r[k].angular0 = u0.c[0]; r[k].angular1 = u0.c[0];
                r[k].targetVelocity = J.params[1]; r[k].max = J.params[2]; r[k].min = -J.params[2]; ++k;
            }
            break;
        case PSX_JOINT_SERVO: {
            rowP2P(r, k, p0, p1, r0, r1);
            rowAng(r, k, cross(u1.c[1], u0.c[0]), dot(u0.c[0], u1.c[1]));
            rowAng(r, k, cross(u1.c[2], u0.c[0]), dot(u0.c[0], u1.c[2]));
            // glm::orientedAngle (gtx/vector_angle.inl): acos(clamp(dot)), negated when dot(ref, cross) < 0
            float ang = std::acos(clampG(dot(u0.c[2], u1.c[2]), -1.f, 1.f));
            if (dot(u0.c[0], cross(u0.c[2], u1.c[2])) < 0.f) ang = -ang;
            r[k].angular0 = u0.c[0]; r[k].angular1 = u0.c[0];
            r[k].c = ang - J.params[0]; r[k].frequency = J.params[1]; r[k].damping = J.params[2]; ++k;
            break;
        }
        case PSX_JOINT_PRISMATIC: {
            V3 d = p1 - p0;
            r[k].linear = u0.c[1]; r[k].angular0 = cross(r0, u0.c[1]); r[k].angular1 = cross(r1, u0.c[1]); r[k].c = dot(d, u0.c[1]); ++k;
            r[k].linear = u0.c[2]; r[k].angular0 = cross(r0, u0.c[2]); r[k].angular1 = cross(r1, u0.c[2]); r[k].c = dot(d, u0.c[2]); ++k;
            rowAng(r, k, cross(u1.c[1], u0.c[0]), dot(u0.c[0], u1.c[1]));
            rowAng(r, k, cross(u1.c[2], u0.c[0]), dot(u0.c[0], u1.c[2]));
            rowAng(r, k, cross(u1.c[2], u0.c[1]), dot(u0.c[1], u1.c[2]));
            float dx = dot(d, u0.c[0]);
            V3 r0xx = cross(r0, u0.c[0]), r1xx = cross(r1, u0.c[0]);
            if (J.makeUpper) {
                r[k].linear = u0.c[0]; r[k].angular0 = r0xx; r[k].angular1 = r1xx; r[k].c = dx - J.params[0]; r[k].min = 0; ++k;
            } else if (J.makeLower) {
                r[k].linear = u0.c[0]; r[k].angular0 = r0xx; r[k].angular1 = r1xx; r[k].c = dx - J.params[1]; r[k].max = 0; ++k;
            }
            if (J.params[2] != 0.f) {
                r[k].linear = u0.c[0]; r[k].angular0 = r0xx; r[k].angular1 = r1xx; r[k].c = dx - J.params[3];
                r[k].frequency = J.params[4]; r[k].damping = J.params[5]; ++k;
            }
            break;
        }
        case PSX_JOINT_GEAR: {
            float a0, a1;
            {
                V3 p1p = p1 + dot(p0 - p1, u0.c[0]) * u0.c[0];
                V3 dir = normalize(p0 - p1p);
                V3 n = cross(u0.c[0], dir);
                M3 mm0 = m3cols(u0.c[0], -n, dir);
                M3 t = mm(transpose(mm0), u0);
                a0 = std::atan2(at(t.c[1], 2), at(t.c[2], 2));
            }
            {
                V3 p0p = p0 + dot(p1 - p0, u1.c[0]) * u1.c[0];
                V3 dir = normalize(p0p - p1);
                V3 n = cross(u1.c[0], dir);
                M3 mm1 = m3cols(u1.c[0], -n, dir);
                M3 t = mm(transpose(u1), mm1);
                a1 = std::atan2(at(t.c[1], 2), at(t.c[2], 2));
            }
            if (!J.gearInit) { J.persistent0 = a0; J.persistent1 = a1; J.gearInit = true; }
            J.virtual0 += angleDiff(a0, J.persistent0);
            J.virtual1 += angleDiff(a1, J.persistent1);
            J.persistent0 = a0; J.persistent1 = a1;
            float ratio = J.params[0];
            r[k].angular0 = u0.c[0] * ratio; r[k].angular1 = -u1.c[0]; r[k].c = J.virtual0 * ratio - J.virtual1; ++k;
            break;
        }
    }
}

// getSolverDesc of each joint type: the row flags in creation order
static void layoutRows(World& w, Joint& J) {
    std::vector<int> f;
    auto add = [&](int flags, int n) { for (int i = 0; i < n; ++i) f.push_back(flags); };
    switch (J.type) {
        case PSX_JOINT_FIXED: add(RF_NONE, 3); add(RF_ANGULAR, 3); break;
        case PSX_JOINT_SPHERICAL: add(RF_NONE, 3); break;
        case PSX_JOINT_UNIVERSAL: add(RF_NONE, 3); add(RF_ANGULAR, 1); break;
        case PSX_JOINT_REVOLUTE: add(RF_NONE, 3); add(RF_ANGULAR, 2); if (J.params[0] != 0.f) add(RF_ANGULAR | RF_LIMITED, 1); break;
        case PSX_JOINT_SERVO: add(RF_NONE, 3); add(RF_ANGULAR, 2); add(RF_ANGULAR | RF_SOFT, 1); break;
        case PSX_JOINT_GEAR: add(RF_ANGULAR, 1); break;
        case PSX_JOINT_PRISMATIC: {
            // PrismaticJoint.cpp:116-155: the limit row exists only while the limit is violated at frame start
            const Body& B0 = w.bodies[J.body0];
            const Body& B1 = w.bodies[J.body1];
            V3 p0 = B0.pos + qrot(B0.q, J.a0p), p1 = B1.pos + qrot(B1.q, J.a1p);
            V3 d = p1 - p0;
            V3 u00 = qrot(qmul(B0.q, J.a0q), {1, 0, 0});
            float dx = dot(d, u00);
            add(RF_NONE, 2); add(RF_ANGULAR, 3);
            if (dx > J.params[0]) { J.makeUpper = true; J.makeLower = false; add(RF_LIMITED, 1); }
            else if (dx < J.params[1]) { J.makeUpper = false; J.makeLower = true; add(RF_LIMITED, 1); }
            else { J.makeUpper = false; J.makeLower = false; }
            if (J.params[2] != 0.f) add(RF_SOFT, 1);
            break;
        }
    }
    const Body& B0 = w.bodies[J.body0];
    const Body& B1 = w.bodies[J.body1];
    int b0 = B0.simulated() ? B0.dyn : -1, b1 = B1.simulated() ? B1.dyn : -1;
    J.rows.assign(f.size(), Row{});
    for (size_t i = 0; i < f.size(); ++i) { J.rows[i].flags = f[i]; J.rows[i].b0 = b0; J.rows[i].b1 = b1; }
    J.r0 = B0.simulated() ? J.a0p - B0.com : J.a0p;
    J.r1 = B1.simulated() ? J.a1p - B1.com : J.a1p;
}

void World::buildJointRows() {
    for (int c = 0; c <= 8; ++c)
        for (int j : colors[c]) layoutRows(*this, joints[j]);
}

// ---------------------------------------------------------------- row preSolve / solve

static const int kFlagOrder[6] = {RF_NONE, RF_ANGULAR, RF_SOFT, RF_LIMITED, RF_ANGULAR | RF_SOFT, RF_ANGULAR | RF_LIMITED};

// Constraint1D::preSolve (Constraint1D.cpp:5-52) and one lane of Constraint1DW::preSolve (Constraint1DW.cpp:5-115)
static void rowPreSolve(Row& r, const std::vector<Mass>& mt, std::vector<Pseudo>& pv, bool simd) {
    float im0 = 0, im1 = 0;
    M3 I0 = m3zero(), I1 = m3zero();
    if (r.b0 >= 0) { im0 = mt[r.b0].invMass; I0 = mt[r.b0].invI; }
    if (r.b1 >= 0) { im1 = mt[r.b1].invMass; I1 = mt[r.b1].invI; }
    bool ang = r.flags & RF_ANGULAR;
    if (simd && ang) { im0 = 0; im1 = 0; }
    r.angular0t = mv(I0, r.angular0);
    r.angular1t = mv(I1, r.angular1);
    r.invEffMass = dot(r.angular0, r.angular0t) + dot(r.angular1, r.angular1t);
    if (!ang) {
        r.invEffMass += dot(r.linear, r.linear) * (im0 + im1);
        r.linear0t = im0 * r.linear;
        r.linear1t = im1 * r.linear;
    }
    if (r.flags & RF_SOFT) return;
    if (!simd) {
        if (!r.c || !r.invEffMass) return;
        float lambda = r.c / r.invEffMass;
        if (r.flags & RF_LIMITED) lambda = clampG(lambda, r.min, r.max);
        if (r.b0 >= 0) {
            if (!ang) pv[r.b0].v += lambda * r.linear0t;
            pv[r.b0].w += lambda * r.angular0t;
            ++pv[r.b0].count;
        }
        if (r.b1 >= 0) {
            if (!ang) pv[r.b1].v -= lambda * r.linear1t;
            pv[r.b1].w -= lambda * r.angular1t;
            ++pv[r.b1].count;
        }
        return;
    }
    bool ngs = (r.invEffMass != 0.f) && (r.c != 0.f);
    if (!ngs) return;
    float lambda = r.c / r.invEffMass;
    if (r.flags & RF_LIMITED) {
        lambda = lambda > r.min ? lambda : r.min;   // _mm_max_ps
        lambda = lambda < r.max ? lambda : r.max;   // _mm_min_ps
    }
    if (r.b0 >= 0) {
        if (!ang) pv[r.b0].v += lambda * r.linear0t;
        pv[r.b0].w += lambda * r.angular0t;
        ++pv[r.b0].count;
    }
    if (r.b1 >= 0) {
        if (!ang) pv[r.b1].v -= lambda * r.linear1t;
        pv[r.b1].w -= lambda * r.angular1t;
        ++pv[r.b1].count;
    }
}

// Constraint1D::solve (Constraint1D.cpp:54-127) / one lane of Constraint1DW::solve (Constraint1DW.cpp:117-233)
static void rowSolve(Row& r, std::vector<Velocity>& vt, float h, bool warm, bool simd) {
    bool ang = r.flags & RF_ANGULAR, soft = r.flags & RF_SOFT, lim = r.flags & RF_LIMITED;
    if (!simd && !r.invEffMass) return;
    V3 v0{0, 0, 0}, w0{0, 0, 0}, v1{0, 0, 0}, w1{0, 0, 0};
    if (r.b0 >= 0) { if (!ang) v0 = vt[r.b0].v; w0 = vt[r.b0].w; }
    if (r.b1 >= 0) { if (!ang) v1 = vt[r.b1].v; w1 = vt[r.b1].w; }
    if (!soft && warm) {
        bool apply = simd ? (std::fabs(r.c) < (float)1e-4 && std::fabs(r.totalLambda) < 10000.f)
                          : !(std::fabs(r.c) > 1e-4 || std::fabs(r.totalLambda) > 10000);
        if (apply) {
            float lw = r.totalLambda * 0.5f;
            r.totalLambda = lw;
            if (simd || r.b0 >= 0) { if (!ang) v0 += lw * r.linear0t; w0 += lw * r.angular0t; }
            if (simd || r.b1 >= 0) { if (!ang) v1 -= lw * r.linear1t; w1 -= lw * r.angular1t; }
        }
    }
    if (simd && !r.invEffMass) return;
    float rv = dot(r.angular1, w1) - dot(r.angular0, w0);
    if (!ang) rv += dot(r.linear, v1) - dot(r.linear, v0);
    float lambda;
    if (simd) {
        float effMass = 1.f / r.invEffMass;
        if (soft) {
            float af = (2.f * 3.14159265358979323846f) * r.frequency;
            float stiffness = af * af * effMass;
            float damping = 2.f * af * r.damping * effMass;
            float gamma = 1.f / (damping + h * stiffness);
            float beta = h * stiffness * gamma;
            lambda = (rv + beta * r.c / h) / (r.invEffMass + gamma / h);
        } else {
            float bias = (float)(0.2 / (double)h);
            lambda = (rv - r.targetVelocity + bias * r.c) * effMass;
        }
    } else {
        if (soft) {
            float af = 2.f * 3.14159265358979323846f * r.frequency;
            float stiffness = af * af / r.invEffMass;
            float damping = 2.f * af * r.damping / r.invEffMass;
            float gamma = 1.f / (damping + h * stiffness);
            float beta = h * stiffness / (damping + h * stiffness);
            lambda = (rv + beta * r.c / h) / (r.invEffMass + gamma / h);
        } else {
            lambda = (rv - r.targetVelocity + 0.2f * r.c / h) / r.invEffMass;
        }
    }
    if (lim) {
        float prev = r.totalLambda;
        r.totalLambda += lambda;
        if (simd) {
            float lo = r.min * h, hi = r.max * h;
            r.totalLambda = r.totalLambda > lo ? r.totalLambda : lo;
            r.totalLambda = r.totalLambda < hi ? r.totalLambda : hi;
        } else {
            r.totalLambda = clampG(r.totalLambda, r.min, r.max);
        }
        lambda = r.totalLambda - prev;
    } else {
        r.totalLambda += lambda;
    }
    if (!simd) {
        // the scalar row applies only this iteration's impulse to the solver velocities: its
        // warm-start impulse changed local copies alone (Constraint1D.cpp:114-127, 158-168)
        if (r.b0 >= 0) { if (!ang) vt[r.b0].v += lambda * r.linear0t; vt[r.b0].w += lambda * r.angular0t; }
        if (r.b1 >= 0) { if (!ang) vt[r.b1].v -= lambda * r.linear1t; vt[r.b1].w -= lambda * r.angular1t; }
        return;
    }
    if (!ang) { v0 += lambda * r.linear0t; v1 -= lambda * r.linear1t; }
    w0 += lambda * r.angular0t;
    w1 -= lambda * r.angular1t;
    if (r.b0 >= 0) { if (!ang) vt[r.b0].v = v0; vt[r.b0].w = w0; }
    if (r.b1 >= 0) { if (!ang) vt[r.b1].v = v1; vt[r.b1].w = w1; }
}

// ---------------------------------------------------------------- contacts (ContactConstraints.cpp)

static void contactPreSolve(Contact& c, const std::vector<Mass>& mt) {
    float im0 = 0, im1 = 0;
    M3 I0 = m3zero(), I1 = m3zero();
    if (c.b0 >= 0) { im0 = mt[c.b0].invMass; I0 = mt[c.b0].invI; }
    if (c.b1 >= 0) { im1 = mt[c.b1].invMass; I1 = mt[c.b1].invI; }
    for (int i = 0; i < c.np; ++i) {
        CPoint& p = c.p[i];
        p.r0xnt = mv(I0, p.r0xn); p.r1xnt = mv(I1, p.r1xn);
        p.r0xtt = mv(I0, p.r0xt); p.r1xtt = mv(I1, p.r1xt);
        p.invEffN = dot(c.n, c.n) * (im0 + im1) + dot(p.r0xn, p.r0xnt) + dot(p.r1xn, p.r1xnt);
        p.invEffT = dot(p.t, p.t) * (im0 + im1) + dot(p.r0xt, p.r0xtt) + dot(p.r1xt, p.r1xtt);
    }
}

static void contactSolve(Contact& c, std::vector<Velocity>& vt, const std::vector<Body>& bodies,
                         const std::vector<int>& dynBodies, bool useBias, float h) {
    for (int i = 0; i < c.np; ++i) {
        CPoint& p = c.p[i];
        if (!p.invEffN) continue;
        V3 v0{0, 0, 0}, w0{0, 0, 0}, v1{0, 0, 0}, w1{0, 0, 0};
        if (c.b0 >= 0) { v0 = vt[c.b0].v; w0 = vt[c.b0].w; }
        if (c.b1 >= 0) { v1 = vt[c.b1].v; w1 = vt[c.b1].w; }
        float rv = dot(-c.n, v0) + dot(-p.r0xn, w0) + dot(c.n, v1) + dot(p.r1xn, w1);
        float effMass = 1.f / p.invEffN;
        float lambda;
        if (c.soft) {
            float af = 2.f * 3.14159265358979323846f * c.frequency;
            float stiffness = af * af * effMass;
            float damping = 2.f * af * c.damping * effMass;
            float gamma = 1.f / (damping + h * stiffness);
            float beta = h * stiffness / (damping + h * stiffness);
            lambda = (rv + beta * p.c / h) / (p.invEffN + gamma / h);
        } else {
            lambda = (rv - p.targetVelocity + (useBias ? 0.1f * p.c / h : 0.f)) * effMass;
        }
        float prev = p.lamN;
        p.lamN += lambda;
        p.lamN = fminG(p.lamN, 0.f);
        lambda = p.lamN - prev;
        if (c.b0 >= 0) {
            vt[c.b0].v += lambda * bodies[dynBodies[c.b0]].invMass * c.n;
            vt[c.b0].w += lambda * p.r0xnt;
        }
        if (c.b1 >= 0) {
            vt[c.b1].v -= lambda * bodies[dynBodies[c.b1]].invMass * c.n;
            vt[c.b1].w -= lambda * p.r1xnt;
        }
    }
    // friction reads the component velocities, not the solver velocities (ContactConstraints.cpp:93-101)
    for (int i = 0; i < c.np; ++i) {
        CPoint& p = c.p[i];
        if (!p.invEffT) continue;
        V3 v0{0, 0, 0}, w0{0, 0, 0}, v1{0, 0, 0}, w1{0, 0, 0};
        if (c.b0 >= 0) { v0 = bodies[dynBodies[c.b0]].vel; w0 = bodies[dynBodies[c.b0]].ang; }
        if (c.b1 >= 0) { v1 = bodies[dynBodies[c.b1]].vel; w1 = bodies[dynBodies[c.b1]].ang; }
        float rv = dot(-p.t, v0) + dot(-p.r0xt, w0) + dot(p.t, v1) + dot(p.r1xt, w1);
        float lambda = rv / p.invEffT;
        float limit = c.friction * p.lamN;
        float prev = p.lamT;
        p.lamT += lambda;
        p.lamT = clampG(p.lamT, limit, -limit);
        lambda = p.lamT - prev;
        if (c.b0 >= 0) {
            vt[c.b0].v += lambda * bodies[dynBodies[c.b0]].invMass * p.t;
            vt[c.b0].w += lambda * p.r0xtt;
        }
        if (c.b1 >= 0) {
            vt[c.b1].v -= lambda * bodies[dynBodies[c.b1]].invMass * p.t;
            vt[c.b1].w -= lambda * p.r1xtt;
        }
    }
}

// ---------------------------------------------------------------- frame

void World::step(float dt) {
    broadphase();
    narrowphase();
    buildJointRows();
    std::vector<int> order;
    orderError = 0;
    if (useOrder) {
        std::map<CacheKey, int> byKey;
        for (size_t i = 0; i < contacts.size(); ++i) {
            const Contact& c = contacts[i];
            const int* pr = &pairs[4 * c.pair];
            byKey[CacheKey{bodies[pr[0]].entity, pr[1], bodies[pr[2]].entity, pr[3], c.tri}] = (int)i;
        }
        for (const CacheKey& k : orderKeys) {
            auto it = byKey.find(k);
            if (it == byKey.end()) { ++orderError; continue; }
            order.push_back(it->second);
            byKey.erase(it);
        }
        orderError += (int)byKey.size();
        useOrder = false;
    } else {
        order.resize(contacts.size());
        for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    }
    size_t nd = dynBodies.size();
    vt.resize(nd); pv.resize(nd); mt.resize(nd);
    float h = dt / substeps;
    for (int m = 0; m < substeps; ++m) {
        // update contact rows (Physecs.cpp:366-427)
        for (Contact& c : contacts) {
            const Body& B0 = bodies[c.body0];
            const Body& B1 = bodies[c.body1];
            V3 com0{0, 0, 0}, v0{0, 0, 0}, w0{0, 0, 0}, com1{0, 0, 0}, v1{0, 0, 0}, w1{0, 0, 0};
            if (B0.simulated()) { com0 = B0.pos + qrot(B0.q, B0.com); v0 = B0.vel; w0 = B0.ang; }
            if (B1.simulated()) { com1 = B1.pos + qrot(B1.q, B1.com); v1 = B1.vel; w1 = B1.ang; }
            for (int k = 0; k < c.np; ++k) {
                CPoint& p = c.p[k];
                V3 r0 = qrot(B0.q, p.r0), r1 = qrot(B1.q, p.r1);
                V3 cp0 = com0 + r0, cp1 = com1 + r1;
                float cn = dot(cp1 - cp0, c.n);
                V3 r0xn = cross(r0, c.n), r1xn = cross(r1, c.n);
                V3 rel = v1 + cross(w1, r1) - v0 - cross(w0, r0);
                float relN = dot(rel, c.n);
                V3 t = rel - relN * c.n;
                float tl = length(t);
                if (tl) t = t / tl;
                p.r0xn = r0xn; p.r1xn = r1xn; p.t = t;
                p.r0xt = cross(r0, t); p.r1xt = cross(r1, t);
                p.c = cn; p.lamN = 0; p.lamT = 0;
            }
        }
        // update joint rows (Physecs.cpp:429-439, Joint.cpp:5-14)
        for (int col = 0; col <= 8; ++col) {
            for (int j : colors[col]) {
                Joint& J = joints[j];
                const Body& B0 = bodies[J.body0];
                const Body& B1 = bodies[J.body1];
                M3 u0 = mat3_cast(qmul(B0.q, J.a0q)), u1 = mat3_cast(qmul(B1.q, J.a1q));
                V3 r0 = qrot(B0.q, J.r0), r1 = qrot(B1.q, J.r1);
                V3 p0 = B0.pos + qrot(B0.q, J.a0p), p1 = B1.pos + qrot(B1.q, J.a1p);
                makeRows(J, p0, p1, r0, r1, u0, u1);
            }
        }
        // integrate velocities (Physecs.cpp:441-469)
        for (size_t i = 0; i < nd; ++i) {
            Body& B = bodies[dynBodies[i]];
            if (B.kinematic) continue;
            M3 rot = mat3_cast(B.q);
            M3 invRot = transpose(rot);
            B.vel += h * V3{0, -g, 0};
            V3 wl = mv(invRot, B.ang);
            M3 I = inverse(B.invI);
            V3 f = h * cross(wl, mv(I, wl));
            M3 J = madd(I, mscale(h, msub(mm(matrixCross3(wl), I), matrixCross3(mv(I, wl)))));
            wl = wl - solve33(J, f);
            B.ang = mv(rot, wl);
            vt[i] = {B.vel, B.ang};
            pv[i] = {{0, 0, 0}, {0, 0, 0}, 0};
            mt[i] = {B.invMass, mm(mm(rot, B.invI), invRot)};
        }
        // preSolve
        for (Contact& c : contacts) contactPreSolve(c, mt);
        for (int col = 0; col <= 8; ++col) {
            bool simd = col < 8;
            if (simd) {
                for (int j : colors[col]) for (int f : kFlagOrder) for (Row& r : joints[j].rows) if (r.flags == f) rowPreSolve(r, mt, pv, true);
            } else {
                for (int f : kFlagOrder) for (int j : colors[col]) for (Row& r : joints[j].rows) if (r.flags == f) rowPreSolve(r, mt, pv, false);
            }
        }
        // iterations (Physecs.cpp:481-490)
        for (int it = 0; it < iterations; ++it) {
            for (int ci : order) contactSolve(contacts[ci], vt, bodies, dynBodies, true, h);
            for (int col = 0; col <= 8; ++col) {
                bool simd = col < 8;
                if (simd) {
                    for (int j : colors[col]) for (int f : kFlagOrder) for (Row& r : joints[j].rows) if (r.flags == f) rowSolve(r, vt, h, it == 0, true);
                } else {
                    for (int f : kFlagOrder) for (int j : colors[col]) for (Row& r : joints[j].rows) if (r.flags == f) rowSolve(r, vt, h, it == 0, false);
                }
            }
        }
        // integrate positions (Physecs.cpp:492-512)
        for (size_t i = 0; i < nd; ++i) {
            Body& B = bodies[dynBodies[i]];
            if (B.kinematic) continue;
            float s = pv[i].count ? 1.f / pv[i].count : 1.f;
            B.pos += h * vt[i].v + s * pv[i].v;
            V3 prevCom = qrot(B.q, B.com);
            V3 wv = 0.5f * (h * vt[i].w + s * pv[i].w);
            B.q = qadd(B.q, qmul(Q4{wv.x, wv.y, wv.z, 0.f}, B.q));
            B.q = qnormalize(B.q);
            B.pos += prevCom - qrot(B.q, B.com);
        }
        // relaxation (Physecs.cpp:514-520)
        for (int ci : order) if (!contacts[ci].soft) contactSolve(contacts[ci], vt, bodies, dynBodies, false, 0.f);
        // write back
        for (size_t i = 0; i < nd; ++i) {
            Body& B = bodies[dynBodies[i]];
            if (B.kinematic) continue;
            B.vel = vt[i].v;
            B.ang = vt[i].w;
        }
    }
    // enter: in this frame's set only; exit: in the last frame's only (Physecs.cpp:537-552)
    for (const auto& k : triggerCacheTemp)
        if (!triggerCache.count(k)) triggerEvents.push_back({frame, 0, k[0], k[1], k[2], k[3]});
    for (const auto& k : triggerCache)
        if (!triggerCacheTemp.count(k)) triggerEvents.push_back({frame, 1, k[0], k[1], k[2], k[3]});
    triggerCache.swap(triggerCacheTemp);
    ++frame;
    cache.swap(cacheTemp);
    for (size_t i = 0; i < nd; ++i) {
        int b = dynBodies[i];
        if (!bodies[b].kinematic) updateBounds(b, true);
    }
}

}  // namespace orc
