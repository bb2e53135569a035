/*
 * port_capi.cpp — C entry points of the CPU oracle (liborc.so).
 * ORACLE (test infrastructure only): called by tests/, smoke() and bench.py's
 * CPU-baseline leg through ctypes; never by the physecs_gb300 product.
 * The entry points and output layouts mirror oracle/ref/ref_capi.cpp so the
 * restatement can be checked against the reference call for call.
 */
#include "world.h"
#include <cstring>

using namespace orc;

extern "C" {

void* orc_scene_create(const psx_scene_desc* d) {
    World* w = new World();
    w->init(d);
    return w;
}

void orc_scene_destroy(void* h) { delete static_cast<World*>(h); }

void orc_scene_step(void* h, float dt) { static_cast<World*>(h)->step(dt); }

void orc_scene_set_knobs(void* h, int substeps, int iterations, float gravity) {
    World* w = static_cast<World*>(h);
    w->substeps = substeps; w->iterations = iterations; w->g = gravity;
}

void orc_scene_read(void* h, float* pos, float* quat, float* vel, float* ang) {
    World* w = static_cast<World*>(h);
    for (size_t b = 0; b < w->bodies.size(); ++b) {
        const Body& B = w->bodies[b];
        if (!B.alive) {   // a destroyed entity reads as zeros
            std::memset(pos + 3 * b, 0, 12); std::memset(quat + 4 * b, 0, 16);
            std::memset(vel + 3 * b, 0, 12); std::memset(ang + 3 * b, 0, 12);
            continue;
        }
        std::memcpy(pos + 3 * b, &B.pos, 12);
        std::memcpy(quat + 4 * b, &B.q, 16);
        V3 v = B.hasDyn ? B.vel : V3{0, 0, 0}, a = B.hasDyn ? B.ang : V3{0, 0, 0};
        std::memcpy(vel + 3 * b, &v, 12);
        std::memcpy(ang + 3 * b, &a, 12);
    }
}

void orc_scene_write(void* h, const float* pos, const float* quat, const float* vel, const float* ang) {
    World* w = static_cast<World*>(h);
    for (size_t b = 0; b < w->bodies.size(); ++b) {
        Body& B = w->bodies[b];
        if (!B.alive) continue;
        std::memcpy(&B.pos, pos + 3 * b, 12);
        std::memcpy(&B.q, quat + 4 * b, 16);
        if (B.hasDyn) { std::memcpy(&B.vel, vel + 3 * b, 12); std::memcpy(&B.ang, ang + 3 * b, 12); }
    }
}

int orc_scene_pairs(void* h, int32_t* out, int cap) {
    World* w = static_cast<World*>(h);
    int n = (int)w->pairs.size() / 4;
    for (int i = 0; i < n && i < cap; ++i) {
        out[4 * i + 0] = (int32_t)w->bodies[w->pairs[4 * i]].entity;
        out[4 * i + 1] = w->pairs[4 * i + 1];
        out[4 * i + 2] = (int32_t)w->bodies[w->pairs[4 * i + 2]].entity;
        out[4 * i + 3] = w->pairs[4 * i + 3];
    }
    return n;
}

int orc_scene_bounds(void* h, int32_t* ids, float* bounds, int cap) {
    World* w = static_cast<World*>(h);
    int n = (int)w->bp.size();
    for (int i = 0; i < n && i < cap; ++i) {
        const BPEntry& e = w->bp[i];
        ids[2 * i] = (int32_t)e.entity; ids[2 * i + 1] = e.col;
        std::memcpy(bounds + 6 * i, &e.b.min, 12);
        std::memcpy(bounds + 6 * i + 3, &e.b.max, 12);
    }
    return n;
}

/* same layout as ref_scene_contacts; ids[3] also carries the source pair index in bits 8.. */
int orc_scene_contacts(void* h, int32_t* ids, float* f, int cap) {
    World* w = static_cast<World*>(h);
    int n = (int)w->contacts.size();
    for (int i = 0; i < n && i < cap; ++i) {
        const Contact& c = w->contacts[i];
        ids[4 * i] = c.b0; ids[4 * i + 1] = c.b1; ids[4 * i + 2] = c.np; ids[4 * i + 3] = c.soft ? 1 : 0;
        float* o = f + 56 * i;
        std::memset(o, 0, 56 * sizeof(float));
        o[0] = c.n.x; o[1] = c.n.y; o[2] = c.n.z; o[3] = c.friction; o[4] = c.frequency; o[5] = c.damping;
        for (int k = 0; k < c.np; ++k) {
            const CPoint& p = c.p[k];
            float* q = o + 8 + 12 * k;
            q[0] = p.r0.x; q[1] = p.r0.y; q[2] = p.r0.z; q[3] = p.r1.x; q[4] = p.r1.y; q[5] = p.r1.z;
            q[6] = p.targetVelocity; q[7] = p.c; q[8] = p.lamN; q[9] = p.lamT;
        }
    }
    return n;
}

int orc_scene_collide(void* h, int n_pairs, const int32_t* pairs, int32_t* ids, float* f, int cap) {
    World* w = static_cast<World*>(h);
    int n = 0;
    std::vector<Manifold> buf;
    for (int i = 0; i < n_pairs; ++i) {
        int b0 = pairs[4 * i], b1 = pairs[4 * i + 2];
        int c0 = w->bodies[b0].cols[pairs[4 * i + 1]], c1 = w->bodies[b1].cols[pairs[4 * i + 3]];
        buf.clear();
        if (!collision(w->colPos(c0), w->colQ(c0), w->colliders[c0].g, w->colPos(c1), w->colQ(c1), w->colliders[c1].g, buf)) continue;
        for (const Manifold& m : buf) {
            if (!m.numPoints) continue;
            if (n < cap) {
                ids[4 * n] = i; ids[4 * n + 1] = m.triangleIndex; ids[4 * n + 2] = m.numPoints; ids[4 * n + 3] = 0;
                float* o = f + 28 * n;
                std::memset(o, 0, 28 * sizeof(float));
                o[0] = m.normal.x; o[1] = m.normal.y; o[2] = m.normal.z;
                for (int k = 0; k < m.numPoints; ++k) {
                    std::memcpy(o + 4 + 6 * k, &m.points[k].p0, 12);
                    std::memcpy(o + 7 + 6 * k, &m.points[k].p1, 12);
                }
            }
            ++n;
        }
    }
    return n;
}

int orc_scene_joint_colors(void* h, int32_t* out, int cap) {
    World* w = static_cast<World*>(h);
    int n = 0;
    for (int c = 0; c <= 8; ++c)
        for (int j : w->colors[c]) {
            if (n < cap) { out[2 * n] = c; out[2 * n + 1] = (int32_t)w->bodies[w->joints[j].body1].entity; }
            ++n;
        }
    return n;
}

/* Solve the next step's contacts in the given order: keys {entity0, collider0, entity1,
 * collider1, triangleIndex} per manifold.  Returns nothing; the count of manifolds that
 * did not match is reported by orc_scene_order_error after the step. */
void orc_scene_set_contact_order(void* h, int n, const int32_t* keys) {
    World* w = static_cast<World*>(h);
    w->orderKeys.clear();
    for (int i = 0; i < n; ++i)
        w->orderKeys.emplace_back((uint32_t)keys[5 * i], keys[5 * i + 1], (uint32_t)keys[5 * i + 2], keys[5 * i + 3], keys[5 * i + 4]);
    w->useOrder = true;
}

int orc_scene_order_error(void* h) { return static_cast<World*>(h)->orderError; }

/* Manifold keys {entity0, collider0, entity1, collider1, triangleIndex} of the last
 * step's contacts, in the same order as orc_scene_contacts. */
int orc_scene_contact_keys(void* h, int32_t* keys, int cap) {
    World* w = static_cast<World*>(h);
    int n = (int)w->contacts.size();
    for (int i = 0; i < n && i < cap; ++i) {
        const Contact& c = w->contacts[i];
        const int* pr = &w->pairs[4 * c.pair];
        keys[5 * i] = (int32_t)w->bodies[pr[0]].entity; keys[5 * i + 1] = pr[1];
        keys[5 * i + 2] = (int32_t)w->bodies[pr[2]].entity; keys[5 * i + 3] = pr[3];
        keys[5 * i + 4] = c.tri;
    }
    return n;
}

/* Broadphase bounds of one collider (desc collider index) at the current pose, without margin. */
void orc_collider_bounds(void* h, int collider, float* out6) {
    World* w = static_cast<World*>(h);
    Bounds b = getBounds(w->colPos(collider), w->colQ(collider), w->colliders[collider].g);
    std::memcpy(out6, &b.min, 12);
    std::memcpy(out6 + 3, &b.max, 12);
}

// n rays of 8 floats {unused, origin xyz, dir xyz, max distance}; per ray the body,
// collider index within it (-1, -1 for no hit), distance and hit position
void orc_scene_raycast(void* h, int n, const float* rays, const uint8_t* accept, int32_t* out_ids, float* out_f) {
    World* w = static_cast<World*>(h);
    for (int i = 0; i < n; ++i) {
        const float* r = rays + 8 * i;
        V3 o = v3(r[1], r[2], r[3]), d = v3(r[4], r[5], r[6]);
        float dist = 0.f;
        int c = w->raycastClosest(o, d, r[7], accept, dist);
        float* of = out_f + 4 * i;
        if (c < 0) {
            out_ids[2 * i] = -1; out_ids[2 * i + 1] = -1;
            of[0] = of[1] = of[2] = of[3] = 0.f;
            continue;
        }
        out_ids[2 * i] = w->colliders[c].body;
        out_ids[2 * i + 1] = w->colliders[c].local;
        V3 p = o + d * dist;   // rayOrig + rayDir * distance (src/Physecs.cpp:624)
        of[0] = dist; of[1] = p.x; of[2] = p.y; of[3] = p.z;
    }
}

// one shape {pos xyz, quat xyzw}, type, params, convex mesh index, data filter; writes
// up to cap (body, collider) pairs and returns the number found
int orc_scene_overlap(void* h, const float* pose, int type, const float* params, int mesh, int filter, int32_t* out, int cap) {
    World* w = static_cast<World*>(h);
    Geometry g;
    g.type = type;
    g.p[0] = params[0]; g.p[1] = params[1]; g.p[2] = params[2];
    if (type == CONVEX_MESH) g.convex = w->convex[mesh].get();
    if (type == TRIANGLE_MESH) return 0;   // a triangle mesh overlaps nothing (Overlap.cpp:194-235)
    std::vector<int> hits;
    w->overlap(v3(pose[0], pose[1], pose[2]), Q4{pose[3], pose[4], pose[5], pose[6]}, g, filter, hits);
    for (int k = 0; k < (int)hits.size() && k < cap; ++k) {
        int c = hits[k];
        out[2 * k] = w->colliders[c].body;
        out[2 * k + 1] = w->colliders[c].local;
    }
    return (int)hits.size();
}

// Scene::overlapWithMinTranslationalDistance for one shape: up to cap records of
// (body, collider) in out_ids and (normal xyz, mtd) in out_f; returns the number found
int orc_scene_overlap_mtd(void* h, const float* pose, int type, const float* params, int mesh, int32_t* out_ids, float* out_f,
                          int cap) {
    World* w = static_cast<World*>(h);
    Geometry g;
    g.type = type;
    g.p[0] = params[0]; g.p[1] = params[1]; g.p[2] = params[2];
    if (type == CONVEX_MESH) g.convex = w->convex[mesh].get();
    if (type == TRIANGLE_MESH) return 0;
    std::vector<World::MtdHit> hits;
    w->overlapMtd(v3(pose[0], pose[1], pose[2]), Q4{pose[3], pose[4], pose[5], pose[6]}, g, hits);
    for (int k = 0; k < (int)hits.size() && k < cap; ++k) {
        int c = hits[k].col;
        out_ids[2 * k] = w->colliders[c].body;
        out_ids[2 * k + 1] = w->colliders[c].local;
        out_f[4 * k] = hits[k].n.x; out_f[4 * k + 1] = hits[k].n.y; out_f[4 * k + 2] = hits[k].n.z; out_f[4 * k + 3] = hits[k].mtd;
    }
    return (int)hits.size();
}

// CharacterController::move of body b; returns its flags
int orc_character_move(void* h, int b, float height, float radius, float max_step, float slope, int iterations,
                       const float* translation) {
    return static_cast<World*>(h)->moveCharacter(b, height, radius, max_step, slope, iterations,
                                                 v3(translation[0], translation[1], translation[2]));
}

void orc_scene_set_contact_filter(void* h, int32_t (*f)(int32_t, int32_t, int32_t, int32_t)) {
    static_cast<World*>(h)->contactFilter = f;
}

void orc_scene_set_can_collide(void* h, int b0, int b1, int can) { static_cast<World*>(h)->setCanCollide(b0, b1, can != 0); }

// an entity made from body 0 of d (meshes: this scene's); returns the body index and
// writes the entity value
int orc_scene_create_body(void* h, const psx_scene_desc* d, uint32_t* entity) {
    World* w = static_cast<World*>(h);
    const int b = w->createBody(d);
    *entity = w->bodies[b].entity;
    return b;
}

void orc_scene_destroy_body(void* h, int b) { static_cast<World*>(h)->destroyBody(b); }

void orc_scene_add_collider(void* h, int b, const psx_scene_desc* d) { static_cast<World*>(h)->addCollider(b, d); }

void orc_scene_clear_colliders(void* h, int b) { static_cast<World*>(h)->clearColliders(b); }

int orc_scene_create_joint(void* h, int type, int b0, int b1, const float* frames, const float* params) {
    return static_cast<World*>(h)->createJoint(type, b0, b1, frames, params);
}

void orc_scene_destroy_joint(void* h, int j) { static_cast<World*>(h)->destroyJoint(j); }

// The joint classes' setters between frames (RevoluteJoint::setDriveEnabled ...,
// include/Physecs/Joints/*.h): joint j's parameter block is replaced; a gear joint keeps
// its accumulated angles (GearJoint.h:10-17).
void orc_scene_set_joint_params(void* h, int j, const float* p) {
    std::memcpy(static_cast<World*>(h)->joints[j].params, p, sizeof(float) * PSX_JOINT_PARAMS);
}

// A batch of registry deltas in array order (psx_body_delta; the scene field is unused)
void orc_scene_apply_deltas(void* h, int n, const psx_body_delta* d) {
    World* w = static_cast<World*>(h);
    for (int i = 0; i < n; ++i) {
        const psx_body_delta& e = d[i];
        if (e.mask & PSX_DELTA_POSE) w->patchPose(e.body, v3(e.pos[0], e.pos[1], e.pos[2]), Q4{e.quat[0], e.quat[1], e.quat[2], e.quat[3]});
        if (e.mask & PSX_DELTA_VELOCITY)
            w->setVelocity(e.body, v3(e.vel[0], e.vel[1], e.vel[2]), v3(e.ang_vel[0], e.ang_vel[1], e.ang_vel[2]));
        if (e.mask & PSX_DELTA_KINEMATIC) w->setIsKinematic(e.body, e.kinematic != 0);
    }
}

// TriangleMesh::build (src/TriangleMesh.cpp:144-164) of the restatement: triangles in the
// tree's order as 20 words each (indices, pad, bounds min/max, normal, centroid, each
// padded to four) and nodes as 8 words (bounds min, triCount, bounds max, index); nodes
// needs room for max(1, 2 n - 1).  Returns the node count.
int orc_trimesh_build(const float* verts, int nv, const uint32_t* idx, int nidx, uint32_t* tris, uint32_t* nodes) {
    std::vector<V3> v(nv);
    for (int i = 0; i < nv; ++i) v[i] = v3(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
    TriangleMesh m;
    m.build(v, std::vector<uint32_t>(idx, idx + nidx));
    auto put = [](uint32_t* o, V3 a) { std::memcpy(o, &a.x, 4); std::memcpy(o + 1, &a.y, 4); std::memcpy(o + 2, &a.z, 4); o[3] = 0; };
    for (size_t t = 0; t < m.triangles.size(); ++t) {
        const Triangle& tr = m.triangles[t];
        uint32_t* o = tris + 20 * t;
        o[0] = tr.idx[0]; o[1] = tr.idx[1]; o[2] = tr.idx[2]; o[3] = 0;
        put(o + 4, tr.bounds.min); put(o + 8, tr.bounds.max); put(o + 12, tr.normal); put(o + 16, tr.centroid);
    }
    for (size_t k = 0; k < m.bvh.size(); ++k) {
        const TriNode& n = m.bvh[k];
        uint32_t* o = nodes + 8 * k;
        put(o, n.bounds.min); o[3] = (uint32_t)n.triCount;
        put(o + 4, n.bounds.max); o[7] = (uint32_t)n.index;
    }
    return (int)m.bvh.size();
}

// The trigger events of the frames stepped since the last call, in step order: up to
// cap records of (frame, kind 0 enter / 1 exit, body0, collider0, body1, collider1),
// removed from the scene; returns the number pending before the call
int orc_scene_trigger_events(void* h, int32_t* out, int cap) {
    World* w = static_cast<World*>(h);
    const int n = (int)w->triggerEvents.size();
    const int m = n < cap ? n : cap;
    for (int k = 0; k < m; ++k) {
        const World::TriggerEvent& e = w->triggerEvents[k];
        int32_t* o = out + 6 * k;
        o[0] = e.frame; o[1] = e.kind; o[2] = e.body0; o[3] = e.col0; o[4] = e.body1; o[5] = e.col1;
    }
    w->triggerEvents.erase(w->triggerEvents.begin(), w->triggerEvents.begin() + m);
    return n;
}

}  // extern "C"
