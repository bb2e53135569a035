/*
 * ref_capi.cpp — a C entry layer over the UNMODIFIED Physecs reference, used
 * only to generate and check golden fixtures (test infrastructure).  It is
 * compiled together with the reference's own sources by oracle/ref/build_ref.py
 * and never linked into the physecs_gb300 product.
 *
 * It builds an entt::registry from a psx_scene_desc exactly the way a Physecs
 * user does (demo/Demo.cpp:29-43: Transform, then RigidBodyCollisionComponent,
 * then RigidBodyDynamicComponent), drives physecs::Scene::simulate, and reads
 * back the scene's internal buffers: the broadphase pair list
 * (src/Physecs.cpp:134-172), the contact constraints (src/Physecs.cpp:274-314)
 * and the per-collider bounds (src/Physecs.cpp:79-90).
 */
#include <unordered_map>
#include <functional>
#include "Physecs.h"
#include "Components.h"
#include "Transform.h"
#include "Collision.h"
#include "ContactManifold.h"
#include "ContactConstraints.h"
#include "BoundsUtil.h"
#include "FixedJoint.h"
#include "RevoluteJoint.h"
#include "SphericalJoint.h"
#include "PrismaticJoint.h"
#include "UniversalJoint.h"
#include "GearJoint.h"
#include "ServoJoint.h"
#include "CharacterController.h"
#include "psx.h"

#include <memory>
#include <vector>

/* src/ConvexMesh.cpp defines ConvexMeshVertices<N>'s constructor as a template
 * without instantiating it; GCC needs an explicit instantiation to construct a
 * ConvexMesh from outside that translation unit. */
#include "ConvexMesh.cpp"
template physecs::ConvexMeshVertices<4>::ConvexMeshVertices(const std::vector<glm::vec3>&&);
#include <cstring>
#include <cstdio>

namespace {

// Records the scene's onTriggerEnter / onTriggerExit callbacks (src/Physecs.cpp:537-552)
// as (frame, kind 0 enter / 1 exit, body0, collider0, body1, collider1), bodies as desc
// indices.
struct TriggerRecorder : physecs::OnTriggerEnterListener, physecs::OnTriggerExitListener {
    std::unordered_map<uint32_t, int> body_of;
    std::vector<int32_t> events;
    int frame = 0;
    void record(int kind, entt::entity e0, int c0, entt::entity e1, int c1) {
        const int32_t r[6] = {frame, kind, body_of.at((uint32_t)e0), c0, body_of.at((uint32_t)e1), c1};
        events.insert(events.end(), r, r + 6);
    }
    void onTriggerEnter(entt::entity e0, int c0, entt::entity e1, int c1) override { record(0, e0, c0, e1, c1); }
    void onTriggerExit(entt::entity e0, int c0, entt::entity e1, int c1) override { record(1, e0, c0, e1, c1); }
};

struct RefWorld {
    entt::registry registry;
    std::unique_ptr<physecs::Scene> scene;
    std::vector<entt::entity> entities;
    std::vector<std::unique_ptr<physecs::ConvexMesh>> convex;
    std::vector<std::unique_ptr<physecs::TriangleMesh>> trimesh;
    TriggerRecorder triggers;
    std::vector<physecs::Joint*> joints;   // by joint index; null once destroyed
};

glm::vec3 v3(const float* p) { return glm::vec3(p[0], p[1], p[2]); }
glm::quat q4(const float* p) { return glm::quat(p[3], p[0], p[1], p[2]); }

physecs::Collider make_collider(RefWorld& w, const psx_scene_desc* d, int c) {
    physecs::Collider col{};
    col.position = v3(d->col_pos + 3 * c);
    col.orientation = q4(d->col_quat + 4 * c);
    const float* p = d->col_params + 4 * c;
    switch (d->col_type[c]) {
        case PSX_SPHERE: col.geometry.type = physecs::SPHERE; col.geometry.sphere = {p[0]}; break;
        case PSX_CAPSULE: col.geometry.type = physecs::CAPSULE; col.geometry.capsule = {p[0], p[1]}; break;
        case PSX_BOX: col.geometry.type = physecs::BOX; col.geometry.box = {glm::vec3(p[0], p[1], p[2])}; break;
        case PSX_CONVEX_MESH:
            col.geometry.type = physecs::CONVEX_MESH;
            col.geometry.convex.mesh = w.convex[d->col_mesh[c]].get();
            col.geometry.convex.scale = glm::vec3(p[0], p[1], p[2]);
            break;
        case PSX_TRIANGLE_MESH:
            col.geometry.type = physecs::TRIANGLE_MESH;
            col.geometry.triangleMesh.mesh = w.trimesh[d->col_mesh[c]].get();
            break;
    }
    const float* m = d->col_material + 3 * c;
    col.material = {m[0], m[1], m[2]};
    col.isTrigger = d->col_is_trigger ? d->col_is_trigger[c] != 0 : false;
    col.enableSimulation = d->col_enable_sim ? d->col_enable_sim[c] != 0 : true;
    col.data = d->col_data ? d->col_data[c] : 0;
    return col;
}

}  // namespace

// Scene::createJoint<T> for a psx joint record, configured as the user sets it up
physecs::Joint* make_joint(RefWorld& w, int type, int b0, int b1, const float* f, const float* p) {
    entt::entity e0 = w.entities[b0];
    entt::entity e1 = w.entities[b1];
    glm::vec3 p0 = v3(f), p1 = v3(f + 7);
    glm::quat o0 = q4(f + 3), o1 = q4(f + 10);
    switch (type) {
        case PSX_JOINT_FIXED: return w.scene->createJoint<physecs::FixedJoint>(e0, p0, o0, e1, p1, o1);
        case PSX_JOINT_REVOLUTE: {
            auto* jt = w.scene->createJoint<physecs::RevoluteJoint>(e0, p0, o0, e1, p1, o1);
            jt->setDriveEnabled(p[0] != 0.f);
            jt->setDriveVelocity(p[1]);
            jt->setDriveMaxTorque(p[2]);
            return jt;
        }
        case PSX_JOINT_SPHERICAL: return w.scene->createJoint<physecs::SphericalJoint>(e0, p0, o0, e1, p1, o1);
        case PSX_JOINT_PRISMATIC: {
            auto* jt = w.scene->createJoint<physecs::PrismaticJoint>(e0, p0, o0, e1, p1, o1);
            jt->setUpperLimit(p[0]);
            jt->setLowerLimit(p[1]);
            jt->setDriveEnabled(p[2] != 0.f);
            jt->setTargetPosition(p[3]);
            jt->setDriveStiffness(p[4]);
            jt->setDriveDamping(p[5]);
            return jt;
        }
        case PSX_JOINT_UNIVERSAL: return w.scene->createJoint<physecs::UniversalJoint>(e0, p0, o0, e1, p1, o1);
        case PSX_JOINT_GEAR: {
            auto* jt = w.scene->createJoint<physecs::GearJoint>(e0, p0, o0, e1, p1, o1);
            jt->setGearRatio(p[0]);
            return jt;
        }
        case PSX_JOINT_SERVO: {
            auto* jt = w.scene->createJoint<physecs::ServoJoint>(e0, p0, o0, e1, p1, o1);
            jt->setTargetAngle(p[0]);
            jt->setDriveStiffness(p[1]);
            jt->setDriveDamping(p[2]);
            return jt;
        }
    }
    return nullptr;
}

extern "C" {

void* ref_scene_create(const psx_scene_desc* d, int num_threads) {
    auto* w = new RefWorld();
    for (int m = 0; m < d->n_convex; ++m) {
        std::vector<glm::vec3> verts;
        for (int v = d->convex_vert_start[m]; v < d->convex_vert_start[m + 1]; ++v) verts.push_back(v3(d->convex_verts + 3 * v));
        std::vector<physecs::ConvexMeshFace> faces;
        for (int f = d->convex_face_start[m]; f < d->convex_face_start[m + 1]; ++f) {
            physecs::ConvexMeshFace face;
            for (int k = d->face_index_start[f]; k < d->face_index_start[f + 1]; ++k) face.indices.push_back(d->face_indices[k]);
            face.normal = v3(d->face_normal + 3 * f);
            face.centroid = v3(d->face_centroid + 3 * f);
            faces.push_back(face);
        }
        w->convex.emplace_back(new physecs::ConvexMesh(std::move(verts), std::move(faces)));
    }
    for (int m = 0; m < d->n_trimesh; ++m) {
        std::vector<glm::vec3> verts;
        for (int v = d->tri_vert_start[m]; v < d->tri_vert_start[m + 1]; ++v) verts.push_back(v3(d->tri_verts + 3 * v));
        std::vector<unsigned int> idx(d->tri_indices + d->tri_index_start[m], d->tri_indices + d->tri_index_start[m + 1]);
        w->trimesh.emplace_back(new physecs::TriangleMesh(verts, idx));
    }
    w->scene.reset(new physecs::Scene(w->registry, num_threads));
    w->scene->setNumSubSteps(d->num_substeps);
    w->scene->setNumIterations(d->num_iterations);
    w->scene->setGravity(d->gravity);
    w->scene->addOnTriggerEnterCallback(&w->triggers);
    w->scene->addOnTriggerExitCallback(&w->triggers);
    for (int b = 0; b < d->n_bodies; ++b) {
        entt::entity e = w->registry.create();
        if ((uint32_t)e != d->entity[b]) {
            std::fprintf(stderr, "ref_scene_create: entity %u != desc %u\n", (uint32_t)e, d->entity[b]);
        }
        w->entities.push_back(e);
        w->triggers.body_of[(uint32_t)e] = b;
        w->registry.emplace<TransformComponent>(e, v3(d->pos + 3 * b), q4(d->quat + 4 * b), glm::vec3(1));
        std::vector<physecs::Collider> cols;
        for (int c = d->collider_start[b]; c < d->collider_start[b + 1]; ++c) cols.push_back(make_collider(*w, d, c));
        w->registry.emplace<physecs::RigidBodyCollisionComponent>(e, cols);
        if (d->flags[b] & PSX_BODY_DYNAMIC) {
            glm::mat3 invI;
            for (int k = 0; k < 9; ++k) invI[k / 3][k % 3] = d->inv_inertia[9 * b + k];
            w->registry.emplace<physecs::RigidBodyDynamicComponent>(
                e, (d->flags[b] & PSX_BODY_KINEMATIC) != 0, v3(d->vel + 3 * b), v3(d->ang_vel + 3 * b),
                d->inv_mass[b], v3(d->com + 3 * b), invI);
        }
    }
    for (int j = 0; j < d->n_joints; ++j)
        w->joints.push_back(make_joint(*w, d->joint_type[j], d->joint_body0[j], d->joint_body1[j], d->joint_frames + 14 * j,
                                       d->joint_params + PSX_JOINT_PARAMS * j));
    return w;
}

void ref_scene_destroy(void* h) {
    auto* w = static_cast<RefWorld*>(h);
    w->scene.reset();
    delete w;
}

void ref_scene_step(void* h, float dt) {
    auto* w = static_cast<RefWorld*>(h);
    w->scene->simulate(dt);
    ++w->triggers.frame;
}

// physecs::CharacterController(scene, entity, height, radius, maxStepHeight, slopeLimit,
// numIterations).move(translation, deltaTime); returns the flags' value
int ref_character_move(void* h, int b, float height, float radius, float max_step, float slope, int iterations,
                       const float* translation, float dt) {
    auto* w = static_cast<RefWorld*>(h);
    physecs::CharacterController cc(*w->scene, w->entities[b], height, radius, max_step, slope, iterations);
    return cc.move(v3(translation), dt).value;
}

// A new entity as a Physecs user makes one (Transform, RigidBodyCollisionComponent, then
// RigidBodyDynamicComponent for a dynamic body) from body 0 of d, whose meshes index this
// scene's; returns the body index and writes the entity value
int ref_scene_create_body(void* h, const psx_scene_desc* d, uint32_t* entity) {
    auto* w = static_cast<RefWorld*>(h);
    entt::entity e = w->registry.create();
    w->registry.emplace<TransformComponent>(e, v3(d->pos), q4(d->quat), glm::vec3(1));
    std::vector<physecs::Collider> cols;
    for (int c = d->collider_start[0]; c < d->collider_start[1]; ++c) cols.push_back(make_collider(*w, d, c));
    w->registry.emplace<physecs::RigidBodyCollisionComponent>(e, cols);
    if (d->flags[0] & PSX_BODY_DYNAMIC) {
        glm::mat3 invI;
        for (int k = 0; k < 9; ++k) invI[k / 3][k % 3] = d->inv_inertia[k];
        w->registry.emplace<physecs::RigidBodyDynamicComponent>(e, (d->flags[0] & PSX_BODY_KINEMATIC) != 0, v3(d->vel),
                                                                 v3(d->ang_vel), d->inv_mass[0], v3(d->com), invI);
    }
    const int b = (int)w->entities.size();
    w->entities.push_back(e);
    w->triggers.body_of[(uint32_t)e] = b;
    *entity = (uint32_t)e;
    return b;
}

// Scene::createJoint between frames (a psx joint record); returns the joint index
int ref_scene_create_joint(void* h, int type, int b0, int b1, const float* frames, const float* params) {
    auto* w = static_cast<RefWorld*>(h);
    w->joints.push_back(make_joint(*w, type, b0, b1, frames, params));
    return (int)w->joints.size() - 1;
}

// The setters of joint j's class with a psx parameter block, as make_joint applies them
void ref_scene_set_joint_params(void* h, int j, const float* p) {
    auto* w = static_cast<RefWorld*>(h);
    physecs::Joint* jt = w->joints[j];
    if (auto* r = dynamic_cast<physecs::RevoluteJoint*>(jt)) {
        r->setDriveEnabled(p[0] != 0.f); r->setDriveVelocity(p[1]); r->setDriveMaxTorque(p[2]);
    } else if (auto* r = dynamic_cast<physecs::PrismaticJoint*>(jt)) {
        r->setUpperLimit(p[0]); r->setLowerLimit(p[1]); r->setDriveEnabled(p[2] != 0.f);
        r->setTargetPosition(p[3]); r->setDriveStiffness(p[4]); r->setDriveDamping(p[5]);
    } else if (auto* r = dynamic_cast<physecs::GearJoint*>(jt)) {
        r->setGearRatio(p[0]);
    } else if (auto* r = dynamic_cast<physecs::ServoJoint*>(jt)) {
        r->setTargetAngle(p[0]); r->setDriveStiffness(p[1]); r->setDriveDamping(p[2]);
    }
}

// Scene::destroyJoint of joint j
void ref_scene_destroy_joint(void* h, int j) {
    auto* w = static_cast<RefWorld*>(h);
    w->scene->destroyJoint(w->joints[j]);
    w->joints[j] = nullptr;
}

// Scene::addCollider(entity of body b, collider 0 of d) / Scene::clearColliders
void ref_scene_add_collider(void* h, int b, const psx_scene_desc* d) {
    auto* w = static_cast<RefWorld*>(h);
    w->scene->addCollider(w->entities[b], make_collider(*w, d, 0));
}

void ref_scene_clear_colliders(void* h, int b) {
    auto* w = static_cast<RefWorld*>(h);
    w->scene->clearColliders(w->entities[b]);
}

// registry.destroy of body b's entity
void ref_scene_destroy_body(void* h, int b) {
    auto* w = static_cast<RefWorld*>(h);
    w->registry.destroy(w->entities[b]);
    w->entities[b] = entt::null;
}

// Scene::setContactFilter with the caller's function (null: the default filter)
void ref_scene_set_contact_filter(void* h, physecs::ContactType (*f)(bool, int, bool, int)) {
    static_cast<RefWorld*>(h)->scene->setContactFilter(f ? f : physecs::defaultContactFilter);
}

// Scene::setCanCollide for the entities of bodies b0 and b1
void ref_scene_set_can_collide(void* h, int b0, int b1, int can) {
    auto* w = static_cast<RefWorld*>(h);
    w->scene->setCanCollide(w->entities[b0], w->entities[b1], can != 0);
}

// Registry deltas as a Physecs user makes them, in array order: a pose written to the
// TransformComponent and patched, velocities written to the RigidBodyDynamicComponent,
// Scene::setIsKinematic (psx_body_delta; the scene field is unused)
void ref_scene_apply_deltas(void* h, int n, const psx_body_delta* d) {
    auto* w = static_cast<RefWorld*>(h);
    for (int i = 0; i < n; ++i) {
        const psx_body_delta& e = d[i];
        entt::entity ent = w->entities[e.body];
        if (e.mask & PSX_DELTA_POSE) {
            auto& t = w->registry.get<TransformComponent>(ent);
            t.position = v3(e.pos);
            t.orientation = q4(e.quat);
            w->registry.patch<TransformComponent>(ent);
        }
        if (e.mask & PSX_DELTA_VELOCITY) {
            auto& dyn = w->registry.get<physecs::RigidBodyDynamicComponent>(ent);
            dyn.velocity = v3(e.vel);
            dyn.angularVelocity = v3(e.ang_vel);
        }
        if (e.mask & PSX_DELTA_KINEMATIC) w->scene->setIsKinematic(ent, e.kinematic != 0);
    }
}

// physecs::TriangleMesh(vertices, indices) of the reference, dumped in the layout of
// orc_trimesh_build (20 words per triangle, 8 per node).  Returns the node count, or -1
// when the constructor throws (a mesh without triangles: its bvh.reserve(2.f * 0 - 1)
// asks for a size_t above the maximum, src/TriangleMesh.cpp:161).
int ref_trimesh_build(const float* verts, int nv, const uint32_t* idx, int nidx, uint32_t* tris, uint32_t* nodes) {
    std::vector<glm::vec3> v(nv);
    for (int i = 0; i < nv; ++i) v[i] = v3(verts + 3 * i);
    std::unique_ptr<physecs::TriangleMesh> mp;
    try {
        mp.reset(new physecs::TriangleMesh(v, std::vector<unsigned int>(idx, idx + nidx)));
    } catch (const std::exception&) {
        return -1;
    }
    const physecs::TriangleMesh& m = *mp;
    auto put = [](uint32_t* o, glm::vec3 a) { std::memcpy(o, &a.x, 4); std::memcpy(o + 1, &a.y, 4); std::memcpy(o + 2, &a.z, 4); o[3] = 0; };
    for (size_t t = 0; t < m.triangles.size(); ++t) {
        const physecs::Triangle& tr = m.triangles[t];
        uint32_t* o = tris + 20 * t;
        o[0] = tr.indices[0]; o[1] = tr.indices[1]; o[2] = tr.indices[2]; o[3] = 0;
        put(o + 4, tr.bounds.min); put(o + 8, tr.bounds.max); put(o + 12, tr.normal); put(o + 16, tr.centroid);
    }
    for (size_t k = 0; k < m.bvh.size(); ++k) {
        const physecs::TriangleMeshBVHNode& n = m.bvh[k];
        uint32_t* o = nodes + 8 * k;
        put(o, n.bounds.min); o[3] = (uint32_t)n.triCount;
        put(o + 4, n.bounds.max); o[7] = (uint32_t)n.index;
    }
    return (int)m.bvh.size();
}

// The trigger callbacks recorded since the last call, in callback order: up to cap
// records of 6 ints, removed; returns the number pending before the call
int ref_scene_trigger_events(void* h, int32_t* out, int cap) {
    auto& ev = static_cast<RefWorld*>(h)->triggers.events;
    const int n = (int)ev.size() / 6;
    const int m = n < cap ? n : cap;
    if (m) std::memcpy(out, ev.data(), sizeof(int32_t) * 6 * m);
    ev.erase(ev.begin(), ev.begin() + 6 * m);
    return n;
}

void ref_scene_set_knobs(void* h, int substeps, int iterations, float gravity) {
    auto* w = static_cast<RefWorld*>(h);
    w->scene->setNumSubSteps(substeps);
    w->scene->setNumIterations(iterations);
    w->scene->setGravity(gravity);
}

/* Body state in desc order. */
void ref_scene_read(void* h, float* pos, float* quat, float* vel, float* ang_vel) {
    auto* w = static_cast<RefWorld*>(h);
    for (size_t b = 0; b < w->entities.size(); ++b) {
        if (w->entities[b] == entt::null) {   // a destroyed entity reads as zeros
            std::memset(pos + 3 * b, 0, 12); std::memset(quat + 4 * b, 0, 16);
            std::memset(vel + 3 * b, 0, 12); std::memset(ang_vel + 3 * b, 0, 12);
            continue;
        }
        auto& t = w->registry.get<TransformComponent>(w->entities[b]);
        pos[3 * b + 0] = t.position.x; pos[3 * b + 1] = t.position.y; pos[3 * b + 2] = t.position.z;
        quat[4 * b + 0] = t.orientation.x; quat[4 * b + 1] = t.orientation.y;
        quat[4 * b + 2] = t.orientation.z; quat[4 * b + 3] = t.orientation.w;
        auto* dyn = w->registry.try_get<physecs::RigidBodyDynamicComponent>(w->entities[b]);
        glm::vec3 v(0), a(0);
        if (dyn) { v = dyn->velocity; a = dyn->angularVelocity; }
        vel[3 * b + 0] = v.x; vel[3 * b + 1] = v.y; vel[3 * b + 2] = v.z;
        ang_vel[3 * b + 0] = a.x; ang_vel[3 * b + 1] = a.y; ang_vel[3 * b + 2] = a.z;
    }
}

/* Overwrite body state (a user patching components between frames). */
void ref_scene_write(void* h, const float* pos, const float* quat, const float* vel, const float* ang_vel) {
    auto* w = static_cast<RefWorld*>(h);
    for (size_t b = 0; b < w->entities.size(); ++b) {
        if (w->entities[b] == entt::null) continue;
        auto& t = w->registry.get<TransformComponent>(w->entities[b]);
        t.position = v3(pos + 3 * b);
        t.orientation = q4(quat + 4 * b);
        auto* dyn = w->registry.try_get<physecs::RigidBodyDynamicComponent>(w->entities[b]);
        if (dyn) { dyn->velocity = v3(vel + 3 * b); dyn->angularVelocity = v3(ang_vel + 3 * b); }
    }
}

/* Broadphase pairs of the last simulate(): {entity0, collider0, entity1, collider1}. */
int ref_scene_pairs(void* h, int32_t* out, int cap) {
    auto* w = static_cast<RefWorld*>(h);
    int n = (int)w->scene->potentialContacts.size();
    for (int i = 0; i < n && i < cap; ++i) {
        auto& p = w->scene->potentialContacts[i];
        out[4 * i + 0] = (int32_t)(uint32_t)p.entity0;
        out[4 * i + 1] = p.colliderIndex0;
        out[4 * i + 2] = (int32_t)(uint32_t)p.entity1;
        out[4 * i + 3] = p.colliderIndex1;
    }
    return n;
}

/* Broadphase entry bounds in broadphase order: ids {entity, collider}, bounds {min, max}. */
int ref_scene_bounds(void* h, int32_t* ids, float* bounds, int cap) {
    auto* w = static_cast<RefWorld*>(h);
    int n = (int)w->scene->broadPhaseEntries.size();
    for (int i = 0; i < n && i < cap; ++i) {
        auto& e = w->scene->broadPhaseEntries[i];
        ids[2 * i + 0] = (int32_t)(uint32_t)e.entity;
        ids[2 * i + 1] = e.colliderIndex;
        bounds[6 * i + 0] = e.bounds.min.x; bounds[6 * i + 1] = e.bounds.min.y; bounds[6 * i + 2] = e.bounds.min.z;
        bounds[6 * i + 3] = e.bounds.max.x; bounds[6 * i + 4] = e.bounds.max.y; bounds[6 * i + 5] = e.bounds.max.z;
    }
    return n;
}

/*
 * Contact constraints of the last simulate(), in solve order.
 * ids: {b0, b1, numPoints, isSoft}; f: 8 + 4*12 floats per manifold:
 *   n(3) friction frequency damping pad pad | per point r0(3) r1(3) targetVelocity c lambdaN lambdaT pad pad
 */
int ref_scene_contacts(void* h, int32_t* ids, float* f, int cap) {
    auto* w = static_cast<RefWorld*>(h);
    int n = (int)w->scene->contactConstraints.size();
    for (int i = 0; i < n && i < cap; ++i) {
        auto& c = w->scene->contactConstraints[i];
        ids[4 * i + 0] = c.b0; ids[4 * i + 1] = c.b1; ids[4 * i + 2] = c.numPoints; ids[4 * i + 3] = c.isSoft;
        float* o = f + 56 * i;
        std::memset(o, 0, 56 * sizeof(float));
        o[0] = c.n.x; o[1] = c.n.y; o[2] = c.n.z; o[3] = c.friction; o[4] = c.frequency; o[5] = c.dampingRatio;
        for (int k = 0; k < c.numPoints; ++k) {
            auto& p = c.contactPointConstraints[k];
            float* q = o + 8 + 12 * k;
            q[0] = p.r0.x; q[1] = p.r0.y; q[2] = p.r0.z; q[3] = p.r1.x; q[4] = p.r1.y; q[5] = p.r1.z;
            q[6] = p.targetVelocity; q[7] = p.c; q[8] = p.totalLambdaN; q[9] = p.totalLambdaT;
        }
    }
    return n;
}

/*
 * Narrowphase of the reference, physecs::collision (src/Collision.cpp:895),
 * run on explicit collider pairs at the scene's current poses exactly as
 * simulate() does (src/Physecs.cpp:188-213).  pairs: {body0, col0, body1, col1}
 * as desc indices (collider index local to the body).  Per manifold out:
 * ids {pair, triangleIndex, numPoints, 0}; f: normal(3) pad, then 4 x {p0(3), p1(3)}.
 */
int ref_scene_collide(void* h, int n_pairs, const int32_t* pairs, int32_t* ids, float* f, int cap) {
    auto* w = static_cast<RefWorld*>(h);
    int n = 0;
    std::vector<physecs::ContactManifold> buf;
    for (int i = 0; i < n_pairs; ++i) {
        entt::entity e0 = w->entities[pairs[4 * i + 0]], e1 = w->entities[pairs[4 * i + 2]];
        auto& col0 = w->registry.get<physecs::RigidBodyCollisionComponent>(e0).colliders[pairs[4 * i + 1]];
        auto& col1 = w->registry.get<physecs::RigidBodyCollisionComponent>(e1).colliders[pairs[4 * i + 3]];
        auto& t0 = w->registry.get<TransformComponent>(e0);
        auto& t1 = w->registry.get<TransformComponent>(e1);
        auto pos0 = t0.position + t0.orientation * col0.position;
        auto or0 = t0.orientation * col0.orientation;
        auto pos1 = t1.position + t1.orientation * col1.position;
        auto or1 = t1.orientation * col1.orientation;
        buf.clear();
        if (!physecs::collision(pos0, or0, col0.geometry, pos1, or1, col1.geometry, buf)) continue;
        for (auto& m : buf) {
            if (!m.numPoints) continue;
            if (n < cap) {
                ids[4 * n + 0] = i; ids[4 * n + 1] = m.triangleIndex; ids[4 * n + 2] = m.numPoints; ids[4 * n + 3] = 0;
                float* o = f + 28 * n;
                std::memset(o, 0, 28 * sizeof(float));
                o[0] = m.normal.x; o[1] = m.normal.y; o[2] = m.normal.z;
                for (int k = 0; k < m.numPoints; ++k) {
                    float* q = o + 4 + 6 * k;
                    q[0] = m.points[k].position0.x; q[1] = m.points[k].position0.y; q[2] = m.points[k].position0.z;
                    q[3] = m.points[k].position1.x; q[4] = m.points[k].position1.y; q[5] = m.points[k].position1.z;
                }
            }
            ++n;
        }
    }
    return n;
}

/* Joint colour chosen by Scene::addJoint (src/Physecs.cpp:690-710), in creation order. */
int ref_scene_joint_colors(void* h, int32_t* out, int cap) {
    auto* w = static_cast<RefWorld*>(h);
    int n = 0;
    for (int c = 0; c <= physecs::Scene::JointGraph::maxColors; ++c) {
        for (auto* j : w->scene->jointGraph.colors[c].joints) {
            if (n < cap) { out[2 * n] = c; out[2 * n + 1] = (int32_t)(uint32_t)j->getEntity1(); }
            ++n;
        }
    }
    return n;
}

// Scene::raycastClosest for n rays of 8 floats {unused, origin xyz, dir xyz, max
// distance}.  accept: per body (nonzero where the filter accepts the body's entity), or
// NULL for the overload without a filter.  Per ray: the body (-1: entt::null) and the
// hit position the reference reports.
void ref_scene_raycast(void* h, int n, const float* rays, const uint8_t* accept, int32_t* out_body, float* out_pos) {
    auto* w = static_cast<RefWorld*>(h);
    std::unordered_map<uint32_t, int> index;
    for (size_t b = 0; b < w->entities.size(); ++b) index[(uint32_t)w->entities[b]] = (int)b;
    std::function<bool(entt::entity)> filter = [&](entt::entity e) {
        auto it = index.find((uint32_t)e);
        return it != index.end() && accept[it->second] != 0;
    };
    for (int i = 0; i < n; ++i) {
        const float* r = rays + 8 * i;
        glm::vec3 o(r[1], r[2], r[3]), d(r[4], r[5], r[6]), hit(0.f);
        entt::entity e = accept ? w->scene->raycastClosest(o, d, r[7], filter, &hit) : w->scene->raycastClosest(o, d, r[7], &hit);
        out_body[i] = e == entt::null ? -1 : index[(uint32_t)e];
        out_pos[3 * i] = hit.x; out_pos[3 * i + 1] = hit.y; out_pos[3 * i + 2] = hit.z;
    }
}

// Scene::overlap for one shape {pos xyz, quat xyzw}, type, params, convex mesh index and
// data filter: up to cap (body, collider) pairs in the reference's order; returns the count
int ref_scene_overlap(void* h, const float* pose, int type, const float* params, int mesh, int filter, int32_t* out, int cap) {
    auto* w = static_cast<RefWorld*>(h);
    std::unordered_map<uint32_t, int> index;
    for (size_t b = 0; b < w->entities.size(); ++b) index[(uint32_t)w->entities[b]] = (int)b;
    physecs::Geometry g{};
    switch (type) {
        case PSX_SPHERE: g.type = physecs::SPHERE; g.sphere = {params[0]}; break;
        case PSX_CAPSULE: g.type = physecs::CAPSULE; g.capsule = {params[0], params[1]}; break;
        case PSX_BOX: g.type = physecs::BOX; g.box = {glm::vec3(params[0], params[1], params[2])}; break;
        case PSX_CONVEX_MESH:
            g.type = physecs::CONVEX_MESH;
            g.convex.mesh = w->convex[mesh].get();
            g.convex.scale = glm::vec3(params[0], params[1], params[2]);
            break;
        default: return 0;
    }
    auto hits = w->scene->overlap(v3(pose), glm::quat(pose[6], pose[3], pose[4], pose[5]), g, filter);
    for (int k = 0; k < (int)hits.size() && k < cap; ++k) {
        out[2 * k] = index[(uint32_t)hits[k].entity];
        out[2 * k + 1] = hits[k].colIndex;
    }
    return (int)hits.size();
}

// Scene::overlapWithMinTranslationalDistance for one shape: up to cap records of
// (body, collider) and (normal xyz, mtd) in the reference's order; returns the count
int ref_scene_overlap_mtd(void* h, const float* pose, int type, const float* params, int mesh, int32_t* out_ids, float* out_f,
                          int cap) {
    auto* w = static_cast<RefWorld*>(h);
    std::unordered_map<uint32_t, int> index;
    for (size_t b = 0; b < w->entities.size(); ++b) index[(uint32_t)w->entities[b]] = (int)b;
    physecs::Geometry g{};
    switch (type) {
        case PSX_SPHERE: g.type = physecs::SPHERE; g.sphere = {params[0]}; break;
        case PSX_CAPSULE: g.type = physecs::CAPSULE; g.capsule = {params[0], params[1]}; break;
        case PSX_BOX: g.type = physecs::BOX; g.box = {glm::vec3(params[0], params[1], params[2])}; break;
        case PSX_CONVEX_MESH:
            g.type = physecs::CONVEX_MESH;
            g.convex.mesh = w->convex[mesh].get();
            g.convex.scale = glm::vec3(params[0], params[1], params[2]);
            break;
        default: return 0;
    }
    auto hits = w->scene->overlapWithMinTranslationalDistance(v3(pose), glm::quat(pose[6], pose[3], pose[4], pose[5]), g);
    for (int k = 0; k < (int)hits.size() && k < cap; ++k) {
        out_ids[2 * k] = index[(uint32_t)hits[k].entity];
        out_ids[2 * k + 1] = hits[k].colIndex;
        out_f[4 * k] = hits[k].normal.x; out_f[4 * k + 1] = hits[k].normal.y; out_f[4 * k + 2] = hits[k].normal.z;
        out_f[4 * k + 3] = hits[k].mtd;
    }
    return (int)hits.size();
}

}  // extern "C"
