/*
 * physecs_gb300/Physecs.inl — the implementation part of physecs_gb300/Physecs.h.
 *
 * Included by Physecs.h in the one translation unit that defines
 * PHYSECS_GB300_IMPLEMENTATION; the application's TransformComponent must be defined
 * before it.  Every failure of the C ABI throws std::runtime_error with
 * psx_last_error_string(): there is no CPU fallback.
 */
#include <algorithm>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>

namespace physecs {

// ---------------------------------------------------------------- Physecs's asset types
// The out-of-line members of the data types the application's headers declare
// (include/Physecs/Bounds.h, ConvexMesh.h, TriangleMesh.h), so that no Physecs library
// is needed.  Their results equal the reference's.

glm::vec3 Bounds::getCenter() const { return (min + max) / 2.f; }

glm::vec3 Bounds::getHalfExtents() const { return max - getCenter(); }

void Bounds::expand(glm::vec3 e) {
    (e.x < 0 ? min.x : max.x) += e.x;
    (e.y < 0 ? min.y : max.y) += e.y;
    (e.z < 0 ? min.z : max.z) += e.z;
}

void Bounds::addMargin(glm::vec3 margin) {
    max += margin;
    min -= margin;
}

float Bounds::area() const {
    const glm::vec3 d = max - min;
    return 2 * (d.x * d.y + d.y * d.z + d.z * d.x);
}

// The vertex buffer is padded to a multiple of N with copies of the last vertex, so the
// hull's support function can take N vertices at a time (src/ConvexMesh.cpp:3-11).
template <int N>
ConvexMeshVertices<N>::ConvexMeshVertices(const std::vector<glm::vec3>&& vertices)
    : buffer(vertices), count((int)vertices.size()) {
    if (!buffer.empty()) buffer.resize(roundUp(count), glm::vec3(buffer.back()));
}
template ConvexMeshVertices<4>::ConvexMeshVertices(const std::vector<glm::vec3>&&);

namespace gb300 {
namespace detail {

[[noreturn]] inline void fail(const char* what) {
    throw std::runtime_error(std::string("physecs_gb300: ") + what + ": " + psx_last_error_string());
}

inline void ok(psx_status s, const char* what) {
    if (s != PSX_OK) fail(what);
}

// The index list each TriangleMesh was built from.  The mesh object keeps its triangles
// in BVH order only, and the device world rebuilds the BVH from the original order, so
// that triangle numbers (contact keys) are the mesh object's.
struct MeshSources {
    std::mutex mu;
    std::unordered_map<const TriangleMesh*, std::vector<unsigned int>> indices;
};
inline MeshSources& mesh_sources() {
    static MeshSources s;
    return s;
}

// psx_world_set_contact_filter calls a plain function while it evaluates its table; the
// application's filter is reached through this slot for the duration of the call.
inline std::mutex& filter_mutex() {
    static std::mutex m;
    return m;
}
inline ContactType (*&filter_slot())(bool, int, bool, int) {
    static ContactType (*f)(bool, int, bool, int) = nullptr;
    return f;
}
inline int32_t filter_trampoline(int32_t t0, int32_t d0, int32_t t1, int32_t d1) {
    return filter_slot()(t0 != 0, d0, t1 != 0, d1) == TRIGGER ? PSX_CONTACT_TRIGGER : PSX_CONTACT_COLLISION;
}

inline void put3(std::vector<float>& v, glm::vec3 a) { v.insert(v.end(), {a.x, a.y, a.z}); }
inline void put4(std::vector<float>& v, glm::quat q) { v.insert(v.end(), {q.x, q.y, q.z, q.w}); }

inline void shape_of(const Geometry& g, psx_overlap_query& q) {
    q.type = (int32_t)g.type;
    q.params[0] = q.params[1] = q.params[2] = 0.f;
    q.mesh = -1;
    switch (g.type) {
        case SPHERE: q.params[0] = g.sphere.radius; break;
        case CAPSULE: q.params[0] = g.capsule.halfHeight; q.params[1] = g.capsule.radius; break;
        case BOX: q.params[0] = g.box.halfExtents.x; q.params[1] = g.box.halfExtents.y; q.params[2] = g.box.halfExtents.z; break;
        case CONVEX_MESH: q.params[0] = g.convex.scale.x; q.params[1] = g.convex.scale.y; q.params[2] = g.convex.scale.z; break;
        default: break;
    }
}

}  // namespace detail
}  // namespace gb300

// physecs::TriangleMesh(vertices, indices) (src/TriangleMesh.cpp:144-164): the binned-SAH
// BVH is built on the device by psx_trimesh_build, with the reference's layout.
TriangleMesh::TriangleMesh(const std::vector<glm::vec3>& verts, const std::vector<unsigned int>& indices)
    : vertices(verts) {
    const int nt = (int)(indices.size() / 3);
    std::vector<psx_trimesh_triangle> tt((size_t)std::max(nt, 1));
    std::vector<psx_trimesh_node> nn((size_t)std::max(1, 2 * nt - 1));
    int32_t n_nodes = 0;
    gb300::detail::ok(psx_trimesh_build(0, reinterpret_cast<const float*>(verts.data()), (int32_t)verts.size(),
                                        indices.data(), (int32_t)indices.size(), tt.data(), nn.data(), &n_nodes),
                      "TriangleMesh");
    triangles.resize((size_t)nt);
    for (int t = 0; t < nt; ++t) {
        const psx_trimesh_triangle& s = tt[(size_t)t];
        Triangle& d = triangles[(size_t)t];
        for (int k = 0; k < 3; ++k) d.indices[k] = s.indices[k];
        d.bounds.min = glm::vec3(s.bounds_min[0], s.bounds_min[1], s.bounds_min[2]);
        d.bounds.max = glm::vec3(s.bounds_max[0], s.bounds_max[1], s.bounds_max[2]);
        d.normal = glm::vec3(s.normal[0], s.normal[1], s.normal[2]);
        d.centroid = glm::vec3(s.centroid[0], s.centroid[1], s.centroid[2]);
    }
    bvh.resize((size_t)n_nodes);
    for (int i = 0; i < n_nodes; ++i) {
        const psx_trimesh_node& s = nn[(size_t)i];
        bvh[(size_t)i].bounds.min = glm::vec3(s.bounds_min[0], s.bounds_min[1], s.bounds_min[2]);
        bvh[(size_t)i].bounds.max = glm::vec3(s.bounds_max[0], s.bounds_max[1], s.bounds_max[2]);
        bvh[(size_t)i].triCount = s.tri_count;
        bvh[(size_t)i].index = s.index;
    }
    auto& src = gb300::detail::mesh_sources();
    std::lock_guard<std::mutex> lock(src.mu);
    src.indices[this] = indices;
}

// TriangleMesh::overlapBvh (src/TriangleMesh.cpp:166-192): the triangles whose node bounds
// meet `bounds`, depth first, left child first.
const std::vector<int>& TriangleMesh::overlapBvh(const Bounds& b) {
    thread_local std::vector<int> out;
    thread_local std::vector<int> stack;
    out.clear();
    stack.clear();
    stack.push_back(rootId);
    while (!stack.empty()) {
        const TriangleMeshBVHNode& node = bvh[(size_t)stack.back()];
        stack.pop_back();
        const bool meet = b.min.x <= node.bounds.max.x && b.max.x >= node.bounds.min.x && b.min.y <= node.bounds.max.y &&
                          b.max.y >= node.bounds.min.y && b.min.z <= node.bounds.max.z && b.max.z >= node.bounds.min.z;
        if (!meet) continue;
        if (node.triCount) {
            for (int i = 0; i < node.triCount; ++i) out.push_back(node.index + i);
        } else {
            stack.push_back(node.index + 1);
            stack.push_back(node.index);
        }
    }
    return out;
}

namespace gb300 {

ContactType defaultContactFilter(bool isTrigger0, int, bool isTrigger1, int) {
    return (isTrigger0 || isTrigger1) ? TRIGGER : COLLISION;
}

// ---------------------------------------------------------------- Scene

// The reference connects these five signals (src/Physecs.cpp:92-98); here they mark the
// topology changed or an entity moved.  numThreads is accepted and unused: the frame runs
// on the GPU.
Scene::Scene(entt::registry& registry, int) : registry_(registry) {
    registry.on_construct<RigidBodyCollisionComponent>().connect<&Scene::onTopology>(this);
    registry.on_destroy<RigidBodyCollisionComponent>().connect<&Scene::onCollisionDestroy>(this);
    registry.on_update<TransformComponent>().connect<&Scene::onMove>(this);
    registry.on_construct<RigidBodyDynamicComponent>().connect<&Scene::onTopology>(this);
    registry.on_destroy<RigidBodyDynamicComponent>().connect<&Scene::onTopology>(this);
}

// As the reference's destructor (src/Physecs.cpp:815-821) the joints are not deleted.
Scene::~Scene() {
    registry_.on_construct<RigidBodyCollisionComponent>().disconnect<&Scene::onTopology>(this);
    registry_.on_destroy<RigidBodyCollisionComponent>().disconnect<&Scene::onCollisionDestroy>(this);
    registry_.on_update<TransformComponent>().disconnect<&Scene::onMove>(this);
    registry_.on_construct<RigidBodyDynamicComponent>().disconnect<&Scene::onTopology>(this);
    registry_.on_destroy<RigidBodyDynamicComponent>().disconnect<&Scene::onTopology>(this);
    release();
}

void Scene::setNumSubSteps(int n) { numSubSteps_ = n; knobsDirty_ = true; }
void Scene::setNumIterations(int n) { numIterations_ = n; knobsDirty_ = true; }
void Scene::setGravity(float g) { g_ = g; knobsDirty_ = true; }

void Scene::release() {
    if (!world_) return;
    for (std::vector<float>* v : {&pos_, &quat_, &vel_, &ang_})
        if (!v->empty()) psx_unpin_host(v->data());
    psx_world_destroy(world_);
    world_ = nullptr;
}

int Scene::convexIndex(const ConvexMesh* m) const {
    for (size_t i = 0; i < convex_.size(); ++i)
        if (convex_[i] == m) return (int)i;
    return -1;
}

// The device world from the registry's current contents: bodies are the entities with a
// collision component in storage order, then dynamic entities without one, then entities
// only a joint names.
void Scene::build() {
    bodies_.clear();
    bodyOf_.clear();
    convex_.clear();
    auto add = [&](entt::entity e) {
        if (bodyOf_.count((uint32_t)e)) return;
        bodyOf_[(uint32_t)e] = (int)bodies_.size();
        bodies_.push_back(e);
    };
    auto& cs = registry_.storage<RigidBodyCollisionComponent>();
    auto& ds = registry_.storage<RigidBodyDynamicComponent>();
    for (size_t i = 0; i < cs.size(); ++i) add(cs.data()[i]);
    for (size_t i = 0; i < ds.size(); ++i) add(ds.data()[i]);
    for (Joint* j : joints_) { add(j->getEntity0()); add(j->getEntity1()); }

    std::vector<uint32_t> entity, flags;
    std::vector<float> pos, quat, vel, ang, inv_mass, com, inv_i;
    std::vector<int32_t> col_start{0};
    std::vector<float> cpos, cquat, cparams, cmat;
    std::vector<int32_t> ctype, cmesh, cdata;
    std::vector<uint8_t> ctrig, cenable;
    std::vector<const TriangleMesh*> tris;
    std::vector<int32_t> col_from;   // the device world's collider each collider continues, or -1
    for (entt::entity e : bodies_) {
        auto prev = deviceCols_.find((uint32_t)e);
        const int first_new = (int)ctype.size();
        if (const auto* col = registry_.try_get<RigidBodyCollisionComponent>(e))
            for (int k = 0; k < (int)col->colliders.size(); ++k)
                col_from.push_back(prev != deviceCols_.end() && k < prev->second.second ? prev->second.first + k : -1);
        (void)first_new;
        const TransformComponent& t = registry_.get<TransformComponent>(e);
        const auto* d = registry_.try_get<RigidBodyDynamicComponent>(e);
        entity.push_back((uint32_t)e);
        flags.push_back(d ? (PSX_BODY_DYNAMIC | (d->isKinematic ? PSX_BODY_KINEMATIC : 0)) : 0);
        detail::put3(pos, t.position);
        detail::put4(quat, t.orientation);
        detail::put3(vel, d ? d->velocity : glm::vec3(0));
        detail::put3(ang, d ? d->angularVelocity : glm::vec3(0));
        inv_mass.push_back(d ? d->invMass : 0.f);
        detail::put3(com, d ? d->com : glm::vec3(0));
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) inv_i.push_back(d ? d->invInertiaTensor[c][r] : 0.f);   // column-major
        if (const auto* col = registry_.try_get<RigidBodyCollisionComponent>(e)) {
            for (const Collider& c : col->colliders) {
                detail::put3(cpos, c.position);
                detail::put4(cquat, c.orientation);
                psx_overlap_query q{};
                detail::shape_of(c.geometry, q);
                ctype.push_back(q.type);
                cparams.insert(cparams.end(), {q.params[0], q.params[1], q.params[2], 0.f});
                int mesh = -1;
                if (c.geometry.type == CONVEX_MESH) {
                    mesh = convexIndex(c.geometry.convex.mesh);
                    if (mesh < 0) { mesh = (int)convex_.size(); convex_.push_back(c.geometry.convex.mesh); }
                } else if (c.geometry.type == TRIANGLE_MESH) {
                    auto it = std::find(tris.begin(), tris.end(), c.geometry.triangleMesh.mesh);
                    mesh = (int)(it - tris.begin());
                    if (it == tris.end()) tris.push_back(c.geometry.triangleMesh.mesh);
                }
                cmesh.push_back(mesh);
                cmat.insert(cmat.end(), {c.material.friction, c.material.restitution, c.material.damping});
                ctrig.push_back(c.isTrigger ? 1 : 0);
                cenable.push_back(c.enableSimulation ? 1 : 0);
                cdata.push_back(c.data);
            }
        }
        col_start.push_back((int32_t)ctype.size());
    }
    // convex meshes: unpadded vertices and polygon faces
    std::vector<int32_t> cv_start{0}, cf_start{0}, fi_start{0}, fidx;
    std::vector<float> cverts, fnorm, fcen;
    for (const ConvexMesh* m : convex_) {
        for (int v = 0; v < m->vertices.size(); ++v) detail::put3(cverts, m->vertices[v]);
        cv_start.push_back((int32_t)(cverts.size() / 3));
        for (const ConvexMeshFace& f : m->faces) {
            fidx.insert(fidx.end(), f.indices.begin(), f.indices.end());
            fi_start.push_back((int32_t)fidx.size());
            detail::put3(fnorm, f.normal);
            detail::put3(fcen, f.centroid);
        }
        cf_start.push_back((int32_t)(fnorm.size() / 3));
    }
    // triangle meshes: vertices and the index list each was built from
    std::vector<int32_t> tv_start{0}, ti_start{0};
    std::vector<float> tverts;
    std::vector<uint32_t> tidx;
    for (const TriangleMesh* m : tris) {
        for (const glm::vec3& v : m->vertices) detail::put3(tverts, v);
        tv_start.push_back((int32_t)(tverts.size() / 3));
        auto& src = detail::mesh_sources();
        std::lock_guard<std::mutex> lock(src.mu);
        auto it = src.indices.find(m);
        if (it != src.indices.end()) {
            tidx.insert(tidx.end(), it->second.begin(), it->second.end());
        } else {   // a mesh built elsewhere: its triangles in their current order
            for (const Triangle& t : m->triangles) tidx.insert(tidx.end(), {t.indices[0], t.indices[1], t.indices[2]});
        }
        ti_start.push_back((int32_t)tidx.size());
    }
    // joints in creation order, with the colours Scene::addJoint gave them
    std::vector<int32_t> jtype, jb0, jb1, jfrom, jcolor;
    std::vector<float> jframes, jparams;
    for (Joint* j : joints_) {
        jfrom.push_back(j->deviceIndex);
        jcolor.push_back(j->getColor());
        jtype.push_back(j->psxKind());
        jb0.push_back(bodyOf_.at((uint32_t)j->getEntity0()));
        jb1.push_back(bodyOf_.at((uint32_t)j->getEntity1()));
        detail::put3(jframes, j->getAnchor0Pos());
        detail::put4(jframes, j->getAnchor0Or());
        detail::put3(jframes, j->getAnchor1Pos());
        detail::put4(jframes, j->getAnchor1Or());
        float p[PSX_JOINT_PARAMS] = {};
        j->psxParams(p);
        jparams.insert(jparams.end(), p, p + PSX_JOINT_PARAMS);
        j->dirty = false;
    }

    psx_scene_desc d{};
    d.n_bodies = (int32_t)bodies_.size();
    d.entity = entity.data(); d.flags = flags.data(); d.pos = pos.data(); d.quat = quat.data();
    d.vel = vel.data(); d.ang_vel = ang.data(); d.inv_mass = inv_mass.data(); d.com = com.data();
    d.inv_inertia = inv_i.data(); d.collider_start = col_start.data();
    d.n_colliders = (int32_t)ctype.size();
    d.col_pos = cpos.data(); d.col_quat = cquat.data(); d.col_type = ctype.data(); d.col_params = cparams.data();
    d.col_mesh = cmesh.data(); d.col_material = cmat.data(); d.col_is_trigger = ctrig.data();
    d.col_enable_sim = cenable.data(); d.col_data = cdata.data();
    d.n_convex = (int32_t)convex_.size();
    d.convex_vert_start = cv_start.data(); d.convex_verts = cverts.data(); d.convex_face_start = cf_start.data();
    d.face_index_start = fi_start.data(); d.face_indices = fidx.data(); d.face_normal = fnorm.data();
    d.face_centroid = fcen.data();
    d.n_trimesh = (int32_t)tris.size();
    d.tri_vert_start = tv_start.data(); d.tri_verts = tverts.data(); d.tri_index_start = ti_start.data();
    d.tri_indices = tidx.data();
    d.n_joints = (int32_t)joints_.size();
    d.joint_type = jtype.data(); d.joint_body0 = jb0.data(); d.joint_body1 = jb1.data();
    d.joint_frames = jframes.data(); d.joint_params = jparams.data();
    d.num_substeps = numSubSteps_; d.num_iterations = numIterations_; d.gravity = g_;
    if (!world_) {
        psx_world_opts o{};
        o.use_graph = 1;
        detail::ok(psx_world_create(&d, 1, &o, &world_), "simulate: world creation");
    } else {
        // the new topology, carrying the old world's bounds, restitution cache, trigger
        // pairs and gear angles over to the colliders and joints that continue
        psx_scene_carry carry{};
        carry.from_scene = 0;
        carry.collider_from = col_from.data();
        carry.joint_from = jfrom.data();
        carry.joint_color = jcolor.data();
        psx_world* next = nullptr;
        detail::ok(psx_world_recreate(world_, &d, 1, &carry, &next), "simulate: topology change");
        release();
        world_ = next;
    }
    rebuild_ = false;
    knobsDirty_ = false;
    deviceCols_.clear();
    for (size_t b = 0; b < bodies_.size(); ++b)
        deviceCols_[(uint32_t)bodies_[b]] = {col_start[b], col_start[b + 1] - col_start[b]};
    for (size_t j = 0; j < joints_.size(); ++j) joints_[j]->deviceIndex = (int)j;
    // setCanCollide and setContactFilter are set again on the new world
    for (const Pair& p : noCollide_) {
        auto a = bodyOf_.find(p.e0), b = bodyOf_.find(p.e1);
        if (a != bodyOf_.end() && b != bodyOf_.end())
            detail::ok(psx_world_set_can_collide(world_, 0, a->second, b->second, 0), "setCanCollide");
    }
    if (filter_ && filter_ != defaultContactFilter) {
        std::lock_guard<std::mutex> lock(detail::filter_mutex());
        detail::filter_slot() = filter_;
        detail::ok(psx_world_set_contact_filter(world_, detail::filter_trampoline), "setContactFilter");
    }
    const size_t n = bodies_.size();
    pos_.assign(3 * n, 0.f); quat_.assign(4 * n, 0.f); vel_.assign(3 * n, 0.f); ang_.assign(3 * n, 0.f);
    if (n)
        for (std::vector<float>* v : {&pos_, &quat_, &vel_, &ang_}) psx_pin_host(v->data(), v->size() * sizeof(float));
}

// Component state into the staging arrays, as the reference reads it each frame.
void Scene::gather() {
    for (size_t b = 0; b < bodies_.size(); ++b) {
        const TransformComponent& t = registry_.get<TransformComponent>(bodies_[b]);
        const auto* d = registry_.try_get<RigidBodyDynamicComponent>(bodies_[b]);
        const glm::vec3 v = d ? d->velocity : glm::vec3(0), w = d ? d->angularVelocity : glm::vec3(0);
        float* p = &pos_[3 * b]; p[0] = t.position.x; p[1] = t.position.y; p[2] = t.position.z;
        float* q = &quat_[4 * b]; q[0] = t.orientation.x; q[1] = t.orientation.y; q[2] = t.orientation.z; q[3] = t.orientation.w;
        float* u = &vel_[3 * b]; u[0] = v.x; u[1] = v.y; u[2] = v.z;
        float* a = &ang_[3 * b]; a[0] = w.x; a[1] = w.y; a[2] = w.z;
    }
}

// The frame's results into the components of simulated bodies (src/Physecs.cpp:503-510, 522-530).
void Scene::scatter() {
    for (size_t b = 0; b < bodies_.size(); ++b) {
        auto* d = registry_.try_get<RigidBodyDynamicComponent>(bodies_[b]);
        if (!d || d->isKinematic) continue;
        TransformComponent& t = registry_.get<TransformComponent>(bodies_[b]);
        const float* p = &pos_[3 * b];
        const float* q = &quat_[4 * b];
        t.position = glm::vec3(p[0], p[1], p[2]);
        t.orientation = glm::quat(q[3], q[0], q[1], q[2]);
        d->velocity = glm::vec3(vel_[3 * b], vel_[3 * b + 1], vel_[3 * b + 2]);
        d->angularVelocity = glm::vec3(ang_[3 * b], ang_[3 * b + 1], ang_[3 * b + 2]);
    }
}

// Brings the device world up to the registry: rebuilt after a topology change, otherwise
// the patched poses' bounds, joint parameters and knobs.  Returns false for an empty world.
bool Scene::sync() {
    if (rebuild_ || !world_) build();
    if (!moved_.empty()) {
        std::vector<psx_body_delta> deltas;
        for (uint32_t e : moved_) {
            auto it = bodyOf_.find(e);
            if (it == bodyOf_.end() || !registry_.all_of<RigidBodyCollisionComponent>(bodies_[(size_t)it->second])) continue;
            const TransformComponent& t = registry_.get<TransformComponent>(bodies_[(size_t)it->second]);
            psx_body_delta r{};
            r.body = it->second;
            r.mask = PSX_DELTA_POSE;
            r.pos[0] = t.position.x; r.pos[1] = t.position.y; r.pos[2] = t.position.z;
            r.quat[0] = t.orientation.x; r.quat[1] = t.orientation.y; r.quat[2] = t.orientation.z; r.quat[3] = t.orientation.w;
            deltas.push_back(r);
        }
        moved_.clear();
        if (!deltas.empty()) detail::ok(psx_world_apply_deltas(world_, (int32_t)deltas.size(), deltas.data()), "registry.patch");
    }
    for (size_t j = 0; j < joints_.size(); ++j) {
        if (!joints_[j]->dirty) continue;
        float p[PSX_JOINT_PARAMS] = {};
        joints_[j]->psxParams(p);
        detail::ok(psx_world_set_joint_params(world_, 0, (int32_t)j, p), "joint setter");
        joints_[j]->dirty = false;
    }
    if (knobsDirty_) {
        detail::ok(psx_world_set_knobs(world_, 0, numSubSteps_, numIterations_, g_), "setNumSubSteps / setNumIterations / setGravity");
        knobsDirty_ = false;
    }
    return !bodies_.empty();
}

void Scene::simulate(float timeStep) {
    if (!sync()) return;
    gather();
    detail::ok(psx_world_simulate_host(world_, timeStep, pos_.data(), quat_.data(), vel_.data(), ang_.data()), "simulate");
    scatter();
    // trigger callbacks of this frame, enters before exits (src/Physecs.cpp:537-552)
    psx_trigger_event ev[256];
    for (;;) {
        int32_t n = 0;
        detail::ok(psx_world_trigger_events(world_, ev, 256, &n, nullptr), "trigger events");
        for (int32_t i = 0; i < n; ++i) {
            const entt::entity e0{ev[i].entity0}, e1{ev[i].entity1};
            if (ev[i].kind == PSX_TRIGGER_ENTER)
                for (OnTriggerEnterListener* cb : enter_) cb->onTriggerEnter(e0, ev[i].collider0, e1, ev[i].collider1);
            else
                for (OnTriggerExitListener* cb : exit_) cb->onTriggerExit(e0, ev[i].collider0, e1, ev[i].collider1);
        }
        if (n < 256) break;
    }
}

// Scene::raycastClosest without a filter (src/Physecs.cpp:606-611) tests an empty
// std::function at every leaf and never reports a hit; so does this overload.  *hitPos
// receives the ray's end.
entt::entity Scene::raycastClosest(glm::vec3 rayOrig, glm::vec3 rayDir, float maxDistance, glm::vec3* hitPos) {
    if (hitPos) *hitPos = rayOrig + rayDir * maxDistance;
    return entt::null;
}

entt::entity Scene::raycastClosest(glm::vec3 rayOrig, glm::vec3 rayDir, float maxDistance,
                                   const std::function<bool(entt::entity)>& filter, glm::vec3* hitPos) {
    if (!filter || !sync()) {
        if (hitPos) *hitPos = rayOrig + rayDir * maxDistance;
        return entt::null;
    }
    gather();
    detail::ok(psx_world_write_bodies(world_, pos_.data(), quat_.data(), vel_.data(), ang_.data()), "raycastClosest");
    std::vector<uint8_t> accept(bodies_.size());
    for (size_t b = 0; b < bodies_.size(); ++b) accept[b] = filter(bodies_[b]) ? 1 : 0;
    psx_ray r{};
    r.origin[0] = rayOrig.x; r.origin[1] = rayOrig.y; r.origin[2] = rayOrig.z;
    r.dir[0] = rayDir.x; r.dir[1] = rayDir.y; r.dir[2] = rayDir.z;
    r.max_distance = maxDistance;
    psx_ray_hit h{};
    detail::ok(psx_world_raycast(world_, 1, &r, accept.data(), &h), "raycastClosest");
    if (h.body < 0) {
        if (hitPos) *hitPos = rayOrig + rayDir * maxDistance;
        return entt::null;
    }
    if (hitPos) *hitPos = glm::vec3(h.pos[0], h.pos[1], h.pos[2]);
    return bodies_[(size_t)h.body];
}

std::vector<OverlapHit> Scene::overlap(glm::vec3 pos, glm::quat ori, Geometry geometry, int filter) {
    std::vector<OverlapHit> out;
    if (geometry.type == TRIANGLE_MESH || !sync()) return out;
    gather();
    detail::ok(psx_world_write_bodies(world_, pos_.data(), quat_.data(), vel_.data(), ang_.data()), "overlap");
    psx_overlap_query q{};
    q.pos[0] = pos.x; q.pos[1] = pos.y; q.pos[2] = pos.z;
    q.quat[0] = ori.x; q.quat[1] = ori.y; q.quat[2] = ori.z; q.quat[3] = ori.w;
    detail::shape_of(geometry, q);
    if (geometry.type == CONVEX_MESH && (q.mesh = convexIndex(geometry.convex.mesh)) < 0)
        throw std::runtime_error("physecs_gb300: overlap: a convex mesh that no collider of the scene uses");
    q.filter = filter;
    for (int32_t cap = 256;; cap *= 4) {
        std::vector<psx_overlap_hit> hits((size_t)cap);
        int32_t count = 0;
        detail::ok(psx_world_overlap(world_, 1, &q, cap, hits.data(), &count), "overlap");
        if (count <= cap) {
            for (int32_t i = 0; i < count; ++i) out.push_back({bodies_[(size_t)hits[(size_t)i].body], hits[(size_t)i].collider});
            return out;
        }
    }
}

std::vector<OverlapMtdHit> Scene::overlapWithMinTranslationalDistance(glm::vec3 pos, glm::quat ori, Geometry geometry) {
    std::vector<OverlapMtdHit> out;
    if (geometry.type == TRIANGLE_MESH || !sync()) return out;
    gather();
    detail::ok(psx_world_write_bodies(world_, pos_.data(), quat_.data(), vel_.data(), ang_.data()),
               "overlapWithMinTranslationalDistance");
    psx_overlap_query q{};
    q.pos[0] = pos.x; q.pos[1] = pos.y; q.pos[2] = pos.z;
    q.quat[0] = ori.x; q.quat[1] = ori.y; q.quat[2] = ori.z; q.quat[3] = ori.w;
    detail::shape_of(geometry, q);
    if (geometry.type == CONVEX_MESH && (q.mesh = convexIndex(geometry.convex.mesh)) < 0)
        throw std::runtime_error("physecs_gb300: overlapWithMinTranslationalDistance: a convex mesh that no collider of "
                                 "the scene uses");
    for (int32_t cap = 256;; cap *= 4) {
        std::vector<psx_overlap_mtd_hit> hits((size_t)cap);
        int32_t count = 0;
        detail::ok(psx_world_overlap_mtd(world_, 1, &q, cap, hits.data(), &count), "overlapWithMinTranslationalDistance");
        if (count <= cap) {
            for (int32_t i = 0; i < count; ++i) {
                const psx_overlap_mtd_hit& h = hits[(size_t)i];
                out.push_back({bodies_[(size_t)h.body], h.collider, glm::vec3(h.normal[0], h.normal[1], h.normal[2]), h.mtd});
            }
            return out;
        }
    }
}

// Scene::addJoint (src/Physecs.cpp:690-710): the pair stops colliding, and the joint takes
// the lowest colour that neither entity's joints use (8 colours, then the overflow).
void Scene::addJoint(Joint* joint) {
    unsigned& c0 = jointColors_[(uint32_t)joint->getEntity0()];
    unsigned& c1 = jointColors_[(uint32_t)joint->getEntity1()];
    const unsigned used = (c0 | c1) & 0xffu;
    int i = 0;
    while (used & (1u << i)) ++i;
    c0 |= 1u << i;
    c1 |= 1u << i;
    joint->setColor(i);
    joints_.push_back(joint);
    rebuild_ = true;
}

// Scene::destroyJoint (src/Physecs.cpp:712-723)
void Scene::destroyJoint(Joint* joint) {
    auto it = std::find(joints_.begin(), joints_.end(), joint);
    if (it == joints_.end()) return;
    joints_.erase(it);
    const uint32_t e0 = (uint32_t)joint->getEntity0(), e1 = (uint32_t)joint->getEntity1();
    noCollide_.erase(Pair{std::min(e0, e1), std::max(e0, e1)});
    jointColors_[e0] &= ~(1u << joint->getColor());
    jointColors_[e1] &= ~(1u << joint->getColor());
    delete joint;
    rebuild_ = true;
}

// Scene::clearColliders / addCollider (src/Physecs.cpp:725-751)
void Scene::clearColliders(entt::entity entity) {
    registry_.get<RigidBodyCollisionComponent>(entity).colliders.clear();
    auto it = deviceCols_.find((uint32_t)entity);
    if (it != deviceCols_.end()) it->second.second = 0;
    rebuild_ = true;
}

void Scene::addCollider(entt::entity entity, const Collider& collider) {
    registry_.get<RigidBodyCollisionComponent>(entity).colliders.push_back(collider);
    rebuild_ = true;
}

// Scene::setIsKinematic (src/Physecs.cpp:753-770)
void Scene::setIsKinematic(entt::entity entity, bool isKinematic) {
    auto& d = registry_.get<RigidBodyDynamicComponent>(entity);
    d.isKinematic = isKinematic;
    if (isKinematic) {
        d.velocity = glm::vec3(0);
        d.angularVelocity = glm::vec3(0);
    }
    auto it = bodyOf_.find((uint32_t)entity);
    if (!world_ || rebuild_ || it == bodyOf_.end()) return;
    psx_body_delta r{};
    r.body = it->second;
    r.mask = PSX_DELTA_KINEMATIC;
    r.kinematic = isKinematic ? 1 : 0;
    // a body jointed in the overflow colour is refused by the device: rebuild instead
    if (psx_world_apply_deltas(world_, 1, &r) != PSX_OK) rebuild_ = true;
}

void Scene::addOnTriggerEnterCallback(OnTriggerEnterListener* cb) { enter_.push_back(cb); }
void Scene::addOnTriggerExitCallback(OnTriggerExitListener* cb) { exit_.push_back(cb); }
void Scene::removeOnTriggerEnterCallback(OnTriggerEnterListener* cb) {
    auto it = std::find(enter_.begin(), enter_.end(), cb);
    if (it != enter_.end()) enter_.erase(it);
}
void Scene::removeOnTriggerExitCallback(OnTriggerExitListener* cb) {
    auto it = std::find(exit_.begin(), exit_.end(), cb);
    if (it != exit_.end()) exit_.erase(it);
}

// Scene::setCanCollide (src/Physecs.cpp:788-793)
void Scene::setCanCollide(entt::entity entity0, entt::entity entity1, bool canCollide) {
    const uint32_t a = (uint32_t)entity0, b = (uint32_t)entity1;
    const Pair p{std::min(a, b), std::max(a, b)};
    if (canCollide) noCollide_.erase(p);
    else noCollide_.insert(p);
    auto i0 = bodyOf_.find(a), i1 = bodyOf_.find(b);
    if (!world_ || rebuild_ || i0 == bodyOf_.end() || i1 == bodyOf_.end()) return;
    detail::ok(psx_world_set_can_collide(world_, 0, i0->second, i1->second, canCollide ? 1 : 0), "setCanCollide");
}

// Scene::setContactFilter (src/Physecs.cpp:795-797)
void Scene::setContactFilter(ContactType (*filter)(bool, int, bool, int)) {
    filter_ = filter;
    if (!world_ || rebuild_) return;
    std::lock_guard<std::mutex> lock(detail::filter_mutex());
    detail::filter_slot() = filter;
    const bool dflt = !filter || filter == defaultContactFilter;
    detail::ok(psx_world_set_contact_filter(world_, dflt ? nullptr : detail::filter_trampoline), "setContactFilter");
}

entt::registry& Scene::getRegistry() { return registry_; }

// The reference never fills its contact point list, so it stays empty here too.
const std::vector<glm::vec3>& Scene::getContactPoints() { return contactPoints_; }

// The query tree lives on the device and is rebuilt for each batch of queries; there is
// no host copy, so the debug view is empty.
const std::vector<BVHNode>& Scene::getBVH() { return bvhNodes_; }
const int Scene::getBHVRootId() { return BVH::null; }

}  // namespace gb300
}  // namespace physecs
