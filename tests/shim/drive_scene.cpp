/*
 * drive_scene.cpp — one application source, compiled two ways (test infrastructure):
 *   -DDRIVE_REFERENCE  against the Physecs reference: <Physecs.h>, linked with the
 *                      reference library built from its sources;
 *   otherwise          against physecs_gb300/Physecs.h, linked with libpsx.so.
 * It does what a Physecs application does (demo/Demo.cpp:9-57): creates entities, emplaces
 * TransformComponent, RigidBodyCollisionComponent and RigidBodyDynamicComponent, builds
 * meshes, creates joints and sets their parameters, and calls Scene::simulate; between
 * frames it applies a scripted list of registry edits.  After every frame it writes each
 * body's pose and velocities.
 *
 *   drive_scene <scene file> <out file>
 * Scene file (little endian), written by tests/shim/scene_file.py:
 *   int32 counts[13]: bodies, colliders, convex meshes, convex faces, face indices,
 *                     convex vertices, joints, substeps, iterations, frames, ops,
 *                     entities the ops create, and one unused (see scene_file.py)
 *   float gravity, then the arrays in psx_scene_desc order, then the ops.
 * Out file: per frame, per body (the scene's, then the ones the ops create): pos[3]
 * quat[4] (x, y, z, w) vel[3] ang_vel[3] as float32; zeros for an entity destroyed or not
 * yet created.
 */
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <vector>

#include <glm/glm.hpp>
#include <glm/gtc/quaternion.hpp>

struct TransformComponent {
    glm::vec3 position;
    glm::quat orientation;
    glm::vec3 scale;
};

#ifdef DRIVE_REFERENCE
#include "Physecs.h"
#include "Components.h"
#include "FixedJoint.h"
#include "GearJoint.h"
#include "PrismaticJoint.h"
#include "RevoluteJoint.h"
#include "ServoJoint.h"
#include "SphericalJoint.h"
#include "UniversalJoint.h"
#else
#define PHYSECS_GB300_IMPLEMENTATION
#include <physecs_gb300/Physecs.h>
#endif

namespace {

struct Reader {
    FILE* f;
    template <class T>
    std::vector<T> read(size_t n) {
        std::vector<T> v(n);
        if (n && std::fread(v.data(), sizeof(T), n, f) != n) throw std::runtime_error("scene file truncated");
        return v;
    }
};

glm::vec3 v3(const float* p) { return glm::vec3(p[0], p[1], p[2]); }
glm::quat q4(const float* p) { return glm::quat(p[3], p[0], p[1], p[2]); }

enum Op {
    OP_KINEMATIC = 1, OP_PATCH = 2, OP_JOINT = 3, OP_VELOCITY = 4,
    OP_DESTROY = 5,        // registry.destroy(entity)
    OP_CLEAR = 6,          // Scene::clearColliders(entity)
    OP_ADD_SPHERE = 7,     // Scene::addCollider(entity, sphere of radius v[0] at offset v[1..3])
    OP_DESTROY_JOINT = 8,  // Scene::destroyJoint(joint)
    OP_SPAWN_SPHERE = 9    // a new dynamic sphere entity: radius v[0], position v[1..3], invMass v[4], invI diag v[5]
};

void set_joint(physecs::Joint* j, int type, const float* p) {
    switch (type) {
        case 1: {
            auto* r = static_cast<physecs::RevoluteJoint*>(j);
            r->setDriveEnabled(p[0] != 0.f); r->setDriveVelocity(p[1]); r->setDriveMaxTorque(p[2]);
            break;
        }
        case 3: {
            auto* r = static_cast<physecs::PrismaticJoint*>(j);
            r->setUpperLimit(p[0]); r->setLowerLimit(p[1]); r->setDriveEnabled(p[2] != 0.f);
            r->setTargetPosition(p[3]); r->setDriveStiffness(p[4]); r->setDriveDamping(p[5]);
            break;
        }
        case 5: static_cast<physecs::GearJoint*>(j)->setGearRatio(p[0]); break;
        case 6: {
            auto* r = static_cast<physecs::ServoJoint*>(j);
            r->setTargetAngle(p[0]); r->setDriveStiffness(p[1]); r->setDriveDamping(p[2]);
            break;
        }
        default: break;
    }
}

int run(const char* in, const char* out) {
    FILE* f = std::fopen(in, "rb");
    if (!f) throw std::runtime_error("cannot open the scene file");
    Reader r{f};
    auto cnt = r.read<int32_t>(13);
    const int nb = cnt[0], nc = cnt[1], nm = cnt[2], nf = cnt[3], nfi = cnt[4], ncv = cnt[5], nj = cnt[6];
    const int substeps = cnt[7], iterations = cnt[8], frames = cnt[9], nops = cnt[10], nspawn = cnt[11];
    const float gravity = r.read<float>(1)[0];
    auto flags = r.read<uint32_t>(nb);
    auto pos = r.read<float>(3 * nb), quat = r.read<float>(4 * nb), vel = r.read<float>(3 * nb), ang = r.read<float>(3 * nb);
    auto inv_mass = r.read<float>(nb), com = r.read<float>(3 * nb), inv_i = r.read<float>(9 * nb);
    auto col_start = r.read<int32_t>(nb + 1);
    auto cpos = r.read<float>(3 * nc), cquat = r.read<float>(4 * nc);
    auto ctype = r.read<int32_t>(nc);
    auto cparams = r.read<float>(4 * nc);
    auto cmesh = r.read<int32_t>(nc);
    auto cmat = r.read<float>(3 * nc);
    auto ctrig = r.read<uint8_t>(nc), cen = r.read<uint8_t>(nc);
    auto cdata = r.read<int32_t>(nc);
    auto cv_start = r.read<int32_t>(nm + 1);
    auto cverts = r.read<float>(3 * ncv);
    auto cf_start = r.read<int32_t>(nm + 1), fi_start = r.read<int32_t>(nf + 1), fidx = r.read<int32_t>(nfi);
    auto fnorm = r.read<float>(3 * nf), fcen = r.read<float>(3 * nf);
    auto jtype = r.read<int32_t>(nj), jb0 = r.read<int32_t>(nj), jb1 = r.read<int32_t>(nj);
    auto jframes = r.read<float>(14 * nj), jparams = r.read<float>(8 * nj);
    auto ops_i = r.read<int32_t>(4 * nops);
    auto ops_f = r.read<float>(8 * nops);
    std::fclose(f);

    std::vector<std::unique_ptr<physecs::ConvexMesh>> meshes;
    for (int m = 0; m < nm; ++m) {
        std::vector<glm::vec3> verts;
        for (int v = cv_start[m]; v < cv_start[m + 1]; ++v) verts.push_back(v3(&cverts[3 * v]));
        std::vector<physecs::ConvexMeshFace> faces;
        for (int k = cf_start[m]; k < cf_start[m + 1]; ++k) {
            physecs::ConvexMeshFace face;
            for (int i = fi_start[k]; i < fi_start[k + 1]; ++i) face.indices.push_back(fidx[i]);
            face.normal = v3(&fnorm[3 * k]);
            face.centroid = v3(&fcen[3 * k]);
            faces.push_back(face);
        }
        meshes.emplace_back(new physecs::ConvexMesh(std::move(verts), std::move(faces)));
    }

    entt::registry registry;
    physecs::Scene scene(registry, 0);
    scene.setNumSubSteps(substeps);
    scene.setNumIterations(iterations);
    scene.setGravity(gravity);
    std::vector<entt::entity> ents;
    for (int b = 0; b < nb; ++b) {
        entt::entity e = registry.create();
        ents.push_back(e);
        registry.emplace<TransformComponent>(e, v3(&pos[3 * b]), q4(&quat[4 * b]), glm::vec3(1));
        std::vector<physecs::Collider> cols;
        for (int c = col_start[b]; c < col_start[b + 1]; ++c) {
            physecs::Collider col{};
            col.position = v3(&cpos[3 * c]);
            col.orientation = q4(&cquat[4 * c]);
            const float* p = &cparams[4 * c];
            switch (ctype[c]) {
                case 0: col.geometry.type = physecs::SPHERE; col.geometry.sphere = {p[0]}; break;
                case 1: col.geometry.type = physecs::CAPSULE; col.geometry.capsule = {p[0], p[1]}; break;
                case 2: col.geometry.type = physecs::BOX; col.geometry.box = {glm::vec3(p[0], p[1], p[2])}; break;
                default:
                    col.geometry.type = physecs::CONVEX_MESH;
                    col.geometry.convex.mesh = meshes[cmesh[c]].get();
                    col.geometry.convex.scale = glm::vec3(p[0], p[1], p[2]);
                    break;
            }
            col.material = {cmat[3 * c], cmat[3 * c + 1], cmat[3 * c + 2]};
            col.isTrigger = ctrig[c] != 0;
            col.enableSimulation = cen[c] != 0;
            col.data = cdata[c];
            cols.push_back(col);
        }
        registry.emplace<physecs::RigidBodyCollisionComponent>(e, cols);
        if (flags[b] & 1u) {
            glm::mat3 invI;
            for (int k = 0; k < 9; ++k) invI[k / 3][k % 3] = inv_i[9 * b + k];
            registry.emplace<physecs::RigidBodyDynamicComponent>(e, (flags[b] & 2u) != 0, v3(&vel[3 * b]), v3(&ang[3 * b]),
                                                                 inv_mass[b], v3(&com[3 * b]), invI);
        }
    }
    std::vector<physecs::Joint*> joints;
    for (int j = 0; j < nj; ++j) {
        const entt::entity e0 = ents[jb0[j]], e1 = ents[jb1[j]];
        const float* fr = &jframes[14 * j];
        const glm::vec3 p0 = v3(fr), p1 = v3(fr + 7);
        const glm::quat o0 = q4(fr + 3), o1 = q4(fr + 10);
        physecs::Joint* jt = nullptr;
        switch (jtype[j]) {
            case 0: jt = scene.createJoint<physecs::FixedJoint>(e0, p0, o0, e1, p1, o1); break;
            case 1: jt = scene.createJoint<physecs::RevoluteJoint>(e0, p0, o0, e1, p1, o1); break;
            case 2: jt = scene.createJoint<physecs::SphericalJoint>(e0, p0, o0, e1, p1, o1); break;
            case 3: jt = scene.createJoint<physecs::PrismaticJoint>(e0, p0, o0, e1, p1, o1); break;
            case 4: jt = scene.createJoint<physecs::UniversalJoint>(e0, p0, o0, e1, p1, o1); break;
            case 5: jt = scene.createJoint<physecs::GearJoint>(e0, p0, o0, e1, p1, o1); break;
            default: jt = scene.createJoint<physecs::ServoJoint>(e0, p0, o0, e1, p1, o1); break;
        }
        set_joint(jt, jtype[j], &jparams[8 * j]);
        joints.push_back(jt);
    }

    FILE* o = std::fopen(out, "wb");
    if (!o) throw std::runtime_error("cannot open the output file");
    std::vector<char> dead(nb + nspawn, 0);
    int next = 0;
    for (int fr = 0; fr < frames; ++fr) {
        // registry edits scheduled before this frame
        for (; next < nops && ops_i[4 * next] == fr; ++next) {
            const int op = ops_i[4 * next + 1], idx = ops_i[4 * next + 2];
            const float* v = &ops_f[8 * next];
            if (op == OP_KINEMATIC) {
                scene.setIsKinematic(ents[idx], v[0] != 0.f);
            } else if (op == OP_PATCH) {
                registry.patch<TransformComponent>(ents[idx], [&](TransformComponent& t) {
                    t.position = v3(v);
                    t.orientation = q4(v + 3);
                });
            } else if (op == OP_JOINT) {
                set_joint(joints[idx], jtype[idx], v);
            } else if (op == OP_VELOCITY) {
                auto& d = registry.get<physecs::RigidBodyDynamicComponent>(ents[idx]);
                d.velocity = v3(v);
                d.angularVelocity = v3(v + 3);
            } else if (op == OP_DESTROY) {
                registry.destroy(ents[idx]);
                dead[idx] = 1;
            } else if (op == OP_CLEAR) {
                scene.clearColliders(ents[idx]);
            } else if (op == OP_ADD_SPHERE) {
                physecs::Collider col{};
                col.position = v3(v + 1);
                col.orientation = glm::quat(1, 0, 0, 0);
                col.geometry.type = physecs::SPHERE;
                col.geometry.sphere = {v[0]};
                col.material = {0.5f, 0.f, 0.f};
                col.enableSimulation = true;
                scene.addCollider(ents[idx], col);
            } else if (op == OP_DESTROY_JOINT) {
                scene.destroyJoint(joints[idx]);
                joints[idx] = nullptr;
            } else if (op == OP_SPAWN_SPHERE) {
                entt::entity e = registry.create();
                ents.push_back(e);
                registry.emplace<TransformComponent>(e, v3(v + 1), glm::quat(1, 0, 0, 0), glm::vec3(1));
                physecs::Collider col{};
                col.orientation = glm::quat(1, 0, 0, 0);
                col.geometry.type = physecs::SPHERE;
                col.geometry.sphere = {v[0]};
                col.material = {0.5f, 0.f, 0.f};
                col.enableSimulation = true;
                registry.emplace<physecs::RigidBodyCollisionComponent>(e, std::vector<physecs::Collider>{col});
                glm::mat3 invI(0.f);
                invI[0][0] = invI[1][1] = invI[2][2] = v[5];
                registry.emplace<physecs::RigidBodyDynamicComponent>(e, false, glm::vec3(0), glm::vec3(0), v[4], glm::vec3(0), invI);
            }
        }
        scene.simulate(1.f / 60.f);
        for (int b = 0; b < nb + nspawn; ++b) {
            float vals[13] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
            if (b < (int)ents.size() && !dead[b]) {
                const auto& t = registry.get<TransformComponent>(ents[b]);
                const auto* d = registry.try_get<physecs::RigidBodyDynamicComponent>(ents[b]);
                const glm::vec3 vv = d ? d->velocity : glm::vec3(0), aa = d ? d->angularVelocity : glm::vec3(0);
                const float row[13] = {t.position.x, t.position.y, t.position.z, t.orientation.x, t.orientation.y,
                                       t.orientation.z, t.orientation.w, vv.x, vv.y, vv.z, aa.x, aa.y, aa.z};
                std::memcpy(vals, row, sizeof vals);
            }
            std::fwrite(vals, sizeof(float), 13, o);
        }
    }
    std::fclose(o);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: drive_scene <scene file> <out file>\n");
        return 1;
    }
    try {
        return run(argv[1], argv[2]);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "drive_scene: %s\n", e.what());
        return 2;
    }
}
