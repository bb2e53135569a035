/*
 * world.h — the CPU oracle's restatement of physecs::Scene::simulate.
 * ORACLE (test infrastructure only; see omath.h).
 */
#pragma once
#include <array>
#include <map>
#include <memory>
#include <set>
#include <tuple>
#include <vector>
#include "geom.h"
#include "psx.h"

namespace orc {

struct Body {
    uint32_t entity;
    bool hasDyn = false, kinematic = false;
    V3 pos; Q4 q;
    V3 vel{0, 0, 0}, ang{0, 0, 0};
    float invMass = 0;
    V3 com{0, 0, 0};
    M3 invI{};
    std::vector<int> cols;      // its colliders' indices, in RigidBodyCollisionComponent order
    int dyn = -1;               // position in dynamic storage (src/Physecs.cpp:271)
    bool alive = true;          // false once its entity is destroyed
    bool simulated() const { return hasDyn && !kinematic; }
};

struct Collider {
    int body;
    int local;                  // index within its body's RigidBodyCollisionComponent
    V3 pos; Q4 q;
    Geometry g;
    float friction, restitution, damping;
    bool trigger, enable;
    int data;
};

struct BPEntry { uint32_t entity; int body; int col; Bounds b; bool enable, dynamic; };

struct CPoint {  // ContactPointConstraints, src/ContactConstraints.h:11-29
    V3 r0, r1, r0xn{}, r1xn{}, t{}, r0xt{}, r1xt{};
    float targetVelocity, c = 0, lamN = 0, lamT = 0;
    V3 r0xnt{}, r1xnt{}, r0xtt{}, r1xtt{};
    float invEffN = 0, invEffT = 0;
};

struct Contact {  // ContactConstraints, src/ContactConstraints.h:31-48
    int body0, body1;  // desc body indices (TransformComponent)
    int b0, b1;        // dynamic indices or -1
    V3 n;
    float friction;
    bool soft;
    float frequency, damping;
    int np;
    CPoint p[4];
    // provenance for ordering / parity
    int pair = -1, manifold = 0, tri = -1;
};

enum RowFlags { RF_NONE = 0, RF_SOFT = 1, RF_ANGULAR = 2, RF_LIMITED = 4 };

struct Row {  // Constraint1D / one lane of Constraint1DW (include/Physecs/Constraint1D*.h)
    int flags;
    int b0, b1;
    V3 linear{0, 0, 0}, angular0{0, 0, 0}, angular1{0, 0, 0};
    float targetVelocity = 0, c = 0, min = -FLT_MAX, max = FLT_MAX, frequency = 0, damping = 0;
    V3 linear0t{0, 0, 0}, linear1t{0, 0, 0}, angular0t{0, 0, 0}, angular1t{0, 0, 0};
    float invEffMass = 0, totalLambda = 0;
};

struct Joint {
    int type;
    int body0, body1;
    V3 a0p, a1p; Q4 a0q, a1q;
    float params[PSX_JOINT_PARAMS];
    int color = -1;
    // persistent per-joint data (PrismaticJoint.h:9-18, GearJoint.h:10-17)
    bool makeUpper = false, makeLower = false;
    float persistent0 = 0, persistent1 = 0, virtual0 = 0, virtual1 = 0;
    bool gearInit = false;
    // per-frame rows, creation order
    std::vector<Row> rows;
    V3 r0, r1;
};

struct Velocity { V3 v, w; };
struct Pseudo { V3 v, w; int count; };
struct Mass { float invMass; M3 invI; };

using CacheKey = std::tuple<uint32_t, int, uint32_t, int, int>;
struct CacheVal { int np; V3 r0[4]; float tv[4]; };

struct World {
    std::vector<Body> bodies;
    std::vector<Collider> colliders;
    std::vector<std::unique_ptr<ConvexMesh>> convex;
    std::vector<std::unique_ptr<TriangleMesh>> tri;
    std::vector<BPEntry> bp;
    std::vector<Joint> joints;
    std::vector<std::vector<int>> colors{9};   // joints per colour (src/Physecs.cpp:690-710)
    std::vector<unsigned char> colorBits;      // per body
    std::map<std::pair<uint32_t, uint32_t>, int> nonColliding;
    // Scene::setContactFilter's function (Physecs.cpp:795-797); null: the default filter
    int32_t (*contactFilter)(int32_t, int32_t, int32_t, int32_t) = nullptr;
    std::vector<int> dynBodies;                // dyn index -> body
    // the registry's entity storage (EnTT 3.12 storage<entity>): the first entAlive are in
    // use, the rest destroyed (their versions bumped), reused most recent first
    std::vector<uint32_t> entPacked;
    size_t entAlive = 0;
    int substeps = 8, iterations = 2;
    float g = 9.81f;

    std::vector<int> pairs;                    // last frame: {body0, col0, body1, col1} (desc indices / local collider)
    std::vector<Contact> contacts;
    std::map<CacheKey, CacheVal> cache, cacheTemp;
    // trigger pairs (Physecs.cpp:200-207, 537-552): the overlapping trigger pairs of the
    // last frame and of this one, {body0, collider0, body1, collider1}, and the enter (kind 0)
    // and exit (kind 1) events of every frame stepped, in step order
    std::set<std::array<int, 4>> triggerCache, triggerCacheTemp;
    struct TriggerEvent { int frame, kind, body0, col0, body1, col1; };
    std::vector<TriggerEvent> triggerEvents;
    int frame = 0;
    std::vector<Velocity> vt;
    std::vector<Pseudo> pv;
    std::vector<Mass> mt;

    // optional explicit contact solve order for the next step, as manifold keys
    // {entity0, collider0, entity1, collider1, triangleIndex}; unmatched keys set orderError
    std::vector<CacheKey> orderKeys;
    bool useOrder = false;
    int orderError = 0;

    void init(const psx_scene_desc* d);
    void step(float dt);
    void broadphase();
    void narrowphase();
    void buildJointRows();
    void updateBounds(int body, bool margin);
    V3 colPos(int c) const;
    Q4 colQ(int c) const;

    // scene queries (query.cpp): the closest accepted ray hit (collider index or -1,
    // accept: per body, NULL for all) and the colliders a shape overlaps, ascending
    int raycastClosest(V3 o, V3 d, float maxd, const uint8_t* accept, float& dist) const;
    void overlap(V3 pos, Q4 ori, const Geometry& g, int filter, std::vector<int>& out) const;
    // Scene::overlapWithMinTranslationalDistance: (collider, normal, mtd) per manifold with points
    struct MtdHit { int col; V3 n; float mtd; int tri; };
    void overlapMtd(V3 pos, Q4 ori, const Geometry& g, std::vector<MtdHit>& out) const;
    // registry changes between frames: a patched pose (onRigidBodyMove -> updateBounds),
    // written velocities, Scene::setIsKinematic (Physecs.cpp:51-54, 78-90, 753-770)
    void patchPose(int b, V3 p, Q4 q);
    void setVelocity(int b, V3 v, V3 w);
    void setIsKinematic(int b, bool kinematic);
    // Scene::setCanCollide (Physecs.cpp:788-793) for bodies b0 and b1
    void setCanCollide(int b0, int b1, bool canCollide);
    // an entity created with Transform, RigidBodyCollisionComponent and (for a dynamic
    // body) RigidBodyDynamicComponent, in that order, from body 0 of d (meshes are this
    // world's); returns the new body's index.  registry.destroy of a body's entity.
    int createBody(const psx_scene_desc* d);
    void destroyBody(int b);
    // Scene::addCollider (collider 0 of d; meshes are this world's) / clearColliders
    // (Physecs.cpp:727-751) for body b
    void addCollider(int b, const psx_scene_desc* d);
    void clearColliders(int b);
    // Scene::createJoint / destroyJoint (Physecs.cpp:690-725) for a psx joint record
    int createJoint(int type, int b0, int b1, const float* frames, const float* params);
    void destroyJoint(int j);
    // CharacterController::move for body b (CharacterController.cpp:5-45); returns the
    // CharacterCollisionFlags value
    int moveCharacter(int b, float height, float radius, float maxStepHeight, float slopeLimit, int iterations, V3 translation);
    // physecs::overlap of two colliders at the given world poses (the trigger test)
    bool overlapColliders(V3 pos0, Q4 or0, int c0, V3 pos1, Q4 or1, int c1) const;
};

}  // namespace orc
