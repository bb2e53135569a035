/*
 * physecs_gb300/Physecs.h — drop-in replacement for Physecs's <Physecs.h>.
 *
 * physecs::Scene over an entt::registry with the public interface of the reference's
 * Scene (include/Physecs/Physecs.h:199-229), simulated on the GPU through the C ABI of
 * psx.h.  Application code that builds its registry and calls Scene, createJoint<T>
 * and the joint setters compiles unchanged against this header.
 *
 * What the application provides, as it does for Physecs itself:
 *   - its TransformComponent { glm::vec3 position; glm::quat orientation; glm::vec3 scale; }
 *     (the layout of src/Transform.h:6-10; demo/Components.h:3-7 defines its own);
 *   - the include paths of Physecs's public data-type headers (Components.h, Colliders.h,
 *     ConvexMesh.h, TriangleMesh.h, Bounds.h, PhysecsAPI.h, BVH.h), GLM and EnTT;
 *   - in exactly one translation unit, after the TransformComponent definition:
 *         #define PHYSECS_GB300_IMPLEMENTATION
 *         #include <physecs_gb300/Physecs.h>
 *     That unit also defines the out-of-line members of Physecs's asset types (Bounds,
 *     ConvexMeshVertices<4>, TriangleMesh, whose BVH is built on the device with the
 *     reference's layout), so the application links libpsx.so instead of Physecs.
 *
 * How the registry reaches the device:
 *   - The same five signals as the reference connect to the registry
 *     (src/Physecs.cpp:92-98).  Creating or destroying a collision or dynamic component,
 *     addCollider, clearColliders, createJoint and destroyJoint change the topology; the
 *     next simulate() rebuilds the device world from the registry with
 *     psx_world_recreate, which carries over what the reference's Scene keeps across
 *     such changes: each remaining collider's broadphase bounds, the restitution cache
 *     and last frame's trigger pairs between remaining colliders, every joint's colour
 *     (Scene::addJoint's lowest free colour, freed again by destroyJoint) and a gear
 *     joint's accumulated angles.
 *   - Every simulate() uploads the components' current pose and velocities (the
 *     reference reads them in place each frame, so direct writes take effect), steps the
 *     world, and writes the results back into TransformComponent and
 *     RigidBodyDynamicComponent of simulated bodies (src/Physecs.cpp:503-510, 522-530).
 *   - registry.patch<TransformComponent> marks the entity moved: its collider bounds get
 *     the margin before the next frame (onRigidBodyMove, src/Physecs.cpp:51-54).
 *   - Joint setters take effect at the next simulate().
 *   - Trigger listeners are called after each simulate(), enters before exits.
 *
 * Classes live in the inline namespace physecs::gb300: application code names them
 * physecs::Scene, physecs::RevoluteJoint ..., and their symbols cannot clash with a
 * Physecs library linked into the same program.
 */
#pragma once

#include <cstdint>
#include <functional>
#include <memory>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include <entt.hpp>
#include <glm/glm.hpp>
#include <glm/gtc/quaternion.hpp>

#include "Components.h"   // physecs::RigidBodyCollisionComponent, RigidBodyDynamicComponent, Collider, meshes
#include "BVH.h"          // physecs::BVHNode (the type of getBVH's result)
#include "psx.h"

struct TransformComponent;

namespace physecs {
inline namespace gb300 {

struct OverlapHit {
    entt::entity entity;
    int colIndex;
};

struct OverlapMtdHit {
    entt::entity entity;
    int colIndex;
    glm::vec3 normal;
    float mtd;
};

class OnTriggerEnterListener {
public:
    virtual void onTriggerEnter(entt::entity, int, entt::entity, int) = 0;
    virtual ~OnTriggerEnterListener() = default;
};

class OnTriggerExitListener {
public:
    virtual void onTriggerExit(entt::entity, int, entt::entity, int) = 0;
    virtual ~OnTriggerExitListener() = default;
};

enum ContactType { COLLISION, TRIGGER };
ContactType defaultContactFilter(bool isTrigger0, int data0, bool isTrigger1, int data1);

class Scene;

// The public interface of physecs::Joint (include/Physecs/Joint.h:47-70).  The joint
// kinds below hold the parameters their setters write and hand them to the device.
class Joint {
    friend class Scene;
    int color = -1;
    bool dirty = false;     // a setter ran since the parameters last reached the device
    int deviceIndex = -1;   // position among the device world's joints, -1 before it has one

protected:
    entt::entity entity0;
    entt::entity entity1;
    glm::vec3 anchor0Pos;
    glm::quat anchor0Or;
    glm::vec3 anchor1Pos;
    glm::quat anchor1Or;

    Joint(entt::entity entity0, glm::vec3 anchor0Pos, glm::quat anchor0Or, entt::entity entity1, glm::vec3 anchor1Pos,
          glm::quat anchor1Or)
        : entity0(entity0), entity1(entity1), anchor0Pos(anchor0Pos), anchor0Or(anchor0Or), anchor1Pos(anchor1Pos),
          anchor1Or(anchor1Or) {}
    void touch() { dirty = true; }

public:
    entt::entity getEntity0() const { return entity0; }
    entt::entity getEntity1() const { return entity1; }
    glm::vec3 getAnchor0Pos() const { return anchor0Pos; }
    glm::quat getAnchor0Or() const { return anchor0Or; }
    glm::vec3 getAnchor1Pos() const { return anchor1Pos; }
    glm::quat getAnchor1Or() const { return anchor1Or; }
    void setColor(int c) { color = c; }
    int getColor() const { return color; }
    // the PSX_JOINT_* kind and the PSX_JOINT_PARAMS parameter block (include psx.h)
    virtual int psxKind() const = 0;
    virtual void psxParams(float* p) const { (void)p; }
    virtual ~Joint() = default;
};

#define PHYSECS_GB300_JOINT_CTOR(T)                                                                                    \
    T(entt::entity entity0, glm::vec3 anchor0Pos, glm::quat anchor0Or, entt::entity entity1, glm::vec3 anchor1Pos,      \
      glm::quat anchor1Or)                                                                                             \
        : Joint(entity0, anchor0Pos, anchor0Or, entity1, anchor1Pos, anchor1Or) {}

class FixedJoint final : public Joint {
public:
    PHYSECS_GB300_JOINT_CTOR(FixedJoint)
    int psxKind() const override { return PSX_JOINT_FIXED; }
};

class SphericalJoint final : public Joint {
public:
    PHYSECS_GB300_JOINT_CTOR(SphericalJoint)
    int psxKind() const override { return PSX_JOINT_SPHERICAL; }
};

class UniversalJoint final : public Joint {
public:
    PHYSECS_GB300_JOINT_CTOR(UniversalJoint)
    int psxKind() const override { return PSX_JOINT_UNIVERSAL; }
};

// include/Physecs/Joints/RevoluteJoint.h:8-25; defaults as RevoluteJointData
class RevoluteJoint final : public Joint {
    bool driveEnabled = false;
    float driveVelocity = 0;
    float driveMaxTorque = 0;

public:
    PHYSECS_GB300_JOINT_CTOR(RevoluteJoint)
    void setDriveEnabled(bool enabled) { driveEnabled = enabled; touch(); }
    void setDriveVelocity(float velocity) { driveVelocity = velocity; touch(); }
    void setDriveMaxTorque(float maxTorque) { driveMaxTorque = maxTorque; touch(); }
    int psxKind() const override { return PSX_JOINT_REVOLUTE; }
    void psxParams(float* p) const override { p[0] = driveEnabled ? 1.f : 0.f; p[1] = driveVelocity; p[2] = driveMaxTorque; }
};

// include/Physecs/Joints/PrismaticJoint.h:7-32; defaults as PrismaticJointData.  The limit
// row is made from the current offset each frame (src/Joints/PrismaticJoint.cpp:117-150).
class PrismaticJoint final : public Joint {
    float upperLimit = 1;
    float lowerLimit = 0;
    bool driveEnabled = false;
    float targetPosition = 0;
    float driveStiffness = 5;
    float driveDamping = 1;

public:
    PHYSECS_GB300_JOINT_CTOR(PrismaticJoint)
    void setUpperLimit(float v) { upperLimit = v; touch(); }
    void setLowerLimit(float v) { lowerLimit = v; touch(); }
    void setDriveEnabled(bool v) { driveEnabled = v; touch(); }
    void setTargetPosition(float v) { targetPosition = v; touch(); }
    void setDriveStiffness(float v) { driveStiffness = v; touch(); }
    void setDriveDamping(float v) { driveDamping = v; touch(); }
    int psxKind() const override { return PSX_JOINT_PRISMATIC; }
    void psxParams(float* p) const override {
        p[0] = upperLimit; p[1] = lowerLimit; p[2] = driveEnabled ? 1.f : 0.f;
        p[3] = targetPosition; p[4] = driveStiffness; p[5] = driveDamping;
    }
};

// include/Physecs/Joints/GearJoint.h:5-25; the accumulated angles live on the device
class GearJoint final : public Joint {
    float gearRatio = 1;

public:
    PHYSECS_GB300_JOINT_CTOR(GearJoint)
    void setGearRatio(float r) { gearRatio = r; touch(); }
    int psxKind() const override { return PSX_JOINT_GEAR; }
    void psxParams(float* p) const override { p[0] = gearRatio; }
};

// include/Physecs/Joints/ServoJoint.h:6-24; defaults as ServoJointData
class ServoJoint final : public Joint {
    float targetAngle = 0;
    float driveStiffness = 30;
    float driveDamping = 1;

public:
    PHYSECS_GB300_JOINT_CTOR(ServoJoint)
    void setTargetAngle(float a) { targetAngle = a; touch(); }
    void setDriveStiffness(float v) { driveStiffness = v; touch(); }
    void setDriveDamping(float v) { driveDamping = v; touch(); }
    int psxKind() const override { return PSX_JOINT_SERVO; }
    void psxParams(float* p) const override { p[0] = targetAngle; p[1] = driveStiffness; p[2] = driveDamping; }
};

#undef PHYSECS_GB300_JOINT_CTOR

// physecs::Scene (include/Physecs/Physecs.h:45-230), public interface unchanged.
class Scene {
public:
    Scene(entt::registry& registry, int numThreads);

    void setNumSubSteps(int numSubSteps);
    void setNumIterations(int numIterations);
    void setGravity(float gravity);
    void simulate(float timeStep);
    entt::entity raycastClosest(glm::vec3 rayOrig, glm::vec3 rayDir, float maxDistance, glm::vec3* hitPos = nullptr);
    entt::entity raycastClosest(glm::vec3 rayOrig, glm::vec3 rayDir, float maxDistance,
                                const std::function<bool(entt::entity)>& filter, glm::vec3* hitPos = nullptr);
    std::vector<OverlapHit> overlap(glm::vec3 pos, glm::quat ori, Geometry geometry, int filter);
    std::vector<OverlapMtdHit> overlapWithMinTranslationalDistance(glm::vec3 pos, glm::quat ori, Geometry geometry);
    template <typename T>
    T* createJoint(entt::entity entity0, glm::vec3 anchor0Pos, glm::quat anchor0Or, entt::entity entity1,
                   glm::vec3 anchor1Pos, glm::quat anchor1Or) {
        T* joint = new T(entity0, anchor0Pos, anchor0Or, entity1, anchor1Pos, anchor1Or);
        addJoint(joint);
        return joint;
    }
    void destroyJoint(Joint* joint);
    void clearColliders(entt::entity entity);
    void addCollider(entt::entity entity, const Collider& collider);
    void setIsKinematic(entt::entity entity, bool isKinematic);
    void addOnTriggerEnterCallback(OnTriggerEnterListener* callback);
    void addOnTriggerExitCallback(OnTriggerExitListener* callback);
    void removeOnTriggerEnterCallback(OnTriggerEnterListener* callback);
    void removeOnTriggerExitCallback(OnTriggerExitListener* callback);
    void setCanCollide(entt::entity entity0, entt::entity entity1, bool canCollide);
    void setContactFilter(ContactType (*filter)(bool, int, bool, int));
    entt::registry& getRegistry();
    const std::vector<glm::vec3>& getContactPoints();
    const std::vector<BVHNode>& getBVH();
    const int getBHVRootId();
    ~Scene();

    // Beyond the reference: the device world (null before the first simulate()), and the
    // status of the last C-ABI call that failed (PSX_OK when none did).
    psx_world* world() const { return world_; }
    psx_status lastError() const { return error_; }

private:
    struct Pair {
        uint32_t e0, e1;
        bool operator==(const Pair& o) const { return e0 == o.e0 && e1 == o.e1; }
    };
    struct PairHash {
        size_t operator()(const Pair& p) const { return std::hash<uint64_t>{}((uint64_t)p.e0 << 32 | p.e1); }
    };

    entt::registry& registry_;
    int numSubSteps_ = 8;      // the reference's defaults (include/Physecs/Physecs.h:156-159)
    int numIterations_ = 2;
    float g_ = 9.81f;
    bool knobsDirty_ = false;
    psx_world* world_ = nullptr;
    bool rebuild_ = true;
    psx_status error_ = PSX_OK;
    std::vector<entt::entity> bodies_;                 // device body order
    std::unordered_map<uint32_t, int> bodyOf_;         // entity -> device body
    std::vector<const ConvexMesh*> convex_;            // device convex mesh order
    std::vector<Joint*> joints_;                       // creation order
    std::unordered_map<uint32_t, unsigned> jointColors_;   // per entity: colours its joints use
    std::unordered_set<Pair, PairHash> noCollide_;     // setCanCollide(false) pairs
    std::unordered_set<uint32_t> moved_;               // entities patched since the last frame
    // per entity: its first collider in the device world and how many of its colliders
    // there continue (clearColliders makes that 0; added colliders are new)
    std::unordered_map<uint32_t, std::pair<int, int>> deviceCols_;
    ContactType (*filter_)(bool, int, bool, int) = nullptr;
    std::vector<OnTriggerEnterListener*> enter_;
    std::vector<OnTriggerExitListener*> exit_;
    std::vector<float> pos_, quat_, vel_, ang_;        // page-locked staging of the body state
    std::vector<glm::vec3> contactPoints_;
    std::vector<BVHNode> bvhNodes_;

    void addJoint(Joint* joint);
    void onTopology(entt::registry&, entt::entity) { rebuild_ = true; }
    void onCollisionDestroy(entt::registry&, entt::entity e) { deviceCols_.erase((uint32_t)e); rebuild_ = true; }
    void onMove(entt::registry&, entt::entity e) { moved_.insert((uint32_t)e); }
    bool check(psx_status s) { if (s != PSX_OK) error_ = s; return s == PSX_OK; }
    void build();
    void release();
    void gather();
    void scatter();
    bool sync();
    int convexIndex(const ConvexMesh* m) const;
};

}  // namespace gb300
}  // namespace physecs

#ifdef PHYSECS_GB300_IMPLEMENTATION
#include "Physecs.inl"
#endif
