/*
 * layout_check.cpp — sizes and member offsets of the registry components that
 * physecs_gb300/Physecs.h reads, as the application's Physecs headers lay them out
 * (test infrastructure).  Prints "name value" lines.
 */
#include <cstddef>
#include <cstdio>

#include <glm/glm.hpp>
#include <glm/gtc/quaternion.hpp>

struct TransformComponent {
    glm::vec3 position;
    glm::quat orientation;
    glm::vec3 scale;
};

#include <physecs_gb300/Physecs.h>

#define P(name, v) std::printf("%s %d\n", name, (int)(v))

int main() {
    using namespace physecs;
    P("TransformComponent", sizeof(TransformComponent));
    P("TransformComponent.position", offsetof(TransformComponent, position));
    P("TransformComponent.orientation", offsetof(TransformComponent, orientation));
    P("TransformComponent.scale", offsetof(TransformComponent, scale));
    P("RigidBodyDynamicComponent", sizeof(RigidBodyDynamicComponent));
    P("RigidBodyDynamicComponent.isKinematic", offsetof(RigidBodyDynamicComponent, isKinematic));
    P("RigidBodyDynamicComponent.velocity", offsetof(RigidBodyDynamicComponent, velocity));
    P("RigidBodyDynamicComponent.angularVelocity", offsetof(RigidBodyDynamicComponent, angularVelocity));
    P("RigidBodyDynamicComponent.invMass", offsetof(RigidBodyDynamicComponent, invMass));
    P("RigidBodyDynamicComponent.com", offsetof(RigidBodyDynamicComponent, com));
    P("RigidBodyDynamicComponent.invInertiaTensor", offsetof(RigidBodyDynamicComponent, invInertiaTensor));
    P("RigidBodyCollisionComponent", sizeof(RigidBodyCollisionComponent));
    P("Collider", sizeof(Collider));
    P("Collider.position", offsetof(Collider, position));
    P("Collider.orientation", offsetof(Collider, orientation));
    P("Collider.geometry", offsetof(Collider, geometry));
    P("Collider.material", offsetof(Collider, material));
    P("Collider.isTrigger", offsetof(Collider, isTrigger));
    P("Collider.enableSimulation", offsetof(Collider, enableSimulation));
    P("Collider.data", offsetof(Collider, data));
    P("Geometry", sizeof(Geometry));
    // glm::quat members as the shim reads them: x, y, z, w
    glm::quat q(4.f, 1.f, 2.f, 3.f);   // (w, x, y, z)
    const float* f = &q.x;
    P("quat.x", (int)q.x);
    P("quat.storage0", (int)f[0]);
    P("quat.storage3", (int)f[3]);
    return 0;
}
