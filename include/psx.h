/*
 * psx.h — C ABI of the GB300-native Physecs simulation hot path.
 *
 * This is the drop-in boundary for physecs::Scene::simulate(timeStep)
 * (Physecs src/Physecs.cpp:112-561).  Plain pointers and sizes only: no C++,
 * no torch, no CUDA types.  The library keeps every scene's state resident in
 * device memory; callers move body state in and out explicitly, the way the
 * reference reads and writes its EnTT components in place.
 *
 * Conventions
 *   - Every entry point returns psx_status; psx_last_error_string() describes
 *     the most recent failure on the calling thread.
 *   - float3 arrays are tightly packed x,y,z; quaternions are x,y,z,w (the
 *     storage order of glm::quat in TransformComponent, src/Transform.h:6-10);
 *     3x3 matrices are column-major (glm::mat3).
 *   - A scene handle is single-threaded: the caller serialises calls on it.
 */
#ifndef PSX_H
#define PSX_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define PSX_API __attribute__((visibility("default")))
#else
#define PSX_API
#endif

typedef enum psx_status {
    PSX_OK = 0,
    PSX_ERR_INVALID_ARG = 1,
    PSX_ERR_OUT_OF_MEMORY = 2,
    PSX_ERR_CAPACITY = 3,     /* a fixed-capacity device buffer overflowed */
    PSX_ERR_TIMEOUT = 4,      /* a bounded device wait gave up */
    PSX_ERR_CUDA = 5,
    PSX_ERR_NOT_READY = 6
} psx_status;

/* physecs::GeometryType, include/Physecs/Colliders.h:9 */
enum {
    PSX_SPHERE = 0,
    PSX_CAPSULE = 1,
    PSX_BOX = 2,
    PSX_CONVEX_MESH = 3,
    PSX_TRIANGLE_MESH = 4
};

/* body flags */
enum {
    PSX_BODY_DYNAMIC = 1,   /* entity carries a RigidBodyDynamicComponent */
    PSX_BODY_KINEMATIC = 2  /* RigidBodyDynamicComponent::isKinematic */
};

/* joint kinds: the Joint subclasses in include/Physecs/Joints/*.h */
enum {
    PSX_JOINT_FIXED = 0,
    PSX_JOINT_REVOLUTE = 1,
    PSX_JOINT_SPHERICAL = 2,
    PSX_JOINT_PRISMATIC = 3,
    PSX_JOINT_UNIVERSAL = 4,
    PSX_JOINT_GEAR = 5,
    PSX_JOINT_SERVO = 6
};

/*
 * Joint parameter block (8 floats per joint), by kind:
 *   REVOLUTE  [driveEnabled, driveVelocity, driveMaxTorque]        (RevoluteJoint.h:11-15)
 *   PRISMATIC [upperLimit, lowerLimit, driveEnabled, targetPosition,
 *              driveStiffness, driveDamping]                         (PrismaticJoint.h:9-18)
 *   GEAR      [gearRatio]                                            (GearJoint.h:10-17)
 *   SERVO     [targetAngle, driveStiffness, driveDamping]            (ServoJoint.h:10-14)
 *   others    unused
 */
#define PSX_JOINT_PARAMS 8

/*
 * A scene as the reference's registry holds it: entities in creation order,
 * each with a TransformComponent, a RigidBodyCollisionComponent (colliders
 * [collider_start[i], collider_start[i+1])) and optionally a
 * RigidBodyDynamicComponent (include/Physecs/Components.h:6-17).
 */
typedef struct psx_scene_desc {
    int32_t n_bodies;
    const uint32_t* entity;        /* [n] entt::entity value; orders pairs (src/Physecs.cpp:158) */
    const uint32_t* flags;         /* [n] PSX_BODY_* */
    const float* pos;              /* [n*3] TransformComponent::position */
    const float* quat;             /* [n*4] TransformComponent::orientation (x,y,z,w) */
    const float* vel;              /* [n*3] RigidBodyDynamicComponent::velocity */
    const float* ang_vel;          /* [n*3] RigidBodyDynamicComponent::angularVelocity */
    const float* inv_mass;         /* [n]   RigidBodyDynamicComponent::invMass */
    const float* com;              /* [n*3] RigidBodyDynamicComponent::com (body frame) */
    const float* inv_inertia;      /* [n*9] RigidBodyDynamicComponent::invInertiaTensor, column-major */
    const int32_t* collider_start; /* [n+1] */

    int32_t n_colliders;
    const float* col_pos;          /* [m*3] Collider::position */
    const float* col_quat;         /* [m*4] Collider::orientation (x,y,z,w) */
    const int32_t* col_type;       /* [m]   PSX_SPHERE.. */
    const float* col_params;       /* [m*4] sphere {r}; capsule {halfHeight, r}; box {hx,hy,hz};
                                             convex {sx,sy,sz}; triangle mesh {} */
    const int32_t* col_mesh;       /* [m]   convex / triangle mesh index, else -1 */
    const float* col_material;     /* [m*3] Material {friction, restitution, damping} */
    const uint8_t* col_is_trigger; /* [m] */
    const uint8_t* col_enable_sim; /* [m] */
    const int32_t* col_data;       /* [m] */

    /* ConvexMesh (include/Physecs/ConvexMesh.h:29-34): vertices and polygon faces */
    int32_t n_convex;
    const int32_t* convex_vert_start;   /* [n_convex+1] into convex_verts (unpadded) */
    const float* convex_verts;          /* [*3] */
    const int32_t* convex_face_start;   /* [n_convex+1] into the face arrays */
    const int32_t* face_index_start;    /* [n_faces+1] into face_indices */
    const int32_t* face_indices;        /* vertex indices local to the mesh */
    const float* face_normal;           /* [n_faces*3] */
    const float* face_centroid;         /* [n_faces*3] */

    /* TriangleMesh (include/Physecs/TriangleMesh.h:24-41): vertices and index triples */
    int32_t n_trimesh;
    const int32_t* tri_vert_start;      /* [n_trimesh+1] into tri_verts */
    const float* tri_verts;             /* [*3] */
    const int32_t* tri_index_start;     /* [n_trimesh+1] into tri_indices (multiple of 3) */
    const uint32_t* tri_indices;

    /* joints in creation order (Scene::createJoint, include/Physecs/Physecs.h:209-214) */
    int32_t n_joints;
    const int32_t* joint_type;     /* [j] PSX_JOINT_* */
    const int32_t* joint_body0;    /* [j] body index */
    const int32_t* joint_body1;    /* [j] body index */
    const float* joint_frames;     /* [j*14] anchor0 pos(3) quat(4), anchor1 pos(3) quat(4) */
    const float* joint_params;     /* [j*PSX_JOINT_PARAMS] */

    /* Scene knobs (include/Physecs/Physecs.h:156-159) */
    int32_t num_substeps;
    int32_t num_iterations;
    float gravity;
} psx_scene_desc;


/* ------------------------------------------------------------------------
 * Worlds: one or many independent scenes stepped together.
 *
 * A world of one scene is the drop-in for physecs::Scene; a world of many
 * scenes is the batched form (every kernel carries per-scene segment offsets).
 * Bodies are addressed scene-major: all bodies of scene 0 in desc order, then
 * scene 1, and so on.
 * ---------------------------------------------------------------------- */
typedef struct psx_world psx_world;

/* Launch shapes of the kernels whose best shape depends on the workload.  None of them
 * changes a result; 0 in a field keeps the default.  psx_world_tune picks them. */
typedef struct psx_launch_config {
    int32_t convex_warps;            /* EPA: warps (pairs) per block, 1-3 (default 1) */
    int32_t convex_blocks_per_sm;    /* EPA: blocks per SM in the grouped kernel's grid (default 8) */
    int32_t analytic_threads;        /* sphere/capsule/box pairs: threads per block, <= 256 (default 64) */
    int32_t analytic_blocks_per_sm;  /* (default 16) */
    int32_t contacts_threads;        /* convex contact generation: threads per block, <= 256 (default 64) */
    int32_t solver_smem_kb;          /* shared memory per 256-thread solver block in KB (default: by scene count) */
    int32_t large_scene_solver;      /* scenes above the block limit: 1 one thread-block cluster each (those whose
                                      * velocities fit the cluster's shared memory), 2 the whole grid, one scene
                                      * after another (default: clusters when two or more scenes fit them) */
    int32_t gjk_blocks_per_sm;       /* GJK (one thread per convex pair): 128-thread blocks per SM, 1-16 (default 16) */
    int32_t epa_lanes;               /* EPA: lanes per overlapping pair, 1, 8, 16 or 32 (default 1); below 32 a block
                                      * is one warp holding 32 / epa_lanes pairs.  1: one lane per pair with the
                                      * warp's new faces built by all of its lanes, and 16 lanes per pair for the
                                      * pairs that need more than 12 steps */
    int32_t solver_threads_min;      /* smallest solver block: 32 or 64 (scenes up to 96 dynamic bodies on 32 or 64
                                      * threads, up to 384 on 128), 128 or 256 (default: 64 for worlds of more block
                                      * scenes than two per SM, else 256) */
    int32_t epa_full_only;           /* 1: no grouped small-polytope pass: the pairs go to the full polytope
                                      * directly, or with epa_lanes 1 after the lane-per-pair pass (lowest latency
                                      * for the slowest pair); 2: the grouped pass between them (highest
                                      * throughput; default) */
    int32_t large_threads;           /* block scenes above 1024 dynamic bodies: threads per block, 128 (four blocks
                                      * an SM), 256 (two) or 512 (one, with the most shared memory; default) */
} psx_launch_config;

typedef struct psx_world_opts {
    int32_t pairs_per_collider;      /* broadphase pair capacity per collider (0: default 8); a collider
                                      * with more than 4.5 times as many partners after it in its tree's
                                      * order costs a second walk of its tree in that frame */
    int32_t manifolds_per_collider;  /* contact manifold capacity per collider (0: default 4) */
    int32_t block_scene_max_dyn;     /* scenes up to this many dynamic bodies run one per CTA (0: default 8192) */
    int32_t use_graph;               /* capture the frame in a CUDA graph after the first step */
    int32_t device;                  /* CUDA device ordinal the world lives on */
    const psx_launch_config* launch; /* kernel launch shapes, or NULL for the defaults */
} psx_world_opts;

/* Scene::Scene(registry, numThreads) plus the registry's contents
 * (src/Physecs.cpp:92-98, onRigidBodyCreate :25-37, addJoint :690-710). */
PSX_API psx_status psx_world_create(const psx_scene_desc* scenes, int32_t n_scenes, const psx_world_opts* opts,
                                    psx_world** out);
/* Scene::~Scene (src/Physecs.cpp:815-821) for every scene of the world. */
PSX_API psx_status psx_world_destroy(psx_world* w);
/* Scene::simulate(timeStep) (src/Physecs.cpp:112-561), `frames` times, every scene.
 * Asynchronous: returns once the work is queued on the world's stream. */
PSX_API psx_status psx_world_step(psx_world* w, float dt, int32_t frames);
/* Like psx_world_step, timed on the world's stream with CUDA events: total_ms for all
 * frames, stage_ms[5] = {broadphase, narrowphase, contact + joint rows, solver,
 * end-of-frame bounds} summed over the frames, kernels = kernels queued.  Waits.
 * A world created with use_graph replays its frame graph here as in psx_world_step;
 * total_ms then spans the replays.  stage_ms (when not NULL) then comes from one more
 * frame, launched eagerly after the timed ones and not counted in total_ms or kernels:
 * its stage times, each multiplied by `frames`. */
PSX_API psx_status psx_world_step_timed(psx_world* w, float dt, int32_t frames, float* total_ms, float* stage_ms,
                                        int64_t* kernels);
/* Waits for queued work and reports a device-side error (capacity, timeout). */
PSX_API psx_status psx_world_synchronize(psx_world* w);
/* The reference has no device waits.  Here a scene above the block limit that is solved
 * by the whole grid (a cooperative launch) waits at a grid barrier between colour steps.
 * Each wait polls at most `polls` times, 64 ns apart (0: the default, 2^23 polls, about
 * half a second), then gives up: every block leaves the solver, the frame's results are
 * not valid, and psx_world_synchronize returns PSX_ERR_TIMEOUT.  Takes effect from the
 * next frame. */
PSX_API psx_status psx_world_set_wait_limit(psx_world* w, int64_t polls);
/* Scene::setNumSubSteps / setNumIterations / setGravity (src/Physecs.cpp:100-110) for one scene (-1: all). */
PSX_API psx_status psx_world_set_knobs(psx_world* w, int32_t scene, int32_t substeps, int32_t iterations, float gravity);
/* Copy every body's TransformComponent and velocities out of / into device memory
 * (pos n*3, quat n*4 x,y,z,w, vel n*3, ang_vel n*3; host pointers, any may be NULL). */
PSX_API psx_status psx_world_read_bodies(psx_world* w, float* pos, float* quat, float* vel, float* ang_vel);
PSX_API psx_status psx_world_write_bodies(psx_world* w, const float* pos, const float* quat, const float* vel,
                                          const float* ang_vel);
/* The same read as psx_world_read_bodies, for callers that must not allocate while
 * they run: a frame loop with a hard deadline (cudaMalloc / cudaMallocHost can stall
 * the device for milliseconds) or a process whose device memory is already handed
 * out to its own pool.  psx_world_read_bodies grows a device staging buffer on first
 * use; this call instead packs the state on the device into one fixed array that
 * the library holds for the whole process (3.4 MB per device) and copies from there
 * into the caller's arrays.  On success it calls no allocator, host or device.
 *   - Limit: worlds of at most 65536 bodies; larger worlds get PSX_ERR_CAPACITY.
 *   - The first call on a device looks up that array's device address; make this
 *     first call before any stream capture begins.
 *   - Every call in the process shares the array.  Calls whose GPU work overlaps
 *     (different streams or host threads at once) race on it; serialise them.
 * It has no counterpart in the reference, where Scene state is host memory. */
PSX_API psx_status psx_world_read_bodies_noalloc(psx_world* w, float* pos, float* quat, float* vel, float* ang_vel);
/* One end-to-end simulate through host buffers: upload the given state, step one
 * frame, download the new state into the same buffers, and wait. */
PSX_API psx_status psx_world_simulate_host(psx_world* w, float dt, float* pos, float* quat, float* vel, float* ang_vel);
/* Autotuner: runs `frames` frames (they advance the world) for each candidate launch
 * shape of each tunable kernel, one kernel at a time, timing its stage with CUDA events;
 * keeps the fastest and writes the chosen configuration to *best.  Results do not
 * depend on the launch shapes; throughput does. */
PSX_API psx_status psx_world_tune(psx_world* w, int32_t frames, psx_launch_config* best);
/* The launch shapes in effect (after defaults, tuning or opts.launch). */
PSX_API psx_status psx_world_launch_config(psx_world* w, psx_launch_config* out);

/* ---- topology changes between frames: bodies, colliders and joints created or destroyed
 * (registry.create / registry.destroy with onRigidBodyCreate / onRigidBodyDelete /
 * onDynamicCreate / onDynamicDelete, Scene::addCollider / clearColliders, createJoint /
 * destroyJoint; src/Physecs.cpp:25-78, 690-751).  The caller describes its scenes as they
 * now are (bodies with their current state, entity values as the registry gives them,
 * joints in the order Scene keeps them) and says what continues from the old world;
 * psx_world_recreate builds the new world and moves over, on the device, what the old
 * world holds beyond the state:
 *   - each continued collider's broadphase bounds (with the 0.01 m margin if its body was
 *     simulated or patched); new colliders get creation bounds, as onRigidBodyCreate and
 *     addCollider give them;
 *   - the restitution cache between continued colliders (src/Physecs.cpp:209-316);
 *   - the trigger pairs of the last frame between continued colliders (:200-207); a pair
 *     that loses a collider exits at the end of the next frame, as the reference's next
 *     frame finds it gone (:545-551), reported with body -1 for a removed body and the
 *     entity value it had;
 *   - a continued gear joint's accumulated angles (GearJoint.h:10-17);
 *   - the frame count, launch shapes, wait limit, CUDA-graph use and device.
 * The contact filter and setCanCollide pairs are the caller's to set again. */
typedef struct psx_scene_carry {
    int32_t from_scene;             /* the old world's scene this scene continues, -1: a new scene */
    const int32_t* collider_from;   /* [n_colliders] the old scene-local collider each collider continues, -1: new */
    const int32_t* joint_from;      /* [n_joints] the old scene-local joint each joint continues, -1: new; NULL: all new */
    const int32_t* joint_color;     /* [n_joints] each joint's colour 0-8 as Scene::addJoint gave it (the lowest colour
                                     * free at both bodies when it was created; 8 is the overflow); NULL: colours
                                     * assigned greedily in the joints' order, as at creation */
} psx_scene_carry;
/* The old world stays valid until the caller destroys it. */
PSX_API psx_status psx_world_recreate(psx_world* from, const psx_scene_desc* scenes, int32_t n_scenes,
                                      const psx_scene_carry* carry, psx_world** out);

/* The setters of the joint classes (RevoluteJoint::setDriveEnabled / setDriveVelocity /
 * setDriveMaxTorque, PrismaticJoint::setUpperLimit ... setDriveDamping, GearJoint::
 * setGearRatio, ServoJoint::setTargetAngle ... setDriveDamping; include/Physecs/Joints/
 * *.h) between frames: the whole PSX_JOINT_PARAMS block of joint `joint` (index within
 * the scene's joints, in creation order) is replaced, ahead of the next frame.  A gear
 * joint keeps its accumulated angles. */
PSX_API psx_status psx_world_set_joint_params(psx_world* w, int32_t scene, int32_t joint, const float* params);

/* ---- filters of the narrowphase */
#define PSX_CONTACT_COLLISION 0
#define PSX_CONTACT_TRIGGER 1
/* ContactType (*)(bool isTrigger0, int data0, bool isTrigger1, int data1) of
 * Scene::setContactFilter (include/Physecs/Physecs.h:42-43, 224): PSX_CONTACT_TRIGGER makes
 * a pair a trigger pair (an overlap test and trigger events, no contact),
 * PSX_CONTACT_COLLISION a colliding one.  Collider 0 is the pair's lower entity. */
typedef int32_t (*psx_contact_filter)(int32_t is_trigger0, int32_t data0, int32_t is_trigger1, int32_t data1);
/* Scene::setContactFilter (src/Physecs.cpp:795-797) for every scene of the world; NULL
 * restores the default filter (a trigger collider makes a trigger pair,
 * src/Physecs.cpp:20-23).  The filter is called on the host once per pair of
 * (isTrigger, data) classes of the world's colliders (at most 1024 classes) and read on
 * the device as a table.  Waits for queued frames. */
PSX_API psx_status psx_world_set_contact_filter(psx_world* w, psx_contact_filter filter);
/* Scene::setCanCollide(entity0, entity1, canCollide) (src/Physecs.cpp:788-793): the pair
 * of bodies joins or leaves the set of pairs that never collide (jointed bodies start
 * in it).  Waits for queued frames. */
PSX_API psx_status psx_world_set_can_collide(psx_world* w, int32_t scene, int32_t body0, int32_t body1,
                                             int32_t can_collide);

/* ---- registry deltas: the changes a Physecs user makes to the registry between frames.
 * A batch applies in array order, each record's fields in the order pose, velocity,
 * kinematic:
 *   PSX_DELTA_POSE      TransformComponent written, then registry.patch: the body's
 *                       collider bounds are recomputed with the 0.01 m margin
 *                       (onRigidBodyMove -> updateBounds, src/Physecs.cpp:51-54, 78-90);
 *   PSX_DELTA_VELOCITY  RigidBodyDynamicComponent velocity and angularVelocity written;
 *   PSX_DELTA_KINEMATIC Scene::setIsKinematic(entity, kinematic) (src/Physecs.cpp:753-770):
 *                       the broadphase's dynamic flag, and zero velocities when it
 *                       becomes kinematic. */
#define PSX_DELTA_POSE 1
#define PSX_DELTA_VELOCITY 2
#define PSX_DELTA_KINEMATIC 4
typedef struct psx_body_delta {
    int32_t scene;
    int32_t body;        /* scene-local body index */
    int32_t mask;        /* PSX_DELTA_* bits */
    int32_t kinematic;   /* PSX_DELTA_KINEMATIC: the new isKinematic */
    float pos[3];
    float quat[4];       /* x, y, z, w */
    float vel[3];
    float ang_vel[3];
} psx_body_delta;
/* Queues a batch of deltas on the world's stream, ahead of the next frame: one upload of
 * the batch (coalesced per body on the host) and one kernel, plus a fix-up of the joints
 * of bodies whose kinematic flag changed.  VELOCITY and KINEMATIC need a dynamic body;
 * KINEMATIC is refused for a body with a joint in the overflow colour (a colour past
 * the eighth, whose solve steps assume the dynamic bodies of creation time). */
PSX_API psx_status psx_world_apply_deltas(psx_world* w, int32_t n, const psx_body_delta* deltas);
/* Page-locks (and releases) a caller's host buffer, e.g. the arrays handed to
 * psx_world_read_bodies / psx_world_write_bodies / psx_world_simulate_host, so that their
 * copies run at the host link's speed instead of through CUDA's own staging buffers. */
PSX_API psx_status psx_pin_host(void* p, size_t bytes);
PSX_API psx_status psx_unpin_host(void* p);

/* ---- triangle meshes: the BVH of physecs::TriangleMesh, built on the device */
typedef struct psx_trimesh_triangle {  /* Triangle (include/Physecs/TriangleMesh.h:9-14) */
    uint32_t indices[3];
    uint32_t pad;
    float bounds_min[4];               /* w = 0 */
    float bounds_max[4];
    float normal[4];
    float centroid[4];
} psx_trimesh_triangle;
typedef struct psx_trimesh_node {      /* TriangleMeshBVHNode (include/Physecs/TriangleMesh.h:16-20) */
    float bounds_min[3];
    int32_t tri_count;                 /* > 0: a leaf over triangles [index, index + tri_count) */
    float bounds_max[3];
    int32_t index;                     /* inner node: its left child (the right one follows) */
} psx_trimesh_node;
/* physecs::TriangleMesh(vertices, indices) (src/TriangleMesh.cpp:144-164) on CUDA device
 * `device`: triangles (n_indices / 3 of them) in the BVH's order and the BVH's nodes,
 * identical to the reference's (binned SAH, 6 buckets; node 0 is the root).  nodes
 * needs room for max(1, 2 * triangles - 1); *n_nodes receives the count.  Every index
 * must be below n_vertices and every vertex finite (PSX_ERR_INVALID_ARG otherwise). */
PSX_API psx_status psx_trimesh_build(int32_t device, const float* vertices, int32_t n_vertices, const uint32_t* indices,
                                     int32_t n_indices, psx_trimesh_triangle* triangles, psx_trimesh_node* nodes,
                                     int32_t* n_nodes);
/* Replaces the vertices of triangle mesh `mesh` of scene `scene` (same vertex count, same
 * indices: an edited terrain), rebuilds its BVH on the device as a new TriangleMesh over
 * them would be built, and recomputes the bounds of the colliders that use it (as at
 * creation, no margin).  Waits for the world's queued frames first. */
PSX_API psx_status psx_world_update_trimesh(psx_world* w, int32_t scene, int32_t mesh, const float* vertices);

/* ---- scene queries against the world's current state */
typedef struct psx_ray {
    int32_t scene;
    float origin[3];
    float dir[3];
    float max_distance;
} psx_ray;
typedef struct psx_ray_hit {
    int32_t body;       /* scene-local body index of the closest hit, -1: none */
    int32_t collider;   /* collider index within that body */
    uint32_t entity;
    float distance;
    float pos[3];       /* origin + dir * distance */
} psx_ray_hit;
/* Scene::raycastClosest(origin, dir, maxDistance, filter, &hitPos) for n rays
 * (src/Physecs.cpp:571-626, src/Raycast.cpp).  accept: one byte per world body
 * (scene-major), nonzero where the filter accepts the body's entity; NULL accepts every
 * entity.  (The reference's overload without a filter never reports a hit, since it
 * tests an empty std::function; a shim for that overload returns entt::null without
 * calling this.)  Among hits at exactly the same distance the collider with the lowest
 * world index wins, where the reference's choice follows its own tree. */
PSX_API psx_status psx_world_raycast(psx_world* w, int32_t n, const psx_ray* rays, const uint8_t* accept,
                                     psx_ray_hit* hits);

typedef struct psx_overlap_query {
    int32_t scene;
    float pos[3];
    float quat[4];      /* x, y, z, w */
    int32_t type;       /* PSX_SPHERE, PSX_CAPSULE, PSX_BOX, PSX_CONVEX_MESH (PSX_TRIANGLE_MESH overlaps nothing) */
    float params[3];    /* as col_params: sphere {r}; capsule {halfHeight, r}; box {halfExtents}; convex {scale} */
    int32_t mesh;       /* convex mesh index within the scene's desc */
    int32_t filter;     /* collider data bits that must meet, 0: any */
} psx_overlap_query;
typedef struct psx_overlap_hit {
    int32_t body;       /* scene-local body index */
    int32_t collider;   /* collider index within that body */
    uint32_t entity;
} psx_overlap_hit;
/* Scene::overlap(pos, ori, geometry, filter) for n shapes (src/Physecs.cpp:628-651,
 * src/Overlap.cpp).  Query i's hits are hits[i * cap, i * cap + min(counts[i], cap));
 * counts[i] is the number found (a count above cap means the list was cut).  The set
 * is the reference's; the order is this world's tree order. */
PSX_API psx_status psx_world_overlap(psx_world* w, int32_t n, const psx_overlap_query* queries, int32_t cap,
                                     psx_overlap_hit* hits, int32_t* counts);

typedef struct psx_overlap_mtd_hit {
    int32_t body;       /* scene-local body index */
    int32_t collider;   /* collider index within that body */
    uint32_t entity;
    float normal[3];    /* the collision's normal, from the collider towards the query shape */
    float mtd;          /* max(0, deepest dot(p0 - p1, normal) over the manifold's points) */
} psx_overlap_mtd_hit;
/* Scene::overlapWithMinTranslationalDistance(pos, ori, geometry) for n shapes
 * (src/Physecs.cpp:653-688): one record per manifold with points of the collision
 * between each collider and the shape (a triangle mesh yields one per touching
 * triangle manifold).  Layout as psx_world_overlap; the filter field is not used. */
PSX_API psx_status psx_world_overlap_mtd(psx_world* w, int32_t n, const psx_overlap_query* queries, int32_t cap,
                                         psx_overlap_mtd_hit* hits, int32_t* counts);
/* physecs::CharacterController (include/Physecs/CharacterController.h:17-41) */
typedef struct psx_character {
    int32_t scene;
    int32_t body;              /* the controller's entity (scene-local body); bodies of a batch differ */
    float height, radius;
    float max_step_height;     /* read only by the step-up test, which never fires (below) */
    float slope_limit;         /* cosine of the steepest slope walked up (default cos 45 degrees) */
    int32_t num_iterations;    /* default 2 */
    float translation[3];
} psx_character;
#define PSX_CHARACTER_DOWN 1
#define PSX_CHARACTER_SIDES 2
#define PSX_CHARACTER_UP 4
#define PSX_CHARACTER_TRUNCATED 0x80   /* an iteration met more than 32 contacts; the rest were skipped */
/* CharacterController::move(translation, deltaTime) (src/CharacterController.cpp:5-45) for
 * n controllers at once, on the device: the capsule (height / 2, radius) above the
 * body is pushed out of what it overlaps, num_iterations times, and the body's pose is
 * patched (its collider bounds get the 0.01 m margin).  flags_out[i] receives the
 * CharacterCollisionFlags value.  As in the reference the step-up test never changes the
 * translation: it calls Scene::raycastClosest without a filter, which never reports a
 * hit (src/Physecs.cpp:580, 615).  The hits of one iteration apply in the order
 * (collider, triangle) where the reference takes its tree's order, and the controllers
 * of one batch see each other at their poses before the batch (the reference moves
 * them one by one).  Waits. */
PSX_API psx_status psx_world_move_characters(psx_world* w, int32_t n, const psx_character* chars, float dt,
                                             uint8_t* flags_out);

/* Trigger events: Scene::simulate's onTriggerEnter / onTriggerExit callbacks
 * (src/Physecs.cpp:537-552; listeners registered by addOnTriggerEnterCallback /
 * addOnTriggerExitCallback, :772-786).  With the default contact filter
 * (src/Physecs.cpp:20-23) a broadphase pair with a trigger collider is a trigger pair:
 * its colliders are tested with physecs::overlap, and a pair overlapping in a frame but
 * not in the frame before enters, a pair overlapping in the frame before but not in this
 * one exits (src/Physecs.cpp:200-207).  A pair's colliders are in the broadphase's order
 * (the lower entity first), as the reference passes them. */
#define PSX_TRIGGER_ENTER 0
#define PSX_TRIGGER_EXIT 1
typedef struct psx_trigger_event {
    int32_t frame;      /* frame that raised it: frames stepped before it since the world's creation */
    int32_t kind;       /* PSX_TRIGGER_ENTER or PSX_TRIGGER_EXIT */
    int32_t scene;
    int32_t body0;      /* scene-local body index (-1: a body removed by psx_world_recreate) */
    int32_t collider0;  /* collider index within that body */
    int32_t body1;
    int32_t collider1;
    uint32_t entity0;
    uint32_t entity1;
} psx_trigger_event;
/* Delivers the trigger events of the frames stepped since the last call (waits for the
 * world's stream): up to cap events into out, ordered by frame, then enter before exit
 * (the reference's order), then scene, bodies and colliders (the reference's order within
 * a frame is its hash set's); events past cap stay queued for the next call.  n_lost
 * (optional) receives the events dropped since the last call because more than the
 * device log's capacity (2 x the pair capacity, at least 4096) piled up between two
 * calls.  A world without trigger colliders delivers none. */
PSX_API psx_status psx_world_trigger_events(psx_world* w, psx_trigger_event* out, int32_t cap, int32_t* n_out,
                                            int64_t* n_lost);
/* counts[12] = {bodies, colliders, dynamic bodies, joints, scenes, pairs, manifolds, error bits,
 *              contact points, joint rows, simulated bodies, kernels queued since creation}
 * (per-frame values describe the last frame) */
PSX_API psx_status psx_world_counts(psx_world* w, int32_t* counts);
/* counts[4] = {convex-mesh pairs, of them overlapping after GJK (EPA runs on these), of
 *             those the ones that outgrew the lane-per-pair EPA (12 steps), and of those
 *             the ones that outgrew the grouped EPA (36 steps)} of the last frame; EPA
 *             schedules that skip a tier report 0 for it */
PSX_API psx_status psx_world_narrow_counts(psx_world* w, int32_t* counts);
/* Inspection of the last frame (synchronises):
 *   pairs: {scene, entity0, collider0, entity1, collider1} per broadphase pair
 *   contacts: ids {scene, b0, b1, np | soft << 8, entity0, collider0, entity1, collider1} per
 *             manifold, b = scene-local dynamic index or -1; f = 56 floats per manifold
 *             (normal, friction, frequency, damping, pad, pad, then per point r0, r1,
 *             targetVelocity, c, lambdaN, lambdaT, pad, pad), in solve order (colour by
 *             colour); meta = {colour, triangleIndex} per manifold
 *   bounds: {min xyz, max xyz} per collider, desc order */
PSX_API int32_t psx_world_get_pairs(psx_world* w, int32_t* out, int32_t cap);
PSX_API int32_t psx_world_get_contacts(psx_world* w, int32_t* ids, float* f, int32_t* meta, int32_t cap);
PSX_API int32_t psx_world_get_bounds(psx_world* w, float* bounds, int32_t cap);
/* Human-readable description of the calling thread's last error. */
PSX_API const char* psx_last_error_string(void);

/* ------------------------------------------------------------------------
 * Serving: continuous batching of independent scene requests.  No counterpart
 * in the reference (one Scene per registry there); each request is a scene as
 * psx_world_create takes it plus a frame count, and its results equal those of
 * a world holding that scene alone.
 *
 * The server holds slots in size classes (class_bodies ascending, bodies per
 * slot including the request's static ones).  Requests carry no joints and no
 * triangle meshes; their convex meshes must equal meshes of mesh_pool (a scene
 * desc of which only the convex-mesh arrays are read).  Single-threaded: the
 * caller serialises calls on one server.
 * ---------------------------------------------------------------------- */
typedef struct psx_server psx_server;

typedef struct psx_server_opts {
    int32_t n_classes;
    const int32_t* class_bodies;      /* [n_classes] body capacity of a slot, ascending */
    const int32_t* class_slots;       /* [n_classes] slots of that class */
    const psx_scene_desc* mesh_pool;  /* convex meshes requests may use, or NULL */
    int32_t pairs_per_collider;       /* as psx_world_opts (0: 16, so that the broadphase keeps every
                                       * collider's pairs from its one tree walk; see psx_world_opts) */
    int32_t manifolds_per_collider;
    int32_t device;
    int32_t eager;                    /* 1: launch every tick's kernels one by one instead of replaying a CUDA graph */
    int32_t profile;                  /* 1: time each tick's stages with CUDA events (ticks then run eagerly);
                                       * psx_server_tick_stages reads them */
    int64_t hbm_budget;               /* device bytes the server may hold, 0: no cap.  Every slot keeps its
                                       * request's state resident, so the budget caps the slots: creation
                                       * fails with PSX_ERR_OUT_OF_MEMORY when they need more */
    const psx_launch_config* launch;  /* kernel launch shapes of the slots' world, or NULL: the world defaults
                                       * with epa_full_only = 1 (frame latency before throughput) */
    int32_t triggers;                 /* 1: the requests' trigger colliders raise events (psx_server_trigger_events);
                                       * 0: they only keep out of contact */
} psx_server_opts;

PSX_API psx_status psx_server_create(const psx_server_opts* opts, psx_server** out);
PSX_API psx_status psx_server_destroy(psx_server* s);
/* Place a request in the smallest free slot that holds it; it runs from the next
 * tick for `frames` frames of dt seconds.  PSX_ERR_CAPACITY: no free slot fits.
 * Admission packs the request into pinned host memory only; its arrays reach the
 * device when the next tick begins, so a request may be admitted while a tick runs. */
PSX_API psx_status psx_server_admit(psx_server* s, const psx_scene_desc* request, int32_t frames, float dt,
                                    int32_t* slot);
/* One frame of every running request, in one batched frame: tick_begin uploads the
 * requests admitted since the last tick and launches the frame without waiting;
 * tick_end waits for it and writes the slots whose request ran its last frame to
 * done[0..min(n,cap)).  Between the two the caller may admit, read finished slots and
 * release slots.  psx_server_tick = tick_begin + tick_end. */
PSX_API psx_status psx_server_tick_begin(psx_server* s);
PSX_API psx_status psx_server_tick_end(psx_server* s, int32_t* done, int32_t cap, int32_t* n_done);
PSX_API psx_status psx_server_tick(psx_server* s, int32_t* done, int32_t cap, int32_t* n_done);
/* Body state of a running or finished request (arrays as psx_world_read_bodies).  A
 * finished request is read beside a tick in flight; a running one after it. */
PSX_API psx_status psx_server_read(psx_server* s, int32_t slot, float* pos, float* quat, float* vel, float* ang_vel);
/* Free a slot (a running request is dropped). */
PSX_API psx_status psx_server_release(psx_server* s, int32_t slot);
/* out[6] = {running, finished, free slots, bodies running, body-frames so far, slots} */
PSX_API psx_status psx_server_stats(psx_server* s, int64_t* out);
/* The world that holds the slots (slot i is scene i), for the inspection entry points
 * (psx_world_counts, psx_world_get_pairs, psx_world_get_contacts).  Owned by the server. */
PSX_API psx_world* psx_server_world(psx_server* s);
/* With opts.profile set: the last finished tick's stage times in ms, out[6] = {staged
 * admissions (uploads and creation bounds), broadphase, narrowphase, contact and joint
 * rows, solver, end-of-frame bounds}. */
PSX_API psx_status psx_server_tick_stages(psx_server* s, float* out);
/* With opts.triggers set: the trigger events of the ticks ended so far, as
 * psx_world_trigger_events gives a world's (Scene::simulate's onTriggerEnter /
 * onTriggerExit, src/Physecs.cpp:537-552), for each request as if it ran alone: scene =
 * the request's slot, frame = frames of the request stepped before it, bodies and
 * colliders indexed within the request, entities the request's.  Events are decoded
 * when their tick ends, so a slot may be released and reused before they are read.
 * Up to cap events into out in tick order (within a tick: frame, enter before exit,
 * slot, bodies, colliders); the rest stay queued.  n_lost (optional): events dropped
 * because the device log overflowed within a tick. */
PSX_API psx_status psx_server_trigger_events(psx_server* s, psx_trigger_event* out, int32_t cap, int32_t* n_out,
                                             int64_t* n_lost);
/* Device memory the server holds (its slots' world and flags), in bytes. */
PSX_API psx_status psx_server_device_bytes(psx_server* s, int64_t* out);

/* ---- single-scene spelling of the same entry points (physecs::Scene) ---- */
typedef psx_world psx_scene;
PSX_API psx_status psx_scene_create(const psx_scene_desc* desc, psx_scene** out);
PSX_API psx_status psx_scene_destroy(psx_scene* s);
PSX_API psx_status psx_scene_simulate(psx_scene* s, float dt);

#ifdef __cplusplus
}
#endif

#endif /* PSX_H */
