// types.cuh — device data layout of a simulated world (one or many scenes).
//
// Bodies, colliders and dynamic bodies live in flat structure-of-arrays buffers
// with per-scene segment offsets, so every kernel serves a single scene and a
// batch of thousands of scenes alike.  float4 elements keep every access 16-byte
// aligned and coalesced.
#pragma once
#include <cstdint>
#include "dmath.cuh"

namespace psx {

enum : int { G_SPHERE = 0, G_CAPSULE = 1, G_BOX = 2, G_CONVEX = 3, G_TRIMESH = 4 };
enum : int { COL_ENABLE = 1, COL_TRIGGER = 2, COL_DYNAMIC = 4 };
enum : int { BODY_DYN = 1, BODY_KIN = 2 };

// device error word bits
enum : int {
    ERR_PAIR_CAPACITY = 1 << 0,
    ERR_MANIFOLD_CAPACITY = 1 << 1,
    ERR_POLY_CAPACITY = 1 << 2,
    ERR_TRI_CAPACITY = 1 << 3,
    ERR_EPA_CAPACITY = 1 << 4,
    ERR_BARRIER_TIMEOUT = 1 << 5,
    ERR_COLOR_CAPACITY = 1 << 6,
    ERR_STACK_CAPACITY = 1 << 7,
    ERR_CACHE_CAPACITY = 1 << 8,
};

constexpr int kMaxPoly = 64;       // polygon vertices after clipping (reference caps at 128, src/Clipping.cpp:6)
constexpr int kTriManifolds = 16;  // manifolds one body may produce against one triangle mesh
constexpr int kTriCandidates = 64; // candidate triangles per body-mesh pair
constexpr int kMaxRowsPerJoint = 8;
constexpr int kMaxColors = 128;    // contact colours per scene
constexpr int kMeshBoundsChunk = 8192;   // triangle-mesh vertices per block in the collider bounds

struct ConvexMeshDev {   // one ConvexMesh
    int vert_start, vert_count_padded, vert_count;
    int face_start, face_count;
};
struct TriMeshDev {
    int vert_start, vert_count, tri_start, tri_count, node_start;
};
struct TriDev {          // Triangle (include/Physecs/TriangleMesh.h:9-14)
    int4 idx;            // three vertex indices (mesh-local), w unused
    float4 bmin, bmax;
    float4 normal, centroid;
};
struct TriNodeDev {      // TriangleMeshBVHNode
    float4 bmin;         // w = triCount (as int bits)
    float4 bmax;         // w = index (as int bits)
};

struct Manifold {
    float4 n;            // normal; w unused
    float4 p0[4];
    float4 p1[4];
    int np, tri, pair, pad;
};

struct ContactPt {
    float4 r0;           // local r0, w = targetVelocity
    float4 r1;           // local r1, w = c
    float4 r0xn;         // w = lambdaN
    float4 r1xn;         // w = lambdaT
    float4 t;            // w = invEffMassN
    float4 r0xt;         // w = invEffMassT
    float4 r1xt;
    float4 r0xnt, r1xnt, r0xtt, r1xtt;
};

struct Contact {         // ContactConstraints (src/ContactConstraints.h:31-48)
    int b0, b1;          // global dynamic index or -1
    int body0, body1;    // global body index
    float4 n;            // w = friction
    float frequency, damping;
    int np, soft;
    int color, scene, pair, tri;
    ContactPt p[4];
};

struct Row {             // Constraint1D / Constraint1DW lane
    float4 linear;       // w = targetVelocity
    float4 angular0;     // w = c
    float4 angular1;     // w = min
    float4 linear0t;     // w = max
    float4 linear1t;     // w = frequency
    float4 angular0t;    // w = dampingRatio
    float4 angular1t;    // w = invEffMass
    float totalLambda;
    int flags, b0, b1;
};

struct JointDev {
    int type, body0, body1, color;   // colour from the reference's greedy colouring
    int b0, b1, simd, nrows;
    float4 a0p, a0q, a1p, a1q;
    float4 r0, r1;                   // anchor relative to COM when dynamic
    float params[8];
    int makeUpper, makeLower, gearInit, pad;
    float persistent0, persistent1, virtual0, virtual1;
    int rowflags[kMaxRowsPerJoint];
};

// Per-substep solver record of one contact (ContactConstraints, src/ContactConstraints.h:31-48),
// written in colour order:
//   n = {normal, friction}   m = {invMass0, invMass1, frequency, damping}
//   i = {dynamic body 0 or -1, dynamic body 1 or -1, numPoints | soft << 8, first point}
struct SHdr {
    float4 n, m;
    int4 i;
};
// One ContactPointConstraints as the iterations read it:
//   a = {r0 x n, lambdaN}          b = {r1 x n, targetVelocity}
//   c = {I0 (r0 x n), bias term}   d = {I1 (r1 x n), effective-mass term}
//   e = {t, lambdaT}               f = {I0 (r0 x t), friction impulse}
//   g = {I1 (r1 x t), live rows: 1 normal (invEffMassN != 0), 2 friction (invEffMassT != 0)}
// Between the row update and preSolve, f/g.xyz hold r0 x t / r1 x t and c.w the separation.
// Friction reads the component velocities, which stay fixed through a substep's
// iterations (ContactConstraints.cpp:93-101), so its unclamped impulse is formed once
// per substep in preSolve with the same operations.
struct SPt {
    float4 a, b, c, d, e, f, g;
};
constexpr int kHdrF4 = 3, kPtF4 = 7;

// one body's registry changes of a batch (the layout of psx_body_delta; body is the
// world body index once the host has coalesced the batch)
enum : int { DELTA_POSE = 1, DELTA_VELOCITY = 2, DELTA_KINEMATIC = 4 };
struct DeltaRec {
    int scene, body, mask, kinematic;
    float pos[3], quat[4], vel[3], ang[3];
};

struct CacheEntry {      // restitution cache (include/Physecs/Physecs.h:127-135)
    unsigned long long key;
    int np, pad;
    float4 r0tv[4];      // local r0 (xyz), targetVelocity (w)
};

struct World {
    int n_scenes, n_bodies, n_colliders, n_dyn, n_joints;
    int key_cbits;       // bits of a collider index in a restitution-cache key (the rest: triangle + 1)
    int* scene_body;     // [S+1]
    int* scene_col;      // [S+1]
    int* scene_dyn;      // [S+1]
    int* scene_joint;    // [S+1]
    int* scene_jsched;   // [S+1] into joint schedule
    float4* knobs;       // [S]: substeps, iterations, gravity, 0
    // bodies
    float4* pos;         // xyz
    float4* quat;
    int4* info;          // entity, flags, dyn index, scene
    int* body_col;       // [n_bodies + 1] each body's first collider
    // dynamic bodies
    int* dyn_body;
    float4* vel;         // component velocity
    float4* ang;
    float4* com;         // xyz com, w invMass
    float4* invI;        // 3 per dynamic body, local inverse inertia columns
    float4* vt_v;        // solver velocities
    float4* vt_w;
    float4* pv_v;        // pseudo velocities, w = constraint count
    float4* pv_w;
    float4* mt;          // 3 per dynamic body, world inverse inertia columns
    // colliders
    int4* col_info;      // body, type, mesh, flags
    float4* col_pos;
    float4* col_quat;
    float4* col_params;
    float4* col_mat;     // friction, restitution, damping, data
    float4* aabb_min;
    float4* aabb_max;
    // assets
    ConvexMeshDev* convex;
    float4* convex_verts;
    int* face_idx_start;   // per face, into face_idx
    int* face_idx;
    float4* face_normal;
    float4* face_centroid;
    TriMeshDev* trimesh;
    float4* tri_verts;
    TriDev* tris;
    TriNodeDev* tri_nodes;
    int4* tri_src;         // per triangle, index order: mesh-local vertex indices, w = mesh's first vertex
    int* trimesh_cols;     // colliders whose shape is a triangle mesh
    int n_trimesh_cols;
    int2* trimesh_chunks;  // (trimesh_cols slot, chunk of kMeshBoundsChunk vertices) for their bounds
    int n_trimesh_chunks;
    unsigned long long* trimesh_keys;   // [6][n_trimesh_cols] bounds reduction keys
    // joints
    JointDev* joints;
    Row* rows;             // kMaxRowsPerJoint per joint
    int* jsched;           // joint indices in solve order (colour, sub-colour)
    int* jsched_step;      // step id per schedule entry
    int* scene_jsteps;     // [S+1] step boundaries into jstep_start
    int* jstep_start;      // start of each step in jsched
    int* jstep_simd;       // 1 for colours 0..7 (4-lane arithmetic), 0 for overflow
    // jointed body pairs, sorted (lo, hi): such pairs never collide (src/Physecs.cpp:209, 694)
    int* col_class;               // with a user contact filter: each collider's (isTrigger, data) class
    unsigned char* filter_table;  // [n_classes^2] 1: TRIGGER for (class of collider 0, class of collider 1)
    int n_classes;
    int2* nc_pairs;
    int n_nc;
    // serving: per-scene flags, null for a plain world (every scene runs, cache on)
    int* scene_active;     // [S] 0: the scene is skipped by the traversal and the solver
    int* scene_fresh;      // [S] 1: first frame of a newly placed scene, no cached contacts
    // errors
    int* err;
};

}  // namespace psx
