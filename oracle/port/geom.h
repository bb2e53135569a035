/*
 * geom.h — shapes, manifolds and narrowphase entry points of the CPU oracle.
 * ORACLE (test infrastructure only; see omath.h).
 */
#pragma once
#include <vector>
#include <cstdint>
#include "omath.h"

namespace orc {

enum GeomType { SPHERE = 0, CAPSULE = 1, BOX = 2, CONVEX_MESH = 3, TRIANGLE_MESH = 4 };

struct ConvexFace { std::vector<int> indices; V3 normal, centroid; };

// include/Physecs/ConvexMesh.h:13-34; the vertex buffer is padded to a multiple
// of four with copies of the last vertex (src/ConvexMesh.cpp:3-11)
struct ConvexMesh {
    std::vector<V3> buffer;  // padded
    int count = 0;           // unpadded vertex count
    std::vector<ConvexFace> faces;
};

struct Triangle { uint32_t idx[3]; Bounds bounds; V3 normal, centroid; };
struct TriNode { Bounds bounds; int triCount = 0; int index = 0; };

// include/Physecs/TriangleMesh.h:24-41, binned-SAH BVH of src/TriangleMesh.cpp
struct TriangleMesh {
    std::vector<V3> vertices;
    std::vector<Triangle> triangles;
    std::vector<TriNode> bvh;
    void build(const std::vector<V3>& verts, const std::vector<uint32_t>& indices);
    void overlap(const Bounds& b, std::vector<int>& out) const;
};

struct Geometry {
    int type;
    float p[3];               // sphere {r}; capsule {halfHeight, r}; box {he}; convex {scale}
    const ConvexMesh* convex = nullptr;
    const TriangleMesh* tri = nullptr;
};

struct ContactPoint { V3 p0, p1; };
struct Manifold {
    int numPoints = 0;
    ContactPoint points[4];
    V3 normal{0, 0, 0};
    int triangleIndex = -1;
};

// physecs::collision, src/Collision.cpp:895-1016
bool collision(V3 pos0, Q4 or0, const Geometry& g0, V3 pos1, Q4 or1, const Geometry& g1, std::vector<Manifold>& out);
// physecs::getBounds, src/BoundsUtil.cpp:23-33
Bounds getBounds(V3 pos, Q4 ori, const Geometry& g);

}  // namespace orc
