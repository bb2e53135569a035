// meshbvh.cuh — the device build of TriangleMesh's BVH (src/TriangleMesh.cpp:7-164).
#pragma once
#include <cuda_runtime.h>
#include <vector>
#include "types.cuh"

namespace psx {

// One mesh of a build: its triangles at [tri_start, tri_start + tri_count) of the
// build-wide triangle arrays (contiguous over all meshes, from 0), its nodes from
// node_start (room for 2 * tri_count - 1, at least 1).
struct BuildMesh { int tri_start, tri_count, vert_start, node_start; };

// Builds every mesh's BVH as the reference's TriangleMesh constructor does: idx holds
// each triangle's three mesh-local vertex indices in the mesh's index order, w = the
// mesh's first vertex in verts.  Writes the triangles in the tree's order to tris_out
// (at each mesh's tri_start) and the nodes to nodes_out; node_counts[m] receives the
// nodes of mesh m.  *err_out is nonzero if a capacity was exceeded (it cannot be with
// the documented sizes).  Waits for the stream.
cudaError_t build_mesh_bvhs(const float4* verts, const int4* idx, const std::vector<BuildMesh>& meshes, TriDev* tris_out,
                            TriNodeDev* nodes_out, std::vector<int>& node_counts, int* err_out, cudaStream_t st);

}  // namespace psx
