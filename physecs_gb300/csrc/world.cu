// world.cu — host runtime and C ABI of the GB300 simulation hot path.
//
// Owns every device buffer of a world (one or many scenes), packs scene
// descriptors into the device layout of types.cuh, reproduces the host-side
// work the reference does when a scene is populated (triangle-mesh BVH build,
// src/TriangleMesh.cpp:7-164; joint colouring, src/Physecs.cpp:690-710), and
// queues one frame as a fixed sequence of kernels on the world's stream.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>
#include "meshbvh.cuh"
#include "runtime.cuh"

using namespace psx;

namespace psx {
namespace rt {

thread_local std::string g_err;

psx_status fail(psx_status s, const std::string& msg) {
    g_err = msg;
    return s;
}

}  // namespace rt
}  // namespace psx

using namespace psx::rt;

namespace {

template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
};

}  // namespace



psx_status psx::rt::validate(const psx_scene_desc& d) {
    if (d.n_bodies <= 0) return fail(PSX_ERR_INVALID_ARG, "scene without bodies");
    if (!d.entity || !d.flags || !d.pos || !d.quat || !d.collider_start) return fail(PSX_ERR_INVALID_ARG, "missing body arrays");
    if (d.collider_start[0] != 0 || d.collider_start[d.n_bodies] != d.n_colliders) return fail(PSX_ERR_INVALID_ARG, "collider_start");
    if (d.n_colliders <= 0) return fail(PSX_ERR_INVALID_ARG, "scene without colliders");
    for (int c = 0; c < d.n_colliders; ++c) {
        int t = d.col_type[c];
        if (t < 0 || t > 4) return fail(PSX_ERR_INVALID_ARG, "collider type");
        if (t == PSX_CONVEX_MESH && (d.col_mesh[c] < 0 || d.col_mesh[c] >= d.n_convex)) return fail(PSX_ERR_INVALID_ARG, "convex mesh index");
        if (t == PSX_TRIANGLE_MESH && (d.col_mesh[c] < 0 || d.col_mesh[c] >= d.n_trimesh)) return fail(PSX_ERR_INVALID_ARG, "triangle mesh index");
    }
    for (int j = 0; j < d.n_joints; ++j) {
        if (d.joint_type[j] < 0 || d.joint_type[j] > 6) return fail(PSX_ERR_INVALID_ARG, "joint type");
        if (d.joint_body0[j] < 0 || d.joint_body0[j] >= d.n_bodies || d.joint_body1[j] < 0 || d.joint_body1[j] >= d.n_bodies)
            return fail(PSX_ERR_INVALID_ARG, "joint body index");
    }
    if (d.num_substeps <= 0 || d.num_iterations < 0) return fail(PSX_ERR_INVALID_ARG, "knobs");
    for (int m = 0; m < d.n_trimesh; ++m) {   // the device BVH build reads vertices by these indices
        const int nv = d.tri_vert_start[m + 1] - d.tri_vert_start[m];
        for (int k = d.tri_index_start[m]; k < d.tri_index_start[m + 1]; ++k)
            if (d.tri_indices[k] >= (uint32_t)nv) return fail(PSX_ERR_INVALID_ARG, "triangle-mesh vertex index");
        for (int v = 3 * d.tri_vert_start[m]; v < 3 * d.tri_vert_start[m + 1]; ++v)
            if (!std::isfinite(d.tri_verts[v])) return fail(PSX_ERR_INVALID_ARG, "triangle-mesh vertex not finite");
    }
    return PSX_OK;
}

psx_status psx::rt::build_world(psx_world* W, const psx_scene_desc* scenes, int S, const psx_world_opts& o) {
    W->n_scenes = S;
    std::vector<int> scene_body{0}, scene_col{0}, scene_dyn{0}, scene_joint{0};
    std::vector<float4> pos, quat, vel, ang, com, invI, col_pos, col_quat, col_params, col_mat;
    std::vector<int4> info, col_info;
    std::vector<int> dyn_body;
    std::vector<ConvexMeshDev> convex;
    std::vector<float4> convex_verts, face_normal, face_centroid;
    std::vector<int> face_idx_start{0}, face_idx;
    std::vector<TriMeshDev> trimesh;
    std::vector<float4> tri_verts;
    std::vector<int4> tri_src;    // per triangle: mesh-local vertex indices, w = the mesh's first vertex
    int n_tri_nodes = 0;
    std::vector<int2> body_joint;       // (body, joint) for every joint end
    std::vector<int> overflow_bodies;   // bodies with a joint in the overflow colour
    std::vector<JointDev> joints;
    std::vector<int2> nc;
    std::vector<int> jsched, jstep_start{0}, scene_jsteps{0};
    for (int s = 0; s < S; ++s) {
        const psx_scene_desc& d = scenes[s];
        PSX_TRY(validate(d));
        int bbase = (int)pos.size(), cbase = (int)col_info.size(), dbase = (int)dyn_body.size();
        int mbase = (int)convex.size(), tbase = (int)trimesh.size(), jbase = (int)joints.size();
        W->h_scene_convex.push_back(mbase);
        W->h_scene_trimesh.push_back(tbase);
        // convex meshes: vertex buffer padded to a multiple of four with the last vertex (src/ConvexMesh.cpp:3-11)
        for (int m = 0; m < d.n_convex; ++m) {
            ConvexMeshDev cm;
            cm.vert_start = (int)convex_verts.size();
            int v0 = d.convex_vert_start[m], v1 = d.convex_vert_start[m + 1];
            cm.vert_count = v1 - v0;
            cm.vert_count_padded = (cm.vert_count + 3) / 4 * 4;
            for (int v = v0; v < v1; ++v) convex_verts.push_back(f4(d.convex_verts[3 * v], d.convex_verts[3 * v + 1], d.convex_verts[3 * v + 2]));
            for (int v = cm.vert_count; v < cm.vert_count_padded; ++v) convex_verts.push_back(convex_verts.back());
            cm.face_start = (int)face_normal.size();
            for (int fi = d.convex_face_start[m]; fi < d.convex_face_start[m + 1]; ++fi) {
                for (int k = d.face_index_start[fi]; k < d.face_index_start[fi + 1]; ++k) face_idx.push_back(d.face_indices[k]);
                face_idx_start.push_back((int)face_idx.size());
                face_normal.push_back(f4(d.face_normal[3 * fi], d.face_normal[3 * fi + 1], d.face_normal[3 * fi + 2]));
                face_centroid.push_back(f4(d.face_centroid[3 * fi], d.face_centroid[3 * fi + 1], d.face_centroid[3 * fi + 2]));
            }
            cm.face_count = (int)face_normal.size() - cm.face_start;
            convex.push_back(cm);
        }
        for (int m = 0; m < d.n_trimesh; ++m) {
            int v0 = d.tri_vert_start[m], v1 = d.tri_vert_start[m + 1];
            int i0 = d.tri_index_start[m], i1 = d.tri_index_start[m + 1];
            // the mesh's triangles in index order; its BVH is built on the device below
            TriMeshDev tm;
            tm.vert_start = (int)tri_verts.size();
            tm.vert_count = v1 - v0;
            tm.tri_start = (int)tri_src.size();
            tm.tri_count = (i1 - i0) / 3;
            tm.node_start = n_tri_nodes;
            n_tri_nodes += std::max(1, 2 * tm.tri_count - 1);
            for (int v = v0; v < v1; ++v) tri_verts.push_back(f4(d.tri_verts[3 * v], d.tri_verts[3 * v + 1], d.tri_verts[3 * v + 2]));
            for (int k = 0; k < tm.tri_count; ++k) {
                const uint32_t* ix = d.tri_indices + i0 + 3 * k;
                tri_src.push_back(make_int4((int)ix[0], (int)ix[1], (int)ix[2], tm.vert_start));
            }
            trimesh.push_back(tm);
        }
        for (int b = 0; b < d.n_bodies; ++b) {
            uint32_t fl = d.flags[b];
            bool dyn = fl & PSX_BODY_DYNAMIC;
            bool sim = dyn && !(fl & PSX_BODY_KINEMATIC);
            int di = -1;
            if (sim) ++W->n_simulated;
            pos.push_back(f4(d.pos[3 * b], d.pos[3 * b + 1], d.pos[3 * b + 2]));
            quat.push_back(f4(d.quat[4 * b], d.quat[4 * b + 1], d.quat[4 * b + 2], d.quat[4 * b + 3]));
            if (dyn) {
                di = (int)dyn_body.size();
                dyn_body.push_back(bbase + b);
                vel.push_back(f4(d.vel[3 * b], d.vel[3 * b + 1], d.vel[3 * b + 2]));
                ang.push_back(f4(d.ang_vel[3 * b], d.ang_vel[3 * b + 1], d.ang_vel[3 * b + 2]));
                com.push_back(f4(d.com[3 * b], d.com[3 * b + 1], d.com[3 * b + 2], d.inv_mass[b]));
                for (int k = 0; k < 3; ++k) invI.push_back(f4(d.inv_inertia[9 * b + 3 * k], d.inv_inertia[9 * b + 3 * k + 1], d.inv_inertia[9 * b + 3 * k + 2]));
            }
            info.push_back(make_int4((int)d.entity[b], (int)fl, di, s));
            W->h_body_col.push_back((int)col_info.size());
            W->h_body_flags.push_back((int)fl);
            W->h_entity.push_back(d.entity[b]);
            W->h_body_dyn.push_back(di);
            for (int c = d.collider_start[b]; c < d.collider_start[b + 1]; ++c) {
                int t = d.col_type[c];
                int mesh = t == PSX_CONVEX_MESH ? mbase + d.col_mesh[c] : (t == PSX_TRIANGLE_MESH ? tbase + d.col_mesh[c] : -1);
                int flags = 0;
                if (!d.col_enable_sim || d.col_enable_sim[c]) flags |= COL_ENABLE;
                if (d.col_is_trigger && d.col_is_trigger[c]) flags |= COL_TRIGGER;
                if (sim) flags |= COL_DYNAMIC;
                col_info.push_back(make_int4(bbase + b, t, mesh, flags));
                W->h_col_trimesh.push_back(t == PSX_TRIANGLE_MESH ? mesh : -1);
                W->h_col_data.push_back(d.col_data ? d.col_data[c] : 0);
                W->h_col_trig.push_back(d.col_is_trigger && d.col_is_trigger[c] ? 1 : 0);
                col_pos.push_back(f4(d.col_pos[3 * c], d.col_pos[3 * c + 1], d.col_pos[3 * c + 2]));
                col_quat.push_back(f4(d.col_quat[4 * c], d.col_quat[4 * c + 1], d.col_quat[4 * c + 2], d.col_quat[4 * c + 3]));
                col_params.push_back(f4(d.col_params[4 * c], d.col_params[4 * c + 1], d.col_params[4 * c + 2], d.col_params[4 * c + 3]));
                col_mat.push_back(f4(d.col_material[3 * c], d.col_material[3 * c + 1], d.col_material[3 * c + 2],
                                     bits_as_float(d.col_data ? d.col_data[c] : 0)));
                W->h_col_local.push_back(c - d.collider_start[b]);
                W->h_col_body.push_back(bbase + b);
            }
        }
        // joints: the reference's greedy per-entity colour bitsets (src/Physecs.cpp:690-710);
        // colours 0-7 are entity-disjoint, colour 8 collects the overflow
        std::vector<unsigned char> bits(d.n_bodies, 0);
        std::vector<std::vector<int>> colors(9);
        const int32_t* forced = s < (int)W->forced_colors.size() ? W->forced_colors[s] : nullptr;
        for (int j = 0; j < d.n_joints; ++j) {
            int b0 = d.joint_body0[j], b1 = d.joint_body1[j];
            unsigned u = bits[b0] | bits[b1];
            int c = __builtin_ctz(~u);
            if (forced) {   // the colour the caller's scene gave the joint when it was created
                c = forced[j];
                if (c < 0 || c > 8 || (c < 8 && (u >> c) & 1u))
                    return fail(PSX_ERR_INVALID_ARG, "joint colour " + std::to_string(c) + " of joint " + std::to_string(j) +
                                                         " is out of range or taken at one of its bodies");
            }
            bits[b0] |= (unsigned char)(1u << c);
            bits[b1] |= (unsigned char)(1u << c);
            colors[c].push_back(j);
            body_joint.push_back(make_int2(bbase + b0, jbase + j));
            body_joint.push_back(make_int2(bbase + b1, jbase + j));
            if (c == 8) overflow_bodies.push_back(bbase + b0), overflow_bodies.push_back(bbase + b1);
            int lo = std::min(bbase + b0, bbase + b1), hi = std::max(bbase + b0, bbase + b1);
            nc.push_back(make_int2(lo, hi));
            JointDev J{};
            J.type = d.joint_type[j];
            J.body0 = bbase + b0; J.body1 = bbase + b1;
            J.color = c; J.simd = c < 8 ? 1 : 0;
            bool s0 = (d.flags[b0] & PSX_BODY_DYNAMIC) && !(d.flags[b0] & PSX_BODY_KINEMATIC);
            bool s1 = (d.flags[b1] & PSX_BODY_DYNAMIC) && !(d.flags[b1] & PSX_BODY_KINEMATIC);
            J.b0 = s0 ? W->h_body_dyn[bbase + b0] : -1;
            J.b1 = s1 ? W->h_body_dyn[bbase + b1] : -1;
            const float* fr = d.joint_frames + 14 * j;
            J.a0p = f4(fr[0], fr[1], fr[2]); J.a0q = f4(fr[3], fr[4], fr[5], fr[6]);
            J.a1p = f4(fr[7], fr[8], fr[9]); J.a1q = f4(fr[10], fr[11], fr[12], fr[13]);
            V3 a0 = {fr[0], fr[1], fr[2]}, a1 = {fr[7], fr[8], fr[9]};
            V3 r0 = s0 ? a0 - V3{d.com[3 * b0], d.com[3 * b0 + 1], d.com[3 * b0 + 2]} : a0;
            V3 r1 = s1 ? a1 - V3{d.com[3 * b1], d.com[3 * b1 + 1], d.com[3 * b1 + 2]} : a1;
            J.r0 = st4(r0); J.r1 = st4(r1);
            for (int k = 0; k < 8; ++k) J.params[k] = d.joint_params ? d.joint_params[PSX_JOINT_PARAMS * j + k] : 0.f;
            joints.push_back(J);
        }
        // solve schedule: one step per reference colour 0-7; the overflow colour is split into
        // steps by creation order so that joints sharing a dynamic body stay ordered
        for (int c = 0; c < 8; ++c) {
            if (colors[c].empty()) continue;
            for (int j : colors[c]) jsched.push_back(jbase + j);
            jstep_start.push_back((int)jsched.size());
        }
        if (!colors[8].empty()) {
            std::map<int, int> level_of_body;
            std::vector<std::vector<int>> levels;
            for (int j : colors[8]) {
                int lv = 0;
                for (int b : {d.joint_body0[j], d.joint_body1[j]}) {
                    bool sim = (d.flags[b] & PSX_BODY_DYNAMIC) && !(d.flags[b] & PSX_BODY_KINEMATIC);
                    if (!sim) continue;
                    auto it = level_of_body.find(b);
                    if (it != level_of_body.end()) lv = std::max(lv, it->second + 1);
                }
                for (int b : {d.joint_body0[j], d.joint_body1[j]}) level_of_body[b] = lv;
                if ((int)levels.size() <= lv) levels.resize(lv + 1);
                levels[lv].push_back(j);
            }
            for (auto& L : levels) {
                for (int j : L) jsched.push_back(jbase + j);
                jstep_start.push_back((int)jsched.size());
            }
        }
        scene_jsteps.push_back((int)jstep_start.size() - 1);
        scene_body.push_back((int)pos.size());
        scene_col.push_back((int)col_info.size());
        scene_dyn.push_back((int)dyn_body.size());
        scene_joint.push_back((int)joints.size());
        W->h_knobs.push_back(f4((float)d.num_substeps, (float)d.num_iterations, d.gravity, 1.f / 60.f));
        int nd = scene_dyn[s + 1] - scene_dyn[s];
        if (nd > o.block_scene_max_dyn) W->grid_scenes_h.push_back(s);
        else if (nd > 1024) W->large_scenes_h.push_back(s);
        else W->block_scenes_h.push_back(s);
    }
    std::sort(nc.begin(), nc.end(), [](int2 a, int2 b) { return a.x < b.x || (a.x == b.x && a.y < b.y); });
    nc.erase(std::unique(nc.begin(), nc.end(), [](int2 a, int2 b) { return a.x == b.x && a.y == b.y; }), nc.end());
    W->h_scene_body = scene_body;
    W->h_body_col.push_back((int)col_info.size());
    {
        const int nb = (int)pos.size();
        std::sort(body_joint.begin(), body_joint.end(), [](int2 a, int2 b) { return a.x < b.x || (a.x == b.x && a.y < b.y); });
        W->h_bj_start.assign(nb + 1, 0);
        for (const int2& e : body_joint) ++W->h_bj_start[e.x + 1];
        for (int b = 0; b < nb; ++b) W->h_bj_start[b + 1] += W->h_bj_start[b];
        W->h_bj.clear();
        for (const int2& e : body_joint) W->h_bj.push_back(e.y);
        W->h_body_overflow.assign(nb, 0);
        for (int b : overflow_bodies) W->h_body_overflow[b] = 1;
        W->h_delta_slot.assign(nb, -1);
    }
    W->h_scene_convex.push_back((int)convex.size());
    W->h_scene_trimesh.push_back((int)trimesh.size());
    W->h_scene_col = scene_col;
    W->h_scene_dyn = scene_dyn;
    World& w = W->w;
    w.n_scenes = S;
    w.n_bodies = (int)pos.size();
    w.n_colliders = (int)col_info.size();
    w.n_dyn = (int)dyn_body.size();
    w.n_joints = (int)joints.size();
    if (w.n_colliders >= (1 << 23)) return fail(PSX_ERR_CAPACITY, "more than 2^23 colliders in one world");
    // restitution-cache keys: as few bits per collider as the world needs, the rest for triangles
    w.key_cbits = 1;
    while ((1ll << w.key_cbits) - 1 < (long long)w.n_colliders) ++w.key_cbits;   // indices below 2^cbits - 1
    const long long tri_max = (1ll << (64 - 2 * w.key_cbits)) - 2;
    for (const TriMeshDev& tm : trimesh)
        if (tm.tri_count > tri_max)
            return fail(PSX_ERR_CAPACITY, "triangle mesh above " + std::to_string(tri_max) + " triangles in a world of " +
                                              std::to_string(w.n_colliders) + " colliders");
    PSX_TRY(W->upload(w.scene_body, scene_body));
    PSX_TRY(W->upload(w.body_col, W->h_body_col));
    PSX_TRY(W->upload(w.scene_col, scene_col));
    PSX_TRY(W->upload(w.scene_dyn, scene_dyn));
    PSX_TRY(W->upload(w.scene_joint, scene_joint));
    W->h_scene_joint = scene_joint;
    PSX_TRY(W->upload(w.knobs, W->h_knobs));
    PSX_TRY(W->upload(w.pos, pos));
    PSX_TRY(W->upload(w.quat, quat));
    PSX_TRY(W->upload(w.info, info));
    PSX_TRY(W->upload(w.dyn_body, dyn_body));
    PSX_TRY(W->upload(w.vel, vel));
    PSX_TRY(W->upload(w.ang, ang));
    PSX_TRY(W->upload(w.com, com));
    PSX_TRY(W->upload(w.invI, invI));
    PSX_TRY(W->alloc(w.vt_v, w.n_dyn));
    PSX_TRY(W->alloc(w.vt_w, w.n_dyn));
    PSX_TRY(W->alloc(w.pv_v, w.n_dyn));
    PSX_TRY(W->alloc(w.pv_w, w.n_dyn));
    PSX_TRY(W->alloc(w.mt, 3 * (size_t)w.n_dyn));
    PSX_TRY(W->upload(w.col_info, col_info));
    PSX_TRY(W->upload(w.col_pos, col_pos));
    PSX_TRY(W->upload(w.col_quat, col_quat));
    PSX_TRY(W->upload(w.col_params, col_params));
    PSX_TRY(W->upload(w.col_mat, col_mat));
    PSX_TRY(W->alloc(w.aabb_min, w.n_colliders));
    PSX_TRY(W->alloc(w.aabb_max, w.n_colliders));
    PSX_TRY(W->upload(w.convex, convex));
    PSX_TRY(W->upload(w.convex_verts, convex_verts));
    PSX_TRY(W->upload(w.face_idx_start, face_idx_start));
    PSX_TRY(W->upload(w.face_idx, face_idx));
    PSX_TRY(W->upload(w.face_normal, face_normal));
    PSX_TRY(W->upload(w.face_centroid, face_centroid));
    PSX_TRY(W->upload(w.trimesh, trimesh));
    PSX_TRY(W->upload(w.tri_verts, tri_verts));
    // triangle-mesh BVHs: every mesh of every scene in one device build
    PSX_TRY(W->upload(w.tri_src, tri_src));
    PSX_TRY(W->alloc(w.tris, tri_src.size()));
    PSX_TRY(W->alloc(w.tri_nodes, n_tri_nodes));
    if (!trimesh.empty()) {
        std::vector<BuildMesh> bm;
        for (const TriMeshDev& tm : trimesh) bm.push_back({tm.tri_start, tm.tri_count, tm.vert_start, tm.node_start});
        std::vector<int> counts;
        int berr = 0;
        PSX_CUDA(cudaDeviceSynchronize());   // the uploads above ran on the legacy stream
        PSX_CUDA(build_mesh_bvhs(w.tri_verts, w.tri_src, bm, w.tris, w.tri_nodes, counts, &berr, W->stream));
        if (berr) return fail(PSX_ERR_CAPACITY, "triangle-mesh BVH build");
    }
    W->h_trimesh = trimesh;
    {
        std::vector<int> tcols;
        for (int c = 0; c < (int)W->h_col_trimesh.size(); ++c) if (W->h_col_trimesh[c] >= 0) tcols.push_back(c);
        PSX_TRY(W->upload(w.trimesh_cols, tcols));
        w.n_trimesh_cols = (int)tcols.size();
        std::vector<int2> tch;
        for (int t = 0; t < (int)tcols.size(); ++t) {
            const int nv = trimesh[W->h_col_trimesh[tcols[t]]].vert_count;
            for (int k = 0; k == 0 || k * kMeshBoundsChunk < nv; ++k) tch.push_back(make_int2(t, k));
        }
        PSX_TRY(W->upload(w.trimesh_chunks, tch));
        w.n_trimesh_chunks = (int)tch.size();
        PSX_TRY(W->alloc(w.trimesh_keys, 6 * tcols.size()));
    }
    PSX_TRY(W->upload(w.joints, joints));
    PSX_TRY(W->alloc(w.rows, (size_t)kMaxRowsPerJoint * std::max(1, w.n_joints)));
    PSX_TRY(W->upload(w.jsched, jsched));
    PSX_TRY(W->upload(w.jstep_start, jstep_start));
    PSX_TRY(W->upload(w.scene_jsteps, scene_jsteps));
    w.scene_jsched = nullptr;
    w.jsched_step = nullptr;
    w.jstep_simd = nullptr;
    PSX_TRY(W->upload_reuse(w.nc_pairs, W->nc_cap, nc));
    w.n_nc = (int)nc.size();
    W->h_nc = nc;
    PSX_TRY(W->alloc(w.err, 1));
    PSX_CUDA(cudaMemset(w.err, 0, sizeof(int)));

    // ---- frame buffers
    FrameBuf& f = W->f;
    int n = w.n_colliders;
    int ppc = o.pairs_per_collider > 0 ? o.pairs_per_collider : 8;
    int mpc = o.manifolds_per_collider > 0 ? o.manifolds_per_collider : 4;
    f.pair_cap = std::max(1024, ppc * n);
    f.man_cap = std::max(1024, mpc * n);
    int tri_pairs = 0;
    for (int s = 0; s < S; ++s) if (scenes[s].n_trimesh) tri_pairs += scenes[s].n_bodies;
    f.tri_cap = std::max(64, 2 * tri_pairs);
    f.cache_cap = 1 << ilog2ceil(2 * f.man_cap);
    PSX_TRY(W->alloc(f.scene_lo, S));
    PSX_TRY(W->alloc(f.scene_hi, S));
    PSX_TRY(W->alloc(f.keys, n));
    PSX_TRY(W->alloc(f.mkey, n));
    PSX_TRY(W->alloc(f.order, n));
    PSX_TRY(W->alloc(f.keys_tmp, n));
    PSX_TRY(W->alloc(f.order_tmp, n));
    PSX_TRY(W->alloc(f.radix_hist, radix_hist_ints(n)));
    BVHNodes& v = f.bvh;
    PSX_TRY(W->alloc(v.left, n)); PSX_TRY(W->alloc(v.right, n)); PSX_TRY(W->alloc(v.parent, n));
    PSX_TRY(W->alloc(v.leaf_parent, n)); PSX_TRY(W->alloc(v.first, n)); PSX_TRY(W->alloc(v.last, n));
    PSX_TRY(W->alloc(v.bmin, n)); PSX_TRY(W->alloc(v.bmax, n)); PSX_TRY(W->alloc(v.visits, n));
    PSX_TRY(W->alloc(f.leaf_cnt, n));
    PSX_TRY(W->alloc(f.leaf_off, n));
    size_t scr = std::max(scan_scratch_ints(std::max(f.pair_cap, n)), scan_scratch_ints(S + 1));
    PSX_TRY(W->alloc(f.scan_scratch, scr));
    PSX_TRY(W->alloc(f.pairs, f.pair_cap));
    PSX_TRY(W->alloc(f.n_pairs, 1));
    PSX_TRY(W->alloc(f.pair_cat, f.pair_cap));
    PSX_TRY(W->alloc(f.cat_count, 10));
    PSX_TRY(W->alloc(f.cat_list, 9 * (size_t)f.pair_cap));
    // the broadphase keeps each leaf's first pairs in the lists' memory until they are
    // placed (k_pairs_place)
    f.trav_k = n > 0 ? (int)std::min<size_t>(1 << 20, 9 * (size_t)f.pair_cap / (2 * (size_t)n)) : 0;
    PSX_TRY(W->alloc(f.trav_tail, 1));
    PSX_TRY(W->alloc(f.man_pair, f.pair_cap));
    epa_save_caps(f.pair_cap, f.lane_saves, f.group_saves);
    PSX_TRY(W->alloc(f.epa_save, epa_save_bytes(f.lane_saves, f.group_saves)));
    PSX_TRY(W->alloc(f.man_tri, (size_t)f.tri_cap * kTriManifolds));
    PSX_TRY(W->alloc(f.pair_tslot, f.pair_cap));
    PSX_TRY(W->alloc(f.pair_nman, f.pair_cap));
    PSX_TRY(W->alloc(f.pair_moff, f.pair_cap));
    PSX_TRY(W->alloc(f.n_man, 1));
    PSX_TRY(W->alloc(f.contacts, f.man_cap));
    PSX_TRY(W->alloc(f.man_scene_cnt, S + 1));
    PSX_TRY(W->alloc(f.scene_man, S + 1));
    PSX_TRY(W->alloc(f.claim, std::max(1, w.n_dyn)));
    PSX_TRY(W->alloc(f.color_of, f.man_cap));
    PSX_TRY(W->alloc(f.corder, f.man_cap));
    PSX_TRY(W->alloc(f.scene_ncolor, S));
    PSX_TRY(W->alloc(f.color_start, (size_t)S * (kMaxColors + 1)));
    PSX_TRY(W->alloc(f.claim_pos, (size_t)S * (kMaxColors + 1)));
    PSX_TRY(W->alloc(f.pt_off, f.man_cap));
    PSX_TRY(W->alloc(f.cbody, f.man_cap));
    PSX_TRY(W->alloc(f.cmask, std::max(1, w.n_dyn)));
    PSX_TRY(W->alloc(f.s_hdr, f.man_cap));
    PSX_TRY(W->alloc(f.s_pts, 4 * (size_t)f.man_cap));
    PSX_TRY(W->alloc(f.cache_a, f.cache_cap));
    PSX_TRY(W->alloc(f.cache_b, f.cache_cap));
    PSX_TRY(W->alloc(f.cache_parity, 1));
    PSX_TRY(W->alloc(f.bar, 4));
    PSX_TRY(W->alloc(f.n_points, 1));
    PSX_TRY(W->alloc(f.n_rows, 1));
    PSX_CUDA(cudaMemset(f.n_points, 0, sizeof(int)));
    PSX_CUDA(cudaMemset(f.n_rows, 0, sizeof(int)));
    PSX_CUDA(cudaMemset(f.bar, 0, 4 * sizeof(unsigned)));
    PSX_CUDA(cudaMemset(f.cache_parity, 0, sizeof(int)));
    PSX_CUDA(cudaMemset(f.cache_a, 0xff, sizeof(CacheEntry) * (size_t)f.cache_cap));
    PSX_CUDA(cudaMemset(f.cache_b, 0xff, sizeof(CacheEntry) * (size_t)f.cache_cap));
    PSX_CUDA(cudaMemset(f.n_pairs, 0, sizeof(int)));
    PSX_CUDA(cudaMemset(f.n_man, 0, sizeof(int)));
    PSX_CUDA(cudaMemset(f.scene_man, 0, sizeof(int) * (S + 1)));
    // trigger sets and the event log, for a world with trigger colliders only
    bool any_trigger = false;
    for (const int4& ci : col_info) any_trigger |= (ci.w & COL_TRIGGER) && (ci.w & COL_ENABLE);
    if (any_trigger) PSX_TRY(alloc_triggers(W));
    // shared memory per solver block: the most a block may have when there are at most as
    // many block scenes as SMs, else a size that keeps two blocks resident per SM (the
    // register budget of the 256-thread solver allows two)
    {
        int dev = 0, sms = 0, optin = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        int want = (int)W->block_scenes_h.size() <= sms ? optin - 5120 : 100 * 1024;   // two blocks per SM
        W->solver_smem = std::max(0, std::min(want, optin - 5120)) / 16 * 16;
        W->solver_smem_large = std::max(0, optin - 5120) / 16 * 16;
    }
    W->big_scenes_h = W->grid_scenes_h;
    {   // longest scenes first, so that none of them starts in the last wave
        auto longer = [&](int a, int b) {
            int na = scene_dyn[a + 1] - scene_dyn[a], nb = scene_dyn[b + 1] - scene_dyn[b];
            return na > nb || (na == nb && a < b);
        };
        std::sort(W->large_scenes_h.begin(), W->large_scenes_h.end(), longer);
    }
    PSX_TRY(W->upload(W->block_scenes, W->block_scenes_h));
    PSX_TRY(W->upload(W->large_scenes, W->large_scenes_h));
    for (int t = 0; t < 3; ++t) PSX_TRY(W->alloc(W->tier_scenes[t], W->block_scenes_h.size()));
    {   // smaller solver blocks pay when more scenes wait than the SMs hold at once; a
        // world of few scenes keeps 256 threads a scene for latency
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        PSX_TRY(partition_tiers(W, (int)W->block_scenes_h.size() > 2 * sms ? 64 : 256));
    }
    PSX_TRY(W->alloc(W->cluster_scenes, W->big_scenes_h.size()));
    PSX_TRY(W->alloc(W->grid_scenes, W->big_scenes_h.size()));
    PSX_TRY(partition_big(W, 0));
    W->scene_bits = S <= 1 ? 0 : ilog2ceil(S);
    {
        // scenes of at most 4096 colliders are sorted block by block in shared memory
        int maxc = 0;
        for (int s = 0; s < S; ++s) maxc = std::max(maxc, scene_col[s + 1] - scene_col[s]);
        int P = 1;
        while (P < maxc) P <<= 1;
        W->scene_sort_pmax = P <= 4096 ? P : 0;   // at most 32 KB of shared memory
    }
    // creation bounds: no margin (src/Physecs.cpp:32)
    launch_aabb(w, 0, W->stream);
    PSX_CUDA(cudaGetLastError());
    PSX_CUDA(cudaStreamSynchronize(W->stream));
    return PSX_OK;
}

// One frame = Scene::simulate for every scene: broadphase, narrowphase, contact rows,
// joint layout, the solver kernel (colouring + all substeps), end-of-frame bounds.
// ev (optional) receives 6 events delimiting the 5 stages.  Returns kernels queued.
int psx::rt::queue_frame(psx_world* W, cudaEvent_t* ev) {
    int k = 0;
    cudaStream_t s = W->stream;
    if (ev) cudaEventRecord(ev[0], s);
    k += launch_broadphase(W->w, W->f, W->scene_bits, W->scene_sort_pmax, s);
    if (ev) cudaEventRecord(ev[1], s);
    k += launch_narrowphase(W->w, W->f, StreamPair{W->aux_stream, W->ev_fork2, W->ev_join2}, W->narrow, s);
    if (ev) cudaEventRecord(ev[2], s);
    k += launch_contacts(W->w, W->f, s);
    k += launch_joint_layout(W->w, W->f, s);
    if (ev) cudaEventRecord(ev[3], s);
    auto tier_smem = [&](int nt) { return std::max(12 * 1024, W->solver_smem * nt / 256) / 16 * 16; };
    const int nt0 = W->threads_min <= 32 ? 32 : 64;
    SolverLaunch L{{W->tier_scenes[0], W->tier_scenes[1], W->tier_scenes[2]},
                   {(int)W->tier_h[0].size(), (int)W->tier_h[1].size(), (int)W->tier_h[2].size()},
                   {tier_smem(nt0), tier_smem(128), W->solver_smem}, nt0,
                   {W->tier_stream[0], W->tier_stream[1]}, W->ev_tfork, {W->ev_tjoin[0], W->ev_tjoin[1]},
                   W->large_scenes, (int)W->large_scenes_h.size(), W->solver_smem_large,
                   W->cluster_scenes, (int)W->cluster_scenes_h.size(),
                   W->grid_scenes, (int)W->grid_scenes_h.size(), W->grid_blocks,
                   W->aux_stream, W->ev_fork, W->ev_join, W->wait_limit, W->large_nt};
    k += launch_solver(W->w, W->f, L, s);
    if (ev) cudaEventRecord(ev[4], s);
    k += launch_aabb(W->w, 1, s);
    if (ev) cudaEventRecord(ev[5], s);
    W->launches += k;
    return k;
}

// One frame, launched from a CUDA graph once the world uses one: the first frame runs
// uncaptured (it sets the kernels' one-time attributes), the second is captured, and
// every later frame replays the graph.
psx_status psx::rt::run_frame(psx_world* W) {
    if (!W->use_graph || W->frames_run == 0) {
        W->frame_kernels = queue_frame(W);
    } else {
        if (!W->graph) {
            cudaGraph_t g;
            PSX_CUDA(cudaStreamBeginCapture(W->stream, cudaStreamCaptureModeThreadLocal));
            int k = queue_frame(W);
            W->launches -= k;   // counted when the graph runs
            PSX_CUDA(cudaStreamEndCapture(W->stream, &g));
            // the nodes keep their launches' priorities (the largest scenes' solver goes first)
            PSX_CUDA(cudaGraphInstantiate(&W->graph, g, cudaGraphInstantiateFlagUseNodePriority));
            cudaGraphDestroy(g);
        }
        PSX_CUDA(cudaGraphLaunch(W->graph, W->stream));
        W->launches += W->frame_kernels;
    }
    ++W->frames_run;
    return PSX_OK;
}

// Validate and apply launch shapes (0 keeps the current value).
psx_status psx::rt::alloc_triggers(psx_world* W) {
    FrameBuf& f = W->f;
    if (f.trig_cap) return PSX_OK;
    const int cap = f.pair_cap, tcap = 1 << ilog2ceil(2 * cap), ecap = std::max(4096, 2 * cap);
    for (int k = 0; k < 2; ++k) {
        PSX_TRY(W->alloc(f.trig_table[k], tcap));
        PSX_TRY(W->alloc(f.trig_keys[k], cap));
        PSX_TRY(W->alloc(f.trig_slot[k], cap));
        PSX_CUDA(cudaMemset(f.trig_table[k], 0xff, sizeof(unsigned long long) * (size_t)tcap));
    }
    PSX_TRY(W->alloc(f.trig_state, 4));
    PSX_TRY(W->alloc(f.trig_evt, ecap));
    PSX_TRY(W->alloc(f.n_evt, 1));
    const int state[4] = {0, 0, 0, (int)W->frames_run};   // events count frames from the world's creation
    PSX_CUDA(cudaMemcpy(f.trig_state, state, sizeof(state), cudaMemcpyHostToDevice));
    PSX_CUDA(cudaMemset(f.n_evt, 0, sizeof(int)));
    f.trig_table_cap = tcap;
    f.evt_cap = ecap;
    f.trig_cap = cap;   // last: the frame launches the trigger kernels from here on
    return PSX_OK;
}

psx_status psx::rt::apply_launch(psx_world* W, const psx_launch_config& c) {
    NarrowShape n = W->narrow;
    if (c.convex_warps) n.convex_warps = c.convex_warps;
    if (c.convex_blocks_per_sm) n.convex_blocks_per_sm = c.convex_blocks_per_sm;
    if (c.analytic_threads) n.analytic_threads = c.analytic_threads;
    if (c.analytic_blocks_per_sm) n.analytic_blocks_per_sm = c.analytic_blocks_per_sm;
    if (c.contacts_threads) n.contacts_threads = c.contacts_threads;
    if (c.gjk_blocks_per_sm) n.gjk_blocks_per_sm = c.gjk_blocks_per_sm;
    if (c.epa_lanes) n.epa_lanes = c.epa_lanes;
    if (c.epa_full_only) n.epa_full_only = c.epa_full_only == 1;
    auto threads_ok = [](int t) { return t == 32 || t == 64 || t == 128 || t == 256; };
    if (n.convex_warps < 1 || n.convex_warps > 3 || n.convex_blocks_per_sm < 1 || n.convex_blocks_per_sm > 32 ||
        !threads_ok(n.analytic_threads) || n.analytic_blocks_per_sm < 1 || n.analytic_blocks_per_sm > 64 ||
        !threads_ok(n.contacts_threads) || n.gjk_blocks_per_sm < 1 || n.gjk_blocks_per_sm > 16 ||
        (n.epa_lanes != 1 && n.epa_lanes != 8 && n.epa_lanes != 16 && n.epa_lanes != 32))
        return fail(PSX_ERR_INVALID_ARG, "launch config out of range");
    int smem = W->solver_smem;
    if (c.solver_smem_kb) {
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        smem = c.solver_smem_kb * 1024;
        if (smem < 16 * 1024 || smem > optin - 5120) return fail(PSX_ERR_INVALID_ARG, "solver shared memory out of range");
    }
    if (c.large_scene_solver < 0 || c.large_scene_solver > 2) return fail(PSX_ERR_INVALID_ARG, "large_scene_solver out of range");
    if (c.large_scene_solver && c.large_scene_solver != W->large_mode) PSX_TRY(partition_big(W, c.large_scene_solver));
    if (c.solver_threads_min && c.solver_threads_min != 32 && c.solver_threads_min != 64 && c.solver_threads_min != 128 &&
        c.solver_threads_min != 256)
        return fail(PSX_ERR_INVALID_ARG, "solver_threads_min must be 32, 64, 128 or 256");
    if (c.solver_threads_min && c.solver_threads_min != W->threads_min) PSX_TRY(partition_tiers(W, c.solver_threads_min));
    if (c.large_threads && c.large_threads != 128 && c.large_threads != 256 && c.large_threads != 512)
        return fail(PSX_ERR_INVALID_ARG, "large_threads must be 128, 256 or 512");
    if (c.large_threads) W->large_nt = c.large_threads;
    W->narrow = n;
    W->solver_smem = smem;
    if (W->graph) { cudaGraphExecDestroy(W->graph); W->graph = nullptr; }   // recaptured with the new shapes
    return PSX_OK;
}

// A cluster holds a scene's velocities in its blocks' shared memory, so it takes the
// scenes whose velocities fit; several cluster scenes are solved side by side, while the
// grid solves its scenes one after another with all SMs.
psx_status psx::rt::partition_big(psx_world* W, int mode) {
    auto fits = [&](int s) {
        int nd = W->h_scene_dyn[s + 1] - W->h_scene_dyn[s];
        int per = (nd + kClusterBlocks - 1) / kClusterBlocks;
        return (size_t)per * 6 * sizeof(float) <= (size_t)W->solver_smem_large;
    };
    if (mode == 0) {
        int n = 0;
        for (int s : W->big_scenes_h) n += fits(s);
        mode = n >= 2 ? 1 : 2;
    }
    W->cluster_scenes_h.clear();
    W->grid_scenes_h.clear();
    for (int s : W->big_scenes_h) (mode == 1 && fits(s) ? W->cluster_scenes_h : W->grid_scenes_h).push_back(s);
    PSX_CUDA(cudaStreamSynchronize(W->stream));
    if (!W->cluster_scenes_h.empty())
        PSX_CUDA(cudaMemcpy(W->cluster_scenes, W->cluster_scenes_h.data(), W->cluster_scenes_h.size() * sizeof(int), cudaMemcpyHostToDevice));
    if (!W->grid_scenes_h.empty())
        PSX_CUDA(cudaMemcpy(W->grid_scenes, W->grid_scenes_h.data(), W->grid_scenes_h.size() * sizeof(int), cudaMemcpyHostToDevice));
    W->grid_blocks = W->grid_scenes_h.empty() ? 0 : solver_grid_blocks();
    W->large_mode = mode;
    return PSX_OK;
}

// Block scenes of up to 96 dynamic bodies run on 64-thread blocks and up to 384 on
// 128-thread blocks (when threads_min allows), the rest on 256: a colour of a small
// scene holds few contacts, and smaller blocks let more scenes share an SM.  Each list
// is ordered longest scene first.
psx_status psx::rt::partition_tiers(psx_world* W, int threads_min) {
    for (auto& t : W->tier_h) t.clear();
    for (int s : W->block_scenes_h) {
        int nd = W->h_scene_dyn[s + 1] - W->h_scene_dyn[s];
        int t = (threads_min <= 64 && nd <= 96) ? 0 : ((threads_min <= 128 && nd <= 384) ? 1 : 2);
        W->tier_h[t].push_back(s);
    }
    PSX_CUDA(cudaStreamSynchronize(W->stream));
    for (int t = 0; t < 3; ++t) {
        auto& v = W->tier_h[t];
        std::stable_sort(v.begin(), v.end(), [&](int a, int b) {
            return W->h_scene_dyn[a + 1] - W->h_scene_dyn[a] > W->h_scene_dyn[b + 1] - W->h_scene_dyn[b];
        });
        if (!v.empty()) PSX_CUDA(cudaMemcpy(W->tier_scenes[t], v.data(), v.size() * sizeof(int), cudaMemcpyHostToDevice));
    }
    W->threads_min = threads_min;
    return PSX_OK;
}

psx_launch_config psx::rt::current_launch(const psx_world* W) {
    psx_launch_config c{};
    c.convex_warps = W->narrow.convex_warps;
    c.convex_blocks_per_sm = W->narrow.convex_blocks_per_sm;
    c.analytic_threads = W->narrow.analytic_threads;
    c.analytic_blocks_per_sm = W->narrow.analytic_blocks_per_sm;
    c.contacts_threads = W->narrow.contacts_threads;
    c.gjk_blocks_per_sm = W->narrow.gjk_blocks_per_sm;
    c.epa_lanes = W->narrow.epa_lanes;
    c.epa_full_only = W->narrow.epa_full_only ? 1 : 2;
    c.solver_smem_kb = W->solver_smem / 1024;
    c.large_scene_solver = W->large_mode;
    c.solver_threads_min = W->threads_min;
    c.large_threads = W->large_nt;
    return c;
}

psx_status psx::rt::check_err(psx_world* W) {
    int e = 0;
    PSX_CUDA(cudaMemcpy(&e, W->w.err, sizeof(int), cudaMemcpyDeviceToHost));
    if (!e) return PSX_OK;
    char buf[160];
    std::snprintf(buf, sizeof buf, "device error bits 0x%x", e);
    if (e & ERR_BARRIER_TIMEOUT) return fail(PSX_ERR_TIMEOUT, buf);
    return fail(PSX_ERR_CAPACITY, buf);
}

extern "C" {

PSX_API const char* psx_last_error_string(void) { return g_err.c_str(); }

PSX_API psx_status psx_world_create(const psx_scene_desc* scenes, int32_t n_scenes, const psx_world_opts* opts, psx_world** out) {
    if (!scenes || n_scenes <= 0 || !out) return fail(PSX_ERR_INVALID_ARG, "psx_world_create: bad arguments");
    psx_world_opts o{};
    if (opts) o = *opts;
    return create_world(scenes, n_scenes, o, 0, {}, out);
}

}  // extern "C"

// A new world: streams and events, then the scenes.  frames_run: the frames an earlier
// world of these scenes ran (trigger events count frames from there); colors: per scene,
// the joints' colours as the caller's scene assigned them, or empty.
psx_status psx::rt::create_world(const psx_scene_desc* scenes, int n_scenes, psx_world_opts o, long long frames_run,
                                 const std::vector<const int32_t*>& colors, psx_world** out) {
    if (o.block_scene_max_dyn <= 0) o.block_scene_max_dyn = 8192;
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) return fail(PSX_ERR_CUDA, "no CUDA device");
    if (o.device < 0 || o.device >= dev_count) return fail(PSX_ERR_INVALID_ARG, "device ordinal");
    if (cudaSetDevice(o.device) != cudaSuccess) return fail(PSX_ERR_CUDA, "cudaSetDevice");
    psx_world* W = new psx_world();
    W->device = o.device;
    W->use_graph = o.use_graph != 0;
    W->opts_used = o;
    W->opts_used.launch = nullptr;
    W->frames_run = frames_run;
    W->forced_colors = colors;
    cudaError_t e = cudaStreamCreateWithFlags(&W->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) {
        // the aux stream carries the longest chains of the frame (the convex pairs' GJK and
        // EPA passes, the largest scenes' solver): its blocks go first
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        e = cudaStreamCreateWithPriority(&W->aux_stream, cudaStreamNonBlocking, greatest);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&W->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&W->ev_join, cudaEventDisableTiming);
    for (int t = 0; t < 2 && e == cudaSuccess; ++t) {
        e = cudaStreamCreateWithFlags(&W->tier_stream[t], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&W->ev_tjoin[t], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&W->ev_tfork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&W->ev_fork2, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&W->ev_join2, cudaEventDisableTiming);
    if (e != cudaSuccess) { delete W; return fail(PSX_ERR_CUDA, cudaGetErrorString(e)); }
    psx_status s = build_world(W, scenes, n_scenes, o);
    W->forced_colors.clear();
    if (s != PSX_OK) { delete W; return s; }
    if (o.launch) {
        s = apply_launch(W, *o.launch);
        if (s != PSX_OK) { delete W; return s; }
    }
    *out = W;
    return PSX_OK;
}

extern "C" {

PSX_API psx_status psx_world_destroy(psx_world* w) {
    if (w) cudaSetDevice(w->device);
    if (!w) return fail(PSX_ERR_INVALID_ARG, "null world");
    cudaStreamSynchronize(w->stream);
    delete w;
    return PSX_OK;
}

PSX_API psx_status psx_world_set_knobs(psx_world* W, int32_t scene, int32_t substeps, int32_t iterations, float gravity) {
    if (W) cudaSetDevice(W->device);
    if (!W || substeps <= 0 || iterations < 0 || scene >= W->n_scenes) return fail(PSX_ERR_INVALID_ARG, "set_knobs");
    for (int s = 0; s < W->n_scenes; ++s) {
        if (scene >= 0 && s != scene) continue;
        W->h_knobs[s].x = (float)substeps; W->h_knobs[s].y = (float)iterations; W->h_knobs[s].z = gravity;
    }
    W->knobs_dirty = true;
    return PSX_OK;
}

PSX_API psx_status psx_world_set_wait_limit(psx_world* W, int64_t polls) {
    if (!W || polls < 0) return fail(PSX_ERR_INVALID_ARG, "psx_world_set_wait_limit: bad arguments");
    PSX_CUDA(cudaSetDevice(W->device));
    if (W->wait_limit != polls) {
        PSX_CUDA(cudaStreamSynchronize(W->stream));
        W->wait_limit = polls;
        if (W->graph) { cudaGraphExecDestroy(W->graph); W->graph = nullptr; }   // recaptured with the new limit
    }
    return PSX_OK;
}

PSX_API psx_status psx_world_step(psx_world* W, float dt, int32_t frames) {
    if (W) cudaSetDevice(W->device);
    if (!W || frames < 0) return fail(PSX_ERR_INVALID_ARG, "psx_world_step");
    if (W->knobs_dirty || W->h_knobs.empty() || W->h_knobs[0].w != dt) {
        for (auto& k : W->h_knobs) k.w = dt;
        PSX_CUDA(cudaMemcpyAsync(W->w.knobs, W->h_knobs.data(), sizeof(float4) * W->h_knobs.size(), cudaMemcpyHostToDevice, W->stream));
        W->knobs_dirty = false;
    }
    for (int i = 0; i < frames; ++i) {
        PSX_TRY(run_frame(W));
    }
    PSX_CUDA(cudaGetLastError());
    return PSX_OK;
}

PSX_API psx_status psx_world_step_timed(psx_world* W, float dt, int32_t frames, float* total_ms, float* stage_ms,
                                        int64_t* kernels) {
    if (W) cudaSetDevice(W->device);
    if (!W || frames <= 0) return fail(PSX_ERR_INVALID_ARG, "psx_world_step_timed");
    if (W->knobs_dirty || W->h_knobs.empty() || W->h_knobs[0].w != dt) {
        for (auto& k : W->h_knobs) k.w = dt;
        PSX_CUDA(cudaMemcpyAsync(W->w.knobs, W->h_knobs.data(), sizeof(float4) * W->h_knobs.size(), cudaMemcpyHostToDevice, W->stream));
        W->knobs_dirty = false;
    }
    size_t need = 6 * (size_t)frames;
    while (W->events.size() < need) {
        cudaEvent_t e;
        PSX_CUDA(cudaEventCreate(&e));
        W->events.push_back(e);
    }
    long long k0 = W->launches;
    if (W->use_graph) {
        // frames as psx_world_step runs them (graph replays after the first two), timed as
        // a whole; then, outside that time, one more frame launched eagerly between stage
        // events gives the stage split
        PSX_CUDA(cudaEventRecord(W->events[0], W->stream));
        for (int i = 0; i < frames; ++i) PSX_TRY(run_frame(W));
        PSX_CUDA(cudaEventRecord(W->events[1], W->stream));
        PSX_CUDA(cudaGetLastError());
        if (kernels) *kernels = W->launches - k0;
        PSX_CUDA(cudaEventSynchronize(W->events[1]));
        float tot = 0;
        PSX_CUDA(cudaEventElapsedTime(&tot, W->events[0], W->events[1]));
        if (total_ms) *total_ms = tot;
        if (stage_ms) {
            queue_frame(W, &W->events[0]);
            ++W->frames_run;
            PSX_CUDA(cudaGetLastError());
            PSX_CUDA(cudaEventSynchronize(W->events[5]));
            for (int s = 0; s < 5; ++s) {
                float ms = 0;
                PSX_CUDA(cudaEventElapsedTime(&ms, W->events[s], W->events[s + 1]));
                stage_ms[s] = ms * frames;
            }
        }
        return check_err(W);
    }
    for (int i = 0; i < frames; ++i) queue_frame(W, &W->events[6 * (size_t)i]);
    W->frames_run += frames;
    PSX_CUDA(cudaGetLastError());
    PSX_CUDA(cudaEventSynchronize(W->events[6 * (size_t)frames - 1]));
    float st[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < frames; ++i) {
        for (int s = 0; s < 5; ++s) {
            float ms = 0;
            PSX_CUDA(cudaEventElapsedTime(&ms, W->events[6 * i + s], W->events[6 * i + s + 1]));
            st[s] += ms;
        }
    }
    float tot = 0;
    PSX_CUDA(cudaEventElapsedTime(&tot, W->events[0], W->events[6 * (size_t)frames - 1]));
    if (total_ms) *total_ms = tot;
    if (stage_ms) for (int s = 0; s < 5; ++s) stage_ms[s] = st[s];
    if (kernels) *kernels = W->launches - k0;
    return check_err(W);
}

// Mean time of one stage (0 broadphase, 1 narrowphase, 2 contact rows, 3 solver) over
// `frames` frames, after one untimed frame with the same shapes.
static psx_status time_stage(psx_world* W, int frames, int stage, float* ms) {
    queue_frame(W);
    W->frames_run += frames + 1;
    size_t need = 6 * (size_t)frames;
    while (W->events.size() < need) {
        cudaEvent_t e;
        PSX_CUDA(cudaEventCreate(&e));
        W->events.push_back(e);
    }
    for (int i = 0; i < frames; ++i) queue_frame(W, &W->events[6 * (size_t)i]);
    PSX_CUDA(cudaStreamSynchronize(W->stream));
    PSX_TRY(check_err(W));
    float sum = 0;
    for (int i = 0; i < frames; ++i) {
        float t = 0;
        PSX_CUDA(cudaEventElapsedTime(&t, W->events[6 * (size_t)i + stage], W->events[6 * (size_t)i + stage + 1]));
        sum += t;
    }
    *ms = sum / frames;
    return PSX_OK;
}

PSX_API psx_status psx_world_tune(psx_world* W, int32_t frames, psx_launch_config* best) {
    if (!W || frames < 1) return fail(PSX_ERR_INVALID_ARG, "psx_world_tune");
    PSX_CUDA(cudaSetDevice(W->device));
    if (W->h_knobs.empty()) return fail(PSX_ERR_INVALID_ARG, "empty world");
    psx_launch_config cur = current_launch(W);
    struct Knob { int stage; std::vector<psx_launch_config> cands; };
    std::vector<Knob> knobs;
    {   // GJK: 128-thread blocks per SM
        Knob k{1, {}};
        for (int b : {4, 8, 12, 16}) {
            psx_launch_config c{};
            c.gjk_blocks_per_sm = b;
            k.cands.push_back(c);
        }
        knobs.push_back(k);
    }
    {   // EPA: lanes per pair, warps per block, blocks per SM (a SmallPoly per pair in shared
        // memory; the registers allow about 28 warps per SM); 1: a lane per pair, with the
        // grouped kernel's blocks for the pairs that outgrow it
        Knob k{1, {}};
        const int cands[][3] = {{32, 1, 15}, {32, 1, 24}, {32, 1, 32}, {32, 2, 12}, {32, 3, 8}, {16, 1, 20}, {8, 1, 12},
                                {1, 1, 8}};
        for (const auto& c3 : cands) {
            psx_launch_config c{};
            c.epa_lanes = c3[0];
            c.convex_warps = c3[1];
            c.convex_blocks_per_sm = c3[2];
            k.cands.push_back(c);
        }
        knobs.push_back(k);
    }
    {   // analytic pairs
        Knob k{1, {}};
        for (int t : {64, 128, 256})
            for (int b : {4, 8, 16}) {
                psx_launch_config c{};
                c.analytic_threads = t;
                c.analytic_blocks_per_sm = b;
                k.cands.push_back(c);
            }
        knobs.push_back(k);
    }
    {   // convex contact generation
        Knob k{1, {}};
        for (int t : {64, 128, 256}) {
            psx_launch_config c{};
            c.contacts_threads = t;
            k.cands.push_back(c);
        }
        knobs.push_back(k);
    }
    if (!W->big_scenes_h.empty()) {   // scenes above the block limit: clusters or the grid
        Knob k{3, {}};
        for (int m : {1, 2}) {
            psx_launch_config c{};
            c.large_scene_solver = m;
            k.cands.push_back(c);
        }
        knobs.push_back(k);
    }
    if (!W->block_scenes_h.empty()) {   // the smallest solver block size
        Knob k{3, {}};
        for (int t : {32, 64, 128, 256}) {
            psx_launch_config c{};
            c.solver_threads_min = t;
            k.cands.push_back(c);
        }
        knobs.push_back(k);
    }
    if (!W->large_scenes_h.empty()) {   // block scenes above 1024 bodies: one big block or several smaller ones an SM
        Knob k{3, {}};
        for (int t : {512, 256, 128}) {
            psx_launch_config c{};
            c.large_threads = t;
            k.cands.push_back(c);
        }
        knobs.push_back(k);
    }
    if (W->block_scenes_h.size() > 152) {   // many small scenes: shared memory per solver block
        Knob k{3, {}};
        for (int kb : {48, 64, 100}) {
            psx_launch_config c{};
            c.solver_smem_kb = kb;
            k.cands.push_back(c);
        }
        knobs.push_back(k);
    }
    for (const Knob& k : knobs) {
        float best_ms = 1e30f;
        psx_launch_config pick = cur;
        for (const psx_launch_config& c : k.cands) {
            PSX_TRY(apply_launch(W, cur));
            PSX_TRY(apply_launch(W, c));
            float ms = 0;
            PSX_TRY(time_stage(W, frames, k.stage, &ms));
            if (ms < best_ms) { best_ms = ms; pick = current_launch(W); }
        }
        cur = pick;
        PSX_TRY(apply_launch(W, cur));
    }
    if (best) *best = cur;
    return PSX_OK;
}

PSX_API psx_status psx_world_launch_config(psx_world* W, psx_launch_config* out) {
    if (!W || !out) return fail(PSX_ERR_INVALID_ARG, "psx_world_launch_config");
    *out = current_launch(W);
    return PSX_OK;
}

PSX_API psx_status psx_world_synchronize(psx_world* W) {
    if (W) cudaSetDevice(W->device);
    if (!W) return fail(PSX_ERR_INVALID_ARG, "null world");
    PSX_CUDA(cudaStreamSynchronize(W->stream));
    return check_err(W);
}

// device staging for the caller's 3-float arrays, grown once
static psx_status body_stage(psx_world* W, float** out) {
    const size_t n = 9 * (size_t)std::max(1, W->w.n_bodies);
    if (W->bstage_n < n) {
        PSX_CUDA(cudaStreamSynchronize(W->stream));
        if (W->bstage) cudaFree(W->bstage);
        W->bstage = nullptr;
        W->bstage_n = 0;
        PSX_CUDA(cudaMalloc(&W->bstage, n * sizeof(float)));
        W->bstage_n = n;
    }
    *out = W->bstage;
    return PSX_OK;
}

// The caller's arrays are copied as they are (page-locked ones through psx_pin_host at the
// link's speed) and repacked on the device.
static psx_status read_bodies(psx_world* W, float* pos, float* quat, float* vel, float* ang, bool sync_after) {
    (void)sync_after;
    const World& w = W->w;
    const size_t nb = w.n_bodies;
    float* st = nullptr;
    PSX_TRY(body_stage(W, &st));
    float *sp = st, *sv = st + 3 * nb, *sa = st + 6 * nb;
    launch_pack_bodies(w, pos ? sp : nullptr, vel ? sv : nullptr, ang ? sa : nullptr, W->stream);
    if (pos) PSX_CUDA(cudaMemcpyAsync(pos, sp, 3 * nb * sizeof(float), cudaMemcpyDeviceToHost, W->stream));
    if (quat) PSX_CUDA(cudaMemcpyAsync(quat, w.quat, nb * sizeof(float4), cudaMemcpyDeviceToHost, W->stream));
    if (vel) PSX_CUDA(cudaMemcpyAsync(vel, sv, 3 * nb * sizeof(float), cudaMemcpyDeviceToHost, W->stream));
    if (ang) PSX_CUDA(cudaMemcpyAsync(ang, sa, 3 * nb * sizeof(float), cudaMemcpyDeviceToHost, W->stream));
    PSX_CUDA(cudaStreamSynchronize(W->stream));
    return PSX_OK;
}

PSX_API psx_status psx_world_read_bodies(psx_world* W, float* pos, float* quat, float* vel, float* ang_vel) {
    if (W) cudaSetDevice(W->device);
    if (!W) return fail(PSX_ERR_INVALID_ARG, "null world");
    return read_bodies(W, pos, quat, vel, ang_vel, true);
}

PSX_API psx_status psx_world_write_bodies(psx_world* W, const float* pos, const float* quat, const float* vel, const float* ang) {
    if (W) cudaSetDevice(W->device);
    if (!W) return fail(PSX_ERR_INVALID_ARG, "null world");
    const World& w = W->w;
    const size_t nb = w.n_bodies;
    float* st = nullptr;
    PSX_TRY(body_stage(W, &st));
    float *sp = st, *sv = st + 3 * nb, *sa = st + 6 * nb;
    if (pos) PSX_CUDA(cudaMemcpyAsync(sp, pos, 3 * nb * sizeof(float), cudaMemcpyHostToDevice, W->stream));
    if (quat) PSX_CUDA(cudaMemcpyAsync(w.quat, quat, nb * sizeof(float4), cudaMemcpyHostToDevice, W->stream));
    if (vel) PSX_CUDA(cudaMemcpyAsync(sv, vel, 3 * nb * sizeof(float), cudaMemcpyHostToDevice, W->stream));
    if (ang) PSX_CUDA(cudaMemcpyAsync(sa, ang, 3 * nb * sizeof(float), cudaMemcpyHostToDevice, W->stream));
    launch_unpack_bodies(w, pos ? sp : nullptr, vel ? sv : nullptr, ang ? sa : nullptr, W->stream);
    PSX_CUDA(cudaStreamSynchronize(W->stream));   // the caller may reuse its arrays on return
    return PSX_OK;
}

// A range whose pages another registration already covers stays as it is (two small
// arrays can share a page); unpinning such a range is then a no-op.
PSX_API psx_status psx_pin_host(void* p, size_t bytes) {
    if (!p || !bytes) return fail(PSX_ERR_INVALID_ARG, "psx_pin_host: bad arguments");
    const cudaError_t e = cudaHostRegister(p, bytes, cudaHostRegisterDefault);
    if (e == cudaErrorHostMemoryAlreadyRegistered) { cudaGetLastError(); return PSX_OK; }
    PSX_CUDA(e);
    return PSX_OK;
}

PSX_API psx_status psx_unpin_host(void* p) {
    if (!p) return fail(PSX_ERR_INVALID_ARG, "psx_unpin_host: null pointer");
    const cudaError_t e = cudaHostUnregister(p);
    if (e == cudaErrorHostMemoryNotRegistered) { cudaGetLastError(); return PSX_OK; }
    PSX_CUDA(e);
    return PSX_OK;
}

PSX_API psx_status psx_world_apply_deltas(psx_world* W, int32_t n, const psx_body_delta* d) {
    if (!W || n < 0 || (n && !d)) return fail(PSX_ERR_INVALID_ARG, "psx_world_apply_deltas: bad arguments");
    if (n == 0) return PSX_OK;
    static_assert(sizeof(psx_body_delta) == sizeof(DeltaRec), "psx_body_delta layout");
    PSX_CUDA(cudaSetDevice(W->device));
    // fold the batch per body, in order: a kinematic toggle zeroes the velocities at its point
    std::vector<DeltaRec> recs;
    psx_status st = PSX_OK;
    for (int i = 0; i < n && st == PSX_OK; ++i) {
        const psx_body_delta& e = d[i];
        if (e.scene < 0 || e.scene >= W->n_scenes || e.body < 0 ||
            e.body >= W->h_scene_body[e.scene + 1] - W->h_scene_body[e.scene] || (e.mask & ~7)) {
            st = fail(PSX_ERR_INVALID_ARG, "psx_world_apply_deltas: scene, body or mask of record " + std::to_string(i));
            break;
        }
        const int b = W->h_scene_body[e.scene] + e.body;
        if ((e.mask & (PSX_DELTA_VELOCITY | PSX_DELTA_KINEMATIC)) && W->h_body_dyn[b] < 0) {
            st = fail(PSX_ERR_INVALID_ARG, "psx_world_apply_deltas: velocity or kinematic flag of a static body");
            break;
        }
        if ((e.mask & PSX_DELTA_KINEMATIC) && W->h_body_overflow[b]) {
            st = fail(PSX_ERR_INVALID_ARG, "psx_world_apply_deltas: kinematic flag of a body jointed in the overflow colour");
            break;
        }
        int& slot = W->h_delta_slot[b];
        if (slot < 0) {
            slot = (int)recs.size();
            DeltaRec r{};
            r.body = b;
            recs.push_back(r);
        }
        DeltaRec& r = recs[slot];
        if (e.mask & PSX_DELTA_POSE) {
            r.mask |= DELTA_POSE;
            for (int k = 0; k < 3; ++k) r.pos[k] = e.pos[k];
            for (int k = 0; k < 4; ++k) r.quat[k] = e.quat[k];
        }
        if (e.mask & PSX_DELTA_VELOCITY) {
            r.mask |= DELTA_VELOCITY;
            for (int k = 0; k < 3; ++k) { r.vel[k] = e.vel[k]; r.ang[k] = e.ang_vel[k]; }
        }
        if (e.mask & PSX_DELTA_KINEMATIC) {
            r.mask |= DELTA_KINEMATIC;
            r.kinematic = e.kinematic != 0;
            if (r.kinematic) {
                r.mask |= DELTA_VELOCITY;
                for (int k = 0; k < 3; ++k) r.vel[k] = r.ang[k] = 0.f;
            }
        }
    }
    for (const DeltaRec& r : recs) W->h_delta_slot[r.body] = -1;
    if (st != PSX_OK) return st;
    // the joints to fix up; the host's kinematic flags change only once the upload and
    // the kernel are queued, so a failed call leaves host and device as they were
    std::vector<int> joints;
    for (const DeltaRec& r : recs) {
        if (!(r.mask & DELTA_KINEMATIC)) continue;
        for (int k = W->h_bj_start[r.body]; k < W->h_bj_start[r.body + 1]; ++k) joints.push_back(W->h_bj[k]);
    }
    std::sort(joints.begin(), joints.end());
    joints.erase(std::unique(joints.begin(), joints.end()), joints.end());
    // one staging buffer (records, then joint ids), reused once its last upload is done
    const size_t rec_b = sizeof(DeltaRec) * recs.size(), bytes = rec_b + sizeof(int) * joints.size();
    if (W->ev_delta) PSX_CUDA(cudaEventSynchronize(W->ev_delta));
    else PSX_CUDA(cudaEventCreateWithFlags(&W->ev_delta, cudaEventDisableTiming));
    if (W->dpin_bytes < bytes) {
        if (W->dpin) cudaFreeHost(W->dpin);
        W->dpin = nullptr;
        W->dpin_bytes = 0;
        PSX_CUDA(cudaMallocHost(&W->dpin, bytes));
        W->dpin_bytes = bytes;
    }
    if (W->ddev_bytes < bytes) {
        PSX_CUDA(cudaStreamSynchronize(W->stream));
        if (W->ddev) cudaFree(W->ddev);
        W->ddev = nullptr;
        W->ddev_bytes = 0;
        PSX_CUDA(cudaMalloc(&W->ddev, bytes));
        W->ddev_bytes = bytes;
    }
    char* hp = reinterpret_cast<char*>(W->dpin);
    std::memcpy(hp, recs.data(), rec_b);
    if (!joints.empty()) std::memcpy(hp + rec_b, joints.data(), sizeof(int) * joints.size());
    PSX_CUDA(cudaMemcpyAsync(W->ddev, hp, bytes, cudaMemcpyHostToDevice, W->stream));
    PSX_CUDA(cudaEventRecord(W->ev_delta, W->stream));
    const DeltaRec* dd = reinterpret_cast<const DeltaRec*>(W->ddev);
    const int* dj = reinterpret_cast<const int*>(W->ddev + rec_b);
    W->launches += launch_apply_deltas(W->w, dd, (int)recs.size(), dj, (int)joints.size(), W->stream);
    PSX_CUDA(cudaGetLastError());
    for (const DeltaRec& r : recs) {
        if (!(r.mask & DELTA_KINEMATIC)) continue;
        int& fl = W->h_body_flags[r.body];
        const bool was_sim = (fl & PSX_BODY_DYNAMIC) && !(fl & PSX_BODY_KINEMATIC);
        fl = r.kinematic ? (fl | PSX_BODY_KINEMATIC) : (fl & ~PSX_BODY_KINEMATIC);
        const bool sim = (fl & PSX_BODY_DYNAMIC) && !(fl & PSX_BODY_KINEMATIC);
        W->n_simulated += (int)sim - (int)was_sim;
    }
    // triangle-mesh colliders of posed bodies
    for (const DeltaRec& r : recs) {
        if (!(r.mask & DELTA_POSE)) continue;
        for (int c = W->h_body_col[r.body]; c < W->h_body_col[r.body + 1]; ++c)
            if (W->h_col_trimesh[c] >= 0) W->launches += launch_trimesh_bounds(W->w, c, c + 1, true, W->stream);
    }
    return PSX_OK;
}

PSX_API psx_status psx_world_set_joint_params(psx_world* W, int32_t scene, int32_t joint, const float* params) {
    if (!W || !params || scene < 0 || scene >= W->n_scenes)
        return fail(PSX_ERR_INVALID_ARG, "psx_world_set_joint_params: bad arguments");
    const int j0 = W->h_scene_joint[scene], j1 = W->h_scene_joint[scene + 1];
    if (joint < 0 || joint >= j1 - j0) return fail(PSX_ERR_INVALID_ARG, "psx_world_set_joint_params: joint index");
    PSX_CUDA(cudaSetDevice(W->device));
    // the joint's parameter block in its device record; every frame reads it (the rows a
    // joint has are laid out per frame), so the change takes effect from the next frame
    float* dst = W->w.joints[j0 + joint].params;
    PSX_CUDA(cudaMemcpyAsync(dst, params, PSX_JOINT_PARAMS * sizeof(float), cudaMemcpyHostToDevice, W->stream));
    return PSX_OK;
}

PSX_API psx_status psx_world_set_contact_filter(psx_world* W, psx_contact_filter fn) {
    if (!W) return fail(PSX_ERR_INVALID_ARG, "psx_world_set_contact_filter: null world");
    PSX_CUDA(cudaSetDevice(W->device));
    PSX_CUDA(cudaStreamSynchronize(W->stream));
    World& w = W->w;
    if (!fn) {
        w.filter_table = nullptr;
    } else {
        // the filter sees only (isTrigger, data) of the two colliders: one call per pair of classes
        std::map<std::pair<int, int>, int> cls;
        std::vector<int> col_class(w.n_colliders);
        std::vector<std::pair<int, int>> key_of;
        for (int c = 0; c < w.n_colliders; ++c) {
            const std::pair<int, int> k{W->h_col_trig[c], W->h_col_data[c]};
            auto it = cls.find(k);
            if (it == cls.end()) {
                it = cls.emplace(k, (int)key_of.size()).first;
                key_of.push_back(k);
            }
            col_class[c] = it->second;
        }
        const int K = (int)key_of.size();
        if (K > 1024) return fail(PSX_ERR_CAPACITY, "psx_world_set_contact_filter: more than 1024 (isTrigger, data) classes");
        std::vector<unsigned char> table((size_t)K * K);
        bool any_trigger = false;
        for (int i = 0; i < K; ++i)
            for (int j = 0; j < K; ++j) {
                const int r = fn(key_of[i].first, key_of[i].second, key_of[j].first, key_of[j].second);
                if (r != PSX_CONTACT_COLLISION && r != PSX_CONTACT_TRIGGER)
                    return fail(PSX_ERR_INVALID_ARG, "psx_world_set_contact_filter: the filter returned " + std::to_string(r));
                table[(size_t)i * K + j] = r == PSX_CONTACT_TRIGGER;
                any_trigger |= r == PSX_CONTACT_TRIGGER;
            }
        if (any_trigger) PSX_TRY(alloc_triggers(W));
        if (!w.col_class) PSX_TRY(W->alloc(w.col_class, std::max(1, w.n_colliders)));
        if (w.n_colliders) PSX_CUDA(cudaMemcpy(w.col_class, col_class.data(), sizeof(int) * w.n_colliders, cudaMemcpyHostToDevice));
        PSX_TRY(W->upload_reuse(w.filter_table, W->filter_cap, table));
        w.n_classes = K;
    }
    if (W->graph) { cudaGraphExecDestroy(W->graph); W->graph = nullptr; }   // the frame reads w by value
    return PSX_OK;
}

PSX_API psx_status psx_world_set_can_collide(psx_world* W, int32_t scene, int32_t body0, int32_t body1, int32_t can_collide) {
    if (!W || scene < 0 || scene >= W->n_scenes) return fail(PSX_ERR_INVALID_ARG, "psx_world_set_can_collide: scene");
    const int nb = W->h_scene_body[scene + 1] - W->h_scene_body[scene];
    if (body0 < 0 || body0 >= nb || body1 < 0 || body1 >= nb) return fail(PSX_ERR_INVALID_ARG, "psx_world_set_can_collide: body");
    PSX_CUDA(cudaSetDevice(W->device));
    const int b0 = W->h_scene_body[scene] + body0, b1 = W->h_scene_body[scene] + body1;
    const int2 key = make_int2(std::min(b0, b1), std::max(b0, b1));
    auto less = [](int2 a, int2 b) { return a.x < b.x || (a.x == b.x && a.y < b.y); };
    auto it = std::lower_bound(W->h_nc.begin(), W->h_nc.end(), key, less);
    const bool present = it != W->h_nc.end() && it->x == key.x && it->y == key.y;
    if (can_collide && present) W->h_nc.erase(it);
    else if (!can_collide && !present) W->h_nc.insert(it, key);
    else return PSX_OK;
    PSX_CUDA(cudaStreamSynchronize(W->stream));
    World& w = W->w;
    PSX_TRY(W->upload_reuse(w.nc_pairs, W->nc_cap, W->h_nc));
    w.n_nc = (int)W->h_nc.size();
    if (W->graph) { cudaGraphExecDestroy(W->graph); W->graph = nullptr; }
    return PSX_OK;
}

PSX_API psx_status psx_world_simulate_host(psx_world* W, float dt, float* pos, float* quat, float* vel, float* ang) {
    if (W) cudaSetDevice(W->device);
    PSX_TRY(psx_world_write_bodies(W, pos, quat, vel, ang));
    PSX_TRY(psx_world_step(W, dt, 1));
    PSX_TRY(read_bodies(W, pos, quat, vel, ang, true));
    return check_err(W);
}

PSX_API psx_status psx_world_counts(psx_world* W, int32_t* counts) {
    if (W) cudaSetDevice(W->device);
    if (!W || !counts) return fail(PSX_ERR_INVALID_ARG, "counts");
    PSX_CUDA(cudaStreamSynchronize(W->stream));
    int np = 0, nm = 0, e = 0, pts = 0, rows = 0;
    PSX_CUDA(cudaMemcpy(&np, W->f.n_pairs, sizeof(int), cudaMemcpyDeviceToHost));
    PSX_CUDA(cudaMemcpy(&nm, W->f.n_man, sizeof(int), cudaMemcpyDeviceToHost));
    PSX_CUDA(cudaMemcpy(&e, W->w.err, sizeof(int), cudaMemcpyDeviceToHost));
    PSX_CUDA(cudaMemcpy(&pts, W->f.n_points, sizeof(int), cudaMemcpyDeviceToHost));
    PSX_CUDA(cudaMemcpy(&rows, W->f.n_rows, sizeof(int), cudaMemcpyDeviceToHost));
    counts[0] = W->w.n_bodies; counts[1] = W->w.n_colliders; counts[2] = W->w.n_dyn; counts[3] = W->w.n_joints;
    counts[4] = W->n_scenes; counts[5] = np; counts[6] = std::min(nm, W->f.man_cap); counts[7] = e;
    counts[8] = pts; counts[9] = rows;
    counts[10] = W->n_simulated;
    counts[11] = (int32_t)std::min<long long>(W->launches, 0x7fffffff);
    return PSX_OK;
}

PSX_API psx_status psx_world_narrow_counts(psx_world* W, int32_t* counts) {
    if (W) cudaSetDevice(W->device);
    if (!W || !counts) return fail(PSX_ERR_INVALID_ARG, "narrow counts");
    PSX_CUDA(cudaStreamSynchronize(W->stream));
    int c[10] = {};
    PSX_CUDA(cudaMemcpy(c, W->f.cat_count, sizeof c, cudaMemcpyDeviceToHost));
    const bool flat = W->narrow.epa_lanes == 1;
    counts[0] = c[1];
    counts[1] = c[3];
    counts[2] = flat ? c[8] : 0;
    counts[3] = W->narrow.epa_full_only ? 0 : c[6];
    return PSX_OK;
}

PSX_API int32_t psx_world_get_pairs(psx_world* W, int32_t* out, int32_t cap) {
    if (W) cudaSetDevice(W->device);
    if (!W) return -1;
    cudaStreamSynchronize(W->stream);
    int np = 0;
    cudaMemcpy(&np, W->f.n_pairs, sizeof(int), cudaMemcpyDeviceToHost);
    std::vector<int2> pr(np);
    if (np) cudaMemcpy(pr.data(), W->f.pairs, np * sizeof(int2), cudaMemcpyDeviceToHost);
    std::vector<int4> ci(W->w.n_colliders);
    cudaMemcpy(ci.data(), W->w.col_info, ci.size() * sizeof(int4), cudaMemcpyDeviceToHost);
    for (int i = 0; i < np && i < cap; ++i) {
        int a = pr[i].x, b = pr[i].y;
        int ba = ci[a].x, bb = ci[b].x;
        int s = (int)(std::upper_bound(W->h_scene_body.begin(), W->h_scene_body.end(), ba) - W->h_scene_body.begin()) - 1;
        out[5 * i + 0] = s;
        out[5 * i + 1] = (int32_t)W->h_entity[ba];
        out[5 * i + 2] = W->h_col_local[a];
        out[5 * i + 3] = (int32_t)W->h_entity[bb];
        out[5 * i + 4] = W->h_col_local[b];
    }
    return np;
}

PSX_API int32_t psx_world_get_contacts(psx_world* W, int32_t* ids, float* f, int32_t* meta, int32_t cap) {
    if (W) cudaSetDevice(W->device);
    if (!W) return -1;
    cudaStreamSynchronize(W->stream);
    int S = W->n_scenes;
    std::vector<int> scene_man(S + 1), cstart((size_t)S * (kMaxColors + 1)), ncol(S);
    cudaMemcpy(scene_man.data(), W->f.scene_man, (S + 1) * sizeof(int), cudaMemcpyDeviceToHost);
    int nm = scene_man[S];
    std::vector<Contact> cs(nm);
    std::vector<int> corder(nm), color_of(nm);
    if (nm) {
        cudaMemcpy(cs.data(), W->f.contacts, nm * sizeof(Contact), cudaMemcpyDeviceToHost);
        cudaMemcpy(corder.data(), W->f.corder, nm * sizeof(int), cudaMemcpyDeviceToHost);
        cudaMemcpy(color_of.data(), W->f.color_of, nm * sizeof(int), cudaMemcpyDeviceToHost);
    }
    std::vector<int2> pr;
    int np = 0;
    cudaMemcpy(&np, W->f.n_pairs, sizeof(int), cudaMemcpyDeviceToHost);
    pr.resize(np);
    if (np) cudaMemcpy(pr.data(), W->f.pairs, np * sizeof(int2), cudaMemcpyDeviceToHost);
    std::vector<int4> ci(W->w.n_colliders);
    cudaMemcpy(ci.data(), W->w.col_info, ci.size() * sizeof(int4), cudaMemcpyDeviceToHost);
    int out = 0;
    for (int s = 0; s < S; ++s) {
        // solve order: colour by colour, contacts of one colour by index
        std::vector<int> idx;
        for (int m = scene_man[s]; m < scene_man[s + 1]; ++m) idx.push_back(m);
        std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return color_of[a] < color_of[b]; });
        for (int m : idx) {
            if (out < cap) {
                const Contact& c = cs[m];
                int d0 = W->h_scene_dyn[s];
                int2 p = pr[c.pair];
                ids[8 * out + 0] = s;
                ids[8 * out + 1] = c.b0 >= 0 ? c.b0 - d0 : -1;
                ids[8 * out + 2] = c.b1 >= 0 ? c.b1 - d0 : -1;
                ids[8 * out + 3] = c.np | (c.soft << 8);
                ids[8 * out + 4] = (int32_t)W->h_entity[ci[p.x].x];
                ids[8 * out + 5] = W->h_col_local[p.x];
                ids[8 * out + 6] = (int32_t)W->h_entity[ci[p.y].x];
                ids[8 * out + 7] = W->h_col_local[p.y];
                float* o = f + 56 * out;
                std::memset(o, 0, 56 * sizeof(float));
                o[0] = c.n.x; o[1] = c.n.y; o[2] = c.n.z; o[3] = c.n.w; o[4] = c.frequency; o[5] = c.damping;
                for (int k = 0; k < c.np; ++k) {
                    const ContactPt& p = c.p[k];
                    float* q = o + 8 + 12 * k;
                    q[0] = p.r0.x; q[1] = p.r0.y; q[2] = p.r0.z; q[3] = p.r1.x; q[4] = p.r1.y; q[5] = p.r1.z;
                    q[6] = p.r0.w; q[7] = p.r1.w; q[8] = p.r0xn.w; q[9] = p.r1xn.w;
                }
                if (meta) { meta[2 * out] = color_of[m]; meta[2 * out + 1] = c.tri; }
            }
            ++out;
        }
    }
    return out;
}

PSX_API int32_t psx_world_get_bounds(psx_world* W, float* bounds, int32_t cap) {
    if (W) cudaSetDevice(W->device);
    if (!W) return -1;
    cudaStreamSynchronize(W->stream);
    int n = W->w.n_colliders;
    std::vector<float4> a(n), b(n);
    cudaMemcpy(a.data(), W->w.aabb_min, n * sizeof(float4), cudaMemcpyDeviceToHost);
    cudaMemcpy(b.data(), W->w.aabb_max, n * sizeof(float4), cudaMemcpyDeviceToHost);
    for (int i = 0; i < n && i < cap; ++i) {
        bounds[6 * i] = a[i].x; bounds[6 * i + 1] = a[i].y; bounds[6 * i + 2] = a[i].z;
        bounds[6 * i + 3] = b[i].x; bounds[6 * i + 4] = b[i].y; bounds[6 * i + 5] = b[i].z;
    }
    return n;
}

PSX_API psx_status psx_scene_create(const psx_scene_desc* desc, psx_scene** out) { return psx_world_create(desc, 1, nullptr, out); }
PSX_API psx_status psx_scene_destroy(psx_scene* s) { return psx_world_destroy(s); }
PSX_API psx_status psx_scene_simulate(psx_scene* s, float dt) {
    if (s) cudaSetDevice(s->device);
    PSX_TRY(psx_world_step(s, dt, 1));
    return psx_world_synchronize(s);
}

}  // extern "C"

// ---------------------------------------------------------------- allocation-free body read
// psx_world_read_bodies repacks the state on the device into a staging buffer that it
// grows with cudaMalloc on first use.  Some callers cannot allocate at all while they run:
// a render or control loop with a per-frame deadline (cudaMalloc / cudaMallocHost can
// stall the whole device for milliseconds), or a process whose device memory is
// reserved up front by its own pool allocator.  psx_world_read_bodies_noalloc serves
// them: a pack kernel writes the caller's layout into one fixed, file-scope device
// array, and plain copies move it into the caller's host arrays.

namespace {

constexpr int kNoAllocMaxBodies = 65536;    // bodies one call can read
constexpr int kNoAllocFloatsPerBody = 13;   // pos 3, quat 4, vel 3, ang_vel 3
constexpr int kNoAllocMaxDevices = 64;

// 3.4 MB shared by every call in the process on a given device.  It keeps the
// last call's contents; the pack kernel rewrites every float a call copies out
// (zero velocities for static bodies included), so nothing stale is returned.
// Calls that overlap on the GPU (two streams, two host threads) race on it.
static __device__ __align__(256) float g_noalloc_scratch[kNoAllocMaxBodies * kNoAllocFloatsPerBody];

std::mutex g_noalloc_mu;
float* g_noalloc_addr[kNoAllocMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device, looked up once per device.
psx_status noalloc_scratch(int device, float** out) {
    if (device < 0 || device >= kNoAllocMaxDevices) return fail(PSX_ERR_INVALID_ARG, "device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[device]) {
        float* p = nullptr;
        PSX_CUDA(cudaGetSymbolAddress((void**)&p, g_noalloc_scratch));
        g_noalloc_addr[device] = p;
    }
    *out = g_noalloc_addr[device];
    return PSX_OK;
}

// One thread per body; writes pos[3n] | quat[4n] | vel[3n] | ang_vel[3n] into out.
__global__ void k_pack_bodies(const float4* __restrict__ pos, const float4* __restrict__ quat,
                              const int4* __restrict__ info, const float4* __restrict__ vel,
                              const float4* __restrict__ ang, int n, float* __restrict__ out) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    float* P = out;
    float* Q = out + 3 * (size_t)n;
    float* V = out + 7 * (size_t)n;
    float* A = out + 10 * (size_t)n;
    float4 p = pos[b], q = quat[b];
    int d = info[b].z;
    float4 v = d >= 0 ? vel[d] : make_float4(0.f, 0.f, 0.f, 0.f);
    float4 a = d >= 0 ? ang[d] : make_float4(0.f, 0.f, 0.f, 0.f);
    P[3 * b] = p.x; P[3 * b + 1] = p.y; P[3 * b + 2] = p.z;
    Q[4 * b] = q.x; Q[4 * b + 1] = q.y; Q[4 * b + 2] = q.z; Q[4 * b + 3] = q.w;
    V[3 * b] = v.x; V[3 * b + 1] = v.y; V[3 * b + 2] = v.z;
    A[3 * b] = a.x; A[3 * b + 1] = a.y; A[3 * b + 2] = a.z;
}

}  // namespace

extern "C" {

PSX_API psx_status psx_world_read_bodies_noalloc(psx_world* W, float* pos, float* quat, float* vel, float* ang_vel) {
    if (!W) return fail(PSX_ERR_INVALID_ARG, "null world");
    PSX_CUDA(cudaSetDevice(W->device));
    const int n = W->w.n_bodies;
    if (n > kNoAllocMaxBodies) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "psx_world_read_bodies_noalloc: world has %d bodies, the limit is %d", n,
                      kNoAllocMaxBodies);
        return fail(PSX_ERR_CAPACITY, buf);
    }
    if (n == 0) return PSX_OK;
    float* scratch = nullptr;
    PSX_TRY(noalloc_scratch(W->device, &scratch));
    const World& w = W->w;
    k_pack_bodies<<<(n + 255) / 256, 256, 0, W->stream>>>(w.pos, w.quat, w.info, w.vel, w.ang, n, scratch);
    PSX_CUDA(cudaGetLastError());
    W->launches += 1;
    const size_t fb = sizeof(float);
    if (pos) PSX_CUDA(cudaMemcpyAsync(pos, scratch, 3 * (size_t)n * fb, cudaMemcpyDeviceToHost, W->stream));
    if (quat) PSX_CUDA(cudaMemcpyAsync(quat, scratch + 3 * (size_t)n, 4 * (size_t)n * fb, cudaMemcpyDeviceToHost, W->stream));
    if (vel) PSX_CUDA(cudaMemcpyAsync(vel, scratch + 7 * (size_t)n, 3 * (size_t)n * fb, cudaMemcpyDeviceToHost, W->stream));
    if (ang_vel) PSX_CUDA(cudaMemcpyAsync(ang_vel, scratch + 10 * (size_t)n, 3 * (size_t)n * fb, cudaMemcpyDeviceToHost, W->stream));
    PSX_CUDA(cudaStreamSynchronize(W->stream));
    return PSX_OK;
}

}  // extern "C"
