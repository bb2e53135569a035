// carry.cu — topology changes between frames: a world rebuilt from the scenes as they
// now are, carrying over what the old world holds beyond the bodies' state.
//
// A Physecs scene changes its topology through the registry and its own calls
// (src/Physecs.cpp): registry.create / destroy fire onRigidBodyCreate / onRigidBodyDelete
// and onDynamicCreate / onDynamicDelete (:25-78), addCollider / clearColliders add and
// remove broadphase entries (:725-751), createJoint / destroyJoint edit the joint graph
// (:690-723).  Everything else the scene keeps across the change is per collider or per
// joint:
//   - each collider's broadphase bounds: a new collider starts with creation bounds
//     (no margin); one that existed keeps the bounds of its last update, with the
//     0.01 m margin once its body was simulated or patched (:79-90, 555-559);
//   - the restitution cache, keyed by the two colliders and the triangle (:209-316);
//   - the trigger pairs overlapping in the last frame (:200-207, 537-552);
//   - each joint's colour, and a gear joint's accumulated angles (GearJoint.h:10-17).
// psx_world_recreate builds a new world from the caller's descriptions and moves those
// over from the old world on the device, through the caller's map from new colliders
// and joints to old ones.  The frame counter, launch shapes, wait limit and graph use
// carry over too.
#include <algorithm>
#include <string>
#include <vector>
#include "runtime.cuh"

using namespace psx;
using namespace psx::rt;

namespace {

// bounds of the continued colliders: dst[k] = src[map[k]] where map[k] >= 0
__global__ void k_carry_bounds(float4* dmin, float4* dmax, const float4* smin, const float4* smax, const int* map, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int o = map[k];
    if (o < 0) return;
    dmin[k] = smin[o];
    dmax[k] = smax[o];
}

// The old world's last cache table into the table the new world's first frame reads:
// every entry whose two colliders continue, under its new key.
__global__ void k_carry_cache(const CacheEntry* src, int src_cap, int src_cbits, const int* omap, CacheEntry* dst,
                              int dst_cap, int dst_cbits, int* err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= src_cap) return;
    const CacheEntry e = src[i];
    if (e.key == kEmpty) return;
    const unsigned long long cm = (1ull << src_cbits) - 1ull;
    const int ca = (int)((e.key >> (64 - src_cbits)) & cm), cb = (int)((e.key >> (64 - 2 * src_cbits)) & cm);
    const int tri = (int)(uint32_t)(e.key & ((1ull << (64 - 2 * src_cbits)) - 1ull)) - 1;
    const int na = omap[ca], nb = omap[cb];
    if (na < 0 || nb < 0) return;
    const unsigned long long key = cache_key(na, nb, tri, dst_cbits);
    const unsigned mask = (unsigned)dst_cap - 1u;
    for (unsigned h = cache_hash(key) & mask, probe = 0; probe < (unsigned)dst_cap; ++probe, h = (h + 1) & mask) {
        const unsigned long long old = atomicCAS(&dst[h].key, kEmpty, key);
        if (old == kEmpty || old == key) {
            dst[h].np = e.np;
            for (int q = 0; q < 4; ++q) dst[h].r0tv[q] = e.r0tv[q];
            return;
        }
    }
    atomicOr(err, ERR_CACHE_CAPACITY);
}

// The old world's last-frame trigger set into the new world's (set 1 of a fresh world,
// which its first frame reads as the last frame's): the pairs whose colliders continue.
__global__ void k_carry_triggers(FrameBuf src, FrameBuf dst, const int* omap, int* err) {
    const int prev = src.trig_state[0] ^ 1;
    const int n = min(src.trig_state[1 + prev], src.trig_cap);
    const unsigned mask = (unsigned)dst.trig_table_cap - 1u;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const unsigned long long key = src.trig_keys[prev][t];
        const int na = omap[(int)(key >> 32)], nb = omap[(int)(unsigned)key];
        if (na < 0 || nb < 0) continue;
        const unsigned long long nk = ((unsigned long long)(unsigned)na << 32) | (unsigned)nb;
        const int i = atomicAdd(&dst.trig_state[2], 1);
        if (i >= dst.trig_cap) { atomicOr(err, ERR_PAIR_CAPACITY); continue; }
        unsigned h = trig_hash(nk) & mask;
        for (unsigned probe = 0; probe <= mask; ++probe, h = (h + 1) & mask)
            if (atomicCAS(&dst.trig_table[1][h], kNoKey, nk) == kNoKey) break;
        dst.trig_keys[1][i] = nk;
        dst.trig_slot[1][i] = (int)h;
    }
}

// a gear joint's accumulated angles (the other joint kinds keep nothing across frames)
__global__ void k_carry_joints(JointDev* dst, const JointDev* src, const int* map, int n) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int o = map[j];
    if (o < 0) return;
    dst[j].gearInit = src[o].gearInit;
    dst[j].persistent0 = src[o].persistent0;
    dst[j].persistent1 = src[o].persistent1;
    dst[j].virtual0 = src[o].virtual0;
    dst[j].virtual1 = src[o].virtual1;
}

template <class T>
struct DevArray {
    T* p = nullptr;
    ~DevArray() { if (p) cudaFree(p); }
    psx_status upload(const std::vector<T>& v) {
        if (v.empty()) return PSX_OK;
        PSX_CUDA(cudaMalloc(&p, v.size() * sizeof(T)));
        PSX_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
        return PSX_OK;
    }
};

}  // namespace

extern "C" {

PSX_API psx_status psx_world_recreate(psx_world* F, const psx_scene_desc* scenes, int32_t n_scenes,
                                      const psx_scene_carry* carry, psx_world** out) {
    if (!F || !scenes || n_scenes <= 0 || !carry || !out) return fail(PSX_ERR_INVALID_ARG, "psx_world_recreate: bad arguments");
    PSX_CUDA(cudaSetDevice(F->device));
    PSX_CUDA(cudaStreamSynchronize(F->stream));
    // new -> old maps over world colliders and joints, and the joints' colours
    std::vector<int> cmap, jmap;
    std::vector<const int32_t*> colors(n_scenes, nullptr);
    for (int s = 0; s < n_scenes; ++s) {
        const psx_scene_desc& d = scenes[s];
        const psx_scene_carry& c = carry[s];
        const int from = c.from_scene;
        if (from >= F->n_scenes || d.n_colliders < 0 || d.n_joints < 0)
            return fail(PSX_ERR_INVALID_ARG, "psx_world_recreate: scene " + std::to_string(s) + " continues a scene the old world lacks");
        const int ocb = from >= 0 ? F->h_scene_col[from] : 0, onc = from >= 0 ? F->h_scene_col[from + 1] - ocb : 0;
        const int ojb = from >= 0 ? F->h_scene_joint[from] : 0, onj = from >= 0 ? F->h_scene_joint[from + 1] - ojb : 0;
        for (int k = 0; k < d.n_colliders; ++k) {
            const int o = from >= 0 && c.collider_from ? c.collider_from[k] : -1;
            if (o >= onc) return fail(PSX_ERR_INVALID_ARG, "psx_world_recreate: collider_from out of range");
            cmap.push_back(o >= 0 ? ocb + o : -1);
        }
        for (int j = 0; j < d.n_joints; ++j) {
            const int o = from >= 0 && c.joint_from ? c.joint_from[j] : -1;
            if (o >= onj) return fail(PSX_ERR_INVALID_ARG, "psx_world_recreate: joint_from out of range");
            jmap.push_back(o >= 0 ? ojb + o : -1);
        }
        colors[s] = c.joint_color;
    }
    std::vector<int> omap(std::max(1, F->w.n_colliders), -1);   // old collider -> new, or -1
    for (size_t k = 0; k < cmap.size(); ++k)
        if (cmap[k] >= 0) {
            if (omap[cmap[k]] >= 0) return fail(PSX_ERR_INVALID_ARG, "psx_world_recreate: two colliders continue one");
            omap[cmap[k]] = (int)k;
        }
    // the last frame's trigger pairs that lose a collider: the reference's next frame
    // finds them missing from its new set and calls onTriggerExit for them
    // (src/Physecs.cpp:545-551); they are reported with body -1 for a removed body
    std::vector<psx_trigger_event> vanished;
    if (F->f.trig_cap) {
        int state[4] = {0, 0, 0, 0};
        PSX_CUDA(cudaMemcpy(state, F->f.trig_state, sizeof state, cudaMemcpyDeviceToHost));
        const int prev = state[0] ^ 1, n = std::min(state[1 + prev], F->f.trig_cap);
        std::vector<unsigned long long> keys(std::max(n, 0));
        if (n > 0) PSX_CUDA(cudaMemcpy(keys.data(), F->f.trig_keys[prev], sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost));
        std::vector<int> new_scene(F->n_scenes, -1);
        for (int s = 0; s < n_scenes; ++s)
            if (carry[s].from_scene >= 0) new_scene[carry[s].from_scene] = s;
        std::vector<int> new_col_body;   // new world collider -> new scene-local body
        for (int s = 0; s < n_scenes; ++s)
            for (int b = 0; b < scenes[s].n_bodies; ++b)
                for (int c = scenes[s].collider_start[b]; c < scenes[s].collider_start[b + 1]; ++c) new_col_body.push_back(b);
        for (unsigned long long k : keys) {
            const int c0 = (int)(k >> 32), c1 = (int)(unsigned)k;
            if (omap[c0] >= 0 && omap[c1] >= 0) continue;
            const int ob0 = F->h_col_body[c0], ob1 = F->h_col_body[c1];
            const int os = (int)(std::upper_bound(F->h_scene_body.begin(), F->h_scene_body.end(), ob0) - F->h_scene_body.begin()) - 1;
            if (os < 0 || new_scene[os] < 0) continue;
            psx_trigger_event e{};
            e.frame = (int)F->frames_run;
            e.kind = PSX_TRIGGER_EXIT;
            e.scene = new_scene[os];
            e.body0 = omap[c0] >= 0 ? new_col_body[omap[c0]] : -1;
            e.collider0 = F->h_col_local[c0];
            e.body1 = omap[c1] >= 0 ? new_col_body[omap[c1]] : -1;
            e.collider1 = F->h_col_local[c1];
            e.entity0 = F->h_entity[ob0];
            e.entity1 = F->h_entity[ob1];
            vanished.push_back(e);
        }
    }
    psx_world* W = nullptr;
    PSX_TRY(create_world(scenes, n_scenes, F->opts_used, F->frames_run, colors, &W));
    W->trig_vanished = F->trig_vanished;
    W->trig_vanished.insert(W->trig_vanished.end(), vanished.begin(), vanished.end());
    W->trig_pending = F->trig_pending;   // delivered events the caller has not drained yet stay queued
    psx_status st = apply_launch(W, current_launch(F));
    W->wait_limit = F->wait_limit;
    DevArray<int> d_cmap, d_jmap, d_omap;
    if (st == PSX_OK) st = d_cmap.upload(cmap);
    if (st == PSX_OK) st = d_jmap.upload(jmap);
    if (st == PSX_OK) st = d_omap.upload(omap);
    if (st != PSX_OK) { psx_world_destroy(W); return st; }
    cudaStream_t s = W->stream;
    if (!cmap.empty())
        k_carry_bounds<<<((int)cmap.size() + 255) / 256, 256, 0, s>>>(W->w.aabb_min, W->w.aabb_max, F->w.aabb_min, F->w.aabb_max,
                                                                      d_cmap.p, (int)cmap.size());
    if (!jmap.empty()) k_carry_joints<<<((int)jmap.size() + 127) / 128, 128, 0, s>>>(W->w.joints, F->w.joints, d_jmap.p, (int)jmap.size());
    // the old world's table written by its last frame is the one its next frame would
    // read; the new world's first frame reads cache_b (its parity starts at 0)
    int parity = 0;
    cudaError_t e = cudaMemcpy(&parity, F->f.cache_parity, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && F->w.n_colliders) {
        const CacheEntry* src = parity ? F->f.cache_a : F->f.cache_b;
        k_carry_cache<<<(F->f.cache_cap + 255) / 256, 256, 0, s>>>(src, F->f.cache_cap, F->w.key_cbits, d_omap.p, W->f.cache_b,
                                                                   W->f.cache_cap, W->w.key_cbits, W->w.err);
    }
    if (e == cudaSuccess && F->f.trig_cap) {
        if (!W->f.trig_cap) st = alloc_triggers(W);
        if (st == PSX_OK) k_carry_triggers<<<152, 128, 0, s>>>(F->f, W->f, d_omap.p, W->w.err);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = fail(PSX_ERR_CUDA, cudaGetErrorString(e));
    if (st == PSX_OK) st = check_err(W);
    if (st != PSX_OK) { psx_world_destroy(W); return st; }
    *out = W;
    return PSX_OK;
}

}  // extern "C"
