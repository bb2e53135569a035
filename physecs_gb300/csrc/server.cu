// server.cu — serving form: continuous batching of independent scene requests.
//
// A server is one world of fixed slots in size classes.  A request (one scene and a
// number of frames) is admitted into a free slot of the smallest class that holds it;
// every tick advances all running slots by one frame in one batched frame; a slot
// whose request has run its frames stops and keeps its final state until the caller
// reads and releases it.  Slots that are not running are skipped by the broadphase
// traversal and the solver (World::scene_active).
//
// A request's results do not depend on which slot it lands in or on the other
// requests in flight: the broadphase order, manifold order and contact colouring
// of a scene depend on that scene alone, and the unused bodies of a slot are
// static, kinematic or disabled.  Trigger events (opts.triggers) are decoded per request
// at the end of each tick: the slot's flags keep a fresh request from seeing the last
// occupant's trigger pairs and drop the exits of a finished one.  Requests carry no
// joints and no triangle meshes
// (the serving workload's scenes have neither); their convex meshes must be meshes
// of the server's pool, matched by content.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <tuple>
#include <vector>
#include "runtime.cuh"

using namespace psx;
using namespace psx::rt;

namespace {

// What decodes a request's trigger events: each slot collider's request body and index
// within that body, each request body's entity, and the world frame of its first tick.
struct ReqMap {
    std::vector<int> col_body, col_local;
    std::vector<uint32_t> entity;
    long long frame0 = 0;
};

struct Slot {
    long long first_tick = 0;                     // the first tick that simulates the request
    int cls = 0, scene = 0;
    int body0 = 0, col0 = 0, dyn0 = 0, cap = 0;   // world ranges: cap + 1 bodies, colliders and dynamic entries
    int state = 0;                                // 0 free, 1 running, 2 finished
    int frames_left = 0;
    int n_bodies = 0;
    std::vector<int> dyn_of;                      // request body -> world dynamic index or -1
    ReqMap map;                                   // the request's trigger-event decoding
};

uint64_t fnv(uint64_t h, const void* p, size_t n) {
    const unsigned char* c = (const unsigned char*)p;
    for (size_t i = 0; i < n; ++i) { h ^= c[i]; h *= 1099511628211ull; }
    return h;
}

uint64_t mesh_hash(const psx_scene_desc& d, int m) {
    uint64_t h = 1469598103934665603ull;
    int v0 = d.convex_vert_start[m], v1 = d.convex_vert_start[m + 1];
    int f0 = d.convex_face_start[m], f1 = d.convex_face_start[m + 1];
    h = fnv(h, d.convex_verts + 3 * v0, sizeof(float) * 3 * (v1 - v0));
    for (int f = f0; f < f1; ++f) {
        int a = d.face_index_start[f], b = d.face_index_start[f + 1];
        int cnt = b - a;
        h = fnv(h, &cnt, sizeof cnt);
        h = fnv(h, d.face_indices + a, sizeof(uint32_t) * cnt);
        h = fnv(h, d.face_normal + 3 * f, sizeof(float) * 3);
        h = fnv(h, d.face_centroid + 3 * f, sizeof(float) * 3);
    }
    return h;
}

// Template scene of one slot: cap + 1 kinematic bodies with one disabled sphere each.
struct TemplateScene {
    std::vector<uint32_t> entity, flags;
    std::vector<float> pos, quat, vel, ang, inv_mass, com, inv_inertia;
    std::vector<int32_t> collider_start, col_type, col_mesh;
    std::vector<float> col_pos, col_quat, col_params, col_material;
    std::vector<uint8_t> col_enable;
    void make(int n, psx_scene_desc& d) {
        entity.resize(n); flags.assign(n, PSX_BODY_DYNAMIC | PSX_BODY_KINEMATIC);
        pos.assign(3 * n, 0.f); quat.assign(4 * n, 0.f); vel.assign(3 * n, 0.f); ang.assign(3 * n, 0.f);
        inv_mass.assign(n, 0.f); com.assign(3 * n, 0.f); inv_inertia.assign(9 * n, 0.f);
        collider_start.resize(n + 1); col_type.assign(n, PSX_SPHERE); col_mesh.assign(n, -1);
        col_pos.assign(3 * n, 0.f); col_quat.assign(4 * n, 0.f); col_params.assign(4 * n, 0.f);
        col_material.assign(3 * n, 0.f); col_enable.assign(n, 0);
        for (int i = 0; i < n; ++i) {
            entity[i] = (uint32_t)i;
            quat[4 * i + 3] = 1.f;
            col_quat[4 * i + 3] = 1.f;
            col_params[4 * i] = 0.1f;
            collider_start[i] = i;
        }
        collider_start[n] = n;
        std::memset(&d, 0, sizeof d);
        d.n_bodies = n; d.n_colliders = n;
        d.entity = entity.data(); d.flags = flags.data(); d.pos = pos.data(); d.quat = quat.data();
        d.vel = vel.data(); d.ang_vel = ang.data(); d.inv_mass = inv_mass.data(); d.com = com.data();
        d.inv_inertia = inv_inertia.data(); d.collider_start = collider_start.data(); d.col_type = col_type.data();
        d.col_mesh = col_mesh.data(); d.col_pos = col_pos.data(); d.col_quat = col_quat.data();
        d.col_params = col_params.data(); d.col_material = col_material.data(); d.col_enable_sim = col_enable.data();
        d.num_substeps = 1; d.num_iterations = 1; d.gravity = 9.81f;
    }
};

}  // namespace

// Host staging of admitted requests: their arrays are packed into pinned memory at
// admission and copied to the device at the start of the next tick.  Two stages
// alternate so that packing never waits for the copies of the tick in flight.
struct Upload {
    void* dst;
    size_t src;   // offset in the stage
    size_t bytes;
};
struct Stage {
    char* pin = nullptr;
    size_t cap = 0, used = 0;
    std::vector<Upload> ups;
    std::vector<int2> aabb;          // collider ranges that need creation bounds
    cudaEvent_t copied = nullptr;    // recorded after the stage's copies
    bool pending = false;            // copies issued, completion not yet observed
};

struct psx_server {
    psx_world* W = nullptr;
    std::vector<Slot> slots;
    std::vector<int> class_cap;
    std::vector<std::vector<int>> free_slots;   // per class
    std::vector<uint64_t> pool_hash;            // convex pool: world mesh index = position
    int* d_active = nullptr;
    int* d_fresh = nullptr;
    std::vector<int> h_active;
    bool active_dirty = true;
    long long body_frames = 0;                  // simulated-body frames run so far
    int64_t device_bytes = 0;                   // device memory of the slots' world and the flags
    // admission packing (host) and staging (pinned)
    std::vector<float4> pos, quat, vel, ang, com, invI, cpos, cquat, cpar, cmat;
    std::vector<int4> info, cinfo;
    std::vector<int> dynb;
    Stage stage[2];
    int cur = 0;
    // tick state
    long long ticks_begun = 0;
    bool in_flight = false;
    cudaEvent_t tick_done = nullptr;
    bool profile = false;            // stage events around each tick (ticks run eagerly)
    cudaEvent_t prof[7] = {};        // tick start, then the frame's six stage events
    int* pin_active = nullptr;       // pinned mirror of h_active for the flag copy
    int* pin_err = nullptr;          // device error word of the last tick
    // trigger events (opts.triggers): decoded at the end of each tick
    bool triggers = false;
    int* pin_nevt = nullptr;                     // the device log's count after the last tick
    std::vector<int> slot_col0;                  // first world collider of each slot, ascending
    std::vector<ReqMap> retired;                 // per slot: the request that a re-admission
                                                 // replaced while a tick it ran was in flight
    std::vector<psx_trigger_event> trig_pending;
    int64_t trig_lost = 0;
    // reads of finished requests run on their own stream, beside the next tick
    cudaStream_t read_stream = nullptr;
    float4* read_pin = nullptr;
    size_t read_cap = 0;
    ~psx_server() {
        if (W) cudaStreamSynchronize(W->stream);
        if (read_stream) { cudaStreamSynchronize(read_stream); cudaStreamDestroy(read_stream); }
        for (Stage& st : stage) {
            if (st.pin) cudaFreeHost(st.pin);
            if (st.copied) cudaEventDestroy(st.copied);
        }
        if (tick_done) cudaEventDestroy(tick_done);
        for (cudaEvent_t e : prof) if (e) cudaEventDestroy(e);
        if (pin_active) cudaFreeHost(pin_active);
        if (pin_err) cudaFreeHost(pin_err);
        if (pin_nevt) cudaFreeHost(pin_nevt);
        if (read_pin) cudaFreeHost(read_pin);
        if (d_active) cudaFree(d_active);
        if (d_fresh) cudaFree(d_fresh);
        delete W;
    }
};

extern "C" {

PSX_API psx_status psx_server_create(const psx_server_opts* o, psx_server** out) {
    if (!o || !out || o->n_classes <= 0 || !o->class_bodies || !o->class_slots)
        return fail(PSX_ERR_INVALID_ARG, "psx_server_create: bad arguments");
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) return fail(PSX_ERR_CUDA, "no CUDA device");
    if (o->device < 0 || o->device >= dev_count) return fail(PSX_ERR_INVALID_ARG, "device ordinal");
    PSX_CUDA(cudaSetDevice(o->device));
    psx_server* S = new psx_server();
    int n_slots = 0;
    for (int c = 0; c < o->n_classes; ++c) {
        if (o->class_bodies[c] < 1 || o->class_slots[c] < 0) { delete S; return fail(PSX_ERR_INVALID_ARG, "slot class"); }
        if (c && o->class_bodies[c] <= o->class_bodies[c - 1]) { delete S; return fail(PSX_ERR_INVALID_ARG, "slot classes must grow"); }
        n_slots += o->class_slots[c];
    }
    if (n_slots == 0) { delete S; return fail(PSX_ERR_INVALID_ARG, "no slots"); }
    // one template scene per slot; the mesh pool rides on the first
    std::vector<TemplateScene> ts(n_slots);
    std::vector<psx_scene_desc> descs(n_slots);
    S->free_slots.resize(o->n_classes);
    int k = 0, body = 0, col = 0, dyn = 0;
    for (int c = 0; c < o->n_classes; ++c) {
        S->class_cap.push_back(o->class_bodies[c]);
        for (int i = 0; i < o->class_slots[c]; ++i, ++k) {
            int cap = o->class_bodies[c];
            ts[k].make(cap + 1, descs[k]);
            Slot sl;
            sl.cls = c; sl.scene = k; sl.cap = cap;
            sl.body0 = body; sl.col0 = col; sl.dyn0 = dyn;
            body += cap + 1; col += cap + 1; dyn += cap + 1;
            S->slots.push_back(sl);
        }
        for (int i = o->class_slots[c] - 1; i >= 0; --i) S->free_slots[c].push_back(k - o->class_slots[c] + i);
    }
    if (o->mesh_pool) {
        const psx_scene_desc& p = *o->mesh_pool;
        descs[0].n_convex = p.n_convex;
        descs[0].convex_vert_start = p.convex_vert_start; descs[0].convex_verts = p.convex_verts;
        descs[0].convex_face_start = p.convex_face_start; descs[0].face_index_start = p.face_index_start;
        descs[0].face_indices = p.face_indices; descs[0].face_normal = p.face_normal;
        descs[0].face_centroid = p.face_centroid;
        for (int m = 0; m < p.n_convex; ++m) S->pool_hash.push_back(mesh_hash(p, m));
    }
    psx_world_opts wo{};
    // piled requests reach about 40 partners a collider: room for 72 keeps their pairs
    // from the broadphase's one walk (4.5 x the pairs per collider)
    wo.pairs_per_collider = o->pairs_per_collider ? o->pairs_per_collider : 16;
    wo.manifolds_per_collider = o->manifolds_per_collider;
    wo.block_scene_max_dyn = 1 << 30;
    wo.use_graph = (o->eager || o->profile) ? 0 : 1;   // a tick is the same fixed kernel sequence every time
    wo.device = o->device;
    // a tick waits for its slowest pair: without shapes from the caller, EPA runs with the
    // full polytope directly (the small-polytope pass serves throughput, and a pair that
    // outgrows it is solved twice)
    psx_launch_config latency{};
    latency.epa_full_only = 1;
    latency.epa_lanes = 16;   // not the lane-per-pair pass: its one block per SM suits full frames
    wo.launch = o->launch ? o->launch : &latency;
    psx_world* W = nullptr;
    psx_status st = psx_world_create(descs.data(), n_slots, &wo, &W);
    if (st != PSX_OK) { delete S; return st; }
    S->W = W;
    // trigger sets and the event log; a trigger pair's events are kept or dropped by its
    // slot's running and fresh flags (k_trigger_enter / k_trigger_exit)
    if (o->triggers && (st = alloc_triggers(W)) != PSX_OK) { delete S; return st; }
    if (cudaMalloc(&S->d_active, sizeof(int) * n_slots) != cudaSuccess ||
        cudaMalloc(&S->d_fresh, sizeof(int) * n_slots) != cudaSuccess) {
        delete S;
        return fail(PSX_ERR_OUT_OF_MEMORY, "server flags");
    }
    cudaMemset(S->d_active, 0, sizeof(int) * n_slots);
    cudaMemset(S->d_fresh, 0, sizeof(int) * n_slots);
    S->device_bytes = (int64_t)W->device_bytes + 2 * (int64_t)sizeof(int) * n_slots;
    if (o->hbm_budget > 0 && S->device_bytes > o->hbm_budget) {
        char buf[200];
        std::snprintf(buf, sizeof buf, "psx_server_create: the slots need %lld device bytes, above the budget of %lld",
                      (long long)S->device_bytes, (long long)o->hbm_budget);
        delete S;
        return fail(PSX_ERR_OUT_OF_MEMORY, buf);
    }
    S->h_active.assign(n_slots, 0);
    W->w.scene_active = S->d_active;
    W->w.scene_fresh = S->d_fresh;
    if (cudaMallocHost(&S->pin_active, sizeof(int) * n_slots) != cudaSuccess ||
        cudaMallocHost(&S->pin_err, sizeof(int)) != cudaSuccess ||
        cudaEventCreateWithFlags(&S->tick_done, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&S->stage[0].copied, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&S->stage[1].copied, cudaEventDisableTiming) != cudaSuccess ||
        cudaStreamCreateWithFlags(&S->read_stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete S;
        return fail(PSX_ERR_OUT_OF_MEMORY, "server host staging");
    }
    *S->pin_err = 0;
    if (o->triggers) {
        if (cudaMallocHost(&S->pin_nevt, sizeof(int)) != cudaSuccess) {
            delete S;
            return fail(PSX_ERR_OUT_OF_MEMORY, "server host staging");
        }
        *S->pin_nevt = 0;
        S->triggers = true;
        for (const Slot& sl : S->slots) S->slot_col0.push_back(sl.col0);
        S->retired.resize(n_slots);
    }
    S->profile = o->profile != 0;
    for (int i = 0; S->profile && i < 7; ++i)
        if (cudaEventCreate(&S->prof[i]) != cudaSuccess) { delete S; return fail(PSX_ERR_CUDA, "server profile events"); }
    PSX_CUDA(cudaDeviceSynchronize());
    *out = S;
    return PSX_OK;
}

PSX_API psx_status psx_server_destroy(psx_server* S) {
    if (!S) return fail(PSX_ERR_INVALID_ARG, "null server");
    cudaSetDevice(S->W->device);
    delete S;
    return PSX_OK;
}

PSX_API psx_status psx_server_admit(psx_server* S, const psx_scene_desc* d, int32_t frames, float dt, int32_t* slot_out) {
    if (!S || !d || !slot_out || frames <= 0 || !(dt > 0.f)) return fail(PSX_ERR_INVALID_ARG, "psx_server_admit: bad arguments");
    PSX_CUDA(cudaSetDevice(S->W->device));
    PSX_TRY(validate(*d));
    if (d->n_joints) return fail(PSX_ERR_INVALID_ARG, "serving requests carry no joints");
    if (d->n_trimesh) return fail(PSX_ERR_INVALID_ARG, "serving requests carry no triangle meshes");
    std::vector<int> mesh_map(d->n_convex, -1);
    for (int m = 0; m < d->n_convex; ++m) {
        uint64_t h = mesh_hash(*d, m);
        for (size_t q = 0; q < S->pool_hash.size(); ++q) if (S->pool_hash[q] == h) { mesh_map[m] = (int)q; break; }
    }
    for (int c = 0; c < d->n_colliders; ++c)
        if (d->col_type[c] == PSX_CONVEX_MESH && mesh_map[d->col_mesh[c]] < 0)
            return fail(PSX_ERR_INVALID_ARG, "convex mesh not in the server's pool");
    int need = std::max(d->n_bodies, d->n_colliders - 1);
    int cls = -1;
    for (size_t c = 0; c < S->class_cap.size(); ++c) {
        if (S->class_cap[c] >= need && !S->free_slots[c].empty()) { cls = (int)c; break; }
    }
    if (cls < 0) {
        bool fits = need <= S->class_cap.back();
        return fail(PSX_ERR_CAPACITY, fits ? "no free slot for this request size" : "request larger than the largest slot class");
    }
    int si = S->free_slots[cls].back();
    S->free_slots[cls].pop_back();
    Slot& sl = S->slots[si];
    const int cap = sl.cap, nb = cap + 1;
    const int inert = sl.body0 + cap;   // kinematic body that absorbs unused dynamic entries
    S->pos.assign(nb, f4(0, 0, 0)); S->quat.assign(nb, f4(0, 0, 0, 1));
    S->info.assign(nb, make_int4(0, 0, -1, sl.scene));
    S->vel.assign(nb, f4(0, 0, 0)); S->ang.assign(nb, f4(0, 0, 0)); S->com.assign(nb, f4(0, 0, 0));
    S->invI.assign(3 * nb, f4(0, 0, 0)); S->dynb.assign(nb, inert);
    S->cpos.assign(nb, f4(0, 0, 0)); S->cquat.assign(nb, f4(0, 0, 0, 1)); S->cpar.assign(nb, f4(0.1f, 0, 0));
    S->cmat.assign(nb, f4(0, 0, 0)); S->cinfo.assign(nb, make_int4(inert, PSX_SPHERE, -1, 0));
    sl.dyn_of.assign(d->n_bodies, -1);
    if (S->triggers) {
        // a tick in flight may have run the slot's previous request: its events are
        // decoded at that tick's end with the map it ran under (a request admitted and
        // released again within the same tick never ran, and its map is simply replaced)
        if (S->in_flight && sl.first_tick <= S->ticks_begun) std::swap(S->retired[si], sl.map);
        ReqMap& m = sl.map;
        m.col_body.resize(d->n_colliders);
        m.col_local.resize(d->n_colliders);
        m.entity.assign(d->entity, d->entity + d->n_bodies);
        for (int b = 0; b < d->n_bodies; ++b)
            for (int c = d->collider_start[b]; c < d->collider_start[b + 1]; ++c) {
                m.col_body[c] = b;
                m.col_local[c] = c - d->collider_start[b];
            }
        m.frame0 = S->W->frames_run;   // the frame of the next tick: every tick begun has counted its frame
    }
    int nd = 0, nsim = 0;
    for (int b = 0; b < d->n_bodies; ++b) {
        uint32_t fl = d->flags[b];
        bool dynb = fl & PSX_BODY_DYNAMIC;
        bool sim = dynb && !(fl & PSX_BODY_KINEMATIC);
        S->pos[b] = f4(d->pos[3 * b], d->pos[3 * b + 1], d->pos[3 * b + 2]);
        S->quat[b] = f4(d->quat[4 * b], d->quat[4 * b + 1], d->quat[4 * b + 2], d->quat[4 * b + 3]);
        int di = -1;
        if (dynb) {
            di = sl.dyn0 + nd;
            S->dynb[nd] = sl.body0 + b;
            S->vel[nd] = f4(d->vel[3 * b], d->vel[3 * b + 1], d->vel[3 * b + 2]);
            S->ang[nd] = f4(d->ang_vel[3 * b], d->ang_vel[3 * b + 1], d->ang_vel[3 * b + 2]);
            S->com[nd] = f4(d->com[3 * b], d->com[3 * b + 1], d->com[3 * b + 2], d->inv_mass[b]);
            for (int q = 0; q < 3; ++q)
                S->invI[3 * nd + q] = f4(d->inv_inertia[9 * b + 3 * q], d->inv_inertia[9 * b + 3 * q + 1], d->inv_inertia[9 * b + 3 * q + 2]);
            sl.dyn_of[b] = di;
            ++nd;
        }
        if (sim) ++nsim;
        S->info[b] = make_int4((int)d->entity[b], (int)fl, di, sl.scene);
        for (int c = d->collider_start[b]; c < d->collider_start[b + 1]; ++c) {
            int t = d->col_type[c];
            int flags = 0;
            if (!d->col_enable_sim || d->col_enable_sim[c]) flags |= COL_ENABLE;
            if (d->col_is_trigger && d->col_is_trigger[c]) flags |= COL_TRIGGER;
            if (sim) flags |= COL_DYNAMIC;
            S->cinfo[c] = make_int4(sl.body0 + b, t, t == PSX_CONVEX_MESH ? mesh_map[d->col_mesh[c]] : -1, flags);
            S->cpos[c] = f4(d->col_pos[3 * c], d->col_pos[3 * c + 1], d->col_pos[3 * c + 2]);
            S->cquat[c] = f4(d->col_quat[4 * c], d->col_quat[4 * c + 1], d->col_quat[4 * c + 2], d->col_quat[4 * c + 3]);
            S->cpar[c] = f4(d->col_params[4 * c], d->col_params[4 * c + 1], d->col_params[4 * c + 2], d->col_params[4 * c + 3]);
            S->cmat[c] = f4(d->col_material[3 * c], d->col_material[3 * c + 1], d->col_material[3 * c + 2],
                            bits_as_float(d->col_data ? d->col_data[c] : 0));
        }
    }
    S->info[cap] = make_int4(-1, PSX_BODY_DYNAMIC | PSX_BODY_KINEMATIC, sl.dyn0 + nd, sl.scene);
    S->dynb[nd] = inert;   // the inert body's own dynamic entry (and every unused one) points at it
    World& w = S->W->w;
    // stage the slot's arrays; they reach the device at the start of the next tick
    Stage& stg = S->stage[S->cur];
    if (stg.pending) {
        PSX_CUDA(cudaEventSynchronize(stg.copied));
        stg.pending = false;
        stg.used = 0;
    }
    const size_t stage_need = stg.used + (size_t)nb * (16 * sizeof(float4)) + 4 * sizeof(float4);
    if (stage_need > stg.cap) {
        size_t new_cap = std::max(stage_need, 2 * stg.cap);
        char* np = nullptr;
        PSX_CUDA(cudaMallocHost(&np, new_cap));
        if (stg.used) std::memcpy(np, stg.pin, stg.used);
        if (stg.pin) cudaFreeHost(stg.pin);
        stg.pin = np;
        stg.cap = new_cap;
    }
    auto up = [&](auto* dst, const auto* src, size_t count, int off) {
        size_t bytes = count * sizeof(src[0]);
        std::memcpy(stg.pin + stg.used, src, bytes);
        stg.ups.push_back(Upload{(void*)(dst + off), stg.used, bytes});
        stg.used += (bytes + 15) / 16 * 16;
    };
    up(w.pos, S->pos.data(), S->pos.size(), sl.body0);
    up(w.quat, S->quat.data(), S->quat.size(), sl.body0);
    up(w.info, S->info.data(), S->info.size(), sl.body0);
    up(w.dyn_body, S->dynb.data(), S->dynb.size(), sl.dyn0);
    up(w.vel, S->vel.data(), S->vel.size(), sl.dyn0);
    up(w.ang, S->ang.data(), S->ang.size(), sl.dyn0);
    up(w.com, S->com.data(), S->com.size(), sl.dyn0);
    up(w.invI, S->invI.data(), S->invI.size(), 3 * sl.dyn0);
    up(w.col_info, S->cinfo.data(), S->cinfo.size(), sl.col0);
    up(w.col_pos, S->cpos.data(), S->cpos.size(), sl.col0);
    up(w.col_quat, S->cquat.data(), S->cquat.size(), sl.col0);
    up(w.col_params, S->cpar.data(), S->cpar.size(), sl.col0);
    up(w.col_mat, S->cmat.data(), S->cmat.size(), sl.col0);
    S->W->h_knobs[sl.scene] = f4((float)d->num_substeps, (float)d->num_iterations, d->gravity, dt);
    up(w.knobs, &S->W->h_knobs[sl.scene], 1, sl.scene);
    const int one = 1;   // first frame: no cached contacts from the slot's previous request
    up(S->d_fresh, &one, 1, sl.scene);
    stg.aabb.push_back(make_int2(sl.col0, sl.col0 + nb));
    sl.first_tick = S->ticks_begun + 1;
    sl.state = 1;
    sl.frames_left = frames;
    sl.n_bodies = d->n_bodies;
    S->h_active[sl.scene] = 1;
    S->active_dirty = true;
    (void)nsim;
    *slot_out = si;
    return PSX_OK;
}

PSX_API psx_status psx_server_tick_begin(psx_server* S) {
    if (!S) return fail(PSX_ERR_INVALID_ARG, "null server");
    if (S->in_flight) return fail(PSX_ERR_INVALID_ARG, "psx_server_tick_begin: a tick is in flight");
    psx_world* W = S->W;
    PSX_CUDA(cudaSetDevice(W->device));
    cudaStream_t st = W->stream;
    Stage& stg = S->stage[S->cur];
    if (S->profile) PSX_CUDA(cudaEventRecord(S->prof[0], st));
    if (!stg.ups.empty()) {
        for (const Upload& u : stg.ups)
            PSX_CUDA(cudaMemcpyAsync(u.dst, stg.pin + u.src, u.bytes, cudaMemcpyHostToDevice, st));
        // creation bounds carry no margin (src/Physecs.cpp:25-37)
        for (int2 r : stg.aabb) launch_aabb_range(W->w, r.x, r.y, 0, st);
        PSX_CUDA(cudaEventRecord(stg.copied, st));
        stg.pending = true;   // the pinned bytes stay untouched until the copies are seen complete
        stg.ups.clear();
        stg.aabb.clear();
        S->cur ^= 1;
    }
    if (S->active_dirty) {
        std::memcpy(S->pin_active, S->h_active.data(), sizeof(int) * S->h_active.size());
        PSX_CUDA(cudaMemcpyAsync(S->d_active, S->pin_active, sizeof(int) * S->h_active.size(), cudaMemcpyHostToDevice, st));
        S->active_dirty = false;
    }
    ++S->ticks_begun;
    if (S->profile) {
        W->frame_kernels = queue_frame(W, S->prof + 1);
        ++W->frames_run;
    } else {
        PSX_TRY(run_frame(W));
    }
    PSX_CUDA(cudaMemsetAsync(S->d_fresh, 0, sizeof(int) * S->h_active.size(), st));
    PSX_CUDA(cudaMemcpyAsync(S->pin_err, W->w.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (S->triggers) PSX_CUDA(cudaMemcpyAsync(S->pin_nevt, W->f.n_evt, sizeof(int), cudaMemcpyDeviceToHost, st));
    PSX_CUDA(cudaEventRecord(S->tick_done, st));
    PSX_CUDA(cudaGetLastError());
    S->in_flight = true;
    return PSX_OK;
}

}  // extern "C"

namespace {

// The tick just ended: its raw events (world frame, kind, world colliders) become request
// events.  A slot's colliders are a fixed range of the world's, so the range gives the
// slot; the request that ran there in this tick gives bodies, colliders and entities.
psx_status drain_triggers(psx_server* S) {
    const int n = *S->pin_nevt;
    if (!n) return PSX_OK;
    psx_world* W = S->W;
    const FrameBuf& f = W->f;
    cudaStream_t st = W->stream;
    const int kept = std::min(n, f.evt_cap);
    std::vector<int4> ev(kept);
    PSX_CUDA(cudaMemcpyAsync(ev.data(), f.trig_evt, sizeof(int4) * kept, cudaMemcpyDeviceToHost, st));
    PSX_CUDA(cudaMemsetAsync(f.n_evt, 0, sizeof(int), st));
    PSX_CUDA(cudaStreamSynchronize(st));
    S->trig_lost += n - kept;
    const long long tick = S->ticks_begun;
    std::vector<psx_trigger_event> batch;
    batch.reserve(kept);
    for (const int4& r : ev) {
        const int si = (int)(std::upper_bound(S->slot_col0.begin(), S->slot_col0.end(), r.z) - S->slot_col0.begin()) - 1;
        if (si < 0) continue;
        const Slot& sl = S->slots[si];
        const ReqMap& m = sl.first_tick <= tick ? sl.map : S->retired[si];
        const int c0 = r.z - sl.col0, c1 = r.w - sl.col0;
        if (c0 < 0 || c1 < 0 || c0 >= (int)m.col_body.size() || c1 >= (int)m.col_body.size()) continue;
        psx_trigger_event e{};
        e.frame = (int)(r.x - m.frame0);
        e.kind = r.y;
        e.scene = si;
        e.body0 = m.col_body[c0];
        e.collider0 = m.col_local[c0];
        e.body1 = m.col_body[c1];
        e.collider1 = m.col_local[c1];
        e.entity0 = m.entity[e.body0];
        e.entity1 = m.entity[e.body1];
        batch.push_back(e);
    }
    // one tick: enter before exit, then slot, bodies and colliders, as a world orders a frame's
    auto key = [](const psx_trigger_event& e) {
        return std::make_tuple(e.kind, e.scene, e.body0, e.collider0, e.body1, e.collider1);
    };
    std::sort(batch.begin(), batch.end(), [&](const psx_trigger_event& a, const psx_trigger_event& b) { return key(a) < key(b); });
    S->trig_pending.insert(S->trig_pending.end(), batch.begin(), batch.end());
    return PSX_OK;
}

}  // namespace

extern "C" {

PSX_API psx_status psx_server_tick_end(psx_server* S, int32_t* done, int32_t cap, int32_t* n_done) {
    if (!S) return fail(PSX_ERR_INVALID_ARG, "null server");
    if (!S->in_flight) return fail(PSX_ERR_INVALID_ARG, "psx_server_tick_end: no tick in flight");
    PSX_CUDA(cudaSetDevice(S->W->device));
    PSX_CUDA(cudaEventSynchronize(S->tick_done));
    S->in_flight = false;
    if (int e = *S->pin_err) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "device error bits 0x%x", e);
        return fail((e & ERR_BARRIER_TIMEOUT) ? PSX_ERR_TIMEOUT : PSX_ERR_CAPACITY, buf);
    }
    if (S->triggers) PSX_TRY(drain_triggers(S));
    int nd = 0;
    for (size_t i = 0; i < S->slots.size(); ++i) {
        Slot& sl = S->slots[i];
        if (sl.state != 1 || sl.first_tick > S->ticks_begun) continue;
        S->body_frames += sl.n_bodies;
        if (--sl.frames_left == 0) {
            sl.state = 2;
            S->h_active[sl.scene] = 0;
            S->active_dirty = true;
            if (done && nd < cap) done[nd] = (int32_t)i;
            ++nd;
        }
    }
    if (n_done) *n_done = nd;
    return PSX_OK;
}

PSX_API psx_status psx_server_tick(psx_server* S, int32_t* done, int32_t cap, int32_t* n_done) {
    PSX_TRY(psx_server_tick_begin(S));
    return psx_server_tick_end(S, done, cap, n_done);
}

PSX_API psx_status psx_server_read(psx_server* S, int32_t slot, float* pos, float* quat, float* vel, float* ang_vel) {
    if (!S || slot < 0 || slot >= (int)S->slots.size()) return fail(PSX_ERR_INVALID_ARG, "psx_server_read: slot");
    Slot& sl = S->slots[slot];
    if (sl.state == 0) return fail(PSX_ERR_INVALID_ARG, "psx_server_read: slot is free");
    psx_world* W = S->W;
    PSX_CUDA(cudaSetDevice(W->device));
    // a finished request is not simulated any more and can be read beside a tick in
    // flight; a running one is read after that tick
    if (sl.state == 1 && S->in_flight) PSX_CUDA(cudaEventSynchronize(S->tick_done));
    int nb = sl.n_bodies, nd = sl.cap + 1;
    size_t n4 = 2 * (size_t)nb + 2 * (size_t)nd;
    if (S->read_cap < n4) {
        if (S->read_pin) cudaFreeHost(S->read_pin);
        S->read_pin = nullptr;
        S->read_cap = 0;
        PSX_CUDA(cudaMallocHost(&S->read_pin, n4 * sizeof(float4)));
        S->read_cap = n4;
    }
    float4 *hp = S->read_pin, *hq = hp + nb, *hv = hq + nb, *ha = hv + nd;
    const World& w = W->w;
    cudaStream_t rs = S->read_stream;
    PSX_CUDA(cudaMemcpyAsync(hp, w.pos + sl.body0, nb * sizeof(float4), cudaMemcpyDeviceToHost, rs));
    PSX_CUDA(cudaMemcpyAsync(hq, w.quat + sl.body0, nb * sizeof(float4), cudaMemcpyDeviceToHost, rs));
    PSX_CUDA(cudaMemcpyAsync(hv, w.vel + sl.dyn0, nd * sizeof(float4), cudaMemcpyDeviceToHost, rs));
    PSX_CUDA(cudaMemcpyAsync(ha, w.ang + sl.dyn0, nd * sizeof(float4), cudaMemcpyDeviceToHost, rs));
    PSX_CUDA(cudaStreamSynchronize(rs));
    for (int b = 0; b < nb; ++b) {
        if (pos) { pos[3 * b] = hp[b].x; pos[3 * b + 1] = hp[b].y; pos[3 * b + 2] = hp[b].z; }
        if (quat) { quat[4 * b] = hq[b].x; quat[4 * b + 1] = hq[b].y; quat[4 * b + 2] = hq[b].z; quat[4 * b + 3] = hq[b].w; }
        int d = sl.dyn_of[b];
        float4 v = d >= 0 ? hv[d - sl.dyn0] : make_float4(0, 0, 0, 0), a = d >= 0 ? ha[d - sl.dyn0] : make_float4(0, 0, 0, 0);
        if (vel) { vel[3 * b] = v.x; vel[3 * b + 1] = v.y; vel[3 * b + 2] = v.z; }
        if (ang_vel) { ang_vel[3 * b] = a.x; ang_vel[3 * b + 1] = a.y; ang_vel[3 * b + 2] = a.z; }
    }
    return PSX_OK;
}

PSX_API psx_status psx_server_release(psx_server* S, int32_t slot) {
    if (!S || slot < 0 || slot >= (int)S->slots.size()) return fail(PSX_ERR_INVALID_ARG, "psx_server_release: slot");
    Slot& sl = S->slots[slot];
    if (sl.state == 0) return fail(PSX_ERR_INVALID_ARG, "psx_server_release: slot is free");
    if (sl.state == 1) { S->h_active[sl.scene] = 0; S->active_dirty = true; }
    sl.state = 0;
    S->free_slots[sl.cls].push_back(slot);
    return PSX_OK;
}

PSX_API psx_status psx_server_trigger_events(psx_server* S, psx_trigger_event* out, int32_t cap, int32_t* n_out,
                                             int64_t* n_lost) {
    if (!S || cap < 0 || (cap && !out) || !n_out) return fail(PSX_ERR_INVALID_ARG, "psx_server_trigger_events: bad arguments");
    if (!S->triggers) return fail(PSX_ERR_INVALID_ARG, "psx_server_trigger_events: the server was created without triggers");
    const int m = (int)std::min<size_t>((size_t)cap, S->trig_pending.size());
    std::copy(S->trig_pending.begin(), S->trig_pending.begin() + m, out);
    S->trig_pending.erase(S->trig_pending.begin(), S->trig_pending.begin() + m);
    *n_out = m;
    if (n_lost) { *n_lost = S->trig_lost; S->trig_lost = 0; }
    return PSX_OK;
}

PSX_API psx_world* psx_server_world(psx_server* S) { return S ? S->W : nullptr; }

PSX_API psx_status psx_server_device_bytes(psx_server* S, int64_t* out) {
    if (!S || !out) return fail(PSX_ERR_INVALID_ARG, "psx_server_device_bytes");
    *out = S->device_bytes;
    return PSX_OK;
}

PSX_API psx_status psx_server_tick_stages(psx_server* S, float* out) {
    if (!S || !out) return fail(PSX_ERR_INVALID_ARG, "psx_server_tick_stages");
    if (!S->profile) return fail(PSX_ERR_INVALID_ARG, "psx_server_tick_stages: the server was created without profile");
    if (S->in_flight || S->ticks_begun == 0) return fail(PSX_ERR_INVALID_ARG, "psx_server_tick_stages: no finished tick");
    PSX_CUDA(cudaSetDevice(S->W->device));
    for (int i = 0; i < 6; ++i) PSX_CUDA(cudaEventElapsedTime(&out[i], S->prof[i], S->prof[i + 1]));
    return PSX_OK;
}

PSX_API psx_status psx_server_stats(psx_server* S, int64_t* out) {
    if (!S || !out) return fail(PSX_ERR_INVALID_ARG, "psx_server_stats");
    int64_t running = 0, finished = 0, freec = 0, bodies = 0;
    for (const Slot& sl : S->slots) {
        if (sl.state == 1) { ++running; bodies += sl.n_bodies; }
        else if (sl.state == 2) ++finished;
        else ++freec;
    }
    out[0] = running; out[1] = finished; out[2] = freec; out[3] = bodies; out[4] = S->body_frames;
    out[5] = (int64_t)S->slots.size();
    return PSX_OK;
}

}  // extern "C"
