// runtime.cuh — host-side state of a world and the runtime helpers shared by the
// C-ABI entry points (world.cu) and the serving loop (server.cu).
#pragma once
#include <cuda_runtime.h>
#include <string>
#include <vector>
#include "frame.cuh"
#include "../../include/psx.h"

namespace psx {
namespace rt {
// records msg for psx_last_error_string() on the calling thread and returns s
psx_status fail(psx_status s, const std::string& msg);
inline float4 f4(float x, float y, float z, float w = 0.f) { return make_float4(x, y, z, w); }
inline int ilog2ceil(int v) { int b = 0; while ((1 << b) < v) ++b; return b; }
}  // namespace rt
}  // namespace psx

#define PSX_CUDA(call)                                                                     \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) return psx::rt::fail(PSX_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define PSX_TRY(expr)                       \
    do {                                    \
        psx_status s_ = (expr);             \
        if (s_ != PSX_OK) return s_;        \
    } while (0)

struct psx_world {
    psx::World w{};
    psx::FrameBuf f{};
    cudaStream_t stream = nullptr;
    std::vector<void*> allocs;
    int n_scenes = 0;
    int scene_bits = 0;     // bits of the scene index in the broadphase sort
    int scene_sort_pmax = 0; // > 0: per-scene sort in shared memory, scenes padded to this size
    std::vector<int> h_scene_body, h_scene_col, h_scene_dyn, h_scene_joint;
    std::vector<uint32_t> h_entity;        // per body
    std::vector<int> h_body_dyn;           // per body: global dyn index or -1
    std::vector<int> h_col_local;          // per collider: index within its body
    std::vector<int> h_col_body;           // per collider: world body index
    std::vector<int> h_scene_convex;       // per scene (+1): first world convex mesh
    std::vector<int> h_scene_trimesh;      // per scene (+1): first world triangle mesh
    std::vector<psx::TriMeshDev> h_trimesh;
    std::vector<int> h_col_trimesh;        // per collider: world triangle mesh, or -1
    std::vector<int> h_col_data;           // per collider: Collider::data
    std::vector<char> h_col_trig;          // per collider: Collider::isTrigger
    std::vector<int2> h_nc;                // non-colliding body pairs (lo, hi), sorted
    size_t nc_cap = 0;                     // device capacity of w.nc_pairs
    size_t filter_cap = 0;                 // device capacity of w.filter_table (bytes)
    // registry deltas
    std::vector<int> h_body_col;           // [n_bodies + 1] each body's first collider
    std::vector<int> h_body_flags;         // PSX_BODY_* as the device holds them
    std::vector<int> h_bj_start, h_bj;     // joints of each body (CSR)
    std::vector<char> h_body_overflow;     // 1: the body has a joint in the overflow colour
    std::vector<int> h_delta_slot;         // per body: its record in the batch being packed, or -1
    psx_body_delta* dpin = nullptr;        // pinned staging of a delta batch (records, then joint ids)
    size_t dpin_bytes = 0;
    char* ddev = nullptr;                  // device copy of the batch
    size_t ddev_bytes = 0;
    cudaEvent_t ev_delta = nullptr;        // the last batch's upload is done
    void* qbuf = nullptr;                  // scene-query staging on the device
    std::vector<psx_trigger_event> trig_pending;   // drained from the device, not yet delivered
    long long trig_lost = 0;               // events past the device log's capacity
    // exits of last-frame trigger pairs whose collider a topology change removed: due at
    // the end of the given frame (psx_world_recreate), delivered with that frame's events
    std::vector<psx_trigger_event> trig_vanished;
    size_t qbuf_bytes = 0;
    std::vector<int> block_scenes_h, grid_scenes_h;
    int* block_scenes = nullptr;
    int* grid_scenes = nullptr;
    int grid_blocks = 0;
    int solver_smem = 0;             // dynamic shared memory per solver block (bytes)
    psx::NarrowShape narrow{1, 8, 64, 16, 64, 16, 1, 0};   // launch shapes of the narrowphase kernels
    long long frames_run = 0;        // frames queued since creation
    int frame_kernels = 0;           // kernels in one frame
    int solver_smem_large = 0;       // the same for the 512-thread blocks of large scenes
    std::vector<int> large_scenes_h; // block scenes above 1024 dynamic bodies
    int* large_scenes = nullptr;
    std::vector<int> big_scenes_h;     // scenes above the block limit
    std::vector<int> cluster_scenes_h; // ... solved by a thread-block cluster each
    int* cluster_scenes = nullptr;     // (grid_scenes: the rest; both sized for every big scene)
    int large_mode = 0;                // 1: clusters where they fit, 2: the whole grid
    long long wait_limit = 0;          // polls of a grid-barrier wait before it gives up (0: the default)
    int large_nt = 512;                // threads per block of the scenes above 1024 dynamic bodies
    psx_world_opts opts_used{};        // the creation options (launch shapes: current_launch)
    std::vector<const int32_t*> forced_colors;   // per scene, while building: joint colours given by the caller
    // block scenes by solver block size (64, 128, 256 threads), each longest first
    std::vector<int> tier_h[3];
    int* tier_scenes[3] = {nullptr, nullptr, nullptr};
    int threads_min = 64;              // smallest solver block size in use
    cudaStream_t tier_stream[2] = {nullptr, nullptr};   // the 64- and 128-thread tiers
    cudaEvent_t ev_tfork = nullptr, ev_tjoin[2] = {nullptr, nullptr};
    cudaStream_t aux_stream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;     // solver: large scenes on the aux stream
    cudaEvent_t ev_fork2 = nullptr, ev_join2 = nullptr;   // narrowphase: convex pairs on the aux stream
    std::vector<float4> h_knobs;
    bool use_graph = false;
    cudaGraphExec_t graph = nullptr;
    float graph_dt = -1.f;
    bool knobs_dirty = true;
    float* bstage = nullptr;               // device staging of body state: pos, vel, ang_vel, 3 floats a body each
    size_t bstage_n = 0;
    int device = 0;
    long long launches = 0;          // kernels queued since creation
    int n_simulated = 0;             // dynamic, non-kinematic bodies
    std::vector<cudaEvent_t> events; // stage events of timed steps
    size_t device_bytes = 0;         // device memory held in allocs

    template <class T>
    psx_status alloc(T*& p, size_t n) {
        if (n == 0) n = 1;
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, n * sizeof(T));
        if (e != cudaSuccess) return psx::rt::fail(PSX_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        allocs.push_back(q);
        device_bytes += n * sizeof(T);
        p = (T*)q;
        return PSX_OK;
    }
    // copies v into p, allocating a larger buffer only when v outgrows *cap
    template <class T>
    psx_status upload_reuse(T*& p, size_t& cap, const std::vector<T>& v) {
        if (v.size() > cap || !p) {
            psx_status s = alloc(p, std::max<size_t>(v.size(), 2 * cap));
            if (s != PSX_OK) return s;
            cap = std::max<size_t>(v.size(), 2 * cap);
        }
        if (!v.empty()) PSX_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
        return PSX_OK;
    }
    template <class T>
    psx_status upload(T*& p, const std::vector<T>& v) {
        psx_status s = alloc(p, v.size());
        if (s != PSX_OK) return s;
        if (!v.empty()) PSX_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
        return PSX_OK;
    }
    ~psx_world() {
        for (cudaEvent_t e : events) cudaEventDestroy(e);
        if (graph) cudaGraphExecDestroy(graph);
        for (void* p : allocs) cudaFree(p);
        if (bstage) cudaFree(bstage);
        if (qbuf) cudaFree(qbuf);
        if (dpin) cudaFreeHost(dpin);
        if (ddev) cudaFree(ddev);
        if (ev_delta) cudaEventDestroy(ev_delta);
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_fork2) cudaEventDestroy(ev_fork2);
        if (ev_join2) cudaEventDestroy(ev_join2);
        if (ev_join) cudaEventDestroy(ev_join);
        if (aux_stream) cudaStreamDestroy(aux_stream);
        for (cudaStream_t t : tier_stream) if (t) cudaStreamDestroy(t);
        if (ev_tfork) cudaEventDestroy(ev_tfork);
        for (cudaEvent_t e : ev_tjoin) if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }
};


namespace psx {
namespace rt {
psx_status validate(const psx_scene_desc& d);
psx_status create_world(const psx_scene_desc* scenes, int n_scenes, psx_world_opts o, long long frames_run,
                        const std::vector<const int32_t*>& colors, psx_world** out);
// packs scenes into W's device buffers and computes the creation bounds
psx_status build_world(psx_world* W, const psx_scene_desc* scenes, int S, const psx_world_opts& o);
// queues one frame on W's stream; ev (optional) receives 6 stage events; returns kernels queued
int queue_frame(psx_world* W, cudaEvent_t* ev = nullptr);
// one frame on W's stream, through W's CUDA graph when it uses one
psx_status run_frame(psx_world* W);
// launch shapes: apply (0 fields keep the current value) and read back
psx_status apply_launch(psx_world* W, const psx_launch_config& c);
psx_launch_config current_launch(const psx_world* W);
// splits the scenes above the block limit between clusters and the grid (mode as
// psx_launch_config::large_scene_solver, 0: by the default rule)
psx_status partition_big(psx_world* W, int mode);
// splits the block scenes into solver block sizes (64 / 128 / 256 threads), the
// smallest size in use being threads_min
psx_status partition_tiers(psx_world* W, int threads_min);
// trigger sets and the event log (a world with trigger pairs)
psx_status alloc_triggers(psx_world* W);
// reads the device error word; maps its bits to a status
psx_status check_err(psx_world* W);
// pinned host staging of at least n4 float4
}  // namespace rt
}  // namespace psx
