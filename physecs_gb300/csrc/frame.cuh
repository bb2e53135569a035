// frame.cuh — per-frame device buffers and the kernel entry points of one frame.
#pragma once
#include "types.cuh"
#include "prims.cuh"

namespace psx {

// Restitution-cache keys: (collider, collider, triangle + 1) in one word; collider indices
// take cbits bits each (every index is below 2^cbits - 1, so no key is all ones, the
// empty mark), the triangle the remaining 64 - 2 cbits.
__device__ __forceinline__ unsigned long long cache_key(int ca, int cb, int tri, int cbits) {
    return ((unsigned long long)(uint32_t)ca << (64 - cbits)) | ((unsigned long long)(uint32_t)cb << (64 - 2 * cbits)) |
           (unsigned long long)(uint32_t)(tri + 1);
}
__device__ __forceinline__ uint32_t cache_hash(unsigned long long k) {
    k ^= k >> 33; k *= 0xff51afd7ed558ccdull; k ^= k >> 33; k *= 0xc4ceb9fe1a85ec53ull; k ^= k >> 33;
    return (uint32_t)k;
}
constexpr unsigned long long kEmpty = ~0ull;

// Trigger-pair keys (collider0 << 32 | collider1) and their tables' hash and empty mark.
constexpr unsigned long long kNoKey = ~0ull;
__device__ __forceinline__ unsigned trig_hash(unsigned long long k) {
    k ^= k >> 33; k *= 0xff51afd7ed558ccdull; k ^= k >> 33; k *= 0xc4ceb9fe1a85ec53ull; k ^= k >> 33;
    return (unsigned)k;
}

struct BVHNodes {
    int* left;        // child index: >= 0 internal node (global), < 0 leaf ~(sorted position)
    int* right;
    int* parent;      // parent of internal nodes (global internal index), -1 for roots
    int* leaf_parent; // parent of each sorted leaf
    int* first;       // sorted-leaf range covered by each internal node
    int* last;
    float4* bmin;
    float4* bmax;
    int* visits;
};

struct FrameBuf {
    // broadphase
    float4* scene_lo;     // [S] centroid bounds for Morton quantisation
    float4* scene_hi;
    uint32_t* keys;       // [n_colliders] sort keys, then the sorted leaves' Morton codes
    uint32_t* mkey;       // [n_colliders] Morton code per collider
    int* order;           // sorted leaf -> collider
    uint32_t* keys_tmp;
    int* order_tmp;
    int* radix_hist;
    BVHNodes bvh;
    int* leaf_cnt;        // [n_colliders] pairs found per sorted leaf
    int* leaf_off;
    int* scan_scratch;
    int trav_k;           // pairs per leaf the walk keeps in cat_list (free until k_classify), 0: none
    int* trav_tail;       // device flag: some leaf found more than trav_k pairs
    int pair_cap;
    int2* pairs;          // collider indices, entity(a) < entity(b)
    int* n_pairs;         // device scalar
    // narrowphase
    int* pair_cat;        // 0 analytic, 1 convex mesh, 2 triangle mesh
    int* cat_count;       // [10]: analytic pairs without a box, convex, triangle-mesh pairs, convex pairs
                          // that overlap, analytic pairs with one box, box-box pairs, overlapping convex
                          // pairs whose EPA polytope outgrew the small one, trigger pairs, overlapping
                          // convex pairs that outgrew the lane-per-pair EPA; [9] the pairs that EPA
                          // has taken so far
    int* cat_list;        // [9 * pair_cap]: the pairs of lists 0-8
    Manifold* man_pair;   // one slot per pair (analytic / convex categories)
    unsigned char* epa_save;   // polytopes handed from one EPA pass to the next (epa_save_bytes())
    int lane_saves, group_saves;   // how many of them the lane-per-pair and grouped passes may hand over
    int tri_cap;          // triangle-mesh pair slots
    Manifold* man_tri;    // kTriManifolds slots per triangle-mesh pair slot
    int* pair_tslot;      // triangle-mesh slot of a pair
    int* pair_nman;
    int* pair_moff;
    int man_cap;
    int* n_man;
    Contact* contacts;    // one per manifold, in pair order
    int* man_scene_cnt;   // [S]
    int* scene_man;       // [S+1]
    // colouring
    unsigned long long* claim;  // [n_dyn] (hashed priority << 32 | contact index)
    int* color_of;        // [man_cap]
    int* corder;          // [man_cap] manifolds sorted by (scene, colour, index)
    int* scene_ncolor;    // [S]
    int* color_start;     // [S * (kMaxColors+1)]
    int* claim_pos;       // [S * (kMaxColors+1)] scatter counters
    // per-substep contact records of scenes whose records do not fit in shared memory
    int* pt_off;          // [man_cap] first point of each contact, colour order
    int2* cbody;          // [man_cap] colouring: scene-local dynamic bodies of each contact
    uint4* cmask;         // [n_dyn] colouring: colours each dynamic body carries (128 bits)
    SHdr* s_hdr;          // [man_cap]
    SPt* s_pts;           // [4 * man_cap]
    // restitution cache: open addressing, two tables; cache_parity selects the current one
    int cache_cap;        // power of two
    CacheEntry* cache_a;
    CacheEntry* cache_b;
    int* cache_parity;
    // trigger pairs (src/Physecs.cpp:200-207, 537-552); trig_cap is 0 when the world has no
    // trigger collider.  Two sets alternate between frames, trig_state[0] selecting this
    // frame's: the keys (collider0 << 32 | collider1) of the overlapping trigger pairs, as a
    // list and in an open-addressing table (~0 = empty) that records each key's slot
    int trig_cap;                          // = pair_cap: every trigger pair is a pair
    int trig_table_cap;                    // power of two >= 2 * trig_cap
    unsigned long long* trig_table[2];
    unsigned long long* trig_keys[2];
    int* trig_slot[2];
    int* trig_state;                       // [4]: parity, keys in set 0, keys in set 1, frame
    int evt_cap;
    int4* trig_evt;                        // [evt_cap] (frame, 0 enter / 1 exit, collider0, collider1)
    int* n_evt;                            // events since the host last drained them (may pass evt_cap)
    // grid barrier: count, generation, flag
    unsigned int* bar;
    // per-frame totals: contact points, joint rows (for throughput accounting)
    int* n_points;
    int* n_rows;
};

// kernel launch helpers (definitions in the .cu files); each returns the number of
// kernels it queued
int launch_aabb(const World& w, int margin_mode, cudaStream_t s);
int launch_aabb_range(const World& w, int c0, int c1, int margin_mode, cudaStream_t s);
// getBoundsTriangleMesh for the triangle-mesh colliders in [c0, c1), with the 0.01 m
// margin of updateBounds or without it
int launch_trimesh_bounds(const World& w, int c0, int c1, bool margin, cudaStream_t s);
// a coalesced batch of registry deltas (one record per body), then the joints of the
// bodies whose kinematic flag changed
int launch_apply_deltas(const World& w, const DeltaRec* d, int n, const int* joints, int nj, cudaStream_t s);
// body state between 3-float device staging (every body) and the world's float4 arrays
int launch_unpack_bodies(const World& w, const float* pos, const float* vel, const float* ang, cudaStream_t s);
int launch_pack_bodies(const World& w, float* pos, float* vel, float* ang, cudaStream_t s);
// scene_sort_pmax > 0: every scene has at most that many colliders (a power of two) and
// is sorted by its own block in shared memory; 0: one radix sort over the whole world
int launch_broadphase(const World& w, FrameBuf& f, int scene_bits, int scene_sort_pmax, cudaStream_t s);
// each scene's LBVH over the current bounds (all_leaves: every collider reachable, for queries)
int launch_bvh_build(const World& w, FrameBuf& f, int scene_bits, int scene_sort_pmax, bool all_leaves, cudaStream_t s);

// scene queries (query.cu); the layouts are psx_ray and psx_overlap_query of include/psx.h
struct RayIn { int scene; float ox, oy, oz, dx, dy, dz, maxd; };
struct RayOut { int collider; float dist; };   // world collider index or -1
struct ShapeIn {
    int scene;
    float px, py, pz, qx, qy, qz, qw;
    int type;
    float p0, p1, p2;
    int mesh;     // world convex mesh index
    int filter;   // collider data bits (0: any)
};
int launch_raycast(const World& w, FrameBuf& f, const RayIn* rays, int n, const unsigned char* accept, RayOut* out,
                   cudaStream_t s);
int launch_overlap(const World& w, FrameBuf& f, const ShapeIn* qs, int n, int cap, int* counts, int* hits, cudaStream_t s);
// one CharacterController::move per record (psx_character layout; body is the world index)
struct CharIn {
    int scene, body;
    float height, radius, max_step_height, slope_limit;
    int iterations;
    float tx, ty, tz;
};
int launch_move_characters(const World& w, FrameBuf& f, const CharIn* cs, int n, unsigned char* flags, float4* moved,
                           cudaStream_t s);
int launch_overlap_mtd(const World& w, FrameBuf& f, const ShapeIn* qs, int n, int cap, int* counts, float4* hits,
                       int* hit_col, cudaStream_t s);
// a second stream with a fork / join event pair, for kernels that may overlap
struct StreamPair {
    cudaStream_t aux;
    cudaEvent_t fork, join;
};
struct NarrowShape {
    int convex_warps, convex_blocks_per_sm;   // EPA: warps per block, blocks per SM
    int analytic_threads, analytic_blocks_per_sm;
    int contacts_threads;
    int gjk_blocks_per_sm;                    // GJK: 128-thread blocks per SM
    int epa_lanes;                            // EPA: lanes per pair (8, 16 or 32; below 32, one warp per block);
                                              // 1: a lane per pair, 16 for the pairs that outgrow it
    int epa_full_only;                        // EPA: skip the small-polytope pass
};
int launch_narrowphase(const World& w, FrameBuf& f, const StreamPair& sp, const NarrowShape& ns, cudaStream_t s);
void epa_save_caps(int pair_cap, int& lane, int& group);
size_t epa_save_bytes(int lane, int group);
// trigger pairs of this frame: overlap tests, enter and exit events, set swap (query.cu)
int launch_triggers(const World& w, FrameBuf& f, cudaStream_t s);
int launch_contacts(const World& w, FrameBuf& f, cudaStream_t s);
// scenes of one frame's solver launch: small block scenes (one 256-thread block each),
// large block scenes (one 512-thread block each, on the aux stream), grid scenes
// (the whole grid, one after another)
constexpr int kClusterBlocks = 8;   // blocks of the cluster that solves one large scene
struct SolverLaunch {
    const int* tier[3]; int n_tier[3]; int smem_tier[3];   // block scenes by block size 32 or 64 / 128 / 256
    int tier0_nt;                                          // threads per block of the smallest tier: 32 or 64
    cudaStream_t tstream[2];                               // streams of the 64- and 128-thread tiers
    cudaEvent_t tfork, tjoin[2];
    const int* large; int n_large; int smem_large;
    const int* cluster; int n_cluster;     // large scenes solved by one cluster each
    const int* grid; int n_grid; int grid_blocks;
    cudaStream_t aux;
    cudaEvent_t fork, join;
    long long wait_limit;                  // polls of a grid-barrier wait (0: kDefaultWaitPolls)
    int large_nt;                          // threads per block of the large block scenes: 128, 256 or 512
};
int launch_solver(const World& w, FrameBuf& f, const SolverLaunch& L, cudaStream_t s);
int solver_grid_blocks();
int launch_joint_layout(const World& w, FrameBuf& f, cudaStream_t s);

}  // namespace psx
