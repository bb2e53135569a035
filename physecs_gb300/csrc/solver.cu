// solver.cu — contact rows, graph colouring, joint rows and the TGS substep loop.
//
// Restates Physecs src/Physecs.cpp:209-531 with src/ContactConstraints.cpp,
// src/Constraint1D.cpp (scalar rows, joint colour 8) and src/Constraint1DW.cpp
// (4-lane rows, joint colours 0-7).  The reference solves every contact serially;
// here contacts are graph-coloured so that each colour is body-disjoint and its
// contacts can be solved in parallel with a result identical to any serial order
// of that colour.  Joints keep the reference's own colouring (colours 0-7 are
// entity-disjoint); the overflow colour is split into sub-colours on the host.
//
// One persistent kernel runs a whole frame of a scene: colouring, then every
// substep's row update, velocity integration, preSolve, iterations, position
// integration, relaxation and write-back.  Small scenes run one per CTA with
// __syncthreads between phases; large scenes run on the whole grid with a
// bounded grid barrier.
#include <cooperative_groups.h>
#include "libm_f32.cuh"
#include <algorithm>
#include "frame.cuh"

namespace psx {

constexpr float kPi = 3.14159265358979323846f;

// ---------------------------------------------------------------- restitution cache


__global__ void k_cache_clear(FrameBuf f) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f.cache_cap) return;
    CacheEntry* cur = f.cache_parity[0] ? f.cache_b : f.cache_a;
    cur[i].key = kEmpty;
}

__global__ void k_cache_flip(FrameBuf f) { f.cache_parity[0] ^= 1; }

// ---------------------------------------------------------------- contact rows (src/Physecs.cpp:215-314)

__global__ void k_build_contacts(World w, FrameBuf f) {
    int np = *f.n_pairs;
    CacheEntry* cur = f.cache_parity[0] ? f.cache_b : f.cache_a;
    const CacheEntry* prev = f.cache_parity[0] ? f.cache_a : f.cache_b;
    unsigned mask = (unsigned)f.cache_cap - 1u;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        int cnt = f.pair_nman[p];
        if (!cnt) continue;
        int off = f.pair_moff[p];
        int2 pr = f.pairs[p];
        int4 cA = w.col_info[pr.x], cB = w.col_info[pr.y];
        int bodyA = cA.x, bodyB = cB.x;
        int4 iA = w.info[bodyA], iB = w.info[bodyB];
        bool simA = (iA.y & BODY_DYN) && !(iA.y & BODY_KIN), simB = (iB.y & BODY_DYN) && !(iB.y & BODY_KIN);
        Q4 qA = ld4(w.quat[bodyA]), qB = ld4(w.quat[bodyB]);
        V3 com0 = {0, 0, 0}, v0 = {0, 0, 0}, w0 = {0, 0, 0}, com1 = {0, 0, 0}, v1 = {0, 0, 0}, w1 = {0, 0, 0};
        if (simA) { com0 = ld3(w.pos[bodyA]) + qrot(qA, ld3(w.com[iA.z])); v0 = ld3(w.vel[iA.z]); w0 = ld3(w.ang[iA.z]); }
        if (simB) { com1 = ld3(w.pos[bodyB]) + qrot(qB, ld3(w.com[iB.z])); v1 = ld3(w.vel[iB.z]); w1 = ld3(w.ang[iB.z]); }
        float4 mA = w.col_mat[pr.x], mB = w.col_mat[pr.y];
        float friction = (mA.x + mB.x) * 0.5f;
        bool soft;
        float freq = 0, damp = 0, rest = 0;
        if (mA.z || mB.z) {
            soft = true;
            if (mA.z && mB.z) { freq = fminG(mA.y, mB.y); damp = fminG(mA.z, mB.z); }
            else if (mA.z) { freq = mA.y; damp = mA.z; }
            else { freq = mB.y; damp = mB.z; }
        } else {
            soft = false;
            rest = (mA.y + mB.y) * 0.5f;
        }
        Q4 iqA = qinverse(qA), iqB = qinverse(qB);
        bool tri = f.pair_cat[p] == 2;
        for (int k = 0; k < cnt; ++k) {
            int idx = off + k;
            if (idx >= f.man_cap) { atomicOr(w.err, ERR_MANIFOLD_CAPACITY); break; }
            const Manifold& m = tri ? f.man_tri[f.pair_tslot[p] * kTriManifolds + k] : f.man_pair[p];
            Contact c;
            c.b0 = simA ? iA.z : -1;
            c.b1 = simB ? iB.z : -1;
            c.body0 = bodyA; c.body1 = bodyB;
            V3 n = ld3(m.n);
            c.n = st4(n, friction);
            c.frequency = freq; c.damping = damp;
            c.np = m.np; c.soft = soft ? 1 : 0;
            c.color = -1; c.scene = iA.w; c.pair = p; c.tri = m.tri;
            unsigned long long key = cache_key(pr.x, pr.y, m.tri, w.key_cbits);
            // previous frame's entry, if any
            const CacheEntry* pe = nullptr;
            const bool fresh = w.scene_fresh && w.scene_fresh[iA.w];
            for (unsigned h = cache_hash(key) & mask, probe = 0; !fresh && probe < (unsigned)f.cache_cap; ++probe, h = (h + 1) & mask) {
                unsigned long long kk = prev[h].key;
                if (kk == key) { pe = &prev[h]; break; }
                if (kk == kEmpty) break;
            }
            CacheEntry ne;
            ne.key = key; ne.np = m.np;
            for (int q = 0; q < m.np; ++q) {
                V3 r0 = ld3(m.p0[q]) - com0;
                V3 r1 = ld3(m.p1[q]) - com1;
                V3 rel = v1 + cross(w1, r1) - v0 - cross(w0, r0);
                float relN = dot(rel, n);
                r0 = qrot(iqA, r0);
                r1 = qrot(iqB, r1);
                float tv = 0;
                bool found = false;
                if (pe) {
                    for (int i = 0; i < pe->np; ++i) {
                        float4 e = pe->r0tv[i];
                        if ((double)distance(r0, ld3(e)) < 0.1) { found = true; tv = e.w; break; }
                    }
                }
                if (!found) tv = -rest * relN;
                ne.r0tv[q] = st4(r0, tv);
                ContactPt& cp = c.p[q];
                cp.r0 = st4(r0, tv);
                cp.r1 = st4(r1, 0.f);
            }
            // insert into this frame's table
            bool placed = false;
            for (unsigned h = cache_hash(key) & mask, probe = 0; probe < (unsigned)f.cache_cap; ++probe, h = (h + 1) & mask) {
                unsigned long long old = atomicCAS(&cur[h].key, kEmpty, key);
                if (old == kEmpty || old == key) {
                    cur[h].np = ne.np;
                    for (int q = 0; q < ne.np; ++q) cur[h].r0tv[q] = ne.r0tv[q];
                    placed = true;
                    break;
                }
            }
            if (!placed) atomicOr(w.err, ERR_CACHE_CAPACITY);
            f.contacts[idx] = c;
            atomicAdd(&f.man_scene_cnt[iA.w], 1);
            atomicAdd(f.n_points, m.np);
        }
    }
}

// ---------------------------------------------------------------- joints

// getSolverDesc of each joint type (src/Joints/*.cpp): row flags in creation order,
// evaluated at frame start; the prismatic limit row exists only while violated.
__global__ void k_joint_layout(World w, int* n_rows) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= w.n_joints) return;
    JointDev J = w.joints[j];
    int f[kMaxRowsPerJoint];
    int n = 0;
    auto add = [&](int fl, int cnt) { for (int i = 0; i < cnt; ++i) f[n++] = fl; };
    enum { RN = 0, RS = 1, RA = 2, RL = 4 };
    switch (J.type) {
        case 0: add(RN, 3); add(RA, 3); break;                                        // fixed
        case 1: add(RN, 3); add(RA, 2); if (J.params[0] != 0.f) add(RA | RL, 1); break;  // revolute
        case 2: add(RN, 3); break;                                                    // spherical
        case 3: {                                                                     // prismatic
            V3 p0 = ld3(w.pos[J.body0]) + qrot(ld4(w.quat[J.body0]), ld3(J.a0p));
            V3 p1 = ld3(w.pos[J.body1]) + qrot(ld4(w.quat[J.body1]), ld3(J.a1p));
            V3 d = p1 - p0;
            V3 u00 = qrot(qmul(ld4(w.quat[J.body0]), ld4(J.a0q)), {1, 0, 0});
            float dx = dot(d, u00);
            add(RN, 2); add(RA, 3);
            if (dx > J.params[0]) { J.makeUpper = 1; J.makeLower = 0; add(RL, 1); }
            else if (dx < J.params[1]) { J.makeUpper = 0; J.makeLower = 1; add(RL, 1); }
            else { J.makeUpper = 0; J.makeLower = 0; }
            if (J.params[2] != 0.f) add(RS, 1);
            break;
        }
        case 4: add(RN, 3); add(RA, 1); break;                                        // universal
        case 5: add(RA, 1); break;                                                    // gear
        default: add(RN, 3); add(RA, 2); add(RA | RS, 1); break;                      // servo
    }
    J.nrows = n;
    atomicAdd(n_rows, n);
    for (int i = 0; i < kMaxRowsPerJoint; ++i) J.rowflags[i] = i < n ? f[i] : -1;
    w.joints[j].makeUpper = J.makeUpper;
    w.joints[j].makeLower = J.makeLower;
    w.joints[j].nrows = n;
    for (int i = 0; i < kMaxRowsPerJoint; ++i) w.joints[j].rowflags[i] = J.rowflags[i];
    for (int i = 0; i < n; ++i) {
        Row r;
        r.linear = make_float4(0, 0, 0, 0);
        r.angular0 = make_float4(0, 0, 0, 0);
        r.angular1 = make_float4(0, 0, 0, -FLT_MAX);
        r.linear0t = make_float4(0, 0, 0, FLT_MAX);
        r.linear1t = make_float4(0, 0, 0, 0);
        r.angular0t = make_float4(0, 0, 0, 0);
        r.angular1t = make_float4(0, 0, 0, 0);
        r.totalLambda = 0;
        r.flags = f[i]; r.b0 = J.b0; r.b1 = J.b1;
        w.rows[j * kMaxRowsPerJoint + i] = r;
    }
}

int launch_joint_layout(const World& w, FrameBuf& f, cudaStream_t s) {
    cudaMemsetAsync(f.n_rows, 0, sizeof(int), s);
    if (!w.n_joints) return 0;
    k_joint_layout<<<(w.n_joints + 127) / 128, 128, 0, s>>>(w, f.n_rows);
    return 1;
}

__device__ __forceinline__ float angleDiffD(float a0, float a1) {  // GearJoint.cpp:5-8
    const float pi = kPi, two_pi = 6.28318530717958647692f;
    float diff = fmodf(a1 - a0 + pi, two_pi) - pi;
    return diff < -pi ? diff + two_pi : diff;
}

// makeConstraints of each joint type (src/Joints/*.cpp, src/JointsUtil.h:8-28), rows in creation order
__device__ void make_joint_rows(const World& w, int j) {
    JointDev& J = w.joints[j];
    Q4 q0 = ld4(w.quat[J.body0]), q1 = ld4(w.quat[J.body1]);
    M3 u0 = mat3_cast(qmul(q0, ld4(J.a0q))), u1 = mat3_cast(qmul(q1, ld4(J.a1q)));
    V3 r0 = qrot(q0, ld3(J.r0)), r1 = qrot(q1, ld3(J.r1));
    V3 p0 = ld3(w.pos[J.body0]) + qrot(q0, ld3(J.a0p)), p1 = ld3(w.pos[J.body1]) + qrot(q1, ld3(J.a1p));
    Row* R = w.rows + j * kMaxRowsPerJoint;
    int k = 0;
    auto lin = [&](V3 l, V3 a0, V3 a1, float c) {
        R[k].linear = st4(l, R[k].linear.w); R[k].angular0 = st4(a0, c); R[k].angular1 = st4(a1, R[k].angular1.w); ++k;
    };
    auto ang = [&](V3 a, float c) {
        R[k].angular0 = st4(a, c); R[k].angular1 = st4(a, R[k].angular1.w); ++k;
    };
    auto p2p = [&]() {
        V3 d = p1 - p0;
        lin({1, 0, 0}, {0, r0.z, -r0.y}, {0, r1.z, -r1.y}, d.x);
        lin({0, 1, 0}, {-r0.z, 0, r0.x}, {-r1.z, 0, r1.x}, d.y);
        lin({0, 0, 1}, {r0.y, -r0.x, 0}, {r1.y, -r1.x, 0}, d.z);
    };
    switch (J.type) {
        case 0:
            p2p();
            ang(cross(u1.c[1], u0.c[0]), dot(u0.c[0], u1.c[1]));
            ang(cross(u1.c[2], u0.c[0]), dot(u0.c[0], u1.c[2]));
            ang(cross(u1.c[2], u0.c[1]), dot(u0.c[1], u1.c[2]));
            break;
        case 2: p2p(); break;
        case 4:
            p2p();
            ang(cross(u1.c[2], u0.c[2]), dot(u0.c[2], u1.c[2]));
            break;
        case 1:
            p2p();
            ang(cross(u1.c[1], u0.c[0]), dot(u0.c[0], u1.c[1]));
            ang(cross(u1.c[2], u0.c[0]), dot(u0.c[0], u1.c[2]));
            if (J.params[0] != 0.f) {
                R[k].angular0 = st4(u0.c[0], R[k].angular0.w);
                R[k].angular1 = st4(u0.c[0], -J.params[2]);
                R[k].linear.w = J.params[1];
                R[k].linear0t.w = J.params[2];
                ++k;
            }
            break;
        case 6: {
            p2p();
            ang(cross(u1.c[1], u0.c[0]), dot(u0.c[0], u1.c[1]));
            ang(cross(u1.c[2], u0.c[0]), dot(u0.c[0], u1.c[2]));
            float a = libm::acosf(clampG(dot(u0.c[2], u1.c[2]), -1.f, 1.f));   // glm::orientedAngle
            if (dot(u0.c[0], cross(u0.c[2], u1.c[2])) < 0.f) a = -a;
            R[k].angular0 = st4(u0.c[0], a - J.params[0]);
            R[k].angular1 = st4(u0.c[0], R[k].angular1.w);
            R[k].linear1t.w = J.params[1];
            R[k].angular0t.w = J.params[2];
            ++k;
            break;
        }
        case 3: {
            V3 d = p1 - p0;
            lin(u0.c[1], cross(r0, u0.c[1]), cross(r1, u0.c[1]), dot(d, u0.c[1]));
            lin(u0.c[2], cross(r0, u0.c[2]), cross(r1, u0.c[2]), dot(d, u0.c[2]));
            ang(cross(u1.c[1], u0.c[0]), dot(u0.c[0], u1.c[1]));
            ang(cross(u1.c[2], u0.c[0]), dot(u0.c[0], u1.c[2]));
            ang(cross(u1.c[2], u0.c[1]), dot(u0.c[1], u1.c[2]));
            float dx = dot(d, u0.c[0]);
            V3 r0xx = cross(r0, u0.c[0]), r1xx = cross(r1, u0.c[0]);
            if (J.makeUpper) {
                R[k].angular1.w = 0.f;  // min = 0
                lin(u0.c[0], r0xx, r1xx, dx - J.params[0]);
            } else if (J.makeLower) {
                R[k].linear0t.w = 0.f;  // max = 0
                lin(u0.c[0], r0xx, r1xx, dx - J.params[1]);
            }
            if (J.params[2] != 0.f) {
                R[k].linear1t.w = J.params[4];
                R[k].angular0t.w = J.params[5];
                lin(u0.c[0], r0xx, r1xx, dx - J.params[3]);
            }
            break;
        }
        default: {  // gear (GearJoint.cpp:10-50)
            float a0, a1;
            {
                V3 p1p = p1 + dot(p0 - p1, u0.c[0]) * u0.c[0];
                V3 dir = normalize(p0 - p1p);
                V3 n = cross(u0.c[0], dir);
                M3 t = mm(transpose(m3cols(u0.c[0], -n, dir)), u0);
                a0 = libm::atan2f(at(t.c[1], 2), at(t.c[2], 2));
            }
            {
                V3 p0p = p0 + dot(p1 - p0, u1.c[0]) * u1.c[0];
                V3 dir = normalize(p0p - p1);
                V3 n = cross(u1.c[0], dir);
                M3 t = mm(transpose(u1), m3cols(u1.c[0], -n, dir));
                a1 = libm::atan2f(at(t.c[1], 2), at(t.c[2], 2));
            }
            if (!J.gearInit) { J.persistent0 = a0; J.persistent1 = a1; J.gearInit = 1; }
            J.virtual0 += angleDiffD(a0, J.persistent0);
            J.virtual1 += angleDiffD(a1, J.persistent1);
            J.persistent0 = a0; J.persistent1 = a1;
            float ratio = J.params[0];
            R[k].angular0 = st4(u0.c[0] * ratio, J.virtual0 * ratio - J.virtual1);
            R[k].angular1 = st4(-u1.c[0], R[k].angular1.w);
            ++k;
            break;
        }
    }
}

// Constraint1D(W)::preSolve for one row (Constraint1D.cpp:5-52 / Constraint1DW.cpp:5-115)
__device__ void row_presolve(const World& w, Row& r, bool simd) {
    int fl = r.flags;
    bool angf = fl & 2, soft = fl & 1, lim = fl & 4;
    float im0 = 0, im1 = 0;
    M3 I0 = m3zero(), I1 = m3zero();
    if (r.b0 >= 0) { im0 = w.com[r.b0].w; I0 = m3cols(ld3(w.mt[3 * r.b0]), ld3(w.mt[3 * r.b0 + 1]), ld3(w.mt[3 * r.b0 + 2])); }
    if (r.b1 >= 0) { im1 = w.com[r.b1].w; I1 = m3cols(ld3(w.mt[3 * r.b1]), ld3(w.mt[3 * r.b1 + 1]), ld3(w.mt[3 * r.b1 + 2])); }
    V3 a0 = ld3(r.angular0), a1 = ld3(r.angular1), l = ld3(r.linear);
    V3 a0t = mv(I0, a0), a1t = mv(I1, a1);
    float inv = dot(a0, a0t) + dot(a1, a1t);
    V3 l0t = ld3(r.linear0t), l1t = ld3(r.linear1t);
    if (!angf) {
        inv += dot(l, l) * (im0 + im1);
        l0t = im0 * l;
        l1t = im1 * l;
    }
    r.angular0t = st4(a0t, r.angular0t.w);
    r.angular1t = st4(a1t, inv);
    r.linear0t = st4(l0t, r.linear0t.w);
    r.linear1t = st4(l1t, r.linear1t.w);
    if (soft) return;
    float c = r.angular0.w, mn = r.angular1.w, mx = r.linear0t.w;
    float lambda;
    if (!simd) {
        if (!c || !inv) return;
        lambda = c / inv;
        if (lim) lambda = clampG(lambda, mn, mx);
    } else {
        if (!(inv != 0.f && c != 0.f)) return;
        lambda = c / inv;
        if (lim) { lambda = lambda > mn ? lambda : mn; lambda = lambda < mx ? lambda : mx; }
    }
    if (r.b0 >= 0) {
        float4 pv = w.pv_v[r.b0], pw = w.pv_w[r.b0];
        V3 v = ld3(pv), wv = ld3(pw);
        if (!angf) v += lambda * l0t;
        wv += lambda * a0t;
        w.pv_v[r.b0] = st4(v, pv.w + 1.f);
        w.pv_w[r.b0] = st4(wv, 0.f);
    }
    if (r.b1 >= 0) {
        float4 pv = w.pv_v[r.b1], pw = w.pv_w[r.b1];
        V3 v = ld3(pv), wv = ld3(pw);
        if (!angf) v -= lambda * l1t;
        wv -= lambda * a1t;
        w.pv_v[r.b1] = st4(v, pv.w + 1.f);
        w.pv_w[r.b1] = st4(wv, 0.f);
    }
}

// Body velocities the iterations work on, as six float arrays of n entries:
//   - in this block's shared memory (s != null, body d at index d - off);
//   - spread over the blocks of a thread-block cluster (rs != null: body d at block
//     (d - off) mod 2^lg, index (d - off) >> lg, through distributed shared memory);
//   - else the world's vt arrays.
struct VelRef {
    float* s;
    float* const* rs;
    float4* v;
    float4* w;
    int off, n, lg;
    __device__ __forceinline__ float* base(int d, int& j) const {
        int i = d - off;
        if (rs) { j = i >> lg; return rs[i & ((1 << lg) - 1)]; }
        j = i;
        return s;
    }
    __device__ __forceinline__ V3 lv(int d) const {
        if (s || rs) { int j; const float* b = base(d, j); return {b[j], b[n + j], b[2 * n + j]}; }
        return ld3(v[d]);
    }
    __device__ __forceinline__ V3 lw(int d) const {
        if (s || rs) { int j; const float* b = base(d, j); return {b[3 * n + j], b[4 * n + j], b[5 * n + j]}; }
        return ld3(w[d]);
    }
    __device__ __forceinline__ void sv(int d, V3 x) const {
        if (s || rs) { int j; float* b = base(d, j); b[j] = x.x; b[n + j] = x.y; b[2 * n + j] = x.z; }
        else v[d] = st4(x);
    }
    __device__ __forceinline__ void sw(int d, V3 x) const {
        if (s || rs) { int j; float* b = base(d, j); b[3 * n + j] = x.x; b[4 * n + j] = x.y; b[5 * n + j] = x.z; }
        else w[d] = st4(x);
    }
};

// Constraint1D(W)::solve for one row (Constraint1D.cpp:54-127 / Constraint1DW.cpp:117-233)
__device__ void row_solve(const World& w, Row& r, float h, bool warm, bool simd, const VelRef vr) {
    int fl = r.flags;
    bool angf = fl & 2, soft = fl & 1, lim = fl & 4;
    float inv = r.angular1t.w;
    if (!simd && !inv) return;
    V3 v0 = {0, 0, 0}, w0 = {0, 0, 0}, v1 = {0, 0, 0}, w1 = {0, 0, 0};
    if (r.b0 >= 0) { if (!angf) v0 = vr.lv(r.b0); w0 = vr.lw(r.b0); }
    if (r.b1 >= 0) { if (!angf) v1 = vr.lv(r.b1); w1 = vr.lw(r.b1); }
    V3 l0t = ld3(r.linear0t), l1t = ld3(r.linear1t), a0t = ld3(r.angular0t), a1t = ld3(r.angular1t);
    float c = r.angular0.w;
    if (!soft && warm) {
        bool apply = simd ? (fabsf(c) < (float)1e-4 && fabsf(r.totalLambda) < 10000.f)
                          : !((double)fabsf(c) > 1e-4 || fabsf(r.totalLambda) > 10000.f);
        if (apply) {
            float lw = r.totalLambda * 0.5f;
            r.totalLambda = lw;
            if (!angf) { v0 += lw * l0t; v1 -= lw * l1t; }
            w0 += lw * a0t;
            w1 -= lw * a1t;
        }
    }
    if (simd && !inv) return;
    V3 a0 = ld3(r.angular0), a1 = ld3(r.angular1), l = ld3(r.linear);
    float rv = dot(a1, w1) - dot(a0, w0);
    if (!angf) rv += dot(l, v1) - dot(l, v0);
    float tvel = r.linear.w, mn = r.angular1.w, mx = r.linear0t.w, freq = r.linear1t.w, damp = r.angular0t.w;
    float lambda;
    if (simd) {
        float eff = 1.f / inv;
        if (soft) {
            float af = (2.f * kPi) * freq;
            float stiffness = af * af * eff;
            float damping = 2.f * af * damp * eff;
            float gamma = 1.f / (damping + h * stiffness);
            float beta = h * stiffness * gamma;
            lambda = (rv + beta * c / h) / (inv + gamma / h);
        } else {
            float bias = (float)(0.2 / (double)h);
            lambda = (rv - tvel + bias * c) * eff;
        }
    } else {
        if (soft) {
            float af = 2.f * kPi * freq;
            float stiffness = af * af / inv;
            float damping = 2.f * af * damp / inv;
            float gamma = 1.f / (damping + h * stiffness);
            float beta = h * stiffness / (damping + h * stiffness);
            lambda = (rv + beta * c / h) / (inv + gamma / h);
        } else {
            lambda = (rv - tvel + 0.2f * c / h) / inv;
        }
    }
    if (lim) {
        float prev = r.totalLambda;
        r.totalLambda += lambda;
        if (simd) {
            float lo = mn * h, hi = mx * h;
            r.totalLambda = r.totalLambda > lo ? r.totalLambda : lo;
            r.totalLambda = r.totalLambda < hi ? r.totalLambda : hi;
        } else {
            r.totalLambda = clampG(r.totalLambda, mn, mx);
        }
        lambda = r.totalLambda - prev;
    } else {
        r.totalLambda += lambda;
    }
    if (!simd) {
        // the scalar row applies only this iteration's impulse (Constraint1D.cpp:158-168)
        if (r.b0 >= 0) {
            if (!angf) vr.sv(r.b0, vr.lv(r.b0) + lambda * l0t);
            vr.sw(r.b0, vr.lw(r.b0) + lambda * a0t);
        }
        if (r.b1 >= 0) {
            if (!angf) vr.sv(r.b1, vr.lv(r.b1) - lambda * l1t);
            vr.sw(r.b1, vr.lw(r.b1) - lambda * a1t);
        }
        return;
    }
    if (!angf) { v0 += lambda * l0t; v1 -= lambda * l1t; }
    w0 += lambda * a0t;
    w1 -= lambda * a1t;
    if (r.b0 >= 0) { if (!angf) vr.sv(r.b0, v0); vr.sw(r.b0, w0); }
    if (r.b1 >= 0) { if (!angf) vr.sv(r.b1, v1); vr.sw(r.b1, w1); }
}

__constant__ int c_flag_order[6] = {0, 2, 1, 4, 3, 6};

__device__ void joint_presolve(const World& w, int j) {
    JointDev& J = w.joints[j];
    Row* R = w.rows + j * kMaxRowsPerJoint;
    for (int fi = 0; fi < 6; ++fi)
        for (int k = 0; k < J.nrows; ++k)
            if (J.rowflags[k] == c_flag_order[fi]) row_presolve(w, R[k], J.simd != 0);
}

__device__ void joint_solve(const World& w, int j, float h, bool warm, const VelRef vr) {
    JointDev& J = w.joints[j];
    Row* R = w.rows + j * kMaxRowsPerJoint;
    for (int fi = 0; fi < 6; ++fi)
        for (int k = 0; k < J.nrows; ++k)
            if (J.rowflags[k] == c_flag_order[fi]) row_solve(w, R[k], h, warm, J.simd != 0, vr);
}

// ---------------------------------------------------------------- contacts (ContactConstraints.cpp)

__device__ __forceinline__ M3 world_invI(const World& w, int d) {
    return m3cols(ld3(w.mt[3 * d]), ld3(w.mt[3 * d + 1]), ld3(w.mt[3 * d + 2]));
}


// update contact rows (src/Physecs.cpp:366-427)
__device__ void contact_update(const World& w, Contact& c, SHdr& H, SPt* P) {
    int4 i0 = w.info[c.body0], i1 = w.info[c.body1];
    Q4 q0 = ld4(w.quat[c.body0]), q1 = ld4(w.quat[c.body1]);
    V3 com0 = {0, 0, 0}, v0 = {0, 0, 0}, w0 = {0, 0, 0}, com1 = {0, 0, 0}, v1 = {0, 0, 0}, w1 = {0, 0, 0};
    if (c.b0 >= 0) { com0 = ld3(w.pos[c.body0]) + qrot(q0, ld3(w.com[i0.z])); v0 = ld3(w.vel[i0.z]); w0 = ld3(w.ang[i0.z]); }
    if (c.b1 >= 0) { com1 = ld3(w.pos[c.body1]) + qrot(q1, ld3(w.com[i1.z])); v1 = ld3(w.vel[i1.z]); w1 = ld3(w.ang[i1.z]); }
    V3 n = ld3(c.n);
    H.n = c.n;
    H.m = make_float4(c.b0 >= 0 ? w.com[c.b0].w : 0.f, c.b1 >= 0 ? w.com[c.b1].w : 0.f, c.frequency, c.damping);
    H.i.x = c.b0;
    H.i.y = c.b1;
    H.i.z = c.np | (c.soft << 8);
    for (int k = 0; k < c.np; ++k) {
        ContactPt& p = c.p[k];
        V3 r0 = qrot(q0, ld3(p.r0)), r1 = qrot(q1, ld3(p.r1));
        V3 cp0 = com0 + r0, cp1 = com1 + r1;
        float cn = dot(cp1 - cp0, n);
        V3 rel = v1 + cross(w1, r1) - v0 - cross(w0, r0);
        float relN = dot(rel, n);
        V3 t = rel - relN * n;
        float tl = length(t);
        if (tl) t = t / tl;
        p.r1.w = cn;
        SPt& q = P[k];
        q.a = st4(cross(r0, n), 0.f);
        q.b = st4(cross(r1, n), p.r0.w);
        q.c.w = cn;
        q.e = st4(t, 0.f);
        q.f = st4(cross(r0, t), 0.f);
        q.g = st4(cross(r1, t), 0.f);
    }
}

// ContactConstraints::preSolve (src/ContactConstraints.cpp:4-31) and the per-substep
// constants of solve (:33-101)
__device__ void contact_presolve(const World& w, SHdr& H, SPt* P, float h) {
    const int b0 = H.i.x, b1 = H.i.y, np = H.i.z & 0xff;
    const bool soft = (H.i.z >> 8) != 0;
    const float im0 = H.m.x, im1 = H.m.y;
    M3 I0 = m3zero(), I1 = m3zero();
    V3 v0 = {0, 0, 0}, w0 = {0, 0, 0}, v1 = {0, 0, 0}, w1 = {0, 0, 0};
    if (b0 >= 0) { I0 = world_invI(w, b0); v0 = ld3(w.vel[b0]); w0 = ld3(w.ang[b0]); }
    if (b1 >= 0) { I1 = world_invI(w, b1); v1 = ld3(w.vel[b1]); w1 = ld3(w.ang[b1]); }
    V3 n = ld3(H.n);
    for (int k = 0; k < np; ++k) {
        SPt& p = P[k];
        V3 r0xn = ld3(p.a), r1xn = ld3(p.b), r0xt = ld3(p.f), r1xt = ld3(p.g), t = ld3(p.e);
        V3 r0xnt = mv(I0, r0xn), r1xnt = mv(I1, r1xn), r0xtt = mv(I0, r0xt), r1xtt = mv(I1, r1xt);
        float invN = dot(n, n) * (im0 + im1) + dot(r0xn, r0xnt) + dot(r1xn, r1xnt);
        float invT = dot(t, t) * (im0 + im1) + dot(r0xt, r0xtt) + dot(r1xt, r1xtt);
        float cc = p.c.w;
        float t1 = 0.f, t2 = 0.f, lamT = 0.f;
        if (invN) {
            float eff = 1.f / invN;
            if (soft) {
                float af = 2.f * kPi * H.m.z;
                float stiffness = af * af * eff;
                float damping = 2.f * af * H.m.w * eff;
                float gamma = 1.f / (damping + h * stiffness);
                float beta = h * stiffness / (damping + h * stiffness);
                t1 = beta * cc / h;
                t2 = invN + gamma / h;
            } else {
                t1 = 0.1f * cc / h;
                t2 = eff;
            }
        }
        if (invT) {
            float rv = dot(-t, v0) + dot(-r0xt, w0) + dot(t, v1) + dot(r1xt, w1);
            lamT = rv / invT;
        }
        int live = (invN ? 1 : 0) | (invT ? 2 : 0);
        p.c = st4(r0xnt, t1);
        p.d = st4(r1xnt, t2);
        p.f = st4(r0xtt, lamT);
        p.g = st4(r1xtt, __int_as_float(live));
    }
}

// ContactConstraints::solve (src/ContactConstraints.cpp:33-124).  No other thread touches
// the contact's bodies within its colour, so their velocities stay in registers from the
// first point to the last; every value equals a reload after each point.
// The step is one dependent chain of up to eight rows, so it is written for latency:
//   * the header and the velocity view come by value (a store through a record pointer
//     then cannot alias them, and nothing is reloaded after it);
//   * the records are read ahead of the chain (the normal rows' all at once, then the
//     friction rows') and the accumulated impulses are written after the last row;
//   * all four rows of each kind are evaluated and a row is kept only when it is live
//     (the reference skips a row whose inverse effective mass is zero; a contact has
//     fewer than four points), so the chain has no branches.  A live row's operations
//     and their order are the reference's.  Branching on the point count instead costs
//     registers that the solver kernels do not have.
__device__ __noinline__ void contact_solve(const SHdr H, SPt* __restrict__ P, bool useBias, const VelRef vr) {
    const V3 n = ld3(H.n);
    const float friction = H.n.w;
    const float im0 = H.m.x, im1 = H.m.y;
    const int b0 = H.i.x, b1 = H.i.y, np = H.i.z & 0xff;
    const bool soft = (H.i.z >> 8) != 0;
    V3 v0 = {0, 0, 0}, w0 = {0, 0, 0}, v1 = {0, 0, 0}, w1 = {0, 0, 0};
    if (b0 >= 0) { v0 = vr.lv(b0); w0 = vr.lw(b0); }
    if (b1 >= 0) { v1 = vr.lv(b1); w1 = vr.lw(b1); }
    // every normal record of the contact is read before the chain; rows past the
    // contact's points read its first point and stay dead
    float4 A[4], B[4], C[4], D[4];
    int live[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const bool has = i < np;
        const SPt* q = P + (has ? i : 0);
        A[i] = q->a; B[i] = q->b; C[i] = q->c; D[i] = q->d;
        live[i] = has ? __float_as_int(q->g.w) : 0;
    }
    bool touched = false;
    float lamN[4], lamT[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const bool on = (live[i] & 1) != 0;
        const V3 r0xn = ld3(A[i]), r1xn = ld3(B[i]);
        float rv = dot(-n, v0) + dot(-r0xn, w0) + dot(n, v1) + dot(r1xn, w1);
        float lambda;
        if (soft) lambda = (rv + C[i].w) / D[i].w;
        else lambda = (rv - B[i].w + (useBias ? C[i].w : 0.f)) * D[i].w;
        const float prev = A[i].w;
        float tot = prev + lambda;
        tot = fminG(tot, 0.f);
        lamN[i] = on ? tot : prev;
        lambda = tot - prev;
        const V3 nv0 = v0 + lambda * im0 * n, nw0 = w0 + lambda * ld3(C[i]);
        const V3 nv1 = v1 - lambda * im1 * n, nw1 = w1 - lambda * ld3(D[i]);
        if (on && b0 >= 0) { v0 = nv0; w0 = nw0; }
        if (on && b1 >= 0) { v1 = nv1; w1 = nw1; }
        touched |= on;
    }
    float4 E[4], F[4], G[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int q = i < np ? i : 0;
        E[i] = P[q].e; F[i] = P[q].f; G[i] = P[q].g;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const bool on = (live[i] & 2) != 0;
        const V3 t = ld3(E[i]);
        float lambda = F[i].w;
        const float limit = friction * lamN[i];
        const float prev = E[i].w;
        float tot = prev + lambda;
        tot = clampG(tot, limit, -limit);
        lamT[i] = tot;
        lambda = tot - prev;
        const V3 nv0 = v0 + lambda * im0 * t, nw0 = w0 + lambda * ld3(F[i]);
        const V3 nv1 = v1 - lambda * im1 * t, nw1 = w1 - lambda * ld3(G[i]);
        if (on && b0 >= 0) { v0 = nv0; w0 = nw0; }
        if (on && b1 >= 0) { v1 = nv1; w1 = nw1; }
        touched |= on;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (live[i] & 1) P[i].a.w = lamN[i];
        if (live[i] & 2) P[i].e.w = lamT[i];
    }
    if (touched) {
        if (b0 >= 0) { vr.sv(b0, v0); vr.sw(b0, w0); }
        if (b1 >= 0) { vr.sv(b1, v1); vr.sw(b1, w1); }
    }
}

// ---------------------------------------------------------------- bodies

// integrate velocities (src/Physecs.cpp:441-469)
__device__ void integrate_velocity(const World& w, int d, float h, float g, const VelRef& vr) {
    int b = w.dyn_body[d];
    if (w.info[b].y & BODY_KIN) return;
    M3 rot = mat3_cast(ld4(w.quat[b]));
    M3 invRot = transpose(rot);
    V3 vel = ld3(w.vel[d]) + h * V3{0, -g, 0};
    V3 ang = ld3(w.ang[d]);
    V3 wl = mv(invRot, ang);
    M3 invIl = m3cols(ld3(w.invI[3 * d]), ld3(w.invI[3 * d + 1]), ld3(w.invI[3 * d + 2]));
    M3 I = inverse(invIl);
    V3 f = h * cross(wl, mv(I, wl));
    M3 J = madd(I, mscale(h, msub(mm(matrixCross3(wl), I), matrixCross3(mv(I, wl)))));
    wl = wl - solve33(J, f);
    ang = mv(rot, wl);
    w.vel[d] = st4(vel);
    w.ang[d] = st4(ang);
    vr.sv(d, vel);
    vr.sw(d, ang);
    w.pv_v[d] = make_float4(0, 0, 0, 0);
    w.pv_w[d] = make_float4(0, 0, 0, 0);
    M3 wi = mm(mm(rot, invIl), invRot);
    w.mt[3 * d] = st4(wi.c[0]);
    w.mt[3 * d + 1] = st4(wi.c[1]);
    w.mt[3 * d + 2] = st4(wi.c[2]);
}

// integrate positions (src/Physecs.cpp:492-512)
__device__ void integrate_position(const World& w, int d, float h, const VelRef& vr) {
    int b = w.dyn_body[d];
    if (w.info[b].y & BODY_KIN) return;
    float4 pv = w.pv_v[d];
    float s = pv.w != 0.f ? 1.f / pv.w : 1.f;
    V3 pos = ld3(w.pos[b]);
    Q4 q = ld4(w.quat[b]);
    V3 com = ld3(w.com[d]);
    pos += h * vr.lv(d) + s * ld3(pv);
    V3 prevCom = qrot(q, com);
    V3 wv = 0.5f * (h * vr.lw(d) + s * ld3(w.pv_w[d]));
    q = qadd(q, qmul(Q4{wv.x, wv.y, wv.z, 0.f}, q));
    q = qnormalize(q);
    pos += prevCom - qrot(q, com);
    w.pos[b] = st4(pos);
    w.quat[b] = st4(q);
}

// ---------------------------------------------------------------- frame kernel

struct BlockSync {
    static constexpr bool kCluster = false;
    __device__ __forceinline__ void sync() const { __syncthreads(); }
    __device__ __forceinline__ int tid() const { return threadIdx.x; }
    __device__ __forceinline__ int nth() const { return blockDim.x; }
    __device__ __forceinline__ bool any(bool v) const { return __syncthreads_or(v) != 0; }
    // bit 0: a == true somewhere, bit 1: b == true somewhere
    __device__ __forceinline__ int any2(bool a, bool b) const {
        return (__syncthreads_or(a) ? 1 : 0) | (__syncthreads_or(b) ? 2 : 0);
    }
    // block-wide maximum of v (v >= -1)
    __device__ int max_int(int v) const {
        __shared__ int mx;
        if (threadIdx.x == 0) mx = -1;
        __syncthreads();
        atomicMax(&mx, v);
        __syncthreads();
        int r = mx;
        __syncthreads();
        return r;
    }
    // first point of each contact (colour order) packed without gaps; returns the point count
    __device__ int point_offsets(FrameBuf& f, int ms, int nc) const {
        __shared__ int part[513];   // solver blocks have at most 512 threads
        const int t = threadIdx.x, T = blockDim.x;
        const int chunk = (nc + T - 1) / T;
        const int k0 = min(nc, t * chunk), k1 = min(nc, k0 + chunk);
        int sum = 0;
        for (int k = k0; k < k1; ++k) sum += f.contacts[f.corder[ms + k]].np;
        part[t] = sum;
        __syncthreads();
        if (t == 0) {
            int acc = 0;
            for (int i = 0; i < T; ++i) { int v = part[i]; part[i] = acc; acc += v; }
            part[T] = acc;
        }
        __syncthreads();
        int acc = part[t];
        for (int k = k0; k < k1; ++k) { f.pt_off[ms + k] = acc; acc += f.contacts[f.corder[ms + k]].np; }
        const int total = part[T];
        __syncthreads();
        return total;
    }
};
struct GridSync {
    static constexpr bool kCluster = false;
    GridBarrier bar;
    int* flag;
    __device__ __forceinline__ void sync() const { bar.sync(); }
    __device__ __forceinline__ int tid() const { return blockIdx.x * blockDim.x + threadIdx.x; }
    __device__ __forceinline__ int nth() const { return gridDim.x * blockDim.x; }
    __device__ __forceinline__ bool any(bool v) const {
        if (threadIdx.x == 0 && blockIdx.x == 0) atomicExch(flag, 0);
        bar.sync();
        if (__syncthreads_or(v) && threadIdx.x == 0) atomicOr(flag, 1);
        bar.sync();
        bool r = *(volatile int*)flag != 0;
        bar.sync();
        return r;
    }
    __device__ __forceinline__ int any2(bool a, bool b) const { return (any(a) ? 1 : 0) | (any(b) ? 2 : 0); }
    // grid-wide maximum of v (v >= -1), through the barrier's spare word
    __device__ int max_int(int v) const {
        int* slot = flag + 1;
        if (threadIdx.x == 0 && blockIdx.x == 0) atomicExch(slot, -1);
        bar.sync();
        atomicMax(slot, v);
        bar.sync();
        int r = *(volatile int*)slot;
        bar.sync();
        return r;
    }
    // four point slots per contact (no cross-block scan in grid mode)
    __device__ int point_offsets(FrameBuf& f, int ms, int nc) const {
        for (int k = tid(); k < nc; k += nth()) f.pt_off[ms + k] = 4 * k;
        bar.sync();
        return 4 * nc;
    }
};

// A thread-block cluster working on one scene: the hardware cluster barrier orders
// shared, distributed-shared and global memory for all its threads; reductions go
// through a small array in block 0's shared memory.
struct ClusterSync {
    static constexpr bool kCluster = true;
    int rank, R, lg;
    float* const* bases;   // every block's dynamic shared memory, mapped
    int* red;              // R ints in block 0's shared memory, mapped
    __device__ __forceinline__ void sync() const { cooperative_groups::this_cluster().sync(); }
    __device__ __forceinline__ int tid() const { return rank * blockDim.x + threadIdx.x; }
    __device__ __forceinline__ int nth() const { return R * blockDim.x; }
    // cluster-wide bitwise OR of v's two low bits (__syncthreads_or only reports "nonzero")
    __device__ int reduce_or(int v) const {
        int b = (__syncthreads_or(v & 1) ? 1 : 0) | (__syncthreads_or(v & 2) ? 2 : 0);
        if (threadIdx.x == 0) red[rank] = b;
        sync();
        int r = 0;
        for (int i = 0; i < R; ++i) r |= red[i];
        sync();
        return r;
    }
    __device__ __forceinline__ bool any(bool v) const { return reduce_or(v ? 1 : 0) != 0; }
    __device__ __forceinline__ int any2(bool a, bool b) const { return reduce_or((a ? 1 : 0) | (b ? 2 : 0)); }
    __device__ int max_int(int v) const {
        __shared__ int bm;
        if (threadIdx.x == 0) bm = -1;
        __syncthreads();
        atomicMax(&bm, v);
        __syncthreads();
        if (threadIdx.x == 0) red[rank] = bm;
        sync();
        int r = -1;
        for (int i = 0; i < R; ++i) r = max(r, red[i]);
        sync();
        return r;
    }
    // four point slots per contact, as in grid mode
    __device__ int point_offsets(FrameBuf& f, int ms, int nc) const {
        for (int k = tid(); k < nc; k += nth()) f.pt_off[ms + k] = 4 * k;
        sync();
        return 4 * nc;
    }
};

// Colouring of one scene's contacts (see solve_scene): first fit, in rounds.  Every
// uncoloured contact proposes the lowest colour that neither of its dynamic bodies
// carries yet (a 128-bit mask per body); each body accepts the lowest proposal, ties
// going to a hashed priority of the contact's index within the scene; a contact
// accepted by both bodies takes its colour.  At most one contact per body is coloured
// per round, so no two contacts of a colour share a dynamic body, and the result does
// not depend on thread timing.  mask[d - ds], claim[d - ds], cb[k], col[k] are indexed
// by scene-local dynamic body and contact.  Contacts that find no colour below
// kMaxColors - 1 form a last colour that one thread solves in contact order; the
// return value is then negative.
template <class S>
__device__ int colour_contacts(const World& w, FrameBuf& f, int ms, int nc, int ds, int nd, const S& sy,
                               unsigned long long* claim, uint4* mask, int2* cb, int* col) {
    const int tid = sy.tid(), nth = sy.nth();
    const unsigned long long kFree = ~0ull;
    for (int d = tid; d < nd; d += nth) { claim[d] = kFree; mask[d] = make_uint4(0, 0, 0, 0); }
    for (int k = tid; k < nc; k += nth) {
        const Contact& c = f.contacts[ms + k];
        cb[k] = make_int2(c.b0 >= 0 ? c.b0 - ds : -1, c.b1 >= 0 ? c.b1 - ds : -1);
        col[k] = -1;
    }
    sy.sync();
    int ncol = 0;
    bool overflow = false;
    for (int round = 0;; ++round) {
        bool left = false, committed = false;
        for (int k = tid; k < nc; k += nth) {
            if (col[k] >= 0) continue;
            const int2 b = cb[k];
            uint4 m0 = b.x >= 0 ? mask[b.x] : make_uint4(0, 0, 0, 0);
            uint4 m1 = b.y >= 0 ? mask[b.y] : make_uint4(0, 0, 0, 0);
            unsigned u[4] = {m0.x | m1.x, m0.y | m1.y, m0.z | m1.z, m0.w | m1.w};
            int c = kMaxColors - 1;
            for (int q = 0; q < 4; ++q)
                if (~u[q]) { c = 32 * q + __ffs(~u[q]) - 1; break; }
            if (c >= kMaxColors - 1) continue;   // no colour left: the serial colour takes it
            unsigned long long v = ((unsigned long long)c << 40) |
                                   ((unsigned long long)(cache_hash((unsigned long long)k * 0x9E3779B97F4A7C15ull + round) & 0xffffu) << 24) |
                                   (unsigned)k;
            if (b.x >= 0) atomicMin(&claim[b.x], v);
            if (b.y >= 0) atomicMin(&claim[b.y], v);
        }
        sy.sync();
        for (int k = tid; k < nc; k += nth) {
            if (col[k] >= 0) continue;
            const int2 b = cb[k];
            unsigned long long v0 = b.x >= 0 ? claim[b.x] : kFree, v1 = b.y >= 0 ? claim[b.y] : kFree;
            bool mine0 = b.x < 0 || (v0 != kFree && (unsigned)(v0 & 0xffffffu) == (unsigned)k);
            bool mine1 = b.y < 0 || (v1 != kFree && (unsigned)(v1 & 0xffffffu) == (unsigned)k);
            if (b.x < 0 && b.y < 0) { col[k] = 0; committed = true; continue; }
            if (mine0 && mine1) {
                int c = (int)((b.x >= 0 ? v0 : v1) >> 40);
                col[k] = c;
                committed = true;
                // each body accepted only this contact this round: plain updates suffice
                unsigned bit = 1u << (c & 31);
                int q = c >> 5;
                if (b.x >= 0) { unsigned* mm = (unsigned*)&mask[b.x]; mm[q] |= bit; }
                if (b.y >= 0) { unsigned* mm = (unsigned*)&mask[b.y]; mm[q] |= bit; }
            } else {
                left = true;
            }
        }
        sy.sync();
        for (int d = tid; d < nd; d += nth) claim[d] = kFree;
        // the lowest proposal of a round always wins both its bodies, so a round without a
        // new colour means every open contact is out of colours
        int flags = sy.any2(left, committed);
        if (!(flags & 1)) break;
        if (!(flags & 2)) { overflow = true; break; }
    }
    // colours used; contacts left without one form a last colour, solved serially
    int top = -1;
    for (int k = tid; k < nc; k += nth) if (col[k] >= 0) top = max(top, col[k]);
    top = sy.max_int(top);
    ncol = top + 1;
    if (overflow) {
        for (int k = tid; k < nc; k += nth) if (col[k] < 0) col[k] = ncol;
        sy.sync();
        return -(ncol + 1);   // negative: the last colour is serial
    }
    return ncol;
}

template <class S>
__device__ void solve_scene(const World& w, FrameBuf& f, int s, const S& sy, float4* smem, int smem_f4) {
    if (w.scene_active && !w.scene_active[s]) return;
    const int tid = sy.tid(), nth = sy.nth();
    int ds = w.scene_dyn[s], de = w.scene_dyn[s + 1];
    int ms = f.scene_man[s], me = f.scene_man[s + 1];
    float4 kn = w.knobs[s];
    int substeps = (int)kn.x, iterations = (int)kn.y;
    float g = kn.z, dt = kn.w;
    int* colstart_g = f.color_start + s * (kMaxColors + 1);
    __shared__ int colstart[kMaxColors + 1];   // this block's copy, read by every colour step
    // ---- graph colouring of the contacts.  Each colour is a maximal set of contacts with
    // no dynamic body in common, grown in rounds: every uncoloured contact whose bodies
    // the colour does not hold yet claims them with a hashed priority, and the contacts
    // that hold all their bodies join the colour.  Priorities use the contact's index
    // within its scene, so a scene is coloured the same way whatever other scenes
    // share the world.  The working arrays (bodies of each contact, colour of each
    // contact, one claim word per dynamic body) live in shared memory when they fit.
    const int nd = de - ds, nc = me - ms;
    const bool col_smem = !S::kCluster && 24 * (size_t)nd + 12 * (size_t)nc <= 16 * (size_t)smem_f4;
    uint4* cmask = col_smem ? (uint4*)smem : f.cmask + ds;
    unsigned long long* claim = col_smem ? (unsigned long long*)(cmask + nd) : f.claim + ds;
    int2* cb = col_smem ? (int2*)(claim + nd) : f.cbody + ms;
    int* col = col_smem ? (int*)(cb + nc) : f.color_of + ms;
    int ncol = colour_contacts(w, f, ms, nc, ds, nd, sy, claim, cmask, cb, col);
    const bool serial_last = ncol < 0;
    if (serial_last) ncol = -ncol;
    // counting sort of the scene's contacts by colour
    for (int k = tid; k <= kMaxColors; k += nth) colstart_g[k] = 0;
    sy.sync();
    for (int k = tid; k < nc; k += nth) { int cl = col[k]; if (cl >= 0) atomicAdd(&colstart_g[cl + 1], 1); }
    sy.sync();
    if (tid == 0) {
        for (int k = 0; k < kMaxColors; ++k) colstart_g[k + 1] += colstart_g[k];
        f.scene_ncolor[s] = ncol;
    }
    sy.sync();
    for (int k = threadIdx.x; k <= kMaxColors; k += blockDim.x) colstart[k] = colstart_g[k];
    __syncthreads();
    for (int k = tid; k < nc; k += nth) {
        int cl = col[k];
        if (col_smem) f.color_of[ms + k] = cl;   // kept for inspection
        if (cl < 0 || (serial_last && cl == ncol - 1)) continue;
        // contacts of one colour touch disjoint bodies and may be solved in any order
        int pos = atomicAdd(&f.claim_pos[s * (kMaxColors + 1) + cl], 1);
        f.corder[ms + colstart[cl] + pos] = ms + k;
    }
    if (serial_last && tid == 0) {
        // the serial colour keeps contact order
        int pos = 0;
        for (int k = 0; k < nc; ++k) if (col[k] == ncol - 1) f.corder[ms + colstart[ncol - 1] + pos++] = ms + k;
    }
    sy.sync();
    // ---- where the substep data lives: velocities and contact records in shared memory
    // when they fit, velocities alone when only they fit, else the world's buffers
    const int ncl = colstart[kMaxColors];   // coloured contacts (all, unless the colour cap was hit)
    int npts = sy.point_offsets(f, ms, ncl);   // first point of each contact -> f.pt_off[ms + k]
    const int vel_f4 = (6 * nd + 3) / 4;
    const bool vel_smem = !S::kCluster && vel_f4 <= smem_f4;
    // contact headers in shared memory when they fit beside the velocities; point records
    // fill what is left, in colour order, up to the first contact whose points no longer
    // fit (contacts ks.. keep theirs in the world's buffer), so a scene slightly too big
    // for shared memory loses only its tail, not every record
    const bool hdr_smem = vel_smem && vel_f4 + kHdrF4 * ncl <= smem_f4;
    const int pbase_f4 = vel_f4 + (hdr_smem ? kHdrF4 * ncl : 0);
    const int pcap = vel_smem ? max(0, (smem_f4 - pbase_f4) / kPtF4) : 0;
    int ks = 0;
    if (vel_smem) {
        int fit = 0;
        for (int k = tid; k < ncl; k += nth) {
            const int end = k + 1 < ncl ? f.pt_off[ms + k + 1] : npts;
            if (end <= pcap) fit = k + 1;
        }
        ks = sy.max_int(fit);
    }
    VelRef vr = vel_smem ? VelRef{(float*)smem, nullptr, nullptr, nullptr, ds, nd, 0}
                         : VelRef{nullptr, nullptr, w.vt_v, w.vt_w, 0, 0, 0};
    if constexpr (S::kCluster) {
        // velocities spread over the cluster's blocks; records and colouring stay global
        const int per = (nd + sy.R - 1) >> sy.lg;
        if (6 * per <= 4 * smem_f4) vr = VelRef{nullptr, sy.bases, nullptr, nullptr, ds, per, sy.lg};
        else vr = VelRef{nullptr, nullptr, w.vt_v, w.vt_w, 0, 0, 0};
    }
    SHdr* H = hdr_smem ? (SHdr*)(smem + vel_f4) : f.s_hdr + ms;
    SPt* const Ps = (SPt*)(smem + pbase_f4);
    SPt* const Pg = f.s_pts + 4 * (size_t)ms;
    auto PK = [&](int k) -> SPt* { return (k < ks ? Ps : Pg) + H[k].i.w; };
    for (int k = tid; k < ncl; k += nth) H[k].i.w = f.pt_off[ms + k];
    sy.sync();
    int js0 = w.scene_jsteps[s], js1 = w.scene_jsteps[s + 1];
    int jb = w.scene_joint[s], je = w.scene_joint[s + 1];
    float h = dt / substeps;
    for (int sub = 0; sub < substeps; ++sub) {
        for (int k = tid; k < ncl; k += nth) contact_update(w, f.contacts[f.corder[ms + k]], H[k], PK(k));
        for (int j = jb + tid; j < je; j += nth) make_joint_rows(w, j);
        sy.sync();
        for (int d = ds + tid; d < de; d += nth) integrate_velocity(w, d, h, g, vr);
        sy.sync();
        for (int k = tid; k < ncl; k += nth) contact_presolve(w, H[k], PK(k), h);
        for (int st = js0; st < js1; ++st) {
            for (int k = w.jstep_start[st] + tid; k < w.jstep_start[st + 1]; k += nth) joint_presolve(w, w.jsched[k]);
            sy.sync();
        }
        sy.sync();
        for (int it = 0; it < iterations; ++it) {
            for (int cl = 0; cl < ncol; ++cl) {
                if (serial_last && cl == ncol - 1) {
                    if (tid == 0)
                        for (int k = colstart[cl]; k < colstart[cl + 1]; ++k) contact_solve(H[k], PK(k), true, vr);
                } else {
                    for (int k = colstart[cl] + tid; k < colstart[cl + 1]; k += nth) contact_solve(H[k], PK(k), true, vr);
                }
                sy.sync();
            }
            for (int st = js0; st < js1; ++st) {
                for (int k = w.jstep_start[st] + tid; k < w.jstep_start[st + 1]; k += nth) joint_solve(w, w.jsched[k], h, it == 0, vr);
                sy.sync();
            }
        }
        for (int d = ds + tid; d < de; d += nth) integrate_position(w, d, h, vr);
        sy.sync();
        for (int cl = 0; cl < ncol; ++cl) {
            if (serial_last && cl == ncol - 1) {
                if (tid == 0)
                    for (int k = colstart[cl]; k < colstart[cl + 1]; ++k)
                        if (!(H[k].i.z >> 8)) contact_solve(H[k], PK(k), false, vr);
            } else {
                for (int k = colstart[cl] + tid; k < colstart[cl + 1]; k += nth)
                    if (!(H[k].i.z >> 8)) contact_solve(H[k], PK(k), false, vr);
            }
            sy.sync();
        }
        for (int d = ds + tid; d < de; d += nth) {
            int b = w.dyn_body[d];
            if (w.info[b].y & BODY_KIN) continue;
            w.vel[d] = st4(vr.lv(d));
            w.ang[d] = st4(vr.lw(d));
        }
        sy.sync();
    }
    // accumulated impulses back into the frame's contacts (inspection only)
    for (int k = tid; k < ncl; k += nth) {
        Contact& c = f.contacts[f.corder[ms + k]];
        const SPt* q = PK(k);
        for (int i = 0; i < c.np; ++i) { c.p[i].r0xn.w = q[i].a.w; c.p[i].r1xn.w = q[i].e.w; }
    }
}

// one scene per block; NT = 32 or 64, 128 or 256 for scenes up to 1024 dynamic bodies (by size), 512 above
template <int NT>
__global__ void __launch_bounds__(NT, 512 / NT) k_solve_block(World w, FrameBuf f, const int* scenes, int smem_f4) {
    extern __shared__ float4 smem[];
    BlockSync sy;
    solve_scene(w, f, scenes[blockIdx.x], sy, smem, smem_f4);
}

static_assert(kBarrierTimeoutBit == ERR_BARRIER_TIMEOUT, "grid barrier error bit");

__global__ void __launch_bounds__(256, 2) k_solve_grid(World w, FrameBuf f, const int* scenes, int n, long long limit) {
    GridSync sy{GridBarrier{f.bar, f.bar + 1, w.err, limit}, (int*)(f.bar + 2)};
    for (int i = 0; i < n; ++i) {
        solve_scene(w, f, scenes[i], sy, nullptr, 0);
        sy.sync();
    }
}

// one cluster of kClusterBlocks blocks per large scene, velocities in distributed shared memory
template <int NT>
__global__ void __launch_bounds__(NT, 1) k_solve_cluster(World w, FrameBuf f, const int* scenes, int smem_f4) {
    extern __shared__ float4 smem[];
    __shared__ float* bases[kClusterBlocks];
    __shared__ int red[kClusterBlocks];
    cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
    const int R = (int)cl.num_blocks(), rank = (int)cl.block_rank();
    if (threadIdx.x < R) bases[threadIdx.x] = cl.map_shared_rank((float*)smem, (int)threadIdx.x);
    int* red0 = cl.map_shared_rank(red, 0);
    int lg = 0;
    while ((1 << lg) < R) ++lg;
    cl.sync();
    ClusterSync sy{rank, R, lg, bases, red0};
    solve_scene(w, f, scenes[blockIdx.x / R], sy, smem, smem_f4);
    cl.sync();   // no block leaves while the others may still read its shared memory
}

__global__ void k_zero_ints(int* p, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = 0;
}

int launch_contacts(const World& w, FrameBuf& f, cudaStream_t s) {
    k_cache_clear<<<(f.cache_cap + 255) / 256, 256, 0, s>>>(f);
    k_zero_ints<<<(w.n_scenes + 256) / 256, 256, 0, s>>>(f.man_scene_cnt, w.n_scenes + 1);
    k_zero_ints<<<1, 32, 0, s>>>(f.n_points, 1);
    k_build_contacts<<<1216, 128, 0, s>>>(w, f);
    scan_exclusive(f.man_scene_cnt, f.scene_man, w.n_scenes + 1, nullptr, f.scan_scratch, s);
    return 4 + 3;
}

int solver_grid_blocks() {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_solve_grid, 256, 0);
    if (per < 1) per = 1;
    return sms * per;
}

// The dynamic shared memory a kernel may use is a per-device attribute: it is set on
// the current device whenever a launch there asks for more than was set before.
constexpr int kMaxDevices = 64;

static void set_kernel_smem(const void* fn, int* done, int bytes) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxDevices) return;
    if (done[dev] < bytes) {
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        done[dev] = bytes;
    }
}

template <int NT>
static void set_smem(int bytes) {
    static int done[kMaxDevices] = {};
    set_kernel_smem((const void*)k_solve_block<NT>, done, bytes);
}

// A solver launch at a scheduling priority: `rank` 0 is the device's highest, each step
// one lower, down to the lowest (the priority is a launch attribute, so a CUDA graph
// captured from it keeps it).  The larger the scenes of a launch, the longer their
// chains and the earlier their blocks should start.
template <int NT>
static void launch_block_ranked(int grid, int smem, cudaStream_t st, int rank, const World& w, FrameBuf& f,
                                const int* scenes) {
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributePriority;
    attr[0].val.priority = greatest < least ? std::min(least, greatest + rank) : greatest;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_solve_block<NT>, w, f, scenes, smem / 16);
}

int launch_solver(const World& w, FrameBuf& f, const SolverLaunch& L, cudaStream_t s) {
    k_zero_ints<<<(w.n_scenes * (kMaxColors + 1) + 255) / 256, 256, 0, s>>>(f.claim_pos, w.n_scenes * (kMaxColors + 1));
    int k = 2;
    // large scenes on a second stream, concurrently with the small ones, and first: their
    // chains are the longest (measured with eager launches: solver stage 7.20 -> 6.65 ms
    // on the 4096-scene frame)
    if (L.n_large) {
        cudaEventRecord(L.fork, s);
        cudaStreamWaitEvent(L.aux, L.fork, 0);
        if (L.large_nt == 128 || L.large_nt == 256) {
            // several blocks an SM, each with its share of the SM's shared memory (beside
            // each block's 1 KB reserve and its static shared memory)
            const int per = L.large_nt == 128 ? 4 : 2;
            const int smem = (L.smem_large + 5120 - per * 6144) / per / 16 * 16;
            if (L.large_nt == 128) {
                set_smem<128>(smem);
                launch_block_ranked<128>(L.n_large, smem, L.aux, 0, w, f, L.large);
            } else {
                set_smem<256>(smem);
                launch_block_ranked<256>(L.n_large, smem, L.aux, 0, w, f, L.large);
            }
        } else {
            set_smem<512>(L.smem_large);
            launch_block_ranked<512>(L.n_large, L.smem_large, L.aux, 0, w, f, L.large);
        }
        cudaEventRecord(L.join, L.aux);
        ++k;
    }
    // block scenes: 64- and 128-thread tiers on their own streams beside the 256-thread one
    if (L.n_tier[0] || L.n_tier[1]) cudaEventRecord(L.tfork, s);
    if (L.n_tier[0]) {
        cudaStreamWaitEvent(L.tstream[0], L.tfork, 0);
        if (L.tier0_nt == 32) {   // one warp a scene: up to 16 scenes an SM
            set_smem<32>(L.smem_tier[0]);
            launch_block_ranked<32>(L.n_tier[0], L.smem_tier[0], L.tstream[0], 3, w, f, L.tier[0]);
        } else {
            set_smem<64>(L.smem_tier[0]);
            launch_block_ranked<64>(L.n_tier[0], L.smem_tier[0], L.tstream[0], 3, w, f, L.tier[0]);
        }
        cudaEventRecord(L.tjoin[0], L.tstream[0]);
        ++k;
    }
    if (L.n_tier[1]) {
        set_smem<128>(L.smem_tier[1]);
        cudaStreamWaitEvent(L.tstream[1], L.tfork, 0);
        launch_block_ranked<128>(L.n_tier[1], L.smem_tier[1], L.tstream[1], 2, w, f, L.tier[1]);
        cudaEventRecord(L.tjoin[1], L.tstream[1]);
        ++k;
    }
    if (L.n_tier[2]) {
        set_smem<256>(L.smem_tier[2]);
        launch_block_ranked<256>(L.n_tier[2], L.smem_tier[2], s, 1, w, f, L.tier[2]);
        ++k;
    }
    if (L.n_tier[0]) cudaStreamWaitEvent(s, L.tjoin[0], 0);
    if (L.n_tier[1]) cudaStreamWaitEvent(s, L.tjoin[1], 0);
    if (L.n_large) cudaStreamWaitEvent(s, L.join, 0);
    if (L.n_cluster) {
        static int cluster_smem[kMaxDevices] = {};
        set_kernel_smem((const void*)k_solve_cluster<512>, cluster_smem, L.smem_large);
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(kClusterBlocks * L.n_cluster);
        cfg.blockDim = dim3(512);
        cfg.dynamicSmemBytes = L.smem_large;
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = kClusterBlocks;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        cudaLaunchKernelEx(&cfg, k_solve_cluster<512>, w, f, L.cluster, L.smem_large / 16);
        ++k;
    }
    if (L.n_grid) {
        World wc = w;
        FrameBuf fc = f;
        const int* gs = L.grid;
        int ng = L.n_grid;
        long long limit = L.wait_limit > 0 ? L.wait_limit : kDefaultWaitPolls;
        // the barrier's words start from zero in every launch, whatever an earlier launch
        // that gave up on a wait left in them
        cudaMemsetAsync(f.bar, 0, 4 * sizeof(unsigned), s);
        void* args[] = {(void*)&wc, (void*)&fc, (void*)&gs, (void*)&ng, (void*)&limit};
        cudaLaunchCooperativeKernel((void*)k_solve_grid, L.grid_blocks, 256, args, 0, s);
        ++k;
    }
    k_cache_flip<<<1, 1, 0, s>>>(f);
    return k;
}

}  // namespace psx
