/*
 * gjk_epa.cpp — support mappings, GJK and EPA of the CPU oracle.
 * ORACLE (test infrastructure only; see omath.h).
 *
 * Restates src/GJK.h:13-292 and src/EPA.h:10-186 including their mixed
 * precision: supports are single precision, the simplex and the polytope are
 * double precision, and every place where the reference passes a dvec3 into a
 * glm::vec3 parameter rounds to float here too.
 */
#include "collide_util.h"
#include <limits>

namespace orc {

// GJK.h:13-128
V3 Support::operator()(V3 dir) const {
    switch (kind) {
        case 0: return pos + dir * radius;
        case 1: return pos + axis * signG(dot(dir, axis)) * halfHeight + dir * radius;
        case 2: {
            V3 s = pos;
            for (int i = 0; i < 3; ++i) s += signG(dot(dir, basis.c[i])) * basis.c[i] * at(he, i);
            return s;
        }
        case 3: {
            V3 d = scale * multiplyTranspose(basis, dir);
            // four lanes scan vertices i, i+4, ...: strict '>' keeps the first
            // maximum per lane, then lanes 1..3 replace lane 0 only on '>' (GJK.h:56-105)
            float best[4];
            int bi[4];
            for (int l = 0; l < 4; ++l) { best[l] = std::numeric_limits<float>::lowest(); bi[l] = l; }
            int n = (int)mesh->buffer.size();
            for (int i = 0; i < n; i += 4) {
                for (int l = 0; l < 4; ++l) {
                    V3 v = mesh->buffer[i + l];
                    float dp = (v.x * d.x + v.y * d.y) + v.z * d.z;
                    if (dp > best[l]) bi[l] = i + l;
                    best[l] = (dp > best[l]) ? dp : best[l];   // _mm_max_ps(dot, max)
                }
            }
            int mi = bi[0];
            float mvv = best[0];
            for (int l = 1; l < 4; ++l) if (best[l] > mvv) { mvv = best[l]; mi = bi[l]; }
            return pos + mv(basis, scale * mesh->buffer[mi]);
        }
        default: {
            if (dot(dir, a) > dot(dir, b)) {
                if (dot(dir, a) > dot(dir, c)) return a;
                return c;
            }
            if (dot(dir, b) > dot(dir, c)) return b;
            return c;
        }
    }
}

static GjkVertex mink(const Support& s0, const Support& s1, V3 dir) {
    V3 a = s0(dir);
    V3 b = s1(-dir);
    return {d3(a - b), d3(a), d3(b)};
}

static float sqrDistPointToLine(V3 p, V3 a, V3 b) {
    V3 r = p - a, d = b - a;
    V3 q = a + dot(r, d) / dot(d, d) * d;
    V3 pq = p - q;
    return dot(pq, pq);
}
static float distPointToPlane(V3 p, V3 o, V3 n) { return std::fabs(dot(p - o, n)); }
static bool isZeroF(V3 v) { return (double)length2(v) < 1e-6; }

static bool checkDirection(const Support& s0, const Support& s1, D3 dir, GjkVertex& v) {
    dir = normalize(dir);
    v = mink(s0, s1, f3(dir));
    return dot(v.pos, dir) >= 0;
}

static bool checkFace(D3 v0, D3 v1, D3 v2, D3 opposite, D3& n) {
    n = cross(v1 - v0, v2 - v0);
    n = signD(dot(v0 - opposite, n)) * n;
    return dot(n, -v0) > (double)0.00001f;
}

static bool containsOrigin(GjkSimplex& s, D3& dir, int& fi) {
    fi = 2;
    if (checkFace(s.v[3].pos, s.v[0].pos, s.v[1].pos, s.v[fi].pos, dir)) return false;
    if (checkFace(s.v[3].pos, s.v[2].pos, s.v[0].pos, s.v[--fi].pos, dir)) return false;
    if (checkFace(s.v[3].pos, s.v[1].pos, s.v[2].pos, s.v[--fi].pos, dir)) return false;
    return true;
}

// completes a degenerate simplex around an origin on the line v0v1 (GJK.h:233-246, 253-265)
static void completeFromLine(const Support& s0, const Support& s1, GjkSimplex& s) {
    D3 dir = cross(s.v[0].pos - s.v[1].pos, D3{0, 1, 0});
    if (isZeroF(f3(dir))) dir = cross(s.v[0].pos - s.v[1].pos, D3{0, 0, 1});
    s.v[2] = mink(s0, s1, f3(normalize(dir)));
    if (sqrDistPointToLine(f3(s.v[2].pos), f3(s.v[0].pos), f3(s.v[1].pos)) < 0.00001f) s.v[2] = mink(s0, s1, f3(-dir));
    dir = normalize(cross(s.v[1].pos - s.v[0].pos, s.v[2].pos - s.v[0].pos));
    s.v[3] = mink(s0, s1, f3(dir));
    if (distPointToPlane(f3(s.v[3].pos), f3(s.v[0].pos), f3(dir)) < 0.0001f) s.v[3] = mink(s0, s1, f3(-dir));
}

// GJK.h:226-292
bool gjk(const Support& s0, const Support& s1, V3 startDir, GjkSimplex& s) {
    D3 dir = d3(normalize(startDir));
    s.v[0] = mink(s0, s1, f3(dir));
    if (isZeroF(f3(s.v[0].pos))) {
        dir = -dir;
        s.v[1] = mink(s0, s1, f3(dir));
        completeFromLine(s0, s1, s);
        return true;
    }
    dir = -s.v[0].pos;
    if (!checkDirection(s0, s1, dir, s.v[1])) return false;
    dir = cross(cross(s.v[0].pos - s.v[1].pos, -s.v[1].pos), s.v[0].pos - s.v[1].pos);
    if (isZeroF(f3(dir))) {
        completeFromLine(s0, s1, s);
        return true;
    }
    if (!checkDirection(s0, s1, dir, s.v[2])) return false;
    dir = cross(s.v[1].pos - s.v[0].pos, s.v[2].pos - s.v[0].pos);
    double sg = signD(dot(-s.v[0].pos, dir));
    if (!sg) {
        dir = normalize(dir);
        s.v[3] = mink(s0, s1, f3(dir));
        if (distPointToPlane(f3(s.v[3].pos), f3(s.v[0].pos), f3(dir)) < 0.0001f) s.v[3] = mink(s0, s1, f3(-dir));
        return true;
    }
    dir = sg * dir;
    if (!checkDirection(s0, s1, dir, s.v[3])) return false;
    int fi;
    for (int i = 0; i < 100; ++i) {
        if (containsOrigin(s, dir, fi)) return true;
        if (!checkDirection(s0, s1, dir, s.v[fi])) return false;
        GjkVertex t = s.v[fi];
        s.v[fi] = s.v[3];
        s.v[3] = t;
    }
    return false;
}

// ---------------------------------------------------------------- EPA (EPA.h)

namespace {
constexpr int kMaxVerts = 4 + 100;
constexpr int kMaxFaces = 2 * kMaxVerts + 8;
constexpr int kMaxEdges = 3 * kMaxFaces;
struct Face { int i[3]; D3 n; };
struct Polytope {
    GjkVertex v[kMaxVerts];
    int nv = 0;
    Face f[kMaxFaces];
    int nf = 0;
    void createFace(int i0, int i1, int i2) {
        D3 n = cross(v[i0].pos - v[i1].pos, v[i2].pos - v[i1].pos);
        double len = length(n);
        if (len) n = n / len;
        if (nf < kMaxFaces) f[nf++] = {{i0, i1, i2}, n};
    }
    void destroyFace(int k) { f[k] = f[nf - 1]; --nf; }
    double dist(const Face& fc) const { return dot(v[fc.i[0]].pos, fc.n); }
    void findClosest(float& distance, D3& n, int& fi) const {
        distance = (float)std::numeric_limits<double>::max();
        for (int k = 0; k < nf; ++k) {
            double d = dist(f[k]);
            if (d < distance) { distance = (float)d; n = f[k].n; fi = k; }
        }
    }
    void insert(const GjkVertex& p) {
        int e0[kMaxEdges], e1[kMaxEdges];
        int ne = 0;
        for (int k = nf - 1; k >= 0; --k) {
            Face& fc = f[k];
            if (dot(fc.n, p.pos - v[fc.i[0]].pos) > 0) {
                int a[3] = {fc.i[0], fc.i[1], fc.i[2]}, b[3] = {fc.i[1], fc.i[2], fc.i[0]};
                bool found[3] = {false, false, false};
                for (int j = 0; j < 3; ++j) {
                    for (int q = ne - 1; q >= 0; --q) {
                        if (e0[q] == b[j] && e1[q] == a[j]) {
                            found[j] = true;
                            e0[q] = e0[ne - 1]; e1[q] = e1[ne - 1]; --ne;
                            break;
                        }
                    }
                }
                for (int j = 0; j < 3; ++j) if (!found[j] && ne < kMaxEdges) { e0[ne] = a[j]; e1[ne] = b[j]; ++ne; }
                destroyFace(k);
            }
        }
        if (nv >= kMaxVerts) return;
        int vi = nv;
        v[nv++] = p;
        for (int q = 0; q < ne; ++q) createFace(vi, e0[q], e1[q]);
    }
    void closestPoints(int fi, V3& cp0, V3& cp1) const {
        const Face& fc = f[fi];
        const GjkVertex& a = v[fc.i[0]];
        const GjkVertex& b = v[fc.i[1]];
        const GjkVertex& c = v[fc.i[2]];
        D3 proj = fc.n + dist(fc);   // EPA.h:108 adds the distance to every component
        V3 v0 = f3(b.pos - a.pos), v1 = f3(c.pos - a.pos), v2 = f3(proj - a.pos);
        double d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1), d20 = dot(v2, v0), d21 = dot(v2, v1);
        double denom = d00 * d11 - d01 * d01;
        double u, vv, w;
        if (denom) {
            vv = (d20 * d11 - d21 * d01) / denom;
            w = (d00 * d21 - d01 * d20) / denom;
            u = 1.0f - vv - w;
        } else {
            w = 0;
            if (d00) { vv = d20 / d00; u = 1.0f - vv; }
            else { vv = 0; u = 1.0; }
        }
        cp0 = f3(u * a.sp0 + vv * b.sp0 + w * c.sp0);
        cp1 = f3(u * a.sp1 + vv * b.sp1 + w * c.sp1);
    }
};
}  // namespace

// EPA.h:170-186
V3 epa(const Support& s0, const Support& s1, GjkSimplex& s, V3& cp0, V3& cp1) {
    static thread_local Polytope p;
    p.nv = 0; p.nf = 0;
    for (int i = 0; i < 4; ++i) p.v[p.nv++] = s.v[i];
    D3 n = cross(p.v[0].pos - p.v[1].pos, p.v[2].pos - p.v[1].pos);
    if (dot(p.v[3].pos - p.v[0].pos, n) < 0) {
        p.createFace(0, 1, 2); p.createFace(3, 1, 0); p.createFace(3, 2, 1); p.createFace(3, 0, 2);
    } else {
        p.createFace(0, 2, 1); p.createFace(3, 2, 0); p.createFace(3, 1, 2); p.createFace(3, 0, 1);
    }
    float minDist;
    D3 normal{0, 0, 0};
    int fi = 0;
    for (int i = 0; i < 100; ++i) {
        p.findClosest(minDist, normal, fi);
        GjkVertex v = mink(s0, s1, f3(normal));
        if (dot(v.pos, normal) - minDist < (double)0.00001f) break;
        p.insert(v);
    }
    p.closestPoints(fi, cp0, cp1);
    return f3(normal);
}

}  // namespace orc
