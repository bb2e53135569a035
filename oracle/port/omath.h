/*
 * omath.h — scalar vector / quaternion / matrix helpers for the CPU oracle.
 *
 * ORACLE (test infrastructure): only tests, smoke() and bench.py's CPU
 * baseline use oracle/.  Each helper evaluates its floating-point operations
 * in the same order as the GLM 0.9.9.8 function the reference calls, so that
 * oracle results can be compared with the reference bit for bit:
 *   dot      (x*x + y*y) + z*z                     glm/detail/func_geometric.inl compute_dot
 *   cross    x.y*y.z - y.y*x.z, ...                compute_cross
 *   q * v    v + ((uv*w) + uuv) * 2                glm/detail/type_quat.inl operator*
 *   mat3(q)  1 - 2(yy+zz), 2(xy+wz), ...           glm/gtc/quaternion.inl mat3_cast
 *   M * v    (m00*x + m10*y) + m20*z               glm/detail/type_mat3x3.inl
 *   inverse  cofactors * (1/det)                   glm/detail/func_matrix.inl
 *   min/max  (y < x) ? y : x / (x < y) ? y : x     glm/detail/func_common.inl
 * Compile with -ffp-contract=off.
 */
#pragma once
#include <cmath>
#include <cfloat>

namespace orc {

struct V3 { float x, y, z; };
struct D3 { double x, y, z; };
struct Q4 { float x, y, z, w; };
struct M3 { V3 c[3]; };   // column-major, like glm::mat3
struct V2 { float x, y; };

inline V3 v3(float x, float y, float z) { return {x, y, z}; }
inline V3 v3s(float s) { return {s, s, s}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline V3 operator/(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline V3 operator+(V3 a, float s) { return {a.x + s, a.y + s, a.z + s}; }
inline V3 operator-(V3 a, float s) { return {a.x - s, a.y - s, a.z - s}; }
inline V3& operator+=(V3& a, V3 b) { a = a + b; return a; }
inline V3& operator-=(V3& a, V3 b) { a = a - b; return a; }
inline float& at(V3& v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
inline float at(const V3& v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

inline float dot(V3 a, V3 b) { V3 t = a * b; return t.x + t.y + t.z; }
inline V3 cross(V3 x, V3 y) { return {x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y}; }
inline float length(V3 v) { return std::sqrt(dot(v, v)); }
inline float length2(V3 v) { return dot(v, v); }
inline float distance(V3 a, V3 b) { return length(a - b); }
inline float distance2(V3 a, V3 b) { return length2(b - a); }
inline V3 normalize(V3 v) { return v * (1.f / std::sqrt(dot(v, v))); }
inline float fminG(float x, float y) { return (y < x) ? y : x; }
inline float fmaxG(float x, float y) { return (x < y) ? y : x; }
inline float clampG(float x, float lo, float hi) { return fminG(fmaxG(x, lo), hi); }
inline V3 vmin(V3 a, V3 b) { return {fminG(a.x, b.x), fminG(a.y, b.y), fminG(a.z, b.z)}; }
inline V3 vmax(V3 a, V3 b) { return {fmaxG(a.x, b.x), fmaxG(a.y, b.y), fmaxG(a.z, b.z)}; }
inline V3 vclamp(V3 x, V3 lo, V3 hi) { return vmin(vmax(x, lo), hi); }
inline V3 vabs(V3 a) { return {std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)}; }
inline float signG(float x) { return (float)(0.f < x) - (float)(x < 0.f); }
inline double signD(double x) { return (double)(0.0 < x) - (double)(x < 0.0); }
inline float mixG(float x, float y, float a) { return x * (1.f - a) + y * a; }
inline float det2(V2 c0, V2 c1) { return c0.x * c1.y - c1.x * c0.y; }
inline V2 operator-(V2 a, V2 b) { return {a.x - b.x, a.y - b.y}; }
inline V2 operator+(V2 a, V2 b) { return {a.x + b.x, a.y + b.y}; }
inline V2 operator-(V2 a) { return {-a.x, -a.y}; }
inline V2 operator*(float s, V2 a) { return {s * a.x, s * a.y}; }

inline D3 d3(V3 v) { return {(double)v.x, (double)v.y, (double)v.z}; }
inline V3 f3(D3 v) { return {(float)v.x, (float)v.y, (float)v.z}; }
inline D3 operator+(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 operator-(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 operator-(D3 a) { return {-a.x, -a.y, -a.z}; }
inline D3 operator*(D3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline D3 operator*(double s, D3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline D3 operator/(D3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
inline D3 operator+(D3 a, double s) { return {a.x + s, a.y + s, a.z + s}; }
inline double dot(D3 a, D3 b) { D3 t = {a.x * b.x, a.y * b.y, a.z * b.z}; return t.x + t.y + t.z; }
inline D3 cross(D3 x, D3 y) { return {x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y}; }
inline double length(D3 v) { return std::sqrt(dot(v, v)); }
inline D3 normalize(D3 v) { return v * (1.0 / std::sqrt(dot(v, v))); }

// quaternion (glm::quat), stored x, y, z, w
inline Q4 q4(float w, float x, float y, float z) { return {x, y, z, w}; }
inline Q4 qmul(Q4 p, Q4 q) {
    return {p.w * q.x + p.x * q.w + p.y * q.z - p.z * q.y,
            p.w * q.y + p.y * q.w + p.z * q.x - p.x * q.z,
            p.w * q.z + p.z * q.w + p.x * q.y - p.y * q.x,
            p.w * q.w - p.x * q.x - p.y * q.y - p.z * q.z};
}
inline V3 qrot(Q4 q, V3 v) {
    V3 qv = {q.x, q.y, q.z};
    V3 uv = cross(qv, v);
    V3 uuv = cross(qv, uv);
    return v + ((uv * q.w) + uuv) * 2.f;
}
inline float qdot(Q4 a, Q4 b) {
    float w = a.w * b.w, x = a.x * b.x, y = a.y * b.y, z = a.z * b.z;
    return (w + x) + (y + z);
}
inline Q4 qinverse(Q4 q) {
    float d = qdot(q, q);
    return {-q.x / d, -q.y / d, -q.z / d, q.w / d};
}
inline Q4 qnormalize(Q4 q) {
    float len = std::sqrt(qdot(q, q));
    if (len <= 0.f) return {0.f, 0.f, 0.f, 1.f};
    float o = 1.f / len;
    return {q.x * o, q.y * o, q.z * o, q.w * o};
}
inline Q4 qadd(Q4 a, Q4 b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }

inline M3 m3cols(V3 a, V3 b, V3 c) { return {{a, b, c}}; }
inline M3 m3zero() { return {{{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}}; }
inline M3 m3diag(float s) { return {{{s, 0, 0}, {0, s, 0}, {0, 0, s}}}; }
inline M3 mat3_cast(Q4 q) {
    float qxx = q.x * q.x, qyy = q.y * q.y, qzz = q.z * q.z;
    float qxz = q.x * q.z, qxy = q.x * q.y, qyz = q.y * q.z;
    float qwx = q.w * q.x, qwy = q.w * q.y, qwz = q.w * q.z;
    M3 r;
    r.c[0] = {1.f - 2.f * (qyy + qzz), 2.f * (qxy + qwz), 2.f * (qxz - qwy)};
    r.c[1] = {2.f * (qxy - qwz), 1.f - 2.f * (qxx + qzz), 2.f * (qyz + qwx)};
    r.c[2] = {2.f * (qxz + qwy), 2.f * (qyz - qwx), 1.f - 2.f * (qxx + qyy)};
    return r;
}
inline V3 mv(const M3& m, V3 v) {
    return {m.c[0].x * v.x + m.c[1].x * v.y + m.c[2].x * v.z,
            m.c[0].y * v.x + m.c[1].y * v.y + m.c[2].y * v.z,
            m.c[0].z * v.x + m.c[1].z * v.y + m.c[2].z * v.z};
}
inline M3 mm(const M3& a, const M3& b) {
    M3 r;
    for (int j = 0; j < 3; ++j) {
        V3 bj = b.c[j];
        r.c[j] = {a.c[0].x * bj.x + a.c[1].x * bj.y + a.c[2].x * bj.z,
                  a.c[0].y * bj.x + a.c[1].y * bj.y + a.c[2].y * bj.z,
                  a.c[0].z * bj.x + a.c[1].z * bj.y + a.c[2].z * bj.z};
    }
    return r;
}
inline M3 transpose(const M3& m) {
    return {{{m.c[0].x, m.c[1].x, m.c[2].x}, {m.c[0].y, m.c[1].y, m.c[2].y}, {m.c[0].z, m.c[1].z, m.c[2].z}}};
}
inline M3 madd(const M3& a, const M3& b) { return {{a.c[0] + b.c[0], a.c[1] + b.c[1], a.c[2] + b.c[2]}}; }
inline M3 msub(const M3& a, const M3& b) { return {{a.c[0] - b.c[0], a.c[1] - b.c[1], a.c[2] - b.c[2]}}; }
inline M3 mscale(float s, const M3& a) { return {{s * a.c[0], s * a.c[1], s * a.c[2]}}; }
inline float m(const M3& a, int c, int r) { return at(a.c[c], r); }
inline float determinant(const M3& a) {
    return +m(a, 0, 0) * (m(a, 1, 1) * m(a, 2, 2) - m(a, 2, 1) * m(a, 1, 2))
           - m(a, 1, 0) * (m(a, 0, 1) * m(a, 2, 2) - m(a, 2, 1) * m(a, 0, 2))
           + m(a, 2, 0) * (m(a, 0, 1) * m(a, 1, 2) - m(a, 1, 1) * m(a, 0, 2));
}
inline M3 inverse(const M3& a) {
    float o = 1.f / (+m(a, 0, 0) * (m(a, 1, 1) * m(a, 2, 2) - m(a, 2, 1) * m(a, 1, 2))
                     - m(a, 1, 0) * (m(a, 0, 1) * m(a, 2, 2) - m(a, 2, 1) * m(a, 0, 2))
                     + m(a, 2, 0) * (m(a, 0, 1) * m(a, 1, 2) - m(a, 1, 1) * m(a, 0, 2)));
    M3 r;
    r.c[0].x = +(m(a, 1, 1) * m(a, 2, 2) - m(a, 2, 1) * m(a, 1, 2)) * o;
    r.c[1].x = -(m(a, 1, 0) * m(a, 2, 2) - m(a, 2, 0) * m(a, 1, 2)) * o;
    r.c[2].x = +(m(a, 1, 0) * m(a, 2, 1) - m(a, 2, 0) * m(a, 1, 1)) * o;
    r.c[0].y = -(m(a, 0, 1) * m(a, 2, 2) - m(a, 2, 1) * m(a, 0, 2)) * o;
    r.c[1].y = +(m(a, 0, 0) * m(a, 2, 2) - m(a, 2, 0) * m(a, 0, 2)) * o;
    r.c[2].y = -(m(a, 0, 0) * m(a, 2, 1) - m(a, 2, 0) * m(a, 0, 1)) * o;
    r.c[0].z = +(m(a, 0, 1) * m(a, 1, 2) - m(a, 1, 1) * m(a, 0, 2)) * o;
    r.c[1].z = -(m(a, 0, 0) * m(a, 1, 2) - m(a, 1, 0) * m(a, 0, 2)) * o;
    r.c[2].z = +(m(a, 0, 0) * m(a, 1, 1) - m(a, 1, 0) * m(a, 0, 1)) * o;
    return r;
}
// glm::matrixCross3 (glm/gtx/matrix_cross_product.inl)
inline M3 matrixCross3(V3 x) {
    M3 r = m3zero();
    r.c[0].y = x.z; r.c[1].x = -x.z; r.c[0].z = -x.y; r.c[2].x = x.y; r.c[1].z = x.x; r.c[2].y = -x.x;
    return r;
}
// MathUtil.h:6-8 multiplyTranspose, :10-21 solve33
inline V3 multiplyTranspose(const M3& a, V3 v) { return {dot(v, a.c[0]), dot(v, a.c[1]), dot(v, a.c[2])}; }
inline V3 solve33(const M3& A, V3 b) {
    V3 c12 = cross(A.c[1], A.c[2]);
    float det = dot(A.c[0], c12);
    if (det == 0.f) return {0, 0, 0};
    float inv = 1.f / det;
    return {inv * dot(b, c12), inv * dot(A.c[0], cross(b, A.c[2])), inv * dot(A.c[0], cross(A.c[1], b))};
}

struct Bounds { V3 min, max; };

}  // namespace orc
