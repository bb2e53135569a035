// dmath.cuh — vector / quaternion / 3x3 matrix arithmetic for the device kernels.
//
// Every function evaluates its float operations in the order of the GLM 0.9.9.8
// function the Physecs reference calls (dot = (x*x + y*y) + z*z, quat * vec =
// v + ((uv*w) + uuv) * 2, mat3_cast, column-major mat3 * vec3, cofactor inverse).
// The library is compiled with -fmad=false and IEEE division / square root, so a
// kernel built on these helpers rounds exactly like the reference's CPU code.
#pragma once
#include <cfloat>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define PSX_HD __host__ __device__ __forceinline__
#else
#define PSX_HD inline
#endif

namespace psx {

struct V3 { float x, y, z; };
struct D3 { double x, y, z; };
struct Q4 { float x, y, z, w; };
struct M3 { V3 c[3]; };
struct V2 { float x, y; };
struct Bounds { V3 min, max; };

PSX_HD V3 v3(float x, float y, float z) { return {x, y, z}; }
PSX_HD V3 v3s(float s) { return {s, s, s}; }
PSX_HD V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
PSX_HD V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
PSX_HD V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
PSX_HD V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
PSX_HD V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
PSX_HD V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
PSX_HD V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
PSX_HD V3 operator/(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
PSX_HD V3 operator+(V3 a, float s) { return {a.x + s, a.y + s, a.z + s}; }
PSX_HD V3 operator-(V3 a, float s) { return {a.x - s, a.y - s, a.z - s}; }
PSX_HD V3& operator+=(V3& a, V3 b) { a = a + b; return a; }
PSX_HD V3& operator-=(V3& a, V3 b) { a = a - b; return a; }
PSX_HD float& at(V3& v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
PSX_HD float at(const V3& v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

PSX_HD float dot(V3 a, V3 b) { V3 t = a * b; return t.x + t.y + t.z; }
PSX_HD V3 cross(V3 x, V3 y) { return {x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y}; }
PSX_HD float length(V3 v) { return sqrtf(dot(v, v)); }
PSX_HD float length2(V3 v) { return dot(v, v); }
PSX_HD float distance(V3 a, V3 b) { return length(a - b); }
PSX_HD float distance2(V3 a, V3 b) { return length2(b - a); }
PSX_HD V3 normalize(V3 v) { return v * (1.f / sqrtf(dot(v, v))); }
PSX_HD float fminG(float x, float y) { return (y < x) ? y : x; }
PSX_HD float fmaxG(float x, float y) { return (x < y) ? y : x; }
PSX_HD float clampG(float x, float lo, float hi) { return fminG(fmaxG(x, lo), hi); }
PSX_HD V3 vmin(V3 a, V3 b) { return {fminG(a.x, b.x), fminG(a.y, b.y), fminG(a.z, b.z)}; }
PSX_HD V3 vmax(V3 a, V3 b) { return {fmaxG(a.x, b.x), fmaxG(a.y, b.y), fmaxG(a.z, b.z)}; }
PSX_HD V3 vclamp(V3 x, V3 lo, V3 hi) { return vmin(vmax(x, lo), hi); }
PSX_HD V3 vabs(V3 a) { return {fabsf(a.x), fabsf(a.y), fabsf(a.z)}; }
PSX_HD float signG(float x) { return (float)(0.f < x) - (float)(x < 0.f); }
PSX_HD double signD(double x) { return (double)(0.0 < x) - (double)(x < 0.0); }
PSX_HD float mixG(float x, float y, float a) { return x * (1.f - a) + y * a; }
PSX_HD float det2(V2 c0, V2 c1) { return c0.x * c1.y - c1.x * c0.y; }
PSX_HD V2 operator-(V2 a, V2 b) { return {a.x - b.x, a.y - b.y}; }
PSX_HD V2 operator+(V2 a, V2 b) { return {a.x + b.x, a.y + b.y}; }
PSX_HD V2 operator-(V2 a) { return {-a.x, -a.y}; }
PSX_HD V2 operator*(float s, V2 a) { return {s * a.x, s * a.y}; }

PSX_HD D3 d3(V3 v) { return {(double)v.x, (double)v.y, (double)v.z}; }
PSX_HD V3 f3(D3 v) { return {(float)v.x, (float)v.y, (float)v.z}; }
PSX_HD D3 operator+(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
PSX_HD D3 operator-(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
PSX_HD D3 operator-(D3 a) { return {-a.x, -a.y, -a.z}; }
PSX_HD D3 operator*(D3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
PSX_HD D3 operator*(double s, D3 a) { return {s * a.x, s * a.y, s * a.z}; }
PSX_HD D3 operator/(D3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
PSX_HD D3 operator+(D3 a, double s) { return {a.x + s, a.y + s, a.z + s}; }
PSX_HD double dot(D3 a, D3 b) { D3 t = {a.x * b.x, a.y * b.y, a.z * b.z}; return t.x + t.y + t.z; }
PSX_HD D3 cross(D3 x, D3 y) { return {x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y}; }
PSX_HD double length(D3 v) { return sqrt(dot(v, v)); }
PSX_HD D3 normalize(D3 v) { return v * (1.0 / sqrt(dot(v, v))); }

PSX_HD Q4 qmul(Q4 p, Q4 q) {
    return {p.w * q.x + p.x * q.w + p.y * q.z - p.z * q.y,
            p.w * q.y + p.y * q.w + p.z * q.x - p.x * q.z,
            p.w * q.z + p.z * q.w + p.x * q.y - p.y * q.x,
            p.w * q.w - p.x * q.x - p.y * q.y - p.z * q.z};
}
PSX_HD V3 qrot(Q4 q, V3 v) {
    V3 qv = {q.x, q.y, q.z};
    V3 uv = cross(qv, v);
    V3 uuv = cross(qv, uv);
    return v + ((uv * q.w) + uuv) * 2.f;
}
PSX_HD float qdot(Q4 a, Q4 b) {
    float w = a.w * b.w, x = a.x * b.x, y = a.y * b.y, z = a.z * b.z;
    return (w + x) + (y + z);
}
PSX_HD Q4 qinverse(Q4 q) {
    float d = qdot(q, q);
    return {-q.x / d, -q.y / d, -q.z / d, q.w / d};
}
PSX_HD Q4 qnormalize(Q4 q) {
    float len = sqrtf(qdot(q, q));
    if (len <= 0.f) return {0.f, 0.f, 0.f, 1.f};
    float o = 1.f / len;
    return {q.x * o, q.y * o, q.z * o, q.w * o};
}
PSX_HD Q4 qadd(Q4 a, Q4 b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }

PSX_HD M3 m3cols(V3 a, V3 b, V3 c) { return {{a, b, c}}; }
PSX_HD M3 m3zero() { M3 r; r.c[0] = {0, 0, 0}; r.c[1] = {0, 0, 0}; r.c[2] = {0, 0, 0}; return r; }
PSX_HD M3 mat3_cast(Q4 q) {
    float qxx = q.x * q.x, qyy = q.y * q.y, qzz = q.z * q.z;
    float qxz = q.x * q.z, qxy = q.x * q.y, qyz = q.y * q.z;
    float qwx = q.w * q.x, qwy = q.w * q.y, qwz = q.w * q.z;
    M3 r;
    r.c[0] = {1.f - 2.f * (qyy + qzz), 2.f * (qxy + qwz), 2.f * (qxz - qwy)};
    r.c[1] = {2.f * (qxy - qwz), 1.f - 2.f * (qxx + qzz), 2.f * (qyz + qwx)};
    r.c[2] = {2.f * (qxz + qwy), 2.f * (qyz - qwx), 1.f - 2.f * (qxx + qyy)};
    return r;
}
PSX_HD V3 mv(const M3& m, V3 v) {
    return {m.c[0].x * v.x + m.c[1].x * v.y + m.c[2].x * v.z,
            m.c[0].y * v.x + m.c[1].y * v.y + m.c[2].y * v.z,
            m.c[0].z * v.x + m.c[1].z * v.y + m.c[2].z * v.z};
}
PSX_HD M3 mm(const M3& a, const M3& b) {
    M3 r;
    for (int j = 0; j < 3; ++j) {
        V3 bj = b.c[j];
        r.c[j] = {a.c[0].x * bj.x + a.c[1].x * bj.y + a.c[2].x * bj.z,
                  a.c[0].y * bj.x + a.c[1].y * bj.y + a.c[2].y * bj.z,
                  a.c[0].z * bj.x + a.c[1].z * bj.y + a.c[2].z * bj.z};
    }
    return r;
}
PSX_HD M3 transpose(const M3& m) {
    M3 r;
    r.c[0] = {m.c[0].x, m.c[1].x, m.c[2].x};
    r.c[1] = {m.c[0].y, m.c[1].y, m.c[2].y};
    r.c[2] = {m.c[0].z, m.c[1].z, m.c[2].z};
    return r;
}
PSX_HD M3 madd(const M3& a, const M3& b) { return {{a.c[0] + b.c[0], a.c[1] + b.c[1], a.c[2] + b.c[2]}}; }
PSX_HD M3 msub(const M3& a, const M3& b) { return {{a.c[0] - b.c[0], a.c[1] - b.c[1], a.c[2] - b.c[2]}}; }
PSX_HD M3 mscale(float s, const M3& a) { return {{s * a.c[0], s * a.c[1], s * a.c[2]}}; }
PSX_HD float mel(const M3& a, int c, int r) { return at(a.c[c], r); }
PSX_HD float determinant(const M3& a) {
    return +mel(a, 0, 0) * (mel(a, 1, 1) * mel(a, 2, 2) - mel(a, 2, 1) * mel(a, 1, 2))
           - mel(a, 1, 0) * (mel(a, 0, 1) * mel(a, 2, 2) - mel(a, 2, 1) * mel(a, 0, 2))
           + mel(a, 2, 0) * (mel(a, 0, 1) * mel(a, 1, 2) - mel(a, 1, 1) * mel(a, 0, 2));
}
PSX_HD M3 inverse(const M3& a) {
    float o = 1.f / determinant(a);
    M3 r;
    r.c[0].x = +(mel(a, 1, 1) * mel(a, 2, 2) - mel(a, 2, 1) * mel(a, 1, 2)) * o;
    r.c[1].x = -(mel(a, 1, 0) * mel(a, 2, 2) - mel(a, 2, 0) * mel(a, 1, 2)) * o;
    r.c[2].x = +(mel(a, 1, 0) * mel(a, 2, 1) - mel(a, 2, 0) * mel(a, 1, 1)) * o;
    r.c[0].y = -(mel(a, 0, 1) * mel(a, 2, 2) - mel(a, 2, 1) * mel(a, 0, 2)) * o;
    r.c[1].y = +(mel(a, 0, 0) * mel(a, 2, 2) - mel(a, 2, 0) * mel(a, 0, 2)) * o;
    r.c[2].y = -(mel(a, 0, 0) * mel(a, 2, 1) - mel(a, 2, 0) * mel(a, 0, 1)) * o;
    r.c[0].z = +(mel(a, 0, 1) * mel(a, 1, 2) - mel(a, 1, 1) * mel(a, 0, 2)) * o;
    r.c[1].z = -(mel(a, 0, 0) * mel(a, 1, 2) - mel(a, 1, 0) * mel(a, 0, 2)) * o;
    r.c[2].z = +(mel(a, 0, 0) * mel(a, 1, 1) - mel(a, 1, 0) * mel(a, 0, 1)) * o;
    return r;
}
PSX_HD M3 matrixCross3(V3 x) {
    M3 r = m3zero();
    r.c[0].y = x.z; r.c[1].x = -x.z; r.c[0].z = -x.y; r.c[2].x = x.y; r.c[1].z = x.x; r.c[2].y = -x.x;
    return r;
}
PSX_HD V3 multiplyTranspose(const M3& a, V3 v) { return {dot(v, a.c[0]), dot(v, a.c[1]), dot(v, a.c[2])}; }
PSX_HD V3 solve33(const M3& A, V3 b) {
    V3 c12 = cross(A.c[1], A.c[2]);
    float det = dot(A.c[0], c12);
    if (det == 0.f) return {0, 0, 0};
    float inv = 1.f / det;
    return {inv * dot(b, c12), inv * dot(A.c[0], cross(b, A.c[2])), inv * dot(A.c[0], cross(A.c[1], b))};
}

#ifdef __CUDACC__
PSX_HD V3 ld3(const float4& a) { return {a.x, a.y, a.z}; }
PSX_HD Q4 ld4(const float4& a) { return {a.x, a.y, a.z, a.w}; }
PSX_HD float4 st4(V3 v, float w = 0.f) { return make_float4(v.x, v.y, v.z, w); }
PSX_HD float4 st4(Q4 q) { return make_float4(q.x, q.y, q.z, q.w); }
PSX_HD float bits_as_float(int i) { float f; memcpy(&f, &i, sizeof f); return f; }
#endif

}  // namespace psx
