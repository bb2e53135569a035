/*
 * collide_util.h — helpers shared by the oracle's narrowphase.
 * ORACLE (test infrastructure only; see omath.h).
 */
#pragma once
#include "geom.h"

namespace orc {

enum { TF_FACE = 0, TF_EDGE = 1, TF_VERTEX = 2 };  // TriangleFeature, src/GeomUtil.h:6-8

// Clipping.cpp caps a clipped polygon at 128 points (src/Clipping.cpp:6)
constexpr int kMaxPoly = 128;
struct Poly { V2 p[kMaxPoly]; int n = 0; };

V3 closestPointOnSegment(V3 point, V3 lineOrig, V3 lineDir, float mn, float mx);
void closestPointsBetweenSegments(V3 o0, V3 d0, float min0, float max0, V3 o1, V3 d1, float min1, float max1, V3& p0, V3& p1);
void closestPointsBetweenSegmentsV(V3 o0, V3 v0, V3 o1, V3 v1, V3& p0, V3& p1);
float sqrDistSegmentAABB(V3 p, V3 dir, float mn, float mx, V3 he, float& t, V3& q);
float sqrDistPointTriangle(V3 p, V3 a, V3 b, V3 c, V3& q, int& feature, int& featureIndex);
float sqrDistSegmentTriangle(V3 p, V3 dir, float mn, float mx, V3 a, V3 b, V3 c, float& t, V3& q, int& feature, int& featureIndex);
float distanceAABBPlane(V3 he, V3 n, float d);

void suthHodgClip(Poly& poly, const V2* clip, int nclip);
bool clipLine(V2& p0, V2& p1, const V2* clip, int n);

void generateContactsPolygonBoxFace(V3 boxCenter, const M3& boxBasis, int boxAxis, int boxAxisSign, V3 he,
                                    V3 incOrig, V3 incNormal, const Poly& poly, int clipX, int clipY,
                                    ContactPoint* cp, int& numPoints);
void generateContactsPolygonPolygonFace(V3 refPos, const M3& refToWorld, V3 refPlaneOrigin, V3 refPlaneNormal,
                                        V3 incOrig, V3 incNormal, const Poly& poly, int clipX, int clipY,
                                        ContactPoint* cp, int& numPoints);

// support mappings (src/GJK.h:13-128)
struct Support {
    int kind;            // 0 sphere, 1 capsule, 2 box, 3 convex, 4 triangle
    V3 pos;
    float radius = 0, halfHeight = 0;
    V3 axis{0, 0, 0};
    M3 basis{};
    V3 he{0, 0, 0};
    const ConvexMesh* mesh = nullptr;
    V3 scale{1, 1, 1};
    V3 a{0, 0, 0}, b{0, 0, 0}, c{0, 0, 0};
    V3 operator()(V3 dir) const;
};

struct GjkVertex { D3 pos, sp0, sp1; };
struct GjkSimplex { GjkVertex v[4]; };

bool gjk(const Support& s0, const Support& s1, V3 startDir, GjkSimplex& s);
V3 epa(const Support& s0, const Support& s1, GjkSimplex& s, V3& cp0, V3& cp1);

}  // namespace orc
