// FP64 restatement of crashcat's convex collision pipeline for the CPU oracle.
//
// TEST INFRASTRUCTURE ONLY (parity oracle, never part of the GPU library).
//
// Each function cites the reference function it follows; the arithmetic is
// kept in the reference's operation order so that the oracle reproduces the
// reference's IEEE-754 double results (compiled with -ffp-contract=off).
#pragma once
#include <algorithm>
#include <array>
#include <cstring>
#include <limits>
#include <vector>

#include "oracle_math.h"

namespace orc {

constexpr double DEFAULT_CONVEX_RADIUS = 0.05;  // src/collision/support.ts:5
constexpr uint32_t EMPTY_SUB_SHAPE_ID = 0xffffffffu;  // src/body/sub-shape.ts:4

enum ShapeType : int { SHAPE_SPHERE = 0, SHAPE_BOX = 1, SHAPE_CAPSULE = 2, SHAPE_CONVEX_HULL = 3, SHAPE_TRIANGLE_MESH = 4,
                       SHAPE_CYLINDER = 5, SHAPE_PLANE = 6, SHAPE_EMPTY = 7, SHAPE_COMPOUND = 8 };

// Triangle mesh as built (src/shapes/utils/triangle-mesh-data.ts, triangle-mesh-bvh.ts): welded
// vertices, triangles (vertex indices, active-edge bits AB 1 / BC 2 / CA 4) in the order the BVH
// build left them, nodes in pre-order (min, max, then the right child's node index or the first
// triangle, then the split axis or -(count + 1) for a leaf)
struct MeshData {
    std::vector<V3> verts;
    std::vector<std::array<int, 4>> tris;
    std::vector<std::array<double, 8>> nodes;
    int subBits = 0;
    Box3 bounds;
};

// ConvexHullShape fields (src/shapes/convex-hull.ts:38-62): points relative to the centre of
// mass, the points shrunk by the convex radius (setConvexHullNoConvexSupport :732-788),
// polygon faces over point indices and their planes (n . x + c = 0)
struct HullData {
    std::vector<V3> points, shrunk;
    std::vector<int> face_first, face_count, vidx;
    std::vector<V3> plane_n;
    std::vector<double> plane_c;
    double convex_radius = 0, volume = 0;
    V3 com{0, 0, 0};
    double inertia[9] = {0};  // unit density, row-major
    Box3 bounds;
};

// Shape data (src/shapes/box.ts:38-70, src/shapes/sphere.ts, src/shapes/capsule.ts, convex-hull.ts)
struct CompoundData;
struct Shape {
    const HullData *hull = nullptr;  // convex hull
    const MeshData *mesh = nullptr;  // triangle mesh
    const CompoundData *compound = nullptr;  // compound shape
    int type = SHAPE_BOX;
    V3 half_extents;          // box
    double convex_radius = 0;  // box
    double radius = 0;         // sphere / capsule / cylinder
    double half_height = 0;    // capsule (segment along Y) / cylinder (along Y)
    double density = 1000;
    V3 pn{0, 1, 0};            // plane: unit normal and constant (n . x + c = 0, solid below)
    double pc = 0, halfExtent = 1000;  // plane: DEFAULT_PLANE_HALF_EXTENT plane.ts:36
    V3 com;                    // shape-local centre of mass
    Box3 aabb;                 // shape-local bounds
    // decorators (scaled.ts, transformed.ts, offset-center-of-mass.ts) as
    // OffsetCenterOfMass(Transformed(Scaled(leaf))): the scale is baked into the leaf's
    // dimensions above; the collision geometry is the leaf at (tPos, tRot) in the body frame
    // (collideTransformedVsShape transformed.ts); com, aabb and innerRadius are the decorated
    // shape's
    bool decorated = false;
    Box3 leafAabb;             // the (scaled) leaf's bounds in its own frame, which its collisions use
    V3 tPos{0, 0, 0};
    Q4 tRot{0, 0, 0, 1};
    double innerRadius = -1;   // getInnerRadius of the decorated shape (< 0: the leaf's)
};
// CompoundShape (compound.ts): convex children at poses in the compound's frame; the compound's
// com, aabb and mass come from them (computeCompoundCenterOfMass :110-141, computeCompound-
// LocalBounds :70-108, computeMassProperties :177-230)
struct CompoundData {
    std::vector<Shape> shapes;
    std::vector<V3> pos;
    std::vector<Q4> rot;
    int subBits = 0;      // the bits subShape.pushIndex gives a child index of shapes.size()
    double innerRadius = 0;  // getInnerRadius :283-289: the least of the children's
    double mass = 0, inertia[9] = {};  // about the compound's centre of mass, row-major
};
// subShape.pushIndex (sub-shape.ts:60-64) of child i onto an empty id: the index in the low
// subBits bits, ones above
inline uint32_t compound_sub_id(const CompoundData &c, int i) {
    if (c.subBits >= 32) return (uint32_t)i;
    return (0xffffffffu & ~((1u << c.subBits) - 1u)) | (uint32_t)i;
}
// child i of a compound at (p, q): the child's world pose (the accumulated transform of
// collideCompoundVsShape :520-526)
inline void compound_child_pose(const CompoundData &c, int i, V3 p, Q4 q, V3 &cp, Q4 &cq) {
    cp = add(p, rotate(q, c.pos[i]));
    cq = qmul(q, c.rot[i]);
}

// the pose of a shape's collision geometry for a body at (p, q)
inline void geometry_pose(const Shape &s, V3 p, Q4 q, V3 &gp, Q4 &gq) {
    if (!s.decorated) {
        gp = p;
        gq = q;
        return;
    }
    gp = add(p, rotate(q, s.tPos));
    gq = qmul(q, s.tRot);
}

// ----------------------------------------------------------------------------
// Support functions (src/collision/support.ts, src/shapes/sphere.ts:173-266)
// ----------------------------------------------------------------------------
enum SupportMode { INCLUDE_CONVEX_RADIUS = 0, EXCLUDE_CONVEX_RADIUS = 1 };
enum SupportKind { SUP_BOX, SUP_SPHERE_POINT, SUP_SPHERE_SURFACE, SUP_CAPSULE_SEGMENT, SUP_CAPSULE_SURFACE, SUP_HULL,
                   SUP_TRIANGLE, SUP_CYLINDER };

struct Support {
    int kind = SUP_BOX;
    const std::vector<V3> *pts = nullptr;  // convex hull support points
    V3 he;                    // box half extents (already shrunk if EXCLUDE)
    double radius = 0;        // sphere/capsule radius used by the surface form
    double half_height = 0;   // capsule
    double convex_radius = 0;  // reported convex radius
    bool transformed = false;  // TransformedSupport (support.ts:228-278)
    M4 m;
    bool add_radius = false;  // AddConvexRadiusSupport (support.ts:282-315)
    double add_r = 0;
    V3 ta, tb, tc;  // TriangleSupport (support.ts:75-142)

    V3 inner(V3 d) const {
        switch (kind) {
            case SUP_BOX:  // boxGetSupport support.ts:323-327
                return {d.x >= 0 ? he.x : -he.x, d.y >= 0 ? he.y : -he.y, d.z >= 0 ? he.z : -he.z};
            case SUP_SPHERE_POINT:  // sphere.ts:184-187
                return {0, 0, 0};
            case SUP_SPHERE_SURFACE: {  // sphere.ts:213-229
                double l = d.x * d.x + d.y * d.y + d.z * d.z;
                if (l > 0) {
                    double s = radius / std::sqrt(l);
                    return {d.x * s, d.y * s, d.z * s};
                }
                return {0, 0, 0};
            }
            case SUP_HULL: {  // the point with the highest projection (convex-hull.ts:588-614, 695-715)
                double best = -1.0 / 0.0;
                V3 bp{0, 0, 0};
                for (const V3 &p : *pts) {
                    double dd = p.x * d.x + p.y * d.y + p.z * d.z;
                    if (dd > best) {
                        best = dd;
                        bp = p;
                    }
                }
                return bp;
            }
            case SUP_TRIANGLE: {  // triangleGetSupport support.ts:83-118
                double d1 = dot(ta, d), d2 = dot(tb, d), d3 = dot(tc, d);
                if (d1 > d2) return d1 > d3 ? ta : tc;
                return d2 > d3 ? tb : tc;
            }
            case SUP_CAPSULE_SEGMENT:  // capsule.ts: segment +-h on Y
                return {0, d.y > 0 ? half_height : -half_height, 0};
            case SUP_CYLINDER: {  // cylinder{No,With}ConvexGetSupport cylinder.ts
                double hl = std::sqrt(d.x * d.x + d.z * d.z);
                V3 o{0, d.y >= 0 ? half_height : -half_height, 0};
                if (hl > 0) {
                    double s = radius / hl;
                    o.x = d.x * s;
                    o.z = d.z * s;
                }
                return o;
            }
            case SUP_CAPSULE_SURFACE: {  // capsuleWithConvexGetSupport capsule.ts:321-338
                double l = d.x * d.x + d.y * d.y + d.z * d.z;
                if (!(l > 0)) return {0, half_height, 0};
                double s = radius / std::sqrt(l);
                return {d.x * s, d.y * s + (d.y > 0 ? half_height : -half_height), d.z * s};
            }
        }
        return {0, 0, 0};
    }
    V3 get(V3 d) const {
        V3 o;
        if (transformed) {
            // transformedGetSupport support.ts:237-258
            V3 ld{m.m[0] * d.x + m.m[1] * d.y + m.m[2] * d.z, m.m[4] * d.x + m.m[5] * d.y + m.m[6] * d.z,
                  m.m[8] * d.x + m.m[9] * d.y + m.m[10] * d.z};
            V3 s = inner(ld);
            o = {m.m[0] * s.x + m.m[4] * s.y + m.m[8] * s.z + m.m[12],
                 m.m[1] * s.x + m.m[5] * s.y + m.m[9] * s.z + m.m[13],
                 m.m[2] * s.x + m.m[6] * s.y + m.m[10] * s.z + m.m[14]};
        } else {
            o = inner(d);
        }
        if (add_radius) {
            // addConvexRadiusGetSupport support.ts:288-301
            double l = d.x * d.x + d.y * d.y + d.z * d.z;
            if (l > 0) {
                double s = add_r / std::sqrt(l);
                o.x += d.x * s;
                o.y += d.y * s;
                o.z += d.z * s;
            }
        }
        return o;
    }
};

// getShapeSupportFunction for unit scale (support.ts:57-69, setBoxSupport support.ts:339-370,
// getSphereSupportFunction sphere.ts:256-266)
inline Support make_support(const Shape &s, SupportMode mode) {
    Support o;
    if (s.type == SHAPE_CONVEX_HULL) {
        // getConvexHullSupportFunction convex-hull.ts:968-997
        o.kind = SUP_HULL;
        if (mode == INCLUDE_CONVEX_RADIUS || s.hull->convex_radius == 0) {
            o.pts = &s.hull->points;
            o.convex_radius = 0;
        } else {
            o.pts = &s.hull->shrunk;
            o.convex_radius = s.hull->convex_radius;
        }
    } else if (s.type == SHAPE_BOX) {
        o.kind = SUP_BOX;
        if (mode == EXCLUDE_CONVEX_RADIUS) {
            double cr = std::min(s.convex_radius * 1.0, DEFAULT_CONVEX_RADIUS);
            o.he = {std::max(0.0, s.half_extents.x - cr), std::max(0.0, s.half_extents.y - cr),
                    std::max(0.0, s.half_extents.z - cr)};
            o.convex_radius = cr;
        } else {
            o.he = s.half_extents;
            o.convex_radius = 0;
        }
    } else if (s.type == SHAPE_CYLINDER) {
        // getCylinderSupportFunction cylinder.ts: the full cylinder, or the one shrunk by the
        // convex radius with that radius reported
        o.kind = SUP_CYLINDER;
        if (mode == INCLUDE_CONVEX_RADIUS) {
            o.half_height = s.half_height;
            o.radius = s.radius;
            o.convex_radius = 0;
        } else {
            o.half_height = s.half_height - s.convex_radius;
            o.radius = s.radius - s.convex_radius;
            o.convex_radius = s.convex_radius;
        }
    } else if (s.type == SHAPE_SPHERE) {
        if (mode == INCLUDE_CONVEX_RADIUS) {
            o.kind = SUP_SPHERE_SURFACE;
            o.radius = s.radius;
            o.convex_radius = 0;
        } else {
            o.kind = SUP_SPHERE_POINT;
            o.convex_radius = s.radius;
        }
    } else {
        o.half_height = s.half_height;
        if (mode == INCLUDE_CONVEX_RADIUS) {
            o.kind = SUP_CAPSULE_SURFACE;
            o.radius = s.radius;
            o.convex_radius = 0;
        } else {
            o.kind = SUP_CAPSULE_SEGMENT;
            o.convex_radius = s.radius;
        }
    }
    return o;
}

// SupportFunctionMode.DEFAULT: the box and the cylinder include their convex radius
// (support.ts:351, cylinder.ts:412), the other shapes exclude it (sphere.ts:258,
// capsule.ts:396, convex-hull.ts:978)
inline Support make_support_default(const Shape &s) {
    return make_support(s, (s.type == SHAPE_BOX || s.type == SHAPE_CYLINDER) ? INCLUDE_CONVEX_RADIUS
                                                                            : EXCLUDE_CONVEX_RADIUS);
}

// ----------------------------------------------------------------------------
// Simplex + closest points (src/collision/simplex.ts, closest-points.ts, gjk.ts)
// ----------------------------------------------------------------------------
struct SimplexPoint {
    V3 y, p, q;
};
struct Simplex {
    SimplexPoint pts[4];
    int size = 0;
};

struct Bary {
    double u = 0, v = 0, w = 0;
    bool valid = false;
};

// computeBarycentricCoordinates2d closest-points.ts:19-47
inline Bary bary2(V3 a, V3 b, double sqtol) {
    Bary o;
    V3 ab = sub(b, a);
    double den = ab.x * ab.x + ab.y * ab.y + ab.z * ab.z;
    if (den < sqtol) {
        if (a.x * a.x + a.y * a.y + a.z * a.z < b.x * b.x + b.y * b.y + b.z * b.z) {
            o.u = 1.0;
            o.v = 0.0;
        } else {
            o.u = 0.0;
            o.v = 1.0;
        }
        o.valid = false;
        return o;
    }
    o.v = -(a.x * ab.x + a.y * ab.y + a.z * ab.z) / den;
    o.u = 1.0 - o.v;
    o.valid = true;
    return o;
}

// computeBarycentricCoordinates3d closest-points.ts:51-152
inline Bary bary3(V3 a, V3 b, V3 c, double sqtol) {
    Bary o;
    V3 ab = sub(b, a), ac = sub(c, a), bc = sub(c, b);
    double d00 = ab.x * ab.x + ab.y * ab.y + ab.z * ab.z;
    double d11 = ac.x * ac.x + ac.y * ac.y + ac.z * ac.z;
    double d22 = bc.x * bc.x + bc.y * bc.y + bc.z * bc.z;
    if (d00 <= d22) {
        double d01 = ab.x * ac.x + ab.y * ac.y + ab.z * ac.z;
        double den = d00 * d11 - d01 * d01;
        if (std::fabs(den) < 1.0e-12) {
            if (d00 > d11) {
                Bary t = bary2(a, b, sqtol);
                o.u = t.u;
                o.v = t.v;
                o.w = 0.0;
            } else {
                Bary t = bary2(a, c, sqtol);
                o.u = t.u;
                o.w = t.v;
                o.v = 0.0;
            }
            o.valid = false;
            return o;
        }
        double a0 = a.x * ab.x + a.y * ab.y + a.z * ab.z;
        double a1 = a.x * ac.x + a.y * ac.y + a.z * ac.z;
        o.v = (d01 * a1 - d11 * a0) / den;
        o.w = (d01 * a0 - d00 * a1) / den;
        o.u = 1.0 - o.v - o.w;
    } else {
        double d12 = ac.x * bc.x + ac.y * bc.y + ac.z * bc.z;
        double den = d11 * d22 - d12 * d12;
        if (std::fabs(den) < 1.0e-12) {
            if (d11 > d22) {
                Bary t = bary2(a, c, sqtol);
                o.u = t.u;
                o.w = t.v;
                o.v = 0.0;
            } else {
                Bary t = bary2(b, c, sqtol);
                o.v = t.u;
                o.w = t.v;
                o.u = 0.0;
            }
            o.valid = false;
            return o;
        }
        double c1 = c.x * ac.x + c.y * ac.y + c.z * ac.z;
        double c2 = c.x * bc.x + c.y * bc.y + c.z * bc.z;
        o.u = (d22 * c1 - d12 * c2) / den;
        o.v = (d11 * c2 - d12 * c1) / den;
        o.w = 1.0 - o.u - o.v;
    }
    o.valid = true;
    return o;
}

struct ClosestPoint {
    V3 point;
    int set = 0;
};

inline double clamp01(double v) { return v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v); }

// computeClosestPointOnLine gjk.ts:33-55
inline ClosestPoint closest_on_line(V3 a, V3 b, double sqtol) {
    Bary br = bary2(a, b, sqtol);
    ClosestPoint o;
    if (br.v <= 0.0) {
        o.point = a;
        o.set = 0b0001;
    } else if (br.u <= 0.0) {
        o.point = b;
        o.set = 0b0010;
    } else {
        o.point = {a.x * br.u + b.x * br.v, a.y * br.u + b.y * br.v, a.z * br.u + b.z * br.v};
        o.set = 0b0011;
    }
    return o;
}

// computeClosestPointOnTriangle gjk.ts:57-350
inline ClosestPoint closest_on_triangle(V3 inA, V3 inB, V3 inC, bool mustIncludeC, double sqtol) {
    ClosestPoint out;
    V3 ac0 = sub(inC, inA), bc0 = sub(inC, inB);
    bool swapAC = bc0.x * bc0.x + bc0.y * bc0.y + bc0.z * bc0.z < ac0.x * ac0.x + ac0.y * ac0.y + ac0.z * ac0.z;
    V3 a = swapAC ? inC : inA;
    V3 c = swapAC ? inA : inC;
    V3 ab = sub(inB, a);
    V3 ac = sub(c, a);
    V3 n{ab.y * ac.z - ab.z * ac.y, ab.z * ac.x - ab.x * ac.z, ab.x * ac.y - ab.y * ac.x};
    double nls = n.x * n.x + n.y * n.y + n.z * n.z;
    if (nls < 1.0e-10) {
        int cs = 0b0100;
        V3 cp = inC;
        double best = inC.x * inC.x + inC.y * inC.y + inC.z * inC.z;
        if (!mustIncludeC) {
            double al = inA.x * inA.x + inA.y * inA.y + inA.z * inA.z;
            if (al < best) {
                cs = 0b0001;
                cp = inA;
                best = al;
            }
            double bl = inB.x * inB.x + inB.y * inB.y + inB.z * inB.z;
            if (bl < best) {
                cs = 0b0010;
                cp = inB;
                best = bl;
            }
        }
        {
            V3 ac2 = sub(c, a);
            double acl = ac2.x * ac2.x + ac2.y * ac2.y + ac2.z * ac2.z;
            if (acl > sqtol) {
                double v = clamp01(-(a.x * ac2.x + a.y * ac2.y + a.z * ac2.z) / acl);
                V3 q{a.x + ac2.x * v, a.y + ac2.y * v, a.z + ac2.z * v};
                double d = q.x * q.x + q.y * q.y + q.z * q.z;
                if (d < best) {
                    cs = 0b0101;
                    cp = q;
                    best = d;
                }
            }
        }
        {
            V3 bc2 = sub(inC, inB);
            double bcl = bc2.x * bc2.x + bc2.y * bc2.y + bc2.z * bc2.z;
            if (bcl > sqtol) {
                double v = clamp01(-(inB.x * bc2.x + inB.y * bc2.y + inB.z * bc2.z) / bcl);
                V3 q{inB.x + bc2.x * v, inB.y + bc2.y * v, inB.z + bc2.z * v};
                double d = q.x * q.x + q.y * q.y + q.z * q.z;
                if (d < best) {
                    cs = 0b0110;
                    cp = q;
                    best = d;
                }
            }
        }
        if (!mustIncludeC) {
            V3 ab2 = sub(inB, inA);
            double abl = ab2.x * ab2.x + ab2.y * ab2.y + ab2.z * ab2.z;
            if (abl > sqtol) {
                double v = clamp01(-(inA.x * ab2.x + inA.y * ab2.y + inA.z * ab2.z) / abl);
                V3 q{inA.x + ab2.x * v, inA.y + ab2.y * v, inA.z + ab2.z * v};
                double d = q.x * q.x + q.y * q.y + q.z * q.z;
                if (d < best) {
                    cs = 0b0011;
                    cp = q;
                }
            }
        }
        out.set = cs;
        out.point = cp;
        return out;
    }
    V3 ap{-a.x, -a.y, -a.z};
    double d1 = ab.x * ap.x + ab.y * ap.y + ab.z * ap.z;
    double d2 = ac.x * ap.x + ac.y * ap.y + ac.z * ap.z;
    if (d1 <= 0.0 && d2 <= 0.0) {
        out.set = swapAC ? 0b0100 : 0b0001;
        out.point = a;
        return out;
    }
    V3 bp{-inB.x, -inB.y, -inB.z};
    double d3 = ab.x * bp.x + ab.y * bp.y + ab.z * bp.z;
    double d4 = ac.x * bp.x + ac.y * bp.y + ac.z * bp.z;
    if (d3 >= 0.0 && d4 <= d3) {
        out.set = 0b0010;
        out.point = inB;
        return out;
    }
    if (d1 * d4 <= d3 * d2 && d1 >= 0.0 && d3 <= 0.0) {
        double v = d1 / (d1 - d3);
        out.set = swapAC ? 0b0110 : 0b0011;
        out.point = {a.x + ab.x * v, a.y + ab.y * v, a.z + ab.z * v};
        return out;
    }
    V3 cpp{-c.x, -c.y, -c.z};
    double d5 = ab.x * cpp.x + ab.y * cpp.y + ab.z * cpp.z;
    double d6 = ac.x * cpp.x + ac.y * cpp.y + ac.z * cpp.z;
    if (d6 >= 0.0 && d5 <= d6) {
        out.set = swapAC ? 0b0001 : 0b0100;
        out.point = c;
        return out;
    }
    if (d5 * d2 <= d1 * d6 && d2 >= 0.0 && d6 <= 0.0) {
        double w = d2 / (d2 - d6);
        out.set = 0b0101;
        out.point = {a.x + ac.x * w, a.y + ac.y * w, a.z + ac.z * w};
        return out;
    }
    double d43 = d4 - d3;
    double d56 = d5 - d6;
    if (d3 * d6 <= d5 * d4 && d43 >= 0.0 && d56 >= 0.0) {
        double w = d43 / (d43 + d56);
        out.set = swapAC ? 0b0011 : 0b0110;
        V3 t = sub(c, inB);
        out.point = {inB.x + t.x * w, inB.y + t.y * w, inB.z + t.z * w};
        return out;
    }
    out.set = 0b0111;
    V3 t{a.x + inB.x + c.x, a.y + inB.y + c.y, a.z + inB.z + c.z};
    double s = (t.x * n.x + t.y * n.y + t.z * n.z) / (3 * nls);
    out.point = {n.x * s, n.y * s, n.z * s};
    return out;
}

// isOriginOutsideOfTrianglePlanes gjk.ts:305-395
inline void origin_outside_planes(int out[4], V3 a, V3 b, V3 c, V3 d, double tol) {
    V3 ab = sub(b, a), ac = sub(c, a), ad = sub(d, a), bd = sub(d, b), bc = sub(c, b);
    V3 abac{ab.y * ac.z - ab.z * ac.y, ab.z * ac.x - ab.x * ac.z, ab.x * ac.y - ab.y * ac.x};
    V3 acad{ac.y * ad.z - ac.z * ad.y, ac.z * ad.x - ac.x * ad.z, ac.x * ad.y - ac.y * ad.x};
    V3 adab{ad.y * ab.z - ad.z * ab.y, ad.z * ab.x - ad.x * ab.z, ad.x * ab.y - ad.y * ab.x};
    V3 bdbc{bd.y * bc.z - bd.z * bc.y, bd.z * bc.x - bd.x * bc.z, bd.x * bc.y - bd.y * bc.x};
    double spx = a.x * abac.x + a.y * abac.y + a.z * abac.z;
    double spy = a.x * acad.x + a.y * acad.y + a.z * acad.z;
    double spz = a.x * adab.x + a.y * adab.y + a.z * adab.z;
    double spw = b.x * bdbc.x + b.y * bdbc.y + b.z * bdbc.z;
    double sdx = ad.x * abac.x + ad.y * abac.y + ad.z * abac.z;
    double sdy = ab.x * acad.x + ab.y * acad.y + ab.z * acad.z;
    double sdz = ac.x * adab.x + ac.y * adab.y + ac.z * adab.z;
    double sdw = -(ab.x * bdbc.x + ab.y * bdbc.y + ab.z * bdbc.z);
    if (sdx > 0 && sdy > 0 && sdz > 0 && sdw > 0) {
        out[0] = spx >= -tol;
        out[1] = spy >= -tol;
        out[2] = spz >= -tol;
        out[3] = spw >= -tol;
        return;
    }
    if (sdx < 0 && sdy < 0 && sdz < 0 && sdw < 0) {
        out[0] = spx <= tol;
        out[1] = spy <= tol;
        out[2] = spz <= tol;
        out[3] = spw <= tol;
        return;
    }
    out[0] = out[1] = out[2] = out[3] = 1;
}

// computeClosestPointOnTetrahedron gjk.ts:399-488
inline ClosestPoint closest_on_tetra(V3 a, V3 b, V3 c, V3 d, bool mustIncludeD, double tol) {
    double sqtol = tol * tol;
    ClosestPoint out;
    out.set = 0b1111;
    out.point = {0, 0, 0};
    double best = std::numeric_limits<double>::infinity();
    int o[4];
    origin_outside_planes(o, a, b, c, d, tol);
    if (o[0]) {
        if (mustIncludeD) {
            out.set = 0b0001;
            out.point = a;
        } else {
            out = closest_on_triangle(a, b, c, false, sqtol);
        }
        best = lensq(out.point);
    }
    if (o[1]) {
        ClosestPoint t = closest_on_triangle(a, c, d, mustIncludeD, sqtol);
        double ds = lensq(t.point);
        if (ds < best) {
            best = ds;
            out.point = t.point;
            out.set = (t.set & 0b0001) + ((t.set & 0b0110) << 1);
        }
    }
    if (o[2]) {
        ClosestPoint t = closest_on_triangle(a, b, d, mustIncludeD, sqtol);
        double ds = lensq(t.point);
        if (ds < best) {
            best = ds;
            out.point = t.point;
            out.set = (t.set & 0b0011) + ((t.set & 0b0100) << 1);
        }
    }
    if (o[3]) {
        ClosestPoint t = closest_on_triangle(b, c, d, mustIncludeD, sqtol);
        double ds = lensq(t.point);
        if (ds < best) {
            out.point = t.point;
            out.set = t.set << 1;
        }
    }
    return out;
}

constexpr double GJK_TOLERANCE = 1e-5;  // gjk.ts:489
constexpr int GJK_MAX_ITERATIONS = 100;  // gjk.ts:490

struct ClosestToSimplex {
    V3 point;
    double sqdist = 0;
    int set = 0;
    bool found = false;
};

// computeClosestPointToSimplex gjk.ts:524-596
inline bool closest_to_simplex(ClosestToSimplex &r, double prev, bool lastPart, const Simplex &s) {
    ClosestPoint cp;
    switch (s.size) {
        case 1:
            cp.set = 0b0001;
            cp.point = s.pts[0].y;
            break;
        case 2:
            cp = closest_on_line(s.pts[0].y, s.pts[1].y, 1e-10);
            break;
        case 3:
            cp = closest_on_triangle(s.pts[0].y, s.pts[1].y, s.pts[2].y, lastPart, 1e-10);
            break;
        default:
            cp = closest_on_tetra(s.pts[0].y, s.pts[1].y, s.pts[2].y, s.pts[3].y, lastPart, 1e-5);
            break;
    }
    double sd = lensq(cp.point);
    if (sd < prev) {
        r.point = cp.point;
        r.sqdist = sd;
        r.set = cp.set;
        r.found = true;
        return true;
    }
    r.found = false;
    return false;
}

struct GjkResult {
    double sqdist = 0;
    V3 axis, pa, pb;
    Simplex simplex;
};

// gjkClosestPoints gjk.ts:1294-1546
inline GjkResult gjk_closest_points(const Support &A, const Support &B, double tolerance, V3 direction,
                                    double maxDistSq) {
    GjkResult out;
    double sqtol = tolerance * tolerance;
    Simplex sx;
    ClosestToSimplex c;
    c.point = direction;
    c.sqdist = direction.x * direction.x + direction.y * direction.y + direction.z * direction.z;
    c.set = 0;
    c.found = true;
    double prev = std::numeric_limits<double>::max();
    int it = 0;
    while (it++ < GJK_MAX_ITERATIONS) {
        V3 p = A.get(c.point);
        V3 q = B.get(neg(c.point));
        V3 w = sub(p, q);
        double d = c.point.x * w.x + c.point.y * w.y + c.point.z * w.z;
        if (d < 0.0 && d * d > c.sqdist * maxDistSq) {
            out.sqdist = std::numeric_limits<double>::max();
            out.axis = c.point;
            return out;
        }
        sx.pts[sx.size] = {w, p, q};
        sx.size++;
        closest_to_simplex(c, prev, true, sx);
        if (!c.found) {
            sx.size--;
            break;
        }
        if (c.set == 0xf) {
            c.point = {0, 0, 0};
            c.sqdist = 0.0;
            break;
        }
        int ns = 0;
        for (int i = 0; i < sx.size; i++) {
            if (c.set & (1 << i)) {
                if (ns != i) sx.pts[ns] = sx.pts[i];
                ns++;
            }
        }
        sx.size = ns;
        if (c.sqdist <= sqtol) {
            c.point = {0, 0, 0};
            c.sqdist = 0.0;
            break;
        }
        double ymax = 0;
        for (int i = 0; i < sx.size; i++) ymax = std::max(ymax, lensq(sx.pts[i].y));
        if (c.sqdist <= GJK_TOLERANCE * ymax) {
            c.point = {0, 0, 0};
            c.sqdist = 0.0;
            break;
        }
        c.point = neg(c.point);
        if (prev - c.sqdist <= GJK_TOLERANCE * prev) break;
        prev = c.sqdist;
    }
    out.pa = {0, 0, 0};
    out.pb = {0, 0, 0};
    out.simplex = sx;
    if (sx.size == 0) {
        out.sqdist = std::numeric_limits<double>::max();
        out.axis = {0, 0, 0};
        return out;
    }
    if (sx.size == 1) {
        out.pa = sx.pts[0].p;
        out.pb = sx.pts[0].q;
    } else if (sx.size == 2) {
        Bary b = bary2(sx.pts[0].y, sx.pts[1].y, 1e-10);
        V3 p0 = sx.pts[0].p, p1 = sx.pts[1].p, q0 = sx.pts[0].q, q1 = sx.pts[1].q;
        out.pa = {p0.x * b.u + p1.x * b.v, p0.y * b.u + p1.y * b.v, p0.z * b.u + p1.z * b.v};
        out.pb = {q0.x * b.u + q1.x * b.v, q0.y * b.u + q1.y * b.v, q0.z * b.u + q1.z * b.v};
    } else if (sx.size == 3) {
        Bary b = bary3(sx.pts[0].y, sx.pts[1].y, sx.pts[2].y, 1e-10);
        V3 p0 = sx.pts[0].p, p1 = sx.pts[1].p, p2 = sx.pts[2].p;
        V3 q0 = sx.pts[0].q, q1 = sx.pts[1].q, q2 = sx.pts[2].q;
        out.pa = {p0.x * b.u + p1.x * b.v + p2.x * b.w, p0.y * b.u + p1.y * b.v + p2.y * b.w,
                  p0.z * b.u + p1.z * b.v + p2.z * b.w};
        out.pb = {q0.x * b.u + q1.x * b.v + q2.x * b.w, q0.y * b.u + q1.y * b.v + q2.y * b.w,
                  q0.z * b.u + q1.z * b.v + q2.z * b.w};
    }
    out.axis = c.point;
    out.sqdist = c.sqdist;
    return out;
}

// ----------------------------------------------------------------------------
// Penetration depth (src/collision/penetration.ts)
// ----------------------------------------------------------------------------
enum PenStatus { NOT_COLLIDING = 0, COLLIDING = 1, INDETERMINATE = 2 };
struct PenDepth {
    int status = NOT_COLLIDING;
    V3 axis, pa, pb;
};

// penetrationDepthStepGJK penetration.ts:35-110
inline PenDepth pen_step_gjk(Simplex &outSimplex, const Support &A, const Support &B, double rA, double rB,
                             V3 dir, double tol) {
    PenDepth o;
    double cr = rA + rB;
    double crs = cr * cr;
    GjkResult g = gjk_closest_points(A, B, tol, dir, crs);
    if (g.sqdist > crs) {
        o.status = NOT_COLLIDING;
        return o;
    }
    o.pa = g.pa;
    o.pb = g.pb;
    o.axis = g.axis;
    outSimplex = g.simplex;
    if (g.sqdist > 0.0) {
        double vl = std::sqrt(g.sqdist);
        o.pa = scale_add(o.pa, o.axis, rA / vl);
        o.pb = scale_add(o.pb, o.axis, -(rB / vl));
        o.status = COLLIDING;
        return o;
    }
    o.status = INDETERMINATE;
    return o;
}

// ---- EPA convex hull builder (src/collision/epa-convex-hull-builder.ts) ----
constexpr int EPA_MAX_TRIANGLES = 256;
constexpr int EPA_MAX_EDGE_LENGTH = 128;
constexpr double EPA_MIN_TRIANGLE_AREA = 1e-10;
constexpr double EPA_BARYCENTRIC_EPSILON = 1e-3;
constexpr int EPA_MAX_POINTS_TO_INCLUDE_ORIGIN_IN_HULL = 32;
constexpr int EPA_MAX_POINTS = 128;

struct EpaTri;
struct EpaEdge {
    int nt = -1;  // neighbour triangle index
    int ne = 0;   // neighbour edge
    int start = 0;
};
struct EpaTri {
    EpaEdge e[3];
    V3 normal, centroid;
    double cls = std::numeric_limits<double>::infinity();
    double lambda[2] = {0, 0};
    bool rel0 = false, interior = false, removed = false, inq = false;
    int index = -1;
};

struct EpaHull {
    std::vector<EpaTri> tris;  // pool, grows to EPA_MAX_TRIANGLES
    std::vector<int> free_list;
    std::vector<int> queue;
    const std::vector<V3> *pos = nullptr;

    bool facing(const EpaTri &t, V3 p) const {
        V3 ab = sub(p, t.centroid);
        return t.normal.x * ab.x + t.normal.y * ab.y + t.normal.z * ab.z > 0.0;
    }
    void push(int ti) {  // pushTriangleToQueue :95-116
        queue.push_back(ti);
        tris[ti].inq = true;
        int cur = (int)queue.size() - 1;
        while (cur > 0) {
            int par = (cur - 1) >> 1;
            if (tris[queue[par]].cls > tris[queue[cur]].cls) {
                std::swap(queue[par], queue[cur]);
                cur = par;
            } else {
                break;
            }
        }
    }
    int pop() {  // popClosestTriangleFromQueue :388-425
        if (queue.empty()) return -1;
        std::swap(queue[queue.size() - 1], queue[0]);
        int count = (int)queue.size() - 1;
        int largest = 0;
        while (true) {
            int child = (largest << 1) + 1;
            if (child >= count) break;
            int prevL = largest;
            if (tris[queue[largest]].cls > tris[queue[child]].cls) largest = child;
            ++child;
            if (child < count && tris[queue[largest]].cls > tris[queue[child]].cls) largest = child;
            if (prevL == largest) break;
            std::swap(queue[prevL], queue[largest]);
        }
        int r = queue.back();
        queue.pop_back();
        return r;
    }
    void link(int t1, int e1, int t2, int e2) {
        tris[t1].e[e1].nt = t2;
        tris[t1].e[e1].ne = e2;
        tris[t2].e[e2].nt = t1;
        tris[t2].e[e2].ne = e1;
    }
    // createTriangle :179-341
    int create(int i1, int i2, int i3) {
        int idx;
        if (!free_list.empty()) {
            idx = free_list.back();
            free_list.pop_back();
        } else {
            idx = (int)tris.size();
            if (idx >= EPA_MAX_TRIANGLES) return -1;
            tris.emplace_back();
            tris.back().index = idx;
        }
        EpaTri &t = tris[idx];
        t.cls = std::numeric_limits<double>::infinity();
        t.lambda[0] = t.lambda[1] = 0.0;
        t.rel0 = t.interior = t.removed = t.inq = false;
        t.e[0].start = i1;
        t.e[1].start = i2;
        t.e[2].start = i3;
        t.e[0].nt = t.e[1].nt = t.e[2].nt = -1;
        V3 y0 = (*pos)[i1], y1 = (*pos)[i2], y2 = (*pos)[i3];
        double cx = (y0.x + y1.x + y2.x) / 3.0, cy = (y0.y + y1.y + y2.y) / 3.0, cz = (y0.z + y1.z + y2.z) / 3.0;
        t.centroid = {cx, cy, cz};
        V3 y10 = sub(y1, y0), y20 = sub(y2, y0), y21 = sub(y2, y1);
        double y20d = y20.x * y20.x + y20.y * y20.y + y20.z * y20.z;
        double y21d = y21.x * y21.x + y21.y * y21.y + y21.z * y21.z;
        if (y20d < y21d) {
            double nx = y10.y * y20.z - y10.z * y20.y, ny = y10.z * y20.x - y10.x * y20.z,
                   nz = y10.x * y20.y - y10.y * y20.x;
            t.normal = {nx, ny, nz};
            double nl = nx * nx + ny * ny + nz * nz;
            if (nl > EPA_MIN_TRIANGLE_AREA) {
                double cdn = cx * nx + cy * ny + cz * nz;
                t.cls = (std::fabs(cdn) * cdn) / nl;
                double y10d = y10.x * y10.x + y10.y * y10.y + y10.z * y10.z;
                double y10y20 = y10.x * y20.x + y10.y * y20.y + y10.z * y20.z;
                double det = y10d * y20d - y10y20 * y10y20;
                if (det > 0.0) {
                    double y0y10 = y0.x * y10.x + y0.y * y10.y + y0.z * y10.z;
                    double y0y20 = y0.x * y20.x + y0.y * y20.y + y0.z * y20.z;
                    double l0 = (y10y20 * y0y20 - y20d * y0y10) / det;
                    double l1 = (y10y20 * y0y10 - y10d * y0y20) / det;
                    t.lambda[0] = l0;
                    t.lambda[1] = l1;
                    t.rel0 = true;
                    if (l0 > -EPA_BARYCENTRIC_EPSILON && l1 > -EPA_BARYCENTRIC_EPSILON &&
                        l0 + l1 < 1.0 + EPA_BARYCENTRIC_EPSILON)
                        t.interior = true;
                }
            }
        } else {
            double nx = y10.y * y21.z - y10.z * y21.y, ny = y10.z * y21.x - y10.x * y21.z,
                   nz = y10.x * y21.y - y10.y * y21.x;
            t.normal = {nx, ny, nz};
            double nl = nx * nx + ny * ny + nz * nz;
            if (nl > EPA_MIN_TRIANGLE_AREA) {
                double cdn = cx * nx + cy * ny + cz * nz;
                t.cls = (std::fabs(cdn) * cdn) / nl;
                double y10d = y10.x * y10.x + y10.y * y10.y + y10.z * y10.z;
                double y10y21 = y10.x * y21.x + y10.y * y21.y + y10.z * y21.z;
                double det = y10d * y21d - y10y21 * y10y21;
                if (det > 0.0) {
                    double y1y10 = y1.x * y10.x + y1.y * y10.y + y1.z * y10.z;
                    double y1y21 = y1.x * y21.x + y1.y * y21.y + y1.z * y21.z;
                    double l0 = (y21d * y1y10 - y10y21 * y1y21) / det;
                    double l1 = (y10y21 * y1y10 - y10d * y1y21) / det;
                    t.lambda[0] = l0;
                    t.lambda[1] = l1;
                    t.rel0 = false;
                    if (l0 > -EPA_BARYCENTRIC_EPSILON && l1 > -EPA_BARYCENTRIC_EPSILON &&
                        l0 + l1 < 1.0 + EPA_BARYCENTRIC_EPSILON)
                        t.interior = true;
                }
            }
        }
        return idx;
    }
    // initialize :347-371
    bool initialize(int i1, int i2, int i3) {
        free_list.resize(tris.size());
        for (size_t i = 0; i < tris.size(); i++) free_list[i] = (int)(tris.size() - 1 - i);
        queue.clear();
        int t1 = create(i1, i2, i3);
        int t2 = create(i1, i3, i2);
        if (t1 < 0 || t2 < 0) return false;
        link(t1, 0, t2, 2);
        link(t1, 1, t2, 1);
        link(t1, 2, t2, 0);
        push(t1);
        push(t2);
        return true;
    }
    // findFacingTriangle :427-452
    int find_facing(V3 p) {
        int best = -1;
        double bestd = 0.0;
        for (size_t i = 0; i < queue.size(); i++) {
            EpaTri &t = tris[queue[i]];
            if (t.removed) continue;
            V3 ab = sub(p, t.centroid);
            double d = dot(t.normal, ab);
            if (d > 0.0) {
                double ds = (d * d) / lensq(t.normal);
                if (ds > bestd) {
                    best = queue[i];
                    bestd = ds;
                }
            }
        }
        return best;
    }
    void free_tri(int ti) { free_list.push_back(ti); }
    void unlink(int ti) {  // unlinkTriangle :458-474
        for (int i = 0; i < 3; i++) {
            EpaEdge &e = tris[ti].e[i];
            if (e.nt >= 0) {
                tris[e.nt].e[e.ne].nt = -1;
                e.nt = -1;
            }
        }
        if (!tris[ti].inq) free_tri(ti);
    }
    // findEdge :476-540
    bool find_edge(int facing_t, V3 vertex, std::vector<EpaEdge> &out) {
        out.clear();
        tris[facing_t].removed = true;
        struct SE {
            int t, edge, iter;
        };
        SE stack[EPA_MAX_EDGE_LENGTH];
        int sp = 0;
        stack[0] = {facing_t, 0, -1};
        int next_expected = -1;
        while (true) {
            SE &cur = stack[sp];
            if (++cur.iter >= 3) {
                unlink(cur.t);
                if (--sp < 0) break;
            } else {
                EpaEdge e = tris[cur.t].e[(cur.edge + cur.iter) % 3];
                int n = e.nt;
                if (n >= 0 && !tris[n].removed) {
                    if (facing(tris[n], vertex)) {
                        tris[n].removed = true;
                        sp++;
                        if (sp >= EPA_MAX_EDGE_LENGTH) return false;  // the reference stack is 128 deep
                        stack[sp] = {n, e.ne, 0};
                    } else {
                        if (e.start != next_expected && next_expected != -1) return false;
                        next_expected = tris[n].e[e.ne].start;
                        out.push_back(e);
                    }
                }
            }
        }
        if (!out.empty() && out[0].start != next_expected) return false;
        return out.size() >= 3;
    }
    // addPoint :542-593
    bool add_point(int facing_t, int idx, double closest, std::vector<int> &outT) {
        V3 p = (*pos)[idx];
        std::vector<EpaEdge> edges;
        if (!find_edge(facing_t, p, edges)) return false;
        int ne = (int)edges.size();
        for (int i = 0; i < ne; i++) {
            int in = (i + 1) % ne;
            int nt = create(edges[i].start, edges[in].start, idx);
            if (nt < 0) return false;
            outT.push_back(nt);
            if ((tris[nt].interior && tris[nt].cls < closest) || tris[nt].cls < 0.0) push(nt);
        }
        for (int i = 0; i < ne; i++) {
            int in = (i + 1) % ne;
            link(outT[i], 0, edges[i].nt, edges[i].ne);
            link(outT[i], 1, outT[in], 2);
        }
        return true;
    }
};

// penetrationDepthStepEPA penetration.ts:214-614
inline bool pen_step_epa(PenDepth &out, const Support &A, const Support &B, double tol, const Simplex &sx) {
    std::vector<V3> Y, P, Q;
    Y.reserve(256);
    P.reserve(256);
    Q.reserve(256);
    for (int i = 0; i < sx.size; i++) {
        Y.push_back(sx.pts[i].y);
        P.push_back(sx.pts[i].p);
        Q.push_back(sx.pts[i].q);
    }
    auto add_sup = [&](V3 d) {
        V3 p = A.get(d);
        V3 q = B.get(neg(d));
        Y.push_back(sub(p, q));
        P.push_back(p);
        Q.push_back(q);
        return (int)Y.size() - 1;
    };
    if (Y.size() == 1) {
        Y.pop_back();
        P.pop_back();
        Q.pop_back();
        add_sup({0, 1, 0});
        add_sup({-1, -1, -1});
        add_sup({1, -1, -1});
        add_sup({0, -1, 1});
    } else if (Y.size() == 2) {
        const double COS120 = std::cos(120.0 * M_PI / 180.0);
        const double SIN120 = std::sin(120.0 * M_PI / 180.0);
        const double OMC = 1 - COS120;
        V3 y0 = Y[0], y1 = Y[1];
        double ax = y1.x - y0.x, ay = y1.y - y0.y, az = y1.z - y0.z;
        double al = std::sqrt(ax * ax + ay * ay + az * az);
        double nx = ax / al, ny = ay / al, nz = az / al;
        double d1x, d1y, d1z;
        if (std::fabs(nx) > std::fabs(ny)) {
            double pl = std::sqrt(nx * nx + nz * nz);
            d1x = nz / pl;
            d1y = 0.0;
            d1z = -nx / pl;
        } else {
            double pl = std::sqrt(ny * ny + nz * nz);
            d1x = 0.0;
            d1y = nz / pl;
            d1z = -ny / pl;
        }
        double r00 = COS120 + nx * nx * OMC, r01 = nx * ny * OMC - nz * SIN120, r02 = nx * nz * OMC + ny * SIN120;
        double r10 = ny * nx * OMC + nz * SIN120, r11 = COS120 + ny * ny * OMC, r12 = ny * nz * OMC - nx * SIN120;
        double r20 = nz * nx * OMC - ny * SIN120, r21 = nz * ny * OMC + nx * SIN120, r22 = COS120 + nz * nz * OMC;
        double d2x = r00 * d1x + r01 * d1y + r02 * d1z, d2y = r10 * d1x + r11 * d1y + r12 * d1z,
               d2z = r20 * d1x + r21 * d1y + r22 * d1z;
        double d3x = r00 * d2x + r01 * d2y + r02 * d2z, d3y = r10 * d2x + r11 * d2y + r12 * d2z,
               d3z = r20 * d2x + r21 * d2y + r22 * d2z;
        add_sup({d1x, d1y, d1z});
        add_sup({d2x, d2y, d2z});
        add_sup({d3x, d3y, d3z});
    }
    EpaHull h;
    h.tris.reserve(EPA_MAX_TRIANGLES);
    h.pos = &Y;
    if (!h.initialize(0, 1, 2)) {
        out.status = NOT_COLLIDING;
        return false;
    }
    std::vector<int> nts;
    for (int i = 3; i < (int)Y.size(); i++) {
        int t = h.find_facing(Y[i]);
        if (t >= 0) {
            nts.clear();
            if (!h.add_point(t, i, std::numeric_limits<double>::max(), nts)) {
                out.status = NOT_COLLIDING;
                return false;
            }
        }
    }
    while (true) {
        if (h.queue.empty()) {
            out.status = NOT_COLLIDING;
            return false;
        }
        int t = h.queue[0];
        if (h.tris[t].removed) {
            h.pop();
            if (h.queue.empty()) {
                out.status = NOT_COLLIDING;
                return false;
            }
            h.free_tri(t);
            continue;
        }
        if (h.tris[t].cls >= 0.0) break;
        h.pop();
        int ni = add_sup(h.tris[t].normal);
        V3 w = Y[ni];
        nts.clear();
        if (!h.facing(h.tris[t], w) || !h.add_point(t, ni, std::numeric_limits<double>::max(), nts)) {
            out.status = NOT_COLLIDING;
            return false;
        }
        h.free_tri(t);
        if (h.queue.empty() || (int)Y.size() >= EPA_MAX_POINTS_TO_INCLUDE_ORIGIN_IN_HULL) {
            out.status = NOT_COLLIDING;
            return false;
        }
    }
    double closest = std::numeric_limits<double>::max();
    int last = -1;
    bool flip = false;
    do {
        int t = h.pop();
        if (t < 0) {
            out.status = NOT_COLLIDING;
            return false;
        }
        if (h.tris[t].removed) {
            h.free_tri(t);
            continue;
        }
        if (h.tris[t].cls >= closest) break;
        if (last >= 0) h.free_tri(last);
        last = t;
        V3 tn = h.tris[t].normal;
        int ni = add_sup(tn);
        V3 w = Y[ni];
        double d = tn.x * w.x + tn.y * w.y + tn.z * w.z;
        if (d < 0.0) {
            out.status = NOT_COLLIDING;
            return false;
        }
        double nls = tn.x * tn.x + tn.y * tn.y + tn.z * tn.z;
        double ds = (d * d) / nls;
        if (ds - h.tris[t].cls < h.tris[t].cls * tol) break;
        closest = std::min(closest, ds);
        if (!h.facing(h.tris[t], w)) break;
        nts.clear();
        if (!h.add_point(t, ni, closest, nts)) break;
        bool defect = false;
        for (int k : nts) {
            const EpaTri &q = h.tris[k];
            if (q.normal.x * q.centroid.x + q.normal.y * q.centroid.y + q.normal.z * q.centroid.z < 0.0) {
                defect = true;
                break;
            }
        }
        if (defect) {
            V3 nn = neg(tn);
            V3 p2 = A.get(nn);
            V3 q2 = B.get(tn);
            V3 w2 = sub(p2, q2);
            double d2 = nn.x * w2.x + nn.y * w2.y + nn.z * w2.z;
            if (d2 < d) flip = true;
            break;
        }
    } while (!h.queue.empty() && (int)Y.size() < EPA_MAX_POINTS);
    if (last < 0) {
        out.status = NOT_COLLIDING;
        return false;
    }
    const EpaTri &L = h.tris[last];
    double nls = L.normal.x * L.normal.x + L.normal.y * L.normal.y + L.normal.z * L.normal.z;
    double cdn = L.centroid.x * L.normal.x + L.centroid.y * L.normal.y + L.centroid.z * L.normal.z;
    V3 pn = scale(L.normal, cdn / nls);
    if (pn.x * pn.x + pn.y * pn.y + pn.z * pn.z < 1e-10) {
        out.status = NOT_COLLIDING;
        return false;
    }
    if (flip) pn = neg(pn);
    V3 xp0 = P[L.e[0].start], xp1 = P[L.e[1].start], xp2 = P[L.e[2].start];
    V3 xq0 = Q[L.e[0].start], xq1 = Q[L.e[1].start], xq2 = Q[L.e[2].start];
    double l0 = L.lambda[0], l1 = L.lambda[1];
    V3 ca, cb;
    if (L.rel0) {
        ca = {xp0.x + (xp1.x - xp0.x) * l0 + (xp2.x - xp0.x) * l1, xp0.y + (xp1.y - xp0.y) * l0 + (xp2.y - xp0.y) * l1,
              xp0.z + (xp1.z - xp0.z) * l0 + (xp2.z - xp0.z) * l1};
        cb = {xq0.x + (xq1.x - xq0.x) * l0 + (xq2.x - xq0.x) * l1, xq0.y + (xq1.y - xq0.y) * l0 + (xq2.y - xq0.y) * l1,
              xq0.z + (xq1.z - xq0.z) * l0 + (xq2.z - xq0.z) * l1};
    } else {
        ca = {xp1.x + (xp0.x - xp1.x) * l0 + (xp2.x - xp1.x) * l1, xp1.y + (xp0.y - xp1.y) * l0 + (xp2.y - xp1.y) * l1,
              xp1.z + (xp0.z - xp1.z) * l0 + (xp2.z - xp1.z) * l1};
        cb = {xq1.x + (xq0.x - xq1.x) * l0 + (xq2.x - xq1.x) * l1, xq1.y + (xq0.y - xq1.y) * l0 + (xq2.y - xq1.y) * l1,
              xq1.z + (xq0.z - xq1.z) * l0 + (xq2.z - xq1.z) * l1};
    }
    out.axis = pn;
    out.pa = ca;
    out.pb = cb;
    out.status = COLLIDING;
    return true;
}

// ----------------------------------------------------------------------------
// Faces, clipping, manifolds (src/utils/face.ts, src/manifold/clip.ts, manifold.ts)
// ----------------------------------------------------------------------------
constexpr int FACE_MAX_VERTICES = 64;
struct Face {
    int n = 0;
    V3 v[FACE_MAX_VERTICES];
};

// transformFace face.ts:30-80 (unit scale)
inline void transform_face(Face &f, V3 p, Q4 q) {
    double qx2 = q.x + q.x, qy2 = q.y + q.y, qz2 = q.z + q.z;
    double qxx = q.x * qx2, qyx = q.y * qx2, qyy = q.y * qy2, qzx = q.z * qx2, qzy = q.z * qy2, qzz = q.z * qz2,
           qwx = q.w * qx2, qwy = q.w * qy2, qwz = q.w * qz2;
    double m00 = (1 - qyy - qzz) * 1.0, m01 = (qyx + qwz) * 1.0, m02 = (qzx - qwy) * 1.0;
    double m10 = (qyx - qwz) * 1.0, m11 = (1 - qxx - qzz) * 1.0, m12 = (qzy + qwx) * 1.0;
    double m20 = (qzx + qwy) * 1.0, m21 = (qzy - qwx) * 1.0, m22 = (1 - qxx - qyy) * 1.0;
    for (int i = 0; i < f.n; i++) {
        V3 a = f.v[i];
        f.v[i] = {m00 * a.x + m10 * a.y + m20 * a.z + p.x, m01 * a.x + m11 * a.y + m21 * a.z + p.y,
                  m02 * a.x + m12 * a.y + m22 * a.z + p.z};
    }
}

// cylinder getSupportingFace cylinder.ts: the side edge facing away from dir, or the cap
// octagon (CYLINDER_CAP_OCTAGON) turned towards dir's horizontal part
inline void cylinder_supporting_face(Face &f, V3 d, double h, double r) {
    static const double OCT[8][3] = {{0.0, 1.0, 1.0},          {0.707106769, 1.0, 0.707106769},
                                     {1.0, 1.0, 0.0},          {0.707106769, 1.0, -0.707106769},
                                     {0.0, 1.0, -1.0},         {-0.707106769, 1.0, -0.707106769},
                                     {-1.0, 1.0, 0.0},         {-0.707106769, 1.0, 0.707106769}};
    double xz = d.x * d.x + d.z * d.z, yy = d.y * d.y;
    if (xz > yy) {
        double fct = -r / std::sqrt(xz);
        f.n = 2;
        f.v[0] = {d.x * fct, h, d.z * fct};
        f.v[1] = {d.x * fct, -h, d.z * fct};
        return;
    }
    double sx = d.y < 0 ? r : -r, sy = d.y < 0 ? h : -h, sz = r;
    double c = 1, sn = 0;
    if (xz > 0.00765427 * yy) {
        double hl = std::sqrt(xz);
        c = d.x / hl;
        sn = d.z / hl;
    }
    f.n = 8;
    for (int i = 0; i < 8; i++) {
        double x = sx * OCT[i][0], y = sy * OCT[i][1], z = sz * OCT[i][2];
        f.v[i] = {x * c - z * sn, y, x * sn + z * c};
    }
}

// box getSupportingFace box.ts:129-332 (scale not inside out)
inline void box_supporting_face(Face &f, V3 dir, V3 he) {
    double hx = he.x, hy = he.y, hz = he.z;
    double ax = std::fabs(dir.x), ay = std::fabs(dir.y), az = std::fabs(dir.z);
    f.n = 4;
    if (ax >= ay && ax >= az) {
        if (dir.x < 0) {
            f.v[0] = {hx, -hy, -hz};
            f.v[1] = {hx, hy, -hz};
            f.v[2] = {hx, hy, hz};
            f.v[3] = {hx, -hy, hz};
        } else {
            f.v[0] = {-hx, -hy, -hz};
            f.v[1] = {-hx, -hy, hz};
            f.v[2] = {-hx, hy, hz};
            f.v[3] = {-hx, hy, -hz};
        }
    } else if (ay >= ax && ay >= az) {
        if (dir.y < 0) {
            f.v[0] = {-hx, hy, -hz};
            f.v[1] = {-hx, hy, hz};
            f.v[2] = {hx, hy, hz};
            f.v[3] = {hx, hy, -hz};
        } else {
            f.v[0] = {-hx, -hy, -hz};
            f.v[1] = {hx, -hy, -hz};
            f.v[2] = {hx, -hy, hz};
            f.v[3] = {-hx, -hy, hz};
        }
    } else {
        if (dir.z < 0) {
            f.v[0] = {-hx, -hy, hz};
            f.v[1] = {hx, -hy, hz};
            f.v[2] = {hx, hy, hz};
            f.v[3] = {-hx, hy, hz};
        } else {
            f.v[0] = {-hx, -hy, -hz};
            f.v[1] = {-hx, hy, -hz};
            f.v[2] = {hx, hy, -hz};
            f.v[3] = {hx, -hy, -hz};
        }
    }
}

// capsule getSupportingFace capsule.ts:192-251: the segment on the side opposite to the
// direction when both caps project within the capsule projection slop, else no face
inline void capsule_supporting_face(Face &f, V3 d, double h, double r) {
    double len = std::sqrt(d.x * d.x + d.z * d.z);
    if (len == 0.0) {
        f.n = 0;
        return;
    }
    double sx = (r / len) * d.x, sz = (r / len) * d.z;
    V3 top{-sx, h, -sz}, bottom{-sx, -h, -sz};
    double pt = top.x * d.x + top.y * d.y + top.z * d.z;
    double pb = bottom.x * d.x + bottom.y * d.y + bottom.z * d.z;
    const double slop = 0.02;  // cCapsuleProjectionSlop
    double dl = std::sqrt(d.x * d.x + d.y * d.y + d.z * d.z);
    if (std::fabs(pt - pb) < slop * dl) {
        f.n = 2;
        f.v[0] = top;
        f.v[1] = bottom;
    } else {
        f.n = 0;
    }
}

// convex hull getSupportingFace convex-hull.ts:479-541 (unit scale): the face whose plane normal
// is most opposed to dir; at most MAX_FACE_VERTICES / 2 = 16 of its vertices
inline void hull_supporting_face(Face &f, V3 dir, const HullData &h) {
    int best = 0;
    double bd = 0;
    for (size_t i = 0; i < h.plane_n.size(); i++) {
        V3 n = h.plane_n[i];
        double d = (n.x * dir.x + n.y * dir.y + n.z * dir.z) / std::sqrt(n.x * n.x + n.y * n.y + n.z * n.z);
        if (i == 0 || d < bd) {
            bd = d;
            best = (int)i;
        }
    }
    int first = h.face_first[best], nv = h.face_count[best];
    const int maxv = 32 / 2;
    int step = (nv + maxv - 1) / maxv;
    f.n = 0;
    for (int i = 0; i < nv; i += step) f.v[f.n++] = h.points[h.vidx[first + i]];
}

// getShapeSupportingFace shapes.ts:489-508 (sphere has no face)
inline void shape_supporting_face(Face &f, const Shape &s, V3 dir, V3 p, Q4 q) {
    if (s.type == SHAPE_CONVEX_HULL) {
        hull_supporting_face(f, dir, *s.hull);
        transform_face(f, p, q);
    } else if (s.type == SHAPE_BOX) {
        box_supporting_face(f, dir, s.half_extents);
        transform_face(f, p, q);
    } else if (s.type == SHAPE_CAPSULE) {
        capsule_supporting_face(f, dir, s.half_height, s.radius);
        if (f.n > 0) transform_face(f, p, q);
    } else if (s.type == SHAPE_CYLINDER) {
        cylinder_supporting_face(f, dir, s.half_height, s.radius);
        transform_face(f, p, q);
    } else {
        f.n = 0;
    }
}

// clipPolyVsPlane clip.ts:13-92
inline void clip_poly_vs_plane(Face &out, const Face &in, V3 o, V3 n) {
    out.n = 0;
    if (in.n < 2) return;
    V3 e1 = in.v[in.n - 1];
    double prevNum = (o.x - e1.x) * n.x + (o.y - e1.y) * n.y + (o.z - e1.z) * n.z;
    bool prevIn = prevNum < 0.0;
    for (int j = 0; j < in.n; j++) {
        V3 e2 = in.v[j];
        double num = (o.x - e2.x) * n.x + (o.y - e2.y) * n.y + (o.z - e2.z) * n.z;
        bool curIn = num < 0.0;
        if (curIn != prevIn) {
            V3 e12 = sub(e2, e1);
            double den = e12.x * n.x + e12.y * n.y + e12.z * n.z;
            if (den != 0.0) {
                double t = prevNum / den;
                if (out.n < FACE_MAX_VERTICES) out.v[out.n] = {e1.x + e12.x * t, e1.y + e12.y * t, e1.z + e12.z * t};
                out.n++;
            } else {
                curIn = prevIn;
            }
        }
        if (curIn) {
            if (out.n < FACE_MAX_VERTICES) out.v[out.n] = e2;
            out.n++;
        }
        prevNum = num;
        prevIn = curIn;
        e1 = e2;
    }
    if (out.n > FACE_MAX_VERTICES) out.n = FACE_MAX_VERTICES;
}

// clipPolyVsPoly clip.ts:108-175
inline void clip_poly_vs_poly(Face &out, const Face &toClip, const Face &clipping, V3 clipNormal) {
    out.n = 0;
    if (toClip.n < 2) return;
    if (clipping.n < 3) return;
    static thread_local Face tmp[2];
    int tmpIdx = 0;
    for (int i = 0; i < clipping.n; i++) {
        V3 c1 = clipping.v[i];
        V3 c2 = clipping.v[(i + 1) % clipping.n];
        V3 e = sub(c2, c1);
        V3 cn{clipNormal.y * e.z - clipNormal.z * e.y, clipNormal.z * e.x - clipNormal.x * e.z,
              clipNormal.x * e.y - clipNormal.y * e.x};
        const Face *src = (i == 0) ? &toClip : (tmpIdx == 0 ? &tmp[0] : &tmp[1]);
        tmpIdx ^= 1;
        Face *dst = (i == clipping.n - 1) ? &out : (tmpIdx == 0 ? &tmp[0] : &tmp[1]);
        clip_poly_vs_plane(*dst, *src, c1, cn);
        if (dst->n < 3) {
            out.n = 0;
            break;
        }
    }
}

struct Manifold {
    int n = 0;
    V3 base;
    V3 relA[FACE_MAX_VERTICES], relB[FACE_MAX_VERTICES];
    V3 normal;
    double depth = 0;
    uint32_t subA = EMPTY_SUB_SHAPE_ID, subB = EMPTY_SUB_SHAPE_ID;
};

// setContactPoint manifold.ts:134-145
inline void set_contact_point(Manifold &m, int i, V3 a, V3 b) {
    m.relA[i] = sub(a, m.base);
    m.relB[i] = sub(b, m.base);
}

// pruneContactPoints manifold.ts:192-311
inline void prune_contact_points(Manifold &m, V3 axis) {
    constexpr double MIN_DISTANCE_SQ = 1.0e-6;
    if (m.n <= 4) return;
    std::vector<V3> proj(m.n);
    std::vector<double> dsq(m.n);
    for (int i = 0; i < m.n; i++) {
        V3 v1 = m.relA[i], v2 = m.relB[i];
        double d = dot(v1, axis);
        proj[i] = scale_add(v1, axis, -d);
        dsq[i] = std::max(MIN_DISTANCE_SQ, lensq(sub(v2, v1)));
    }
    int p1 = 0;
    double mm = std::max(MIN_DISTANCE_SQ, lensq(proj[0])) * dsq[0];
    for (int i = 1; i < m.n; i++) {
        double met = std::max(MIN_DISTANCE_SQ, lensq(proj[i])) * dsq[i];
        if (met > mm) {
            mm = met;
            p1 = i;
        }
    }
    int p2 = -1;
    mm = -std::numeric_limits<double>::infinity();
    for (int i = 0; i < m.n; i++) {
        if (i != p1) {
            double met = std::max(MIN_DISTANCE_SQ, lensq(sub(proj[i], proj[p1]))) * dsq[i];
            if (met > mm) {
                mm = met;
                p2 = i;
            }
        }
    }
    int p3 = -1, p4 = -1;
    double minD = 0.0, maxD = 0.0;
    V3 edge = sub(proj[p2], proj[p1]);
    V3 perp = cross(edge, axis);
    for (int i = 0; i < m.n; i++) {
        if (i != p1 && i != p2) {
            double d = dot(sub(proj[i], proj[p1]), perp);
            if (d < minD) {
                minD = d;
                p3 = i;
            } else if (d > maxD) {
                maxD = d;
                p4 = i;
            }
        }
    }
    int order[4] = {p1, p3, p2, p4};
    int o = 0;
    for (int k = 0; k < 4; k++) {
        int s = order[k];
        if (s != -1) {
            if (o != s) {
                m.relA[o] = m.relA[s];
                m.relB[o] = m.relB[s];
            }
            o++;
        }
    }
    m.n = o;
}

// clipPolyVsEdge clip.ts:190-363: the polygon's crossings of the plane through the edge
// (normal = clipNormal x edge), snapped onto the edge projected into the polygon's plane
inline void clip_poly_vs_edge(Face &out, const Face &poly, V3 ev1, V3 ev2, V3 clipNormal) {
    out.n = 0;
    if (poly.n < 3) return;
    V3 edge = sub(ev2, ev1);
    V3 en = cross(clipNormal, edge);
    V3 p0 = poly.v[0], p1 = poly.v[1], p2 = poly.v[2];
    V3 pn = cross(sub(p2, p0), sub(p1, p0));
    double pl2 = dot(pn, pn);
    V3 v1 = scale_add(ev1, pn, dot(sub(p0, ev1), pn) / pl2);
    V3 v2 = scale_add(ev2, pn, dot(sub(p0, ev2), pn) / pl2);
    V3 v12 = sub(v2, v1);
    double v12l2 = dot(v12, v12);
    V3 e1 = poly.v[poly.n - 1];
    double prevNum = dot(sub(ev1, e1), en);
    bool prevIn = prevNum < 0.0;
    for (int j = 0; j < poly.n; j++) {
        V3 e2 = poly.v[j];
        double num = dot(sub(ev1, e2), en);
        bool curIn = num < 0.0;
        if (curIn != prevIn) {
            V3 e12 = sub(e2, e1);
            double den = dot(e12, en);
            V3 c = den != 0.0 ? scale_add(e1, e12, prevNum / den) : e1;
            double proj = dot(sub(c, v1), v12);
            V3 o = proj < 0.0 ? v1 : (proj > v12l2 ? v2 : c);
            if (out.n < FACE_MAX_VERTICES) out.v[out.n] = o;
            out.n++;
        }
        prevNum = num;
        prevIn = curIn;
        e1 = e2;
    }
    if (out.n > FACE_MAX_VERTICES) out.n = FACE_MAX_VERTICES;
}

// manifoldBetweenTwoFaces manifold.ts:345-444
inline void manifold_between_faces(Manifold &out, V3 cp1, V3 cp2, V3 axis, double maxDist, const Face &f1,
                                   const Face &f2) {
    out.n = 0;
    if (f1.n < 2 || f2.n < 3) {
        set_contact_point(out, 0, cp1, cp2);
        out.n = 1;
        return;
    }
    static thread_local Face clipped;
    clipped.n = 0;
    if (f1.n >= 3) {
        clip_poly_vs_poly(clipped, f2, f1, axis);
    } else if (f1.n == 2) {
        clip_poly_vs_edge(clipped, f2, f1.v[0], f1.v[1], axis);
    }
    V3 po = f1.v[0];
    V3 e1 = f1.v[1];
    V3 first = sub(e1, po);
    V3 pn;
    if (f1.n >= 3) {
        V3 second = sub(f1.v[2], po);
        pn = cross(first, second);
    } else {
        V3 perp = cross(first, axis);
        pn = cross(perp, first);
    }
    double adn = dot(axis, pn);
    if (adn != 0.0) {
        double al = len(axis);
        for (int i = 0; i < clipped.n; i++) {
            V3 p2 = clipped.v[i];
            double dist = dot(sub(p2, po), pn) / adn;
            if (dist * al < maxDist) {
                V3 p1 = scale_add(p2, axis, -dist);
                set_contact_point(out, out.n, p1, p2);
                out.n++;
                if (out.n >= FACE_MAX_VERTICES) break;
            }
        }
    }
    if (out.n == 0) {
        set_contact_point(out, 0, cp1, cp2);
        out.n = 1;
    }
}

// Hit produced by a shape-vs-shape collision (collide-shape-vs-shape.ts:8-31)
struct Hit {
    V3 pa, pb, axis;
    double penetration = 0;
    uint32_t subA = EMPTY_SUB_SHAPE_ID, subB = EMPTY_SUB_SHAPE_ID;
    Face faceA, faceB;
};

struct CollideSettings {
    double maxSeparation = 0.02;
    double collisionTolerance = 1e-4;
    double penetrationTolerance = 1e-4;
    bool collectFaces = true;
    bool collideWithBackfaces = false;  // the narrowphase's; collideShape queries default to true
};

// collideConvexVsConvex convex.ts:257-346 + collideConvexVsConvexLocal convex.ts:359-641
// Returns true and fills `hit` when the shapes touch within the separation distance.
inline bool collide_convex_vs_convex(Hit &hit, const CollideSettings &cs, const Shape &sa, V3 pA, Q4 qA,
                                     const Shape &sb, V3 pB, Q4 qB) {
    double iax = -qA.x, iay = -qA.y, iaz = -qA.z, iaw = qA.w;
    Q4 rel{iaw * qB.x + iax * qB.w + iay * qB.z - iaz * qB.y, iaw * qB.y - iax * qB.z + iay * qB.w + iaz * qB.x,
           iaw * qB.z + iax * qB.y - iay * qB.x + iaz * qB.w, iaw * qB.w - iax * qB.x - iay * qB.y - iaz * qB.z};
    double abx = pB.x - pA.x, aby = pB.y - pA.y, abz = pB.z - pA.z;
    double qx = iax, qy = iay, qz = iaz, qw = iaw;
    double uvx = qy * abz - qz * aby + qw * abx, uvy = qz * abx - qx * abz + qw * aby,
           uvz = qx * aby - qy * abx + qw * abz;
    double uuvx = qy * uvz - qz * uvy, uuvy = qz * uvx - qx * uvz, uuvz = qx * uvy - qy * uvx;
    V3 posBInA{abx + 2 * uuvx, aby + 2 * uuvy, abz + 2 * uuvz};

    Support supA = make_support(sa, EXCLUDE_CONVEX_RADIUS);
    Support supB = make_support(sb, EXCLUDE_CONVEX_RADIUS);
    supB.transformed = true;
    supB.m = mat4_from_rt(rel, posBInA);
    V3 axis = posBInA;
    if (axis.x * axis.x + axis.y * axis.y + axis.z * axis.z <= 1e-12) axis = {1, 0, 0};
    Simplex sx;
    double maxSep = cs.maxSeparation;
    PenDepth pd = pen_step_gjk(sx, supA, supB, supA.convex_radius + maxSep, supB.convex_radius, axis,
                               cs.collisionTolerance);
    if (pd.status == NOT_COLLIDING) return false;
    if (pd.status == INDETERMINATE) {
        maxSep = std::min(maxSep, 1.0);
        Support a2 = make_support(sa, INCLUDE_CONVEX_RADIUS);
        Support b2 = make_support(sb, INCLUDE_CONVEX_RADIUS);
        a2.add_radius = true;
        a2.add_r = maxSep;
        b2.transformed = true;
        b2.m = mat4_from_rt(rel, posBInA);
        if (!pen_step_epa(pd, a2, b2, cs.penetrationTolerance, sx)) return false;
    }
    double dx = pd.pa.x - pd.pb.x, dy = pd.pa.y - pd.pb.y, dz = pd.pa.z - pd.pb.z;
    double penetration = std::sqrt(dx * dx + dy * dy + dz * dz) - maxSep;
    // collector.earlyOutFraction is Number.MAX_VALUE for the narrowphase collectors (update.ts:349)
    V3 pax = pd.axis;
    double pal = std::sqrt(pax.x * pax.x + pax.y * pax.y + pax.z * pax.z);
    if (pal > 0.0) {
        double corr = maxSep / pal;
        pd.pa.x += pax.x * -corr;
        pd.pa.y += pax.y * -corr;
        pd.pa.z += pax.z * -corr;
    }
    auto to_world = [&](V3 v) {
        double qax = qA.x, qay = qA.y, qaz = qA.z, qaw = qA.w;
        double ux = qay * v.z - qaz * v.y + qaw * v.x, uy = qaz * v.x - qax * v.z + qaw * v.y,
               uz = qax * v.y - qay * v.x + qaw * v.z;
        double wx = qay * uz - qaz * uy, wy = qaz * ux - qax * uz, wz = qax * uy - qay * ux;
        return V3{v.x + 2 * wx, v.y + 2 * wy, v.z + 2 * wz};
    };
    V3 ca = to_world(pd.pa);
    hit.pa = {ca.x + pA.x, ca.y + pA.y, ca.z + pA.z};
    V3 cb = to_world(pd.pb);
    hit.pb = {cb.x + pA.x, cb.y + pA.y, cb.z + pA.z};
    hit.axis = to_world(pd.axis);
    hit.penetration = penetration;
    hit.subA = EMPTY_SUB_SHAPE_ID;
    hit.subB = EMPTY_SUB_SHAPE_ID;
    hit.faceA.n = 0;
    hit.faceB.n = 0;
    if (cs.collectFaces) {
        shape_supporting_face(hit.faceA, sa, neg(pd.axis), pA, qA);
        double cx = -rel.x, cy = -rel.y, cz = -rel.z, cw = rel.w;
        V3 fa = pd.axis;
        double px = cy * fa.z - cz * fa.y + cw * fa.x, py = cz * fa.x - cx * fa.z + cw * fa.y,
               pz = cx * fa.y - cy * fa.x + cw * fa.z;
        double ddx = cy * pz - cz * py, ddy = cz * px - cx * pz, ddz = cx * py - cy * px;
        V3 dirB{fa.x + 2 * ddx, fa.y + 2 * ddy, fa.z + 2 * ddz};
        V3 pbw = to_world(posBInA);
        V3 posB{pbw.x + pA.x, pbw.y + pA.y, pbw.z + pA.z};
        Q4 quatB{qA.w * rel.x + qA.x * rel.w + qA.y * rel.z - qA.z * rel.y,
                 qA.w * rel.y - qA.x * rel.z + qA.y * rel.w + qA.z * rel.x,
                 qA.w * rel.z + qA.x * rel.y - qA.y * rel.x + qA.z * rel.w,
                 qA.w * rel.w - qA.x * rel.x - qA.y * rel.y - qA.z * rel.z};
        shape_supporting_face(hit.faceB, sb, dirB, posB, quatB);
    }
    return true;
}

// collideSphereVsSphere sphere.ts:319-410
inline bool collide_sphere_vs_sphere(Hit &hit, const Shape &sa, V3 pA, const Shape &sb, V3 pB) {
    double rA = sa.radius * 1.0, rB = sb.radius * 1.0;
    double dx = pB.x - pA.x, dy = pB.y - pA.y, dz = pB.z - pA.z;
    double ds = dx * dx + dy * dy + dz * dz;
    double rs = rA + rB;
    if (ds >= rs * rs) return false;
    double d = std::sqrt(ds);
    double pen = rs - d;
    V3 n;
    if (d > 0) {
        double inv = 1 / d;
        n = {dx * inv, dy * inv, dz * inv};
    } else {
        n = {0, 1, 0};
    }
    hit.pa = {pA.x + n.x * rA, pA.y + n.y * rA, pA.z + n.z * rA};
    hit.pb = {pB.x - n.x * rB, pB.y - n.y * rB, pB.z - n.z * rB};
    hit.axis = n;
    hit.penetration = pen;
    hit.subA = hit.subB = EMPTY_SUB_SHAPE_ID;
    hit.faceA.n = 0;
    hit.faceB.n = 0;
    return true;
}

// ----------------------------------------------------------------------------
// Shape cast (gjk.ts:853-1259, penetration.ts:621-699, convex.ts:675-900)
// ----------------------------------------------------------------------------
struct CastHit {
    double fraction = 0;
    V3 pa, pb, axis;  // world-space points and the unnormalised penetration axis
};

// ---- plane shape (src/shapes/plane.ts) ------------------------------------------------
// getOrthogonalBasis :210-233
inline void plane_basis(V3 n, V3 &p1, V3 &p2) {
    p1 = cross(n, V3{0, 1, 0});
    double l = lensq(p1);
    p1 = l < 1e-6 ? V3{1, 0, 0} : scale(p1, 1 / std::sqrt(l));
    p2 = normalize(cross(p1, n));
    p1 = normalize(cross(n, p2));
}
// getPlaneVertices :235-271
inline void plane_vertices(V3 out[4], V3 n, double c, double he) {
    V3 p1, p2;
    plane_basis(n, p1, p2);
    p1 = scale(p1, he);
    p2 = scale(p2, he);
    V3 pt = scale(n, -c);
    out[0] = add(pt, add(p1, p2));
    out[1] = add(pt, sub(p1, p2));
    out[2] = sub(pt, add(p1, p2));
    out[3] = add(pt, add(neg(p1), p2));
}
// computePlaneLocalBounds :273-295: the face's corners and the corners one half extent behind
inline Box3 plane_local_bounds(V3 n, double c, double he) {
    V3 v[4];
    plane_vertices(v, n, c, he);
    Box3 b{{1e300, 1e300, 1e300}, {-1e300, -1e300, -1e300}};
    auto grow = [&](V3 p) {
        b.mn = {std::min(b.mn.x, p.x), std::min(b.mn.y, p.y), std::min(b.mn.z, p.z)};
        b.mx = {std::max(b.mx.x, p.x), std::max(b.mx.y, p.y), std::max(b.mx.z, p.z)};
    };
    for (V3 p : v) {
        grow(p);
        grow(sub(p, scale(n, he)));
    }
    return b;
}
// transformPlane :196-208 for a rotation and translation
inline void transform_plane(V3 &n, double &c, V3 n0, double c0, Q4 q, V3 t) {
    n = rotate(q, n0);
    c = c0 - dot(t, n);
}
// getAdaptivePlaneSupportingFace :655-706: a square on the world plane centred under the convex
// shape's position, |size of its bounds| from the centre to each side
inline void plane_adaptive_face(Face &f, const Shape &convex, V3 convexPos, V3 nw, double cw) {
    V3 center = sub(convexPos, scale(nw, dot(nw, convexPos) + cw));
    V3 p1, p2;
    plane_basis(nw, p1, p2);
    const Box3 &a = convex.decorated ? convex.leafAabb : convex.aabb;
    double size = len(sub(a.mx, a.mn));
    p1 = scale(p1, size);
    p2 = scale(p2, size);
    f.n = 4;
    f.v[0] = add(center, add(p1, p2));
    f.v[1] = add(center, sub(p1, p2));
    f.v[2] = sub(center, add(p1, p2));
    f.v[3] = add(center, add(neg(p1), p2));
}
// collideConvexVsPlane :474-629: A convex at (pA, qA), B the plane shape at (pB, qB)
inline bool collide_convex_vs_plane(Hit &hit, const CollideSettings &cs, const Shape &sa, V3 pA, Q4 qA,
                                    const Shape &sb, V3 pB, Q4 qB) {
    // the plane in A's frame: inverse(A) x B
    Q4 iqA = qconj(qA);
    V3 nl;
    double cl;
    transform_plane(nl, cl, sb.pn, sb.pc, qmul(iqA, qB), rotate(iqA, sub(pB, pA)));
    Support S = make_support_default(sa);
    V3 sp = S.get(neg(nl));
    double sd = dot(nl, sp) + cl;
    double cr = S.convex_radius;
    double pen = -sd + cr;
    if (!(pen > -cs.maxSeparation)) return false;
    V3 p1 = sub(sp, scale(nl, cr)), p2 = sub(sp, scale(nl, sd));
    hit.pa = add(pA, rotate(qA, p1));
    hit.pb = add(pA, rotate(qA, p2));
    hit.axis = rotate(qA, neg(nl));
    hit.penetration = pen;
    hit.faceA.n = hit.faceB.n = 0;
    if (cs.collectFaces) {
        shape_supporting_face(hit.faceA, sa, nl, pA, qA);
        if (hit.faceA.n > 0) {
            V3 nw;
            double cw;
            transform_plane(nw, cw, sb.pn, sb.pc, qB, pB);
            plane_adaptive_face(hit.faceB, sa, pA, nw, cw);
        }
    }
    return true;
}
// castRayVsPlane :320-398 (treatConvexAsSolid, back faces culled unless asked)
inline bool cast_ray_vs_plane(const Shape &s, V3 pos, Q4 q, V3 origin, V3 dir, double length, bool solid,
                              bool backfaces, double maxFraction, double &fraction) {
    V3 n;
    double c;
    transform_plane(n, c, s.pn, s.pc, q, pos);
    double d = dot(n, origin) + c;
    if (solid && d <= 0.0 && maxFraction > 0.0) {
        fraction = 0;
        return true;
    }
    double dn = dot(dir, n);
    if (std::fabs(dn) < 1e-10) return false;
    if (!backfaces && dn > 0.0) return false;
    double f = -d / dn / length;
    if (f >= 0.0 && f < maxFraction) {
        fraction = f;
        return true;
    }
    return false;
}
// collidePointVsPlane :404-460
inline bool point_in_plane(const Shape &s, V3 pos, Q4 q, V3 point) {
    V3 n;
    double c;
    transform_plane(n, c, s.pn, s.pc, q, pos);
    return dot(n, point) + c < 0.0;
}
// castConvexVsPlane :727-918: the plane's own (unposed) equation against the world support point,
// the hit's points carried by the plane body's transform, as the reference computes them
inline bool cast_convex_vs_plane(CastHit &hit, const Shape &sa, V3 pA, Q4 qA, V3 disp, const Shape &sb, V3 pB, Q4 qB,
                                 double earlyOut, bool backfaces) {
    const V3 n = sb.pn;
    Support S = make_support_default(sa);
    V3 nInA = neg(rotate(qconj(qA), n));
    V3 spw = add(pA, rotate(qA, S.get(nInA)));
    double sd = dot(n, spw) + sb.pc;
    double cr = S.convex_radius;
    double pen = -sd + cr;
    double dn = dot(disp, n);
    double fraction;
    V3 p1, p2;
    Q4 hq = qB;
    V3 ht = pB;
    if (pen > 0.0) {
        if (!backfaces && dn > 0.0) return false;
        if (pen <= -earlyOut) return false;
        fraction = 0;
        p1 = add(pB, rotate(qB, sub(spw, scale(n, cr))));
        p2 = add(pB, rotate(qB, sub(spw, scale(n, sd))));
    } else if (dn < 0.0) {
        fraction = pen / dn;
        if (fraction >= earlyOut) return false;
        // mat4.translate(planeToWorld, disp x fraction): the translation goes through the rotation
        ht = add(pB, rotate(qB, scale(disp, fraction)));
        p1 = add(ht, rotate(qB, sub(spw, scale(n, cr))));
        p2 = p1;
    } else {
        return false;
    }
    hit.fraction = fraction;
    hit.pa = p1;
    hit.pb = p2;
    // vec3.transformMat4 of -n by comHit (a point transform: the translation is added)
    hit.axis = add(ht, rotate(hq, neg(n)));
    return true;
}

// gjkCastShape gjk.ts:853-1259.  A (already placed in B's space) moves by disp, B is fixed;
// returns false on a miss, else the time of impact and the closest points at that time.
inline bool gjk_cast_shape(double &lambdaOut, V3 &pa, V3 &pb, V3 &axisOut, const Support &A, const Support &B,
                           V3 disp, double tol, double rA, double rB, double maxLambda) {
    double sqtol = tol * tol;
    const double sumR = rA + rB;
    Simplex sx;
    double lambda = 0.0;
    V3 x{0, 0, 0};
    // the starting direction: the negated support of B plus the negated support of A at the
    // zero direction (gjk.ts:882-897)
    V3 q = neg(B.get({0, 0, 0}));
    V3 p = A.get({0, 0, 0});
    V3 v = sub(q, p);
    double vLenSq = std::numeric_limits<double>::max();
    bool allowRestart = false;
    V3 prevV{0, 0, 0};
    for (int it = 0; it < GJK_MAX_ITERATIONS; it++) {
        p = A.get(neg(v));
        q = B.get(v);
        V3 w = sub(x, sub(q, p));
        double vdw = dot(v, w) - sumR * std::sqrt(lensq(v));
        if (vdw > 0.0) {
            double vdr = dot(v, disp);
            if (vdr >= -1.0e-18) return false;
            double old = lambda;
            lambda -= vdw / vdr;
            if (old == lambda) break;
            if (lambda >= maxLambda) return false;
            x = scale(disp, lambda);
            vLenSq = std::numeric_limits<double>::max();
            sqtol = (tol + sumR) * (tol + sumR);
            allowRestart = true;
        }
        sx.pts[sx.size].p = p;
        sx.pts[sx.size].q = q;
        sx.size++;
        for (int i = 0; i < sx.size; i++) sx.pts[i].y = add(sub(x, sx.pts[i].q), sx.pts[i].p);
        ClosestToSimplex c;
        if (closest_to_simplex(c, vLenSq, false, sx)) {
            vLenSq = c.sqdist;
            v = c.point;
        } else {
            if (!allowRestart) break;
            allowRestart = false;
            sx.pts[0].p = p;
            sx.pts[0].q = q;
            sx.size = 1;
            v = sub(x, q);
            vLenSq = std::numeric_limits<double>::max();
            continue;
        }
        if (c.set == 0xf) break;
        // updatePointSetPQ gjk.ts:799-813
        int ns = 0;
        for (int i = 0; i < sx.size; i++)
            if (c.set & (1 << i)) {
                if (ns != i) {
                    sx.pts[ns].p = sx.pts[i].p;
                    sx.pts[ns].q = sx.pts[i].q;
                }
                ns++;
            }
        sx.size = ns;
        if (vLenSq <= sqtol) break;
        prevV = v;
    }
    for (int i = 0; i < sx.size; i++) sx.pts[i].y = add(sub(x, sx.pts[i].q), sx.pts[i].p);
    double vl = std::sqrt(lensq(v));
    V3 nv = vl > 0 ? scale(v, 1 / vl) : V3{0, 0, 0};
    V3 sa{0, 0, 0}, sb{0, 0, 0};
    if (sx.size == 1) {
        sb = sx.pts[0].q;
        sa = sx.pts[0].p;
    } else if (sx.size == 2) {
        Bary b = bary2(sx.pts[0].y, sx.pts[1].y, 1e-10);
        sb = add(scale(sx.pts[0].q, b.u), scale(sx.pts[1].q, b.v));
        sa = add(scale(sx.pts[0].p, b.u), scale(sx.pts[1].p, b.v));
    } else if (sx.size >= 3) {
        Bary b = bary3(sx.pts[0].y, sx.pts[1].y, sx.pts[2].y, 1e-10);
        sb = add(add(scale(sx.pts[0].q, b.u), scale(sx.pts[1].q, b.v)), scale(sx.pts[2].q, b.w));
        sa = add(add(scale(sx.pts[0].p, b.u), scale(sx.pts[1].p, b.v)), scale(sx.pts[2].p, b.w));
    }
    if (sx.size >= 1) {
        pb = scale_add(sb, nv, rB);
        pa = lambda > 0.0 ? pb : scale_add(sa, nv, -rA);
    } else {
        pa = pb = {0, 0, 0};
    }
    lambdaOut = lambda;
    axisOut = sumR > 0.0 ? neg(v) : neg(prevV);
    return true;
}

// castConvexVsConvex convex.ts:675-742 and castConvexVsConvexLocal convex.ts:744-900 with
// penetrationCastShape penetration.ts:621-699, for the continuous-collision query
// (update.ts:1210-1240): no deepest point, no faces, back faces culled.  maxLambda is the
// collector's early-out fraction.
inline bool cast_convex_vs_convex(CastHit &hit, const Shape &sa, V3 pA, Q4 qA, V3 disp, const Shape &sb, V3 pB,
                                  Q4 qB, double maxLambda, bool collideWithBackfaces) {
    Q4 iqB = qconj(qB);
    V3 posAInB = rotate(iqB, sub(pA, pB));
    Q4 qAInB = qmul(iqB, qA);
    V3 dInB = rotate(iqB, disp);
    Support A = make_support(sa, EXCLUDE_CONVEX_RADIUS);
    Support B = make_support(sb, EXCLUDE_CONVEX_RADIUS);
    A.transformed = true;
    A.m = mat4_from_rt(qAInB, posAInB);
    const double tol = 1e-4;
    double lambda;
    V3 pa, pb, axis;
    if (!gjk_cast_shape(lambda, pa, pb, axis, A, B, dInB, tol, A.convex_radius, B.convex_radius, maxLambda))
        return false;
    // an axis shorter than the tolerance is replaced by the cast direction (penetration.ts:693-698)
    if (lensq(axis) < tol * tol) axis = dInB;
    if (lambda > 1.0) return false;
    if (!collideWithBackfaces && dot(axis, dInB) <= 0) return false;
    if (lambda >= maxLambda) return false;
    hit.pa = add(rotate(qB, pa), pB);
    hit.pb = add(rotate(qB, pb), pB);
    hit.axis = rotate(qB, axis);
    hit.fraction = lambda;
    return true;
}

// ----------------------------------------------------------------------------
// Triangle meshes (src/shapes/triangle-mesh.ts, src/collision/active-edges.ts, triangle.ts)
// ----------------------------------------------------------------------------
// fixNormal active-edges.ts:74-153
inline V3 fix_normal(V3 v0, V3 v1, V3 v2, V3 tn, int active, V3 point, V3 normal, V3 move) {
    if (active == 0b111) return normal;
    double nl = len(normal), tl = len(tn);
    if (dot(move, normal) * tl < dot(move, tn) * nl) return normal;
    if (active == 0) return tn;
    if (dot(tn, normal) > 0.999848 * nl * tl) return normal;
    Bary b = bary3(sub(v0, point), sub(v1, point), sub(v2, point), 1e-10);
    const double E = 1.0e-4, OME = 1.0 - 1.0e-4;
    int edge;
    if (b.u > OME)
        edge = 0b101;
    else if (b.v > OME)
        edge = 0b011;
    else if (b.w > OME)
        edge = 0b110;
    else if (b.u < E)
        edge = 0b010;
    else if (b.v < E)
        edge = 0b100;
    else if (b.w < E)
        edge = 0b001;
    else
        return tn;
    return (active & edge) ? normal : tn;
}

// getClosestPointOnTriangle triangle.ts:62-197 (query point at the origin); feature bits:
// vertices A 1, B 2, C 4, an edge its two vertices, the face 7
inline V3 closest_point_on_triangle(V3 a, V3 b, V3 c, double &dsq, int &feature) {
    V3 ab = sub(b, a), ac = sub(c, a);
    V3 n = cross(ab, ac);
    double nl2 = lensq(n);
    if (nl2 < 1e-10) {  // handleDegenerateTriangle triangle.ts:199-287
        V3 best = c;
        feature = 0b100;
        double bd = lensq(c);
        if (lensq(a) < bd) best = a, bd = lensq(a), feature = 0b001;
        if (lensq(b) < bd) best = b, bd = lensq(b), feature = 0b010;
        const double EPS2 = 1.1920929e-7 * 1.1920929e-7;
        auto edge = [&](V3 p, V3 e, int f) {
            double el = lensq(e);
            if (el > EPS2) {
                double v = std::max(0.0, std::min(1.0, -dot(p, e) / el));
                V3 q = scale_add(p, e, v);
                double d = lensq(q);
                if (d < bd) best = q, bd = d, feature = f;
            }
        };
        edge(a, ac, 0b101);
        edge(b, sub(c, b), 0b110);
        edge(a, ab, 0b011);
        dsq = bd;
        return best;
    }
    double d1 = -dot(ab, a), d2 = -dot(ac, a);
    if (d1 <= 0 && d2 <= 0) return dsq = lensq(a), feature = 0b001, a;
    double d3 = -dot(ab, b), d4 = -dot(ac, b);
    if (d3 >= 0 && d4 <= d3) return dsq = lensq(b), feature = 0b010, b;
    if (d1 * d4 <= d3 * d2 && d1 >= 0 && d3 <= 0) {
        V3 p = scale_add(a, ab, d1 / (d1 - d3));
        return dsq = lensq(p), feature = 0b011, p;
    }
    double d5 = -dot(ab, c), d6 = -dot(ac, c);
    if (d6 >= 0 && d5 <= d6) return dsq = lensq(c), feature = 0b100, c;
    if (d5 * d2 <= d1 * d6 && d2 >= 0 && d6 <= 0) {
        V3 p = scale_add(a, ac, d2 / (d2 - d6));
        return dsq = lensq(p), feature = 0b101, p;
    }
    double d43 = d4 - d3, d56 = d5 - d6;
    if (d3 * d6 <= d5 * d4 && d43 >= 0 && d56 >= 0) {
        V3 p = scale_add(b, sub(c, b), d43 / (d43 + d56));
        return dsq = lensq(p), feature = 0b110, p;
    }
    double sc = dot(add(add(a, b), c), n) / (3 * nl2);
    V3 p = scale(n, sc);
    return dsq = lensq(p), feature = 0b111, p;
}

inline uint32_t mesh_sub_shape_id(const MeshData &m, int tri) {  // subShape.pushIndex sub-shape.ts:60-64
    uint32_t mask = m.subBits >= 32 ? 0xffffffffu : ((1u << m.subBits) - 1u);
    return (0xffffffffu & ~mask) | (uint32_t)tri;
}

inline bool node_hits_box(const std::array<double, 8> &nd, const Box3 &q) {  // nodeIntersectsBox bvh.ts:178-196
    return nd[0] <= q.mx.x && nd[3] >= q.mn.x && nd[1] <= q.mx.y && nd[4] >= q.mn.y && nd[2] <= q.mx.z && nd[5] >= q.mn.z;
}

// the mesh BVH walk of the collide functions (triangle-mesh.ts:1122-1134, 1359-1385): a node
// that meets the query box is opened, the child whose centre is nearer the query point first
template <class F>
inline void mesh_walk(const MeshData &M, const Box3 &q, V3 qc, F &&leaf) {
    if (M.nodes.empty()) return;
    std::vector<int> stack{0};
    while (!stack.empty()) {
        int node = stack.back();
        stack.pop_back();
        const auto &nd = M.nodes[node];
        if (!node_hits_box(nd, q)) continue;
        if (nd[7] < 0) {
            int start = (int)nd[6], count = (int)(-nd[7]) - 1;
            for (int t = start; t < start + count; t++) leaf(t);
            continue;
        }
        int left = node + 1, right = (int)nd[6];
        auto centre = [&](int k) {
            const auto &c = M.nodes[k];
            return V3{(c[0] + c[3]) * 0.5, (c[1] + c[4]) * 0.5, (c[2] + c[5]) * 0.5};
        };
        double ld = lensq(sub(qc, centre(left))), rd = lensq(sub(qc, centre(right)));
        if (ld <= rd) {
            stack.push_back(right);
            stack.push_back(left);
        } else {
            stack.push_back(left);
            stack.push_back(right);
        }
    }
}

inline bool box_overlap_incl(const Box3 &a, const Box3 &b) {
    return a.mn.x <= b.mx.x && a.mx.x >= b.mn.x && a.mn.y <= b.mx.y && a.mx.y >= b.mn.y && a.mn.z <= b.mx.z &&
           a.mx.z >= b.mn.z;
}

// collideConvexVsTriangleMesh triangle-mesh.ts:1026-1386 (unit scale): hits in world space,
// A the convex shape, B the mesh
inline void collide_convex_vs_mesh(std::vector<Hit> &out, const CollideSettings &cs, const Shape &sa, V3 pA, Q4 qA,
                                   const Shape &sb, V3 pB, Q4 qB, V3 movement) {
    const MeshData &M = *sb.mesh;
    Q4 iqA = qconj(qA), iqB = qconj(qB);
    Q4 m2cQ = qmul(iqA, qB);
    V3 m2cP = rotate(iqA, sub(pB, pA));
    Q4 cInMQ = qmul(iqB, qA);
    V3 cInMP = rotate(iqB, sub(pA, pB));
    const double ms = cs.maxSeparation;
    const Box3 &la = sa.decorated ? sa.leafAabb : sa.aabb;
    Box3 b1{sub(la.mn, V3{ms, ms, ms}), add(la.mx, V3{ms, ms, ms})};
    Box3 b12{{1e300, 1e300, 1e300}, {-1e300, -1e300, -1e300}};
    for (int c = 0; c < 8; c++) {
        const Box3 &lb = sa.decorated ? sa.leafAabb : sa.aabb;
        V3 p{(c & 1) ? lb.mx.x : lb.mn.x, (c & 2) ? lb.mx.y : lb.mn.y, (c & 4) ? lb.mx.z : lb.mn.z};
        V3 q = add(rotate(cInMQ, p), cInMP);
        b12.mn = {std::min(b12.mn.x, q.x), std::min(b12.mn.y, q.y), std::min(b12.mn.z, q.z)};
        b12.mx = {std::max(b12.mx.x, q.x), std::max(b12.mx.y, q.y), std::max(b12.mx.z, q.z)};
    }
    b12 = {sub(b12.mn, V3{ms, ms, ms}), add(b12.mx, V3{ms, ms, ms})};
    Support supA = make_support(sa, EXCLUDE_CONVEX_RADIUS);
    V3 qc = scale(add(b12.mn, b12.mx), 0.5);
    mesh_walk(M, b12, qc, [&](int t) {
        const auto &tr = M.tris[t];
        V3 a = add(rotate(m2cQ, M.verts[tr[0]]), m2cP), b = add(rotate(m2cQ, M.verts[tr[1]]), m2cP),
           c = add(rotate(m2cQ, M.verts[tr[2]]), m2cP);
        Box3 tb{{std::min(a.x, std::min(b.x, c.x)), std::min(a.y, std::min(b.y, c.y)), std::min(a.z, std::min(b.z, c.z))},
                {std::max(a.x, std::max(b.x, c.x)), std::max(a.y, std::max(b.y, c.y)), std::max(a.z, std::max(b.z, c.z))}};
        if (!box_overlap_incl(tb, b1)) return;
        V3 n = cross(sub(b, a), sub(c, a));
        bool backFacing = dot(n, a) > 0.0;
        if (backFacing && !cs.collideWithBackfaces) return;
        Support tri;
        tri.kind = SUP_TRIANGLE;
        tri.ta = a;
        tri.tb = b;
        tri.tc = c;
        tri.convex_radius = 0;
        V3 axis = neg(n);
        axis = lensq(axis) < 1e-10 ? V3{1, 0, 0} : normalize(axis);
        double maxSep = ms;
        Simplex sx;
        PenDepth pd = pen_step_gjk(sx, supA, tri, supA.convex_radius + maxSep, 0, axis, cs.collisionTolerance);
        if (pd.status == NOT_COLLIDING) return;
        if (pd.status == INDETERMINATE) {
            maxSep = std::min(maxSep, 1.0);
            Support a2 = make_support(sa, INCLUDE_CONVEX_RADIUS);
            a2.add_radius = true;
            a2.add_r = maxSep;
            if (!pen_step_epa(pd, a2, tri, cs.penetrationTolerance, sx)) return;
        }
        double penetration = distance(pd.pa, pd.pb) - maxSep;
        double al = len(pd.axis);
        if (al > 0.0) pd.pa = scale_add(pd.pa, pd.axis, -(maxSep / al));
        if (tr[3] != 0b111) {
            V3 mv = rotate(iqA, movement);
            V3 tn = backFacing ? n : neg(n);
            pd.axis = fix_normal(a, b, c, tn, tr[3], pd.pb, pd.axis, mv);
        }
        Hit h;
        h.pa = add(rotate(qA, pd.pa), pA);
        h.pb = add(rotate(qA, pd.pb), pA);
        h.axis = rotate(qA, pd.axis);
        h.penetration = penetration;
        h.subA = EMPTY_SUB_SHAPE_ID;
        h.subB = mesh_sub_shape_id(M, t);
        shape_supporting_face(h.faceA, sa, neg(pd.axis), pA, qA);
        h.faceB.n = 3;
        h.faceB.v[0] = add(rotate(qA, a), pA);
        h.faceB.v[1] = add(rotate(qA, b), pA);
        h.faceB.v[2] = add(rotate(qA, c), pA);
        out.push_back(h);
    });
}

// collideSphereVsTriangleMesh triangle-mesh.ts:1418-1712 (unit scale)
inline void collide_sphere_vs_mesh(std::vector<Hit> &out, const CollideSettings &cs, const Shape &sa, V3 pA,
                                   const Shape &sb, V3 pB, Q4 qB, V3 movement) {
    static const int FEATURE_TO_ACTIVE_EDGES[8] = {0b000, 0b101, 0b011, 0b001, 0b110, 0b100, 0b010, 0b000};
    const MeshData &M = *sb.mesh;
    const double r = sa.radius, ms = cs.maxSeparation;
    const double maxSq = (r + ms) * (r + ms);
    Q4 iqB = qconj(qB);
    V3 c = rotate(iqB, sub(pA, pB));
    double er = r + ms;
    Box3 q{{c.x - er, c.y - er, c.z - er}, {c.x + er, c.y + er, c.z + er}};
    mesh_walk(M, q, c, [&](int t) {
        const auto &tr = M.tris[t];
        V3 sv0 = M.verts[tr[0]], sv1 = M.verts[tr[1]], sv2 = M.verts[tr[2]];
        V3 v0 = sub(sv0, c), v1 = sub(sv1, c), v2 = sub(sv2, c);
        V3 tn = cross(sub(v1, v0), sub(v2, v0));
        bool back = dot(tn, v0) > 0;
        if (back && !cs.collideWithBackfaces) return;
        double dsq;
        int feature;
        V3 p2 = closest_point_on_triangle(v0, v1, v2, dsq, feature);
        if (dsq > maxSq) return;
        double pen = r - std::sqrt(dsq);
        V3 axis = dsq > 0 ? normalize(p2) : V3{0, 1, 0};
        V3 p1 = scale(axis, r);
        if (feature != 0b111 && tr[3] != 0b111 && (tr[3] & FEATURE_TO_ACTIVE_EDGES[feature]) == 0) {
            V3 mv = rotate(iqB, movement);
            V3 nax = back ? tn : neg(tn);
            if (dot(mv, axis) * len(nax) >= dot(mv, nax)) axis = nax;
        }
        Hit h;
        h.pa = add(rotate(qB, add(c, p1)), pB);
        h.pb = add(rotate(qB, add(c, p2)), pB);
        h.axis = rotate(qB, axis);
        h.penetration = pen;
        h.subA = EMPTY_SUB_SHAPE_ID;
        h.subB = mesh_sub_shape_id(M, t);
        h.faceA.n = 0;
        h.faceB.n = 3;
        h.faceB.v[0] = add(rotate(qB, sv0), pB);
        h.faceB.v[1] = add(rotate(qB, sv1), pB);
        h.faceB.v[2] = add(rotate(qB, sv2), pB);
        out.push_back(h);
    });
}

// rayDistanceToBox3 cast-utils.ts:14-49: the entry fraction of the segment origin + t * dir
// (t in [0, length]) into the box, +inf on a miss
inline double ray_fraction_to_box(V3 o, V3 d, double length, const Box3 &b) {
    double t0 = 0, t1 = length;
    const double oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
    const double mn[3] = {b.mn.x, b.mn.y, b.mn.z}, mx[3] = {b.mx.x, b.mx.y, b.mx.z};
    for (int i = 0; i < 3; i++) {
        if (std::fabs(dd[i]) < 1e-10) {
            if (oo[i] < mn[i] || oo[i] > mx[i]) return std::numeric_limits<double>::infinity();
        } else {
            double inv = 1.0 / dd[i];
            double a = (mn[i] - oo[i]) * inv, c = (mx[i] - oo[i]) * inv;
            t0 = std::max(t0, std::min(a, c));
            t1 = std::min(t1, std::max(a, c));
            if (t1 < t0) return std::numeric_limits<double>::infinity();
        }
    }
    return t0 >= 0 ? t0 / length : std::numeric_limits<double>::infinity();
}

// A shape cast hit handed to a cast collector: fraction, world points, the unnormalised
// penetration axis.  The collector returns nothing; earlyOut() is its current early-out fraction.
struct CastMeshHit {
    double fraction;
    V3 pa, pb, axis;
    uint32_t sub = EMPTY_SUB_SHAPE_ID;  // the triangle's sub-shape id
};

// castConvexVsTriangleMesh triangle-mesh.ts:638-1019 with the default cast settings the
// continuous-collision visitor uses (tolerances 0.01, SupportFunctionMode.DEFAULT, no deepest
// point, back faces culled, no movement direction)
template <class Add, class EarlyOut>
inline void cast_convex_vs_mesh(const Shape &sa, V3 pA, Q4 qA, V3 disp, const Shape &sb, V3 pB, Q4 qB, Add &&onHit,
                                EarlyOut &&earlyOut) {
    const MeshData &M = *sb.mesh;
    if (M.nodes.empty()) return;
    Q4 iqB = qconj(qB);
    V3 posAInB = rotate(iqB, sub(pA, pB));
    Q4 qAInB = qmul(iqB, qA);
    V3 dInB = rotate(iqB, disp);
    Box3 base{{1e300, 1e300, 1e300}, {-1e300, -1e300, -1e300}};
    for (int c = 0; c < 8; c++) {
        const Box3 &lb = sa.decorated ? sa.leafAabb : sa.aabb;
        V3 p{(c & 1) ? lb.mx.x : lb.mn.x, (c & 2) ? lb.mx.y : lb.mn.y, (c & 4) ? lb.mx.z : lb.mn.z};
        V3 q = add(rotate(qAInB, p), posAInB);
        base.mn = {std::min(base.mn.x, q.x), std::min(base.mn.y, q.y), std::min(base.mn.z, q.z)};
        base.mx = {std::max(base.mx.x, q.x), std::max(base.mx.y, q.y), std::max(base.mx.z, q.z)};
    }
    // SupportFunctionMode.DEFAULT: a box keeps its full extent (box.ts / support.ts:364), the
    // other shapes their core with the convex radius (sphere.ts:258, capsule.ts:396, convex-hull.ts:978)
    Support supA = make_support(sa, sa.type == SHAPE_BOX ? INCLUDE_CONVEX_RADIUS : EXCLUDE_CONVEX_RADIUS);
    V3 origin = scale(add(base.mn, base.mx), 0.5);
    double rlen = len(dInB);
    V3 rdir = rlen > 1e-10 ? normalize(dInB) : V3{0, 0, 0};
    V3 half = scale(sub(base.mx, base.mn), 0.5);
    std::vector<std::pair<int, double>> stack{{0, 0.0}};
    while (!stack.empty()) {
        auto [node, dist] = stack.back();
        stack.pop_back();
        if (dist >= earlyOut()) continue;
        const auto &nd = M.nodes[node];
        if (nd[7] < 0) {
            int start = (int)nd[6], count = (int)(-nd[7]) - 1;
            for (int t = start; t < start + count; t++) {
                const auto &tr = M.tris[t];
                V3 a = M.verts[tr[0]], b = M.verts[tr[1]], c = M.verts[tr[2]];
                Box3 tb{{std::min(a.x, std::min(b.x, c.x)) - half.x, std::min(a.y, std::min(b.y, c.y)) - half.y,
                         std::min(a.z, std::min(b.z, c.z)) - half.z},
                        {std::max(a.x, std::max(b.x, c.x)) + half.x, std::max(a.y, std::max(b.y, c.y)) + half.y,
                         std::max(a.z, std::max(b.z, c.z)) + half.z}};
                if (!(ray_fraction_to_box(origin, rdir, rlen, tb) < std::numeric_limits<double>::infinity())) continue;
                if (earlyOut() <= 0) return;
                V3 n = cross(sub(b, a), sub(c, a));
                if (dot(n, dInB) > 0) continue;  // back face
                Support tri;
                tri.kind = SUP_TRIANGLE;
                tri.ta = a;
                tri.tb = b;
                tri.tc = c;
                Support A = supA;
                A.transformed = true;
                A.m = mat4_from_rt(qAInB, posAInB);
                double lambda;
                V3 pa, pb, ax;
                const double tol = 0.01;
                if (!gjk_cast_shape(lambda, pa, pb, ax, A, tri, dInB, tol, supA.convex_radius, 0.0, earlyOut()))
                    continue;
                if (lensq(ax) < tol * tol) ax = dInB;  // penetration.ts:693-698
                double depth = len(sub(pa, pb));
                if (lambda == 0 && -depth >= earlyOut()) continue;
                if (tr[3] != 0b111)  // fixNormal with the triangle normal as given (back faces culled)
                    ax = fix_normal(a, b, c, n, tr[3], pb, ax, V3{0, 0, 0});
                onHit(CastMeshHit{lambda, add(rotate(qB, pa), pB), add(rotate(qB, pb), pB), rotate(qB, ax),
                                  mesh_sub_shape_id(M, t)});
            }
            continue;
        }
        int left = node + 1, right = (int)nd[6];
        auto grown = [&](int k) {
            const auto &c = M.nodes[k];
            return Box3{{c[0] - half.x, c[1] - half.y, c[2] - half.z}, {c[3] + half.x, c[4] + half.y, c[5] + half.z}};
        };
        double ld = ray_fraction_to_box(origin, rdir, rlen, grown(left));
        double rd = ray_fraction_to_box(origin, rdir, rlen, grown(right));
        if (ld <= rd) {
            if (rd < earlyOut()) stack.push_back({right, rd});
            if (ld < earlyOut()) stack.push_back({left, ld});
        } else {
            if (ld < earlyOut()) stack.push_back({left, ld});
            if (rd < earlyOut()) stack.push_back({right, rd});
        }
    }
}

// rayCylinder / raySphereFromOrigin sphere-triangle.ts:17-83, 156-195
inline double ray_cylinder(V3 dir, V3 ca, V3 cb, double r) {
    V3 axis = sub(cb, ca), start = neg(ca);
    double sda = dot(start, axis), dda = dot(dir, axis), eda = sda + dda;
    if (sda < 0 && eda < 0) return std::numeric_limits<double>::infinity();
    double al2 = lensq(axis);
    if (sda > al2 && eda > al2) return std::numeric_limits<double>::infinity();
    double a = al2 * lensq(dir) - dda * dda;
    if (std::fabs(a) < 1e-6) return std::numeric_limits<double>::infinity();
    double b = al2 * dot(start, dir) - dda * sda;
    double c = al2 * (lensq(start) - r * r) - sda * sda;
    double det = b * b - a * c;
    if (det < 0) return std::numeric_limits<double>::infinity();
    double t = -(b + std::sqrt(det)) / a;
    if (t < 0 || t > 1) return std::numeric_limits<double>::infinity();
    double hda = sda + t * dda;
    if (hda < 0 || hda > al2) return std::numeric_limits<double>::infinity();
    return t;
}
inline double ray_sphere_from_origin(V3 dir, V3 c, double r) {
    double a = lensq(dir), b = -2 * dot(dir, c), cc = lensq(c) - r * r;
    double disc = b * b - 4 * a * cc;
    if (disc < 0) return cc <= 0 ? 0 : std::numeric_limits<double>::infinity();
    if (a < 1e-10) return cc <= 0 ? 0 : std::numeric_limits<double>::infinity();
    double sq = std::sqrt(disc);
    double t1 = (-b - sq) / (2 * a), t2 = (-b + sq) / (2 * a);
    if (t1 > t2) std::swap(t1, t2);
    if (t1 >= 0 && t1 <= 1) return t1;
    if (t2 >= 0 && t2 <= 1) return 0;
    if (t1 < 0 && t2 > 1) return 0;
    return std::numeric_limits<double>::infinity();
}

// castSphereVsTriangleMesh triangle-mesh.ts:1870-2236 with castSphereVsTriangleMeshAddHit
// :1781-1868 (default cast settings, no movement direction).  The hit's penetration axis is the
// negated contact normal (:1847-1848).
template <class Add, class EarlyOut>
inline void cast_sphere_vs_mesh(const Shape &sa, V3 pA, V3 disp, const Shape &sb, V3 pB, Q4 qB, Add &&onHit,
                                EarlyOut &&earlyOut) {
    const MeshData &M = *sb.mesh;
    if (M.nodes.empty()) return;
    const double r = sa.radius;
    Q4 iqB = qconj(qB);
    V3 start = rotate(iqB, sub(pA, pB)), dir = rotate(iqB, disp);
    V3 end = add(start, dir);
    Box3 sw{{std::min(start.x, end.x) - r, std::min(start.y, end.y) - r, std::min(start.z, end.z) - r},
            {std::max(start.x, end.x) + r, std::max(start.y, end.y) + r, std::max(start.z, end.z) + r}};
    V3 qc = scale(add(sw.mn, sw.mx), 0.5);
    uint32_t cur_sub = EMPTY_SUB_SHAPE_ID;
    auto emit = [&](bool back, V3 tn, int active, double fraction, V3 ca, V3 cbp, V3 cn) {
        V3 fn = cn;
        if (active != 0b111) {  // movement direction zero: the normal kept unless the check below flips it
            V3 tnf = back ? tn : neg(tn);
            V3 mv{0, 0, 0};
            if (dot(mv, cn) * len(tnf) < dot(mv, tnf) * len(cn)) fn = tnf;
        }
        V3 pa = add(rotate(qB, add(start, ca)), pB), pb = add(rotate(qB, add(start, cbp)), pB);
        V3 nw = normalize(rotate(qB, fn));
        onHit(CastMeshHit{fraction, pa, pb, neg(nw), cur_sub});
    };
    mesh_walk(M, sw, qc, [&](int t) {
        cur_sub = mesh_sub_shape_id(M, t);
        const auto &tr = M.tris[t];
        V3 rv0 = sub(M.verts[tr[0]], start), rv1 = sub(M.verts[tr[1]], start), rv2 = sub(M.verts[tr[2]], start);
        V3 tn = cross(sub(rv1, rv0), sub(rv2, rv0));
        double tl = len(tn);
        if (tl == 0) return;
        tn = scale(tn, 1.0 / tl);
        double ndd = dot(tn, dir);
        bool back = ndd > 0;
        if (back) return;
        int active = tr[3];
        // already touching at the start
        if (std::fabs(dot(rv0, tn)) <= r) {
            double dsq;
            int feature;
            V3 q = closest_point_on_triangle(rv0, rv1, rv2, dsq, feature);
            if (dsq <= r * r) {
                double ql = std::sqrt(dsq);
                double pen = r - ql;
                if (-pen >= earlyOut()) return;
                V3 cn = ql > 0 ? scale(q, 1 / ql) : V3{0, 1, 0};
                emit(back, tn, active, 0.0, scale_add(q, cn, pen), q, cn);
                return;
            }
        }
        // the plane
        double andd = std::fabs(ndd);
        if (andd > 1e-6) {
            V3 d = scale(tn, (ndd > 0 ? 1.0 : (ndd < 0 ? -1.0 : 0.0)) * r);
            double pi = dot(sub(rv0, d), tn) / ndd;
            if (pi * andd >= -r && pi < earlyOut() && pi >= 0) {
                V3 p = scale_add(d, dir, pi);
                V3 v0r = sub(rv0, p), v1r = sub(rv1, p), v2r = sub(rv2, p);
                V3 nn = cross(v1r, v2r);
                double nl = len(nn);
                if (nl > 0) {
                    double area = dot(nn, tn) / nl;
                    if (area > 0) {
                        double u = dot(cross(v1r, v2r), tn) / (area * nl), v = dot(cross(v2r, v0r), tn) / (area * nl),
                               w = dot(cross(v0r, v1r), tn) / (area * nl);
                        if (u >= 0 && v >= 0 && w >= 0) {
                            emit(back, tn, 0b111, pi, p, p, back ? tn : neg(tn));
                            return;
                        }
                    }
                }
            }
        }
        // edges and vertices
        double f = std::numeric_limits<double>::infinity();
        f = std::min(f, ray_cylinder(dir, rv0, rv1, r));
        f = std::min(f, ray_cylinder(dir, rv1, rv2, r));
        f = std::min(f, ray_cylinder(dir, rv2, rv0, r));
        f = std::min(f, ray_sphere_from_origin(dir, rv0, r));
        f = std::min(f, ray_sphere_from_origin(dir, rv1, r));
        f = std::min(f, ray_sphere_from_origin(dir, rv2, r));
        if (f >= 0 && f < earlyOut()) {
            V3 p = scale(dir, f);
            double dsq;
            int feature;
            V3 q = closest_point_on_triangle(sub(rv0, p), sub(rv1, p), sub(rv2, p), dsq, feature);
            V3 cn = normalize(q);
            V3 cp = add(p, q);
            emit(back, tn, active, f, cp, cp, cn);
        }
    });
}

// ----------------------------------------------------------------------------
// Ray casts (query.ts:78-90, convex.ts:54-126, gjk.ts:622-790, triangle-mesh.ts castRay)
// ----------------------------------------------------------------------------
// gjkCastRay gjk.ts:622-790: the ray origin + lambda * dir against a support in its own frame;
// false when the ray misses before maxLambda
inline bool gjk_cast_ray(double &lambdaOut, V3 origin, V3 dir, double tol, const Support &S, double maxLambda) {
    const double sqtol = tol * tol;
    Simplex sx;
    double lambda = 0.0;
    V3 x = origin;
    V3 p = S.get({0, 0, 0});
    V3 v = sub(x, p);
    double vls = std::numeric_limits<double>::max();
    bool allowRestart = false;
    for (int it = 0; it < GJK_MAX_ITERATIONS; it++) {
        p = S.get(v);
        V3 w = sub(x, p);
        double vdw = dot(v, w);
        if (vdw > 0.0) {
            double vdr = dot(v, dir);
            if (vdr >= -1.0e-18) return false;
            double old = lambda;
            lambda -= vdw / vdr;
            if (old == lambda) break;
            if (lambda >= maxLambda) return false;
            x = scale_add(origin, dir, lambda);
            vls = std::numeric_limits<double>::max();
            allowRestart = true;
        }
        sx.pts[sx.size].p = p;
        sx.size++;
        for (int i = 0; i < sx.size; i++) sx.pts[i].y = sub(x, sx.pts[i].p);
        ClosestToSimplex c;
        if (closest_to_simplex(c, vls, false, sx)) {
            vls = c.sqdist;
            v = c.point;
        } else {
            if (!allowRestart) break;
            allowRestart = false;
            sx.pts[0].p = p;
            sx.size = 1;
            v = sub(x, p);
            vls = std::numeric_limits<double>::max();
            continue;
        }
        if (c.set == 0xf) break;
        int ns = 0;
        for (int i = 0; i < sx.size; i++)
            if (c.set & (1 << i)) {
                if (ns != i) sx.pts[ns].p = sx.pts[i].p;
                ns++;
            }
        sx.size = ns;
        if (vls <= sqtol) break;
    }
    lambdaOut = lambda;
    return true;
}

// raycast3.intersectsTriangle of mathcat 0.0.10 (not vendored), taken as the Moller-Trumbore
// test over t in [0, length] along the ray's direction, back faces culled when asked; the hit's
// fraction is t / length
inline bool ray_triangle(V3 o, V3 d, double length, V3 a, V3 b, V3 c, bool cullBack, double &fraction) {
    const double EPS = 1e-10;
    V3 e1 = sub(b, a), e2 = sub(c, a);
    V3 pv = cross(d, e2);
    double det = dot(e1, pv);
    if (cullBack ? det < EPS : std::fabs(det) < EPS) return false;
    double inv = 1.0 / det;
    V3 tv = sub(o, a);
    double u = dot(tv, pv) * inv;
    if (u < 0 || u > 1) return false;
    V3 qv = cross(tv, e1);
    double v = dot(d, qv) * inv;
    if (v < 0 || u + v > 1) return false;
    double t = dot(e2, qv) * inv;
    if (t < 0 || t > length) return false;
    fraction = t / length;
    return true;
}

// castRayVsShape for one body (castRayVsConvex convex.ts:54-126, castRayVsTriangleMesh
// triangle-mesh.ts): the closest hit below maxFraction, its sub-shape id
inline bool cast_ray_vs_shape(const Shape &s, V3 pos, Q4 q, V3 origin, V3 dir, double length, bool solid,
                              double maxFraction, double &fraction, uint32_t &subId) {
    if (s.type == SHAPE_COMPOUND) {  // castRayVsCompound compound.ts:350-421: each child, the closest
        const CompoundData &C = *s.compound;
        double best = maxFraction;
        bool found = false;
        for (int i = 0; i < (int)C.shapes.size(); i++) {
            if (best <= 0) break;
            V3 cp;
            Q4 cq;
            compound_child_pose(C, i, pos, q, cp, cq);
            double f;
            uint32_t sub;
            if (cast_ray_vs_shape(C.shapes[i], cp, cq, origin, dir, length, solid, best, f, sub) && f < best) {
                best = f;
                found = true;
                subId = compound_sub_id(C, i);
            }
        }
        if (found) fraction = best;
        return found;
    }
    Q4 iq = qconj(q);
    V3 lo = rotate(iq, sub(origin, pos)), ld = rotate(iq, dir);
    if (s.type == SHAPE_TRIANGLE_MESH) {
        const MeshData &M = *s.mesh;
        if (M.nodes.empty()) return false;
        bool found = false;
        double best = maxFraction;
        std::vector<std::pair<int, double>> stack{{0, -std::numeric_limits<double>::infinity()}};
        while (!stack.empty()) {
            if (best <= 0) break;
            auto [node, dist] = stack.back();
            stack.pop_back();
            if (dist >= best) continue;
            const auto &nd = M.nodes[node];
            if (nd[7] < 0) {
                int start = (int)nd[6], count = (int)(-nd[7]) - 1;
                for (int t = start; t < start + count; t++) {
                    const auto &tr = M.tris[t];
                    double f;
                    if (ray_triangle(lo, ld, length, M.verts[tr[0]], M.verts[tr[1]], M.verts[tr[2]], true, f) &&
                        f < best) {
                        best = f;
                        found = true;
                        subId = mesh_sub_shape_id(M, t);
                    }
                }
                continue;
            }
            int left = node + 1, right = (int)nd[6];
            auto box = [&](int k) {
                const auto &c = M.nodes[k];
                return Box3{{c[0], c[1], c[2]}, {c[3], c[4], c[5]}};
            };
            double ldist = ray_fraction_to_box(lo, ld, length, box(left)), rdist = ray_fraction_to_box(lo, ld, length, box(right));
            if (ldist <= rdist) {
                if (rdist < best) stack.push_back({right, rdist});
                if (ldist < best) stack.push_back({left, ldist});
            } else {
                if (ldist < best) stack.push_back({left, ldist});
                if (rdist < best) stack.push_back({right, rdist});
            }
        }
        if (found) fraction = best;
        return found;
    }
    if (s.type == SHAPE_EMPTY) return false;
    if (s.type == SHAPE_PLANE) {
        subId = EMPTY_SUB_SHAPE_ID;
        return cast_ray_vs_plane(s, pos, q, origin, dir, length, solid, false, maxFraction, fraction);
    }
    Support S = make_support(s, INCLUDE_CONVEX_RADIUS);
    double lambda;
    if (!gjk_cast_ray(lambda, lo, scale(ld, length), 1e-3, S, maxFraction)) return false;
    if (!(solid || lambda > 0.0)) return false;
    fraction = std::max(0.0, lambda);
    subId = EMPTY_SUB_SHAPE_ID;
    return true;
}

// castRayVsTriangleMesh triangle-mesh.ts:259-432 with the AllCastRayCollector (cast-ray-vs-shape.ts
// :66-94): its early-out fraction stays INITIAL_EARLY_OUT_FRACTION, so every triangle hit below it
// is added, in walk order, as (fraction, sub-shape id); back faces culled
inline void mesh_ray_all_hits(const MeshData &M, V3 o, V3 d, double length,
                              std::vector<std::pair<double, uint32_t>> &hits) {
    const double early = 1.0 + 1e-4;
    if (M.nodes.empty()) return;
    std::vector<std::pair<int, double>> stack{{0, -std::numeric_limits<double>::infinity()}};
    while (!stack.empty()) {
        auto [node, dist] = stack.back();
        stack.pop_back();
        if (dist >= early) continue;
        const auto &nd = M.nodes[node];
        if (nd[7] < 0) {
            int start = (int)nd[6], count = (int)(-nd[7]) - 1;
            for (int t = start; t < start + count; t++) {
                const auto &tr = M.tris[t];
                double f;
                if (ray_triangle(o, d, length, M.verts[tr[0]], M.verts[tr[1]], M.verts[tr[2]], true, f) && f < early)
                    hits.push_back({f, mesh_sub_shape_id(M, t)});
            }
            continue;
        }
        int left = node + 1, right = (int)nd[6];
        auto box = [&](int k) {
            const auto &c = M.nodes[k];
            return Box3{{c[0], c[1], c[2]}, {c[3], c[4], c[5]}};
        };
        double ldist = ray_fraction_to_box(o, d, length, box(left)), rdist = ray_fraction_to_box(o, d, length, box(right));
        if (rdist < early) stack.push_back({right, rdist});
        if (ldist < early) stack.push_back({left, ldist});
    }
}

// the hit count of a ray through a mesh with every hit kept (hitCountCollector
// triangle-mesh.ts:441-467: its early-out fraction stays INITIAL_EARLY_OUT_FRACTION, so every
// node the ray enters is walked) and the sub-shape id of the last hit in walk order
inline int mesh_ray_hit_count(const MeshData &M, V3 o, V3 d, double length, uint32_t &lastSub) {
    const double early = 1.0 + 1e-4;
    int count = 0;
    if (M.nodes.empty()) return 0;
    std::vector<std::pair<int, double>> stack{{0, -std::numeric_limits<double>::infinity()}};
    while (!stack.empty()) {
        auto [node, dist] = stack.back();
        stack.pop_back();
        if (dist >= early) continue;
        const auto &nd = M.nodes[node];
        if (nd[7] < 0) {
            int start = (int)nd[6], n = (int)(-nd[7]) - 1;
            for (int t = start; t < start + n; t++) {
                const auto &tr = M.tris[t];
                double f;
                if (ray_triangle(o, d, length, M.verts[tr[0]], M.verts[tr[1]], M.verts[tr[2]], false, f) && f < early) {
                    count++;
                    lastSub = mesh_sub_shape_id(M, t);
                }
            }
            continue;
        }
        int left = node + 1, right = (int)nd[6];
        auto box = [&](int k) {
            const auto &c = M.nodes[k];
            return Box3{{c[0], c[1], c[2]}, {c[3], c[4], c[5]}};
        };
        double ldist = ray_fraction_to_box(o, d, length, box(left)), rdist = ray_fraction_to_box(o, d, length, box(right));
        if (ldist <= rdist) {
            if (rdist < early) stack.push_back({right, rdist});
            if (ldist < early) stack.push_back({left, ldist});
        } else {
            if (ldist < early) stack.push_back({left, ldist});
            if (rdist < early) stack.push_back({right, rdist});
        }
    }
    return count;
}

inline bool box_contains(const Box3 &b, V3 p) {  // box3.containsPoint
    return p.x >= b.mn.x && p.x <= b.mx.x && p.y >= b.mn.y && p.y <= b.mx.y && p.z >= b.mn.z && p.z <= b.mx.z;
}

// collidePointVsShape for one body: collidePointVsSphere sphere.ts:272-301, collidePointVsBox
// box.ts:370-410, collidePointVsConvex convex.ts:142-216 (GJK of the INCLUDE_CONVEX_RADIUS support
// against the point, collisionTolerance 1e-4 by default), collidePointVsTriangleMesh
// triangle-mesh.ts:482-570 (odd-even count of a +Y ray 1.1 x the mesh height long, back faces
// counted).  True when the point is inside; subId is the mesh's last-hit triangle.
inline bool point_in_shape(const Shape &s, V3 pos, Q4 q, V3 point, double tol, uint32_t &subId) {
    subId = EMPTY_SUB_SHAPE_ID;
    if (s.type == SHAPE_EMPTY) return false;
    if (s.type == SHAPE_COMPOUND) {  // collidePointVsCompound compound.ts:423-492: the first child
        const CompoundData &C = *s.compound;
        for (int i = 0; i < (int)C.shapes.size(); i++) {
            V3 cp;
            Q4 cq;
            compound_child_pose(C, i, pos, q, cp, cq);
            uint32_t sub;
            if (point_in_shape(C.shapes[i], cp, cq, point, tol, sub)) {
                subId = compound_sub_id(C, i);
                return true;
            }
        }
        return false;
    }
    if (s.type == SHAPE_PLANE) return point_in_plane(s, pos, q, point);
    V3 l = sub(point, pos);
    if (s.type == SHAPE_SPHERE) return dot(l, l) <= s.radius * s.radius;
    V3 lp = rotate(qconj(q), l);
    if (s.type == SHAPE_BOX)
        return std::fabs(lp.x) <= s.half_extents.x && std::fabs(lp.y) <= s.half_extents.y &&
               std::fabs(lp.z) <= s.half_extents.z;
    const Box3 &la = s.decorated ? s.leafAabb : s.aabb;
    if (!box_contains(la, lp)) return false;
    if (s.type == SHAPE_TRIANGLE_MESH) {
        double h = la.mx.y - la.mn.y;
        uint32_t last = EMPTY_SUB_SHAPE_ID;
        int n = mesh_ray_hit_count(*s.mesh, lp, {0, 1, 0}, h * 1.1, last);
        if ((n & 1) == 0) return false;
        subId = last;
        return true;
    }
    Support S = make_support(s, INCLUDE_CONVEX_RADIUS);
    Support P;
    P.kind = SUP_SPHERE_POINT;
    P.transformed = true;
    P.m = mat4_from_rt({0, 0, 0, 1}, lp);
    V3 dir = lp;
    if (dot(dir, dir) < 1e-10) dir = {0, 1, 0};
    GjkResult g = gjk_closest_points(S, P, tol, dir, 0.0);
    return g.sqdist <= tol * tol;
}

// the hits of a body pair in narrowphase order (collideShapeVsShape narrowphase.ts:172-238 with
// the mesh registrations triangle-mesh.ts:223-237: a mesh as shape A runs the convex-vs-mesh
// function reversed, collide-shape-vs-shape.ts:227-354)
inline void collide_hits(std::vector<Hit> &out, const CollideSettings &cs, const Shape &sa, V3 pA, Q4 qA,
                         const Shape &sb, V3 pB, Q4 qB, V3 movement);

// collideShapeVsShape narrowphase.ts:172-238 (dispatch for the supported convex shapes)
inline bool collide_shapes(Hit &hit, const CollideSettings &cs, const Shape &sa, V3 pA, Q4 qA, const Shape &sb,
                           V3 pB, Q4 qB) {
    if (sa.type == SHAPE_EMPTY || sb.type == SHAPE_EMPTY) return false;
    if (sa.type == SHAPE_PLANE && sb.type == SHAPE_PLANE) return false;
    if (sb.type == SHAPE_PLANE) return collide_convex_vs_plane(hit, cs, sa, pA, qA, sb, pB, qB);
    if (sa.type == SHAPE_PLANE) {  // reversedCollideShapeVsShape collide-shape-vs-shape.ts:227-354
        if (!collide_convex_vs_plane(hit, cs, sb, pB, qB, sa, pA, qA)) return false;
        std::swap(hit.pa, hit.pb);
        hit.axis = neg(hit.axis);
        std::swap(hit.faceA, hit.faceB);
        return true;
    }
    if (sa.type == SHAPE_SPHERE && sb.type == SHAPE_SPHERE) return collide_sphere_vs_sphere(hit, sa, pA, sb, pB);
    return collide_convex_vs_convex(hit, cs, sa, pA, qA, sb, pB, qB);
}

inline void collide_hits(std::vector<Hit> &out, const CollideSettings &cs, const Shape &sa, V3 pA, Q4 qA,
                         const Shape &sb, V3 pB, Q4 qB, V3 movement) {
    if (sa.type == SHAPE_COMPOUND || sb.type == SHAPE_COMPOUND) {
        // collideCompoundVsShape / collideShapeVsCompound compound.ts:494-678: each child in turn
        // (A's first when both are compounds), its sub-shape id pushed onto the hits
        const bool onA = sa.type == SHAPE_COMPOUND;
        const CompoundData &C = *(onA ? sa : sb).compound;
        for (int i = 0; i < (int)C.shapes.size(); i++) {
            V3 cp;
            Q4 cq;
            compound_child_pose(C, i, onA ? pA : pB, onA ? qA : qB, cp, cq);
            const size_t first = out.size();
            if (onA)
                collide_hits(out, cs, C.shapes[i], cp, cq, sb, pB, qB, movement);
            else
                collide_hits(out, cs, sa, pA, qA, C.shapes[i], cp, cq, movement);
            const uint32_t id = compound_sub_id(C, i);
            for (size_t k = first; k < out.size(); k++) (onA ? out[k].subA : out[k].subB) = id;
        }
        return;
    }
    const bool ma = sa.type == SHAPE_TRIANGLE_MESH, mb = sb.type == SHAPE_TRIANGLE_MESH;
    if (ma && mb) return;
    if (sa.type == SHAPE_EMPTY || sb.type == SHAPE_EMPTY) return;  // empty-shape.ts: registers nothing
    // a plane collides with convex shapes only (plane.ts register :297-308)
    if ((ma && sb.type == SHAPE_PLANE) || (mb && sa.type == SHAPE_PLANE)) return;
    if (mb) {
        if (sa.type == SHAPE_SPHERE)
            collide_sphere_vs_mesh(out, cs, sa, pA, sb, pB, qB, movement);
        else
            collide_convex_vs_mesh(out, cs, sa, pA, qA, sb, pB, qB, movement);
        return;
    }
    if (ma) {
        size_t first = out.size();
        if (sb.type == SHAPE_SPHERE)
            collide_sphere_vs_mesh(out, cs, sb, pB, sa, pA, qA, movement);
        else
            collide_convex_vs_mesh(out, cs, sb, pB, qB, sa, pA, qA, movement);
        for (size_t i = first; i < out.size(); i++) {  // createInvertedCollector collide-shape-vs-shape.ts:227-270
            Hit &h = out[i];
            std::swap(h.pa, h.pb);
            h.axis = neg(h.axis);
            std::swap(h.subA, h.subB);
            std::swap(h.faceA, h.faceB);
        }
        return;
    }
    Hit h;
    if (collide_shapes(h, cs, sa, pA, qA, sb, pB, qB)) out.push_back(h);
}

}  // namespace orc
