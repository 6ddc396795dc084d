// Narrowphase: convex GJK / EPA, supporting faces, polygon clipping and
// contact point reduction, one body pair per thread.
//
// Reference: narrowphase (src/update.ts:714-850), collideConvexVsConvex and
// collideConvexVsConvexLocal (src/shapes/convex.ts:257-641),
// gjkClosestPoints (src/collision/gjk.ts:1294-1546), penetrationDepthStepGJK /
// penetrationDepthStepEPA (src/collision/penetration.ts:35-614), the EPA hull
// (src/collision/epa-convex-hull-builder.ts), box supporting faces
// (src/shapes/box.ts:129-332), manifoldBetweenTwoFaces / pruneContactPoints
// (src/manifold/manifold.ts:192-444), clipPolyVsPoly (src/manifold/clip.ts),
// collideSphereVsSphere (src/shapes/sphere.ts:319-410).
//
// GJK, faces and clipping run in FP32 with contact points kept relative to
// body A's position.  Pairs whose shrunk shapes overlap (GJK INDETERMINATE) are
// queued for a second kernel that runs EPA in FP64 with its polytope in a
// per-thread slice of global scratch memory.
#include <mutex>

#include <math_constants.h>

#include "cc_internal.cuh"

namespace cc {

static __constant__ DevSettings c_settings;

void upload_settings_narrowphase(const DevSettings &s, cudaStream_t st) {
    cudaMemcpyToSymbolAsync(c_settings, &s, sizeof(DevSettings), 0, cudaMemcpyHostToDevice, st);
}

template <typename S>
struct V {
    S x, y, z;
};
template <typename S>
__device__ __forceinline__ V<S> mk(S x, S y, S z) {
    return V<S>{x, y, z};
}
template <typename S>
__device__ __forceinline__ V<S> operator+(V<S> a, V<S> b) {
    return {a.x + b.x, a.y + b.y, a.z + b.z};
}
template <typename S>
__device__ __forceinline__ V<S> operator-(V<S> a, V<S> b) {
    return {a.x - b.x, a.y - b.y, a.z - b.z};
}
template <typename S>
__device__ __forceinline__ V<S> operator-(V<S> a) {
    return {-a.x, -a.y, -a.z};
}
template <typename S>
__device__ __forceinline__ V<S> operator*(V<S> a, S s) {
    return {a.x * s, a.y * s, a.z * s};
}
template <typename S>
__device__ __forceinline__ S dot(V<S> a, V<S> b) {
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename S>
__device__ __forceinline__ S lsq(V<S> a) {
    return a.x * a.x + a.y * a.y + a.z * a.z;
}
template <typename S>
__device__ __forceinline__ V<S> crs(V<S> a, V<S> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename S>
__device__ __forceinline__ S sq_root(S v);
template <>
__device__ __forceinline__ float sq_root<float>(float v) {
    return sqrtf(v);
}
template <>
__device__ __forceinline__ double sq_root<double>(double v) {
    return sqrt(v);
}
template <typename S>
__device__ __forceinline__ S s_abs(S v) {
    return v < S(0) ? -v : v;
}
template <typename S>
__device__ __forceinline__ S s_max_value();
template <>
__device__ __forceinline__ float s_max_value<float>() {
    return 3.402823466e38f;
}
template <>
__device__ __forceinline__ double s_max_value<double>() {
    return 1.7976931348623157e308;
}

// quaternion (x y z w) helpers in precision S
template <typename S>
struct Q {
    S x, y, z, w;
};
template <typename S>
__device__ __forceinline__ V<S> qrotS(Q<S> q, V<S> v) {
    V<S> u{q.x, q.y, q.z};
    V<S> t = crs(u, v) * S(2);
    return v + t * q.w + crs(u, t);
}
template <typename S>
__device__ __forceinline__ Q<S> qmulS(Q<S> a, Q<S> b) {
    return {a.x * b.w + a.w * b.x + a.y * b.z - a.z * b.y, a.y * b.w + a.w * b.y + a.z * b.x - a.x * b.z,
            a.z * b.w + a.w * b.z + a.x * b.y - a.y * b.x, a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z};
}

// ---------------------------------------------------------------------------
// support functions
// ---------------------------------------------------------------------------
enum { SUP_BOX = 0, SUP_POINT = 1, SUP_SPHERE = 2, SUP_CAPSULE_SEGMENT = 3, SUP_CAPSULE_SURFACE = 4, SUP_HULL = 5,
       SUP_TRIANGLE = 6, SUP_CYLINDER = 7 };
// the world's convex hull arrays, as the support functions read them
struct HullView {
    const DevHull *hulls;
    const float4 *points, *shrunk;
};
__device__ __forceinline__ HullView hull_view(const DevWorld &w) { return HullView{w.hulls, w.hull_points, w.hull_shrunk}; }
// H: the support may be a convex hull (the contact-only narrowphase instance compiles it out);
// T: it may be a mesh triangle (only the mesh passes compile it in)
template <typename S, bool H = true, bool T = false>
struct Sup {
    int kind;
    const float4 *hp;  // hull support points (original or shrunk) and their count
    int hn;
    V<S> he;      // box half extents
    S radius;     // sphere surface radius
    S convex_radius;
    bool transformed;
    V<S> r0, r1, r2, t;  // rows of the rotation and translation (B in A's frame)
    S add_r;
    __device__ V<S> inner(V<S> d) const {
        if (kind == SUP_BOX) return {d.x >= S(0) ? he.x : -he.x, d.y >= S(0) ? he.y : -he.y, d.z >= S(0) ? he.z : -he.z};
        if (H && kind == SUP_HULL) {  // the point with the highest projection (convex-hull.ts:588-614, 695-715)
            S best = -s_max_value<S>();
            V<S> bp{S(0), S(0), S(0)};
            bool any = false;
            for (int k = 0; k < hn; k++) {
                float4 p = hp[k];
                S dd = S(p.x) * d.x + S(p.y) * d.y + S(p.z) * d.z;
                if (!any || dd > best) {
                    best = dd;
                    bp = {S(p.x), S(p.y), S(p.z)};
                    any = true;
                }
            }
            return bp;
        }
        if (T && kind == SUP_TRIANGLE) {
            // triangleGetSupport support.ts:83-118: the vertex with the largest projection (an
            // untransformed triangle keeps its vertices in r0, r1, r2)
            S d1 = dot(r0, d), d2 = dot(r1, d), d3 = dot(r2, d);
            if (d1 > d2) return d1 > d3 ? r0 : r2;
            return d2 > d3 ? r1 : r2;
        }
        if (kind == SUP_POINT) return {S(0), S(0), S(0)};
        if (kind == SUP_CYLINDER) {  // cylinder{No,With}ConvexGetSupport cylinder.ts
            const S hl = sq_root(d.x * d.x + d.z * d.z);
            V<S> o{S(0), d.y >= S(0) ? he.y : -he.y, S(0)};
            if (hl > S(0)) {
                const S sc = radius / hl;
                o.x = d.x * sc;
                o.z = d.z * sc;
            }
            return o;
        }
        // capsule: segment +-h on Y (capsuleNoConvexGetSupport capsule.ts:268-275)
        if (kind == SUP_CAPSULE_SEGMENT) return {S(0), d.y > S(0) ? he.y : -he.y, S(0)};
        S l = lsq(d);
        if (kind == SUP_CAPSULE_SURFACE) {  // capsuleWithConvexGetSupport capsule.ts:321-338
            if (!(l > S(0))) return {S(0), he.y, S(0)};
            S sc = radius / sq_root(l);
            return {d.x * sc, d.y * sc + (d.y > S(0) ? he.y : -he.y), d.z * sc};
        }
        if (l > S(0)) return d * (radius / sq_root(l));
        return {S(0), S(0), S(0)};
    }
    __device__ V<S> get(V<S> d) const {
        V<S> o;
        if (transformed) {
            // local direction = R^T d ; point = R s + t
            V<S> ld{r0.x * d.x + r1.x * d.y + r2.x * d.z, r0.y * d.x + r1.y * d.y + r2.y * d.z,
                    r0.z * d.x + r1.z * d.y + r2.z * d.z};
            V<S> s = inner(ld);
            o = {dot(r0, s) + t.x, dot(r1, s) + t.y, dot(r2, s) + t.z};
        } else {
            o = inner(d);
        }
        if (add_r != S(0)) {
            S l = lsq(d);
            if (l > S(0)) o = o + d * (add_r / sq_root(l));
        }
        return o;
    }
};

// setBoxSupport support.ts:339-370 / getSphereSupportFunction sphere.ts:256-266
template <typename S, bool H = true, bool T = false>
__device__ Sup<S, H, T> make_sup(int shape, float4 sp, bool exclude, const HullView &hv) {
    Sup<S, H, T> o;
    o.transformed = false;
    o.add_r = S(0);
    o.radius = S(0);
    o.he = {S(0), S(0), S(0)};
    o.hp = nullptr;
    o.hn = 0;
    if (H && shape == SHAPE_HULL && hv.hulls) {
        // getConvexHullSupportFunction convex-hull.ts:968-997: the shrunk points with the convex
        // radius when it is excluded (and not zero), else the points themselves
        const DevHull &h = hv.hulls[hull_of(sp)];
        o.kind = SUP_HULL;
        o.hn = h.num_points;
        if (exclude && h.convex_radius != 0.f) {
            o.hp = hv.shrunk + h.first_point;
            o.convex_radius = S(h.convex_radius);
        } else {
            o.hp = hv.points + h.first_point;
            o.convex_radius = S(0);
        }
    } else if (shape == SHAPE_BOX) {
        o.kind = SUP_BOX;
        if (exclude) {
            S cr = S(sp.w) < S(0.05) ? S(sp.w) : S(0.05);
            o.he = {S(sp.x) - cr > S(0) ? S(sp.x) - cr : S(0), S(sp.y) - cr > S(0) ? S(sp.y) - cr : S(0),
                    S(sp.z) - cr > S(0) ? S(sp.z) - cr : S(0)};
            o.convex_radius = cr;
        } else {
            o.he = {S(sp.x), S(sp.y), S(sp.z)};
            o.convex_radius = S(0);
        }
    } else if (shape == SHAPE_CYLINDER) {
        // getCylinderSupportFunction cylinder.ts (half height sp.x, radius sp.y, convex radius sp.z)
        o.kind = SUP_CYLINDER;
        if (exclude) {
            o.he = {S(0), S(sp.x) - S(sp.z), S(0)};
            o.radius = S(sp.y) - S(sp.z);
            o.convex_radius = S(sp.z);
        } else {
            o.he = {S(0), S(sp.x), S(0)};
            o.radius = S(sp.y);
            o.convex_radius = S(0);
        }
    } else if (shape == SHAPE_CAPSULE) {
        // getCapsuleSupportFunction capsule.ts:390-404 (radius sp.x, half height sp.y)
        o.he = {S(0), S(sp.y), S(0)};
        if (exclude) {
            o.kind = SUP_CAPSULE_SEGMENT;
            o.convex_radius = S(sp.x);
        } else {
            o.kind = SUP_CAPSULE_SURFACE;
            o.radius = S(sp.x);
            o.convex_radius = S(0);
        }
    } else {
        if (exclude) {
            o.kind = SUP_POINT;
            o.convex_radius = S(sp.x);
        } else {
            o.kind = SUP_SPHERE;
            o.radius = S(sp.x);
            o.convex_radius = S(0);
        }
    }
    return o;
}
template <typename S, bool H, bool T>
__device__ void set_transform(Sup<S, H, T> &s, Q<S> q, V<S> p) {
    S x2 = q.x + q.x, y2 = q.y + q.y, z2 = q.z + q.z;
    S xx = q.x * x2, xy = q.x * y2, xz = q.x * z2, yy = q.y * y2, yz = q.y * z2, zz = q.z * z2;
    S wx = q.w * x2, wy = q.w * y2, wz = q.w * z2;
    s.r0 = {S(1) - (yy + zz), xy - wz, xz + wy};
    s.r1 = {xy + wz, S(1) - (xx + zz), yz - wx};
    s.r2 = {xz - wy, yz + wx, S(1) - (xx + yy)};
    s.t = p;
    s.transformed = true;
}

// ---------------------------------------------------------------------------
// GJK (gjk.ts), templated on precision
// ---------------------------------------------------------------------------
template <typename S>
struct SP {
    V<S> y, p, q;
};
template <typename S>
struct Simplex {
    SP<S> pts[4];
    int size;
};
template <typename S>
struct Bary {
    S u, v, w;
};
template <typename S>
__device__ Bary<S> bary2(V<S> a, V<S> b, S sqtol) {
    Bary<S> o{S(0), S(0), S(0)};
    V<S> ab = b - a;
    S den = lsq(ab);
    if (den < sqtol) {
        if (lsq(a) < lsq(b)) {
            o.u = S(1);
            o.v = S(0);
        } else {
            o.u = S(0);
            o.v = S(1);
        }
        return o;
    }
    o.v = -dot(a, ab) / den;
    o.u = S(1) - o.v;
    return o;
}
template <typename S>
__device__ Bary<S> bary3(V<S> a, V<S> b, V<S> c, S sqtol) {
    Bary<S> o{S(0), S(0), S(0)};
    V<S> ab = b - a, ac = c - a, bc = c - b;
    S d00 = lsq(ab), d11 = lsq(ac), d22 = lsq(bc);
    if (d00 <= d22) {
        S d01 = dot(ab, ac);
        S den = d00 * d11 - d01 * d01;
        if (s_abs(den) < S(1.0e-12)) {
            if (d00 > d11) {
                Bary<S> t = bary2(a, b, sqtol);
                o.u = t.u;
                o.v = t.v;
                o.w = S(0);
            } else {
                Bary<S> t = bary2(a, c, sqtol);
                o.u = t.u;
                o.w = t.v;
                o.v = S(0);
            }
            return o;
        }
        S a0 = dot(a, ab), a1 = dot(a, ac);
        o.v = (d01 * a1 - d11 * a0) / den;
        o.w = (d01 * a0 - d00 * a1) / den;
        o.u = S(1) - o.v - o.w;
    } else {
        S d12 = dot(ac, bc);
        S den = d11 * d22 - d12 * d12;
        if (s_abs(den) < S(1.0e-12)) {
            if (d11 > d22) {
                Bary<S> t = bary2(a, c, sqtol);
                o.u = t.u;
                o.w = t.v;
                o.v = S(0);
            } else {
                Bary<S> t = bary2(b, c, sqtol);
                o.v = t.u;
                o.w = t.v;
                o.u = S(0);
            }
            return o;
        }
        S c1 = dot(c, ac), c2 = dot(c, bc);
        o.u = (d22 * c1 - d12 * c2) / den;
        o.v = (d11 * c2 - d12 * c1) / den;
        o.w = S(1) - o.u - o.v;
    }
    return o;
}
template <typename S>
struct CP {
    V<S> p;
    int set;
};
template <typename S>
__device__ __forceinline__ S clamp01(S v) {
    return v < S(0) ? S(0) : (v > S(1) ? S(1) : v);
}
template <typename S>
__device__ CP<S> closest_line(V<S> a, V<S> b, S sqtol) {
    Bary<S> br = bary2(a, b, sqtol);
    if (br.v <= S(0)) return {a, 1};
    if (br.u <= S(0)) return {b, 2};
    return {a * br.u + b * br.v, 3};
}
template <typename S>
__device__ CP<S> closest_tri(V<S> inA, V<S> inB, V<S> inC, bool mustC, S sqtol) {
    V<S> ac0 = inC - inA, bc0 = inC - inB;
    bool swapAC = lsq(bc0) < lsq(ac0);
    V<S> a = swapAC ? inC : inA;
    V<S> c = swapAC ? inA : inC;
    V<S> ab = inB - a, ac = c - a;
    V<S> n = crs(ab, ac);
    S nls = lsq(n);
    if (nls < S(1.0e-10)) {
        int cs = 4;
        V<S> cp = inC;
        S best = lsq(inC);
        if (!mustC) {
            S al = lsq(inA);
            if (al < best) {
                cs = 1;
                cp = inA;
                best = al;
            }
            S bl = lsq(inB);
            if (bl < best) {
                cs = 2;
                cp = inB;
                best = bl;
            }
        }
        {
            V<S> e = c - a;
            S el = lsq(e);
            if (el > sqtol) {
                S v = clamp01(-dot(a, e) / el);
                V<S> q = a + e * v;
                S d = lsq(q);
                if (d < best) {
                    cs = 5;
                    cp = q;
                    best = d;
                }
            }
        }
        {
            V<S> e = inC - inB;
            S el = lsq(e);
            if (el > sqtol) {
                S v = clamp01(-dot(inB, e) / el);
                V<S> q = inB + e * v;
                S d = lsq(q);
                if (d < best) {
                    cs = 6;
                    cp = q;
                    best = d;
                }
            }
        }
        if (!mustC) {
            V<S> e = inB - inA;
            S el = lsq(e);
            if (el > sqtol) {
                S v = clamp01(-dot(inA, e) / el);
                V<S> q = inA + e * v;
                S d = lsq(q);
                if (d < best) {
                    cs = 3;
                    cp = q;
                }
            }
        }
        return {cp, cs};
    }
    V<S> ap = -a;
    S d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= S(0) && d2 <= S(0)) return {a, swapAC ? 4 : 1};
    V<S> bp = -inB;
    S d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= S(0) && d4 <= d3) return {inB, 2};
    if (d1 * d4 <= d3 * d2 && d1 >= S(0) && d3 <= S(0)) {
        S v = d1 / (d1 - d3);
        return {a + ab * v, swapAC ? 6 : 3};
    }
    V<S> cpv = -c;
    S d5 = dot(ab, cpv), d6 = dot(ac, cpv);
    if (d6 >= S(0) && d5 <= d6) return {c, swapAC ? 1 : 4};
    if (d5 * d2 <= d1 * d6 && d2 >= S(0) && d6 <= S(0)) {
        S ww = d2 / (d2 - d6);
        return {a + ac * ww, 5};
    }
    S d43 = d4 - d3, d56 = d5 - d6;
    if (d3 * d6 <= d5 * d4 && d43 >= S(0) && d56 >= S(0)) {
        S ww = d43 / (d43 + d56);
        return {inB + (c - inB) * ww, swapAC ? 3 : 6};
    }
    V<S> t = a + inB + c;
    S sc = dot(t, n) / (S(3) * nls);
    return {n * sc, 7};
}
template <typename S>
__device__ void outside_planes(int o[4], V<S> a, V<S> b, V<S> c, V<S> d, S tol) {
    V<S> ab = b - a, ac = c - a, ad = d - a, bd = d - b, bc = c - b;
    V<S> abac = crs(ab, ac), acad = crs(ac, ad), adab = crs(ad, ab), bdbc = crs(bd, bc);
    S spx = dot(a, abac), spy = dot(a, acad), spz = dot(a, adab), spw = dot(b, bdbc);
    S sdx = dot(ad, abac), sdy = dot(ab, acad), sdz = dot(ac, adab), sdw = -dot(ab, bdbc);
    if (sdx > S(0) && sdy > S(0) && sdz > S(0) && sdw > S(0)) {
        o[0] = spx >= -tol;
        o[1] = spy >= -tol;
        o[2] = spz >= -tol;
        o[3] = spw >= -tol;
        return;
    }
    if (sdx < S(0) && sdy < S(0) && sdz < S(0) && sdw < S(0)) {
        o[0] = spx <= tol;
        o[1] = spy <= tol;
        o[2] = spz <= tol;
        o[3] = spw <= tol;
        return;
    }
    o[0] = o[1] = o[2] = o[3] = 1;
}
template <typename S>
__device__ CP<S> closest_tetra(V<S> a, V<S> b, V<S> c, V<S> d, bool mustD, S tol) {
    S sqtol = tol * tol;
    CP<S> out{{S(0), S(0), S(0)}, 15};
    S best = s_max_value<S>();
    int o[4];
    outside_planes(o, a, b, c, d, tol);
    if (o[0]) {
        if (mustD)
            out = {a, 1};
        else
            out = closest_tri(a, b, c, false, sqtol);
        best = lsq(out.p);
    }
    if (o[1]) {
        CP<S> t = closest_tri(a, c, d, mustD, sqtol);
        S ds = lsq(t.p);
        if (ds < best) {
            best = ds;
            out.p = t.p;
            out.set = (t.set & 1) + ((t.set & 6) << 1);
        }
    }
    if (o[2]) {
        CP<S> t = closest_tri(a, b, d, mustD, sqtol);
        S ds = lsq(t.p);
        if (ds < best) {
            best = ds;
            out.p = t.p;
            out.set = (t.set & 3) + ((t.set & 4) << 1);
        }
    }
    if (o[3]) {
        CP<S> t = closest_tri(b, c, d, mustD, sqtol);
        S ds = lsq(t.p);
        if (ds < best) {
            out.p = t.p;
            out.set = t.set << 1;
        }
    }
    return out;
}

template <typename S>
struct GjkOut {
    S sqdist;
    V<S> axis, pa, pb;
};

// gjkClosestPoints gjk.ts:1294-1546
template <typename S, class SA, class SB>
__device__ GjkOut<S> gjk(const SA &A, const SB &B, S tolerance, V<S> dir, S maxDistSq, Simplex<S> &sx) {
    GjkOut<S> out;
    const S GJK_TOL = S(1e-5);
    S sqtol = tolerance * tolerance;
    sx.size = 0;
    V<S> v = dir;
    S vls = lsq(dir);
    S prev = s_max_value<S>();
    int it = 0;
    while (it++ < 100) {
        V<S> p = A.get(v);
        V<S> q = B.get(-v);
        V<S> w = p - q;
        S d = dot(v, w);
        if (d < S(0) && d * d > vls * maxDistSq) {
            out.sqdist = s_max_value<S>();
            out.axis = v;
            return out;
        }
        sx.pts[sx.size] = {w, p, q};
        sx.size++;
        CP<S> cp;
        switch (sx.size) {
            case 1:
                cp = {sx.pts[0].y, 1};
                break;
            case 2:
                cp = closest_line(sx.pts[0].y, sx.pts[1].y, S(1e-10));
                break;
            case 3:
                cp = closest_tri(sx.pts[0].y, sx.pts[1].y, sx.pts[2].y, true, S(1e-10));
                break;
            default:
                cp = closest_tetra(sx.pts[0].y, sx.pts[1].y, sx.pts[2].y, sx.pts[3].y, true, S(1e-5));
                break;
        }
        S nd = lsq(cp.p);
        if (!(nd < prev)) {
            sx.size--;
            break;
        }
        v = cp.p;
        vls = nd;
        if (cp.set == 0xf) {
            v = {S(0), S(0), S(0)};
            vls = S(0);
            break;
        }
        int ns = 0;
        for (int i = 0; i < sx.size; i++) {
            if (cp.set & (1 << i)) {
                if (ns != i) sx.pts[ns] = sx.pts[i];
                ns++;
            }
        }
        sx.size = ns;
        if (vls <= sqtol) {
            v = {S(0), S(0), S(0)};
            vls = S(0);
            break;
        }
        S ymax = S(0);
        for (int i = 0; i < sx.size; i++) {
            S l = lsq(sx.pts[i].y);
            ymax = ymax > l ? ymax : l;
        }
        if (vls <= GJK_TOL * ymax) {
            v = {S(0), S(0), S(0)};
            vls = S(0);
            break;
        }
        v = -v;
        if (prev - vls <= GJK_TOL * prev) break;
        prev = vls;
    }
    out.pa = {S(0), S(0), S(0)};
    out.pb = {S(0), S(0), S(0)};
    if (sx.size == 0) {
        out.sqdist = s_max_value<S>();
        out.axis = {S(0), S(0), S(0)};
        return out;
    }
    if (sx.size == 1) {
        out.pa = sx.pts[0].p;
        out.pb = sx.pts[0].q;
    } else if (sx.size == 2) {
        Bary<S> b = bary2(sx.pts[0].y, sx.pts[1].y, S(1e-10));
        out.pa = sx.pts[0].p * b.u + sx.pts[1].p * b.v;
        out.pb = sx.pts[0].q * b.u + sx.pts[1].q * b.v;
    } else if (sx.size == 3) {
        Bary<S> b = bary3(sx.pts[0].y, sx.pts[1].y, sx.pts[2].y, S(1e-10));
        out.pa = sx.pts[0].p * b.u + sx.pts[1].p * b.v + sx.pts[2].p * b.w;
        out.pb = sx.pts[0].q * b.u + sx.pts[1].q * b.v + sx.pts[2].q * b.w;
    }
    out.axis = v;
    out.sqdist = vls;
    return out;
}

// ---------------------------------------------------------------------------
// faces, clipping, reduction (FP32, coordinates relative to body A)
// ---------------------------------------------------------------------------
// Faces and clipped polygons hold at most N vertices: 16 for the pairs of boxes, spheres and
// capsules (4-vertex faces, 8-vertex clips), 32 when a hull takes part (a hull face gives at
// most MAX_FACE_VERTICES / 2 = 16 vertices, convex-hull.ts:88, 515-517, and a clip of two such
// faces up to 32).  The small instance keeps the common pairs' local frames small.
constexpr int FMAX_FACE = 32;  // MAX_FACE_VERTICES (convex-hull.ts:88)
template <int N>
struct FaceN {
    int n;
    float3 v[N];
};

// box getSupportingFace box.ts:129-332 (unit scale), then rotate + translate
template <int N>
__device__ void box_face(FaceN<N> &f, float3 dir, float4 he4, float4 q, float3 t) {
    float hx = he4.x, hy = he4.y, hz = he4.z;
    float ax = fabsf(dir.x), ay = fabsf(dir.y), az = fabsf(dir.z);
    f.n = 4;
    if (ax >= ay && ax >= az) {
        if (dir.x < 0.f) {
            f.v[0] = f3(hx, -hy, -hz);
            f.v[1] = f3(hx, hy, -hz);
            f.v[2] = f3(hx, hy, hz);
            f.v[3] = f3(hx, -hy, hz);
        } else {
            f.v[0] = f3(-hx, -hy, -hz);
            f.v[1] = f3(-hx, -hy, hz);
            f.v[2] = f3(-hx, hy, hz);
            f.v[3] = f3(-hx, hy, -hz);
        }
    } else if (ay >= ax && ay >= az) {
        if (dir.y < 0.f) {
            f.v[0] = f3(-hx, hy, -hz);
            f.v[1] = f3(-hx, hy, hz);
            f.v[2] = f3(hx, hy, hz);
            f.v[3] = f3(hx, hy, -hz);
        } else {
            f.v[0] = f3(-hx, -hy, -hz);
            f.v[1] = f3(hx, -hy, -hz);
            f.v[2] = f3(hx, -hy, hz);
            f.v[3] = f3(-hx, -hy, hz);
        }
    } else {
        if (dir.z < 0.f) {
            f.v[0] = f3(-hx, -hy, hz);
            f.v[1] = f3(hx, -hy, hz);
            f.v[2] = f3(hx, hy, hz);
            f.v[3] = f3(-hx, hy, hz);
        } else {
            f.v[0] = f3(-hx, -hy, -hz);
            f.v[1] = f3(-hx, hy, -hz);
            f.v[2] = f3(hx, hy, -hz);
            f.v[3] = f3(hx, -hy, -hz);
        }
    }
    Mat3 m = quat_to_mat(q);
    for (int i = 0; i < 4; i++) f.v[i] = mmul(m, f.v[i]) + t;
}

// capsule getSupportingFace capsule.ts:192-251: the segment on the side opposite to dir
// (body space) when both caps project within the capsule projection slop, else no face;
// rotated by q and moved by t
// cylinder getSupportingFace cylinder.ts (half height sp.x, radius sp.y): the side edge facing
// away from d, or the cap octagon (CYLINDER_CAP_OCTAGON) turned towards d's horizontal part
template <int N>
__device__ void cylinder_face(FaceN<N> &f, float3 d, float4 sp, float4 q, float3 t) {
    const float OCTX[8] = {0.0f, 0.707106769f, 1.0f, 0.707106769f, 0.0f, -0.707106769f, -1.0f, -0.707106769f};
    const float OCTZ[8] = {1.0f, 0.707106769f, 0.0f, -0.707106769f, -1.0f, -0.707106769f, 0.0f, 0.707106769f};
    const float h = sp.x, r = sp.y;
    const float xz = d.x * d.x + d.z * d.z, yy = d.y * d.y;
    if (xz > yy) {
        const float fct = -r / sqrtf(xz);
        f.n = 2;
        f.v[0] = qrot(q, f3(d.x * fct, h, d.z * fct)) + t;
        f.v[1] = qrot(q, f3(d.x * fct, -h, d.z * fct)) + t;
        return;
    }
    const float sx = d.y < 0.f ? r : -r, sy = d.y < 0.f ? h : -h, sz = r;
    float c = 1.f, sn = 0.f;
    if (xz > 0.00765427f * yy) {
        const float hl = sqrtf(xz);
        c = d.x / hl;
        sn = d.z / hl;
    }
    f.n = 8;
    for (int i = 0; i < 8; i++) {
        const float x = sx * OCTX[i], z = sz * OCTZ[i];
        f.v[i] = qrot(q, f3(x * c - z * sn, sy, x * sn + z * c)) + t;
    }
}
template <int N>
__device__ void capsule_face(FaceN<N> &f, float3 d, float4 sp, float4 q, float3 t) {
    float r = sp.x, h = sp.y;
    float len = sqrtf(d.x * d.x + d.z * d.z);
    f.n = 0;
    if (len == 0.f) return;
    float sx = (r / len) * d.x, sz = (r / len) * d.z;
    float3 top = f3(-sx, h, -sz), bottom = f3(-sx, -h, -sz);
    float pt = dot3(top, d), pb = dot3(bottom, d);
    const float slop = 0.02f;  // cCapsuleProjectionSlop
    if (fabsf(pt - pb) < slop * sqrtf(lensq3(d))) {
        f.n = 2;
        f.v[0] = qrot(q, top) + t;
        f.v[1] = qrot(q, bottom) + t;
    }
}

// convex hull getSupportingFace convex-hull.ts:479-541 (unit scale): the face whose plane
// normal is most opposed to dir, at most 16 of its vertices, rotated by q and moved by t
// ---- plane shape (src/shapes/plane.ts): shape record (unit normal xyz, constant) --------
// getOrthogonalBasis plane.ts:210-233
__device__ void plane_basis(float3 n, float3 &p1, float3 &p2) {
    p1 = cross3(n, f3(0.f, 1.f, 0.f));
    const float l = lensq3(p1);
    p1 = l < 1e-6f ? f3(1.f, 0.f, 0.f) : p1 * (1.f / sqrtf(l));
    p2 = normalize3(cross3(p1, n));
    p1 = normalize3(cross3(n, p2));
}
// the plane of a body at (p, q): transformPlane plane.ts:196-208
__device__ __forceinline__ void plane_world(float4 sp, float3 p, float4 q, float3 &n, float &c) {
    n = qrot(q, xyz(sp));
    c = sp.w - dot3(p, n);
}
// getAdaptivePlaneSupportingFace plane.ts:655-706: a square on the world plane (nw, cw) centred
// under cpos with half side |size| (the convex leaf's bounds diagonal), minus t
template <int N>
__device__ void plane_face(FaceN<N> &f, float3 nw, float cw, float3 cpos, float size, float3 t) {
    const float3 center = cpos - nw * (dot3(nw, cpos) + cw);
    float3 p1, p2;
    plane_basis(nw, p1, p2);
    p1 = p1 * size;
    p2 = p2 * size;
    f.n = 4;
    f.v[0] = center + (p1 + p2) - t;
    f.v[1] = center + (p1 - p2) - t;
    f.v[2] = center - (p1 + p2) - t;
    f.v[3] = center + (p2 - p1) - t;
}
__device__ float convex_bounds_size(const DevWorld &w, uint32_t f, float4 sp);
// SupportFunctionMode.DEFAULT: box and cylinder include their convex radius, the rest exclude it
__device__ __forceinline__ bool default_excludes(int shape) { return shape != SHAPE_BOX && shape != SHAPE_CYLINDER; }

template <int N>
__device__ void hull_face(FaceN<N> &f, float3 dir, const DevWorld &w, float4 sp, float4 q, float3 t) {
    const DevHull &h = w.hulls[hull_of(sp)];
    int best = 0;
    float bd = 0.f;
    for (int i = 0; i < h.num_faces; i++) {
        float4 pl = w.hull_planes[h.first_face + i];
        float3 n = f3(pl.x, pl.y, pl.z);
        float d = dot3(n, dir) / sqrtf(lensq3(n));
        if (i == 0 || d < bd) {
            bd = d;
            best = i;
        }
    }
    int2 fc = w.hull_faces[h.first_face + best];
    const int maxv = FMAX_FACE / 2;
    int step = (fc.y + maxv - 1) / maxv;
    f.n = 0;
    for (int i = 0; i < fc.y && f.n < N; i += step) {
        float4 p = w.hull_points[w.hull_vidx[fc.x + i]];
        f.v[f.n++] = qrot(q, f3(p.x, p.y, p.z)) + t;
    }
}

// clipPolyVsPlane clip.ts:13-92
template <int N>
__device__ void clip_plane(FaceN<N> &out, const FaceN<N> &in, float3 o, float3 n) {
    out.n = 0;
    if (in.n < 2) return;
    float3 e1 = in.v[in.n - 1];
    float prevNum = dot3(o - e1, n);
    bool prevIn = prevNum < 0.f;
    for (int j = 0; j < in.n; j++) {
        float3 e2 = in.v[j];
        float num = dot3(o - e2, n);
        bool curIn = num < 0.f;
        if (curIn != prevIn) {
            float3 e12 = e2 - e1;
            float den = dot3(e12, n);
            if (den != 0.f) {
                float t = prevNum / den;
                if (out.n < N) out.v[out.n++] = e1 + e12 * t;
            } else {
                curIn = prevIn;
            }
        }
        if (curIn && out.n < N) out.v[out.n++] = e2;
        prevNum = num;
        prevIn = curIn;
        e1 = e2;
    }
}

// clipPolyVsPoly clip.ts:108-175
template <int N>
__device__ void clip_poly(FaceN<N> &out, const FaceN<N> &toClip, const FaceN<N> &clipping, float3 cn) {
    out.n = 0;
    if (toClip.n < 2 || clipping.n < 3) return;
    FaceN<N> t0, t1;
    int tmpIdx = 0;
    for (int i = 0; i < clipping.n; i++) {
        float3 c1 = clipping.v[i];
        float3 c2 = clipping.v[(i + 1) % clipping.n];
        float3 pn = cross3(cn, c2 - c1);
        const FaceN<N> *src = (i == 0) ? &toClip : (tmpIdx == 0 ? &t0 : &t1);
        tmpIdx ^= 1;
        FaceN<N> *dst = (i == clipping.n - 1) ? &out : (tmpIdx == 0 ? &t0 : &t1);
        clip_plane(*dst, *src, c1, pn);
        if (dst->n < 3) {
            out.n = 0;
            return;
        }
    }
}

template <int N>
struct PtsN {
    int n;
    float3 a[N], b[N];
};

// pruneContactPoints manifold.ts:192-311
template <int N>
__device__ void prune(PtsN<N> &m, float3 axis) {
    const float MIN_D = 1.0e-6f;
    if (m.n <= 4) return;
    float3 proj[N];
    float dsq[N];
    for (int i = 0; i < m.n; i++) {
        float d = dot3(m.a[i], axis);
        proj[i] = m.a[i] - axis * d;
        dsq[i] = fmaxf(MIN_D, lensq3(m.b[i] - m.a[i]));
    }
    int p1 = 0;
    float mm = fmaxf(MIN_D, lensq3(proj[0])) * dsq[0];
    for (int i = 1; i < m.n; i++) {
        float met = fmaxf(MIN_D, lensq3(proj[i])) * dsq[i];
        if (met > mm) {
            mm = met;
            p1 = i;
        }
    }
    int p2 = -1;
    mm = -3.0e38f;
    for (int i = 0; i < m.n; i++) {
        if (i == p1) continue;
        float met = fmaxf(MIN_D, lensq3(proj[i] - proj[p1])) * dsq[i];
        if (met > mm) {
            mm = met;
            p2 = i;
        }
    }
    int p3 = -1, p4 = -1;
    float minD = 0.f, maxD = 0.f;
    float3 perp = cross3(proj[p2] - proj[p1], axis);
    for (int i = 0; i < m.n; i++) {
        if (i == p1 || i == p2) continue;
        float d = dot3(proj[i] - proj[p1], perp);
        if (d < minD) {
            minD = d;
            p3 = i;
        } else if (d > maxD) {
            maxD = d;
            p4 = i;
        }
    }
    int ord[4] = {p1, p3, p2, p4};
    float3 ka[4], kb[4];
    int o = 0;
    for (int k = 0; k < 4; k++) {
        if (ord[k] >= 0) {
            ka[o] = m.a[ord[k]];
            kb[o] = m.b[ord[k]];
            o++;
        }
    }
    for (int k = 0; k < o; k++) {
        m.a[k] = ka[k];
        m.b[k] = kb[k];
    }
    m.n = o;
}

// clipPolyVsEdge clip.ts:190-363: crossings of the polygon with the plane through the edge
// (normal = clip normal x edge), snapped onto the edge projected into the polygon's plane
template <int N>
__device__ void clip_poly_vs_edge(FaceN<N> &out, const FaceN<N> &poly, float3 ev1, float3 ev2, float3 cn) {
    out.n = 0;
    if (poly.n < 3) return;
    float3 en = cross3(cn, ev2 - ev1);
    float3 p0 = poly.v[0];
    float3 pn = cross3(poly.v[2] - p0, poly.v[1] - p0);
    float pl2 = lensq3(pn);
    float3 v1 = ev1 + pn * (dot3(p0 - ev1, pn) / pl2);
    float3 v2 = ev2 + pn * (dot3(p0 - ev2, pn) / pl2);
    float3 v12 = v2 - v1;
    float v12l2 = lensq3(v12);
    float3 e1 = poly.v[poly.n - 1];
    float prevNum = dot3(ev1 - e1, en);
    bool prevIn = prevNum < 0.f;
    for (int j = 0; j < poly.n; j++) {
        float3 e2 = poly.v[j];
        float num = dot3(ev1 - e2, en);
        bool curIn = num < 0.f;
        if (curIn != prevIn && out.n < N) {
            float3 e12 = e2 - e1;
            float den = dot3(e12, en);
            float3 c = den != 0.f ? e1 + e12 * (prevNum / den) : e1;
            float proj = dot3(c - v1, v12);
            out.v[out.n++] = proj < 0.f ? v1 : (proj > v12l2 ? v2 : c);
        }
        prevNum = num;
        prevIn = curIn;
        e1 = e2;
    }
}

// manifoldBetweenTwoFaces manifold.ts:345-444 (polygon faces)
template <int N>
__device__ void manifold_faces(PtsN<N> &out, float3 cp1, float3 cp2, float3 axis, float maxDist, const FaceN<N> &f1,
                               const FaceN<N> &f2) {
    out.n = 0;
    if (f1.n < 2 || f2.n < 3) {
        out.a[0] = cp1;
        out.b[0] = cp2;
        out.n = 1;
        return;
    }
    FaceN<N> clipped;
    clipped.n = 0;
    if (f1.n >= 3)
        clip_poly(clipped, f2, f1, axis);
    else
        clip_poly_vs_edge(clipped, f2, f1.v[0], f1.v[1], axis);
    float3 po = f1.v[0];
    float3 first = f1.v[1] - po;
    float3 pn;
    if (f1.n >= 3)
        pn = cross3(first, f1.v[2] - po);
    else
        pn = cross3(cross3(first, axis), first);
    float adn = dot3(axis, pn);
    if (adn != 0.f) {
        float al = sqrtf(lensq3(axis));
        for (int i = 0; i < clipped.n; i++) {
            float3 p2 = clipped.v[i];
            float dist = dot3(p2 - po, pn) / adn;
            if (dist * al < maxDist) {
                out.a[out.n] = p2 - axis * dist;
                out.b[out.n] = p2;
                out.n++;
                if (out.n >= N) break;
            }
        }
    }
    if (out.n == 0) {
        out.a[0] = cp1;
        out.b[0] = cp2;
        out.n = 1;
    }
}

// Turns one hit (relative to A's position) into a manifold: update.ts:385-558
// for a convex pair (a single hit, so a single manifold).
template <int N>
__device__ void emit_manifold(DevWorld &w, int a, int b, float3 pa, float3 pb, float3 axis, float penetration,
                              bool faces) {
    uint32_t fa = w.flags[a], fb = w.flags[b];
    float3 posA, posB;
    float4 qa, qb;
    geom_pose(w, a, fa, posA, qa);
    geom_pose(w, b, fb, posB, qb);
    PtsN<N> pts;
    float maxd = c_settings.spec_dist + c_settings.manifold_tol;
    float3 nrm = normalize3(axis);
    bool haveFaces = false;
    FaceN<N> fA, fB;
    fA.n = 0;
    fB.n = 0;
    if (faces) {
        // face directions in body space: A uses -axis, B uses axis (both rotated into the body frames)
        float3 axA = qrot_inv(qa, axis);
        float3 axB = qrot_inv(qb, axis);
        if (shape_of(fa) == SHAPE_BOX) box_face(fA, -axA, w.shape[a], qa, f3(0.f, 0.f, 0.f));
        if (shape_of(fa) == SHAPE_CAPSULE) capsule_face(fA, -axA, w.shape[a], qa, f3(0.f, 0.f, 0.f));
        if (shape_of(fa) == SHAPE_HULL) hull_face(fA, -axA, w, w.shape[a], qa, f3(0.f, 0.f, 0.f));
        if (shape_of(fb) == SHAPE_HULL) hull_face(fB, axB, w, w.shape[b], qb, posB - posA);
        if (shape_of(fb) == SHAPE_BOX) box_face(fB, axB, w.shape[b], qb, posB - posA);
        if (shape_of(fb) == SHAPE_CAPSULE) capsule_face(fB, axB, w.shape[b], qb, posB - posA);
        if (shape_of(fa) == SHAPE_CYLINDER) cylinder_face(fA, -axA, w.shape[a], qa, f3(0.f, 0.f, 0.f));
        if (shape_of(fb) == SHAPE_CYLINDER) cylinder_face(fB, axB, w.shape[b], qb, posB - posA);
        // a plane's face is the square under the convex body, made when the convex face has
        // vertices (collideConvexVsPlane plane.ts:588-606)
        if (shape_of(fa) == SHAPE_PLANE && fB.n > 0) {
            float3 nw;
            float cw;
            plane_world(w.shape[a], posA, qa, nw, cw);
            plane_face(fA, nw, cw, posB, convex_bounds_size(w, fb, w.shape[b]), posA);
        }
        if (shape_of(fb) == SHAPE_PLANE && fA.n > 0) {
            float3 nw;
            float cw;
            plane_world(w.shape[b], posB, qb, nw, cw);
            plane_face(fB, nw, cw, posA, convex_bounds_size(w, fa, w.shape[a]), posA);
        }
        haveFaces = fA.n >= 2 && fB.n >= 3;
    }
    if (haveFaces) {
        manifold_faces(pts, pa, pb, axis, maxd, fA, fB);
    } else {
        pts.n = 1;
        pts.a[0] = pa;
        pts.b[0] = pb;
    }
    if (pts.n > 32) prune(pts, nrm);
    nrm = normalize3(nrm);
    if (pts.n > 4) prune(pts, nrm);
    int slot = atomicAdd(&w.ctr->num_manifolds, 1);
    if (slot >= w.max_manifolds) {
        atomicOr(&w.ctr->overflow, OVF_MANIFOLDS);
        return;
    }
    Manifold m;
    m.a = a;
    m.b = b;
    m.n = pts.n;
    m.base = posA;
    m.normal = nrm;
    m.depth = penetration;
    for (int k = 0; k < 4; k++) {
        m.ra[k] = k < pts.n ? pts.a[k] : f3(0.f, 0.f, 0.f);
        m.rb[k] = k < pts.n ? pts.b[k] : f3(0.f, 0.f, 0.f);
    }
    m.sub_a = m.sub_b = 0xffffffffu;
    w.manifolds[slot] = m;
}

struct EpaItem {
    int a, b;
    int size;
    int pad;
    float3 y[4], p[4], q[4];
    int tri;  // -1: a convex pair; else a = the convex body, b = the mesh body, this triangle
};

// The collide class of a pair, by the shapes' collide routine: the pairs the mesh and compound
// passes take, plane pairs, sphere pairs, then the GJK pairs by their most expensive shape.
__device__ __forceinline__ int pair_class(uint32_t fa, uint32_t fb) {
    const int sa = shape_of(fa), sb = shape_of(fb);
    const int lo = min(sa, sb), hi = max(sa, sb);
    if (lo == SHAPE_EMPTY || hi == SHAPE_EMPTY || sa == SHAPE_MESH || sb == SHAPE_MESH || sa == SHAPE_COMPOUND ||
        sb == SHAPE_COMPOUND)
        return 0;
    if (sa == SHAPE_PLANE || sb == SHAPE_PLANE) return 1;
    if (sa == SHAPE_HULL || sb == SHAPE_HULL) return 2;
    if (lo == SHAPE_SPHERE && hi == SHAPE_SPHERE) return 3;
    if (sa == SHAPE_CYLINDER || sb == SHAPE_CYLINDER) return 4;
    if (sa == SHAPE_CAPSULE || sb == SHAPE_CAPSULE) return 5;
    if (sa == SHAPE_SPHERE || sb == SHAPE_SPHERE) return 6;  // a sphere against a box
    return 7;                                                // box against box
}

// k_pair_order: the pairs' indices grouped by collide class into w.pair_order (classes in order,
// any order inside a class).  Pass 0 counts the classes, pass 1 places the indices; one atomic
// per class present in a warp.
template <int PASS>
__global__ void k_pair_order(DevWorld w) {
    const int np = min(w.ctr->num_pairs, w.max_pairs);
    const int lane = threadIdx.x & 31;
    for (int base = blockIdx.x * blockDim.x; base < np; base += gridDim.x * blockDim.x) {
        const int pi = base + threadIdx.x;  // the warp's lanes stay together through the loop
        const bool live = pi < np;
        int c = -1;
        if (live) {
            const int2 pr = w.pairs[pi];
            c = pair_class(w.flags[pr.x], w.flags[pr.y]);
        }
        const unsigned same = __match_any_sync(0xffffffffu, c);
        const int leader = __ffs(same) - 1;
        int slot = 0;
        if (live && lane == leader)
            slot = atomicAdd(PASS == 0 ? &w.ctr->pair_class[c] : &w.ctr->pair_class_fill[c], __popc(same));
        slot = __shfl_sync(same, slot, leader);
        if (PASS == 1 && live) {
            int off = 0;
            for (int k = 0; k < c; k++) off += w.ctr->pair_class[k];
            w.pair_order[off + slot + __popc(same & ((1u << lane) - 1u))] = pi;
        }
    }
}

// narrowphase for one pair: order A/B (update.ts:74), dispatch, GJK
// HULLS: the pairs with a convex hull (launched only when the world has hulls); the other
// instance takes every other pair, without the hull code
template <bool HULLS>
__global__ void __launch_bounds__(128) k_narrowphase(DevWorld w, EpaItem *epa_items) {
    int np = min(w.ctr->num_pairs, w.max_pairs);
    for (int pk = blockIdx.x * blockDim.x + threadIdx.x; pk < np; pk += gridDim.x * blockDim.x) {
        const int pi = w.pair_order[pk];  // grouped by collide class
        int2 pr = w.pairs[pi];
        int a = pr.x, b = pr.y;
        uint32_t fa = w.flags[a], fb = w.flags[b];
        int ma = motion_of(fa), mb = motion_of(fb);
        if (ma > mb || (ma == mb && b < a)) {
            int t = a;
            a = b;
            b = t;
            uint32_t tf = fa;
            fa = fb;
            fb = tf;
        }
        float maxSep = ((fa | fb) & F_SENSOR) ? 0.f : c_settings.spec_dist;
        float3 pa3, pb3;
        float4 qa, qb;
        geom_pose(w, a, fa, pa3, qa);
        geom_pose(w, b, fb, pb3, qb);
        const float4 pa4 = make_float4(pa3.x, pa3.y, pa3.z, 0.f), pb4 = make_float4(pb3.x, pb3.y, pb3.z, 0.f);
        float4 sa = w.shape[a], sb = w.shape[b];
        int sha = shape_of(fa), shb = shape_of(fb);
        if (sha == SHAPE_EMPTY || shb == SHAPE_EMPTY) continue;  // empty-shape.ts registers no collide function
        if (sha == SHAPE_MESH || shb == SHAPE_MESH) {  // the mesh passes take these pairs
            if (sha == SHAPE_PLANE || shb == SHAPE_PLANE) continue;  // no mesh-vs-plane function
            if (!HULLS) {
                int k = atomicAdd(&w.ctr->num_mesh_pairs, 1);
                if (k < w.max_pairs) w.mesh_pairs[k] = pi;
            }
            continue;
        }
        if (sha == SHAPE_COMPOUND || shb == SHAPE_COMPOUND) {  // the compound pass takes these pairs
            if (!HULLS) {
                const int k = atomicAdd(&w.ctr->num_compound_pairs, 1);
                if (k < w.max_pairs) w.compound_pairs[k] = pi;
            }
            continue;
        }
        if ((sha == SHAPE_HULL || shb == SHAPE_HULL) != HULLS) continue;
        if (sha == SHAPE_PLANE || shb == SHAPE_PLANE) {
            // collideConvexVsPlane plane.ts:474-629, reversed when the plane is A (the usual case:
            // the plane is static); a plane against a plane has no collide function
            if (sha == SHAPE_PLANE && shb == SHAPE_PLANE) continue;
            const bool planeA = sha == SHAPE_PLANE;
            const float3 pC = planeA ? pb3 : pa3, pP = planeA ? pa3 : pb3;
            const float4 qC = planeA ? qb : qa, qP = planeA ? qa : qb;
            const float4 sC = planeA ? sb : sa, sP = planeA ? sa : sb;
            const int shC = planeA ? shb : sha;
            // the plane in the convex body's frame
            const float3 nl = qrot_inv(qC, qrot(qP, xyz(sP)));
            const float cl = sP.w - dot3(qrot_inv(qC, pP - pC), nl);
            const Sup<float, HULLS> S = make_sup<float, HULLS>(shC, sC, default_excludes(shC), hull_view(w));
            const V<float> spv = S.get(V<float>{-nl.x, -nl.y, -nl.z});
            const float3 sp3 = f3(spv.x, spv.y, spv.z);
            const float sd = dot3(nl, sp3) + cl, cr = S.convex_radius;
            const float pen = -sd + cr;
            if (!(pen > -maxSep)) continue;
            const float3 p1 = pC + qrot(qC, sp3 - nl * cr), p2 = pC + qrot(qC, sp3 - nl * sd);
            const float3 ax = qrot(qC, -nl);  // from the convex body into the plane
            // points relative to A's position; the axis from A to B
            if (planeA)
                emit_manifold<HULLS ? 32 : 16>(w, a, b, p2 - pa3, p1 - pa3, -ax, pen, true);
            else
                emit_manifold<HULLS ? 32 : 16>(w, a, b, p1 - pa3, p2 - pa3, ax, pen, true);
            continue;
        }
        if (sha == SHAPE_SPHERE && shb == SHAPE_SPHERE) {
            // collideSphereVsSphere sphere.ts:319-410 (no speculative distance)
            float3 d = xyz(pb4) - xyz(pa4);
            float dsq = lensq3(d);
            float rs = sa.x + sb.x;
            if (dsq >= rs * rs) continue;
            float dist = sqrtf(dsq);
            float3 n = dist > 0.f ? d * (1.f / dist) : f3(0.f, 1.f, 0.f);
            emit_manifold<16>(w, a, b, n * sa.x, d - n * sb.x, n, rs - dist, false);
            continue;
        }
        // collideConvexVsConvex convex.ts:257-346: B in A's local frame
        Q<float> qA{qa.x, qa.y, qa.z, qa.w}, qB{qb.x, qb.y, qb.z, qb.w};
        Q<float> iA{-qa.x, -qa.y, -qa.z, qa.w};
        Q<float> rel = qmulS(iA, qB);
        V<float> ab{pb4.x - pa4.x, pb4.y - pa4.y, pb4.z - pa4.z};
        V<float> posBInA = qrotS(iA, ab);
        const HullView hv = hull_view(w);
        Sup<float, HULLS> supA = make_sup<float, HULLS>(sha, sa, true, hv);
        Sup<float, HULLS> supB = make_sup<float, HULLS>(shb, sb, true, hv);
        set_transform(supB, rel, posBInA);
        V<float> axis = posBInA;
        if (lsq(axis) <= 1e-12f) axis = {1.f, 0.f, 0.f};
        float rA = supA.convex_radius + maxSep, rB = supB.convex_radius;
        float cr = rA + rB;
        Simplex<float> sx;
        GjkOut<float> g = gjk(supA, supB, c_settings.collision_tol, axis, cr * cr, sx);
        if (g.sqdist > cr * cr) continue;  // NOT_COLLIDING
        if (!(g.sqdist > 0.f)) {
            // INDETERMINATE: EPA in FP64 in a second pass
            int e = atomicAdd(&w.ctr->num_epa, 1);
            if (e >= w.max_epa) {
                atomicOr(&w.ctr->overflow, OVF_EPA);
                continue;
            }
            EpaItem it;
            it.a = a;
            it.b = b;
            it.size = sx.size;
            it.pad = 0;
            it.tri = -1;
            for (int k = 0; k < 4; k++) {
                SP<float> s = sx.pts[k < sx.size ? k : 0];
                it.y[k] = f3(s.y.x, s.y.y, s.y.z);
                it.p[k] = f3(s.p.x, s.p.y, s.p.z);
                it.q[k] = f3(s.q.x, s.q.y, s.q.z);
            }
            epa_items[e] = it;
            continue;
        }
        // COLLIDING: penetrationDepthStepGJK penetration.ts:84-106
        float vl = sqrtf(g.sqdist);
        V<float> pa = g.pa + g.axis * (rA / vl);
        V<float> pb = g.pb + g.axis * (-(rB / vl));
        V<float> dd = pa - pb;
        float penetration = sqrtf(lsq(dd)) - maxSep;
        float al = sqrtf(lsq(g.axis));
        if (al > 0.f) pa = pa + g.axis * (-(maxSep / al));
        V<float> paw = qrotS(qA, pa), pbw = qrotS(qA, pb), axw = qrotS(qA, g.axis);
        emit_manifold<HULLS ? 32 : 16>(w, a, b, f3(paw.x, paw.y, paw.z), f3(pbw.x, pbw.y, pbw.z),
                                       f3(axw.x, axw.y, axw.z), penetration, true);
    }
}

// ---------------------------------------------------------------------------
// EPA (penetration.ts:214-614 + epa-convex-hull-builder.ts) in FP64.
//
// The hull algorithm is written once over a storage policy:
//  * PackedStore: a compact polytope (32 support points, 64 triangles) with every
//    array interleaved across the 64 threads of a block ([element][thread]), so a
//    warp touching the same element of its lanes' polytopes reads one or two
//    cache lines.  The reference's polytopes stay far below these limits (on the
//    seeded scenes: 15 points and 25 triangles at most).
//  * BigStore: the reference's limits (128 points, 256 triangles, 128-edge
//    horizon) in a per-thread slice.  Items whose polytope outgrows the packed
//    limits are re-run from their GJK simplex with this store, so every item gets
//    the reference's behaviour at the reference's limits.
// ---------------------------------------------------------------------------
// the real type of the polytope arithmetic
using R = double;
constexpr R R_EPS_INTERIOR = R(1e-3);           // interior test margin (:287-289)
constexpr R R_ONE_PLUS_EPS = R(1.0 + 1e-3);
constexpr R R_MIN_NORMAL_SQ = R(1e-10);         // degenerate-normal threshold (:255, :300)
constexpr R R_THIRD = R(1.0 / 3.0);
constexpr int EPA_MAX_TRI = 256;
constexpr int EPA_PTS_CAP = 160;
constexpr int EPA_QUEUE_CAP = 512;
constexpr int EPA_EDGE_CAP = 128;
constexpr int EPA_BLOCK = 64;

// triangle flags
enum : int { TF_REL0 = 1, TF_INTERIOR = 2, TF_REMOVED = 4, TF_INQ = 8 };

struct EpaTri {
    V<R> normal, centroid;
    R cls;
    int nt[3];
    int ne[3];
    int st[3];
    int flags;
};
struct EpaScratch {
    V<R> Y[EPA_PTS_CAP], P[EPA_PTS_CAP], Qp[EPA_PTS_CAP];
    EpaTri tri[EPA_MAX_TRI];
    int queue[EPA_QUEUE_CAP];
    int freel[EPA_MAX_TRI];
    int edge_nt[EPA_EDGE_CAP], edge_ne[EPA_EDGE_CAP], edge_st[EPA_EDGE_CAP];
    int stk_t[EPA_EDGE_CAP], stk_e[EPA_EDGE_CAP], stk_i[EPA_EDGE_CAP];
    int newt[EPA_EDGE_CAP];
};
size_t epa_scratch_bytes() { return sizeof(EpaScratch); }

struct BigStore {
    static constexpr int PTS = EPA_PTS_CAP, TRI = EPA_MAX_TRI, QCAP = EPA_QUEUE_CAP, ECAP = EPA_EDGE_CAP;
    static constexpr bool PACKED = false;
    EpaScratch *s;
    __device__ V<R> Y(int i) const { return s->Y[i]; }
    __device__ V<R> P(int i) const { return s->P[i]; }
    __device__ V<R> Q(int i) const { return s->Qp[i]; }
    __device__ void set_point(int i, V<R> y, V<R> p, V<R> q) {
        s->Y[i] = y;
        s->P[i] = p;
        s->Qp[i] = q;
    }
    __device__ V<R> normal(int t) const { return s->tri[t].normal; }
    __device__ V<R> centroid(int t) const { return s->tri[t].centroid; }
    __device__ R cls(int t) const { return s->tri[t].cls; }
    __device__ int flags(int t) const { return s->tri[t].flags; }
    __device__ int st(int t, int k) const { return s->tri[t].st[k]; }
    __device__ int nt(int t, int k) const { return s->tri[t].nt[k]; }
    __device__ int ne(int t, int k) const { return s->tri[t].ne[k]; }
    __device__ void set_geom(int t, V<R> n, V<R> c, R cls) {
        s->tri[t].normal = n;
        s->tri[t].centroid = c;
        s->tri[t].cls = cls;
    }
    __device__ void set_flags(int t, int f) { s->tri[t].flags = f; }
    __device__ void set_st(int t, int a, int b, int c) {
        s->tri[t].st[0] = a;
        s->tri[t].st[1] = b;
        s->tri[t].st[2] = c;
    }
    __device__ void set_nb(int t, int k, int n, int e) {
        s->tri[t].nt[k] = n;
        s->tri[t].ne[k] = e;
    }
    __device__ int q(int i) const { return s->queue[i]; }
    __device__ void set_q(int i, int t) { s->queue[i] = t; }
    __device__ int fr(int i) const { return s->freel[i]; }
    __device__ void set_fr(int i, int t) { s->freel[i] = t; }
    __device__ void set_edge(int i, int n, int e, int st) {
        s->edge_nt[i] = n;
        s->edge_ne[i] = e;
        s->edge_st[i] = st;
    }
    __device__ int edge_nt(int i) const { return s->edge_nt[i]; }
    __device__ int edge_ne(int i) const { return s->edge_ne[i]; }
    __device__ int edge_st(int i) const { return s->edge_st[i]; }
    __device__ void set_stk(int i, int t, int e, int k) {
        s->stk_t[i] = t;
        s->stk_e[i] = e;
        s->stk_i[i] = k;
    }
    __device__ int stk_t(int i) const { return s->stk_t[i]; }
    __device__ int stk_e(int i) const { return s->stk_e[i]; }
    __device__ int stk_i(int i) const { return s->stk_i[i]; }
    __device__ void set_stk_i(int i, int k) { s->stk_i[i] = k; }
    __device__ int newt(int i) const { return s->newt[i]; }
    __device__ void set_newt(int i, int t) { s->newt[i] = t; }
};

// one block's packed polytopes: element e of thread j lives at [e][j]
constexpr int PK_PTS = 32, PK_TRI = 64, PK_Q = 64, PK_E = 32;
struct PackedBlock {
    R yx[PK_PTS][EPA_BLOCK], yy[PK_PTS][EPA_BLOCK], yz[PK_PTS][EPA_BLOCK];
    R px[PK_PTS][EPA_BLOCK], py[PK_PTS][EPA_BLOCK], pz[PK_PTS][EPA_BLOCK];
    R qx[PK_PTS][EPA_BLOCK], qy[PK_PTS][EPA_BLOCK], qz[PK_PTS][EPA_BLOCK];
    R nx[PK_TRI][EPA_BLOCK], ny[PK_TRI][EPA_BLOCK], nz[PK_TRI][EPA_BLOCK];
    R cx[PK_TRI][EPA_BLOCK], cy[PK_TRI][EPA_BLOCK], cz[PK_TRI][EPA_BLOCK];
    R cl[PK_TRI][EPA_BLOCK];
    float fnx[PK_TRI][EPA_BLOCK], fny[PK_TRI][EPA_BLOCK], fnz[PK_TRI][EPA_BLOCK];  // FP32 copies of the
    float fcx[PK_TRI][EPA_BLOCK], fcy[PK_TRI][EPA_BLOCK], fcz[PK_TRI][EPA_BLOCK];  // normal and centroid
    uint32_t vf[PK_TRI][EPA_BLOCK];   // st0 | st1 << 8 | st2 << 16 | flags << 24
    uint32_t nbt[PK_TRI][EPA_BLOCK];  // neighbour triangles, 8 bits each (0xff: none)
    uint32_t nbe[PK_TRI][EPA_BLOCK];  // neighbour edges, 8 bits each
    uint8_t queue[PK_Q][EPA_BLOCK];
    uint8_t freel[PK_TRI][EPA_BLOCK];
    uint8_t e_nt[PK_E][EPA_BLOCK], e_ne[PK_E][EPA_BLOCK], e_st[PK_E][EPA_BLOCK];
    uint8_t s_t[PK_E][EPA_BLOCK], s_e[PK_E][EPA_BLOCK], s_i[PK_E][EPA_BLOCK];
    uint8_t nw[PK_E][EPA_BLOCK];
};
size_t epa_packed_block_bytes() { return sizeof(PackedBlock); }

struct PackedStore {
    static constexpr int PTS = PK_PTS, TRI = PK_TRI, QCAP = PK_Q, ECAP = PK_E;
    static constexpr bool PACKED = true;
    PackedBlock *b;
    int j;  // thread within the block
    __device__ V<R> Y(int i) const { return {b->yx[i][j], b->yy[i][j], b->yz[i][j]}; }
    __device__ V<R> P(int i) const { return {b->px[i][j], b->py[i][j], b->pz[i][j]}; }
    __device__ V<R> Q(int i) const { return {b->qx[i][j], b->qy[i][j], b->qz[i][j]}; }
    __device__ void set_point(int i, V<R> y, V<R> p, V<R> q) {
        b->yx[i][j] = y.x;
        b->yy[i][j] = y.y;
        b->yz[i][j] = y.z;
        b->px[i][j] = p.x;
        b->py[i][j] = p.y;
        b->pz[i][j] = p.z;
        b->qx[i][j] = q.x;
        b->qy[i][j] = q.y;
        b->qz[i][j] = q.z;
    }
    __device__ V<R> normal(int t) const { return {b->nx[t][j], b->ny[t][j], b->nz[t][j]}; }
    __device__ V<R> centroid(int t) const { return {b->cx[t][j], b->cy[t][j], b->cz[t][j]}; }
    __device__ R cls(int t) const { return b->cl[t][j]; }
    __device__ int flags(int t) const { return (int)(b->vf[t][j] >> 24); }
    __device__ int st(int t, int k) const { return (int)((b->vf[t][j] >> (8 * k)) & 0xffu); }
    __device__ int nt(int t, int k) const {
        uint32_t v = (b->nbt[t][j] >> (8 * k)) & 0xffu;
        return v == 0xffu ? -1 : (int)v;
    }
    __device__ int ne(int t, int k) const { return (int)((b->nbe[t][j] >> (8 * k)) & 0xffu); }
    __device__ void set_geom(int t, V<R> n, V<R> c, R cls) {
        b->nx[t][j] = n.x;
        b->ny[t][j] = n.y;
        b->nz[t][j] = n.z;
        b->cx[t][j] = c.x;
        b->cy[t][j] = c.y;
        b->cz[t][j] = c.z;
        b->cl[t][j] = cls;
        b->fnx[t][j] = (float)n.x;
        b->fny[t][j] = (float)n.y;
        b->fnz[t][j] = (float)n.z;
        b->fcx[t][j] = (float)c.x;
        b->fcy[t][j] = (float)c.y;
        b->fcz[t][j] = (float)c.z;
    }
    __device__ float3 normal32(int t) const { return make_float3(b->fnx[t][j], b->fny[t][j], b->fnz[t][j]); }
    __device__ float3 centroid32(int t) const { return make_float3(b->fcx[t][j], b->fcy[t][j], b->fcz[t][j]); }
    __device__ void set_flags(int t, int f) { b->vf[t][j] = (b->vf[t][j] & 0x00ffffffu) | ((uint32_t)f << 24); }
    __device__ void set_st(int t, int a, int c, int d) {
        b->vf[t][j] = (b->vf[t][j] & 0xff000000u) | (uint32_t)a | ((uint32_t)c << 8) | ((uint32_t)d << 16);
    }
    __device__ void set_nb(int t, int k, int n, int e) {
        uint32_t sh = 8 * k, m = ~(0xffu << sh);
        b->nbt[t][j] = (b->nbt[t][j] & m) | ((uint32_t)(n < 0 ? 0xff : n) << sh);
        b->nbe[t][j] = (b->nbe[t][j] & m) | ((uint32_t)e << sh);
    }
    __device__ int q(int i) const { return b->queue[i][j]; }
    __device__ void set_q(int i, int t) { b->queue[i][j] = (uint8_t)t; }
    __device__ int fr(int i) const { return b->freel[i][j]; }
    __device__ void set_fr(int i, int t) { b->freel[i][j] = (uint8_t)t; }
    __device__ void set_edge(int i, int n, int e, int st) {
        b->e_nt[i][j] = (uint8_t)n;
        b->e_ne[i][j] = (uint8_t)e;
        b->e_st[i][j] = (uint8_t)st;
    }
    __device__ int edge_nt(int i) const { return b->e_nt[i][j]; }
    __device__ int edge_ne(int i) const { return b->e_ne[i][j]; }
    __device__ int edge_st(int i) const { return b->e_st[i][j]; }
    __device__ void set_stk(int i, int t, int e, int k) {
        b->s_t[i][j] = (uint8_t)t;
        b->s_e[i][j] = (uint8_t)e;
        b->s_i[i][j] = (uint8_t)k;
    }
    __device__ int stk_t(int i) const { return b->s_t[i][j]; }
    __device__ int stk_e(int i) const { return b->s_e[i][j]; }
    __device__ int stk_i(int i) const { return (int)(int8_t)b->s_i[i][j]; }
    __device__ void set_stk_i(int i, int k) { b->s_i[i][j] = (uint8_t)(int8_t)k; }
    __device__ int newt(int i) const { return b->nw[i][j]; }
    __device__ void set_newt(int i, int t) { b->nw[i][j] = (uint8_t)t; }
};

// The geometry half of createTriangle (epa-convex-hull-builder.ts:179-345) for slot idx of the
// polytope in store s: centroid, normal, closest distance and the interior flags.  Returns whether
// the face's normal and centroid have dot(n, c) < 0, the defect test penetration.ts:485-486
// takes on every new face.
template <class S>
__device__ bool tri_geom(S &s, int idx, int i1, int i2, int i3) {
    int fl = 0;
    R cls = 1.0 / 0.0;
    V<R> y0 = s.Y(i1), y1 = s.Y(i2), y2 = s.Y(i3);
    // centroid (:219-225): the division by 3 is a multiplication by 1/3 here
    V<R> c{(y0.x + y1.x + y2.x) * R_THIRD, (y0.y + y1.y + y2.y) * R_THIRD, (y0.z + y1.z + y2.z) * R_THIRD};
    V<R> y10 = y1 - y0, y20 = y2 - y0, y21 = y2 - y1;
    R y20d = lsq(y20), y21d = lsq(y21);
    // the interior test l0 > -1e-3, l1 > -1e-3, l0 + l1 < 1 + 1e-3 is taken on the numerators
    // (det > 0); the lambdas of the triangle the result uses are divided out in epa()
    V<R> n;
    if (y20d < y21d) {
        n = crs(y10, y20);
        R nl = lsq(n);
        if (nl > R_MIN_NORMAL_SQ) {
            R cdn = dot(c, n);
            cls = (s_abs(cdn) * cdn) / nl;
            R y10d = lsq(y10), y1020 = dot(y10, y20);
            R det = y10d * y20d - y1020 * y1020;
            if (det > 0.0) {
                R a = dot(y0, y10), b = dot(y0, y20);
                R l0n = y1020 * b - y20d * a, l1n = y1020 * a - y10d * b;
                fl |= TF_REL0;
                if (l0n > -R_EPS_INTERIOR * det && l1n > -R_EPS_INTERIOR * det && l0n + l1n < R_ONE_PLUS_EPS * det)
                    fl |= TF_INTERIOR;
            }
        }
    } else {
        n = crs(y10, y21);
        R nl = lsq(n);
        if (nl > R_MIN_NORMAL_SQ) {
            R cdn = dot(c, n);
            cls = (s_abs(cdn) * cdn) / nl;
            R y10d = lsq(y10), y1021 = dot(y10, y21);
            R det = y10d * y21d - y1021 * y1021;
            if (det > 0.0) {
                R a = dot(y1, y10), b = dot(y1, y21);
                R l0n = y21d * a - y1021 * b, l1n = y1021 * a - y10d * b;
                if (l0n > -R_EPS_INTERIOR * det && l1n > -R_EPS_INTERIOR * det && l0n + l1n < R_ONE_PLUS_EPS * det)
                    fl |= TF_INTERIOR;
            }
        }
    }
    s.set_geom(idx, n, c, cls);
    s.set_flags(idx, fl);
    return dot(n, c) < 0.0;
}

// An integer key with the order of the doubles it comes from (-0 and +0 equal, no NaNs here):
// the heap and the face selection compare closest distances with integer instructions, which
// keeps them off the FP64 pipe.
__device__ __forceinline__ unsigned long long order_key(R x) {
    long long b = __double_as_longlong(x);
    if (b == (long long)0x8000000000000000ull) b = 0;
    return b < 0 ? ~(unsigned long long)b : ((unsigned long long)b | 0x8000000000000000ull);
}

template <class S>
struct Hull {
    S st;
    int ntri, nfree, nq, npts;
    int pts_limit;  // support points this store may hold (at most S::PTS)
    bool overflow;  // a packed limit was exceeded: the item must be re-run with the reference's limits
    __device__ bool facing(int t, V<R> p) const { return dot(st.normal(t), p - st.centroid(t)) > 0.0; }
    __device__ R cls(int t) const { return st.cls(t); }
    __device__ int flags(int t) const { return st.flags(t); }
    __device__ void add_flags(int t, int f) { st.set_flags(t, st.flags(t) | f); }
    // pushTriangleToQueue epa-convex-hull-builder.ts:95-116
    __device__ void push(int t) {
        if (nq >= S::QCAP) {
            if (S::PACKED) overflow = true;
            return;
        }
        st.set_q(nq, t);
        add_flags(t, TF_INQ);
        int cur = nq++;
        while (cur > 0) {
            int par = (cur - 1) >> 1;
            int qp = st.q(par), qc = st.q(cur);
            if (order_key(st.cls(qp)) > order_key(st.cls(qc))) {
                st.set_q(par, qc);
                st.set_q(cur, qp);
                cur = par;
            } else {
                break;
            }
        }
    }
    __device__ int pop() {
        if (nq == 0) return -1;
        int last = st.q(nq - 1);
        st.set_q(nq - 1, st.q(0));
        st.set_q(0, last);
        int count = nq - 1;
        int largest = 0;
        while (true) {
            int child = (largest << 1) + 1;
            if (child >= count) break;
            int prevL = largest;
            if (order_key(st.cls(st.q(largest))) > order_key(st.cls(st.q(child)))) largest = child;
            ++child;
            if (child < count && order_key(st.cls(st.q(largest))) > order_key(st.cls(st.q(child)))) largest = child;
            if (prevL == largest) break;
            int t2 = st.q(prevL);
            st.set_q(prevL, st.q(largest));
            st.set_q(largest, t2);
        }
        nq--;
        return st.q(nq);
    }
    __device__ void link(int t1, int e1, int t2, int e2) {
        st.set_nb(t1, e1, t2, e2);
        st.set_nb(t2, e2, t1, e1);
    }
    // createTriangle epa-convex-hull-builder.ts:179-345: a slot (alloc) and its geometry (tri_geom)
    __device__ int alloc(int i1, int i2, int i3) {
        int idx;
        if (nfree > 0) {
            idx = st.fr(--nfree);
        } else {
            if (ntri >= S::TRI) {
                if (S::PACKED) overflow = true;
                return -1;
            }
            idx = ntri++;
        }
        st.set_st(idx, i1, i2, i3);
        for (int k = 0; k < 3; k++) st.set_nb(idx, k, -1, 0);
        return idx;
    }
    __device__ int create(int i1, int i2, int i3) {
        int idx = alloc(i1, i2, i3);
        if (idx >= 0) tri_geom(st, idx, i1, i2, i3);
        return idx;
    }
    // barycentric lambdas of triangle t (the second half of createTriangle)
    __device__ void lambdas(int t, R &l0, R &l1, bool &rel0) const {
        V<R> y0 = st.Y(st.st(t, 0)), y1 = st.Y(st.st(t, 1)), y2 = st.Y(st.st(t, 2));
        V<R> y10 = y1 - y0, y20 = y2 - y0, y21 = y2 - y1;
        R y20d = lsq(y20), y21d = lsq(y21);
        l0 = l1 = 0.0;
        rel0 = false;
        if (y20d < y21d) {
            if (!(lsq(crs(y10, y20)) > R_MIN_NORMAL_SQ)) return;
            R y10d = lsq(y10), y1020 = dot(y10, y20);
            R det = y10d * y20d - y1020 * y1020;
            if (det > 0.0) {
                R a = dot(y0, y10), b = dot(y0, y20);
                l0 = (y1020 * b - y20d * a) / det;
                l1 = (y1020 * a - y10d * b) / det;
                rel0 = true;
            }
        } else {
            if (!(lsq(crs(y10, y21)) > R_MIN_NORMAL_SQ)) return;
            R y10d = lsq(y10), y1021 = dot(y10, y21);
            R det = y10d * y21d - y1021 * y1021;
            if (det > 0.0) {
                R a = dot(y1, y10), b = dot(y1, y21);
                l0 = (y21d * a - y1021 * b) / det;
                l1 = (y1021 * a - y10d * b) / det;
            }
        }
    }
    __device__ void free_tri(int t) {
        if (nfree < S::TRI) st.set_fr(nfree++, t);
    }
    __device__ void unlink(int t) {
        for (int i = 0; i < 3; i++) {
            int n = st.nt(t, i);
            if (n >= 0) {
                st.set_nb(n, st.ne(t, i), -1, 0);
                st.set_nb(t, i, -1, 0);
            }
        }
        if (!(flags(t) & TF_INQ)) free_tri(t);
    }
    // findFacingTriangle epa-convex-hull-builder.ts:420-474
    __device__ int find_facing(V<R> p) {
        int best = -1;
        R bestd = 0.0;
        for (int i = 0; i < nq; i++) {
            int t = st.q(i);
            if (flags(t) & TF_REMOVED) continue;
            V<R> n = st.normal(t);
            R d = dot(n, p - st.centroid(t));
            if (d > 0.0) {
                R dsq = (d * d) / lsq(n);
                if (dsq > bestd) {
                    best = t;
                    bestd = dsq;
                }
            }
        }
        return best;
    }
    // The facing test of every triangle slot below `upto` against p, as a bit mask.  The lanes of a
    // warp run the loop together (upto is the same on every lane), so the FP64 tests issue with
    // every lane whose polytope has that slot; find_edge then reads the bits (the geometry of a
    // triangle does not change while its flags do).  Packed store only (at most 64 slots).
    //
    // The test is taken in FP32 on the faces' FP32 copies first.  Rounding the inputs and the
    // FP32 arithmetic move the dot product by at most about 6 x 2^-24 x S, S = sum |n_i|
    // (|p_i| + |c_i|); when the FP32 value is further than 2^-19 x S from zero its sign is the
    // exact sign, and so the sign the FP64 test gives.  Closer calls are taken in FP64.
    __device__ unsigned long long facing_mask(V<R> p, int upto) const {
        const float px = (float)p.x, py = (float)p.y, pz = (float)p.z;
        const float ax = fabsf(px), ay = fabsf(py), az = fabsf(pz);
        unsigned long long m = 0ull;
        for (int t = 0; t < upto; t++) {
            if (t >= ntri) continue;
            const float3 n = st.normal32(t), c = st.centroid32(t);
            const float r = n.x * (px - c.x) + n.y * (py - c.y) + n.z * (pz - c.z);
            const float e = 1.9073486328125e-06f *  // 2^-19
                            (fabsf(n.x) * (ax + fabsf(c.x)) + fabsf(n.y) * (ay + fabsf(c.y)) + fabsf(n.z) * (az + fabsf(c.z)));
            bool f;
            if (r > e)
                f = true;
            else if (r < -e)
                f = false;
            else
                f = facing(t, p);
            if (f) m |= 1ull << t;
        }
        return m;
    }
    __device__ bool facing_of(int t, V<R> vtx, const unsigned long long *mask) const {
        return mask ? ((*mask >> t) & 1ull) != 0 : facing(t, vtx);
    }
    // findEdge epa-convex-hull-builder.ts:476-540; returns the edge count or -1.  mask: the facing
    // bits of the triangle slots (facing_mask), or null to test them as they are met
    __device__ int find_edge(int ft, V<R> vtx, const unsigned long long *mask = nullptr) {
        int ne = 0;
        add_flags(ft, TF_REMOVED);
        int sp = 0;
        st.set_stk(0, ft, 0, -1);
        int next_expected = -1;
        int guard = 0;
        while (guard++ < 100000) {
            int ct = st.stk_t(sp);
            int si = st.stk_i(sp) + 1;
            st.set_stk_i(sp, si);
            if (si >= 3) {
                unlink(ct);
                if (--sp < 0) break;
            } else {
                int ei = (st.stk_e(sp) + si) % 3;
                int n = st.nt(ct, ei);
                int nen = st.ne(ct, ei);
                int est = st.st(ct, ei);
                if (n >= 0 && !(flags(n) & TF_REMOVED)) {
                    if (facing_of(n, vtx, mask)) {
                        add_flags(n, TF_REMOVED);
                        sp++;
                        if (sp >= S::ECAP) {
                            if (S::PACKED) overflow = true;
                            return -1;
                        }
                        st.set_stk(sp, n, nen, 0);
                    } else {
                        if (est != next_expected && next_expected != -1) return -1;
                        next_expected = st.st(n, nen);
                        if (ne >= S::ECAP) {
                            if (S::PACKED) overflow = true;
                            return -1;
                        }
                        st.set_edge(ne, n, nen, est);
                        ne++;
                    }
                }
            }
        }
        if (ne > 0 && st.edge_st(0) != next_expected) return -1;
        return ne >= 3 ? ne : -1;
    }
    // addPoint epa-convex-hull-builder.ts:541-600
    __device__ int add_point(int ft, int idx, R closest, const unsigned long long *mask = nullptr) {
        int ne = find_edge(ft, st.Y(idx), mask);
        if (ne < 0) return -1;
        for (int i = 0; i < ne; i++) {
            int in = (i + 1) % ne;
            int nt = create(st.edge_st(i), st.edge_st(in), idx);
            if (nt < 0) return -1;
            st.set_newt(i, nt);
            if (((flags(nt) & TF_INTERIOR) && cls(nt) < closest) || cls(nt) < 0.0) push(nt);
        }
        for (int i = 0; i < ne; i++) {
            int in = (i + 1) % ne;
            link(st.newt(i), 0, st.edge_nt(i), st.edge_ne(i));
            link(st.newt(i), 1, st.newt(in), 2);
        }
        return ne;
    }
    // addPoint in two halves around the new faces' geometry, which the lock-step pass spreads
    // over the warp (warp_tri_geom): the horizon and the new faces' slots in addPoint's order,
    // then, once their geometry is written, the queue and the links
    __device__ int add_point_slots(int ft, int idx, const unsigned long long *mask) {
        int ne = find_edge(ft, st.Y(idx), mask);
        if (ne < 0) return -1;
        for (int i = 0; i < ne; i++) {
            int nt = alloc(st.edge_st(i), st.edge_st((i + 1) % ne), idx);
            if (nt < 0) return -1;
            st.set_newt(i, nt);
        }
        return ne;
    }
    __device__ void add_point_links(int ne, R closest) {
        for (int i = 0; i < ne; i++) {
            int nt = st.newt(i);
            if (((flags(nt) & TF_INTERIOR) && cls(nt) < closest) || cls(nt) < 0.0) push(nt);
        }
        for (int i = 0; i < ne; i++) {
            int in = (i + 1) % ne;
            link(st.newt(i), 0, st.edge_nt(i), st.edge_ne(i));
            link(st.newt(i), 1, st.newt(in), 2);
        }
    }
    template <class SA, class SB>
    __device__ int add_sup(const SA &A, const SB &B, V<R> d) {
        if (npts >= pts_limit) {
            if (S::PACKED) overflow = true;
            return -1;
        }
        V<R> p = A.get(d), q = B.get(-d);
        int i = npts++;
        st.set_point(i, p - q, p, q);
        return i;
    }
    // an FP64 GJK simplex the polytope starts from
    __device__ void start(const Simplex<R> &sx) {
        pts_limit = S::PTS;
        npts = sx.size;
        nq = ntri = nfree = 0;
        overflow = false;
        for (int k = 0; k < sx.size; k++) st.set_point(k, sx.pts[k].y, sx.pts[k].p, sx.pts[k].q);
    }
    // the GJK simplex the polytope starts from
    __device__ void start(const EpaItem &it, int limit = S::PTS) {
        pts_limit = limit < S::PTS ? limit : S::PTS;
        npts = it.size;
        nq = ntri = nfree = 0;
        overflow = false;
        for (int k = 0; k < it.size; k++) {
            V<R> y{R(it.y[k].x), R(it.y[k].y), R(it.y[k].z)}, p{R(it.p[k].x), R(it.p[k].y), R(it.p[k].z)};
            V<R> q{R(it.q[k].x), R(it.q[k].y), R(it.q[k].z)};
            st.set_point(k, y, p, q);
        }
    }
};

// penetrationDepthStepEPA penetration.ts:214-614, in three parts: the seed polytope
// (epa_seed), the growth until the origin is inside and the expansion towards the closest face
// (epa_loops, or the lock-step rounds of k_epa), and the result from the last face (epa_result).
constexpr R EPA_MAXD = 1.7976931348623157e308;

// the simplex filled to a tetrahedron, its first two triangles and the remaining simplex points
// (penetration.ts:226-345); false when it cannot start
template <class S, class SA, class SB>
__device__ bool epa_seed(Hull<S> &h, const SA &A, const SB &B) {
    if (h.npts == 1) {
        h.npts = 0;
        h.add_sup(A, B, {0.0, 1.0, 0.0});
        h.add_sup(A, B, {-1.0, -1.0, -1.0});
        h.add_sup(A, B, {1.0, -1.0, -1.0});
        h.add_sup(A, B, {0.0, -1.0, 1.0});
    } else if (h.npts == 2) {
        constexpr R C120 = R(-0.4999999999999998), S120 = R(0.8660254037844387), OMC = R(1.4999999999999998);
        V<R> y0 = h.st.Y(0), y1 = h.st.Y(1);
        V<R> ax = y1 - y0;
        R al = sq_root(lsq(ax));
        R nx = ax.x / al, ny = ax.y / al, nz = ax.z / al;
        V<R> d1;
        if (s_abs(nx) > s_abs(ny)) {
            R pl = sq_root(nx * nx + nz * nz);
            d1 = {nz / pl, 0.0, -nx / pl};
        } else {
            R pl = sq_root(ny * ny + nz * nz);
            d1 = {0.0, nz / pl, -ny / pl};
        }
        R r00 = C120 + nx * nx * OMC, r01 = nx * ny * OMC - nz * S120, r02 = nx * nz * OMC + ny * S120;
        R r10 = ny * nx * OMC + nz * S120, r11 = C120 + ny * ny * OMC, r12 = ny * nz * OMC - nx * S120;
        R r20 = nz * nx * OMC - ny * S120, r21 = nz * ny * OMC + nx * S120, r22 = C120 + nz * nz * OMC;
        V<R> d2{r00 * d1.x + r01 * d1.y + r02 * d1.z, r10 * d1.x + r11 * d1.y + r12 * d1.z,
                     r20 * d1.x + r21 * d1.y + r22 * d1.z};
        V<R> d3{r00 * d2.x + r01 * d2.y + r02 * d2.z, r10 * d2.x + r11 * d2.y + r12 * d2.z,
                     r20 * d2.x + r21 * d2.y + r22 * d2.z};
        h.add_sup(A, B, d1);
        h.add_sup(A, B, d2);
        h.add_sup(A, B, d3);
    }
    if (h.npts < 3) return false;
    h.ntri = 0;
    h.nfree = 0;
    h.nq = 0;
    int t1 = h.create(0, 1, 2), t2 = h.create(0, 2, 1);
    if (t1 < 0 || t2 < 0) return false;
    h.link(t1, 0, t2, 2);
    h.link(t1, 1, t2, 1);
    h.link(t1, 2, t2, 0);
    h.push(t1);
    h.push(t2);
    for (int i = 3; i < h.npts; i++) {
        int t = h.find_facing(h.st.Y(i));
        if (t >= 0 && h.add_point(t, i, EPA_MAXD) < 0) return false;
    }
    return true;
}

// the contact from the last face the expansion kept (penetration.ts:509-614)
template <class S>
__device__ bool epa_result(Hull<S> &h, int last, bool flip, V<R> &outAxis, V<R> &outPa, V<R> &outPb) {
    if (h.overflow) return false;
    if (last < 0) return false;
    V<R> ln = h.st.normal(last);
    R nls = lsq(ln);
    V<R> pn = ln * (dot(h.st.centroid(last), ln) / nls);
    if (lsq(pn) < R_MIN_NORMAL_SQ) return false;
    if (flip) pn = -pn;
    R l0, l1;
    bool rel0;
    h.lambdas(last, l0, l1, rel0);
    int s0 = h.st.st(last, 0), s1 = h.st.st(last, 1), s2 = h.st.st(last, 2);
    V<R> xp0 = h.st.P(s0), xp1 = h.st.P(s1), xp2 = h.st.P(s2);
    V<R> xq0 = h.st.Q(s0), xq1 = h.st.Q(s1), xq2 = h.st.Q(s2);
    if (rel0) {
        outPa = xp0 + (xp1 - xp0) * l0 + (xp2 - xp0) * l1;
        outPb = xq0 + (xq1 - xq0) * l0 + (xq2 - xq0) * l1;
    } else {
        outPa = xp1 + (xp0 - xp1) * l0 + (xp2 - xp1) * l1;
        outPb = xq1 + (xq0 - xq1) * l0 + (xq2 - xq1) * l1;
    }
    outAxis = pn;
    return true;
}

// The whole EPA of one pair, sequentially; true and the result on success
template <class S, class SA, class SB>
__device__ bool epa(Hull<S> &h, const SA &A, const SB &B, R tol, V<R> &outAxis,
                    V<R> &outPa, V<R> &outPb) {
    const R MAXD = EPA_MAXD;
    if (!epa_seed(h, A, B)) return false;
    int guard = 0;
    while (guard++ < 4096) {
        if (h.nq == 0) return false;
        int t = h.st.q(0);
        if (h.flags(t) & TF_REMOVED) {
            h.pop();
            if (h.nq == 0) return false;
            h.free_tri(t);
            continue;
        }
        if (h.cls(t) >= 0.0) break;
        h.pop();
        int ni = h.add_sup(A, B, h.st.normal(t));
        if (ni < 0) return false;
        if (!h.facing(t, h.st.Y(ni)) || h.add_point(t, ni, MAXD) < 0) return false;
        h.free_tri(t);
        if (h.nq == 0 || h.npts >= 32) return false;
    }
    R closest = MAXD;
    int last = -1;
    bool flip = false;
    guard = 0;
    do {
        int t = h.pop();
        if (t < 0) return false;
        if (h.flags(t) & TF_REMOVED) {
            h.free_tri(t);
            continue;
        }
        if (h.cls(t) >= closest) break;
        if (last >= 0) h.free_tri(last);
        last = t;
        V<R> tn = h.st.normal(t);
        int ni = h.add_sup(A, B, tn);
        if (ni < 0) break;
        V<R> wv = h.st.Y(ni);
        R d = dot(tn, wv);
        if (d < 0.0) return false;
        R dsq = (d * d) / lsq(tn);
        if (dsq - h.cls(t) < h.cls(t) * tol) break;
        closest = closest < dsq ? closest : dsq;
        if (!h.facing(t, wv)) break;
        int ne = h.add_point(t, ni, closest);
        if (ne < 0) break;
        bool defect = false;
        for (int k = 0; k < ne; k++) {
            int q = h.st.newt(k);
            if (dot(h.st.normal(q), h.st.centroid(q)) < 0.0) {
                defect = true;
                break;
            }
        }
        if (defect) {
            V<R> nn = -tn;
            V<R> w2 = A.get(nn) - B.get(tn);
            if (dot(nn, w2) < d) flip = true;
            break;
        }
    } while (h.nq > 0 && h.npts < 128 && guard++ < 4096);
    return epa_result(h, last, flip, outAxis, outPa, outPb);
}

// The same EPA with the growth and expansion loops cut into rounds that the lanes of a warp run
// together: select a face (pop), one support point, the checks, and the horizon walk with the new
// faces.  Each lane's polytope sees exactly the operations of epa(), in the same order; only the
// facing tests of the horizon walk are taken for every face slot up front (facing_mask), in a loop
// the lanes share, so that the FP64 work issues with most lanes of the warp active (on GB300 an
// FP64 warp instruction costs the same whatever the number of active lanes).
enum : int { EPA_DONE = 0, EPA_GROW = 1, EPA_EXPAND = 2, EPA_FAIL = 3 };
// one lane's EPA in progress: the locals of epa() between its loops
struct EpaLane {
    int phase, gguard, eguard, last;
    R closest;
    bool flip;
    __device__ void begin(bool seeded) {
        phase = seeded ? EPA_GROW : EPA_FAIL;
        gguard = eguard = 0;
        last = -1;
        closest = EPA_MAXD;
        flip = false;
    }
    __device__ bool running() const { return phase == EPA_GROW || phase == EPA_EXPAND; }
};

// The geometry of the new faces of every lane of the warp, spread over the lanes.  Lane l of
// the warp owns ne_l new faces (0 when it has none) whose slots and corners add_point_slots has
// written; the warp's faces are numbered in lane order and lane k computes faces k, k + 32, ...,
// reading the owner's points and writing the owner's face slots in the block's packed store.
// Each face is computed exactly as Hull::create computes it, so the polytopes are bit-identical
// to the one-lane-at-a-time construction.  Returns whether one of the calling lane's own new faces
// failed the defect test.  Every lane of the warp calls it together.
__device__ bool warp_tri_geom(const PackedStore &st, int ne, int ni) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    int incl = ne;
    for (int o = 1; o < 32; o <<= 1) {
        int v = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(FULL, incl, 31);
    const int excl = incl - ne;
    bool defect = false;
    __syncwarp();  // the owners' corners and slots are visible to the lanes that build the faces
    for (int r = 0; r < total; r += 32) {
        const int f = r + lane;
        // the owner of face f: the first lane whose inclusive count is above f
        int owner = 0;
        for (int step = 16; step > 0; step >>= 1) {
            int v = __shfl_sync(FULL, incl, owner + step - 1);
            if (v <= f) owner += step;
        }
        const int o_ne = __shfl_sync(FULL, ne, owner & 31);
        const int o_ex = __shfl_sync(FULL, excl, owner & 31);
        const int o_ni = __shfl_sync(FULL, ni, owner & 31);
        bool d = false;
        if (f < total) {
            PackedStore so = st;
            so.j = (threadIdx.x & ~31) + owner;
            const int i = f - o_ex;
            const int nxt = i + 1 < o_ne ? i + 1 : 0;
            d = tri_geom(so, so.newt(i), so.edge_st(i), so.edge_st(nxt), o_ni);
        }
        const unsigned m = __ballot_sync(FULL, d);
        // this lane's faces among the round's 32
        const int lo = max(excl - r, 0), hi = min(excl + ne - r, 32);
        if (lo < hi) {
            const unsigned bits = (hi - lo == 32 ? FULL : ((1u << (hi - lo)) - 1u)) << lo;
            if (m & bits) defect = true;
        }
    }
    __syncwarp();  // the faces' geometry is visible to their owners
    return defect;
}

// one round of epa()'s growth / expansion loops for the lanes that are running
template <class S, class SA, class SB>
__device__ void epa_round(EpaLane &L, Hull<S> &h, const SA &A, const SB &B, R tol) {
    static_assert(S::TRI <= 64, "the facing mask holds one bit per face slot");
    const R MAXD = EPA_MAXD;
    // select: the face to expand (the loop heads of epa()).  Faces removed by an earlier
    // horizon are popped and dropped here, inside the same round, so that every lane with a
    // polytope left reaches the support and the new faces together.
    bool work = false;
    int t = -1;
    while (!work && (L.phase == EPA_GROW || L.phase == EPA_EXPAND)) {
        if (L.phase == EPA_GROW) {
            if (!(L.gguard++ < 4096)) {
                L.phase = EPA_EXPAND;
            } else if (h.nq == 0) {
                L.phase = EPA_FAIL;
            } else {
                t = h.st.q(0);
                if (h.flags(t) & TF_REMOVED) {
                    h.pop();
                    if (h.nq == 0)
                        L.phase = EPA_FAIL;
                    else
                        h.free_tri(t);
                } else if (order_key(h.cls(t)) >= order_key(0.0)) {
                    L.phase = EPA_EXPAND;
                } else {
                    h.pop();
                    work = true;
                }
            }
        } else {
            t = h.pop();
            if (t < 0) {
                L.phase = EPA_FAIL;
            } else if (h.flags(t) & TF_REMOVED) {
                h.free_tri(t);
                if (!(h.nq > 0 && h.npts < 128 && L.eguard++ < 4096)) L.phase = EPA_DONE;
            } else if (order_key(h.cls(t)) >= order_key(L.closest)) {
                L.phase = EPA_DONE;
            } else {
                if (L.last >= 0) h.free_tri(L.last);
                L.last = t;
                work = true;
            }
        }
    }
    // one support point along the face normal
    V<R> tn{0.0, 0.0, 0.0};
    int ni = -1;
    if (work) {
        tn = h.st.normal(t);
        ni = h.add_sup(A, B, tn);
        if (ni < 0) {
            L.phase = L.phase == EPA_GROW ? EPA_FAIL : EPA_DONE;
            work = false;
        }
    }
    // the checks of the new point
    R d = 0.0;
    if (work) {
        V<R> wv = h.st.Y(ni);
        if (L.phase == EPA_GROW) {
            if (!h.facing(t, wv)) {
                L.phase = EPA_FAIL;
                work = false;
            }
        } else {
            d = dot(tn, wv);
            if (d < 0.0) {
                L.phase = EPA_FAIL;
                work = false;
            } else {
                R dsq = (d * d) / lsq(tn);
                if (dsq - h.cls(t) < h.cls(t) * tol) {
                    L.phase = EPA_DONE;
                    work = false;
                } else {
                    L.closest = L.closest < dsq ? L.closest : dsq;
                    if (!h.facing(t, wv)) {
                        L.phase = EPA_DONE;
                        work = false;
                    }
                }
            }
        }
    }
    // the horizon and the new faces: the slots per lane, the faces' geometry over the warp, then
    // the queue and the links per lane
    int ne = -1;
    if (work) {
        const int upto = __reduce_max_sync(__activemask(), h.ntri);
        const unsigned long long mask = h.facing_mask(h.st.Y(ni), upto);
        ne = h.add_point_slots(t, ni, &mask);
    }
    const bool defect = warp_tri_geom(h.st, ne > 0 ? ne : 0, ni);
    if (work) {
        if (ne >= 0) h.add_point_links(ne, L.phase == EPA_GROW ? MAXD : L.closest);
        if (L.phase == EPA_GROW) {
            if (ne < 0) {
                L.phase = EPA_FAIL;
            } else {
                h.free_tri(t);
                if (h.nq == 0 || h.npts >= 32) L.phase = EPA_FAIL;
            }
        } else if (ne < 0) {
            L.phase = EPA_DONE;
        } else {
            if (defect) {
                V<R> nn = -tn;
                V<R> w2 = A.get(nn) - B.get(tn);
                if (dot(nn, w2) < d) L.flip = true;
                L.phase = EPA_DONE;
            } else if (!(h.nq > 0 && h.npts < 128 && L.eguard++ < 4096)) {
                L.phase = EPA_DONE;
            }
        }
    }
}

// Supports of one queued pair in A's local frame (convex.ts:440-452): EPA runs on the full
// shapes with the speculative distance (at most 1) added to A as a radius.
template <bool H>
__device__ void epa_setup(const DevWorld &w, const EpaItem &it, Sup<R, H> &A, Sup<R, H> &B, R &maxSep) {
    int a = it.a, b = it.b;
    uint32_t fa = w.flags[a], fb = w.flags[b];
    float maxSepF = ((fa | fb) & F_SENSOR) ? 0.f : c_settings.spec_dist;
    maxSep = R(maxSepF < 1.f ? maxSepF : 1.f);
    float3 pa4, pb4;
    float4 qa, qb;
    geom_pose(w, a, fa, pa4, qa);
    geom_pose(w, b, fb, pb4, qb);
    Q<R> iA{R(-qa.x), R(-qa.y), R(-qa.z), R(qa.w)};
    Q<R> qB{R(qb.x), R(qb.y), R(qb.z), R(qb.w)};
    Q<R> rel = qmulS(iA, qB);
    V<R> ab{R(pb4.x) - R(pa4.x), R(pb4.y) - R(pa4.y), R(pb4.z) - R(pa4.z)};
    V<R> posBInA = qrotS(iA, ab);
    A = make_sup<R, H>(shape_of(fa), w.shape[a], false, hull_view(w));
    A.add_r = maxSep;
    B = make_sup<R, H>(shape_of(fb), w.shape[b], false, hull_view(w));
    set_transform(B, rel, posBInA);
}

// a body's convex sub-shapes: a compound's children at their composed poses, or its own shape
struct SubShape {
    int shape;
    float4 sp;
    float3 pos;
    float4 quat;
    uint32_t sub;  // subShape.pushIndex of the child index, 0xffffffff for a body's own shape
};
__device__ __forceinline__ int sub_count(const DevWorld &w, int b, uint32_t f) {
    return shape_of(f) == SHAPE_COMPOUND ? w.compounds[compound_of(w.shape[b])].count : 1;
}
__device__ SubShape sub_shape(const DevWorld &w, int b, uint32_t f, int i) {
    SubShape s;
    geom_pose(w, b, f, s.pos, s.quat);
    if (shape_of(f) != SHAPE_COMPOUND) {
        s.shape = shape_of(f);
        s.sp = w.shape[b];
        s.sub = 0xffffffffu;
        return s;
    }
    const DevCompound &C = w.compounds[compound_of(w.shape[b])];
    const DevChild ch = w.children[C.first + i];
    s.shape = __float_as_int(ch.pos.w);
    s.sp = ch.params;
    s.pos = s.pos + qrot(s.quat, xyz(ch.pos));  // the accumulated transform :520-526
    s.quat = qmul(s.quat, ch.quat);
    s.sub = C.sub_bits >= 32 ? (uint32_t)i : ((0xffffffffu & ~((1u << C.sub_bits) - 1u)) | (uint32_t)i);
    return s;
}
// a mesh triangle's EPA (collideConvexVsTriangleMesh triangle-mesh.ts:1226-1247): A the convex
// body with its radius and the separation, B the triangle's vertices in A's frame
__device__ void epa_setup_mesh(const DevWorld &w, const EpaItem &it, Sup<R> &A, Sup<R, true, true> &B, R &maxSep) {
    int a = it.a, b = it.b;
    uint32_t fa = w.flags[a], fb = w.flags[b];
    float maxSepF = ((fa | fb) & F_SENSOR) ? 0.f : c_settings.spec_dist;
    maxSep = R(maxSepF < 1.f ? maxSepF : 1.f);
    // the convex side: the body's shape, or a compound's child (its index above bit 24)
    const int ti = it.tri & 0xffffff, ci = (it.tri >> 24) - 1;
    const SubShape cs = sub_shape(w, a, fa, ci >= 0 ? ci : 0);
    float3 pb4;
    float4 qb;
    const float3 pa4 = cs.pos;
    const float4 qa = cs.quat;
    geom_pose(w, b, fb, pb4, qb);
    Q<R> iA{R(-qa.x), R(-qa.y), R(-qa.z), R(qa.w)};
    Q<R> rel = qmulS(iA, Q<R>{R(qb.x), R(qb.y), R(qb.z), R(qb.w)});
    V<R> posBInA = qrotS(iA, V<R>{R(pb4.x) - R(pa4.x), R(pb4.y) - R(pa4.y), R(pb4.z) - R(pa4.z)});
    A = make_sup<R>(cs.shape, cs.sp, false, hull_view(w));
    A.add_r = maxSep;
    const int4 t = w.mesh_tris[w.meshes[mesh_of(w.shape[b])].first_tri + ti];
    const int vi[3] = {t.x, t.y, t.z};
    V<R> v[3];
    for (int k = 0; k < 3; k++) {
        float4 m = w.mesh_verts[vi[k]];
        v[k] = posBInA + qrotS(rel, V<R>{R(m.x), R(m.y), R(m.z)});
    }
    B = make_sup<R, true, true>(SHAPE_SPHERE, make_float4(0.f, 0.f, 0.f, 0.f), false, hull_view(w));
    B.kind = SUP_TRIANGLE;
    B.r0 = v[0];
    B.r1 = v[1];
    B.r2 = v[2];
    B.convex_radius = R(0);
}

// The hit of one item (penetrationDepthStepEPA :502-548) written back into the item for
// k_epa_emit: size = 1 with pa in y[0], pb in p[0], axis in q[0] and the depth in pad
// (all in world orientation, relative to A's position), or size = 0 for no contact.
__device__ void epa_finish(const DevWorld &w, EpaItem &it, bool ok, R maxSep, V<R> axis, V<R> pa,
                           V<R> pb) {
    if (!ok) {
        it.size = 0;
        return;
    }
    float3 pa_unused;
    float4 qa;
    geom_pose(w, it.a, w.flags[it.a], pa_unused, qa);
    // mesh items keep the convex body's frame: the mesh pass fixes the normal there
    Q<R> qA = it.tri >= 0 ? Q<R>{R(0), R(0), R(0), R(1)} : Q<R>{R(qa.x), R(qa.y), R(qa.z), R(qa.w)};
    V<R> dd = pa - pb;
    R penetration = sq_root(lsq(dd)) - maxSep;
    R al = sq_root(lsq(axis));
    if (al > 0.0) pa = pa + axis * (-(maxSep / al));
    V<R> paw = qrotS(qA, pa), pbw = qrotS(qA, pb), axw = qrotS(qA, axis);
    it.size = 1;
    it.y[0] = f3((float)(paw.x), (float)(paw.y), (float)(paw.z));
    it.p[0] = f3((float)(pbw.x), (float)(pbw.y), (float)(pbw.z));
    it.q[0] = f3((float)(axw.x), (float)(axw.y), (float)(axw.z));
    it.pad = __float_as_int((float)(penetration));
}

// Packed pass.  fetch_warp = 1: the lanes of a warp run their items in lock-step rounds
// (epa_round), and a lane whose polytope is done writes its result and takes the next item at
// once, so the warp stays full until the queue runs dry; fetch_warp = 0: each thread takes its
// next item as soon as it finishes one and runs it alone (epa).  Items that outgrow the packed
// limits go to the fallback list.
template <bool H>
__device__ __forceinline__ void epa_packed_item(DevWorld &w, EpaItem *items, int i, Hull<PackedStore> &h,
                                                int *fallback, int pts_limit) {
    EpaItem &it = items[i];
    if (it.tri >= 0) return;  // mesh triangles: k_epa_mesh
    Sup<R, H> A, B;
    R maxSep;
    epa_setup(w, it, A, B, maxSep);
    h.start(it, pts_limit);
    V<R> axis, pa, pb;
    bool ok = epa(h, A, B, R(c_settings.penetration_tol), axis, pa, pb);
    if (h.overflow) {
        fallback[atomicAdd(&w.ctr->epa_fallback, 1)] = i;
        return;
    }
    epa_finish(w, it, ok, maxSep, axis, pa, pb);
}

// H: the world has convex hulls (without them the support code leaves the hull loop out)
template <bool H>
__global__ void __launch_bounds__(EPA_BLOCK) k_epa(DevWorld w, EpaItem *items, PackedBlock *blocks,
                                                   int *fallback, int pts_limit, int fetch_warp) {
    int ne = min(w.ctr->num_epa, w.max_epa);
    Hull<PackedStore> h;
    h.st.b = blocks + blockIdx.x;
    h.st.j = threadIdx.x;
    if (!fetch_warp) {
        for (int i = atomicAdd(&w.ctr->epa_cursor, 1); i < ne; i = atomicAdd(&w.ctr->epa_cursor, 1))
            epa_packed_item<H>(w, items, i, h, fallback, pts_limit);
        return;
    }
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const R tol = R(c_settings.penetration_tol);
    int item = -1;           // the item this lane's polytope belongs to
    bool exhausted = false;  // the queue has nothing left for this lane
    EpaLane L;
    L.phase = EPA_DONE;
    Sup<R, H> A, B;
    R maxSep = 0.0;
    while (true) {
        // a lane whose polytope is done writes the result and takes the next item
        const bool idle = !L.running();
        if (idle && item >= 0) {
            V<R> axis{0.0, 0.0, 0.0}, pa{0.0, 0.0, 0.0}, pb{0.0, 0.0, 0.0};
            bool ok = L.phase != EPA_FAIL && epa_result(h, L.last, L.flip, axis, pa, pb);
            if (h.overflow)
                fallback[atomicAdd(&w.ctr->epa_fallback, 1)] = item;
            else
                epa_finish(w, items[item], ok, maxSep, axis, pa, pb);
            item = -1;
        }
        const bool need = idle && !exhausted;
        const unsigned want = __ballot_sync(FULL, need);
        if (want) {
            const int leader = __ffs(want) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(&w.ctr->epa_cursor, __popc(want));
            base = __shfl_sync(FULL, base, leader);
            if (need) {
                const int i = base + __popc(want & below);
                if (i >= ne) {
                    exhausted = true;
                } else if (items[i].tri < 0) {  // mesh triangles: k_epa_mesh
                    item = i;
                    epa_setup(w, items[i], A, B, maxSep);
                    h.start(items[i], pts_limit);
                    L.begin(epa_seed(h, A, B));
                }
            }
        }
        if (!__any_sync(FULL, L.running() || item >= 0 || !exhausted)) break;
        epa_round(L, h, A, B, tol);
    }
}

// Fallback pass with the reference's limits, for the items the packed pass handed over.
template <bool H>
__global__ void __launch_bounds__(EPA_BLOCK) k_epa_big(DevWorld w, EpaItem *items, EpaScratch *scratch,
                                                       const int *fallback) {
    int nf = w.ctr->epa_fallback;
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    Hull<BigStore> h;
    h.st.s = scratch + tid;
    for (int k = tid; k < nf; k += gridDim.x * blockDim.x) {
        EpaItem &it = items[fallback[k]];
        Sup<R, H> A, B;
        R maxSep;
        epa_setup(w, it, A, B, maxSep);
        h.start(it);
        V<R> axis, pa, pb;
        bool ok = epa(h, A, B, R(c_settings.penetration_tol), axis, pa, pb);
        epa_finish(w, it, ok, maxSep, axis, pa, pb);
    }
}

// The mesh triangles' EPA items, with the reference's polytope limits (after the fallback pass,
// whose scratch it reuses)
__global__ void __launch_bounds__(EPA_BLOCK) k_epa_mesh(DevWorld w, EpaItem *items, EpaScratch *scratch) {
    int ne = min(w.ctr->num_epa, w.max_epa);
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    Hull<BigStore> h;
    h.st.s = scratch + tid;
    for (int k = tid; k < ne; k += gridDim.x * blockDim.x) {
        EpaItem &it = items[k];
        if (it.tri < 0) continue;
        Sup<R> A;
        Sup<R, true, true> B;
        R maxSep;
        epa_setup_mesh(w, it, A, B, maxSep);
        h.start(it);
        V<R> axis, pa, pb;
        bool ok = epa(h, A, B, R(c_settings.penetration_tol), axis, pa, pb);
        epa_finish(w, it, ok, maxSep, axis, pa, pb);
    }
}

// Manifolds of the EPA hits (faces, clipping, reduction in FP32), one item per thread.
template <bool HULLS>
__global__ void __launch_bounds__(128) k_epa_emit(DevWorld w, const EpaItem *items) {
    int ne = min(w.ctr->num_epa, w.max_epa);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ne; i += gridDim.x * blockDim.x) {
        const EpaItem &it = items[i];
        if (it.size != 1 || it.tri >= 0) continue;
        bool hull = shape_of(w.flags[it.a]) == SHAPE_HULL || shape_of(w.flags[it.b]) == SHAPE_HULL;
        if (hull != HULLS) continue;
        emit_manifold<HULLS ? 32 : 16>(w, it.a, it.b, it.y[0], it.p[0], it.q[0], __int_as_float(it.pad), true);
    }
}

size_t epa_item_bytes() { return sizeof(EpaItem); }

// ---------------------------------------------------------------------------
// triangle meshes: collideConvexVsTriangleMesh triangle-mesh.ts:1026-1386 and
// collideSphereVsTriangleMesh :1418-1712 into narrowphaseWithReductionCollector
// (update.ts:385-558), one mesh pair per thread
// ---------------------------------------------------------------------------
constexpr int MESH_MAXM = 4;     // manifolds a mesh pair keeps in the first passes
constexpr int MESH_BIG_M = 32;   // the reference's pool (update.ts:358-361), for the pairs that need more
constexpr int MESH_MAXP = 56;    // points of one manifold before its prune (at most 32 + one hit's)
constexpr int MESH_STACK = 64;

template <int M>
struct MeshReduceT {
    int nm;
    float3 normal[M];  // accumulated (unnormalised) normals
    float depth[M];
    uint32_t sub_a[M], sub_b[M];
    PtsN<MESH_MAXP> pts[M];
    bool dropped;  // a new normal group arrived with every slot taken
};
using MeshReduce = MeshReduceT<MESH_MAXM>;
size_t mesh_big_slot_bytes() { return sizeof(MeshReduceT<MESH_BIG_M>); }

// addHit update.ts:385-519 (points relative to the base, the narrowphase's body A)
template <int N, int M>
__device__ void mesh_add_hit(MeshReduceT<M> &r, float3 pa, float3 pb, float3 axis, float penetration, uint32_t sa,
                             uint32_t sb, const FaceN<N> &fA, const FaceN<N> &fB) {
    const float3 n = normalize3(axis);
    int m = -1;
    for (int i = 0; i < r.nm; i++)
        if (dot3(n, r.normal[i]) >= c_settings.normal_cos) {
            m = i;
            break;
        }
    if (m < 0) {
        if (r.nm >= M) {
            // pool full: the shallowest manifold makes way for a deeper hit
            int sh = 0;
            for (int i = 1; i < r.nm; i++)
                if (r.depth[i] < r.depth[sh]) sh = i;
            r.dropped = true;
            if (penetration < r.depth[sh]) return;
            m = sh;
        } else {
            m = r.nm++;
        }
        r.pts[m].n = 0;
        r.normal[m] = n;
        r.depth[m] = penetration;
        r.sub_a[m] = sa;
        r.sub_b[m] = sb;
    } else {
        r.normal[m] = r.normal[m] + n;
    }
    PtsN<N> tmp;
    const float maxd = c_settings.spec_dist + c_settings.manifold_tol;
    if (fA.n >= 2 && fB.n >= 3) {
        manifold_faces(tmp, pa, pb, axis, maxd, fA, fB);
    } else {
        tmp.n = 1;
        tmp.a[0] = pa;
        tmp.b[0] = pb;
    }
    PtsN<MESH_MAXP> &P = r.pts[m];
    for (int i = 0; i < tmp.n && P.n < 64 && P.n < MESH_MAXP; i++) {
        P.a[P.n] = tmp.a[i];
        P.b[P.n] = tmp.b[i];
        P.n++;
    }
    if (penetration > r.depth[m]) r.depth[m] = penetration;
    if (P.n > 32) prune(P, r.normal[m]);
}

// finalizeAndCreateConstraints update.ts:525-558: the manifolds into the contact pipeline
template <int M>
__device__ void mesh_emit(DevWorld &w, MeshReduceT<M> &r, int a, int b, float3 base) {
    for (int i = 0; i < r.nm; i++) {
        PtsN<MESH_MAXP> &P = r.pts[i];
        float3 nrm = normalize3(r.normal[i]);
        if (P.n > 4) prune(P, nrm);
        if (P.n <= 0) continue;
        int slot = atomicAdd(&w.ctr->num_manifolds, 1);
        if (slot >= w.max_manifolds) {
            atomicOr(&w.ctr->overflow, OVF_MANIFOLDS);
            return;
        }
        Manifold m;
        m.a = a;
        m.b = b;
        m.n = P.n;
        m.base = base;
        m.normal = nrm;
        m.depth = r.depth[i];
        for (int k = 0; k < 4; k++) {
            m.ra[k] = k < P.n ? P.a[k] : f3(0.f, 0.f, 0.f);
            m.rb[k] = k < P.n ? P.b[k] : f3(0.f, 0.f, 0.f);
        }
        m.sub_a = r.sub_a[i];
        m.sub_b = r.sub_b[i];
        w.manifolds[slot] = m;
    }
    if (r.dropped) atomicAdd(&w.ctr->mesh_reduced, 1);
}

// fixNormal active-edges.ts:74-153 (shape A's frame, the point relative to A)
__device__ float3 fix_normal(float3 v0, float3 v1, float3 v2, float3 tn, int active, float3 point, float3 normal,
                             float3 move) {
    if (active == 0b111) return normal;
    const float nl = sqrtf(lensq3(normal)), tl = sqrtf(lensq3(tn));
    if (dot3(move, normal) * tl < dot3(move, tn) * nl) return normal;
    if (active == 0) return tn;
    if (dot3(tn, normal) > 0.999848f * nl * tl) return normal;  // within 1 degree
    Bary<float> bc = bary3(V<float>{v0.x - point.x, v0.y - point.y, v0.z - point.z},
                           V<float>{v1.x - point.x, v1.y - point.y, v1.z - point.z},
                           V<float>{v2.x - point.x, v2.y - point.y, v2.z - point.z}, 1e-10f);
    const float E = 1.0e-4f, OME = 1.0f - 1.0e-4f;
    int edge;
    if (bc.u > OME)
        edge = 0b101;
    else if (bc.v > OME)
        edge = 0b011;
    else if (bc.w > OME)
        edge = 0b110;
    else if (bc.u < E)
        edge = 0b010;
    else if (bc.v < E)
        edge = 0b100;
    else if (bc.w < E)
        edge = 0b001;
    else
        return tn;
    return (active & edge) ? normal : tn;
}

// getClosestPointOnTriangle triangle.ts:62-197 (the query point at the origin); feature bits
// A 1, B 2, C 4, edges their vertex pairs, the face 7
__device__ float3 closest_on_triangle(float3 a, float3 b, float3 c, float &dsq, int &feature) {
    float3 ab = b - a, ac = c - a;
    float3 n = cross3(ab, ac);
    float nl2 = lensq3(n);
    if (nl2 < 1e-10f) {
        // degenerate: the nearest of the vertices and edges (handleDegenerateTriangle :199-287)
        float3 best = c;
        feature = 0b100;
        float bd = lensq3(c);
        if (lensq3(a) < bd) {
            best = a, bd = lensq3(a), feature = 0b001;
        }
        if (lensq3(b) < bd) {
            best = b, bd = lensq3(b), feature = 0b010;
        }
        const float EPS2 = 1.1920929e-7f * 1.1920929e-7f;
        auto edge = [&](float3 p, float3 e, int f) {
            float el = lensq3(e);
            if (el > EPS2) {
                float v = fmaxf(0.f, fminf(1.f, -dot3(p, e) / el));
                float3 q = p + e * v;
                float d = lensq3(q);
                if (d < bd) best = q, bd = d, feature = f;
            }
        };
        edge(a, ac, 0b101);
        edge(b, c - b, 0b110);
        edge(a, ab, 0b011);
        dsq = bd;
        return best;
    }
    float d1 = -dot3(ab, a), d2 = -dot3(ac, a);
    if (d1 <= 0.f && d2 <= 0.f) {
        dsq = lensq3(a), feature = 0b001;
        return a;
    }
    float d3 = -dot3(ab, b), d4 = -dot3(ac, b);
    if (d3 >= 0.f && d4 <= d3) {
        dsq = lensq3(b), feature = 0b010;
        return b;
    }
    if (d1 * d4 <= d3 * d2 && d1 >= 0.f && d3 <= 0.f) {
        float v = d1 / (d1 - d3);
        float3 p = a + ab * v;
        dsq = lensq3(p), feature = 0b011;
        return p;
    }
    float d5 = -dot3(ab, c), d6 = -dot3(ac, c);
    if (d6 >= 0.f && d5 <= d6) {
        dsq = lensq3(c), feature = 0b100;
        return c;
    }
    if (d5 * d2 <= d1 * d6 && d2 >= 0.f && d6 <= 0.f) {
        float v = d2 / (d2 - d6);
        float3 p = a + ac * v;
        dsq = lensq3(p), feature = 0b101;
        return p;
    }
    float d43 = d4 - d3, d56 = d5 - d6;
    if (d3 * d6 <= d5 * d4 && d43 >= 0.f && d56 >= 0.f) {
        float v = d43 / (d43 + d56);
        float3 p = b + (c - b) * v;
        dsq = lensq3(p), feature = 0b110;
        return p;
    }
    float sc = dot3(a + b + c, n) / (3.f * nl2);
    float3 p = n * sc;
    dsq = lensq3(p), feature = 0b111;
    return p;
}

__device__ __forceinline__ bool node_hits_box(const float4 &lo, const float4 &hi, float3 qlo, float3 qhi) {
    return lo.x <= qhi.x && hi.x >= qlo.x && lo.y <= qhi.y && hi.y >= qlo.y && lo.z <= qhi.z && hi.z >= qlo.z;
}

// the convex shape's local bounds (box.ts:77-84, sphere, capsule.ts:84-94, convex-hull.ts:214-231)
__device__ void convex_local_bounds(const DevWorld &w, uint32_t f, float4 sp, float3 &lo, float3 &hi) {
    int s = shape_of(f);
    if (s == SHAPE_HULL) {
        const DevHull &h = w.hulls[hull_of(sp)];
        lo = xyz(h.lo);
        hi = xyz(h.hi);
    } else if (s == SHAPE_BOX) {
        lo = f3(-sp.x, -sp.y, -sp.z);
        hi = f3(sp.x, sp.y, sp.z);
    } else if (s == SHAPE_CAPSULE) {
        lo = f3(-sp.x, -(sp.y + sp.x), -sp.x);
        hi = f3(sp.x, sp.y + sp.x, sp.x);
    } else if (s == SHAPE_CYLINDER) {
        lo = f3(-sp.y, -sp.x, -sp.y);
        hi = f3(sp.y, sp.x, sp.y);
    } else {
        lo = f3(-sp.x, -sp.x, -sp.x);
        hi = f3(sp.x, sp.x, sp.x);
    }
}
// |size| of a convex leaf's local bounds (box3.size + vec3.length, plane.ts:680-681)
__device__ float convex_bounds_size(const DevWorld &w, uint32_t f, float4 sp) {
    float3 lo, hi;
    convex_local_bounds(w, f, sp, lo, hi);
    return sqrtf(lensq3(hi - lo));
}

// One mesh pair k.  PASS 0: pairs with no triangle in need of EPA are reduced and emitted; a
// pair with some reserves one EPA item per such triangle, in traversal order, and waits.
// PASS 1 (after the EPA passes): those pairs again, each such triangle taking its item.
// PASS 2: a pair whose hits wanted more than the 4 manifolds of the first passes' pool, again
// with the reference's pool of 32 (red in global memory) and its EPA items, if it has some.
// A pair of the first passes that overflows its pool is handed to PASS 2 instead of emitted.
template <int PASS, int M>
__device__ void mesh_pair(DevWorld &w, EpaItem *epa_items, int k, MeshReduceT<M> &red) {
    {
        if (PASS == 1 && w.mesh_epa_base[k] < 0) return;
        int2 pr = w.pairs[w.mesh_pairs[k]];
        int a = pr.x, b = pr.y;
        uint32_t fa = w.flags[a], fb = w.flags[b];
        int ma = motion_of(fa), mb = motion_of(fb);
        if (ma > mb || (ma == mb && b < a)) {  // narrowphase order (update.ts:74)
            int t = a;
            a = b;
            b = t;
            uint32_t tf = fa;
            fa = fb;
            fb = tf;
        }
        if (PASS == 0) w.mesh_epa_base[k] = -1;
        const bool meshA = shape_of(fa) == SHAPE_MESH, meshB = shape_of(fb) == SHAPE_MESH;
        if (meshA == meshB) return;  // mesh against mesh: no collide function (triangle-mesh.ts:223-237)
        // collideTriangleMeshVsConvex = the convex-vs-mesh function with the hit reversed
        // (reversedCollideShapeVsShape collide-shape-vs-shape.ts:227-354)
        const bool inverted = meshA;
        const int cv = inverted ? b : a, mh = inverted ? a : b;
        const uint32_t fcb = inverted ? fb : fa;  // the convex body's flags
        float3 base, pm;
        float4 qbase, qm4;
        geom_pose(w, a, fa, base, qbase);
        const float maxSepIn = ((fa | fb) & F_SENSOR) ? 0.f : c_settings.spec_dist;
        geom_pose(w, mh, w.flags[mh], pm, qm4);
        const Q<float> qM{qm4.x, qm4.y, qm4.z, qm4.w}, iqM{-qm4.x, -qm4.y, -qm4.z, qm4.w};
        const DevMesh &M = w.meshes[mesh_of(w.shape[mh])];
        // activeEdgeMovementDirection: A's velocity minus B's in the narrowphase order (update.ts:729-733)
        const float3 moveW = xyz(w.linvel[a]) - xyz(w.linvel[b]);
        // a compound collides child by child (collideCompoundVsShape compound.ts:494-578)
        const bool compound = shape_of(fcb) == SHAPE_COMPOUND;
        const int ncv = sub_count(w, cv, fcb);
        red.nm = 0;
        red.dropped = false;
        int epa_needed = 0, epa_next = 0;
        const int epa_base = PASS >= 1 ? w.mesh_epa_base[k] : -1;
        const int epa_count = PASS >= 1 ? w.mesh_epa_count[k] : 0;
        for (int round = 0; round < 2; round++) {  // PASS 0 runs a second round to fill the EPA items
            if (round == 1 && (PASS >= 1 || epa_needed == 0)) break;
            int reserve = -1;
            if (round == 1) {
                // the whole block or nothing: the EPA passes read every item below min(num_epa, max_epa)
                int cur = *(volatile int *)&w.ctr->num_epa;
                for (int guard = 0; guard < (1 << 20); guard++) {
                    if (cur + epa_needed > w.max_epa) break;
                    int prev = atomicCAS(&w.ctr->num_epa, cur, cur + epa_needed);
                    if (prev == cur) {
                        reserve = cur;
                        break;
                    }
                    cur = prev;
                }
                if (reserve < 0) {
                    atomicOr(&w.ctr->overflow, OVF_EPA);
                    break;
                }
                w.mesh_epa_base[k] = reserve;
                w.mesh_epa_count[k] = epa_needed;
                epa_next = 0;
            }
            for (int ci = 0; ci < ncv; ci++) {
            const SubShape csub = sub_shape(w, cv, fcb, ci);
            const uint32_t fc = shape_bits(csub.shape);
            const float3 pc = csub.pos;
            const float4 qc4 = csub.quat;
            const float3 cvRel = pc - base;  // the convex shape's position relative to the base
            const Q<float> qC{qc4.x, qc4.y, qc4.z, qc4.w}, iqC{-qc4.x, -qc4.y, -qc4.z, qc4.w};
            // mesh into the convex shape's frame, and the convex shape into the mesh's frame
            const Q<float> m2c = qmulS(iqC, qM);
            const V<float> m2cPos = qrotS(iqC, V<float>{pm.x - pc.x, pm.y - pc.y, pm.z - pc.z});
            const Q<float> cInM = qmulS(iqM, qC);
            const V<float> cInMPos = qrotS(iqM, V<float>{pc.x - pm.x, pc.y - pm.y, pc.z - pm.z});
            const float4 sc = csub.sp;
            const bool sphere = csub.shape == SHAPE_SPHERE;
            // query bounds in the mesh frame and the traversal's reference point
            float3 qlo, qhi, qcenter, blo1, bhi1;
            V<float> sphereC{0.f, 0.f, 0.f};
            if (sphere) {
                sphereC = cInMPos;
                const float er = sc.x + maxSepIn;
                qlo = f3(sphereC.x - er, sphereC.y - er, sphereC.z - er);
                qhi = f3(sphereC.x + er, sphereC.y + er, sphereC.z + er);
                qcenter = f3(sphereC.x, sphereC.y, sphereC.z);
            } else {
                float3 llo, lhi;
                convex_local_bounds(w, fc, sc, llo, lhi);
                blo1 = llo - f3(maxSepIn, maxSepIn, maxSepIn);
                bhi1 = lhi + f3(maxSepIn, maxSepIn, maxSepIn);
                // box3.transformMat4 of the local bounds (8 corners), grown by the separation
                qlo = f3(3.0e38f, 3.0e38f, 3.0e38f);
                qhi = f3(-3.0e38f, -3.0e38f, -3.0e38f);
                for (int c = 0; c < 8; c++) {
                    V<float> p{(c & 1) ? lhi.x : llo.x, (c & 2) ? lhi.y : llo.y, (c & 4) ? lhi.z : llo.z};
                    V<float> q = qrotS(cInM, p) + cInMPos;
                    qlo = f3(fminf(qlo.x, q.x), fminf(qlo.y, q.y), fminf(qlo.z, q.z));
                    qhi = f3(fmaxf(qhi.x, q.x), fmaxf(qhi.y, q.y), fmaxf(qhi.z, q.z));
                }
                qlo = qlo - f3(maxSepIn, maxSepIn, maxSepIn);
                qhi = qhi + f3(maxSepIn, maxSepIn, maxSepIn);
                qcenter = (qlo + qhi) * 0.5f;
            }
            const HullView hv = hull_view(w);
            Sup<float> supA;
            if (!sphere) supA = make_sup<float>(shape_of(fc), sc, true, hv);
            int stack[MESH_STACK];
            int sp = 0;
            stack[sp++] = 0;
            while (sp > 0) {
                const int node = stack[--sp];
                const float4 nlo = w.mesh_nodes[2 * (M.first_node + node)], nhi = w.mesh_nodes[2 * (M.first_node + node) + 1];
                if (!node_hits_box(nlo, nhi, qlo, qhi)) continue;
                const int aux = __float_as_int(nlo.w), tag = __float_as_int(nhi.w);
                if (tag >= 0) {
                    // internal: the nearer child (centre to centre) is visited first
                    const int left = node + 1, right = aux;
                    float4 l0 = w.mesh_nodes[2 * (M.first_node + left)], l1 = w.mesh_nodes[2 * (M.first_node + left) + 1];
                    float4 r0 = w.mesh_nodes[2 * (M.first_node + right)], r1 = w.mesh_nodes[2 * (M.first_node + right) + 1];
                    float ld = lensq3(qcenter - (xyz(l0) + xyz(l1)) * 0.5f);
                    float rd = lensq3(qcenter - (xyz(r0) + xyz(r1)) * 0.5f);
                    if (sp + 2 > MESH_STACK) {
                        atomicOr(&w.ctr->overflow, OVF_SLOTS);
                        continue;
                    }
                    if (ld <= rd) {
                        stack[sp++] = right;
                        stack[sp++] = left;
                    } else {
                        stack[sp++] = left;
                        stack[sp++] = right;
                    }
                    continue;
                }
                const int tcount = -tag - 1;
                for (int ti = aux; ti < aux + tcount; ti++) {
                    const int4 tr = w.mesh_tris[M.first_tri + ti];
                    const float3 m0 = xyz(w.mesh_verts[tr.x]), m1 = xyz(w.mesh_verts[tr.y]), m2 = xyz(w.mesh_verts[tr.z]);
                    const uint32_t tsub = M.sub_bits >= 32 ? (uint32_t)ti
                                                           : ((0xffffffffu & ~((1u << M.sub_bits) - 1u)) | (uint32_t)ti);
                    float3 hpa, hpb, hax;  // hit in the convex-first order, relative to the base
                    float hpen;
                    FaceN<32> fConvex, fTri;
                    fConvex.n = 0;
                    fTri.n = 0;
                    if (sphere) {
                        // collideSphereVsTriangleMesh triangle-mesh.ts:1510-1646, in the mesh frame
                        const float r = sc.x;
                        const float3 c = f3(sphereC.x, sphereC.y, sphereC.z);
                        const float3 v0 = m0 - c, v1 = m1 - c, v2 = m2 - c;
                        const float3 tn = cross3(v1 - v0, v2 - v0);
                        const bool back = dot3(tn, v0) > 0.f;
                        if (back) continue;
                        float dsq;
                        int feature;
                        float3 p2 = closest_on_triangle(v0, v1, v2, dsq, feature);
                        if (dsq > (r + maxSepIn) * (r + maxSepIn)) continue;
                        hpen = r - sqrtf(dsq);
                        float3 ax = dsq > 0.f ? normalize3(p2) : f3(0.f, 1.f, 0.f);
                        const float3 p1 = ax * r;
                        const int feat_edges[8] = {0b000, 0b101, 0b011, 0b001, 0b110, 0b100, 0b010, 0b000};
                        if (feature != 0b111 && tr.w != 0b111 && (tr.w & feat_edges[feature]) == 0) {
                            const V<float> mv = qrotS(iqM, V<float>{moveW.x, moveW.y, moveW.z});
                            const float3 mvm = f3(mv.x, mv.y, mv.z);
                            const float3 nax = back ? tn : -tn;
                            if (dot3(mvm, ax) * sqrtf(lensq3(nax)) >= dot3(mvm, nax)) ax = nax;
                        }
                        auto to_base = [&](float3 v) {
                            V<float> q = qrotS(qM, V<float>{v.x, v.y, v.z});
                            return f3(q.x, q.y, q.z) + (pm - base);
                        };
                        hpa = to_base(c + p1);
                        hpb = to_base(c + p2);
                        V<float> aw = qrotS(qM, V<float>{ax.x, ax.y, ax.z});
                        hax = f3(aw.x, aw.y, aw.z);
                        fTri.n = 3;
                        fTri.v[0] = to_base(m0);
                        fTri.v[1] = to_base(m1);
                        fTri.v[2] = to_base(m2);
                    } else {
                        // collideConvexVsTriangleMesh triangle-mesh.ts:1140-1386, in the convex body's frame
                        auto to_c = [&](float3 v) {
                            V<float> q = qrotS(m2c, V<float>{v.x, v.y, v.z}) + m2cPos;
                            return f3(q.x, q.y, q.z);
                        };
                        const float3 t0 = to_c(m0), t1 = to_c(m1), t2 = to_c(m2);
                        const float3 tlo = f3(fminf(t0.x, fminf(t1.x, t2.x)), fminf(t0.y, fminf(t1.y, t2.y)),
                                              fminf(t0.z, fminf(t1.z, t2.z)));
                        const float3 thi = f3(fmaxf(t0.x, fmaxf(t1.x, t2.x)), fmaxf(t0.y, fmaxf(t1.y, t2.y)),
                                              fmaxf(t0.z, fmaxf(t1.z, t2.z)));
                        if (!(tlo.x <= bhi1.x && thi.x >= blo1.x && tlo.y <= bhi1.y && thi.y >= blo1.y &&
                              tlo.z <= bhi1.z && thi.z >= blo1.z))
                            continue;
                        const float3 tn = cross3(t1 - t0, t2 - t0);
                        if (dot3(tn, t0) > 0.f) continue;  // back facing
                        Sup<float, true, true> supT =
                            make_sup<float, true, true>(SHAPE_SPHERE, make_float4(0.f, 0.f, 0.f, 0.f), false, hv);
                        supT.kind = SUP_TRIANGLE;
                        supT.r0 = V<float>{t0.x, t0.y, t0.z};
                        supT.r1 = V<float>{t1.x, t1.y, t1.z};
                        supT.r2 = V<float>{t2.x, t2.y, t2.z};
                        supT.convex_radius = 0.f;
                        V<float> axis{-tn.x, -tn.y, -tn.z};
                        if (lsq(axis) < 1e-10f)
                            axis = {1.f, 0.f, 0.f};
                        else
                            axis = axis * (1.f / sq_root(lsq(axis)));
                        float maxSep = maxSepIn;
                        const float rA = supA.convex_radius + maxSep;
                        Simplex<float> sx;
                        GjkOut<float> g = gjk(supA, supT, c_settings.collision_tol, axis, rA * rA, sx);
                        if (g.sqdist > rA * rA) continue;  // NOT_COLLIDING
                        V<float> pa, pb, pax;
                        if (!(g.sqdist > 0.f)) {
                            // INDETERMINATE: EPA in FP64 (penetrationDepthStepEPA) through the EPA passes
                            maxSep = fminf(maxSep, 1.f);
                            if (PASS == 0) {
                                if (round == 0) {
                                    epa_needed++;
                                    continue;
                                }
                                EpaItem it;
                                it.a = cv;
                                it.b = mh;
                                it.tri = compound ? (ti | ((ci + 1) << 24)) : ti;  // a child's: its index above bit 24
                                it.size = sx.size;
                                it.pad = 0;
                                for (int q = 0; q < 4; q++) {
                                    SP<float> s = sx.pts[q < sx.size ? q : 0];
                                    it.y[q] = f3(s.y.x, s.y.y, s.y.z);
                                    it.p[q] = f3(s.p.x, s.p.y, s.p.z);
                                    it.q[q] = f3(s.q.x, s.q.y, s.q.z);
                                }
                                if (epa_next < epa_needed) epa_items[reserve + epa_next++] = it;
                                continue;
                            }
                            if (epa_next >= epa_count) continue;
                            const EpaItem &it = epa_items[epa_base + epa_next++];
                            if (it.size != 1) continue;  // EPA found no contact
                            pa = V<float>{it.y[0].x, it.y[0].y, it.y[0].z};
                            pb = V<float>{it.p[0].x, it.p[0].y, it.p[0].z};
                            pax = V<float>{it.q[0].x, it.q[0].y, it.q[0].z};
                            hpen = __int_as_float(it.pad);
                        } else {
                            if (PASS == 0 && round == 1) continue;  // only the EPA items are filled
                            // COLLIDING: penetrationDepthStepGJK penetration.ts:84-106
                            const float vl = sqrtf(g.sqdist);
                            pa = g.pa + g.axis * (rA / vl);
                            pb = g.pb;
                            pax = g.axis;
                            V<float> dd = pa - pb;
                            hpen = sqrtf(lsq(dd)) - maxSep;
                            const float al = sqrtf(lsq(pax));
                            if (al > 0.f) pa = pa + pax * (-(maxSep / al));
                        }
                        if (PASS == 0 && round == 1) continue;
                        if (tr.w != 0b111) {  // active edges: fixNormal
                            const V<float> mv = qrotS(iqC, V<float>{moveW.x, moveW.y, moveW.z});
                            float3 fixed = fix_normal(t0, t1, t2, -tn, tr.w, f3(pb.x, pb.y, pb.z),
                                                      f3(pax.x, pax.y, pax.z), f3(mv.x, mv.y, mv.z));
                            pax = V<float>{fixed.x, fixed.y, fixed.z};
                        }
                        auto to_base = [&](V<float> v) {
                            V<float> q = qrotS(qC, v);
                            return f3(q.x, q.y, q.z) + cvRel;
                        };
                        hpa = to_base(pa);
                        hpb = to_base(pb);
                        V<float> aw = qrotS(qC, pax);
                        hax = f3(aw.x, aw.y, aw.z);
                        // supporting faces: the convex shape's along -axis, the triangle
                        const float3 axl = f3(pax.x, pax.y, pax.z);
                        const int s = shape_of(fc);
                        if (s == SHAPE_BOX) box_face(fConvex, -axl, sc, qc4, cvRel);
                        if (s == SHAPE_CAPSULE) capsule_face(fConvex, -axl, sc, qc4, cvRel);
                        if (s == SHAPE_HULL) hull_face(fConvex, -axl, w, sc, qc4, cvRel);
                        if (s == SHAPE_CYLINDER) cylinder_face(fConvex, -axl, sc, qc4, cvRel);
                        fTri.n = 3;
                        fTri.v[0] = to_base(V<float>{t0.x, t0.y, t0.z});
                        fTri.v[1] = to_base(V<float>{t1.x, t1.y, t1.z});
                        fTri.v[2] = to_base(V<float>{t2.x, t2.y, t2.z});
                    }
                    if (PASS != 2) atomicAdd(&w.ctr->num_mesh_hits, 1);
                    if (inverted)  // the inverted collector: points, axis, sub-shape ids and faces swapped
                        mesh_add_hit(red, hpb, hpa, -hax, hpen, tsub, csub.sub, fTri, fConvex);
                    else
                        mesh_add_hit(red, hpa, hpb, hax, hpen, csub.sub, tsub, fConvex, fTri);
                }
            }
            }  // children
        }
        if (PASS == 0 && epa_needed > 0) return;  // finished by the second pass
        if (PASS != 2 && red.dropped && w.mesh_big) {  // the pool overflowed: the 32-manifold pass takes it
            const int o = atomicAdd(&w.ctr->num_mesh_big, 1);
            if (o < w.max_pairs) {
                w.mesh_big[o] = k;
                return;
            }
        }
        mesh_emit(w, red, a, b, base);
    }
}

template <int PASS>
__global__ void __launch_bounds__(64) k_mesh_narrowphase(DevWorld w, EpaItem *epa_items) {
    const int npairs = min(w.ctr->num_mesh_pairs, w.max_pairs);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < npairs; k += gridDim.x * blockDim.x) {
        MeshReduce red;
        mesh_pair<PASS, MESH_MAXM>(w, epa_items, k, red);
    }
}
// the pairs whose hits overflowed the 4-manifold pool, with the reference's 32 (one global slot
// per thread)
__global__ void __launch_bounds__(64) k_mesh_big(DevWorld w, EpaItem *epa_items) {
    const int nbig = min(w.ctr->num_mesh_big, w.max_pairs);
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    MeshReduceT<MESH_BIG_M> &red = ((MeshReduceT<MESH_BIG_M> *)w.mesh_big_red)[tid];
    for (int j = tid; j < nbig; j += gridDim.x * blockDim.x) mesh_pair<2, MESH_BIG_M>(w, epa_items, w.mesh_big[j], red);
}


// ---------------------------------------------------------------------------
// compound pairs (compound.ts collideCompoundVsShape / collideShapeVsCompound :494-678): the
// sub-shapes of each body (a compound's children at their composed poses, or the body's own
// convex shape) collided pairwise, A's first, every hit into the reduction pool
// ---------------------------------------------------------------------------
// the supporting face of a convex sub-shape along a world direction, relative to the base
template <int N>
__device__ void sub_face(FaceN<N> &f, const DevWorld &w, const SubShape &s, float3 dir, float3 base) {
    const float3 d = qrot_inv(s.quat, dir), t = s.pos - base;
    if (s.shape == SHAPE_BOX) box_face(f, d, s.sp, s.quat, t);
    if (s.shape == SHAPE_CAPSULE) capsule_face(f, d, s.sp, s.quat, t);
    if (s.shape == SHAPE_HULL) hull_face(f, d, w, s.sp, s.quat, t);
    if (s.shape == SHAPE_CYLINDER) cylinder_face(f, d, s.sp, s.quat, t);
}
// collideShapeVsShape (narrowphase.ts:172-238) of two sub-shapes, one of them possibly a plane:
// the hit, relative to the base, with both supporting faces into the pool (EPA in FP64 on the
// thread's polytope, from the FP32 GJK simplex as the narrowphase's EPA starts)
template <int M>
__device__ void collide_sub(const DevWorld &w, const HullView &hv, EpaScratch *slot, const SubShape &A,
                            const SubShape &B, float maxSep, float3 base, MeshReduceT<M> &red) {
    if (A.shape == SHAPE_EMPTY || B.shape == SHAPE_EMPTY) return;
    if (A.shape == SHAPE_PLANE && B.shape == SHAPE_PLANE) return;
    FaceN<32> fA, fB;
    fA.n = fB.n = 0;
    float3 pa, pb, ax;
    float pen;
    if (A.shape == SHAPE_PLANE || B.shape == SHAPE_PLANE) {  // collideConvexVsPlane plane.ts:474-629
        const bool planeA = A.shape == SHAPE_PLANE;
        const SubShape &Cv = planeA ? B : A, &P = planeA ? A : B;
        const float3 nl = qrot_inv(Cv.quat, qrot(P.quat, xyz(P.sp)));
        const float cl = P.sp.w - dot3(qrot_inv(Cv.quat, P.pos - Cv.pos), nl);
        const Sup<float> S = make_sup<float>(Cv.shape, Cv.sp, default_excludes(Cv.shape), hv);
        const V<float> spv = S.get(V<float>{-nl.x, -nl.y, -nl.z});
        const float3 sp3 = f3(spv.x, spv.y, spv.z);
        const float sd = dot3(nl, sp3) + cl, cr = S.convex_radius;
        pen = -sd + cr;
        if (!(pen > -maxSep)) return;
        const float3 p1 = Cv.pos + qrot(Cv.quat, sp3 - nl * cr), p2 = Cv.pos + qrot(Cv.quat, sp3 - nl * sd);
        const float3 axc = qrot(Cv.quat, -nl);  // from the convex shape into the plane
        pa = planeA ? p2 : p1;
        pb = planeA ? p1 : p2;
        ax = planeA ? -axc : axc;
        // the convex face, then the plane's square under it (plane.ts:588-606)
        float3 llo, lhi;
        convex_local_bounds(w, shape_bits(Cv.shape), Cv.sp, llo, lhi);
        const float size = sqrtf(lensq3(lhi - llo));
        float3 nw;
        float cw;
        plane_world(P.sp, P.pos, P.quat, nw, cw);
        if (planeA) {
            sub_face(fB, w, B, ax, base);
            if (fB.n > 0) plane_face(fA, nw, cw, B.pos, size, base);
        } else {
            sub_face(fA, w, A, -ax, base);
            if (fA.n > 0) plane_face(fB, nw, cw, A.pos, size, base);
        }
    } else if (A.shape == SHAPE_SPHERE && B.shape == SHAPE_SPHERE) {  // collideSphereVsSphere sphere.ts:319-410
        const float3 d = B.pos - A.pos;
        const float dsq = lensq3(d), rs = A.sp.x + B.sp.x;
        if (dsq >= rs * rs) return;
        const float dist = sqrtf(dsq);
        const float3 nn = dist > 0.f ? d * (1.f / dist) : f3(0.f, 1.f, 0.f);
        pa = A.pos + nn * A.sp.x;
        pb = B.pos - nn * B.sp.x;
        ax = nn;
        pen = rs - dist;
    } else {  // collideConvexVsConvex convex.ts:257-641: B in A's frame
        const Q<float> qA{A.quat.x, A.quat.y, A.quat.z, A.quat.w}, iA{-A.quat.x, -A.quat.y, -A.quat.z, A.quat.w};
        const Q<float> rel = qmulS(iA, Q<float>{B.quat.x, B.quat.y, B.quat.z, B.quat.w});
        const V<float> posBInA = qrotS(iA, V<float>{B.pos.x - A.pos.x, B.pos.y - A.pos.y, B.pos.z - A.pos.z});
        const Sup<float> supA = make_sup<float>(A.shape, A.sp, true, hv);
        Sup<float> supB = make_sup<float>(B.shape, B.sp, true, hv);
        set_transform(supB, rel, posBInA);
        V<float> axis = posBInA;
        if (lsq(axis) <= 1e-12f) axis = {1.f, 0.f, 0.f};
        const float rA = supA.convex_radius + maxSep, rB = supB.convex_radius, cr = rA + rB;
        Simplex<float> sx;
        const GjkOut<float> g = gjk(supA, supB, c_settings.collision_tol, axis, cr * cr, sx);
        if (g.sqdist > cr * cr) return;  // NOT_COLLIDING
        V<float> lpa, lpb, lax;
        if (!(g.sqdist > 0.f)) {  // INDETERMINATE: EPA in FP64 with the separation clamped to 1
            const R msE = R(fminf(maxSep, 1.f));
            const Q<R> iAr{R(iA.x), R(iA.y), R(iA.z), R(iA.w)};
            Sup<R> EA = make_sup<R>(A.shape, A.sp, false, hv);
            EA.add_r = msE;
            Sup<R> EB = make_sup<R>(B.shape, B.sp, false, hv);
            set_transform(EB, qmulS(iAr, Q<R>{R(B.quat.x), R(B.quat.y), R(B.quat.z), R(B.quat.w)}),
                          qrotS(iAr, V<R>{R(B.pos.x) - R(A.pos.x), R(B.pos.y) - R(A.pos.y), R(B.pos.z) - R(A.pos.z)}));
            EpaItem it;
            it.a = it.b = 0;
            it.size = sx.size;
            it.pad = 0;
            it.tri = -1;
            for (int k = 0; k < 4; k++) {
                SP<float> sp = sx.pts[k < sx.size ? k : 0];
                it.y[k] = f3(sp.y.x, sp.y.y, sp.y.z);
                it.p[k] = f3(sp.p.x, sp.p.y, sp.p.z);
                it.q[k] = f3(sp.q.x, sp.q.y, sp.q.z);
            }
            Hull<BigStore> h;
            h.st.s = slot;
            h.start(it);
            V<R> eax, ea, eb;
            if (!epa(h, EA, EB, R(c_settings.penetration_tol), eax, ea, eb)) return;  // convex.ts:331
            const V<R> dd = ea - eb;
            const R al = sq_root(lsq(eax));
            pen = (float)(sq_root(lsq(dd)) - msE);
            if (al > R(0)) ea = ea + eax * (-(msE / al));
            lpa = V<float>{(float)ea.x, (float)ea.y, (float)ea.z};
            lpb = V<float>{(float)eb.x, (float)eb.y, (float)eb.z};
            lax = V<float>{(float)eax.x, (float)eax.y, (float)eax.z};
        } else {  // COLLIDING: penetrationDepthStepGJK penetration.ts:84-106
            const float vl = sqrtf(g.sqdist);
            lpa = g.pa + g.axis * (rA / vl);
            lpb = g.pb + g.axis * (-(rB / vl));
            const V<float> dd = lpa - lpb;
            pen = sqrtf(lsq(dd)) - maxSep;
            const float al = sqrtf(lsq(g.axis));
            if (al > 0.f) lpa = lpa + g.axis * (-(maxSep / al));
            lax = g.axis;
        }
        const V<float> paw = qrotS(qA, lpa), pbw = qrotS(qA, lpb), axw = qrotS(qA, lax);
        pa = A.pos + f3(paw.x, paw.y, paw.z);
        pb = A.pos + f3(pbw.x, pbw.y, pbw.z);
        ax = f3(axw.x, axw.y, axw.z);
        sub_face(fA, w, A, -ax, base);
        sub_face(fB, w, B, ax, base);
    }
    mesh_add_hit(red, pa - base, pb - base, ax, pen, A.sub, B.sub, fA, fB);
}

// one compound pair per thread, the reduction pool of 32 manifolds and an EPA polytope in global
// memory (the mesh passes' slots, used at another time of the step)
__global__ void __launch_bounds__(64) k_compound_pairs(DevWorld w) {
    const int np = min(w.ctr->num_compound_pairs, w.max_pairs);
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    MeshReduceT<MESH_BIG_M> &red = ((MeshReduceT<MESH_BIG_M> *)w.mesh_big_red)[tid];
    EpaScratch *slot = (EpaScratch *)w.epa_scratch + tid;
    const HullView hv = hull_view(w);
    for (int k = tid; k < np; k += gridDim.x * blockDim.x) {
        int2 pr = w.pairs[w.compound_pairs[k]];
        int a = pr.x, b = pr.y;
        uint32_t fa = w.flags[a], fb = w.flags[b];
        const int ma = motion_of(fa), mb = motion_of(fb);
        if (ma > mb || (ma == mb && b < a)) {  // narrowphase order (update.ts:74)
            const int t = a;
            a = b;
            b = t;
            const uint32_t tf = fa;
            fa = fb;
            fb = tf;
        }
        const float maxSep = ((fa | fb) & F_SENSOR) ? 0.f : c_settings.spec_dist;
        float3 base;
        float4 qbase;
        geom_pose(w, a, fa, base, qbase);
        red.nm = 0;
        red.dropped = false;
        const int na = sub_count(w, a, fa), nb = sub_count(w, b, fb);
        for (int i = 0; i < na; i++) {
            const SubShape A = sub_shape(w, a, fa, i);
            for (int j = 0; j < nb; j++) collide_sub(w, hv, slot, A, sub_shape(w, b, fb, j), maxSep, base, red);
        }
        mesh_emit(w, red, a, b, base);
    }
}

void launch_mesh_narrowphase(DevWorld &w, int pass, cudaStream_t s) {
    EpaItem *items = (EpaItem *)w.epa_items;
    if (pass == 0) {
        k_mesh_narrowphase<0><<<device_sm_count() * 4, 64, 0, s>>>(w, items);
    } else {
        k_mesh_narrowphase<1><<<device_sm_count() * 4, 64, 0, s>>>(w, items);
        if (w.mesh_big) k_mesh_big<<<MESH_BIG_THREADS / 64, 64, 0, s>>>(w, items);
    }
}

// ---------------------------------------------------------------------------
// continuous collision: the shape cast of each LINEAR_CAST body against the world
// ---------------------------------------------------------------------------
// gjkCastShape gjk.ts:853-1259: A, placed in B's frame, moves by disp; B is fixed.  Returns
// false on a miss, else the time of impact, the closest points then and the unnormalised
// separating axis (closest points found without the last point being required,
// computeClosestPointToSimplex gjk.ts:524-596).
template <typename S, class SA, class SB>
__device__ bool gjk_cast(S &lambda_out, V<S> &pa, V<S> &pb, V<S> &axis_out, const SA &A, const SB &B, V<S> disp,
                         S tol, S rA, S rB, S maxLambda) {
    S sqtol = tol * tol;
    const S sumR = rA + rB;
    Simplex<S> sx;
    sx.size = 0;
    S lambda = S(0);
    V<S> x{S(0), S(0), S(0)};
    const V<S> zero{S(0), S(0), S(0)};
    V<S> q = -B.get(zero);
    V<S> p = A.get(zero);
    V<S> v = q - p;  // the starting direction (gjk.ts:882-897)
    S vls = s_max_value<S>();
    bool allow_restart = false;
    V<S> prev_v{S(0), S(0), S(0)};
    for (int it = 0; it < 100; it++) {
        p = A.get(-v);
        q = B.get(v);
        V<S> wv = x - (q - p);
        S vdw = dot(v, wv) - sumR * sq_root(lsq(v));
        if (vdw > S(0)) {
            S vdr = dot(v, disp);
            if (vdr >= S(-1.0e-18)) return false;
            S old = lambda;
            lambda -= vdw / vdr;
            if (old == lambda) break;
            if (lambda >= maxLambda) return false;
            x = disp * lambda;
            vls = s_max_value<S>();
            sqtol = (tol + sumR) * (tol + sumR);
            allow_restart = true;
        }
        sx.pts[sx.size].p = p;
        sx.pts[sx.size].q = q;
        sx.size++;
        for (int i = 0; i < sx.size; i++) sx.pts[i].y = x - sx.pts[i].q + sx.pts[i].p;
        CP<S> cp;
        switch (sx.size) {
            case 1:
                cp = {sx.pts[0].y, 1};
                break;
            case 2:
                cp = closest_line(sx.pts[0].y, sx.pts[1].y, S(1e-10));
                break;
            case 3:
                cp = closest_tri(sx.pts[0].y, sx.pts[1].y, sx.pts[2].y, false, S(1e-10));
                break;
            default:
                cp = closest_tetra(sx.pts[0].y, sx.pts[1].y, sx.pts[2].y, sx.pts[3].y, false, S(1e-5));
                break;
        }
        S nd = lsq(cp.p);
        if (nd < vls) {
            vls = nd;
            v = cp.p;
        } else {
            if (!allow_restart) break;
            allow_restart = false;
            sx.pts[0].p = p;
            sx.pts[0].q = q;
            sx.size = 1;
            v = x - q;
            vls = s_max_value<S>();
            continue;
        }
        if (cp.set == 0xf) break;
        int ns = 0;  // updatePointSetPQ gjk.ts:799-813
        for (int i = 0; i < sx.size; i++)
            if (cp.set & (1 << i)) {
                if (ns != i) {
                    sx.pts[ns].p = sx.pts[i].p;
                    sx.pts[ns].q = sx.pts[i].q;
                }
                ns++;
            }
        sx.size = ns;
        if (vls <= sqtol) break;
        prev_v = v;
    }
    for (int i = 0; i < sx.size; i++) sx.pts[i].y = x - sx.pts[i].q + sx.pts[i].p;
    S vl = sq_root(lsq(v));
    V<S> nv = vl > S(0) ? v * (S(1) / vl) : zero;
    V<S> sa = zero, sb = zero;
    if (sx.size == 1) {
        sa = sx.pts[0].p;
        sb = sx.pts[0].q;
    } else if (sx.size == 2) {
        Bary<S> b = bary2(sx.pts[0].y, sx.pts[1].y, S(1e-10));
        sa = sx.pts[0].p * b.u + sx.pts[1].p * b.v;
        sb = sx.pts[0].q * b.u + sx.pts[1].q * b.v;
    } else if (sx.size >= 3) {
        Bary<S> b = bary3(sx.pts[0].y, sx.pts[1].y, sx.pts[2].y, S(1e-10));
        sa = sx.pts[0].p * b.u + sx.pts[1].p * b.v + sx.pts[2].p * b.w;
        sb = sx.pts[0].q * b.u + sx.pts[1].q * b.v + sx.pts[2].q * b.w;
    }
    if (sx.size >= 1) {
        pb = sb + nv * rB;
        pa = lambda > S(0) ? pb : sa + nv * (-rA);
    } else {
        pa = pb = zero;
    }
    lambda_out = lambda;
    axis_out = sumR > S(0) ? -v : -prev_v;
    return true;
}

// entry t of the segment o + t d, t in [0, len], into a box, or +inf on a miss
// (rayDistanceToBox3 cast-utils.ts:14-49, the slab test the casts use)
__device__ __forceinline__ float ray_box_entry(float3 o, float3 d, float len, float3 lo, float3 hi) {
    float t0 = 0.f, t1 = len;
    const float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
    const float mn[3] = {lo.x, lo.y, lo.z}, mx[3] = {hi.x, hi.y, hi.z};
#pragma unroll
    for (int i = 0; i < 3; i++) {
        if (fabsf(dd[i]) < 1e-10f) {
            if (oo[i] < mn[i] || oo[i] > mx[i]) return CUDART_INF_F;
        } else {
            float inv = 1.f / dd[i];
            float a = (mn[i] - oo[i]) * inv, c = (mx[i] - oo[i]) * inv;
            t0 = fmaxf(t0, fminf(a, c));
            t1 = fminf(t1, fmaxf(a, c));
            if (t1 < t0) return CUDART_INF_F;
        }
    }
    return t0;
}

// rayDistanceToBox3 cast-utils.ts:14-49 (the entry fraction, +inf on a miss)
__device__ __forceinline__ float ray_fraction_to_box(float3 o, float3 d, float len, float3 lo, float3 hi) {
    float t = ray_box_entry(o, d, len, lo, hi);
    return t < CUDART_INF_F ? t / len : CUDART_INF_F;
}
// rayCylinder / raySphereFromOrigin sphere-triangle.ts:17-83, 156-195
__device__ float ray_cylinder(float3 dir, float3 ca, float3 cb, float r) {
    float3 axis = cb - ca, st = -ca;
    float sda = dot3(st, axis), dda = dot3(dir, axis), eda = sda + dda;
    if (sda < 0.f && eda < 0.f) return CUDART_INF_F;
    float al2 = lensq3(axis);
    if (sda > al2 && eda > al2) return CUDART_INF_F;
    float a = al2 * lensq3(dir) - dda * dda;
    if (fabsf(a) < 1e-6f) return CUDART_INF_F;
    float b = al2 * dot3(st, dir) - dda * sda;
    float c = al2 * (lensq3(st) - r * r) - sda * sda;
    float det = b * b - a * c;
    if (det < 0.f) return CUDART_INF_F;
    float t = -(b + sqrtf(det)) / a;
    if (t < 0.f || t > 1.f) return CUDART_INF_F;
    float hda = sda + t * dda;
    if (hda < 0.f || hda > al2) return CUDART_INF_F;
    return t;
}
__device__ float ray_sphere_from_origin(float3 dir, float3 c, float r) {
    float a = lensq3(dir), b = -2.f * dot3(dir, c), cc = lensq3(c) - r * r;
    float disc = b * b - 4.f * a * cc;
    if (disc < 0.f || a < 1e-10f) return cc <= 0.f ? 0.f : CUDART_INF_F;
    float sq = sqrtf(disc);
    float t1 = (-b - sq) / (2.f * a), t2 = (-b + sq) / (2.f * a);
    if (t1 > t2) {
        float t = t1;
        t1 = t2;
        t2 = t;
    }
    if (t1 >= 0.f && t1 <= 1.f) return t1;
    if (t2 >= 0.f && t2 <= 1.f) return 0.f;
    if (t1 < 0.f && t2 > 1.f) return 0.f;
    return CUDART_INF_F;
}

// castConvexVsPlane plane.ts:727-918 for a convex support S of the moving shape at (pA, qA)
// (SupportFunctionMode.DEFAULT) against a plane body at (pP, qP): the plane's own equation
// against the world support point, the hit carried by the plane body's transform, as the
// reference computes them; back faces culled
__device__ bool cast_vs_plane(const Sup<float> &S, float3 pA, float4 qA, float3 disp, float4 spP, float3 pP,
                              float4 qP, float early, float &frac, float3 &paw, float3 &axw) {
    const float3 n = xyz(spP);
    const float3 nA = -qrot_inv(qA, n);
    const V<float> s = S.get(V<float>{nA.x, nA.y, nA.z});
    const float3 spw = pA + qrot(qA, f3(s.x, s.y, s.z));
    const float sd = dot3(n, spw) + spP.w, cr = S.convex_radius, pen = -sd + cr;
    const float dn = dot3(disp, n);
    float3 ht = pP;
    if (pen > 0.f) {
        if (dn > 0.f || pen <= -early) return false;
        frac = 0.f;
        paw = pP + qrot(qP, spw - n * cr);
    } else if (dn < 0.f) {
        frac = pen / dn;
        if (frac >= early) return false;
        ht = pP + qrot(qP, disp * frac);
        paw = ht + qrot(qP, spw - n * cr);
    } else {
        return false;
    }
    axw = ht + qrot(qP, -n);  // vec3.transformMat4 of -n: a point transform
    return true;
}

// a triangle's sub-shape id (subShape.pushIndex sub-shape.ts:60-64: the index in the low bits,
// ones above)
__device__ __forceinline__ uint32_t tri_sub_id(const DevMesh &M, int ti) {
    return M.sub_bits >= 32 ? (uint32_t)ti : ((0xffffffffu & ~((1u << M.sub_bits) - 1u)) | (uint32_t)ti);
}

// the convex shapes a cast or collide query may be: sphere, box, capsule, cylinder, or a convex
// hull of the world (its index as int bits, as bodies keep it)
__device__ __forceinline__ bool query_shape_ok(const DevWorld &w, int shape, float4 sp) {
    if (shape == SHAPE_HULL) return (unsigned)hull_of(sp) < (unsigned)w.num_hulls;
    return shape == SHAPE_SPHERE || shape == SHAPE_BOX || shape == SHAPE_CAPSULE || shape == SHAPE_CYLINDER;
}

// castConvexVsTriangleMesh triangle-mesh.ts:638-1019 and castSphereVsTriangleMesh :1781-2236
// for the continuous-collision visitor (default cast settings: tolerances 0.01, support mode
// DEFAULT, back faces culled, no movement direction, no deepest point).  collect(fraction,
// world point on A, world penetration axis, the triangle's sub-shape id) is the collector; fps its
// early-out fraction.
template <class Collect>
__device__ void ccd_cast_mesh(const DevWorld &w, uint32_t fa, float4 sa, float3 pA, float4 qA4, float3 disp, int b,
                              const float &fps, Collect &&collect) {
    const DevMesh &M = w.meshes[mesh_of(w.shape[b])];
    if (M.num_tris == 0) return;
    float3 pB;
    float4 qB4;
    geom_pose(w, b, w.flags[b], pB, qB4);
    const Q<float> qB{qB4.x, qB4.y, qB4.z, qB4.w}, iqB{-qB4.x, -qB4.y, -qB4.z, qB4.w};
    auto toB = [&](float3 v) {
        V<float> q = qrotS(iqB, V<float>{v.x, v.y, v.z});
        return f3(q.x, q.y, q.z);
    };
    auto toW = [&](float3 v) {
        V<float> q = qrotS(qB, V<float>{v.x, v.y, v.z});
        return f3(q.x, q.y, q.z);
    };
    const float3 dInB = toB(disp);
    const float4 *nodes = w.mesh_nodes + 2 * M.first_node;
    int stack[MESH_STACK];
    float sdist[MESH_STACK];
    if (shape_of(fa) == SHAPE_SPHERE) {
        const float r = sa.x;
        const float3 start = toB(pA - pB), end = start + dInB;
        const float3 lo = f3(fminf(start.x, end.x) - r, fminf(start.y, end.y) - r, fminf(start.z, end.z) - r);
        const float3 hi = f3(fmaxf(start.x, end.x) + r, fmaxf(start.y, end.y) + r, fmaxf(start.z, end.z) + r);
        const float3 qc = (lo + hi) * 0.5f;
        // castSphereVsTriangleMeshAddHit :1781-1868: the penetration axis is the negated contact normal
        uint32_t tsub = 0xffffffffu;
        auto emit = [&](float fraction, float3 cp, float3 cn) {
            collect(fraction, toW(start + cp) + pB, -normalize3(toW(cn)), tsub);
        };
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            const int node = stack[--sp];
            const float4 nlo = nodes[2 * node], nhi = nodes[2 * node + 1];
            if (!node_hits_box(nlo, nhi, lo, hi)) continue;
            const int aux = __float_as_int(nlo.w), tag = __float_as_int(nhi.w);
            if (tag >= 0) {
                const int left = node + 1, right = aux;
                float ld = lensq3(qc - (xyz(nodes[2 * left]) + xyz(nodes[2 * left + 1])) * 0.5f);
                float rd = lensq3(qc - (xyz(nodes[2 * right]) + xyz(nodes[2 * right + 1])) * 0.5f);
                if (sp + 2 > MESH_STACK) continue;
                if (ld <= rd) {
                    stack[sp++] = right;
                    stack[sp++] = left;
                } else {
                    stack[sp++] = left;
                    stack[sp++] = right;
                }
                continue;
            }
            for (int ti = aux; ti < aux + (-tag - 1); ti++) {
                const int4 tr = w.mesh_tris[M.first_tri + ti];
                tsub = tri_sub_id(M, ti);
                const float3 v0 = xyz(w.mesh_verts[tr.x]) - start, v1 = xyz(w.mesh_verts[tr.y]) - start,
                             v2 = xyz(w.mesh_verts[tr.z]) - start;
                float3 tn = cross3(v1 - v0, v2 - v0);
                const float tl = sqrtf(lensq3(tn));
                if (tl == 0.f) continue;
                tn = tn * (1.f / tl);
                const float ndd = dot3(tn, dInB);
                if (ndd > 0.f) continue;  // back face
                if (fabsf(dot3(v0, tn)) <= r) {  // touching at the start
                    float dsq;
                    int feature;
                    float3 q = closest_on_triangle(v0, v1, v2, dsq, feature);
                    if (dsq <= r * r) {
                        const float ql = sqrtf(dsq), pen = r - ql;
                        if (-pen >= fps) continue;
                        const float3 cn = ql > 0.f ? q * (1.f / ql) : f3(0.f, 1.f, 0.f);
                        emit(0.f, q + cn * pen, cn);
                        continue;
                    }
                }
                if (fabsf(ndd) > 1e-6f) {  // the plane
                    const float3 d = tn * ((ndd > 0.f ? 1.f : (ndd < 0.f ? -1.f : 0.f)) * r);
                    const float pi = dot3(v0 - d, tn) / ndd;
                    if (pi * fabsf(ndd) >= -r && pi < fps && pi >= 0.f) {
                        const float3 p = d + dInB * pi;
                        const float3 a0 = v0 - p, a1 = v1 - p, a2 = v2 - p;
                        const float3 nn = cross3(a1, a2);
                        const float nl = sqrtf(lensq3(nn));
                        if (nl > 0.f) {
                            const float area = dot3(nn, tn) / nl;
                            if (area > 0.f) {
                                const float u = dot3(cross3(a1, a2), tn) / (area * nl),
                                            v = dot3(cross3(a2, a0), tn) / (area * nl),
                                            ww = dot3(cross3(a0, a1), tn) / (area * nl);
                                if (u >= 0.f && v >= 0.f && ww >= 0.f) {
                                    emit(pi, p, -tn);
                                    continue;
                                }
                            }
                        }
                    }
                }
                float f = CUDART_INF_F;  // edges and vertices
                f = fminf(f, ray_cylinder(dInB, v0, v1, r));
                f = fminf(f, ray_cylinder(dInB, v1, v2, r));
                f = fminf(f, ray_cylinder(dInB, v2, v0, r));
                f = fminf(f, ray_sphere_from_origin(dInB, v0, r));
                f = fminf(f, ray_sphere_from_origin(dInB, v1, r));
                f = fminf(f, ray_sphere_from_origin(dInB, v2, r));
                if (f >= 0.f && f < fps) {
                    const float3 p = dInB * f;
                    float dsq;
                    int feature;
                    const float3 q = closest_on_triangle(v0 - p, v1 - p, v2 - p, dsq, feature);
                    emit(f, p + q, normalize3(q));
                }
            }
        }
        return;
    }
    // the GJK cast of the convex shape: A placed in the mesh's frame
    const Q<float> qAq{qA4.x, qA4.y, qA4.z, qA4.w};
    const Q<float> qAInB = qmulS(iqB, qAq);
    const float3 posAInB = toB(pA - pB);
    float3 llo, lhi;
    convex_local_bounds(w, fa, sa, llo, lhi);
    float3 blo = f3(3.0e38f, 3.0e38f, 3.0e38f), bhi = f3(-3.0e38f, -3.0e38f, -3.0e38f);
    for (int c = 0; c < 8; c++) {
        V<float> p{(c & 1) ? lhi.x : llo.x, (c & 2) ? lhi.y : llo.y, (c & 4) ? lhi.z : llo.z};
        V<float> q = qrotS(qAInB, p);
        float3 qq = f3(q.x, q.y, q.z) + posAInB;
        blo = f3(fminf(blo.x, qq.x), fminf(blo.y, qq.y), fminf(blo.z, qq.z));
        bhi = f3(fmaxf(bhi.x, qq.x), fmaxf(bhi.y, qq.y), fmaxf(bhi.z, qq.z));
    }
    const HullView hv = hull_view(w);
    // SupportFunctionMode.DEFAULT: the full box, the other shapes' core with their radius
    Sup<float> supA = make_sup<float>(shape_of(fa), sa, shape_of(fa) != SHAPE_BOX, hv);
    const float crA = supA.convex_radius;
    set_transform(supA, qAInB, V<float>{posAInB.x, posAInB.y, posAInB.z});
    const float3 origin = (blo + bhi) * 0.5f, half = (bhi - blo) * 0.5f;
    const float rlen = sqrtf(lensq3(dInB));
    const float3 rdir = rlen > 1e-10f ? dInB * (1.f / rlen) : f3(0.f, 0.f, 0.f);
    const V<float> dv{dInB.x, dInB.y, dInB.z};
    int sp = 0;
    stack[sp] = 0;
    sdist[sp++] = 0.f;
    while (sp > 0) {
        --sp;
        const int node = stack[sp];
        if (sdist[sp] >= fps) continue;
        const float4 nlo = nodes[2 * node], nhi = nodes[2 * node + 1];
        const int aux = __float_as_int(nlo.w), tag = __float_as_int(nhi.w);
        if (tag >= 0) {
            const int left = node + 1, right = aux;
            float ld = ray_fraction_to_box(origin, rdir, rlen, xyz(nodes[2 * left]) - half,
                                           xyz(nodes[2 * left + 1]) + half);
            float rd = ray_fraction_to_box(origin, rdir, rlen, xyz(nodes[2 * right]) - half,
                                           xyz(nodes[2 * right + 1]) + half);
            if (sp + 2 > MESH_STACK) continue;
            if (ld <= rd) {
                if (rd < fps) stack[sp] = right, sdist[sp++] = rd;
                if (ld < fps) stack[sp] = left, sdist[sp++] = ld;
            } else {
                if (ld < fps) stack[sp] = left, sdist[sp++] = ld;
                if (rd < fps) stack[sp] = right, sdist[sp++] = rd;
            }
            continue;
        }
        for (int ti = aux; ti < aux + (-tag - 1); ti++) {
            const int4 tr = w.mesh_tris[M.first_tri + ti];
            const float3 a = xyz(w.mesh_verts[tr.x]), bb = xyz(w.mesh_verts[tr.y]), c = xyz(w.mesh_verts[tr.z]);
            const float3 tlo = f3(fminf(a.x, fminf(bb.x, c.x)), fminf(a.y, fminf(bb.y, c.y)), fminf(a.z, fminf(bb.z, c.z)));
            const float3 thi = f3(fmaxf(a.x, fmaxf(bb.x, c.x)), fmaxf(a.y, fmaxf(bb.y, c.y)), fmaxf(a.z, fmaxf(bb.z, c.z)));
            if (!(ray_box_entry(origin, rdir, rlen, tlo - half, thi + half) < CUDART_INF_F)) continue;
            if (fps <= 0.f) return;
            const float3 n = cross3(bb - a, c - a);
            if (dot3(n, dInB) > 0.f) continue;  // back face
            Sup<float, true, true> supT = make_sup<float, true, true>(SHAPE_SPHERE, make_float4(0.f, 0.f, 0.f, 0.f), false, hv);
            supT.kind = SUP_TRIANGLE;
            supT.r0 = V<float>{a.x, a.y, a.z};
            supT.r1 = V<float>{bb.x, bb.y, bb.z};
            supT.r2 = V<float>{c.x, c.y, c.z};
            supT.convex_radius = 0.f;
            float lambda;
            V<float> cpa, cpb, ax;
            if (!gjk_cast(lambda, cpa, cpb, ax, supA, supT, dv, 0.01f, crA, 0.f, fps)) continue;
            if (lsq(ax) < 0.01f * 0.01f) ax = dv;  // penetration.ts:693-698
            const float depth = sqrtf(lsq(cpa - cpb));
            if (lambda == 0.f && -depth >= fps) continue;
            float3 axf = f3(ax.x, ax.y, ax.z);
            if (tr.w != 0b111) axf = fix_normal(a, bb, c, n, tr.w, f3(cpb.x, cpb.y, cpb.z), axf, f3(0.f, 0.f, 0.f));
            collect(lambda, toW(f3(cpa.x, cpa.y, cpa.z)) + pB, toW(axf), tri_sub_id(M, ti));
        }
    }
}

// findCCDContacts update.ts:1354-1470: one thread per record.  The swept bounds are cast
// through the refitted tree (dbvt.castAABB dbvt.ts:869-975: a ray from the swept centre along
// the displacement against boxes grown by the swept half extents, nodes past the distance cull
// skipped), every body found goes through the visitor's filters (update.ts:1153-1206) and the
// shape cast (castConvexVsConvex convex.ts:675-900, back faces culled), and the collector keeps
// the earliest fraction plus slop (update.ts:1044-1109); of equal ones the lower body index, the
// first in the reference's candidate order for bodies of one tree leaf level.
constexpr int CCD_STACK = 64;
__global__ void __launch_bounds__(128) k_ccd_find(DevWorld w, const int2 *node_world, float dt) {
    const int nr = w.ctr->num_ccd;
    const int n = w.n;
    const HullView hv = hull_view(w);
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nr; r += gridDim.x * blockDim.x) {
        CcdRec &c = w.ccd[r];
        const int a = c.body;
        const uint32_t fa = w.flags[a];
        const float3 delta = xyz(c.delta);
        const float thr_sq = c.delta.w, max_pen = c.normal.w;
        const float3 alo = xyz(w.aabb_lo[a]), ahi = xyz(w.aabb_hi[a]);
        const float3 slo = f3(fminf(alo.x, alo.x + delta.x), fminf(alo.y, alo.y + delta.y), fminf(alo.z, alo.z + delta.z));
        const float3 shi = f3(fmaxf(ahi.x, ahi.x + delta.x), fmaxf(ahi.y, ahi.y + delta.y), fmaxf(ahi.z, ahi.z + delta.z));
        const float3 origin = (slo + shi) * 0.5f, half = (shi - slo) * 0.5f;
        const float clen = sqrtf(lensq3(delta));
        const float3 cdir = normalize3(delta);
        const float3 half_a = (ahi - alo) * 0.5f;
        const int wa = w.world[a];
        const uint32_t allowed = c_settings.cast_pairs[layer_of(fa)];
        const uint2 ga = w.groups[a];
        float3 pA;
        float4 qA;
        geom_pose(w, a, fa, pA, qA);
        const Sup<float> supA0 = make_sup<float>(shape_of(fa), w.shape[a], true, hv);
        float best_fps = c.fps, best_frac = c.point.w;
        int best = -1;
        float3 best_n = f3(0.f, 0.f, 0.f), best_p = f3(0.f, 0.f, 0.f);
        int stack[CCD_STACK];
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            int node = stack[--sp];
            int2 nw = node_world[node];
            if (wa < nw.x || wa > nw.y) continue;
            float3 nlo = xyz(w.node_lo[node]) - half, nhi = xyz(w.node_hi[node]) + half;
            float t = ray_box_entry(origin, cdir, clen, nlo, nhi);
            if (!(t < CUDART_INF_F) || t / clen > clen) continue;
            if (node < n - 1) {
                int2 ch = w.node_child[node];
                if (sp + 2 <= CCD_STACK) {
                    stack[sp++] = ch.y;
                    stack[sp++] = ch.x;
                } else {
                    atomicOr(&w.ctr->overflow, OVF_SLOTS);
                }
                continue;
            }
            const int b = w.order[node - (n - 1)];
            const uint32_t fb = w.flags[b];
            if (!(allowed & (1u << layer_of(fb)))) continue;
            const uint2 gb = w.groups[b];
            if (!((ga.x & gb.y) != 0u && (gb.x & ga.y) != 0u)) continue;
            // ccdBodyVisitor.visit update.ts:1153-1206
            if (b == a) continue;
            const int cb = w.ccd_index[b];
            if (cb >= 0 && a > b) continue;  // a pair of cast bodies is cast once, by the lower index
            if (fb & F_SENSOR) continue;
            float3 rel = delta;
            if (cb >= 0) rel = rel - xyz(w.ccd[cb].delta);
            if (lensq3(rel) < thr_sq) continue;
            const float3 blo = xyz(w.aabb_lo[b]) - half_a, bhi = xyz(w.aabb_hi[b]) + half_a;
            if (!(ray_box_entry(xyz(w.pos[a]), rel, sqrtf(lensq3(rel)), blo, bhi) < CUDART_INF_F)) continue;
            // ccdCastShapeCollector.addHit update.ts:1044-1109
            auto collect = [&](float lambda, float3 paw, float3 axw, uint32_t = 0xffffffffu) {
                const float3 nrm = normalize3(axw);
                const float den = dot3(nrm, delta);
                if (den <= max_pen) return;
                const float fps = lambda + max_pen / den;
                if (!(fps < best_fps || (fps == best_fps && best >= 0 && b < best))) return;
                best = b;
                best_fps = fps;
                best_frac = lambda;
                best_n = nrm;
                float3 pt = paw;
                // calculateBodyMotion update.ts:984-994
                if (motion_of(fb) != STATIC && (fb & F_LINEAR_CAST)) {
                    float3 mb = xyz(w.linvel[b]) * dt;
                    if (lensq3(mb) > 1e-12f) pt = pt + mb * lambda;
                }
                best_p = pt;
            };
            if (shape_of(fb) == SHAPE_EMPTY || shape_of(fa) == SHAPE_EMPTY) continue;
            if (shape_of(fb) == SHAPE_MESH) {
                ccd_cast_mesh(w, fa, w.shape[a], pA, qA, rel, b, best_fps, collect);
                continue;
            }
            if (shape_of(fb) == SHAPE_PLANE) {
                float3 pB, paw, axw;
                float4 qB;
                float frac;
                geom_pose(w, b, fb, pB, qB);
                const Sup<float> S = make_sup<float>(shape_of(fa), w.shape[a], default_excludes(shape_of(fa)), hv);
                if (cast_vs_plane(S, pA, qA, rel, w.shape[b], pB, qB, best_fps, frac, paw, axw)) collect(frac, paw, axw);
                continue;
            }
            // castConvexVsConvex: A in B's frame; a compound target child by child
            // (castShapeVsCompound compound.ts:776-866)
            const int nsub = sub_count(w, b, fb);
            for (int ci = 0; ci < nsub; ci++) {
                const SubShape cs = sub_shape(w, b, fb, ci);
                const float3 pB = cs.pos;
                const float4 qB = cs.quat;
                const Q<float> iqB{-qB.x, -qB.y, -qB.z, qB.w};
                const V<float> posAInB = qrotS(iqB, V<float>{pA.x - pB.x, pA.y - pB.y, pA.z - pB.z});
                const Q<float> qAInB = qmulS(iqB, Q<float>{qA.x, qA.y, qA.z, qA.w});
                const V<float> dInB = qrotS(iqB, V<float>{rel.x, rel.y, rel.z});
                Sup<float> supA = supA0;
                set_transform(supA, qAInB, posAInB);
                const Sup<float> supB = make_sup<float>(cs.shape, cs.sp, true, hv);
                float lambda;
                V<float> cpa, cpb, ax;
                if (!gjk_cast(lambda, cpa, cpb, ax, supA, supB, dInB, 1e-4f, supA.convex_radius, supB.convex_radius,
                              best_fps))
                    continue;
                // penetrationCastShape penetration.ts:693-698: a too short axis becomes the cast direction
                if (lsq(ax) < 1e-4f * 1e-4f) ax = dInB;
                if (lambda > 1.f || dot(ax, dInB) <= 0.f || lambda >= best_fps) continue;
                const Q<float> qBq{qB.x, qB.y, qB.z, qB.w};
                const V<float> axw = qrotS(qBq, ax);
                const V<float> paw = qrotS(qBq, cpa);
                collect(lambda, f3(paw.x + pB.x, paw.y + pB.y, paw.z + pB.z), f3(axw.x, axw.y, axw.z));
            }
        }
        if (best >= 0) {
            c.hit = best;
            c.fps = best_fps;
            c.normal = make_float4(best_n.x, best_n.y, best_n.z, max_pen);
            c.point = make_float4(best_p.x, best_p.y, best_p.z, best_frac);
            atomicAdd(&w.ctr->num_ccd_hits, 1);
        }
    }
}

void launch_ccd_find(DevWorld &w, float dt, cudaStream_t s) {
    k_ccd_find<<<grid_for(w.n, 128, 16), 128, 0, s>>>(w, w.node_world, dt);
}

// ---------------------------------------------------------------------------
// world queries: castRay (query.ts:78-90) with the closest-hit collector
// (ClosestCastRayCollector cast-ray-vs-shape.ts:180-205), one thread per ray
// ---------------------------------------------------------------------------
// gjkCastRay gjk.ts:622-790: origin + lambda * dir against a support in its own frame; false
// when the ray misses before maxLambda
template <typename S, class SA>
__device__ bool gjk_cast_ray(S &lambda_out, V<S> origin, V<S> dir, S tol, const SA &A, S maxLambda) {
    const S sqtol = tol * tol;
    Simplex<S> sx;
    sx.size = 0;
    S lambda = S(0);
    V<S> x = origin;
    V<S> p = A.get(V<S>{S(0), S(0), S(0)});
    V<S> v = x - p;
    S vls = s_max_value<S>();
    bool allow_restart = false;
    for (int it = 0; it < 100; it++) {
        p = A.get(v);
        const V<S> wv = x - p;
        const S vdw = dot(v, wv);
        if (vdw > S(0)) {
            const S vdr = dot(v, dir);
            if (vdr >= S(-1.0e-18)) return false;
            const S old = lambda;
            lambda -= vdw / vdr;
            if (old == lambda) break;
            if (lambda >= maxLambda) return false;
            x = origin + dir * lambda;
            vls = s_max_value<S>();
            allow_restart = true;
        }
        sx.pts[sx.size].p = p;
        sx.size++;
        for (int i = 0; i < sx.size; i++) sx.pts[i].y = x - sx.pts[i].p;
        CP<S> cp;
        switch (sx.size) {
            case 1:
                cp = {sx.pts[0].y, 1};
                break;
            case 2:
                cp = closest_line(sx.pts[0].y, sx.pts[1].y, S(1e-10));
                break;
            case 3:
                cp = closest_tri(sx.pts[0].y, sx.pts[1].y, sx.pts[2].y, false, S(1e-10));
                break;
            default:
                cp = closest_tetra(sx.pts[0].y, sx.pts[1].y, sx.pts[2].y, sx.pts[3].y, false, S(1e-5));
                break;
        }
        const S nd = lsq(cp.p);
        if (nd < vls) {
            vls = nd;
            v = cp.p;
        } else {
            if (!allow_restart) break;
            allow_restart = false;
            sx.pts[0].p = p;
            sx.size = 1;
            v = x - p;
            vls = s_max_value<S>();
            continue;
        }
        if (cp.set == 0xf) break;
        int ns = 0;
        for (int i = 0; i < sx.size; i++)
            if (cp.set & (1 << i)) {
                if (ns != i) sx.pts[ns].p = sx.pts[i].p;
                ns++;
            }
        sx.size = ns;
        if (vls <= sqtol) break;
    }
    lambda_out = lambda;
    return true;
}

// raycast3.intersectsTriangle of mathcat 0.0.10 (not vendored), taken as the Moller-Trumbore test
// over t in [0, len] along the ray direction with back faces culled when asked; the hit's fraction
// is t / len
__device__ __forceinline__ bool ray_triangle(float3 o, float3 d, float len, float3 a, float3 b, float3 c,
                                             bool cull_back, float &fraction) {
    const float3 e1 = b - a, e2 = c - a;
    const float3 pv = cross3(d, e2);
    const float det = dot3(e1, pv);
    if (cull_back ? det < 1e-10f : fabsf(det) < 1e-10f) return false;
    const float inv = 1.f / det;
    const float3 tv = o - a;
    const float u = dot3(tv, pv) * inv;
    if (u < 0.f || u > 1.f) return false;
    const float3 qv = cross3(tv, e1);
    const float v = dot3(d, qv) * inv;
    if (v < 0.f || u + v > 1.f) return false;
    const float t = dot3(e2, qv) * inv;
    if (t < 0.f || t > len) return false;
    fraction = t / len;
    return true;
}

// castRayVsTriangleMesh triangle-mesh.ts:259-430: the closest triangle below max_f of the mesh of
// body b, the ray in the mesh's frame; nearer child first, subtrees beyond the best hit skipped
// castRayVsTriangleMesh triangle-mesh.ts:259-432 in the mesh's frame: every triangle hit below
// the collector's early-out fraction `early` (read live: on_hit(fraction, sub-shape id) may lower
// it) in the walk's nearer-child-first order; the walk ends once early <= 0
template <class OnHit>
__device__ void ray_mesh_walk(const DevWorld &w, int b, float3 o, float3 d, float len, bool cull_back,
                              const float &early, OnHit &&on_hit) {
    const DevMesh &M = w.meshes[mesh_of(w.shape[b])];
    if (M.num_tris == 0) return;
    const float4 *nodes = w.mesh_nodes + 2 * M.first_node;
    int stack[MESH_STACK];
    float sdist[MESH_STACK];
    int sp = 0;
    stack[sp] = 0;
    sdist[sp++] = -CUDART_INF_F;
    const float &best = early;
    while (sp > 0) {
        if (best <= 0.f) break;
        --sp;
        const int node = stack[sp];
        if (sdist[sp] >= best) continue;
        const float4 nlo = nodes[2 * node], nhi = nodes[2 * node + 1];
        const int aux = __float_as_int(nlo.w), tag = __float_as_int(nhi.w);
        if (tag < 0) {
            for (int ti = aux; ti < aux + (-tag - 1); ti++) {
                const int4 tr = w.mesh_tris[M.first_tri + ti];
                float f;
                if (ray_triangle(o, d, len, xyz(w.mesh_verts[tr.x]), xyz(w.mesh_verts[tr.y]), xyz(w.mesh_verts[tr.z]),
                                 cull_back, f) &&
                    f < best)
                    on_hit(f, M.sub_bits >= 32 ? (uint32_t)ti
                                               : ((0xffffffffu & ~((1u << M.sub_bits) - 1u)) | (uint32_t)ti));
            }
            continue;
        }
        const int left = node + 1, right = aux;
        const float ld = ray_fraction_to_box(o, d, len, xyz(nodes[2 * left]), xyz(nodes[2 * left + 1]));
        const float rd = ray_fraction_to_box(o, d, len, xyz(nodes[2 * right]), xyz(nodes[2 * right + 1]));
        if (sp + 2 > MESH_STACK) {
            atomicOr(&w.ctr->overflow, OVF_SLOTS);
            continue;
        }
        if (ld <= rd) {
            if (rd < best) { stack[sp] = right; sdist[sp++] = rd; }
            if (ld < best) { stack[sp] = left; sdist[sp++] = ld; }
        } else {
            if (ld < best) { stack[sp] = left; sdist[sp++] = ld; }
            if (rd < best) { stack[sp] = right; sdist[sp++] = rd; }
        }
    }
}
// the closest hit of the walk (ClosestCastRayCollector: each hit lowers the early-out fraction)
__device__ bool ray_vs_mesh(const DevWorld &w, int b, float3 o, float3 d, float len, bool cull_back, float max_f,
                            float &fraction, uint32_t &sub) {
    float best = max_f;
    bool found = false;
    ray_mesh_walk(w, b, o, d, len, cull_back, best, [&](float f, uint32_t s) {
        best = f;
        found = true;
        sub = s;
    });
    if (found) fraction = best;
    return found;
}

// castRayVsConvex convex.ts:54-126 (the INCLUDE_CONVEX_RADIUS support, tolerance 1e-3) of one
// convex shape at (pB, qB)
__device__ bool ray_vs_convex(const HullView &hv, int shape, float4 sp, float3 pB, float4 qB, float3 o, float3 d,
                              float len, uint32_t flags, float max_f, float &fraction) {
    const float3 lo = qrot_inv(qB, o - pB), ld = qrot_inv(qB, d);
    const Sup<float> sup = make_sup<float>(shape, sp, false, hv);
    float lambda;
    if (!gjk_cast_ray(lambda, V<float>{lo.x, lo.y, lo.z}, V<float>{ld.x * len, ld.y * len, ld.z * len}, 1e-3f, sup,
                      max_f))
        return false;
    if (!((flags & CC_RAY_SOLID) || lambda > 0.f)) return false;
    fraction = fmaxf(0.f, lambda);
    return true;
}

// castRayVsShape for one body (castRayVsConvex convex.ts:54-126 with the INCLUDE_CONVEX_RADIUS
// support and tolerance 1e-3, or the mesh walk): the hit below max_f and its sub-shape id.
// MESH selects the triangle-mesh branch, so that each kernel instance holds only one of them.
template <bool MESH>
__device__ bool ray_vs_body(const DevWorld &w, const HullView &hv, int b, float3 o, float3 d, float len,
                            uint32_t flags, float max_f, float &fraction, uint32_t &sub) {
    const uint32_t fb = w.flags[b];
    float3 pB;
    float4 qB;
    geom_pose(w, b, fb, pB, qB);
    const float3 lo = qrot_inv(qB, o - pB), ld = qrot_inv(qB, d);
    if (MESH) return ray_vs_mesh(w, b, lo, ld, len, !(flags & CC_RAY_BACKFACES), max_f, fraction, sub);
    if (shape_of(fb) == SHAPE_EMPTY) return false;
    if (shape_of(fb) == SHAPE_PLANE) {  // castRayVsPlane plane.ts:320-398
        float3 n;
        float c;
        plane_world(w.shape[b], pB, qB, n, c);
        const float dist = dot3(n, o) + c;
        sub = 0xffffffffu;
        if ((flags & CC_RAY_SOLID) && dist <= 0.f && max_f > 0.f) {
            fraction = 0.f;
            return true;
        }
        const float dn = dot3(d, n);
        if (fabsf(dn) < 1e-10f) return false;
        if (!(flags & CC_RAY_BACKFACES) && dn > 0.f) return false;
        const float f = -dist / dn / len;
        if (!(f >= 0.f && f < max_f)) return false;
        fraction = f;
        return true;
    }
    if (shape_of(fb) == SHAPE_COMPOUND) {  // castRayVsCompound compound.ts:350-421: the children's closest
        bool found = false;
        float best = max_f;
        const int nc = sub_count(w, b, fb);
        for (int i = 0; i < nc && best > 0.f; i++) {
            const SubShape cs = sub_shape(w, b, fb, i);
            float f;
            if (ray_vs_convex(hv, cs.shape, cs.sp, cs.pos, cs.quat, o, d, len, flags, best, f) && f < best) {
                best = f;
                found = true;
                sub = cs.sub;
            }
        }
        if (found) fraction = best;
        return found;
    }
    sub = 0xffffffffu;
    return ray_vs_convex(hv, shape_of(fb), w.shape[b], pB, qB, o, d, len, flags, max_f, fraction);
}

// broadphase.castRay / dbvt.castRay (broadphase.ts:280-298, dbvt.ts:779-865) over the world's
// subtree of the device tree: every body whose box the segment enters and that passes the filter
// is cast, into one of the collectors of cast-ray-vs-shape.ts:66-205:
//   COLLECT_CLOSEST: the least fraction wins, ties to the lower body index (hits[r]);
//   COLLECT_ANY: the first hit of the walk ends it (hits[r], counts[r] = 0 or 1);
//   COLLECT_ALL: every hit below the initial early-out fraction, one per convex body and one per
//     triangle of a mesh, appended to hits[r * cap ...] while room is left; counts[r] the total.
// PASS 0 casts every body; with meshes present, PASS 1 casts the meshes alone and PASS 2 the
// convex bodies, starting from PASS 1's hits (so the ground's hit culls what lies beyond it, and
// each instance carries one shape family's code).
template <int PASS, int MODE>
__global__ void __launch_bounds__(128) k_cast_rays(DevWorld w, const int2 *node_world, const DevRay *rays,
                                                   const int *order, int nr, DevRayFilter flt, DevRayHit *hits,
                                                   int cap, int *counts) {
    const int n = w.n;
    const HullView hv = hull_view(w);
    const float INITIAL = 1.f + 1e-4f;  // INITIAL_EARLY_OUT_FRACTION cast-utils.ts:3
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nr; k += gridDim.x * blockDim.x) {
        const int r = order ? order[k] : k;
        const DevRay ry = rays[r];
        const float3 o = f3(ry.origin[0], ry.origin[1], ry.origin[2]);
        const float3 d = f3(ry.direction[0], ry.direction[1], ry.direction[2]);
        const float len = ry.length;
        const int wr = ry.world;
        float best = INITIAL;
        int hit = -1;
        uint32_t hsub = 0xffffffffu;
        int cnt = 0;
        DevRayHit *out = hits + (size_t)r * (MODE == COLLECT_ALL ? cap : 1);
        if (PASS == 2) {
            if (MODE == COLLECT_CLOSEST) {
                const DevRayHit h0 = hits[r];
                if (h0.body >= 0) {
                    best = h0.fraction;
                    hit = h0.body;
                    hsub = h0.sub_shape_id;
                }
            } else {
                cnt = counts[r];
                if (MODE == COLLECT_ANY && cnt > 0) continue;  // PASS 1 found one
            }
        }
        // ANY: the hit ends the walk (SHOULD_EARLY_OUT_FRACTION); ALL: appended while room is left
        auto add = [&](int b, float f, uint32_t sub) {
            if (MODE == COLLECT_ALL && cnt < cap) {
                DevRayHit h;
                h.body = b;
                h.fraction = f;
                h.sub_shape_id = sub;
                h.pad = 0;
                out[cnt] = h;
            }
            if (MODE == COLLECT_ANY) {
                hit = b;
                best = f;
                hsub = sub;
            }
            cnt++;
        };
        if (n > 0 && wr >= 0 && wr < w.num_worlds && len > 0.f) {
            // Nearer child first, and a subtree whose box the ray enters beyond the best hit (by more
            // than twice the GJK tolerance, 1e-3 m) is skipped: a shape lies inside its box, so no hit
            // in it can come first.  The reference casts every body whose box the segment enters; the
            // least fraction is the same.  ANY and ALL keep the initial early-out fraction.
            int stack[CCD_STACK];
            float sdist[CCD_STACK];
            int sp = 0;
            const float t_root = ray_box_entry(o, d, len, xyz(w.node_lo[0]), xyz(w.node_hi[0]));
            if (t_root < CUDART_INF_F) {
                stack[sp] = 0;
                sdist[sp++] = t_root;
            }
            while (sp > 0) {
                if (MODE == COLLECT_ANY && cnt > 0) break;
                --sp;
                const int node = stack[sp];
                if (sdist[sp] > best * len + 2e-3f) continue;
                const int2 nw = node_world[node];
                if (wr < nw.x || wr > nw.y) continue;
                if (node < n - 1) {
                    const int2 ch = w.node_child[node];
                    const float tl = ray_box_entry(o, d, len, xyz(w.node_lo[ch.x]), xyz(w.node_hi[ch.x]));
                    const float tr = ray_box_entry(o, d, len, xyz(w.node_lo[ch.y]), xyz(w.node_hi[ch.y]));
                    if (sp + 2 > CCD_STACK) {
                        atomicOr(&w.ctr->overflow, OVF_SLOTS);
                        continue;
                    }
                    const int far_n = tl <= tr ? ch.y : ch.x, near_n = tl <= tr ? ch.x : ch.y;
                    const float far_t = fmaxf(tl, tr), near_t = fminf(tl, tr);
                    if (far_t < CUDART_INF_F) {
                        stack[sp] = far_n;
                        sdist[sp++] = far_t;
                    }
                    if (near_t < CUDART_INF_F) {
                        stack[sp] = near_n;
                        sdist[sp++] = near_t;
                    }
                    continue;
                }
                const int b = w.order[node - (n - 1)];
                if (w.world[b] != wr) continue;
                const uint32_t fb = w.flags[b];
                if (!(flt.layer_mask & (1u << layer_of(fb)))) continue;
                const uint2 gb = w.groups[b];
                if (!((flt.groups & gb.y) != 0u && (gb.x & flt.mask) != 0u)) continue;
                const bool is_mesh = shape_of(fb) == SHAPE_MESH;
                if (is_mesh ? PASS == 2 : PASS == 1) continue;
                float f;
                uint32_t sub;
                if (MODE != COLLECT_CLOSEST) {
                    if (is_mesh) {  // every triangle hit (AnyCastRayCollector / AllCastRayCollector)
                        float3 pB;
                        float4 qB;
                        geom_pose(w, b, fb, pB, qB);
                        float early = INITIAL;
                        ray_mesh_walk(w, b, qrot_inv(qB, o - pB), qrot_inv(qB, d), len,
                                      !(flt.flags & CC_RAY_BACKFACES), early, [&](float fh, uint32_t sh) {
                                          add(b, fh, sh);
                                          if (MODE == COLLECT_ANY) early = 0.f;
                                      });
                    } else if (shape_of(fb) == SHAPE_COMPOUND) {  // one hit per child (castRayVsCompound)
                        const int nc = sub_count(w, b, fb);
                        for (int i = 0; i < nc; i++) {
                            if (MODE == COLLECT_ANY && cnt > 0) break;
                            const SubShape cs = sub_shape(w, b, fb, i);
                            if (ray_vs_convex(hv, cs.shape, cs.sp, cs.pos, cs.quat, o, d, len, flt.flags, INITIAL, f))
                                add(b, f, cs.sub);
                        }
                    } else if (ray_vs_body<false>(w, hv, b, o, d, len, flt.flags, INITIAL, f, sub)) {
                        add(b, f, sub);
                    }
                    continue;
                }
                // a later-found body of lower index may still take an equal fraction
                const float max_f = (hit >= 0 && b < hit) ? nextafterf(best, CUDART_INF_F) : best;
                const bool ok = is_mesh ? ray_vs_body<true>(w, hv, b, o, d, len, flt.flags, max_f, f, sub)
                                        : ray_vs_body<false>(w, hv, b, o, d, len, flt.flags, max_f, f, sub);
                if (!ok) continue;
                if (f < best || (f == best && b < hit)) {
                    best = f;
                    hit = b;
                    hsub = sub;
                }
            }
        }
        if (MODE != COLLECT_CLOSEST) counts[r] = cnt;
        if (MODE == COLLECT_ALL) continue;
        DevRayHit h;
        h.body = hit;
        h.fraction = hit >= 0 ? best : 1.f;
        h.sub_shape_id = hsub;
        h.pad = 0;
        out[0] = h;
    }
}

// ---------------------------------------------------------------------------
// world queries: collidePoint (query.ts:470-490) with every hit collected
// ---------------------------------------------------------------------------
// the odd-even count of collidePointVsTriangleMesh triangle-mesh.ts:482-570: a +Y ray from the
// point, 1.1 x the mesh height long, back faces counted, every hit kept (hitCountCollector
// :441-467 never lowers its early-out fraction); last = the last hit's sub-shape id in walk order
__device__ int mesh_ray_hit_count(const DevWorld &w, const DevMesh &M, float3 o, float len, uint32_t &last) {
    const float early = 1.f + 1e-4f;
    const float3 d = f3(0.f, 1.f, 0.f);
    const float4 *nodes = w.mesh_nodes + 2 * M.first_node;
    int stack[MESH_STACK];
    float sdist[MESH_STACK];
    int sp = 0, count = 0;
    stack[sp] = 0;
    sdist[sp++] = -CUDART_INF_F;
    while (sp > 0) {
        --sp;
        const int node = stack[sp];
        if (sdist[sp] >= early) continue;
        const float4 nlo = nodes[2 * node], nhi = nodes[2 * node + 1];
        const int aux = __float_as_int(nlo.w), tag = __float_as_int(nhi.w);
        if (tag < 0) {
            for (int ti = aux; ti < aux + (-tag - 1); ti++) {
                const int4 tr = w.mesh_tris[M.first_tri + ti];
                float f;
                if (ray_triangle(o, d, len, xyz(w.mesh_verts[tr.x]), xyz(w.mesh_verts[tr.y]), xyz(w.mesh_verts[tr.z]),
                                 false, f) &&
                    f < early) {
                    count++;
                    last = M.sub_bits >= 32 ? (uint32_t)ti : ((0xffffffffu & ~((1u << M.sub_bits) - 1u)) | (uint32_t)ti);
                }
            }
            continue;
        }
        const int left = node + 1, right = aux;
        const float ld = ray_fraction_to_box(o, d, len, xyz(nodes[2 * left]), xyz(nodes[2 * left + 1]));
        const float rd = ray_fraction_to_box(o, d, len, xyz(nodes[2 * right]), xyz(nodes[2 * right + 1]));
        if (sp + 2 > MESH_STACK) {
            atomicOr(&w.ctr->overflow, OVF_SLOTS);
            continue;
        }
        if (ld <= rd) {
            if (rd < early) { stack[sp] = right; sdist[sp++] = rd; }
            if (ld < early) { stack[sp] = left; sdist[sp++] = ld; }
        } else {
            if (ld < early) { stack[sp] = left; sdist[sp++] = ld; }
            if (rd < early) { stack[sp] = right; sdist[sp++] = rd; }
        }
    }
    return count;
}

// collidePointVsShape of one convex shape at (pB, qB): sphere.ts:272-301 (distance), box.ts:370-410
// (half extents), convex.ts:142-216 (local bounds, then GJK of the INCLUDE_CONVEX_RADIUS support
// against the point with the query's collision tolerance)
__device__ bool point_in_convex(const HullView &hv, int shape, float4 sp, float3 pB, float4 qB, float3 p, float tol) {
    const float3 l = p - pB;
    if (shape == SHAPE_SPHERE) return lensq3(l) <= sp.x * sp.x;
    const float3 lp = qrot_inv(qB, l);
    if (shape == SHAPE_BOX) return fabsf(lp.x) <= sp.x && fabsf(lp.y) <= sp.y && fabsf(lp.z) <= sp.z;
    float3 lo, hi;  // the shape's local bounds: capsule.ts computeCapsuleAABB, the hull's points
    if (shape == SHAPE_HULL) {
        const DevHull &h = hv.hulls[hull_of(sp)];
        lo = xyz(h.lo);
        hi = xyz(h.hi);
    } else if (shape == SHAPE_CYLINDER) {  // cylinder.ts calculateAABB
        lo = f3(-sp.y, -sp.x, -sp.y);
        hi = f3(sp.y, sp.x, sp.y);
    } else {
        const float th = sp.y + sp.x;
        lo = f3(-sp.x, -th, -sp.x);
        hi = f3(sp.x, th, sp.x);
    }
    if (lp.x < lo.x || lp.x > hi.x || lp.y < lo.y || lp.y > hi.y || lp.z < lo.z || lp.z > hi.z) return false;
    const Sup<float> A = make_sup<float>(shape, sp, false, hv);
    Sup<float> P = make_sup<float>(SHAPE_SPHERE, make_float4(0.f, 0.f, 0.f, 0.f), true, hv);
    set_transform(P, Q<float>{0.f, 0.f, 0.f, 1.f}, V<float>{lp.x, lp.y, lp.z});
    V<float> dir{lp.x, lp.y, lp.z};
    if (lsq(dir) < 1e-10f) dir = V<float>{0.f, 1.f, 0.f};
    Simplex<float> sx;
    sx.size = 0;
    const GjkOut<float> g = gjk(A, P, tol, dir, 0.f, sx);
    return g.sqdist <= tol * tol;
}

// collidePointVsShape for one body: the convex shapes above, the plane (plane.ts:404-460), a
// compound's first child holding the point (compound.ts:423-492), triangle-mesh.ts:482-570 (local
// bounds, odd-even count)
__device__ bool point_in_body(const DevWorld &w, const HullView &hv, int b, float3 p, float tol, uint32_t &sub) {
    sub = 0xffffffffu;
    const uint32_t fb = w.flags[b];
    const float4 sp = w.shape[b];
    float3 pB;
    float4 qB;
    geom_pose(w, b, fb, pB, qB);
    const int shape = shape_of(fb);
    if (shape == SHAPE_EMPTY) return false;
    if (shape == SHAPE_PLANE) {  // collidePointVsPlane plane.ts:404-460
        float3 n;
        float c;
        plane_world(sp, pB, qB, n, c);
        return dot3(n, p) + c < 0.f;
    }
    if (shape == SHAPE_COMPOUND) {
        const int nc = sub_count(w, b, fb);
        for (int i = 0; i < nc; i++) {
            const SubShape cs = sub_shape(w, b, fb, i);
            if (point_in_convex(hv, cs.shape, cs.sp, cs.pos, cs.quat, p, tol)) {
                sub = cs.sub;
                return true;
            }
        }
        return false;
    }
    if (shape == SHAPE_MESH) {
        const float3 lp = qrot_inv(qB, p - pB);
        const DevMesh &M = w.meshes[mesh_of(sp)];
        if (M.num_tris == 0) return false;
        if (lp.x < M.lo.x || lp.x > M.hi.x || lp.y < M.lo.y || lp.y > M.hi.y || lp.z < M.lo.z || lp.z > M.hi.z)
            return false;
        uint32_t last = 0xffffffffu;
        if ((mesh_ray_hit_count(w, M, lp, (M.hi.y - M.lo.y) * 1.1f, last) & 1) == 0) return false;
        sub = last;
        return true;
    }
    return point_in_convex(hv, shape, sp, pB, qB, p, tol);
}

// broadphase.intersectPoint / dbvt.intersectPoint (broadphase.ts:314-324, dbvt.ts:683-740) over the
// world's subtree: every body whose box holds the point and that passes the filter is tested;
// the hit count, and the lowest body index among the hits with its sub-shape id
__global__ void __launch_bounds__(128) k_collide_points(DevWorld w, const int2 *node_world, const float4 *pts, int np,
                                                        DevRayFilter flt, float tol, int4 *out) {
    const int n = w.n;
    const HullView hv = hull_view(w);
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < np; r += gridDim.x * blockDim.x) {
        const float4 q = pts[r];
        const float3 p = xyz(q);
        const int wr = __float_as_int(q.w);
        int count = 0, first = -1;
        uint32_t fsub = 0xffffffffu;
        if (n > 0 && wr >= 0 && wr < w.num_worlds) {
            int stack[CCD_STACK];
            int sp = 0;
            stack[sp++] = 0;
            while (sp > 0) {
                const int node = stack[--sp];
                const int2 nw = node_world[node];
                if (wr < nw.x || wr > nw.y) continue;
                const float4 lo = w.node_lo[node], hi = w.node_hi[node];
                if (p.x < lo.x || p.x > hi.x || p.y < lo.y || p.y > hi.y || p.z < lo.z || p.z > hi.z) continue;
                if (node < n - 1) {
                    const int2 ch = w.node_child[node];
                    if (sp + 2 <= CCD_STACK) {
                        stack[sp++] = ch.y;
                        stack[sp++] = ch.x;
                    } else {
                        atomicOr(&w.ctr->overflow, OVF_SLOTS);
                    }
                    continue;
                }
                const int b = w.order[node - (n - 1)];
                if (w.world[b] != wr) continue;
                const uint32_t fb = w.flags[b];
                if (!(flt.layer_mask & (1u << layer_of(fb)))) continue;
                const uint2 gb = w.groups[b];
                if (!((flt.groups & gb.y) != 0u && (gb.x & flt.mask) != 0u)) continue;
                uint32_t sub;
                if (!point_in_body(w, hv, b, p, tol, sub)) continue;
                count++;
                if (first < 0 || b < first) {
                    first = b;
                    fsub = sub;
                }
            }
        }
        out[r] = make_int4(count, first, (int)fsub, 0);
    }
}

void launch_collide_points(DevWorld &w, const float4 *pts, int np, const DevRayFilter &f, float tol, int4 *out,
                           cudaStream_t s) {
    if (np <= 0) return;
    k_collide_points<<<grid_for(np, 128, 16), 128, 0, s>>>(w, w.node_world, pts, np, f, tol, out);
}

// ---------------------------------------------------------------------------
// world queries: castShape (query.ts:196-214) with the closest-hit collector
// (ClosestCastShapeCollector cast-shape-vs-shape.ts:199-217), default cast settings
// ---------------------------------------------------------------------------
// broadphase.castAABB (broadphase.ts:327-345) of the cast shape's start box along the
// displacement over the world's subtree, nearer child first and subtrees beyond the best hit
// skipped; castShapeVsShape per body: castConvexVsConvexLocal convex.ts:744-830 (EXCLUDE supports,
// tolerance 1e-4, back faces dropped), or for a mesh the sphere's own cast or
// castConvexVsTriangleMesh (ccd_cast_mesh, the same default settings).
// PASS 0 casts every body; with meshes present PASS 1 casts the meshes and PASS 2 the convex
// bodies from PASS 1's hits, as the ray queries do.  MODE picks the collector of
// cast-shape-vs-shape.ts:165-226 as for the rays: the closest hit, the first hit found, or every
// hit (one per convex body, one per mesh triangle) appended to hits[k * cap ...].
template <int PASS, int MODE>
__global__ void __launch_bounds__(128, 4) k_cast_shapes(DevWorld w, const int2 *node_world, const DevShapeCast *qs,
                                                     int nq, DevRayFilter flt, DevShapeCastHit *hits, int cap,
                                                     int *counts) {
    const int n = w.n;
    const HullView hv = hull_view(w);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nq; k += gridDim.x * blockDim.x) {
        const DevShapeCast q = qs[k];
        const int shape = q.shape_type;
        const float4 sa = make_float4(q.params[0], q.params[1], q.params[2], q.params[3]);
        const uint32_t fa = shape_bits(shape);
        const float3 pA = f3(q.position[0], q.position[1], q.position[2]);
        const float4 qA = make_float4(q.quaternion[0], q.quaternion[1], q.quaternion[2], q.quaternion[3]);
        const float3 disp = f3(q.displacement[0], q.displacement[1], q.displacement[2]);
        const int wr = q.world;
        float best = 1.f + 1e-4f;  // INITIAL_EARLY_OUT_FRACTION cast-utils.ts:3
        const float INITIAL = best;
        int hit = -1;
        uint32_t hsub = 0xffffffffu;
        float3 hn = f3(0.f, 0.f, 0.f), hp = f3(0.f, 0.f, 0.f);
        int cnt = 0;
        DevShapeCastHit *out = hits + (size_t)k * (MODE == COLLECT_ALL ? cap : 1);
        if (PASS == 2) {
            if (MODE == COLLECT_CLOSEST) {
                const DevShapeCastHit h0 = hits[k];
                if (h0.body >= 0) {
                    hit = h0.body;
                    best = h0.fraction;
                    hn = f3(h0.normal[0], h0.normal[1], h0.normal[2]);
                    hp = f3(h0.point[0], h0.point[1], h0.point[2]);
                    hsub = h0.sub_shape_id;
                }
            } else {
                cnt = counts[k];
                if (MODE == COLLECT_ANY && cnt > 0) continue;  // PASS 1 found one
            }
        }
        // the early-out fraction of the ANY and ALL collectors: the initial one, 0 after ANY's hit
        float early = INITIAL;
        const bool valid = query_shape_ok(w, shape, sa);
        if (valid && n > 0 && wr >= 0 && wr < w.num_worlds) {
            // the start box: the local bounds through the pose (box3.transformMat4 query.ts:206-208)
            float3 llo, lhi;
            convex_local_bounds(w, fa, sa, llo, lhi);
            const float3 hl = (lhi - llo) * 0.5f, centre = pA + qrot(qA, (lhi + llo) * 0.5f);
            const float3 ex = qrot(qA, f3(1.f, 0.f, 0.f)), ey = qrot(qA, f3(0.f, 1.f, 0.f)),
                         ez = qrot(qA, f3(0.f, 0.f, 1.f));
            const float3 half = f3(fabsf(ex.x) * hl.x + fabsf(ey.x) * hl.y + fabsf(ez.x) * hl.z,
                                   fabsf(ex.y) * hl.x + fabsf(ey.y) * hl.y + fabsf(ez.y) * hl.z,
                                   fabsf(ex.z) * hl.x + fabsf(ey.z) * hl.y + fabsf(ez.z) * hl.z);
            const float clen = sqrtf(lensq3(disp));
            const float3 cdir = clen > 0.f ? disp * (1.f / clen) : f3(0.f, 0.f, 0.f);
            const Sup<float> supA0 = make_sup<float>(shape, sa, true, hv);
            auto entry = [&](int node) {
                return ray_box_entry(centre, cdir, clen, xyz(w.node_lo[node]) - half, xyz(w.node_hi[node]) + half);
            };
            int stack[CCD_STACK];
            float sdist[CCD_STACK];
            int sp = 0;
            const float t_root = entry(0);
            if (t_root < CUDART_INF_F) {
                stack[sp] = 0;
                sdist[sp++] = t_root;
            }
            while (sp > 0) {
                if (MODE == COLLECT_ANY && cnt > 0) break;
                --sp;
                const int node = stack[sp];
                if (sdist[sp] > best * clen + 2e-2f) continue;  // beyond the best hit by twice the mesh tolerance
                const int2 nw = node_world[node];
                if (wr < nw.x || wr > nw.y) continue;
                if (node < n - 1) {
                    const int2 ch = w.node_child[node];
                    const float tl = entry(ch.x), tr = entry(ch.y);
                    if (sp + 2 > CCD_STACK) {
                        atomicOr(&w.ctr->overflow, OVF_SLOTS);
                        continue;
                    }
                    const int far_n = tl <= tr ? ch.y : ch.x, near_n = tl <= tr ? ch.x : ch.y;
                    const float far_t = fmaxf(tl, tr), near_t = fminf(tl, tr);
                    if (far_t < CUDART_INF_F) {
                        stack[sp] = far_n;
                        sdist[sp++] = far_t;
                    }
                    if (near_t < CUDART_INF_F) {
                        stack[sp] = near_n;
                        sdist[sp++] = near_t;
                    }
                    continue;
                }
                const int b = w.order[node - (n - 1)];
                if (w.world[b] != wr) continue;
                const uint32_t fb = w.flags[b];
                if (!(flt.layer_mask & (1u << layer_of(fb)))) continue;
                const uint2 gb = w.groups[b];
                if (!((flt.groups & gb.y) != 0u && (gb.x & flt.mask) != 0u)) continue;
                auto collect = [&](float lambda, float3 paw, float3 axw, uint32_t sub = 0xffffffffu) {
                    if (MODE != COLLECT_CLOSEST) {
                        if (!(lambda < early)) return;
                        if (MODE == COLLECT_ANY) early = 0.f;  // SHOULD_EARLY_OUT_FRACTION
                        if (MODE == COLLECT_ALL && cnt >= cap) {
                            cnt++;
                            return;
                        }
                        DevShapeCastHit h;
                        h.body = b;
                        h.fraction = lambda;
                        const float3 nn = -normalize3(axw);
                        h.normal[0] = nn.x, h.normal[1] = nn.y, h.normal[2] = nn.z;
                        h.point[0] = paw.x, h.point[1] = paw.y, h.point[2] = paw.z;
                        h.sub_shape_id = sub;
                        h.pad = 0;
                        out[MODE == COLLECT_ALL ? cnt : 0] = h;
                        cnt++;
                        return;
                    }
                    if (!(lambda < best || (lambda == best && hit >= 0 && b < hit))) return;
                    best = lambda;
                    hit = b;
                    hsub = sub;
                    hn = -normalize3(axw);
                    hp = paw;
                };
                const float &limit = MODE == COLLECT_CLOSEST ? best : early;
                if (shape_of(fb) == SHAPE_EMPTY) continue;
                if (shape_of(fb) == SHAPE_MESH) {
                    if (PASS != 2) ccd_cast_mesh(w, fa, sa, pA, qA, disp, b, limit, collect);
                    continue;
                }
                if (shape_of(fb) == SHAPE_PLANE) {
                    if (PASS == 1) continue;
                    float3 pB, paw, axw;
                    float4 qB;
                    float frac;
                    geom_pose(w, b, fb, pB, qB);
                    const Sup<float> S = make_sup<float>(shape, sa, default_excludes(shape), hv);
                    if (cast_vs_plane(S, pA, qA, disp, w.shape[b], pB, qB, limit, frac, paw, axw)) collect(frac, paw, axw);
                    continue;
                }
                if (PASS == 1) continue;
                // a convex body, or a compound child by child (castShapeVsCompound compound.ts:776-866)
                const int nsub = sub_count(w, b, fb);
                for (int ci = 0; ci < nsub; ci++) {
                    if (MODE == COLLECT_ANY && cnt > 0) break;
                    const SubShape cs = sub_shape(w, b, fb, ci);
                    const float3 pB = cs.pos;
                    const float4 qB = cs.quat;
                    const Q<float> iqB{-qB.x, -qB.y, -qB.z, qB.w};
                    const V<float> posAInB = qrotS(iqB, V<float>{pA.x - pB.x, pA.y - pB.y, pA.z - pB.z});
                    const Q<float> qAInB = qmulS(iqB, Q<float>{qA.x, qA.y, qA.z, qA.w});
                    const V<float> dInB = qrotS(iqB, V<float>{disp.x, disp.y, disp.z});
                    Sup<float> supA = supA0;
                    set_transform(supA, qAInB, posAInB);
                    const Sup<float> supB = make_sup<float>(cs.shape, cs.sp, true, hv);
                    const float max_l = MODE != COLLECT_CLOSEST ? early
                                        : (hit >= 0 && b < hit) ? nextafterf(best, CUDART_INF_F)
                                                                : best;
                    float lambda;
                    V<float> cpa, cpb, ax;
                    if (!gjk_cast(lambda, cpa, cpb, ax, supA, supB, dInB, 1e-4f, supA.convex_radius,
                                  supB.convex_radius, max_l))
                        continue;
                    // penetrationCastShape penetration.ts:693-698: a too short axis becomes the cast direction
                    if (lsq(ax) < 1e-4f * 1e-4f) ax = dInB;
                    if (lambda > 1.f || dot(ax, dInB) <= 0.f || lambda >= max_l) continue;
                    const Q<float> qBq{qB.x, qB.y, qB.z, qB.w};
                    const V<float> axw = qrotS(qBq, ax);
                    const V<float> paw = qrotS(qBq, cpa);
                    collect(lambda, f3(paw.x + pB.x, paw.y + pB.y, paw.z + pB.z), f3(axw.x, axw.y, axw.z), cs.sub);
                }
            }
        }
        if (MODE != COLLECT_CLOSEST) counts[k] = cnt;
        if (MODE == COLLECT_ALL || (MODE == COLLECT_ANY && cnt > 0)) continue;
        DevShapeCastHit h;
        h.body = hit;
        h.fraction = hit >= 0 ? best : 1.f;
        h.normal[0] = hn.x, h.normal[1] = hn.y, h.normal[2] = hn.z;
        h.point[0] = hp.x, h.point[1] = hp.y, h.point[2] = hp.z;
        h.sub_shape_id = hit >= 0 ? hsub : 0xffffffffu;
        h.pad = 0;
        out[0] = h;
    }
}

// ---------------------------------------------------------------------------
// world queries: collideShape (query.ts:286-311) with the closest, any and all-hit collectors
// (ClosestCollideShapeCollector, AnyCollideShapeCollector, AllCollideShapeCollector,
// collide-shape-vs-shape.ts:82-176)
// ---------------------------------------------------------------------------
// penetrationDepthStepEPA (penetration.ts:214-614) from an FP64 GJK simplex on one thread's
// polytope.  A collide query runs GJK in FP64 as well (the query is no hot path), so EPA starts
// from the simplex the FP64 restatement reaches: on a flat Minkowski difference (a box through a
// triangle) EPA can stop on a different face when started elsewhere.
template <class SB>
__device__ bool query_epa(EpaScratch *slot, const Simplex<R> &sx, const Sup<R> &A, const SB &B, R tol,
                          V<R> &axis, V<R> &pa, V<R> &pb) {
    Hull<BigStore> h;
    h.st.s = slot;
    h.start(sx);
    return epa(h, A, B, tol, axis, pa, pb);
}


// collideConvexVsTriangleMesh triangle-mesh.ts:1140-1386 / collideSphereVsTriangleMesh
// :1418-1712 of the query shape A at (pA, qA) against mesh body b at (pB, qB), no movement
// direction (active edges take the triangle normal): every triangle hit through add
template <class Add>
__device__ bool collide_query_mesh(const DevWorld &w, const HullView &hv, EpaScratch *slot, int shA, float4 sa,
                                   float3 pA, float4 qA4, int b, float3 pB, float4 qB4, const DevCollideSettings &cs,
                                   Add &&add) {
    const DevMesh &M = w.meshes[mesh_of(w.shape[b])];
    if (M.num_tris == 0) return true;
    const float ms = cs.max_separation;
    const Q<float> qA{qA4.x, qA4.y, qA4.z, qA4.w}, iqA{-qA4.x, -qA4.y, -qA4.z, qA4.w};
    const Q<float> qM{qB4.x, qB4.y, qB4.z, qB4.w}, iqM{-qB4.x, -qB4.y, -qB4.z, qB4.w};
    const Q<float> cInM = qmulS(iqM, qA);
    const V<float> cInMPos = qrotS(iqM, V<float>{pA.x - pB.x, pA.y - pB.y, pA.z - pB.z});
    const bool sphere = shA == SHAPE_SPHERE;
    float3 qlo, qhi, qcenter, blo1 = f3(0.f, 0.f, 0.f), bhi1 = f3(0.f, 0.f, 0.f);
    if (sphere) {
        const float er = sa.x + ms;
        qcenter = f3(cInMPos.x, cInMPos.y, cInMPos.z);
        qlo = qcenter - f3(er, er, er);
        qhi = qcenter + f3(er, er, er);
    } else {
        float3 llo, lhi;
        convex_local_bounds(w, shape_bits(shA), sa, llo, lhi);
        blo1 = llo - f3(ms, ms, ms);
        bhi1 = lhi + f3(ms, ms, ms);
        qlo = f3(3.0e38f, 3.0e38f, 3.0e38f);
        qhi = f3(-3.0e38f, -3.0e38f, -3.0e38f);
        for (int c = 0; c < 8; c++) {
            V<float> p{(c & 1) ? lhi.x : llo.x, (c & 2) ? lhi.y : llo.y, (c & 4) ? lhi.z : llo.z};
            V<float> q = qrotS(cInM, p) + cInMPos;
            qlo = f3(fminf(qlo.x, q.x), fminf(qlo.y, q.y), fminf(qlo.z, q.z));
            qhi = f3(fmaxf(qhi.x, q.x), fmaxf(qhi.y, q.y), fmaxf(qhi.z, q.z));
        }
        qlo = qlo - f3(ms, ms, ms);
        qhi = qhi + f3(ms, ms, ms);
        qcenter = (qlo + qhi) * 0.5f;
    }
    Sup<R> supA;
    if (!sphere) supA = make_sup<R>(shA, sa, true, hv);
    const Q<R> m2cR = qmulS(Q<R>{R(-qA4.x), R(-qA4.y), R(-qA4.z), R(qA4.w)}, Q<R>{R(qB4.x), R(qB4.y), R(qB4.z), R(qB4.w)});
    const V<R> m2cPosR = qrotS(Q<R>{R(-qA4.x), R(-qA4.y), R(-qA4.z), R(qA4.w)},
                               V<R>{R(pB.x) - R(pA.x), R(pB.y) - R(pA.y), R(pB.z) - R(pA.z)});
    int stack[MESH_STACK];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const int node = stack[--sp];
        const float4 nlo = w.mesh_nodes[2 * (M.first_node + node)], nhi = w.mesh_nodes[2 * (M.first_node + node) + 1];
        if (!node_hits_box(nlo, nhi, qlo, qhi)) continue;
        const int aux = __float_as_int(nlo.w), tag = __float_as_int(nhi.w);
        if (tag >= 0) {  // internal: the nearer child (centre to centre) first
            const int left = node + 1, right = aux;
            const float4 l0 = w.mesh_nodes[2 * (M.first_node + left)], l1 = w.mesh_nodes[2 * (M.first_node + left) + 1];
            const float4 r0 = w.mesh_nodes[2 * (M.first_node + right)],
                         r1 = w.mesh_nodes[2 * (M.first_node + right) + 1];
            const float ld = lensq3(qcenter - (xyz(l0) + xyz(l1)) * 0.5f);
            const float rd = lensq3(qcenter - (xyz(r0) + xyz(r1)) * 0.5f);
            if (sp + 2 > MESH_STACK) {
                atomicOr(&w.ctr->overflow, OVF_SLOTS);
                continue;
            }
            stack[sp++] = ld <= rd ? right : left;
            stack[sp++] = ld <= rd ? left : right;
            continue;
        }
        for (int ti = aux; ti < aux + (-tag - 1); ti++) {
            const int4 tr = w.mesh_tris[M.first_tri + ti];
            const float3 m0 = xyz(w.mesh_verts[tr.x]), m1 = xyz(w.mesh_verts[tr.y]), m2 = xyz(w.mesh_verts[tr.z]);
            const uint32_t tsub =
                M.sub_bits >= 32 ? (uint32_t)ti : ((0xffffffffu & ~((1u << M.sub_bits) - 1u)) | (uint32_t)ti);
            if (sphere) {  // in the mesh frame
                const float r = sa.x;
                const float3 c = qcenter;
                const float3 v0 = m0 - c, v1 = m1 - c, v2 = m2 - c;
                const float3 tn = cross3(v1 - v0, v2 - v0);
                const bool back = dot3(tn, v0) > 0.f;
                if (back && !cs.backfaces) continue;
                float dsq;
                int feature;
                const float3 p2 = closest_on_triangle(v0, v1, v2, dsq, feature);
                if (dsq > (r + ms) * (r + ms)) continue;
                const float pen = r - sqrtf(dsq);
                float3 ax = dsq > 0.f ? normalize3(p2) : f3(0.f, 1.f, 0.f);
                const float3 p1 = ax * r;
                const int feat_edges[8] = {0b000, 0b101, 0b011, 0b001, 0b110, 0b100, 0b010, 0b000};
                // an inactive edge or vertex: with no movement direction the triangle normal wins
                if (feature != 0b111 && tr.w != 0b111 && (tr.w & feat_edges[feature]) == 0) ax = back ? tn : -tn;
                auto to_w = [&](float3 v) {
                    V<float> q = qrotS(qM, V<float>{v.x, v.y, v.z});
                    return f3(q.x, q.y, q.z) + pB;
                };
                V<float> aw = qrotS(qM, V<float>{ax.x, ax.y, ax.z});
                if (!add(b, tsub, pen, to_w(c + p1), to_w(c + p2), normalize3(f3(aw.x, aw.y, aw.z)))) return false;
                continue;
            }
            // in the query shape's frame, FP64
            auto to_c = [&](float3 v) { return qrotS(m2cR, V<R>{R(v.x), R(v.y), R(v.z)}) + m2cPosR; };
            const V<R> T0 = to_c(m0), T1 = to_c(m1), T2 = to_c(m2);
            const V<R> tlo{fmin(T0.x, fmin(T1.x, T2.x)), fmin(T0.y, fmin(T1.y, T2.y)), fmin(T0.z, fmin(T1.z, T2.z))};
            const V<R> thi{fmax(T0.x, fmax(T1.x, T2.x)), fmax(T0.y, fmax(T1.y, T2.y)), fmax(T0.z, fmax(T1.z, T2.z))};
            if (!(tlo.x <= R(bhi1.x) && thi.x >= R(blo1.x) && tlo.y <= R(bhi1.y) && thi.y >= R(blo1.y) &&
                  tlo.z <= R(bhi1.z) && thi.z >= R(blo1.z)))
                continue;
            const V<R> tn = crs(T1 - T0, T2 - T0);
            const bool back = dot(tn, T0) > R(0);
            if (back && !cs.backfaces) continue;
            Sup<R, true, true> supT = make_sup<R, true, true>(SHAPE_SPHERE, make_float4(0.f, 0.f, 0.f, 0.f), false, hv);
            supT.kind = SUP_TRIANGLE;
            supT.r0 = T0;
            supT.r1 = T1;
            supT.r2 = T2;
            supT.convex_radius = R(0);
            V<R> axis{-tn.x, -tn.y, -tn.z};
            axis = lsq(axis) < R(1e-10) ? V<R>{R(1), R(0), R(0)} : axis * (R(1) / sq_root(lsq(axis)));
            const R rA = supA.convex_radius + R(ms);
            Simplex<R> sx;
            GjkOut<R> g = gjk(supA, supT, R(cs.collision_tol), axis, rA * rA, sx);
            if (g.sqdist > rA * rA) continue;  // NOT_COLLIDING
            V<R> pa, pb, pax;
            R pen;
            if (!(g.sqdist > R(0))) {  // INDETERMINATE: EPA
                const R msE = R(fminf(ms, 1.f));
                Sup<R> A = make_sup<R>(shA, sa, false, hv);
                A.add_r = msE;
                if (!query_epa(slot, sx, A, supT, R(cs.penetration_tol), pax, pa, pb)) continue;
                const V<R> dd = pa - pb;
                const R al = sq_root(lsq(pax));
                pen = sq_root(lsq(dd)) - msE;
                if (al > R(0)) pa = pa + pax * (-(msE / al));
            } else {  // COLLIDING: penetrationDepthStepGJK penetration.ts:84-106
                const R vl = sq_root(g.sqdist);
                pa = g.pa + g.axis * (rA / vl);
                pb = g.pb;
                pax = g.axis;
                const V<R> dd = pa - pb;
                pen = sq_root(lsq(dd)) - R(ms);
                const R al = sq_root(lsq(pax));
                if (al > R(0)) pa = pa + pax * (-(R(ms) / al));
            }
            if (tr.w != 0b111) {  // active edges: fixNormal with no movement direction
                auto f3r = [](V<R> v) { return f3((float)v.x, (float)v.y, (float)v.z); };
                const float3 tnf = f3r(tn);
                const float3 fixed = fix_normal(f3r(T0), f3r(T1), f3r(T2), back ? tnf : -tnf, tr.w, f3r(pb), f3r(pax),
                                                f3(0.f, 0.f, 0.f));
                pax = V<R>{R(fixed.x), R(fixed.y), R(fixed.z)};
            }
            const Q<R> qAr{R(qA4.x), R(qA4.y), R(qA4.z), R(qA4.w)};
            const V<R> paw = qrotS(qAr, pa), pbw = qrotS(qAr, pb), axw = qrotS(qAr, pax);
            if (!add(b, tsub, (float)pen, f3((float)paw.x, (float)paw.y, (float)paw.z) + pA,
                     f3((float)pbw.x, (float)pbw.y, (float)pbw.z) + pA,
                     normalize3(f3((float)axw.x, (float)axw.y, (float)axw.z))))
                return false;
        }
    }
    return true;
}

// collideShapeVsShape (narrowphase.ts:172-238) of the query shape A against one shape of body b
// (shB, sb at pB, qB; subB its sub-shape id): the hit(s) through add(body, sub-shape id,
// penetration, point on A, point on B, unit axis), all world space; false once add asks the walk
// to stop
template <class Add>
__device__ bool collide_query_shape(const DevWorld &w, const HullView &hv, EpaScratch *slot, int shA, float4 sa,
                                    float3 pA, float4 qA, int b, int shB, float4 sb, float3 pB, float4 qB,
                                    uint32_t subB, const DevCollideSettings &cs, Add &&add) {
    if (shB == SHAPE_EMPTY) return true;  // empty-shape.ts registers no collide function
    const float ms = cs.max_separation;
    if (shB == SHAPE_MESH) return collide_query_mesh(w, hv, slot, shA, sa, pA, qA, b, pB, qB, cs, add);
    if (shB == SHAPE_PLANE) {  // collideConvexVsPlane plane.ts:474-629, the plane in A's frame
        const float3 nl = qrot_inv(qA, qrot(qB, xyz(sb)));
        const float cl = sb.w - dot3(qrot_inv(qA, pB - pA), nl);
        const Sup<float> S = make_sup<float>(shA, sa, default_excludes(shA), hv);
        const V<float> spv = S.get(V<float>{-nl.x, -nl.y, -nl.z});
        const float3 sp3 = f3(spv.x, spv.y, spv.z);
        const float sd = dot3(nl, sp3) + cl, cr = S.convex_radius;
        const float pen = -sd + cr;
        if (!(pen > -ms)) return true;
        return add(b, subB, pen, pA + qrot(qA, sp3 - nl * cr), pA + qrot(qA, sp3 - nl * sd), qrot(qA, -nl));
    }
    if (shA == SHAPE_SPHERE && shB == SHAPE_SPHERE) {  // collideSphereVsSphere sphere.ts:319-410
        const float3 d = pB - pA;
        const float dsq = lensq3(d), rs = sa.x + sb.x;
        if (dsq >= rs * rs) return true;
        const float dist = sqrtf(dsq);
        const float3 nn = dist > 0.f ? d * (1.f / dist) : f3(0.f, 1.f, 0.f);
        return add(b, subB, rs - dist, pA + nn * sa.x, pB - nn * sb.x, nn);
    }
    // collideConvexVsConvex convex.ts:257-346: B in A's local frame, GJK and EPA in FP64
    const Q<R> qAr{R(qA.x), R(qA.y), R(qA.z), R(qA.w)}, iA{R(-qA.x), R(-qA.y), R(-qA.z), R(qA.w)};
    const Q<R> rel = qmulS(iA, Q<R>{R(qB.x), R(qB.y), R(qB.z), R(qB.w)});
    const V<R> posBInA = qrotS(iA, V<R>{R(pB.x) - R(pA.x), R(pB.y) - R(pA.y), R(pB.z) - R(pA.z)});
    const Sup<R> supA = make_sup<R>(shA, sa, true, hv);
    Sup<R> supB = make_sup<R>(shB, sb, true, hv);
    set_transform(supB, rel, posBInA);
    V<R> axis = posBInA;
    if (lsq(axis) <= R(1e-12)) axis = {R(1), R(0), R(0)};
    const R rA = supA.convex_radius + R(ms), rB = supB.convex_radius, cr = rA + rB;
    Simplex<R> sx;
    const GjkOut<R> g = gjk(supA, supB, R(cs.collision_tol), axis, cr * cr, sx);
    if (g.sqdist > cr * cr) return true;  // NOT_COLLIDING
    V<R> pa, pb, ax;
    R pen;
    if (!(g.sqdist > R(0))) {  // INDETERMINATE: EPA with the separation clamped to 1 (convex.ts:448)
        const R msE = R(fminf(ms, 1.f));
        Sup<R> A = make_sup<R>(shA, sa, false, hv);
        A.add_r = msE;
        Sup<R> B = make_sup<R>(shB, sb, false, hv);
        set_transform(B, rel, posBInA);
        if (!query_epa(slot, sx, A, B, R(cs.penetration_tol), ax, pa, pb)) return true;  // convex.ts:331
        const V<R> dd = pa - pb;
        const R al = sq_root(lsq(ax));
        pen = sq_root(lsq(dd)) - msE;
        if (al > R(0)) pa = pa + ax * (-(msE / al));
    } else {  // COLLIDING: penetrationDepthStepGJK penetration.ts:84-106
        const R vl = sq_root(g.sqdist);
        pa = g.pa + g.axis * (rA / vl);
        pb = g.pb + g.axis * (-(rB / vl));
        const V<R> dd = pa - pb;
        pen = sq_root(lsq(dd)) - R(ms);
        const R al = sq_root(lsq(g.axis));
        if (al > R(0)) pa = pa + g.axis * (-(R(ms) / al));
        ax = g.axis;
    }
    const V<R> paw = qrotS(qAr, pa), pbw = qrotS(qAr, pb), axw = qrotS(qAr, ax);
    return add(b, subB, (float)pen, f3((float)paw.x, (float)paw.y, (float)paw.z) + pA,
               f3((float)pbw.x, (float)pbw.y, (float)pbw.z) + pA,
               normalize3(f3((float)axw.x, (float)axw.y, (float)axw.z)));
}

// the query shape A against body b: each of a compound's children (collideShapeVsCompound
// compound.ts:580-678), else the body's own shape
template <class Add>
__device__ bool collide_query_body(const DevWorld &w, const HullView &hv, EpaScratch *slot, int shA, float4 sa,
                                   float3 pA, float4 qA, int b, const DevCollideSettings &cs, Add &&add) {
    const uint32_t fb = w.flags[b];
    const int nsub = sub_count(w, b, fb);
    for (int i = 0; i < nsub; i++) {
        const SubShape s = sub_shape(w, b, fb, i);
        if (!collide_query_shape(w, hv, slot, shA, sa, pA, qA, b, s.shape, s.sp, s.pos, s.quat, s.sub, cs, add))
            return false;
    }
    return true;
}

// broadphase.intersectAABB (broadphase.ts:300-312) of the query's box, grown by the separation
// distance, over the world's subtree; every body that passes the filter is collided with
// collideShapeVsShape into the collector:
//   COLLECT_CLOSEST: the deepest penetration (ties to the lower body index, then sub-shape id);
//   COLLECT_ANY: the first hit of the walk ends it;
//   COLLECT_ALL: every hit appended to hits[k * cap ...] while room is left.
// One EPA polytope per thread (the world's reference-limit EPA slots), so the grid is the slot count.
template <int MODE>
__global__ void __launch_bounds__(64) k_collide_shapes(DevWorld w, const int2 *node_world, const DevCollideShape *qs,
                                                       int nq, DevRayFilter flt, DevCollideSettings cs, int cap,
                                                       DevCollideHit *hits, int *counts) {
    const int n = w.n;
    const HullView hv = hull_view(w);
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    EpaScratch *slot = (EpaScratch *)w.epa_scratch + tid;
    for (int k = tid; k < nq; k += gridDim.x * blockDim.x) {
        const DevCollideShape q = qs[k];
        const int shA = q.shape_type;
        const float4 sa = make_float4(q.params[0], q.params[1], q.params[2], q.params[3]);
        const float3 pA = f3(q.position[0], q.position[1], q.position[2]);
        const float4 qA = make_float4(q.quaternion[0], q.quaternion[1], q.quaternion[2], q.quaternion[3]);
        const int wr = q.world;
        DevCollideHit best;
        best.body = -1;
        best.sub_shape_id = 0xffffffffu;
        best.penetration = 0.f;
        for (int c = 0; c < 3; c++) best.point_a[c] = best.point_b[c] = best.axis[c] = 0.f;
        int cnt = 0;
        DevCollideHit *out = hits + (size_t)k * (MODE == COLLECT_ALL ? cap : 1);
        auto add = [&](int b, uint32_t sub, float pen, float3 pa, float3 pb, float3 ax) -> bool {
            const bool take = MODE != COLLECT_CLOSEST || cnt == 0 || pen > best.penetration ||
                              (pen == best.penetration &&
                               (b < best.body || (b == best.body && sub < best.sub_shape_id)));
            if (take && !(MODE == COLLECT_ALL && cnt >= cap)) {
                DevCollideHit h;
                h.body = b;
                h.sub_shape_id = sub;
                h.penetration = pen;
                h.point_a[0] = pa.x, h.point_a[1] = pa.y, h.point_a[2] = pa.z;
                h.point_b[0] = pb.x, h.point_b[1] = pb.y, h.point_b[2] = pb.z;
                h.axis[0] = ax.x, h.axis[1] = ax.y, h.axis[2] = ax.z;
                if (MODE == COLLECT_ALL)
                    out[cnt] = h;
                else
                    best = h;
            }
            if (MODE == COLLECT_CLOSEST) {
                cnt = 1;
                return true;
            }
            cnt++;
            return MODE == COLLECT_ALL;
        };
        const bool valid = query_shape_ok(w, shA, sa);
        if (valid && n > 0 && wr >= 0 && wr < w.num_worlds) {
            // box3.transformMat4 of the local bounds, grown by the separation (query.ts:294-298)
            float3 llo, lhi;
            convex_local_bounds(w, shape_bits(shA), sa, llo, lhi);
            const float3 hl = (lhi - llo) * 0.5f, centre = pA + qrot(qA, (lhi + llo) * 0.5f);
            const float3 ex = qrot(qA, f3(1.f, 0.f, 0.f)), ey = qrot(qA, f3(0.f, 1.f, 0.f)),
                         ez = qrot(qA, f3(0.f, 0.f, 1.f));
            const float m = cs.max_separation;
            const float3 half = f3(fabsf(ex.x) * hl.x + fabsf(ey.x) * hl.y + fabsf(ez.x) * hl.z + m,
                                   fabsf(ex.y) * hl.x + fabsf(ey.y) * hl.y + fabsf(ez.y) * hl.z + m,
                                   fabsf(ex.z) * hl.x + fabsf(ey.z) * hl.y + fabsf(ez.z) * hl.z + m);
            const float3 lo = centre - half, hi = centre + half;
            auto overlaps = [&](int node) {
                const float4 a = w.node_lo[node], c = w.node_hi[node];
                return a.x <= hi.x && c.x >= lo.x && a.y <= hi.y && c.y >= lo.y && a.z <= hi.z && c.z >= lo.z;
            };
            int stack[CCD_STACK];
            int sp = 0;
            if (overlaps(0)) stack[sp++] = 0;
            bool go = true;
            while (sp > 0 && go) {
                const int node = stack[--sp];
                const int2 nw = node_world[node];
                if (wr < nw.x || wr > nw.y) continue;
                if (node < n - 1) {
                    const int2 ch = w.node_child[node];
                    if (sp + 2 > CCD_STACK) {
                        atomicOr(&w.ctr->overflow, OVF_SLOTS);
                        continue;
                    }
                    if (overlaps(ch.y)) stack[sp++] = ch.y;
                    if (overlaps(ch.x)) stack[sp++] = ch.x;
                    continue;
                }
                const int b = w.order[node - (n - 1)];
                if (w.world[b] != wr) continue;
                const uint32_t fb = w.flags[b];
                if (!(flt.layer_mask & (1u << layer_of(fb)))) continue;
                const uint2 gb = w.groups[b];
                if (!((flt.groups & gb.y) != 0u && (gb.x & flt.mask) != 0u)) continue;
                go = collide_query_body(w, hv, slot, shA, sa, pA, qA, b, cs, add);
            }
        }
        counts[k] = cnt;
        if (MODE != COLLECT_ALL) out[0] = best;
    }
}

// the first min(count, cap) hits of each query of an ALL collector in a fixed order (insertion sort)
template <class H, class Less>
__device__ void sort_hits(H *a, int m, Less less) {
    for (int i = 1; i < m; i++) {
        const H x = a[i];
        int j = i - 1;
        while (j >= 0 && less(x, a[j])) {
            a[j + 1] = a[j];
            j--;
        }
        a[j + 1] = x;
    }
}
__global__ void k_sort_ray_hits(DevRayHit *hits, const int *counts, int nq, int cap) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nq) return;
    sort_hits(hits + (size_t)k * cap, min(counts[k], cap), [](const DevRayHit &x, const DevRayHit &y) {
        if (x.fraction != y.fraction) return x.fraction < y.fraction;
        if (x.body != y.body) return x.body < y.body;
        return x.sub_shape_id < y.sub_shape_id;
    });
}
__global__ void k_sort_cast_hits(DevShapeCastHit *hits, const int *counts, int nq, int cap) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nq) return;
    sort_hits(hits + (size_t)k * cap, min(counts[k], cap), [](const DevShapeCastHit &x, const DevShapeCastHit &y) {
        if (x.fraction != y.fraction) return x.fraction < y.fraction;
        if (x.body != y.body) return x.body < y.body;
        return x.sub_shape_id < y.sub_shape_id;
    });
}
__global__ void k_sort_collide_hits(DevCollideHit *hits, const int *counts, int nq, int cap) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nq) return;
    sort_hits(hits + (size_t)k * cap, min(counts[k], cap), [](const DevCollideHit &x, const DevCollideHit &y) {
        if (x.body != y.body) return x.body < y.body;
        return x.sub_shape_id < y.sub_shape_id;
    });
}

void launch_collide_shapes(DevWorld &w, const DevCollideShape *qs, int nq, const DevRayFilter &f,
                           const DevCollideSettings &cs, int mode, int cap, DevCollideHit *hits, int *counts,
                           cudaStream_t s) {
    if (nq <= 0) return;
    const int blocks = std::min(EPA_BIG_THREADS, (nq + 63) / 64 * 64) / 64;  // one EPA slot per thread
    if (mode == COLLECT_ANY)
        k_collide_shapes<COLLECT_ANY><<<blocks, 64, 0, s>>>(w, w.node_world, qs, nq, f, cs, 1, hits, counts);
    else if (mode == COLLECT_ALL)
        k_collide_shapes<COLLECT_ALL><<<blocks, 64, 0, s>>>(w, w.node_world, qs, nq, f, cs, cap, hits, counts);
    else
        k_collide_shapes<COLLECT_CLOSEST><<<blocks, 64, 0, s>>>(w, w.node_world, qs, nq, f, cs, 1, hits, counts);
    if (mode == COLLECT_ALL) k_sort_collide_hits<<<(nq + 127) / 128, 128, 0, s>>>(hits, counts, nq, cap);
}

template <int MODE>
static void cast_shapes_mode(DevWorld &w, const DevShapeCast *qs, int nq, const DevRayFilter &f, DevShapeCastHit *hits,
                             int cap, int *counts, cudaStream_t s) {
    if (w.num_mesh_bodies > 0) {
        k_cast_shapes<1, MODE><<<grid_for(nq, 128, 16), 128, 0, s>>>(w, w.node_world, qs, nq, f, hits, cap, counts);
        k_cast_shapes<2, MODE><<<grid_for(nq, 128, 16), 128, 0, s>>>(w, w.node_world, qs, nq, f, hits, cap, counts);
    } else {
        k_cast_shapes<0, MODE><<<grid_for(nq, 128, 16), 128, 0, s>>>(w, w.node_world, qs, nq, f, hits, cap, counts);
    }
}
void launch_cast_shapes(DevWorld &w, const DevShapeCast *qs, int nq, const DevRayFilter &f, DevShapeCastHit *hits,
                        cudaStream_t s, int mode, int cap, int *counts) {
    if (nq <= 0) return;
    if (mode == COLLECT_ANY) {
        cast_shapes_mode<COLLECT_ANY>(w, qs, nq, f, hits, 1, counts, s);
    } else if (mode == COLLECT_ALL) {
        cast_shapes_mode<COLLECT_ALL>(w, qs, nq, f, hits, cap, counts, s);
        k_sort_cast_hits<<<(nq + 127) / 128, 128, 0, s>>>(hits, counts, nq, cap);
    } else {
        cast_shapes_mode<COLLECT_CLOSEST>(w, qs, nq, f, hits, 1, nullptr, s);
    }
}

template <int MODE>
static void cast_rays_mode(DevWorld &w, const DevRay *rays, const int *order, int nr, const DevRayFilter &f,
                           DevRayHit *hits, int cap, int *counts, cudaStream_t s) {
    if (w.num_mesh_bodies > 0) {
        k_cast_rays<1, MODE><<<grid_for(nr, 128, 16), 128, 0, s>>>(w, w.node_world, rays, order, nr, f, hits, cap,
                                                                  counts);
        k_cast_rays<2, MODE><<<grid_for(nr, 128, 16), 128, 0, s>>>(w, w.node_world, rays, order, nr, f, hits, cap,
                                                                  counts);
    } else {
        k_cast_rays<0, MODE><<<grid_for(nr, 128, 16), 128, 0, s>>>(w, w.node_world, rays, order, nr, f, hits, cap,
                                                                  counts);
    }
}
void launch_cast_rays(DevWorld &w, const DevRay *rays, const int *order, int nr, const DevRayFilter &f,
                      DevRayHit *hits, cudaStream_t s, int mode, int cap, int *counts) {
    if (nr <= 0) return;
    if (mode == COLLECT_ANY) {
        cast_rays_mode<COLLECT_ANY>(w, rays, order, nr, f, hits, 1, counts, s);
    } else if (mode == COLLECT_ALL) {
        cast_rays_mode<COLLECT_ALL>(w, rays, order, nr, f, hits, cap, counts, s);
        k_sort_ray_hits<<<(nr + 127) / 128, 128, 0, s>>>(hits, counts, nr, cap);
    } else {
        cast_rays_mode<COLLECT_CLOSEST>(w, rays, order, nr, f, hits, 1, nullptr, s);
    }
}

void launch_mesh_narrowphase(DevWorld &w, int pass, cudaStream_t s);

void launch_narrowphase(DevWorld &w, float, cudaStream_t s, cudaEvent_t mid) {
    EpaItem *items = (EpaItem *)w.epa_items;
    k_pair_order<0><<<grid_for(w.max_pairs, 256), 256, 0, s>>>(w);
    k_pair_order<1><<<grid_for(w.max_pairs, 256), 256, 0, s>>>(w);
    k_narrowphase<false><<<device_sm_count() * 8, 128, 0, s>>>(w, items);
    if (w.num_hulls > 0) k_narrowphase<true><<<device_sm_count() * 8, 128, 0, s>>>(w, items);
    if (w.num_mesh_bodies > 0) launch_mesh_narrowphase(w, 0, s);
    if (mid) cudaEventRecord(mid, s);
    if (w.num_hulls > 0) {
        k_epa<true><<<w.epa_threads / EPA_BLOCK, EPA_BLOCK, 0, s>>>(
            w, items, (PackedBlock *)w.epa_packed, w.epa_fallback, w.epa_packed_points, w.epa_fetch_warp);
        k_epa_big<true><<<EPA_BIG_THREADS / EPA_BLOCK, EPA_BLOCK, 0, s>>>(w, items, (EpaScratch *)w.epa_scratch,
                                                                          w.epa_fallback);
    } else {
        k_epa<false><<<w.epa_threads / EPA_BLOCK, EPA_BLOCK, 0, s>>>(
            w, items, (PackedBlock *)w.epa_packed, w.epa_fallback, w.epa_packed_points, w.epa_fetch_warp);
        k_epa_big<false><<<EPA_BIG_THREADS / EPA_BLOCK, EPA_BLOCK, 0, s>>>(w, items, (EpaScratch *)w.epa_scratch,
                                                                           w.epa_fallback);
    }
    k_epa_emit<false><<<device_sm_count() * 8, 128, 0, s>>>(w, items);
    if (w.num_hulls > 0) k_epa_emit<true><<<device_sm_count() * 8, 128, 0, s>>>(w, items);
    if (w.num_mesh_bodies > 0) {
        k_epa_mesh<<<EPA_BIG_THREADS / EPA_BLOCK, EPA_BLOCK, 0, s>>>(w, items, (EpaScratch *)w.epa_scratch);
        launch_mesh_narrowphase(w, 1, s);
    }
    if (w.num_compound_bodies > 0) k_compound_pairs<<<MESH_BIG_THREADS / 64, 64, 0, s>>>(w);
}

// ---------------------------------------------------------------------------
// Allocation-free penetration query (cc_penetration_static).  The same GJK and
// EPA device code as the world's narrowphase, run on caller-owned device
// buffers; the EPA polytopes and the queue of EPA items live in file-scope
// device arrays, so the call allocates nothing.
// ---------------------------------------------------------------------------
struct StaticQueue {
    int count;  // items queued by the GJK pass; cleared at the start of every call
    int pad[63];
};
static __device__ __align__(256) EpaScratch g_static_slots[CC_STATIC_EPA_SLOTS];
static __device__ __align__(256) EpaItem g_static_items[CC_STATIC_MAX_QUERIES];
static __device__ __align__(256) StaticQueue g_static_queue;

__device__ __forceinline__ void pose_of(const cc_shape_pose &s, float4 &pos, float4 &quat, float4 &prm) {
    pos = make_float4(s.position[0], s.position[1], s.position[2], 0.f);
    quat = make_float4(s.quaternion[0], s.quaternion[1], s.quaternion[2], s.quaternion[3]);
    prm = make_float4(s.shape_params[0], s.shape_params[1], s.shape_params[2], s.shape_params[3]);
}

__device__ __forceinline__ void write_hit(cc_penetration_result &r, float3 posA, float3 pa, float3 pb, float3 axis,
                                          float depth, int used_epa) {
    float3 n = normalize3(axis);
    r.hit = 1;
    r.normal[0] = n.x;
    r.normal[1] = n.y;
    r.normal[2] = n.z;
    r.depth = depth;
    r.point_a[0] = posA.x + pa.x;
    r.point_a[1] = posA.y + pa.y;
    r.point_a[2] = posA.z + pa.z;
    r.point_b[0] = posA.x + pb.x;
    r.point_b[1] = posA.y + pb.y;
    r.point_b[2] = posA.z + pb.z;
    r.used_epa = used_epa;
}

// GJK pass, one query per thread: the dispatch and GJK step of k_narrowphase;
// INDETERMINATE pairs are queued for the EPA pass.
__global__ void __launch_bounds__(128) k_static_gjk(const cc_penetration_query *qs, int n, cc_penetration_result *res,
                                                    EpaItem *items, StaticQueue *queue, float collision_tol) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const cc_penetration_query &qy = qs[i];
    cc_penetration_result r;
    r.hit = 0;
    r.normal[0] = r.normal[1] = r.normal[2] = 0.f;
    r.depth = 0.f;
    r.point_a[0] = r.point_a[1] = r.point_a[2] = 0.f;
    r.point_b[0] = r.point_b[1] = r.point_b[2] = 0.f;
    r.used_epa = 0;
    float4 pa4, pb4, qa, qb, sa, sb;
    pose_of(qy.a, pa4, qa, sa);
    pose_of(qy.b, pb4, qb, sb);
    int sha = qy.a.shape_type, shb = qy.b.shape_type;
    float maxSep = qy.max_separation;
    if (sha < SHAPE_SPHERE || sha > SHAPE_CAPSULE || shb < SHAPE_SPHERE || shb > SHAPE_CAPSULE) {
        // hulls and meshes keep their data in a world, and other values name no shape
        r.hit = CC_PENETRATION_UNSUPPORTED;
        res[i] = r;
        return;
    }
    if (sha == SHAPE_SPHERE && shb == SHAPE_SPHERE) {
        float3 d = xyz(pb4) - xyz(pa4);
        float dsq = lensq3(d);
        float rs = sa.x + sb.x;
        if (dsq < rs * rs) {
            float dist = sqrtf(dsq);
            float3 nn = dist > 0.f ? d * (1.f / dist) : f3(0.f, 1.f, 0.f);
            write_hit(r, xyz(pa4), nn * sa.x, d - nn * sb.x, nn, rs - dist, 0);
        }
        res[i] = r;
        return;
    }
    Q<float> qA{qa.x, qa.y, qa.z, qa.w}, qB{qb.x, qb.y, qb.z, qb.w};
    Q<float> iA{-qa.x, -qa.y, -qa.z, qa.w};
    Q<float> rel = qmulS(iA, qB);
    V<float> ab{pb4.x - pa4.x, pb4.y - pa4.y, pb4.z - pa4.z};
    V<float> posBInA = qrotS(iA, ab);
    const HullView none{nullptr, nullptr, nullptr};  // the static query takes no hull shapes
    Sup<float> supA = make_sup<float>(sha, sa, true, none);
    Sup<float> supB = make_sup<float>(shb, sb, true, none);
    set_transform(supB, rel, posBInA);
    V<float> axis = posBInA;
    if (lsq(axis) <= 1e-12f) axis = {1.f, 0.f, 0.f};
    float rA = supA.convex_radius + maxSep, rB = supB.convex_radius;
    float cr = rA + rB;
    Simplex<float> sx;
    GjkOut<float> g = gjk(supA, supB, collision_tol, axis, cr * cr, sx);
    if (g.sqdist > cr * cr) {
        res[i] = r;
        return;
    }
    if (!(g.sqdist > 0.f)) {
        // every query fits the queue (count <= CC_STATIC_MAX_QUERIES is checked on the host)
        int e = atomicAdd(&queue->count, 1);
        EpaItem it;
        it.a = i;
        it.b = i;
        it.size = sx.size;
        it.pad = 0;
        for (int k = 0; k < 4; k++) {
            SP<float> s = sx.pts[k < sx.size ? k : 0];
            it.y[k] = f3(s.y.x, s.y.y, s.y.z);
            it.p[k] = f3(s.p.x, s.p.y, s.p.z);
            it.q[k] = f3(s.q.x, s.q.y, s.q.z);
        }
        items[e] = it;
        r.used_epa = 1;
        res[i] = r;
        return;
    }
    float vl = sqrtf(g.sqdist);
    V<float> pa = g.pa + g.axis * (rA / vl);
    V<float> pb = g.pb + g.axis * (-(rB / vl));
    V<float> dd = pa - pb;
    float penetration = sqrtf(lsq(dd)) - maxSep;
    float al = sqrtf(lsq(g.axis));
    if (al > 0.f) pa = pa + g.axis * (-(maxSep / al));
    V<float> paw = qrotS(qA, pa), pbw = qrotS(qA, pb), axw = qrotS(qA, g.axis);
    write_hit(r, xyz(pa4), f3(paw.x, paw.y, paw.z), f3(pbw.x, pbw.y, pbw.z), f3(axw.x, axw.y, axw.z), penetration,
              0);
    res[i] = r;
}

// EPA pass: CC_STATIC_EPA_SLOTS threads, each owning one static polytope,
// stride over the queued items (the arithmetic of epa_pair).
__global__ void __launch_bounds__(64) k_static_epa(const cc_penetration_query *qs, cc_penetration_result *res,
                                                   const EpaItem *items, const StaticQueue *queue,
                                                   EpaScratch *slots, float penetration_tol) {
    int ne = queue->count;
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= CC_STATIC_EPA_SLOTS) return;
    EpaScratch *mine = slots + tid;
    for (int j = tid; j < ne; j += CC_STATIC_EPA_SLOTS) {
        const EpaItem &it = items[j];
        const cc_penetration_query &qy = qs[it.a];
        float4 pa4, pb4, qa, qb, sa, sb;
        pose_of(qy.a, pa4, qa, sa);
        pose_of(qy.b, pb4, qb, sb);
        R maxSep = R(qy.max_separation < 1.f ? qy.max_separation : 1.f);
        Q<R> iA{R(-qa.x), R(-qa.y), R(-qa.z), R(qa.w)};
        Q<R> qB{R(qb.x), R(qb.y), R(qb.z), R(qb.w)}, qA{R(qa.x), R(qa.y), R(qa.z), R(qa.w)};
        Q<R> rel = qmulS(iA, qB);
        V<R> ab{R(pb4.x) - R(pa4.x), R(pb4.y) - R(pa4.y), R(pb4.z) - R(pa4.z)};
        V<R> posBInA = qrotS(iA, ab);
        const HullView none{nullptr, nullptr, nullptr};
        Sup<R> A = make_sup<R>(qy.a.shape_type, sa, false, none);
        Sup<R> B = make_sup<R>(qy.b.shape_type, sb, false, none);
        A.add_r = maxSep;
        set_transform(B, rel, posBInA);
        Hull<BigStore> h;
        h.st.s = mine;
        h.start(it);
        V<R> axis, pa, pb;
        if (!epa(h, A, B, R(penetration_tol), axis, pa, pb)) continue;  // no contact (convex.ts:331)
        V<R> dd = pa - pb;
        R penetration = sq_root(lsq(dd)) - maxSep;
        R al = sq_root(lsq(axis));
        if (al > R(0)) pa = pa + axis * (-(maxSep / al));
        V<R> paw = qrotS(qA, pa), pbw = qrotS(qA, pb), axw = qrotS(qA, axis);
        cc_penetration_result r;
        write_hit(r, xyz(pa4), f3((float)(paw.x), (float)(paw.y), (float)(paw.z)),
                  f3((float)(pbw.x), (float)(pbw.y), (float)(pbw.z)),
                  f3((float)(axw.x), (float)(axw.y), (float)(axw.z)), (float)(penetration), 1);
        res[it.a] = r;
    }
}

// Addresses of the static arrays on one device, looked up once.
struct StaticArrays {
    EpaScratch *slots;
    EpaItem *items;
    StaticQueue *queue;
};
constexpr int STATIC_MAX_DEVICES = 64;
static StaticArrays g_static_addr[STATIC_MAX_DEVICES];
static bool g_static_ready[STATIC_MAX_DEVICES];
static std::mutex g_static_mutex;

static int static_arrays(StaticArrays &out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return CC_ERR_CUDA;
    if (dev < 0 || dev >= STATIC_MAX_DEVICES) return CC_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_static_mutex);
    if (!g_static_ready[dev]) {
        StaticArrays a;
        if (cudaGetSymbolAddress((void **)&a.slots, g_static_slots) != cudaSuccess) return CC_ERR_CUDA;
        if (cudaGetSymbolAddress((void **)&a.items, g_static_items) != cudaSuccess) return CC_ERR_CUDA;
        if (cudaGetSymbolAddress((void **)&a.queue, g_static_queue) != cudaSuccess) return CC_ERR_CUDA;
        g_static_addr[dev] = a;
        g_static_ready[dev] = true;
    }
    out = g_static_addr[dev];
    return CC_OK;
}

}  // namespace cc

extern "C" int cc_penetration_static(const cc_penetration_query *queries, int32_t count,
                                     cc_penetration_result *results, float collision_tolerance,
                                     float penetration_tolerance, void *stream) {
    using namespace cc;
    if (count < 0 || (count > 0 && (queries == nullptr || results == nullptr))) return CC_ERR_INVALID;
    if (!(collision_tolerance > 0.f) || !(penetration_tolerance > 0.f)) return CC_ERR_INVALID;
    if (count > CC_STATIC_MAX_QUERIES) return CC_ERR_CAPACITY;
    if (count == 0) return CC_OK;
    StaticArrays a;
    int r = static_arrays(a);
    if (r != CC_OK) return r;
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemsetAsync(&a.queue->count, 0, sizeof(int), s) != cudaSuccess) return CC_ERR_CUDA;
    k_static_gjk<<<(count + 127) / 128, 128, 0, s>>>(queries, count, results, a.items, a.queue, collision_tolerance);
    k_static_epa<<<CC_STATIC_EPA_SLOTS / 64 + (CC_STATIC_EPA_SLOTS % 64 != 0), 64, 0, s>>>(
        queries, results, a.items, a.queue, a.slots, penetration_tolerance);
    return cudaGetLastError() == cudaSuccess ? CC_OK : CC_ERR_CUDA;
}
