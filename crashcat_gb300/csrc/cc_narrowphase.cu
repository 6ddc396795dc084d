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
enum { SUP_BOX = 0, SUP_POINT = 1, SUP_SPHERE = 2 };
template <typename S>
struct Sup {
    int kind;
    V<S> he;      // box half extents
    S radius;     // sphere surface radius
    S convex_radius;
    bool transformed;
    V<S> r0, r1, r2, t;  // rows of the rotation and translation (B in A's frame)
    S add_r;
    __device__ V<S> inner(V<S> d) const {
        if (kind == SUP_BOX) return {d.x >= S(0) ? he.x : -he.x, d.y >= S(0) ? he.y : -he.y, d.z >= S(0) ? he.z : -he.z};
        if (kind == SUP_POINT) return {S(0), S(0), S(0)};
        S l = lsq(d);
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
template <typename S>
__device__ Sup<S> make_sup(int shape, float4 sp, bool exclude) {
    Sup<S> o;
    o.transformed = false;
    o.add_r = S(0);
    o.radius = S(0);
    o.he = {S(0), S(0), S(0)};
    if (shape == SHAPE_BOX) {
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
template <typename S>
__device__ void set_transform(Sup<S> &s, Q<S> q, V<S> p) {
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
template <typename S>
__device__ GjkOut<S> gjk(const Sup<S> &A, const Sup<S> &B, S tolerance, V<S> dir, S maxDistSq, Simplex<S> &sx) {
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
constexpr int FMAX = 16;
struct Face {
    int n;
    float3 v[FMAX];
};

// box getSupportingFace box.ts:129-332 (unit scale), then rotate + translate
__device__ void box_face(Face &f, float3 dir, float4 he4, float4 q, float3 t) {
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

// clipPolyVsPlane clip.ts:13-92
__device__ void clip_plane(Face &out, const Face &in, float3 o, float3 n) {
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
                if (out.n < FMAX) out.v[out.n++] = e1 + e12 * t;
            } else {
                curIn = prevIn;
            }
        }
        if (curIn && out.n < FMAX) out.v[out.n++] = e2;
        prevNum = num;
        prevIn = curIn;
        e1 = e2;
    }
}

// clipPolyVsPoly clip.ts:108-175
__device__ void clip_poly(Face &out, const Face &toClip, const Face &clipping, float3 cn) {
    out.n = 0;
    if (toClip.n < 2 || clipping.n < 3) return;
    Face t0, t1;
    int tmpIdx = 0;
    for (int i = 0; i < clipping.n; i++) {
        float3 c1 = clipping.v[i];
        float3 c2 = clipping.v[(i + 1) % clipping.n];
        float3 pn = cross3(cn, c2 - c1);
        const Face *src = (i == 0) ? &toClip : (tmpIdx == 0 ? &t0 : &t1);
        tmpIdx ^= 1;
        Face *dst = (i == clipping.n - 1) ? &out : (tmpIdx == 0 ? &t0 : &t1);
        clip_plane(*dst, *src, c1, pn);
        if (dst->n < 3) {
            out.n = 0;
            return;
        }
    }
}

struct Pts {
    int n;
    float3 a[FMAX], b[FMAX];
};

// pruneContactPoints manifold.ts:192-311
__device__ void prune(Pts &m, float3 axis) {
    const float MIN_D = 1.0e-6f;
    if (m.n <= 4) return;
    float3 proj[FMAX];
    float dsq[FMAX];
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

// manifoldBetweenTwoFaces manifold.ts:345-444 (polygon faces)
__device__ void manifold_faces(Pts &out, float3 cp1, float3 cp2, float3 axis, float maxDist, const Face &f1,
                               const Face &f2) {
    out.n = 0;
    if (f1.n < 2 || f2.n < 3) {
        out.a[0] = cp1;
        out.b[0] = cp2;
        out.n = 1;
        return;
    }
    Face clipped;
    clipped.n = 0;
    if (f1.n >= 3) clip_poly(clipped, f2, f1, axis);
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
                if (out.n >= FMAX) break;
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
__device__ void emit_manifold(DevWorld &w, int a, int b, float3 pa, float3 pb, float3 axis, float penetration,
                              bool faces) {
    float4 qa = w.quat[a], qb = w.quat[b];
    float3 posA = xyz(w.pos[a]), posB = xyz(w.pos[b]);
    uint32_t fa = w.flags[a], fb = w.flags[b];
    Pts pts;
    float maxd = c_settings.spec_dist + c_settings.manifold_tol;
    float3 nrm = normalize3(axis);
    bool haveFaces = false;
    Face fA, fB;
    fA.n = 0;
    fB.n = 0;
    if (faces) {
        // face directions in body space: A uses -axis, B uses axis (both rotated into the body frames)
        float3 axA = qrot_inv(qa, axis);
        float3 axB = qrot_inv(qb, axis);
        if (shape_of(fa) == SHAPE_BOX) box_face(fA, -axA, w.shape[a], qa, f3(0.f, 0.f, 0.f));
        if (shape_of(fb) == SHAPE_BOX) box_face(fB, axB, w.shape[b], qb, posB - posA);
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
    w.manifolds[slot] = m;
}

struct EpaItem {
    int a, b;
    int size;
    int pad;
    float3 y[4], p[4], q[4];
};

// narrowphase for one pair: order A/B (update.ts:74), dispatch, GJK
__global__ void __launch_bounds__(128) k_narrowphase(DevWorld w, EpaItem *epa_items) {
    int np = min(w.ctr->num_pairs, w.max_pairs);
    for (int pi = blockIdx.x * blockDim.x + threadIdx.x; pi < np; pi += gridDim.x * blockDim.x) {
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
        float4 pa4 = w.pos[a], pb4 = w.pos[b];
        float4 qa = w.quat[a], qb = w.quat[b];
        float4 sa = w.shape[a], sb = w.shape[b];
        int sha = shape_of(fa), shb = shape_of(fb);
        if (sha == SHAPE_SPHERE && shb == SHAPE_SPHERE) {
            // collideSphereVsSphere sphere.ts:319-410 (no speculative distance)
            float3 d = xyz(pb4) - xyz(pa4);
            float dsq = lensq3(d);
            float rs = sa.x + sb.x;
            if (dsq >= rs * rs) continue;
            float dist = sqrtf(dsq);
            float3 n = dist > 0.f ? d * (1.f / dist) : f3(0.f, 1.f, 0.f);
            emit_manifold(w, a, b, n * sa.x, d - n * sb.x, n, rs - dist, false);
            continue;
        }
        // collideConvexVsConvex convex.ts:257-346: B in A's local frame
        Q<float> qA{qa.x, qa.y, qa.z, qa.w}, qB{qb.x, qb.y, qb.z, qb.w};
        Q<float> iA{-qa.x, -qa.y, -qa.z, qa.w};
        Q<float> rel = qmulS(iA, qB);
        V<float> ab{pb4.x - pa4.x, pb4.y - pa4.y, pb4.z - pa4.z};
        V<float> posBInA = qrotS(iA, ab);
        Sup<float> supA = make_sup<float>(sha, sa, true);
        Sup<float> supB = make_sup<float>(shb, sb, true);
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
        emit_manifold(w, a, b, f3(paw.x, paw.y, paw.z), f3(pbw.x, pbw.y, pbw.z), f3(axw.x, axw.y, axw.z),
                      penetration, true);
    }
}

// ---------------------------------------------------------------------------
// EPA (penetration.ts:214-614 + epa-convex-hull-builder.ts) in FP64 with the
// polytope in a per-thread slice of global scratch memory
// ---------------------------------------------------------------------------
constexpr int EPA_MAX_TRI = 256;
constexpr int EPA_PTS_CAP = 160;
constexpr int EPA_QUEUE_CAP = 512;

struct EpaTri {
    V<double> normal, centroid;
    double cls;
    double l0, l1;
    int nt[3];
    int ne[3];
    int st[3];
    int flags;  // 1 rel0, 2 interior, 4 removed, 8 inq
};
struct EpaScratch {
    V<double> Y[EPA_PTS_CAP], P[EPA_PTS_CAP], Qp[EPA_PTS_CAP];
    EpaTri tri[EPA_MAX_TRI];
    int queue[EPA_QUEUE_CAP];
    int freel[EPA_MAX_TRI];
    int edge_nt[128], edge_ne[128], edge_st[128];
    int stk_t[128], stk_e[128], stk_i[128];
    int newt[128];
};
size_t epa_scratch_bytes() { return sizeof(EpaScratch); }
size_t epa_item_bytes();

struct EpaHull {
    EpaScratch *s;
    int ntri, nfree, nq, npts;
    __device__ bool facing(int t, V<double> p) const {
        const EpaTri &T = s->tri[t];
        return dot(T.normal, p - T.centroid) > 0.0;
    }
    __device__ void push(int t) {
        if (nq >= EPA_QUEUE_CAP) return;
        s->queue[nq] = t;
        s->tri[t].flags |= 8;
        int cur = nq++;
        while (cur > 0) {
            int par = (cur - 1) >> 1;
            if (s->tri[s->queue[par]].cls > s->tri[s->queue[cur]].cls) {
                int tmp = s->queue[par];
                s->queue[par] = s->queue[cur];
                s->queue[cur] = tmp;
                cur = par;
            } else {
                break;
            }
        }
    }
    __device__ int pop() {
        if (nq == 0) return -1;
        int tmp = s->queue[nq - 1];
        s->queue[nq - 1] = s->queue[0];
        s->queue[0] = tmp;
        int count = nq - 1;
        int largest = 0;
        while (true) {
            int child = (largest << 1) + 1;
            if (child >= count) break;
            int prevL = largest;
            if (s->tri[s->queue[largest]].cls > s->tri[s->queue[child]].cls) largest = child;
            ++child;
            if (child < count && s->tri[s->queue[largest]].cls > s->tri[s->queue[child]].cls) largest = child;
            if (prevL == largest) break;
            int t2 = s->queue[prevL];
            s->queue[prevL] = s->queue[largest];
            s->queue[largest] = t2;
        }
        nq--;
        return s->queue[nq];
    }
    __device__ void link(int t1, int e1, int t2, int e2) {
        s->tri[t1].nt[e1] = t2;
        s->tri[t1].ne[e1] = e2;
        s->tri[t2].nt[e2] = t1;
        s->tri[t2].ne[e2] = e1;
    }
    __device__ int create(int i1, int i2, int i3) {
        int idx;
        if (nfree > 0) {
            idx = s->freel[--nfree];
        } else {
            if (ntri >= EPA_MAX_TRI) return -1;
            idx = ntri++;
        }
        EpaTri &t = s->tri[idx];
        t.cls = 1.0 / 0.0;
        t.l0 = t.l1 = 0.0;
        t.flags = 0;
        t.st[0] = i1;
        t.st[1] = i2;
        t.st[2] = i3;
        t.nt[0] = t.nt[1] = t.nt[2] = -1;
        t.ne[0] = t.ne[1] = t.ne[2] = 0;
        V<double> y0 = s->Y[i1], y1 = s->Y[i2], y2 = s->Y[i3];
        V<double> c{(y0.x + y1.x + y2.x) / 3.0, (y0.y + y1.y + y2.y) / 3.0, (y0.z + y1.z + y2.z) / 3.0};
        t.centroid = c;
        V<double> y10 = y1 - y0, y20 = y2 - y0, y21 = y2 - y1;
        double y20d = lsq(y20), y21d = lsq(y21);
        if (y20d < y21d) {
            V<double> n = crs(y10, y20);
            t.normal = n;
            double nl = lsq(n);
            if (nl > 1e-10) {
                double cdn = dot(c, n);
                t.cls = (fabs(cdn) * cdn) / nl;
                double y10d = lsq(y10), y1020 = dot(y10, y20);
                double det = y10d * y20d - y1020 * y1020;
                if (det > 0.0) {
                    double a = dot(y0, y10), b = dot(y0, y20);
                    double l0 = (y1020 * b - y20d * a) / det, l1 = (y1020 * a - y10d * b) / det;
                    t.l0 = l0;
                    t.l1 = l1;
                    t.flags |= 1;
                    if (l0 > -1e-3 && l1 > -1e-3 && l0 + l1 < 1.0 + 1e-3) t.flags |= 2;
                }
            }
        } else {
            V<double> n = crs(y10, y21);
            t.normal = n;
            double nl = lsq(n);
            if (nl > 1e-10) {
                double cdn = dot(c, n);
                t.cls = (fabs(cdn) * cdn) / nl;
                double y10d = lsq(y10), y1021 = dot(y10, y21);
                double det = y10d * y21d - y1021 * y1021;
                if (det > 0.0) {
                    double a = dot(y1, y10), b = dot(y1, y21);
                    double l0 = (y21d * a - y1021 * b) / det, l1 = (y1021 * a - y10d * b) / det;
                    t.l0 = l0;
                    t.l1 = l1;
                    if (l0 > -1e-3 && l1 > -1e-3 && l0 + l1 < 1.0 + 1e-3) t.flags |= 2;
                }
            }
        }
        return idx;
    }
    __device__ void free_tri(int t) {
        if (nfree < EPA_MAX_TRI) s->freel[nfree++] = t;
    }
    __device__ void unlink(int t) {
        for (int i = 0; i < 3; i++) {
            int n = s->tri[t].nt[i];
            if (n >= 0) {
                s->tri[n].nt[s->tri[t].ne[i]] = -1;
                s->tri[t].nt[i] = -1;
            }
        }
        if (!(s->tri[t].flags & 8)) free_tri(t);
    }
    __device__ int find_facing(V<double> p) {
        int best = -1;
        double bestd = 0.0;
        for (int i = 0; i < nq; i++) {
            int t = s->queue[i];
            const EpaTri &T = s->tri[t];
            if (T.flags & 4) continue;
            double d = dot(T.normal, p - T.centroid);
            if (d > 0.0) {
                double dsq = (d * d) / lsq(T.normal);
                if (dsq > bestd) {
                    best = t;
                    bestd = dsq;
                }
            }
        }
        return best;
    }
    // findEdge epa-convex-hull-builder.ts:476-540; returns edge count or -1
    __device__ int find_edge(int ft, V<double> vtx) {
        int ne = 0;
        s->tri[ft].flags |= 4;
        int sp = 0;
        s->stk_t[0] = ft;
        s->stk_e[0] = 0;
        s->stk_i[0] = -1;
        int next_expected = -1;
        int guard = 0;
        while (guard++ < 100000) {
            int ct = s->stk_t[sp];
            if (++s->stk_i[sp] >= 3) {
                unlink(ct);
                if (--sp < 0) break;
            } else {
                int ei = (s->stk_e[sp] + s->stk_i[sp]) % 3;
                int n = s->tri[ct].nt[ei];
                int nen = s->tri[ct].ne[ei];
                int est = s->tri[ct].st[ei];
                if (n >= 0 && !(s->tri[n].flags & 4)) {
                    if (facing(n, vtx)) {
                        s->tri[n].flags |= 4;
                        sp++;
                        if (sp >= 128) return -1;
                        s->stk_t[sp] = n;
                        s->stk_e[sp] = nen;
                        s->stk_i[sp] = 0;
                    } else {
                        if (est != next_expected && next_expected != -1) return -1;
                        next_expected = s->tri[n].st[nen];
                        if (ne >= 128) return -1;
                        s->edge_nt[ne] = n;
                        s->edge_ne[ne] = nen;
                        s->edge_st[ne] = est;
                        ne++;
                    }
                }
            }
        }
        if (ne > 0 && s->edge_st[0] != next_expected) return -1;
        return ne >= 3 ? ne : -1;
    }
    __device__ int add_point(int ft, int idx, double closest) {
        int ne = find_edge(ft, s->Y[idx]);
        if (ne < 0) return -1;
        for (int i = 0; i < ne; i++) {
            int in = (i + 1) % ne;
            int nt = create(s->edge_st[i], s->edge_st[in], idx);
            if (nt < 0) return -1;
            s->newt[i] = nt;
            const EpaTri &T = s->tri[nt];
            if (((T.flags & 2) && T.cls < closest) || T.cls < 0.0) push(nt);
        }
        for (int i = 0; i < ne; i++) {
            int in = (i + 1) % ne;
            link(s->newt[i], 0, s->edge_nt[i], s->edge_ne[i]);
            link(s->newt[i], 1, s->newt[in], 2);
        }
        return ne;
    }
};

__device__ int epa_add_sup(EpaHull &h, const Sup<double> &A, const Sup<double> &B, V<double> d) {
    if (h.npts >= EPA_PTS_CAP) return -1;
    V<double> p = A.get(d), q = B.get(-d);
    int i = h.npts++;
    h.s->Y[i] = p - q;
    h.s->P[i] = p;
    h.s->Qp[i] = q;
    return i;
}

// returns true and the penetration result on success
__device__ bool epa(EpaHull &h, const Sup<double> &A, const Sup<double> &B, double tol, V<double> &outAxis,
                    V<double> &outPa, V<double> &outPb) {
    const double MAXD = 1.7976931348623157e308;
    if (h.npts == 1) {
        h.npts = 0;
        epa_add_sup(h, A, B, {0.0, 1.0, 0.0});
        epa_add_sup(h, A, B, {-1.0, -1.0, -1.0});
        epa_add_sup(h, A, B, {1.0, -1.0, -1.0});
        epa_add_sup(h, A, B, {0.0, -1.0, 1.0});
    } else if (h.npts == 2) {
        const double C120 = -0.4999999999999998, S120 = 0.8660254037844387, OMC = 1.0 - C120;
        V<double> y0 = h.s->Y[0], y1 = h.s->Y[1];
        V<double> ax = y1 - y0;
        double al = sqrt(lsq(ax));
        double nx = ax.x / al, ny = ax.y / al, nz = ax.z / al;
        V<double> d1;
        if (fabs(nx) > fabs(ny)) {
            double pl = sqrt(nx * nx + nz * nz);
            d1 = {nz / pl, 0.0, -nx / pl};
        } else {
            double pl = sqrt(ny * ny + nz * nz);
            d1 = {0.0, nz / pl, -ny / pl};
        }
        double r00 = C120 + nx * nx * OMC, r01 = nx * ny * OMC - nz * S120, r02 = nx * nz * OMC + ny * S120;
        double r10 = ny * nx * OMC + nz * S120, r11 = C120 + ny * ny * OMC, r12 = ny * nz * OMC - nx * S120;
        double r20 = nz * nx * OMC - ny * S120, r21 = nz * ny * OMC + nx * S120, r22 = C120 + nz * nz * OMC;
        V<double> d2{r00 * d1.x + r01 * d1.y + r02 * d1.z, r10 * d1.x + r11 * d1.y + r12 * d1.z,
                     r20 * d1.x + r21 * d1.y + r22 * d1.z};
        V<double> d3{r00 * d2.x + r01 * d2.y + r02 * d2.z, r10 * d2.x + r11 * d2.y + r12 * d2.z,
                     r20 * d2.x + r21 * d2.y + r22 * d2.z};
        epa_add_sup(h, A, B, d1);
        epa_add_sup(h, A, B, d2);
        epa_add_sup(h, A, B, d3);
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
        int t = h.find_facing(h.s->Y[i]);
        if (t >= 0 && h.add_point(t, i, MAXD) < 0) return false;
    }
    int guard = 0;
    while (guard++ < 4096) {
        if (h.nq == 0) return false;
        int t = h.s->queue[0];
        if (h.s->tri[t].flags & 4) {
            h.pop();
            if (h.nq == 0) return false;
            h.free_tri(t);
            continue;
        }
        if (h.s->tri[t].cls >= 0.0) break;
        h.pop();
        int ni = epa_add_sup(h, A, B, h.s->tri[t].normal);
        if (ni < 0) return false;
        if (!h.facing(t, h.s->Y[ni]) || h.add_point(t, ni, MAXD) < 0) return false;
        h.free_tri(t);
        if (h.nq == 0 || h.npts >= 32) return false;
    }
    double closest = MAXD;
    int last = -1;
    bool flip = false;
    guard = 0;
    do {
        int t = h.pop();
        if (t < 0) return false;
        if (h.s->tri[t].flags & 4) {
            h.free_tri(t);
            continue;
        }
        if (h.s->tri[t].cls >= closest) break;
        if (last >= 0) h.free_tri(last);
        last = t;
        V<double> tn = h.s->tri[t].normal;
        int ni = epa_add_sup(h, A, B, tn);
        if (ni < 0) break;
        V<double> wv = h.s->Y[ni];
        double d = dot(tn, wv);
        if (d < 0.0) return false;
        double dsq = (d * d) / lsq(tn);
        if (dsq - h.s->tri[t].cls < h.s->tri[t].cls * tol) break;
        closest = closest < dsq ? closest : dsq;
        if (!h.facing(t, wv)) break;
        int ne = h.add_point(t, ni, closest);
        if (ne < 0) break;
        bool defect = false;
        for (int k = 0; k < ne; k++) {
            const EpaTri &q = h.s->tri[h.s->newt[k]];
            if (dot(q.normal, q.centroid) < 0.0) {
                defect = true;
                break;
            }
        }
        if (defect) {
            V<double> nn = -tn;
            V<double> w2 = A.get(nn) - B.get(tn);
            if (dot(nn, w2) < d) flip = true;
            break;
        }
    } while (h.nq > 0 && h.npts < 128 && guard++ < 4096);
    if (last < 0) return false;
    const EpaTri &L = h.s->tri[last];
    double nls = lsq(L.normal);
    V<double> pn = L.normal * (dot(L.centroid, L.normal) / nls);
    if (lsq(pn) < 1e-10) return false;
    if (flip) pn = -pn;
    V<double> xp0 = h.s->P[L.st[0]], xp1 = h.s->P[L.st[1]], xp2 = h.s->P[L.st[2]];
    V<double> xq0 = h.s->Qp[L.st[0]], xq1 = h.s->Qp[L.st[1]], xq2 = h.s->Qp[L.st[2]];
    if (L.flags & 1) {
        outPa = xp0 + (xp1 - xp0) * L.l0 + (xp2 - xp0) * L.l1;
        outPb = xq0 + (xq1 - xq0) * L.l0 + (xq2 - xq0) * L.l1;
    } else {
        outPa = xp1 + (xp0 - xp1) * L.l0 + (xp2 - xp1) * L.l1;
        outPb = xq1 + (xq0 - xq1) * L.l0 + (xq2 - xq1) * L.l1;
    }
    outAxis = pn;
    return true;
}

// Runs the FP64 EPA stage for one queued pair with the given scratch slice.
__device__ void epa_pair(DevWorld &w, const EpaItem &it, EpaScratch *scratch) {
    int a = it.a, b = it.b;
    uint32_t fa = w.flags[a], fb = w.flags[b];
    float maxSepF = ((fa | fb) & F_SENSOR) ? 0.f : c_settings.spec_dist;
    double maxSep = (double)maxSepF < 1.0 ? (double)maxSepF : 1.0;
    float4 pa4 = w.pos[a], pb4 = w.pos[b], qa = w.quat[a], qb = w.quat[b];
    Q<double> iA{-(double)qa.x, -(double)qa.y, -(double)qa.z, (double)qa.w};
    Q<double> qB{qb.x, qb.y, qb.z, qb.w}, qA{qa.x, qa.y, qa.z, qa.w};
    Q<double> rel = qmulS(iA, qB);
    V<double> ab{(double)pb4.x - (double)pa4.x, (double)pb4.y - (double)pa4.y, (double)pb4.z - (double)pa4.z};
    V<double> posBInA = qrotS(iA, ab);
    Sup<double> A = make_sup<double>(shape_of(fa), w.shape[a], false);
    Sup<double> B = make_sup<double>(shape_of(fb), w.shape[b], false);
    A.add_r = maxSep;
    set_transform(B, rel, posBInA);
    EpaHull h;
    h.s = scratch;
    h.npts = it.size;
    for (int k = 0; k < it.size; k++) {
        scratch->Y[k] = {it.y[k].x, it.y[k].y, it.y[k].z};
        scratch->P[k] = {it.p[k].x, it.p[k].y, it.p[k].z};
        scratch->Qp[k] = {it.q[k].x, it.q[k].y, it.q[k].z};
    }
    V<double> axis, pa, pb;
    if (!epa(h, A, B, (double)c_settings.penetration_tol, axis, pa, pb)) return;
    V<double> dd = pa - pb;
    double penetration = sqrt(lsq(dd)) - maxSep;
    double al = sqrt(lsq(axis));
    if (al > 0.0) pa = pa + axis * (-(maxSep / al));
    V<double> paw = qrotS(qA, pa), pbw = qrotS(qA, pb), axw = qrotS(qA, axis);
    emit_manifold(w, a, b, f3((float)paw.x, (float)paw.y, (float)paw.z), f3((float)pbw.x, (float)pbw.y, (float)pbw.z),
                  f3((float)axw.x, (float)axw.y, (float)axw.z), (float)penetration, true);
}

__global__ void __launch_bounds__(64) k_epa(DevWorld w, const EpaItem *items, EpaScratch *scratch) {
    int ne = min(w.ctr->num_epa, w.max_epa);
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    EpaScratch *mine = scratch + tid;
    for (int i = tid; i < ne; i += gridDim.x * blockDim.x) epa_pair(w, items[i], mine);
}

size_t epa_item_bytes() { return sizeof(EpaItem); }

void launch_narrowphase(DevWorld &w, float, cudaStream_t s, cudaEvent_t mid) {
    EpaItem *items = (EpaItem *)w.epa_items;
    k_narrowphase<<<NUM_SMS * 8, 128, 0, s>>>(w, items);
    if (mid) cudaEventRecord(mid, s);
    k_epa<<<w.epa_threads / 64, 64, 0, s>>>(w, items, (EpaScratch *)w.epa_scratch);
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
    if ((sha != SHAPE_SPHERE && sha != SHAPE_BOX) || (shb != SHAPE_SPHERE && shb != SHAPE_BOX)) {
        res[i] = r;  // unknown shape type: reported as no hit
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
    Sup<float> supA = make_sup<float>(sha, sa, true);
    Sup<float> supB = make_sup<float>(shb, sb, true);
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
        double maxSep = (double)qy.max_separation < 1.0 ? (double)qy.max_separation : 1.0;
        Q<double> iA{-(double)qa.x, -(double)qa.y, -(double)qa.z, (double)qa.w};
        Q<double> qB{qb.x, qb.y, qb.z, qb.w}, qA{qa.x, qa.y, qa.z, qa.w};
        Q<double> rel = qmulS(iA, qB);
        V<double> ab{(double)pb4.x - (double)pa4.x, (double)pb4.y - (double)pa4.y, (double)pb4.z - (double)pa4.z};
        V<double> posBInA = qrotS(iA, ab);
        Sup<double> A = make_sup<double>(qy.a.shape_type, sa, false);
        Sup<double> B = make_sup<double>(qy.b.shape_type, sb, false);
        A.add_r = maxSep;
        set_transform(B, rel, posBInA);
        EpaHull h;
        h.s = mine;
        h.npts = it.size;
        for (int k = 0; k < it.size; k++) {
            mine->Y[k] = {it.y[k].x, it.y[k].y, it.y[k].z};
            mine->P[k] = {it.p[k].x, it.p[k].y, it.p[k].z};
            mine->Qp[k] = {it.q[k].x, it.q[k].y, it.q[k].z};
        }
        V<double> axis, pa, pb;
        if (!epa(h, A, B, (double)penetration_tol, axis, pa, pb)) continue;  // no contact (convex.ts:331)
        V<double> dd = pa - pb;
        double penetration = sqrt(lsq(dd)) - maxSep;
        double al = sqrt(lsq(axis));
        if (al > 0.0) pa = pa + axis * (-(maxSep / al));
        V<double> paw = qrotS(qA, pa), pbw = qrotS(qA, pb), axw = qrotS(qA, axis);
        cc_penetration_result r;
        write_hit(r, xyz(pa4), f3((float)paw.x, (float)paw.y, (float)paw.z),
                  f3((float)pbw.x, (float)pbw.y, (float)pbw.z), f3((float)axw.x, (float)axw.y, (float)axw.z),
                  (float)penetration, 1);
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
