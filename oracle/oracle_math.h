// FP64 vector / quaternion / matrix helpers for the CPU oracle.
//
// TEST INFRASTRUCTURE ONLY: this header belongs to the parity oracle and is
// never linked into the GPU library.
//
// The reference (isaac-mason/crashcat) takes its vector maths from the
// third-party package `mathcat@0.0.10` (package.json:44-46,
// pnpm-lock.yaml:2176-2178), which is not vendored.  mathcat follows the
// gl-matrix conventions (column-major Mat4, [x,y,z,w] quaternions); the
// helpers below restate the published gl-matrix algorithms.  Choices that no
// reference test pins (vec3.length as sqrt of the dot product rather than
// Math.hypot, box overlap inclusive) are the oracle's own: mathcat 0.0.10 is
// not vendored with the reference, so no test pins them.
#pragma once
#include <cmath>
#include <cstdint>

namespace orc {

struct V3 {
    double x = 0, y = 0, z = 0;
};
struct Q4 {
    double x = 0, y = 0, z = 0, w = 1;
};
struct Box3 {
    V3 mn, mx;
};

inline V3 v3(double x, double y, double z) { return V3{x, y, z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 scale(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 neg(V3 a) { return {-a.x, -a.y, -a.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double lensq(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
inline double len(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
// gl-matrix vec3.cross
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// gl-matrix vec3.scaleAndAdd: a + b * s
inline V3 scale_add(V3 a, V3 b, double s) { return {a.x + b.x * s, a.y + b.y * s, a.z + b.z * s}; }
// gl-matrix vec3.normalize: multiply by the reciprocal square root
inline V3 normalize(V3 a) {
    double l = a.x * a.x + a.y * a.y + a.z * a.z;
    if (l > 0) l = 1.0 / std::sqrt(l);
    return {a.x * l, a.y * l, a.z * l};
}
inline double distance(V3 a, V3 b) { return len(sub(a, b)); }

// gl-matrix quat.multiply(a, b)
inline Q4 qmul(Q4 a, Q4 b) {
    return {a.x * b.w + a.w * b.x + a.y * b.z - a.z * b.y, a.y * b.w + a.w * b.y + a.z * b.x - a.x * b.z,
            a.z * b.w + a.w * b.z + a.x * b.y - a.y * b.x, a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z};
}
inline Q4 qnormalize(Q4 a) {
    double l = a.x * a.x + a.y * a.y + a.z * a.z + a.w * a.w;
    if (l > 0) l = 1.0 / std::sqrt(l);
    return {a.x * l, a.y * l, a.z * l, a.w * l};
}
inline Q4 qconj(Q4 a) { return {-a.x, -a.y, -a.z, a.w}; }
// gl-matrix quat.setAxisAngle
inline Q4 qaxis_angle(V3 axis, double rad) {
    rad = rad * 0.5;
    double s = std::sin(rad);
    return {s * axis.x, s * axis.y, s * axis.z, std::cos(rad)};
}
// gl-matrix vec3.transformQuat
inline V3 rotate(Q4 q, V3 a) {
    double qx = q.x, qy = q.y, qz = q.z, qw = q.w;
    double x = a.x, y = a.y, z = a.z;
    double uvx = qy * z - qz * y, uvy = qz * x - qx * z, uvz = qx * y - qy * x;
    double uuvx = qy * uvz - qz * uvy, uuvy = qz * uvx - qx * uvz, uuvz = qx * uvy - qy * uvx;
    double w2 = qw * 2;
    uvx *= w2;
    uvy *= w2;
    uvz *= w2;
    uuvx *= 2;
    uuvy *= 2;
    uuvz *= 2;
    return {x + uvx + uuvx, y + uvy + uuvy, z + uvz + uuvz};
}

// Column-major 4x4 matrix, gl-matrix layout.
struct M4 {
    double m[16];
};
// gl-matrix mat4.fromQuat
inline M4 mat4_from_quat(Q4 q) {
    M4 o{};
    double x = q.x, y = q.y, z = q.z, w = q.w;
    double x2 = x + x, y2 = y + y, z2 = z + z;
    double xx = x * x2, yx = y * x2, yy = y * y2, zx = z * x2, zy = z * y2, zz = z * z2, wx = w * x2,
           wy = w * y2, wz = w * z2;
    o.m[0] = 1 - yy - zz;
    o.m[1] = yx + wz;
    o.m[2] = zx - wy;
    o.m[3] = 0;
    o.m[4] = yx - wz;
    o.m[5] = 1 - xx - zz;
    o.m[6] = zy + wx;
    o.m[7] = 0;
    o.m[8] = zx + wy;
    o.m[9] = zy - wx;
    o.m[10] = 1 - xx - yy;
    o.m[11] = 0;
    o.m[12] = 0;
    o.m[13] = 0;
    o.m[14] = 0;
    o.m[15] = 1;
    return o;
}
// gl-matrix mat4.fromRotationTranslation
inline M4 mat4_from_rt(Q4 q, V3 v) {
    M4 o{};
    double x = q.x, y = q.y, z = q.z, w = q.w;
    double x2 = x + x, y2 = y + y, z2 = z + z;
    double xx = x * x2, xy = x * y2, xz = x * z2, yy = y * y2, yz = y * z2, zz = z * z2, wx = w * x2,
           wy = w * y2, wz = w * z2;
    o.m[0] = 1 - (yy + zz);
    o.m[1] = xy + wz;
    o.m[2] = xz - wy;
    o.m[3] = 0;
    o.m[4] = xy - wz;
    o.m[5] = 1 - (xx + zz);
    o.m[6] = yz + wx;
    o.m[7] = 0;
    o.m[8] = xz + wy;
    o.m[9] = yz - wx;
    o.m[10] = 1 - (xx + yy);
    o.m[11] = 0;
    o.m[12] = v.x;
    o.m[13] = v.y;
    o.m[14] = v.z;
    o.m[15] = 1;
    return o;
}
// gl-matrix mat4.multiply3x3Vec (rotation part times vector)
inline V3 m3mul(const M4 &a, V3 v) {
    return {a.m[0] * v.x + a.m[4] * v.y + a.m[8] * v.z, a.m[1] * v.x + a.m[5] * v.y + a.m[9] * v.z,
            a.m[2] * v.x + a.m[6] * v.y + a.m[10] * v.z};
}
// transposed rotation times vector (inverse rotation)
inline V3 m3tmul(const M4 &a, V3 v) {
    return {a.m[0] * v.x + a.m[1] * v.y + a.m[2] * v.z, a.m[4] * v.x + a.m[5] * v.y + a.m[6] * v.z,
            a.m[8] * v.x + a.m[9] * v.y + a.m[10] * v.z};
}

// box3.intersectsBox3 (inclusive bounds)
inline bool box_overlap(const Box3 &a, const Box3 &b) {
    return !(a.mx.x < b.mn.x || a.mn.x > b.mx.x || a.mx.y < b.mn.y || a.mn.y > b.mx.y || a.mx.z < b.mn.z ||
             a.mn.z > b.mx.z);
}
inline Box3 box_expand(const Box3 &a, double m) {
    return {{a.mn.x - m, a.mn.y - m, a.mn.z - m}, {a.mx.x + m, a.mx.y + m, a.mx.z + m}};
}

}  // namespace orc
