// Swing-twist decomposition and limit clamping (src/constraints/constraint-part/
// swing-twist-constraint-part.ts), shared by the device solve and the host setters
// (setTargetOrientationCS clamps its target with the same function).
#pragma once
#include "cc_internal.cuh"

namespace cc {

enum : int { CL_TWIST_MIN = 1, CL_TWIST_MAX = 2, CL_Y_MIN = 4, CL_Y_MAX = 8, CL_Z_MIN = 16, CL_Z_MAX = 32 };
__host__ __device__ inline float4 qscale4(float4 q, float s) { return make_float4(q.x * s, q.y * s, q.z * s, q.w * s); }
__host__ __device__ inline float4 qconj4(float4 q) { return make_float4(-q.x, -q.y, -q.z, q.w); }
// getSwingTwist :252-269: q = swing * twist, swing.x = 0, twist.y = twist.z = 0
__host__ __device__ inline void get_swing_twist(float4 q, float4 &swing, float4 &twist) {
    float s = sqrtf(q.w * q.w + q.x * q.x);
    if (s != 0.f) {
        twist = make_float4(q.x / s, 0.f, 0.f, q.w / s);
        swing = make_float4(0.f, (q.w * q.y - q.x * q.z) / s, (q.w * q.z + q.x * q.y) / s, s);
    } else {
        twist = make_float4(0.f, 0.f, 0.f, 1.f);
        swing = q;
    }
}
__host__ __device__ inline bool min_shorter(float dmin, float dmax) {  // distanceToMinShorter :239-246
    float a = fabsf(dmin);
    if (a > 1.f) a = 2.f - a;
    float b = fabsf(dmax);
    if (b > 1.f) b = 2.f - b;
    return a < b;
}
// getClosestPointOnEllipse :412-462 in FP64: Newton iteration on the Lagrange multiplier,
// at most 100 steps
__host__ __device__ inline void ellipse_closest(double px, double py, double a, double b, double &ox, double &oy) {
    double aSq = a * a, bSq = b * b, t = 0.0;
    for (int i = 0; i < 100; i++) {
        double ta = t + aSq, tb = t + bSq;
        double ga = a * px / ta, gb = b * py / tb;
        double gt = ga * ga + gb * gb - 1.0;
        if (fabs(gt) < 1e-6) {
            ox = aSq * px / ta;
            oy = bSq * py / tb;
            return;
        }
        double d = -2.0 * (aSq * px * px / (ta * ta * ta) + bSq * py * py / (tb * tb * tb));
        t = t - gt / d;
    }
    ox = aSq * px / (t + aSq);
    oy = bSq * py / (t + bSq);
}
// clampSwingTwist :278-402
// (P: a record holding the swing-twist limits, the swing-twist joint's or the six-DOF joint's)
template <class P>
__host__ __device__ inline int clamp_swing_twist(const P &p, float4 &swing, float4 &twist) {
    int cl = 0;
    bool neg_s = swing.w < 0.f, neg_t = twist.w < 0.f;
    if (neg_s) swing = qscale4(swing, -1.f);
    if (neg_t) twist = qscale4(twist, -1.f);
    int rf = p.rotation_flags;
    if (rf & ST_TWIST_LOCKED) {
        if (twist.x != 0.f) cl |= CL_TWIST_MIN | CL_TWIST_MAX;
        twist = make_float4(0.f, 0.f, 0.f, 1.f);
    } else if (!(rf & ST_TWIST_FREE)) {
        float dmin = p.sin_twist_min - twist.x, dmax = twist.x - p.sin_twist_max;
        if (dmin > 0.f || dmax > 0.f) {
            if (min_shorter(dmin, dmax)) {
                twist = make_float4(p.sin_twist_min, 0.f, 0.f, p.cos_twist_min);
                cl |= CL_TWIST_MIN;
            } else {
                twist = make_float4(p.sin_twist_max, 0.f, 0.f, p.cos_twist_max);
                cl |= CL_TWIST_MAX;
            }
        }
    }
    if (rf & ST_SWING_Y_LOCKED) {
        if (rf & ST_SWING_Z_LOCKED) {
            if (swing.y != 0.f) cl |= CL_Y_MIN | CL_Y_MAX;
            if (swing.z != 0.f) cl |= CL_Z_MIN | CL_Z_MAX;
            swing = make_float4(0.f, 0.f, 0.f, 1.f);
        } else {
            if (swing.y != 0.f) cl |= CL_Y_MIN | CL_Y_MAX;
            float dmin = p.sin_z_min - swing.z, dmax = swing.z - p.sin_z_max;
            if (dmin > 0.f || dmax > 0.f) {
                if (min_shorter(dmin, dmax)) {
                    swing = make_float4(0.f, 0.f, p.sin_z_min, p.cos_z_min);
                    cl |= CL_Z_MIN;
                } else {
                    swing = make_float4(0.f, 0.f, p.sin_z_max, p.cos_z_max);
                    cl |= CL_Z_MAX;
                }
            } else if (cl & CL_Y_MIN) {
                float z = swing.z;
                swing = make_float4(0.f, 0.f, z, sqrtf(1.f - z * z));
            }
        }
    } else if (rf & ST_SWING_Z_LOCKED) {
        if (swing.z != 0.f) cl |= CL_Z_MIN | CL_Z_MAX;
        float dmin = p.sin_y_min - swing.y, dmax = swing.y - p.sin_y_max;
        if (dmin > 0.f || dmax > 0.f) {
            if (min_shorter(dmin, dmax)) {
                swing = make_float4(0.f, p.sin_y_min, 0.f, p.cos_y_min);
                cl |= CL_Y_MIN;
            } else {
                swing = make_float4(0.f, p.sin_y_max, 0.f, p.cos_y_max);
                cl |= CL_Y_MAX;
            }
        } else if (cl & CL_Z_MIN) {
            float y = swing.y;
            swing = make_float4(0.f, y, 0.f, sqrtf(1.f - y * y));
        }
    } else if (p.swing_type == 0) {  // cone: the swing (y, z) inside the ellipse of the sines
        float y = swing.y, z = swing.z, a = p.sin_y_max, b = p.sin_z_max;
        if (a > 0.f && b > 0.f) {
            float e = y * y / (a * a) + z * z / (b * b);
            if (e > 1.f) {
                double cy, cz;
                ellipse_closest(y, z, a, b, cy, cz);
                float fy = (float)cy, fz = (float)cz;
                swing = make_float4(0.f, fy, fz, sqrtf(fmaxf(0.f, 1.f - fy * fy - fz * fz)));
                cl |= CL_Y_MIN | CL_Y_MAX | CL_Z_MIN | CL_Z_MAX;
            }
        }
    } else {  // pyramid: the half angles clamped independently
        float hy = atan2f(swing.y, swing.w), hz = atan2f(swing.z, swing.w);
        float cy = fmaxf(p.y_half_min, fminf(p.y_half_max, hy));
        float cz = fmaxf(p.z_half_min, fminf(p.z_half_max, hz));
        if (hy != cy || hz != cz) {
            float sy = sinf(cy), coy = cosf(cy), sz = sinf(cz), coz = cosf(cz);
            float ny = sy * coz, nz = coy * sz, nw = coy * coz;
            float l = sqrtf(ny * ny + nz * nz + nw * nw);
            swing = make_float4(0.f, ny / l, nz / l, nw / l);
            cl |= CL_Y_MIN | CL_Y_MAX | CL_Z_MIN | CL_Z_MAX;
        }
    }
    if (neg_s) swing = qscale4(swing, -1.f);
    if (neg_t) twist = qscale4(twist, -1.f);
    return cl;
}
}  // namespace cc
