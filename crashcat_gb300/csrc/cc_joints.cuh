// User joints on the device: setup, warm start, velocity and position solve of the point,
// distance, hinge, slider, fixed, cone and swing-twist joints (src/constraints/*-constraint.ts)
// and the constraint parts they are built from (constraint-part/point-, axis-, dual-axis-,
// hinge-rotation-, angle-, swing-twist-, rotation-euler-constraint-part.ts, spring-part.ts).  FP32 like the contact
// solver; the 3x3 and 2x2 effective-mass inversions and the swing ellipse projection run in
// FP64.  Body state is read and written in global memory; the joints of an island are solved
// in order by one thread of the per-CTA island solve.
// Included by cc_solver.cu inside namespace cc (it uses that file's c_settings and rotation_step,
// and the swing-twist clamping of cc_swing.cuh).
#pragma once

// ---- 3x3 helpers, row-major float[9] ------------------------------------------------
__device__ __forceinline__ void jm_from_sym(float o[9], const Sym3 &s) {
    o[0] = s.xx; o[1] = s.xy; o[2] = s.xz;
    o[3] = s.xy; o[4] = s.yy; o[5] = s.yz;
    o[6] = s.xz; o[7] = s.yz; o[8] = s.zz;
}
__device__ __forceinline__ void jm_cross(float o[9], float3 v) {  // [v]x, [v]x w = v x w
    o[0] = 0.f; o[1] = -v.z; o[2] = v.y;
    o[3] = v.z; o[4] = 0.f; o[5] = -v.x;
    o[6] = -v.y; o[7] = v.x; o[8] = 0.f;
}
__device__ __forceinline__ void jm_mm(float o[9], const float a[9], const float b[9]) {
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) o[3 * r + c] = a[3 * r] * b[c] + a[3 * r + 1] * b[3 + c] + a[3 * r + 2] * b[6 + c];
}
__device__ __forceinline__ void jm_mm_bt(float o[9], const float a[9], const float b[9]) {  // a b^T
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++)
            o[3 * r + c] = a[3 * r] * b[3 * c] + a[3 * r + 1] * b[3 * c + 1] + a[3 * r + 2] * b[3 * c + 2];
}
__device__ __forceinline__ float3 jm_mv(const float a[9], float3 v) {
    return f3(a[0] * v.x + a[1] * v.y + a[2] * v.z, a[3] * v.x + a[4] * v.y + a[5] * v.z,
              a[6] * v.x + a[7] * v.y + a[8] * v.z);
}
// mat4.invert3x3 as the adjugate over the determinant, in FP64; singular when det == 0
__device__ bool jm_invert(float o[9], const float m[9]) {
    double a00 = m[0], a01 = m[3], a02 = m[6];  // a(col)(row) as the column-major original
    double a10 = m[1], a11 = m[4], a12 = m[7];
    double a20 = m[2], a21 = m[5], a22 = m[8];
    double b01 = a22 * a11 - a12 * a21, b11 = -a22 * a10 + a12 * a20, b21 = a21 * a10 - a11 * a20;
    double det = a00 * b01 + a01 * b11 + a02 * b21;
    if (det == 0.0) return false;
    det = 1.0 / det;
    double r[9];
    r[0] = b01 * det;
    r[1] = (-a22 * a01 + a02 * a21) * det;
    r[2] = (a12 * a01 - a02 * a11) * det;
    r[3] = b11 * det;
    r[4] = (a22 * a00 - a02 * a20) * det;
    r[5] = (-a12 * a00 + a02 * a10) * det;
    r[6] = b21 * det;
    r[7] = (-a21 * a00 + a01 * a20) * det;
    r[8] = (a11 * a00 - a01 * a10) * det;
    // r holds columns (r[3c + k] = element (k, c)); store row-major
    for (int c = 0; c < 3; c++)
        for (int k = 0; k < 3; k++) o[3 * k + c] = (float)r[3 * c + k];
    return true;
}
__device__ __forceinline__ Sym3 sym_zero() { return Sym3{0, 0, 0, 0, 0, 0}; }
__device__ __forceinline__ void sym_store(float o[6], const Sym3 &s) {
    o[0] = s.xx; o[1] = s.xy; o[2] = s.xz; o[3] = s.yy; o[4] = s.yz; o[5] = s.zz;
}
__device__ __forceinline__ Sym3 sym_load(const float o[6]) { return Sym3{o[0], o[1], o[2], o[3], o[4], o[5]}; }

struct JBody {
    int i;
    int motion;
    float im;
    Sym3 I;  // world inverse inertia (zero unless dynamic)
};
// with_I: the world inverse inertia is needed (setup and position solves); the velocity
// solves use what setup cached in the joint
__device__ __forceinline__ JBody jbody(const DevWorld &w, int i, bool with_I = true) {
    JBody b;
    uint32_t f = w.flags[i];
    b.i = i;
    b.motion = motion_of(f);
    b.im = w.inv_inertia[i].w;
    b.I = (with_I && b.motion == DYNAMIC)
              ? world_inv_inertia(w.quat[i], w.inertia_rot[i], xyz(w.inv_inertia[i]), dof_of(f))
              : sym_zero();
    return b;
}
__device__ __forceinline__ void add_lin(DevWorld &w, int i, float3 d) {
    float4 v = w.linvel[i];
    w.linvel[i] = make_float4(v.x + d.x, v.y + d.y, v.z + d.z, v.w);
}
__device__ __forceinline__ void add_ang(DevWorld &w, int i, float3 d) {
    float4 v = w.angvel[i];
    w.angvel[i] = make_float4(v.x + d.x, v.y + d.y, v.z + d.z, v.w);
}

// ---- spring part ----------------------------------------------------------------------
__device__ float spring_settings(float &soft, float &bias_out, float dt, float iem, float bias, float C, int mode,
                                 float fs, float damping) {
    float k, c;
    if (mode == 0) {  // FREQUENCY_AND_DAMPING
        float em = 1.f / iem;
        if (!(fs > 0.f)) {
            soft = 0.f;
            bias_out = bias;
            return em;
        }
        float omega = 2.f * 3.14159265358979f * fs;
        k = em * omega * omega;
        c = 2.f * em * damping * omega;
    } else {
        if (!(fs > 0.f)) {
            soft = 0.f;
            bias_out = bias;
            return 1.f / iem;
        }
        k = fs;
        c = damping;
    }
    soft = 1.f / (dt * (c + dt * k));
    bias_out = bias + dt * k * soft * C;
    return 1.f / (iem + soft);
}

// ---- point part (point-constraint-part.ts) ---------------------------------------------
__device__ void point_deactivate(DevPoint &p) {
    for (int k = 0; k < 9; k++) p.eff[k] = 0.f;
    p.lambda = f3(0.f, 0.f, 0.f);
    p.active = 0;
}
__device__ void point_calc(DevPoint &p, const JBody &A, const JBody &B, float4 qa, float4 qb, float3 lp1, float3 lp2) {
    p.r1 = qrot(qa, lp1);
    p.r2 = qrot(qb, lp2);
    float iem[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    float sm = 0.f;
    float I[9], X[9], T[9], T2[9];
    if (A.motion == DYNAMIC) {
        sm += A.im;
        jm_from_sym(I, A.I);
        jm_cross(X, p.r1);
        jm_mm(p.invI1_r1X, I, X);
        jm_mm(T, X, I);
        jm_mm_bt(T2, T, X);
        for (int k = 0; k < 9; k++) iem[k] += T2[k];
    } else {
        for (int k = 0; k < 9; k++) p.invI1_r1X[k] = 0.f;
    }
    if (B.motion == DYNAMIC) {
        sm += B.im;
        jm_from_sym(I, B.I);
        jm_cross(X, p.r2);
        jm_mm(p.invI2_r2X, I, X);
        jm_mm(T, X, I);
        jm_mm_bt(T2, T, X);
        for (int k = 0; k < 9; k++) iem[k] += T2[k];
    } else {
        for (int k = 0; k < 9; k++) p.invI2_r2X[k] = 0.f;
    }
    iem[0] += sm;
    iem[4] += sm;
    iem[8] += sm;
    if (jm_invert(p.eff, iem))
        p.active = 1;
    else
        point_deactivate(p);
}
__device__ bool point_apply(DevWorld &w, const DevPoint &p, const JBody &A, const JBody &B, float3 l) {
    if (lensq3(l) == 0.f) return false;
    if (A.motion == DYNAMIC) {
        add_lin(w, A.i, l * (-A.im));
        add_ang(w, A.i, -jm_mv(p.invI1_r1X, l));
    }
    if (B.motion == DYNAMIC) {
        add_lin(w, B.i, l * B.im);
        add_ang(w, B.i, jm_mv(p.invI2_r2X, l));
    }
    return true;
}
__device__ void point_warm(DevWorld &w, DevPoint &p, const JBody &A, const JBody &B, float ratio) {
    if (!p.active) return;
    p.lambda = p.lambda * ratio;
    point_apply(w, p, A, B, p.lambda);
}
__device__ bool point_solve_velocity(DevWorld &w, DevPoint &p, const JBody &A, const JBody &B) {
    if (!p.active) return false;
    float3 jv = xyz(w.linvel[A.i]) - cross3(p.r1, xyz(w.angvel[A.i])) - xyz(w.linvel[B.i]) +
                cross3(p.r2, xyz(w.angvel[B.i]));
    float3 l = jm_mv(p.eff, jv);
    p.lambda = p.lambda + l;
    return point_apply(w, p, A, B, l);
}

// position steps (rigid-body-step.ts:16-97)
__device__ __forceinline__ void add_position_step(DevWorld &w, int i, float3 d) {
    float4 c = w.com[i];
    float3 p = f3(c.x + d.x, c.y + d.y, c.z + d.z);
    int dof = dof_of(w.flags[i]);
    if (!(dof & 1)) p.x = 0.f;
    if (!(dof & 2)) p.y = 0.f;
    if (!(dof & 4)) p.z = 0.f;
    w.com[i] = make_float4(p.x, p.y, p.z, 0.f);
}
__device__ __forceinline__ void add_rotation(DevWorld &w, int i, float3 a) { w.quat[i] = rotation_step(w.quat[i], a); }

// solvePositionConstraint of the point part, after point_calc on the current poses
__device__ bool point_solve_position(DevWorld &w, DevPoint &p, const JBody &A, const JBody &B, float beta) {
    if (!p.active) return false;
    float3 sep = xyz(w.com[B.i]) + p.r2 - xyz(w.com[A.i]) - p.r1;
    if (lensq3(sep) < 1e-12f) return false;
    float3 l = jm_mv(p.eff, sep) * (-beta);
    if (A.motion == DYNAMIC) {
        add_position_step(w, A.i, l * (-A.im));
        add_rotation(w, A.i, -jm_mv(p.invI1_r1X, l));
    }
    if (B.motion == DYNAMIC) {
        add_position_step(w, B.i, l * B.im);
        add_rotation(w, B.i, jm_mv(p.invI2_r2X, l));
    }
    return true;
}

// ---- hinge rotation part (hinge-rotation-constraint-part.ts) --------------------------
__device__ __forceinline__ float3 perpendicular3(float3 v) {
    if (fabsf(v.x) > fabsf(v.y)) {
        float l = sqrtf(v.x * v.x + v.z * v.z);
        return f3(v.z / l, 0.f, -v.x / l);
    }
    float l = sqrtf(v.y * v.y + v.z * v.z);
    return f3(0.f, v.z / l, -v.y / l);
}
__device__ void hrot_deactivate(DevHinge &j) {
    j.r_eff[0] = j.r_eff[1] = j.r_eff[2] = j.r_eff[3] = 0.f;
    j.r_lambda[0] = j.r_lambda[1] = 0.f;
}
__device__ __forceinline__ bool hrot_active(const DevHinge &j) {
    return j.r_eff[0] != 0.f || j.r_eff[1] != 0.f || j.r_eff[2] != 0.f || j.r_eff[3] != 0.f;
}
__device__ void hrot_calc(DevHinge &j, const JBody &A, const JBody &B, float3 axis1, float3 axis2) {
    j.a1 = axis1;
    float3 a2 = axis2;
    float d = dot3(j.a1, a2);
    if (d <= 1.0e-3f) {
        float3 perp = a2 + j.a1 * (-d);
        if (lensq3(perp) < 1.0e-6f) perp = perpendicular3(j.a1);
        perp = normalize3(perp);
        a2 = j.a1 * 0.01f + perp * 0.99f;
        a2 = normalize3(a2);
    }
    j.b2 = perpendicular3(a2);
    j.c2 = cross3(a2, j.b2);
    sym_store(j.invI1, A.I);
    sym_store(j.invI2, B.I);
    j.b2xA1 = cross3(j.b2, j.a1);
    j.c2xA1 = cross3(j.c2, j.a1);
    Sym3 sum{A.I.xx + B.I.xx, A.I.xy + B.I.xy, A.I.xz + B.I.xz, A.I.yy + B.I.yy, A.I.yz + B.I.yz, A.I.zz + B.I.zz};
    float3 t = symmul(sum, j.b2xA1);
    double k0 = dot3(j.b2xA1, t), k2 = dot3(j.c2xA1, t);
    t = symmul(sum, j.c2xA1);
    double k1 = dot3(j.b2xA1, t), k3 = dot3(j.c2xA1, t);
    double det = k0 * k3 - k1 * k2;
    if (fabs(det) < 1e-10) {
        hrot_deactivate(j);
        return;
    }
    double id = 1.0 / det;
    j.r_eff[0] = (float)(k3 * id);
    j.r_eff[1] = (float)(-k1 * id);
    j.r_eff[2] = (float)(-k2 * id);
    j.r_eff[3] = (float)(k0 * id);
}
__device__ bool hrot_apply(DevWorld &w, const DevHinge &j, const JBody &A, const JBody &B, float l0, float l1) {
    if (l0 == 0.f && l1 == 0.f) return false;
    float3 imp = j.b2xA1 * l0 + j.c2xA1 * l1;
    if (A.motion == DYNAMIC) add_ang(w, A.i, -symmul(sym_load(j.invI1), imp));
    if (B.motion == DYNAMIC) add_ang(w, B.i, symmul(sym_load(j.invI2), imp));
    return true;
}
__device__ bool hrot_solve_velocity(DevWorld &w, DevHinge &j, const JBody &A, const JBody &B) {
    if (!hrot_active(j)) return false;
    float j0 = 0.f, j1 = 0.f;
    if (A.motion != STATIC) {
        float3 wa = xyz(w.angvel[A.i]);
        j0 += dot3(j.b2xA1, wa);
        j1 += dot3(j.c2xA1, wa);
    }
    if (B.motion != STATIC) {
        float3 wb = xyz(w.angvel[B.i]);
        j0 -= dot3(j.b2xA1, wb);
        j1 -= dot3(j.c2xA1, wb);
    }
    float l0 = j.r_eff[0] * j0 + j.r_eff[1] * j1, l1 = j.r_eff[2] * j0 + j.r_eff[3] * j1;
    j.r_lambda[0] += l0;
    j.r_lambda[1] += l1;
    return hrot_apply(w, j, A, B, l0, l1);
}

// ---- angle part (angle-constraint-part.ts) ---------------------------------------------
__device__ __forceinline__ void angle_deactivate(DevAngle &p) {
    p.eff = 0.f;
    p.lambda = 0.f;
}
__device__ float angle_iem(DevAngle &p, const JBody &A, const JBody &B, float3 axis) {
    p.i1 = A.motion == DYNAMIC ? symmul(A.I, axis) : f3(0.f, 0.f, 0.f);
    p.i2 = B.motion == DYNAMIC ? symmul(B.I, axis) : f3(0.f, 0.f, 0.f);
    return dot3(axis, p.i1 + p.i2);
}
__device__ void angle_calc(DevAngle &p, const JBody &A, const JBody &B, float3 axis, float bias) {
    float iem = angle_iem(p, A, B, axis);
    if (iem == 0.f) {
        angle_deactivate(p);
    } else {
        p.eff = 1.f / iem;
        p.soft = 0.f;
        p.bias = bias;
    }
}
__device__ void angle_calc_settings(DevAngle &p, float dt, const JBody &A, const JBody &B, float3 axis, float bias,
                                    float C, int mode, float fs, float damping) {
    float iem = angle_iem(p, A, B, axis);
    if (iem == 0.f)
        angle_deactivate(p);
    else
        p.eff = spring_settings(p.soft, p.bias, dt, iem, bias, C, mode, fs, damping);
}
__device__ bool angle_apply(DevWorld &w, const DevAngle &p, const JBody &A, const JBody &B, float l) {
    if (l == 0.f) return false;
    if (A.motion == DYNAMIC) add_ang(w, A.i, -(p.i1 * l));
    if (B.motion == DYNAMIC) add_ang(w, B.i, p.i2 * l);
    return true;
}
__device__ void angle_warm(DevWorld &w, DevAngle &p, const JBody &A, const JBody &B, float ratio) {
    p.lambda *= ratio;
    angle_apply(w, p, A, B, p.lambda);
}
__device__ bool angle_solve_velocity(DevWorld &w, DevAngle &p, const JBody &A, const JBody &B, float3 axis, float mn,
                                     float mx) {
    if (p.eff == 0.f) return false;
    float jv = 0.f;
    if (A.motion != STATIC) jv += dot3(axis, xyz(w.angvel[A.i]));
    if (B.motion != STATIC) jv -= dot3(axis, xyz(w.angvel[B.i]));
    float l = p.eff * (jv - (p.soft * p.lambda + p.bias));
    float nl = fmaxf(mn, fminf(mx, p.lambda + l));
    float dl = nl - p.lambda;
    p.lambda = nl;
    return angle_apply(w, p, A, B, dl);
}

// ---- hinge (hinge-constraint.ts) -------------------------------------------------------
__device__ __forceinline__ float center_angle(float a) {
    const float PI = 3.14159265358979f;
    while (a > PI) a -= 2.f * PI;
    while (a < -PI) a += 2.f * PI;
    return a;
}
// calculateA1AndTheta
__device__ void hinge_theta(DevHinge &j, float4 qa, float4 qb) {
    if (!(j.h.flags & JF_LIMITS) && j.motor_state == 0 && !(j.max_friction_torque > 0.f)) return;
    float3 wh = qrot(qa, j.lh1);
    j.wh1 = wh;
    float4 rel = qmul(qmul(qb, j.inv_initial), make_float4(-qa.x, -qa.y, -qa.z, qa.w));
    float ad = wh.x * rel.x + wh.y * rel.y + wh.z * rel.z;
    j.theta = rel.w == 0.f ? 3.14159265358979f : 2.f * atanf(ad / rel.w);
}
__device__ __forceinline__ float hinge_to_limit(const DevHinge &j) {
    float dmn = center_angle(j.theta - j.limits_min), dmx = center_angle(j.theta - j.limits_max);
    return fabsf(dmn) < fabsf(dmx) ? dmn : dmx;
}
__device__ __forceinline__ bool hinge_min_closest(const DevHinge &j) {
    return fabsf(center_angle(j.theta - j.limits_min)) < fabsf(center_angle(j.theta - j.limits_max));
}
__device__ void hinge_limit_props(DevHinge &j, const JBody &A, const JBody &B, float dt) {
    if ((j.h.flags & JF_LIMITS) && (j.theta <= j.limits_min || j.theta >= j.limits_max))
        angle_calc_settings(j.limit, dt, A, B, j.wh1, 0.f, hinge_to_limit(j), j.limits_spring_mode, j.limits_freq,
                            j.limits_damping);
    else
        angle_deactivate(j.limit);
}
__device__ void hinge_motor_props(DevHinge &j, const JBody &A, const JBody &B, float dt) {
    if (j.motor_state == 0) {
        if (j.max_friction_torque > 0.f)
            angle_calc(j.motor, A, B, j.wh1, 0.f);
        else
            angle_deactivate(j.motor);
    } else if (j.motor_state == 1) {
        angle_calc(j.motor, A, B, j.wh1, -j.target_angular_velocity);
    } else {
        if (j.motor_freq > 0.f)
            angle_calc_settings(j.motor, dt, A, B, j.wh1, 0.f, center_angle(j.theta - j.target_angle),
                                j.motor_spring_mode, j.motor_freq, j.motor_damping);
        else
            angle_deactivate(j.motor);
    }
}
// setupVelocity
__device__ void hinge_setup(DevWorld &w, DevHinge &j, float dt) {
    JBody A = jbody(w, j.h.a), B = jbody(w, j.h.b);
    float4 qa = w.quat[j.h.a], qb = w.quat[j.h.b];
    point_calc(j.pt, A, B, qa, qb, j.lp1, j.lp2);
    hrot_calc(j, A, B, qrot(qa, j.lh1), qrot(qb, j.lh2));
    hinge_theta(j, qa, qb);
    hinge_limit_props(j, A, B, dt);
    hinge_motor_props(j, A, B, dt);
}
// warmStartVelocity: motor, point, rotation, limits
__device__ void hinge_warm(DevWorld &w, DevHinge &j, float ratio) {
    JBody A = jbody(w, j.h.a, false), B = jbody(w, j.h.b, false);
    angle_warm(w, j.motor, A, B, ratio);
    point_warm(w, j.pt, A, B, ratio);
    j.r_lambda[0] *= ratio;
    j.r_lambda[1] *= ratio;
    hrot_apply(w, j, A, B, j.r_lambda[0], j.r_lambda[1]);
    angle_warm(w, j.limit, A, B, ratio);
}
// solveVelocity
__device__ bool hinge_solve_velocity(DevWorld &w, DevHinge &j, float dt) {
    JBody A = jbody(w, j.h.a, false), B = jbody(w, j.h.b, false);
    const float INF = __int_as_float(0x7f800000);
    bool motor = false, limit = false;
    if (j.motor.eff != 0.f) {
        if (j.motor_state == 0) {
            float ml = j.max_friction_torque * dt;
            motor = angle_solve_velocity(w, j.motor, A, B, j.wh1, -ml, ml);
        } else {
            motor = angle_solve_velocity(w, j.motor, A, B, j.wh1, dt * j.min_torque, dt * j.max_torque);
        }
    }
    bool pos = point_solve_velocity(w, j.pt, A, B);
    bool rot = hrot_solve_velocity(w, j, A, B);
    if (j.limit.eff != 0.f) {
        float mn, mx;
        if (j.limits_min == j.limits_max) {
            mn = -INF;
            mx = INF;
        } else if (hinge_min_closest(j)) {
            mn = 0.f;
            mx = INF;
        } else {
            mn = -INF;
            mx = 0.f;
        }
        limit = angle_solve_velocity(w, j.limit, A, B, j.wh1, mn, mx);
    }
    return motor || pos || rot || limit;
}
// solvePosition
__device__ bool hinge_solve_position(DevWorld &w, DevHinge &j, float dt) {
    const float beta = c_settings.baumgarte;
    JBody A = jbody(w, j.h.a), B = jbody(w, j.h.b);
    point_calc(j.pt, A, B, w.quat[j.h.a], w.quat[j.h.b], j.lp1, j.lp2);
    bool pos = point_solve_position(w, j.pt, A, B, beta);
    A = jbody(w, j.h.a);
    B = jbody(w, j.h.b);
    float4 qa = w.quat[j.h.a], qb = w.quat[j.h.b];
    hrot_calc(j, A, B, qrot(qa, j.lh1), qrot(qb, j.lh2));
    bool rot = false;
    if (hrot_active(j)) {
        float c0 = dot3(j.a1, j.b2), c1 = dot3(j.a1, j.c2);
        if (!(fabsf(c0) < 1e-10f && fabsf(c1) < 1e-10f)) {
            float l0 = -beta * (j.r_eff[0] * c0 + j.r_eff[1] * c1), l1 = -beta * (j.r_eff[2] * c0 + j.r_eff[3] * c1);
            float3 imp = j.b2xA1 * l0 + j.c2xA1 * l1;
            if (A.motion == DYNAMIC) add_rotation(w, A.i, -symmul(sym_load(j.invI1), imp));
            if (B.motion == DYNAMIC) add_rotation(w, B.i, symmul(sym_load(j.invI2), imp));
            rot = true;
        }
    }
    bool limit = false;
    if ((j.h.flags & JF_LIMITS) && !(j.limits_freq > 0.f)) {
        A = jbody(w, j.h.a);
        B = jbody(w, j.h.b);
        hinge_theta(j, w.quat[j.h.a], w.quat[j.h.b]);
        hinge_limit_props(j, A, B, dt);
        float C = hinge_to_limit(j);
        if (j.limit.eff != 0.f && C != 0.f && j.limit.soft == 0.f) {
            float l = -j.limit.eff * beta * C;
            if (A.motion == DYNAMIC) add_rotation(w, A.i, -(j.limit.i1 * l));
            if (B.motion == DYNAMIC) add_rotation(w, B.i, j.limit.i2 * l);
            limit = true;
        }
    }
    return pos || rot || limit;
}

// ---- swing-twist limits (swing-twist-constraint-part.ts) -------------------------------
// calculateConstraintProperties :481-652 (limit axes and their angle parts)
template <class P>
__device__ void st_calc(P &p, const JBody &A, const JBody &B, float4 q, float4 c2w) {
    float4 sw, tw;
    get_swing_twist(q, sw, tw);
    float4 csw = sw, ctw = tw;
    int cl = clamp_swing_twist(p, csw, ctw);
    int rf = p.rotation_flags;
    const float3 X = f3(1.f, 0.f, 0.f), Y = f3(0.f, 1.f, 0.f), Z = f3(0.f, 0.f, 1.f);
    float4 t2w = qmul(c2w, sw);
    if (rf & ST_SWING_Y_LOCKED) {
        p.ws_y = qrot(t2w, Y);
        p.ws_z = qrot(t2w, Z);
        angle_calc(p.sy, A, B, p.ws_y, 0.f);
        if (rf & ST_SWING_Z_LOCKED) {
            angle_calc(p.sz, A, B, p.ws_z, 0.f);
        } else if (cl & (CL_Z_MIN | CL_Z_MAX)) {
            if (cl & CL_Z_MIN) p.ws_z = -p.ws_z;
            angle_calc(p.sz, A, B, p.ws_z, 0.f);
        } else {
            angle_deactivate(p.sz);
        }
    } else if (rf & ST_SWING_Z_LOCKED) {
        p.ws_y = qrot(t2w, Y);
        p.ws_z = qrot(t2w, Z);
        if (cl & (CL_Y_MIN | CL_Y_MAX)) {
            if (cl & CL_Y_MIN) p.ws_y = -p.ws_y;
            angle_calc(p.sy, A, B, p.ws_y, 0.f);
        } else {
            angle_deactivate(p.sy);
        }
        angle_calc(p.sz, A, B, p.ws_z, 0.f);
    } else if ((rf & ST_SWING_YZ_FREE) != ST_SWING_YZ_FREE) {
        if (cl & (CL_Y_MIN | CL_Y_MAX | CL_Z_MIN | CL_Z_MAX)) {
            float3 current = qrot(t2w, X), desired = qrot(qmul(c2w, csw), X);
            float3 c = cross3(desired, current);
            float l = sqrtf(lensq3(c));
            if (l > 1e-6f) {
                p.ws_y = c * (1.f / l);
                angle_calc(p.sy, A, B, p.ws_y, 0.f);
            } else {
                angle_deactivate(p.sy);
            }
        } else {
            angle_deactivate(p.sy);
        }
        angle_deactivate(p.sz);
    } else {
        angle_deactivate(p.sy);
        angle_deactivate(p.sz);
    }
    if (rf & ST_TWIST_LOCKED) {
        p.ws_twist = qrot(t2w, X);
        angle_calc(p.tw, A, B, p.ws_twist, 0.f);
    } else if (!(rf & ST_TWIST_FREE)) {
        if (cl & (CL_TWIST_MIN | CL_TWIST_MAX)) {
            p.ws_twist = qrot(t2w, X);
            if (cl & CL_TWIST_MIN) p.ws_twist = -p.ws_twist;
            angle_calc(p.tw, A, B, p.ws_twist, 0.f);
        } else {
            angle_deactivate(p.tw);
        }
    } else {
        angle_deactivate(p.tw);
    }
}
// solvePositionConstraint :743-776 through a RotationEulerConstraintPart
// (rotation-euler-constraint-part.ts calculateConstraintProperties, solvePositionConstraint)
template <class P>
__device__ bool st_solve_position(DevWorld &w, P &p, const JBody &A, const JBody &B, float4 q, float beta) {
    float4 sw, tw;
    get_swing_twist(q, sw, tw);
    if (clamp_swing_twist(p, sw, tw) == 0) return false;
    float4 inv_initial = qmul(p.c2b2, qconj4(qmul(qmul(p.c2b1, sw), tw)));
    float I1[9], I2[9], S[9], eff[9];
    jm_from_sym(I1, A.I);
    jm_from_sym(I2, B.I);
    for (int k = 0; k < 9; k++) S[k] = I1[k] + I2[k];
    if (!jm_invert(eff, S))
        for (int k = 0; k < 9; k++) eff[k] = 0.f;
    float4 qa = w.quat[A.i], qb = w.quat[B.i];
    float4 diff = qmul(qmul(qb, inv_initial), qconj4(qa));
    if (diff.w < 0.f) diff = qscale4(diff, -1.f);
    float3 err = f3(2.f * diff.x, 2.f * diff.y, 2.f * diff.z);
    if (lensq3(err) < 1e-12f) return false;
    float3 l = jm_mv(eff, err) * (-beta);
    if (A.motion == DYNAMIC) add_rotation(w, A.i, -jm_mv(I1, l));
    if (B.motion == DYNAMIC) add_rotation(w, B.i, jm_mv(I2, l));
    return true;
}
// warm start and velocity solve of the three limit parts (swing-twist-constraint-part.ts
// warmStart, solveVelocityConstraint): swing Y, swing Z, twist
template <class P>
__device__ void st_warm(DevWorld &w, P &p, const JBody &A, const JBody &B, float ratio) {
    angle_warm(w, p.sy, A, B, ratio);
    angle_warm(w, p.sz, A, B, ratio);
    angle_warm(w, p.tw, A, B, ratio);
}
template <class P>
__device__ bool st_solve_velocity(DevWorld &w, P &p, const JBody &A, const JBody &B) {
    const float INF = __int_as_float(0x7f800000);
    bool imp = false;
    if (p.sy.eff != 0.f)
        imp = angle_solve_velocity(w, p.sy, A, B, p.ws_y, -INF, p.sin_y_min == p.sin_y_max ? INF : 0.f) || imp;
    if (p.sz.eff != 0.f)
        imp = angle_solve_velocity(w, p.sz, A, B, p.ws_z, -INF, p.sin_z_min == p.sin_z_max ? INF : 0.f) || imp;
    if (p.tw.eff != 0.f)
        imp = angle_solve_velocity(w, p.tw, A, B, p.ws_twist, -INF, p.sin_twist_min == p.sin_twist_max ? INF : 0.f) ||
              imp;
    return imp;
}

// ---- swing-twist (swing-twist-constraint.ts) ------------------------------------------
// setupVelocity :484-666
__device__ void swing_setup(DevWorld &w, DevSwing &j, float dt) {
    JBody A = jbody(w, j.h.a), B = jbody(w, j.h.b);
    float4 qa = w.quat[j.h.a], qb = w.quat[j.h.b];
    point_calc(j.pt, A, B, qa, qb, j.lp1, j.lp2);
    float4 c1w = qmul(qa, j.c2b1), c2w = qmul(qb, j.c2b2);
    float4 q = qmul(qconj4(c1w), c2w);
    st_calc(j, A, B, q, c1w);
    if (j.swing_motor_state != 0 || j.twist_motor_state != 0 || j.max_friction_torque > 0.f) {
        j.ws_motor[0] = qrot(c2w, f3(1.f, 0.f, 0.f));
        j.ws_motor[1] = qrot(c2w, f3(0.f, 1.f, 0.f));
        j.ws_motor[2] = qrot(c2w, f3(0.f, 0.f, 1.f));
        float e[3] = {0.f, 0.f, 0.f};
        if (j.swing_motor_state == 2 || j.twist_motor_state == 2) {
            float4 t = j.target_q;
            if (q.x * t.x + q.y * t.y + q.z * t.z + q.w * t.w < 0.f) t = qscale4(t, -1.f);
            float4 d = qmul(qconj4(q), t);
            e[0] = -2.f * d.x;
            e[1] = -2.f * d.y;
            e[2] = -2.f * d.z;
        }
        float tav[3] = {j.target_w.x, j.target_w.y, j.target_w.z};
        if (j.swing_motor_state == 0) {
            if (j.max_friction_torque > 0.f) {
                for (int i = 1; i < 3; i++) angle_calc(j.motor[i], A, B, j.ws_motor[i], 0.f);
            } else {
                for (int i = 0; i < 3; i++) angle_deactivate(j.motor[i]);
            }
        } else if (j.swing_motor_state == 1) {
            for (int i = 1; i < 3; i++) angle_calc(j.motor[i], A, B, j.ws_motor[i], -tav[i]);
        } else if (j.swing_freq > 0.f) {
            for (int i = 1; i < 3; i++)
                angle_calc_settings(j.motor[i], dt, A, B, j.ws_motor[i], 0.f, e[i], j.swing_spring_mode, j.swing_freq,
                                    j.swing_damping);
        } else {
            for (int i = 1; i < 3; i++) angle_deactivate(j.motor[i]);
        }
        if (j.twist_motor_state == 0) {
            if (j.max_friction_torque > 0.f)
                angle_calc(j.motor[0], A, B, j.ws_motor[0], 0.f);
            else
                angle_deactivate(j.motor[0]);
        } else if (j.twist_motor_state == 1) {
            angle_calc(j.motor[0], A, B, j.ws_motor[0], -tav[0]);
        } else if (j.twist_freq > 0.f) {
            angle_calc_settings(j.motor[0], dt, A, B, j.ws_motor[0], 0.f, e[0], j.twist_spring_mode, j.twist_freq,
                                j.twist_damping);
        } else {
            angle_deactivate(j.motor[0]);
        }
    } else {
        for (int i = 0; i < 3; i++) angle_deactivate(j.motor[i]);
    }
}
// warmStartVelocity :668-680: motors, limits, point
__device__ void swing_warm(DevWorld &w, DevSwing &j, float ratio) {
    JBody A = jbody(w, j.h.a, false), B = jbody(w, j.h.b, false);
    for (int i = 0; i < 3; i++) angle_warm(w, j.motor[i], A, B, ratio);
    angle_warm(w, j.sy, A, B, ratio);
    angle_warm(w, j.sz, A, B, ratio);
    angle_warm(w, j.tw, A, B, ratio);
    point_warm(w, j.pt, A, B, ratio);
}
// solveVelocity :682-748
__device__ bool swing_solve_velocity(DevWorld &w, DevSwing &j, float dt) {
    JBody A = jbody(w, j.h.a, false), B = jbody(w, j.h.b, false);
    const float INF = __int_as_float(0x7f800000);
    bool imp = false;
    if (j.motor[0].eff != 0.f) {
        float mn, mx;
        if (j.twist_motor_state == 0) {
            mx = dt * j.max_friction_torque;
            mn = -mx;
        } else {
            mn = dt * j.twist_min_torque;
            mx = dt * j.twist_max_torque;
        }
        imp = angle_solve_velocity(w, j.motor[0], A, B, j.ws_motor[0], mn, mx) || imp;
    }
    if (j.motor[1].eff != 0.f) {
        float mn, mx;
        if (j.swing_motor_state == 0) {
            mx = dt * j.max_friction_torque;
            mn = -mx;
        } else {
            mn = dt * j.swing_min_torque;
            mx = dt * j.swing_max_torque;
        }
        for (int i = 1; i < 3; i++) imp = angle_solve_velocity(w, j.motor[i], A, B, j.ws_motor[i], mn, mx) || imp;
    }
    if (j.sy.eff != 0.f)
        imp = angle_solve_velocity(w, j.sy, A, B, j.ws_y, -INF, j.sin_y_min == j.sin_y_max ? INF : 0.f) || imp;
    if (j.sz.eff != 0.f)
        imp = angle_solve_velocity(w, j.sz, A, B, j.ws_z, -INF, j.sin_z_min == j.sin_z_max ? INF : 0.f) || imp;
    if (j.tw.eff != 0.f)
        imp = angle_solve_velocity(w, j.tw, A, B, j.ws_twist, -INF, j.sin_twist_min == j.sin_twist_max ? INF : 0.f) ||
              imp;
    imp = point_solve_velocity(w, j.pt, A, B) || imp;
    return imp;
}
// solvePosition :757-800: rotation limits, then the point from the corrected poses
__device__ bool swing_solve_position(DevWorld &w, DevSwing &j) {
    const float beta = c_settings.baumgarte;
    JBody A = jbody(w, j.h.a), B = jbody(w, j.h.b);
    float4 qa = w.quat[j.h.a], qb = w.quat[j.h.b];
    float4 q = qmul(qconj4(qmul(qa, j.c2b1)), qmul(qb, j.c2b2));
    bool imp = st_solve_position(w, j, A, B, q, beta);
    A = jbody(w, j.h.a);
    B = jbody(w, j.h.b);
    point_calc(j.pt, A, B, w.quat[j.h.a], w.quat[j.h.b], j.lp1, j.lp2);
    imp = point_solve_position(w, j.pt, A, B, beta) || imp;
    return imp;
}

// ---- velocity steps with the translation DOF lock (motion-properties.ts:702-720) ----------
__device__ __forceinline__ void add_lin_locked(DevWorld &w, int i, float3 d) {
    float4 v = w.linvel[i];
    float3 n = f3(v.x + d.x, v.y + d.y, v.z + d.z);
    const int dof = dof_of(w.flags[i]);
    if (!(dof & 1)) n.x = 0.f;
    if (!(dof & 2)) n.y = 0.f;
    if (!(dof & 4)) n.z = 0.f;
    w.linvel[i] = make_float4(n.x, n.y, n.z, v.w);
}
// AngleConstraintPart.solvePositionConstraint (angle-constraint-part.ts)
__device__ bool angle_solve_position(DevWorld &w, const DevAngle &p, const JBody &A, const JBody &B, float C,
                                     float beta) {
    if (C == 0.f || p.eff == 0.f || p.soft != 0.f) return false;
    const float l = -p.eff * beta * C;
    if (A.motion == DYNAMIC) add_rotation(w, A.i, -(p.i1 * l));
    if (B.motion == DYNAMIC) add_rotation(w, B.i, p.i2 * l);
    return true;
}

// ---- rotation-euler part (rotation-euler-constraint-part.ts) -------------------------
__device__ __forceinline__ void euler_deactivate(DevEuler &p) {
    for (int k = 0; k < 9; k++) p.eff[k] = 0.f;
    p.lambda = f3(0.f, 0.f, 0.f);
}
// calculateConstraintProperties :127-156: K = (I1^-1 + I2^-1)^-1, inverted in FP64
__device__ void euler_calc(DevEuler &p, const JBody &A, const JBody &B) {
    sym_store(p.invI1, A.I);
    sym_store(p.invI2, B.I);
    Sym3 sum{A.I.xx + B.I.xx, A.I.xy + B.I.xy, A.I.xz + B.I.xz, A.I.yy + B.I.yy, A.I.yz + B.I.yz, A.I.zz + B.I.zz};
    float m[9];
    jm_from_sym(m, sum);
    if (!jm_invert(p.eff, m)) euler_deactivate(p);
}
__device__ bool euler_apply(DevWorld &w, const DevEuler &p, const JBody &A, const JBody &B, float3 l) {
    if (lensq3(l) == 0.f) return false;
    if (A.motion == DYNAMIC) add_ang(w, A.i, -symmul(sym_load(p.invI1), l));
    if (B.motion == DYNAMIC) add_ang(w, B.i, symmul(sym_load(p.invI2), l));
    return true;
}
__device__ void euler_warm(DevWorld &w, DevEuler &p, const JBody &A, const JBody &B, float ratio) {
    p.lambda = p.lambda * ratio;
    euler_apply(w, p, A, B, p.lambda);
}
__device__ bool euler_solve_velocity(DevWorld &w, DevEuler &p, const JBody &A, const JBody &B) {
    float3 w1 = A.motion != STATIC ? xyz(w.angvel[A.i]) : f3(0.f, 0.f, 0.f);
    float3 w2 = B.motion != STATIC ? xyz(w.angvel[B.i]) : f3(0.f, 0.f, 0.f);
    float3 l = jm_mv(p.eff, w1 - w2);
    p.lambda = p.lambda + l;
    return euler_apply(w, p, A, B, l);
}
// solvePositionConstraint :256-311: error 2 xyz of q2 invInitial q1^-1 with w made positive
__device__ bool euler_solve_position(DevWorld &w, const DevEuler &p, const JBody &A, const JBody &B, float4 inv_initial,
                                     float beta) {
    float4 diff = qmul(qmul(w.quat[B.i], inv_initial), qconj4(w.quat[A.i]));
    if (diff.w < 0.f) diff = make_float4(-diff.x, -diff.y, -diff.z, -diff.w);
    float3 err = f3(2.f * diff.x, 2.f * diff.y, 2.f * diff.z);
    if (lensq3(err) < 1e-12f) return false;
    float3 l = jm_mv(p.eff, err) * (-beta);
    if (A.motion == DYNAMIC) add_rotation(w, A.i, -symmul(sym_load(p.invI1), l));
    if (B.motion == DYNAMIC) add_rotation(w, B.i, symmul(sym_load(p.invI2), l));
    return true;
}

// ---- axis part of a joint (axis-constraint-part.ts) ----------------------------------
__device__ float axis_iem(DevAxis &p, const JBody &A, const JBody &B, float3 r1, float3 r2, float3 ax) {
    float iem = 0.f;
    p.r1xa = p.r2xa = p.i1 = p.i2 = f3(0.f, 0.f, 0.f);
    if (A.motion == DYNAMIC) {
        p.r1xa = cross3(r1, ax);
        p.i1 = symmul(A.I, p.r1xa);
        iem += A.im + dot3(p.i1, p.r1xa);
    }
    if (B.motion == DYNAMIC) {
        p.r2xa = cross3(r2, ax);
        p.i2 = symmul(B.I, p.r2xa);
        iem += B.im + dot3(p.i2, p.r2xa);
    }
    return iem;
}
__device__ __forceinline__ void axis_deactivate(DevAxis &p) {
    p.eff = 0.f;
    p.lambda = 0.f;
}
__device__ void axis_calc(DevAxis &p, const JBody &A, const JBody &B, float3 r1, float3 r2, float3 ax, float bias) {
    float iem = axis_iem(p, A, B, r1, r2, ax);
    if (iem == 0.f) {
        axis_deactivate(p);
    } else {
        p.eff = 1.f / iem;
        p.soft = 0.f;
        p.bias = bias;
    }
}
__device__ void axis_calc_settings(DevAxis &p, float dt, const JBody &A, const JBody &B, float3 r1, float3 r2,
                                   float3 ax, float bias, float C, int mode, float fs, float damping) {
    float iem = axis_iem(p, A, B, r1, r2, ax);
    if (iem == 0.f)
        axis_deactivate(p);
    else
        p.eff = spring_settings(p.soft, p.bias, dt, iem, bias, C, mode, fs, damping);
}
__device__ void axis_push(DevWorld &w, const DevAxis &p, const JBody &A, const JBody &B, float3 ax, float l) {
    if (A.motion == DYNAMIC) {
        add_lin_locked(w, A.i, ax * (-l * A.im));
        add_ang(w, A.i, -(p.i1 * l));
    }
    if (B.motion == DYNAMIC) {
        add_lin_locked(w, B.i, ax * (l * B.im));
        add_ang(w, B.i, p.i2 * l);
    }
}
__device__ void axis_warm(DevWorld &w, DevAxis &p, const JBody &A, const JBody &B, float3 ax, float ratio) {
    p.lambda *= ratio;
    if (p.lambda == 0.f) return;
    axis_push(w, p, A, B, ax, p.lambda);
}
// solveVelocityConstraint: getTotalLambda :578-625, clamp, applyLambda :640-707
__device__ bool axis_solve_velocity(DevWorld &w, DevAxis &p, const JBody &A, const JBody &B, float3 ax, float mn,
                                    float mx) {
    const bool mA = A.motion != STATIC, mB = B.motion != STATIC;
    float jv = 0.f;
    if (mA && mB)
        jv = dot3(ax, xyz(w.linvel[A.i]) - xyz(w.linvel[B.i]));
    else if (mA)
        jv = dot3(ax, xyz(w.linvel[A.i]));
    else if (mB)
        jv = -dot3(ax, xyz(w.linvel[B.i]));
    if (mA) jv += dot3(p.r1xa, xyz(w.angvel[A.i]));
    if (mB) jv -= dot3(p.r2xa, xyz(w.angvel[B.i]));
    float tl = p.lambda + p.eff * (jv - (p.soft * p.lambda + p.bias));
    tl = fmaxf(mn, fminf(mx, tl));
    const float dl = tl - p.lambda;
    p.lambda = tl;
    if (dl == 0.f) return false;
    axis_push(w, p, A, B, ax, dl);
    return true;
}
// solvePositionConstraintWithMassOverride :790-847
__device__ bool axis_solve_position(DevWorld &w, const DevAxis &p, const JBody &A, const JBody &B, float3 ax, float C,
                                    float beta) {
    if (C == 0.f || p.eff == 0.f || p.soft != 0.f) return false;
    const float l = -p.eff * beta * C;
    if (A.motion == DYNAMIC) {
        add_position_step(w, A.i, ax * (-l * A.im));
        add_rotation(w, A.i, -(p.i1 * l));
    }
    if (B.motion == DYNAMIC) {
        add_position_step(w, B.i, ax * (l * B.im));
        add_rotation(w, B.i, p.i2 * l);
    }
    return true;
}

// ---- dual-axis part (dual-axis-constraint-part.ts) -----------------------------------
__device__ __forceinline__ void dual_deactivate(DevDual &p) {
    p.lambda[0] = p.lambda[1] = 0.f;
    p.eff[0] = p.eff[1] = p.eff[2] = p.eff[3] = 0.f;
}
__device__ __forceinline__ bool dual_active(const DevDual &p) {
    return p.eff[0] != 0.f || p.eff[1] != 0.f || p.eff[2] != 0.f || p.eff[3] != 0.f;
}
// calculateConstraintProperties :78-140; the 2x2 inversion (mat2.invert) in FP64
__device__ void dual_calc(DevDual &p, const JBody &A, float3 r1u, const JBody &B, float3 r2, float3 n1, float3 n2) {
    double iem[4] = {0.0, 0.0, 0.0, 0.0};
    p.r1xn1 = p.r1xn2 = p.r2xn1 = p.r2xn2 = p.i1n1 = p.i1n2 = p.i2n1 = p.i2n2 = f3(0.f, 0.f, 0.f);
    if (A.motion == DYNAMIC) {
        p.r1xn1 = cross3(r1u, n1);
        p.r1xn2 = cross3(r1u, n2);
        p.i1n1 = symmul(A.I, p.r1xn1);
        p.i1n2 = symmul(A.I, p.r1xn2);
        iem[0] += A.im + dot3(p.r1xn1, p.i1n1);
        iem[1] += dot3(p.r1xn2, p.i1n1);
        iem[2] += dot3(p.r1xn1, p.i1n2);
        iem[3] += A.im + dot3(p.r1xn2, p.i1n2);
    }
    if (B.motion == DYNAMIC) {
        p.r2xn1 = cross3(r2, n1);
        p.r2xn2 = cross3(r2, n2);
        p.i2n1 = symmul(B.I, p.r2xn1);
        p.i2n2 = symmul(B.I, p.r2xn2);
        iem[0] += B.im + dot3(p.r2xn1, p.i2n1);
        iem[1] += dot3(p.r2xn2, p.i2n1);
        iem[2] += dot3(p.r2xn1, p.i2n2);
        iem[3] += B.im + dot3(p.r2xn2, p.i2n2);
    }
    double det = iem[0] * iem[3] - iem[2] * iem[1];
    if (det == 0.0) {
        dual_deactivate(p);
        return;
    }
    det = 1.0 / det;
    p.eff[0] = (float)(iem[3] * det);
    p.eff[1] = (float)(-iem[1] * det);
    p.eff[2] = (float)(-iem[2] * det);
    p.eff[3] = (float)(iem[0] * det);
}
__device__ void dual_push(DevWorld &w, const DevDual &p, const JBody &A, const JBody &B, float3 n1, float3 n2, float l0,
                          float l1) {
    const float3 imp = n1 * l0 + n2 * l1;
    if (A.motion == DYNAMIC) {
        add_lin_locked(w, A.i, imp * (-A.im));
        add_ang(w, A.i, -(p.i1n1 * l0 + p.i1n2 * l1));
    }
    if (B.motion == DYNAMIC) {
        add_lin_locked(w, B.i, imp * B.im);
        add_ang(w, B.i, p.i2n1 * l0 + p.i2n2 * l1);
    }
}
__device__ void dual_warm(DevWorld &w, DevDual &p, const JBody &A, const JBody &B, float3 n1, float3 n2, float ratio) {
    if (!dual_active(p)) return;
    p.lambda[0] *= ratio;
    p.lambda[1] *= ratio;
    if (p.lambda[0] == 0.f && p.lambda[1] == 0.f) return;
    dual_push(w, p, A, B, n1, n2, p.lambda[0], p.lambda[1]);
}
__device__ bool dual_solve_velocity(DevWorld &w, DevDual &p, const JBody &A, const JBody &B, float3 n1, float3 n2) {
    if (!dual_active(p)) return false;
    const bool mA = A.motion != STATIC, mB = B.motion != STATIC;
    float j0 = 0.f, j1 = 0.f;
    if (mA) {
        const float3 v = xyz(w.linvel[A.i]), av = xyz(w.angvel[A.i]);
        j0 += dot3(n1, v) + dot3(p.r1xn1, av);
        j1 += dot3(n2, v) + dot3(p.r1xn2, av);
    }
    if (mB) {
        const float3 v = xyz(w.linvel[B.i]), av = xyz(w.angvel[B.i]);
        j0 -= dot3(n1, v) + dot3(p.r2xn1, av);
        j1 -= dot3(n2, v) + dot3(p.r2xn2, av);
    }
    const float l0 = p.eff[0] * j0 + p.eff[2] * j1, l1 = p.eff[1] * j0 + p.eff[3] * j1;
    p.lambda[0] += l0;
    p.lambda[1] += l1;
    if (l0 == 0.f && l1 == 0.f) return false;
    dual_push(w, p, A, B, n1, n2, l0, l1);
    return true;
}
__device__ bool dual_solve_position(DevWorld &w, const DevDual &p, const JBody &A, const JBody &B, float3 u, float3 n1,
                                    float3 n2, float beta) {
    if (!dual_active(p)) return false;
    const float c0 = dot3(u, n1), c1 = dot3(u, n2);
    if (c0 == 0.f && c1 == 0.f) return false;
    const float l0 = -beta * (p.eff[0] * c0 + p.eff[2] * c1), l1 = -beta * (p.eff[1] * c0 + p.eff[3] * c1);
    if (l0 == 0.f && l1 == 0.f) return false;
    const float3 imp = n1 * l0 + n2 * l1;
    if (A.motion == DYNAMIC) {
        add_position_step(w, A.i, imp * (-A.im));
        add_rotation(w, A.i, -(p.i1n1 * l0 + p.i1n2 * l1));
    }
    if (B.motion == DYNAMIC) {
        add_position_step(w, B.i, imp * B.im);
        add_rotation(w, B.i, p.i2n1 * l0 + p.i2n2 * l1);
    }
    return true;
}

// ---- point joint (point-constraint.ts:186-244) ---------------------------------------
__device__ void pointj_setup(DevWorld &w, DevJoint &j) {
    JBody A = jbody(w, j.h.a), B = jbody(w, j.h.b);
    point_calc(j.pt, A, B, w.quat[j.h.a], w.quat[j.h.b], j.lp1, j.lp2);
}
__device__ bool pointj_solve_position(DevWorld &w, DevJoint &j) {
    JBody A = jbody(w, j.h.a), B = jbody(w, j.h.b);
    point_calc(j.pt, A, B, w.quat[j.h.a], w.quat[j.h.b], j.lp1, j.lp2);
    return point_solve_position(w, j.pt, A, B, c_settings.baumgarte);
}

// ---- fixed joint (fixed-constraint.ts:299-395) ---------------------------------------
__device__ void fixed_setup(DevWorld &w, DevJoint &j) {
    JBody A = jbody(w, j.h.a), B = jbody(w, j.h.b);
    euler_calc(j.rot, A, B);
    point_calc(j.pt, A, B, w.quat[j.h.a], w.quat[j.h.b], j.lp1, j.lp2);
}
__device__ bool fixed_solve_position(DevWorld &w, DevJoint &j) {
    const float beta = c_settings.baumgarte;
    JBody A = jbody(w, j.h.a), B = jbody(w, j.h.b);
    euler_calc(j.rot, A, B);
    bool rot = euler_solve_position(w, j.rot, A, B, j.inv_initial, beta);
    A = jbody(w, j.h.a);
    B = jbody(w, j.h.b);
    point_calc(j.pt, A, B, w.quat[j.h.a], w.quat[j.h.b], j.lp1, j.lp2);
    bool pos = point_solve_position(w, j.pt, A, B, beta);
    return rot || pos;
}

// ---- distance joint (distance-constraint.ts:270-465) ---------------------------------
__device__ void distance_calc(DevWorld &w, DevJoint &j, const JBody &A, const JBody &B, float dt) {
    const float3 ca = xyz(w.com[j.h.a]), cb = xyz(w.com[j.h.b]);
    j.wp1 = qrot(w.quat[j.h.a], j.lp1) + ca;
    j.wp2 = qrot(w.quat[j.h.b], j.lp2) + cb;
    const float3 delta = j.wp2 - j.wp1;
    const float dl = sqrtf(lensq3(delta));
    if (dl > 0.f) j.wn = delta * (1.f / dl);
    const float3 r1u = j.wp2 - ca, r2 = j.wp2 - cb;
    const float INF = __int_as_float(0x7f800000);
    float C;
    if (j.min_dist == j.max_dist) {  // a rod: both directions
        C = dl - j.min_dist;
        j.min_lambda = -INF;
        j.max_lambda = INF;
    } else if (dl <= j.min_dist) {  // too close: push apart only
        C = dl - j.min_dist;
        j.min_lambda = 0.f;
        j.max_lambda = INF;
    } else if (dl >= j.max_dist) {  // too far: pull together only
        C = dl - j.max_dist;
        j.min_lambda = -INF;
        j.max_lambda = 0.f;
    } else {
        axis_deactivate(j.ax);
        return;
    }
    axis_calc_settings(j.ax, dt, A, B, r1u, r2, j.wn, 0.f, C, j.spring_mode, j.spring_freq, j.spring_damping);
}
__device__ bool distance_solve_position(DevWorld &w, DevJoint &j, float dt) {
    if (j.spring_freq > 0.f) return false;
    // the error on the world points of the last property calculation (setup, or the previous
    // position iteration), then the properties are refreshed (solvePosition :420-458)
    const float d = dot3(j.wp2 - j.wp1, j.wn);
    float err = 0.f;
    if (d < j.min_dist)
        err = d - j.min_dist;
    else if (d > j.max_dist)
        err = d - j.max_dist;
    if (err == 0.f) return false;
    JBody A = jbody(w, j.h.a), B = jbody(w, j.h.b);
    distance_calc(w, j, A, B, dt);
    return axis_solve_position(w, j.ax, A, B, j.wn, err, c_settings.baumgarte);
}

// ---- cone joint (cone-constraint.ts:321-448) -----------------------------------------
__device__ void cone_rot_calc(DevWorld &w, DevJoint &j, const JBody &A, const JBody &B) {
    const float3 t1 = qrot(w.quat[j.h.a], j.lt1), t2 = qrot(w.quat[j.h.b], j.lt2);
    j.cos_theta = dot3(t1, t2);
    if (j.cos_theta < j.cos_half_cone) {
        const float3 ra = cross3(t2, t1);
        const float l = sqrtf(lensq3(ra));
        if (l > 1e-6f) j.w_rot_axis = ra * (1.f / l);
        angle_calc(j.ang, A, B, j.w_rot_axis, 0.f);
    } else {
        angle_deactivate(j.ang);
    }
}
__device__ void cone_setup(DevWorld &w, DevJoint &j) {
    JBody A = jbody(w, j.h.a), B = jbody(w, j.h.b);
    point_calc(j.pt, A, B, w.quat[j.h.a], w.quat[j.h.b], j.lp1, j.lp2);
    cone_rot_calc(w, j, A, B);
}
__device__ bool cone_solve_position(DevWorld &w, DevJoint &j) {
    const float beta = c_settings.baumgarte;
    JBody A = jbody(w, j.h.a), B = jbody(w, j.h.b);
    point_calc(j.pt, A, B, w.quat[j.h.a], w.quat[j.h.b], j.lp1, j.lp2);
    bool pos = point_solve_position(w, j.pt, A, B, beta);
    A = jbody(w, j.h.a);
    B = jbody(w, j.h.b);
    cone_rot_calc(w, j, A, B);
    bool rot = false;
    if (j.ang.eff != 0.f) rot = angle_solve_position(w, j.ang, A, B, j.cos_theta - j.cos_half_cone, beta);
    return pos || rot;
}

// ---- slider joint (slider-constraint.ts:546-1038) ------------------------------------
enum : int { SL_LIMITS = 1 };
__device__ void slider_r1r2u(DevWorld &w, DevJoint &j) {  // calculateR1R2U :546-562
    j.r1 = qrot(w.quat[j.h.a], j.lp1);
    j.r2 = qrot(w.quat[j.h.b], j.lp2);
    j.u = xyz(w.com[j.h.b]) - xyz(w.com[j.h.a]) + j.r2 - j.r1;
}
__device__ void slider_axis_pos(DevWorld &w, DevJoint &j) {  // calculateSlidingAxisAndPosition :564-577
    if ((j.slider_flags & SL_LIMITS) || j.motor_state != 0 || j.max_friction_force > 0.f) {
        j.ws = qrot(w.quat[j.h.a], j.ls1);
        j.d = dot3(j.u, j.ws);
    }
}
__device__ void slider_pos_calc(DevWorld &w, DevJoint &j, const JBody &A, const JBody &B) {  // :579-609
    const float4 qa = w.quat[j.h.a];
    j.n1 = qrot(qa, j.ln1);
    j.n2 = qrot(qa, j.ln2);
    dual_calc(j.dual, A, j.r1 + j.u, B, j.r2, j.n1, j.n2);
}
__device__ void slider_limits_calc(DevJoint &j, const JBody &A, const JBody &B, float dt) {  // :611-696
    if (!(j.slider_flags & SL_LIMITS)) {
        axis_deactivate(j.ax);
        return;
    }
    const bool below = j.d <= j.limits_min, above = j.d >= j.limits_max;
    if (below || above) {
        const float err = below ? j.d - j.limits_min : j.d - j.limits_max;
        if (j.limits_freq > 0.f)
            axis_calc_settings(j.ax, dt, A, B, j.r1 + j.u, j.r2, j.ws, 0.f, err, j.limits_spring_mode, j.limits_freq,
                               j.limits_damping);
        else
            axis_calc(j.ax, A, B, j.r1 + j.u, j.r2, j.ws, 0.f);
    } else {
        axis_deactivate(j.ax);
    }
}
__device__ void slider_motor_calc(DevJoint &j, const JBody &A, const JBody &B, float dt) {  // :698-785
    const float3 r1u = j.r1 + j.u;
    if (j.motor_state == 0) {
        if (j.max_friction_force > 0.f)
            axis_calc(j.motor, A, B, r1u, j.r2, j.ws, 0.f);
        else
            axis_deactivate(j.motor);
    } else if (j.motor_state == 1) {
        axis_calc(j.motor, A, B, r1u, j.r2, j.ws, -j.target_velocity);
    } else if (j.motor_freq > 0.f) {
        axis_calc_settings(j.motor, dt, A, B, r1u, j.r2, j.ws, 0.f, j.d - j.target_position, j.motor_spring_mode,
                           j.motor_freq, j.motor_damping);
    } else {
        axis_deactivate(j.motor);
    }
}
__device__ void slider_setup(DevWorld &w, DevJoint &j, float dt) {  // setupVelocity :787-827
    JBody A = jbody(w, j.h.a), B = jbody(w, j.h.b);
    slider_r1r2u(w, j);
    slider_pos_calc(w, j, A, B);
    euler_calc(j.rot, A, B);
    slider_axis_pos(w, j);
    slider_limits_calc(j, A, B, dt);
    slider_motor_calc(j, A, B, dt);
}
__device__ void slider_warm(DevWorld &w, DevJoint &j, const JBody &A, const JBody &B, float ratio) {  // :829-877
    if (j.motor.eff != 0.f) axis_warm(w, j.motor, A, B, j.ws, ratio);
    dual_warm(w, j.dual, A, B, j.n1, j.n2, ratio);
    euler_warm(w, j.rot, A, B, ratio);
    if (j.ax.eff != 0.f) axis_warm(w, j.ax, A, B, j.ws, ratio);
}
__device__ bool slider_solve_velocity(DevWorld &w, DevJoint &j, const JBody &A, const JBody &B, float dt) {  // :879-958
    const float INF = __int_as_float(0x7f800000);
    bool motor = false, limit = false;
    if (j.motor.eff != 0.f) {
        if (j.motor_state == 0) {
            const float ml = j.max_friction_force * dt;
            motor = axis_solve_velocity(w, j.motor, A, B, j.ws, -ml, ml);
        } else {
            motor = axis_solve_velocity(w, j.motor, A, B, j.ws, dt * j.min_force, dt * j.max_force);
        }
    }
    bool pos = dual_solve_velocity(w, j.dual, A, B, j.n1, j.n2);
    bool rot = euler_solve_velocity(w, j.rot, A, B);
    if (j.ax.eff != 0.f) {
        float mn, mx;
        if (j.limits_min == j.limits_max) {
            mn = -INF;
            mx = INF;
        } else if (j.d <= j.limits_min) {
            mn = 0.f;
            mx = INF;
        } else {
            mn = -INF;
            mx = 0.f;
        }
        limit = axis_solve_velocity(w, j.ax, A, B, j.ws, mn, mx);
    }
    return motor || pos || rot || limit;
}
__device__ bool slider_solve_position(DevWorld &w, DevJoint &j, float dt) {  // :960-1038
    const float beta = c_settings.baumgarte;
    JBody A = jbody(w, j.h.a), B = jbody(w, j.h.b);
    slider_r1r2u(w, j);
    slider_pos_calc(w, j, A, B);
    bool pos = dual_solve_position(w, j.dual, A, B, j.u, j.n1, j.n2, beta);
    A = jbody(w, j.h.a);
    B = jbody(w, j.h.b);
    euler_calc(j.rot, A, B);
    bool rot = euler_solve_position(w, j.rot, A, B, j.inv_initial, beta);
    bool limit = false;
    if ((j.slider_flags & SL_LIMITS) && !(j.limits_freq > 0.f)) {
        A = jbody(w, j.h.a);
        B = jbody(w, j.h.b);
        slider_r1r2u(w, j);
        slider_axis_pos(w, j);
        slider_limits_calc(j, A, B, dt);
        if (j.ax.eff != 0.f) {
            const float err = j.d <= j.limits_min ? j.d - j.limits_min : j.d - j.limits_max;
            limit = axis_solve_position(w, j.ax, A, B, j.ws, err, beta);
        }
    }
    return pos || rot || limit;
}

// ---- the joints of one record (point, distance, fixed, cone, slider) -----------------
__device__ void other_setup(DevWorld &w, DevJoint &j, float dt) {
    switch (j.type) {
    case JT_POINT: pointj_setup(w, j); break;
    case JT_DISTANCE: {
        JBody A = jbody(w, j.h.a), B = jbody(w, j.h.b);
        distance_calc(w, j, A, B, dt);
        break;
    }
    case JT_FIXED: fixed_setup(w, j); break;
    case JT_CONE: cone_setup(w, j); break;
    case JT_SLIDER: slider_setup(w, j, dt); break;
    }
}
__device__ void other_warm(DevWorld &w, DevJoint &j, float ratio) {
    JBody A = jbody(w, j.h.a, false), B = jbody(w, j.h.b, false);
    switch (j.type) {
    case JT_POINT: point_warm(w, j.pt, A, B, ratio); break;
    case JT_DISTANCE: axis_warm(w, j.ax, A, B, j.wn, ratio); break;
    case JT_FIXED:
        euler_warm(w, j.rot, A, B, ratio);
        point_warm(w, j.pt, A, B, ratio);
        break;
    case JT_CONE:
        point_warm(w, j.pt, A, B, ratio);
        if (j.ang.eff != 0.f) angle_warm(w, j.ang, A, B, ratio);
        break;
    case JT_SLIDER: slider_warm(w, j, A, B, ratio); break;
    }
}
__device__ bool other_solve_velocity(DevWorld &w, DevJoint &j, float dt) {
    JBody A = jbody(w, j.h.a, false), B = jbody(w, j.h.b, false);
    switch (j.type) {
    case JT_POINT: return point_solve_velocity(w, j.pt, A, B);
    case JT_DISTANCE:
        return j.ax.eff != 0.f && axis_solve_velocity(w, j.ax, A, B, j.wn, j.min_lambda, j.max_lambda);
    case JT_FIXED: {
        bool rot = euler_solve_velocity(w, j.rot, A, B);
        bool pos = point_solve_velocity(w, j.pt, A, B);
        return rot || pos;
    }
    case JT_CONE: {
        const float INF = __int_as_float(0x7f800000);
        bool pos = point_solve_velocity(w, j.pt, A, B);
        bool rot = j.ang.eff != 0.f && angle_solve_velocity(w, j.ang, A, B, j.w_rot_axis, 0.f, INF);
        return pos || rot;
    }
    case JT_SLIDER: return slider_solve_velocity(w, j, A, B, dt);
    }
    return false;
}
__device__ bool other_solve_position(DevWorld &w, DevJoint &j, float dt) {
    switch (j.type) {
    case JT_POINT: return pointj_solve_position(w, j);
    case JT_DISTANCE: return distance_solve_position(w, j, dt);
    case JT_FIXED: return fixed_solve_position(w, j);
    case JT_CONE: return cone_solve_position(w, j);
    case JT_SLIDER: return slider_solve_position(w, j, dt);
    }
    return false;
}

// ---- six-DOF joint (six-dof-constraint.ts) -------------------------------------------
__device__ __forceinline__ bool sd_fixed(const DevSixDof &j, int a) { return (j.fixed_axis >> a) & 1; }
__device__ __forceinline__ bool sd_free(const DevSixDof &j, int a) { return (j.free_axis >> a) & 1; }
__device__ __forceinline__ bool sd_trans_constrained(const DevSixDof &j) { return (j.free_axis & 7) != 7; }
__device__ __forceinline__ bool sd_trans_fully(const DevSixDof &j) {
    return (j.fixed_axis & 7) == 7 && !(j.flags & SD_SPRING_LIMITS);
}
__device__ __forceinline__ bool sd_rot_constrained(const DevSixDof &j) { return (j.free_axis & 56) != 56; }
__device__ __forceinline__ bool sd_rot_fully(const DevSixDof &j) { return (j.fixed_axis & 56) == 56; }
__device__ __forceinline__ bool sd_friction(const DevSixDof &j, int a) {
    return !sd_fixed(j, a) && j.max_friction[a] > 0.f;
}
// getTwistAroundAxis :37-49
__device__ float4 twist_around(float4 q, float3 axis) {
    const float d = q.x * axis.x + q.y * axis.y + q.z * axis.z;
    const float l = d * d + q.w * q.w;
    if (!(l > 1e-10f)) return make_float4(0.f, 0.f, 0.f, 1.f);
    const float il = 1.f / sqrtf(l);
    return make_float4(d * axis.x * il, d * axis.y * il, d * axis.z * il, q.w * il);
}
// getPositionConstraintProperties :535-566
__device__ void sd_position_props(const DevWorld &w, const DevSixDof &j, float3 &r1u, float3 &r2, float3 &u) {
    const float3 ca = xyz(w.com[j.h.a]), cb = xyz(w.com[j.h.b]);
    const float3 p1 = qrot(w.quat[j.h.a], j.lp1) + ca, p2 = qrot(w.quat[j.h.b], j.lp2) + cb;
    r1u = p2 - ca;
    r2 = p2 - cb;
    u = p2 - p1;
}
__device__ __forceinline__ float f3_at(float3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
// setupVelocity :568-881
__device__ void sixdof_setup(DevWorld &w, DevSixDof &j, float dt) {
    JBody A = jbody(w, j.h.a), B = jbody(w, j.h.b);
    const float4 qa = w.quat[j.h.a], qb = w.quat[j.h.b];
    const float4 c1w = qmul(qa, j.c2b1);
    const float3 E[3] = {f3(1.f, 0.f, 0.f), f3(0.f, 1.f, 0.f), f3(0.f, 0.f, 1.f)};
    for (int i = 0; i < 3; i++) j.t_axis[i] = qrot(c1w, E[i]);
    if (sd_trans_fully(j)) {
        point_calc(j.pt, A, B, qa, qb, j.lp1, j.lp2);
    } else if (sd_trans_constrained(j) || (j.flags & SD_TRANS_MOTOR)) {
        float3 r1u, r2, u;
        sd_position_props(w, j, r1u, r2, u);
        for (int i = 0; i < 3; i++) {
            const float3 ta = j.t_axis[i];
            const float d = dot3(ta, u);
            j.disp[i] = d;
            bool on = false;
            float C = 0.f;
            if (sd_fixed(j, i)) {
                C = d - j.limit_min[i];
                on = true;
            } else if (!sd_free(j, i)) {
                if (d <= j.limit_min[i]) {
                    C = d - j.limit_min[i];
                    on = true;
                } else if (d >= j.limit_max[i]) {
                    C = d - j.limit_max[i];
                    on = true;
                }
            }
            if (on) {
                if (j.limits_freq[i] > 0.f)
                    axis_calc_settings(j.trans[i], dt, A, B, r1u, r2, ta, 0.f, C, j.limits_spring_mode[i],
                                       j.limits_freq[i], j.limits_damping[i]);
                else
                    axis_calc(j.trans[i], A, B, r1u, r2, ta, 0.f);
            } else {
                axis_deactivate(j.trans[i]);
            }
            if (j.motor_state[i] == 0) {
                if (sd_friction(j, i))
                    axis_calc(j.motor_t[i], A, B, r1u, r2, ta, 0.f);
                else
                    axis_deactivate(j.motor_t[i]);
            } else if (j.motor_state[i] == 1) {
                axis_calc(j.motor_t[i], A, B, r1u, r2, ta, -f3_at(j.target_v, i));
            } else if (j.motor_freq[i] > 0.f) {
                axis_calc_settings(j.motor_t[i], dt, A, B, r1u, r2, ta, 0.f, dot3(ta, u) - f3_at(j.target_p, i),
                                   j.motor_spring_mode[i], j.motor_freq[i], j.motor_damping[i]);
            } else {
                axis_deactivate(j.motor_t[i]);
            }
        }
    }
    const float4 c2w = qmul(qb, j.c2b2);
    const float4 q = qmul(qconj4(c1w), c2w);
    if (sd_rot_fully(j)) {
        euler_calc(j.rot, A, B);
    } else if (sd_rot_constrained(j) || (j.flags & SD_ROT_MOTOR)) {
        if (sd_rot_constrained(j)) {
            st_calc(j, A, B, q, c1w);
        } else {
            angle_deactivate(j.sy);
            angle_deactivate(j.sz);
            angle_deactivate(j.tw);
        }
        if (j.flags & SD_ROT_MOTOR) {
            for (int i = 0; i < 3; i++) j.r_axis[i] = qrot(c2w, E[i]);
            float4 t = j.target_q;
            if (q.x * t.x + q.y * t.y + q.z * t.z + q.w * t.w < 0.f) t = qscale4(t, -1.f);
            const float4 diff = qmul(qconj4(q), t);
            float4 pd;
            switch (j.rot_pos_motor) {
                case 1: pd = twist_around(diff, E[0]); break;
                case 2: pd = twist_around(diff, E[1]); break;
                case 4: pd = twist_around(diff, E[2]); break;
                case 3: pd = qmul(diff, qconj4(twist_around(diff, E[2]))); break;
                case 5: pd = qmul(diff, qconj4(twist_around(diff, E[1]))); break;
                case 6: pd = qmul(diff, qconj4(twist_around(diff, E[0]))); break;
                default: pd = diff; break;
            }
            const float err[3] = {-2.f * pd.x, -2.f * pd.y, -2.f * pd.z};
            for (int i = 0; i < 3; i++) {
                const int a = 3 + i;
                if (j.motor_state[a] == 0) {
                    if (sd_friction(j, a))
                        angle_calc(j.motor_r[i], A, B, j.r_axis[i], 0.f);
                    else
                        angle_deactivate(j.motor_r[i]);
                } else if (j.motor_state[a] == 1) {
                    angle_calc(j.motor_r[i], A, B, j.r_axis[i], -f3_at(j.target_w, i));
                } else if (j.motor_freq[a] > 0.f) {
                    angle_calc_settings(j.motor_r[i], dt, A, B, j.r_axis[i], 0.f, err[i], j.motor_spring_mode[a],
                                        j.motor_freq[a], j.motor_damping[a]);
                } else {
                    angle_deactivate(j.motor_r[i]);
                }
            }
        }
    }
}
// warmStartVelocity :883-942
__device__ void sixdof_warm(DevWorld &w, DevSixDof &j, float ratio) {
    JBody A = jbody(w, j.h.a, false), B = jbody(w, j.h.b, false);
    if (j.flags & SD_TRANS_MOTOR)
        for (int i = 0; i < 3; i++)
            if (j.motor_t[i].eff != 0.f) axis_warm(w, j.motor_t[i], A, B, j.t_axis[i], ratio);
    if (j.flags & SD_ROT_MOTOR)
        for (int i = 0; i < 3; i++)
            if (j.motor_r[i].eff != 0.f) angle_warm(w, j.motor_r[i], A, B, ratio);
    if (sd_rot_fully(j))
        euler_warm(w, j.rot, A, B, ratio);
    else if (sd_rot_constrained(j))
        st_warm(w, j, A, B, ratio);
    if (sd_trans_fully(j)) {
        point_warm(w, j.pt, A, B, ratio);
    } else if (sd_trans_constrained(j)) {
        for (int i = 0; i < 3; i++)
            if (j.trans[i].eff != 0.f) axis_warm(w, j.trans[i], A, B, j.t_axis[i], ratio);
    }
}
// solveVelocity :966-1082 (returns false, as the reference does)
__device__ bool sixdof_solve_velocity(DevWorld &w, DevSixDof &j, float dt) {
    JBody A = jbody(w, j.h.a, false), B = jbody(w, j.h.b, false);
    const float INF = __int_as_float(0x7f800000);
    if (j.flags & SD_TRANS_MOTOR)
        for (int i = 0; i < 3; i++) {
            if (j.motor_t[i].eff == 0.f) continue;
            if (j.motor_state[i] == 0) {
                const float ml = j.max_friction[i] * dt;
                axis_solve_velocity(w, j.motor_t[i], A, B, j.t_axis[i], -ml, ml);
            } else {
                axis_solve_velocity(w, j.motor_t[i], A, B, j.t_axis[i], dt * j.motor_min_force[i],
                                    dt * j.motor_max_force[i]);
            }
        }
    if (j.flags & SD_ROT_MOTOR)
        for (int i = 0; i < 3; i++) {
            const int a = 3 + i;
            if (j.motor_r[i].eff == 0.f) continue;
            if (j.motor_state[a] == 0) {
                const float ml = j.max_friction[a] * dt;
                angle_solve_velocity(w, j.motor_r[i], A, B, j.r_axis[i], -ml, ml);
            } else {
                angle_solve_velocity(w, j.motor_r[i], A, B, j.r_axis[i], dt * j.motor_min_force[a],
                                     dt * j.motor_max_force[a]);
            }
        }
    if (sd_rot_fully(j))
        euler_solve_velocity(w, j.rot, A, B);
    else if (sd_rot_constrained(j))
        st_solve_velocity(w, j, A, B);
    if (sd_trans_fully(j)) {
        point_solve_velocity(w, j.pt, A, B);
    } else if (sd_trans_constrained(j)) {
        for (int i = 0; i < 3; i++) {
            if (j.trans[i].eff == 0.f) continue;
            float mn = -INF, mx = INF;
            if (!sd_fixed(j, i)) {
                if (j.disp[i] <= j.limit_min[i])
                    mn = 0.f;
                else if (j.disp[i] >= j.limit_max[i])
                    mx = 0.f;
            }
            axis_solve_velocity(w, j.trans[i], A, B, j.t_axis[i], mn, mx);
        }
    }
    return false;
}
// quat.fromEuler for an 'xyz' euler (mathcat): q = qx qy qz
__device__ float4 quat_from_euler_xyz(float x, float y, float z) {
    const float c1 = cosf(0.5f * x), s1 = sinf(0.5f * x), c2 = cosf(0.5f * y), s2 = sinf(0.5f * y),
                c3 = cosf(0.5f * z), s3 = sinf(0.5f * z);
    return make_float4(s1 * c2 * c3 + c1 * s2 * s3, c1 * s2 * c3 - s1 * c2 * s3, c1 * c2 * s3 + s1 * s2 * c3,
                       c1 * c2 * c3 - s1 * s2 * s3);
}
// solvePosition :1084-1236
__device__ bool sixdof_solve_position(DevWorld &w, DevSixDof &j) {
    const float beta = c_settings.baumgarte;
    bool imp = false;
    JBody A = jbody(w, j.h.a), B = jbody(w, j.h.b);
    if (sd_rot_fully(j)) {
        const float4 off = qmul(j.c2b1, quat_from_euler_xyz(j.limit_min[3], j.limit_min[4], j.limit_min[5]));
        const float4 inv_initial = qmul(j.c2b2, qconj4(off));
        euler_calc(j.rot, A, B);
        imp = euler_solve_position(w, j.rot, A, B, inv_initial, beta) || imp;
    } else if (sd_rot_constrained(j)) {
        const float4 c1w = qmul(w.quat[j.h.a], j.c2b1), c2w = qmul(w.quat[j.h.b], j.c2b2);
        imp = st_solve_position(w, j, A, B, qmul(qconj4(c1w), c2w), beta) || imp;
    }
    A = jbody(w, j.h.a);
    B = jbody(w, j.h.b);
    if (sd_trans_fully(j)) {
        const float3 lp1 = j.lp1 + qrot(j.c2b1, f3(j.limit_min[0], j.limit_min[1], j.limit_min[2]));
        point_calc(j.pt, A, B, w.quat[j.h.a], w.quat[j.h.b], lp1, j.lp2);
        imp = point_solve_position(w, j.pt, A, B, beta) || imp;
    } else if (sd_trans_constrained(j)) {
        const float3 E[3] = {f3(1.f, 0.f, 0.f), f3(0.f, 1.f, 0.f), f3(0.f, 0.f, 1.f)};
        for (int i = 0; i < 3; i++) {
            if (j.limits_freq[i] > 0.f) continue;
            float3 r1u, r2, u;
            sd_position_props(w, j, r1u, r2, u);
            const float3 ta = qrot(qmul(w.quat[j.h.a], j.c2b1), E[i]);
            float err = 0.f;
            if (sd_fixed(j, i)) {
                err = dot3(u, ta) - j.limit_min[i];
            } else if (!sd_free(j, i)) {
                const float d = dot3(u, ta);
                if (d <= j.limit_min[i])
                    err = d - j.limit_min[i];
                else if (d >= j.limit_max[i])
                    err = d - j.limit_max[i];
            }
            if (err != 0.f) {
                A = jbody(w, j.h.a);
                B = jbody(w, j.h.b);
                axis_calc(j.trans[i], A, B, r1u, r2, ta, 0.f);
                imp = axis_solve_position(w, j.trans[i], A, B, ta, err, beta) || imp;
            }
        }
    }
    return imp;
}

// ---- dispatch on the joint id (the id helpers are in cc_internal.cuh) ------------------
__device__ void joint_setup(DevWorld &w, int id, float dt) {
    const int t = joint_type_of(id), i = joint_index_of(id);
    if (t == JT_SIX_DOF)
        sixdof_setup(w, w.sixdofs[i], dt);
    else if (t == JT_SWING)
        swing_setup(w, w.swings[i], dt);
    else if (t == JT_HINGE)
        hinge_setup(w, w.hinges[i], dt);
    else
        other_setup(w, other_joint(w, id), dt);
}
__device__ void joint_warm(DevWorld &w, int id, float ratio) {
    const int t = joint_type_of(id), i = joint_index_of(id);
    if (t == JT_SIX_DOF)
        sixdof_warm(w, w.sixdofs[i], ratio);
    else if (t == JT_SWING)
        swing_warm(w, w.swings[i], ratio);
    else if (t == JT_HINGE)
        hinge_warm(w, w.hinges[i], ratio);
    else
        other_warm(w, other_joint(w, id), ratio);
}
__device__ bool joint_solve_velocity(DevWorld &w, int id, float dt) {
    const int t = joint_type_of(id), i = joint_index_of(id);
    if (t == JT_SIX_DOF) return sixdof_solve_velocity(w, w.sixdofs[i], dt);
    if (t == JT_SWING) return swing_solve_velocity(w, w.swings[i], dt);
    if (t == JT_HINGE) return hinge_solve_velocity(w, w.hinges[i], dt);
    return other_solve_velocity(w, other_joint(w, id), dt);
}
__device__ bool joint_solve_position(DevWorld &w, int id, float dt) {
    const int t = joint_type_of(id), i = joint_index_of(id);
    if (t == JT_SIX_DOF) return sixdof_solve_position(w, w.sixdofs[i]);
    if (t == JT_SWING) return swing_solve_position(w, w.swings[i]);
    if (t == JT_HINGE) return hinge_solve_position(w, w.hinges[i], dt);
    return other_solve_position(w, other_joint(w, id), dt);
}
