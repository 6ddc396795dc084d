// Hinge joints on the device: setup, warm start, velocity and position solve of
// src/constraints/hinge-constraint.ts and the constraint parts it is built from
// (point-constraint-part.ts, hinge-rotation-constraint-part.ts, angle-constraint-part.ts,
// spring-part.ts).  FP32 like the contact solver; the 3x3 and 2x2 effective-mass inversions
// run in FP64.  Body state is read and written in global memory; a joint is solved by one
// thread (the per-thread island solve, or thread 0 of the per-CTA solve).
// Included by cc_solver.cu inside namespace cc (it uses that file's c_settings and rotation_step).
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

// ---- point part --------------------------------------------------------------------
__device__ void point_calc(DevHinge &j, const JBody &A, const JBody &B, float4 qa, float4 qb) {
    j.r1 = qrot(qa, j.lp1);
    j.r2 = qrot(qb, j.lp2);
    float iem[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    float sm = 0.f;
    float I[9], X[9], T[9], T2[9];
    if (A.motion == DYNAMIC) {
        sm += A.im;
        jm_from_sym(I, A.I);
        jm_cross(X, j.r1);
        jm_mm(j.invI1_r1X, I, X);
        jm_mm(T, X, I);
        jm_mm_bt(T2, T, X);
        for (int k = 0; k < 9; k++) iem[k] += T2[k];
    } else {
        for (int k = 0; k < 9; k++) j.invI1_r1X[k] = 0.f;
    }
    if (B.motion == DYNAMIC) {
        sm += B.im;
        jm_from_sym(I, B.I);
        jm_cross(X, j.r2);
        jm_mm(j.invI2_r2X, I, X);
        jm_mm(T, X, I);
        jm_mm_bt(T2, T, X);
        for (int k = 0; k < 9; k++) iem[k] += T2[k];
    } else {
        for (int k = 0; k < 9; k++) j.invI2_r2X[k] = 0.f;
    }
    iem[0] += sm;
    iem[4] += sm;
    iem[8] += sm;
    if (jm_invert(j.p_eff, iem)) {
        j.p_active = 1;
    } else {
        for (int k = 0; k < 9; k++) j.p_eff[k] = 0.f;
        j.p_lambda = f3(0.f, 0.f, 0.f);
        j.p_active = 0;
    }
}
__device__ bool point_apply(DevWorld &w, const DevHinge &j, const JBody &A, const JBody &B, float3 l) {
    if (lensq3(l) == 0.f) return false;
    if (A.motion == DYNAMIC) {
        add_lin(w, A.i, l * (-A.im));
        add_ang(w, A.i, -jm_mv(j.invI1_r1X, l));
    }
    if (B.motion == DYNAMIC) {
        add_lin(w, B.i, l * B.im);
        add_ang(w, B.i, jm_mv(j.invI2_r2X, l));
    }
    return true;
}
__device__ bool point_solve_velocity(DevWorld &w, DevHinge &j, const JBody &A, const JBody &B) {
    if (!j.p_active) return false;
    float3 jv = xyz(w.linvel[A.i]) - cross3(j.r1, xyz(w.angvel[A.i])) - xyz(w.linvel[B.i]) +
                cross3(j.r2, xyz(w.angvel[B.i]));
    float3 l = jm_mv(j.p_eff, jv);
    j.p_lambda = j.p_lambda + l;
    return point_apply(w, j, A, B, l);
}

// ---- hinge rotation part -------------------------------------------------------------
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

// ---- angle parts (limit: l_*, motor: m_*) -----------------------------------------------
struct AngleRef {
    float3 &i1, &i2;
    float &eff, &soft, &bias, &lambda;
};
__device__ __forceinline__ AngleRef limit_part(DevHinge &j) {
    return AngleRef{j.l_i1, j.l_i2, j.l_eff, j.l_soft, j.l_bias, j.l_lambda};
}
__device__ __forceinline__ AngleRef motor_part(DevHinge &j) {
    return AngleRef{j.m_i1, j.m_i2, j.m_eff, j.m_soft, j.m_bias, j.m_lambda};
}
__device__ __forceinline__ void angle_deactivate(AngleRef p) {
    p.eff = 0.f;
    p.lambda = 0.f;
}
__device__ float angle_iem(AngleRef p, const JBody &A, const JBody &B, float3 axis) {
    p.i1 = A.motion == DYNAMIC ? symmul(A.I, axis) : f3(0.f, 0.f, 0.f);
    p.i2 = B.motion == DYNAMIC ? symmul(B.I, axis) : f3(0.f, 0.f, 0.f);
    return dot3(axis, p.i1 + p.i2);
}
__device__ void angle_calc(AngleRef p, const JBody &A, const JBody &B, float3 axis, float bias) {
    float iem = angle_iem(p, A, B, axis);
    if (iem == 0.f) {
        angle_deactivate(p);
    } else {
        p.eff = 1.f / iem;
        p.soft = 0.f;
        p.bias = bias;
    }
}
__device__ void angle_calc_settings(AngleRef p, float dt, const JBody &A, const JBody &B, float3 axis, float bias,
                                    float C, int mode, float fs, float damping) {
    float iem = angle_iem(p, A, B, axis);
    if (iem == 0.f)
        angle_deactivate(p);
    else
        p.eff = spring_settings(p.soft, p.bias, dt, iem, bias, C, mode, fs, damping);
}
__device__ bool angle_apply(DevWorld &w, AngleRef p, const JBody &A, const JBody &B, float l) {
    if (l == 0.f) return false;
    if (A.motion == DYNAMIC) add_ang(w, A.i, -(p.i1 * l));
    if (B.motion == DYNAMIC) add_ang(w, B.i, p.i2 * l);
    return true;
}
__device__ bool angle_solve_velocity(DevWorld &w, AngleRef p, const JBody &A, const JBody &B, float3 axis, float mn,
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

// ---- hinge ---------------------------------------------------------------------------
__device__ __forceinline__ float center_angle(float a) {
    const float PI = 3.14159265358979f;
    while (a > PI) a -= 2.f * PI;
    while (a < -PI) a += 2.f * PI;
    return a;
}
// calculateA1AndTheta
__device__ void hinge_theta(DevHinge &j, float4 qa, float4 qb) {
    if (!(j.flags & JF_LIMITS) && j.motor_state == 0 && !(j.max_friction_torque > 0.f)) return;
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
    if ((j.flags & JF_LIMITS) && (j.theta <= j.limits_min || j.theta >= j.limits_max))
        angle_calc_settings(limit_part(j), dt, A, B, j.wh1, 0.f, hinge_to_limit(j), j.limits_spring_mode,
                            j.limits_freq, j.limits_damping);
    else
        angle_deactivate(limit_part(j));
}
__device__ void hinge_motor_props(DevHinge &j, const JBody &A, const JBody &B, float dt) {
    if (j.motor_state == 0) {
        if (j.max_friction_torque > 0.f)
            angle_calc(motor_part(j), A, B, j.wh1, 0.f);
        else
            angle_deactivate(motor_part(j));
    } else if (j.motor_state == 1) {
        angle_calc(motor_part(j), A, B, j.wh1, -j.target_angular_velocity);
    } else {
        if (j.motor_freq > 0.f)
            angle_calc_settings(motor_part(j), dt, A, B, j.wh1, 0.f, center_angle(j.theta - j.target_angle),
                                j.motor_spring_mode, j.motor_freq, j.motor_damping);
        else
            angle_deactivate(motor_part(j));
    }
}
__device__ __forceinline__ bool hinge_active(const DevWorld &w, const DevHinge &j) {
    return (j.flags & JF_ENABLED) && !(sleeping_of(w.flags[j.a]) && sleeping_of(w.flags[j.b]));
}
// setupVelocity
__device__ void hinge_setup(DevWorld &w, DevHinge &j, float dt) {
    JBody A = jbody(w, j.a), B = jbody(w, j.b);
    float4 qa = w.quat[j.a], qb = w.quat[j.b];
    point_calc(j, A, B, qa, qb);
    hrot_calc(j, A, B, qrot(qa, j.lh1), qrot(qb, j.lh2));
    hinge_theta(j, qa, qb);
    hinge_limit_props(j, A, B, dt);
    hinge_motor_props(j, A, B, dt);
}
// warmStartVelocity: motor, point, rotation, limits
__device__ void hinge_warm(DevWorld &w, DevHinge &j, float ratio) {
    JBody A = jbody(w, j.a, false), B = jbody(w, j.b, false);
    j.m_lambda *= ratio;
    angle_apply(w, motor_part(j), A, B, j.m_lambda);
    if (j.p_active) {
        j.p_lambda = j.p_lambda * ratio;
        point_apply(w, j, A, B, j.p_lambda);
    }
    j.r_lambda[0] *= ratio;
    j.r_lambda[1] *= ratio;
    hrot_apply(w, j, A, B, j.r_lambda[0], j.r_lambda[1]);
    j.l_lambda *= ratio;
    angle_apply(w, limit_part(j), A, B, j.l_lambda);
}
// solveVelocity
__device__ bool hinge_solve_velocity(DevWorld &w, DevHinge &j, float dt) {
    JBody A = jbody(w, j.a, false), B = jbody(w, j.b, false);
    const float INF = __int_as_float(0x7f800000);
    bool motor = false, limit = false;
    if (j.m_eff != 0.f) {
        if (j.motor_state == 0) {
            float ml = j.max_friction_torque * dt;
            motor = angle_solve_velocity(w, motor_part(j), A, B, j.wh1, -ml, ml);
        } else {
            motor = angle_solve_velocity(w, motor_part(j), A, B, j.wh1, dt * j.min_torque, dt * j.max_torque);
        }
    }
    bool pos = point_solve_velocity(w, j, A, B);
    bool rot = hrot_solve_velocity(w, j, A, B);
    if (j.l_eff != 0.f) {
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
        limit = angle_solve_velocity(w, limit_part(j), A, B, j.wh1, mn, mx);
    }
    return motor || pos || rot || limit;
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

// solvePosition
__device__ bool hinge_solve_position(DevWorld &w, DevHinge &j, float dt) {
    const float beta = c_settings.baumgarte;
    JBody A = jbody(w, j.a), B = jbody(w, j.b);
    point_calc(j, A, B, w.quat[j.a], w.quat[j.b]);
    bool pos = false;
    if (j.p_active) {
        float3 sep = xyz(w.com[j.b]) + j.r2 - xyz(w.com[j.a]) - j.r1;
        if (!(lensq3(sep) < 1e-12f)) {
            float3 l = jm_mv(j.p_eff, sep) * (-beta);
            if (A.motion == DYNAMIC) {
                add_position_step(w, A.i, l * (-A.im));
                add_rotation(w, A.i, -jm_mv(j.invI1_r1X, l));
            }
            if (B.motion == DYNAMIC) {
                add_position_step(w, B.i, l * B.im);
                add_rotation(w, B.i, jm_mv(j.invI2_r2X, l));
            }
            pos = true;
        }
    }
    A = jbody(w, j.a);
    B = jbody(w, j.b);
    float4 qa = w.quat[j.a], qb = w.quat[j.b];
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
    if ((j.flags & JF_LIMITS) && !(j.limits_freq > 0.f)) {
        A = jbody(w, j.a);
        B = jbody(w, j.b);
        hinge_theta(j, w.quat[j.a], w.quat[j.b]);
        hinge_limit_props(j, A, B, dt);
        float C = hinge_to_limit(j);
        if (j.l_eff != 0.f && C != 0.f && j.l_soft == 0.f) {
            float l = -j.l_eff * beta * C;
            if (A.motion == DYNAMIC) add_rotation(w, A.i, -(j.l_i1 * l));
            if (B.motion == DYNAMIC) add_rotation(w, B.i, j.l_i2 * l);
            limit = true;
        }
    }
    return pos || rot || limit;
}

__device__ __forceinline__ bool hinge_before(const DevHinge &x, const DevHinge &y) {
    if (x.priority != y.priority) return x.priority < y.priority;
    return x.index < y.index;
}

