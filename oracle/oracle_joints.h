// FP64 restatement of crashcat's hinge joint and the constraint parts it is built from
// (TEST INFRASTRUCTURE: the parity oracle).  Follows, function by function:
//   src/constraints/hinge-constraint.ts, src/constraints/constraint-part/point-constraint-part.ts,
//   hinge-rotation-constraint-part.ts, angle-constraint-part.ts, spring-part.ts.
// 3x3 matrices are stored by columns like the reference's column-major mat4 (element (r, c)
// at m[c][r]); mathcat's mat4.invert3x3 is restated as the adjugate over the determinant,
// singular when the determinant is exactly zero.
// Included by oracle.cpp inside namespace orc, after the body helpers it uses; the data
// types are in oracle_joint_types.h.
#pragma once

inline M3 m3_zero() {
    M3 r;
    for (int c = 0; c < 3; c++)
        for (int k = 0; k < 3; k++) r.m[c][k] = 0;
    return r;
}
inline M3 m3_from_m4(const M4 &a) {
    M3 r;
    for (int c = 0; c < 3; c++)
        for (int k = 0; k < 3; k++) r.m[c][k] = a.m[c * 4 + k];
    return r;
}
inline V3 m3_mul(const M3 &a, V3 v) {  // mat4.multiply3x3Vec
    return {a.m[0][0] * v.x + a.m[1][0] * v.y + a.m[2][0] * v.z, a.m[0][1] * v.x + a.m[1][1] * v.y + a.m[2][1] * v.z,
            a.m[0][2] * v.x + a.m[1][2] * v.y + a.m[2][2] * v.z};
}
inline M3 m3_mm(const M3 &a, const M3 &b) {  // mat4.multiply3x3: a * b
    M3 r;
    for (int c = 0; c < 3; c++)
        for (int k = 0; k < 3; k++) r.m[c][k] = a.m[0][k] * b.m[c][0] + a.m[1][k] * b.m[c][1] + a.m[2][k] * b.m[c][2];
    return r;
}
inline M3 m3_mm_rt(const M3 &a, const M3 &b) {  // mat4.multiply3x3RightTransposed: a * b^T
    M3 r;
    for (int c = 0; c < 3; c++)
        for (int k = 0; k < 3; k++) r.m[c][k] = a.m[0][k] * b.m[0][c] + a.m[1][k] * b.m[1][c] + a.m[2][k] * b.m[2][c];
    return r;
}
inline M3 m3_add(const M3 &a, const M3 &b) {
    M3 r;
    for (int c = 0; c < 3; c++)
        for (int k = 0; k < 3; k++) r.m[c][k] = a.m[c][k] + b.m[c][k];
    return r;
}
inline M3 m3_cross(V3 v) {  // mat4.crossProductMatrix: [v]x, so [v]x w = v x w
    M3 r = m3_zero();
    r.m[1][0] = -v.z;
    r.m[2][0] = v.y;
    r.m[0][1] = v.z;
    r.m[2][1] = -v.x;
    r.m[0][2] = -v.y;
    r.m[1][2] = v.x;
    return r;
}
inline bool m3_invert(M3 &out, const M3 &a) {  // mat4.invert3x3
    double a00 = a.m[0][0], a01 = a.m[0][1], a02 = a.m[0][2];
    double a10 = a.m[1][0], a11 = a.m[1][1], a12 = a.m[1][2];
    double a20 = a.m[2][0], a21 = a.m[2][1], a22 = a.m[2][2];
    double b01 = a22 * a11 - a12 * a21, b11 = -a22 * a10 + a12 * a20, b21 = a21 * a10 - a11 * a20;
    double det = a00 * b01 + a01 * b11 + a02 * b21;
    if (det == 0.0) return false;
    det = 1.0 / det;
    out.m[0][0] = b01 * det;
    out.m[0][1] = (-a22 * a01 + a02 * a21) * det;
    out.m[0][2] = (a12 * a01 - a02 * a11) * det;
    out.m[1][0] = b11 * det;
    out.m[1][1] = (a22 * a00 - a02 * a20) * det;
    out.m[1][2] = (-a12 * a00 + a02 * a10) * det;
    out.m[2][0] = b21 * det;
    out.m[2][1] = (-a21 * a00 + a01 * a20) * det;
    out.m[2][2] = (a11 * a00 - a01 * a10) * det;
    return true;
}

// spring-settings.ts / spring-part.ts
inline double spring_helper(SpringPart &p, double dt, double iem, double bias, double C, double k, double c) {
    p.softness = 1.0 / (dt * (c + dt * k));
    p.bias = bias + dt * k * p.softness * C;
    return 1.0 / (iem + p.softness);
}
inline double spring_with_settings(SpringPart &p, double dt, double iem, double bias, double C,
                                   const SpringSettings &s) {
    if (s.mode == FREQUENCY_AND_DAMPING) {
        double em = 1.0 / iem;
        if (s.frequencyOrStiffness > 0) {
            double omega = 2.0 * M_PI * s.frequencyOrStiffness;
            double k = em * omega * omega, c = 2.0 * em * s.damping * omega;
            return spring_helper(p, dt, iem, bias, C, k, c);
        }
        p.softness = 0;
        p.bias = bias;
        return em;
    }
    if (s.frequencyOrStiffness > 0) return spring_helper(p, dt, iem, bias, C, s.frequencyOrStiffness, s.damping);
    p.softness = 0;
    p.bias = bias;
    return 1.0 / iem;
}

// world inverse inertia of a body (zero unless dynamic) and its product with a vector
inline M3 world_inv_inertia(const Body &b) {
    if (b.motion != DYNAMIC) return m3_zero();
    return m3_from_m4(inv_inertia_for_rotation(b, mat4_from_quat(b.quat)));
}

// ---- PointConstraintPart ----------------------------------------------------------
inline void point_deactivate(PointPart &p) {
    p.effMass = m3_zero();
    p.totalLambda = {0, 0, 0};
    p.active = false;
}
inline void point_calc(PointPart &p, const Body &A, V3 r1Local, const Body &B, V3 r2Local) {
    M3 RA = m3_from_m4(mat4_from_quat(A.quat)), RB = m3_from_m4(mat4_from_quat(B.quat));
    p.r1 = m3_mul(RA, r1Local);
    p.r2 = m3_mul(RB, r2Local);
    M3 iem = m3_zero();
    double sm = 0;
    if (A.motion == DYNAMIC) {
        sm += A.invMass;
        M3 I = world_inv_inertia(A), X = m3_cross(p.r1);
        p.invI1_r1X = m3_mm(I, X);
        iem = m3_add(iem, m3_mm_rt(m3_mm(X, I), X));
    } else {
        p.invI1_r1X = m3_zero();
    }
    if (B.motion == DYNAMIC) {
        sm += B.invMass;
        M3 I = world_inv_inertia(B), X = m3_cross(p.r2);
        p.invI2_r2X = m3_mm(I, X);
        iem = m3_add(iem, m3_mm_rt(m3_mm(X, I), X));
    } else {
        p.invI2_r2X = m3_zero();
    }
    iem.m[0][0] += sm;
    iem.m[1][1] += sm;
    iem.m[2][2] += sm;
    if (m3_invert(p.effMass, iem)) {
        p.active = true;
    } else {
        point_deactivate(p);
    }
}
inline bool point_apply(PointPart &p, Body &A, Body &B, V3 l) {
    if (lensq(l) == 0) return false;
    if (A.motion == DYNAMIC) {
        A.linvel = scale_add(A.linvel, l, -A.invMass);
        A.angvel = sub(A.angvel, m3_mul(p.invI1_r1X, l));
    }
    if (B.motion == DYNAMIC) {
        B.linvel = scale_add(B.linvel, l, B.invMass);
        B.angvel = add(B.angvel, m3_mul(p.invI2_r2X, l));
    }
    return true;
}
inline void point_warm(PointPart &p, Body &A, Body &B, double ratio) {
    if (!p.active) return;
    p.totalLambda = scale(p.totalLambda, ratio);
    point_apply(p, A, B, p.totalLambda);
}
inline bool point_solve_velocity(PointPart &p, Body &A, Body &B) {
    if (!p.active) return false;
    V3 jv = A.linvel;
    jv = sub(jv, cross(p.r1, A.angvel));
    jv = sub(jv, B.linvel);
    jv = add(jv, cross(p.r2, B.angvel));
    V3 l = m3_mul(p.effMass, jv);
    p.totalLambda = add(p.totalLambda, l);
    return point_apply(p, A, B, l);
}

// ---- HingeRotationConstraintPart ----------------------------------------------------
inline V3 perpendicular(V3 v) {  // getPerpendicularVector hinge-rotation-constraint-part.ts
    if (std::fabs(v.x) > std::fabs(v.y)) {
        double l = std::sqrt(v.x * v.x + v.z * v.z);
        return {v.z / l, 0, -v.x / l};
    }
    double l = std::sqrt(v.y * v.y + v.z * v.z);
    return {0, v.z / l, -v.y / l};
}
inline void hrot_deactivate(HingeRotPart &p) {
    for (double &e : p.eff) e = 0;
    p.totalLambda[0] = p.totalLambda[1] = 0;
}
inline bool hrot_active(const HingeRotPart &p) { return p.eff[0] != 0 || p.eff[1] != 0 || p.eff[2] != 0 || p.eff[3] != 0; }
inline void hrot_calc(HingeRotPart &p, const Body &A, const Body &B, V3 axis1, V3 axis2) {
    p.a1 = axis1;
    V3 a2 = axis2;
    double d = dot(p.a1, a2);
    if (d <= 1.0e-3) {
        V3 perp = scale_add(a2, p.a1, -d);
        if (lensq(perp) < 1.0e-6) perp = perpendicular(p.a1);
        perp = normalize(perp);
        a2 = scale(p.a1, 0.01);
        a2 = scale_add(a2, perp, 0.99);
        a2 = normalize(a2);
    }
    p.b2 = perpendicular(a2);
    p.c2 = cross(a2, p.b2);
    p.invI1 = world_inv_inertia(A);
    p.invI2 = world_inv_inertia(B);
    p.b2xA1 = cross(p.b2, p.a1);
    p.c2xA1 = cross(p.c2, p.a1);
    M3 sum = m3_add(p.invI1, p.invI2);
    V3 t = m3_mul(sum, p.b2xA1);
    double k0 = dot(p.b2xA1, t), k2 = dot(p.c2xA1, t);
    t = m3_mul(sum, p.c2xA1);
    double k1 = dot(p.b2xA1, t), k3 = dot(p.c2xA1, t);
    double det = k0 * k3 - k1 * k2;
    if (std::fabs(det) < 1e-10) {
        hrot_deactivate(p);
        return;
    }
    double id = 1.0 / det;
    p.eff[0] = k3 * id;
    p.eff[1] = -k1 * id;
    p.eff[2] = -k2 * id;
    p.eff[3] = k0 * id;
}
inline bool hrot_apply(HingeRotPart &p, Body &A, Body &B, double l0, double l1) {
    if (l0 == 0 && l1 == 0) return false;
    V3 imp = scale(p.b2xA1, l0);
    imp = scale_add(imp, p.c2xA1, l1);
    if (A.motion == DYNAMIC) A.angvel = sub(A.angvel, m3_mul(p.invI1, imp));
    if (B.motion == DYNAMIC) B.angvel = add(B.angvel, m3_mul(p.invI2, imp));
    return true;
}
inline void hrot_warm(HingeRotPart &p, Body &A, Body &B, double ratio) {
    p.totalLambda[0] *= ratio;
    p.totalLambda[1] *= ratio;
    hrot_apply(p, A, B, p.totalLambda[0], p.totalLambda[1]);
}
inline bool hrot_solve_velocity(HingeRotPart &p, Body &A, Body &B) {
    if (!hrot_active(p)) return false;
    double j0 = 0, j1 = 0;
    if (A.motion != STATIC) {
        j0 += dot(p.b2xA1, A.angvel);
        j1 += dot(p.c2xA1, A.angvel);
    }
    if (B.motion != STATIC) {
        j0 -= dot(p.b2xA1, B.angvel);
        j1 -= dot(p.c2xA1, B.angvel);
    }
    double l0 = p.eff[0] * j0 + p.eff[1] * j1, l1 = p.eff[2] * j0 + p.eff[3] * j1;
    p.totalLambda[0] += l0;
    p.totalLambda[1] += l1;
    return hrot_apply(p, A, B, l0, l1);
}

// ---- AngleConstraintPart -----------------------------------------------------------
inline void angle_deactivate(AnglePart &p) {
    p.effMass = 0;
    p.totalLambda = 0;
}
inline bool angle_active(const AnglePart &p) { return p.effMass != 0; }
inline double angle_iem(AnglePart &p, const Body &A, const Body &B, V3 axis) {
    p.invI1_Axis = A.motion == DYNAMIC ? m3_mul(world_inv_inertia(A), axis) : V3{0, 0, 0};
    p.invI2_Axis = B.motion == DYNAMIC ? m3_mul(world_inv_inertia(B), axis) : V3{0, 0, 0};
    V3 s = add(p.invI1_Axis, p.invI2_Axis);
    return axis.x * s.x + axis.y * s.y + axis.z * s.z;
}
inline void angle_calc(AnglePart &p, const Body &A, const Body &B, V3 axis, double bias) {
    double iem = angle_iem(p, A, B, axis);
    if (iem == 0) {
        angle_deactivate(p);
    } else {
        p.effMass = 1.0 / iem;
        p.spring.softness = 0;
        p.spring.bias = bias;
    }
}
inline void angle_calc_settings(AnglePart &p, double dt, const Body &A, const Body &B, V3 axis, double bias, double C,
                                const SpringSettings &s) {
    double iem = angle_iem(p, A, B, axis);
    if (iem == 0)
        angle_deactivate(p);
    else
        p.effMass = spring_with_settings(p.spring, dt, iem, bias, C, s);
}
inline bool angle_apply(AnglePart &p, Body &A, Body &B, double l) {
    if (l == 0) return false;
    if (A.motion == DYNAMIC) A.angvel = sub(A.angvel, scale(p.invI1_Axis, l));
    if (B.motion == DYNAMIC) B.angvel = add(B.angvel, scale(p.invI2_Axis, l));
    return true;
}
inline void angle_warm(AnglePart &p, Body &A, Body &B, double ratio) {
    p.totalLambda *= ratio;
    angle_apply(p, A, B, p.totalLambda);
}
inline bool angle_solve_velocity(AnglePart &p, Body &A, Body &B, V3 axis, double mn, double mx) {
    if (!angle_active(p)) return false;
    double jv = 0;
    if (A.motion != STATIC) jv += dot(axis, A.angvel);
    if (B.motion != STATIC) jv -= dot(axis, B.angvel);
    double l = p.effMass * (jv - (p.spring.softness * p.totalLambda + p.spring.bias));
    double nl = std::max(mn, std::min(mx, p.totalLambda + l));
    double dl = nl - p.totalLambda;
    p.totalLambda = nl;
    return angle_apply(p, A, B, dl);
}

// ---- HingeConstraint ---------------------------------------------------------------

inline double center_angle(double a) {  // centerAngleAroundZero
    while (a > M_PI) a -= 2 * M_PI;
    while (a < -M_PI) a += 2 * M_PI;
    return a;
}
// calculateA1AndTheta hinge-constraint.ts
inline void hinge_theta(HingeJoint &j, const Body &A, const Body &B) {
    if (!j.hasLimits && j.motorState == MOTOR_OFF && j.maxFrictionTorque <= 0) return;
    V3 wh = rotate(A.quat, j.lh1);
    j.wh1 = wh;
    Q4 rel = qmul(qmul(B.quat, j.invInitial), qconj(A.quat));
    double axisDot = wh.x * rel.x + wh.y * rel.y + wh.z * rel.z;
    j.theta = rel.w == 0 ? M_PI : 2 * std::atan(axisDot / rel.w);
}
inline double hinge_smallest_to_limit(const HingeJoint &j) {
    double dmn = center_angle(j.theta - j.limitsMin), dmx = center_angle(j.theta - j.limitsMax);
    return std::fabs(dmn) < std::fabs(dmx) ? dmn : dmx;
}
inline bool hinge_min_closest(const HingeJoint &j) {
    double dmn = center_angle(j.theta - j.limitsMin), dmx = center_angle(j.theta - j.limitsMax);
    return std::fabs(dmn) < std::fabs(dmx);
}
inline void hinge_limit_props(HingeJoint &j, const Body &A, const Body &B, double dt) {
    if (j.hasLimits && (j.theta <= j.limitsMin || j.theta >= j.limitsMax))
        angle_calc_settings(j.limit, dt, A, B, j.wh1, 0, hinge_smallest_to_limit(j), j.limitsSpring);
    else
        angle_deactivate(j.limit);
}
inline void hinge_motor_props(HingeJoint &j, const Body &A, const Body &B, double dt) {
    switch (j.motorState) {
        case MOTOR_OFF:
            if (j.maxFrictionTorque > 0)
                angle_calc(j.motor, A, B, j.wh1, 0);
            else
                angle_deactivate(j.motor);
            break;
        case MOTOR_VELOCITY:
            angle_calc(j.motor, A, B, j.wh1, -j.targetAngularVelocity);
            break;
        case MOTOR_POSITION:
            if (j.motorSpring.frequencyOrStiffness > 0)
                angle_calc_settings(j.motor, dt, A, B, j.wh1, 0, center_angle(j.theta - j.targetAngle), j.motorSpring);
            else
                angle_deactivate(j.motor);
            break;
    }
}
// setupVelocity hinge-constraint.ts
inline void hinge_setup(HingeJoint &j, const Body &A, const Body &B, double dt) {
    V3 h1 = rotate(A.quat, j.lh1), h2 = rotate(B.quat, j.lh2);
    point_calc(j.point, A, j.lp1, B, j.lp2);
    hrot_calc(j.rot, A, B, h1, h2);
    hinge_theta(j, A, B);
    hinge_limit_props(j, A, B, dt);
    hinge_motor_props(j, A, B, dt);
}
inline void hinge_warm(HingeJoint &j, Body &A, Body &B, double ratio) {
    angle_warm(j.motor, A, B, ratio);
    point_warm(j.point, A, B, ratio);
    hrot_warm(j.rot, A, B, ratio);
    angle_warm(j.limit, A, B, ratio);
}
inline bool hinge_solve_velocity(HingeJoint &j, Body &A, Body &B, double dt) {
    bool motor = false, limit = false;
    const double INF = 1.0 / 0.0;
    if (angle_active(j.motor)) {
        if (j.motorState == MOTOR_OFF) {
            double ml = j.maxFrictionTorque * dt;
            motor = angle_solve_velocity(j.motor, A, B, j.wh1, -ml, ml);
        } else {
            motor = angle_solve_velocity(j.motor, A, B, j.wh1, dt * j.minTorqueLimit, dt * j.maxTorqueLimit);
        }
    }
    bool pos = point_solve_velocity(j.point, A, B);
    bool rot = hrot_solve_velocity(j.rot, A, B);
    if (angle_active(j.limit)) {
        double mn, mx;
        if (j.limitsMin == j.limitsMax) {
            mn = -INF;
            mx = INF;
        } else if (hinge_min_closest(j)) {
            mn = 0;
            mx = INF;
        } else {
            mn = -INF;
            mx = 0;
        }
        limit = angle_solve_velocity(j.limit, A, B, j.wh1, mn, mx);
    }
    return motor || pos || rot || limit;
}

// ---- position solves (solvePositionConstraint of each part, hinge solvePosition) ----
inline bool point_solve_position(PointPart &p, Body &A, Body &B, double baumgarte) {
    if (!p.active) return false;
    V3 sep = sub(sub(add(B.com, p.r2), A.com), p.r1);
    if (lensq(sep) < 1e-12) return false;
    V3 l = scale(m3_mul(p.effMass, sep), -baumgarte);
    if (A.motion == DYNAMIC) {
        A.com = sub(A.com, scale(l, A.invMass));
        apply_dof_pos(A);
        sub_rotation_step(A, m3_mul(p.invI1_r1X, l));
    }
    if (B.motion == DYNAMIC) {
        B.com = add(B.com, scale(l, B.invMass));
        apply_dof_pos(B);
        add_rotation_step(B, m3_mul(p.invI2_r2X, l));
    }
    return true;
}
inline bool hrot_solve_position(HingeRotPart &p, Body &A, Body &B, double baumgarte) {
    if (!hrot_active(p)) return false;
    double c0 = dot(p.a1, p.b2), c1 = dot(p.a1, p.c2);
    if (std::fabs(c0) < 1e-10 && std::fabs(c1) < 1e-10) return false;
    double l0 = -baumgarte * (p.eff[0] * c0 + p.eff[1] * c1), l1 = -baumgarte * (p.eff[2] * c0 + p.eff[3] * c1);
    V3 imp = scale_add(scale(p.b2xA1, l0), p.c2xA1, l1);
    if (A.motion == DYNAMIC) sub_rotation_step(A, m3_mul(p.invI1, imp));
    if (B.motion == DYNAMIC) add_rotation_step(B, m3_mul(p.invI2, imp));
    return true;
}
inline bool angle_solve_position(AnglePart &p, Body &A, Body &B, double C, double baumgarte) {
    if (C == 0 || !angle_active(p) || p.spring.softness != 0) return false;
    double l = -p.effMass * baumgarte * C;
    if (A.motion == DYNAMIC) sub_rotation_step(A, scale(p.invI1_Axis, l));
    if (B.motion == DYNAMIC) add_rotation_step(B, scale(p.invI2_Axis, l));
    return true;
}
inline bool hinge_solve_position(HingeJoint &j, Body &A, Body &B, double dt, double baumgarte) {
    point_calc(j.point, A, j.lp1, B, j.lp2);
    bool pos = point_solve_position(j.point, A, B, baumgarte);
    V3 h1 = rotate(A.quat, j.lh1), h2 = rotate(B.quat, j.lh2);
    hrot_calc(j.rot, A, B, h1, h2);
    bool rot = hrot_solve_position(j.rot, A, B, baumgarte);
    bool limit = false;
    if (j.hasLimits && j.limitsSpring.frequencyOrStiffness <= 0) {
        hinge_theta(j, A, B);
        hinge_limit_props(j, A, B, dt);
        if (angle_active(j.limit)) limit = angle_solve_position(j.limit, A, B, hinge_smallest_to_limit(j), baumgarte);
    }
    return pos || rot || limit;
}

// quat.fromMat3 (Shoemake's method, as gl-matrix) for getInvInitialOrientationXZ
inline Q4 quat_from_m3(const M3 &m) {
    const double *f = &m.m[0][0];  // column-major 3x3
    double tr = f[0] + f[4] + f[8];
    Q4 o;
    if (tr > 0.0) {
        double r = std::sqrt(tr + 1.0);
        o.w = 0.5 * r;
        r = 0.5 / r;
        o.x = (f[5] - f[7]) * r;
        o.y = (f[6] - f[2]) * r;
        o.z = (f[1] - f[3]) * r;
    } else {
        int i = 0;
        if (f[4] > f[0]) i = 1;
        if (f[8] > f[i * 3 + i]) i = 2;
        int j = (i + 1) % 3, k = (i + 2) % 3;
        double q[3];
        double r = std::sqrt(f[i * 3 + i] - f[j * 3 + j] - f[k * 3 + k] + 1.0);
        q[i] = 0.5 * r;
        r = 0.5 / r;
        o.w = (f[j * 3 + k] - f[k * 3 + j]) * r;
        q[j] = (f[j * 3 + i] + f[i * 3 + j]) * r;
        q[k] = (f[k * 3 + i] + f[i * 3 + k]) * r;
        o.x = q[0];
        o.y = q[1];
        o.z = q[2];
    }
    return o;
}
// getInvInitialOrientationXZ hinge-constraint.ts
inline Q4 inv_initial_orientation_xz(V3 n1, V3 h1, V3 n2, V3 h2) {
    const double eps = 1e-6;
    if (std::fabs(n1.x - n2.x) < eps && std::fabs(n1.y - n2.y) < eps && std::fabs(n1.z - n2.z) < eps &&
        std::fabs(h1.x - h2.x) < eps && std::fabs(h1.y - h2.y) < eps && std::fabs(h1.z - h2.z) < eps)
        return {0, 0, 0, 1};
    V3 y1 = cross(h1, n1), y2 = cross(h2, n2);
    M3 m1, m2;  // columns: normal, y, hinge (mat3.fromValues fills column by column)
    V3 c1[3] = {n1, y1, h1}, c2[3] = {n2, y2, h2};
    for (int c = 0; c < 3; c++) {
        m1.m[c][0] = c1[c].x;
        m1.m[c][1] = c1[c].y;
        m1.m[c][2] = c1[c].z;
        m2.m[c][0] = c2[c].x;
        m2.m[c][1] = c2[c].y;
        m2.m[c][2] = c2[c].z;
    }
    Q4 q1 = quat_from_m3(m1), q2 = quat_from_m3(m2);
    return qmul(q2, qconj(q1));
}
