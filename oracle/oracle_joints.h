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

// ---- SwingTwistConstraintPart (swing-twist-constraint-part.ts) ----------------------
// setLimits :140-236
inline void st_set_limits(SwingTwistPart &p, double twistMin, double twistMax, double swingYMin, double swingYMax,
                          double swingZMin, double swingZMax) {
    const double locked = 0.5 * M_PI / 180.0, freeA = 179.5 * M_PI / 180.0;
    p.swingYHalfMin = 0.5 * swingYMin;
    p.swingYHalfMax = 0.5 * swingYMax;
    p.swingZHalfMin = 0.5 * swingZMin;
    p.swingZHalfMax = 0.5 * swingZMax;
    p.rotationFlags = 0;
    auto axis = [&](double mn, double mx, int lockedFlag, int freeFlag, double &sMin, double &sMax, double &cMin,
                    double &cMax) {
        if (mn > -locked && mx < locked) {
            p.rotationFlags |= lockedFlag;
            sMin = sMax = 0;
            cMin = cMax = 1;
        } else if (mn < -freeA && mx > freeA) {
            p.rotationFlags |= freeFlag;
            sMin = -1;
            sMax = 1;
            cMin = cMax = 0;
        } else {
            sMin = std::sin(0.5 * mn);
            sMax = std::sin(0.5 * mx);
            cMin = std::cos(0.5 * mn);
            cMax = std::cos(0.5 * mx);
        }
    };
    axis(twistMin, twistMax, TWIST_X_LOCKED, TWIST_X_FREE, p.sinTwistHalfMin, p.sinTwistHalfMax, p.cosTwistHalfMin,
         p.cosTwistHalfMax);
    axis(swingYMin, swingYMax, SWING_Y_LOCKED, SWING_Y_FREE, p.sinSwingYHalfMin, p.sinSwingYHalfMax, p.cosSwingYHalfMin,
         p.cosSwingYHalfMax);
    axis(swingZMin, swingZMax, SWING_Z_LOCKED, SWING_Z_FREE, p.sinSwingZHalfMin, p.sinSwingZHalfMax, p.cosSwingZHalfMin,
         p.cosSwingZHalfMax);
}
// distanceToMinShorter :239-246
inline bool distance_to_min_shorter(double dMin, double dMax) {
    double a = std::fabs(dMin);
    if (a > 1) a = 2 - a;
    double b = std::fabs(dMax);
    if (b > 1) b = 2 - b;
    return a < b;
}
// getSwingTwist :252-269: q = swing * twist, swing.x = 0, twist.y = twist.z = 0
inline void get_swing_twist(Q4 q, Q4 &swing, Q4 &twist) {
    double s = std::sqrt(q.w * q.w + q.x * q.x);
    if (s != 0) {
        twist = {q.x / s, 0, 0, q.w / s};
        swing = {0, (q.w * q.y - q.x * q.z) / s, (q.w * q.z + q.x * q.y) / s, s};
    } else {
        twist = {0, 0, 0, 1};
        swing = q;
    }
}
inline Q4 qscale(Q4 q, double s) { return {q.x * s, q.y * s, q.z * s, q.w * s}; }
// getClosestPointOnEllipse :412-462 (Newton iteration on the Lagrange multiplier)
inline void closest_point_on_ellipse(double px, double py, double a, double b, double &ox, double &oy) {
    if (a <= 0) {
        ox = 0;
        oy = py >= 0 ? b : -b;
        return;
    }
    if (b <= 0) {
        ox = px >= 0 ? a : -a;
        oy = 0;
        return;
    }
    double aSq = a * a, bSq = b * b, t = 0;
    for (int i = 0; i < 100; i++) {
        double ta = t + aSq, tb = t + bSq;
        double ga = a * px / ta, gb = b * py / tb;
        double gt = ga * ga + gb * gb - 1;
        if (std::fabs(gt) < 1e-6) {
            ox = aSq * px / ta;
            oy = bSq * py / tb;
            return;
        }
        double d = -2 * (aSq * px * px / (ta * ta * ta) + bSq * py * py / (tb * tb * tb));
        t = t - gt / d;
    }
    ox = aSq * px / (t + aSq);
    oy = bSq * py / (t + bSq);
}
// clampSwingTwist :278-402
inline int clamp_swing_twist(const SwingTwistPart &p, Q4 &swing, Q4 &twist) {
    int clamped = 0;
    bool negSwing = swing.w < 0, negTwist = twist.w < 0;
    if (negSwing) swing = qscale(swing, -1);
    if (negTwist) twist = qscale(twist, -1);
    if (p.rotationFlags & TWIST_X_LOCKED) {
        if (twist.x != 0) clamped |= TWIST_MIN | TWIST_MAX;
        twist = {0, 0, 0, 1};
    } else if (!(p.rotationFlags & TWIST_X_FREE)) {
        double dMin = p.sinTwistHalfMin - twist.x, dMax = twist.x - p.sinTwistHalfMax;
        if (dMin > 0 || dMax > 0) {
            if (distance_to_min_shorter(dMin, dMax)) {
                twist = {p.sinTwistHalfMin, 0, 0, p.cosTwistHalfMin};
                clamped |= TWIST_MIN;
            } else {
                twist = {p.sinTwistHalfMax, 0, 0, p.cosTwistHalfMax};
                clamped |= TWIST_MAX;
            }
        }
    }
    if (p.rotationFlags & SWING_Y_LOCKED) {
        if (p.rotationFlags & SWING_Z_LOCKED) {
            if (swing.y != 0) clamped |= SWING_Y_MIN | SWING_Y_MAX;
            if (swing.z != 0) clamped |= SWING_Z_MIN | SWING_Z_MAX;
            swing = {0, 0, 0, 1};
        } else {
            if (swing.y != 0) clamped |= SWING_Y_MIN | SWING_Y_MAX;
            double dMin = p.sinSwingZHalfMin - swing.z, dMax = swing.z - p.sinSwingZHalfMax;
            if (dMin > 0 || dMax > 0) {
                if (distance_to_min_shorter(dMin, dMax)) {
                    swing = {0, 0, p.sinSwingZHalfMin, p.cosSwingZHalfMin};
                    clamped |= SWING_Z_MIN;
                } else {
                    swing = {0, 0, p.sinSwingZHalfMax, p.cosSwingZHalfMax};
                    clamped |= SWING_Z_MAX;
                }
            } else if (clamped & SWING_Y_MIN) {
                double z = swing.z;
                swing = {0, 0, z, std::sqrt(1 - z * z)};
            }
        }
    } else if (p.rotationFlags & SWING_Z_LOCKED) {
        if (swing.z != 0) clamped |= SWING_Z_MIN | SWING_Z_MAX;
        double dMin = p.sinSwingYHalfMin - swing.y, dMax = swing.y - p.sinSwingYHalfMax;
        if (dMin > 0 || dMax > 0) {
            if (distance_to_min_shorter(dMin, dMax)) {
                swing = {0, p.sinSwingYHalfMin, 0, p.cosSwingYHalfMin};
                clamped |= SWING_Y_MIN;
            } else {
                swing = {0, p.sinSwingYHalfMax, 0, p.cosSwingYHalfMax};
                clamped |= SWING_Y_MAX;
            }
        } else if (clamped & SWING_Z_MIN) {
            double y = swing.y;
            swing = {0, y, 0, std::sqrt(1 - y * y)};
        }
    } else if (p.swingType == SWING_CONE) {
        double y = swing.y, z = swing.z, a = p.sinSwingYHalfMax, b = p.sinSwingZHalfMax;
        if (a > 0 && b > 0) {
            double e = y * y / (a * a) + z * z / (b * b);
            if (e > 1) {
                double cy, cz;
                closest_point_on_ellipse(y, z, a, b, cy, cz);
                double nw = std::sqrt(std::max(0.0, 1 - cy * cy - cz * cz));
                swing = {0, cy, cz, nw};
                clamped |= SWING_Y_MIN | SWING_Y_MAX | SWING_Z_MIN | SWING_Z_MAX;
            }
        }
    } else {
        double hy = std::atan2(swing.y, swing.w), hz = std::atan2(swing.z, swing.w);
        double cy = std::max(p.swingYHalfMin, std::min(p.swingYHalfMax, hy));
        double cz = std::max(p.swingZHalfMin, std::min(p.swingZHalfMax, hz));
        if (hy != cy || hz != cz) {
            double sy = std::sin(cy), coy = std::cos(cy), sz = std::sin(cz), coz = std::cos(cz);
            double ny = sy * coz, nz = coy * sz, nw = coy * coz;
            double l = std::sqrt(ny * ny + nz * nz + nw * nw);
            swing = {0, ny / l, nz / l, nw / l};
            clamped |= SWING_Y_MIN | SWING_Y_MAX | SWING_Z_MIN | SWING_Z_MAX;
        }
    }
    if (negSwing) swing = qscale(swing, -1);
    if (negTwist) twist = qscale(twist, -1);
    return clamped;
}
// calculateConstraintProperties :481-652
inline void st_calc(SwingTwistPart &p, const Body &A, const Body &B, Q4 q, Q4 c2w) {
    Q4 sw, tw;
    get_swing_twist(q, sw, tw);
    Q4 csw = sw, ctw = tw;
    int clamped = clamp_swing_twist(p, csw, ctw);
    const V3 X{1, 0, 0}, Y{0, 1, 0}, Z{0, 0, 1};
    if (p.rotationFlags & SWING_Y_LOCKED) {
        Q4 t2w = qmul(c2w, sw);
        p.wsSwingY = rotate(t2w, Y);
        p.wsSwingZ = rotate(t2w, Z);
        if (p.rotationFlags & SWING_Z_LOCKED) {
            angle_calc(p.swingY, A, B, p.wsSwingY, 0);
            angle_calc(p.swingZ, A, B, p.wsSwingZ, 0);
        } else {
            angle_calc(p.swingY, A, B, p.wsSwingY, 0);
            if (clamped & (SWING_Z_MIN | SWING_Z_MAX)) {
                if (clamped & SWING_Z_MIN) p.wsSwingZ = neg(p.wsSwingZ);
                angle_calc(p.swingZ, A, B, p.wsSwingZ, 0);
            } else {
                angle_deactivate(p.swingZ);
            }
        }
    } else if (p.rotationFlags & SWING_Z_LOCKED) {
        Q4 t2w = qmul(c2w, sw);
        p.wsSwingY = rotate(t2w, Y);
        p.wsSwingZ = rotate(t2w, Z);
        if (clamped & (SWING_Y_MIN | SWING_Y_MAX)) {
            if (clamped & SWING_Y_MIN) p.wsSwingY = neg(p.wsSwingY);
            angle_calc(p.swingY, A, B, p.wsSwingY, 0);
        } else {
            angle_deactivate(p.swingY);
        }
        angle_calc(p.swingZ, A, B, p.wsSwingZ, 0);
    } else if ((p.rotationFlags & SWING_YZ_FREE) != SWING_YZ_FREE) {
        if (clamped & (SWING_Y_MIN | SWING_Y_MAX | SWING_Z_MIN | SWING_Z_MAX)) {
            V3 current = rotate(qmul(c2w, sw), X), desired = rotate(qmul(c2w, csw), X);
            V3 c = cross(desired, current);
            double l = len(c);
            if (l > 1e-6) {
                p.wsSwingY = scale(c, 1 / l);
                angle_calc(p.swingY, A, B, p.wsSwingY, 0);
            } else {
                angle_deactivate(p.swingY);
            }
        } else {
            angle_deactivate(p.swingY);
        }
        angle_deactivate(p.swingZ);
    } else {
        angle_deactivate(p.swingY);
        angle_deactivate(p.swingZ);
    }
    if (p.rotationFlags & TWIST_X_LOCKED) {
        p.wsTwist = rotate(qmul(c2w, sw), X);
        angle_calc(p.twist, A, B, p.wsTwist, 0);
    } else if (!(p.rotationFlags & TWIST_X_FREE)) {
        if (clamped & (TWIST_MIN | TWIST_MAX)) {
            p.wsTwist = rotate(qmul(c2w, sw), X);
            if (clamped & TWIST_MIN) p.wsTwist = neg(p.wsTwist);
            angle_calc(p.twist, A, B, p.wsTwist, 0);
        } else {
            angle_deactivate(p.twist);
        }
    } else {
        angle_deactivate(p.twist);
    }
}
inline void st_warm(SwingTwistPart &p, Body &A, Body &B, double ratio) {
    angle_warm(p.swingY, A, B, ratio);
    angle_warm(p.swingZ, A, B, ratio);
    angle_warm(p.twist, A, B, ratio);
}
// solveVelocityConstraint :670-722
inline bool st_solve_velocity(SwingTwistPart &p, Body &A, Body &B) {
    const double INF = 1.0 / 0.0;
    bool imp = false;
    if (angle_active(p.swingY)) {
        double mx = p.sinSwingYHalfMin == p.sinSwingYHalfMax ? INF : 0;
        imp = angle_solve_velocity(p.swingY, A, B, p.wsSwingY, -INF, mx) || imp;
    }
    if (angle_active(p.swingZ)) {
        double mx = p.sinSwingZHalfMin == p.sinSwingZHalfMax ? INF : 0;
        imp = angle_solve_velocity(p.swingZ, A, B, p.wsSwingZ, -INF, mx) || imp;
    }
    if (angle_active(p.twist)) {
        double mx = p.sinTwistHalfMin == p.sinTwistHalfMax ? INF : 0;
        imp = angle_solve_velocity(p.twist, A, B, p.wsTwist, -INF, mx) || imp;
    }
    return imp;
}
// solvePositionConstraint :743-776 with RotationEulerConstraintPart
// (rotation-euler-constraint-part.ts calculateConstraintProperties, solvePositionConstraint)
inline bool st_solve_position(SwingTwistPart &p, Body &A, Body &B, Q4 q, Q4 c2b1, Q4 c2b2, double baumgarte) {
    Q4 sw, tw;
    get_swing_twist(q, sw, tw);
    int clamped = clamp_swing_twist(p, sw, tw);
    if (clamped == 0) return false;
    Q4 invInitial = qmul(c2b2, qconj(qmul(qmul(c2b1, sw), tw)));
    M3 I1 = world_inv_inertia(A), I2 = world_inv_inertia(B), eff;
    if (!m3_invert(eff, m3_add(I1, I2))) eff = m3_zero();
    Q4 diff = qmul(qmul(B.quat, invInitial), qconj(A.quat));
    if (diff.w < 0) diff = qscale(diff, -1);
    V3 err{2 * diff.x, 2 * diff.y, 2 * diff.z};
    if (lensq(err) < 1e-12) return false;
    V3 l = scale(m3_mul(eff, err), -baumgarte);
    if (A.motion == DYNAMIC) sub_rotation_step(A, m3_mul(I1, l));
    if (B.motion == DYNAMIC) add_rotation_step(B, m3_mul(I2, l));
    return true;
}

// ---- SwingTwistConstraint (swing-twist-constraint.ts) --------------------------------
inline void swing_update_limits(SwingTwistJoint &j) {  // updateLimits :300-310
    st_set_limits(j.st, j.twistMin, j.twistMax, -j.planeHalfCone, j.planeHalfCone, -j.normalHalfCone, j.normalHalfCone);
}
// setupVelocity :484-666
inline void swing_setup(SwingTwistJoint &j, const Body &A, const Body &B, double dt) {
    point_calc(j.point, A, j.lp1, B, j.lp2);
    Q4 c1w = qmul(A.quat, j.c2b1), c2w = qmul(B.quat, j.c2b2);
    Q4 q = qmul(qconj(c1w), c2w);
    st_calc(j.st, A, B, q, c1w);
    if (j.swingMotorState != MOTOR_OFF || j.twistMotorState != MOTOR_OFF || j.maxFrictionTorque > 0) {
        const V3 E[3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
        for (int i = 0; i < 3; i++) j.wsMotorAxis[i] = rotate(c2w, E[i]);
        V3 err{0, 0, 0};
        if (j.swingMotorState == MOTOR_POSITION || j.twistMotorState == MOTOR_POSITION) {
            Q4 t = j.targetOrientation;
            if (q.x * t.x + q.y * t.y + q.z * t.z + q.w * t.w < 0) t = qscale(t, -1);
            Q4 d = qmul(qconj(q), t);
            err = {-2 * d.x, -2 * d.y, -2 * d.z};
        }
        double e[3] = {err.x, err.y, err.z};
        double tav[3] = {j.targetAngularVelocity.x, j.targetAngularVelocity.y, j.targetAngularVelocity.z};
        switch (j.swingMotorState) {
            case MOTOR_OFF:
                if (j.maxFrictionTorque > 0) {
                    for (int i = 1; i < 3; i++) angle_calc(j.motor[i], A, B, j.wsMotorAxis[i], 0);
                } else {
                    for (int i = 0; i < 3; i++) angle_deactivate(j.motor[i]);
                }
                break;
            case MOTOR_VELOCITY:
                for (int i = 1; i < 3; i++) angle_calc(j.motor[i], A, B, j.wsMotorAxis[i], -tav[i]);
                break;
            case MOTOR_POSITION:
                if (j.swingMotorSpring.frequencyOrStiffness > 0) {
                    for (int i = 1; i < 3; i++)
                        angle_calc_settings(j.motor[i], dt, A, B, j.wsMotorAxis[i], 0, e[i], j.swingMotorSpring);
                } else {
                    for (int i = 1; i < 3; i++) angle_deactivate(j.motor[i]);
                }
                break;
        }
        switch (j.twistMotorState) {
            case MOTOR_OFF:
                if (j.maxFrictionTorque > 0)
                    angle_calc(j.motor[0], A, B, j.wsMotorAxis[0], 0);
                else
                    angle_deactivate(j.motor[0]);
                break;
            case MOTOR_VELOCITY:
                angle_calc(j.motor[0], A, B, j.wsMotorAxis[0], -tav[0]);
                break;
            case MOTOR_POSITION:
                if (j.twistMotorSpring.frequencyOrStiffness > 0)
                    angle_calc_settings(j.motor[0], dt, A, B, j.wsMotorAxis[0], 0, e[0], j.twistMotorSpring);
                else
                    angle_deactivate(j.motor[0]);
                break;
        }
    } else {
        for (int i = 0; i < 3; i++) angle_deactivate(j.motor[i]);
    }
}
// warmStartVelocity :668-680: motors, limits, point
inline void swing_warm(SwingTwistJoint &j, Body &A, Body &B, double ratio) {
    for (int i = 0; i < 3; i++) angle_warm(j.motor[i], A, B, ratio);
    st_warm(j.st, A, B, ratio);
    point_warm(j.point, A, B, ratio);
}
// solveVelocity :682-748
inline bool swing_solve_velocity(SwingTwistJoint &j, Body &A, Body &B, double dt) {
    bool imp = false;
    if (angle_active(j.motor[0])) {
        double mn, mx;
        if (j.twistMotorState == MOTOR_OFF) {
            mx = dt * j.maxFrictionTorque;
            mn = -mx;
        } else {
            mn = dt * j.twistMinTorque;
            mx = dt * j.twistMaxTorque;
        }
        imp = angle_solve_velocity(j.motor[0], A, B, j.wsMotorAxis[0], mn, mx) || imp;
    }
    if (angle_active(j.motor[1])) {
        double mn, mx;
        if (j.swingMotorState == MOTOR_OFF) {
            mx = dt * j.maxFrictionTorque;
            mn = -mx;
        } else {
            mn = dt * j.swingMinTorque;
            mx = dt * j.swingMaxTorque;
        }
        for (int i = 1; i < 3; i++) imp = angle_solve_velocity(j.motor[i], A, B, j.wsMotorAxis[i], mn, mx) || imp;
    }
    imp = st_solve_velocity(j.st, A, B) || imp;
    imp = point_solve_velocity(j.point, A, B) || imp;
    return imp;
}
// solvePosition :757-800: rotation limits, then the point from the corrected poses
inline bool swing_solve_position(SwingTwistJoint &j, Body &A, Body &B, double baumgarte) {
    Q4 c1w = qmul(A.quat, j.c2b1), c2w = qmul(B.quat, j.c2b2);
    Q4 q = qmul(qconj(c1w), c2w);
    bool imp = st_solve_position(j.st, A, B, q, j.c2b1, j.c2b2, baumgarte);
    point_calc(j.point, A, j.lp1, B, j.lp2);
    imp = point_solve_position(j.point, A, B, baumgarte) || imp;
    return imp;
}

// ---- RotationEulerConstraintPart (rotation-euler-constraint-part.ts) -----------------
inline void euler_deactivate(EulerPart &p) {  // deactivate :49-52
    p.effMass = m3_zero();
    p.totalLambda = {0, 0, 0};
}
// getInvInitialOrientationXY :71-111; vec3.equals is mathcat's (gl-matrix's) approximate
// comparison, |a - b| <= 1e-6 max(1, |a|, |b|) per component
inline bool vec3_equals(V3 a, V3 b) {
    auto eq = [](double x, double y) {
        return std::fabs(x - y) <= 1e-6 * std::max(1.0, std::max(std::fabs(x), std::fabs(y)));
    };
    return eq(a.x, b.x) && eq(a.y, b.y) && eq(a.z, b.z);
}
inline Q4 axes_to_quat(V3 x, V3 y) {  // quat.fromMat3 of the columns (x, y, x cross y)
    V3 z = cross(x, y);
    M3 m;
    V3 c[3] = {x, y, z};
    for (int k = 0; k < 3; k++) {
        m.m[k][0] = c[k].x;
        m.m[k][1] = c[k].y;
        m.m[k][2] = c[k].z;
    }
    return quat_from_m3(m);
}
inline Q4 inv_initial_orientation_xy(V3 x1, V3 y1, V3 x2, V3 y2) {
    if (vec3_equals(x1, x2) && vec3_equals(y1, y2)) return {0, 0, 0, 1};
    return qmul(axes_to_quat(x2, y2), qconj(axes_to_quat(x1, y1)));
}
// calculateConstraintProperties :127-156
inline void euler_calc(EulerPart &p, const Body &A, const Body &B) {
    p.invI1 = world_inv_inertia(A);
    p.invI2 = world_inv_inertia(B);
    if (!m3_invert(p.effMass, m3_add(p.invI1, p.invI2))) euler_deactivate(p);
}
// applyVelocityStep :226-247
inline bool euler_apply(EulerPart &p, Body &A, Body &B, V3 l) {
    if (lensq(l) == 0) return false;
    if (A.motion == DYNAMIC) A.angvel = sub(A.angvel, m3_mul(p.invI1, l));
    if (B.motion == DYNAMIC) B.angvel = add(B.angvel, m3_mul(p.invI2, l));
    return true;
}
inline void euler_warm(EulerPart &p, Body &A, Body &B, double ratio) {  // warmStart :158-169
    p.totalLambda = scale(p.totalLambda, ratio);
    euler_apply(p, A, B, p.totalLambda);
}
inline bool euler_solve_velocity(EulerPart &p, Body &A, Body &B) {  // solveVelocityConstraint :176-213
    V3 w1 = A.motion != STATIC ? A.angvel : V3{0, 0, 0};
    V3 w2 = B.motion != STATIC ? B.angvel : V3{0, 0, 0};
    V3 l = m3_mul(p.effMass, sub(w1, w2));
    p.totalLambda = add(p.totalLambda, l);
    return euler_apply(p, A, B, l);
}
// solvePositionConstraint :256-311: error = 2 xyz of q2 invInitial q1^-1 (w made positive)
inline bool euler_solve_position(EulerPart &p, Body &A, Body &B, Q4 invInitial, double baumgarte) {
    Q4 diff = qmul(qmul(B.quat, invInitial), qconj(A.quat));
    if (diff.w < 0) diff = {-diff.x, -diff.y, -diff.z, -diff.w};
    V3 err{2 * diff.x, 2 * diff.y, 2 * diff.z};
    if (lensq(err) < 1e-12) return false;
    V3 l = scale(m3_mul(p.effMass, err), -baumgarte);
    if (A.motion == DYNAMIC) sub_rotation_step(A, m3_mul(p.invI1, l));
    if (B.motion == DYNAMIC) add_rotation_step(B, m3_mul(p.invI2, l));
    return true;
}

// ---- AxisConstraintPart with a spring, and its position solve ------------------------
inline M4 world_inv_inertia4(const Body &b) {
    M4 r{};
    if (b.motion == DYNAMIC) r = inv_inertia_for_rotation(b, mat4_from_quat(b.quat));
    return r;
}
inline double dyn_inv_mass(const Body &b) { return b.motion == DYNAMIC ? b.invMass : 0.0; }
// calculateConstraintPropertiesWithSettings axis-constraint-part.ts:400-440
inline void axis_calc_settings(AxisPart &p, double dt, const Body &A, const Body &B, V3 r1, V3 r2, V3 ax, double bias,
                               double C, const SpringSettings &s) {
    double iem = inv_eff_mass(p, A, B, dyn_inv_mass(A), dyn_inv_mass(B), world_inv_inertia4(A),
                              world_inv_inertia4(B), r1, r2, ax);
    if (iem == 0) {
        p.effMass = 0;
        p.totalLambda = 0;
        return;
    }
    SpringPart sp;
    p.effMass = spring_with_settings(sp, dt, iem, bias, C, s);
    p.softness = sp.softness;
    p.bias = sp.bias;
}
inline void axis_calc(AxisPart &p, const Body &A, const Body &B, V3 r1, V3 r2, V3 ax, double bias) {
    calc_props(p, A, B, dyn_inv_mass(A), dyn_inv_mass(B), world_inv_inertia4(A), world_inv_inertia4(B), r1, r2, ax,
               bias);
}
inline void axis_deactivate(AxisPart &p) {
    p.effMass = 0;
    p.totalLambda = 0;
}
// solveVelocityConstraint :557-570 (getTotalLambda, clamp, applyLambda)
inline bool axis_solve_velocity(AxisPart &p, Body &A, Body &B, V3 ax, double mn, double mx) {
    double tl = total_lambda(p, A, B, ax);
    return apply_lambda(p, A, B, dyn_inv_mass(A), dyn_inv_mass(B), ax, std::max(mn, std::min(mx, tl)));
}
// solvePositionConstraintWithMassOverride :790-847
inline bool axis_solve_position(AxisPart &p, Body &A, Body &B, V3 ax, double C, double baumgarte) {
    if (C == 0 || p.effMass == 0 || p.softness != 0) return false;
    double l = -p.effMass * baumgarte * C;
    if (A.motion == DYNAMIC) {
        A.com = sub(A.com, scale(ax, l * A.invMass));
        apply_dof_pos(A);
        sub_rotation_step(A, scale(p.invI1, l));
    }
    if (B.motion == DYNAMIC) {
        B.com = add(B.com, scale(ax, l * B.invMass));
        apply_dof_pos(B);
        add_rotation_step(B, scale(p.invI2, l));
    }
    return true;
}

// ---- DualAxisConstraintPart (dual-axis-constraint-part.ts) ---------------------------
inline void dual_deactivate(DualAxisPart &p) {
    p.totalLambda[0] = p.totalLambda[1] = 0;
    for (double &e : p.eff) e = 0;
}
inline bool dual_active(const DualAxisPart &p) { return p.eff[0] != 0 || p.eff[1] != 0 || p.eff[2] != 0 || p.eff[3] != 0; }
// calculateConstraintProperties :78-140 (mat2.invert: null when the determinant is 0)
inline void dual_calc(DualAxisPart &p, const Body &A, V3 r1u, const Body &B, V3 r2, V3 n1, V3 n2) {
    double iem[4] = {0, 0, 0, 0};
    auto side = [&](const Body &b, V3 r, V3 &c1, V3 &c2, V3 &i1, V3 &i2) {
        c1 = cross(r, n1);
        c2 = cross(r, n2);
        M3 I = world_inv_inertia(b);
        i1 = m3_mul(I, c1);
        i2 = m3_mul(I, c2);
        iem[0] += b.invMass + dot(c1, i1);
        iem[1] += dot(c2, i1);
        iem[2] += dot(c1, i2);
        iem[3] += b.invMass + dot(c2, i2);
    };
    if (A.motion == DYNAMIC) side(A, r1u, p.r1xn1, p.r1xn2, p.i1n1, p.i1n2);
    if (B.motion == DYNAMIC) side(B, r2, p.r2xn1, p.r2xn2, p.i2n1, p.i2n2);
    double det = iem[0] * iem[3] - iem[2] * iem[1];
    if (det == 0) {
        dual_deactivate(p);
        return;
    }
    det = 1.0 / det;
    p.eff[0] = iem[3] * det;
    p.eff[1] = -iem[1] * det;
    p.eff[2] = -iem[2] * det;
    p.eff[3] = iem[0] * det;
}
inline void dual_apply(DualAxisPart &p, Body &A, Body &B, V3 n1, V3 n2, double l0, double l1) {
    V3 imp = scale_add(scale(n1, l0), n2, l1);
    if (A.motion == DYNAMIC) {
        A.linvel = sub(A.linvel, scale(imp, A.invMass));
        apply_dof_lin(A);
        A.angvel = sub(A.angvel, scale_add(scale(p.i1n1, l0), p.i1n2, l1));
    }
    if (B.motion == DYNAMIC) {
        B.linvel = add(B.linvel, scale(imp, B.invMass));
        apply_dof_lin(B);
        B.angvel = add(B.angvel, scale_add(scale(p.i2n1, l0), p.i2n2, l1));
    }
}
inline void dual_warm(DualAxisPart &p, Body &A, Body &B, V3 n1, V3 n2, double ratio) {  // warmStart :148-186
    if (!dual_active(p)) return;
    p.totalLambda[0] *= ratio;
    p.totalLambda[1] *= ratio;
    if (p.totalLambda[0] == 0 && p.totalLambda[1] == 0) return;
    dual_apply(p, A, B, n1, n2, p.totalLambda[0], p.totalLambda[1]);
}
// solveVelocityConstraint :194-267
inline bool dual_solve_velocity(DualAxisPart &p, Body &A, Body &B, V3 n1, V3 n2) {
    if (!dual_active(p)) return false;
    bool mA = A.motion != STATIC, mB = B.motion != STATIC;
    double j0 = 0, j1 = 0;
    if (mA && mB) {
        j0 = dot(n1, A.linvel) - dot(n1, B.linvel);
        j1 = dot(n2, A.linvel) - dot(n2, B.linvel);
    } else if (mA) {
        j0 = dot(n1, A.linvel);
        j1 = dot(n2, A.linvel);
    } else if (mB) {
        j0 = -dot(n1, B.linvel);
        j1 = -dot(n2, B.linvel);
    }
    if (mA) {
        j0 += dot(p.r1xn1, A.angvel);
        j1 += dot(p.r1xn2, A.angvel);
    }
    if (mB) {
        j0 -= dot(p.r2xn1, B.angvel);
        j1 -= dot(p.r2xn2, B.angvel);
    }
    double l0 = p.eff[0] * j0 + p.eff[2] * j1, l1 = p.eff[1] * j0 + p.eff[3] * j1;  // vec2.transformMat2
    p.totalLambda[0] += l0;
    p.totalLambda[1] += l1;
    if (l0 == 0 && l1 == 0) return false;
    dual_apply(p, A, B, n1, n2, l0, l1);
    return true;
}
// solvePositionConstraint :275-330
inline bool dual_solve_position(DualAxisPart &p, Body &A, Body &B, V3 u, V3 n1, V3 n2, double baumgarte) {
    if (!dual_active(p)) return false;
    double c0 = dot(u, n1), c1 = dot(u, n2);
    if (c0 == 0 && c1 == 0) return false;
    double l0 = -baumgarte * (p.eff[0] * c0 + p.eff[2] * c1), l1 = -baumgarte * (p.eff[1] * c0 + p.eff[3] * c1);
    if (l0 == 0 && l1 == 0) return false;
    V3 imp = scale_add(scale(n1, l0), n2, l1);
    if (A.motion == DYNAMIC) {
        A.com = sub(A.com, scale(imp, A.invMass));
        apply_dof_pos(A);
        sub_rotation_step(A, scale_add(scale(p.i1n1, l0), p.i1n2, l1));
    }
    if (B.motion == DYNAMIC) {
        B.com = add(B.com, scale(imp, B.invMass));
        apply_dof_pos(B);
        add_rotation_step(B, scale_add(scale(p.i2n1, l0), p.i2n2, l1));
    }
    return true;
}

// ---- PointConstraint (point-constraint.ts:186-244) -----------------------------------
inline void pointj_setup(PointJoint &j, const Body &A, const Body &B) { point_calc(j.point, A, j.lp1, B, j.lp2); }
inline void pointj_warm(PointJoint &j, Body &A, Body &B, double ratio) { point_warm(j.point, A, B, ratio); }
inline bool pointj_solve_velocity(PointJoint &j, Body &A, Body &B) { return point_solve_velocity(j.point, A, B); }
inline bool pointj_solve_position(PointJoint &j, Body &A, Body &B, double baumgarte) {
    point_calc(j.point, A, j.lp1, B, j.lp2);
    return point_solve_position(j.point, A, B, baumgarte);
}

// ---- FixedConstraint (fixed-constraint.ts:299-395) -----------------------------------
inline void fixed_setup(FixedJoint &j, const Body &A, const Body &B) {
    euler_calc(j.rot, A, B);
    point_calc(j.point, A, j.lp1, B, j.lp2);
}
inline void fixed_warm(FixedJoint &j, Body &A, Body &B, double ratio) {
    euler_warm(j.rot, A, B, ratio);
    point_warm(j.point, A, B, ratio);
}
inline bool fixed_solve_velocity(FixedJoint &j, Body &A, Body &B) {
    bool rot = euler_solve_velocity(j.rot, A, B);
    bool pos = point_solve_velocity(j.point, A, B);
    return rot || pos;
}
inline bool fixed_solve_position(FixedJoint &j, Body &A, Body &B, double baumgarte) {
    euler_calc(j.rot, A, B);
    bool rot = euler_solve_position(j.rot, A, B, j.invInitial, baumgarte);
    point_calc(j.point, A, j.lp1, B, j.lp2);
    bool pos = point_solve_position(j.point, A, B, baumgarte);
    return rot || pos;
}

// ---- DistanceConstraint (distance-constraint.ts:270-465) -----------------------------
// calculateDistanceConstraintProperties :270-373
inline void distance_calc(DistanceJoint &j, const Body &A, const Body &B, double dt) {
    j.wp1 = add(rotate(A.quat, j.lp1), A.com);
    j.wp2 = add(rotate(B.quat, j.lp2), B.com);
    V3 delta = sub(j.wp2, j.wp1);
    double dl = len(delta);
    if (dl > 0) j.wn = scale(delta, 1 / dl);
    V3 r1u = sub(j.wp2, A.com), r2 = sub(j.wp2, B.com);
    if (j.minDistance == j.maxDistance) {
        axis_calc_settings(j.axis, dt, A, B, r1u, r2, j.wn, 0, dl - j.minDistance, j.spring);
        j.minLambda = -1.0 / 0.0;
        j.maxLambda = 1.0 / 0.0;
    } else if (dl <= j.minDistance) {
        axis_calc_settings(j.axis, dt, A, B, r1u, r2, j.wn, 0, dl - j.minDistance, j.spring);
        j.minLambda = 0;
        j.maxLambda = 1.0 / 0.0;
    } else if (dl >= j.maxDistance) {
        axis_calc_settings(j.axis, dt, A, B, r1u, r2, j.wn, 0, dl - j.maxDistance, j.spring);
        j.minLambda = -1.0 / 0.0;
        j.maxLambda = 0;
    } else {
        axis_deactivate(j.axis);
    }
}
inline void distance_warm(DistanceJoint &j, Body &A, Body &B, double ratio) {
    warm_start(j.axis, A, B, dyn_inv_mass(A), dyn_inv_mass(B), j.wn, ratio);
}
inline bool distance_solve_velocity(DistanceJoint &j, Body &A, Body &B) {
    if (j.axis.effMass == 0) return false;
    return axis_solve_velocity(j.axis, A, B, j.wn, j.minLambda, j.maxLambda);
}
// solvePosition :420-458: the error is measured on the world points of the last property
// calculation (setup, or the previous position iteration), then the properties are refreshed
inline bool distance_solve_position(DistanceJoint &j, Body &A, Body &B, double dt, double baumgarte) {
    if (j.spring.frequencyOrStiffness > 0) return false;
    double d = dot(sub(j.wp2, j.wp1), j.wn);
    double err = 0;
    if (d < j.minDistance)
        err = d - j.minDistance;
    else if (d > j.maxDistance)
        err = d - j.maxDistance;
    if (err == 0) return false;
    distance_calc(j, A, B, dt);
    return axis_solve_position(j.axis, A, B, j.wn, err, baumgarte);
}

// ---- ConeConstraint (cone-constraint.ts:321-448) -------------------------------------
// calculateRotationConstraintProperties :321-347
inline void cone_rot_calc(ConeJoint &j, const Body &A, const Body &B) {
    V3 t1 = rotate(A.quat, j.lt1), t2 = rotate(B.quat, j.lt2);
    j.cosTheta = dot(t1, t2);
    if (j.cosTheta < j.cosHalfCone) {
        V3 ra = cross(t2, t1);
        double l = len(ra);
        if (l > 1e-6) j.wRotAxis = scale(ra, 1 / l);
        angle_calc(j.angle, A, B, j.wRotAxis, 0);
    } else {
        angle_deactivate(j.angle);
    }
}
inline void cone_setup(ConeJoint &j, const Body &A, const Body &B) {
    point_calc(j.point, A, j.lp1, B, j.lp2);
    cone_rot_calc(j, A, B);
}
inline void cone_warm(ConeJoint &j, Body &A, Body &B, double ratio) {
    point_warm(j.point, A, B, ratio);
    if (angle_active(j.angle)) angle_warm(j.angle, A, B, ratio);
}
inline bool cone_solve_velocity(ConeJoint &j, Body &A, Body &B) {
    bool pos = point_solve_velocity(j.point, A, B);
    bool rot = false;
    if (angle_active(j.angle)) rot = angle_solve_velocity(j.angle, A, B, j.wRotAxis, 0, 1.0 / 0.0);
    return pos || rot;
}
inline bool cone_solve_position(ConeJoint &j, Body &A, Body &B, double baumgarte) {
    point_calc(j.point, A, j.lp1, B, j.lp2);
    bool pos = point_solve_position(j.point, A, B, baumgarte);
    cone_rot_calc(j, A, B);
    bool rot = false;
    if (angle_active(j.angle)) rot = angle_solve_position(j.angle, A, B, j.cosTheta - j.cosHalfCone, baumgarte);
    return pos || rot;
}

// ---- SliderConstraint (slider-constraint.ts:546-1038) --------------------------------
inline void slider_r1r2u(SliderJoint &j, const Body &A, const Body &B) {  // calculateR1R2U :546-562
    j.r1 = m3mul(mat4_from_quat(A.quat), j.lp1);
    j.r2 = m3mul(mat4_from_quat(B.quat), j.lp2);
    j.u = sub(add(sub(B.com, A.com), j.r2), j.r1);
}
inline void slider_axis_pos(SliderJoint &j, const Body &A) {  // calculateSlidingAxisAndPosition :564-577
    if (j.hasLimits || j.motorState != MOTOR_OFF || j.maxFrictionForce > 0) {
        j.wSlider = m3mul(mat4_from_quat(A.quat), j.lSlider1);
        j.d = dot(j.u, j.wSlider);
    }
}
inline void slider_pos_calc(SliderJoint &j, const Body &A, const Body &B) {  // :579-609
    M4 RA = mat4_from_quat(A.quat);
    j.n1 = m3mul(RA, j.lNormal1);
    j.n2 = m3mul(RA, j.lNormal2);
    dual_calc(j.pos, A, add(j.r1, j.u), B, j.r2, j.n1, j.n2);
}
inline void slider_limits_calc(SliderJoint &j, const Body &A, const Body &B, double dt) {  // :611-696
    if (!j.hasLimits) {
        axis_deactivate(j.limits);
        return;
    }
    bool below = j.d <= j.limitsMin, above = j.d >= j.limitsMax;
    if (below || above) {
        double err = below ? j.d - j.limitsMin : j.d - j.limitsMax;
        V3 r1u = add(j.r1, j.u);
        if (j.limitsSpring.frequencyOrStiffness > 0)
            axis_calc_settings(j.limits, dt, A, B, r1u, j.r2, j.wSlider, 0, err, j.limitsSpring);
        else
            axis_calc(j.limits, A, B, r1u, j.r2, j.wSlider, 0);
    } else {
        axis_deactivate(j.limits);
    }
}
inline void slider_motor_calc(SliderJoint &j, const Body &A, const Body &B, double dt) {  // :698-785
    V3 r1u = add(j.r1, j.u);
    if (j.motorState == MOTOR_OFF) {
        if (j.maxFrictionForce > 0)
            axis_calc(j.motor, A, B, r1u, j.r2, j.wSlider, 0);
        else
            axis_deactivate(j.motor);
    } else if (j.motorState == MOTOR_VELOCITY) {
        axis_calc(j.motor, A, B, r1u, j.r2, j.wSlider, -j.targetVelocity);
    } else if (j.motorSpring.frequencyOrStiffness > 0) {
        axis_calc_settings(j.motor, dt, A, B, r1u, j.r2, j.wSlider, 0, j.d - j.targetPosition, j.motorSpring);
    } else {
        axis_deactivate(j.motor);
    }
}
inline void slider_setup(SliderJoint &j, const Body &A, const Body &B, double dt) {  // setupVelocity :787-827
    slider_r1r2u(j, A, B);
    slider_pos_calc(j, A, B);
    euler_calc(j.rot, A, B);
    slider_axis_pos(j, A);
    slider_limits_calc(j, A, B, dt);
    slider_motor_calc(j, A, B, dt);
}
inline void slider_warm(SliderJoint &j, Body &A, Body &B, double ratio) {  // warmStartVelocity :829-877
    if (j.motor.effMass != 0) warm_start(j.motor, A, B, dyn_inv_mass(A), dyn_inv_mass(B), j.wSlider, ratio);
    dual_warm(j.pos, A, B, j.n1, j.n2, ratio);
    euler_warm(j.rot, A, B, ratio);
    if (j.limits.effMass != 0) warm_start(j.limits, A, B, dyn_inv_mass(A), dyn_inv_mass(B), j.wSlider, ratio);
}
inline bool slider_solve_velocity(SliderJoint &j, Body &A, Body &B, double dt) {  // solveVelocity :879-958
    bool motor = false, limit = false;
    if (j.motor.effMass != 0) {
        if (j.motorState == MOTOR_OFF) {
            double ml = j.maxFrictionForce * dt;
            motor = axis_solve_velocity(j.motor, A, B, j.wSlider, -ml, ml);
        } else {
            motor = axis_solve_velocity(j.motor, A, B, j.wSlider, dt * j.minForceLimit, dt * j.maxForceLimit);
        }
    }
    bool pos = dual_solve_velocity(j.pos, A, B, j.n1, j.n2);
    bool rot = euler_solve_velocity(j.rot, A, B);
    if (j.limits.effMass != 0) {
        double mn, mx;
        if (j.limitsMin == j.limitsMax) {
            mn = -1.0 / 0.0;
            mx = 1.0 / 0.0;
        } else if (j.d <= j.limitsMin) {
            mn = 0;
            mx = 1.0 / 0.0;
        } else {
            mn = -1.0 / 0.0;
            mx = 0;
        }
        limit = axis_solve_velocity(j.limits, A, B, j.wSlider, mn, mx);
    }
    return motor || pos || rot || limit;
}
inline bool slider_solve_position(SliderJoint &j, Body &A, Body &B, double dt, double baumgarte) {  // :960-1038
    slider_r1r2u(j, A, B);
    slider_pos_calc(j, A, B);
    bool pos = dual_solve_position(j.pos, A, B, j.u, j.n1, j.n2, baumgarte);
    euler_calc(j.rot, A, B);
    bool rot = euler_solve_position(j.rot, A, B, j.invInitial, baumgarte);
    bool limit = false;
    if (j.hasLimits && !(j.limitsSpring.frequencyOrStiffness > 0)) {
        slider_r1r2u(j, A, B);
        slider_axis_pos(j, A);
        slider_limits_calc(j, A, B, dt);
        if (j.limits.effMass != 0) {
            double err = j.d <= j.limitsMin ? j.d - j.limitsMin : j.d - j.limitsMax;
            limit = axis_solve_position(j.limits, A, B, j.wSlider, err, baumgarte);
        }
    }
    return pos || rot || limit;
}

// swingTwistConstraintPart.deactivate: the three limit parts
inline void st_deactivate(SwingTwistPart &p) {
    angle_deactivate(p.swingY);
    angle_deactivate(p.swingZ);
    angle_deactivate(p.twist);
}

// ---- SixDOFConstraint (six-dof-constraint.ts) -----------------------------------------
inline bool sd_fixed(const SixDofJoint &j, int a) { return (j.fixedAxis & (1 << a)) != 0; }
inline bool sd_free(const SixDofJoint &j, int a) { return (j.freeAxis & (1 << a)) != 0; }
inline bool sd_trans_constrained(const SixDofJoint &j) { return (j.freeAxis & 7) != 7; }
inline bool sd_trans_fully(const SixDofJoint &j) { return (j.fixedAxis & 7) == 7 && !j.hasSpringLimits; }
inline bool sd_rot_constrained(const SixDofJoint &j) { return (j.freeAxis & 56) != 56; }
inline bool sd_rot_fully(const SixDofJoint &j) { return (j.fixedAxis & 56) == 56; }
inline bool sd_friction(const SixDofJoint &j, int a) { return !sd_fixed(j, a) && j.maxFriction[a] > 0; }
// updateTranslationLimits / updateRotationLimits / updateFixedFreeAxis and the cached motor
// flags (:240-333), applied after creation and after every setter
inline void sd_update(SixDofJoint &j) {
    for (int i = 0; i < 3; i++)
        if (j.limitMin[i] > j.limitMax[i]) j.limitMin[i] = j.limitMax[i] = 0;
    if (j.swingType == SWING_CONE) {
        j.limitMax[4] = std::max(0.0, j.limitMax[4]);
        j.limitMax[5] = std::max(0.0, j.limitMax[5]);
        j.limitMin[4] = -j.limitMax[4];
        j.limitMin[5] = -j.limitMax[5];
    }
    for (int i = 3; i < 6; i++) {
        j.limitMin[i] = std::max(-M_PI, std::min(M_PI, j.limitMin[i]));
        j.limitMax[i] = std::max(-M_PI, std::min(M_PI, j.limitMax[i]));
        if (j.limitMin[i] > j.limitMax[i]) j.limitMin[i] = j.limitMax[i] = 0;
    }
    j.st.swingType = j.swingType;
    st_set_limits(j.st, j.limitMin[3], j.limitMax[3], j.limitMin[4], j.limitMax[4], j.limitMin[5], j.limitMax[5]);
    j.freeAxis = j.fixedAxis = 0;
    for (int a = 0; a < 6; a++) {
        double lim = a >= 3 ? M_PI : 1.0 / 0.0;
        if (j.limitMin[a] >= j.limitMax[a])
            j.fixedAxis |= 1 << a;
        else if (j.limitMin[a] <= -lim && j.limitMax[a] >= lim)
            j.freeAxis |= 1 << a;
    }
    j.hasSpringLimits = j.limitsSpring[0].frequencyOrStiffness > 0 || j.limitsSpring[1].frequencyOrStiffness > 0 ||
                        j.limitsSpring[2].frequencyOrStiffness > 0;
    j.translationMotorActive = j.rotationMotorActive = false;
    for (int i = 0; i < 3; i++) {
        j.translationMotorActive = j.translationMotorActive || j.motorState[i] != MOTOR_OFF || sd_friction(j, i);
        j.rotationMotorActive = j.rotationMotorActive || j.motorState[3 + i] != MOTOR_OFF || sd_friction(j, 3 + i);
    }
    j.rotationPositionMotorActive = 0;
    for (int i = 0; i < 3; i++)
        if (j.motorState[3 + i] == MOTOR_POSITION) j.rotationPositionMotorActive |= 1 << i;
}
// getTwistAroundAxis :37-49
inline Q4 twist_around(Q4 q, V3 axis) {
    double d = q.x * axis.x + q.y * axis.y + q.z * axis.z;
    double l = d * d + q.w * q.w;
    if (!(l > 1e-10)) return {0, 0, 0, 1};
    double il = 1 / std::sqrt(l);
    return {d * axis.x * il, d * axis.y * il, d * axis.z * il, q.w * il};
}
// getPositionConstraintProperties :535-566
inline void sd_position_props(const SixDofJoint &j, const Body &A, const Body &B, V3 &r1u, V3 &r2, V3 &u) {
    V3 p1 = add(rotate(A.quat, j.lp1), A.com), p2 = add(rotate(B.quat, j.lp2), B.com);
    r1u = sub(p2, A.com);
    r2 = sub(p2, B.com);
    u = sub(p2, p1);
}
inline V3 m4_column(const M4 &m, int i) { return {m.m[4 * i], m.m[4 * i + 1], m.m[4 * i + 2]}; }
// setupVelocity :568-881
inline void sixdof_setup(SixDofJoint &j, const Body &A, const Body &B, double dt) {
    Q4 c1w = qmul(A.quat, j.c2b1);
    M4 ax = mat4_from_quat(c1w);
    for (int i = 0; i < 3; i++) j.translationAxis[i] = m4_column(ax, i);
    if (sd_trans_fully(j)) {
        point_calc(j.point, A, j.lp1, B, j.lp2);
    } else if (sd_trans_constrained(j) || j.translationMotorActive) {
        V3 r1u, r2, u;
        sd_position_props(j, A, B, r1u, r2, u);
        for (int i = 0; i < 3; i++) {
            const V3 ta = j.translationAxis[i];
            double d = dot(ta, u);
            j.displacement[i] = d;
            bool on = false;
            double C = 0;
            if (sd_fixed(j, i)) {
                C = d - j.limitMin[i];
                on = true;
            } else if (!sd_free(j, i)) {
                if (d <= j.limitMin[i]) {
                    C = d - j.limitMin[i];
                    on = true;
                } else if (d >= j.limitMax[i]) {
                    C = d - j.limitMax[i];
                    on = true;
                }
            }
            if (on) {
                if (j.limitsSpring[i].frequencyOrStiffness > 0)
                    axis_calc_settings(j.translation[i], dt, A, B, r1u, r2, ta, 0, C, j.limitsSpring[i]);
                else
                    axis_calc(j.translation[i], A, B, r1u, r2, ta, 0);
            } else {
                axis_deactivate(j.translation[i]);
            }
            if (j.motorState[i] == MOTOR_OFF) {
                if (sd_friction(j, i))
                    axis_calc(j.motorTranslation[i], A, B, r1u, r2, ta, 0);
                else
                    axis_deactivate(j.motorTranslation[i]);
            } else if (j.motorState[i] == MOTOR_VELOCITY) {
                axis_calc(j.motorTranslation[i], A, B, r1u, r2, ta, -(&j.targetVelocity.x)[i]);
            } else if (j.motorSpring[i].frequencyOrStiffness > 0) {
                axis_calc_settings(j.motorTranslation[i], dt, A, B, r1u, r2, ta, 0,
                                   dot(ta, u) - (&j.targetPosition.x)[i], j.motorSpring[i]);
            } else {
                axis_deactivate(j.motorTranslation[i]);
            }
        }
    }
    Q4 c2w = qmul(B.quat, j.c2b2);
    Q4 q = qmul(qconj(c1w), c2w);
    if (sd_rot_fully(j)) {
        euler_calc(j.rot, A, B);
    } else if (sd_rot_constrained(j) || j.rotationMotorActive) {
        if (sd_rot_constrained(j))
            st_calc(j.st, A, B, q, c1w);
        else
            st_deactivate(j.st);
        if (j.rotationMotorActive) {
            M4 rm = mat4_from_quat(c2w);
            for (int i = 0; i < 3; i++) j.rotationAxis[i] = m4_column(rm, i);
            Q4 t = j.targetOrientation;
            if (q.x * t.x + q.y * t.y + q.z * t.z + q.w * t.w < 0) t = qscale(t, -1);
            Q4 diff = qmul(qconj(q), t), pd;
            const V3 X{1, 0, 0}, Y{0, 1, 0}, Z{0, 0, 1};
            switch (j.rotationPositionMotorActive) {
                case 1: pd = twist_around(diff, X); break;
                case 2: pd = twist_around(diff, Y); break;
                case 4: pd = twist_around(diff, Z); break;
                case 3: pd = qmul(diff, qconj(twist_around(diff, Z))); break;
                case 5: pd = qmul(diff, qconj(twist_around(diff, Y))); break;
                case 6: pd = qmul(diff, qconj(twist_around(diff, X))); break;
                default: pd = diff; break;
            }
            double err[3] = {-2 * pd.x, -2 * pd.y, -2 * pd.z};
            for (int i = 0; i < 3; i++) {
                const int a = 3 + i;
                if (j.motorState[a] == MOTOR_OFF) {
                    if (sd_friction(j, a))
                        angle_calc(j.motorRotation[i], A, B, j.rotationAxis[i], 0);
                    else
                        angle_deactivate(j.motorRotation[i]);
                } else if (j.motorState[a] == MOTOR_VELOCITY) {
                    angle_calc(j.motorRotation[i], A, B, j.rotationAxis[i], -(&j.targetAngularVelocity.x)[i]);
                } else if (j.motorSpring[a].frequencyOrStiffness > 0) {
                    angle_calc_settings(j.motorRotation[i], dt, A, B, j.rotationAxis[i], 0, err[i], j.motorSpring[a]);
                } else {
                    angle_deactivate(j.motorRotation[i]);
                }
            }
        }
    }
}
// warmStartVelocity :883-942
inline void sixdof_warm(SixDofJoint &j, Body &A, Body &B, double ratio) {
    double imA = dyn_inv_mass(A), imB = dyn_inv_mass(B);
    if (j.translationMotorActive)
        for (int i = 0; i < 3; i++)
            if (j.motorTranslation[i].effMass != 0)
                warm_start(j.motorTranslation[i], A, B, imA, imB, j.translationAxis[i], ratio);
    if (j.rotationMotorActive)
        for (int i = 0; i < 3; i++)
            if (angle_active(j.motorRotation[i])) angle_warm(j.motorRotation[i], A, B, ratio);
    if (sd_rot_fully(j))
        euler_warm(j.rot, A, B, ratio);
    else if (sd_rot_constrained(j))
        st_warm(j.st, A, B, ratio);
    if (sd_trans_fully(j)) {
        point_warm(j.point, A, B, ratio);
    } else if (sd_trans_constrained(j)) {
        for (int i = 0; i < 3; i++)
            if (j.translation[i].effMass != 0) warm_start(j.translation[i], A, B, imA, imB, j.translationAxis[i], ratio);
    }
}
// solveVelocity :966-1082 (returns false, as the reference does)
inline bool sixdof_solve_velocity(SixDofJoint &j, Body &A, Body &B, double dt) {
    if (j.translationMotorActive)
        for (int i = 0; i < 3; i++) {
            if (j.motorTranslation[i].effMass == 0) continue;
            if (j.motorState[i] == MOTOR_OFF) {
                double ml = j.maxFriction[i] * dt;
                axis_solve_velocity(j.motorTranslation[i], A, B, j.translationAxis[i], -ml, ml);
            } else {
                axis_solve_velocity(j.motorTranslation[i], A, B, j.translationAxis[i], dt * j.motorMinForce[i],
                                    dt * j.motorMaxForce[i]);
            }
        }
    if (j.rotationMotorActive)
        for (int i = 0; i < 3; i++) {
            const int a = 3 + i;
            if (!angle_active(j.motorRotation[i])) continue;
            if (j.motorState[a] == MOTOR_OFF) {
                double ml = j.maxFriction[a] * dt;
                angle_solve_velocity(j.motorRotation[i], A, B, j.rotationAxis[i], -ml, ml);
            } else {
                angle_solve_velocity(j.motorRotation[i], A, B, j.rotationAxis[i], dt * j.motorMinForce[a],
                                     dt * j.motorMaxForce[a]);
            }
        }
    if (sd_rot_fully(j))
        euler_solve_velocity(j.rot, A, B);
    else if (sd_rot_constrained(j))
        st_solve_velocity(j.st, A, B);
    if (sd_trans_fully(j)) {
        point_solve_velocity(j.point, A, B);
    } else if (sd_trans_constrained(j)) {
        for (int i = 0; i < 3; i++) {
            if (j.translation[i].effMass == 0) continue;
            double mn = -1.0 / 0.0, mx = 1.0 / 0.0;
            if (!sd_fixed(j, i)) {
                if (j.displacement[i] <= j.limitMin[i])
                    mn = 0;
                else if (j.displacement[i] >= j.limitMax[i])
                    mx = 0;
            }
            axis_solve_velocity(j.translation[i], A, B, j.translationAxis[i], mn, mx);
        }
    }
    return false;
}
// quat.fromEuler for an 'xyz' euler (mathcat, unpinned): the rotation X then Y then Z applied
// to the frame, q = qx qy qz
inline Q4 quat_from_euler_xyz(double x, double y, double z) {
    double c1 = std::cos(x / 2), s1 = std::sin(x / 2), c2 = std::cos(y / 2), s2 = std::sin(y / 2), c3 = std::cos(z / 2),
           s3 = std::sin(z / 2);
    return {s1 * c2 * c3 + c1 * s2 * s3, c1 * s2 * c3 - s1 * c2 * s3, c1 * c2 * s3 + s1 * s2 * c3,
            c1 * c2 * c3 - s1 * s2 * s3};
}
// solvePosition :1084-1236
inline bool sixdof_solve_position(SixDofJoint &j, Body &A, Body &B, double baumgarte) {
    bool imp = false;
    if (sd_rot_fully(j)) {
        Q4 off = qmul(j.c2b1, quat_from_euler_xyz(j.limitMin[3], j.limitMin[4], j.limitMin[5]));
        Q4 invInitial = qmul(j.c2b2, qconj(off));
        euler_calc(j.rot, A, B);
        imp = euler_solve_position(j.rot, A, B, invInitial, baumgarte) || imp;
    } else if (sd_rot_constrained(j)) {
        Q4 c1w = qmul(A.quat, j.c2b1), c2w = qmul(B.quat, j.c2b2);
        Q4 q = qmul(qconj(c1w), c2w);
        imp = st_solve_position(j.st, A, B, q, j.c2b1, j.c2b2, baumgarte) || imp;
    }
    if (sd_trans_fully(j)) {
        V3 lp1 = add(j.lp1, rotate(j.c2b1, V3{j.limitMin[0], j.limitMin[1], j.limitMin[2]}));
        point_calc(j.point, A, lp1, B, j.lp2);
        imp = point_solve_position(j.point, A, B, baumgarte) || imp;
    } else if (sd_trans_constrained(j)) {
        for (int i = 0; i < 3; i++) {
            if (j.limitsSpring[i].frequencyOrStiffness > 0) continue;
            V3 r1u, r2, u;
            sd_position_props(j, A, B, r1u, r2, u);
            V3 e{i == 0 ? 1.0 : 0.0, i == 1 ? 1.0 : 0.0, i == 2 ? 1.0 : 0.0};
            V3 ta = rotate(qmul(A.quat, j.c2b1), e);
            double err = 0;
            if (sd_fixed(j, i)) {
                err = dot(u, ta) - j.limitMin[i];
            } else if (!sd_free(j, i)) {
                double d = dot(u, ta);
                if (d <= j.limitMin[i])
                    err = d - j.limitMin[i];
                else if (d >= j.limitMax[i])
                    err = d - j.limitMax[i];
            }
            if (err != 0) {
                axis_calc(j.translation[i], A, B, r1u, r2, ta, 0);
                imp = axis_solve_position(j.translation[i], A, B, ta, err, baumgarte) || imp;
            }
        }
    }
    return imp;
}
