// Data of crashcat's hinge joint and its constraint parts (TEST INFRASTRUCTURE: the parity
// oracle): src/constraints/hinge-constraint.ts, constraint-part/{point,hinge-rotation,angle,
// spring}-*.ts.  Included by oracle.cpp inside namespace orc, before the World; the functions
// are in oracle_joints.h.
#pragma once

struct M3 {
    double m[3][3];  // m[col][row], like the reference's column-major mat4
};

// spring-settings.ts / spring-part.ts
enum SpringMode { FREQUENCY_AND_DAMPING = 0, STIFFNESS_AND_DAMPING = 1 };
struct SpringSettings {
    int mode = FREQUENCY_AND_DAMPING;
    double frequencyOrStiffness = 0, damping = 0;
};
struct SpringPart {
    double bias = 0, softness = 0;
};

// PointConstraintPart point-constraint-part.ts
struct PointPart {
    V3 r1, r2;
    M3 invI1_r1X, invI2_r2X, effMass;
    V3 totalLambda{0, 0, 0};
    bool active = false;
};

// HingeRotationConstraintPart hinge-rotation-constraint-part.ts
struct HingeRotPart {
    V3 a1, b2, c2, b2xA1, c2xA1;
    M3 invI1, invI2;
    double eff[4] = {0, 0, 0, 0};
    double totalLambda[2] = {0, 0};
};

// AngleConstraintPart angle-constraint-part.ts
struct AnglePart {
    V3 invI1_Axis{0, 0, 0}, invI2_Axis{0, 0, 0};
    double effMass = 0;
    SpringPart spring;
    double totalLambda = 0;
};

// HingeConstraint hinge-constraint.ts (motor settings default: motor-settings.ts:53-66)
enum MotorState { MOTOR_OFF = 0, MOTOR_VELOCITY = 1, MOTOR_POSITION = 2 };
struct HingeJoint {
    int a = 0, b = 0;
    int priority = 0, index = 0;
    bool enabled = true;
    V3 lp1, lp2, lh1, lh2, ln1, ln2;
    Q4 invInitial{0, 0, 0, 1};
    double theta = 0;
    V3 wh1{0, 0, 0};
    bool hasLimits = false;
    double limitsMin = -M_PI, limitsMax = M_PI;
    SpringSettings limitsSpring;
    int motorState = MOTOR_OFF;
    double targetAngularVelocity = 0, targetAngle = 0, maxFrictionTorque = 0;
    SpringSettings motorSpring{FREQUENCY_AND_DAMPING, 2.0, 1.0};
    double minTorqueLimit = -1.0 / 0.0, maxTorqueLimit = 1.0 / 0.0;
    PointPart point;
    HingeRotPart rot;
    AnglePart limit, motor;
};
