// Data of crashcat's user joints and their constraint parts (TEST INFRASTRUCTURE: the parity
// oracle): src/constraints/{point,distance,hinge,slider,fixed,cone,swing-twist}-constraint.ts,
// constraint-part/{point,hinge-rotation,angle,rotation-euler,dual-axis,swing-twist,spring}-*.ts.
// Included by oracle.cpp inside namespace orc, before the World; the functions
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
    int velOverride = 0, posOverride = 0;  // numVelocityStepsOverride / numPositionStepsOverride
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

// SwingTwistConstraintPart swing-twist-constraint-part.ts:47-84 (limits as sines and cosines of
// half angles; rotation flags :26-35)
enum SwingType { SWING_CONE = 0, SWING_PYRAMID = 1 };
enum RotationFlags {
    TWIST_X_LOCKED = 1,
    SWING_Y_LOCKED = 2,
    SWING_Z_LOCKED = 4,
    TWIST_X_FREE = 8,
    SWING_Y_FREE = 16,
    SWING_Z_FREE = 32,
    SWING_YZ_FREE = 48
};
enum ClampedAxis { TWIST_MIN = 1, TWIST_MAX = 2, SWING_Y_MIN = 4, SWING_Y_MAX = 8, SWING_Z_MIN = 16, SWING_Z_MAX = 32 };
struct SwingTwistPart {
    int swingType = SWING_CONE, rotationFlags = 0;
    double sinTwistHalfMin = 0, sinTwistHalfMax = 0, cosTwistHalfMin = 1, cosTwistHalfMax = 1;
    double swingYHalfMin = 0, swingYHalfMax = 0, sinSwingYHalfMin = 0, sinSwingYHalfMax = 0, cosSwingYHalfMin = 1,
           cosSwingYHalfMax = 1;
    double swingZHalfMin = 0, swingZHalfMax = 0, sinSwingZHalfMin = 0, sinSwingZHalfMax = 0, cosSwingZHalfMin = 1,
           cosSwingZHalfMax = 1;
    V3 wsSwingY{0, 0, 0}, wsSwingZ{0, 0, 0}, wsTwist{0, 0, 0};
    AnglePart swingY, swingZ, twist;
};

// SwingTwistConstraint swing-twist-constraint.ts:35-85
struct SwingTwistJoint {
    int a = 0, b = 0;
    int priority = 0, index = 0;
    int velOverride = 0, posOverride = 0;
    bool enabled = true;
    V3 lp1, lp2;
    Q4 c2b1{0, 0, 0, 1}, c2b2{0, 0, 0, 1};  // constraint space to body space
    double normalHalfCone = 0, planeHalfCone = 0, twistMin = 0, twistMax = 0, maxFrictionTorque = 0;
    int swingMotorState = MOTOR_OFF, twistMotorState = MOTOR_OFF;
    V3 targetAngularVelocity{0, 0, 0};
    Q4 targetOrientation{0, 0, 0, 1};
    SpringSettings swingMotorSpring{FREQUENCY_AND_DAMPING, 2.0, 1.0}, twistMotorSpring{FREQUENCY_AND_DAMPING, 2.0, 1.0};
    double swingMinTorque = -1.0 / 0.0, swingMaxTorque = 1.0 / 0.0, twistMinTorque = -1.0 / 0.0,
           twistMaxTorque = 1.0 / 0.0;
    V3 wsMotorAxis[3];
    PointPart point;
    SwingTwistPart st;
    AnglePart motor[3];  // twist, swing Y, swing Z
};

// RotationEulerConstraintPart rotation-euler-constraint-part.ts (3 rotational rows)
struct EulerPart {
    M3 invI1, invI2, effMass;
    V3 totalLambda{0, 0, 0};
};

// DualAxisConstraintPart dual-axis-constraint-part.ts (2 translational rows); effMass as
// mathcat's column-major mat2: [m00, m10, m01, m11]
struct DualAxisPart {
    V3 r1xn1{0, 0, 0}, r1xn2{0, 0, 0}, r2xn1{0, 0, 0}, r2xn2{0, 0, 0};
    V3 i1n1{0, 0, 0}, i1n2{0, 0, 0}, i2n1{0, 0, 0}, i2n2{0, 0, 0};
    double eff[4] = {0, 0, 0, 0};
    double totalLambda[2] = {0, 0};
};

// fields every joint type carries (constraints.ts makeConstraintBase)
struct JointBase {
    int a = 0, b = 0;
    int priority = 0, index = 0;
    int velOverride = 0, posOverride = 0;
    bool enabled = true;
};

// PointConstraint point-constraint.ts:21-26
struct PointJoint : JointBase {
    V3 lp1, lp2;
    PointPart point;
};

// FixedConstraint fixed-constraint.ts:28-46
struct FixedJoint : JointBase {
    V3 lp1, lp2;
    Q4 invInitial{0, 0, 0, 1};
    PointPart point;
    EulerPart rot;
};

// DistanceConstraint distance-constraint.ts:24-49
struct DistanceJoint : JointBase {
    V3 lp1, lp2;
    double minDistance = 0, maxDistance = 0;
    SpringSettings spring;
    V3 wp1{0, 0, 0}, wp2{0, 0, 0}, wn{0, 1, 0};
    double minLambda = 0, maxLambda = 0;
    AxisPart axis;
};

// ConeConstraint cone-constraint.ts:24-46
struct ConeJoint : JointBase {
    V3 lp1, lp2, lt1{1, 0, 0}, lt2{1, 0, 0};
    double cosHalfCone = 1;
    V3 wRotAxis{0, 1, 0};
    double cosTheta = 1;
    PointPart point;
    AnglePart angle;
};

// SliderConstraint slider-constraint.ts:56-101 (motor settings: motor-settings.ts:37-51)
struct SliderJoint : JointBase {
    V3 lp1, lp2, lSlider1, lNormal1, lNormal2;
    Q4 invInitial{0, 0, 0, 1};
    V3 r1{0, 0, 0}, r2{0, 0, 0}, u{0, 0, 0}, wSlider{0, 0, 0}, n1{0, 0, 0}, n2{0, 0, 0};
    double d = 0;
    bool hasLimits = false;
    double limitsMin = -1.0 / 0.0, limitsMax = 1.0 / 0.0;
    SpringSettings limitsSpring;
    int motorState = MOTOR_OFF;
    double targetVelocity = 0, targetPosition = 0, maxFrictionForce = 0;
    SpringSettings motorSpring{FREQUENCY_AND_DAMPING, 2.0, 1.0};
    double minForceLimit = -1.0 / 0.0, maxForceLimit = 1.0 / 0.0;
    DualAxisPart pos;
    EulerPart rot;
    AxisPart limits, motor;
};

// SixDOFConstraint six-dof-constraint.ts:66-117 (defaults makeSixDOFConstraint :119-163)
struct SixDofJoint : JointBase {
    V3 lp1, lp2;
    Q4 c2b1{0, 0, 0, 1}, c2b2{0, 0, 0, 1};  // constraintToBody1 / 2
    double limitMin[6] = {-1.0 / 0.0, -1.0 / 0.0, -1.0 / 0.0, -M_PI, -M_PI, -M_PI};
    double limitMax[6] = {1.0 / 0.0, 1.0 / 0.0, 1.0 / 0.0, M_PI, M_PI, M_PI};
    SpringSettings limitsSpring[3];
    double maxFriction[6] = {0, 0, 0, 0, 0, 0};
    int motorState[6] = {MOTOR_OFF, MOTOR_OFF, MOTOR_OFF, MOTOR_OFF, MOTOR_OFF, MOTOR_OFF};
    SpringSettings motorSpring[6];
    double motorMinForce[6] = {-1.0 / 0.0, -1.0 / 0.0, -1.0 / 0.0, -1.0 / 0.0, -1.0 / 0.0, -1.0 / 0.0};
    double motorMaxForce[6] = {1.0 / 0.0, 1.0 / 0.0, 1.0 / 0.0, 1.0 / 0.0, 1.0 / 0.0, 1.0 / 0.0};
    V3 targetVelocity{0, 0, 0}, targetAngularVelocity{0, 0, 0}, targetPosition{0, 0, 0};
    Q4 targetOrientation{0, 0, 0, 1};
    int swingType = SWING_CONE;
    V3 translationAxis[3], rotationAxis[3];
    double displacement[3] = {0, 0, 0};
    int freeAxis = 0, fixedAxis = 0;
    bool translationMotorActive = false, rotationMotorActive = false, hasSpringLimits = false;
    int rotationPositionMotorActive = 0;
    AxisPart translation[3], motorTranslation[3];
    PointPart point;
    SwingTwistPart st;
    EulerPart rot;
    AnglePart motorRotation[3];
};
