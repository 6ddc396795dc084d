// FP64 CPU restatement of crashcat's per-step world update (`updateWorld`,
// src/update.ts:45-239) used as the parity oracle and the timed CPU baseline.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the GPU library links, loads or calls
// this code; only tests/, __graft_entry__.smoke() and bench.py's CPU baseline
// use it.  The restatement covers the bodies, shapes and settings the GPU path
// supports (box and sphere bodies, static / kinematic / dynamic motion,
// discrete motion quality, no user joints, no listener).
//
// Parity notes:
//  * JS numbers are IEEE doubles, so FP64 C++ with -ffp-contract=off
//    reproduces the reference's arithmetic except for sin/cos and the
//    mathcat choices documented in oracle_math.h.
//  * The reference finds pairs with a DBVT; the pair SET it reports depends
//    only on the tight-AABB predicate at the leaves (dbvt.ts:669), so the
//    oracle uses a median-split BVH over the same predicate.  Pair ORDER has no
//    effect on the step's results because the solver sorts each island's
//    contacts by (sortKey, idA, idB) (contact-constraints.ts:1240-1264).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <array>
#include <map>
#include <memory>
#include <numeric>
#include <set>
#include <tuple>
#include <vector>

#include "oracle_frozen.h"
#include "oracle_collide.h"

namespace orc {

enum MotionType : int { STATIC = 0, KINEMATIC = 1, DYNAMIC = 2 };
enum Combine : int { C_AVERAGE = 0, C_MULTIPLY = 1, C_MIN = 2, C_MAX = 3, C_GEOMETRIC_MEAN = 4 };
constexpr int64_t INACTIVE = 9007199254740991LL;  // Number.MAX_SAFE_INTEGER, sleep.ts:8

// WorldSettings defaults, world-settings.ts:224-264
struct Settings {
    V3 gravity{0, -9.81, 0};
    bool gravityEnabled = true;
    double preserveLambdaMaxDistSq = 0.01 * 0.01;
    double collisionTolerance = 1e-4, penetrationTolerance = 1e-4;
    double speculativeContactDistance = 0.02, manifoldTolerance = 1e-3;
    bool useManifoldReduction = true;
    double normalCosMaxDeltaRotation = std::cos((5 * M_PI) / 180);
    double minVelocityForRestitution = 1;
    int velocityIterations = 10, positionIterations = 2;
    bool warmStarting = true;
    double penetrationSlop = 0.02, baumgarteFactor = 0.2, maxPenetrationDistance = 0.2;
    bool allowSleeping = true;
    double timeBeforeSleep = 0.5, pointVelocitySleepThreshold = 0.03;
    // ccd (world-settings.ts:258-262)
    double linearCastThreshold = 0.05, linearCastMaxPenetration = 0.25, ccdMinVelocityForRestitution = 1.0;
};

struct SleepSphere {
    V3 c;
    double r = 0;
};

// RigidBody + MotionProperties (rigid-body.ts:142-252, motion-properties.ts:25-69)
struct Body {
    int index = 0;
    int64_t id = 0;
    Shape shape;
    V3 position, com;
    Q4 quat;
    int motion = DYNAMIC;
    V3 linvel, angvel, force, torque;
    V3 invInertiaDiag;
    Q4 inertiaRot;
    double invMass = 0, linDamp = 0.05, angDamp = 0.05, maxLin = 500, maxAng = 0.25 * M_PI * 60, gravityFactor = 1;
    int dof = 0b111111;
    int velOverride = 0, posOverride = 0;
    SleepSphere spheres[3];
    bool allowSleeping = true;
    double sleepTimer = 0;
    double friction = 0.2, restitution = 0;
    int frictionCombine = C_GEOMETRIC_MEAN, restitutionCombine = C_MAX;
    uint32_t groups = 0xffffffffu, mask = 0xffffffffu;
    bool sensor = false, collideKinematicVsNonDynamic = false, useManifoldReduction = true;
    bool linearCast = false;  // MotionQuality.LINEAR_CAST
    int ccdIndex = -1;        // this step's CCD record, or -1
    bool sleeping = false;
    Box3 aabb;
    int objectLayer = 0;
    int64_t activeIndex = INACTIVE;
    int islandIndex = -1;
};

struct CachedPoint {
    V3 p1, p2;
    double ln = 0, lt1 = 0, lt2 = 0;
};
// Contact (contacts.ts:9-81): persistent record keyed by ids + sub-shape ids
struct Contact {
    int64_t idA, idB;
    uint32_t subA, subB;
    bool processed = false;
    V3 normalB;
    int n = 0;
    CachedPoint pts[4];
};
using ContactKey = std::tuple<int64_t, int64_t, uint32_t, uint32_t>;

// AxisConstraintPart (axis-constraint-part.ts:23-60)
struct AxisPart {
    V3 r1xa, r2xa, invI1, invI2;
    double effMass = 0, totalLambda = 0, softness = 0, bias = 0;
};
struct WorldContactPoint {
    V3 posA, posB, localA, localB;
    AxisPart n, t1, t2;
    int prevPoint = -1;  // cached point whose impulses warm-started this one (-1: none)
};
struct ContactConstraint {
    int bodyA, bodyB;
    uint32_t subA, subB;
    V3 normal, t1, t2;
    double friction, restitution;
    int n = 0;
    WorldContactPoint pts[4];
    double invMassA, invMassB;
    M4 invIA, invIB;
    double invIScaleA = 1, invIScaleB = 1;
    ContactKey contactKey;
    uint32_t sortKey;
    bool hasPrev = false;  // the contact existed in the previous step
};

struct Island {
    std::vector<int64_t> bodyIndices;  // active indices
    std::vector<int> contactIndices;
    std::vector<int> jointIndices;
    int velSteps = 0, posSteps = 0;
};

#include "oracle_joint_types.h"

struct Layers {
    int nObj = 0, nBp = 0;
    std::vector<int> objToBp;
    std::vector<uint8_t> objPairs, objVsBp, bpPairs;
};

struct World {
    Settings s;
    Layers layers;
    std::vector<Body> bodies;
    std::vector<int> activeBodyIndices;
    int64_t activeCount = 0;
    int nextSequence = 0;
    std::map<ContactKey, Contact> contacts;
    // contact events of the last step: (type 1 added / 2 persisted / 3 removed, body index A, body index B)
    // at the listener call sites (contact-constraints.ts:494-499, contacts.ts:305-307)
    std::vector<std::array<int64_t, 3>> events;
    std::vector<HingeJoint> joints;
    std::vector<SwingTwistJoint> swings;
    std::vector<PointJoint> points;
    std::vector<DistanceJoint> distances;
    std::vector<FixedJoint> fixeds;
    std::vector<ConeJoint> cones;
    std::vector<SliderJoint> sliders;
    std::vector<SixDofJoint> sixdofs;
    std::vector<std::unique_ptr<HullData>> hulls;  // convex hull shapes the bodies refer to
    std::vector<std::unique_ptr<MeshData>> meshes;  // triangle meshes the bodies refer to
    std::vector<std::unique_ptr<CompoundData>> compounds;  // compound shapes the bodies refer to
    // skip broadphase pairs of bodies that share an enabled joint: the declarative form of the
    // ragdoll example's onBodyPairValidate (examples/src/example-ragdoll.ts:487-489)
    bool skipJointPairs = false;
    std::vector<ContactConstraint> constraints;
    std::vector<Island> islands;
    double prevDt = 0;
    // diagnostic: solve each island's contacts in greedy-colour order (the order a
    // colour-parallel sweep realises) instead of the reference's sorted order
    bool colouredOrder = false;
    int reorderedIslands = 0;
    // per-step diagnostics
    std::vector<std::pair<int, int>> pairs;
    std::vector<Manifold> manifolds;  // manifolds that produced constraints, after id ordering
    std::vector<std::pair<int, int>> manifoldBodies;
    std::vector<double> manifoldLambda;  // summed normal impulse per manifold after the solve
    double bodySteps = 0;
    // continuous collision: this step's records (ccd.ts:20-57) and the two constraint parts
    // that applyCCD keeps across calls (update.ts:1413-1414): their accumulated lambdas carry
    // from one CCD impulse to the next, within a step and across steps
    struct CCDRecord {
        int body = -1, hit = -1;
        V3 delta, normal, point;
        double fraction = 1, fps = 1, thresholdSq = 0, maxPenetration = 0;
        double friction = 0, restitution = 0;
    };
    std::vector<CCDRecord> ccd;
    double ccdNormalLambda = 0, ccdFrictionLambda = 0;
    int ccdHits = 0;  // records whose cast hit a body, last step
    // the rows of the last step's velocity solve, in the frozen-replay layout of oracle_frozen.h
    // (recorded when recordTape is set)
    bool recordTape = false;
    std::vector<double> tapeBodies, tapeCons, tapeV2;
    double tapeRatio = 0;
};

// ---------------------------------------------------------------------------
// Mass and motion properties
// ---------------------------------------------------------------------------
// setMassAndInertiaOfSolidBox mass-properties.ts:36-52 / sphere.ts:97-123
static void shape_mass(const Shape &s, double &mass, V3 &inertiaDiag) {
    if (s.type == SHAPE_COMPOUND) {  // the tensor goes through set_mass_properties_tensor
        mass = s.compound->mass;
        inertiaDiag = {0, 0, 0};
        return;
    }
    if (s.type == SHAPE_BOX) {
        V3 full = scale(s.half_extents, 2);
        mass = full.x * full.y * full.z * s.density;
        V3 sq{full.x * full.x, full.y * full.y, full.z * full.z};
        inertiaDiag = {(sq.y + sq.z) * (mass / 12.0), (sq.x + sq.z) * (mass / 12.0), (sq.x + sq.y) * (mass / 12.0)};
    } else if (s.type == SHAPE_SPHERE) {
        double r2 = s.radius * s.radius;
        mass = (4.0 / 3.0) * M_PI * s.radius * r2 * s.density;
        double in = (2.0 / 5.0) * mass * r2;
        inertiaDiag = {in, in, in};
    } else if (s.type == SHAPE_CYLINDER) {
        // computeMassProperties cylinder.ts
        mass = M_PI * s.radius * s.radius * 2 * s.half_height * s.density;
        double iyy = 0.5 * mass * s.radius * s.radius;
        double ixx = 0.5 * iyy + (mass * 4 * s.half_height * s.half_height) / 12;
        inertiaDiag = {ixx, iyy, ixx};
    } else if (s.type == SHAPE_CONVEX_HULL) {
        // computeMassProperties convex-hull.ts:453-459: the inertia tensor goes through
        // set_mass_properties_tensor
        mass = s.hull->volume * s.density;
        inertiaDiag = {0, 0, 0};
    } else if (s.type == SHAPE_CAPSULE) {
        // computeMassProperties capsule.ts:119-157 (cylinder plus two hemispheres)
        double r = s.radius, h = s.half_height;
        double volume = M_PI * r * r * (2 * h) + (4.0 / 3.0) * M_PI * r * r * r;
        mass = volume * s.density;
        double r2 = r * r, height = 2.0 * h;
        double cyl = M_PI * height * r2 * s.density;
        double hemi = ((2.0 * M_PI) / 3.0) * r2 * r * s.density;
        double height2 = height * height;
        double iy = r2 * cyl * 0.5;
        double ixz = cyl * ((1.0 / 12.0) * height2 + (1.0 / 4.0) * r2);
        double hxz = hemi * ((2.0 / 5.0) * r2 + h * h + (3.0 / 8.0) * h * r);
        double hy = hemi * (2.0 / 5.0) * r2;
        inertiaDiag = {ixz + hxz, iy + hy, ixz + hxz};
    } else {
        mass = 0;
        inertiaDiag = {0, 0, 0};
    }
}

// setMassProperties motion-properties.ts:419-491 for a diagonal inertia tensor
// (the Jacobi decomposition exits immediately with an identity rotation when
// all off-diagonal terms are zero, motion-properties.ts:232-245).
static void set_mass_properties(Body &b, double mass, V3 d) {
    int tr = b.dof & 0b111, rot = (b.dof >> 3) & 0b111;
    b.invMass = tr == 0 ? 0.0 : 1.0 / mass;
    if (rot == 0) {
        b.invInertiaDiag = {0, 0, 0};
        b.inertiaRot = {0, 0, 0, 1};
    } else {
        double l = d.x * d.x + d.y * d.y + d.z * d.z;
        const double EPS = 1e-10;  // EPSILON, motion-properties.ts:178
        if (l > EPS * EPS) {
            b.invInertiaDiag = {d.x != 0 ? 1.0 / d.x : 0, d.y != 0 ? 1.0 / d.y : 0, d.z != 0 ? 1.0 / d.z : 0};
            b.inertiaRot = {0, 0, 0, 1};
        } else {
            double si = 2.5 * b.invMass;
            b.invInertiaDiag = {si, si, si};
            b.inertiaRot = {0, 0, 0, 1};
        }
    }
}

inline Q4 quat_from_m3(const M3 &m);  // quat.fromMat3, oracle_joints.h

// setMassProperties for a full inertia tensor (motion-properties.ts:419-491): the principal
// moments and axes by cyclic Jacobi rotations (decomposePrincipalMomentsOfInertia
// mass-properties.ts:181-300 diagonalises the same symmetric matrix); the world inverse inertia
// R diag(1/d) R^T does not depend on the order or signs the decomposition picks.
static void set_mass_properties_tensor(Body &b, double mass, const double *unit_inertia, double density) {
    double a[3][3], v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) a[r][c] = unit_inertia[3 * r + c] * density;
    for (int sweep = 0; sweep < 50; sweep++) {
        if (std::fabs(a[0][1]) + std::fabs(a[0][2]) + std::fabs(a[1][2]) < 1e-300) break;
        for (int p = 0; p < 2; p++)
            for (int q = p + 1; q < 3; q++) {
                if (a[p][q] == 0) continue;
                double th = (a[q][q] - a[p][p]) / (2 * a[p][q]);
                double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1));
                double c = 1 / std::sqrt(t * t + 1), sn = t * c;
                for (int k = 0; k < 3; k++) {
                    double x = a[k][p], y = a[k][q];
                    a[k][p] = c * x - sn * y;
                    a[k][q] = sn * x + c * y;
                }
                for (int k = 0; k < 3; k++) {
                    double x = a[p][k], y = a[q][k];
                    a[p][k] = c * x - sn * y;
                    a[q][k] = sn * x + c * y;
                }
                for (int k = 0; k < 3; k++) {
                    double x = v[k][p], y = v[k][q];
                    v[k][p] = c * x - sn * y;
                    v[k][q] = sn * x + c * y;
                }
            }
    }
    double det = v[0][0] * (v[1][1] * v[2][2] - v[1][2] * v[2][1]) - v[0][1] * (v[1][0] * v[2][2] - v[1][2] * v[2][0]) +
                 v[0][2] * (v[1][0] * v[2][1] - v[1][1] * v[2][0]);
    if (det < 0)
        for (int k = 0; k < 3; k++) v[k][2] = -v[k][2];
    set_mass_properties(b, mass, V3{a[0][0], a[1][1], a[2][2]});
    int rot = (b.dof >> 3) & 0b111;
    if (rot != 0) {
        M3 m;  // columns = principal axes
        for (int c = 0; c < 3; c++)
            for (int r = 0; r < 3; r++) m.m[c][r] = v[r][c];
        b.inertiaRot = quat_from_m3(m);
    }
}

// getInverseInertiaForRotation motion-properties.ts:494-621
static M4 inv_inertia_for_rotation(const Body &b, const M4 &R) {
    Q4 q = b.inertiaRot;
    double qx2 = q.x + q.x, qy2 = q.y + q.y, qz2 = q.z + q.z;
    double qxx = q.x * qx2, qyx = q.y * qx2, qyy = q.y * qy2, qzx = q.z * qx2, qzy = q.z * qy2, qzz = q.z * qz2,
           qwx = q.w * qx2, qwy = q.w * qy2, qwz = q.w * qz2;
    double i00 = 1 - qyy - qzz, i01 = qyx + qwz, i02 = qzx - qwy;
    double i10 = qyx - qwz, i11 = 1 - qxx - qzz, i12 = qzy + qwx;
    double i20 = qzx + qwy, i21 = qzy - qwx, i22 = 1 - qxx - qyy;
    const double *m = R.m;
    double b00 = m[0], b01 = m[1], b02 = m[2], b10 = m[4], b11 = m[5], b12 = m[6], b20 = m[8], b21 = m[9],
           b22 = m[10];
    double r00 = b00 * i00 + b10 * i01 + b20 * i02, r01 = b01 * i00 + b11 * i01 + b21 * i02,
           r02 = b02 * i00 + b12 * i01 + b22 * i02;
    double r10 = b00 * i10 + b10 * i11 + b20 * i12, r11 = b01 * i10 + b11 * i11 + b21 * i12,
           r12 = b02 * i10 + b12 * i11 + b22 * i12;
    double r20 = b00 * i20 + b10 * i21 + b20 * i22, r21 = b01 * i20 + b11 * i21 + b21 * i22,
           r22 = b02 * i20 + b12 * i21 + b22 * i22;
    double d0 = b.invInertiaDiag.x, d1 = b.invInertiaDiag.y, d2 = b.invInertiaDiag.z;
    double s00 = d0 * r00, s01 = d0 * r01, s02 = d0 * r02, s10 = d1 * r10, s11 = d1 * r11, s12 = d1 * r12,
           s20 = d2 * r20, s21 = d2 * r21, s22 = d2 * r22;
    M4 o{};
    o.m[0] = s00 * r00 + s10 * r10 + s20 * r20;
    o.m[1] = s00 * r01 + s10 * r11 + s20 * r21;
    o.m[2] = s00 * r02 + s10 * r12 + s20 * r22;
    o.m[4] = s01 * r00 + s11 * r10 + s21 * r20;
    o.m[5] = s01 * r01 + s11 * r11 + s21 * r21;
    o.m[6] = s01 * r02 + s11 * r12 + s21 * r22;
    o.m[8] = s02 * r00 + s12 * r10 + s22 * r20;
    o.m[9] = s02 * r01 + s12 * r11 + s22 * r21;
    o.m[10] = s02 * r02 + s12 * r12 + s22 * r22;
    o.m[15] = 1;
    int ar = (b.dof >> 3) & 0b111;
    if (ar != 0b111) {
        double mx = ar & 1 ? 1.0 : 0.0, my = ar & 2 ? 1.0 : 0.0, mz = ar & 4 ? 1.0 : 0.0;
        o.m[0] *= mx * mx;
        o.m[1] *= my * mx;
        o.m[2] *= mz * mx;
        o.m[4] *= mx * my;
        o.m[5] *= my * my;
        o.m[6] *= mz * my;
        o.m[8] *= mx * mz;
        o.m[9] *= my * mz;
        o.m[10] *= mz * mz;
    }
    return o;
}

// ---------------------------------------------------------------------------
// Transform / AABB / sleep helpers
// ---------------------------------------------------------------------------
// updateCenterOfMassPosition rigid-body.ts:527-536
static void update_com(Body &b) { b.com = add(rotate(b.quat, b.shape.com), b.position); }
// updatePositionFromCenterOfMass rigid-body.ts:545-553
static void update_pos_from_com(Body &b) { b.position = sub(b.com, rotate(b.quat, b.shape.com)); }
// updateAABB rigid-body.ts:561-674
static void update_aabb(Body &b) {
    const Box3 &s = b.shape.aabb;
    M4 R = mat4_from_quat(b.quat);
    const double *m = R.m;
    double xs[2] = {s.mn.x, s.mx.x}, ys[2] = {s.mn.y, s.mx.y}, zs[2] = {s.mn.z, s.mx.z};
    // corner order: (min,min,min) (max,min,min) (min,max,min) (max,max,min) ...
    double mnx = 0, mny = 0, mnz = 0, mxx = 0, mxy = 0, mxz = 0;
    for (int c = 0; c < 8; c++) {
        double x = xs[c & 1], y = ys[(c >> 1) & 1], z = zs[(c >> 2) & 1];
        double wx = m[0] * x + m[4] * y + m[8] * z + b.position.x;
        double wy = m[1] * x + m[5] * y + m[9] * z + b.position.y;
        double wz = m[2] * x + m[6] * y + m[10] * z + b.position.z;
        if (c == 0) {
            mnx = mxx = wx;
            mny = mxy = wy;
            mnz = mxz = wz;
        } else {
            mnx = std::min(mnx, wx);
            mny = std::min(mny, wy);
            mnz = std::min(mnz, wz);
            mxx = std::max(mxx, wx);
            mxy = std::max(mxy, wy);
            mxz = std::max(mxz, wz);
        }
    }
    b.aabb = {{mnx, mny, mnz}, {mxx, mxy, mxz}};
}
static void set_transform(Body &b) {
    update_com(b);
    update_aabb(b);
}

// getSleepTestPoints sleep.ts:22-74
static void sleep_points(const Body &b, V3 out[3]) {
    out[0] = b.com;
    const Box3 &a = b.shape.aabb;
    V3 e{(a.mx.x - a.mn.x) * 0.5, (a.mx.y - a.mn.y) * 0.5, (a.mx.z - a.mn.z) * 0.5};
    int lowest;
    if (e.x <= e.y && e.x <= e.z)
        lowest = 0;
    else if (e.y <= e.z)
        lowest = 1;
    else
        lowest = 2;
    V3 X{1, 0, 0}, Y{0, 1, 0}, Z{0, 0, 1};
    if (lowest == 0) {
        out[1] = scale_add(b.com, rotate(b.quat, Y), e.y);
        out[2] = scale_add(b.com, rotate(b.quat, Z), e.z);
    } else if (lowest == 1) {
        out[1] = scale_add(b.com, rotate(b.quat, X), e.x);
        out[2] = scale_add(b.com, rotate(b.quat, Z), e.z);
    } else {
        out[1] = scale_add(b.com, rotate(b.quat, X), e.x);
        out[2] = scale_add(b.com, rotate(b.quat, Y), e.y);
    }
}
static void reset_sleep_spheres(Body &b, V3 p[3]) {
    for (int i = 0; i < 3; i++) {
        b.spheres[i].c = p[i];
        b.spheres[i].r = 0;
    }
    b.sleepTimer = 0;
}
// resetSleepTimer sleep.ts:123-130
static void reset_sleep_timer(Body &b) {
    if (b.motion != DYNAMIC) return;
    V3 p[3];
    sleep_points(b, p);
    reset_sleep_spheres(b, p);
}
// updateSleepState sleep.ts:88-117
static bool update_sleep_state(Body &b, double dt, double maxMove, double tbs) {
    if (!b.allowSleeping || b.sensor) return false;
    V3 p[3];
    sleep_points(b, p);
    for (int i = 0; i < 3; i++) {
        SleepSphere &s = b.spheres[i];
        double d = distance(s.c, p[i]);
        s.r = std::max(s.r, d);
        if (s.r > maxMove) {
            reset_sleep_spheres(b, p);
            return false;
        }
    }
    b.sleepTimer += dt;
    return b.sleepTimer >= tbs;
}
// addBodyToActiveBodies / removeBodyFromActiveBodies sleep.ts:132-166
static void add_active(World &w, Body &b) {
    if (b.activeIndex != INACTIVE) return;
    b.activeIndex = w.activeCount;
    if ((int64_t)w.activeBodyIndices.size() <= w.activeCount) w.activeBodyIndices.resize(w.activeCount + 1);
    w.activeBodyIndices[w.activeCount] = b.index;
    w.activeCount++;
}
static void remove_active(World &w, Body &b) {
    if (b.activeIndex == INACTIVE) return;
    int64_t last = w.activeCount - 1;
    if (b.activeIndex != last) {
        int lastBody = w.activeBodyIndices[last];
        w.activeBodyIndices[b.activeIndex] = lastBody;
        w.bodies[lastBody].activeIndex = b.activeIndex;
    }
    b.activeIndex = INACTIVE;
    w.activeCount--;
}
// sleep / wake sleep.ts:169-203
static void sleep_body(World &w, Body &b) {
    if (b.motion == STATIC || b.sleeping) return;
    remove_active(w, b);
    b.sleeping = true;
    b.linvel = {0, 0, 0};
    b.angvel = {0, 0, 0};
}
static void wake_body(World &w, Body &b) {
    if (b.motion == STATIC) return;
    reset_sleep_timer(b);
    if (!b.sleeping) return;
    b.sleeping = false;
    add_active(w, b);
}

// ---------------------------------------------------------------------------
// Broadphase (broadphase.ts:44-277)
// ---------------------------------------------------------------------------
static bool should_query(const Body &b) { return b.motion != STATIC && !b.sleeping; }
static int64_t dedup_index(const Body &b) { return should_query(b) ? (int64_t)b.index : INACTIVE; }

struct BvhNode {
    Box3 box;
    int left = -1, right = -1, first = 0, count = 0;
};
static void bvh_build(const std::vector<Body> &bodies, std::vector<int> &idx, std::vector<BvhNode> &nodes, int first,
                      int count) {
    int ni = (int)nodes.size();
    nodes.emplace_back();
    Box3 bx = bodies[idx[first]].aabb;
    for (int i = first + 1; i < first + count; i++) {
        const Box3 &a = bodies[idx[i]].aabb;
        bx.mn = {std::min(bx.mn.x, a.mn.x), std::min(bx.mn.y, a.mn.y), std::min(bx.mn.z, a.mn.z)};
        bx.mx = {std::max(bx.mx.x, a.mx.x), std::max(bx.mx.y, a.mx.y), std::max(bx.mx.z, a.mx.z)};
    }
    nodes[ni].box = bx;
    if (count <= 4) {
        nodes[ni].first = first;
        nodes[ni].count = count;
        return;
    }
    V3 ext = sub(bx.mx, bx.mn);
    int axis = (ext.x >= ext.y && ext.x >= ext.z) ? 0 : (ext.y >= ext.z ? 1 : 2);
    auto key = [&](int i) {
        const Box3 &a = bodies[i].aabb;
        return axis == 0 ? a.mn.x + a.mx.x : (axis == 1 ? a.mn.y + a.mx.y : a.mn.z + a.mx.z);
    };
    int mid = first + count / 2;
    std::nth_element(idx.begin() + first, idx.begin() + mid, idx.begin() + first + count,
                     [&](int a, int b) { return key(a) < key(b) || (key(a) == key(b) && a < b); });
    int l = (int)nodes.size();
    bvh_build(bodies, idx, nodes, first, mid - first);
    int r = (int)nodes.size();
    bvh_build(bodies, idx, nodes, mid, first + count - mid);
    nodes[ni].left = l;
    nodes[ni].right = r;
}

// User joints of every type under one id, as the reference's ConstraintId packs them
// (constraint-id.ts:1-35): the ConstraintType above bit 24, the per-type index below.
// joint_ids lists them type by type, each in creation order, the order in which the
// reference walks its constraint pools (constraints.ts:264-318, islands.ts:210-225).
enum JointType {
    JT_POINT = 0, JT_DISTANCE = 1, JT_HINGE = 2, JT_SLIDER = 3, JT_FIXED = 4, JT_CONE = 5, JT_SWING = 6, JT_SIX_DOF = 7
};
constexpr int JOINT_TYPE_SHIFT = 24, JOINT_INDEX_MASK = (1 << JOINT_TYPE_SHIFT) - 1;
inline int joint_type(int id) { return id >> JOINT_TYPE_SHIFT; }
inline int joint_index(int id) { return id & JOINT_INDEX_MASK; }
struct JointInfo {
    int a, b, priority, index, type;
    bool enabled;
    int velOverride, posOverride;
};
static const JointBase &joint_base(const World &w, int id) {
    int i = joint_index(id);
    switch (joint_type(id)) {
    case JT_POINT: return w.points[i];
    case JT_DISTANCE: return w.distances[i];
    case JT_SLIDER: return w.sliders[i];
    case JT_FIXED: return w.fixeds[i];
    case JT_CONE: return w.cones[i];
    case JT_SIX_DOF: return w.sixdofs[i];
    default: break;
    }
    static const JointBase none;
    return none;
}
static std::vector<int> joint_ids(const World &w) {
    std::vector<int> ids;
    size_t count[8] = {w.points.size(), w.distances.size(), w.joints.size(), w.sliders.size(),
                       w.fixeds.size(),  w.cones.size(),     w.swings.size(), w.sixdofs.size()};
    for (int t = 0; t < 8; t++)
        for (size_t i = 0; i < count[t]; i++) ids.push_back((t << JOINT_TYPE_SHIFT) | (int)i);
    return ids;
}
static JointInfo joint_info(const World &w, int id) {
    int t = joint_type(id), i = joint_index(id);
    if (t == JT_SWING) {
        const SwingTwistJoint &j = w.swings[i];
        return {j.a, j.b, j.priority, j.index, t, j.enabled, j.velOverride, j.posOverride};
    }
    if (t == JT_HINGE) {
        const HingeJoint &j = w.joints[i];
        return {j.a, j.b, j.priority, j.index, t, j.enabled, j.velOverride, j.posOverride};
    }
    const JointBase &j = joint_base(w, id);
    return {j.a, j.b, j.priority, j.index, t, j.enabled, j.velOverride, j.posOverride};
}

static void find_colliding_pairs(World &w) {
    w.pairs.clear();
    std::set<std::pair<int, int>> joined;  // body pairs that share an enabled joint
    if (w.skipJointPairs)
        for (int id : joint_ids(w)) {
            JointInfo ji = joint_info(w, id);
            if (ji.enabled) joined.insert({std::min(ji.a, ji.b), std::max(ji.a, ji.b)});
        }
    std::vector<int> idx(w.bodies.size());
    std::iota(idx.begin(), idx.end(), 0);
    std::vector<BvhNode> nodes;
    if (!idx.empty()) bvh_build(w.bodies, idx, nodes, 0, (int)idx.size());
    // bodies sorted (stably) by broadphase layer, broadphase.ts:235-239
    std::vector<int> order(w.bodies.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return w.layers.objToBp[w.bodies[a].objectLayer] < w.layers.objToBp[w.bodies[b].objectLayer];
    });
    std::vector<int> cand;
    std::vector<int> stack;
    for (int qi : order) {
        Body &A = w.bodies[qi];
        if (!should_query(A)) continue;
        Box3 E = box_expand(A.aabb, w.s.speculativeContactDistance);
        int la = A.objectLayer, bpa = w.layers.objToBp[la];
        cand.clear();
        stack.clear();
        stack.push_back(0);
        while (!stack.empty()) {
            int n = stack.back();
            stack.pop_back();
            if (!box_overlap(nodes[n].box, E)) continue;
            if (nodes[n].left >= 0) {
                stack.push_back(nodes[n].left);
                stack.push_back(nodes[n].right);
                continue;
            }
            for (int k = 0; k < nodes[n].count; k++) cand.push_back(idx[nodes[n].first + k]);
        }
        std::sort(cand.begin(), cand.end());
        for (int bi : cand) {
            Body &B = w.bodies[bi];
            int lb = B.objectLayer, bpb = w.layers.objToBp[lb];
            // layer gating of the per-layer tree query (broadphase.ts:252-272)
            if (!w.layers.objVsBp[la * w.layers.nBp + bpb]) continue;
            if (!w.layers.bpPairs[bpa * w.layers.nBp + bpb]) continue;
            // dbvt.intersectAABB leaf filters (dbvt.ts:645-670)
            if (!((A.groups & B.mask) != 0 && (B.groups & A.mask) != 0)) continue;
            if (!w.layers.objPairs[la * w.layers.nObj + lb]) continue;
            if (!box_overlap(B.aabb, E)) continue;
            // CollisionBodyPairVisitor.visit broadphase.ts:83-138
            if (A.id == B.id) continue;
            if (dedup_index(A) >= dedup_index(B)) continue;
            if (A.motion == STATIC && B.motion == STATIC) continue;
            if (!A.collideKinematicVsNonDynamic && !B.collideKinematicVsNonDynamic && A.motion != DYNAMIC &&
                B.motion != DYNAMIC && !(A.motion == KINEMATIC && B.sensor) && !(B.motion == KINEMATIC && A.sensor))
                continue;
            // onBodyPairValidate (broadphase.ts:112-123) as the declarative joint-pair filter
            if (w.skipJointPairs && joined.count({std::min(A.index, B.index), std::max(A.index, B.index)})) continue;
            w.pairs.push_back({A.index, B.index});
        }
    }
}

// ---------------------------------------------------------------------------
// Contact constraints (contact-constraints.ts)
// ---------------------------------------------------------------------------
static double combine(double a, double b, int ma, int mb) {  // combine-material.ts:40-57
    static const int prio[5] = {0, 1, 3, 4, 2};                // AVERAGE, MULTIPLY, MIN, MAX, GEOMETRIC_MEAN
    int mode = prio[ma] >= prio[mb] ? ma : mb;
    switch (mode) {
        case C_MULTIPLY:
            return a * b;
        case C_MIN:
            return std::min(a, b);
        case C_MAX:
            return std::max(a, b);
        case C_GEOMETRIC_MEAN:
            return std::sqrt(a * b);
        default:
            return (a + b) / 2;
    }
}

// calculateInverseEffectiveMass axis-constraint-part.ts:86-148.  For a
// non-dynamic body the cross terms are zeroed (the reference leaves stale
// values there, which only kinematic bodies ever read).
static double inv_eff_mass(AxisPart &p, const Body &A, const Body &B, double imA, double imB, const M4 &IA,
                           const M4 &IB, V3 r1, V3 r2, V3 ax) {
    double iem = 0;
    p.r1xa = p.r2xa = p.invI1 = p.invI2 = {0, 0, 0};
    if (A.motion == DYNAMIC) {
        p.r1xa = {r1.y * ax.z - r1.z * ax.y, r1.z * ax.x - r1.x * ax.z, r1.x * ax.y - r1.y * ax.x};
        V3 c = p.r1xa;
        p.invI1 = {IA.m[0] * c.x + IA.m[4] * c.y + IA.m[8] * c.z, IA.m[1] * c.x + IA.m[5] * c.y + IA.m[9] * c.z,
                   IA.m[2] * c.x + IA.m[6] * c.y + IA.m[10] * c.z};
        iem += imA + (p.invI1.x * c.x + p.invI1.y * c.y + p.invI1.z * c.z);
    }
    if (B.motion == DYNAMIC) {
        p.r2xa = {r2.y * ax.z - r2.z * ax.y, r2.z * ax.x - r2.x * ax.z, r2.x * ax.y - r2.y * ax.x};
        V3 c = p.r2xa;
        p.invI2 = {IB.m[0] * c.x + IB.m[4] * c.y + IB.m[8] * c.z, IB.m[1] * c.x + IB.m[5] * c.y + IB.m[9] * c.z,
                   IB.m[2] * c.x + IB.m[6] * c.y + IB.m[10] * c.z};
        iem += imB + (p.invI2.x * c.x + p.invI2.y * c.y + p.invI2.z * c.z);
    }
    return iem;
}
// calculateConstraintProperties axis-constraint-part.ts:165-200
static void calc_props(AxisPart &p, const Body &A, const Body &B, double imA, double imB, const M4 &IA, const M4 &IB,
                       V3 r1, V3 r2, V3 ax, double bias) {
    double iem = inv_eff_mass(p, A, B, imA, imB, IA, IB, r1, r2, ax);
    if (iem == 0) {
        p.effMass = 0;
        p.totalLambda = 0;
    } else {
        p.effMass = 1 / iem;
        p.softness = 0;
        p.bias = bias;
    }
}
static bool part_active(const AxisPart &p) { return p.effMass != 0; }

// calculateNormalVelocityBias contact-constraints.ts:288-423
static double normal_velocity_bias(const Body &A, const Body &B, V3 pA, V3 pB, V3 n, V3 rA, V3 rB, double e,
                                   double dt, V3 g, double minVel) {
    bool aM = A.motion != STATIC, bM = B.motion != STATIC, aD = A.motion == DYNAMIC, bD = B.motion == DYNAMIC;
    auto vel_at = [](const Body &b, V3 r) {
        return V3{b.linvel.x + (b.angvel.y * r.z - b.angvel.z * r.y), b.linvel.y + (b.angvel.z * r.x - b.angvel.x * r.z),
                  b.linvel.z + (b.angvel.x * r.y - b.angvel.y * r.x)};
    };
    V3 rv;
    if (aM && bM) {
        V3 v1 = vel_at(A, rA), v2 = vel_at(B, rB);
        rv = sub(v2, v1);
    } else if (aM) {
        rv = neg(vel_at(A, rA));
    } else if (bM) {
        rv = vel_at(B, rB);
    } else {
        return 0;
    }
    double nv = rv.x * n.x + rv.y * n.y + rv.z * n.z;
    V3 d = sub(pA, pB);
    double pen = d.x * n.x + d.y * n.y + d.z * n.z;
    double spec = std::max(0.0, -pen / dt);
    if (e > 0 && nv < -minVel) {
        if (nv < -spec) {
            double rx = 0, ry = 0, rz = 0;
            if (aM && bM) {
                double gs = B.gravityFactor - A.gravityFactor;
                rx += g.x * gs;
                ry += g.y * gs;
                rz += g.z * gs;
            } else if (aM) {
                rx += g.x * -A.gravityFactor;
                ry += g.y * -A.gravityFactor;
                rz += g.z * -A.gravityFactor;
            } else if (bM) {
                rx += g.x * B.gravityFactor;
                ry += g.y * B.gravityFactor;
                rz += g.z * B.gravityFactor;
            }
            if (aD) {
                double fs = -A.invMass;
                rx += A.force.x * fs;
                ry += A.force.y * fs;
                rz += A.force.z * fs;
            }
            if (bD) {
                double fs = B.invMass;
                rx += B.force.x * fs;
                ry += B.force.y * fs;
                rz += B.force.z * fs;
            }
            double adn = rx * n.x + ry * n.y + rz * n.z;
            double fdv = std::min(0.0, adn * dt);
            return e * (nv - fdv);
        }
        return spec;
    }
    return spec;
}

// computeContactSortKey contact-constraints.ts:1222-1231
static uint32_t sort_key(int a, int b, uint32_t sa, uint32_t sb) {
    int32_t h = 0;
    auto step = [](int32_t h, int64_t v) { return (int32_t)(uint32_t)((int64_t)h * 31 + v); };
    h = step(h, a);
    h = step(h, b);
    h = step(h, (int32_t)sa);
    h = step(h, (int32_t)sb);
    return (uint32_t)h;
}

// addContactConstraint contact-constraints.ts:437-857 (no listener)
static bool add_contact_constraint(World &w, Body *A, Body *B, Manifold m, double dt) {
    if (A->id > B->id) {
        std::swap(A, B);
        // swapShapes manifold.ts:86-105
        m.normal = neg(m.normal);
        std::swap(m.subA, m.subB);
        for (int i = 0; i < m.n; i++) std::swap(m.relA[i], m.relB[i]);
    }
    ContactKey key{A->id, B->id, m.subA, m.subB};
    auto it = w.contacts.find(key);
    bool existing = it != w.contacts.end();
    w.events.push_back({existing ? 2 : 1, A->id & 0xffffffffLL, B->id & 0xffffffffLL});
    Contact prev;
    if (existing) prev = it->second;
    Contact &c = w.contacts[key];
    if (!existing) {
        c.idA = A->id;
        c.idB = B->id;
        c.subA = m.subA;
        c.subB = m.subB;
    }
    c.processed = true;
    M4 rotA = mat4_from_quat(A->quat), rotB = mat4_from_quat(B->quat);
    V3 nw = m.normal;
    c.normalB = normalize(V3{rotB.m[0] * nw.x + rotB.m[1] * nw.y + rotB.m[2] * nw.z,
                             rotB.m[4] * nw.x + rotB.m[5] * nw.y + rotB.m[6] * nw.z,
                             rotB.m[8] * nw.x + rotB.m[9] * nw.y + rotB.m[10] * nw.z});
    c.n = m.n;
    double friction = combine(A->friction, B->friction, A->frictionCombine, B->frictionCombine);
    double restitution = combine(A->restitution, B->restitution, A->restitutionCombine, B->restitutionCombine);
    bool isSensor = A->sensor || B->sensor;
    if (!isSensor && ((A->motion == DYNAMIC && A->invMass != 0) || (B->motion == DYNAMIC && B->invMass != 0))) {
        w.constraints.emplace_back();
        ContactConstraint &cc = w.constraints.back();
        cc.bodyA = A->index;
        cc.bodyB = B->index;
        cc.subA = m.subA;
        cc.subB = m.subB;
        cc.contactKey = key;
        cc.sortKey = sort_key(A->index, B->index, m.subA, m.subB);
        cc.hasPrev = existing;
        cc.normal = m.normal;
        double nx = cc.normal.x, ny = cc.normal.y, nz = cc.normal.z;
        if (std::fabs(nx) > std::fabs(ny)) {
            double tl = std::sqrt(nx * nx + nz * nz);
            cc.t1 = {nz / tl, 0, -nx / tl};
        } else {
            double tl = std::sqrt(ny * ny + nz * nz);
            cc.t1 = {0, nz / tl, -ny / tl};
        }
        cc.t2 = {ny * cc.t1.z - nz * cc.t1.y, nz * cc.t1.x - nx * cc.t1.z, nx * cc.t1.y - ny * cc.t1.x};
        cc.friction = friction;
        cc.restitution = restitution;
        cc.invMassA = A->invMass * 1.0;
        cc.invMassB = B->invMass * 1.0;
        cc.invIScaleA = 1;
        cc.invIScaleB = 1;
        std::memset(&cc.invIA, 0, sizeof(M4));
        std::memset(&cc.invIB, 0, sizeof(M4));
        if (A->motion == DYNAMIC) cc.invIA = inv_inertia_for_rotation(*A, rotA);
        if (B->motion == DYNAMIC) cc.invIB = inv_inertia_for_rotation(*B, rotB);
        cc.n = 0;
        for (int i = 0; i < m.n; i++) {
            WorldContactPoint &cp = cc.pts[cc.n];
            cc.n++;
            cp.posA = add(m.base, m.relA[i]);
            cp.posB = add(m.base, m.relB[i]);
            V3 la = sub(cp.posA, A->com), lb = sub(cp.posB, B->com);
            cp.localA = m3tmul(rotA, la);
            cp.localB = m3tmul(rotB, lb);
            bool set = false;
            if (existing) {
                for (int j = 0; j < prev.n; j++) {
                    const CachedPoint &p = prev.pts[j];
                    V3 d1 = sub(cp.localA, p.p1), d2 = sub(cp.localB, p.p2);
                    double s1 = d1.x * d1.x + d1.y * d1.y + d1.z * d1.z;
                    double s2 = d2.x * d2.x + d2.y * d2.y + d2.z * d2.z;
                    double th = w.s.preserveLambdaMaxDistSq;
                    if (s1 < th && s2 < th) {
                        cp.n.totalLambda = p.ln;
                        cp.t1.totalLambda = p.lt1;
                        cp.t2.totalLambda = p.lt2;
                        cp.prevPoint = j;
                        set = true;
                        break;
                    }
                }
            }
            if (!set) {
                cp.n.totalLambda = 0;
                cp.t1.totalLambda = 0;
                cp.t2.totalLambda = 0;
            }
            V3 mid{(cp.posA.x + cp.posB.x) * 0.5, (cp.posA.y + cp.posB.y) * 0.5, (cp.posA.z + cp.posB.z) * 0.5};
            V3 rA = sub(mid, A->com), rB = sub(mid, B->com);
            double nb = normal_velocity_bias(*A, *B, cp.posA, cp.posB, cc.normal, rA, rB, restitution, dt, w.s.gravity,
                                             w.s.minVelocityForRestitution);
            calc_props(cp.n, *A, *B, cc.invMassA, cc.invMassB, cc.invIA, cc.invIB, rA, rB, cc.normal, nb);
            if (friction > 0) {
                // zero surface velocity: calculateFrictionBias contact-constraints.ts:252-266 returns 0
                calc_props(cp.t1, *A, *B, cc.invMassA, cc.invMassB, cc.invIA, cc.invIB, rA, rB, cc.t1, 0.0);
                calc_props(cp.t2, *A, *B, cc.invMassA, cc.invMassB, cc.invIA, cc.invIB, rA, rB, cc.t2, 0.0);
            } else {
                cp.t1.effMass = 0;
                cp.t1.totalLambda = 0;
                cp.t2.effMass = 0;
                cp.t2.totalLambda = 0;
            }
            CachedPoint &cpt = c.pts[i];
            cpt.p1 = cp.localA;
            cpt.p2 = cp.localB;
            cpt.ln = cp.n.totalLambda;
            cpt.lt1 = cp.t1.totalLambda;
            cpt.lt2 = cp.t2.totalLambda;
        }
        w.manifolds.push_back(m);
        w.manifoldBodies.push_back({A->index, B->index});
        return true;
    }
    for (int i = 0; i < m.n; i++) {
        V3 pa = add(m.base, m.relA[i]), pb = add(m.base, m.relB[i]);
        V3 la = sub(pa, A->com), lb = sub(pb, B->com);
        c.pts[i].p1 = m3tmul(rotA, la);
        c.pts[i].p2 = m3tmul(rotB, lb);
        c.pts[i].ln = c.pts[i].lt1 = c.pts[i].lt2 = 0;
    }
    return false;
}

// narrowphase update.ts:714-850 with the reduction collector update.ts:333-563
static bool narrowphase(World &w, Body *A, Body *B, double dt) {
    CollideSettings cs;
    cs.collectFaces = true;
    cs.collisionTolerance = w.s.collisionTolerance;
    cs.penetrationTolerance = w.s.penetrationTolerance;
    cs.maxSeparation = (A->sensor || B->sensor) ? 0 : w.s.speculativeContactDistance;
    // activeEdgeMovementDirection update.ts:729-733
    V3 movement = sub(A->linvel, B->linvel);
    std::vector<Hit> hits;
    V3 gpA, gpB;
    Q4 gqA, gqB;
    geometry_pose(A->shape, A->position, A->quat, gpA, gqA);
    geometry_pose(B->shape, B->position, B->quat, gpB, gqB);
    collide_hits(hits, cs, A->shape, gpA, gqA, B->shape, gpB, gqB, movement);
    // narrowphaseWithReductionCollector.addHit update.ts:385-519: hits whose normal is within
    // normalCosMaxDeltaRotation of a manifold's accumulated normal join it, at most 32 manifolds
    const double maxContactDistance = w.s.speculativeContactDistance + w.s.manifoldTolerance;
    std::vector<Manifold> ms;
    for (const Hit &hit : hits) {
        V3 n = normalize(hit.axis);
        int found = -1;
        for (size_t i = 0; i < ms.size(); i++)
            if (dot(n, ms[i].normal) >= w.s.normalCosMaxDeltaRotation) {
                found = (int)i;
                break;
            }
        if (found < 0) {
            if (ms.size() >= 32) {
                int sh = 0;
                for (int i = 1; i < (int)ms.size(); i++)
                    if (ms[i].depth < ms[sh].depth) sh = i;
                if (hit.penetration < ms[sh].depth) continue;
                found = sh;
            } else {
                ms.emplace_back();
                found = (int)ms.size() - 1;
            }
            Manifold &m = ms[found];
            m = Manifold();
            m.base = A->position;
            m.normal = n;
            m.depth = hit.penetration;
            m.subA = hit.subA;
            m.subB = hit.subB;
        } else {
            ms[found].normal = add(ms[found].normal, n);
        }
        Manifold &m = ms[found];
        Manifold tmp;
        tmp.base = A->position;
        if (hit.faceA.n >= 2 && hit.faceB.n >= 3) {
            manifold_between_faces(tmp, hit.pa, hit.pb, hit.axis, maxContactDistance, hit.faceA, hit.faceB);
        } else {
            set_contact_point(tmp, 0, hit.pa, hit.pb);
            tmp.n = 1;
        }
        for (int i = 0; i < tmp.n; i++) {
            if (m.n >= 64) break;
            m.relA[m.n] = tmp.relA[i];
            m.relB[m.n] = tmp.relB[i];
            m.n++;
        }
        if (hit.penetration > m.depth) m.depth = hit.penetration;
        if (m.n > 32) prune_contact_points(m, m.normal);
    }
    // finalizeAndCreateConstraints update.ts:525-558
    bool created = false;
    for (Manifold &m : ms) {
        m.normal = normalize(m.normal);
        if (m.n > 4) prune_contact_points(m, m.normal);
        if (m.n > 0) created = add_contact_constraint(w, A, B, m, dt) || created;
    }
    return created;
}

// ---------------------------------------------------------------------------
// Solver (contact-constraints.ts:906-1216, axis-constraint-part.ts:500-847)
// ---------------------------------------------------------------------------
static void apply_dof_lin(Body &b) {
    int t = b.dof & 0b111;
    if (!(t & 1)) b.linvel.x = 0;
    if (!(t & 2)) b.linvel.y = 0;
    if (!(t & 4)) b.linvel.z = 0;
}
static void warm_start(AxisPart &p, Body &A, Body &B, double imA, double imB, V3 ax, double ratio) {
    p.totalLambda *= ratio;
    if (p.totalLambda == 0) return;
    if (A.motion == DYNAMIC) {
        V3 imp = scale(ax, p.totalLambda * imA);
        A.linvel = sub(A.linvel, imp);
        apply_dof_lin(A);
        V3 ai = scale(p.invI1, p.totalLambda);
        A.angvel = sub(A.angvel, ai);
    }
    if (B.motion == DYNAMIC) {
        V3 imp = scale(ax, p.totalLambda * imB);
        B.linvel = add(B.linvel, imp);
        apply_dof_lin(B);
        V3 ai = scale(p.invI2, p.totalLambda);
        B.angvel = add(B.angvel, ai);
    }
}
// getTotalLambda axis-constraint-part.ts:578-625
static double total_lambda(const AxisPart &p, const Body &A, const Body &B, V3 ax) {
    bool mA = A.motion != STATIC, mB = B.motion != STATIC;
    double jv;
    if (mA && mB) {
        double dx = A.linvel.x - B.linvel.x, dy = A.linvel.y - B.linvel.y, dz = A.linvel.z - B.linvel.z;
        jv = ax.x * dx + ax.y * dy + ax.z * dz;
    } else if (mA) {
        jv = ax.x * A.linvel.x + ax.y * A.linvel.y + ax.z * A.linvel.z;
    } else if (mB) {
        jv = -(ax.x * B.linvel.x + ax.y * B.linvel.y + ax.z * B.linvel.z);
    } else {
        jv = 0;
    }
    if (mA) jv += p.r1xa.x * A.angvel.x + p.r1xa.y * A.angvel.y + p.r1xa.z * A.angvel.z;
    if (mB) jv -= p.r2xa.x * B.angvel.x + p.r2xa.y * B.angvel.y + p.r2xa.z * B.angvel.z;
    double lambda = p.effMass * (jv - (p.softness * p.totalLambda + p.bias));
    return p.totalLambda + lambda;
}
// applyLambda axis-constraint-part.ts:640-707
static bool apply_lambda(AxisPart &p, Body &A, Body &B, double imA, double imB, V3 ax, double tl) {
    double dl = tl - p.totalLambda;
    p.totalLambda = tl;
    if (dl == 0) return false;
    if (A.motion == DYNAMIC) {
        double ls = dl * imA;
        A.linvel.x -= ax.x * ls;
        A.linvel.y -= ax.y * ls;
        A.linvel.z -= ax.z * ls;
        apply_dof_lin(A);
        A.angvel.x -= p.invI1.x * dl;
        A.angvel.y -= p.invI1.y * dl;
        A.angvel.z -= p.invI1.z * dl;
    }
    if (B.motion == DYNAMIC) {
        double ls = dl * imB;
        B.linvel.x += ax.x * ls;
        B.linvel.y += ax.y * ls;
        B.linvel.z += ax.z * ls;
        apply_dof_lin(B);
        B.angvel.x += p.invI2.x * dl;
        B.angvel.y += p.invI2.y * dl;
        B.angvel.z += p.invI2.z * dl;
    }
    return true;
}

static void warm_start_all(World &w, double ratio) {
    for (ContactConstraint &c : w.constraints) {
        Body &A = w.bodies[c.bodyA], &B = w.bodies[c.bodyB];
        for (int i = 0; i < c.n; i++) {
            WorldContactPoint &cp = c.pts[i];
            if (part_active(cp.t1) || part_active(cp.t2)) {
                warm_start(cp.t1, A, B, c.invMassA, c.invMassB, c.t1, ratio);
                warm_start(cp.t2, A, B, c.invMassA, c.invMassB, c.t2, ratio);
            }
            warm_start(cp.n, A, B, c.invMassA, c.invMassB, c.normal, ratio);
        }
    }
}

// solveVelocityConstraintsForIsland contact-constraints.ts:963-1053
static void solve_velocity(World &w, const std::vector<int> &ids) {
    for (int ci : ids) {
        ContactConstraint &c = w.constraints[ci];
        Body &A = w.bodies[c.bodyA], &B = w.bodies[c.bodyB];
        if (A.motion != DYNAMIC && B.motion != DYNAMIC) continue;
        for (int i = 0; i < c.n; i++) {
            WorldContactPoint &cp = c.pts[i];
            if (part_active(cp.t1) || part_active(cp.t2)) {
                double l1 = total_lambda(cp.t1, A, B, c.t1);
                double l2 = total_lambda(cp.t2, A, B, c.t2);
                double mf = c.friction * cp.n.totalLambda;
                double fm = l1 * l1 + l2 * l2;
                double mfs = mf * mf;
                if (fm > mfs) {
                    double s = mf / std::sqrt(fm);
                    l1 *= s;
                    l2 *= s;
                }
                apply_lambda(cp.t1, A, B, c.invMassA, c.invMassB, c.t1, l1);
                apply_lambda(cp.t2, A, B, c.invMassA, c.invMassB, c.t2, l2);
            }
        }
        for (int i = 0; i < c.n; i++) {
            WorldContactPoint &cp = c.pts[i];
            double tl = total_lambda(cp.n, A, B, c.normal);
            apply_lambda(cp.n, A, B, c.invMassA, c.invMassB, c.normal, std::max(0.0, tl));
        }
    }
}

// rigid-body-step.ts:16-97
static void add_rotation_step(Body &b, V3 a) {
    double l = len(a);
    if (l > 1.0e-6) {
        V3 axis = scale(a, 1 / l);
        Q4 r = qaxis_angle(axis, l);
        b.quat = qnormalize(qmul(r, b.quat));
    }
}
static void sub_rotation_step(Body &b, V3 a) {
    double l = len(a);
    if (l > 1.0e-6) {
        V3 axis = scale(a, 1 / l);
        Q4 r = qaxis_angle(axis, -l);
        b.quat = qnormalize(qmul(r, b.quat));
    }
}
static void apply_dof_pos(Body &b) {
    int t = b.dof & 0b111;
    if (!(t & 1)) b.com.x = 0;
    if (!(t & 2)) b.com.y = 0;
    if (!(t & 4)) b.com.z = 0;
}

#include "oracle_joints.h"

// ConstraintDef dispatch of every joint type (constraints.ts:264-342)
static void joint_setup(World &w, int id, double dt) {
    int i = joint_index(id);
    switch (joint_type(id)) {
    case JT_POINT: { PointJoint &j = w.points[i]; pointj_setup(j, w.bodies[j.a], w.bodies[j.b]); break; }
    case JT_DISTANCE: { DistanceJoint &j = w.distances[i]; distance_calc(j, w.bodies[j.a], w.bodies[j.b], dt); break; }
    case JT_HINGE: { HingeJoint &j = w.joints[i]; hinge_setup(j, w.bodies[j.a], w.bodies[j.b], dt); break; }
    case JT_SLIDER: { SliderJoint &j = w.sliders[i]; slider_setup(j, w.bodies[j.a], w.bodies[j.b], dt); break; }
    case JT_FIXED: { FixedJoint &j = w.fixeds[i]; fixed_setup(j, w.bodies[j.a], w.bodies[j.b]); break; }
    case JT_CONE: { ConeJoint &j = w.cones[i]; cone_setup(j, w.bodies[j.a], w.bodies[j.b]); break; }
    case JT_SWING: { SwingTwistJoint &j = w.swings[i]; swing_setup(j, w.bodies[j.a], w.bodies[j.b], dt); break; }
    case JT_SIX_DOF: { SixDofJoint &j = w.sixdofs[i]; sixdof_setup(j, w.bodies[j.a], w.bodies[j.b], dt); break; }
    }
}
static void joint_warm(World &w, int id, double ratio) {
    int i = joint_index(id);
    switch (joint_type(id)) {
    case JT_POINT: { PointJoint &j = w.points[i]; pointj_warm(j, w.bodies[j.a], w.bodies[j.b], ratio); break; }
    case JT_DISTANCE: { DistanceJoint &j = w.distances[i]; distance_warm(j, w.bodies[j.a], w.bodies[j.b], ratio); break; }
    case JT_HINGE: { HingeJoint &j = w.joints[i]; hinge_warm(j, w.bodies[j.a], w.bodies[j.b], ratio); break; }
    case JT_SLIDER: { SliderJoint &j = w.sliders[i]; slider_warm(j, w.bodies[j.a], w.bodies[j.b], ratio); break; }
    case JT_FIXED: { FixedJoint &j = w.fixeds[i]; fixed_warm(j, w.bodies[j.a], w.bodies[j.b], ratio); break; }
    case JT_CONE: { ConeJoint &j = w.cones[i]; cone_warm(j, w.bodies[j.a], w.bodies[j.b], ratio); break; }
    case JT_SWING: { SwingTwistJoint &j = w.swings[i]; swing_warm(j, w.bodies[j.a], w.bodies[j.b], ratio); break; }
    case JT_SIX_DOF: { SixDofJoint &j = w.sixdofs[i]; sixdof_warm(j, w.bodies[j.a], w.bodies[j.b], ratio); break; }
    }
}
static bool joint_solve_velocity(World &w, int id, double dt) {
    int i = joint_index(id);
    switch (joint_type(id)) {
    case JT_POINT: { PointJoint &j = w.points[i]; return pointj_solve_velocity(j, w.bodies[j.a], w.bodies[j.b]); }
    case JT_DISTANCE: { DistanceJoint &j = w.distances[i]; return distance_solve_velocity(j, w.bodies[j.a], w.bodies[j.b]); }
    case JT_HINGE: { HingeJoint &j = w.joints[i]; return hinge_solve_velocity(j, w.bodies[j.a], w.bodies[j.b], dt); }
    case JT_SLIDER: { SliderJoint &j = w.sliders[i]; return slider_solve_velocity(j, w.bodies[j.a], w.bodies[j.b], dt); }
    case JT_FIXED: { FixedJoint &j = w.fixeds[i]; return fixed_solve_velocity(j, w.bodies[j.a], w.bodies[j.b]); }
    case JT_CONE: { ConeJoint &j = w.cones[i]; return cone_solve_velocity(j, w.bodies[j.a], w.bodies[j.b]); }
    case JT_SWING: { SwingTwistJoint &j = w.swings[i]; return swing_solve_velocity(j, w.bodies[j.a], w.bodies[j.b], dt); }
    case JT_SIX_DOF: { SixDofJoint &j = w.sixdofs[i]; return sixdof_solve_velocity(j, w.bodies[j.a], w.bodies[j.b], dt); }
    }
    return false;
}
static bool joint_solve_position(World &w, int id, double dt) {
    int i = joint_index(id);
    double beta = w.s.baumgarteFactor;
    switch (joint_type(id)) {
    case JT_POINT: { PointJoint &j = w.points[i]; return pointj_solve_position(j, w.bodies[j.a], w.bodies[j.b], beta); }
    case JT_DISTANCE: {
        DistanceJoint &j = w.distances[i];
        return distance_solve_position(j, w.bodies[j.a], w.bodies[j.b], dt, beta);
    }
    case JT_HINGE: { HingeJoint &j = w.joints[i]; return hinge_solve_position(j, w.bodies[j.a], w.bodies[j.b], dt, beta); }
    case JT_SLIDER: { SliderJoint &j = w.sliders[i]; return slider_solve_position(j, w.bodies[j.a], w.bodies[j.b], dt, beta); }
    case JT_FIXED: { FixedJoint &j = w.fixeds[i]; return fixed_solve_position(j, w.bodies[j.a], w.bodies[j.b], beta); }
    case JT_CONE: { ConeJoint &j = w.cones[i]; return cone_solve_position(j, w.bodies[j.a], w.bodies[j.b], beta); }
    case JT_SWING: { SwingTwistJoint &j = w.swings[i]; return swing_solve_position(j, w.bodies[j.a], w.bodies[j.b], beta); }
    case JT_SIX_DOF: { SixDofJoint &j = w.sixdofs[i]; return sixdof_solve_position(j, w.bodies[j.a], w.bodies[j.b], beta); }
    }
    return false;
}

// solvePositionConstraintsForIsland contact-constraints.ts:1098-1216
static bool solve_position(World &w, const std::vector<int> &ids) {
    bool any = false;
    for (int ci : ids) {
        ContactConstraint &c = w.constraints[ci];
        Body &A = w.bodies[c.bodyA], &B = w.bodies[c.bodyB];
        if (A.motion != DYNAMIC && B.motion != DYNAMIC) continue;
        M4 rotA = mat4_from_quat(A.quat), rotB = mat4_from_quat(B.quat);
        M4 IA{}, IB{};
        if (A.motion == DYNAMIC) IA = inv_inertia_for_rotation(A, rotA);
        if (B.motion == DYNAMIC) IB = inv_inertia_for_rotation(B, rotB);
        for (int i = 0; i < c.n; i++) {
            WorldContactPoint &cp = c.pts[i];
            V3 wra = m3mul(rotA, cp.localA);
            V3 pa = add(A.com, wra);
            V3 wrb = m3mul(rotB, cp.localB);
            V3 pb = add(B.com, wrb);
            V3 pv = sub(pb, pa);
            double sep = (pv.x * c.normal.x + pv.y * c.normal.y + pv.z * c.normal.z) + w.s.penetrationSlop;
            sep = std::max(sep, -w.s.maxPenetrationDistance);
            if (sep >= 0) continue;
            V3 mid{(pa.x + pb.x) * 0.5, (pa.y + pb.y) * 0.5, (pa.z + pb.z) * 0.5};
            V3 rA = sub(mid, A.com), rB = sub(mid, B.com);
            // calculateConstraintPropertiesWithMassOverride axis-constraint-part.ts:225-264
            M4 sIA = IA, sIB = IB;
            for (int k = 0; k < 16; k++) {
                sIA.m[k] *= c.invIScaleA;
                sIB.m[k] *= c.invIScaleB;
            }
            calc_props(cp.n, A, B, c.invMassA, c.invMassB, sIA, sIB, rA, rB, c.normal, 0);
            // solvePositionConstraintWithMassOverride axis-constraint-part.ts:790-847
            AxisPart &p = cp.n;
            if (sep == 0 || !part_active(p) || p.softness != 0) continue;
            double lambda = -p.effMass * w.s.baumgarteFactor * sep;
            if (A.motion == DYNAMIC) {
                V3 imp = scale(c.normal, lambda * c.invMassA);
                A.com = sub(A.com, imp);
                apply_dof_pos(A);
                sub_rotation_step(A, scale(p.invI1, lambda));
            }
            if (B.motion == DYNAMIC) {
                V3 imp = scale(c.normal, lambda * c.invMassB);
                B.com = add(B.com, imp);
                apply_dof_pos(B);
                add_rotation_step(B, scale(p.invI2, lambda));
            }
            any = true;
        }
    }
    return any;
}

// ---------------------------------------------------------------------------
// Islands (islands.ts)
// ---------------------------------------------------------------------------
static void build_islands(World &w) {
    int64_t na = w.activeCount;
    std::vector<int64_t> links(na), bodyIslands(na, 0);
    for (int64_t i = 0; i < na; i++) links[i] = i;
    for (Body &b : w.bodies) b.islandIndex = -1;
    auto lowest = [&](int64_t i) {
        while (links[i] != i) i = links[i];
        return i;
    };
    // linkBodies islands.ts:103-140
    auto link_bodies = [&](int64_t a, int64_t b) {
        if (a < na && b < na) {
            int64_t f = lowest(a), s = lowest(b);
            if (f != s) {
                if (f < s)
                    links[s] = f;
                else
                    links[f] = s;
                int64_t lo = std::min(f, s);
                if (links[a] > lo) links[a] = lo;
                if (links[b] > lo) links[b] = lo;
            }
        }
    };
    std::vector<int64_t> contactLinks(w.constraints.size(), INACTIVE);
    for (size_t ci = 0; ci < w.constraints.size(); ci++) {
        const ContactConstraint &c = w.constraints[ci];
        Body &A = w.bodies[c.bodyA], &B = w.bodies[c.bodyB];
        if (A.activeIndex != INACTIVE && B.activeIndex != INACTIVE) link_bodies(A.activeIndex, B.activeIndex);
        contactLinks[ci] = std::min(A.activeIndex, B.activeIndex);
    }
    // linkUserConstraints islands.ts:209-224, linkConstraint :163-178
    std::vector<int> jointIds = joint_ids(w);
    std::vector<int64_t> jointLinks(jointIds.size(), INACTIVE);
    for (size_t k = 0; k < jointIds.size(); k++) {
        JointInfo j = joint_info(w, jointIds[k]);
        if (!j.enabled) continue;
        Body &A = w.bodies[j.a], &B = w.bodies[j.b];
        if (A.activeIndex == INACTIVE && B.activeIndex == INACTIVE) continue;
        if (A.activeIndex != INACTIVE && B.activeIndex != INACTIVE) link_bodies(A.activeIndex, B.activeIndex);
        jointLinks[k] = std::min(A.activeIndex, B.activeIndex);
    }
    // finalize islands.ts:240-389
    int ni = 0;
    for (int64_t i = 0; i < na; i++) {
        int64_t l = links[i];
        if (l != i) {
            bodyIslands[i] = bodyIslands[l];
        } else {
            bodyIslands[i] = ni++;
        }
    }
    std::vector<Island> isl(ni);
    for (int64_t ai = 0; ai < na; ai++) {
        int bi = w.activeBodyIndices[ai];
        isl[bodyIslands[ai]].bodyIndices.push_back(ai);
        w.bodies[bi].islandIndex = (int)bodyIslands[ai];
    }
    for (size_t ci = 0; ci < contactLinks.size(); ci++) {
        int64_t ab = contactLinks[ci];
        if (ab >= INACTIVE) continue;
        isl[bodyIslands[ab]].contactIndices.push_back((int)ci);
    }
    for (size_t k = 0; k < jointLinks.size(); k++) {
        int64_t ab = jointLinks[k];
        if (ab >= INACTIVE) continue;
        isl[bodyIslands[ab]].jointIndices.push_back(jointIds[k]);
    }
    std::stable_sort(isl.begin(), isl.end(), [](const Island &a, const Island &b) {
        return a.contactIndices.size() + a.jointIndices.size() > b.contactIndices.size() + b.jointIndices.size();
    });
    for (Island &is : isl) {
        int vs = 0, ps = 0;
        bool dv = false, dp = false;
        for (int64_t ai : is.bodyIndices) {
            Body &b = w.bodies[w.activeBodyIndices[ai]];
            if (b.motion != DYNAMIC) continue;
            vs = std::max(vs, b.velOverride);
            dv = dv || b.velOverride == 0;
            ps = std::max(ps, b.posOverride);
            dp = dp || b.posOverride == 0;
        }
        // getConstraintIterationOverrides of the island's user constraints (hinge-constraint.ts:819-827)
        for (int id : is.jointIndices) {
            JointInfo ji = joint_info(w, id);
            int jv = ji.velOverride, jp = ji.posOverride;
            vs = std::max(vs, jv);
            dv = dv || jv == 0;
            ps = std::max(ps, jp);
            dp = dp || jp == 0;
        }
        if (dv) vs = std::max(vs, w.s.velocityIterations);
        if (dp) ps = std::max(ps, w.s.positionIterations);
        is.velSteps = vs;
        is.posSteps = ps;
    }
    w.islands = std::move(isl);
}

// checkIslandSleep islands.ts:392-423
static void check_island_sleep(World &w, Island &is, double dt) {
    if (!w.s.allowSleeping) return;
    double tbs = w.s.timeBeforeSleep;
    double maxMove = w.s.pointVelocitySleepThreshold * tbs;
    bool all = true;
    for (int64_t ai : is.bodyIndices) {
        Body &b = w.bodies[w.activeBodyIndices[ai]];
        if (b.motion != DYNAMIC) continue;
        bool cs = update_sleep_state(b, dt, maxMove, tbs);
        all = all && cs;
    }
    if (all) {
        for (int64_t ai : is.bodyIndices) {
            Body &b = w.bodies[w.activeBodyIndices[ai]];
            if (b.motion == DYNAMIC) sleep_body(w, b);
        }
    }
}

// ---------------------------------------------------------------------------
// The step: updateWorld update.ts:45-239 (no listener, no joints, no CCD bodies)
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// Continuous collision detection for LINEAR_CAST bodies (update.ts:896-976, 979-1700, ccd.ts)
// ---------------------------------------------------------------------------
// getInnerRadius box.ts:333-335, sphere.ts:147-149, capsule.ts:254-256, convex-hull.ts:549-558
static double inner_radius(const Shape &s) {
    if (s.decorated && s.innerRadius >= 0) return s.innerRadius;
    if (s.type == SHAPE_COMPOUND) return s.compound->innerRadius;
    switch (s.type) {
        case SHAPE_BOX:
            return std::min(s.half_extents.x, std::min(s.half_extents.y, s.half_extents.z));
        case SHAPE_CYLINDER:  // cylinder.ts getInnerRadius
            return std::min(s.half_height, s.radius);
        case SHAPE_CONVEX_HULL: {
            double r = std::numeric_limits<double>::max();
            for (double c : s.hull->plane_c) r = std::min(r, -c);
            return std::max(0.0, r);
        }
        default:
            return s.radius;
    }
}

// Slab test of the segment origin + t * dir, t in [0, length], against a box: the entry t, or
// +inf on a miss.  rayDistanceToBox3 cast-utils.ts:14-49 (which returns t / length); the same
// slab test stands for mathcat 0.0.10's raycast3.intersectsBox3, which the reference calls with
// the ray's direction as given (normalised in dbvt.ts:888, the raw displacement in
// update.ts:1201-1204).
static double ray_box_entry(V3 o, V3 d, double length, const Box3 &b) {
    double t0 = 0, t1 = length;
    const double oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
    const double mn[3] = {b.mn.x, b.mn.y, b.mn.z}, mx[3] = {b.mx.x, b.mx.y, b.mx.z};
    for (int i = 0; i < 3; i++) {
        if (std::fabs(dd[i]) < 1e-10) {
            if (oo[i] < mn[i] || oo[i] > mx[i]) return std::numeric_limits<double>::infinity();
        } else {
            double inv = 1.0 / dd[i];
            double a = (mn[i] - oo[i]) * inv, c = (mx[i] - oo[i]) * inv;
            t0 = std::max(t0, std::min(a, c));
            t1 = std::min(t1, std::max(a, c));
            if (t1 < t0) return std::numeric_limits<double>::infinity();
        }
    }
    return t0;
}

static Box3 box_grow(const Box3 &b, V3 e) { return {sub(b.mn, e), add(b.mx, e)}; }

// findCCDContacts update.ts:1354-1470 with the broadphase cast (broadphase.ts:327-343,
// dbvt.ts:869-975), the body visitor (update.ts:1118-1250) and the collector
// (update.ts:1003-1115).  The candidates are every body in index order; the first of equal
// fractions wins, as the collector keeps only strictly earlier hits.  The dynamic tree's
// distance cull (dbvt.ts:905) compares against fattened leaf boxes that depend on the tree's
// history; the exact box stands in for them here.  The contact-manifold block that follows the
// cast in the reference (update.ts:1395-1466) is never entered, because the collector's
// reset() (update.ts:1036-1042) clears hasHit after every visit.
static void find_ccd_contacts(World &w, double dt) {
    for (World::CCDRecord &c : w.ccd) {
        Body &A = w.bodies[c.body];
        Box3 end{add(A.aabb.mn, c.delta), add(A.aabb.mx, c.delta)};
        Box3 swept{{std::min(A.aabb.mn.x, end.mn.x), std::min(A.aabb.mn.y, end.mn.y), std::min(A.aabb.mn.z, end.mn.z)},
                   {std::max(A.aabb.mx.x, end.mx.x), std::max(A.aabb.mx.y, end.mx.y), std::max(A.aabb.mx.z, end.mx.z)}};
        V3 origin = scale(add(swept.mn, swept.mx), 0.5);
        V3 half = scale(sub(swept.mx, swept.mn), 0.5);
        double castLen = len(c.delta);
        V3 castDir = normalize(c.delta);
        V3 halfA = scale(sub(A.aabb.mx, A.aabb.mn), 0.5);
        int la = A.objectLayer;
        for (Body &B : w.bodies) {
            int lb = B.objectLayer;
            // broadphase layer and leaf filters of the tree cast (broadphase.ts:334-335,
            // dbvt.ts:905-966)
            if (!w.layers.objVsBp[la * w.layers.nBp + w.layers.objToBp[lb]]) continue;
            if (!((A.groups & B.mask) != 0 && (B.groups & A.mask) != 0)) continue;
            if (!w.layers.objPairs[la * w.layers.nObj + lb]) continue;
            double t = ray_box_entry(origin, castDir, castLen, box_grow(B.aabb, half));
            if (!(t < std::numeric_limits<double>::infinity()) || t / castLen > castLen) continue;
            // ccdBodyVisitor.visit update.ts:1153-1250
            if (B.index == A.index) continue;
            const World::CCDRecord *cb = B.ccdIndex >= 0 ? &w.ccd[B.ccdIndex] : nullptr;
            if (cb && c.body > cb->body) continue;
            if (B.sensor) continue;
            V3 rel = cb ? sub(c.delta, cb->delta) : c.delta;
            if (lensq(rel) < c.thresholdSq) continue;
            double relLen = len(rel);
            if (!(ray_box_entry(A.position, rel, relLen, box_grow(B.aabb, halfA)) <
                  std::numeric_limits<double>::infinity()))
                continue;
            V3 gpA, gpB;
            Q4 gqA, gqB;
            geometry_pose(A.shape, A.position, A.quat, gpA, gqA);
            geometry_pose(B.shape, B.position, B.quat, gpB, gqB);
            // ccdCastShapeCollector.addHit update.ts:1044-1109
            auto collect = [&](double fraction, V3 pa, V3 axis) {
                V3 n = normalize(axis);
                double den = dot(n, c.delta);
                if (den <= c.maxPenetration) return;
                double fps = fraction + c.maxPenetration / den;
                if (fps >= c.fps) return;
                c.hit = B.index;
                c.fraction = fraction;
                c.fps = fps;
                c.normal = n;
                // calculateBodyMotion update.ts:984-994: a moving LINEAR_CAST body B counts its
                // velocity step, whether or not it took the continuous path this step
                V3 mB{0, 0, 0};
                if (B.motion != STATIC && B.linearCast) mB = scale(B.linvel, dt);
                c.point = lensq(mB) > 1e-12 ? add(pa, scale(mB, fraction)) : pa;
                c.friction = combine(A.friction, B.friction, A.frictionCombine, B.frictionCombine);
                c.restitution = combine(A.restitution, B.restitution, A.restitutionCombine, B.restitutionCombine);
            };
            if (B.shape.type == SHAPE_EMPTY || A.shape.type == SHAPE_EMPTY) continue;
            if (B.shape.type == SHAPE_COMPOUND) {  // castShapeVsCompound compound.ts:776-866: each child
                const CompoundData &C = *B.shape.compound;
                for (int i = 0; i < (int)C.shapes.size(); i++) {
                    V3 cp;
                    Q4 cq;
                    compound_child_pose(C, i, gpB, gqB, cp, cq);
                    CastHit h;
                    if (cast_convex_vs_convex(h, A.shape, gpA, gqA, rel, C.shapes[i], cp, cq, c.fps, false))
                        collect(h.fraction, h.pa, h.axis);
                }
                continue;
            }
            if (B.shape.type == SHAPE_PLANE) {  // castConvexVsPlane plane.ts:727-918
                CastHit h;
                if (cast_convex_vs_plane(h, A.shape, gpA, gqA, rel, B.shape, gpB, gqB, c.fps, false))
                    collect(h.fraction, h.pa, h.axis);
                continue;
            }
            if (B.shape.type == SHAPE_TRIANGLE_MESH) {
                // castShapeVsShape dispatch (triangle-mesh.ts:223-237): the sphere's own cast
                // for spheres, the GJK cast for the other shapes; the collector's early-out
                // fraction tightens with each hit
                auto onHit = [&](const CastMeshHit &h) { collect(h.fraction, h.pa, h.axis); };
                auto earlyOut = [&]() { return c.fps; };
                if (A.shape.type == SHAPE_SPHERE)
                    cast_sphere_vs_mesh(A.shape, gpA, rel, B.shape, gpB, gqB, onHit, earlyOut);
                else
                    cast_convex_vs_mesh(A.shape, gpA, gqA, rel, B.shape, gpB, gqB, onHit, earlyOut);
                continue;
            }
            CastHit h;
            if (!cast_convex_vs_convex(h, A.shape, gpA, gqA, rel, B.shape, gpB, gqB, c.fps, false)) continue;
            collect(h.fraction, h.pa, h.axis);
        }
    }
}

static void clamp_velocities(Body &b) {  // clampLinearVelocity / clampAngularVelocity motion-properties.ts:624-639
    if (lensq(b.linvel) > b.maxLin * b.maxLin) b.linvel = scale(normalize(b.linvel), b.maxLin);
    if (lensq(b.angvel) > b.maxAng * b.maxAng) b.angvel = scale(normalize(b.angvel), b.maxAng);
}

// applyCCD update.ts:1420-1580: one normal and one friction iteration at the time of impact.
// The two parts keep their accumulated lambdas from earlier calls (module-scope scratch in the
// reference); the normal impulse itself does not depend on them, the friction bound does.
static void apply_ccd(World &w, const World::CCDRecord &c, Body &A, Body &B) {
    if (A.motion != DYNAMIC) return;
    V3 r1 = sub(c.point, scale_add(A.com, c.delta, c.fraction));
    V3 r2 = sub(c.point, B.com);
    V3 v1 = add(A.linvel, cross(A.angvel, r1));
    V3 v2 = B.motion != STATIC ? add(B.linvel, cross(B.angvel, r2)) : V3{0, 0, 0};
    V3 rel = sub(v2, v1);
    double nv = dot(rel, c.normal);
    if (nv >= 0) return;
    double bias = (c.restitution > 0 && nv < -w.s.ccdMinVelocityForRestitution) ? c.restitution * nv : 0;
    double imA = A.invMass, imB = B.motion == DYNAMIC ? B.invMass : 0;
    M4 IA = inv_inertia_for_rotation(A, mat4_from_quat(A.quat));
    M4 IB{};
    if (B.motion == DYNAMIC) IB = inv_inertia_for_rotation(B, mat4_from_quat(B.quat));
    AxisPart np;
    np.totalLambda = w.ccdNormalLambda;
    calc_props(np, A, B, imA, imB, IA, IB, r1, r2, c.normal, bias);
    apply_lambda(np, A, B, imA, imB, c.normal, total_lambda(np, A, B, c.normal));
    w.ccdNormalLambda = np.totalLambda;
    if (c.friction > 0) {
        V3 tv = sub(rel, scale(c.normal, nv));
        double tl2 = lensq(tv);
        if (tl2 > 1e-12) {
            V3 dir = scale(tv, 1.0 / std::sqrt(tl2));
            double maxF = c.friction * np.totalLambda;
            AxisPart fp;
            fp.totalLambda = w.ccdFrictionLambda;
            calc_props(fp, A, B, imA, imB, IA, IB, r1, r2, dir, 0);
            double tl = total_lambda(fp, A, B, dir);
            apply_lambda(fp, A, B, imA, imB, dir, std::max(-maxF, std::min(maxF, tl)));
            w.ccdFrictionLambda = fp.totalLambda;
        }
    }
    clamp_velocities(A);
    if (B.motion == DYNAMIC) clamp_velocities(B);
}

// sortCCDBodies update.ts:1583-1611 and resolveCCDContacts update.ts:1616-1670.  After the sort
// a body's record index still names the slot it was created in, so the cascade below reads
// the record that the sort put in that slot, as the reference does.
static void resolve_ccd_contacts(World &w) {
    std::sort(w.ccd.begin(), w.ccd.end(), [](const World::CCDRecord &a, const World::CCDRecord &b) {
        if (a.fps != b.fps) return a.fps < b.fps;
        return a.body < b.body;
    });
    for (size_t i = 0; i < w.ccd.size(); i++) {
        World::CCDRecord &c = w.ccd[i];
        Body &A = w.bodies[c.body];
        if (c.hit == -1) {
            A.position = add(A.position, c.delta);
            set_transform(A);
            continue;
        }
        Body &B = w.bodies[c.hit];
        if (B.ccdIndex >= 0) {
            World::CCDRecord &cb = w.ccd[B.ccdIndex];
            if (cb.hit != -1 && cb.fraction > c.fraction) {
                cb.hit = -1;
                cb.fps = c.fraction;
            }
        }
        apply_ccd(w, c, A, B);
        A.position = add(A.position, scale(c.delta, c.fps));
        set_transform(A);
        if (B.sleeping) wake_body(w, B);
    }
}

// The rows the velocity solve starts from (oracle_frozen.h layout): per body the velocities
// after the force integration, the world inverse inertia, the inverse mass and flags; per
// contact constraint the axes, friction, inverse masses and per point the moment arms to the
// contact midpoint (as addContactConstraint computes them, contact-constraints.ts:700-720),
// effective masses, bias, the cached (pre-ratio) impulses and the cached point they came from.
static void record_tape_rows(World &w, double dt) {
    using namespace orc_frozen;
    const size_t n = w.bodies.size();
    w.tapeBodies.assign(n * BODY_ROW, 0.0);
    for (size_t i = 0; i < n; i++) {
        const Body &b = w.bodies[i];
        double *o = &w.tapeBodies[i * BODY_ROW];
        o[0] = b.linvel.x, o[1] = b.linvel.y, o[2] = b.linvel.z;
        o[3] = b.angvel.x, o[4] = b.angvel.y, o[5] = b.angvel.z;
        const bool dyn = b.motion == DYNAMIC && !b.sleeping;
        if (dyn) {
            M4 I = inv_inertia_for_rotation(b, mat4_from_quat(b.quat));
            const int idx[9] = {0, 1, 2, 4, 5, 6, 8, 9, 10};
            for (int k = 0; k < 9; k++) o[6 + k] = I.m[idx[k]];
        }
        o[15] = b.invMass;
        o[16] = (double)((dyn ? T_DYNAMIC : 0) | (b.motion != STATIC ? T_MOVING : 0) | (b.dof << 8));
    }
    w.tapeRatio = (w.s.warmStarting && w.prevDt > 0) ? dt / w.prevDt : 0.0;
    w.tapeCons.assign(w.constraints.size() * CON_ROW, 0.0);
    for (size_t k = 0; k < w.constraints.size(); k++) {
        const ContactConstraint &c = w.constraints[k];
        const Body &A = w.bodies[c.bodyA], &B = w.bodies[c.bodyB];
        double *r = &w.tapeCons[k * CON_ROW];
        r[0] = c.bodyA, r[1] = c.bodyB, r[2] = c.n, r[3] = A.islandIndex, r[4] = c.hasPrev ? 1 : 0;
        r[5] = (double)c.sortKey;
        const V3 ax[3] = {c.normal, c.t1, c.t2};
        for (int x = 0; x < 3; x++) r[6 + 3 * x] = ax[x].x, r[7 + 3 * x] = ax[x].y, r[8 + 3 * x] = ax[x].z;
        r[15] = c.friction, r[16] = c.invMassA, r[17] = c.invMassB;
        for (int q = 0; q < c.n; q++) {
            const WorldContactPoint &cp = c.pts[q];
            double *pt = r + CON_HEAD + q * POINT_ROW;
            V3 mid{(cp.posA.x + cp.posB.x) * 0.5, (cp.posA.y + cp.posB.y) * 0.5, (cp.posA.z + cp.posB.z) * 0.5};
            V3 rA = sub(mid, A.com), rB = sub(mid, B.com);
            pt[0] = rA.x, pt[1] = rA.y, pt[2] = rA.z, pt[3] = rB.x, pt[4] = rB.y, pt[5] = rB.z;
            const AxisPart *parts[3] = {&cp.n, &cp.t1, &cp.t2};
            for (int x = 0; x < 3; x++) pt[6 + x] = parts[x]->effMass, pt[10 + x] = parts[x]->totalLambda;
            pt[9] = cp.n.bias;
            pt[13] = cp.prevPoint;
        }
        for (int q = c.n; q < 4; q++) (r + CON_HEAD + q * POINT_ROW)[13] = -1;
    }
}
// the final impulses of each constraint and the post-solve velocities of every body
static void record_tape_finals(World &w) {
    using namespace orc_frozen;
    for (size_t k = 0; k < w.constraints.size(); k++) {
        const ContactConstraint &c = w.constraints[k];
        for (int q = 0; q < c.n; q++) {
            double *pt = &w.tapeCons[k * CON_ROW + CON_HEAD + q * POINT_ROW];
            pt[14] = c.pts[q].n.totalLambda, pt[15] = c.pts[q].t1.totalLambda, pt[16] = c.pts[q].t2.totalLambda;
        }
    }
    w.tapeV2.assign(w.bodies.size() * 6, 0.0);
    for (size_t i = 0; i < w.bodies.size(); i++) {
        const Body &b = w.bodies[i];
        double *o = &w.tapeV2[i * 6];
        o[0] = b.linvel.x, o[1] = b.linvel.y, o[2] = b.linvel.z, o[3] = b.angvel.x, o[4] = b.angvel.y, o[5] = b.angvel.z;
    }
}

static void step(World &w, double dt) {
    // ccd.clear ccd.ts:108-124
    w.ccd.clear();
    for (Body &b : w.bodies) b.ccdIndex = -1;
    w.constraints.clear();
    w.manifoldLambda.clear();
    w.manifolds.clear();
    w.manifoldBodies.clear();
    for (auto &kv : w.contacts) kv.second.processed = false;
    w.events.clear();
    // accelerationIntegrationUpdate update.ts:245-319
    for (Body &b : w.bodies) {
        if (b.motion != DYNAMIC || b.sleeping) continue;
        double gs = w.s.gravityEnabled ? b.gravityFactor : 0;
        V3 g = w.s.gravity;
        double ax = (b.force.x * b.invMass + g.x * gs) * dt;
        double ay = (b.force.y * b.invMass + g.y * gs) * dt;
        double az = (b.force.z * b.invMass + g.z * gs) * dt;
        b.linvel.x += ax;
        b.linvel.y += ay;
        b.linvel.z += az;
        double ldf = std::max(0.0, 1 - b.linDamp * dt);
        b.linvel = scale(b.linvel, ldf);
        double ls = b.linvel.x * b.linvel.x + b.linvel.y * b.linvel.y + b.linvel.z * b.linvel.z;
        if (ls > b.maxLin * b.maxLin) b.linvel = scale(b.linvel, b.maxLin / std::sqrt(ls));
        apply_dof_lin(b);
        M4 R = mat4_from_quat(b.quat);
        M4 I = inv_inertia_for_rotation(b, R);
        V3 t = b.torque;
        b.angvel.x += (I.m[0] * t.x + I.m[4] * t.y + I.m[8] * t.z) * dt;
        b.angvel.y += (I.m[1] * t.x + I.m[5] * t.y + I.m[9] * t.z) * dt;
        b.angvel.z += (I.m[2] * t.x + I.m[6] * t.y + I.m[10] * t.z) * dt;
        double adf = std::max(0.0, 1 - b.angDamp * dt);
        b.angvel = scale(b.angvel, adf);
        double as = b.angvel.x * b.angvel.x + b.angvel.y * b.angvel.y + b.angvel.z * b.angvel.z;
        if (as > b.maxAng * b.maxAng) b.angvel = scale(b.angvel, b.maxAng / std::sqrt(as));
        int r = (b.dof >> 3) & 0b111;
        if (!(r & 1)) b.angvel.x = 0;
        if (!(r & 2)) b.angvel.y = 0;
        if (!(r & 4)) b.angvel.z = 0;
    }
    find_colliding_pairs(w);
    for (auto &pr : w.pairs) {
        Body *A = &w.bodies[pr.first], *B = &w.bodies[pr.second];
        if (A->motion > B->motion || (A->motion == B->motion && B->id < A->id)) std::swap(A, B);
        bool created = narrowphase(w, A, B, dt);
        if (created) {
            if (A->motion == DYNAMIC && A->sleeping) wake_body(w, *A);
            if (B->motion == DYNAMIC && B->sleeping) wake_body(w, *B);
        }
        // destroyStaleContactsBetweenBodies: a convex pair has a single contact key, so any
        // unprocessed record between A and B is removed with the unprocessed sweep below.
    }
    // destroyUnprocessedContacts contacts.ts:534-553
    for (auto it = w.contacts.begin(); it != w.contacts.end();) {
        if (!it->second.processed) {
            w.events.push_back({3, it->second.idA & 0xffffffffLL, it->second.idB & 0xffffffffLL});
            it = w.contacts.erase(it);
        } else {
            ++it;
        }
    }
    if (dt > 0) {
        // wakeBodiesInUserConstraints update.ts:863-888
        for (int id : joint_ids(w)) {
            JointInfo j = joint_info(w, id);
            if (!j.enabled) continue;
            Body &A = w.bodies[j.a], &B = w.bodies[j.b];
            bool act = !A.sleeping || !B.sleeping, dyn = A.motion == DYNAMIC || B.motion == DYNAMIC;
            if (act && dyn) {
                if (A.sleeping && A.motion == DYNAMIC) wake_body(w, A);
                if (B.sleeping && B.motion == DYNAMIC) wake_body(w, B);
            }
        }
        build_islands(w);
        // updateSleeping + setupVelocityConstraints constraints.ts:264-287
        auto joint_active = [&](int id) {
            JointInfo j = joint_info(w, id);
            return j.enabled && !(w.bodies[j.a].sleeping && w.bodies[j.b].sleeping);
        };
        for (int id : joint_ids(w)) {
            if (!joint_active(id)) continue;
            joint_setup(w, id, dt);
        }
        if (w.recordTape) record_tape_rows(w, dt);
        if (w.s.warmStarting) {
            double ratio = (w.s.warmStarting && w.prevDt > 0) ? dt / w.prevDt : 0.0;
            warm_start_all(w, ratio);
            for (int id : joint_ids(w)) {
                if (!joint_active(id)) continue;
                joint_warm(w, id, ratio);
            }
        }
        w.prevDt = dt;
        for (Island &is : w.islands) {
            if (is.contactIndices.empty() && is.jointIndices.empty()) continue;
            // sortConstraintIds constraints.ts:248-261: (priority, then the per-type index); the
            // stable sort keeps the type order of the island's list for equal keys
            std::stable_sort(is.jointIndices.begin(), is.jointIndices.end(), [&](int a, int b) {
                JointInfo ja = joint_info(w, a), jb = joint_info(w, b);
                if (ja.priority != jb.priority) return ja.priority < jb.priority;
                return ja.index < jb.index;
            });
            // sortContactIndices contact-constraints.ts:1240-1264 (JS sort is stable)
            std::stable_sort(is.contactIndices.begin(), is.contactIndices.end(), [&](int a, int b) {
                const ContactConstraint &ca = w.constraints[a], &cb = w.constraints[b];
                if (ca.sortKey != cb.sortKey) return ca.sortKey < cb.sortKey;
                int64_t ia = w.bodies[ca.bodyA].id, ib = w.bodies[cb.bodyA].id;
                if (ia != ib) return ia < ib;
                return w.bodies[ca.bodyB].id < w.bodies[cb.bodyB].id;
            });
            if (w.colouredOrder) {
                std::vector<int> &ci = is.contactIndices;
                std::vector<int> col(ci.size(), -1);
                std::map<int, size_t> claim;
                for (int round = 0;; round++) {
                    claim.clear();
                    bool left = false;
                    for (size_t k = 0; k < ci.size(); k++) {
                        if (col[k] >= 0) continue;
                        left = true;
                        const ContactConstraint &c = w.constraints[ci[k]];
                        for (int bi : {c.bodyA, c.bodyB})
                            if (w.bodies[bi].motion == DYNAMIC && !claim.count(bi)) claim[bi] = k;
                    }
                    if (!left) break;
                    for (size_t k = 0; k < ci.size(); k++) {
                        if (col[k] >= 0) continue;
                        const ContactConstraint &c = w.constraints[ci[k]];
                        bool ok = true;
                        for (int bi : {c.bodyA, c.bodyB})
                            if (w.bodies[bi].motion == DYNAMIC && claim[bi] != k) ok = false;
                        if (ok) col[k] = round;
                    }
                }
                std::vector<size_t> ord(ci.size());
                std::iota(ord.begin(), ord.end(), 0);
                std::stable_sort(ord.begin(), ord.end(), [&](size_t a, size_t b) { return col[a] < col[b]; });
                std::vector<int> re(ci.size());
                for (size_t k = 0; k < ord.size(); k++) re[k] = ci[ord[k]];
                if (re != ci) w.reorderedIslands++;
                ci = re;
            }
            for (int i = 0; i < is.velSteps; i++) {
                if (!is.contactIndices.empty()) solve_velocity(w, is.contactIndices);
                for (int ji : is.jointIndices) joint_solve_velocity(w, ji, dt);
            }
        }
        if (w.recordTape) record_tape_finals(w);
        // storeAppliedImpulses contact-constraints.ts:1061-1076
        w.manifoldLambda.assign(w.constraints.size(), 0.0);
        for (size_t k = 0; k < w.constraints.size(); k++)
            for (int i = 0; i < w.constraints[k].n; i++) w.manifoldLambda[k] += w.constraints[k].pts[i].n.totalLambda;
        for (ContactConstraint &c : w.constraints) {
            Contact &ct = w.contacts[c.contactKey];
            for (int i = 0; i < c.n; i++) {
                ct.pts[i].ln = c.pts[i].n.totalLambda;
                ct.pts[i].lt1 = c.pts[i].t1.totalLambda;
                ct.pts[i].lt2 = c.pts[i].t2.totalLambda;
            }
        }
        // velocityIntegrationUpdate update.ts:896-976
        for (Body &b : w.bodies) {
            if (b.motion == STATIC || b.sleeping) continue;
            if (b.motion == DYNAMIC) {
                // clampLinearVelocity / clampAngularVelocity motion-properties.ts:624-639
                if (lensq(b.linvel) > b.maxLin * b.maxLin) b.linvel = scale(normalize(b.linvel), b.maxLin);
                if (lensq(b.angvel) > b.maxAng * b.maxAng) b.angvel = scale(normalize(b.angvel), b.maxAng);
            }
            V3 rv = scale(b.angvel, dt);
            double angle = len(rv);
            if (angle > 1e-6) {
                V3 axis = scale(rv, 1 / angle);
                Q4 rq = qaxis_angle(axis, angle);
                b.quat = qnormalize(qmul(rq, b.quat));
            }
            V3 disp = scale(b.linvel, dt);
            // LINEAR_CAST dynamic non-sensor bodies moving more than the threshold defer their
            // translation to the continuous-collision pass (update.ts:930-968)
            if (b.linearCast && b.motion == DYNAMIC && !b.sensor) {
                double inner = inner_radius(b.shape);
                double thr = w.s.linearCastThreshold * inner;
                if (lensq(disp) > thr * thr) {
                    World::CCDRecord c;
                    c.body = b.index;
                    c.delta = disp;
                    c.thresholdSq = thr * thr;
                    c.maxPenetration = std::min(w.s.penetrationSlop, w.s.linearCastMaxPenetration * inner);
                    b.ccdIndex = (int)w.ccd.size();
                    w.ccd.push_back(c);
                    set_transform(b);  // setQuaternion: the rotation about the body position
                    continue;
                }
            }
            b.com = add(b.com, disp);
            update_pos_from_com(b);
            set_transform(b);
        }
        find_ccd_contacts(w, dt);
        w.ccdHits = 0;
        for (const World::CCDRecord &c : w.ccd) w.ccdHits += c.hit >= 0;
        resolve_ccd_contacts(w);
        for (Island &is : w.islands) {
            if (is.contactIndices.empty() && is.jointIndices.empty()) continue;
            for (int i = 0; i < is.posSteps; i++) {
                bool applied = false;
                if (!is.contactIndices.empty()) applied = solve_position(w, is.contactIndices);
                for (int ji : is.jointIndices) applied = joint_solve_position(w, ji, dt) || applied;
                if (!applied) break;
            }
        }
        // updateBodyPositions update.ts:322-330
        for (Body &b : w.bodies) {
            if (b.motion == STATIC || b.sleeping) continue;
            update_pos_from_com(b);
            set_transform(b);
        }
        for (Island &is : w.islands) check_island_sleep(w, is, dt);
    }
    for (Body &b : w.bodies) {
        if (b.motion == STATIC || b.sleeping) continue;
        b.force = {0, 0, 0};
        b.torque = {0, 0, 0};
    }
}

}  // namespace orc

// ===========================================================================
// C ABI used by the Python test harness (ctypes).
// ===========================================================================
using namespace orc;

extern "C" {

// Body description: one row of doubles per body, layout shared with the
// Python scene builder (crashcat_gb300/scenes.py BODY_FIELDS).
enum {
    F_SHAPE = 0,       // 0 sphere, 1 box, 2 capsule (F_P0 radius, F_P0 + 1 half height)
    F_P0 = 1,          // shape params (box hx,hy,hz,convexRadius ; sphere r)
    F_DENSITY = 5,
    F_MOTION = 6,
    F_POS = 7,
    F_QUAT = 10,
    F_LINVEL = 14,
    F_ANGVEL = 17,
    F_FRICTION = 20,
    F_RESTITUTION = 21,
    F_LAYER = 22,
    F_GRAVITY_FACTOR = 23,
    F_LIN_DAMP = 24,
    F_ANG_DAMP = 25,
    F_ALLOW_SLEEP = 26,
    F_WORLD = 27,
    F_GROUPS = 28,
    F_MASK = 29,
    F_MOTION_QUALITY = 30,  // 0 discrete, 1 linear cast (MotionQuality motion-properties.ts:8-26)
    F_VEL_OVERRIDE = 31,    // numVelocityStepsOverride / numPositionStepsOverride (motion-properties.ts:59-61)
    F_POS_OVERRIDE = 32,
    F_SCALE = 33,           // ScaledShape.scale (0 components read as 1)
    F_TPOS = 36,            // TransformedShape.position
    F_TROT = 39,            // TransformedShape.quaternion (all zero: identity)
    F_COM_OFFSET = 43,      // OffsetCenterOfMassShape.offset
    F_MASS_MODE = 46,       // MassPropertiesOverride: 0 from the shape, 1 mass given, 2 mass and inertia given
    F_MASS = 47,            // RigidBodySettings.mass / massPropertiesOverride.mass
    F_INERTIA = 48,         // massPropertiesOverride inertia xx xy xz yy yz zz
    F_COUNT = 54
};

void *orc_world_create(const double *settings, int n_obj, const int *obj_to_bp, int n_bp, const uint8_t *obj_pairs,
                       const uint8_t *obj_vs_bp, const uint8_t *bp_pairs) {
    World *w = new World();
    Settings &s = w->s;
    s.gravity = {settings[0], settings[1], settings[2]};
    s.speculativeContactDistance = settings[3];
    s.manifoldTolerance = settings[4];
    s.collisionTolerance = settings[5];
    s.penetrationTolerance = settings[6];
    s.normalCosMaxDeltaRotation = settings[7];
    s.preserveLambdaMaxDistSq = settings[8];
    s.velocityIterations = (int)settings[9];
    s.positionIterations = (int)settings[10];
    s.warmStarting = settings[11] != 0;
    s.penetrationSlop = settings[12];
    s.baumgarteFactor = settings[13];
    s.maxPenetrationDistance = settings[14];
    s.minVelocityForRestitution = settings[15];
    s.allowSleeping = settings[16] != 0;
    s.timeBeforeSleep = settings[17];
    s.pointVelocitySleepThreshold = settings[18];
    s.gravityEnabled = settings[19] != 0;
    s.linearCastThreshold = settings[20];
    s.linearCastMaxPenetration = settings[21];
    s.ccdMinVelocityForRestitution = settings[22];
    w->layers.nObj = n_obj;
    w->layers.nBp = n_bp;
    w->layers.objToBp.assign(obj_to_bp, obj_to_bp + n_obj);
    w->layers.objPairs.assign(obj_pairs, obj_pairs + n_obj * n_obj);
    w->layers.objVsBp.assign(obj_vs_bp, obj_vs_bp + n_obj * n_bp);
    w->layers.bpPairs.assign(bp_pairs, bp_pairs + n_bp * n_bp);
    return w;
}

void orc_world_destroy(void *wp) { delete (World *)wp; }

// rigidBody.create rigid-body.ts:390-434 for each row
// Shape fields of a body row (F_SHAPE, F_DENSITY, F_P0..F_P0 + 3); false for an unknown type.
// The decorators of a body row around its leaf shape, nested as
// OffsetCenterOfMass(Transformed(Scaled(leaf))): the scale baked into the leaf (box half
// extents |s| per axis with the convex radius min(r min|s|, 0.05) of setBoxSupport
// support.ts:343-372; sphere and capsule |s.x|, sphere.ts:195-197, capsule.ts:308-318), the
// local bounds of computeScaledLocalBounds / computeTransformedLocalBounds (scaled.ts,
// transformed.ts), the centre of mass of computeTransformedCenterOfMass +
// computeOffsetCenterOfMassCenterOfMass and the inner radius min|s| x the leaf's (scaled.ts
// getInnerRadius).  A scaled convex hull or mesh is refused.
static bool decorate(Shape &s, const double *r) {
    V3 sc{r[F_SCALE], r[F_SCALE + 1], r[F_SCALE + 2]};
    if (sc.x == 0) sc.x = 1;
    if (sc.y == 0) sc.y = 1;
    if (sc.z == 0) sc.z = 1;
    V3 tp{r[F_TPOS], r[F_TPOS + 1], r[F_TPOS + 2]};
    Q4 tq{r[F_TROT], r[F_TROT + 1], r[F_TROT + 2], r[F_TROT + 3]};
    if (tq.x == 0 && tq.y == 0 && tq.z == 0 && tq.w == 0) tq = {0, 0, 0, 1};
    V3 off{r[F_COM_OFFSET], r[F_COM_OFFSET + 1], r[F_COM_OFFSET + 2]};
    const bool scaled = sc.x != 1 || sc.y != 1 || sc.z != 1;
    const bool transformed = tp.x != 0 || tp.y != 0 || tp.z != 0 || tq.x != 0 || tq.y != 0 || tq.z != 0 || tq.w != 1;
    const bool offset = off.x != 0 || off.y != 0 || off.z != 0;
    if (!scaled && !transformed && !offset) return true;
    const V3 as{std::fabs(sc.x), std::fabs(sc.y), std::fabs(sc.z)};
    const double minScale = std::min(as.x, std::min(as.y, as.z));
    const double leafInner = inner_radius(s);
    if (scaled) {
        if (s.type == SHAPE_CONVEX_HULL || s.type == SHAPE_TRIANGLE_MESH) return false;
        if (s.type == SHAPE_BOX) {
            s.half_extents = {s.half_extents.x * as.x, s.half_extents.y * as.y, s.half_extents.z * as.z};
            s.convex_radius = std::min(s.convex_radius * minScale, 0.05);
        } else if (s.type == SHAPE_CYLINDER) {  // setCylinder*Support cylinder.ts: |s.x| throughout
            s.radius *= as.x;
            s.half_height *= as.x;
            s.convex_radius *= as.x;
        } else {
            s.radius *= as.x;
            s.half_height *= as.x;
        }
        // computeScaledLocalBounds: the leaf's bounds times |s| per axis
        s.aabb = {{s.aabb.mn.x * as.x, s.aabb.mn.y * as.y, s.aabb.mn.z * as.z},
                  {s.aabb.mx.x * as.x, s.aabb.mx.y * as.y, s.aabb.mx.z * as.z}};
        // computeScaledCenterOfMass reads the scaled shape's own (zero) centre of mass
        s.com = {0, 0, 0};
    }
    s.leafAabb = s.aabb;
    if (transformed) {
        Box3 b{{1e300, 1e300, 1e300}, {-1e300, -1e300, -1e300}};
        for (int c = 0; c < 8; c++) {
            V3 k{(c & 1) ? s.aabb.mx.x : s.aabb.mn.x, (c & 2) ? s.aabb.mx.y : s.aabb.mn.y,
                 (c & 4) ? s.aabb.mx.z : s.aabb.mn.z};
            V3 t = add(rotate(tq, k), tp);
            b.mn = {std::min(b.mn.x, t.x), std::min(b.mn.y, t.y), std::min(b.mn.z, t.z)};
            b.mx = {std::max(b.mx.x, t.x), std::max(b.mx.y, t.y), std::max(b.mx.z, t.z)};
        }
        s.aabb = b;
        s.com = add(rotate(tq, s.com), tp);
    }
    s.com = add(s.com, off);
    s.decorated = true;
    s.tPos = tp;
    s.tRot = tq;
    s.innerRadius = (scaled ? minScale : 1.0) * leafInner;
    return true;
}

// computeCompoundLocalBounds compound.ts:70-108: the children's bounds' corners through their poses
static Box3 compound_bounds(const CompoundData &c) {
    Box3 b{{1e300, 1e300, 1e300}, {-1e300, -1e300, -1e300}};
    for (size_t i = 0; i < c.shapes.size(); i++) {
        const Box3 &a = c.shapes[i].aabb;
        for (int k = 0; k < 8; k++) {
            V3 p{(k & 1) ? a.mx.x : a.mn.x, (k & 2) ? a.mx.y : a.mn.y, (k & 4) ? a.mx.z : a.mn.z};
            V3 q = add(rotate(c.rot[i], p), c.pos[i]);
            b.mn = {std::min(b.mn.x, q.x), std::min(b.mn.y, q.y), std::min(b.mn.z, q.z)};
            b.mx = {std::max(b.mx.x, q.x), std::max(b.mx.y, q.y), std::max(b.mx.z, q.z)};
        }
    }
    return b;
}
static V3 compound_com(const CompoundData &c);

static bool shape_from_row(Shape &s, const double *r, const World *w = nullptr) {
    s.type = (int)r[F_SHAPE];
    s.density = r[F_DENSITY];
    s.com = {0, 0, 0};
    if (s.type == SHAPE_CONVEX_HULL) {  // F_P0: the hull index
        int h = (int)r[F_P0];
        if (!w || h < 0 || h >= (int)w->hulls.size()) return false;
        s.hull = w->hulls[h].get();
        s.com = s.hull->com;
        s.aabb = s.hull->bounds;
        s.convex_radius = s.hull->convex_radius;
    } else if (s.type == SHAPE_COMPOUND) {  // F_P0: the compound index; no decorators on it
        int c = (int)r[F_P0];
        if (!w || c < 0 || c >= (int)w->compounds.size()) return false;
        s.compound = w->compounds[c].get();
        s.aabb = compound_bounds(*s.compound);
        s.com = compound_com(*s.compound);
        if (!decorate(s, r)) return false;
        return !s.decorated;
    } else if (s.type == SHAPE_TRIANGLE_MESH) {  // F_P0: the mesh index
        int m = (int)r[F_P0];
        if (!w || m < 0 || m >= (int)w->meshes.size()) return false;
        s.mesh = w->meshes[m].get();
        s.aabb = s.mesh->bounds;
    } else if (s.type == SHAPE_BOX) {
        s.half_extents = {r[F_P0], r[F_P0 + 1], r[F_P0 + 2]};
        s.convex_radius = r[F_P0 + 3];
        s.aabb = {neg(s.half_extents), s.half_extents};
    } else if (s.type == SHAPE_SPHERE) {
        s.radius = r[F_P0];
        s.aabb = {{-s.radius, -s.radius, -s.radius}, {s.radius, s.radius, s.radius}};
    } else if (s.type == SHAPE_EMPTY) {  // empty-shape.ts: a point of bounds, no mass
        s.aabb = {{0, 0, 0}, {0, 0, 0}};
    } else if (s.type == SHAPE_PLANE) {
        // plane.ts create :77-98: the normal normalised, the constant as given
        s.pn = normalize(V3{r[F_P0], r[F_P0 + 1], r[F_P0 + 2]});
        s.pc = r[F_P0 + 3];
        if (!(lensq(s.pn) > 0)) return false;
        s.aabb = plane_local_bounds(s.pn, s.pc, s.halfExtent);
    } else if (s.type == SHAPE_CYLINDER) {
        // cylinder.ts: half height along Y, radius, convex radius (update: 0 <= cr <= h, r)
        s.half_height = r[F_P0];
        s.radius = r[F_P0 + 1];
        s.convex_radius = r[F_P0 + 2];
        if (!(s.convex_radius >= 0 && s.half_height >= s.convex_radius && s.radius >= s.convex_radius)) return false;
        s.aabb = {{-s.radius, -s.half_height, -s.radius}, {s.radius, s.half_height, s.radius}};
    } else if (s.type == SHAPE_CAPSULE) {
        // capsule.ts:84-94: segment +-halfHeight on Y with radius r
        s.radius = r[F_P0];
        s.half_height = r[F_P0 + 1];
        double th = s.half_height + s.radius;
        s.aabb = {{-s.radius, -th, -s.radius}, {s.radius, th, s.radius}};
    } else {
        return false;
    }
    return decorate(s, r);
}

// computeMassProperties of OffsetCenterOfMass(Transformed(Scaled(leaf))): the leaf's mass
// and inertia, massProperties.scale (mass-properties.ts:59-112), rotate (:121-160) and
// translate (:168-205); I is row-major
static void decorated_mass(const double *r, const World *w, double &mass, double I[9]) {
    double row[F_COUNT];
    for (int k = 0; k < F_COUNT; k++) row[k] = r[k];
    for (int k = F_SCALE; k < F_COUNT; k++) row[k] = 0;  // the leaf alone
    Shape leaf;
    shape_from_row(leaf, row, w);
    V3 d;
    shape_mass(leaf, mass, d);
    double t[9] = {d.x, 0, 0, 0, d.y, 0, 0, 0, d.z};
    if (leaf.type == SHAPE_CONVEX_HULL)
        for (int k = 0; k < 9; k++) t[k] = leaf.hull->inertia[k] * leaf.density;
    V3 sc{r[F_SCALE], r[F_SCALE + 1], r[F_SCALE + 2]};
    if (sc.x == 0) sc.x = 1;
    if (sc.y == 0) sc.y = 1;
    if (sc.z == 0) sc.z = 1;
    if (sc.x != 1 || sc.y != 1 || sc.z != 1) {
        double half = 0.5 * (t[0] + t[4] + t[8]);
        double q0 = sc.x * sc.x * (half - t[0]), q1 = sc.y * sc.y * (half - t[4]), q2 = sc.z * sc.z * (half - t[8]);
        double ms = std::fabs(sc.x * sc.y * sc.z);
        double n[9] = {q1 + q2, sc.x * sc.y * t[1], sc.x * sc.z * t[2], sc.x * sc.y * t[3], q0 + q2, sc.y * sc.z * t[5],
                       sc.x * sc.z * t[6], sc.y * sc.z * t[7], q0 + q1};
        for (int k = 0; k < 9; k++) t[k] = n[k] * ms;
        mass *= ms;
    }
    Q4 tq{r[F_TROT], r[F_TROT + 1], r[F_TROT + 2], r[F_TROT + 3]};
    if (!(tq.x == 0 && tq.y == 0 && tq.z == 0 && tq.w == 0) && !(tq.x == 0 && tq.y == 0 && tq.z == 0 && tq.w == 1)) {
        M4 R4 = mat4_from_quat(tq);  // column-major: element (i, j) at m[4 j + i]
        double rt[9], o[9];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double acc = 0;
                for (int k = 0; k < 3; k++) acc += R4.m[4 * k + i] * t[3 * k + j];
                rt[3 * i + j] = acc;
            }
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double acc = 0;
                for (int k = 0; k < 3; k++) acc += rt[3 * i + k] * R4.m[4 * k + j];
                o[3 * i + j] = acc;
            }
        for (int k = 0; k < 9; k++) t[k] = o[k];
    }
    V3 off{r[F_COM_OFFSET], r[F_COM_OFFSET + 1], r[F_COM_OFFSET + 2]};
    if (off.x != 0 || off.y != 0 || off.z != 0) {
        double dd = dot(off, off), v[3] = {off.x, off.y, off.z};
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) t[3 * i + j] += mass * ((i == j ? dd : 0.0) - v[i] * v[j]);
    }
    for (int k = 0; k < 9; k++) I[k] = t[k];
}

// Mass properties of a body row (rigid-body.ts setRigidBody :309-326, updateShape :676-700,
// MotionProperties.setMassProperties motion-properties.ts:419-491); -1 when the row asks for a
// mass the shape cannot give
static int setup_mass(Body &b, const Shape &s, const double *r, const World *w) {
    double mass;
    V3 idiag;
    shape_mass(s, mass, idiag);
    // meshes and planes have no mass (triangle-mesh.ts:153-158, plane.ts:120-122)
    if ((s.type == SHAPE_TRIANGLE_MESH || s.type == SHAPE_PLANE) && b.motion == DYNAMIC) return -1;
    const int massMode = (int)r[F_MASS_MODE];
    if (massMode != 0 && b.motion != STATIC && s.type != SHAPE_TRIANGLE_MESH && s.type != SHAPE_PLANE) {
        // rigid-body.ts setRigidBody :309-326 and updateShape :676-700: a given mass scales the
        // shape's inertia (scaleToMass mass-properties.ts:220-240), or mass and inertia given
        double I[9];
        if (s.decorated) {
            decorated_mass(r, w, mass, I);
        } else if (s.type == SHAPE_CONVEX_HULL) {
            for (int k = 0; k < 9; k++) I[k] = s.hull->inertia[k] * s.density;
        } else if (s.type == SHAPE_COMPOUND) {
            for (int k = 0; k < 9; k++) I[k] = s.compound->inertia[k];
        } else {
            double t[9] = {idiag.x, 0, 0, 0, idiag.y, 0, 0, 0, idiag.z};
            for (int k = 0; k < 9; k++) I[k] = t[k];
        }
        if (massMode == 1) {
            double m = r[F_MASS];
            if (mass > 0)
                for (int k = 0; k < 9; k++) I[k] *= m / mass;
            mass = m;
        } else {
            const double *t = r + F_INERTIA;
            double g[9] = {t[0], t[1], t[2], t[1], t[3], t[4], t[2], t[4], t[5]};
            for (int k = 0; k < 9; k++) I[k] = g[k];
            mass = r[F_MASS];
        }
        if ((b.dof & 7) != 0 && !(mass > 0)) return -1;  // setMassProperties asserts a mass
        set_mass_properties_tensor(b, mass, I, 1.0);
    } else if (b.motion != STATIC && s.type != SHAPE_TRIANGLE_MESH && s.type != SHAPE_PLANE) {
        if ((b.dof & 7) != 0 && !(mass > 0)) return -1;  // an empty shape needs a given mass
        if (s.decorated) {
            double I[9];
            decorated_mass(r, w, mass, I);
            set_mass_properties_tensor(b, mass, I, 1.0);
        } else if (s.type == SHAPE_CONVEX_HULL) {
            set_mass_properties_tensor(b, mass, s.hull->inertia, s.density);
        } else if (s.type == SHAPE_COMPOUND) {
            set_mass_properties_tensor(b, mass, s.compound->inertia, 1.0);
        } else {
            set_mass_properties(b, mass, idiag);
        }
    }
    return 0;
}

int orc_add_bodies(void *wp, const double *rows, int n) {
    World &w = *(World *)wp;
    for (int i = 0; i < n; i++) {
        const double *r = rows + (size_t)i * F_COUNT;
        Body b;
        b.index = (int)w.bodies.size();
        int seq = w.nextSequence;
        w.nextSequence = (w.nextSequence + 1) & ((1 << 20) - 1);
        b.id = (int64_t)b.index + (int64_t)seq * 4294967296LL;
        Shape &s = b.shape;
        if (!shape_from_row(s, r, &w)) return -1;
        b.position = {r[F_POS], r[F_POS + 1], r[F_POS + 2]};
        b.quat = {r[F_QUAT], r[F_QUAT + 1], r[F_QUAT + 2], r[F_QUAT + 3]};
        b.motion = (int)r[F_MOTION];
        b.linvel = {r[F_LINVEL], r[F_LINVEL + 1], r[F_LINVEL + 2]};
        b.angvel = {r[F_ANGVEL], r[F_ANGVEL + 1], r[F_ANGVEL + 2]};
        b.friction = r[F_FRICTION];
        b.restitution = r[F_RESTITUTION];
        b.objectLayer = (int)r[F_LAYER];
        b.gravityFactor = r[F_GRAVITY_FACTOR];
        b.linDamp = r[F_LIN_DAMP];
        b.angDamp = r[F_ANG_DAMP];
        b.allowSleeping = r[F_ALLOW_SLEEP] != 0;
        b.linearCast = r[F_MOTION_QUALITY] == 1;
        if (b.linearCast && s.type == SHAPE_COMPOUND) return -1;  // a cast compound is not restated
        b.velOverride = (int)r[F_VEL_OVERRIDE];
        b.posOverride = (int)r[F_POS_OVERRIDE];
        b.groups = (uint32_t)r[F_GROUPS];
        b.mask = (uint32_t)r[F_MASK];
        if (setup_mass(b, s, r, &w) != 0) return -1;
        update_com(b);
        update_aabb(b);
        w.bodies.push_back(b);
        Body &bb = w.bodies.back();
        if (bb.motion == DYNAMIC) reset_sleep_timer(bb);
        if (bb.motion != STATIC && !bb.sleeping) add_active(w, bb);
    }
    return 0;
}

int orc_body_count(void *wp) { return (int)((World *)wp)->bodies.size(); }

// Hinge joint (hinge-constraint.ts create), 36 doubles:
//  0 bodyA, 1 bodyB, 2-4 pointA, 5-7 pointB, 8-10 hingeAxisA, 11-13 hingeAxisB, 14-16 normalAxisA,
//  17-19 normalAxisB, 20 space (0 world, 1 local), 21 limitsMin, 22 limitsMax,
//  23-25 limits spring (mode, frequency or stiffness, damping), 26 maxFrictionTorque,
//  27 motor state (0 off, 1 velocity, 2 position), 28 target angular velocity, 29 target angle,
//  30-32 motor spring (mode, frequency or stiffness, damping), 33 min torque, 34 max torque,
//  35 priority.  Returns the joint index or -1.
int orc_add_hinge(void *wp, const double *d) {
    World &w = *(World *)wp;
    int a = (int)d[0], b = (int)d[1];
    if (a < 0 || b < 0 || a >= (int)w.bodies.size() || b >= (int)w.bodies.size()) return -1;
    const Body &A = w.bodies[a], &B = w.bodies[b];
    HingeJoint j;
    j.a = a;
    j.b = b;
    j.index = (int)w.joints.size();
    j.priority = (int)d[35];
    j.velOverride = (int)d[36];
    j.posOverride = (int)d[37];
    V3 pA{d[2], d[3], d[4]}, pB{d[5], d[6], d[7]};
    V3 h1 = normalize(V3{d[8], d[9], d[10]}), h2 = normalize(V3{d[11], d[12], d[13]});
    V3 n1 = normalize(V3{d[14], d[15], d[16]}), n2 = normalize(V3{d[17], d[18], d[19]});
    if ((int)d[20] == 0) {
        Q4 iqA = qconj(A.quat), iqB = qconj(B.quat);
        j.lp1 = rotate(iqA, sub(pA, A.com));
        j.lp2 = rotate(iqB, sub(pB, B.com));
        j.lh1 = rotate(iqA, h1);
        j.lh2 = rotate(iqB, h2);
        j.ln1 = rotate(iqA, n1);
        j.ln2 = rotate(iqB, n2);
        Q4 r0 = inv_initial_orientation_xz(n1, h1, n2, h2);
        j.invInitial = qmul(qmul(iqB, r0), A.quat);
    } else {
        j.lp1 = pA;
        j.lp2 = pB;
        j.lh1 = h1;
        j.lh2 = h2;
        j.ln1 = n1;
        j.ln2 = n2;
        j.invInitial = inv_initial_orientation_xz(rotate(A.quat, n1), rotate(A.quat, h1), rotate(B.quat, n2),
                                                  rotate(B.quat, h2));
    }
    double mn = d[21], mx = d[22];
    if (mn <= -M_PI && mx >= M_PI) {
        j.hasLimits = false;
        j.limitsMin = -M_PI;
        j.limitsMax = M_PI;
    } else {
        j.hasLimits = true;
        j.limitsMin = std::max(mn, -M_PI);
        j.limitsMax = std::min(mx, M_PI);
    }
    j.limitsSpring = {(int)d[23], d[24], d[25]};
    j.maxFrictionTorque = d[26];
    j.motorSpring = {(int)d[30], d[31], d[32]};
    j.minTorqueLimit = d[33];
    j.maxTorqueLimit = d[34];
    // setMotorState / setTargetAngularVelocity / setTargetAngle (hinge-constraint.ts)
    j.motorState = (int)d[27];
    j.targetAngularVelocity = d[28];
    j.targetAngle = j.hasLimits ? std::max(j.limitsMin, std::min(j.limitsMax, d[29])) : d[29];
    w.joints.push_back(j);
    return j.index;
}
void orc_set_skip_joint_pairs(void *wp, int on) { ((World *)wp)->skipJointPairs = on != 0; }

// A convex hull shape given by its data (the hull construction itself is not part of the
// step): np points and shrunk points (3 doubles each, relative to the centre of mass), nf faces
// (first face vertex, count), nv face vertex indices, planes (nf x 4: normal, constant),
// scal = convex radius, volume, com xyz, inertia (9, unit density, row-major), bounds min xyz,
// max xyz (20 doubles).  Returns the hull index.
int orc_add_hull(void *wp, int np, const double *points, const double *shrunk, int nf, const int *faces, int nv,
                 const int *vidx, const double *planes, const double *scal) {
    World &w = *(World *)wp;
    auto h = std::make_unique<HullData>();
    for (int i = 0; i < np; i++) {
        h->points.push_back({points[3 * i], points[3 * i + 1], points[3 * i + 2]});
        h->shrunk.push_back({shrunk[3 * i], shrunk[3 * i + 1], shrunk[3 * i + 2]});
    }
    for (int f = 0; f < nf; f++) {
        h->face_first.push_back(faces[2 * f]);
        h->face_count.push_back(faces[2 * f + 1]);
        h->plane_n.push_back({planes[4 * f], planes[4 * f + 1], planes[4 * f + 2]});
        h->plane_c.push_back(planes[4 * f + 3]);
    }
    for (int k = 0; k < nv; k++) h->vidx.push_back(vidx[k]);
    h->convex_radius = scal[0];
    h->volume = scal[1];
    h->com = {scal[2], scal[3], scal[4]};
    for (int k = 0; k < 9; k++) h->inertia[k] = scal[5 + k];
    h->bounds = {{scal[14], scal[15], scal[16]}, {scal[17], scal[18], scal[19]}};
    w.hulls.push_back(std::move(h));
    return (int)w.hulls.size() - 1;
}

// Swing-twist joint (swing-twist-constraint.ts create :180-296), 47 doubles:
//  0 bodyA, 1 bodyB, 2-4 position1, 5-7 position2, 8-10 twistAxis1, 11-13 planeAxis1,
//  14-16 twistAxis2, 17-19 planeAxis2, 20 space (0 world, 1 local), 21 swingType (0 cone, 1 pyramid),
//  22 normalHalfConeAngle, 23 planeHalfConeAngle, 24 twistMinAngle, 25 twistMaxAngle,
//  26 maxFrictionTorque, 27 swing motor state, 28 twist motor state, 29-31 target angular velocity,
//  32-35 target orientation (x y z w, constraint space), 36-38 swing motor spring (mode, f, d),
//  39-41 twist motor spring, 42-43 swing motor torque limits (min, max), 44-45 twist motor torque
//  limits, 46 priority.  Returns the joint index or -1.
// a triangle mesh as built: nv vertices (x y z), nt triangles (a b c active-edge bits), nn
// nodes (8 each: min, max, right child node or first triangle, axis or -(count + 1))
int orc_add_mesh(void *wp, int nv, const double *verts, int nt, const int *tris, int nn, const double *nodes) {
    World &w = *(World *)wp;
    auto m = std::make_unique<MeshData>();
    for (int i = 0; i < nv; i++) m->verts.push_back({verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]});
    for (int t = 0; t < nt; t++) m->tris.push_back({tris[4 * t], tris[4 * t + 1], tris[4 * t + 2], tris[4 * t + 3]});
    for (int k = 0; k < nn; k++) {
        std::array<double, 8> nd;
        for (int j = 0; j < 8; j++) nd[j] = nodes[8 * k + j];
        m->nodes.push_back(nd);
    }
    unsigned maxi = nt > 0 ? (unsigned)(nt - 1) : 0u;
    m->subBits = maxi == 0 ? 0 : 32 - __builtin_clz(maxi);
    if (nn > 0) m->bounds = {{nodes[0], nodes[1], nodes[2]}, {nodes[3], nodes[4], nodes[5]}};
    w.meshes.push_back(std::move(m));
    return (int)w.meshes.size() - 1;
}

// compound.ts create / update (:43-57, :143-147) and computeMassProperties (:177-230): children
// given as 13 doubles (shape type, 4 shape params, position xyz, quaternion xyzw, density);
// convex children only (sphere, box, capsule, cylinder, a hull of this world).  Returns the
// compound index, or -1.
static V3 compound_com(const CompoundData &c) {
    // computeCompoundCenterOfMass :110-141: the children's centres of mass weighted by mass
    V3 acc{0, 0, 0};
    double total = 0;
    for (size_t i = 0; i < c.shapes.size(); i++) {
        double m;
        V3 d;
        shape_mass(c.shapes[i], m, d);
        acc = add(acc, scale(add(c.pos[i], rotate(c.rot[i], c.shapes[i].com)), m));
        total += m;
    }
    return total > 0 ? scale(acc, 1.0 / total) : V3{0, 0, 0};
}
int orc_add_compound(void *wp, const double *rows, int n) {
    World &w = *(World *)wp;
    if (n <= 0) return -1;
    auto c = std::make_unique<CompoundData>();
    for (int i = 0; i < n; i++) {
        const double *q = rows + 13 * i;
        double row[F_COUNT] = {};
        row[F_SHAPE] = q[0];
        for (int k = 0; k < 4; k++) row[F_P0 + k] = q[1 + k];
        row[F_DENSITY] = q[12];
        Shape ch;
        if (!shape_from_row(ch, row, &w)) return -1;
        if (ch.type != SHAPE_SPHERE && ch.type != SHAPE_BOX && ch.type != SHAPE_CAPSULE && ch.type != SHAPE_CYLINDER &&
            ch.type != SHAPE_CONVEX_HULL)
            return -1;
        c->shapes.push_back(ch);
        c->pos.push_back({q[5], q[6], q[7]});
        c->rot.push_back(Q4{q[8], q[9], q[10], q[11]});
    }
    unsigned maxi = (unsigned)(n - 1);
    c->subBits = maxi == 0 ? 0 : 32 - __builtin_clz(maxi);
    c->innerRadius = std::numeric_limits<double>::max();
    for (const Shape &ch : c->shapes) c->innerRadius = std::min(c->innerRadius, inner_radius(ch));
    const V3 com = compound_com(*c);
    double I[9] = {};
    c->mass = 0;
    for (int i = 0; i < n; i++) {
        const Shape &ch = c->shapes[i];
        double m;
        V3 d;
        shape_mass(ch, m, d);
        double t[9] = {d.x, 0, 0, 0, d.y, 0, 0, 0, d.z};
        if (ch.type == SHAPE_CONVEX_HULL)
            for (int k = 0; k < 9; k++) t[k] = ch.hull->inertia[k] * ch.density;
        // massProperties.rotate (mass-properties.ts:121-160): R I R^T
        M4 R4 = mat4_from_quat(c->rot[i]);  // column-major: element (i, j) at m[4 j + i]
        double rt[9], o[9];
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                double acc = 0;
                for (int k = 0; k < 3; k++) acc += R4.m[4 * k + a] * t[3 * k + b];
                rt[3 * a + b] = acc;
            }
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                double acc = 0;
                for (int k = 0; k < 3; k++) acc += rt[3 * a + k] * R4.m[4 * k + b];
                o[3 * a + b] = acc;
            }
        // massProperties.translate (:168-205) by the child's centre of mass from the compound's
        V3 off = sub(add(c->pos[i], rotate(c->rot[i], ch.com)), com);
        double dd = dot(off, off), v[3] = {off.x, off.y, off.z};
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) I[3 * a + b] += o[3 * a + b] + m * ((a == b ? dd : 0.0) - v[a] * v[b]);
        c->mass += m;
    }
    for (int k = 0; k < 9; k++) c->inertia[k] = I[k];
    w.compounds.push_back(std::move(c));
    return (int)w.compounds.size() - 1;
}

int orc_add_swing_twist(void *wp, const double *d) {
    World &w = *(World *)wp;
    int a = (int)d[0], b = (int)d[1];
    if (a < 0 || b < 0 || a >= (int)w.bodies.size() || b >= (int)w.bodies.size()) return -1;
    const Body &A = w.bodies[a], &B = w.bodies[b];
    SwingTwistJoint j;
    j.a = a;
    j.b = b;
    j.index = (int)w.swings.size();
    j.priority = (int)d[46];
    j.velOverride = (int)d[47];
    j.posOverride = (int)d[48];
    V3 t1 = normalize(V3{d[8], d[9], d[10]}), p1 = normalize(V3{d[11], d[12], d[13]});
    V3 t2 = normalize(V3{d[14], d[15], d[16]}), p2 = normalize(V3{d[17], d[18], d[19]});
    V3 n1 = cross(p1, t1), n2 = cross(p2, t2);
    // constraint space X = twist, Y = normal, Z = plane (columns of the rotation)
    M3 m1, m2;
    V3 c1[3] = {t1, n1, p1}, c2[3] = {t2, n2, p2};
    for (int c = 0; c < 3; c++) {
        m1.m[c][0] = c1[c].x;
        m1.m[c][1] = c1[c].y;
        m1.m[c][2] = c1[c].z;
        m2.m[c][0] = c2[c].x;
        m2.m[c][1] = c2[c].y;
        m2.m[c][2] = c2[c].z;
    }
    j.c2b1 = quat_from_m3(m1);
    j.c2b2 = quat_from_m3(m2);
    V3 pos1{d[2], d[3], d[4]}, pos2{d[5], d[6], d[7]};
    if ((int)d[20] == 0) {
        Q4 iqA = qconj(A.quat), iqB = qconj(B.quat);
        j.lp1 = rotate(iqA, sub(pos1, A.com));
        j.lp2 = rotate(iqB, sub(pos2, B.com));
        j.c2b1 = qmul(iqA, j.c2b1);
        j.c2b2 = qmul(iqB, j.c2b2);
    } else {
        j.lp1 = pos1;
        j.lp2 = pos2;
    }
    j.normalHalfCone = d[22];
    j.planeHalfCone = d[23];
    j.twistMin = d[24];
    j.twistMax = d[25];
    j.st.swingType = (int)d[21];
    swing_update_limits(j);
    j.maxFrictionTorque = d[26];
    j.swingMotorState = (int)d[27];
    j.twistMotorState = (int)d[28];
    j.targetAngularVelocity = {d[29], d[30], d[31]};
    // setTargetOrientationCS :405-416: clamped into the limits
    Q4 to{d[32], d[33], d[34], d[35]}, sw, tw;
    get_swing_twist(to, sw, tw);
    j.targetOrientation = clamp_swing_twist(j.st, sw, tw) != 0 ? qmul(sw, tw) : to;
    j.swingMotorSpring = {(int)d[36], d[37], d[38]};
    j.twistMotorSpring = {(int)d[39], d[40], d[41]};
    j.swingMinTorque = d[42];
    j.swingMaxTorque = d[43];
    j.twistMinTorque = d[44];
    j.twistMaxTorque = d[45];
    w.swings.push_back(j);
    return j.index;
}
// Point, distance, fixed, cone and slider joints (the create functions of point-, distance-,
// fixed-, cone- and slider-constraint.ts) from a flat record of doubles:
//   0 bodyA, 1 bodyB, 2 space (0 world, 1 local), 3 priority, 4 velocity override,
//   5 position override, 6 enabled, then per type:
//   point     7-9 pointA, 10-12 pointB
//   distance  7-9 pointA, 10-12 pointB, 13 minDistance, 14 maxDistance (< 0: unset),
//             15-17 spring (mode, frequency or stiffness, damping)
//   fixed     7 autoDetectPoint, 8-10 point1, 11-13 point2, 14-16 axisX1, 17-19 axisY1,
//             20-22 axisX2, 23-25 axisY2
//   cone      7-9 pointA, 10-12 pointB, 13-15 twistAxisA, 16-18 twistAxisB, 19 halfConeAngle
//   slider    7 autoDetectPoint, 8-10 pointA, 11-13 pointB, 14-16 sliderAxisA, 17-19 sliderAxisB,
//             20-22 normalAxisA, 23-25 normalAxisB, 26 limitsMin, 27 limitsMax,
//             28-30 limits spring, 31 maxFrictionForce, 32-34 motor spring, 35 min force,
//             36 max force, 37 motor state, 38 target velocity, 39 target position
//             (37-39 through setMotorState / setTargetVelocity / setTargetPosition)
//   six-DOF   7-9 position1, 10-12 position2, 13-15 axisX1, 16-18 axisY1, 19-21 axisX2, 22-24 axisY2,
//             25 swingType, 26-31 limitMin, 32-37 limitMax, 38-43 maxFriction, 44-52 limits
//             springs (3 x mode, frequency or stiffness, damping), 53-70 motor springs (6 x 3),
//             71-76 motor min force, 77-82 motor max force, 83-88 motor states, 89-91 target
//             velocity, 92-94 target angular velocity, 95-97 target position, 98-101 target
//             orientation (83-101 through setMotorState and the setTarget*CS setters)
// Returns the joint's per-type index, or -1.
int orc_add_joint(void *wp, int type, const double *d) {
    World &w = *(World *)wp;
    int a = (int)d[0], b = (int)d[1];
    if (a < 0 || b < 0 || a >= (int)w.bodies.size() || b >= (int)w.bodies.size()) return -1;
    const Body &A = w.bodies[a], &B = w.bodies[b];
    const bool world_space = (int)d[2] == 0;
    const Q4 iqA = qconj(A.quat), iqB = qconj(B.quat);
    auto base = [&](JointBase &j, int index) {
        j.a = a;
        j.b = b;
        j.index = index;
        j.priority = (int)d[3];
        j.velOverride = (int)d[4];
        j.posOverride = (int)d[5];
        j.enabled = d[6] != 0;
    };
    auto v = [&](int k) { return V3{d[k], d[k + 1], d[k + 2]}; };
    // the anchor of autoDetectPoint: the inverse-mass-weighted mean of the centres of mass
    auto anchor = [&]() {
        double im = A.invMass + B.invMass;
        if (im == 0) return A.com;
        return add(scale(A.com, A.invMass / im), scale(B.com, B.invMass / im));
    };
    switch (type) {
    case JT_POINT: {
        PointJoint j;
        base(j, (int)w.points.size());
        if (world_space) {
            j.lp1 = rotate(iqA, sub(v(7), A.com));
            j.lp2 = rotate(iqB, sub(v(10), B.com));
        } else {
            j.lp1 = v(7);
            j.lp2 = v(10);
        }
        w.points.push_back(j);
        return j.index;
    }
    case JT_DISTANCE: {  // distance-constraint.ts create :121-214
        DistanceJoint j;
        base(j, (int)w.distances.size());
        if (world_space) {
            j.lp1 = rotate(iqA, sub(v(7), A.com));
            j.lp2 = rotate(iqB, sub(v(10), B.com));
            j.wp1 = v(7);
            j.wp2 = v(10);
        } else {
            j.lp1 = v(7);
            j.lp2 = v(10);
            j.wp1 = add(rotate(A.quat, j.lp1), A.com);
            j.wp2 = add(rotate(B.quat, j.lp2), B.com);
        }
        double dist = len(sub(j.wp2, j.wp1));
        double mn = d[13], mx = d[14];
        if (mn < 0 && mx < 0) {
            j.minDistance = j.maxDistance = dist;
        } else {
            j.minDistance = mn < 0 ? std::min(dist, mx) : mn;
            j.maxDistance = mx < 0 ? std::max(dist, mn) : mx;
        }
        j.spring = {(int)d[15], d[16], d[17]};
        w.distances.push_back(j);
        return j.index;
    }
    case JT_FIXED: {  // fixed-constraint.ts create :131-262
        FixedJoint j;
        base(j, (int)w.fixeds.size());
        Q4 r0 = inv_initial_orientation_xy(normalize(v(14)), normalize(v(17)), normalize(v(20)), normalize(v(23)));
        if (world_space) {
            if (d[7] != 0) {
                V3 p = anchor();
                j.lp1 = rotate(iqA, sub(p, A.com));
                j.lp2 = rotate(iqB, sub(p, B.com));
            } else {
                j.lp1 = rotate(iqA, sub(v(8), A.com));
                j.lp2 = rotate(iqB, sub(v(11), B.com));
            }
            j.invInitial = qmul(qmul(iqB, r0), A.quat);
        } else {
            j.lp1 = v(8);
            j.lp2 = v(11);
            j.invInitial = r0;
        }
        w.fixeds.push_back(j);
        return j.index;
    }
    case JT_CONE: {  // cone-constraint.ts create :150-230
        ConeJoint j;
        base(j, (int)w.cones.size());
        V3 t1 = normalize(v(13)), t2 = normalize(v(16));
        j.cosHalfCone = std::cos(d[19]);
        // getNormalizedPerpendicular :118-136
        double ax = std::fabs(t1.x), ay = std::fabs(t1.y), az = std::fabs(t1.z);
        V3 perp = (ax <= ay && ax <= az) ? V3{0, -t1.z, t1.y} : (ay <= az ? V3{t1.z, 0, -t1.x} : V3{-t1.y, t1.x, 0});
        j.wRotAxis = normalize(perp);
        if (world_space) {
            j.lp1 = rotate(iqA, sub(v(7), A.com));
            j.lp2 = rotate(iqB, sub(v(10), B.com));
            j.lt1 = rotate(iqA, t1);
            j.lt2 = rotate(iqB, t2);
        } else {
            j.lp1 = v(7);
            j.lp2 = v(10);
            j.lt1 = t1;
            j.lt2 = t2;
            j.wRotAxis = rotate(A.quat, j.wRotAxis);
        }
        w.cones.push_back(j);
        return j.index;
    }
    case JT_SLIDER: {  // slider-constraint.ts create :261-412 and the setters :488-525
        SliderJoint j;
        base(j, (int)w.sliders.size());
        V3 s1 = normalize(v(14)), s2 = normalize(v(17)), n1 = normalize(v(20)), n2 = normalize(v(23));
        // getInvInitialOrientationXY :203-259 (exact component test with eps 1e-6)
        const double eps = 1e-6;
        Q4 r0{0, 0, 0, 1};
        if (!(std::fabs(s1.x - s2.x) < eps && std::fabs(s1.y - s2.y) < eps && std::fabs(s1.z - s2.z) < eps &&
              std::fabs(n1.x - n2.x) < eps && std::fabs(n1.y - n2.y) < eps && std::fabs(n1.z - n2.z) < eps))
            r0 = qmul(axes_to_quat(s2, n2), qconj(axes_to_quat(s1, n1)));
        if (world_space) {
            if (d[7] != 0) {
                V3 p = anchor();
                j.lp1 = rotate(iqA, sub(p, A.com));
                j.lp2 = rotate(iqB, sub(p, B.com));
            } else {
                j.lp1 = rotate(iqA, sub(v(8), A.com));
                j.lp2 = rotate(iqB, sub(v(11), B.com));
            }
            j.lSlider1 = normalize(rotate(iqA, s1));
            j.lNormal1 = normalize(rotate(iqA, n1));
            j.lNormal2 = cross(j.lSlider1, j.lNormal1);
            j.invInitial = qmul(qmul(iqB, r0), A.quat);
        } else {
            j.lp1 = v(8);
            j.lp2 = v(11);
            j.lSlider1 = s1;
            j.lNormal1 = n1;
            j.lNormal2 = cross(j.lSlider1, j.lNormal1);
            j.invInitial = r0;
        }
        j.limitsMin = std::min(d[26], 0.0);
        j.limitsMax = std::max(d[27], 0.0);
        j.hasLimits = j.limitsMin != -1.0 / 0.0 || j.limitsMax != 1.0 / 0.0;
        j.limitsSpring = {(int)d[28], d[29], d[30]};
        j.maxFrictionForce = d[31];
        j.motorSpring = {(int)d[32], d[33], d[34]};
        j.minForceLimit = d[35];
        j.maxForceLimit = d[36];
        j.motorState = (int)d[37];
        j.targetVelocity = d[38];
        j.targetPosition = j.hasLimits ? std::max(j.limitsMin, std::min(j.limitsMax, d[39])) : d[39];
        w.sliders.push_back(j);
        return j.index;
    }
    case JT_SIX_DOF: {  // six-dof-constraint.ts create :335-480 and the setters :1262-1299
        SixDofJoint j;
        base(j, (int)w.sixdofs.size());
        auto frame = [&](V3 x, V3 y) { return axes_to_quat(normalize(x), normalize(y)); };
        j.c2b1 = frame(v(13), v(16));
        j.c2b2 = frame(v(19), v(22));
        if (world_space) {
            j.lp1 = rotate(iqA, sub(v(7), A.com));
            j.lp2 = rotate(iqB, sub(v(10), B.com));
            j.c2b1 = qmul(iqA, j.c2b1);
            j.c2b2 = qmul(iqB, j.c2b2);
        } else {
            j.lp1 = v(7);
            j.lp2 = v(10);
        }
        j.swingType = (int)d[25];
        for (int k = 0; k < 6; k++) {
            j.limitMin[k] = d[26 + k];
            j.limitMax[k] = d[32 + k];
            j.maxFriction[k] = d[38 + k];
            j.motorSpring[k] = {(int)d[53 + 3 * k], d[54 + 3 * k], d[55 + 3 * k]};
            j.motorMinForce[k] = d[71 + k];
            j.motorMaxForce[k] = d[77 + k];
            j.motorState[k] = (int)d[83 + k];
        }
        for (int k = 0; k < 3; k++) j.limitsSpring[k] = {(int)d[44 + 3 * k], d[45 + 3 * k], d[46 + 3 * k]};
        sd_update(j);
        j.targetVelocity = v(89);
        j.targetAngularVelocity = v(92);
        j.targetPosition = v(95);
        Q4 to{d[98], d[99], d[100], d[101]}, sw, tw;  // setTargetOrientationCS: clamped into the limits
        get_swing_twist(to, sw, tw);
        clamp_swing_twist(j.st, sw, tw);
        j.targetOrientation = qmul(sw, tw);
        w.sixdofs.push_back(j);
        return j.index;
    }
    default: return -1;
    }
}
// Total impulses of one joint (getTotalLambda* of each type): point 3 (point part),
// distance 1, fixed 6 (point, rotation), cone 4 (point, angle), slider 2 + 3 + 1 + 1
// (position, rotation, limits, motor), six-DOF 18 (3 translation rows, point, rotation, swing Y,
// swing Z, twist, 3 translation motors, 3 rotation motors).  Returns the count written, or -1.
int orc_get_joint_lambdas(void *wp, int type, int index, double *out) {
    World &w = *(World *)wp;
    auto put3 = [&](int k, V3 a) {
        out[k] = a.x;
        out[k + 1] = a.y;
        out[k + 2] = a.z;
    };
    switch (type) {
    case JT_POINT:
        if (index < 0 || index >= (int)w.points.size()) return -1;
        put3(0, w.points[index].point.totalLambda);
        return 3;
    case JT_DISTANCE:
        if (index < 0 || index >= (int)w.distances.size()) return -1;
        out[0] = w.distances[index].axis.totalLambda;
        return 1;
    case JT_FIXED:
        if (index < 0 || index >= (int)w.fixeds.size()) return -1;
        put3(0, w.fixeds[index].point.totalLambda);
        put3(3, w.fixeds[index].rot.totalLambda);
        return 6;
    case JT_CONE:
        if (index < 0 || index >= (int)w.cones.size()) return -1;
        put3(0, w.cones[index].point.totalLambda);
        out[3] = w.cones[index].angle.totalLambda;
        return 4;
    case JT_SLIDER: {
        if (index < 0 || index >= (int)w.sliders.size()) return -1;
        const SliderJoint &j = w.sliders[index];
        out[0] = j.pos.totalLambda[0];
        out[1] = j.pos.totalLambda[1];
        put3(2, j.rot.totalLambda);
        out[5] = j.limits.totalLambda;
        out[6] = j.motor.totalLambda;
        return 7;
    }
    case JT_SIX_DOF: {
        if (index < 0 || index >= (int)w.sixdofs.size()) return -1;
        const SixDofJoint &j = w.sixdofs[index];
        for (int k = 0; k < 3; k++) out[k] = j.translation[k].totalLambda;
        put3(3, j.point.totalLambda);
        put3(6, j.rot.totalLambda);
        out[9] = j.st.swingY.totalLambda;
        out[10] = j.st.swingZ.totalLambda;
        out[11] = j.st.twist.totalLambda;
        for (int k = 0; k < 3; k++) out[12 + k] = j.motorTranslation[k].totalLambda;
        for (int k = 0; k < 3; k++) out[15 + k] = j.motorRotation[k].totalLambda;
        return 18;
    }
    default: return -1;
    }
}
// getCurrentPosition slider-constraint.ts:460-476 of one slider, or NaN
double orc_slider_position(void *wp, int index) {
    World &w = *(World *)wp;
    if (index < 0 || index >= (int)w.sliders.size()) return 0.0 / 0.0;
    const SliderJoint &j = w.sliders[index];
    const Body &A = w.bodies[j.a], &B = w.bodies[j.b];
    V3 u = sub(add(sub(B.com, A.com), rotate(B.quat, j.lp2)), rotate(A.quat, j.lp1));
    return dot(u, rotate(A.quat, j.lSlider1));
}

// Contact events of the last step, 3 int64 per event (type, body index A, body index B); returns the count.
int orc_get_events(void *wp, int64_t *out, int cap) {
    const World &w = *(World *)wp;
    int n = (int)w.events.size();
    for (int i = 0; i < n && i < cap; i++)
        for (int k = 0; k < 3; k++) out[3 * i + k] = w.events[i][k];
    return n;
}
void orc_set_coloured_order(void *wp, int on) { ((World *)wp)->colouredOrder = on != 0; }
int orc_reordered_islands(void *wp) { return ((World *)wp)->reorderedIslands; }

// state rows: pos3 quat4 linvel3 angvel3 com3 sleeping1 = 17 doubles
int orc_get_state(void *wp, double *out) {
    World &w = *(World *)wp;
    for (size_t i = 0; i < w.bodies.size(); i++) {
        const Body &b = w.bodies[i];
        double *o = out + i * 17;
        o[0] = b.position.x;
        o[1] = b.position.y;
        o[2] = b.position.z;
        o[3] = b.quat.x;
        o[4] = b.quat.y;
        o[5] = b.quat.z;
        o[6] = b.quat.w;
        o[7] = b.linvel.x;
        o[8] = b.linvel.y;
        o[9] = b.linvel.z;
        o[10] = b.angvel.x;
        o[11] = b.angvel.y;
        o[12] = b.angvel.z;
        o[13] = b.com.x;
        o[14] = b.com.y;
        o[15] = b.com.z;
        o[16] = b.sleeping ? 1.0 : 0.0;
    }
    return 0;
}

// Overwrite pose and velocity (rigidBody.setTransform + setLinearVelocity /
// setAngularVelocity without waking semantics beyond the reference's own).
int orc_set_state(void *wp, const double *in) {
    World &w = *(World *)wp;
    for (size_t i = 0; i < w.bodies.size(); i++) {
        Body &b = w.bodies[i];
        const double *o = in + i * 17;
        b.position = {o[0], o[1], o[2]};
        b.quat = {o[3], o[4], o[5], o[6]};
        b.linvel = {o[7], o[8], o[9]};
        b.angvel = {o[10], o[11], o[12]};
        set_transform(b);
    }
    return 0;
}

int orc_step(void *wp, double dt, int n_steps) {
    World &w = *(World *)wp;
    for (int i = 0; i < n_steps; i++) step(w, dt);
    return 0;
}

int orc_pair_count(void *wp) { return (int)((World *)wp)->pairs.size(); }
int orc_get_pairs(void *wp, int *out) {
    World &w = *(World *)wp;
    for (size_t i = 0; i < w.pairs.size(); i++) {
        out[2 * i] = w.pairs[i].first;
        out[2 * i + 1] = w.pairs[i].second;
    }
    return 0;
}

// AABBs (min3 max3) per body
int orc_get_aabbs(void *wp, double *out) {
    World &w = *(World *)wp;
    for (size_t i = 0; i < w.bodies.size(); i++) {
        const Box3 &a = w.bodies[i].aabb;
        double *o = out + 6 * i;
        o[0] = a.mn.x;
        o[1] = a.mn.y;
        o[2] = a.mn.z;
        o[3] = a.mx.x;
        o[4] = a.mx.y;
        o[5] = a.mx.z;
    }
    return 0;
}

// Manifolds created during the last step (after id ordering).  Row layout:
// bodyA, bodyB, n, normal3, depth, then 4 x (pointA3 pointB3) world space = 32 doubles.
int orc_manifold_count(void *wp) { return (int)((World *)wp)->manifolds.size(); }
int orc_get_manifolds(void *wp, double *out) {
    World &w = *(World *)wp;
    for (size_t i = 0; i < w.manifolds.size(); i++) {
        const Manifold &m = w.manifolds[i];
        double *o = out + 32 * i;
        o[0] = w.manifoldBodies[i].first;
        o[1] = w.manifoldBodies[i].second;
        o[2] = m.n;
        o[3] = m.normal.x;
        o[4] = m.normal.y;
        o[5] = m.normal.z;
        o[6] = m.depth;
        o[7] = i < w.manifoldLambda.size() ? w.manifoldLambda[i] : 0;
        for (int k = 0; k < 4; k++) {
            double *p = o + 8 + 6 * k;
            if (k < m.n) {
                V3 a = add(m.base, m.relA[k]), b = add(m.base, m.relB[k]);
                p[0] = a.x;
                p[1] = a.y;
                p[2] = a.z;
                p[3] = b.x;
                p[4] = b.y;
                p[5] = b.z;
            } else {
                for (int j = 0; j < 6; j++) p[j] = 0;
            }
        }
    }
    return 0;
}

// Island statistics of the last step: number of islands with contacts.
int orc_island_count(void *wp) { return (int)((World *)wp)->islands.size(); }
// Island.numVelocitySteps / numPositionSteps of the last step, per body (2 ints; -1 when the body
// is in no island)
void orc_get_island_iterations(void *wp, int *out) {
    World &w = *(World *)wp;
    for (size_t i = 0; i < w.bodies.size(); i++) out[2 * i] = out[2 * i + 1] = -1;
    for (const Island &is : w.islands)
        for (int64_t ai : is.bodyIndices) {
            int bi = w.activeBodyIndices[ai];
            out[2 * bi] = is.velSteps;
            out[2 * bi + 1] = is.posSteps;
        }
}
// sub-shape ids of the manifolds, in orc_get_manifolds order (2 per manifold, id order)
int orc_get_manifold_subs(void *wp, uint32_t *out) {
    World &w = *(World *)wp;
    for (size_t i = 0; i < w.manifolds.size(); i++) {
        out[2 * i] = w.manifolds[i].subA;
        out[2 * i + 1] = w.manifolds[i].subB;
    }
    return (int)w.manifolds.size();
}
// fixNormal active-edges.ts:74-153 on 8 vec3 inputs (v0 v1 v2 triangle normal point normal movement,
// and active bits in in[24]): 1 when it keeps the normal, 0 when it returns the triangle normal
int orc_fix_normal(const double *in) {
    auto v = [&](int k) { return V3{in[3 * k], in[3 * k + 1], in[3 * k + 2]}; };
    V3 tn = v(3), n = v(5);
    V3 r = fix_normal(v(0), v(1), v(2), tn, (int)in[24], v(4), n, v(6));
    if (r.x == n.x && r.y == n.y && r.z == n.z) return 1;
    if (r.x == tn.x && r.y == tn.y && r.z == tn.z) return 0;
    return -1;
}
// continuous collision of the last step: records, and records whose cast hit a body
void orc_ccd_counts(void *wp, int *out) {
    out[0] = (int)((World *)wp)->ccd.size();
    out[1] = ((World *)wp)->ccdHits;
}

// the convex shapes a cast or collide query may be (a hull names one of the world's hulls)
static bool query_shape(int t) {
    return t == SHAPE_SPHERE || t == SHAPE_BOX || t == SHAPE_CAPSULE || t == SHAPE_CYLINDER || t == SHAPE_CONVEX_HULL;
}

// castRay query.ts:78-90 with the closest-hit collector (cast-ray-vs-shape.ts:180-205): each ray
// (origin xyz, direction xyz unit, length) against every body whose current AABB the segment
// enters (dbvt.castRay dbvt.ts:779-865) and that passes the filter (object layer bit in
// layerMask, collision group/mask); hit = (body index, fraction, sub-shape id) or body -1.
// Ties in fraction go to the lower body index.
void orc_cast_rays(void *wp, const double *rays, int n, uint32_t layerMask, uint32_t groups, uint32_t mask,
                   int treatConvexAsSolid, double *fractions, int *bodies, uint32_t *subs) {
    World &W = *(World *)wp;
    for (auto &b : W.bodies) update_aabb(b);
    for (int r = 0; r < n; r++) {
        const double *ry = rays + 7 * r;
        V3 o{ry[0], ry[1], ry[2]}, d{ry[3], ry[4], ry[5]};
        double len = ry[6];
        double best = 1.0 + 1e-4;  // INITIAL_EARLY_OUT_FRACTION cast-utils.ts:3
        int hit = -1;
        uint32_t hsub = EMPTY_SUB_SHAPE_ID;
        for (auto &b : W.bodies) {
            if (!((groups & b.mask) != 0 && (b.groups & mask) != 0)) continue;
            if (!(layerMask & (1u << b.objectLayer))) continue;
            if (!(ray_fraction_to_box(o, d, len, b.aabb) < std::numeric_limits<double>::infinity())) continue;
            double f;
            uint32_t sub;
            V3 gp;
            Q4 gq;
            geometry_pose(b.shape, b.position, b.quat, gp, gq);
            if (!cast_ray_vs_shape(b.shape, gp, gq, o, d, len, treatConvexAsSolid != 0, best, f, sub)) continue;
            if (f < best || (f == best && hit >= 0 && b.index < hit)) {
                best = f;
                hit = b.index;
                hsub = sub;
            }
        }
        fractions[r] = hit >= 0 ? best : 1.0;
        bodies[r] = hit;
        subs[r] = hsub;
    }
}

// collidePoint query.ts:470-490 with every hit collected (createAllCollidePointCollector): per
// point (xyz) the number of bodies that contain it, the lowest such body index (-1 if none) and
// that body's sub-shape id; bodies whose current AABB contains the point and that pass the filter
// (dbvt.intersectPoint dbvt.ts:683-740)
void orc_collide_points(void *wp, const double *pts, int n, uint32_t layerMask, uint32_t groups, uint32_t mask,
                        double tol, int *counts, int *bodies, uint32_t *subs) {
    World &W = *(World *)wp;
    for (auto &b : W.bodies) update_aabb(b);
    for (int r = 0; r < n; r++) {
        V3 p{pts[3 * r], pts[3 * r + 1], pts[3 * r + 2]};
        int c = 0, first = -1;
        uint32_t fsub = EMPTY_SUB_SHAPE_ID;
        for (auto &b : W.bodies) {
            if (!((groups & b.mask) != 0 && (b.groups & mask) != 0)) continue;
            if (!(layerMask & (1u << b.objectLayer))) continue;
            if (!box_contains(b.aabb, p)) continue;
            uint32_t sub;
            V3 gp;
            Q4 gq;
            geometry_pose(b.shape, b.position, b.quat, gp, gq);
            if (!point_in_shape(b.shape, gp, gq, p, tol, sub)) continue;
            if (c++ == 0) {
                first = b.index;
                fsub = sub;
            }
        }
        counts[r] = c;
        bodies[r] = first;
        subs[r] = fsub;
    }
}

// castShape query.ts:196-214 with the closest-hit collector (ClosestCastShapeCollector
// cast-shape-vs-shape.ts:199-217) and the default cast settings (createDefaultCastShapeSettings
// :116-127): each query (shape type, 4 shape params, position xyz, quaternion xyzw, displacement
// xyz; 15 doubles) is cast against every body that passes the filter (a body out of reach of the
// swept box cannot be hit, so this is the set broadphase.castAABB visits, less the misses) by
// castShapeVsShape: castConvexVsConvex convex.ts:744-830, or for a mesh the sphere's own cast or
// castConvexVsTriangleMesh.  Out per query: fraction, normal (-penetration axis, normalised),
// contact point on the cast shape (7 doubles); the body (-1 on a miss) and its sub-shape id (a mesh
// triangle's, else 0xffffffff; subs may be NULL).  Ties go to the lower
// body index.
int orc_cast_shapes(void *wp, const double *qs, int n, uint32_t layerMask, uint32_t groups, uint32_t mask,
                    double *out, int *bodies, uint32_t *subs) {
    World &W = *(World *)wp;
    for (int r = 0; r < n; r++) {
        const double *q = qs + 15 * r;
        double row[F_COUNT] = {};
        row[F_SHAPE] = q[0];
        row[F_DENSITY] = 1000.0;
        for (int k = 0; k < 4; k++) row[F_P0 + k] = q[1 + k];
        Shape sa;
        if (!shape_from_row(sa, row, &W) || !query_shape(sa.type)) return -1;
        V3 pA{q[5], q[6], q[7]}, disp{q[12], q[13], q[14]};
        Q4 qA{q[8], q[9], q[10], q[11]};
        double best = 1.0 + 1e-4;  // INITIAL_EARLY_OUT_FRACTION cast-utils.ts:3
        int hit = -1;
        uint32_t hsub = EMPTY_SUB_SHAPE_ID;
        V3 hn{0, 0, 0}, hp{0, 0, 0};
        for (auto &B : W.bodies) {
            if (!((groups & B.mask) != 0 && (B.groups & mask) != 0)) continue;
            if (!(layerMask & (1u << B.objectLayer))) continue;
            V3 gpB;
            Q4 gqB;
            geometry_pose(B.shape, B.position, B.quat, gpB, gqB);
            auto collect = [&](double fraction, V3 pa, V3 axis, uint32_t sub = EMPTY_SUB_SHAPE_ID) {
                if (!(fraction < best || (fraction == best && hit >= 0 && B.index < hit))) return;
                best = fraction;
                hit = B.index;
                hsub = sub;
                hn = neg(normalize(axis));
                hp = pa;
            };
            if (B.shape.type == SHAPE_EMPTY) continue;
            if (B.shape.type == SHAPE_COMPOUND) {  // castShapeVsCompound compound.ts:776-866
                const CompoundData &C = *B.shape.compound;
                for (int i = 0; i < (int)C.shapes.size(); i++) {
                    V3 cp;
                    Q4 cq;
                    compound_child_pose(C, i, gpB, gqB, cp, cq);
                    CastHit h;
                    const double maxL = (hit >= 0 && B.index < hit) ? std::nextafter(best, 2.0) : best;
                    if (cast_convex_vs_convex(h, sa, pA, qA, disp, C.shapes[i], cp, cq, maxL, false))
                        collect(h.fraction, h.pa, h.axis, compound_sub_id(C, i));
                }
                continue;
            }
            if (B.shape.type == SHAPE_PLANE) {
                CastHit h;
                if (cast_convex_vs_plane(h, sa, pA, qA, disp, B.shape, gpB, gqB, best, false))
                    collect(h.fraction, h.pa, h.axis);
                continue;
            }
            if (B.shape.type == SHAPE_TRIANGLE_MESH) {
                auto onHit = [&](const CastMeshHit &h) { collect(h.fraction, h.pa, h.axis, h.sub); };
                auto earlyOut = [&]() { return best; };
                if (sa.type == SHAPE_SPHERE)
                    cast_sphere_vs_mesh(sa, pA, disp, B.shape, gpB, gqB, onHit, earlyOut);
                else
                    cast_convex_vs_mesh(sa, pA, qA, disp, B.shape, gpB, gqB, onHit, earlyOut);
                continue;
            }
            CastHit h;
            const double maxL = (hit >= 0 && B.index < hit) ? std::nextafter(best, 2.0) : best;
            if (!cast_convex_vs_convex(h, sa, pA, qA, disp, B.shape, gpB, gqB, maxL, false)) continue;
            collect(h.fraction, h.pa, h.axis);
        }
        double *o = out + 7 * r;
        o[0] = hit >= 0 ? best : 1.0;
        o[1] = hn.x, o[2] = hn.y, o[3] = hn.z;
        o[4] = hp.x, o[5] = hp.y, o[6] = hp.z;
        bodies[r] = hit;
        if (subs) subs[r] = hsub;
    }
    return 0;
}

// castRay query.ts:78-90 with the AllCastRayCollector (cast-ray-vs-shape.ts:66-94): per ray
// (7 doubles as orc_cast_rays) every hit of every body whose AABB the segment enters and that
// passes the filter: a convex body's one hit below INITIAL_EARLY_OUT_FRACTION, each triangle hit
// of a mesh (back faces culled).  Sorted by fraction, body index, sub-shape id; the first cap
// written to fractions / bodies / subs[r * cap ...], counts[r] = the number found.
void orc_cast_rays_all(void *wp, const double *rays, int n, uint32_t layerMask, uint32_t groups, uint32_t mask,
                       int treatConvexAsSolid, int cap, double *fractions, int *bodies, uint32_t *subs, int *counts) {
    World &W = *(World *)wp;
    for (auto &b : W.bodies) update_aabb(b);
    const double initial = 1.0 + 1e-4;
    for (int r = 0; r < n; r++) {
        const double *ry = rays + 7 * r;
        V3 o{ry[0], ry[1], ry[2]}, d{ry[3], ry[4], ry[5]};
        double len = ry[6];
        struct H {
            double f;
            int b;
            uint32_t sub;
        };
        std::vector<H> hs;
        for (auto &b : W.bodies) {
            if (!((groups & b.mask) != 0 && (b.groups & mask) != 0)) continue;
            if (!(layerMask & (1u << b.objectLayer))) continue;
            if (!(ray_fraction_to_box(o, d, len, b.aabb) < std::numeric_limits<double>::infinity())) continue;
            V3 gp;
            Q4 gq;
            geometry_pose(b.shape, b.position, b.quat, gp, gq);
            if (b.shape.type == SHAPE_COMPOUND) {  // castRayVsCompound: each child's hit
                const CompoundData &C = *b.shape.compound;
                for (int i = 0; i < (int)C.shapes.size(); i++) {
                    V3 cp;
                    Q4 cq;
                    compound_child_pose(C, i, gp, gq, cp, cq);
                    double f;
                    uint32_t sb;
                    if (cast_ray_vs_shape(C.shapes[i], cp, cq, o, d, len, treatConvexAsSolid != 0, initial, f, sb))
                        hs.push_back({f, b.index, compound_sub_id(C, i)});
                }
                continue;
            }
            if (b.shape.type == SHAPE_TRIANGLE_MESH) {
                Q4 iq = qconj(gq);
                std::vector<std::pair<double, uint32_t>> th;
                mesh_ray_all_hits(*b.shape.mesh, rotate(iq, sub(o, gp)), rotate(iq, d), len, th);
                for (auto &t : th) hs.push_back({t.first, b.index, t.second});
                continue;
            }
            double f;
            uint32_t sb;
            if (cast_ray_vs_shape(b.shape, gp, gq, o, d, len, treatConvexAsSolid != 0, initial, f, sb))
                hs.push_back({f, b.index, sb});
        }
        std::sort(hs.begin(), hs.end(), [](const H &x, const H &y) {
            if (x.f != y.f) return x.f < y.f;
            if (x.b != y.b) return x.b < y.b;
            return x.sub < y.sub;
        });
        counts[r] = (int)hs.size();
        for (int k = 0; k < (int)hs.size() && k < cap; k++) {
            fractions[r * cap + k] = hs[k].f;
            bodies[r * cap + k] = hs[k].b;
            subs[r * cap + k] = hs[k].sub;
        }
    }
}

// castShape query.ts:196-214 with the AllCastShapeCollector (cast-shape-vs-shape.ts:165-197):
// per query (15 doubles as orc_cast_shapes) every hit below INITIAL_EARLY_OUT_FRACTION: a convex
// body's or a plane's one hit, each triangle hit of a mesh.  Sorted by fraction, body, sub-shape
// id; the first cap written as 7 doubles (fraction, normal, point) to out[(r * cap + k) * 7],
// bodies and subs[r * cap + k]; counts[r] = the number found.
int orc_cast_shapes_all(void *wp, const double *qs, int n, uint32_t layerMask, uint32_t groups, uint32_t mask,
                        int cap, double *out, int *bodies, uint32_t *subs, int *counts) {
    World &W = *(World *)wp;
    const double initial = 1.0 + 1e-4;
    for (int r = 0; r < n; r++) {
        const double *q = qs + 15 * r;
        double row[F_COUNT] = {};
        row[F_SHAPE] = q[0];
        row[F_DENSITY] = 1000.0;
        for (int k = 0; k < 4; k++) row[F_P0 + k] = q[1 + k];
        Shape sa;
        if (!shape_from_row(sa, row, &W) || !query_shape(sa.type)) return -1;
        V3 pA{q[5], q[6], q[7]}, disp{q[12], q[13], q[14]};
        Q4 qA{q[8], q[9], q[10], q[11]};
        struct H {
            double f;
            int b;
            uint32_t sub;
            V3 n, p;
        };
        std::vector<H> hs;
        for (auto &B : W.bodies) {
            if (!((groups & B.mask) != 0 && (B.groups & mask) != 0)) continue;
            if (!(layerMask & (1u << B.objectLayer))) continue;
            V3 gpB;
            Q4 gqB;
            geometry_pose(B.shape, B.position, B.quat, gpB, gqB);
            auto collect = [&](double fraction, V3 pa, V3 axis, uint32_t sub = EMPTY_SUB_SHAPE_ID) {
                if (fraction < initial) hs.push_back({fraction, B.index, sub, neg(normalize(axis)), pa});
            };
            if (B.shape.type == SHAPE_EMPTY) continue;
            if (B.shape.type == SHAPE_COMPOUND) {
                const CompoundData &C = *B.shape.compound;
                for (int i = 0; i < (int)C.shapes.size(); i++) {
                    V3 cp;
                    Q4 cq;
                    compound_child_pose(C, i, gpB, gqB, cp, cq);
                    CastHit h;
                    if (cast_convex_vs_convex(h, sa, pA, qA, disp, C.shapes[i], cp, cq, initial, false))
                        collect(h.fraction, h.pa, h.axis, compound_sub_id(C, i));
                }
                continue;
            }
            if (B.shape.type == SHAPE_PLANE) {
                CastHit h;
                if (cast_convex_vs_plane(h, sa, pA, qA, disp, B.shape, gpB, gqB, initial, false))
                    collect(h.fraction, h.pa, h.axis);
                continue;
            }
            if (B.shape.type == SHAPE_TRIANGLE_MESH) {
                auto onHit = [&](const CastMeshHit &h) { collect(h.fraction, h.pa, h.axis, h.sub); };
                auto earlyOut = [&]() { return initial; };
                if (sa.type == SHAPE_SPHERE)
                    cast_sphere_vs_mesh(sa, pA, disp, B.shape, gpB, gqB, onHit, earlyOut);
                else
                    cast_convex_vs_mesh(sa, pA, qA, disp, B.shape, gpB, gqB, onHit, earlyOut);
                continue;
            }
            CastHit h;
            if (cast_convex_vs_convex(h, sa, pA, qA, disp, B.shape, gpB, gqB, initial, false))
                collect(h.fraction, h.pa, h.axis);
        }
        std::sort(hs.begin(), hs.end(), [](const H &x, const H &y) {
            if (x.f != y.f) return x.f < y.f;
            if (x.b != y.b) return x.b < y.b;
            return x.sub < y.sub;
        });
        counts[r] = (int)hs.size();
        for (int k = 0; k < (int)hs.size() && k < cap; k++) {
            double *o = out + (size_t)(r * cap + k) * 7;
            o[0] = hs[k].f;
            o[1] = hs[k].n.x, o[2] = hs[k].n.y, o[3] = hs[k].n.z;
            o[4] = hs[k].p.x, o[5] = hs[k].p.y, o[6] = hs[k].p.z;
            bodies[r * cap + k] = hs[k].b;
            subs[r * cap + k] = hs[k].sub;
        }
    }
    return 0;
}

// collideShape query.ts:286-311 with the AllCollideShapeCollector (collide-shape-vs-shape.ts
// :82-113): per query (shape type, 4 shape params, position xyz, quaternion xyzw; 12 doubles)
// every hit of collideShapeVsShape (collide_hits, no movement direction) against every body whose
// current AABB meets the query's box (the shape's local bounds through its pose, grown by the
// separation: broadphase.intersectAABB) and that passes the filter.  settings: maxSeparation,
// collisionTolerance, penetrationTolerance, collideWithBackfaces.  Sorted by body, sub-shape id;
// the first cap written as 10 doubles (penetration, point on the query shape, point on the body,
// unit axis) to out[(r * cap + k) * 10], bodies / subs[r * cap + k]; counts[r] = the number found.
int orc_collide_shapes_all(void *wp, const double *qs, int n, uint32_t layerMask, uint32_t groups, uint32_t mask,
                           const double *settings, int cap, double *out, int *bodies, uint32_t *subs, int *counts) {
    World &W = *(World *)wp;
    for (auto &b : W.bodies) update_aabb(b);
    CollideSettings cs;
    cs.maxSeparation = settings[0];
    cs.collisionTolerance = settings[1];
    cs.penetrationTolerance = settings[2];
    cs.collideWithBackfaces = settings[3] != 0;
    cs.collectFaces = false;
    for (int r = 0; r < n; r++) {
        const double *q = qs + 12 * r;
        double row[F_COUNT] = {};
        row[F_SHAPE] = q[0];
        row[F_DENSITY] = 1000.0;
        for (int k = 0; k < 4; k++) row[F_P0 + k] = q[1 + k];
        Body qb;
        if (!shape_from_row(qb.shape, row, &W) || !query_shape(qb.shape.type)) return -1;
        qb.position = {q[5], q[6], q[7]};
        qb.quat = {q[8], q[9], q[10], q[11]};
        update_aabb(qb);
        const double m = cs.maxSeparation;
        Box3 E{sub(qb.aabb.mn, V3{m, m, m}), add(qb.aabb.mx, V3{m, m, m})};
        struct H {
            int b;
            Hit h;
        };
        std::vector<H> hs;
        for (auto &B : W.bodies) {
            if (!((groups & B.mask) != 0 && (B.groups & mask) != 0)) continue;
            if (!(layerMask & (1u << B.objectLayer))) continue;
            if (!box_overlap(B.aabb, E)) continue;
            V3 gp;
            Q4 gq;
            geometry_pose(B.shape, B.position, B.quat, gp, gq);
            std::vector<Hit> out1;
            collide_hits(out1, cs, qb.shape, qb.position, qb.quat, B.shape, gp, gq, V3{0, 0, 0});
            for (auto &h : out1) hs.push_back({B.index, h});
        }
        std::stable_sort(hs.begin(), hs.end(), [](const H &x, const H &y) {
            if (x.b != y.b) return x.b < y.b;
            return x.h.subB < y.h.subB;
        });
        counts[r] = (int)hs.size();
        for (int k = 0; k < (int)hs.size() && k < cap; k++) {
            const Hit &h = hs[k].h;
            V3 ax = normalize(h.axis);
            double *o = out + (size_t)(r * cap + k) * 10;
            o[0] = h.penetration;
            o[1] = h.pa.x, o[2] = h.pa.y, o[3] = h.pa.z;
            o[4] = h.pb.x, o[5] = h.pb.y, o[6] = h.pb.z;
            o[7] = ax.x, o[8] = ax.y, o[9] = ax.z;
            bodies[r * cap + k] = hs[k].b;
            subs[r * cap + k] = h.subB;
        }
    }
    return 0;
}

// ---- unit-level entry points for the known-answer tests -------------------
// Faces are passed as n vertices (xyz doubles).  Returns the output vertex count.
int orc_clip_poly_vs_plane(const double *poly, int n, const double *origin, const double *normal, double *out) {
    Face in, o;
    in.n = n;
    for (int i = 0; i < n; i++) in.v[i] = {poly[3 * i], poly[3 * i + 1], poly[3 * i + 2]};
    clip_poly_vs_plane(o, in, {origin[0], origin[1], origin[2]}, {normal[0], normal[1], normal[2]});
    for (int i = 0; i < o.n; i++) {
        out[3 * i] = o.v[i].x;
        out[3 * i + 1] = o.v[i].y;
        out[3 * i + 2] = o.v[i].z;
    }
    return o.n;
}
int orc_clip_poly_vs_poly(const double *poly, int n, const double *clip, int m, const double *normal, double *out) {
    Face a, c, o;
    a.n = n;
    for (int i = 0; i < n; i++) a.v[i] = {poly[3 * i], poly[3 * i + 1], poly[3 * i + 2]};
    c.n = m;
    for (int i = 0; i < m; i++) c.v[i] = {clip[3 * i], clip[3 * i + 1], clip[3 * i + 2]};
    clip_poly_vs_poly(o, a, c, {normal[0], normal[1], normal[2]});
    for (int i = 0; i < o.n; i++) {
        out[3 * i] = o.v[i].x;
        out[3 * i + 1] = o.v[i].y;
        out[3 * i + 2] = o.v[i].z;
    }
    return o.n;
}
// manifoldBetweenTwoFaces with baseOffset 0; writes pointsA then pointsB (n x 3 each).
int orc_manifold_between_faces(const double *cp1, const double *cp2, const double *axis, double maxDist,
                               const double *f1, int n1, const double *f2, int n2, double *outA, double *outB) {
    Face a, b;
    a.n = n1;
    b.n = n2;
    for (int i = 0; i < n1; i++) a.v[i] = {f1[3 * i], f1[3 * i + 1], f1[3 * i + 2]};
    for (int i = 0; i < n2; i++) b.v[i] = {f2[3 * i], f2[3 * i + 1], f2[3 * i + 2]};
    Manifold m;
    m.base = {0, 0, 0};
    manifold_between_faces(m, {cp1[0], cp1[1], cp1[2]}, {cp2[0], cp2[1], cp2[2]}, {axis[0], axis[1], axis[2]},
                           maxDist, a, b);
    for (int i = 0; i < m.n; i++) {
        outA[3 * i] = m.relA[i].x;
        outA[3 * i + 1] = m.relA[i].y;
        outA[3 * i + 2] = m.relA[i].z;
        outB[3 * i] = m.relB[i].x;
        outB[3 * i + 1] = m.relB[i].y;
        outB[3 * i + 2] = m.relB[i].z;
    }
    return m.n;
}
// pruneContactPoints on n points (relative to base 0); returns the kept count, rewrites in place.
int orc_prune_contact_points(double *ptsA, double *ptsB, int n, const double *axis) {
    Manifold m;
    m.n = n;
    for (int i = 0; i < n; i++) {
        m.relA[i] = {ptsA[3 * i], ptsA[3 * i + 1], ptsA[3 * i + 2]};
        m.relB[i] = {ptsB[3 * i], ptsB[3 * i + 1], ptsB[3 * i + 2]};
    }
    prune_contact_points(m, {axis[0], axis[1], axis[2]});
    for (int i = 0; i < m.n; i++) {
        ptsA[3 * i] = m.relA[i].x;
        ptsA[3 * i + 1] = m.relA[i].y;
        ptsA[3 * i + 2] = m.relA[i].z;
        ptsB[3 * i] = m.relB[i].x;
        ptsB[3 * i + 1] = m.relB[i].y;
        ptsB[3 * i + 2] = m.relB[i].z;
    }
    return m.n;
}
// Barycentric coordinates (u, v, w, valid) of the closest point to the origin.
void orc_barycentric(const double *a, const double *b, const double *c, int n, double sqtol, double *out) {
    Bary r;
    if (n == 2)
        r = bary2({a[0], a[1], a[2]}, {b[0], b[1], b[2]}, sqtol);
    else
        r = bary3({a[0], a[1], a[2]}, {b[0], b[1], b[2]}, {c[0], c[1], c[2]}, sqtol);
    out[0] = r.u;
    out[1] = r.v;
    out[2] = r.w;
    out[3] = r.valid ? 1 : 0;
}
// Single shape pair collision (world space).  shape rows as in orc_add_bodies (F_SHAPE..F_P0+3).
// out: found, pointA3, pointB3, axis3, penetration, faceA n, faceB n  (13 doubles)
int orc_collide_pair(const double *rowA, const double *rowB, double maxSep, double *out) {
    Shape s[2];
    V3 p[2];
    Q4 q[2];
    const double *rows[2] = {rowA, rowB};
    for (int k = 0; k < 2; k++) {
        const double *r = rows[k];
        if (!shape_from_row(s[k], r)) return -1;
        p[k] = {r[F_POS], r[F_POS + 1], r[F_POS + 2]};
        q[k] = {r[F_QUAT], r[F_QUAT + 1], r[F_QUAT + 2], r[F_QUAT + 3]};
    }
    CollideSettings cs;
    cs.maxSeparation = maxSep;
    Hit h;
    V3 gp[2];
    Q4 gq[2];
    for (int k = 0; k < 2; k++) geometry_pose(s[k], p[k], q[k], gp[k], gq[k]);
    bool f = collide_shapes(h, cs, s[0], gp[0], gq[0], s[1], gp[1], gq[1]);
    out[0] = f ? 1 : 0;
    out[1] = h.pa.x;
    out[2] = h.pa.y;
    out[3] = h.pa.z;
    out[4] = h.pb.x;
    out[5] = h.pb.y;
    out[6] = h.pb.z;
    out[7] = h.axis.x;
    out[8] = h.axis.y;
    out[9] = h.axis.z;
    out[10] = h.penetration;
    out[11] = h.faceA.n;
    out[12] = h.faceB.n;
    return f ? 1 : 0;
}
// World-space inverse inertia (3x3 column-major) for a body row at its orientation.
void orc_inverse_inertia(const double *row, double *out9) {
    Body b;
    Shape &s = b.shape;
    shape_from_row(s, row);
    b.motion = DYNAMIC;
    setup_mass(b, s, row, nullptr);
    b.quat = {row[F_QUAT], row[F_QUAT + 1], row[F_QUAT + 2], row[F_QUAT + 3]};
    M4 I = inv_inertia_for_rotation(b, mat4_from_quat(b.quat));
    int k = 0;
    for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++) out9[k++] = I.m[c * 4 + r];
}

// Record (1) or stop recording (0) the rows of each step's velocity solve.
void orc_set_record_tape(void *wp, int on) { ((World *)wp)->recordTape = on != 0; }
// The last recorded step: body rows (n x BODY_ROW), contact rows (count x CON_ROW), post-solve
// velocities (n x 6) and the warm-start ratio; returns the contact count (arrays may be NULL).
int orc_get_solver_tape(void *wp, double *bodies, double *cons, double *v2, double *ratio) {
    World &w = *(World *)wp;
    if (bodies) std::copy(w.tapeBodies.begin(), w.tapeBodies.end(), bodies);
    if (cons) std::copy(w.tapeCons.begin(), w.tapeCons.end(), cons);
    if (v2) std::copy(w.tapeV2.begin(), w.tapeV2.end(), v2);
    if (ratio) *ratio = w.tapeRatio;
    return (int)(w.tapeCons.size() / orc_frozen::CON_ROW);
}
// Frozen-contact replay of a taped rollout (oracle_frozen.h).  mode 0: the real parts are the
// tape's at every step and the dual parts carry the derivative along (dv, dw, dmu): out =
// [loss at the tape, directional derivative].  mode 1: the replay's own trajectory from the
// initial state moved by eps x (dv, dw, dmu): out = [loss(eps), its derivative along the
// direction]; the loss is taken against a replay at eps = 0.  v2_out (steps x n x 6) and
// lam_out (contacts x 12) receive the replay's post-solve velocities and final impulses.
int orc_frozen_rollout(int n, int steps, int worlds, int iters, double dt, const double *consts,
                       const double *bodies, const double *v0, const double *ratio, const int *con_off,
                       const double *cons, const double *x_final, const double *targets, int mode, double eps,
                       const double *dv, const double *dw, const double *dmu, double *out, double *v2_out,
                       double *lam_out) {
    using namespace orc_frozen;
    if (n <= 0 || steps <= 0 || (mode != 0 && mode != 1)) return -1;
    Tape T;
    T.n = n, T.steps = steps, T.worlds = worlds, T.iters = iters, T.dt = dt;
    T.consts = consts, T.bodies = bodies, T.v0 = v0, T.ratio = ratio, T.con_off = con_off, T.cons = cons;
    T.x_final = x_final, T.targets = targets;
    std::vector<V3s<double>> ref;
    if (mode == 1) {
        Replay<double> nominal(T, 1);
        nominal.run(0.0, nullptr, nullptr, nullptr);
        ref = nominal.vsum;
    }
    Replay<Dual> r(T, mode);
    r.v2_out = v2_out;
    r.lam_out = lam_out;
    r.run(eps, dv, dw, dmu);
    Dual L = r.loss(mode == 1 ? &ref : nullptr);
    out[0] = L.v;
    out[1] = L.d;
    return 0;
}

}  // extern "C"
