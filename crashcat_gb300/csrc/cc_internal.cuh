// Internal device data layout and helpers of the GB300 world step.
//
// Body state lives in device memory as structure-of-arrays of float4 rows so
// that every per-body kernel issues 16-byte coalesced loads.  One handle can
// hold many independent worlds (the batched form); every body carries its
// world index and pairs never cross worlds.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "../../include/crashcat_gpu.h"

namespace cc {

// ---------------------------------------------------------------------------
// body flag word
// ---------------------------------------------------------------------------
enum : uint32_t {
    F_MOTION_MASK = 0x3u,        // bits 0-1: STATIC / KINEMATIC / DYNAMIC
    F_SLEEPING = 1u << 2,
    F_ALLOW_SLEEP = 1u << 3,
    F_SENSOR = 1u << 4,
    F_KIN_VS_NONDYN = 1u << 5,
    F_SHAPE_SHIFT = 6,           // bits 6-8 shape type
    F_DOF_SHIFT = 9,             // bits 9-14 allowed DOFs
    F_FCOMB_SHIFT = 15,          // bits 15-17 friction combine mode
    F_RCOMB_SHIFT = 18,          // bits 18-20 restitution combine mode
    F_LAYER_SHIFT = 21,          // bits 21-25 object layer
    F_LINEAR_CAST = 1u << 26,    // MotionQuality.LINEAR_CAST
    F_DECORATED = 1u << 27,      // the shape has decorators (DevWorld::frames)
    F_SHAPE_HI = 1u << 28,       // the shape type's fourth bit
};
__host__ __device__ inline int motion_of(uint32_t f) { return (int)(f & F_MOTION_MASK); }
__host__ __device__ inline int shape_of(uint32_t f) { return (int)(((f >> F_SHAPE_SHIFT) & 7u) | ((f >> 25) & 8u)); }
// the flag bits of a shape type (bits 6-8 and 28)
__host__ __device__ inline uint32_t shape_bits(int shape) {
    return ((uint32_t)(shape & 7) << F_SHAPE_SHIFT) | ((uint32_t)(shape & 8) << 25);
}
__host__ __device__ inline int dof_of(uint32_t f) { return (int)((f >> F_DOF_SHIFT) & 63u); }
__host__ __device__ inline int layer_of(uint32_t f) { return (int)((f >> F_LAYER_SHIFT) & 31u); }
__host__ __device__ inline bool sleeping_of(uint32_t f) { return (f & F_SLEEPING) != 0; }

constexpr int STATIC = 0, KINEMATIC = 1, DYNAMIC = 2;
constexpr int SHAPE_SPHERE = 0, SHAPE_BOX = 1, SHAPE_CAPSULE = 2, SHAPE_HULL = 3, SHAPE_MESH = 4, SHAPE_CYLINDER = 5,
              SHAPE_PLANE = 6, SHAPE_EMPTY = 7,  // an empty shape (empty-shape.ts) collides with nothing
              SHAPE_COMPOUND = 8;

// Per-step overflow flags (status bits in DevCounters::overflow)
enum : int { OVF_PAIRS = 1, OVF_MANIFOLDS = 2, OVF_EPA = 4, OVF_ISLAND = 8, OVF_CACHE = 16, OVF_SLOTS = 32,
             OVF_TIMEOUT = 64 };

// Device-resident counters of one step (one 128-byte line).
// Islands of the per-thread and per-warp solve tiers are listed by size, most constraints first:
// the per-thread tier by its contact count (0 to 15, and 16 or more), the per-warp tier by the
// power of two above its contact count less one (9-16, 17-32, 33-64, 65-128, 129-256).  Each
// bucket is a list of the body capacity.
constexpr int SMALL_BUCKETS = 17, MID_BUCKETS = 5;
// The narrowphase takes the broadphase pairs grouped by the shapes' collide routine
// (pair_class), so that the lanes of a warp run one routine.
constexpr int PAIR_CLASSES = 8;

struct DevCounters {
    int num_pairs;
    int num_manifolds;
    int num_epa;
    int num_islands;
    int num_large_islands;
    int num_small_islands;
    int overflow;
    int num_points;
    int num_awake;
    int max_island_constraints;
    int island_cursor;
    int large_cursor;
    int num_mid_islands;
    int mid_cursor;
    int epa_cursor;
    int epa_fallback;  // EPA items handed to the pass with the reference's polytope limits
    int num_removed;   // contact pairs of the previous step not found in this step
    int num_giant_islands;              // islands solved by the whole grid (cooperative launch)
    unsigned int bar_count, bar_gen;    // grid barrier of the giant-island solve
    int bar_error;                      // a bounded grid-barrier wait gave up
    int giant_left[2], giant_any[2], giant_sleep;
    int giant_colours;  // most colours of a giant island this step
    int num_small_joint_islands, num_large_joint_islands;  // islands with joints per tier
    int num_ccd;       // bodies that took the continuous-collision path this step
    int num_ccd_hits;  // of them, those whose cast hit a body
    int num_mesh_pairs;   // broadphase pairs with a triangle mesh body
    int num_mesh_hits;    // triangle hits reported to the mesh pairs' reduction
    int mesh_reduced;     // mesh pairs whose hits needed more manifolds than the reference's pool of 32
    int num_mesh_big;     // mesh pairs run again with the 32-manifold pool (their hits overflowed 4)
    int num_compound_pairs;  // broadphase pairs with a compound body and no mesh
    int small_bucket[SMALL_BUCKETS];  // per-thread tier islands by contact count
    int mid_bucket[MID_BUCKETS];      // per-warp tier islands by size class
    int mid_cursor_s;                 // cursor of the per-warp tier's small instance
    int pair_class[PAIR_CLASSES];     // broadphase pairs per collide class
    int pair_class_fill[PAIR_CLASSES];
    int pad2[1];
};

// Settings copied into constant memory once per world.
struct DevSettings {
    float gravity[3];
    int gravity_enabled;
    float spec_dist;
    float manifold_tol;
    float collision_tol;
    float penetration_tol;
    float normal_cos;
    float preserve_lambda_dsq;
    int vel_iters;
    int pos_iters;
    int warm_starting;
    float slop;
    float baumgarte;
    float max_pen;
    float min_vel_restitution;
    int allow_sleeping;
    float time_before_sleep;
    float sleep_threshold;
    float ccd_threshold, ccd_max_penetration, ccd_min_vel_restitution;  // WorldSettings.ccd
    uint32_t allowed_pairs[CC_MAX_LAYERS];  // combined layer predicate, bit j of [i]
    // layer predicate of the continuous-collision cast: object layer pair enabled AND the
    // querying layer may query the other's broadphase layer (broadphase.ts:334-335, dbvt.ts:954)
    uint32_t cast_pairs[CC_MAX_LAYERS];
    int small_island_max_cons;  // islands up to this many contacts run on one thread
    int small_island_max_joints;  // islands with joints: up to this many joints run on one thread
    unsigned wait_polls;        // polls of a bounded device wait (grid barrier) before it gives up
    int link_attempts;          // attempts of one union-find link before it gives up (OVF_ISLAND)
    int test_withhold_block;    // test hook: block 0 of the whole-grid solve skips its barriers
};

// Manifold produced by the narrowphase for one body pair (<= 4 points),
// points stored relative to the position of body `base`.
struct Manifold {
    int a, b;          // narrowphase order (A has the lower motion type)
    int n;
    float3 base;       // position of A when the pair was collided
    float3 normal;     // A -> B, normalised
    float depth;
    float3 ra[4];      // point on A relative to base (= position of A)
    float3 rb[4];
    uint32_t sub_a, sub_b;  // sub-shape ids (0xffffffff for a convex shape; a mesh triangle's id)
};

// Contact constraint in solver form (one per manifold that creates a constraint).
struct ContactPoint {
    float3 rA, rB;          // moment arms from the centres of mass (midpoint - com)
    float3 localA, localB;  // contact points in body space (for the position solve)
    float eff_n, eff_t1, eff_t2;
    float lam_n, lam_t1, lam_t2;
    float bias_n;
    float pad;
};
struct ContactConstraint {
    int a, b;              // body indices ordered by id
    int n;
    int island;
    float3 normal;
    float friction;
    float3 t1;
    float invMassA;
    float3 t2;
    float invMassB;
    uint32_t sort_key;
    int cache_slot;
    int pad0, pad1;
    ContactPoint p[4];
};

constexpr unsigned long long EMPTY_KEY = 0xffffffffffffffffull;  // free slot of the contact cache tables

// Contact cache record (contacts.ts:9-81): persistent across steps.
struct CacheRecord {
    unsigned long long key;  // (idxA << 32) | idxB, both ordered by id
    int n;
    int pad;
    float3 p1[4];
    float3 p2[4];
    float ln[4], lt1[4], lt2[4];
};

// Adjoint rollout (cc_adjoint.cu): one step's tape, taken between the contact setup and the
// solver, indexed like the world's per-step arrays.
struct TapeStep {
    ContactConstraint *cons;  // constraint rows by manifold index
    int *valid;               // constraint index of each manifold (-1: no constraint)
    float4 *v, *w, *q;        // velocities after force integration, orientation before the solve
    uint32_t *flags;
    int *isl_off, *isl_cnt;   // per island: first entry in isl_cons, contact count
    int *isl_cons;
    int *counts;              // [manifolds, islands]
};
// State a rollout resumes from: body state and the contact cache table the next step reads.
struct Checkpoint {
    float4 *pos, *quat, *com, *linvel, *angvel, *force, *torque, *sleep_sph;
    float *sleep_timer;
    uint32_t *flags;
    unsigned long long *keys;
    CacheRecord *recs;
    int *parity;
};
constexpr double ADJ_MU_SCALE = 1073741824.0;  // 2^30: fixed-point scale of AdjBuffers::mu_body
struct AdjBuffers {
    float4 *vbar, *wbar;    // adjoints of the linear / angular velocity
    float4 *xbar;           // dL/dx of each body
    float4 *vwork, *wwork;  // replayed velocities
    float4 *iw;             // world inverse inertia (2 per body) of the step being reversed
    float *u_tape;          // pre-projection value of every row update: iterations x manifolds x 12
    float *lam_bar;         // adjoint of every row's impulse: manifolds x 12
    float *mu_con;          // dL/d(combined friction) per constraint
    unsigned long long *mu_body;  // dL/d(friction) per body in 34.30 fixed point (order-free sums)
    float dt;
};

// Hinge joint (src/constraints/hinge-constraint.ts) with the state of its constraint parts:
// point (point-constraint-part.ts), hinge rotation (hinge-rotation-constraint-part.ts), and
// the limit and motor angle parts (angle-constraint-part.ts, spring-part.ts).
enum : int { JF_ENABLED = 1, JF_LIMITS = 2 };
// Convex hull shape (src/shapes/convex-hull.ts): points relative to the centre of mass, the
// points shrunk by the convex radius, polygon faces and their planes.  A hull body's shape
// record holds (hull index as int bits, convex radius, 0, 0).
struct DevHull {
    int first_point, num_points, first_face, num_faces;
    float convex_radius, inner_radius, pad0, pad1;
    float4 com;     // centre of mass in the input frame (xyz)
    float4 lo, hi;  // bounds of the points (xyz)
};

// Shape decorators of one body (src/shapes/scaled.ts, transformed.ts, offset-center-of-mass.ts),
// nested as OffsetCenterOfMass(Transformed(Scaled(leaf))): the scale is baked into the leaf's
// shape record; the collision geometry is the leaf at (t_pos, t_rot) in the body frame; com,
// the inner radius and the local bounds are the decorated shape's.
struct DevFrame {
    float4 t_pos;         // TransformedShape.position (xyz) | getInnerRadius of the decorated shape (w)
    float4 t_rot;         // TransformedShape.quaternion
    float4 com;           // centre of mass of the decorated shape in the body frame (xyz)
    double lo[3], hi[3];  // local bounds of the decorated shape
};

// Triangle mesh shape (src/shapes/triangle-mesh.ts, utils/triangle-mesh-data.ts and
// triangle-mesh-bvh.ts): welded vertices, triangles (vertex indices, active-edge bits) and
// the BVH in pre-order, two float4 per node: (min xyz, right child node or first triangle as
// int bits) and (max xyz, split axis or -(triangle count + 1) as int bits).  A mesh body's
// shape record holds (mesh index as int bits, 0, 0, 0).
struct DevMesh {
    int first_vertex, first_tri, first_node, num_tris;
    int sub_bits;  // bits of the triangle index in the sub-shape id (subShape.pushIndex sub-shape.ts:60-64)
    int pad0, pad1, pad2;
    float4 lo, hi;  // bounds of the root node
};
constexpr int MESH_KEY_BITS = 21;  // body indices and triangle indices in a mesh contact's cache key

// user joints of every type share one id space, packed as the reference's ConstraintId
// (constraint-id.ts:1-35): the ConstraintType above bit 24, the per-type index below
enum : int { JT_POINT = 0, JT_DISTANCE = 1, JT_HINGE = 2, JT_SLIDER = 3, JT_FIXED = 4, JT_CONE = 5, JT_SWING = 6,
             JT_SIX_DOF = 7, JT_TYPES = 8 };
constexpr int JOINT_TYPE_SHIFT = 24, JOINT_INDEX_MASK = (1 << JOINT_TYPE_SHIFT) - 1;

// fields every joint type starts with
struct DevJointHead {
    int a, b;             // body indices
    int priority, index;  // constraintPriority and the per-type creation index (sort key)
    int flags;            // JF_*
    int island;           // island of this step (-1: in none)
    int iter_ovr;         // velocity | position << 8 iteration overrides (0: the world's counts)
};
// PointConstraintPart (point-constraint-part.ts)
struct DevPoint {
    float3 r1, r2;
    float invI1_r1X[9], invI2_r2X[9], eff[9];  // row-major 3x3
    float3 lambda;
    int active;
};
// AngleConstraintPart (angle-constraint-part.ts)
struct DevAngle {
    float3 i1, i2;  // I1^-1 axis, I2^-1 axis
    float eff, soft, bias, lambda;
};

// RotationEulerConstraintPart (rotation-euler-constraint-part.ts): 3 rotational rows
struct DevEuler {
    float invI1[6], invI2[6];  // symmetric xx xy xz yy yz zz
    float eff[9];              // row-major
    float3 lambda;
};
// AxisConstraintPart (axis-constraint-part.ts) of a joint: one row along a world axis
struct DevAxis {
    float3 r1xa, r2xa, i1, i2;  // (r1 + u) x axis, r2 x axis, and the inverse inertias times them
    float eff, soft, bias, lambda;
};
// DualAxisConstraintPart (dual-axis-constraint-part.ts): 2 translational rows; eff as the
// reference's column-major mat2 [m00, m10, m01, m11]
struct DevDual {
    float3 r1xn1, r1xn2, r2xn1, r2xn2, i1n1, i1n2, i2n1, i2n2;
    float eff[4], lambda[2];
};

// Point, distance, fixed, cone and slider joints in one record (point-, distance-, fixed-,
// cone-, slider-constraint.ts): the fields of the joint's type are used, the rest stay zero.
struct DevJoint {
    DevJointHead h;
    int type;                     // JT_POINT .. JT_CONE
    float3 lp1, lp2;              // attachment points from the centres of mass, body space
    float4 inv_initial;           // fixed, slider: inverse initial relative orientation
    // distance
    float min_dist, max_dist;
    int spring_mode;
    float spring_freq, spring_damping;
    // cone: twist axes (body space), cosine of the half cone angle
    float3 lt1, lt2;
    float cos_half_cone;
    // slider: axis and normals (body A space), limits, friction and motor
    float3 ls1, ln1, ln2;
    int slider_flags;             // bit 0: limits
    float limits_min, limits_max;
    int limits_spring_mode;
    float limits_freq, limits_damping, max_friction_force;
    int motor_state, motor_spring_mode;
    float motor_freq, motor_damping, min_force, max_force, target_velocity, target_position;
    // per-step state
    float3 wp1, wp2, wn;          // distance: world points and normal
    float min_lambda, max_lambda;
    float3 w_rot_axis;            // cone: rotation axis of the limit
    float cos_theta;
    float3 r1, r2, u, ws, n1, n2; // slider: arms, separation, world axis and normals
    float d;                      // slider: position along the axis
    DevPoint pt;
    DevEuler rot;
    DevAxis ax, motor;            // distance row, cone unused; slider limits (ax) and motor
    DevAngle ang;                 // cone limit
    DevDual dual;                 // slider position rows
};

struct DevHinge {
    DevJointHead h;
    int motor_state, limits_spring_mode, motor_spring_mode;
    float3 lp1, lp2, lh1, lh2;  // attachment points (from the centre of mass) and hinge axes, body space
    float4 inv_initial;         // inverse initial relative orientation
    float limits_min, limits_max, limits_freq, limits_damping;
    float max_friction_torque, target_angular_velocity, target_angle;
    float motor_freq, motor_damping, min_torque, max_torque;
    // per-step state
    float theta;
    float3 wh1;  // world hinge axis of body A
    DevPoint pt;
    // hinge rotation part
    float3 a1, b2, c2, b2xA1, c2xA1;
    float invI1[6], invI2[6];  // symmetric xx xy xz yy yz zz
    float r_eff[4], r_lambda[2];
    DevAngle limit, motor;
};

// SwingTwistConstraint (swing-twist-constraint.ts) with its SwingTwistConstraintPart limits
// (swing-twist-constraint-part.ts): sines and cosines of the half-angle limits
enum : int { ST_TWIST_LOCKED = 1, ST_SWING_Y_LOCKED = 2, ST_SWING_Z_LOCKED = 4, ST_TWIST_FREE = 8,
             ST_SWING_Y_FREE = 16, ST_SWING_Z_FREE = 32, ST_SWING_YZ_FREE = 48 };
struct DevSwing {
    DevJointHead h;
    int swing_type, rotation_flags;
    int swing_motor_state, twist_motor_state, swing_spring_mode, twist_spring_mode;
    float3 lp1, lp2;
    float4 c2b1, c2b2;  // constraint space to body space
    float normal_half_cone, plane_half_cone, twist_min, twist_max, max_friction_torque;
    float sin_twist_min, sin_twist_max, cos_twist_min, cos_twist_max;
    float y_half_min, y_half_max, sin_y_min, sin_y_max, cos_y_min, cos_y_max;
    float z_half_min, z_half_max, sin_z_min, sin_z_max, cos_z_min, cos_z_max;
    float3 target_w;  // target angular velocity, constraint space of body B
    float4 target_q;  // target orientation, constraint space
    float swing_freq, swing_damping, twist_freq, twist_damping;
    float swing_min_torque, swing_max_torque, twist_min_torque, twist_max_torque;
    // per-step state
    float3 ws_y, ws_z, ws_twist, ws_motor[3];
    DevPoint pt;
    DevAngle sy, sz, tw, motor[3];  // limits (swing Y, swing Z, twist), motors (twist, swing Y, swing Z)
};

// SixDOFConstraint (six-dof-constraint.ts:66-117): per-axis limits, friction and motors over
// translation X Y Z and rotation X Y Z of the constraint frame; the rotation limits through the
// swing-twist part (the same fields as DevSwing's, read by the same templates)
enum : int { SD_TRANS_MOTOR = 1, SD_ROT_MOTOR = 2, SD_SPRING_LIMITS = 4 };
struct DevSixDof {
    DevJointHead h;
    int swing_type, rotation_flags;
    int free_axis, fixed_axis, flags, rot_pos_motor;  // axis bits; SD_*; rotation position motors (bits 0-2)
    float3 lp1, lp2;
    float4 c2b1, c2b2;  // constraint space to body space
    float limit_min[6], limit_max[6], max_friction[6];
    int limits_spring_mode[3];
    float limits_freq[3], limits_damping[3];
    int motor_state[6], motor_spring_mode[6];
    float motor_freq[6], motor_damping[6], motor_min_force[6], motor_max_force[6];
    float3 target_v, target_w, target_p;
    float4 target_q;
    // swing-twist part limits (sines and cosines of half angles)
    float sin_twist_min, sin_twist_max, cos_twist_min, cos_twist_max;
    float y_half_min, y_half_max, sin_y_min, sin_y_max, cos_y_min, cos_y_max;
    float z_half_min, z_half_max, sin_z_min, sin_z_max, cos_z_min, cos_z_max;
    // per-step state
    float3 t_axis[3], r_axis[3];
    float disp[3];
    float3 ws_y, ws_z, ws_twist;
    DevAngle sy, sz, tw;
    DevAxis trans[3], motor_t[3];
    DevAngle motor_r[3];
    DevPoint pt;
    DevEuler rot;
};

// impulse adjoints handed from one step's reverse to the previous step's, keyed by body pair
struct AdjHandoff {
    unsigned long long *keys;  // cache_cap entries, EMPTY_KEY when free
    float *vals;               // 12 per entry: 4 points x (t1, t2, n)
};

// One body's continuous-collision record of a step (CCDBody ccd.ts:20-57)
struct CcdRec {
    float4 delta;   // displacement of the step | squared cast threshold
    float4 normal;  // contact normal | maximum penetration
    float4 point;   // contact point | fraction of the displacement at the hit
    float fps;      // fraction plus the penetration allowance
    float friction, restitution;  // combined materials of the hit
    int body, hit;  // the body, the body it hits (-1: none)
    int slot;       // creation rank inside its world (bodies in index order)
    int pad[2];
};

// a compound shape: its children's range and the bits of a child index in a sub-shape id
struct DevCompound {
    int first, count, sub_bits, pad;
};
// one child: its shape record (as a body's; a hull's index as int bits), its pose in the
// compound's frame, its shape type (int bits in pos.w)
struct DevChild {
    float4 params, pos, quat;
};

struct DevWorld {
    int n;          // bodies in use
    int cap;        // body capacity
    int max_pairs, max_manifolds, max_epa, cache_cap;
    int num_worlds;
    // body SoA
    float4 *pos, *quat, *com, *linvel, *angvel, *force, *torque;
    float4 *inv_inertia;  // xyz inverse inertia diagonal, w inverse mass
    float4 *inertia_rot;
    float4 *shape;        // box: hx hy hz convexRadius ; sphere: r
    float4 *material;     // friction, restitution, gravity factor, 0
    float4 *damping;      // linear damping, angular damping, max linear v, max angular v
    uint32_t *flags;
    uint2 *groups;        // collision groups, mask
    int *world;
    float4 *sleep_sph;    // 3 per body: centre xyz, radius w
    float *sleep_timer;
    double *aabb64;       // 6 per body, exact FP64 bounds
    float4 *aabb_lo, *aabb_hi;  // FP32 bounds rounded outward
    int *wake;            // wake requests raised by the contact setup
    // broadphase
    unsigned long long *morton, *morton_alt;
    int *order, *order_alt;
    int *node_parent;     // 2n-1 nodes: internal [0, n-1), leaves [n-1, 2n-1)
    int2 *node_child;
    float4 *node_lo, *node_hi;  // node bounds (w of lo = min world, w of hi = max world, as float bits)
    int *node_flag;
    int *pair_count;      // per body count of pairs it reports
    int *pair_offset;
    int2 *pair_slots;     // per body fixed slots
    int2 *pairs;
    int *pair_order;  // the pairs' indices grouped by collide class (k_pair_order)
    // narrowphase
    Manifold *manifolds;
    int *manifold_valid;
    int *epa_list;
    // constraints
    ContactConstraint *cons;
    int *cons_of_manifold;
    CacheRecord *cache_prev, *cache_cur;
    // islands
    int *uf_parent;
    int *island_of_body;
    int *island_id_of_root;
    int *island_body_count, *island_cons_count;
    int *island_body_off, *island_cons_off;
    int *island_bodies, *island_cons;
    int *island_fill_b, *island_fill_c;
    uint32_t *iter_ovr;  // per body: velocity | position << 8 iteration overrides (0: the world's counts)
    int *island_iters;   // per island: max velocity override, max position override, defaults wanted (bits 0/1)
    int *island_order;
    float4 *inv_inertia_world;   // 2 per body: xx xy xz yy | yz zz 0 0
    // scan scratch
    int *scan_tmp;
    DevCounters *ctr;
    // broadphase scratch
    unsigned int *scene;   // ordered-int scene bounds of AABB centres
    int2 *node_world;      // world range of each LBVH node
    // narrowphase scratch
    void *epa_items;
    void *epa_packed;      // packed EPA polytopes, one per thread of the packed pass
    void *epa_scratch;     // polytopes with the reference's limits, one per thread of the fallback pass
    int *epa_fallback;     // items the packed pass handed to the fallback pass
    int epa_threads;       // threads of the packed EPA pass
    int epa_packed_points; // support points a packed polytope may hold before its item falls back
    int epa_fetch_warp;    // EPA items taken 32 at a time per warp (1) or one at a time per thread (0)
    cudaStream_t aux_stream;   // second stream: the per-CTA island solve runs beside the per-warp one
    cudaStream_t aux2_stream;  // third stream: the per-thread island solve beside both
    cudaStream_t aux3_stream;  // fourth stream: the per-warp solve of the islands past 32 contacts
    cudaEvent_t ev_fork, ev_join, ev_join2, ev_join3;
    int warp_blocks_per_sm;  // launch shape of the per-warp island solve
    int warp_carveout;       // shared-memory carveout (percent) of the per-warp island solve
    // persistent contact cache (double buffered by parity)
    unsigned long long *cache_keys[2];
    CacheRecord *cache_recs[2];
    int *cache_parity;
    // island solve scratch
    int *root_flag;
    int *small_list, *large_list;
    int *scratch_order, *scratch_colour, *scratch_claim;
    int *contact_event;               // per manifold: 1 added, 2 persisted (listener.ts:58-79)
    unsigned long long *removed_keys;  // pairs in contact last step but not this step
    int *mid_list;    // islands solved by one warp each
    DevFrame *frames;  // per body: shape decorators (allocated with the first decorated body)
    // hinge joints and their island lists
    DevHinge *hinges;
    int num_hinges, max_hinges;
    DevSwing *swings;
    int num_swings, max_swings;
    // point, distance, fixed, cone and slider joints, sorted by (type, per-type index)
    DevJoint *others;
    int num_others, max_others;
    DevSixDof *sixdofs;
    int num_sixdofs, max_sixdofs;
    int type_count[JT_TYPES];  // joints of each type (hinges and swing-twists included)
    int type_first[JT_TYPES];  // first record of each type in others
    int skip_joint_pairs;              // broadphase skips body pairs that share an enabled joint
    int *joint_partners;               // JOINT_PARTNERS per body: other bodies joined to it (-1: none)
    int *island_joint_count, *island_joint_off, *island_fill_j;
    int *small_joint_list, *large_joint_list;  // islands with joints of the per-thread / per-CTA tiers
    // 5 x max_joints: as scattered | by (type, index) | by (priority, index, type) | colour of
    // each ranked joint | ranked joints grouped by colour (per-CTA solve)
    int *island_joints;
    int max_joints;      // capacity of the per-island joint lists
    int *joint_wake;     // flag: some joint has to wake a body this step
    int *body_local;  // index of a body inside its island's body list (per-warp solve)
    // convex hull shapes
    DevHull *hulls;
    int num_hulls;
    float4 *hull_points, *hull_shrunk, *hull_planes;  // planes: normal xyz, constant w
    int2 *hull_faces;                                  // first vertex index, vertex count
    int *hull_vidx;
    // giant islands (more constraints than giant_min): solved by the whole grid
    int giant_min;
    int giant_blocks;                      // blocks of the cooperative launch (co-resident)
    int *giant_list;
    unsigned long long *giant_claim;       // 4 x cap: contact claims, two parities | joint claims, two parities
    int *giant_count;  // 4 x (GIANT_COLOURS + 2): contact colour offsets, contact fill cursors, joint offsets, joint fill
    // triangle meshes
    DevMesh *meshes;
    int num_meshes;
    int num_mesh_bodies;  // bodies with a mesh shape (0: the mesh passes are not launched)
    float4 *mesh_verts;
    int4 *mesh_tris;      // a b c (vertex indices into mesh_verts), active-edge bits
    float4 *mesh_nodes;   // 2 per node
    int *mesh_pairs;      // pairs with a mesh body this step (index into pairs)
    int *mesh_epa_base;   // per mesh pair: its first EPA item, -1 when it needs none
    int *mesh_epa_count;  // per mesh pair: its EPA items
    int *mesh_big;        // mesh pairs handed to the 32-manifold pass this step
    // compound shapes (compound.ts): per compound its children's range, per child its shape
    struct DevCompound *compounds;
    struct DevChild *children;
    int num_compounds;
    int num_compound_bodies;
    int *compound_pairs;  // pairs with a compound body and no mesh this step (index into pairs)
    void *mesh_big_red;   // MESH_BIG_THREADS reduction slots of 32 manifolds
    // continuous collision (LINEAR_CAST bodies, update.ts:896-1670)
    int num_linear_cast;  // bodies with LINEAR_CAST motion quality (0: the single-pass solve)
    int *ccd_flag;        // per body: deferred its translation this step
    int *ccd_slot;        // per body: exclusive scan of ccd_flag (its record)
    int *ccd_index;       // per body: its record this step, -1 for none
    CcdRec *ccd;          // records in body order
    int *ccd_world_off;   // num_worlds + 1: records per world, then their offsets
    int *ccd_world_fill;  // num_worlds: scatter cursors
    int *ccd_seg;         // records grouped by world
    float2 *ccd_lambda;   // per world: accumulated lambdas of the normal and friction parts
    int *ccd_scan_tmp;    // scan scratch over the worlds
};

// the mesh index of a mesh body's shape record (same int-bits encoding as hull_of)
__host__ __device__ inline int mesh_of(float4 sp) {
#ifdef __CUDA_ARCH__
    return __float_as_int(sp.x);
#else
    int v;
    memcpy(&v, &sp.x, sizeof(int));
    return v;
#endif
}
// the compound index of a compound body's shape record (the same int-bits encoding)
__host__ __device__ inline int compound_of(float4 sp) {
#ifdef __CUDA_ARCH__
    return __float_as_int(sp.x);
#else
    int v;
    memcpy(&v, &sp.x, sizeof(int));
    return v;
#endif
}
__host__ __device__ inline int hull_of(float4 sp) {
#ifdef __CUDA_ARCH__
    return __float_as_int(sp.x);
#else
    int v;
    memcpy(&v, &sp.x, sizeof(int));
    return v;
#endif
}
// body i's shape's centre of mass in the body frame (zero for the undecorated shapes but the hull)
__device__ inline float3 shape_com(const DevWorld &w, int i, uint32_t f, float4 sp) {
    if (f & F_DECORATED) {
        const float4 c = w.frames[i].com;
        return make_float3(c.x, c.y, c.z);
    }
    if (shape_of(f) != SHAPE_HULL) return make_float3(0.f, 0.f, 0.f);
    float4 c = w.hulls[hull_of(sp)].com;
    return make_float3(c.x, c.y, c.z);
}

// getInnerRadius box.ts:333-335, sphere.ts:147-149, capsule.ts:254-256, convex-hull.ts:549-558, cylinder.ts
__device__ inline float shape_inner_radius(const DevWorld &w, int i, uint32_t f, float4 sp) {
    if (f & F_DECORATED) return w.frames[i].t_pos.w;  // scaled.ts getInnerRadius: min|s| x the leaf's
    int s = shape_of(f);
    if (s == SHAPE_BOX) return fminf(sp.x, fminf(sp.y, sp.z));
    if (s == SHAPE_HULL) return w.hulls[hull_of(sp)].inner_radius;
    if (s == SHAPE_CYLINDER) return fminf(sp.x, sp.y);  // cylinder.ts getInnerRadius
    return sp.x;  // sphere and capsule radius
}

// ---- user joints of every type under one id ---------------------------------------------
__device__ __forceinline__ int joint_total(const DevWorld &w) {
    return w.num_hinges + w.num_swings + w.num_others + w.num_sixdofs;
}
__device__ __forceinline__ int joint_type_of(int id) { return id >> JOINT_TYPE_SHIFT; }
__device__ __forceinline__ int joint_index_of(int id) { return id & JOINT_INDEX_MASK; }
// the k-th joint in type order, each type in creation order (the order in which the reference
// walks its constraint pools, constraints.ts:264-318)
__device__ __forceinline__ int joint_id_at(const DevWorld &w, int k) {
    for (int t = 0; t < JT_TYPES; t++) {
        const int c = w.type_count[t];
        if (k < c) return (t << JOINT_TYPE_SHIFT) | k;
        k -= c;
    }
    return -1;
}
__device__ __forceinline__ DevJoint &other_joint(const DevWorld &w, int id) {
    return w.others[w.type_first[joint_type_of(id)] + joint_index_of(id)];
}
__device__ __forceinline__ DevJointHead &joint_head(const DevWorld &w, int id) {
    const int t = joint_type_of(id), i = joint_index_of(id);
    if (t == JT_HINGE) return w.hinges[i].h;
    if (t == JT_SWING) return w.swings[i].h;
    if (t == JT_SIX_DOF) return w.sixdofs[i].h;
    return w.others[w.type_first[t] + i].h;
}
__device__ __forceinline__ bool joint_active(const DevWorld &w, const DevJointHead &h) {
    return (h.flags & JF_ENABLED) && !(sleeping_of(w.flags[h.a]) && sleeping_of(w.flags[h.b]));
}
// solve order inside an island: (priority, per-type index, type) (constraints.ts:248-261, a
// stable sort of a list built type by type)
__device__ __forceinline__ bool joint_before(const DevWorld &w, int x, int y) {
    const DevJointHead &a = joint_head(w, x), &b = joint_head(w, y);
    if (a.priority != b.priority) return a.priority < b.priority;
    if (a.index != b.index) return a.index < b.index;
    return joint_type_of(x) < joint_type_of(y);
}


// ---------------------------------------------------------------------------
// float3 / quaternion helpers (FP32 device path)
// ---------------------------------------------------------------------------
__host__ __device__ inline float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__host__ __device__ inline float3 xyz(float4 a) { return make_float3(a.x, a.y, a.z); }
__host__ __device__ inline float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ inline float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ inline float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__host__ __device__ inline float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ inline float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ inline float lensq3(float3 a) { return dot3(a, a); }
__host__ __device__ inline float3 cross3(float3 a, float3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ inline float3 normalize3(float3 a) {
    float l = lensq3(a);
    if (l > 0.f) l = rsqrtf(l);
    return a * l;
}
// rotate vector by quaternion (x,y,z,w)
__host__ __device__ inline float3 qrot(float4 q, float3 v) {
    float3 u = f3(q.x, q.y, q.z);
    float3 t = cross3(u, v) * 2.f;
    return v + t * q.w + cross3(u, t);
}
__host__ __device__ inline float3 qrot_inv(float4 q, float3 v) { return qrot(make_float4(-q.x, -q.y, -q.z, q.w), v); }
__host__ __device__ inline float4 qmul(float4 a, float4 b) {
    return make_float4(a.x * b.w + a.w * b.x + a.y * b.z - a.z * b.y, a.y * b.w + a.w * b.y + a.z * b.x - a.x * b.z,
                       a.z * b.w + a.w * b.z + a.x * b.y - a.y * b.x, a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z);
}
// the pose of body i's collision geometry: the body's, composed with TransformedShape's
// (collideTransformedVsShape transformed.ts passes the inner shape pos + q t, q r)
__device__ __forceinline__ void geom_pose(const DevWorld &w, int i, uint32_t f, float3 &p, float4 &q) {
    p = make_float3(w.pos[i].x, w.pos[i].y, w.pos[i].z);
    q = w.quat[i];
    if (f & F_DECORATED) {
        const DevFrame &d = w.frames[i];
        p = p + qrot(q, make_float3(d.t_pos.x, d.t_pos.y, d.t_pos.z));
        q = qmul(q, d.t_rot);
    }
}
__device__ inline float4 qnormalize(float4 q) {
    float l = q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w;
    if (l > 0.f) l = rsqrtf(l);
    return make_float4(q.x * l, q.y * l, q.z * l, q.w * l);
}
// rotation matrix rows from a quaternion: r0, r1, r2 are the ROWS of R
struct Mat3 {
    float3 r0, r1, r2;
};
__host__ __device__ inline Mat3 quat_to_mat(float4 q) {
    float x2 = q.x + q.x, y2 = q.y + q.y, z2 = q.z + q.z;
    float xx = q.x * x2, yx = q.y * x2, yy = q.y * y2, zx = q.z * x2, zy = q.z * y2, zz = q.z * z2;
    float wx = q.w * x2, wy = q.w * y2, wz = q.w * z2;
    Mat3 m;
    m.r0 = f3(1.f - yy - zz, yx - wz, zx + wy);
    m.r1 = f3(yx + wz, 1.f - xx - zz, zy - wx);
    m.r2 = f3(zx - wy, zy + wx, 1.f - xx - yy);
    return m;
}
__host__ __device__ inline float3 mmul(const Mat3 &m, float3 v) { return f3(dot3(m.r0, v), dot3(m.r1, v), dot3(m.r2, v)); }
__host__ __device__ inline float3 mtmul(const Mat3 &m, float3 v) {
    return m.r0 * v.x + m.r1 * v.y + m.r2 * v.z;
}

// Symmetric 3x3 (world inverse inertia): xx xy xz yy yz zz
struct Sym3 {
    float xx, xy, xz, yy, yz, zz;
};
__host__ __device__ inline float3 symmul(const Sym3 &s, float3 v) {
    return f3(s.xx * v.x + s.xy * v.y + s.xz * v.z, s.xy * v.x + s.yy * v.y + s.yz * v.z,
              s.xz * v.x + s.yz * v.y + s.zz * v.z);
}
// I^-1_world = R Ri diag(d) (R Ri)^T, masked by the rotation DOFs
// (getInverseInertiaForRotation, motion-properties.ts:494-621)
__device__ inline Sym3 world_inv_inertia(float4 q, float4 inertia_rot, float3 d, int dof) {
    Mat3 m = quat_to_mat(qmul(q, inertia_rot));
    // columns of R*Ri are c0 = (r0.x, r1.x, r2.x) ...
    float3 c0 = f3(m.r0.x, m.r1.x, m.r2.x), c1 = f3(m.r0.y, m.r1.y, m.r2.y), c2 = f3(m.r0.z, m.r1.z, m.r2.z);
    Sym3 s;
    s.xx = d.x * c0.x * c0.x + d.y * c1.x * c1.x + d.z * c2.x * c2.x;
    s.xy = d.x * c0.x * c0.y + d.y * c1.x * c1.y + d.z * c2.x * c2.y;
    s.xz = d.x * c0.x * c0.z + d.y * c1.x * c1.z + d.z * c2.x * c2.z;
    s.yy = d.x * c0.y * c0.y + d.y * c1.y * c1.y + d.z * c2.y * c2.y;
    s.yz = d.x * c0.y * c0.z + d.y * c1.y * c1.z + d.z * c2.y * c2.z;
    s.zz = d.x * c0.z * c0.z + d.y * c1.z * c1.z + d.z * c2.z * c2.z;
    int ar = (dof >> 3) & 7;
    if (ar != 7) {
        float mx = (ar & 1) ? 1.f : 0.f, my = (ar & 2) ? 1.f : 0.f, mz = (ar & 4) ? 1.f : 0.f;
        s.xx *= mx * mx;
        s.xy *= mx * my;
        s.xz *= mx * mz;
        s.yy *= my * my;
        s.yz *= my * mz;
        s.zz *= mz * mz;
    }
    return s;
}

// An island's iteration counts (islands.ts:344-386): the largest override among its dynamic
// bodies and joints, raised to the world's count when any of them asks for the default (0).
__device__ __forceinline__ void island_iterations(const DevWorld &w, int isl, int def_vel, int def_pos, int &vel,
                                                  int &pos) {
    const int *s = w.island_iters + 3 * (size_t)isl;
    const int f = s[2];
    vel = s[0];
    pos = s[1];
    if (f & 1) vel = vel > def_vel ? vel : def_vel;
    if (f & 2) pos = pos > def_pos ? pos : def_pos;
}

// grid sizing: multiples of the current device's SM count (152 on GB300), read once per
// device with cudaDevAttrMultiProcessorCount
int device_sm_count();
inline int grid_for(int n, int block, int max_blocks_per_sm = 8) {
    int g = (n + block - 1) / block;
    int cap = device_sm_count() * max_blocks_per_sm;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return g;
}

// host launchers implemented in the .cu files
void launch_integrate_forces(DevWorld &w, float dt, cudaStream_t s);
void launch_broadphase(DevWorld &w, cudaStream_t s);
void launch_narrowphase(DevWorld &w, float dt, cudaStream_t s, cudaEvent_t mid = nullptr);
void launch_contacts_and_islands(DevWorld &w, float dt, float warm_ratio, cudaStream_t s);
// phase: SOLVE_ALL runs each island's whole solve in one pass; a world with LINEAR_CAST bodies
// runs SOLVE_VELOCITY (through the integration), the continuous-collision pass, then
// SOLVE_POSITION (position iterations, positions, sleeping)
enum : int { SOLVE_ALL = 0, SOLVE_VELOCITY = 1, SOLVE_POSITION = 2 };
void launch_solver(DevWorld &w, float dt, float warm_ratio, cudaStream_t s, cudaEvent_t mid = nullptr,
                   int phase = SOLVE_ALL);
void launch_ccd(DevWorld &w, float dt, cudaStream_t s);
void launch_ccd_bounds(DevWorld &w, float dt, cudaStream_t s);
void launch_ccd_find(DevWorld &w, float dt, cudaStream_t s);

// world ray queries: a ray is origin, length, unit direction and the world it is cast in; its hit
// is the body (-1 on a miss), the fraction of the length and the sub-shape id
struct DevRay {
    float origin[3];
    float length;
    float direction[3];
    int world;
};
struct DevRayHit {
    int body;
    float fraction;
    uint32_t sub_shape_id;
    int pad;
};
enum : int { CC_RAY_SOLID = 1, CC_RAY_BACKFACES = 2 };  // treatConvexAsSolid, collideWithBackfaces
struct DevRayFilter {
    uint32_t layer_mask, groups, mask;
    int flags;
};
// the boxes and the tree of the current poses, for queries between steps
void launch_query_tree(DevWorld &w, cudaStream_t s);
// order: the rays sorted by world and the Morton code of their origin (coherent warps), from
// launch_ray_order; keys/keys_alt 2 x nr, idx/idx_alt 2 x nr, tmp radix_tmp_ints(nr)
void launch_ray_order(DevWorld &w, const DevRay *rays, int nr, unsigned long long *keys, int *idx, int *tmp,
                      cudaStream_t s);
// the hit collectors of the queries: closest, any (the first found) and all (cast-ray-vs-shape.ts
// :66-205, cast-shape-vs-shape.ts:165-226, collide-shape-vs-shape.ts:82-176)
enum : int { COLLECT_CLOSEST = 0, COLLECT_ANY = 1, COLLECT_ALL = 2 };
// hits: nr x (mode ALL ? cap : 1) records; counts (modes ANY and ALL): hits found per ray.  Mode ALL
// leaves each ray's first min(count, cap) hits sorted by fraction, body, sub-shape id.
void launch_cast_rays(DevWorld &w, const DevRay *rays, const int *order, int nr, const DevRayFilter &f,
                      DevRayHit *hits, cudaStream_t s, int mode = COLLECT_CLOSEST, int cap = 1,
                      int *counts = nullptr);
// shape casts: a sphere, box or capsule (params as a body's shape record) at a pose, moved by a
// displacement, in a world; the hit: body (-1), fraction, normal, contact point on the cast shape
struct DevShapeCast {
    int shape_type;
    float params[4];
    float position[3];
    float quaternion[4];
    float displacement[3];
    int world;
};
struct DevShapeCastHit {
    int body;
    float fraction;
    float normal[3];
    float point[3];
    uint32_t sub_shape_id;  // the mesh triangle's, else 0xffffffff
    int pad;
};
void launch_cast_shapes(DevWorld &w, const DevShapeCast *qs, int nq, const DevRayFilter &f, DevShapeCastHit *hits,
                        cudaStream_t s, int mode = COLLECT_CLOSEST, int cap = 1, int *counts = nullptr);
// collide queries: a sphere, box or capsule at a pose in a world; the hit: body, sub-shape id of
// the body (a mesh triangle), penetration, contact points on the query shape and on the body, the
// unit penetration axis (world space)
struct DevCollideShape {
    int shape_type;
    float params[4];
    float position[3];
    float quaternion[4];
    int world;
};
struct DevCollideHit {
    int body;
    uint32_t sub_shape_id;
    float penetration;
    float point_a[3], point_b[3], axis[3];
};
struct DevCollideSettings {
    float max_separation, collision_tol, penetration_tol;
    int backfaces;
};
// hits: nq x (mode ALL ? cap : 1); counts: hits found per query (every mode).  Mode ALL leaves each
// query's first min(count, cap) hits sorted by body, then sub-shape id.
void launch_collide_shapes(DevWorld &w, const DevCollideShape *qs, int nq, const DevRayFilter &f,
                           const DevCollideSettings &cs, int mode, int cap, DevCollideHit *hits, int *counts,
                           cudaStream_t s);
// points: xyz and the world (int bits in w); out: hit count, lowest body hit (-1), its sub-shape id
void launch_collide_points(DevWorld &w, const float4 *pts, int np, const DevRayFilter &f, float tol, int4 *out,
                           cudaStream_t s);
int giant_blocks_for_device();
void launch_update_bounds(DevWorld &w, cudaStream_t s);
void upload_settings(const DevSettings &s, double spec64, cudaStream_t st);
void launch_cache_begin(DevWorld &w, cudaStream_t s);
size_t epa_scratch_bytes();
size_t mesh_big_slot_bytes();
constexpr int MESH_BIG_THREADS = 256;  // threads (and 32-manifold slots) of the mesh pairs' big-pool pass
void upload_settings_adjoint(const DevSettings &s, cudaStream_t st);
void launch_tape_record(DevWorld &w, TapeStep &t, cudaStream_t s);
void launch_tape_export(DevWorld &w, TapeStep &t, cc_tape_body *bodies, cc_tape_contact *cons, cudaStream_t s);
void checkpoint_save(const DevWorld &w, Checkpoint &c, cudaStream_t s);
void checkpoint_restore(DevWorld &w, const Checkpoint &c, cudaStream_t s);
void launch_rollout_loss(const DevWorld &w, const float *targets, unsigned long long *sums, float *loss, AdjBuffers &a,
                         cudaStream_t s);
void launch_adjoint_step(DevWorld &w, TapeStep &t, AdjBuffers &a, float dt, float ratio, const AdjHandoff &in,
                         const AdjHandoff &out, cudaStream_t s);
size_t epa_packed_block_bytes();
size_t epa_item_bytes();
inline int epa_default_max_threads() { return device_sm_count() * 4 * 64; }  // one polytope per resident EPA thread
inline int epa_max_threads() { return device_sm_count() * 8 * 64; }          // upper bound of the launch-shape override
constexpr int EPA_BIG_THREADS = 1024;  // threads of the fallback pass with the reference's polytope limits
constexpr int JOINT_PARTNERS = 8;      // joined bodies remembered per body for the broadphase pair filter
constexpr int GIANT_COLOURS = 1024;    // colours of the giant-island solve; the rest go to one thread in order

// scan / sort utilities (cc_scan.cu)
void exclusive_scan_int(const int *in, int *out, int n, int *total, int *tmp, cudaStream_t s);
void radix_sort_pairs_u64(unsigned long long *keys, unsigned long long *keys_alt, int *vals, int *vals_alt, int n,
                          int bits, int *tmp, cudaStream_t s, const int *n_dev = nullptr);
size_t scan_tmp_ints(int n);
size_t radix_tmp_ints(int n);

}  // namespace cc
