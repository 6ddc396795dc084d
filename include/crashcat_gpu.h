/*
 * crashcat_gpu.h - C ABI of the GB300 (sm_103a) implementation of crashcat's
 * per-step world update.
 *
 * Every entry point returns an int status (CC_OK = 0).  No C++ exception and
 * no torch type crosses this boundary; all arrays are plain host pointers
 * owned by the caller, except where a function says "device pointer".
 *
 * Reference interface replaced by each entry point (paths inside
 * isaac-mason/crashcat):
 *   cc_world_settings_default  <- createWorldSettings        src/world-settings.ts:224-264
 *   cc_world_create            <- createWorld                src/world.ts:46-58
 *   cc_world_destroy           <- (world dropped by the GC)  src/world.ts:12-39
 *   cc_world_add_bodies        <- rigidBody.create           src/body/rigid-body.ts:390-434
 *   cc_world_step              <- updateWorld                src/update.ts:45-239
 *   cc_world_step_host         <- updateWorld, with the body state read from
 *                                 and written back to host arrays (the form a
 *                                 Node-API addon binds)      src/update.ts:45
 *   cc_world_get_state         <- reading body.position / quaternion /
 *                                 motionProperties.linearVelocity / angularVelocity /
 *                                 sleeping                   src/body/rigid-body.ts:142-252
 *   cc_world_set_state         <- rigidBody.setTransform / setLinearVelocity /
 *                                 setAngularVelocity         src/body/rigid-body.ts:758-774,
 *                                                            src/body/motion-properties.ts:647-672
 *   cc_world_get_pairs         <- world.broadphase.pairs     src/broadphase/broadphase.ts:30-35
 *   cc_world_get_manifolds     <- contact manifolds handed to
 *                                 addContactConstraint        src/constraints/contact-constraints.ts:437
 *   cc_world_get_contact_events <- Listener.onContactAdded / onContactPersisted /
 *                                 onContactRemoved, as a post-step buffer  src/listener.ts:58-98
 *   cc_world_add_convex_hull   <- convexHull.create          src/shapes/convex-hull.ts:106-446
 *   cc_world_get_convex_hull   <- reading the ConvexHullShape fields  src/shapes/convex-hull.ts:38-62
 *   cc_convex_hull_build       <- convexHull.create without a world   src/shapes/convex-hull.ts:106-446
 *   cc_world_add_triangle_mesh <- triangleMesh.create        src/shapes/triangle-mesh.ts:114-140
 *   cc_triangle_mesh_build     <- buildTriangleMesh without a world
 *                                                            src/shapes/utils/triangle-mesh-builder.ts:62-231
 *   cc_world_get_triangle_mesh <- reading the TriangleMeshShape data and BVH
 *                                                            src/shapes/utils/triangle-mesh-data.ts:17-25
 *   cc_world_add_hinges        <- hingeConstraint.create     src/constraints/hinge-constraint.ts:240-387
 *   cc_world_set_hinge_*       <- hingeConstraint setters    src/constraints/hinge-constraint.ts:429-465
 *   cc_world_get_hinge_angles  <- hingeConstraint.getCurrentAngle  src/constraints/hinge-constraint.ts:467-474
 *   cc_world_add_swing_twists  <- swingTwistConstraint.create src/constraints/swing-twist-constraint.ts:180-296
 *   cc_world_set_swing_twist_* <- swingTwistConstraint setters src/constraints/swing-twist-constraint.ts:319-416
 *   cc_world_set_skip_joint_pairs <- a Listener.onBodyPairValidate rejecting joined bodies
 *                                 src/broadphase/broadphase.ts:112-123
 *   cc_world_step_taped        <- updateWorld, then reading world.contactConstraints
 *                                 src/constraints/contact-constraints.ts:32-146
 *   cc_world_autotune          <- (no counterpart: launch shapes of this library)
 *   cc_world_get_stats         <- (no counterpart: per-step counters)
 *   cc_status_string           <- assert() messages          src/utils/assert.ts:1-9
 */
#ifndef CRASHCAT_GPU_H
#define CRASHCAT_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum cc_status {
    CC_OK = 0,
    CC_ERR_INVALID = 1,   /* bad argument */
    CC_ERR_CAPACITY = 2,  /* a per-step buffer overflowed; results of that step are incomplete */
    CC_ERR_TIMEOUT = 3,   /* a bounded device-side wait gave up */
    CC_ERR_NAN = 4,       /* non-finite body state detected */
    CC_ERR_CUDA = 5,      /* a CUDA runtime call failed */
    CC_ERR_UNSUPPORTED = 6
};

/* cc_body_desc.shape_params per type: sphere (radius); box (half extents x y z, convex radius);
 * capsule (radius, half height of the segment on Y); convex hull (hull index); triangle mesh
 * (mesh index); cylinder (half height on Y, radius, convex radius, with 0 <= convex radius <=
 * both; src/shapes/cylinder.ts); plane (normal x y z, normalised on creation, and the constant
 * of n . x + c = 0, solid below; src/shapes/plane.ts, half extent 1000, static or kinematic
 * bodies only: a plane has no mass); empty (no parameters, no collision, no mass;
 * src/shapes/empty-shape.ts). */
enum cc_shape_type { CC_SHAPE_SPHERE = 0, CC_SHAPE_BOX = 1, CC_SHAPE_CAPSULE = 2, CC_SHAPE_CONVEX_HULL = 3,
                     CC_SHAPE_TRIANGLE_MESH = 4, CC_SHAPE_CYLINDER = 5, CC_SHAPE_PLANE = 6, CC_SHAPE_EMPTY = 7,
                     CC_SHAPE_COMPOUND = 8 };
enum cc_motion_type { CC_STATIC = 0, CC_KINEMATIC = 1, CC_DYNAMIC = 2 };
enum cc_mass_mode { CC_MASS_FROM_SHAPE = 0, CC_MASS_GIVEN = 1, CC_MASS_AND_INERTIA_GIVEN = 2 };
enum cc_motion_quality { CC_MOTION_DISCRETE = 0, CC_MOTION_LINEAR_CAST = 1 };  /* MotionQuality motion-properties.ts:8-26 */
enum cc_combine_mode { CC_COMBINE_AVERAGE = 0, CC_COMBINE_MULTIPLY = 1, CC_COMBINE_MIN = 2, CC_COMBINE_MAX = 3,
                       CC_COMBINE_GEOMETRIC_MEAN = 4 };

#define CC_MAX_LAYERS 32

/* WorldSettings (src/world-settings.ts:4-222).  Layer tables follow
 * src/layers.ts: bit j of object_pairs[i] = objectLayerPairs[i][j], bit b of
 * object_vs_broadphase[i] = objectVsBroadphase[i][b], bit b of
 * broadphase_pairs[a] = broadphasePairs[a][b]. */
typedef struct cc_world_settings {
    double gravity[3];
    int32_t gravity_enabled;
    double speculative_contact_distance;
    double manifold_tolerance;
    double collision_tolerance;
    double penetration_tolerance;
    double normal_cos_max_delta_rotation;
    double contact_point_preserve_lambda_max_dist_sq;
    int32_t velocity_iterations;
    int32_t position_iterations;
    int32_t warm_starting;
    double penetration_slop;
    double baumgarte_factor;
    double max_penetration_distance;
    double min_velocity_for_restitution;
    int32_t allow_sleeping;
    double time_before_sleep;
    double point_velocity_sleep_threshold;
    int32_t num_object_layers;
    int32_t num_broadphase_layers;
    int32_t object_to_broadphase[CC_MAX_LAYERS];
    uint32_t object_pairs[CC_MAX_LAYERS];
    uint32_t object_vs_broadphase[CC_MAX_LAYERS];
    uint32_t broadphase_pairs[CC_MAX_LAYERS];
    /* capacities of the device world (0 = derive from max_bodies) */
    int32_t max_bodies;
    int32_t max_pairs;
    int32_t max_manifolds;
    /* number of independent worlds held by this handle (batched form); bodies
     * name their world in cc_body_desc.world */
    int32_t num_worlds;
    /* WorldSettings.ccd (world-settings.ts:198-221): a LINEAR_CAST body whose step moves it
     * more than linearCastThreshold x its inner radius is cast along its motion */
    double ccd_linear_cast_threshold;
    double ccd_linear_cast_max_penetration;
    double ccd_min_velocity_for_restitution;
    /* bounds of the device-side waits (no counterpart in the reference: the single-threaded step
     * never waits).  device_wait_polls: polls of a grid barrier of the whole-grid island solve
     * before it gives up, sets CC_ERR_TIMEOUT for the step and every block leaves (0: 2^21, about
     * 0.2 s).  island_link_attempts: compare-and-swap attempts of one union-find link before it
     * gives up; the step then skips its solve and returns CC_ERR_CAPACITY (0: 2^20). */
    int32_t device_wait_polls;
    int32_t island_link_attempts;
} cc_world_settings;

/* RigidBodySettings (src/body/rigid-body.ts:37-139) for the supported shapes.
 * shape_params: box = half extents xyz + convex radius; sphere = radius;
 * capsule = radius, half height of the cylinder (along local Y, src/shapes/capsule.ts);
 * convex hull = the hull index from cc_world_add_convex_hull (shape_params[0], a whole number). */
typedef struct cc_body_desc {
    int32_t shape_type;
    float shape_params[4];
    float density;
    int32_t motion_type;
    int32_t object_layer;
    int32_t world;
    int32_t allow_sleeping;
    float position[3];
    float quaternion[4];
    float linear_velocity[3];
    float angular_velocity[3];
    float friction;
    float restitution;
    float gravity_factor;
    float linear_damping;
    float angular_damping;
    float max_linear_velocity;
    float max_angular_velocity;
    int32_t friction_combine;
    int32_t restitution_combine;
    uint32_t collision_groups;
    uint32_t collision_mask;
    int32_t allowed_dofs;
    int32_t motion_quality;  /* cc_motion_quality */
    /* MotionProperties.numVelocityStepsOverride / numPositionStepsOverride
     * (src/body/motion-properties.ts:59-61): 0 = the world's iteration counts.  An island
     * runs the largest override of its dynamic bodies and joints, and at least the world's
     * count when any of them is 0 (src/islands.ts:344-386).  At most 255. */
    int32_t num_velocity_steps_override;
    int32_t num_position_steps_override;
    /* Shape decorators around the shape above (src/shapes/scaled.ts, transformed.ts,
     * offset-center-of-mass.ts), nested as OffsetCenterOfMassShape(TransformedShape(
     * ScaledShape(shape))); all zero = no decorator.
     *  - shape_scale: ScaledShape.scale, a zero component reads as 1.  The scale is baked into
     *    the shape: box half extents |s| per axis with the convex radius min(r min|s|, 0.05)
     *    (setBoxSupport support.ts:343-372); sphere and capsule |s.x| (sphere.ts:195-197,
     *    capsule.ts:308-318).  A scaled convex hull or triangle mesh is CC_ERR_UNSUPPORTED.
     *    Mass properties follow massProperties.scale (mass-properties.ts:59-112).
     *  - shape_position / shape_quaternion: TransformedShape, the shape's pose in the body
     *    frame (all-zero quaternion = identity); collisions, casts and queries see the shape
     *    there (collideTransformedVsShape, transformed.ts).
     *  - com_offset: OffsetCenterOfMassShape.offset, moves the centre of mass (and the
     *    inertia by the parallel-axis term) but not the collision geometry. */
    float shape_scale[3];
    float shape_position[3];
    float shape_quaternion[4];
    float com_offset[3];
    /* Mass properties (RigidBodySettings.mass / massPropertiesOverride, rigid-body.ts:309-326,
     * 676-700): cc_mass_mode; with CC_MASS_GIVEN the shape's inertia is scaled to `mass`
     * (scaleToMass mass-properties.ts:220-240); with CC_MASS_AND_INERTIA_GIVEN `mass` and
     * `inertia` (xx xy xz yy yz zz, about the centre of mass, body frame) are used as given.
     * A dynamic body whose shape has no mass (empty) needs one of them. */
    int32_t mass_properties_mode;
    float mass;
    float inertia[6];
} cc_body_desc;

/* Per-step counters of the last completed step. */
typedef struct cc_stats {
    int32_t num_bodies;
    int32_t num_awake;
    int32_t num_pairs;
    int32_t num_manifolds;
    int32_t num_contact_points;
    int32_t num_epa;
    int32_t num_islands;
    int32_t max_island_constraints;
    int32_t overflow_flags;
    int32_t gpu_launches_per_step;
    float last_call_ms; /* device time of the last cc_world_step call (CUDA events on the world's stream) */
    int32_t num_giant_islands; /* islands solved by the whole grid in the last step */
    int32_t giant_colours;     /* colours of the largest of them */
    int32_t num_ccd;           /* LINEAR_CAST bodies cast along their motion in the last step */
    int32_t num_ccd_hits;      /* of them, those whose cast hit a body (findCCDContacts update.ts:1354) */
    int32_t num_mesh_pairs;    /* broadphase pairs with a triangle mesh body */
    int32_t num_mesh_hits;     /* triangle hits handed to those pairs' reduction */
    int32_t mesh_reduced;      /* mesh pairs whose hits wanted more manifolds than the reference's pool of 32 */
    int32_t mesh_big;          /* mesh pairs whose hits needed more than 4 manifolds (run again with 32) */
} cc_stats;

typedef struct cc_world cc_world;

/* One child of a compound shape (src/shapes/compound.ts CompoundShapeChild): a convex shape
 * (sphere, box, capsule, cylinder, or a convex hull of the world, shape_params as a body's),
 * its pose in the compound's frame and its density (the compound's mass, centre of mass and
 * inertia sum the children's, compound.ts:110-230). */
typedef struct cc_compound_child {
    int32_t shape_type;
    float shape_params[4];
    float position[3];
    float quaternion[4];  /* x, y, z, w */
    float density;
} cc_compound_child;

int cc_world_settings_default(cc_world_settings *out);
int cc_world_create(const cc_world_settings *settings, cc_world **out);
int cc_world_destroy(cc_world *world);
int cc_world_add_bodies(cc_world *world, const cc_body_desc *bodies, int32_t n, int32_t *out_index);
/* compound.create (compound.ts:43-57) from n >= 1 convex children; *out_index is the index a
 * body names in shape_params[0] with shape_type CC_SHAPE_COMPOUND.  A compound body takes no
 * decorators and no LINEAR_CAST motion quality (CC_ERR_UNSUPPORTED); its density field is
 * unused (the children carry theirs). */
int cc_world_add_compound(cc_world *world, const cc_compound_child *children, int32_t n, int32_t *out_index);
int cc_world_num_bodies(const cc_world *world, int32_t *out);

/* Advance every world held by the handle by n_steps steps of dt seconds; the
 * body state stays resident in device memory.  Blocks until the steps end. */
int cc_world_step(cc_world *world, float dt, int32_t n_steps);

/* One step with the body state exchanged through host arrays: the
 * per-body state rows (cc_world_set_state layout) are uploaded, the world is
 * stepped once, and the new state is written to state_out. */
int cc_world_step_host(cc_world *world, float dt, const float *state_in, float *state_out);

/* State rows of 16 floats per body: position[3] quaternion[4]
 * linear_velocity[3] angular_velocity[3] center_of_mass[3]; plus one byte
 * per body for the sleeping flag (may be NULL). */
int cc_world_get_state(cc_world *world, float *rows, uint8_t *sleeping);
int cc_world_set_state(cc_world *world, const float *rows);

/* Broadphase pairs of the last step as (query body index, other body index). */
int cc_world_get_pairs(cc_world *world, int32_t *out, int32_t capacity, int32_t *count);

/* Contact manifolds of the last step, 32 floats each: bodyA, bodyB (ordered by
 * id), point count, normal[3] (A to B), penetration depth, summed normal
 * impulse of the contact after the velocity solve, then 4 x (world point on
 * A[3], world point on B[3]). */
int cc_world_get_manifolds(cc_world *world, float *out, int32_t capacity, int32_t *count);
/* The sub-shape ids (A, B) of the same manifolds, in the same order: 0xffffffff for a convex
 * shape, a mesh triangle's id (subShape.pushIndex sub-shape.ts:60-64) for a mesh. */
int cc_world_get_manifold_sub_shapes(cc_world *world, uint32_t *out, int32_t capacity, int32_t *count);

int cc_world_get_stats(cc_world *world, cc_stats *out);

/* Contact events of the last step, the event buffer that stands in for the listener
 * callbacks onContactAdded / onContactPersisted / onContactRemoved (src/listener.ts:58-98;
 * fired at src/constraints/contact-constraints.ts:494-499 and src/contacts.ts:305-307), which
 * kernels cannot call.  3 ints per event: type (1 added, 2 persisted, 3 removed), body A,
 * body B (body indices, A < B), sorted by (type, A, B).  *count is the number of events
 * (more than capacity when out is too small). */
int cc_world_get_contact_events(cc_world *world, int32_t *out, int32_t capacity, int32_t *count);

/* ---------------------------------------------------------------------------
 * Convex hull shapes (src/shapes/convex-hull.ts).  convexHull.create
 * (convex-hull.ts:106-446): the hull of the points (hull tolerance 1e-3), its
 * centre of mass, volume and unit-density inertia, the points relative to the
 * centre of mass, the convex radius (convex_radius < 0 selects the default
 * 0.05) reduced for thin hulls and sharp vertices.  At most 256 hull vertices;
 * flat or degenerate input returns CC_ERR_INVALID.  Bodies name the hull in
 * cc_body_desc.shape_params[0] with shape_type CC_SHAPE_CONVEX_HULL; a body's
 * position is the frame of the input points, its centre of mass position +
 * rotation x com.
 * ------------------------------------------------------------------------- */
typedef struct cc_hull_info {
    int32_t num_points, num_faces, num_face_vertices;
    float convex_radius, volume, inner_radius;
    float com[3];           /* centre of mass in the input frame */
    float inertia[9];       /* about the centre of mass at unit density, row-major */
    float bounds_min[3], bounds_max[3];  /* of the points, relative to the centre of mass */
} cc_hull_info;

int cc_world_add_convex_hull(cc_world *world, const float *points, int32_t n, float convex_radius,
                             int32_t *out_hull);
/* The same construction without a world (host only, no device needed): fills info and, where
 * not NULL, the arrays of cc_world_get_convex_hull below (call once with NULL arrays to size
 * them). */
int cc_convex_hull_build(const float *in_points, int32_t n, float convex_radius, cc_hull_info *info, float *points,
                         float *shrunk, int32_t *faces, int32_t *face_vertices, float *planes, int32_t *point_faces);
/* Read back a built hull: info always; then, where not NULL, points and shrunk points
 * (num_points x 3 floats, relative to the centre of mass; shrunk = moved inwards by the convex
 * radius, the support points of the GJK pass), faces (num_faces x 2: first face vertex, count),
 * face_vertices (num_face_vertices point indices), planes (num_faces x 4: normal, constant),
 * point_faces (num_points x 4: count, then up to 3 face indices). */
int cc_world_get_convex_hull(cc_world *world, int32_t hull, cc_hull_info *info, float *points, float *shrunk,
                             int32_t *faces, int32_t *face_vertices, float *planes, int32_t *point_faces);

/* ---------------------------------------------------------------------------
 * Triangle meshes (src/shapes/triangle-mesh.ts).  triangleMesh.create builds the mesh
 * (buildTriangleMesh triangle-mesh-builder.ts:62-231): vertices welded on a 1e-8 grid,
 * degenerate triangles (|edge cross| < degenerate_tolerance) and duplicates dropped, active
 * edges from the dihedral cosine threshold, a BVH of at most 8 triangles per leaf split at
 * the middle of the longest centre extent.  The triangle order the BVH leaves defines the
 * triangle indices (sub-shape ids).  A mesh has no mass (triangle-mesh.ts:153-158): mesh
 * bodies are static or kinematic, named by the mesh index in shape_params[0] with shape_type
 * CC_SHAPE_TRIANGLE_MESH.  Positions and tolerances are FP64, as the reference builds; the
 * device keeps the welded vertices in FP32.  Limits of this library: at most 2^21 - 1 triangles per mesh, and a
 * world holding a mesh body has at most 2^21 - 1 bodies (the contact key packs both).
 * degenerate_tolerance < 0 selects the default 1e-6, active_edge_cos < -1 the default
 * cos 5 degrees (0.996195); a negative cosine keeps every edge active.
 * ------------------------------------------------------------------------- */
typedef struct cc_mesh_info {
    int32_t num_vertices, num_triangles, num_nodes;
    float bounds_min[3], bounds_max[3];
} cc_mesh_info;

int cc_world_add_triangle_mesh(cc_world *world, const double *positions, int32_t num_vertices,
                               const int32_t *indices, int32_t num_triangles, double degenerate_tolerance,
                               double active_edge_cos, int32_t *out_mesh);
/* The same construction without a world: info and, where not NULL, the arrays of
 * cc_world_get_triangle_mesh. */
int cc_triangle_mesh_build(const double *positions, int32_t num_vertices, const int32_t *indices,
                           int32_t num_triangles, double degenerate_tolerance, double active_edge_cos,
                           cc_mesh_info *info, float *vertices, int32_t *triangles, float *normals, float *nodes);
/* Read back a built mesh: vertices (num_vertices x 3), triangles (num_triangles x 4: vertex
 * indices a b c, active-edge bits AB 1 / BC 2 / CA 4), normals (num_triangles x 3), nodes
 * (num_nodes x 8: min xyz, max xyz, then the right child's node index or the first triangle,
 * then the split axis or -(triangle count + 1) for a leaf; nodes in pre-order, a left child
 * right after its parent). */
int cc_world_get_triangle_mesh(cc_world *world, int32_t mesh, cc_mesh_info *info, float *vertices,
                               int32_t *triangles, float *normals, float *nodes);

/* ---------------------------------------------------------------------------
 * Hinge joints (src/constraints/hinge-constraint.ts).  HingeConstraintSettings
 * (hinge-constraint.ts:125-164) with its SpringSettings (src/constraints/
 * constraint-part/spring-settings.ts) and MotorSettings (motor-settings.ts)
 * flattened.  A joint joins two bodies of the same world; it links their
 * islands, is set up, warm started and solved after the island's contacts in
 * (priority, creation order), as updateWorld does (src/update.ts:100-165).
 * ------------------------------------------------------------------------- */
enum cc_constraint_space { CC_SPACE_WORLD = 0, CC_SPACE_LOCAL = 1 };
enum cc_spring_mode { CC_SPRING_FREQUENCY_AND_DAMPING = 0, CC_SPRING_STIFFNESS_AND_DAMPING = 1 };
enum cc_motor_state { CC_MOTOR_OFF = 0, CC_MOTOR_VELOCITY = 1, CC_MOTOR_POSITION = 2 };

typedef struct cc_spring_settings {
    int32_t mode;                      /* cc_spring_mode */
    float frequency_or_stiffness;      /* Hz, or N/m (N m/rad); 0 = rigid */
    float damping;                     /* damping ratio, or N s/m */
} cc_spring_settings;

typedef struct cc_hinge_desc {
    int32_t body_a, body_b;            /* body indices (cc_world_add_bodies order) */
    int32_t space;                     /* cc_constraint_space of the points and axes below */
    float point_a[3], point_b[3];      /* pivot on each body */
    float hinge_axis_a[3], hinge_axis_b[3];    /* normalised on creation */
    float normal_axis_a[3], normal_axis_b[3];  /* angle reference, perpendicular to the hinge axis */
    float limits_min, limits_max;      /* radians; [-pi, pi] or wider = no limits */
    cc_spring_settings limits_spring;  /* soft limits (frequency 0 = hard) */
    float max_friction_torque;         /* N m while the motor is off */
    int32_t motor_state;               /* cc_motor_state */
    float target_angular_velocity;     /* rad/s (velocity motor) */
    float target_angle;                /* rad (position motor); clamped to the limits */
    cc_spring_settings motor_spring;   /* position motor spring (reference default: frequency 2 Hz, damping 1) */
    float min_torque_limit, max_torque_limit;  /* N m (reference default: -inf, +inf) */
    int32_t priority;                  /* constraintPriority: lower is solved first */
    int32_t enabled;
    int32_t num_velocity_steps_override; /* hinge-constraint.ts:161-163, 0: the world's count */
    int32_t num_position_steps_override;
} cc_hinge_desc;

/* hingeConstraint.create (hinge-constraint.ts:240-387) for n joints; out_index (may be NULL)
 * receives each joint's index.  Bodies must exist and belong to one world.  World-space points
 * and axes are taken against the bodies' current poses. */
int cc_world_add_hinges(cc_world *world, const cc_hinge_desc *hinges, int32_t n, int32_t *out_index);

/* setLimits / setMotorState / setTargetAngularVelocity / setTargetAngle / enabled
 * (hinge-constraint.ts:429-465, ConstraintBase.enabled) of one joint. */
int cc_world_set_hinge_limits(cc_world *world, int32_t index, float limits_min, float limits_max);
int cc_world_set_hinge_motor(cc_world *world, int32_t index, int32_t motor_state, float target_angular_velocity,
                             float target_angle);
int cc_world_set_hinge_enabled(cc_world *world, int32_t index, int32_t enabled);

/* getCurrentAngle (hinge-constraint.ts:467-474) of every joint, n floats. */
int cc_world_get_hinge_angles(cc_world *world, float *out, int32_t capacity);

/* ---------------------------------------------------------------------------
 * Swing-twist joints (src/constraints/swing-twist-constraint.ts), the ragdoll
 * joint: a point constraint plus swing limits (a cone, or a pyramid, about the
 * constraint's Y and Z axes) and twist limits (about its X axis), with optional
 * swing and twist motors.  SwingTwistConstraintSettings
 * (swing-twist-constraint.ts:121-159) flattened; constraint space X = twist
 * axis, Z = plane axis, Y = plane x twist.  Joints of both types share the
 * island solve: ordered by (priority, per-type creation index, type).
 * ------------------------------------------------------------------------- */
enum cc_swing_type { CC_SWING_CONE = 0, CC_SWING_PYRAMID = 1 };

typedef struct cc_swing_twist_desc {
    int32_t body_a, body_b;
    int32_t space;                             /* cc_constraint_space */
    float position_a[3], position_b[3];        /* pivot on each body */
    float twist_axis_a[3], plane_axis_a[3];    /* normalised on creation */
    float twist_axis_b[3], plane_axis_b[3];
    int32_t swing_type;                        /* cc_swing_type */
    float normal_half_cone_angle;              /* swing limit about Z, radians */
    float plane_half_cone_angle;               /* swing limit about Y, radians */
    float twist_min_angle, twist_max_angle;    /* radians, in [-pi, pi] */
    float max_friction_torque;                 /* N m while a motor is off */
    int32_t swing_motor_state, twist_motor_state;  /* cc_motor_state */
    float target_angular_velocity[3];          /* rad/s, constraint space of body B */
    float target_orientation[4];               /* constraint space (x y z w); clamped to the limits */
    cc_spring_settings swing_motor_spring, twist_motor_spring;
    float swing_min_torque_limit, swing_max_torque_limit;
    float twist_min_torque_limit, twist_max_torque_limit;
    int32_t priority;
    int32_t enabled;
    int32_t num_velocity_steps_override; /* swing-twist-constraint.ts settings, 0: the world's count */
    int32_t num_position_steps_override;
} cc_swing_twist_desc;

/* swingTwistConstraint.create (swing-twist-constraint.ts:180-296) for n joints. */
int cc_world_add_swing_twists(cc_world *world, const cc_swing_twist_desc *joints, int32_t n, int32_t *out_index);

/* setNormalHalfConeAngle / setPlaneHalfConeAngle / setTwistMinAngle / setTwistMaxAngle
 * (swing-twist-constraint.ts:319-341) of one joint. */
int cc_world_set_swing_twist_limits(cc_world *world, int32_t index, float normal_half_cone_angle,
                                    float plane_half_cone_angle, float twist_min_angle, float twist_max_angle);
/* setSwingMotorState / setTwistMotorState (a change resets the motor parts' impulses),
 * setTargetAngularVelocityCS, setTargetOrientationCS, setMaxFrictionTorque
 * (swing-twist-constraint.ts:343-416); target_angular_velocity 3 floats, target_orientation 4. */
int cc_world_set_swing_twist_motor(cc_world *world, int32_t index, int32_t swing_motor_state,
                                   int32_t twist_motor_state, const float *target_angular_velocity,
                                   const float *target_orientation, float max_friction_torque);
int cc_world_set_swing_twist_enabled(cc_world *world, int32_t index, int32_t enabled);

/* ---------------------------------------------------------------------------
 * Point, distance, fixed, cone and slider joints (src/constraints/point-, distance-,
 * fixed-, cone- and slider-constraint.ts).  Every joint type keeps its own index space, as
 * the reference's per-type constraint pools do; the *_index arguments below are those
 * per-type indices.  Joints are solved after an island's contacts in (priority, index,
 * type) order (constraints.ts:248-261); the types are numbered as the reference's
 * ConstraintType (constraint-id.ts:24-36).
 * ------------------------------------------------------------------------- */
enum cc_joint_type {
    CC_JOINT_POINT = 0, CC_JOINT_DISTANCE = 1, CC_JOINT_HINGE = 2, CC_JOINT_SLIDER = 3,
    CC_JOINT_FIXED = 4, CC_JOINT_CONE = 5, CC_JOINT_SWING_TWIST = 6
};

/* PointConstraintSettings (point-constraint.ts:44-63): removes the 3 translational DOF. */
typedef struct cc_point_desc {
    int32_t body_a, body_b;
    int32_t space;                     /* cc_constraint_space of the points */
    float point_a[3], point_b[3];
    int32_t priority, enabled;
    int32_t num_velocity_steps_override, num_position_steps_override;
} cc_point_desc;
/* pointConstraint.create (point-constraint.ts:66-139) for n joints. */
int cc_world_add_point_joints(cc_world *world, const cc_point_desc *joints, int32_t n, int32_t *out_index);

/* DistanceConstraintSettings (distance-constraint.ts:58-82): keeps the attachment points
 * between min_distance and max_distance (a negative value is unset: both unset = the current
 * distance; one unset = the current distance clamped by the other), with an optional spring. */
typedef struct cc_distance_desc {
    int32_t body_a, body_b;
    int32_t space;
    float point_a[3], point_b[3];
    float min_distance, max_distance;
    cc_spring_settings spring;         /* frequency 0 = rigid */
    int32_t priority, enabled;
    int32_t num_velocity_steps_override, num_position_steps_override;
} cc_distance_desc;
/* distanceConstraint.create (distance-constraint.ts:96-204) for n joints. */
int cc_world_add_distance_joints(cc_world *world, const cc_distance_desc *joints, int32_t n, int32_t *out_index);
/* setDistance (distance-constraint.ts:484-493): a negative value keeps the current bound;
 * min > max makes both their mean. */
int cc_world_set_distance(cc_world *world, int32_t index, float min_distance, float max_distance);

/* FixedConstraintSettings (fixed-constraint.ts:63-101): welds two bodies.  The pivot is
 * point_a / point_b (the reference's omitted point is the body's centre of mass), or, with
 * auto_detect_point, the inverse-mass-weighted mean of the two centres of mass (world space
 * only).  The axes give the relative orientation to hold (defaults: X = (1,0,0), Y = (0,1,0)). */
typedef struct cc_fixed_desc {
    int32_t body_a, body_b;
    int32_t space;
    int32_t auto_detect_point;
    float point_a[3], point_b[3];
    float axis_x_a[3], axis_y_a[3], axis_x_b[3], axis_y_b[3];
    int32_t priority, enabled;
    int32_t num_velocity_steps_override, num_position_steps_override;
} cc_fixed_desc;
/* fixedConstraint.create (fixed-constraint.ts:103-250) for n joints. */
int cc_world_add_fixed_joints(cc_world *world, const cc_fixed_desc *joints, int32_t n, int32_t *out_index);

/* ConeConstraintSettings (cone-constraint.ts:94-116): a point constraint plus a cone limit
 * on the angle between the two twist axes. */
typedef struct cc_cone_desc {
    int32_t body_a, body_b;
    int32_t space;
    float point_a[3], point_b[3];
    float twist_axis_a[3], twist_axis_b[3];  /* normalised on creation */
    float half_cone_angle;                   /* radians (0: the axes stay aligned) */
    int32_t priority, enabled;
    int32_t num_velocity_steps_override, num_position_steps_override;
} cc_cone_desc;
/* coneConstraint.create (cone-constraint.ts:150-230) for n joints. */
int cc_world_add_cone_joints(cc_world *world, const cc_cone_desc *joints, int32_t n, int32_t *out_index);
/* setHalfConeAngle (cone-constraint.ts:262-264): clamped to [0, pi]. */
int cc_world_set_cone_half_angle(cc_world *world, int32_t index, float half_cone_angle);

/* SliderConstraintSettings (slider-constraint.ts:152-179): one translational DOF along the
 * slider axis, with limits (soft with a spring), friction while the motor is off, and a
 * velocity or position motor.  motor_state / target_velocity / target_position are applied
 * after creation as setMotorState / setTargetVelocity / setTargetPosition do. */
typedef struct cc_slider_desc {
    int32_t body_a, body_b;
    int32_t space;
    int32_t auto_detect_point;
    float point_a[3], point_b[3];
    float slider_axis_a[3], slider_axis_b[3];
    float normal_axis_a[3], normal_axis_b[3];
    float limits_min, limits_max;      /* metres; -inf / +inf = no limit; min is raised to <= 0, max to >= 0 */
    cc_spring_settings limits_spring;
    float max_friction_force;          /* N while the motor is off */
    cc_spring_settings motor_spring;   /* position motor (reference default: frequency 2 Hz, damping 1) */
    float min_force_limit, max_force_limit;  /* N (reference default: -inf, +inf) */
    int32_t motor_state;               /* cc_motor_state */
    float target_velocity;             /* m/s */
    float target_position;             /* m, clamped to the limits */
    int32_t priority, enabled;
    int32_t num_velocity_steps_override, num_position_steps_override;
} cc_slider_desc;
/* sliderConstraint.create (slider-constraint.ts:261-412) for n joints. */
int cc_world_add_slider_joints(cc_world *world, const cc_slider_desc *joints, int32_t n, int32_t *out_index);
/* setLimits / setMotorState + setTargetVelocity + setTargetPosition (slider-constraint.ts:488-520). */
int cc_world_set_slider_limits(cc_world *world, int32_t index, float limits_min, float limits_max);
int cc_world_set_slider_motor(cc_world *world, int32_t index, int32_t motor_state, float target_velocity,
                              float target_position);
/* getCurrentPosition (slider-constraint.ts:460-476) of every slider, n floats. */
int cc_world_get_slider_positions(cc_world *world, float *out, int32_t capacity);

/* SixDOFConstraintSettings (src/constraints/six-dof-constraint.ts:60-117).  Axes 0-2 are the
 * translations along the constraint frame's X, Y, Z, axes 3-5 the rotations about them (3 twist,
 * 4 swing Y, 5 swing Z).  An axis with limit_min >= limit_max is fixed (at limit_min); one with
 * [-inf, +inf] (translation) or [-pi, pi] (rotation) is free; anything else is limited.  The
 * constraint frame of body A (B) has columns axis_x_a, axis_y_a and their cross product.
 * motor_state / target_* are applied after creation as setMotorState / setTarget*CS do; the
 * target orientation is clamped into the rotation limits.  Reference defaults: limits free,
 * no friction, motor springs 10 Hz (translation) and 2 Hz (rotation) with damping 1, motor
 * forces unbounded, target orientation identity. */
typedef struct cc_six_dof_desc {
    int32_t body_a, body_b;
    int32_t space;
    int32_t swing_type;                /* cc_swing_type of the rotation limits */
    float position_a[3], position_b[3];
    float axis_x_a[3], axis_y_a[3];
    float axis_x_b[3], axis_y_b[3];
    float limit_min[6], limit_max[6];  /* metres (0-2) and radians (3-5) */
    float max_friction[6];             /* N or N m while an axis' motor is off */
    cc_spring_settings limits_spring[3];  /* soft translation limits when frequency_or_stiffness > 0 */
    cc_spring_settings motor_spring[6];   /* position motors */
    float motor_min_force[6], motor_max_force[6];
    int32_t motor_state[6];            /* cc_motor_state per axis */
    float target_velocity[3];          /* m/s along the constraint axes */
    float target_angular_velocity[3];  /* rad/s about the constraint axes */
    float target_position[3];          /* m, constraint space */
    float target_orientation[4];       /* x y z w, body B's constraint frame relative to A's */
    int32_t priority, enabled;
    int32_t num_velocity_steps_override, num_position_steps_override;
} cc_six_dof_desc;
/* sixDOFConstraint.create (six-dof-constraint.ts:335-480) for n joints. */
int cc_world_add_six_dof_joints(cc_world *world, const cc_six_dof_desc *joints, int32_t n, int32_t *out_index);
/* setTranslationLimits then setRotationLimits (six-dof-constraint.ts:1238-1260): 6 + 6 floats. */
int cc_world_set_six_dof_limits(cc_world *world, int32_t index, const float *limit_min, const float *limit_max);
/* setMaxFriction and setMotorState per axis, setTargetVelocityCS, setTargetAngularVelocityCS,
 * setTargetPositionCS, setTargetOrientationCS (six-dof-constraint.ts:1262-1306). */
int cc_world_set_six_dof_motor(cc_world *world, int32_t index, const int32_t *motor_state,
                               const float *target_velocity, const float *target_angular_velocity,
                               const float *target_position, const float *target_orientation,
                               const float *max_friction);

/* ConstraintBase.enabled of one joint of any type (cc_joint_type). */
int cc_world_set_joint_enabled(cc_world *world, int32_t type, int32_t index, int32_t enabled);
/* The accumulated impulses of one joint after the last step (getTotalLambda* of each type):
 * point 3 (point part); distance 1; fixed 6 (point, rotation); cone 4 (point, cone angle);
 * slider 7 (2 position, 3 rotation, limits, motor); six-DOF 18 (3 translation limits, point 3,
 * rotation 3, swing Y, swing Z, twist, 3 translation motors, 3 rotation motors).  *count
 * receives the number written. */
int cc_world_get_joint_lambdas(cc_world *world, int32_t type, int32_t index, float *out, int32_t capacity,
                               int32_t *count);

/* on != 0: the broadphase skips body pairs that share an enabled joint, the declarative form
 * of a Listener.onBodyPairValidate that rejects them (src/broadphase/broadphase.ts:112-123; the
 * ragdoll example's filter).  Each body may then share joints with at most 8 other bodies
 * (CC_ERR_CAPACITY otherwise). */
int cc_world_set_skip_joint_pairs(cc_world *world, int32_t on);

/* Stage profiler with no reference counterpart: runs n_steps steps (eager
 * launches) with CUDA events between the stages and writes the mean
 * milliseconds of [integrate forces, broadphase, narrowphase (GJK, faces,
 * clipping), EPA, contacts and islands, per-thread island solve, per-CTA
 * island solve] into stage_ms (n_stages >= 7). */
int cc_world_profile_steps(cc_world *world, float dt, int32_t n_steps, float *stage_ms, int32_t n_stages);

/* The velocity and position iteration counts of the island each body was solved in
 * during the last step (Island.numVelocitySteps / numPositionSteps, src/islands.ts:344-386):
 * 2 ints per body; -1, -1 for a body in no island (static or sleeping). */
int cc_world_get_island_iterations(cc_world *world, int32_t *out);

/* Diagnostic readout with no reference counterpart: island index per body of
 * the last step (-1 for static or sleeping bodies) and, per contact
 * constraint, the rows (bodyA, bodyB, island). */
int cc_world_debug_islands(cc_world *world, int32_t *island_of_body, int32_t *cons_rows, int32_t capacity,
                           int32_t *count);

/* Gradient of a rollout.  No counterpart in the reference: a vector-Jacobian product of
 * n_steps world steps from the current state, differentiating the velocity solve (warm start
 * and PGS, src/constraints/contact-constraints.ts:906-1053) and the integration
 * (src/update.ts:245-319, 896-976) of every step over that step's fixed contact set; the
 * contact geometry and the position-solve corrections of each step are constants, and the
 * warm start carries impulse adjoints from one step to the one before it through the contact
 * cache match.
 *   loss = sum over worlds w of |centroid_w - targets[w]|^2, the centroid taken over the
 *          world's dynamic bodies after the last step (targets: num_worlds x 3 floats);
 *   loss (num_worlds floats), grad_linvel / grad_angvel (n x 3 floats: dloss / d initial
 *   linear / angular velocity of each body) and grad_friction (n floats: dloss / d friction
 *   coefficient of each body) are written when not NULL.
 * The forward pass keeps a checkpoint every checkpoint_every steps; the backward pass
 * recomputes each segment from its checkpoint.  The world ends in the state after the
 * n_steps forward steps.  Device memory for tapes and checkpoints is allocated on the first
 * call and kept with the world. */
int cc_world_rollout_grad(cc_world *world, float dt, int32_t n_steps, int32_t checkpoint_every,
                          const float *targets, float *loss, float *grad_linvel, float *grad_angvel,
                          float *grad_friction);

/* ---------------------------------------------------------------------------
 * Launch-shape autotuner (no counterpart in the reference, which runs on one
 * thread).  Times candidate launch shapes on the world's current state and keeps
 * the fastest: coordinate descent over the EPA pass's resident blocks per SM and
 * its lock-step rounds, the per-warp island tier's blocks per SM, the largest
 * island solved by one thread, and (when the world has islands of thousands of
 * constraints) the size from which the whole grid solves an island.  Every trial
 * restores the state the call started from (bodies, contact cache, joint
 * impulses), runs one untimed step and then steps_per_trial timed steps (CUDA
 * events), so the call leaves the world where it found it.  A candidate must be
 * 2 % faster to replace the current shape.  Each island's solve order and each
 * EPA polytope are the same under every shape, so results change at most by the
 * FP32 rounding of the kernel that solves an island.
 * ------------------------------------------------------------------------- */
typedef struct cc_tune_report {
    float default_ms;            /* ms per step with the shapes the world had */
    float tuned_ms;              /* ms per step with the shapes it keeps */
    int32_t trials;
    int32_t epa_blocks_per_sm;   /* 64-thread EPA blocks per SM */
    int32_t epa_lockstep;        /* 1: a warp runs its 32 EPA items in lock-step rounds */
    int32_t warp_blocks_per_sm;  /* blocks of the per-warp island tier per SM */
    int32_t small_island_max_contacts;  /* islands up to this many contacts: one thread */
    int32_t giant_min;           /* islands with more constraints: the whole grid */
    int32_t graph_kernels_per_step;  /* kernel nodes of the captured step graph */
} cc_tune_report;

int cc_world_autotune(cc_world *world, float dt, int32_t steps_per_trial, cc_tune_report *report);

/* ---------------------------------------------------------------------------
 * One step with its solver rows read back: reading world.contactConstraints
 * after updateWorld (src/constraints/contact-constraints.ts:32-146, the rows
 * addContactConstraint builds at :437-857) together with the body velocities
 * the velocity solve starts from.  These are exactly the constants over which
 * cc_world_rollout_grad differentiates a step, so a host-side replay of the
 * rows (a frozen-contact forward, or a dual-number pass) checks the adjoint.
 *
 *   bodies   : one cc_tape_body per body (num_bodies), written when not NULL;
 *   contacts : the step's contact constraints in manifold order, up to capacity;
 *              *count = the number of constraints (more than capacity: the call
 *              returns CC_ERR_CAPACITY after the step, with nothing written);
 *   warm_ratio: the warm-start ratio dt / previous dt the step used.
 * The step itself is the one cc_world_step(world, dt, 1) takes.
 * ------------------------------------------------------------------------- */
enum { CC_TAPE_DYNAMIC = 1,  /* dynamic and awake: takes impulses in this step's solve */
       CC_TAPE_MOVING = 2 }; /* not static: its velocity enters the rows */

typedef struct cc_tape_body {
    float linear_velocity[3];   /* after the force integration, before the warm start */
    float angular_velocity[3];
    float inv_inertia[6];       /* world-space inverse inertia at the step's orientation:
                                   xx, xy, xz, yy, yz, zz (DOF mask applied) */
    float inv_mass;
    uint32_t flags;             /* CC_TAPE_* | DOF mask << 8 (cc_body_desc.allowed_dofs) */
} cc_tape_body;

typedef struct cc_tape_point {
    float r_a[3], r_b[3];       /* moment arms from the centres of mass to the contact midpoint */
    float eff_normal, eff_tangent1, eff_tangent2;  /* effective masses; 0: row inactive */
    float bias_normal;          /* calculateNormalVelocityBias */
    float lambda_normal, lambda_tangent1, lambda_tangent2;  /* warm-start impulses from the
                                   contact cache, before the warm-start ratio */
    float final_normal, final_tangent1, final_tangent2;     /* after the velocity iterations */
    int32_t prev_point;         /* cached point of the previous step it matched (-1: none) */
} cc_tape_point;

typedef struct cc_tape_contact {
    int32_t body_a, body_b;     /* body indices, ordered by id */
    int32_t num_points;
    int32_t island;
    int32_t has_prev;           /* the pair had a contact in the previous step's cache */
    uint32_t sort_key;          /* computeContactSortKey */
    float normal[3], tangent1[3], tangent2[3];
    float friction;             /* combined friction */
    float inv_mass_a, inv_mass_b;
    cc_tape_point points[4];
} cc_tape_contact;

int cc_world_step_taped(cc_world *world, float dt, cc_tape_body *bodies, cc_tape_contact *contacts,
                        int32_t capacity, int32_t *count, float *warm_ratio);

/* ---------------------------------------------------------------------------
 * World ray queries: castRay (src/query.ts:78-90) with the closest-hit
 * collector (createClosestCastRayCollector, src/collision/cast-ray-vs-shape.ts:
 * 180-205), a batch of rays per call.
 *
 * Each ray is cast against the bodies of its world at their current poses
 * (the boxes and tree are rebuilt from the poses before the rays are cast).
 * A body is a candidate when the segment origin + t * direction, t in
 * [0, length], enters its bounding box (dbvt.castRay, src/broadphase/
 * dbvt.ts:779-865), its object layer bit is set in object_layer_mask
 * (filterObjectLayer) and the groups pass (shouldPairCollide with the filter's
 * collision_group and collision_mask).  Convex shapes are cast with gjkCastRay
 * (castRayVsConvex, src/shapes/convex.ts:54-126); triangle meshes walk their
 * BVH (castRayVsTriangleMesh, src/shapes/triangle-mesh.ts:259-430).
 *
 * hit.body is the body index (-1 on a miss), hit.fraction the fraction of the
 * length (1 on a miss), hit.sub_shape_id the triangle's sub-shape id for a
 * mesh, else 0xffffffff.  Equal fractions go to the lower body index.
 * direction must be unit length (the reference normalises it, query.ts).
 * flags: CC_CAST_RAY_TREAT_CONVEX_AS_SOLID (a ray starting inside a convex
 * shape hits at fraction 0; the reference default) and
 * CC_CAST_RAY_COLLIDE_WITH_BACKFACES (mesh triangles seen from behind count).
 *
 *   cc_world_cast_rays: host arrays; returns when the hits are written.
 *   cc_world_cast_rays_device: device arrays; queued on the world's stream.
 * count < 0 or a NULL argument: CC_ERR_INVALID; count 0 does nothing.
 * ------------------------------------------------------------------------- */
#define CC_CAST_RAY_TREAT_CONVEX_AS_SOLID 1
#define CC_CAST_RAY_COLLIDE_WITH_BACKFACES 2

typedef struct cc_ray {
    float origin[3];
    float length;
    float direction[3];  /* unit */
    int32_t world;
} cc_ray;

typedef struct cc_ray_hit {
    int32_t body;
    float fraction;
    uint32_t sub_shape_id;
    int32_t reserved;
} cc_ray_hit;

typedef struct cc_query_filter {
    uint32_t object_layer_mask;  /* bit per object layer */
    uint32_t collision_group;
    uint32_t collision_mask;
    int32_t flags;               /* CC_CAST_RAY_* */
} cc_query_filter;

int cc_world_cast_rays(cc_world *world, const cc_ray *rays, int32_t count, const cc_query_filter *filter,
                       cc_ray_hit *hits);
int cc_world_cast_rays_device(cc_world *world, const cc_ray *rays, int32_t count, const cc_query_filter *filter,
                              cc_ray_hit *hits);

/* ---------------------------------------------------------------------------
 * World shape casts: castShape (src/query.ts:196-214) with the closest-hit
 * collector (ClosestCastShapeCollector, src/collision/cast-shape-vs-shape.ts:
 * 199-217) and createDefaultCastShapeSettings (:116-127), a batch per call.
 *
 * A sphere, box, capsule, cylinder or convex hull (shape_params as
 * cc_body_desc: a cylinder's convex radius at most its half height and
 * radius, a hull's index among the world's hulls) at position and
 * quaternion moves by displacement in its world.  Every body that passes the
 * filter (flags unused) and that the swept box reaches (broadphase.castAABB)
 * is cast with castShapeVsShape:
 *   - a convex body: castConvexVsConvex (src/shapes/convex.ts:744-830);
 *   - a mesh: the sphere's own cast or castConvexVsTriangleMesh.
 * hit.body is the body index (-1: miss), hit.fraction the fraction of the
 * displacement (1 on a miss), hit.normal the reference's hit normal (the
 * penetration axis negated and normalised), hit.point the contact point on
 * the cast shape, world space, hit.sub_shape_id the mesh triangle's sub-shape
 * id (0xffffffff for other shapes).  Equal fractions go to the lower body index.
 * Other cast shapes: CC_ERR_INVALID from cc_world_cast_shapes.
 *   cc_world_cast_shapes: host arrays; returns when the hits are written.
 *   cc_world_cast_shapes_device: device arrays; queued on the world's stream.
 *     The host does not read the device array, so the kernel checks each cast:
 *     one with another shape comes back as a miss (body -1, fraction 1).
 * A tree walk that outgrows its stack (64 nodes) drops the subtree it could
 * not push, so a hit may be missed: cc_world_cast_shapes then returns
 * CC_ERR_CAPACITY (the hits are still written).
 * ------------------------------------------------------------------------- */
typedef struct cc_shape_cast {
    int32_t shape_type;     /* CC_SHAPE_SPHERE, _BOX, _CAPSULE, _CYLINDER or _CONVEX_HULL */
    float shape_params[4];  /* as cc_body_desc.shape_params */
    float position[3];
    float quaternion[4];    /* x, y, z, w */
    float displacement[3];
    int32_t world;
} cc_shape_cast;

typedef struct cc_shape_cast_hit {
    int32_t body;
    float fraction;
    float normal[3];
    float point[3];
    uint32_t sub_shape_id;  /* the mesh triangle hit, else 0xffffffff */
    int32_t reserved;
} cc_shape_cast_hit;

int cc_world_cast_shapes(cc_world *world, const cc_shape_cast *casts, int32_t count, const cc_query_filter *filter,
                         cc_shape_cast_hit *hits);
int cc_world_cast_shapes_device(cc_world *world, const cc_shape_cast *casts, int32_t count,
                                const cc_query_filter *filter, cc_shape_cast_hit *hits);

/* ---------------------------------------------------------------------------
 * World point queries: collidePoint (src/query.ts:470-490) with every hit
 * collected (createAllCollidePointCollector), a batch of points per call.
 *
 * Bodies of the point's world whose bounding box holds the point
 * (dbvt.intersectPoint, src/broadphase/dbvt.ts:683-740) and that pass the
 * filter (flags unused) are tested with collidePointVsShape:
 *   - sphere: distance (src/shapes/sphere.ts:272-301);
 *   - box: half extents (src/shapes/box.ts:370-410);
 *   - capsule and convex hull: local bounds, then GJK against the point with
 *     collision_tolerance (src/shapes/convex.ts:142-216; the reference's
 *     default is 1e-4);
 *   - triangle mesh: local bounds, then the odd-even count of a +Y ray
 *     (src/shapes/triangle-mesh.ts:482-570).
 * hit.count is the number of bodies holding the point.  hit.body is the
 * lowest such body index (-1: none) and hit.sub_shape_id its sub-shape id:
 * the last triangle the mesh's ray met, else 0xffffffff.
 *   cc_world_collide_points: host arrays; returns when the hits are written.
 *   cc_world_collide_points_device: device arrays; queued on the world's stream.
 * ------------------------------------------------------------------------- */
typedef struct cc_point {
    float position[3];
    int32_t world;
} cc_point;

typedef struct cc_point_hit {
    int32_t count;
    int32_t body;
    uint32_t sub_shape_id;
    int32_t reserved;
} cc_point_hit;

int cc_world_collide_points(cc_world *world, const cc_point *points, int32_t count, const cc_query_filter *filter,
                            float collision_tolerance, cc_point_hit *hits);
int cc_world_collide_points_device(cc_world *world, const cc_point *points, int32_t count,
                                   const cc_query_filter *filter, float collision_tolerance, cc_point_hit *hits);

/* ---------------------------------------------------------------------------
 * Hit collectors of the batched queries: the closest hit, any hit, or all hits
 * (ClosestCastRayCollector / AnyCastRayCollector / AllCastRayCollector,
 * src/collision/cast-ray-vs-shape.ts:66-205; the cast-shape collectors,
 * cast-shape-vs-shape.ts:165-226; the collide-shape collectors,
 * collide-shape-vs-shape.ts:82-176).
 *
 * hits holds count x max_hits records, query i's at hits[i * max_hits]:
 *   CC_COLLECT_CLOSEST: one record per query, as cc_world_cast_rays /
 *     cc_world_cast_shapes write it (collide: the deepest penetration, ties to
 *     the lower body index, then sub-shape id); counts[i] 0 or 1 (counts may be
 *     NULL).
 *   CC_COLLECT_ANY: one record, the first hit the device tree walk meets (the
 *     walk and a mesh's triangle walk stop there); counts[i] 0 or 1.  Which hit
 *     is "first" follows the device tree, not the reference's dbvt.
 *   CC_COLLECT_ALL: every hit below the initial early-out fraction (casts) or
 *     within the separation distance (collide): one per convex body, one per
 *     mesh triangle.  counts[i] = the number found (required); the first
 *     min(counts[i], max_hits) records are sorted by fraction, body index,
 *     sub-shape id (rays and shape casts), or body, sub-shape id (collide).  A query with more hits than max_hits makes
 *     the call return CC_ERR_CAPACITY; which of its hits were kept is then
 *     unspecified (call again with the largest count).
 * The reference's All collectors keep hits in traversal order; these sort them.
 * ------------------------------------------------------------------------- */
enum cc_collector { CC_COLLECT_CLOSEST = 0, CC_COLLECT_ANY = 1, CC_COLLECT_ALL = 2 };

int cc_world_cast_rays_collect(cc_world *world, const cc_ray *rays, int32_t count, const cc_query_filter *filter,
                               int32_t collector, int32_t max_hits, cc_ray_hit *hits, int32_t *counts);
int cc_world_cast_shapes_collect(cc_world *world, const cc_shape_cast *casts, int32_t count,
                                 const cc_query_filter *filter, int32_t collector, int32_t max_hits,
                                 cc_shape_cast_hit *hits, int32_t *counts);

/* ---------------------------------------------------------------------------
 * World collide queries: collideShape (src/query.ts:286-311) with a collector
 * above.  A sphere, box or capsule (shape_params as cc_body_desc) at position
 * and quaternion, in its world.  Every body that passes the filter (flags
 * unused) and whose box meets the query's box (the local bounds through the
 * rotation, grown by max_separation_distance: broadphase.intersectAABB) is
 * collided with collideShapeVsShape (narrowphase.ts:172-238):
 *   - a convex body: collideConvexVsConvex (src/shapes/convex.ts:257-641;
 *     GJK, then EPA in FP64 when the cores overlap) or sphere-vs-sphere;
 *   - a plane: collideConvexVsPlane (src/shapes/plane.ts:474-629);
 *   - a mesh: collideConvexVsTriangleMesh / collideSphereVsTriangleMesh
 *     (src/shapes/triangle-mesh.ts), one hit per triangle, active edges
 *     honoured with no movement direction;
 *   - an empty shape: nothing.
 * The hit (CollideShapeHit collide-shape-vs-shape.ts:8-31, without faces):
 * body index, the body's sub-shape id (a mesh triangle, else 0xffffffff),
 * penetration (negative down to -max_separation_distance for a separated
 * pair), the contact points on the query shape and on the body, and the unit
 * penetration axis (the direction to move the body out), all world space.
 * Settings as createDefaultCollideShapeSettings (:202-212) names them; its
 * defaults: 0, 1e-4, 1e-4, back faces on.  Other query shapes or a negative
 * separation: CC_ERR_INVALID.
 * ------------------------------------------------------------------------- */
typedef struct cc_collide_shape {
    int32_t shape_type;     /* CC_SHAPE_SPHERE, CC_SHAPE_BOX or CC_SHAPE_CAPSULE */
    float shape_params[4];
    float position[3];
    float quaternion[4];    /* x, y, z, w */
    int32_t world;
} cc_collide_shape;

typedef struct cc_collide_shape_hit {
    int32_t body;
    uint32_t sub_shape_id;
    float penetration;
    float point_a[3];       /* on the query shape */
    float point_b[3];       /* on the body */
    float axis[3];          /* unit penetration axis */
} cc_collide_shape_hit;

typedef struct cc_collide_shape_settings {
    float max_separation_distance;
    float collision_tolerance;
    float penetration_tolerance;
    int32_t collide_with_backfaces;
} cc_collide_shape_settings;

int cc_world_collide_shapes(cc_world *world, const cc_collide_shape *shapes, int32_t count,
                            const cc_query_filter *filter, const cc_collide_shape_settings *settings,
                            int32_t collector, int32_t max_hits, cc_collide_shape_hit *hits, int32_t *counts);

/* ---------------------------------------------------------------------------
 * Allocation-free penetration query.  It has no counterpart in the reference:
 * it is this library's narrowphase of one convex pair (FP32 GJK, then FP64 EPA
 * when the shrunk shapes overlap) offered as a batch query on caller-owned
 * device buffers, with no world handle.
 *
 * Why it exists: a world handle reserves its EPA polytopes (about 47 KB per
 * EPA thread) when it is created.  Some callers cannot allocate device memory
 * at the point where they want to ask "how deep do these shape pairs overlap":
 * a frame loop with a fixed device-memory budget, a host thread that must not
 * stall the device (cudaMalloc and cudaFree synchronise it), or code that only
 * owns buffers handed to it by another allocator.  This entry point runs on
 * CC_STATIC_EPA_SLOTS polytopes and a queue of CC_STATIC_MAX_QUERIES items
 * held in file-scope device arrays of the library (about 20 MB per device,
 * held until the process exits), and calls no cudaMalloc, cudaFree or other
 * allocating routine.
 *
 * Use:
 *   - queries and results are DEVICE pointers to count elements;
 *     stream is a cudaStream_t (NULL = the legacy default stream).  The call
 *     returns after queueing its kernels; results are valid once the stream
 *     has been synchronised.
 *   - the first call on each device looks up the address of the static
 *     arrays with cudaGetSymbolAddress (with that device current); make that
 *     first call before any stream capture begins.
 *   - count > CC_STATIC_MAX_QUERIES returns CC_ERR_CAPACITY and queues
 *     nothing; count < 0 or a NULL buffer returns CC_ERR_INVALID; count == 0
 *     queues nothing and returns CC_OK.
 *   - shapes: sphere, box and capsule.  A query naming any other shape type
 *     (a convex hull or a triangle mesh, whose data lives in a world, or a
 *     value that names no shape) gets hit = CC_PENETRATION_UNSUPPORTED in its
 *     result.  The check runs on the device, so it is reported per query and
 *     not as the call's status, which would need a wait on the stream.
 *   - the EPA queue counter must start at zero: every call clears it on the
 *     stream before its first kernel.
 *   - the arrays are shared by every call on the device: two calls whose
 *     kernels overlap on the GPU (different streams, or different host
 *     threads) race on them.  Serialise calls on one stream.
 *   - A and B are taken in the given order (a world puts the body of lower
 *     motion type, then of lower id, first); max_separation is the
 *     speculative contact distance of the world settings (0 for sensors).
 * ------------------------------------------------------------------------- */
#define CC_STATIC_MAX_QUERIES 32768
#define CC_STATIC_EPA_SLOTS 304

typedef struct cc_shape_pose {
    int32_t shape_type;     /* cc_shape_type */
    float shape_params[4];  /* as cc_body_desc.shape_params */
    float position[3];
    float quaternion[4];    /* x, y, z, w */
} cc_shape_pose;

typedef struct cc_penetration_query {
    cc_shape_pose a;
    cc_shape_pose b;
    float max_separation;
} cc_penetration_query;

#define CC_PENETRATION_UNSUPPORTED (-CC_ERR_UNSUPPORTED)

typedef struct cc_penetration_result {
    int32_t hit;        /* 1: the shapes are closer than max_separation; 0: they are not;
                           CC_PENETRATION_UNSUPPORTED: a shape type this query cannot take */
    float normal[3];    /* unit contact normal, A to B, world space */
    float depth;        /* penetration depth (negative: separation) */
    float point_a[3];   /* deepest point on A, world space */
    float point_b[3];   /* deepest point on B, world space */
    int32_t used_epa;   /* 1 when the shrunk shapes overlapped and EPA ran */
} cc_penetration_result;

int cc_penetration_static(const cc_penetration_query *queries, int32_t count, cc_penetration_result *results,
                          float collision_tolerance, float penetration_tolerance, void *stream);

const char *cc_status_string(int status);

#ifdef __cplusplus
}
#endif
#endif /* CRASHCAT_GPU_H */
