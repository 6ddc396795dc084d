"""ctypes binding of the C ABI declared in include/crashcat_gpu.h.

The shared library is built in-tree (``crashcat_gb300/libcrashcat_gpu.so``).
Loading fails loudly when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcrashcat_gpu.so")

CC_OK = 0
CC_ERR_INVALID = 1
CC_ERR_CAPACITY = 2
CC_ERR_TIMEOUT = 3
CC_ERR_NAN = 4
CC_ERR_CUDA = 5
CC_ERR_UNSUPPORTED = 6

SHAPE_SPHERE = 0
SHAPE_BOX = 1
SHAPE_CAPSULE = 2
SHAPE_CONVEX_HULL = 3
SHAPE_TRIANGLE_MESH = 4
SHAPE_CYLINDER = 5
SHAPE_PLANE = 6
SHAPE_EMPTY = 7
SHAPE_COMPOUND = 8
STATIC, KINEMATIC, DYNAMIC = 0, 1, 2
COMBINE_AVERAGE, COMBINE_MULTIPLY, COMBINE_MIN, COMBINE_MAX, COMBINE_GEOMETRIC_MEAN = 0, 1, 2, 3, 4
MAX_LAYERS = 32
STATE_FLOATS = 16  # position[3] quaternion[4] linear_velocity[3] angular_velocity[3] center_of_mass[3]


class Settings(C.Structure):
    _fields_ = [
        ("gravity", C.c_double * 3),
        ("gravity_enabled", C.c_int32),
        ("speculative_contact_distance", C.c_double),
        ("manifold_tolerance", C.c_double),
        ("collision_tolerance", C.c_double),
        ("penetration_tolerance", C.c_double),
        ("normal_cos_max_delta_rotation", C.c_double),
        ("contact_point_preserve_lambda_max_dist_sq", C.c_double),
        ("velocity_iterations", C.c_int32),
        ("position_iterations", C.c_int32),
        ("warm_starting", C.c_int32),
        ("penetration_slop", C.c_double),
        ("baumgarte_factor", C.c_double),
        ("max_penetration_distance", C.c_double),
        ("min_velocity_for_restitution", C.c_double),
        ("allow_sleeping", C.c_int32),
        ("time_before_sleep", C.c_double),
        ("point_velocity_sleep_threshold", C.c_double),
        ("num_object_layers", C.c_int32),
        ("num_broadphase_layers", C.c_int32),
        ("object_to_broadphase", C.c_int32 * MAX_LAYERS),
        ("object_pairs", C.c_uint32 * MAX_LAYERS),
        ("object_vs_broadphase", C.c_uint32 * MAX_LAYERS),
        ("broadphase_pairs", C.c_uint32 * MAX_LAYERS),
        ("max_bodies", C.c_int32),
        ("max_pairs", C.c_int32),
        ("max_manifolds", C.c_int32),
        ("num_worlds", C.c_int32),
        ("ccd_linear_cast_threshold", C.c_double),
        ("ccd_linear_cast_max_penetration", C.c_double),
        ("ccd_min_velocity_for_restitution", C.c_double),
        ("device_wait_polls", C.c_int32),
        ("island_link_attempts", C.c_int32),
    ]


class TuneReport(C.Structure):
    _fields_ = [("default_ms", C.c_float), ("tuned_ms", C.c_float), ("trials", C.c_int32),
                ("epa_blocks_per_sm", C.c_int32), ("epa_lockstep", C.c_int32), ("warp_blocks_per_sm", C.c_int32),
                ("small_island_max_contacts", C.c_int32), ("giant_min", C.c_int32),
                ("graph_kernels_per_step", C.c_int32)]


class HullInfo(C.Structure):
    _fields_ = [("num_points", C.c_int32), ("num_faces", C.c_int32), ("num_face_vertices", C.c_int32),
                ("convex_radius", C.c_float), ("volume", C.c_float), ("inner_radius", C.c_float),
                ("com", C.c_float * 3), ("inertia", C.c_float * 9), ("bounds_min", C.c_float * 3),
                ("bounds_max", C.c_float * 3)]


CAST_RAY_TREAT_CONVEX_AS_SOLID = 1
CAST_RAY_COLLIDE_WITH_BACKFACES = 2

# cc_ray: origin xyz, length, unit direction xyz, world; cc_ray_hit: body, fraction, sub-shape id
RAY_DTYPE = np.dtype([("origin", np.float32, 3), ("length", np.float32), ("direction", np.float32, 3),
                      ("world", np.int32)])
RAY_HIT_DTYPE = np.dtype([("body", np.int32), ("fraction", np.float32), ("sub_shape_id", np.uint32),
                          ("reserved", np.int32)])

# cc_point: position xyz, world; cc_point_hit: count, lowest body hit, its sub-shape id
POINT_DTYPE = np.dtype([("position", np.float32, 3), ("world", np.int32)])
POINT_HIT_DTYPE = np.dtype([("count", np.int32), ("body", np.int32), ("sub_shape_id", np.uint32),
                            ("reserved", np.int32)])

# cc_shape_cast / cc_shape_cast_hit
SHAPE_CAST_DTYPE = np.dtype([("shape_type", np.int32), ("shape_params", np.float32, 4), ("position", np.float32, 3),
                             ("quaternion", np.float32, 4), ("displacement", np.float32, 3), ("world", np.int32)])
SHAPE_CAST_HIT_DTYPE = np.dtype([("body", np.int32), ("fraction", np.float32), ("normal", np.float32, 3),
                                 ("point", np.float32, 3), ("sub_shape_id", np.uint32), ("reserved", np.int32)])
# a compound shape's child (cc_compound_child)
COMPOUND_CHILD_DTYPE = np.dtype([("shape_type", np.int32), ("shape_params", np.float32, 4),
                                 ("position", np.float32, 3), ("quaternion", np.float32, 4),
                                 ("density", np.float32)])

# query collectors (cc_collector) and the collide query's records
COLLECT_CLOSEST, COLLECT_ANY, COLLECT_ALL = 0, 1, 2
COLLIDE_SHAPE_DTYPE = np.dtype([("shape_type", np.int32), ("shape_params", np.float32, 4),
                                ("position", np.float32, 3), ("quaternion", np.float32, 4), ("world", np.int32)])
COLLIDE_SHAPE_HIT_DTYPE = np.dtype([("body", np.int32), ("sub_shape_id", np.uint32), ("penetration", np.float32),
                                    ("point_a", np.float32, 3), ("point_b", np.float32, 3),
                                    ("axis", np.float32, 3)])


class CollideShapeSettings(C.Structure):
    _fields_ = [("max_separation_distance", C.c_float), ("collision_tolerance", C.c_float),
                ("penetration_tolerance", C.c_float), ("collide_with_backfaces", C.c_int32)]


class QueryFilter(C.Structure):
    _fields_ = [("object_layer_mask", C.c_uint32), ("collision_group", C.c_uint32),
                ("collision_mask", C.c_uint32), ("flags", C.c_int32)]


class MeshInfo(C.Structure):
    _fields_ = [("num_vertices", C.c_int32), ("num_triangles", C.c_int32), ("num_nodes", C.c_int32),
                ("bounds_min", C.c_float * 3), ("bounds_max", C.c_float * 3)]


class Stats(C.Structure):
    _fields_ = [(n, C.c_int32) for n in (
        "num_bodies", "num_awake", "num_pairs", "num_manifolds", "num_contact_points", "num_epa",
        "num_islands", "max_island_constraints", "overflow_flags", "gpu_launches_per_step")] + [
        ("last_call_ms", C.c_float), ("num_giant_islands", C.c_int32), ("giant_colours", C.c_int32),
        ("num_ccd", C.c_int32), ("num_ccd_hits", C.c_int32), ("num_mesh_pairs", C.c_int32),
        ("num_mesh_hits", C.c_int32), ("mesh_reduced", C.c_int32), ("mesh_big", C.c_int32)]


# numpy mirror of cc_body_desc (natural C alignment, 4-byte fields only)
BODY_DTYPE = np.dtype([
    ("shape_type", np.int32), ("shape_params", np.float32, 4), ("density", np.float32),
    ("motion_type", np.int32), ("object_layer", np.int32), ("world", np.int32), ("allow_sleeping", np.int32),
    ("position", np.float32, 3), ("quaternion", np.float32, 4), ("linear_velocity", np.float32, 3),
    ("angular_velocity", np.float32, 3), ("friction", np.float32), ("restitution", np.float32),
    ("gravity_factor", np.float32), ("linear_damping", np.float32), ("angular_damping", np.float32),
    ("max_linear_velocity", np.float32), ("max_angular_velocity", np.float32),
    ("friction_combine", np.int32), ("restitution_combine", np.int32),
    ("collision_groups", np.uint32), ("collision_mask", np.uint32), ("allowed_dofs", np.int32),
    ("motion_quality", np.int32),
    ("num_velocity_steps_override", np.int32), ("num_position_steps_override", np.int32),
    ("shape_scale", np.float32, 3), ("shape_position", np.float32, 3), ("shape_quaternion", np.float32, 4),
    ("com_offset", np.float32, 3),
    ("mass_properties_mode", np.int32), ("mass", np.float32), ("inertia", np.float32, 6),
])
MASS_FROM_SHAPE, MASS_GIVEN, MASS_AND_INERTIA_GIVEN = 0, 1, 2
MOTION_DISCRETE, MOTION_LINEAR_CAST = 0, 1

# cc_world_step_taped: the rows of one step's velocity solve (cc_tape_body / cc_tape_contact)
TAPE_DYNAMIC, TAPE_MOVING = 1, 2
TAPE_BODY_DTYPE = np.dtype([("linear_velocity", np.float32, 3), ("angular_velocity", np.float32, 3),
                            ("inv_inertia", np.float32, 6), ("inv_mass", np.float32), ("flags", np.uint32)])
TAPE_POINT_DTYPE = np.dtype([("r_a", np.float32, 3), ("r_b", np.float32, 3), ("eff_normal", np.float32),
                             ("eff_tangent1", np.float32), ("eff_tangent2", np.float32), ("bias_normal", np.float32),
                             ("lambda_normal", np.float32), ("lambda_tangent1", np.float32),
                             ("lambda_tangent2", np.float32), ("final_normal", np.float32),
                             ("final_tangent1", np.float32), ("final_tangent2", np.float32),
                             ("prev_point", np.int32)])
TAPE_CONTACT_DTYPE = np.dtype([("body_a", np.int32), ("body_b", np.int32), ("num_points", np.int32),
                               ("island", np.int32), ("has_prev", np.int32), ("sort_key", np.uint32),
                               ("normal", np.float32, 3), ("tangent1", np.float32, 3), ("tangent2", np.float32, 3),
                               ("friction", np.float32), ("inv_mass_a", np.float32), ("inv_mass_b", np.float32),
                               ("points", TAPE_POINT_DTYPE, 4)])

EXPORTS = {
    "cc_world_settings_default": ([C.POINTER(Settings)], C.c_int),
    "cc_world_create": ([C.POINTER(Settings), C.POINTER(C.c_void_p)], C.c_int),
    "cc_world_destroy": ([C.c_void_p], C.c_int),
    "cc_world_add_bodies": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p], C.c_int),
    "cc_world_num_bodies": ([C.c_void_p, C.POINTER(C.c_int32)], C.c_int),
    "cc_world_step": ([C.c_void_p, C.c_float, C.c_int32], C.c_int),
    "cc_world_step_host": ([C.c_void_p, C.c_float, C.c_void_p, C.c_void_p], C.c_int),
    "cc_world_get_state": ([C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "cc_world_set_state": ([C.c_void_p, C.c_void_p], C.c_int),
    "cc_world_get_pairs": ([C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)], C.c_int),
    "cc_world_get_manifolds": ([C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)], C.c_int),
    "cc_world_get_stats": ([C.c_void_p, C.POINTER(Stats)], C.c_int),
    "cc_world_get_contact_events": ([C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)], C.c_int),
    "cc_world_get_island_iterations": ([C.c_void_p, C.c_void_p], C.c_int),
    "cc_world_debug_islands": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)], C.c_int),
    "cc_world_profile_steps": ([C.c_void_p, C.c_float, C.c_int32, C.c_void_p, C.c_int32], C.c_int),
    "cc_world_rollout_grad": ([C.c_void_p, C.c_float, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.c_void_p, C.c_void_p], C.c_int),
    "cc_world_autotune": ([C.c_void_p, C.c_float, C.c_int32, C.POINTER(TuneReport)], C.c_int),
    "cc_world_step_taped": ([C.c_void_p, C.c_float, C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_int32),
                             C.POINTER(C.c_float)], C.c_int),
    "cc_penetration_static": ([C.c_void_p, C.c_int32, C.c_void_p, C.c_float, C.c_float, C.c_void_p], C.c_int),
    "cc_world_add_hinges": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p], C.c_int),
    "cc_world_add_triangle_mesh": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_double, C.c_double,
                                    C.POINTER(C.c_int32)], C.c_int),
    "cc_triangle_mesh_build": ([C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_double, C.c_double, C.c_void_p,
                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "cc_world_get_triangle_mesh": ([C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p], C.c_int),
    "cc_world_get_manifold_sub_shapes": ([C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)], C.c_int),
    "cc_world_collide_points": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_float, C.c_void_p], C.c_int),
    "cc_world_collide_points_device": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_float, C.c_void_p],
                                       C.c_int),
    "cc_world_cast_shapes": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p], C.c_int),
    "cc_world_cast_shapes_device": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p], C.c_int),
    "cc_world_cast_rays": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p], C.c_int),
    "cc_world_add_compound": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p], C.c_int),
    "cc_world_cast_rays_collect": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_int32,
                                    C.c_void_p, C.c_void_p], C.c_int),
    "cc_world_cast_shapes_collect": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_int32,
                                      C.c_void_p, C.c_void_p], C.c_int),
    "cc_world_collide_shapes": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32,
                                 C.c_void_p, C.c_void_p], C.c_int),
    "cc_world_cast_rays_device": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p], C.c_int),
    "cc_world_add_convex_hull": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_float, C.POINTER(C.c_int32)], C.c_int),
    "cc_world_get_convex_hull": ([C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "cc_convex_hull_build": ([C.c_void_p, C.c_int32, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                              C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "cc_world_set_hinge_limits": ([C.c_void_p, C.c_int32, C.c_float, C.c_float], C.c_int),
    "cc_world_set_hinge_motor": ([C.c_void_p, C.c_int32, C.c_int32, C.c_float, C.c_float], C.c_int),
    "cc_world_set_hinge_enabled": ([C.c_void_p, C.c_int32, C.c_int32], C.c_int),
    "cc_world_get_hinge_angles": ([C.c_void_p, C.c_void_p, C.c_int32], C.c_int),
    "cc_world_set_skip_joint_pairs": ([C.c_void_p, C.c_int32], C.c_int),
    "cc_world_add_swing_twists": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p], C.c_int),
    "cc_world_set_swing_twist_limits": ([C.c_void_p, C.c_int32, C.c_float, C.c_float, C.c_float, C.c_float], C.c_int),
    "cc_world_set_swing_twist_motor": ([C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                        C.c_float], C.c_int),
    "cc_world_set_swing_twist_enabled": ([C.c_void_p, C.c_int32, C.c_int32], C.c_int),
    "cc_world_add_point_joints": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p], C.c_int),
    "cc_world_add_distance_joints": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p], C.c_int),
    "cc_world_add_fixed_joints": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p], C.c_int),
    "cc_world_add_cone_joints": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p], C.c_int),
    "cc_world_add_slider_joints": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p], C.c_int),
    "cc_world_set_distance": ([C.c_void_p, C.c_int32, C.c_float, C.c_float], C.c_int),
    "cc_world_set_cone_half_angle": ([C.c_void_p, C.c_int32, C.c_float], C.c_int),
    "cc_world_set_slider_limits": ([C.c_void_p, C.c_int32, C.c_float, C.c_float], C.c_int),
    "cc_world_set_slider_motor": ([C.c_void_p, C.c_int32, C.c_int32, C.c_float, C.c_float], C.c_int),
    "cc_world_get_slider_positions": ([C.c_void_p, C.c_void_p, C.c_int32], C.c_int),
    "cc_world_set_joint_enabled": ([C.c_void_p, C.c_int32, C.c_int32, C.c_int32], C.c_int),
    "cc_world_get_joint_lambdas": ([C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)],
                                   C.c_int),
    "cc_world_add_six_dof_joints": ([C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p], C.c_int),
    "cc_world_set_six_dof_limits": ([C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p], C.c_int),
    "cc_world_set_six_dof_motor": ([C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p], C.c_int),
    "cc_status_string": ([C.c_int], C.c_char_p),
}

# cc_hinge_desc (4-byte fields only) and its enums
SPACE_WORLD, SPACE_LOCAL = 0, 1
SPRING_FREQUENCY_AND_DAMPING, SPRING_STIFFNESS_AND_DAMPING = 0, 1
MOTOR_OFF, MOTOR_VELOCITY, MOTOR_POSITION = 0, 1, 2
SPRING_DTYPE = np.dtype([("mode", np.int32), ("frequency_or_stiffness", np.float32), ("damping", np.float32)])
HINGE_DTYPE = np.dtype([
    ("body_a", np.int32), ("body_b", np.int32), ("space", np.int32),
    ("point_a", np.float32, 3), ("point_b", np.float32, 3),
    ("hinge_axis_a", np.float32, 3), ("hinge_axis_b", np.float32, 3),
    ("normal_axis_a", np.float32, 3), ("normal_axis_b", np.float32, 3),
    ("limits_min", np.float32), ("limits_max", np.float32), ("limits_spring", SPRING_DTYPE),
    ("max_friction_torque", np.float32), ("motor_state", np.int32),
    ("target_angular_velocity", np.float32), ("target_angle", np.float32), ("motor_spring", SPRING_DTYPE),
    ("min_torque_limit", np.float32), ("max_torque_limit", np.float32),
    ("priority", np.int32), ("enabled", np.int32),
    ("num_velocity_steps_override", np.int32), ("num_position_steps_override", np.int32),
])


def hinge_defaults(n: int) -> np.ndarray:
    """n hinge records with hingeConstraint.create's defaults (hinge-constraint.ts:240-387):
    no limits, rigid limit spring, motor off, position-motor spring 2 Hz / damping 1,
    unbounded motor torque, priority 0, enabled."""
    h = np.zeros(n, HINGE_DTYPE)
    h["limits_min"] = -np.pi
    h["limits_max"] = np.pi
    h["motor_spring"]["frequency_or_stiffness"] = 2.0
    h["motor_spring"]["damping"] = 1.0
    h["min_torque_limit"] = -np.inf
    h["max_torque_limit"] = np.inf
    h["enabled"] = 1
    return h


# cc_swing_twist_desc
SWING_CONE, SWING_PYRAMID = 0, 1
SWING_TWIST_DTYPE = np.dtype([
    ("body_a", np.int32), ("body_b", np.int32), ("space", np.int32),
    ("position_a", np.float32, 3), ("position_b", np.float32, 3),
    ("twist_axis_a", np.float32, 3), ("plane_axis_a", np.float32, 3),
    ("twist_axis_b", np.float32, 3), ("plane_axis_b", np.float32, 3),
    ("swing_type", np.int32), ("normal_half_cone_angle", np.float32), ("plane_half_cone_angle", np.float32),
    ("twist_min_angle", np.float32), ("twist_max_angle", np.float32), ("max_friction_torque", np.float32),
    ("swing_motor_state", np.int32), ("twist_motor_state", np.int32),
    ("target_angular_velocity", np.float32, 3), ("target_orientation", np.float32, 4),
    ("swing_motor_spring", SPRING_DTYPE), ("twist_motor_spring", SPRING_DTYPE),
    ("swing_min_torque_limit", np.float32), ("swing_max_torque_limit", np.float32),
    ("twist_min_torque_limit", np.float32), ("twist_max_torque_limit", np.float32),
    ("priority", np.int32), ("enabled", np.int32),
    ("num_velocity_steps_override", np.int32), ("num_position_steps_override", np.int32),
])


def swing_twist_defaults(n: int) -> np.ndarray:
    """n swing-twist records with swingTwistConstraint.create's defaults
    (swing-twist-constraint.ts:180-296): cone swing, all limits 0 (locked), motors off with
    2 Hz / damping 1 springs and unbounded torque, identity target, priority 0, enabled."""
    h = np.zeros(n, SWING_TWIST_DTYPE)
    h["target_orientation"] = (0.0, 0.0, 0.0, 1.0)
    for f in ("swing_motor_spring", "twist_motor_spring"):
        h[f]["frequency_or_stiffness"] = 2.0
        h[f]["damping"] = 1.0
    h["swing_min_torque_limit"] = h["twist_min_torque_limit"] = -np.inf
    h["swing_max_torque_limit"] = h["twist_max_torque_limit"] = np.inf
    h["enabled"] = 1
    return h


# cc_joint_type (the reference's ConstraintType) and the point, distance, fixed, cone and
# slider joint descriptions
JOINT_POINT, JOINT_DISTANCE, JOINT_HINGE, JOINT_SLIDER, JOINT_FIXED, JOINT_CONE, JOINT_SWING_TWIST, JOINT_SIX_DOF = range(8)
_JOINT_TAIL = [("priority", np.int32), ("enabled", np.int32),
               ("num_velocity_steps_override", np.int32), ("num_position_steps_override", np.int32)]
POINT_JOINT_DTYPE = np.dtype([("body_a", np.int32), ("body_b", np.int32), ("space", np.int32),
                        ("point_a", np.float32, 3), ("point_b", np.float32, 3)] + _JOINT_TAIL)
DISTANCE_JOINT_DTYPE = np.dtype([("body_a", np.int32), ("body_b", np.int32), ("space", np.int32),
                           ("point_a", np.float32, 3), ("point_b", np.float32, 3),
                           ("min_distance", np.float32), ("max_distance", np.float32),
                           ("spring", SPRING_DTYPE)] + _JOINT_TAIL)
FIXED_JOINT_DTYPE = np.dtype([("body_a", np.int32), ("body_b", np.int32), ("space", np.int32),
                        ("auto_detect_point", np.int32), ("point_a", np.float32, 3), ("point_b", np.float32, 3),
                        ("axis_x_a", np.float32, 3), ("axis_y_a", np.float32, 3),
                        ("axis_x_b", np.float32, 3), ("axis_y_b", np.float32, 3)] + _JOINT_TAIL)
CONE_JOINT_DTYPE = np.dtype([("body_a", np.int32), ("body_b", np.int32), ("space", np.int32),
                       ("point_a", np.float32, 3), ("point_b", np.float32, 3),
                       ("twist_axis_a", np.float32, 3), ("twist_axis_b", np.float32, 3),
                       ("half_cone_angle", np.float32)] + _JOINT_TAIL)
SLIDER_JOINT_DTYPE = np.dtype([("body_a", np.int32), ("body_b", np.int32), ("space", np.int32),
                         ("auto_detect_point", np.int32), ("point_a", np.float32, 3), ("point_b", np.float32, 3),
                         ("slider_axis_a", np.float32, 3), ("slider_axis_b", np.float32, 3),
                         ("normal_axis_a", np.float32, 3), ("normal_axis_b", np.float32, 3),
                         ("limits_min", np.float32), ("limits_max", np.float32), ("limits_spring", SPRING_DTYPE),
                         ("max_friction_force", np.float32), ("motor_spring", SPRING_DTYPE),
                         ("min_force_limit", np.float32), ("max_force_limit", np.float32),
                         ("motor_state", np.int32), ("target_velocity", np.float32),
                         ("target_position", np.float32)] + _JOINT_TAIL)
SIX_DOF_JOINT_DTYPE = np.dtype([("body_a", np.int32), ("body_b", np.int32), ("space", np.int32),
                                ("swing_type", np.int32), ("position_a", np.float32, 3), ("position_b", np.float32, 3),
                                ("axis_x_a", np.float32, 3), ("axis_y_a", np.float32, 3),
                                ("axis_x_b", np.float32, 3), ("axis_y_b", np.float32, 3),
                                ("limit_min", np.float32, 6), ("limit_max", np.float32, 6),
                                ("max_friction", np.float32, 6), ("limits_spring", SPRING_DTYPE, 3),
                                ("motor_spring", SPRING_DTYPE, 6), ("motor_min_force", np.float32, 6),
                                ("motor_max_force", np.float32, 6), ("motor_state", np.int32, 6),
                                ("target_velocity", np.float32, 3), ("target_angular_velocity", np.float32, 3),
                                ("target_position", np.float32, 3), ("target_orientation", np.float32, 4)]
                               + _JOINT_TAIL)
JOINT_DTYPES = {JOINT_POINT: POINT_JOINT_DTYPE, JOINT_DISTANCE: DISTANCE_JOINT_DTYPE,
                JOINT_FIXED: FIXED_JOINT_DTYPE, JOINT_CONE: CONE_JOINT_DTYPE, JOINT_SLIDER: SLIDER_JOINT_DTYPE,
                JOINT_SIX_DOF: SIX_DOF_JOINT_DTYPE}
JOINT_ADDERS = {JOINT_POINT: "cc_world_add_point_joints", JOINT_DISTANCE: "cc_world_add_distance_joints",
                JOINT_FIXED: "cc_world_add_fixed_joints", JOINT_CONE: "cc_world_add_cone_joints",
                JOINT_SLIDER: "cc_world_add_slider_joints", JOINT_SIX_DOF: "cc_world_add_six_dof_joints"}


def joint_defaults(joint_type: int, n: int) -> np.ndarray:
    """n records of a point, distance, fixed, cone or slider joint with the reference's create
    defaults: world space, enabled, priority 0; distance bounds unset (the current distance);
    fixed axes X = (1,0,0), Y = (0,1,0); slider without limits, motor off, position-motor spring
    2 Hz / damping 1 and unbounded force (slider-constraint.ts:380-404, motor-settings.ts:37-51)."""
    h = np.zeros(n, JOINT_DTYPES[joint_type])
    h["enabled"] = 1
    if joint_type == JOINT_DISTANCE:
        h["min_distance"] = h["max_distance"] = -1.0
    elif joint_type == JOINT_FIXED:
        h["axis_x_a"] = h["axis_x_b"] = (1.0, 0.0, 0.0)
        h["axis_y_a"] = h["axis_y_b"] = (0.0, 1.0, 0.0)
    elif joint_type == JOINT_SIX_DOF:  # six-dof-constraint.ts:119-163, 405-430
        h["axis_x_a"] = h["axis_x_b"] = (1.0, 0.0, 0.0)
        h["axis_y_a"] = h["axis_y_b"] = (0.0, 1.0, 0.0)
        h["limit_min"] = (-np.inf, -np.inf, -np.inf, -np.pi, -np.pi, -np.pi)
        h["limit_max"] = (np.inf, np.inf, np.inf, np.pi, np.pi, np.pi)
        h["motor_spring"]["frequency_or_stiffness"] = (10.0, 10.0, 10.0, 2.0, 2.0, 2.0)
        h["motor_spring"]["damping"] = 1.0
        h["motor_min_force"] = -np.inf
        h["motor_max_force"] = np.inf
        h["target_orientation"] = (0.0, 0.0, 0.0, 1.0)
    elif joint_type == JOINT_SLIDER:
        h["limits_min"] = -np.inf
        h["limits_max"] = np.inf
        h["motor_spring"]["frequency_or_stiffness"] = 2.0
        h["motor_spring"]["damping"] = 1.0
        h["min_force_limit"] = -np.inf
        h["max_force_limit"] = np.inf
    return h


# cc_penetration_static limits and record layouts (numpy mirrors of the C structs)
STATIC_MAX_QUERIES = 32768
STATIC_EPA_SLOTS = 304
PENETRATION_UNSUPPORTED = -CC_ERR_UNSUPPORTED  # cc_penetration_result.hit of a shape type the query cannot take
SHAPE_POSE_DTYPE = np.dtype([("shape_type", np.int32), ("shape_params", np.float32, 4),
                             ("position", np.float32, 3), ("quaternion", np.float32, 4)])
PEN_QUERY_DTYPE = np.dtype([("a", SHAPE_POSE_DTYPE), ("b", SHAPE_POSE_DTYPE), ("max_separation", np.float32)])
PEN_RESULT_DTYPE = np.dtype([("hit", np.int32), ("normal", np.float32, 3), ("depth", np.float32),
                             ("point_a", np.float32, 3), ("point_b", np.float32, 3), ("used_epa", np.int32)])

_lib = None


class CCError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__(f"{what}: {status_string(status)} (status {status})")
        self.status = status


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(the CUDA path has no CPU fallback)")
    lib = C.CDLL(path)
    for name, (args, res) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def status_string(status: int) -> str:
    try:
        return load().cc_status_string(status).decode()
    except Exception:  # library not loadable: describe the code locally
        return {0: "ok", 1: "invalid argument", 2: "capacity", 3: "timeout", 4: "nan", 5: "cuda",
                6: "unsupported"}.get(status, "unknown")


def check(status: int, what: str) -> None:
    if status != CC_OK:
        raise CCError(status, what)


def ptr(a: np.ndarray) -> C.c_void_p:
    assert a.flags["C_CONTIGUOUS"]
    return C.c_void_p(a.ctypes.data)


def _hull_arrays(call) -> dict:
    """Runs a hull export (cc_convex_hull_build / cc_world_get_convex_hull) twice: sizes, then data."""
    info = HullInfo()
    check(call(C.byref(info), None, None, None, None, None, None), "convex hull")
    npt, nf, nv = info.num_points, info.num_faces, info.num_face_vertices
    pts = np.zeros((npt, 3), np.float32)
    shr = np.zeros((npt, 3), np.float32)
    faces = np.zeros((nf, 2), np.int32)
    vidx = np.zeros(max(nv, 1), np.int32)
    planes = np.zeros((nf, 4), np.float32)
    pf = np.zeros((npt, 4), np.int32)
    check(call(C.byref(info), ptr(pts), ptr(shr), ptr(faces), ptr(vidx), ptr(planes), ptr(pf)), "convex hull")
    return {"points": pts, "shrunk": shr, "faces": faces, "face_vertices": vidx[:nv], "planes": planes,
            "point_faces": pf, "convex_radius": info.convex_radius, "volume": info.volume,
            "inner_radius": info.inner_radius, "com": np.array(info.com[:], np.float32),
            "inertia": np.array(info.inertia[:], np.float32).reshape(3, 3),
            "bounds_min": np.array(info.bounds_min[:], np.float32),
            "bounds_max": np.array(info.bounds_max[:], np.float32)}


def _mesh_arrays(call) -> dict:
    """Runs a mesh export (cc_triangle_mesh_build / cc_world_get_triangle_mesh) twice: sizes, then data."""
    info = MeshInfo()
    check(call(C.byref(info), None, None, None, None), "triangle mesh")
    nv, nt, nn = info.num_vertices, info.num_triangles, info.num_nodes
    verts = np.zeros((max(nv, 1), 3), np.float32)
    tris = np.zeros((max(nt, 1), 4), np.int32)
    normals = np.zeros((max(nt, 1), 3), np.float32)
    nodes = np.zeros((max(nn, 1), 8), np.float32)
    check(call(C.byref(info), ptr(verts), ptr(tris), ptr(normals), ptr(nodes)), "triangle mesh")
    return {"vertices": verts[:nv], "triangles": tris[:nt], "normals": normals[:nt], "nodes": nodes[:nn],
            "bounds_min": np.array(info.bounds_min[:], np.float32),
            "bounds_max": np.array(info.bounds_max[:], np.float32)}


def build_triangle_mesh(positions, indices, degenerate_tolerance: float = -1.0,
                        active_edge_cos: float = -2.0) -> dict:
    """cc_triangle_mesh_build: the mesh as triangleMesh.create builds it (host only):
    vertices, triangles (a b c active-edge bits), normals, BVH nodes."""
    lib = load()
    p = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
    ix = np.ascontiguousarray(indices, dtype=np.int32).reshape(-1, 3)
    return _mesh_arrays(lambda info, *a: lib.cc_triangle_mesh_build(
        ptr(p), len(p), ptr(ix), len(ix), C.c_double(degenerate_tolerance), C.c_double(active_edge_cos), info, *a))


def build_convex_hull(points, convex_radius: float = -1.0) -> dict:
    """cc_convex_hull_build: the hull of the points as convexHull.create makes it (host only)."""
    lib = load()
    p = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
    return _hull_arrays(lambda info, *a: lib.cc_convex_hull_build(ptr(p), len(p), C.c_float(convex_radius), info, *a))
