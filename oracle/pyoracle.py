"""ctypes wrapper of the FP64 CPU oracle (oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg; never by the library.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

F_COUNT = 54  # doubles per body row, see oracle.cpp (enum F_*)
STATE = 17    # pos3 quat4 linvel3 angvel3 com3 sleeping

_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        import importlib.util
        spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(HERE, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    lib = C.CDLL(LIB)
    vp, dp, ip, i32 = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_int
    sig = {
        "orc_world_create": ([dp, i32, ip, i32, vp, vp, vp], vp),
        "orc_world_destroy": ([vp], None),
        "orc_add_bodies": ([vp, dp, i32], i32),
        "orc_body_count": ([vp], i32),
        "orc_set_coloured_order": ([vp, i32], None),
        "orc_reordered_islands": ([vp], i32),
        "orc_get_state": ([vp, dp], i32),
        "orc_set_state": ([vp, dp], i32),
        "orc_step": ([vp, C.c_double, i32], i32),
        "orc_pair_count": ([vp], i32),
        "orc_get_pairs": ([vp, ip], i32),
        "orc_get_aabbs": ([vp, dp], i32),
        "orc_manifold_count": ([vp], i32),
        "orc_get_manifolds": ([vp, dp], i32),
        "orc_island_count": ([vp], i32),
        "orc_ccd_counts": ([vp, ip], None),
        "orc_collide_points": ([vp, dp, i32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_double, ip, ip, vp], None),
        "orc_cast_shapes": ([vp, dp, i32, C.c_uint32, C.c_uint32, C.c_uint32, dp, ip, vp], i32),
        "orc_cast_rays": ([vp, dp, i32, C.c_uint32, C.c_uint32, C.c_uint32, i32, dp, ip, vp], None),
        "orc_add_compound": ([vp, dp, i32], i32),
        "orc_cast_rays_all": ([vp, dp, i32, C.c_uint32, C.c_uint32, C.c_uint32, i32, i32, dp, ip, vp, ip], None),
        "orc_cast_shapes_all": ([vp, dp, i32, C.c_uint32, C.c_uint32, C.c_uint32, i32, dp, ip, vp, ip], i32),
        "orc_collide_shapes_all": ([vp, dp, i32, C.c_uint32, C.c_uint32, C.c_uint32, dp, i32, dp, ip, vp, ip],
                                   i32),
        "orc_add_mesh": ([vp, i32, dp, i32, C.c_void_p, i32, dp], i32),
        "orc_get_manifold_subs": ([vp, C.c_void_p], i32),
        "orc_fix_normal": ([dp], i32),
        "orc_clip_poly_vs_plane": ([dp, i32, dp, dp, dp], i32),
        "orc_clip_poly_vs_poly": ([dp, i32, dp, i32, dp, dp], i32),
        "orc_manifold_between_faces": ([dp, dp, dp, C.c_double, dp, i32, dp, i32, dp, dp], i32),
        "orc_prune_contact_points": ([dp, dp, i32, dp], i32),
        "orc_barycentric": ([dp, dp, dp, i32, C.c_double, dp], None),
        "orc_collide_pair": ([dp, dp, C.c_double, dp], i32),
        "orc_inverse_inertia": ([dp, dp], None),
        "orc_get_events": ([vp, C.c_void_p, i32], i32),
        "orc_add_hinge": ([vp, dp], i32),
        "orc_set_skip_joint_pairs": ([vp, i32], None),
        "orc_add_swing_twist": ([vp, dp], i32),
        "orc_add_joint": ([vp, i32, dp], i32),
        "orc_get_joint_lambdas": ([vp, i32, i32, dp], i32),
        "orc_slider_position": ([vp, i32], C.c_double),
        "orc_add_hull": ([vp, i32, dp, dp, i32, C.c_void_p, i32, C.c_void_p, dp, dp], i32),
        "orc_set_record_tape": ([vp, i32], None),
        "orc_get_island_iterations": ([vp, ip], None),
        "orc_get_solver_tape": ([vp, vp, vp, vp, vp], i32),
        "orc_frozen_rollout": ([i32, i32, i32, i32, C.c_double, dp, dp, dp, dp, ip, dp, dp, dp, i32, C.c_double,
                                vp, vp, vp, dp, vp, vp], i32),
    }
    for k, (a, r) in sig.items():
        f = getattr(lib, k)
        f.argtypes = a
        f.restype = r
    _lib = lib
    return lib


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_int))


def rows_from_bodies(b: np.ndarray) -> np.ndarray:
    """BODY_DTYPE array -> oracle rows (the FP32 inputs promoted exactly to FP64)."""
    n = len(b)
    r = np.zeros((n, F_COUNT), dtype=np.float64)
    r[:, 0] = b["shape_type"]
    r[:, 1:5] = b["shape_params"].astype(np.float64)
    r[:, 5] = b["density"]
    r[:, 6] = b["motion_type"]
    r[:, 7:10] = b["position"]
    r[:, 10:14] = b["quaternion"]
    r[:, 14:17] = b["linear_velocity"]
    r[:, 17:20] = b["angular_velocity"]
    r[:, 20] = b["friction"]
    r[:, 21] = b["restitution"]
    r[:, 22] = b["object_layer"]
    r[:, 23] = b["gravity_factor"]
    r[:, 24] = b["linear_damping"]
    r[:, 25] = b["angular_damping"]
    r[:, 26] = b["allow_sleeping"]
    r[:, 27] = b["world"]
    r[:, 28] = b["collision_groups"]
    r[:, 29] = b["collision_mask"]
    r[:, 30] = b["motion_quality"]
    r[:, 31] = b["num_velocity_steps_override"]
    r[:, 32] = b["num_position_steps_override"]
    r[:, 33:36] = b["shape_scale"]
    r[:, 36:39] = b["shape_position"]
    r[:, 39:43] = b["shape_quaternion"]
    r[:, 43:46] = b["com_offset"]
    r[:, 46] = b["mass_properties_mode"]
    r[:, 47] = b["mass"]
    r[:, 48:54] = b["inertia"]
    return np.ascontiguousarray(r)


def settings_array(ws) -> np.ndarray:
    """WorldSettings (crashcat_gb300.world) -> the oracle's settings vector."""
    s = np.zeros(23, dtype=np.float64)
    s[0:3] = ws.gravity
    s[3] = ws.speculative_contact_distance
    s[4] = ws.manifold_tolerance
    s[5] = ws.collision_tolerance
    s[6] = ws.penetration_tolerance
    s[7] = ws.normal_cos_max_delta_rotation
    s[8] = ws.contact_point_preserve_lambda_max_dist_sq
    s[9] = ws.velocity_iterations
    s[10] = ws.position_iterations
    s[11] = 1.0 if ws.warm_starting else 0.0
    s[12] = ws.penetration_slop
    s[13] = ws.baumgarte_factor
    s[14] = ws.max_penetration_distance
    s[15] = ws.min_velocity_for_restitution
    s[16] = 1.0 if ws.allow_sleeping else 0.0
    s[17] = ws.time_before_sleep
    s[18] = ws.point_velocity_sleep_threshold
    s[19] = 1.0 if ws.gravity_enabled else 0.0
    s[20] = ws.ccd_linear_cast_threshold
    s[21] = ws.ccd_linear_cast_max_penetration
    s[22] = ws.ccd_min_velocity_for_restitution
    return s


class OracleWorld:
    """One oracle world built from the same bodies and settings as a GPU world."""

    def __init__(self, ws, bodies: np.ndarray, hulls=(), meshes=(), compounds=()):
        """hulls / meshes: convex hull and triangle mesh records as GpuWorld.get_convex_hull /
        get_triangle_mesh return them, in index order (the bodies name them by index);
        compounds: arrays of _lib.COMPOUND_CHILD_DTYPE records, in index order."""
        lib = load()
        self.lib = lib
        L = ws.layers
        n_obj, n_bp = len(L.object_to_broadphase), L.broadphase_layers
        obj_to_bp = np.array(L.object_to_broadphase, dtype=np.int32)
        op = np.zeros((n_obj, n_obj), dtype=np.uint8)
        ovb = np.zeros((n_obj, n_bp), dtype=np.uint8)
        bpp = np.zeros((n_bp, n_bp), dtype=np.uint8)
        for a in range(n_obj):
            for b in range(n_obj):
                op[a, b] = (L.object_pairs[a] >> b) & 1
            for b in range(n_bp):
                ovb[a, b] = (L.object_vs_broadphase[a] >> b) & 1
        for a in range(n_bp):
            for b in range(n_bp):
                bpp[a, b] = (L.broadphase_pairs[a] >> b) & 1
        self._keep = (op, ovb, bpp, obj_to_bp)
        s = settings_array(ws)
        self.h = lib.orc_world_create(dptr(s), n_obj, iptr(obj_to_bp), n_bp, op.ctypes.data, ovb.ctypes.data,
                                      bpp.ctypes.data)
        for h in hulls:
            self.add_hull(h)
        for m in meshes:
            self.add_mesh(m)
        for c in compounds:
            self.add_compound(c)
        rows = rows_from_bodies(bodies)
        assert lib.orc_add_bodies(self.h, dptr(rows), len(rows)) == 0
        self.n = len(rows)

    def add_compound(self, children) -> int:
        """A compound shape from child records (shape_type, shape_params, position, quaternion,
        density); returns its index."""
        rows = np.zeros((len(children), 13), dtype=np.float64)
        rows[:, 0] = children["shape_type"]
        rows[:, 1:5] = children["shape_params"]
        rows[:, 5:8] = children["position"]
        rows[:, 8:12] = children["quaternion"]
        rows[:, 12] = children["density"]
        k = self.lib.orc_add_compound(self.h, dptr(rows), len(rows))
        assert k >= 0, "orc_add_compound: children must be convex shapes of this world"
        return k

    def add_mesh(self, m) -> int:
        v = np.ascontiguousarray(m["vertices"], dtype=np.float64)
        t = np.ascontiguousarray(m["triangles"], dtype=np.int32)
        nd = np.ascontiguousarray(m["nodes"], dtype=np.float64)
        k = self.lib.orc_add_mesh(self.h, len(v), dptr(v), len(t), t.ctypes.data, len(nd), dptr(nd))
        assert k >= 0
        return k

    def manifold_sub_shapes(self) -> np.ndarray:
        """Sub-shape ids (A, B) of the manifolds, in manifolds() order."""
        n = self.lib.orc_manifold_count(self.h)
        o = np.zeros((max(n, 1), 2), dtype=np.uint32)
        self.lib.orc_get_manifold_subs(self.h, o.ctypes.data)
        return o[:n]

    def add_hull(self, h) -> int:
        pts = np.ascontiguousarray(h["points"], dtype=np.float64)
        shr = np.ascontiguousarray(h["shrunk"], dtype=np.float64)
        faces = np.ascontiguousarray(h["faces"], dtype=np.int32)
        vidx = np.ascontiguousarray(h["face_vertices"], dtype=np.int32)
        planes = np.ascontiguousarray(h["planes"], dtype=np.float64)
        scal = np.concatenate([[h["convex_radius"], h["volume"]], h["com"], np.ravel(h["inertia"]),
                               h["bounds_min"], h["bounds_max"]]).astype(np.float64)
        k = self.lib.orc_add_hull(self.h, len(pts), dptr(pts), dptr(shr), len(faces), faces.ctypes.data, len(vidx),
                                  vidx.ctypes.data, dptr(planes), dptr(scal))
        assert k >= 0
        return k

    def close(self):
        if self.h:
            self.lib.orc_world_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, dt: float, n: int = 1):
        self.lib.orc_step(self.h, dt, n)

    def state(self) -> np.ndarray:
        o = np.zeros((self.n, STATE), dtype=np.float64)
        self.lib.orc_get_state(self.h, dptr(o))
        return o

    def set_state(self, st: np.ndarray):
        st = np.ascontiguousarray(st, dtype=np.float64)
        self.lib.orc_set_state(self.h, dptr(st))

    def pairs(self) -> np.ndarray:
        n = self.lib.orc_pair_count(self.h)
        o = np.zeros((max(n, 1), 2), dtype=np.int32)
        self.lib.orc_get_pairs(self.h, iptr(o))
        return o[:n]

    def ccd_counts(self) -> tuple[int, int]:
        """Continuous collision of the last step: (bodies cast, casts that hit a body)."""
        o = np.zeros(2, dtype=np.int32)
        self.lib.orc_ccd_counts(self.h, iptr(o))
        return int(o[0]), int(o[1])

    def cast_rays(self, rays: np.ndarray, layer_mask: int = 0xFFFFFFFF, groups: int = 0xFFFFFFFF,
                  mask: int = 0xFFFFFFFF, treat_convex_as_solid: bool = True):
        """Closest hit of each ray (origin xyz, unit direction xyz, length) over the world's
        bodies: (fraction float64, body int32 (-1 on a miss), sub-shape id uint32)."""
        rays = np.ascontiguousarray(rays, dtype=np.float64).reshape(-1, 7)
        n = rays.shape[0]
        fr = np.zeros(max(n, 1), dtype=np.float64)
        bo = np.zeros(max(n, 1), dtype=np.int32)
        su = np.zeros(max(n, 1), dtype=np.uint32)
        self.lib.orc_cast_rays(self.h, dptr(rays), n, layer_mask, groups, mask, int(treat_convex_as_solid),
                               dptr(fr), iptr(bo), su.ctypes.data)
        return fr[:n], bo[:n], su[:n]

    def collide_points(self, points: np.ndarray, layer_mask: int = 0xFFFFFFFF, groups: int = 0xFFFFFFFF,
                       mask: int = 0xFFFFFFFF, tolerance: float = 1e-4):
        """Per point: (number of bodies containing it, the lowest such body (-1: none), its
        sub-shape id)."""
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        n = pts.shape[0]
        co = np.zeros(max(n, 1), dtype=np.int32)
        bo = np.zeros(max(n, 1), dtype=np.int32)
        su = np.zeros(max(n, 1), dtype=np.uint32)
        self.lib.orc_collide_points(self.h, dptr(pts), n, layer_mask, groups, mask, tolerance, iptr(co), iptr(bo),
                                    su.ctypes.data)
        return co[:n], bo[:n], su[:n]

    def cast_shapes(self, queries: np.ndarray, layer_mask: int = 0xFFFFFFFF, groups: int = 0xFFFFFFFF,
                    mask: int = 0xFFFFFFFF, with_subs: bool = False):
        """Closest hit of each shape cast (shape type, 4 params, position xyz, quaternion xyzw,
        displacement xyz): (fraction, normal xyz, point on the cast shape xyz) rows, the body hit
        (-1 on a miss) and, with_subs, its sub-shape id."""
        q = np.ascontiguousarray(queries, dtype=np.float64).reshape(-1, 15)
        n = q.shape[0]
        out = np.zeros((max(n, 1), 7), dtype=np.float64)
        bo = np.zeros(max(n, 1), dtype=np.int32)
        su = np.zeros(max(n, 1), dtype=np.uint32)
        if self.lib.orc_cast_shapes(self.h, dptr(q), n, layer_mask, groups, mask, dptr(out), iptr(bo),
                                    su.ctypes.data) != 0:
            raise ValueError("orc_cast_shapes: a cast shape must be a sphere, box, capsule, cylinder or one of the world's hulls")
        return (out[:n], bo[:n], su[:n]) if with_subs else (out[:n], bo[:n])

    def cast_rays_all(self, rays: np.ndarray, cap: int, layer_mask: int = 0xFFFFFFFF, groups: int = 0xFFFFFFFF,
                      mask: int = 0xFFFFFFFF, treat_convex_as_solid: bool = True):
        """Every hit of each ray (AllCastRayCollector), sorted by fraction, body, sub-shape id:
        (fractions (n, cap), bodies (n, cap), sub-shape ids (n, cap), counts (n))."""
        rays = np.ascontiguousarray(rays, dtype=np.float64).reshape(-1, 7)
        n = rays.shape[0]
        fr = np.zeros((max(n, 1), cap), dtype=np.float64)
        bo = np.full((max(n, 1), cap), -1, dtype=np.int32)
        su = np.zeros((max(n, 1), cap), dtype=np.uint32)
        co = np.zeros(max(n, 1), dtype=np.int32)
        self.lib.orc_cast_rays_all(self.h, dptr(rays), n, layer_mask, groups, mask, int(treat_convex_as_solid), cap,
                                   dptr(fr), iptr(bo), su.ctypes.data, iptr(co))
        return fr[:n], bo[:n], su[:n], co[:n]

    def cast_shapes_all(self, queries: np.ndarray, cap: int, layer_mask: int = 0xFFFFFFFF,
                        groups: int = 0xFFFFFFFF, mask: int = 0xFFFFFFFF):
        """Every hit of each shape cast (AllCastShapeCollector), sorted by fraction, body, sub-shape
        id: ((n, cap, 7) rows of fraction, normal, point; bodies (n, cap); sub-shape ids (n, cap);
        counts (n))."""
        q = np.ascontiguousarray(queries, dtype=np.float64).reshape(-1, 15)
        n = q.shape[0]
        out = np.zeros((max(n, 1), cap, 7), dtype=np.float64)
        bo = np.full((max(n, 1), cap), -1, dtype=np.int32)
        su = np.zeros((max(n, 1), cap), dtype=np.uint32)
        co = np.zeros(max(n, 1), dtype=np.int32)
        if self.lib.orc_cast_shapes_all(self.h, dptr(q), n, layer_mask, groups, mask, cap, dptr(out), iptr(bo),
                                        su.ctypes.data, iptr(co)) != 0:
            raise ValueError("orc_cast_shapes_all: a cast shape must be a sphere, box, capsule, cylinder or one of the world's hulls")
        return out[:n], bo[:n], su[:n], co[:n]

    def collide_shapes_all(self, queries: np.ndarray, cap: int, max_separation: float = 0.0,
                           collision_tolerance: float = 1e-4, penetration_tolerance: float = 1e-4,
                           backfaces: bool = True, layer_mask: int = 0xFFFFFFFF, groups: int = 0xFFFFFFFF,
                           mask: int = 0xFFFFFFFF):
        """Every hit of each collide query (shape type, 4 params, position xyz, quaternion xyzw)
        (AllCollideShapeCollector), sorted by body, sub-shape id: ((n, cap, 10) rows of
        penetration, point on the query shape, point on the body, unit axis; bodies (n, cap);
        sub-shape ids (n, cap); counts (n))."""
        q = np.ascontiguousarray(queries, dtype=np.float64).reshape(-1, 12)
        n = q.shape[0]
        st = np.array([max_separation, collision_tolerance, penetration_tolerance, float(backfaces)])
        out = np.zeros((max(n, 1), cap, 10), dtype=np.float64)
        bo = np.full((max(n, 1), cap), -1, dtype=np.int32)
        su = np.zeros((max(n, 1), cap), dtype=np.uint32)
        co = np.zeros(max(n, 1), dtype=np.int32)
        if self.lib.orc_collide_shapes_all(self.h, dptr(q), n, layer_mask, groups, mask, dptr(st), cap, dptr(out),
                                           iptr(bo), su.ctypes.data, iptr(co)) != 0:
            raise ValueError("orc_collide_shapes_all: a query shape must be a sphere, box, capsule, cylinder or one of the world's hulls")
        return out[:n], bo[:n], su[:n], co[:n]

    def aabbs(self) -> np.ndarray:
        o = np.zeros((self.n, 6), dtype=np.float64)
        self.lib.orc_get_aabbs(self.h, dptr(o))
        return o

    def add_hinge(self, desc: np.ndarray) -> int:
        """Hinge joint from a 38-double descriptor (oracle.cpp orc_add_hinge layout)."""
        d = np.ascontiguousarray(desc, dtype=np.float64)
        k = self.lib.orc_add_hinge(self.h, dptr(d))
        assert k >= 0
        return k

    def add_hinge_record(self, h) -> int:
        """Hinge joint from a cc_hinge_desc record (fields by name)."""
        d = np.zeros(38, dtype=np.float64)
        d[0], d[1] = h["body_a"], h["body_b"]
        for k, f in enumerate(("point_a", "point_b", "hinge_axis_a", "hinge_axis_b", "normal_axis_a", "normal_axis_b")):
            d[2 + 3 * k: 5 + 3 * k] = h[f]
        d[20] = h["space"]
        d[21], d[22] = h["limits_min"], h["limits_max"]
        d[23:26] = (h["limits_spring"]["mode"], h["limits_spring"]["frequency_or_stiffness"],
                    h["limits_spring"]["damping"])
        d[26], d[27], d[28], d[29] = (h["max_friction_torque"], h["motor_state"], h["target_angular_velocity"],
                                      h["target_angle"])
        d[30:33] = (h["motor_spring"]["mode"], h["motor_spring"]["frequency_or_stiffness"],
                    h["motor_spring"]["damping"])
        d[33], d[34], d[35] = h["min_torque_limit"], h["max_torque_limit"], h["priority"]
        d[36], d[37] = h["num_velocity_steps_override"], h["num_position_steps_override"]
        return self.add_hinge(d)

    def add_swing_twist_record(self, h) -> int:
        """Swing-twist joint from a cc_swing_twist_desc record (fields by name)."""
        d = np.zeros(49, dtype=np.float64)
        d[0], d[1] = h["body_a"], h["body_b"]
        for k, f in enumerate(("position_a", "position_b", "twist_axis_a", "plane_axis_a", "twist_axis_b",
                               "plane_axis_b")):
            d[2 + 3 * k: 5 + 3 * k] = h[f]
        d[20], d[21] = h["space"], h["swing_type"]
        d[22], d[23] = h["normal_half_cone_angle"], h["plane_half_cone_angle"]
        d[24], d[25], d[26] = h["twist_min_angle"], h["twist_max_angle"], h["max_friction_torque"]
        d[27], d[28] = h["swing_motor_state"], h["twist_motor_state"]
        d[29:32] = h["target_angular_velocity"]
        d[32:36] = h["target_orientation"]
        for k, f in enumerate(("swing_motor_spring", "twist_motor_spring")):
            d[36 + 3 * k: 39 + 3 * k] = (h[f]["mode"], h[f]["frequency_or_stiffness"], h[f]["damping"])
        d[42], d[43] = h["swing_min_torque_limit"], h["swing_max_torque_limit"]
        d[44], d[45] = h["twist_min_torque_limit"], h["twist_max_torque_limit"]
        d[46] = h["priority"]
        d[47], d[48] = h["num_velocity_steps_override"], h["num_position_steps_override"]
        k = self.lib.orc_add_swing_twist(self.h, dptr(d))
        assert k >= 0
        return k

    def add_joint_record(self, joint_type: int, h) -> int:
        """Point, distance, fixed, cone or slider joint from a record of the C description
        (crashcat_gb300._lib.JOINT_DTYPES; fields by name) in the orc_add_joint layout."""
        d = np.zeros(102, dtype=np.float64)
        d[0], d[1], d[2] = h["body_a"], h["body_b"], h["space"]
        d[3], d[4], d[5], d[6] = (h["priority"], h["num_velocity_steps_override"], h["num_position_steps_override"],
                                  h["enabled"])

        def put(k, fields):
            for f in fields:
                d[k:k + 3] = h[f]
                k += 3
            return k

        def spring(k, f):
            d[k:k + 3] = (h[f]["mode"], h[f]["frequency_or_stiffness"], h[f]["damping"])

        if joint_type == 0:  # point
            put(7, ("point_a", "point_b"))
        elif joint_type == 1:  # distance
            put(7, ("point_a", "point_b"))
            d[13], d[14] = h["min_distance"], h["max_distance"]
            spring(15, "spring")
        elif joint_type == 4:  # fixed
            d[7] = h["auto_detect_point"]
            put(8, ("point_a", "point_b", "axis_x_a", "axis_y_a", "axis_x_b", "axis_y_b"))
        elif joint_type == 5:  # cone
            put(7, ("point_a", "point_b", "twist_axis_a", "twist_axis_b"))
            d[19] = h["half_cone_angle"]
        elif joint_type == 3:  # slider
            d[7] = h["auto_detect_point"]
            put(8, ("point_a", "point_b", "slider_axis_a", "slider_axis_b", "normal_axis_a", "normal_axis_b"))
            d[26], d[27] = h["limits_min"], h["limits_max"]
            spring(28, "limits_spring")
            d[31] = h["max_friction_force"]
            spring(32, "motor_spring")
            d[35], d[36] = h["min_force_limit"], h["max_force_limit"]
            d[37], d[38], d[39] = h["motor_state"], h["target_velocity"], h["target_position"]
        elif joint_type == 7:  # six-DOF
            put(7, ("position_a", "position_b", "axis_x_a", "axis_y_a", "axis_x_b", "axis_y_b"))
            d[25] = h["swing_type"]
            d[26:32], d[32:38], d[38:44] = h["limit_min"], h["limit_max"], h["max_friction"]
            for k in range(3):
                sp = h["limits_spring"][k]
                d[44 + 3 * k:47 + 3 * k] = (sp["mode"], sp["frequency_or_stiffness"], sp["damping"])
            for k in range(6):
                sp = h["motor_spring"][k]
                d[53 + 3 * k:56 + 3 * k] = (sp["mode"], sp["frequency_or_stiffness"], sp["damping"])
            d[71:77], d[77:83], d[83:89] = h["motor_min_force"], h["motor_max_force"], h["motor_state"]
            d[89:92], d[92:95], d[95:98] = h["target_velocity"], h["target_angular_velocity"], h["target_position"]
            d[98:102] = h["target_orientation"]
        else:
            raise ValueError(f"joint type {joint_type}")
        k = self.lib.orc_add_joint(self.h, int(joint_type), dptr(d))
        assert k >= 0
        return k

    def joint_lambdas(self, joint_type: int, index: int) -> np.ndarray:
        out = np.zeros(18, dtype=np.float64)
        n = self.lib.orc_get_joint_lambdas(self.h, int(joint_type), int(index), dptr(out))
        assert n >= 0
        return out[:n]

    def slider_position(self, index: int) -> float:
        return float(self.lib.orc_slider_position(self.h, int(index)))

    def set_skip_joint_pairs(self, on: bool) -> None:
        self.lib.orc_set_skip_joint_pairs(self.h, 1 if on else 0)

    def contact_events(self) -> dict:
        """Contact events of the last step: {'added' | 'persisted' | 'removed': set of (a, b)}."""
        n = self.lib.orc_get_events(self.h, None, 0)
        out = np.zeros((max(n, 1), 3), dtype=np.int64)
        self.lib.orc_get_events(self.h, C.c_void_p(out.ctypes.data), n)
        names = {1: "added", 2: "persisted", 3: "removed"}
        ev = {v: set() for v in names.values()}
        for t, a, b in out[:n].tolist():
            ev[names[t]].add((a, b))
        return ev

    def island_iterations(self) -> np.ndarray:
        """(velocity, position) steps of each body's island in the last step, [n, 2] (-1: none)."""
        o = np.zeros((self.n, 2), dtype=np.int32)
        self.lib.orc_get_island_iterations(self.h, iptr(o))
        return o

    def step_taped(self, dt: float):
        """One step with the rows of its velocity solve (orc_get_solver_tape): returns
        (body rows [n, 17], contact rows [k, 86], post-solve velocities [n, 6], warm-start ratio)
        in the layout of oracle_frozen.h."""
        self.lib.orc_set_record_tape(self.h, 1)
        self.lib.orc_step(self.h, dt, 1)
        k = self.lib.orc_get_solver_tape(self.h, None, None, None, None)
        bodies = np.zeros((self.n, BODY_ROW))
        cons = np.zeros((max(k, 1), CON_ROW))
        v2 = np.zeros((self.n, 6))
        ratio = C.c_double(0.0)
        self.lib.orc_get_solver_tape(self.h, bodies.ctypes.data, cons.ctypes.data, v2.ctypes.data, C.byref(ratio))
        return bodies, cons[:k], v2, float(ratio.value)

    def manifolds(self) -> np.ndarray:
        n = self.lib.orc_manifold_count(self.h)
        o = np.zeros((max(n, 1), 32), dtype=np.float64)
        self.lib.orc_get_manifolds(self.h, dptr(o))
        return o[:n]


def state_to_gpu_rows(st: np.ndarray) -> np.ndarray:
    """oracle state rows (17 doubles) -> GPU state rows (16 floats)."""
    return np.ascontiguousarray(st[:, :16], dtype=np.float32)


def gpu_rows_to_state(rows: np.ndarray) -> np.ndarray:
    o = np.zeros((len(rows), STATE), dtype=np.float64)
    o[:, :16] = rows
    return o


def fix_normal(v0, v1, v2, triangle_normal, active_edges, point, normal, movement) -> int:
    """fixNormal (active-edges.ts:74-153) in the oracle: 1 when it keeps the normal, 0 when it
    returns the triangle normal."""
    a = np.zeros(25, dtype=np.float64)
    for k, v in enumerate((v0, v1, v2, triangle_normal, point, normal, movement)):
        a[3 * k: 3 * k + 3] = v
    a[24] = active_edges
    return load().orc_fix_normal(dptr(a))


# ---------------------------------------------------------------------------
# frozen-contact replay of a taped rollout (oracle_frozen.h)
# ---------------------------------------------------------------------------
BODY_ROW, CONST_ROW, CON_HEAD, POINT_ROW = 17, 6, 18, 17
CON_ROW = CON_HEAD + 4 * POINT_ROW
TAPE_DYNAMIC, TAPE_MOVING = 1, 2


def tape_consts(bodies: np.ndarray, dt: float) -> np.ndarray:
    """Per body (world, in the loss, friction, friction combine mode, linear and angular damping
    factors max(0, 1 - c dt)) from a BODY_DTYPE array."""
    c = np.zeros((len(bodies), CONST_ROW))
    c[:, 0] = bodies["world"]
    c[:, 1] = bodies["motion_type"] == 2
    c[:, 2] = bodies["friction"].astype(np.float64)
    c[:, 3] = bodies["friction_combine"]
    c[:, 4] = np.maximum(0.0, 1.0 - bodies["linear_damping"].astype(np.float64) * dt)
    c[:, 5] = np.maximum(0.0, 1.0 - bodies["angular_damping"].astype(np.float64) * dt)
    return c


def tape_rows_from_gpu(tb: np.ndarray, tc: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """cc_tape_body / cc_tape_contact records (crashcat_gb300._lib TAPE_*_DTYPE) -> the replay's
    body rows [n, 17] and contact rows [k, 86]."""
    b = np.zeros((len(tb), BODY_ROW))
    b[:, 0:3] = tb["linear_velocity"]
    b[:, 3:6] = tb["angular_velocity"]
    s = tb["inv_inertia"].astype(np.float64)  # xx xy xz yy yz zz -> 3x3 column-major
    b[:, 6:15] = s[:, [0, 1, 2, 1, 3, 4, 2, 4, 5]]
    b[:, 15] = tb["inv_mass"]
    b[:, 16] = tb["flags"]
    c = np.zeros((len(tc), CON_ROW))
    c[:, 0] = tc["body_a"]
    c[:, 1] = tc["body_b"]
    c[:, 2] = tc["num_points"]
    c[:, 3] = tc["island"]
    c[:, 4] = tc["has_prev"]
    c[:, 5] = tc["sort_key"]
    c[:, 6:9] = tc["normal"]
    c[:, 9:12] = tc["tangent1"]
    c[:, 12:15] = tc["tangent2"]
    c[:, 15] = tc["friction"]
    c[:, 16] = tc["inv_mass_a"]
    c[:, 17] = tc["inv_mass_b"]
    for q in range(4):
        p = tc["points"][:, q]
        o = CON_HEAD + q * POINT_ROW
        c[:, o:o + 3] = p["r_a"]
        c[:, o + 3:o + 6] = p["r_b"]
        c[:, o + 6] = p["eff_normal"]
        c[:, o + 7] = p["eff_tangent1"]
        c[:, o + 8] = p["eff_tangent2"]
        c[:, o + 9] = p["bias_normal"]
        c[:, o + 10] = p["lambda_normal"]
        c[:, o + 11] = p["lambda_tangent1"]
        c[:, o + 12] = p["lambda_tangent2"]
        c[:, o + 13] = np.where(q < tc["num_points"], p["prev_point"], -1)
        c[:, o + 14] = p["final_normal"]
        c[:, o + 15] = p["final_tangent1"]
        c[:, o + 16] = p["final_tangent2"]
    return b, c


class FrozenTape:
    """The rows of every step of a rollout, for orc_frozen_rollout: consts [n, 6], then per step
    the body rows, the velocities at the step's start [n, 6], the warm-start ratio and the
    contact rows; finish() takes the positions after the last step."""

    def __init__(self, consts: np.ndarray, targets: np.ndarray, velocity_iterations: int, dt: float):
        self.consts = np.ascontiguousarray(consts, dtype=np.float64)
        self.targets = np.ascontiguousarray(targets, dtype=np.float64).reshape(-1, 3)
        self.iters = int(velocity_iterations)
        self.dt = float(dt)
        self.bodies, self.v0, self.ratio, self.cons = [], [], [], []
        self.x_final = None

    def add_step(self, body_rows, v0, ratio, con_rows):
        self.bodies.append(np.asarray(body_rows, dtype=np.float64))
        self.v0.append(np.asarray(v0, dtype=np.float64))
        self.ratio.append(float(ratio))
        self.cons.append(np.asarray(con_rows, dtype=np.float64).reshape(-1, CON_ROW))

    def finish(self, x_final):
        self.x_final = np.ascontiguousarray(x_final, dtype=np.float64)

    def replay(self, mode: int, eps: float = 0.0, dv=None, dw=None, dmu=None, want_v2: bool = False):
        """mode 0: (loss at the tape, its derivative along (dv, dw, dmu)); mode 1: (loss of the
        replay's own trajectory moved by eps along the direction, its derivative there).
        With want_v2 also the post-solve velocities [steps, n, 6] and the final impulses
        [contacts, 4, 3] of the replay."""
        lib = load()
        n, steps = len(self.consts), len(self.bodies)
        bodies = np.ascontiguousarray(np.stack(self.bodies))
        v0 = np.ascontiguousarray(np.stack(self.v0))
        ratio = np.ascontiguousarray(self.ratio, dtype=np.float64)
        off = np.zeros(steps + 1, dtype=np.int32)
        off[1:] = np.cumsum([len(c) for c in self.cons])
        cons = np.ascontiguousarray(np.concatenate(self.cons) if off[-1] else np.zeros((1, CON_ROW)))

        def opt(a, shape):
            if a is None:
                return None, None
            a = np.ascontiguousarray(a, dtype=np.float64).reshape(shape)
            return a, a.ctypes.data

        dv_a, dv_p = opt(dv, (n, 3))
        dw_a, dw_p = opt(dw, (n, 3))
        dm_a, dm_p = opt(dmu, (n,))
        out = np.zeros(2)
        v2 = np.zeros((steps, n, 6)) if want_v2 else None
        lam = np.zeros((max(int(off[-1]), 1), 4, 3)) if want_v2 else None
        st = lib.orc_frozen_rollout(n, steps, len(self.targets), self.iters, self.dt, dptr(self.consts), dptr(bodies),
                                    dptr(v0), dptr(ratio), iptr(off), dptr(cons), dptr(self.x_final),
                                    dptr(self.targets), mode, eps, dv_p, dw_p, dm_p, dptr(out),
                                    v2.ctypes.data if want_v2 else None, lam.ctypes.data if want_v2 else None)
        assert st == 0
        if want_v2:
            return float(out[0]), float(out[1]), v2, lam[: int(off[-1])]
        return float(out[0]), float(out[1])
