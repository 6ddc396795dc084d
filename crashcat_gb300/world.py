"""Host-side mirror of crashcat's world / body / update API over the C ABI.

The reference's user-facing calls (src/index.ts) map as follows:

    createWorldSettings()            -> create_world_settings()           world-settings.ts:224
    addBroadphaseLayer / addObjectLayer / enableCollision                 world-settings.ts:267-284
    createWorld(settings)            -> create_world(settings)            world.ts:46
    rigidBody.create(world, {...})   -> create_body(world, RigidBodySettings(...))   rigid-body.ts:390
    updateWorld(world, listener, dt) -> update_world(world, None, dt)     update.ts:45

The device world is created lazily on the first ``update_world`` with every
body added so far; later bodies are appended to it.  Body state lives on the
device; ``RigidBody`` views read it back on demand.  Listener callbacks
cannot run inside kernels: ``update_world`` calls a listener's
onContactAdded / onContactPersisted / onContactRemoved after the step from the
library's event buffer, and rejects onBodyPairValidate / onContactValidate.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
from typing import Optional

import numpy as np

from . import _lib
from ._lib import BODY_DTYPE, STATE_FLOATS, check, ptr
from . import scenes as _sc


# ---------------------------------------------------------------------------
# settings and layers (src/world-settings.ts, src/layers.ts)
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class Layers:
    broadphase_layers: int = 0
    object_to_broadphase: list = dataclasses.field(default_factory=list)
    object_pairs: list = dataclasses.field(default_factory=list)        # per object layer: bitmask of object layers
    object_vs_broadphase: list = dataclasses.field(default_factory=list)  # per object layer: bitmask of bp layers
    broadphase_pairs: list = dataclasses.field(default_factory=list)     # per bp layer: bitmask of bp layers


@dataclasses.dataclass
class WorldSettings:
    gravity: tuple = (0.0, -9.81, 0.0)
    gravity_enabled: bool = True
    speculative_contact_distance: float = 0.02
    manifold_tolerance: float = 1e-3
    collision_tolerance: float = 1e-4
    penetration_tolerance: float = 1e-4
    normal_cos_max_delta_rotation: float = math.cos(5 * math.pi / 180)
    contact_point_preserve_lambda_max_dist_sq: float = 0.01 * 0.01
    velocity_iterations: int = 10
    position_iterations: int = 2
    warm_starting: bool = True
    penetration_slop: float = 0.02
    baumgarte_factor: float = 0.2
    max_penetration_distance: float = 0.2
    min_velocity_for_restitution: float = 1.0
    ccd_linear_cast_threshold: float = 0.05
    ccd_linear_cast_max_penetration: float = 0.25
    ccd_min_velocity_for_restitution: float = 1.0
    allow_sleeping: bool = True
    time_before_sleep: float = 0.5
    point_velocity_sleep_threshold: float = 0.03
    layers: Layers = dataclasses.field(default_factory=Layers)
    num_worlds: int = 1
    max_bodies: int = 0
    # bounds of the device-side waits (0: the library's defaults); see cc_world_settings
    device_wait_polls: int = 0
    island_link_attempts: int = 0

    def to_c(self, max_bodies: int) -> _lib.Settings:
        s = _lib.Settings()
        for k in range(3):
            s.gravity[k] = self.gravity[k]
        s.gravity_enabled = int(self.gravity_enabled)
        for f in ("speculative_contact_distance", "manifold_tolerance", "collision_tolerance",
                  "penetration_tolerance", "normal_cos_max_delta_rotation",
                  "contact_point_preserve_lambda_max_dist_sq", "penetration_slop", "baumgarte_factor",
                  "max_penetration_distance", "min_velocity_for_restitution", "time_before_sleep",
                  "point_velocity_sleep_threshold", "ccd_linear_cast_threshold",
                  "ccd_linear_cast_max_penetration", "ccd_min_velocity_for_restitution"):
            setattr(s, f, float(getattr(self, f)))
        s.velocity_iterations = self.velocity_iterations
        s.position_iterations = self.position_iterations
        s.warm_starting = int(self.warm_starting)
        s.allow_sleeping = int(self.allow_sleeping)
        L = self.layers
        if not L.object_to_broadphase:
            raise ValueError("world settings need at least one object layer (add_object_layer)")
        s.num_object_layers = len(L.object_to_broadphase)
        s.num_broadphase_layers = L.broadphase_layers
        for i, bp in enumerate(L.object_to_broadphase):
            s.object_to_broadphase[i] = bp
            s.object_pairs[i] = L.object_pairs[i]
            s.object_vs_broadphase[i] = L.object_vs_broadphase[i]
        for i in range(L.broadphase_layers):
            s.broadphase_pairs[i] = L.broadphase_pairs[i]
        s.max_bodies = max(1, max_bodies)
        s.num_worlds = self.num_worlds
        s.device_wait_polls = self.device_wait_polls
        s.island_link_attempts = self.island_link_attempts
        return s


def create_world_settings() -> WorldSettings:
    """createWorldSettings (world-settings.ts:224-264)."""
    return WorldSettings()


def add_broadphase_layer(settings: WorldSettings) -> int:
    """layers.addBroadphaseLayer (layers.ts:26-45)."""
    L = settings.layers
    if L.broadphase_layers >= _lib.MAX_LAYERS:
        raise ValueError("at most 32 broadphase layers")
    L.broadphase_layers += 1
    L.broadphase_pairs.append(0)
    return L.broadphase_layers - 1


def add_object_layer(settings: WorldSettings, broadphase_layer: int) -> int:
    """layers.addObjectLayer (layers.ts:47-71): the layer may query its own broadphase layer."""
    L = settings.layers
    if len(L.object_to_broadphase) >= _lib.MAX_LAYERS:
        raise ValueError("at most 32 object layers")
    L.object_to_broadphase.append(broadphase_layer)
    L.object_pairs.append(0)
    L.object_vs_broadphase.append(1 << broadphase_layer)
    return len(L.object_to_broadphase) - 1


def enable_collision(settings: WorldSettings, a: int, b: int) -> None:
    """layers.enableCollision (layers.ts:73-100)."""
    L = settings.layers
    L.object_pairs[a] |= 1 << b
    L.object_pairs[b] |= 1 << a
    bpa, bpb = L.object_to_broadphase[a], L.object_to_broadphase[b]
    L.broadphase_pairs[bpa] |= 1 << bpb
    L.broadphase_pairs[bpb] |= 1 << bpa
    L.object_vs_broadphase[a] |= 1 << bpb
    L.object_vs_broadphase[b] |= 1 << bpa


def disable_collision(settings: WorldSettings, a: int, b: int) -> None:
    """layers.disableCollision (layers.ts:102-110): only the object pair table changes."""
    L = settings.layers
    L.object_pairs[a] &= ~(1 << b)
    L.object_pairs[b] &= ~(1 << a)


def standard_settings(**overrides) -> WorldSettings:
    """The two-layer setup of the reference's tests (tst/helpers.ts:5-26)."""
    s = create_world_settings()
    bp_moving = add_broadphase_layer(s)
    bp_static = add_broadphase_layer(s)
    moving = add_object_layer(s, bp_moving)
    static = add_object_layer(s, bp_static)
    enable_collision(s, moving, moving)
    enable_collision(s, moving, static)
    for k, v in overrides.items():
        setattr(s, k, v)
    return s


# ---------------------------------------------------------------------------
# shapes and bodies
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class Box:
    half_extents: tuple
    convex_radius: float = _sc.DEFAULT_CONVEX_RADIUS
    density: float = _sc.DEFAULT_DENSITY


@dataclasses.dataclass
class Sphere:
    radius: float
    density: float = _sc.DEFAULT_DENSITY


@dataclasses.dataclass
class RigidBodySettings:
    """RigidBodySettings (rigid-body.ts:37-118) for the supported shapes."""
    shape: object
    object_layer: int
    motion_type: int = _lib.DYNAMIC
    position: tuple = (0.0, 0.0, 0.0)
    quaternion: tuple = (0.0, 0.0, 0.0, 1.0)
    linear_velocity: tuple = (0.0, 0.0, 0.0)
    angular_velocity: tuple = (0.0, 0.0, 0.0)
    friction: float = _sc.DEFAULT_FRICTION
    restitution: float = _sc.DEFAULT_RESTITUTION
    gravity_factor: float = 1.0
    linear_damping: float = _sc.DEFAULT_DAMPING
    angular_damping: float = _sc.DEFAULT_DAMPING
    max_linear_velocity: float = _sc.DEFAULT_MAX_LINEAR_VELOCITY
    max_angular_velocity: float = _sc.DEFAULT_MAX_ANGULAR_VELOCITY
    allow_sleeping: bool = True
    friction_combine: int = _lib.COMBINE_GEOMETRIC_MEAN
    restitution_combine: int = _lib.COMBINE_MAX
    collision_groups: int = 0xFFFFFFFF
    collision_mask: int = 0xFFFFFFFF
    allowed_degrees_of_freedom: int = 0b111111
    world: int = 0
    # motionProperties.numVelocityStepsOverride / numPositionStepsOverride (motion-properties.ts:59-61)
    num_velocity_steps_override: int = 0
    num_position_steps_override: int = 0


def body_desc(s: RigidBodySettings) -> np.ndarray:
    d = np.zeros(1, dtype=BODY_DTYPE)
    if isinstance(s.shape, Box):
        d["shape_type"] = _lib.SHAPE_BOX
        d["shape_params"][0, :3] = s.shape.half_extents
        d["shape_params"][0, 3] = s.shape.convex_radius
        d["density"] = s.shape.density
    elif isinstance(s.shape, Sphere):
        d["shape_type"] = _lib.SHAPE_SPHERE
        d["shape_params"][0, 0] = s.shape.radius
        d["density"] = s.shape.density
    else:
        raise TypeError(f"unsupported shape {type(s.shape).__name__}: box and sphere are supported")
    d["motion_type"] = s.motion_type
    d["object_layer"] = s.object_layer
    d["world"] = s.world
    d["allow_sleeping"] = int(s.allow_sleeping)
    d["position"] = s.position
    d["quaternion"] = s.quaternion
    d["linear_velocity"] = s.linear_velocity
    d["angular_velocity"] = s.angular_velocity
    for f in ("friction", "restitution", "gravity_factor", "linear_damping", "angular_damping",
              "max_linear_velocity", "max_angular_velocity", "friction_combine", "restitution_combine",
              "collision_groups", "collision_mask"):
        d[f] = getattr(s, f)
    d["allowed_dofs"] = s.allowed_degrees_of_freedom
    d["num_velocity_steps_override"] = s.num_velocity_steps_override
    d["num_position_steps_override"] = s.num_position_steps_override
    return d


class GpuWorld:
    """Owns one cc_world handle (one or many independent worlds)."""

    def __init__(self, settings: WorldSettings, max_bodies: int):
        lib = _lib.load()
        self._lib = lib
        self.settings = settings
        cs = settings.to_c(max_bodies)
        h = C.c_void_p()
        check(lib.cc_world_create(C.byref(cs), C.byref(h)), "cc_world_create")
        self.handle = h
        self.n = 0

    def close(self) -> None:
        if self.handle:
            self._lib.cc_world_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_bodies(self, bodies: np.ndarray) -> np.ndarray:
        bodies = np.ascontiguousarray(bodies, dtype=BODY_DTYPE)
        out = np.zeros(len(bodies), dtype=np.int32)
        check(self._lib.cc_world_add_bodies(self.handle, ptr(bodies), len(bodies), ptr(out)), "cc_world_add_bodies")
        self.n += len(bodies)
        return out

    def step(self, dt: float, n_steps: int = 1) -> int:
        st = self._lib.cc_world_step(self.handle, C.c_float(dt), n_steps)
        if st not in (_lib.CC_OK, _lib.CC_ERR_CAPACITY):
            check(st, "cc_world_step")
        return st

    def step_host(self, dt: float, state_in: np.ndarray, state_out: np.ndarray) -> int:
        st = self._lib.cc_world_step_host(self.handle, C.c_float(dt), ptr(state_in), ptr(state_out))
        if st not in (_lib.CC_OK, _lib.CC_ERR_CAPACITY):
            check(st, "cc_world_step_host")
        return st

    def get_state(self):
        rows = np.zeros((self.n, STATE_FLOATS), dtype=np.float32)
        sl = np.zeros(self.n, dtype=np.uint8)
        check(self._lib.cc_world_get_state(self.handle, ptr(rows), ptr(sl)), "cc_world_get_state")
        return rows, sl

    def set_state(self, rows: np.ndarray) -> None:
        rows = np.ascontiguousarray(rows, dtype=np.float32)
        assert rows.shape == (self.n, STATE_FLOATS)
        check(self._lib.cc_world_set_state(self.handle, ptr(rows)), "cc_world_set_state")

    def get_pairs(self) -> np.ndarray:
        cnt = C.c_int32()
        check(self._lib.cc_world_get_pairs(self.handle, None, 0, C.byref(cnt)), "cc_world_get_pairs")
        out = np.zeros((max(cnt.value, 1), 2), dtype=np.int32)
        check(self._lib.cc_world_get_pairs(self.handle, ptr(out), cnt.value, C.byref(cnt)), "cc_world_get_pairs")
        return out[: cnt.value]

    def get_manifolds(self) -> np.ndarray:
        cnt = C.c_int32()
        check(self._lib.cc_world_get_manifolds(self.handle, None, 0, C.byref(cnt)), "cc_world_get_manifolds")
        out = np.zeros((max(cnt.value, 1), 32), dtype=np.float32)
        check(self._lib.cc_world_get_manifolds(self.handle, ptr(out), cnt.value, C.byref(cnt)),
              "cc_world_get_manifolds")
        return out[: cnt.value]

    def island_iterations(self) -> np.ndarray:
        """(velocity, position) iteration counts of the island each body was solved in during the
        last step, [n, 2]; -1 for bodies in no island (cc_world_get_island_iterations)."""
        out = np.zeros((max(self.n, 1), 2), dtype=np.int32)
        check(self._lib.cc_world_get_island_iterations(self.handle, ptr(out)), "cc_world_get_island_iterations")
        return out[: self.n]

    def debug_islands(self):
        cnt = C.c_int32()
        check(self._lib.cc_world_debug_islands(self.handle, None, None, 0, C.byref(cnt)), "cc_world_debug_islands")
        iob = np.zeros(max(self.n, 1), dtype=np.int32)
        rows = np.zeros((max(cnt.value, 1), 3), dtype=np.int32)
        check(self._lib.cc_world_debug_islands(self.handle, ptr(iob), ptr(rows), cnt.value, C.byref(cnt)),
              "cc_world_debug_islands")
        return iob[: self.n], rows[: cnt.value]

    STAGES = ("integrate_forces", "broadphase", "narrowphase", "epa", "contacts_islands", "solve_small_islands",
              "solve_large_islands")

    def profile_steps(self, dt: float, n_steps: int) -> dict:
        """Mean milliseconds per stage over n_steps eager steps bracketed by CUDA events."""
        out = np.zeros(8, dtype=np.float32)
        st = self._lib.cc_world_profile_steps(self.handle, C.c_float(dt), n_steps, ptr(out), 8)
        if st not in (_lib.CC_OK, _lib.CC_ERR_CAPACITY):
            check(st, "cc_world_profile_steps")
        return {k: float(out[i]) for i, k in enumerate(self.STAGES)}

    def rollout_grad(self, dt: float, n_steps: int, targets: np.ndarray, checkpoint_every: int = 10):
        """Loss and gradients of an n_steps rollout from the current state (cc_world_rollout_grad):
        returns (loss per world, dL/d linear velocity [n, 3], dL/d angular velocity [n, 3],
        dL/d friction [n]).  The world ends in the state after the rollout."""
        n = self.n
        targets = np.ascontiguousarray(targets, dtype=np.float32).reshape(-1, 3)
        loss = np.zeros(len(targets), dtype=np.float32)
        gv = np.zeros((n, 3), dtype=np.float32)
        gw = np.zeros((n, 3), dtype=np.float32)
        gm = np.zeros(n, dtype=np.float32)
        _lib.check(self._lib.cc_world_rollout_grad(self.handle, C.c_float(dt), n_steps, checkpoint_every,
                                                  _lib.ptr(targets), _lib.ptr(loss), _lib.ptr(gv), _lib.ptr(gw),
                                                  _lib.ptr(gm)), "cc_world_rollout_grad")
        return loss, gv, gw, gm

    def autotune(self, dt: float, steps_per_trial: int = 3) -> dict:
        """cc_world_autotune: times candidate launch shapes on the current state (which it leaves
        as it found it) and keeps the fastest; returns the report as a dict."""
        rep = _lib.TuneReport()
        check(self._lib.cc_world_autotune(self.handle, C.c_float(dt), steps_per_trial, C.byref(rep)),
              "cc_world_autotune")
        return {f: getattr(rep, f) for f, _ in _lib.TuneReport._fields_}

    def step_taped(self, dt: float, capacity: int | None = None):
        """One step with the rows of its velocity solve (cc_world_step_taped): returns
        (bodies [n] TAPE_BODY_DTYPE, contacts TAPE_CONTACT_DTYPE, warm-start ratio, status)."""
        bodies = np.zeros(self.n, dtype=_lib.TAPE_BODY_DTYPE)
        cap = capacity if capacity is not None else max(self.n * 8, 1024)
        cons = np.zeros(cap, dtype=_lib.TAPE_CONTACT_DTYPE)
        cnt = C.c_int32(0)
        ratio = C.c_float(0.0)
        st = self._lib.cc_world_step_taped(self.handle, C.c_float(dt), _lib.ptr(bodies), _lib.ptr(cons), cap,
                                           C.byref(cnt), C.byref(ratio))
        if st not in (_lib.CC_OK, _lib.CC_ERR_CAPACITY):
            check(st, "cc_world_step_taped")
        if cnt.value > cap:
            raise RuntimeError(f"cc_world_step_taped: {cnt.value} constraints exceed the capacity {cap}")
        return bodies, cons[: cnt.value], float(ratio.value), st

    def contact_events(self) -> np.ndarray:
        """Contact events of the last step as rows (type 1 added / 2 persisted / 3 removed,
        body A, body B), A < B, sorted (cc_world_get_contact_events)."""
        cnt = C.c_int32(0)
        self._lib.cc_world_get_contact_events(self.handle, None, 0, C.byref(cnt))
        out = np.zeros((max(cnt.value, 1), 3), dtype=np.int32)
        st = self._lib.cc_world_get_contact_events(self.handle, ptr(out), cnt.value, C.byref(cnt))
        if st not in (_lib.CC_OK, _lib.CC_ERR_CAPACITY):
            check(st, "cc_world_get_contact_events")
        return out[: cnt.value]

    # ---- convex hull shapes (convex-hull.ts) ----
    def add_convex_hull(self, points, convex_radius: float = -1.0) -> int:
        """cc_world_add_convex_hull: the hull index bodies name in shape_params[0]
        (convex_radius < 0: the default 0.05)."""
        p = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
        out = C.c_int32(-1)
        check(self._lib.cc_world_add_convex_hull(self.handle, ptr(p), len(p), C.c_float(convex_radius),
                                                 C.byref(out)), "cc_world_add_convex_hull")
        return out.value

    def get_convex_hull(self, index: int) -> dict:
        """cc_world_get_convex_hull: the built hull's arrays (the oracle takes them as its shape data)."""
        return _lib._hull_arrays(
            lambda info, *a: self._lib.cc_world_get_convex_hull(self.handle, index, info, *a))

    # ---- triangle meshes (triangle-mesh.ts) ----
    def add_triangle_mesh(self, positions, indices, degenerate_tolerance: float = -1.0,
                          active_edge_cos: float = -2.0) -> int:
        """cc_world_add_triangle_mesh: the mesh index bodies name in shape_params[0]
        (mesh bodies are static or kinematic)."""
        p = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        ix = np.ascontiguousarray(indices, dtype=np.int32).reshape(-1, 3)
        out = C.c_int32(-1)
        check(self._lib.cc_world_add_triangle_mesh(self.handle, ptr(p), len(p), ptr(ix), len(ix),
                                                   C.c_double(degenerate_tolerance), C.c_double(active_edge_cos),
                                                   C.byref(out)), "cc_world_add_triangle_mesh")
        return out.value

    def add_compound(self, children: np.ndarray) -> int:
        """cc_world_add_compound: a compound shape from _lib.COMPOUND_CHILD_DTYPE records; the index
        compound bodies name in shape_params[0]."""
        children = np.ascontiguousarray(children, dtype=_lib.COMPOUND_CHILD_DTYPE)
        out = C.c_int32(-1)
        check(self._lib.cc_world_add_compound(self.handle, children.ctypes.data, len(children), C.byref(out)),
              "cc_world_add_compound")
        return out.value

    def get_triangle_mesh(self, index: int) -> dict:
        """cc_world_get_triangle_mesh: the built mesh's arrays (the oracle takes them as its shape data)."""
        return _lib._mesh_arrays(
            lambda info, *a: self._lib.cc_world_get_triangle_mesh(self.handle, index, info, *a))

    def get_manifold_sub_shapes(self) -> np.ndarray:
        """cc_world_get_manifold_sub_shapes: (sub-shape id A, sub-shape id B) per manifold, in
        get_manifolds order."""
        n = C.c_int32(0)
        check(self._lib.cc_world_get_manifold_sub_shapes(self.handle, None, 0, C.byref(n)),
              "cc_world_get_manifold_sub_shapes")
        out = np.zeros((max(n.value, 1), 2), dtype=np.uint32)
        check(self._lib.cc_world_get_manifold_sub_shapes(self.handle, ptr(out), n.value, C.byref(n)),
              "cc_world_get_manifold_sub_shapes")
        return out[:n.value]

    # ---- world queries (query.ts) ----
    def cast_rays(self, rays: np.ndarray, object_layer_mask: int = 0xFFFFFFFF, collision_group: int = 0xFFFFFFFF,
                  collision_mask: int = 0xFFFFFFFF, treat_convex_as_solid: bool = True,
                  collide_with_backfaces: bool = False) -> np.ndarray:
        """cc_world_cast_rays: the closest hit of each ray (a _lib.RAY_DTYPE array, or rows of
        origin xyz, unit direction xyz, length[, world]) as a _lib.RAY_HIT_DTYPE array."""
        rays = np.asarray(rays)
        if rays.dtype != _lib.RAY_DTYPE:
            rows = np.asarray(rays, np.float64).reshape(len(rays), -1)
            r = np.zeros(len(rows), _lib.RAY_DTYPE)
            r["origin"], r["direction"], r["length"] = rows[:, 0:3], rows[:, 3:6], rows[:, 6]
            r["world"] = rows[:, 7].astype(np.int32) if rows.shape[1] > 7 else 0
            rays = r
        rays = np.ascontiguousarray(rays)
        hits = np.zeros(len(rays), _lib.RAY_HIT_DTYPE)
        flags = (_lib.CAST_RAY_TREAT_CONVEX_AS_SOLID if treat_convex_as_solid else 0) | (
            _lib.CAST_RAY_COLLIDE_WITH_BACKFACES if collide_with_backfaces else 0)
        f = _lib.QueryFilter(object_layer_mask, collision_group, collision_mask, flags)
        check(self._lib.cc_world_cast_rays(self.handle, rays.ctypes.data, len(rays), C.byref(f), hits.ctypes.data),
              "cc_world_cast_rays")
        return hits

    def cast_shapes(self, casts: np.ndarray, object_layer_mask: int = 0xFFFFFFFF, collision_group: int = 0xFFFFFFFF,
                    collision_mask: int = 0xFFFFFFFF) -> np.ndarray:
        """cc_world_cast_shapes: the closest hit of each shape cast (a _lib.SHAPE_CAST_DTYPE array)
        as a _lib.SHAPE_CAST_HIT_DTYPE array."""
        casts = np.ascontiguousarray(casts, dtype=_lib.SHAPE_CAST_DTYPE)
        hits = np.zeros(len(casts), _lib.SHAPE_CAST_HIT_DTYPE)
        f = _lib.QueryFilter(object_layer_mask, collision_group, collision_mask, 0)
        check(self._lib.cc_world_cast_shapes(self.handle, casts.ctypes.data, len(casts), C.byref(f), hits.ctypes.data),
              "cc_world_cast_shapes")
        return hits

    def cast_rays_collect(self, rays: np.ndarray, collector: int, max_hits: int = 1,
                          object_layer_mask: int = 0xFFFFFFFF, collision_group: int = 0xFFFFFFFF,
                          collision_mask: int = 0xFFFFFFFF, treat_convex_as_solid: bool = True,
                          collide_with_backfaces: bool = False):
        """cc_world_cast_rays_collect: (hits as a (n, max_hits) _lib.RAY_HIT_DTYPE array, counts)."""
        rays = np.ascontiguousarray(rays, dtype=_lib.RAY_DTYPE)
        hits = np.zeros((len(rays), max_hits), _lib.RAY_HIT_DTYPE)
        counts = np.zeros(len(rays), np.int32)
        flags = (_lib.CAST_RAY_TREAT_CONVEX_AS_SOLID if treat_convex_as_solid else 0) | (
            _lib.CAST_RAY_COLLIDE_WITH_BACKFACES if collide_with_backfaces else 0)
        f = _lib.QueryFilter(object_layer_mask, collision_group, collision_mask, flags)
        check(self._lib.cc_world_cast_rays_collect(self.handle, rays.ctypes.data, len(rays), C.byref(f), collector,
                                                   max_hits, hits.ctypes.data, counts.ctypes.data),
              "cc_world_cast_rays_collect")
        return hits, counts

    def cast_shapes_collect(self, casts: np.ndarray, collector: int, max_hits: int = 1,
                            object_layer_mask: int = 0xFFFFFFFF, collision_group: int = 0xFFFFFFFF,
                            collision_mask: int = 0xFFFFFFFF):
        """cc_world_cast_shapes_collect: (hits as a (n, max_hits) _lib.SHAPE_CAST_HIT_DTYPE array,
        counts)."""
        casts = np.ascontiguousarray(casts, dtype=_lib.SHAPE_CAST_DTYPE)
        hits = np.zeros((len(casts), max_hits), _lib.SHAPE_CAST_HIT_DTYPE)
        counts = np.zeros(len(casts), np.int32)
        f = _lib.QueryFilter(object_layer_mask, collision_group, collision_mask, 0)
        check(self._lib.cc_world_cast_shapes_collect(self.handle, casts.ctypes.data, len(casts), C.byref(f),
                                                     collector, max_hits, hits.ctypes.data, counts.ctypes.data),
              "cc_world_cast_shapes_collect")
        return hits, counts

    def collide_shapes(self, shapes: np.ndarray, collector: int = _lib.COLLECT_CLOSEST, max_hits: int = 1,
                       max_separation_distance: float = 0.0, collision_tolerance: float = 1e-4,
                       penetration_tolerance: float = 1e-4, collide_with_backfaces: bool = True,
                       object_layer_mask: int = 0xFFFFFFFF, collision_group: int = 0xFFFFFFFF,
                       collision_mask: int = 0xFFFFFFFF):
        """cc_world_collide_shapes (collideShape with createDefaultCollideShapeSettings' defaults):
        (hits as a (n, max_hits) _lib.COLLIDE_SHAPE_HIT_DTYPE array, counts)."""
        shapes = np.ascontiguousarray(shapes, dtype=_lib.COLLIDE_SHAPE_DTYPE)
        hits = np.zeros((len(shapes), max_hits), _lib.COLLIDE_SHAPE_HIT_DTYPE)
        counts = np.zeros(len(shapes), np.int32)
        f = _lib.QueryFilter(object_layer_mask, collision_group, collision_mask, 0)
        cs = _lib.CollideShapeSettings(max_separation_distance, collision_tolerance, penetration_tolerance,
                                       int(collide_with_backfaces))
        check(self._lib.cc_world_collide_shapes(self.handle, shapes.ctypes.data, len(shapes), C.byref(f),
                                                C.byref(cs), collector, max_hits, hits.ctypes.data,
                                                counts.ctypes.data), "cc_world_collide_shapes")
        return hits, counts

    def collide_points(self, points: np.ndarray, object_layer_mask: int = 0xFFFFFFFF,
                       collision_group: int = 0xFFFFFFFF, collision_mask: int = 0xFFFFFFFF,
                       collision_tolerance: float = 1e-4) -> np.ndarray:
        """cc_world_collide_points: per point (a _lib.POINT_DTYPE array, or rows of xyz[, world])
        the number of bodies holding it, the lowest of them and its sub-shape id, as a
        _lib.POINT_HIT_DTYPE array."""
        points = np.asarray(points)
        if points.dtype != _lib.POINT_DTYPE:
            rows = np.asarray(points, np.float64).reshape(len(points), -1)
            p = np.zeros(len(rows), _lib.POINT_DTYPE)
            p["position"] = rows[:, 0:3]
            p["world"] = rows[:, 3].astype(np.int32) if rows.shape[1] > 3 else 0
            points = p
        points = np.ascontiguousarray(points)
        hits = np.zeros(len(points), _lib.POINT_HIT_DTYPE)
        f = _lib.QueryFilter(object_layer_mask, collision_group, collision_mask, 0)
        check(self._lib.cc_world_collide_points(self.handle, points.ctypes.data, len(points), C.byref(f),
                                                collision_tolerance, hits.ctypes.data), "cc_world_collide_points")
        return hits

    # ---- hinge joints (hinge-constraint.ts) ----
    def add_hinges(self, hinges: np.ndarray) -> np.ndarray:
        """cc_world_add_hinges: records of _lib.HINGE_DTYPE; returns the joint indices."""
        hinges = np.ascontiguousarray(hinges, dtype=_lib.HINGE_DTYPE)
        out = np.zeros(len(hinges), dtype=np.int32)
        check(self._lib.cc_world_add_hinges(self.handle, ptr(hinges), len(hinges), ptr(out)), "cc_world_add_hinges")
        return out

    def set_hinge_limits(self, index: int, lo: float, hi: float) -> None:
        check(self._lib.cc_world_set_hinge_limits(self.handle, index, C.c_float(lo), C.c_float(hi)),
              "cc_world_set_hinge_limits")

    def set_hinge_motor(self, index: int, state: int, target_angular_velocity: float = 0.0,
                        target_angle: float = 0.0) -> None:
        check(self._lib.cc_world_set_hinge_motor(self.handle, index, state, C.c_float(target_angular_velocity),
                                                 C.c_float(target_angle)), "cc_world_set_hinge_motor")

    def set_hinge_enabled(self, index: int, enabled: bool) -> None:
        check(self._lib.cc_world_set_hinge_enabled(self.handle, index, int(bool(enabled))),
              "cc_world_set_hinge_enabled")

    def hinge_angles(self, n: int) -> np.ndarray:
        out = np.zeros(max(n, 1), dtype=np.float32)
        check(self._lib.cc_world_get_hinge_angles(self.handle, ptr(out), n), "cc_world_get_hinge_angles")
        return out[:n]

    def add_swing_twists(self, joints: np.ndarray) -> np.ndarray:
        """cc_world_add_swing_twists: records of _lib.SWING_TWIST_DTYPE; returns the joint indices."""
        joints = np.ascontiguousarray(joints, dtype=_lib.SWING_TWIST_DTYPE)
        out = np.zeros(len(joints), dtype=np.int32)
        check(self._lib.cc_world_add_swing_twists(self.handle, ptr(joints), len(joints), ptr(out)),
              "cc_world_add_swing_twists")
        return out

    def set_swing_twist_limits(self, index: int, normal_half_cone: float, plane_half_cone: float,
                               twist_min: float, twist_max: float) -> None:
        check(self._lib.cc_world_set_swing_twist_limits(self.handle, index, C.c_float(normal_half_cone),
                                                        C.c_float(plane_half_cone), C.c_float(twist_min),
                                                        C.c_float(twist_max)), "cc_world_set_swing_twist_limits")

    def set_swing_twist_motor(self, index: int, swing_state: int, twist_state: int, target_angular_velocity=(0, 0, 0),
                              target_orientation=(0, 0, 0, 1), max_friction_torque: float = 0.0) -> None:
        tw = np.asarray(target_angular_velocity, dtype=np.float32)
        tq = np.asarray(target_orientation, dtype=np.float32)
        check(self._lib.cc_world_set_swing_twist_motor(self.handle, index, swing_state, twist_state, ptr(tw), ptr(tq),
                                                       C.c_float(max_friction_torque)),
              "cc_world_set_swing_twist_motor")

    def set_swing_twist_enabled(self, index: int, enabled: bool) -> None:
        check(self._lib.cc_world_set_swing_twist_enabled(self.handle, index, int(bool(enabled))),
              "cc_world_set_swing_twist_enabled")

    def set_skip_joint_pairs(self, on: bool) -> None:
        check(self._lib.cc_world_set_skip_joint_pairs(self.handle, int(bool(on))), "cc_world_set_skip_joint_pairs")

    def add_joints(self, joint_type: int, joints: np.ndarray) -> np.ndarray:
        """cc_world_add_{point,distance,fixed,cone,slider,six_dof}_joints: records of
        _lib.JOINT_DTYPES[joint_type]; returns the joints' per-type indices."""
        fn = _lib.JOINT_ADDERS[joint_type]
        joints = np.ascontiguousarray(joints, dtype=_lib.JOINT_DTYPES[joint_type])
        out = np.zeros(len(joints), dtype=np.int32)
        check(getattr(self._lib, fn)(self.handle, ptr(joints), len(joints), ptr(out)), fn)
        return out

    def set_joint_enabled(self, joint_type: int, index: int, enabled: bool) -> None:
        check(self._lib.cc_world_set_joint_enabled(self.handle, joint_type, index, int(bool(enabled))),
              "cc_world_set_joint_enabled")

    def joint_lambdas(self, joint_type: int, index: int) -> np.ndarray:
        """cc_world_get_joint_lambdas: the accumulated impulses of one joint after the last step."""
        out = np.zeros(18, dtype=np.float32)
        n = C.c_int32(0)
        check(self._lib.cc_world_get_joint_lambdas(self.handle, joint_type, index, ptr(out), 18, C.byref(n)),
              "cc_world_get_joint_lambdas")
        return out[:n.value]

    def set_distance(self, index: int, min_distance: float, max_distance: float) -> None:
        check(self._lib.cc_world_set_distance(self.handle, index, C.c_float(min_distance), C.c_float(max_distance)),
              "cc_world_set_distance")

    def set_cone_half_angle(self, index: int, half_cone_angle: float) -> None:
        check(self._lib.cc_world_set_cone_half_angle(self.handle, index, C.c_float(half_cone_angle)),
              "cc_world_set_cone_half_angle")

    def set_slider_limits(self, index: int, lo: float, hi: float) -> None:
        check(self._lib.cc_world_set_slider_limits(self.handle, index, C.c_float(lo), C.c_float(hi)),
              "cc_world_set_slider_limits")

    def set_slider_motor(self, index: int, state: int, target_velocity: float = 0.0,
                         target_position: float = 0.0) -> None:
        check(self._lib.cc_world_set_slider_motor(self.handle, index, state, C.c_float(target_velocity),
                                                  C.c_float(target_position)), "cc_world_set_slider_motor")

    def set_six_dof_limits(self, index: int, limit_min, limit_max) -> None:
        """setTranslationLimits + setRotationLimits of six-DOF joint ``index`` (6 + 6 values)."""
        mn = np.ascontiguousarray(limit_min, dtype=np.float32).reshape(6)
        mx = np.ascontiguousarray(limit_max, dtype=np.float32).reshape(6)
        check(self._lib.cc_world_set_six_dof_limits(self.handle, index, ptr(mn), ptr(mx)),
              "cc_world_set_six_dof_limits")

    def set_six_dof_motor(self, index: int, motor_state, target_velocity=(0.0, 0.0, 0.0),
                          target_angular_velocity=(0.0, 0.0, 0.0), target_position=(0.0, 0.0, 0.0),
                          target_orientation=(0.0, 0.0, 0.0, 1.0), max_friction=(0.0,) * 6) -> None:
        """setMaxFriction + setMotorState per axis and the constraint-space targets of six-DOF
        joint ``index``."""
        ms = np.ascontiguousarray(motor_state, dtype=np.int32).reshape(6)
        arrs = [np.ascontiguousarray(v, dtype=np.float32).reshape(k) for v, k in
                ((target_velocity, 3), (target_angular_velocity, 3), (target_position, 3),
                 (target_orientation, 4), (max_friction, 6))]
        check(self._lib.cc_world_set_six_dof_motor(self.handle, index, ptr(ms), *[ptr(x) for x in arrs]),
              "cc_world_set_six_dof_motor")

    def slider_positions(self, n: int) -> np.ndarray:
        out = np.zeros(max(n, 1), dtype=np.float32)
        check(self._lib.cc_world_get_slider_positions(self.handle, ptr(out), n), "cc_world_get_slider_positions")
        return out[:n]

    def stats(self) -> dict:
        s = _lib.Stats()
        check(self._lib.cc_world_get_stats(self.handle, C.byref(s)), "cc_world_get_stats")
        return {f: getattr(s, f) for f, _ in _lib.Stats._fields_}


# ---------------------------------------------------------------------------
# reference-shaped facade
# ---------------------------------------------------------------------------
class RigidBody:
    """View of one body; pose and velocities are read from the device world."""

    def __init__(self, world: "World", index: int):
        self._world = world
        self.index = index
        self.id = index  # bodies are never recycled: id order equals index order

    def _row(self):
        return self._world._state()[0][self.index]

    @property
    def position(self):
        return self._row()[0:3].copy()

    @property
    def quaternion(self):
        return self._row()[3:7].copy()

    @property
    def linear_velocity(self):
        return self._row()[7:10].copy()

    @property
    def angular_velocity(self):
        return self._row()[10:13].copy()

    @property
    def sleeping(self) -> bool:
        return bool(self._world._state()[1][self.index])


class World:
    """createWorld (world.ts:46-58)."""

    def __init__(self, settings: WorldSettings, max_bodies: int = 0):
        self.settings = settings
        self._pending: list = []
        self._gpu: Optional[GpuWorld] = None
        self._max_bodies = max_bodies
        self._cache = None
        self.bodies: list = []

    def _flush(self) -> None:
        if self._gpu is None:
            cap = self._max_bodies or max(1024, 2 * len(self._pending))
            self._gpu = GpuWorld(self.settings, cap)
        if self._pending:
            self._gpu.add_bodies(np.concatenate(self._pending))
            self._pending = []
        self._cache = None

    def _state(self):
        self._flush()
        if self._cache is None:
            self._cache = self._gpu.get_state()
        return self._cache


def create_world(settings: WorldSettings, max_bodies: int = 0) -> World:
    return World(settings, max_bodies)


def create_body(world: World, settings: RigidBodySettings) -> RigidBody:
    """rigidBody.create (rigid-body.ts:390-434)."""
    world._pending.append(body_desc(settings))
    b = RigidBody(world, len(world.bodies))
    world.bodies.append(b)
    world._cache = None
    return b


_EVENT_CALLBACKS = {1: "onContactAdded", 2: "onContactPersisted", 3: "onContactRemoved"}
_UNSUPPORTED_CALLBACKS = ("onBodyPairValidate", "onContactValidate")


def update_world(world: World, listener, time_step: float) -> None:
    """updateWorld (update.ts:45): one step of every body in the world on the GPU.

    A listener (listener.ts:23-99) may observe contacts: after the step its
    onContactAdded / onContactPersisted / onContactRemoved are called with the two
    RigidBody handles (ordered by id) for every event of the step, read from the
    library's event buffer.  Callbacks that decide the step itself (onBodyPairValidate,
    onContactValidate, edits of ContactSettings) cannot run inside kernels and are
    rejected."""
    if listener is not None:
        for name in _UNSUPPORTED_CALLBACKS:
            if getattr(listener, name, None) is not None:
                raise NotImplementedError(f"{name} cannot run inside the GPU step")
    world._flush()
    st = world._gpu.step(time_step, 1)
    world._cache = None
    if st != _lib.CC_OK:
        check(st, "updateWorld")
    if listener is not None and any(getattr(listener, n, None) for n in _EVENT_CALLBACKS.values()):
        for kind, a, b in world._gpu.contact_events():
            fn = getattr(listener, _EVENT_CALLBACKS[kind], None)
            if fn is not None:
                fn(world.bodies[a], world.bodies[b])
