"""Seeded synthetic scenes for the benchmark workloads and the parity tests.

A scene is a ``BODY_DTYPE`` array (the C ``cc_body_desc`` layout) plus the
world settings it runs with.  No public dataset is involved: every workload is
generated from a numpy PCG64 generator with a recorded seed, following the
shapes, sizes and value ranges of the workload descriptions.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from typing import Optional

from ._lib import (BODY_DTYPE, COMBINE_GEOMETRIC_MEAN, COMBINE_MAX, COMPOUND_CHILD_DTYPE, DYNAMIC, MOTOR_OFF,
                   MOTOR_POSITION, MOTOR_VELOCITY, SHAPE_BOX, SHAPE_CAPSULE, SHAPE_COMPOUND, SHAPE_CONVEX_HULL,
                   SHAPE_CYLINDER, SHAPE_EMPTY,
                   SHAPE_PLANE, SHAPE_SPHERE, SHAPE_TRIANGLE_MESH, STATIC,
                   SWING_CONE, SWING_PYRAMID, JOINT_CONE, JOINT_DISTANCE, JOINT_FIXED, JOINT_POINT, JOINT_SIX_DOF,
                   JOINT_SLIDER, SPRING_DTYPE, SPRING_FREQUENCY_AND_DAMPING, SPRING_STIFFNESS_AND_DAMPING,
                   hinge_defaults, joint_defaults, swing_twist_defaults)

# object layers of the reference's test helper (tst/helpers.ts:5-26)
LAYER_MOVING = 0
LAYER_NOT_MOVING = 1

# DEFAULT_RIGID_BODY_SETTINGS (src/body/rigid-body.ts:120-139)
DEFAULT_FRICTION = 0.2
DEFAULT_RESTITUTION = 0.0
DEFAULT_DAMPING = 0.05
DEFAULT_MAX_LINEAR_VELOCITY = 500.0
DEFAULT_MAX_ANGULAR_VELOCITY = 0.25 * math.pi * 60.0
DEFAULT_CONVEX_RADIUS = 0.05  # src/collision/support.ts:5
DEFAULT_DENSITY = 1000.0  # src/shapes/shapes.ts:121


@dataclasses.dataclass
class Scene:
    name: str
    bodies: np.ndarray
    dt: float
    steps: int
    velocity_iterations: int = 10
    position_iterations: int = 2
    num_worlds: int = 1
    seed: int = 0
    hinges: Optional[np.ndarray] = None  # cc_hinge_desc records (_lib.HINGE_DTYPE)
    swings: Optional[np.ndarray] = None  # cc_swing_twist_desc records (_lib.SWING_TWIST_DTYPE)
    joints: Optional[dict] = None  # {joint type: records of _lib.JOINT_DTYPES[type]} of the other joint types
    hull_points: Optional[list] = None  # point sets of the convex hulls, in hull index order
    skip_joint_pairs: bool = False
    gravity: tuple = (0.0, -9.81, 0.0)
    mesh: Optional[tuple] = None  # (positions, indices) of the triangle mesh body shapes name as index 0

    @property
    def n(self) -> int:
        return len(self.bodies)


def blank_bodies(n: int) -> np.ndarray:
    b = np.zeros(n, dtype=BODY_DTYPE)
    b["density"] = DEFAULT_DENSITY
    b["motion_type"] = DYNAMIC
    b["object_layer"] = LAYER_MOVING
    b["allow_sleeping"] = 1
    b["quaternion"] = (0.0, 0.0, 0.0, 1.0)
    b["friction"] = DEFAULT_FRICTION
    b["restitution"] = DEFAULT_RESTITUTION
    b["gravity_factor"] = 1.0
    b["linear_damping"] = DEFAULT_DAMPING
    b["angular_damping"] = DEFAULT_DAMPING
    b["max_linear_velocity"] = DEFAULT_MAX_LINEAR_VELOCITY
    b["max_angular_velocity"] = DEFAULT_MAX_ANGULAR_VELOCITY
    b["friction_combine"] = COMBINE_GEOMETRIC_MEAN
    b["restitution_combine"] = COMBINE_MAX
    b["collision_groups"] = 0xFFFFFFFF
    b["collision_mask"] = 0xFFFFFFFF
    b["allowed_dofs"] = 0b111111
    return b


def set_box(b: np.ndarray, idx, half_extents, convex_radius: float = DEFAULT_CONVEX_RADIUS) -> None:
    b["shape_type"][idx] = SHAPE_BOX
    he = np.asarray(half_extents, dtype=np.float32)
    b["shape_params"][idx, 0:3] = he
    b["shape_params"][idx, 3] = convex_radius


def set_sphere(b: np.ndarray, idx, radius) -> None:
    b["shape_type"][idx] = SHAPE_SPHERE
    b["shape_params"][idx, 0] = radius
    b["shape_params"][idx, 1:] = 0.0


def set_capsule(b: np.ndarray, idx, radius, half_height) -> None:
    """Capsule along local Y (src/shapes/capsule.ts): radius, half height of the cylinder."""
    b["shape_type"][idx] = SHAPE_CAPSULE
    b["shape_params"][idx, 0] = radius
    b["shape_params"][idx, 1] = half_height
    b["shape_params"][idx, 2:] = 0.0


def set_cylinder(b: np.ndarray, idx, half_height, radius, convex_radius: float = DEFAULT_CONVEX_RADIUS) -> None:
    """Cylinder along local Y (src/shapes/cylinder.ts): half height, radius, convex radius."""
    b["shape_type"][idx] = SHAPE_CYLINDER
    b["shape_params"][idx, 0] = half_height
    b["shape_params"][idx, 1] = radius
    b["shape_params"][idx, 2] = convex_radius
    b["shape_params"][idx, 3] = 0.0


def set_plane(b: np.ndarray, idx, normal, constant: float = 0.0) -> None:
    """Plane (src/shapes/plane.ts): n . x + c = 0 in the body frame, solid below; static or
    kinematic bodies only."""
    b["shape_type"][idx] = SHAPE_PLANE
    b["shape_params"][idx, 0:3] = normal
    b["shape_params"][idx, 3] = constant


def set_empty(b: np.ndarray, idx) -> None:
    """Empty shape (src/shapes/empty-shape.ts): no collision and no mass."""
    b["shape_type"][idx] = SHAPE_EMPTY
    b["shape_params"][idx] = 0.0


def set_compound(b: np.ndarray, idx, compound_index: int) -> None:
    """A compound body (src/shapes/compound.ts): the index from GpuWorld.add_compound in
    shape_params[0]; mass and inertia come from the children's densities."""
    b["shape_type"][idx] = SHAPE_COMPOUND
    b["shape_params"][idx] = 0.0
    b["shape_params"][idx, 0] = float(compound_index)


def compound_children(specs) -> np.ndarray:
    """Child records from (kind, params, position[, quaternion[, density]]) tuples, kind one of
    sphere, box, capsule, cylinder, hull (params: the hull index)."""
    kinds = {"sphere": SHAPE_SPHERE, "box": SHAPE_BOX, "capsule": SHAPE_CAPSULE, "cylinder": SHAPE_CYLINDER,
             "hull": SHAPE_CONVEX_HULL}
    c = np.zeros(len(specs), COMPOUND_CHILD_DTYPE)
    for i, sp in enumerate(specs):
        kind, params, pos = sp[0], sp[1], sp[2]
        q = sp[3] if len(sp) > 3 else (0.0, 0.0, 0.0, 1.0)
        c["shape_type"][i] = kinds[kind]
        p = list(params)
        if kind == "box" and len(p) == 3:
            p.append(DEFAULT_CONVEX_RADIUS)
        if kind == "cylinder" and len(p) == 2:
            p.append(DEFAULT_CONVEX_RADIUS)
        c["shape_params"][i, :len(p)] = p
        c["position"][i] = pos
        c["quaternion"][i] = q
        c["density"][i] = sp[4] if len(sp) > 4 else 1000.0
    return c


def set_hull(b: np.ndarray, idx, hull_index: int) -> None:
    """A convex hull body: the hull index from GpuWorld.add_convex_hull in shape_params[0]."""
    b["shape_type"][idx] = SHAPE_CONVEX_HULL
    b["shape_params"][idx, 0] = float(hull_index)
    b["shape_params"][idx, 1:] = 0.0


def ellipsoid_hull_points(rng: np.random.Generator, k: int, axes) -> np.ndarray:
    """k points drawn uniformly on the surface of an ellipsoid with the given semi-axes (the
    mixed convex pile's hulls: 16-32 points, axes 0.3-0.8 m)."""
    d = rng.normal(size=(k, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return (d * np.asarray(axes)).astype(np.float32)


def static_floor(b: np.ndarray, idx: int, half=(50.0, 0.5, 50.0), y=-0.5, friction=0.5, world=0) -> None:
    set_box(b, idx, half)
    b["motion_type"][idx] = STATIC
    b["object_layer"][idx] = LAYER_NOT_MOVING
    b["position"][idx] = (0.0, y, 0.0)
    b["friction"][idx] = friction
    b["world"][idx] = world


def random_quaternions(rng: np.random.Generator, n: int) -> np.ndarray:
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return q.astype(np.float32)


def cube_heap(n_side: int = 10, seed: int = 1) -> Scene:
    """1,000 dynamic boxes (half extents 0.5 m, density 1000, friction 0.5,
    restitution 0) on an n_side^3 grid with 1.1 m spacing and uniform +-0.05 m
    jitter, dropped onto a static 100 x 1 x 100 m box floor; dt 1/60, 10/2
    iterations, 600 steps."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = n_side ** 3
    b = blank_bodies(n + 1)
    static_floor(b, 0, friction=0.5)
    idx = np.arange(1, n + 1)
    set_box(b, idx, (0.5, 0.5, 0.5))
    b["friction"][idx] = 0.5
    b["restitution"][idx] = 0.0
    g = np.stack(np.meshgrid(np.arange(n_side), np.arange(n_side), np.arange(n_side), indexing="ij"), -1).reshape(-1, 3)
    pos = np.empty((n, 3))
    pos[:, 0] = (g[:, 0] - (n_side - 1) / 2) * 1.1
    pos[:, 1] = 1.0 + g[:, 1] * 1.1
    pos[:, 2] = (g[:, 2] - (n_side - 1) / 2) * 1.1
    pos += rng.uniform(-0.05, 0.05, size=(n, 3))
    b["position"][idx] = pos.astype(np.float32)
    return Scene("cube_heap", b, dt=1.0 / 60.0, steps=600, velocity_iterations=10, position_iterations=2, seed=seed)


def batched_worlds(num_worlds: int = 4096, seed: int = 4, n_min: int = 8, n_max: int = 512) -> Scene:
    """num_worlds independent worlds with body counts drawn log-uniformly from
    [n_min, n_max]; boxes (half extents 0.2-0.8 m) and spheres (r 0.2-0.6 m),
    each world with its own static floor and seeded drop positions on a jittered
    3 m grid (wide enough for the largest rotated box); dt 1/120, 8/2
    iterations, 1,000 steps."""
    rng = np.random.Generator(np.random.PCG64(seed))
    counts = np.rint(np.exp(rng.uniform(math.log(n_min), math.log(n_max), size=num_worlds))).astype(np.int64)
    counts = np.clip(counts, n_min, n_max)
    total = int(counts.sum()) + num_worlds
    b = blank_bodies(total)
    o = 0
    for wi in range(num_worlds):
        static_floor(b, o, half=(30.0, 0.5, 30.0), friction=0.5, world=wi)
        o += 1
        c = int(counts[wi])
        sl = slice(o, o + c)
        b["world"][sl] = wi
        is_box = rng.random(c) < 0.5
        he = rng.uniform(0.2, 0.8, size=(c, 3)).astype(np.float32)
        r = rng.uniform(0.2, 0.6, size=c).astype(np.float32)
        for k in range(c):
            if is_box[k]:
                set_box(b, o + k, he[k])
            else:
                set_sphere(b, o + k, r[k])
        side = 8
        layer = np.arange(c) // (side * side)
        cell = np.arange(c) % (side * side)
        pos = np.stack([(cell % side - (side - 1) / 2) * 3.0, 1.5 + layer * 3.0, (cell // side - (side - 1) / 2) * 3.0], 1)
        pos += rng.uniform(-0.1, 0.1, size=(c, 3))
        b["position"][sl] = pos.astype(np.float32)
        b["quaternion"][sl] = random_quaternions(rng, c)
        b["friction"][sl] = 0.5
        o += c
    return Scene("batched_worlds", b, dt=1.0 / 120.0, steps=1000, velocity_iterations=8, position_iterations=2,
                 num_worlds=num_worlds, seed=seed)


def random_pairs_scene(n: int = 200, seed: int = 7, extent: float = 6.0, box_fraction: float = 0.6,
                       capsule_fraction: float = 0.0) -> Scene:
    """Boxes, spheres and (optionally) capsules at random poses inside a small region
    above a floor: a contact-rich state for stage-level parity (broadphase pairs,
    contacts).  Capsules: radius 0.2-0.4 m, half height 0.3-0.8 m."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = blank_bodies(n + 1)
    static_floor(b, 0, half=(20.0, 0.5, 20.0), friction=0.5)
    idx = np.arange(1, n + 1)
    is_box = rng.random(n) < box_fraction
    is_capsule = rng.random(n) < capsule_fraction
    for k, i in enumerate(idx):
        if is_capsule[k]:
            set_capsule(b, i, rng.uniform(0.2, 0.4), rng.uniform(0.3, 0.8))
        elif is_box[k]:
            set_box(b, i, rng.uniform(0.2, 0.7, size=3))
        else:
            set_sphere(b, i, rng.uniform(0.2, 0.6))
    pos = rng.uniform((-extent, 0.1, -extent), (extent, 2.5, extent), size=(n, 3))
    b["position"][idx] = pos.astype(np.float32)
    b["quaternion"][idx] = random_quaternions(rng, n)
    b["linear_velocity"][idx] = rng.normal(scale=1.0, size=(n, 3)).astype(np.float32)
    b["angular_velocity"][idx] = rng.normal(scale=1.0, size=(n, 3)).astype(np.float32)
    b["friction"][idx] = rng.uniform(0.1, 1.0, size=n).astype(np.float32)
    return Scene("random_pairs", b, dt=1.0 / 60.0, steps=1, seed=seed)


def resting_boxes(n: int = 64, seed: int = 3, spacing: float = 3.0) -> Scene:
    """Separated boxes resting (slightly penetrating) on a floor: every island
    holds one contact, so the solve order cannot differ from the reference."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = blank_bodies(n + 1)
    static_floor(b, 0, half=(60.0, 0.5, 60.0), friction=0.5)
    idx = np.arange(1, n + 1)
    side = int(math.ceil(math.sqrt(n)))
    he = rng.uniform(0.3, 0.6, size=(n, 3)).astype(np.float32)
    for k, i in enumerate(idx):
        set_box(b, i, he[k])
    gx = (np.arange(n) % side - side / 2) * spacing
    gz = (np.arange(n) // side - side / 2) * spacing
    y = he[:, 1] - rng.uniform(0.0, 0.01, size=n)
    b["position"][idx] = np.stack([gx, y, gz], 1).astype(np.float32)
    b["linear_velocity"][idx] = rng.normal(scale=0.3, size=(n, 3)).astype(np.float32)
    b["angular_velocity"][idx] = rng.normal(scale=0.3, size=(n, 3)).astype(np.float32)
    b["friction"][idx] = 0.5
    return Scene("resting_boxes", b, dt=1.0 / 60.0, steps=1, seed=seed)


def free_fall(n: int = 256, seed: int = 11) -> Scene:
    """Bodies far apart in free fall with spin: no contacts, pure integration."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = blank_bodies(n)
    for i in range(n):
        if i % 2:
            set_box(b, i, rng.uniform(0.2, 0.8, size=3))
        else:
            set_sphere(b, i, rng.uniform(0.2, 0.6))
    side = int(math.ceil(n ** (1 / 3)))
    g = np.stack(np.meshgrid(np.arange(side), np.arange(side), np.arange(side), indexing="ij"), -1).reshape(-1, 3)[:n]
    b["position"] = (g * 10.0 + np.array([0.0, 100.0, 0.0])).astype(np.float32)
    b["quaternion"] = random_quaternions(rng, n)
    b["linear_velocity"] = rng.normal(scale=2.0, size=(n, 3)).astype(np.float32)
    b["angular_velocity"] = rng.normal(scale=2.0, size=(n, 3)).astype(np.float32)
    b["allow_sleeping"] = 0
    return Scene("free_fall", b, dt=1.0 / 60.0, steps=30, seed=seed)


def box_stack(height: int = 10, seed: int = 21, half: float = 0.5, jitter: float = 0.02) -> Scene:
    """A single column of boxes with small seeded offsets, 1 cm above each other."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = blank_bodies(height + 1)
    static_floor(b, 0, half=(20.0, 0.5, 20.0), friction=0.5)
    idx = np.arange(1, height + 1)
    set_box(b, idx, (half, half, half))
    b["friction"][idx] = 0.5
    pos = np.zeros((height, 3))
    pos[:, 1] = half + 0.01 + np.arange(height) * (2 * half + 0.01)
    pos[:, [0, 2]] = rng.uniform(-jitter, jitter, size=(height, 2))
    b["position"][idx] = pos.astype(np.float32)
    return Scene("box_stack", b, dt=1.0 / 60.0, steps=120, seed=seed)


def box_row(count: int = 6, seed: int = 31, gap: float = -0.005) -> Scene:
    """A row of equal boxes resting on the floor, each slightly pressed into its
    neighbour: one island whose contacts split into several colours."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = blank_bodies(count + 1)
    static_floor(b, 0, half=(20.0, 0.5, 20.0), friction=0.5)
    idx = np.arange(1, count + 1)
    set_box(b, idx, (0.5, 0.5, 0.5))
    b["friction"][idx] = 0.5
    pos = np.zeros((count, 3))
    pos[:, 0] = np.arange(count) * (1.0 + gap)
    pos[:, 1] = 0.5 - 0.003
    pos[:, 2] = rng.uniform(-0.05, 0.05, size=count)
    b["position"][idx] = pos.astype(np.float32)
    b["linear_velocity"][idx] = rng.normal(scale=0.5, size=(count, 3)).astype(np.float32)
    return Scene("box_row", b, dt=1.0 / 60.0, steps=1, seed=seed)


def box_pyramid(base: int = 8, seed: int = 41, gap: float = -0.004) -> Scene:
    """A 2-D pyramid of equal boxes (rows of base, base-1, ..., 1) resting on the
    floor, each box pressed slightly into its neighbours: one island of about
    3 x base^2 / 2 contacts, solved by one warp up to 256 contacts."""
    rng = np.random.Generator(np.random.PCG64(seed))
    count = base * (base + 1) // 2
    b = blank_bodies(count + 1)
    static_floor(b, 0, half=(30.0, 0.5, 30.0), friction=0.5)
    idx = np.arange(1, count + 1)
    set_box(b, idx, (0.5, 0.5, 0.5))
    b["friction"][idx] = 0.5
    pos = []
    for row in range(base):
        for k in range(base - row):
            pos.append(((k + 0.5 * row) * (1.0 + gap), 0.5 - 0.003 + row * (1.0 - 0.006), 0.0))
    pos = np.asarray(pos)
    pos[:, 2] = rng.uniform(-0.03, 0.03, size=count)
    b["position"][idx] = pos.astype(np.float32)
    b["linear_velocity"][idx] = rng.normal(scale=0.3, size=(count, 3)).astype(np.float32)
    return Scene("box_pyramid", b, dt=1.0 / 60.0, steps=1, seed=seed)


def diff_rollout_worlds(num_worlds: int = 1024, seed: int = 5, boxes: int = 64) -> tuple:
    """Differentiable-rollout workload: num_worlds worlds of `boxes` boxes (half extents
    0.25-0.5 m, density 500-2000 kg/m^3, friction 0.1-1.0 per body) resting on their own
    floor on an 8-wide grid, with seeded initial linear (horizontal, up to 3 m/s per axis)
    and angular (up to 1 rad/s per axis) velocities so that they slide, spin and collide;
    120 steps at dt 1/60.  Returns (scene, targets): one seeded target point per world, within 2 m of
    the world's initial centroid.  Sleeping is off for this workload (the settings the
    caller builds pass allow_sleeping=False)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = blank_bodies(num_worlds * (boxes + 1))
    targets = np.zeros((num_worlds, 3), dtype=np.float32)
    side = 8
    o = 0
    for wi in range(num_worlds):
        static_floor(b, o, half=(20.0, 0.5, 20.0), friction=0.5, world=wi)
        o += 1
        sl = slice(o, o + boxes)
        b["world"][sl] = wi
        he = rng.uniform(0.25, 0.5, size=(boxes, 3)).astype(np.float32)
        for k in range(boxes):
            set_box(b, o + k, he[k])
        b["density"][sl] = rng.uniform(500.0, 2000.0, size=boxes).astype(np.float32)
        layer = np.arange(boxes) // (side * side)
        cell = np.arange(boxes) % (side * side)
        pos = np.stack([(cell % side - (side - 1) / 2) * 1.6, he[:, 1] + layer * 1.1,
                        (cell // side - (side - 1) / 2) * 1.6], 1)
        b["position"][sl] = pos.astype(np.float32)
        vel = np.zeros((boxes, 3))
        vel[:, 0] = rng.uniform(-3.0, 3.0, size=boxes)
        vel[:, 2] = rng.uniform(-3.0, 3.0, size=boxes)
        b["linear_velocity"][sl] = vel.astype(np.float32)
        b["angular_velocity"][sl] = rng.uniform(-1.0, 1.0, size=(boxes, 3)).astype(np.float32)
        b["friction"][sl] = rng.uniform(0.1, 1.0, size=boxes).astype(np.float32)
        b["allow_sleeping"][sl] = 0
        targets[wi] = pos.mean(0) + np.array([rng.uniform(-2, 2), 0.0, rng.uniform(-2, 2)])
        o += boxes
    sc = Scene("diff_rollout_worlds", b, dt=1.0 / 60.0, steps=120, velocity_iterations=10, position_iterations=2,
               num_worlds=num_worlds, seed=seed)
    return sc, targets


def capsules_on_floor(n: int = 16, seed: int = 51) -> Scene:
    """Capsules lying on the floor in a spaced row, their axis tilted 2-6 degrees so that
    one cap touches first (a perfectly level capsule has no unique deepest point along
    its segment), plus a few standing upright.  The static floor is body A, so each
    contact is a single point (update.ts:474)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = blank_bodies(n + 1)
    static_floor(b, 0, half=(30.0, 0.5, 30.0), friction=0.5)
    idx = np.arange(1, n + 1)
    r = rng.uniform(0.2, 0.4, size=n).astype(np.float32)
    h = rng.uniform(0.3, 0.8, size=n).astype(np.float32)
    for k, i in enumerate(idx):
        set_capsule(b, i, r[k], h[k])
    upright = np.arange(n) % 4 == 3
    tilt = np.radians(rng.uniform(2.0, 6.0, n))
    # lowest point of a lying capsule tilted by `tilt`: r + h sin(tilt) below its centre
    y = np.where(upright, h + r, r + h * np.sin(tilt)) - 0.003
    pos = np.stack([(np.arange(n) - (n - 1) / 2) * 3.0, y, rng.uniform(-0.1, 0.1, n)], 1)
    b["position"][idx] = pos.astype(np.float32)
    yaw = rng.uniform(0, np.pi, n)
    # lying: rotate local Y onto the floor plane (90 degrees less the tilt, about a horizontal
    # axis at angle yaw)
    q = []
    for k in range(n):
        if upright[k]:
            q.append((0.0, math.sin(yaw[k] / 2), 0.0, math.cos(yaw[k] / 2)))
        else:
            ax = (math.cos(yaw[k]), 0.0, math.sin(yaw[k]))
            half = (math.pi / 2 - tilt[k]) / 2
            q.append((ax[0] * math.sin(half), 0.0, ax[2] * math.sin(half), math.cos(half)))
    b["quaternion"][idx] = np.asarray(q, dtype=np.float32)
    b["linear_velocity"][idx] = rng.normal(scale=0.3, size=(n, 3)).astype(np.float32)
    b["friction"][idx] = 0.5
    return Scene("capsules_on_floor", b, dt=1.0 / 60.0, steps=1, seed=seed)


def bouncing_spheres(n: int = 48, seed: int = 61) -> Scene:
    """Spheres (restitution 0.6-0.9) dropped from 0.5-2 m above the floor, spaced apart:
    every contact with the floor is added, persists for a few steps, and is removed when the
    sphere bounces off, so the contact events of the listener cycle through all three kinds."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = blank_bodies(n + 1)
    static_floor(b, 0, half=(40.0, 0.5, 40.0), friction=0.5)
    idx = np.arange(1, n + 1)
    r = rng.uniform(0.2, 0.5, size=n).astype(np.float32)
    for k, i in enumerate(idx):
        set_sphere(b, i, r[k])
    side = int(math.ceil(math.sqrt(n)))
    pos = np.stack([(np.arange(n) % side) * 3.0 - 10.0, r + rng.uniform(0.5, 2.0, n), (np.arange(n) // side) * 3.0 - 10.0], 1)
    b["position"][idx] = pos.astype(np.float32)
    b["restitution"][idx] = rng.uniform(0.6, 0.9, size=n).astype(np.float32)
    b["allow_sleeping"][idx] = 0
    return Scene("bouncing_spheres", b, dt=1.0 / 60.0, steps=120, seed=seed)


def hinge_chains(num_chains: int = 4, links: int = 6, seed: int = 71, limits: bool = True) -> Scene:
    """Chains of boxes (0.8 x 0.2 x 0.2 m) joined end to end by hinges about Z, each hung
    from a static anchor and released horizontally, so they swing down under gravity.  Every
    other chain has limits of +-40 degrees on its joints (soft, 20 Hz, on the last chain);
    joined bodies do not collide (the ragdoll example's pair filter).  Chains are 3 m apart
    in Z and do not touch one another."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = num_chains * (links + 1)
    b = blank_bodies(n)
    h = hinge_defaults(num_chains * links)
    k = 0
    for c in range(num_chains):
        a = c * (links + 1)
        set_box(b, a, (0.1, 0.1, 0.1))
        b["motion_type"][a] = STATIC
        b["object_layer"][a] = LAYER_NOT_MOVING
        z = 3.0 * c
        b["position"][a] = (0.0, 5.0, z)
        prev, pivot_x = a, 0.0
        for i in range(links):
            j = a + 1 + i
            set_box(b, j, (0.4, 0.1, 0.1))
            b["position"][j] = (pivot_x + 0.5, 5.0, z)
            b["linear_velocity"][j] = (0.0, 0.0, rng.uniform(-0.05, 0.05))
            h[k]["body_a"], h[k]["body_b"] = prev, j
            h[k]["point_a"] = h[k]["point_b"] = (pivot_x, 5.0, z)
            h[k]["hinge_axis_a"] = h[k]["hinge_axis_b"] = (0.0, 0.0, 1.0)
            h[k]["normal_axis_a"] = h[k]["normal_axis_b"] = (1.0, 0.0, 0.0)
            if limits and c % 2 == 1:
                h[k]["limits_min"], h[k]["limits_max"] = -np.radians(40.0), np.radians(40.0)
                if c == num_chains - 1:
                    h[k]["limits_spring"]["frequency_or_stiffness"] = 20.0
                    h[k]["limits_spring"]["damping"] = 0.5
            prev, pivot_x = j, pivot_x + 1.0
            k += 1
    b["allow_sleeping"][:] = 0
    return Scene("hinge_chains", b, dt=1.0 / 60.0, steps=60, seed=seed, hinges=h, skip_joint_pairs=True)


def hinge_motors(n: int = 6, seed: int = 81) -> Scene:
    """Wings (3 x 0.2 x 0.2 m boxes) hinged about Z at their centre to static posts, one per
    motor configuration: velocity motors at -5 and 3 rad/s (one with its torque capped at
    200 N m), position motors driven to 60 and -30 degrees, a free wing held by 5 N m of
    hinge friction, and a wing with limits of -20..70 degrees.  Gravity acts on a wing that
    starts off balance (it is shifted 0.3 m from the pivot along its length)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = blank_bodies(2 * n)
    h = hinge_defaults(n)
    for i in range(n):
        post, wing = 2 * i, 2 * i + 1
        x = 5.0 * i
        set_box(b, post, (0.1, 0.1, 0.1))
        b["motion_type"][post] = STATIC
        b["object_layer"][post] = LAYER_NOT_MOVING
        b["position"][post] = (x, 3.0, -1.0)
        set_box(b, wing, (1.5, 0.1, 0.1))
        b["position"][wing] = (x + 0.3, 3.0, 0.0)
        b["quaternion"][wing] = (0.0, 0.0, math.sin(0.05), math.cos(0.05))
        h[i]["body_a"], h[i]["body_b"] = post, wing
        h[i]["point_a"] = h[i]["point_b"] = (x, 3.0, 0.0)
        h[i]["hinge_axis_a"] = h[i]["hinge_axis_b"] = (0.0, 0.0, 1.0)
        h[i]["normal_axis_a"] = h[i]["normal_axis_b"] = (1.0, 0.0, 0.0)
        b["angular_velocity"][wing] = (0.0, 0.0, rng.uniform(-0.5, 0.5))
    h[0]["motor_state"], h[0]["target_angular_velocity"] = MOTOR_VELOCITY, -5.0
    h[1]["motor_state"], h[1]["target_angular_velocity"] = MOTOR_VELOCITY, 3.0
    h[1]["min_torque_limit"], h[1]["max_torque_limit"] = -200.0, 200.0
    h[2]["motor_state"], h[2]["target_angle"] = MOTOR_POSITION, np.radians(60.0)
    h[3]["motor_state"], h[3]["target_angle"] = MOTOR_POSITION, -np.radians(30.0)
    h[3]["motor_spring"]["mode"], h[3]["motor_spring"]["frequency_or_stiffness"] = 1, 4000.0
    h[3]["motor_spring"]["damping"] = 300.0
    h[4]["motor_state"], h[4]["max_friction_torque"] = MOTOR_OFF, 5.0
    if n > 5:
        h[5]["limits_min"], h[5]["limits_max"] = -np.radians(20.0), np.radians(70.0)
    b["allow_sleeping"][:] = 0
    return Scene("hinge_motors", b, dt=1.0 / 60.0, steps=90, seed=seed, hinges=h)


def _qmul(a, b):
    ax, ay, az, aw = a
    bx, by, bz, bw = b
    return np.array([aw * bx + ax * bw + ay * bz - az * by, aw * by - ax * bz + ay * bw + az * bx,
                     aw * bz + ax * by - ay * bx + az * bw, aw * bw - ax * bx - ay * by - az * bz])


def _qrot(q, v):
    ux, uy, uz, w = float(q[0]), float(q[1]), float(q[2]), float(q[3])
    vx, vy, vz = float(v[0]), float(v[1]), float(v[2])
    tx, ty, tz = 2.0 * (uy * vz - uz * vy), 2.0 * (uz * vx - ux * vz), 2.0 * (ux * vy - uy * vx)
    return np.array([vx + w * tx + (uy * tz - uz * ty), vy + w * ty + (uz * tx - ux * tz),
                     vz + w * tz + (ux * ty - uy * tx)])


def _tangent(axis):
    """getTangent of the ragdoll example (examples/src/example-ragdoll.ts:431-445)."""
    ax, ay, az = np.abs(axis)
    if ax <= ay and ax <= az:
        t = np.array([0.0, -axis[2], axis[1]])
    elif ay <= az:
        t = np.array([axis[2], 0.0, -axis[0]])
    else:
        t = np.array([-axis[1], axis[0], 0.0])
    return t / np.linalg.norm(t)


# ragdoll topology of examples/src/example-ragdoll.ts:75-301 at scale 1.8, with capsule parts:
# part -> (centre in the ragdoll frame, limb axis, length, thickness)
def _ragdoll_parts(scale: float = 1.8):
    sd, ual, lal, uas, las = 0.45 * scale, 0.4 * scale, 0.4 * scale, 0.15 * scale, 0.15 * scale
    nl, hr, ubl, pl, ps = 0.1 * scale, 0.2 * scale, 0.6 * scale, 0.2 * scale, 0.25 * scale
    ull, uls, lls, lll = 0.5 * scale, 0.15 * scale, 0.15 * scale, 0.5 * scale
    lower_leg_y = lll / 2
    upper_leg_y = lower_leg_y + lll / 2 + ull / 2
    pelvis_y = upper_leg_y + ull / 2 + pl / 2
    upper_body_y = pelvis_y + pl / 2 + ubl / 2
    head_y = upper_body_y + ubl / 2 + hr / 2 + nl
    arm_y = upper_body_y + ubl / 2
    Y, X = (0.0, 1.0, 0.0), (1.0, 0.0, 0.0)
    parts = {
        "upper_body": ((0, upper_body_y, 0), Y, ubl, sd * 0.6),
        "head": ((0, head_y, 0), Y, hr * 1.4, hr * 1.2),
        "upper_left_arm": ((-sd / 2 - ual / 2, arm_y, 0), X, ual, uas),
        "lower_left_arm": ((-sd / 2 - ual - lal / 2, arm_y, 0), X, lal, las),
        "upper_right_arm": ((sd / 2 + ual / 2, arm_y, 0), X, ual, uas),
        "lower_right_arm": ((sd / 2 + ual + lal / 2, arm_y, 0), X, lal, las),
        "pelvis": ((0, pelvis_y, 0), Y, pl, ps),
        "upper_left_leg": ((-sd / 3, upper_leg_y, 0), Y, ull, uls),
        "lower_left_leg": ((-sd / 3, lower_leg_y, 0), Y, lll, lls),
        "upper_right_leg": ((sd / 3, upper_leg_y, 0), Y, ull, uls),
        "lower_right_leg": ((sd / 3, lower_leg_y, 0), Y, lll, lls),
    }
    # joints: (kind, body A, body B, pivot in the ragdoll frame, twist / hinge axis)
    joints = [
        ("swing", "head", "upper_body", (0, upper_body_y + ubl / 2, 0), Y),                  # neck
        ("hinge", "lower_left_leg", "upper_left_leg", (-sd / 3, lll, 0), X),                 # knees
        ("hinge", "lower_right_leg", "upper_right_leg", (sd / 3, lll, 0), X),
        ("swing", "upper_left_leg", "pelvis", (-sd / 3, upper_leg_y + ull / 2, 0), Y),       # hips
        ("swing", "upper_right_leg", "pelvis", (sd / 3, upper_leg_y + ull / 2, 0), Y),
        ("swing", "pelvis", "upper_body", (0, pelvis_y + pl / 2, 0), Y),                     # spine
        ("swing", "upper_body", "upper_left_arm", (-sd / 2, arm_y, 0), X),                   # shoulders
        ("swing", "upper_body", "upper_right_arm", (sd / 2, arm_y, 0), X),
        ("hinge", "lower_left_arm", "upper_left_arm", (-sd / 2 - ual, arm_y, 0), (0.0, 0.0, 1.0)),  # elbows
        ("hinge", "lower_right_arm", "upper_right_arm", (sd / 2 + ual, arm_y, 0), (0.0, 0.0, 1.0)),
    ]
    return parts, joints


def _rot(axis, angle):
    """Rotation matrix of `angle` about the unit `axis`."""
    a = np.asarray(axis, dtype=np.float64)
    a = a / np.linalg.norm(a)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + math.sin(angle) * K + (1 - math.cos(angle)) * (K @ K)


def _mat_to_quat(R):
    """Unit quaternion (x, y, z, w) of a rotation matrix."""
    tr = R[0, 0] + R[1, 1] + R[2, 2]
    if tr > 0:
        s = math.sqrt(tr + 1.0) * 2
        q = [(R[2, 1] - R[1, 2]) / s, (R[0, 2] - R[2, 0]) / s, (R[1, 0] - R[0, 1]) / s, 0.25 * s]
    elif R[0, 0] > R[1, 1] and R[0, 0] > R[2, 2]:
        s = math.sqrt(1.0 + R[0, 0] - R[1, 1] - R[2, 2]) * 2
        q = [0.25 * s, (R[0, 1] + R[1, 0]) / s, (R[0, 2] + R[2, 0]) / s, (R[2, 1] - R[1, 2]) / s]
    elif R[1, 1] > R[2, 2]:
        s = math.sqrt(1.0 + R[1, 1] - R[0, 0] - R[2, 2]) * 2
        q = [(R[0, 1] + R[1, 0]) / s, 0.25 * s, (R[1, 2] + R[2, 1]) / s, (R[0, 2] - R[2, 0]) / s]
    else:
        s = math.sqrt(1.0 + R[2, 2] - R[0, 0] - R[1, 1]) * 2
        q = [(R[0, 2] + R[2, 0]) / s, (R[1, 2] + R[2, 1]) / s, 0.25 * s, (R[1, 0] - R[0, 1]) / s]
    q = np.array(q)
    return q / np.linalg.norm(q)


def _segment_distances(p0, p1, q0, q1):
    """Distances between the segments p0[k]-p1[k] and q0[k]-q1[k] (clamped closest points)."""
    d1, d2, r = p1 - p0, q1 - q0, p0 - q0
    a, e, f = (d1 * d1).sum(1), (d2 * d2).sum(1), (d2 * r).sum(1)
    c, b = (d1 * r).sum(1), (d1 * d2).sum(1)
    den = a * e - b * b
    s = np.where(den > 1e-12, np.clip((b * f - c * e) / np.where(den > 1e-12, den, 1.0), 0.0, 1.0), 0.0)
    t = (b * s + f) / e
    lo, hi = t < 0.0, t > 1.0
    s = np.where(lo, np.clip(-c / a, 0.0, 1.0), np.where(hi, np.clip((b - c) / a, 0.0, 1.0), s))
    t = np.clip(t, 0.0, 1.0)
    return np.linalg.norm((p0 + d1 * s[:, None]) - (q0 + d2 * t[:, None]), axis=1)


def _pose_overlaps(T, parts, joints, margin: float = 0.05) -> bool:
    """Whether two parts that share no joint overlap (capsule segments closer than their radii)."""
    names = list(parts)
    joined = {frozenset((na, nb)) for _, na, nb, _, _ in joints}
    ends0, ends1, rad = [], [], []
    for name in names:
        c, axis, length, thick = parts[name]
        R, t = T[name]
        hh = max(length / 2 - thick / 2, 0.05)
        ax = R @ np.asarray(axis, dtype=np.float64) * hh
        mid = R @ np.asarray(c, dtype=np.float64) + t
        ends0.append(mid - ax)
        ends1.append(mid + ax)
        rad.append(thick / 2)
    ii, jj = zip(*[(i, j) for i in range(len(names)) for j in range(i + 1, len(names))
                   if frozenset((names[i], names[j])) not in joined])
    ii, jj = np.array(ii), np.array(jj)
    e0, e1, rad = np.array(ends0), np.array(ends1), np.array(rad)
    d = _segment_distances(e0[ii], e1[ii], e0[jj], e1[jj])
    return bool((d < rad[ii] + rad[jj] + margin).any())


def _ragdoll_pose(rng, parts, joints, cones, twist, fill: float = 0.6, tries: int = 64):
    """A seeded random pose: every joint turned by a random angle inside `fill` of its limits,
    the parts placed by walking the joint tree out from the upper body; poses in which two parts
    that share no joint overlap are drawn again.  Returns per part the rotation R and
    translation t of the pose in the ragdoll frame (rest point x -> R x + t)."""
    for _ in range(tries):
        T = _ragdoll_pose_once(rng, parts, joints, cones, twist, fill)
        if not _pose_overlaps(T, parts, joints):
            return T
    return {name: (np.eye(3), np.zeros(3)) for name in parts}


def _ragdoll_pose_once(rng, parts, joints, cones, twist, fill):
    T = {name: (np.eye(3), np.zeros(3)) for name in parts}
    placed = {"upper_body"}
    done = set()
    while len(done) < len(joints):
        for j, (kind, na, nbn, piv, axis) in enumerate(joints):
            if j in done or (na in placed) == (nbn in placed):
                continue
            child, parent = (na, nbn) if nbn in placed else (nbn, na)
            a = np.asarray(axis, dtype=np.float64)
            if kind == "hinge":
                lo, hi = (-2.0, 0.05) if axis[0] else (-0.05, 2.2)
                theta = rng.uniform(lo, hi) * fill
                # the hinge angle is B's rotation relative to A about the axis; the child is A
                Rj = _rot(a, -theta if child == na else theta)
            else:
                u = _tangent(a)
                v = np.cross(a, u)
                phi = rng.uniform(0.0, 2 * math.pi)
                s_axis = math.cos(phi) * u + math.sin(phi) * v
                Rj = _rot(s_axis, rng.uniform(0.0, fill * cones[j])) @ _rot(a, rng.uniform(-fill, fill) * twist)
            Rp, tp = T[parent]
            P = Rp @ np.asarray(piv, dtype=np.float64) + tp
            Rw = Rp @ Rj @ Rp.T
            T[child] = (Rw @ Rp, Rw @ (tp - P) + P)
            placed.add(child)
            done.add(j)
    return T


def ragdolls(num: int = 2000, seed: int = 3, arena: float = 60.0, spacing: float = 4.4,
             cone_deg=(30.0, 80.0), twist_deg: float = 45.0, random_poses: bool = True) -> Scene:
    """Jointed ragdolls: per ragdoll 11 capsule bodies (the ragdoll example's parts and
    sizes at scale 1.8) joined by 4 hinges (knees, elbows) and 6 swing-twist joints (neck,
    spine, hips, shoulders; cone half-angles drawn from U(30, 80) degrees per joint, twist
    limits +-45 degrees, motors off), each ragdoll at a seeded random orientation on a grid
    inside an arena of 6 static walls (a 60 m box).  With random_poses every joint starts
    turned by a seeded random angle inside 60 % of its limits (hinges along their axis, swing
    about a random axis across the twist axis plus a twist); the joints are created in that
    pose, each body's joint axes turned with it, so the pose is a bend of the joint and not its
    zero.  Joined bodies do not collide (the ragdoll example's pair filter); dt 1/60, 12
    velocity / 4 position iterations."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pose_rng = np.random.Generator(np.random.PCG64(seed + 1000))
    parts, joints = _ragdoll_parts()
    names = list(parts)
    nb_r = len(names)
    walls = 6
    b = blank_bodies(walls + num * nb_r)
    half = arena / 2
    t = 1.0
    wall_specs = [((half + t, t, half + t), (0, -t, 0)), ((half + t, t, half + t), (0, arena + t, 0)),
                  ((t, half, half + t), (-half - t, half, 0)), ((t, half, half + t), (half + t, half, 0)),
                  ((half + t, half, t), (0, half, -half - t)), ((half + t, half, t), (0, half, half + t))]
    for k, (he, pos) in enumerate(wall_specs):
        set_box(b, k, he)
        b["motion_type"][k] = STATIC
        b["object_layer"][k] = LAYER_NOT_MOVING
        b["position"][k] = pos
        b["friction"][k] = 0.5
    n_side = int(math.floor((arena - 2.0) / spacing))
    cells = [(i, j, k) for j in range(n_side) for i in range(n_side) for k in range(n_side)]
    assert num <= len(cells), "arena too small for that many ragdolls"
    h_all = hinge_defaults(num * 4)
    s_all = swing_twist_defaults(num * 6)
    hk = sk = 0
    centre = np.array([0.0, 1.6, 0.0])
    for r in range(num):
        i, j, k = cells[r]
        origin = np.array([-half + 1.0 + spacing * (i + 0.5), 1.0 + spacing * (j + 0.5), -half + 1.0 + spacing * (k + 0.5)])
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        cones = [np.radians(rng.uniform(*cone_deg)) if kind == "swing" else 0.0 for kind, *_ in joints]
        T = (_ragdoll_pose(pose_rng, parts, joints, cones, np.radians(twist_deg)) if random_poses
             else {name: (np.eye(3), np.zeros(3)) for name in parts})
        base = walls + r * nb_r
        idx = {}
        for p, name in enumerate(names):
            c, axis, length, thick = parts[name]
            bi = base + p
            idx[name] = bi
            radius = thick / 2
            set_capsule(b, bi, radius, max(length / 2 - radius, 0.05))
            R, t = T[name]
            b["position"][bi] = origin + _qrot(q, R @ np.asarray(c, dtype=np.float64) + t - centre)
            # capsules lie along local Y: arms are turned onto X
            qp = np.array([0.0, 0.0, -math.sin(math.pi / 4), math.cos(math.pi / 4)]) if axis[0] else np.array([0, 0, 0, 1.0])
            b["quaternion"][bi] = _qmul(_qmul(q, _mat_to_quat(R)), qp)
            b["restitution"][bi] = 0.0

        def turned(name, v):  # a rest-frame direction carried by a part's pose, then the ragdoll's orientation
            return _qrot(q, T[name][0] @ np.asarray(v, dtype=np.float64))

        for jn, (kind, na, nbn, piv, axis) in enumerate(joints):
            RB, tB = T[nbn]
            pw = origin + _qrot(q, RB @ np.asarray(piv, dtype=np.float64) + tB - centre)
            if kind == "hinge":
                h = h_all[hk]
                hk += 1
                h["body_a"], h["body_b"] = idx[na], idx[nbn]
                h["point_a"] = h["point_b"] = pw
                h["hinge_axis_a"], h["hinge_axis_b"] = turned(na, axis), turned(nbn, axis)
                limb = np.array([1.0, 0, 0]) if axis[2] else np.array([0, 1.0, 0])
                h["normal_axis_a"], h["normal_axis_b"] = turned(na, limb), turned(nbn, limb)
                h["limits_min"], h["limits_max"] = (-2.0, 0.05) if axis[0] else (-0.05, 2.2)
            else:
                sj = s_all[sk]
                sk += 1
                sj["body_a"], sj["body_b"] = idx[na], idx[nbn]
                sj["position_a"] = sj["position_b"] = pw
                tg = _tangent(np.asarray(axis, dtype=np.float64))
                sj["twist_axis_a"], sj["twist_axis_b"] = turned(na, axis), turned(nbn, axis)
                sj["plane_axis_a"], sj["plane_axis_b"] = turned(na, tg), turned(nbn, tg)
                sj["swing_type"] = SWING_CONE
                sj["normal_half_cone_angle"] = sj["plane_half_cone_angle"] = cones[jn]
                sj["twist_min_angle"], sj["twist_max_angle"] = -np.radians(twist_deg), np.radians(twist_deg)
    return Scene("ragdolls", b, dt=1.0 / 60.0, steps=600, velocity_iterations=12, position_iterations=4,
                 seed=seed, hinges=h_all, swings=s_all, skip_joint_pairs=True)


def swing_twist_chains(seed: int = 91) -> Scene:
    """Four chains of five boxes (0.2 x 0.8 x 0.2 m) hung from static anchors by swing-twist
    joints and released tilted 60 degrees, so that the cone limits engage: a cone of 30
    degrees, an elliptic cone (20 and 50 degrees), a pyramid of +-30 degrees about Z and +-20
    degrees about Y, and a chain with its twist and its swing about Y
    locked (limits inside +-0.5 degrees) and its swing about Z limited to 40 degrees; each link
    starts with a spin about its own axis so that the twist limits (+-15 degrees) engage too."""
    rng = np.random.Generator(np.random.PCG64(seed))
    links, chains = 5, 4
    b = blank_bodies(chains * (links + 1))
    sj = swing_twist_defaults(chains * links)
    tilt = math.radians(60.0)
    d = np.array([math.sin(tilt), -math.cos(tilt), 0.0])  # chain direction, down and out
    qt = np.array([0.0, 0.0, math.sin(tilt / 2), math.cos(tilt / 2)])
    k = 0
    for c in range(chains):
        a = c * (links + 1)
        set_box(b, a, (0.1, 0.1, 0.1))
        b["motion_type"][a] = STATIC
        b["object_layer"][a] = LAYER_NOT_MOVING
        top = np.array([0.0, 8.0, 3.0 * c])
        b["position"][a] = top
        prev = a
        for i in range(links):
            j = a + 1 + i
            set_box(b, j, (0.1, 0.4, 0.1))
            b["position"][j] = top + d * (0.5 + i * 1.0)
            b["quaternion"][j] = qt
            b["angular_velocity"][j] = d * rng.uniform(2.0, 4.0)
            h = sj[k]
            h["body_a"], h["body_b"] = prev, j
            h["position_a"] = h["position_b"] = top + d * (i * 1.0)
            h["twist_axis_a"] = h["twist_axis_b"] = d
            h["plane_axis_a"] = h["plane_axis_b"] = (0.0, 0.0, 1.0)
            h["twist_min_angle"], h["twist_max_angle"] = -math.radians(15.0), math.radians(15.0)
            if c == 0:
                h["normal_half_cone_angle"] = h["plane_half_cone_angle"] = math.radians(30.0)
            elif c == 1:
                h["normal_half_cone_angle"], h["plane_half_cone_angle"] = math.radians(20.0), math.radians(50.0)
            elif c == 2:
                h["swing_type"] = SWING_PYRAMID
                h["normal_half_cone_angle"], h["plane_half_cone_angle"] = math.radians(30.0), math.radians(20.0)
            else:
                h["normal_half_cone_angle"], h["plane_half_cone_angle"] = math.radians(40.0), math.radians(0.2)
                h["twist_min_angle"], h["twist_max_angle"] = 0.0, 0.0
            prev = j
            k += 1
    b["allow_sleeping"][:] = 0
    return Scene("swing_twist_chains", b, dt=1.0 / 60.0, steps=90, seed=seed, swings=sj, skip_joint_pairs=True)


def mixed_convex_pile(n: int = 400, seed: int = 2, extent: float = 12.0, heights=(1.0, 8.0), floor: bool = True,
                      speeds=(0.0, 0.0), fast_fraction: float = 0.0) -> Scene:
    """The mixed convex pile's bodies: shape type uniform over spheres (r 0.2-0.6 m), boxes
    (half extents 0.2-0.8 m), capsules (r 0.2-0.4 m, half height 0.3-0.8 m) and convex hulls of
    16-32 points on an ellipsoid (semi-axes 0.3-0.8 m), dropped from the given heights over an
    area of 1.6 extent x 1.6 extent m onto a static box floor (the terrain mesh of the full
    workload is not part of this scene), at seeded random orientations; fast_fraction of the bodies get
    speeds drawn from `speeds` in a random direction."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nb = n + (1 if floor else 0)
    b = blank_bodies(nb)
    k0 = 0
    if floor:  # three times the drop area, so that nothing rolls off the edge
        static_floor(b, 0, half=(3 * extent, 0.5, 3 * extent), friction=0.5)
        k0 = 1
    idx = np.arange(k0, nb)
    kinds = rng.integers(0, 4, size=n)
    hulls = []
    for j, i in enumerate(idx):
        if kinds[j] == 0:
            set_sphere(b, i, rng.uniform(0.2, 0.6))
        elif kinds[j] == 1:
            set_box(b, i, rng.uniform(0.2, 0.8, size=3))
        elif kinds[j] == 2:
            set_capsule(b, i, rng.uniform(0.2, 0.4), rng.uniform(0.3, 0.8))
        else:
            k = int(rng.integers(16, 33))
            hulls.append(ellipsoid_hull_points(rng, k, rng.uniform(0.3, 0.8, size=3)))
            set_hull(b, i, len(hulls) - 1)
    b["position"][idx] = np.stack([rng.uniform(-extent * 0.8, extent * 0.8, n), rng.uniform(*heights, n),
                                   rng.uniform(-extent * 0.8, extent * 0.8, n)], 1).astype(np.float32)
    b["quaternion"][idx] = random_quaternions(rng, n)
    fast = rng.random(n) < fast_fraction
    if fast.any():
        d = rng.normal(size=(int(fast.sum()), 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        b["linear_velocity"][idx[fast]] = (d * rng.uniform(*speeds, size=(len(d), 1))).astype(np.float32)
    b["friction"][idx] = 0.5
    return Scene("mixed_convex_pile", b, dt=1.0 / 60.0, steps=300, velocity_iterations=8, position_iterations=2,
                 seed=seed, hull_points=hulls)


def ccd_gallery(num_worlds: int = 1, seed: int = 101, arrival_steps: int = 3) -> Scene:
    """Fast LINEAR_CAST bodies (MotionQuality.LINEAR_CAST, update.ts:930-968) against thin walls,
    per world:

    * a static floor and a static wall 10 cm thick (half extents 0.05 x 3 x 6) at x = 8;
    * five bullets of every shape (spheres of radius 0.12-0.2, a spinning box, a capsule, a
      convex hull) at 150-260 m/s, aimed at the wall at small angles;
    * a bullet with restitution 0.6 (it bounces off the wall);
    * a dynamic box in front of the wall hit by one bullet (impulse into a dynamic body);
    * two bullets flying head-on into each other (a pair of cast bodies, z = 10).

    The dynamic box is LINEAR_CAST too: at rest it stays below the cast threshold and moves
    discretely, once hit it is cast.

    The bullets start far enough back to arrive after about ``arrival_steps`` steps at 60 Hz.
    Hull points: one ellipsoid per world (hull index = world).
    """
    rng = np.random.default_rng(seed)
    per = 12
    n = per * num_worlds
    b = blank_bodies(n)
    hulls = []
    for wd in range(num_worlds):
        o = wd * per
        b["world"][o:o + per] = wd
        static_floor(b, o, half=(40.0, 0.5, 40.0), world=wd)
        set_box(b, o + 1, (0.05, 3.0, 6.0))
        b["motion_type"][o + 1] = STATIC
        b["object_layer"][o + 1] = LAYER_NOT_MOVING
        b["position"][o + 1] = (8.0, 3.0, 0.0)
        hulls.append(ellipsoid_hull_points(rng, 20, (0.15, 0.12, 0.1)))
        bullets = range(o + 2, o + 7)
        for k, i in enumerate(bullets):
            speed = rng.uniform(150.0, 260.0)
            y = 1.0 + 0.8 * k
            z = rng.uniform(-3.0, 3.0)
            ang = rng.uniform(-0.25, 0.25)
            d = np.array([math.cos(ang), rng.uniform(-0.05, 0.05), math.sin(ang)])
            d /= np.linalg.norm(d)
            start = np.array([8.0, y, z]) - d * speed / 60.0 * (arrival_steps - 0.5)
            b["position"][i] = start
            b["linear_velocity"][i] = d * speed
            b["motion_quality"][i] = 1
            b["gravity_factor"][i] = 0.0
            b["allow_sleeping"][i] = 0
        set_sphere(b, o + 2, 0.2)
        set_sphere(b, o + 3, 0.12)
        set_box(b, o + 4, (0.1, 0.08, 0.25))
        b["angular_velocity"][o + 4] = (3.0, 7.0, -2.0)
        set_capsule(b, o + 5, 0.08, 0.15)
        b["quaternion"][o + 5] = (0.0, 0.0, math.sin(math.pi / 4), math.cos(math.pi / 4))
        set_hull(b, o + 6, wd)
        # a bouncing bullet
        i = o + 7
        set_sphere(b, i, 0.15)
        b["restitution"][i] = 0.6
        b["position"][i] = (8.0 - 200.0 / 60.0 * (arrival_steps - 0.5), 5.0, -4.0)
        b["linear_velocity"][i] = (200.0, 0.0, 0.0)
        b["motion_quality"][i] = 1
        b["gravity_factor"][i] = 0.0
        # a dynamic box in front of the wall, hit by a bullet
        set_box(b, o + 8, (0.4, 0.4, 0.4))
        b["position"][o + 8] = (6.0, 0.4, 5.0)
        b["motion_quality"][o + 8] = 1  # below the cast threshold until the bullet hits it
        i = o + 9
        set_sphere(b, i, 0.1)
        b["position"][i] = (6.0 - 180.0 / 60.0 * (arrival_steps - 0.5), 0.45, 5.0)
        b["linear_velocity"][i] = (180.0, 0.0, 0.0)
        b["motion_quality"][i] = 1
        b["gravity_factor"][i] = 0.0
        # two bullets head-on
        for i, x, v in ((o + 10, -4.0, 160.0), (o + 11, 4.0, -160.0)):
            set_sphere(b, i, 0.15)
            b["position"][i] = (x, 2.0, 10.0)
            b["linear_velocity"][i] = (v, 0.0, 0.0)
            b["motion_quality"][i] = 1
            b["gravity_factor"][i] = 0.0
    sc = Scene("ccd_gallery", b, dt=1.0 / 60.0, steps=8, num_worlds=num_worlds, seed=seed, hull_points=hulls)
    return sc


def heightfield(n_cells: int = 256, cell: float = 1.0, amplitude: float = 4.0, seed: int = 2,
                octaves: int = 3) -> tuple:
    """A terrain of n_cells x n_cells square cells of the given size centred on the origin, two
    triangles per cell wound upwards, the height value noise (bilinear interpolation of random
    lattice values over octaves of halving period) scaled to +-amplitude/2.  The rolling
    terrain of the 20,000-body mixed workload (256 x 256 cells of 1 m, amplitude 4 m, 131,072
    triangles).  Returns (positions (float32, (n+1)^2 x 3), indices (int32, 2 n^2 x 3))."""
    rng = np.random.default_rng(seed)
    n = n_cells + 1
    h = np.zeros((n, n))
    for o in range(octaves):
        period = max(2, n_cells // (4 << o))
        g = n_cells // period + 2
        lattice = rng.uniform(-1.0, 1.0, (g, g))
        u = np.arange(n) / period
        i0 = np.floor(u).astype(int)
        f = u - i0
        a = lattice[i0][:, i0]
        b = lattice[i0 + 1][:, i0]
        c = lattice[i0][:, i0 + 1]
        d = lattice[i0 + 1][:, i0 + 1]
        fx = f[:, None]
        fz = f[None, :]
        h += (a * (1 - fx) * (1 - fz) + b * fx * (1 - fz) + c * (1 - fx) * fz + d * fx * fz) / (2 ** o)
    h *= 0.5 * amplitude / max(1e-9, np.abs(h).max())
    xs = (np.arange(n) - n_cells / 2.0) * cell
    X, Z = np.meshgrid(xs, xs, indexing="ij")
    pos = np.stack([X, h, Z], axis=-1).reshape(-1, 3).astype(np.float32)
    idx = []
    for i in range(n_cells):
        for j in range(n_cells):
            v00, v10, v01, v11 = i * n + j, (i + 1) * n + j, i * n + j + 1, (i + 1) * n + j + 1
            # counter-clockwise seen from above (+Y): normals point up
            idx.append((v00, v01, v10))
            idx.append((v10, v01, v11))
    return pos, np.array(idx, dtype=np.int32)


def mesh_drop(n: int = 64, n_cells: int = 24, seed: int = 5, amplitude: float = 2.0,
              heights=(1.0, 4.0), fast_fraction: float = 0.0) -> Scene:
    """Bodies of every shape (spheres, boxes, capsules, convex hulls; the mixed pile's size
    ranges) dropped on a heightfield terrain of n_cells x n_cells 1 m cells (one static mesh
    body, index 0; hull points per hull body, mesh data in scene.mesh).  fast_fraction of the
    bodies start at 20-60 m/s in a random downward direction."""
    rng = np.random.default_rng(seed)
    pos, idx = heightfield(n_cells, 1.0, amplitude, seed)
    b = blank_bodies(n + 1)
    b["shape_type"][0] = SHAPE_TRIANGLE_MESH
    b["shape_params"][0] = 0.0
    b["motion_type"][0] = STATIC
    b["object_layer"][0] = LAYER_NOT_MOVING
    b["friction"][0] = 0.5
    hulls = []
    half = 0.4 * n_cells
    for i in range(1, n + 1):
        k = rng.integers(0, 4)
        if k == 0:
            set_sphere(b, i, rng.uniform(0.2, 0.6))
        elif k == 1:
            set_box(b, i, rng.uniform(0.2, 0.8, 3))
        elif k == 2:
            set_capsule(b, i, rng.uniform(0.2, 0.4), rng.uniform(0.3, 0.8))
        else:
            hulls.append(ellipsoid_hull_points(rng, int(rng.integers(16, 33)), rng.uniform(0.3, 0.8, 3)))
            set_hull(b, i, len(hulls) - 1)
        b["position"][i] = (rng.uniform(-half, half), rng.uniform(*heights) + amplitude / 2 + 1.0,
                            rng.uniform(-half, half))
        b["friction"][i] = 0.5
    b["quaternion"][1:] = random_quaternions(rng, n)
    fast = rng.random(n) < fast_fraction
    for i in np.nonzero(fast)[0] + 1:
        d = rng.normal(size=3)
        d[1] = -abs(d[1]) - 0.5
        d /= np.linalg.norm(d)
        b["linear_velocity"][i] = d * rng.uniform(20.0, 60.0)
        b["motion_quality"][i] = 1
    sc = Scene("mesh_drop", b, dt=1.0 / 60.0, steps=120, seed=seed, hull_points=hulls)
    sc.mesh = (pos, idx)
    return sc


def joint_zoo(seed: int = 91) -> Scene:
    """One world of every point, distance, fixed, cone and slider joint configuration, each
    group hung from (or slid along) its own static post, 4 m apart in Z so no group touches
    another; joined bodies do not collide (the ragdoll example's pair filter).  Released under
    gravity with small seeded sideways velocities:

    * point: two chains of 4 boxes (0.4 x 0.1 x 0.1 m) joined end to end by ball joints and
      released horizontally, the second with 0.5 m/s sideways;
    * distance: a rigid 1.5 m rod to a sphere released horizontally; a slack rope (0.5..2 m)
      to a sphere 1 m below its post; a stiff spring (2000 N/m, 1 m rest length) to a sphere
      hung 0.3 m below its rest length;
    * fixed: a cantilever of two boxes welded end to end to a post; a free pair of welded
      boxes thrown spinning as one rigid body;
    * cone: two pendulum capsules with 30 degree cones about the hanging direction, started
      20 degrees out and swinging outwards;
    * slider: a box on a 30 degree incline rail with limits -1..1 m; a velocity motor (2 m/s)
      and a position motor (0.5 m) on horizontal rails; a horizontal slide held back by 20 N of
      friction; a slider between two free boxes."""
    rng = np.random.Generator(np.random.PCG64(seed))
    rows = []   # (shape, params, position, quaternion, static, linear velocity, angular velocity)

    def body(shape, params, pos, static=False, q=(0.0, 0.0, 0.0, 1.0), v=(0.0, 0.0, 0.0), w=(0.0, 0.0, 0.0)):
        rows.append((shape, params, pos, q, static, v, w))
        return len(rows) - 1

    def post(pos):
        return body("box", (0.1, 0.1, 0.1), pos, static=True)

    J = {t: [] for t in (JOINT_POINT, JOINT_DISTANCE, JOINT_FIXED, JOINT_CONE, JOINT_SLIDER)}

    def joint(t, a, b, **f):
        r = joint_defaults(t, 1)[0]
        r["body_a"], r["body_b"] = a, b
        for k, v in f.items():
            if isinstance(v, dict):
                for kk, vv in v.items():
                    r[k][kk] = vv
            else:
                r[k] = v
        J[t].append(r)

    jitter = lambda: (0.0, 0.0, float(rng.uniform(-0.05, 0.05)))
    # point: ball-joint chains
    for c in range(2):
        z = 4.0 * c
        prev, x = post((0.0, 8.0, z)), 0.0
        for i in range(4):
            v = (0.0, 0.0, 0.5) if c == 1 else jitter()
            j = body("box", (0.4, 0.1, 0.1), (x + 0.5, 8.0, z), v=v)
            joint(JOINT_POINT, prev, j, point_a=(x, 8.0, z), point_b=(x, 8.0, z))
            prev, x = j, x + 1.0
    # distance: rod, slack rope, spring
    z = 8.0
    a = post((0.0, 8.0, z))
    s1 = body("sphere", (0.2,), (1.5, 8.0, z), v=jitter())
    joint(JOINT_DISTANCE, a, s1, point_a=(0.0, 8.0, z), point_b=(1.5, 8.0, z))
    a = post((3.0, 8.0, z))
    s2 = body("sphere", (0.2,), (3.0, 7.0, z), v=(0.3, 0.0, 0.0))
    joint(JOINT_DISTANCE, a, s2, point_a=(3.0, 8.0, z), point_b=(3.0, 7.0, z), min_distance=0.5, max_distance=2.0)
    a = post((6.0, 8.0, z))
    s3 = body("sphere", (0.2,), (6.0, 6.7, z))
    joint(JOINT_DISTANCE, a, s3, point_a=(6.0, 8.0, z), point_b=(6.0, 6.7, z), min_distance=1.0, max_distance=1.0,
          spring={"mode": SPRING_STIFFNESS_AND_DAMPING, "frequency_or_stiffness": 2000.0, "damping": 0.0})
    # fixed: cantilever and a free welded pair
    z = 12.0
    a = post((0.0, 8.0, z))
    f1 = body("box", (0.4, 0.1, 0.1), (0.5, 8.0, z))
    f2 = body("box", (0.4, 0.1, 0.1), (1.5, 8.0, z))
    joint(JOINT_FIXED, a, f1, point_a=(0.0, 8.0, z), point_b=(0.0, 8.0, z))
    joint(JOINT_FIXED, f1, f2, point_a=(1.0, 8.0, z), point_b=(1.0, 8.0, z))
    spin = np.array([0.5, 1.0, 2.0])
    g1 = body("box", (0.3, 0.2, 0.1), (4.0, 8.0, z), v=(1.0, 2.0, 0.0), w=tuple(spin))
    # the second box moves with the first as one rigid body: v2 = v1 + w x (p2 - p1)
    v2 = np.array([1.0, 2.0, 0.0]) + np.cross(spin, np.array([0.5, 0.4, 0.0]))
    g2 = body("box", (0.2, 0.3, 0.1), (4.5, 8.4, z), v=tuple(v2), w=tuple(spin))
    joint(JOINT_FIXED, g1, g2, auto_detect_point=1)
    # cone: pendulums 20 degrees out, swinging outwards
    z = 16.0
    for c in range(2):
        x = 4.0 * c
        a = post((x, 8.0, z))
        ang = math.radians(20.0)
        d = (math.sin(ang), -math.cos(ang), 0.0) if c == 0 else (0.0, -math.cos(ang), math.sin(ang))
        q = (0.0, 0.0, math.sin(ang / 2), math.cos(ang / 2)) if c == 0 else (-math.sin(ang / 2), 0.0, 0.0, math.cos(ang / 2))
        centre = (x + 0.8 * d[0], 8.0 + 0.8 * d[1], z + 0.8 * d[2])
        sp = 3.0
        v = (sp * math.cos(ang), sp * math.sin(ang), 0.0) if c == 0 else (0.0, sp * math.sin(ang), sp * math.cos(ang))
        k = body("capsule", (0.1, 0.6), centre, q=q, v=v)
        joint(JOINT_CONE, a, k, point_a=(x, 8.0, z), point_b=(x, 8.0, z), twist_axis_a=(0.0, -1.0, 0.0),
              twist_axis_b=d, half_cone_angle=math.radians(30.0))
    # slider: incline with limits, velocity and position motors, friction, free pair
    z = 20.0
    a = post((0.0, 8.0, z))
    ax = (math.cos(math.radians(30.0)), -math.sin(math.radians(30.0)), 0.0)
    n_ax = (math.sin(math.radians(30.0)), math.cos(math.radians(30.0)), 0.0)
    b1 = body("box", (0.2, 0.2, 0.2), (0.0, 8.0, z))
    joint(JOINT_SLIDER, a, b1, point_a=(0.0, 8.0, z), point_b=(0.0, 8.0, z), slider_axis_a=ax, slider_axis_b=ax,
          normal_axis_a=n_ax, normal_axis_b=n_ax, limits_min=-1.0, limits_max=1.0)
    for i, (state, tv, tp) in enumerate(((1, 2.0, 0.0), (2, 0.0, 0.5))):
        a = post((6.0 + 6.0 * i, 8.0, z))
        bm = body("box", (0.2, 0.2, 0.2), (6.0 + 6.0 * i, 8.0, z))
        joint(JOINT_SLIDER, a, bm, point_a=(6.0 + 6.0 * i, 8.0, z), point_b=(6.0 + 6.0 * i, 8.0, z),
              slider_axis_a=(1.0, 0.0, 0.0), slider_axis_b=(1.0, 0.0, 0.0),
              normal_axis_a=(0.0, 1.0, 0.0), normal_axis_b=(0.0, 1.0, 0.0), motor_state=state, target_velocity=tv,
              target_position=tp)
    a = post((18.0, 8.0, z))
    bf = body("box", (0.2, 0.2, 0.2), (18.0, 8.0, z), v=(3.0, 0.0, 0.0))
    joint(JOINT_SLIDER, a, bf, point_a=(18.0, 8.0, z), point_b=(18.0, 8.0, z), slider_axis_a=(1.0, 0.0, 0.0),
          slider_axis_b=(1.0, 0.0, 0.0),
          normal_axis_a=(0.0, 1.0, 0.0), normal_axis_b=(0.0, 1.0, 0.0), max_friction_force=20.0)
    p1 = body("box", (0.3, 0.2, 0.2), (28.0, 8.0, z), v=(0.0, 1.0, 0.0), w=(0.0, 0.0, 1.0))
    p2 = body("box", (0.2, 0.2, 0.2), (29.0, 8.0, z), v=(2.0, 1.0, 0.0), w=(0.0, 0.0, 1.0))
    joint(JOINT_SLIDER, p1, p2, slider_axis_a=(1.0, 0.0, 0.0), slider_axis_b=(1.0, 0.0, 0.0),
          normal_axis_a=(0.0, 1.0, 0.0), normal_axis_b=(0.0, 1.0, 0.0), auto_detect_point=1)

    b = blank_bodies(len(rows))
    for i, (shape, params, pos, q, static, v, w) in enumerate(rows):
        if shape == "box":
            set_box(b, i, params)
        elif shape == "sphere":
            set_sphere(b, i, params[0])
        else:
            set_capsule(b, i, params[0], params[1])
        b["position"][i] = pos
        b["quaternion"][i] = q
        b["linear_velocity"][i] = v
        b["angular_velocity"][i] = w
        if static:
            b["motion_type"][i] = STATIC
            b["object_layer"][i] = LAYER_NOT_MOVING
    b["linear_damping"] = 0.0
    b["angular_damping"] = 0.0
    b["allow_sleeping"][:] = 0
    joints = {t: np.array(r, dtype=joint_defaults(t, 0).dtype) for t, r in J.items()}
    return Scene("joint_zoo", b, dt=1.0 / 60.0, steps=120, seed=seed, joints=joints, skip_joint_pairs=True)


def six_dof_zoo(seed: int = 93) -> Scene:
    """One world of six-DOF joint configurations (src/constraints/six-dof-constraint.ts), each
    on its own static post, 4 m apart in Z; joined bodies do not collide.  Constraint frames
    are given in world space with the bodies unrotated, so every joint starts at its rest pose:

    * locked: all six axes fixed, a 1 m cantilever box (a weld);
    * ball: translations fixed, rotations free, a capsule pendulum pushed at 3 m/s;
    * cone: translations fixed, twist free, swing cone of 30 degrees, the same push;
    * pyramid: translations fixed, twist +-10 degrees, swing Y +-20 and Z +-40 degrees, two
      pendulums pushed across each swing axis (X twist points down, Y along world X, Z along
      world Z: a push along world X swings about Z, one along world Z about Y);
    * prismatic: X limited to [-1, 1] m along a 30 degree incline, everything else fixed;
    * translation motors along free X: velocity 2 m/s, position 0.5 m;
    * rotation motors about free X (Y, Z rotation and translations fixed, pivot at the centre of
      mass): velocity 3 rad/s, position 45 degrees of twist;
    * friction: free X with 20 N of friction, box launched at 3 m/s;
    * soft limit: Y limited to [-0.1, 0.1] m with a 2 Hz / 0.5 damping limit spring, hanging;
    * a free pair of boxes welded by all six axes, thrown spinning."""
    rng = np.random.Generator(np.random.PCG64(seed))
    rows = []

    def body(shape, params, pos, static=False, v=(0.0, 0.0, 0.0), w=(0.0, 0.0, 0.0)):
        rows.append((shape, params, pos, static, v, w))
        return len(rows) - 1

    def post(pos):
        return body("box", (0.1, 0.1, 0.1), pos, static=True)

    recs = []
    INF, PI = float("inf"), math.pi
    FREE_MIN, FREE_MAX = (-INF, -INF, -INF, -PI, -PI, -PI), (INF, INF, INF, PI, PI, PI)

    def joint(a, b, pos_a, pos_b=None, lmin=FREE_MIN, lmax=FREE_MAX, **f):
        r = joint_defaults(JOINT_SIX_DOF, 1)[0]
        r["body_a"], r["body_b"] = a, b
        r["position_a"] = pos_a
        r["position_b"] = pos_a if pos_b is None else pos_b
        r["limit_min"], r["limit_max"] = lmin, lmax
        for k, v in f.items():
            if isinstance(v, dict):
                for kk, vv in v.items():
                    r[k][kk] = vv
            else:
                r[k] = v
        recs.append(r)

    zero6 = (0.0,) * 6
    down = dict(axis_x_a=(0.0, -1.0, 0.0), axis_y_a=(1.0, 0.0, 0.0), axis_x_b=(0.0, -1.0, 0.0),
                axis_y_b=(1.0, 0.0, 0.0))
    jit = lambda: float(rng.uniform(-0.05, 0.05))
    # locked cantilever
    a = post((0.0, 8.0, 0.0))
    c = body("box", (0.4, 0.1, 0.1), (0.5, 8.0, 0.0))
    joint(a, c, (0.0, 8.0, 0.0), lmin=zero6, lmax=zero6)
    # ball, cone, pyramid pendulums: capsule centres 0.8 m below their pivots
    specs = [(4.0, (0.0, 0.0, 0.0, -PI, -PI, -PI), (0.0, 0.0, 0.0, PI, PI, PI), 0, (3.0, 0.0, jit())),
             (8.0, (0.0, 0.0, 0.0, -PI, -math.radians(30), -math.radians(30)),
              (0.0, 0.0, 0.0, PI, math.radians(30), math.radians(30)), 0, (3.0, 0.0, jit())),
             (12.0, (0.0, 0.0, 0.0, -math.radians(10), -math.radians(20), -math.radians(40)),
              (0.0, 0.0, 0.0, math.radians(10), math.radians(20), math.radians(40)), 1, (3.0, 0.0, 0.0)),
             (12.0, (0.0, 0.0, 0.0, -math.radians(10), -math.radians(20), -math.radians(40)),
              (0.0, 0.0, 0.0, math.radians(10), math.radians(20), math.radians(40)), 1, (0.0, 0.0, 3.0))]
    for k, (z, lmin, lmax, swing, v) in enumerate(specs):
        x = 4.0 * k
        a = post((x, 8.0, z))
        p = body("capsule", (0.1, 0.6), (x, 7.2, z), v=v)
        joint(a, p, (x, 8.0, z), lmin=lmin, lmax=lmax, swing_type=swing, **down)
    # prismatic incline: X along the incline (downhill), Y its normal
    z = 16.0
    ax = (math.cos(math.radians(30.0)), -math.sin(math.radians(30.0)), 0.0)
    n_ax = (math.sin(math.radians(30.0)), math.cos(math.radians(30.0)), 0.0)
    a = post((0.0, 8.0, z))
    b1 = body("box", (0.2, 0.2, 0.2), (0.0, 8.0, z))
    joint(a, b1, (0.0, 8.0, z), lmin=(-1.0,) + zero6[1:], lmax=(1.0,) + zero6[1:], axis_x_a=ax, axis_y_a=n_ax,
          axis_x_b=ax, axis_y_b=n_ax)
    # translation motors along free X
    z = 20.0
    for i, (state, tv, tp) in enumerate(((1, 2.0, 0.0), (2, 0.0, 0.5))):
        x = 6.0 * i
        a = post((x, 8.0, z))
        bm = body("box", (0.2, 0.2, 0.2), (x, 8.0, z))
        ms = [0] * 6
        ms[0] = state
        joint(a, bm, (x, 8.0, z), lmin=(-INF,) + zero6[1:], lmax=(INF,) + zero6[1:], motor_state=ms,
              target_velocity=(tv, 0.0, 0.0), target_position=(tp, 0.0, 0.0))
    # rotation motors about free X
    for i, state in enumerate((1, 2)):
        x = 12.0 + 6.0 * i
        a = post((x, 8.0, z))
        bm = body("box", (0.3, 0.2, 0.1), (x, 8.0, z))
        ms = [0] * 6
        ms[3] = state
        h = math.radians(45.0) / 2
        joint(a, bm, (x, 8.0, z), lmin=zero6[:3] + (-PI, 0.0, 0.0), lmax=zero6[:3] + (PI, 0.0, 0.0), motor_state=ms,
              target_angular_velocity=(3.0, 0.0, 0.0), target_orientation=(math.sin(h), 0.0, 0.0, math.cos(h)))
    # friction along free X
    z = 24.0
    a = post((0.0, 8.0, z))
    bf = body("box", (0.2, 0.2, 0.2), (0.0, 8.0, z), v=(3.0, 0.0, 0.0))
    joint(a, bf, (0.0, 8.0, z), lmin=(-INF,) + zero6[1:], lmax=(INF,) + zero6[1:],
          max_friction=(20.0, 0.0, 0.0, 0.0, 0.0, 0.0))
    # soft limit on Y (up)
    a = post((6.0, 8.0, z))
    bs = body("box", (0.2, 0.2, 0.2), (6.0, 8.0, z))
    sp = np.zeros(3, dtype=SPRING_DTYPE)
    sp[1] = (SPRING_FREQUENCY_AND_DAMPING, 2.0, 0.5)
    joint(a, bs, (6.0, 8.0, z), lmin=(0.0, -0.1, 0.0, 0.0, 0.0, 0.0), lmax=(0.0, 0.1, 0.0, 0.0, 0.0, 0.0),
          limits_spring=sp)
    # free welded pair
    z = 28.0
    spin = np.array([0.5, 1.0, 2.0])
    g1 = body("box", (0.3, 0.2, 0.1), (4.0, 8.0, z), v=(1.0, 2.0, 0.0), w=tuple(spin))
    v2 = np.array([1.0, 2.0, 0.0]) + np.cross(spin, np.array([0.5, 0.4, 0.0]))
    g2 = body("box", (0.2, 0.3, 0.1), (4.5, 8.4, z), v=tuple(v2), w=tuple(spin))
    joint(g1, g2, (4.25, 8.2, z), lmin=zero6, lmax=zero6)

    b = blank_bodies(len(rows))
    for i, (shape, params, pos, static, v, w) in enumerate(rows):
        if shape == "box":
            set_box(b, i, params)
        else:
            set_capsule(b, i, params[0], params[1])
        b["position"][i] = pos
        b["linear_velocity"][i] = v
        b["angular_velocity"][i] = w
        if static:
            b["motion_type"][i] = STATIC
            b["object_layer"][i] = LAYER_NOT_MOVING
    b["linear_damping"] = 0.0
    b["angular_damping"] = 0.0
    b["allow_sleeping"][:] = 0
    joints = {JOINT_SIX_DOF: np.array(recs, dtype=joint_defaults(JOINT_SIX_DOF, 0).dtype)}
    return Scene("six_dof_zoo", b, dt=1.0 / 60.0, steps=120, seed=seed, joints=joints, skip_joint_pairs=True)


def decorated_pile(n: int = 120, seed: int = 6, extent: float = 4.0, heights=(0.5, 4.0), grid: float = 0.0) -> Scene:
    """n decorated convex bodies (src/shapes/transformed.ts, scaled.ts, offset-center-of-mass.ts)
    dropped on a static box floor, a seeded mix of: a box rotated and shifted in its body frame
    (TransformedShape); a non-uniformly scaled box (ScaledShape); a uniformly scaled sphere; a
    capsule laid along X by its transform; a box with its centre of mass moved off its middle
    (OffsetCenterOfMassShape); a scaled box that is also transformed and offset; a cylinder
    (src/shapes/cylinder.ts); and a uniformly scaled cylinder laid on its side.  Random
    orientations, drop heights in ``heights``, positions within +-``extent`` in X and Z, or with
    ``grid`` > 0 on a square grid of that spacing (bodies that never touch one another)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = blank_bodies(n + 1)
    set_box(b, 0, (50.0, 0.5, 50.0))
    b["motion_type"][0] = STATIC
    b["object_layer"][0] = LAYER_NOT_MOVING
    b["position"][0] = (0.0, -0.5, 0.0)

    def rand_quat():
        q = rng.normal(size=4)
        return q / np.linalg.norm(q)

    for i in range(1, n + 1):
        kind = int(rng.integers(0, 8))
        if kind in (6, 7):  # cylinders: plain, and laid on their side by the transform, scaled
            set_cylinder(b, i, float(rng.uniform(0.15, 0.35)), float(rng.uniform(0.15, 0.3)))
            if kind == 7:
                b["shape_quaternion"][i] = (math.sin(math.pi / 4), 0.0, 0.0, math.cos(math.pi / 4))
                b["shape_scale"][i] = float(rng.uniform(0.8, 1.3))
        elif kind in (0, 4, 5):
            set_box(b, i, tuple(rng.uniform(0.15, 0.4, 3)))
        elif kind == 1:
            set_box(b, i, (0.25, 0.25, 0.25))
        elif kind == 2:
            set_sphere(b, i, float(rng.uniform(0.15, 0.3)))
        else:
            set_capsule(b, i, float(rng.uniform(0.1, 0.2)), float(rng.uniform(0.2, 0.4)))
        if kind in (0, 5):
            b["shape_position"][i] = rng.uniform(-0.2, 0.2, 3)
            b["shape_quaternion"][i] = rand_quat()
        if kind == 1:
            b["shape_scale"][i] = rng.uniform(0.6, 1.8, 3)
        if kind == 2:
            b["shape_scale"][i] = float(rng.uniform(0.7, 1.5))
        if kind == 3:
            b["shape_quaternion"][i] = (0.0, 0.0, math.sin(math.pi / 4), math.cos(math.pi / 4))
        if kind in (4, 5):
            b["com_offset"][i] = rng.uniform(-0.1, 0.1, 3)
        if kind == 5:
            b["shape_scale"][i] = rng.uniform(0.7, 1.3, 3)
        b["position"][i] = (rng.uniform(-extent, extent), rng.uniform(*heights), rng.uniform(-extent, extent))
        if grid > 0:
            side = int(math.ceil(math.sqrt(n)))
            b["position"][i, 0] = grid * ((i - 1) % side)
            b["position"][i, 2] = grid * ((i - 1) // side)
        b["quaternion"][i] = rand_quat()
    return Scene("decorated_pile", b, dt=1.0 / 60.0, steps=120, seed=seed)


def plane_drop(n: int = 40, seed: int = 9, grid: float = 0.0) -> Scene:
    """n convex bodies (boxes, spheres, capsules, cylinders; a third of them with a given mass,
    src/body/rigid-body.ts:309-326) dropped onto a static plane shape (src/shapes/plane.ts)
    tilted 10 degrees about Z, with a static empty-shape body (empty-shape.ts) among them that
    nothing collides with.  Positions within +-3 m in X and Z (or on a ``grid``-spaced square),
    heights 0.5 to 2.5 m above the plane."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = blank_bodies(n + 2)
    tilt = math.radians(10.0)
    set_plane(b, 0, (-math.sin(tilt), math.cos(tilt), 0.0), 0.0)
    b["motion_type"][0] = STATIC
    b["object_layer"][0] = LAYER_NOT_MOVING
    set_empty(b, 1)
    b["motion_type"][1] = STATIC
    b["object_layer"][1] = LAYER_NOT_MOVING
    b["position"][1] = (0.0, 1.0, 0.0)
    side = int(math.ceil(math.sqrt(n)))
    for i in range(2, n + 2):
        kind = int(rng.integers(0, 4))
        if kind == 0:
            set_box(b, i, tuple(rng.uniform(0.15, 0.35, 3)))
        elif kind == 1:
            set_sphere(b, i, float(rng.uniform(0.15, 0.3)))
        elif kind == 2:
            set_capsule(b, i, float(rng.uniform(0.1, 0.2)), float(rng.uniform(0.2, 0.4)))
        else:
            set_cylinder(b, i, float(rng.uniform(0.15, 0.3)), float(rng.uniform(0.15, 0.3)))
        if i % 3 == 0:
            b["mass_properties_mode"][i] = 1
            b["mass"][i] = float(rng.uniform(5.0, 50.0))
        x, z = rng.uniform(-3.0, 3.0), rng.uniform(-3.0, 3.0)
        if grid > 0:
            x, z = grid * ((i - 2) % side) - grid * side / 2, grid * ((i - 2) // side) - grid * side / 2
        b["position"][i] = (x, x * math.tan(tilt) + rng.uniform(0.5, 2.5), z)
        q = rng.normal(size=4)
        b["quaternion"][i] = q / np.linalg.norm(q)
    return Scene("plane_drop", b, dt=1.0 / 60.0, steps=120, seed=seed)
