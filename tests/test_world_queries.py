"""World ray queries: castRay (src/query.ts:78-90) with the closest-hit collector
(createClosestCastRayCollector, src/collision/cast-ray-vs-shape.ts:180-205).

Known answers (CPU, the oracle): the cases of tst/query.test.ts (a unit box hit from -5 along +x
at fraction 0.4 of 10, missed from 5 above), tst/collision/cast-ray-vs-shape.test.ts (a unit
sphere 5 along +x hit at 4 of 1000; the ray offset by 0.1 still hits; single triangles hit from
the front, missed from behind and when parallel; of two stacked triangles the nearer is kept) and
tst/collision/cast-ray-treat-convex-as-solid.test.ts (a ray starting inside a sphere, box or
capsule hits at fraction 0 when convex shapes are solid and not at all otherwise; from 3 m outside
a unit sphere it hits at (3 - 1) / 10 = 0.2).  The reference asserts most of these as ranges; the
exact values follow from the geometry and are asserted to the GJK tolerance (1e-3 m along the ray).

mathcat's raycast3.intersectsTriangle is not vendored with the reference; both sides take it as
the Moller-Trumbore test over [0, length] with back faces culled unless asked, so the triangle
cases pin the mesh walk and the culling rule, not the library's own arithmetic.

GPU tolerances (FP32 device, FP64 oracle, the same poses):
  * the known answers: the same hit or miss, fraction within 2e-6 of length 1000 (1e-4 of 10);
  * 4,096 random rays through a terrain with a mixed pile: the same body for at least 99 % of
    rays (grazing rays and near-ties may go either way in FP32), fraction within 1e-4 where the
    bodies agree, the same triangle sub-shape id for at least 99 % of mesh hits;
  * filters and worlds: bit-exact selection (a layer or group that excludes a body never hits
    it; a ray of world k only hits bodies of world k).
"""
import math

import numpy as np
import pytest

from crashcat_gb300 import _lib, scenes, world
from oracle import pyoracle


def ray(o, d, length):
    d = np.asarray(d, np.float64)
    d = d / np.linalg.norm(d)
    return [*o, *d, length]


def one_body(kind, pos=(0.0, 0.0, 0.0), **kw):
    b = scenes.blank_bodies(1)
    if kind == "sphere":
        scenes.set_sphere(b, 0, kw.get("radius", 1.0))
    elif kind == "box":
        scenes.set_box(b, 0, kw.get("half", (1.0, 1.0, 1.0)))
    elif kind == "capsule":
        scenes.set_capsule(b, 0, kw.get("radius", 0.5), kw.get("half_height", 1.0))
    b["position"][0] = pos
    b["motion_type"][0] = _lib.STATIC
    b["object_layer"][0] = scenes.LAYER_NOT_MOVING
    return b


def mesh_body():
    b = scenes.blank_bodies(1)
    b["shape_type"][0] = _lib.SHAPE_TRIANGLE_MESH
    b["shape_params"][0] = 0.0
    b["motion_type"][0] = _lib.STATIC
    b["object_layer"][0] = scenes.LAYER_NOT_MOVING
    return b


# (name, body kind, body position, ray, solid, expected fraction or None for a miss)
CONVEX_CASES = [
    ("query_box_hit", "box", (0, 0, 0), ray((-5, 0, 0), (1, 0, 0), 10), True, 0.4),
    ("query_box_miss_above", "box", (0, 0, 0), ray((-5, 5, 0), (1, 0, 0), 10), True, None),
    ("sphere_from_outside", "sphere", (5, 0, 0), ray((0, 0, 0), (1, 0, 0), 1000), True, 0.004),
    ("sphere_offset_ray", "sphere", (5, 0, 0), ray((0, -0.1, 0), (1, 0, 0), 1000), True,
     (5 - math.sqrt(1 - 0.01)) / 1000),
    ("sphere_example_case", "sphere", (2, 0.044676984915871, 0), ray((-3, 0, 0), (1, 0, 0), 10), True,
     (5 - math.sqrt(1 - 0.044676984915871 ** 2)) / 10),
    ("sphere_miss_side", "sphere", (5, 0, 0), ray((0, 2, 0), (1, 0, 0), 1000), True, None),
    ("box_pointing_away", "box", (5, 0, 0), ray((0, 0, 0), (-1, 0, 0), 1000), True, None),
    ("solid_sphere_inside", "sphere", (0, 0, 0), ray((0, 0, 0), (1, 0, 0), 10), True, 0.0),
    ("hollow_sphere_inside", "sphere", (0, 0, 0), ray((0, 0, 0), (1, 0, 0), 10), False, None),
    ("solid_sphere_outside", "sphere", (0, 0, 0), ray((-3, 0, 0), (1, 0, 0), 10), True, 0.2),
    ("hollow_sphere_outside", "sphere", (0, 0, 0), ray((-3, 0, 0), (1, 0, 0), 10), False, 0.2),
    ("solid_box_inside", "box", (0, 0, 0), ray((0, 0, 0), (1, 0, 0), 10), True, 0.0),
    ("hollow_box_inside", "box", (0, 0, 0), ray((0, 0, 0), (1, 0, 0), 10), False, None),
    ("solid_capsule_inside", "capsule", (0, 0, 0), ray((0, 0, 0), (1, 0, 0), 10), True, 0.0),
    ("hollow_capsule_inside", "capsule", (0, 0, 0), ray((0, 0, 0), (1, 0, 0), 10), False, None),
]

TRI = [0, 0, 0, 1, 0, 0, 0, 1, 0]
# (name, positions, indices, ray, expected fraction or None, the hit triangle's z)
MESH_CASES = [
    ("triangle_front", TRI, [0, 2, 1], ray((0.2, 0.2, -1), (0, 0, 1), 1000), 0.001, 0.0),
    ("triangle_behind", TRI, [0, 1, 2], ray((0.2, 0.2, 1), (0, 0, 1), 1000), None, None),
    ("triangle_parallel", TRI, [0, 1, 2], ray((0.2, 0.2, 1), (1, 0, 0), 1000), None, None),
    ("two_triangles_nearest", TRI + [0, 0, 1, 1, 0, 1, 0, 1, 1], [0, 2, 1, 3, 5, 4],
     ray((0.2, 0.2, -1), (0, 0, 1), 1000), 0.001, 0.0),
    ("two_triangles_from_above", TRI + [0, 0, 1, 1, 0, 1, 0, 1, 1], [0, 1, 2, 3, 4, 5],
     ray((0.2, 0.2, 3), (0, 0, -1), 1000), 0.002, 1.0),
]


def oracle_single(bodies, mesh=None):
    return pyoracle.OracleWorld(world.standard_settings(), bodies, (), [mesh] if mesh is not None else ())


@pytest.mark.parametrize("case", CONVEX_CASES, ids=[c[0] for c in CONVEX_CASES])
def test_oracle_convex_known_answers(oracle_lib, case):
    _, kind, pos, r, solid, want = case
    o = oracle_single(one_body(kind, pos))
    fr, bo, su = o.cast_rays(np.array([r]), treat_convex_as_solid=solid)
    if want is None:
        assert bo[0] == -1
    else:
        assert bo[0] == 0
        assert abs(fr[0] - want) <= 1e-3 / r[6] + 1e-12, (fr[0], want)
        assert su[0] == 0xFFFFFFFF


def mesh_triangle_z(m, sub):
    """z of the first vertex of the triangle a sub-shape id names (subShape.pushIndex
    sub-shape.ts:60-64: the index in the low bits(triangle count - 1) bits, ones above)."""
    bits = max(len(m["triangles"]) - 1, 0).bit_length()
    tri = int(sub) & ((1 << bits) - 1)
    assert (int(sub) | ((1 << bits) - 1)) == 0xFFFFFFFF
    return float(m["vertices"][m["triangles"][tri, 0], 2])


@pytest.mark.parametrize("case", MESH_CASES, ids=[c[0] for c in MESH_CASES])
def test_oracle_mesh_known_answers(gpu_lib, oracle_lib, case):
    _, p, idx, r, want, z = case
    m = _lib.build_triangle_mesh(np.array(p, np.float64).reshape(-1, 3), np.array(idx, np.int64).reshape(-1, 3))
    o = oracle_single(mesh_body(), m)
    fr, bo, su = o.cast_rays(np.array([r]))
    if want is None:
        assert bo[0] == -1
        return
    assert bo[0] == 0
    assert abs(fr[0] - want) < 1e-12
    assert mesh_triangle_z(m, su[0]) == z


def test_oracle_backfaces_culled(gpu_lib, oracle_lib):
    """Back faces are culled by default (createDefaultCastRaySettings collideWithBackfaces false;
    the mesh walk passes !collideWithBackfaces to intersectsTriangle, triangle-mesh.ts:366-373)."""
    m = _lib.build_triangle_mesh(np.array(TRI, np.float64).reshape(-1, 3), np.array([[0, 1, 2]]))
    o = oracle_single(mesh_body(), m)
    r = np.array([ray((0.2, 0.2, 1), (0, 0, -1), 10)])
    assert o.cast_rays(r)[1][0] == 0  # front face from +z: (1,0,0) x (0,1,0) points to +z
    r = np.array([ray((0.2, 0.2, -1), (0, 0, 1), 10)])
    assert o.cast_rays(r)[1][0] == -1


def test_oracle_closest_body_and_filters(oracle_lib):
    """Closest of several bodies along the ray; a body outside the filter is passed over."""
    b = scenes.blank_bodies(3)
    for i, x in enumerate((9.0, 3.0, 6.0)):
        scenes.set_sphere(b, i, 0.5)
        b["position"][i] = (x, 0, 0)
        b["motion_type"][i] = _lib.STATIC
        b["object_layer"][i] = scenes.LAYER_NOT_MOVING
    b["collision_groups"][1] = 2
    o = oracle_single(b)
    r = np.array([ray((0, 0, 0), (1, 0, 0), 20)])
    fr, bo, _ = o.cast_rays(r)
    assert bo[0] == 1 and abs(fr[0] - 2.5 / 20) < 1e-4
    fr, bo, _ = o.cast_rays(r, mask=~2 & 0xFFFFFFFF)
    assert bo[0] == 2 and abs(fr[0] - 5.5 / 20) < 1e-4
    fr, bo, _ = o.cast_rays(r, layer_mask=0)
    assert bo[0] == -1


# ---------------------------------------------------------------------------
# GPU against the oracle
# ---------------------------------------------------------------------------
@pytest.mark.gpu
def test_gpu_known_answers(gpu_lib, oracle_lib):
    for _, kind, pos, r, solid, want in CONVEX_CASES:
        g = world.GpuWorld(world.standard_settings(), 4)
        g.add_bodies(one_body(kind, pos))
        h = g.cast_rays(np.array([r]), treat_convex_as_solid=solid)
        if want is None:
            assert h["body"][0] == -1, (kind, r)
        else:
            assert h["body"][0] == 0, (kind, r)
            assert abs(float(h["fraction"][0]) - want) <= 2e-3 / r[6] + 2e-6, (kind, r, h["fraction"][0], want)
    for _, p, idx, r, want, z in MESH_CASES:
        pos = np.array(p, np.float64).reshape(-1, 3)
        ind = np.array(idx, np.int64).reshape(-1, 3)
        g = world.GpuWorld(world.standard_settings(), 4)
        g.add_triangle_mesh(pos, ind)
        g.add_bodies(mesh_body())
        h = g.cast_rays(np.array([r]))
        if want is None:
            assert h["body"][0] == -1
            continue
        assert h["body"][0] == 0
        assert abs(float(h["fraction"][0]) - want) < 1e-6
        assert mesh_triangle_z(g.get_triangle_mesh(0), h["sub_shape_id"][0]) == z
    # collideWithBackfaces: the triangle seen from behind counts when asked
    g = world.GpuWorld(world.standard_settings(), 4)
    g.add_triangle_mesh(np.array(TRI, np.float64).reshape(-1, 3), np.array([[0, 1, 2]]))
    g.add_bodies(mesh_body())
    r = np.array([ray((0.2, 0.2, -1), (0, 0, 1), 10)])
    assert g.cast_rays(r)["body"][0] == -1
    h = g.cast_rays(r, collide_with_backfaces=True)
    assert h["body"][0] == 0 and abs(float(h["fraction"][0]) - 0.1) < 1e-6


def random_rays(rng, n, half, top):
    o = np.stack([rng.uniform(-half, half, n), rng.uniform(top * 0.5, top, n), rng.uniform(-half, half, n)], 1)
    d = rng.normal(size=(n, 3))
    d[:, 1] = -np.abs(d[:, 1]) - 0.3
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o, d, rng.uniform(5.0, 30.0, (n, 1))], 1)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [5, 6])
def test_gpu_rays_through_terrain_pile(gpu_lib, oracle_lib, seed):
    sc = scenes.mesh_drop(n=120, n_cells=16, seed=seed, heights=(0.0, 3.0))
    ws = world.standard_settings()
    g = world.GpuWorld(ws, sc.n + 16)
    for p in sc.hull_points or ():
        g.add_convex_hull(p)
    g.add_triangle_mesh(*sc.mesh)
    g.add_bodies(sc.bodies)
    hulls = [g.get_convex_hull(i) for i in range(len(sc.hull_points or ()))]
    o = pyoracle.OracleWorld(ws, sc.bodies, hulls, [g.get_triangle_mesh(0)])
    g.step(sc.dt, 30)
    rows, _ = g.get_state()
    st = o.state()
    st[:, 0:13] = rows[:, 0:13]
    o.set_state(st)
    rng = np.random.default_rng(seed)
    rays = random_rays(rng, 4096, 7.0, 8.0)
    h = g.cast_rays(rays)
    fr, bo, su = o.cast_rays(rays)
    same = h["body"] == bo
    assert same.mean() >= 0.99, same.mean()
    assert (bo >= 0).sum() > 2000  # most rays reach something
    hit = same & (bo >= 0)
    assert np.abs(h["fraction"][hit] - fr[hit]).max() < 1e-4
    mesh = hit & (bo == 0)
    assert mesh.sum() > 500
    assert (h["sub_shape_id"][mesh] == su[mesh]).mean() >= 0.99
    # a filter that leaves out the static layer never hits the terrain
    h2 = g.cast_rays(rays, object_layer_mask=~(1 << scenes.LAYER_NOT_MOVING) & 0xFFFFFFFF)
    assert not (h2["body"] == 0).any()
    fr2, bo2, _ = o.cast_rays(rays, layer_mask=~(1 << scenes.LAYER_NOT_MOVING) & 0xFFFFFFFF)
    assert (h2["body"] == bo2).mean() >= 0.99


@pytest.mark.gpu
def test_gpu_rays_stay_in_their_world(gpu_lib, oracle_lib):
    """Worlds share the device tree; a ray only meets bodies of its own world.  Every world holds
    the same spheres shifted by the world index along z, so a ray of world k hits body k * 4 + j."""
    nw, per = 64, 4
    b = scenes.blank_bodies(nw * per)
    for k in range(nw):
        for j in range(per):
            i = k * per + j
            scenes.set_sphere(b, i, 0.4)
            b["position"][i] = (2.0 * j + 2.0, 0.0, 0.0)
            b["motion_type"][i] = _lib.STATIC
            b["object_layer"][i] = scenes.LAYER_NOT_MOVING
            b["world"][i] = k
    ws = world.standard_settings()
    ws.num_worlds = nw
    g = world.GpuWorld(ws, nw * per)
    g.add_bodies(b)
    rays = np.zeros((nw, 8))
    rays[:, 3] = 1.0
    rays[:, 6] = 20.0
    rays[:, 7] = np.arange(nw)
    h = g.cast_rays(rays)
    np.testing.assert_array_equal(h["body"], np.arange(nw) * per)
    np.testing.assert_allclose(h["fraction"], 1.6 / 20.0, atol=1e-4)


@pytest.mark.gpu
def test_gpu_shape_casts_stay_in_their_world(gpu_lib):
    """Worlds share the device tree; a shape cast only meets bodies of its own world.  Every world
    of 64 holds the same spheres, so the sphere cast of world k hits body k * 4; a terrain mesh in
    world 0 is hit by a cast down from world 0 and missed by the same cast from a world without
    bodies, as are the spheres.  No tree walk outgrows its stack (the call would return
    CC_ERR_CAPACITY)."""
    nw, per = 64, 4
    sc = scenes.mesh_drop(n=1, n_cells=12, seed=5, heights=(0.0, 1.0))
    b = scenes.blank_bodies(nw * per)
    for k in range(nw):
        for j in range(per):
            i = k * per + j
            scenes.set_sphere(b, i, 0.4)
            b["position"][i] = (2.0 * j + 2.0, 5.0, 0.0)
            b["motion_type"][i] = _lib.STATIC
            b["object_layer"][i] = scenes.LAYER_NOT_MOVING
            b["world"][i] = k
    terrain = sc.bodies[:1].copy()
    terrain["world"][0] = 0
    bodies = np.concatenate([b, terrain])
    ws = world.standard_settings()
    ws.num_worlds = nw + 1  # the last world has no bodies
    g = world.GpuWorld(ws, len(bodies))
    g.add_triangle_mesh(*sc.mesh)
    g.add_bodies(bodies)
    casts = np.zeros(nw + 3, _lib.SHAPE_CAST_DTYPE)
    casts["shape_type"] = _lib.SHAPE_SPHERE
    casts["shape_params"][:, 0] = 0.2
    casts["quaternion"][:, 3] = 1.0
    casts["position"][:nw] = (0.0, 5.0, 0.0)
    casts["displacement"][:nw] = (20.0, 0.0, 0.0)
    casts["world"][:nw] = np.arange(nw)
    casts["position"][nw:] = [(0.0, 5.0, 0.0), (0.5, 4.0, 0.5), (0.5, 4.0, 0.5)]
    casts["displacement"][nw:] = [(20.0, 0.0, 0.0), (0.0, -8.0, 0.0), (0.0, -8.0, 0.0)]
    casts["world"][nw:] = [nw, 0, nw]
    h = g.cast_shapes(casts)
    np.testing.assert_array_equal(h["body"][:nw], np.arange(nw) * per)
    np.testing.assert_allclose(h["fraction"][:nw], 1.4 / 20.0, atol=1e-4)
    assert h["body"][nw] == -1 and h["body"][nw + 2] == -1
    assert h["body"][nw + 1] == nw * per and 0.0 < h["fraction"][nw + 1] < 1.0


# ---------------------------------------------------------------------------
# collidePoint (query.ts:470-490): the reference's known answers
# (tst/query.test.ts collidePoint, tst/collision/collide-point-vs-shape.test.ts)
# ---------------------------------------------------------------------------
Q45Y = (0.0, math.sin(math.pi / 8), 0.0, math.cos(math.pi / 8))  # 45 degrees about +Y
# (name, body kind, kwargs, body position, quaternion, point, inside)
POINT_CASES = [
    ("query_box_inside", "box", {}, (0, 0, 0), None, (0.5, 0.5, 0.5), True),
    ("query_box_outside", "box", {}, (0, 0, 0), None, (5, 5, 5), False),
    ("sphere_centre", "sphere", {}, (0, 0, 0), None, (0, 0, 0), True),
    ("sphere_translated", "sphere", {}, (5, 3, -2), None, (5, 3, -2), True),
    ("sphere_surface", "sphere", {}, (0, 0, 0), None, (1, 0, 0), True),
    ("sphere_outside", "sphere", {}, (0, 0, 0), None, (2, 0, 0), False),
    ("sphere_outside_unscaled", "sphere", {}, (0, 0, 0), None, (1.5, 0, 0), False),
    ("box_centre", "box", {}, (0, 0, 0), None, (0, 0, 0), True),
    ("box_off_centre", "box", {"half": (2, 2, 2)}, (0, 0, 0), None, (1, 1, 1), True),
    ("box_face", "box", {}, (0, 0, 0), None, (1, 0, 0), True),
    ("box_corner", "box", {}, (0, 0, 0), None, (1, 1, 1), True),
    ("box_outside", "box", {}, (0, 0, 0), None, (2, 0, 0), False),
    ("box_rotated_45", "box", {}, (0, 0, 0), Q45Y, (1.4, 0, 0), True),
    ("box_rotated_inside", "box", {}, (0, 0, 0), Q45Y, (0.5, 0, 0), True),
    ("box_translated", "box", {}, (5, 3, -2), None, (5, 3, -2), True),
    ("box_translated_rotated", "box", {}, (10, 5, 3), Q45Y, (11, 5, 3), True),
    ("capsule_cap_inside", "capsule", {}, (0, 0, 0), None, (0, 1.4, 0), True),
    ("capsule_cap_outside", "capsule", {}, (0, 0, 0), None, (0, 1.6, 0), False),
    ("capsule_side_inside", "capsule", {}, (0, 0, 0), None, (0.45, 0, 0), True),
    ("capsule_side_outside", "capsule", {}, (0, 0, 0), None, (0.55, 0, 0), False),
]

CUBE_INDICES = [0, 1, 3, 0, 3, 2, 4, 7, 5, 4, 6, 7, 2, 3, 6, 3, 7, 6, 1, 0, 4, 1, 4, 5, 1, 7, 3, 1, 5, 7, 0, 2, 6,
                0, 6, 4]


def randomized_cube(seed=7):
    """The test's cube with each corner scaled by 0.1-0.3 per axis (seeded here)."""
    rng = np.random.default_rng(seed)
    base = np.array([[x, y, z] for y in (-1.0, 1.0) for z in (-1.0, 1.0) for x in (-1.0, 1.0)])
    return base * rng.uniform(0.1, 0.3, (8, 3))


# (name, mesh body position, point, inside)
MESH_POINT_CASES = [
    ("cube_centre", (0, 0, 0), (0, 0, 0), True),
    ("cube_far_outside", (0, 0, 0), (5, 0, 0), False),
    ("cube_translated", (10, 5, 3), (10, 5, 3), True),
]


@pytest.mark.parametrize("case", POINT_CASES, ids=[c[0] for c in POINT_CASES])
def test_oracle_point_known_answers(oracle_lib, case):
    _, kind, kw, pos, q, p, inside = case
    b = one_body(kind, pos, **kw)
    if q is not None:
        b["quaternion"][0] = q
    co, bo, su = oracle_single(b).collide_points(np.array([p], np.float64))
    assert (co[0] == 1) == inside and (bo[0] == 0) == inside
    assert su[0] == 0xFFFFFFFF


@pytest.mark.parametrize("case", MESH_POINT_CASES, ids=[c[0] for c in MESH_POINT_CASES])
def test_oracle_mesh_point_known_answers(gpu_lib, oracle_lib, case):
    _, pos, p, inside = case
    m = _lib.build_triangle_mesh(randomized_cube(), np.array(CUBE_INDICES).reshape(-1, 3))
    b = mesh_body()
    b["position"][0] = pos
    co, bo, su = oracle_single(b, m).collide_points(np.array([p], np.float64))
    assert (co[0] == 1) == inside
    if inside:
        assert su[0] != 0xFFFFFFFF  # the last triangle the +Y ray met


@pytest.mark.gpu
def test_gpu_point_known_answers(gpu_lib, oracle_lib):
    for _, kind, kw, pos, q, p, inside in POINT_CASES:
        b = one_body(kind, pos, **kw)
        if q is not None:
            b["quaternion"][0] = q
        g = world.GpuWorld(world.standard_settings(), 4)
        g.add_bodies(b)
        h = g.collide_points(np.array([p], np.float64))
        assert (h["count"][0] == 1) == inside, (kind, p)
        assert (h["body"][0] == 0) == inside
    m_pos, m_idx = randomized_cube(), np.array(CUBE_INDICES).reshape(-1, 3)
    for _, pos, p, inside in MESH_POINT_CASES:
        g = world.GpuWorld(world.standard_settings(), 4)
        g.add_triangle_mesh(m_pos, m_idx)
        b = mesh_body()
        b["position"][0] = pos
        g.add_bodies(b)
        o = oracle_single(b, g.get_triangle_mesh(0))
        h = g.collide_points(np.array([p], np.float64))
        co, bo, su = o.collide_points(np.array([p], np.float64))
        assert (h["count"][0] == 1) == inside
        assert h["sub_shape_id"][0] == su[0]


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [5, 6])
def test_gpu_points_in_terrain_pile(gpu_lib, oracle_lib, seed):
    """Points scattered through a terrain pile: under the terrain (odd-even count of the open
    heightfield), in bodies, in several bodies, in none."""
    sc = scenes.mesh_drop(n=120, n_cells=16, seed=seed, heights=(0.0, 3.0))
    ws = world.standard_settings()
    g = world.GpuWorld(ws, sc.n + 16)
    for p in sc.hull_points or ():
        g.add_convex_hull(p)
    g.add_triangle_mesh(*sc.mesh)
    g.add_bodies(sc.bodies)
    hulls = [g.get_convex_hull(i) for i in range(len(sc.hull_points or ()))]
    o = pyoracle.OracleWorld(ws, sc.bodies, hulls, [g.get_triangle_mesh(0)])
    g.step(sc.dt, 30)
    rows, _ = g.get_state()
    st = o.state()
    st[:, 0:13] = rows[:, 0:13]
    o.set_state(st)
    rng = np.random.default_rng(seed)
    # half of the points near body centres (inside something), half anywhere in the pile's box
    near = rows[rng.integers(1, sc.n, 4096), 0:3] + rng.normal(scale=0.3, size=(4096, 3))
    anywhere = np.stack([rng.uniform(-7, 7, 4096), rng.uniform(-3, 6, 4096), rng.uniform(-7, 7, 4096)], 1)
    pts = np.concatenate([near, anywhere])
    h = g.collide_points(pts)
    co, bo, su = o.collide_points(pts)
    assert (h["count"] == co).mean() >= 0.995
    assert (h["body"] == bo).mean() >= 0.995
    assert (co > 0).mean() > 0.25 and (bo == 0).sum() > 300 and (co > 1).sum() > 0
    mesh = (bo == 0) & (h["body"] == 0)
    assert (h["sub_shape_id"][mesh] == su[mesh]).mean() >= 0.99


# ---------------------------------------------------------------------------
# castShape (query.ts:196-214) with the closest-hit collector and the default cast settings
# ---------------------------------------------------------------------------
SHAPE_IDS = {"sphere": _lib.SHAPE_SPHERE, "box": _lib.SHAPE_BOX, "capsule": _lib.SHAPE_CAPSULE}


def cast_row(kind, params, pos, disp, q=(0.0, 0.0, 0.0, 1.0)):
    p = list(params) + [0.0] * (4 - len(params))
    return [SHAPE_IDS[kind], *p, *pos, *q, *disp]


def cast_array(rows, worlds=None):
    rows = np.asarray(rows, np.float64).reshape(-1, 15)
    c = np.zeros(len(rows), _lib.SHAPE_CAST_DTYPE)
    c["shape_type"] = rows[:, 0].astype(np.int32)
    c["shape_params"], c["position"] = rows[:, 1:5], rows[:, 5:8]
    c["quaternion"], c["displacement"] = rows[:, 8:12], rows[:, 12:15]
    c["world"] = 0 if worlds is None else worlds
    return c


# (name, cast kind, params, start, displacement, expected fraction or None): tst/query.test.ts's
# sphere sweeps against a unit box at the origin, and a box and a capsule swept the same way
SHAPE_CAST_CASES = [
    ("query_sphere_hits_box", "sphere", (0.5,), (-3, 0, 0), (6, 0, 0), 1.5 / 6),
    ("query_sphere_misses_box", "sphere", (0.5,), (-5, 5, 0), (10, 0, 0), None),
    ("box_hits_box", "box", (0.5, 0.5, 0.5, 0.05), (-4, 0, 0), (8, 0, 0), 2.5 / 8),
    ("capsule_hits_box_from_above", "capsule", (0.3, 0.5), (0, 5, 0), (0, -8, 0), 3.2 / 8),
    ("sphere_moving_away", "sphere", (0.5,), (-3, 0, 0), (-6, 0, 0), None),
]


@pytest.mark.parametrize("case", SHAPE_CAST_CASES, ids=[c[0] for c in SHAPE_CAST_CASES])
def test_oracle_shape_cast_known_answers(oracle_lib, case):
    _, kind, params, start, disp, want = case
    o = oracle_single(one_body("box"))
    out, bo = o.cast_shapes(np.array([cast_row(kind, params, start, disp)]))
    if want is None:
        assert bo[0] == -1
        return
    assert bo[0] == 0
    assert abs(out[0, 0] - want) < 2e-3 / np.linalg.norm(disp) + 1e-9, (out[0, 0], want)
    d = np.asarray(disp, np.float64) / np.linalg.norm(disp)
    np.testing.assert_allclose(out[0, 1:4], -d, atol=1e-3)  # the normal faces the cast back


@pytest.mark.gpu
def test_gpu_shape_cast_known_answers(gpu_lib, oracle_lib):
    for _, kind, params, start, disp, want in SHAPE_CAST_CASES:
        g = world.GpuWorld(world.standard_settings(), 4)
        g.add_bodies(one_body("box"))
        h = g.cast_shapes(cast_array([cast_row(kind, params, start, disp)]))
        if want is None:
            assert h["body"][0] == -1, kind
            continue
        assert h["body"][0] == 0, kind
        assert abs(float(h["fraction"][0]) - want) < 3e-3 / np.linalg.norm(disp), (kind, h["fraction"][0], want)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [5, 6])
def test_gpu_shape_casts_through_terrain_pile(gpu_lib, oracle_lib, seed):
    """Spheres, boxes and capsules swept down through a terrain pile, against the oracle at the
    same poses: the same body for at least 97 % of casts (FP32 and the casts' own tolerances,
    1e-4 m convex and 1e-2 m mesh, decide near-ties); where the bodies agree, 99 % of the hit
    distances within 2e-3 m and all within 0.1 m (a grazing cast can converge on another face in
    FP32: one cast of 1,024 was 0.07 m off)."""
    sc = scenes.mesh_drop(n=120, n_cells=16, seed=seed, heights=(0.0, 3.0))
    ws = world.standard_settings()
    g = world.GpuWorld(ws, sc.n + 16)
    for p in sc.hull_points or ():
        g.add_convex_hull(p)
    g.add_triangle_mesh(*sc.mesh)
    g.add_bodies(sc.bodies)
    hulls = [g.get_convex_hull(i) for i in range(len(sc.hull_points or ()))]
    o = pyoracle.OracleWorld(ws, sc.bodies, hulls, [g.get_triangle_mesh(0)])
    g.step(sc.dt, 30)
    rows, _ = g.get_state()
    st = o.state()
    st[:, 0:13] = rows[:, 0:13]
    o.set_state(st)
    rng = np.random.default_rng(seed)
    n = 1024
    kinds = rng.integers(0, 3, n)
    params = np.zeros((n, 4))
    params[kinds == 0, 0] = rng.uniform(0.1, 0.4, (kinds == 0).sum())
    params[kinds == 1, 0:3] = rng.uniform(0.1, 0.4, ((kinds == 1).sum(), 3))
    params[kinds == 1, 3] = 0.05
    params[kinds == 2, 0:2] = rng.uniform(0.1, 0.3, ((kinds == 2).sum(), 2))
    start = np.stack([rng.uniform(-6, 6, n), rng.uniform(7, 10, n), rng.uniform(-6, 6, n)], 1)
    disp = np.stack([rng.uniform(-2, 2, n), rng.uniform(-14, -10, n), rng.uniform(-2, 2, n)], 1)
    q = scenes.random_quaternions(rng, n)
    rows_ = np.concatenate([kinds[:, None], params, start, q, disp], 1)
    h = g.cast_shapes(cast_array(rows_))
    out, bo = o.cast_shapes(rows_)
    same = h["body"] == bo
    assert same.mean() >= 0.97, same.mean()
    assert (bo >= 0).mean() > 0.9 and (bo == 0).sum() > 100 and (bo > 0).sum() > 50
    hit = same & (bo >= 0)
    lens = np.linalg.norm(disp, axis=1)
    err = np.abs((h["fraction"][hit] - out[hit, 0]) * lens[hit])
    assert np.quantile(err, 0.99) < 2e-3 and err.max() < 0.1, (np.quantile(err, 0.99), err.max())
