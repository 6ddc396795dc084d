"""collideShape (src/query.ts:286-311) and the any-hit / all-hit collectors of the ray, shape-cast
and collide queries (src/collision/cast-ray-vs-shape.ts:66-156, cast-shape-vs-shape.ts:165-226,
collide-shape-vs-shape.ts:82-176).

Known answers (CPU, the oracle; exact from the geometry, to the GJK/EPA tolerances):
  * a sphere of 0.5 m centred 1.3 m from a unit box penetrates it by 0.2 m along -x (the axis
    points from the query shape into the body); 1.6 m away it misses, unless the separation
    distance is 0.2 m, when it hits with penetration -0.1 m;
  * a sphere of 0.5 m against a sphere of 1 m 1.2 m away: 0.3 m along +x;
  * a box of half extent 0.5 m centred 0.8 m inside a unit box (cores overlap: EPA): 0.7 m;
  * an upright capsule (radius 0.3 m, half height 0.5 m) whose bottom is 0.2 m into a unit box's
    top face: 0.2 m along -y; a box 0.2 m into a plane: 0.2 m;
  * a sphere of 0.5 m whose centre is 0.3 m above a single triangle: 0.2 m; from behind the
    triangle only when back faces count (the query default);
  * the all-hit ray collector through three spheres on a line returns the three in order of
    fraction; a filter removes exactly the filtered body.

GPU tolerances (the same poses; casts in FP32 on the device, collide queries in FP64 as the
oracle): the known answers within 1e-3 m; on a terrain pile the all-hit lists equal the oracle's
(the same bodies and sub-shape ids) for at least 97 % of queries (grazing contacts within the
tolerances may go either way); cast fractions of matched hits within 2e-3 m for 99 %; collide
penetrations within 1e-5 m for 95 % (EPA's early stop on a box through a triangle follows the
rounding, see the test); the closest collide hit is the oracle's deepest; the any-hit of every
query is one of the oracle's all-hit list.
"""
import numpy as np
import pytest

from crashcat_gb300 import _lib, scenes, world
from oracle import pyoracle

SPH, BOX, CAP = _lib.SHAPE_SPHERE, _lib.SHAPE_BOX, _lib.SHAPE_CAPSULE


def static_bodies(specs):
    """specs: (kind, params, position); static, not-moving layer."""
    b = scenes.blank_bodies(len(specs))
    for i, (kind, params, pos) in enumerate(specs):
        if kind == "sphere":
            scenes.set_sphere(b, i, params[0])
        elif kind == "box":
            scenes.set_box(b, i, params)
        elif kind == "capsule":
            scenes.set_capsule(b, i, params[0], params[1])
        elif kind == "plane":
            scenes.set_plane(b, i, (0.0, 1.0, 0.0), 0.0)
        b["position"][i] = pos
        b["motion_type"][i] = _lib.STATIC
        b["object_layer"][i] = scenes.LAYER_NOT_MOVING
    return b


def qrow(shape, params, pos, q=(0.0, 0.0, 0.0, 1.0)):
    p = list(params) + [0.0] * (4 - len(params))
    return [shape, *p, *pos, *q]


def qarray(rows, worlds=None):
    rows = np.asarray(rows, np.float64).reshape(-1, 12)
    c = np.zeros(len(rows), _lib.COLLIDE_SHAPE_DTYPE)
    c["shape_type"] = rows[:, 0].astype(np.int32)
    c["shape_params"], c["position"], c["quaternion"] = rows[:, 1:5], rows[:, 5:8], rows[:, 8:12]
    c["world"] = 0 if worlds is None else worlds
    return c


TRI = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float64)

# (name, bodies, query row, max separation, expected penetration or None, expected axis)
UNIT_BOX = [("box", (1.0, 1.0, 1.0), (0.0, 0.0, 0.0))]
COLLIDE_CASES = [
    ("sphere_into_box", UNIT_BOX, qrow(SPH, (0.5,), (1.3, 0, 0)), 0.0, 0.2, (-1, 0, 0)),
    ("sphere_apart", UNIT_BOX, qrow(SPH, (0.5,), (1.6, 0, 0)), 0.0, None, None),
    ("sphere_within_separation", UNIT_BOX, qrow(SPH, (0.5,), (1.6, 0, 0)), 0.2, -0.1, (-1, 0, 0)),
    ("sphere_into_sphere", [("sphere", (1.0,), (1.2, 0.0, 0.0))], qrow(SPH, (0.5,), (0, 0, 0)), 0.0, 0.3,
     (1, 0, 0)),
    ("box_deep_in_box", UNIT_BOX, qrow(BOX, (0.5, 0.5, 0.5, 0.05), (0.8, 0, 0)), 0.0, 0.7, (-1, 0, 0)),
    ("capsule_on_box", UNIT_BOX, qrow(CAP, (0.3, 0.5), (0, 1.6, 0)), 0.0, 0.2, (0, -1, 0)),
    ("box_into_plane", [("plane", (), (0.0, 0.0, 0.0))], qrow(BOX, (0.5, 0.5, 0.5, 0.05), (0, 0.3, 0)), 0.0, 0.2,
     (0, -1, 0)),
]


def oracle_of(bodies, mesh=None):
    return pyoracle.OracleWorld(world.standard_settings(), bodies, (), [mesh] if mesh is not None else ())


def gpu_of(bodies, mesh=None):
    g = world.GpuWorld(world.standard_settings(), len(bodies) + 8)
    if mesh is not None:
        g.add_triangle_mesh(*mesh)
    g.add_bodies(bodies)
    return g


def mesh_bodies():
    b = scenes.blank_bodies(1)
    b["shape_type"][0] = _lib.SHAPE_TRIANGLE_MESH
    b["shape_params"][0] = 0.0
    b["motion_type"][0] = _lib.STATIC
    b["object_layer"][0] = scenes.LAYER_NOT_MOVING
    return b


# ---------------------------------------------------------------------------
# the oracle (CPU)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("case", COLLIDE_CASES, ids=[c[0] for c in COLLIDE_CASES])
def test_oracle_collide_known_answers(oracle_lib, case):
    _, specs, row, ms, pen, axis = case
    o = oracle_of(static_bodies(specs))
    out, bo, su, co = o.collide_shapes_all(np.array([row]), 4, max_separation=ms)
    if pen is None:
        assert co[0] == 0
        return
    assert co[0] == 1 and bo[0, 0] == 0 and su[0, 0] == 0xFFFFFFFF
    assert abs(out[0, 0, 0] - pen) < 1e-3, out[0, 0, 0]
    np.testing.assert_allclose(out[0, 0, 7:10], axis, atol=1e-3)
    # the deepest point of the query shape lies the penetration beyond the body's along the axis
    d = (out[0, 0, 1:4] - out[0, 0, 4:7]) @ np.asarray(axis, np.float64)
    assert abs(d - pen) < 1e-3, d


@pytest.mark.parametrize("backfaces", [True, False])
def test_oracle_collide_triangle(gpu_lib, oracle_lib, backfaces):
    """A sphere 0.3 m above a triangle facing it: 0.2 m; from behind only with back faces."""
    for idx, front in (([0, 1, 2], True), ([0, 2, 1], False)):
        m = _lib.build_triangle_mesh(TRI, np.array([idx]))
        o = oracle_of(mesh_bodies(), m)
        out, bo, su, co = o.collide_shapes_all(np.array([qrow(SPH, (0.5,), (0.2, 0.2, 0.3))]), 4, backfaces=backfaces)
        if not front and not backfaces:
            assert co[0] == 0
            continue
        # one triangle takes no sub-shape bits (subShape.pushIndex of index 0 of 1)
        assert co[0] == 1 and bo[0, 0] == 0 and su[0, 0] == 0xFFFFFFFF
        assert abs(out[0, 0, 0] - 0.2) < 1e-9
        out, bo, su, co = o.collide_shapes_all(np.array([qrow(BOX, (0.2, 0.2, 0.2, 0.05), (0.3, 0.3, 0.15))]), 4,
                                               backfaces=backfaces)
        assert co[0] == 1 and abs(out[0, 0, 0] - 0.05) < 1e-3, out[0, 0, 0]


CUBE = np.array([[x, y, z] for x in (-0.5, 0.5) for y in (-0.5, 0.5) for z in (-0.5, 0.5)], np.float64)


def test_oracle_cylinder_and_hull_queries(gpu_lib, oracle_lib):
    """An upright cylinder (half height 0.5, radius 0.3) whose base is 0.1 m into a unit box's
    top face, and a hull of a 1 m cube 0.2 m into it: collide 0.1 m and 0.2 m along -y.  Raised
    by 1 m and cast 3 m straight down, they touch the face after 0.9 m and 0.8 m."""
    hull = _lib.build_convex_hull(CUBE, 0.0)
    o = pyoracle.OracleWorld(world.standard_settings(), static_bodies(UNIT_BOX), [hull], ())
    rows = np.array([qrow(_lib.SHAPE_CYLINDER, (0.5, 0.3, 0.05), (0, 1.4, 0)),
                     qrow(_lib.SHAPE_CONVEX_HULL, (0.0,), (0.3, 1.3, 0.0))])
    out, bo, su, co = o.collide_shapes_all(rows, 4)
    assert (co == 1).all() and (bo[:, 0] == 0).all()
    np.testing.assert_allclose(out[:, 0, 0], [0.1, 0.2], atol=1e-3)
    np.testing.assert_allclose(out[:, 0, 7:10], [[0, -1, 0], [0, -1, 0]], atol=1e-3)
    casts = np.concatenate([rows + np.array([0] * 6 + [1.0] + [0] * 5), np.tile([0, -3.0, 0], (2, 1))], 1)
    out, bo = o.cast_shapes(casts)
    # from 0.1 m / 0.2 m into the box, raised 1 m: 0.9 m / 0.8 m of the 3 m displacement
    np.testing.assert_allclose(out[:, 0], [0.9 / 3, 0.8 / 3], atol=2e-3)


def line_of_spheres():
    return static_bodies([("sphere", (0.5,), (9.0, 0.0, 0.0)), ("sphere", (0.5,), (3.0, 0.0, 0.0)),
                          ("sphere", (0.5,), (6.0, 0.0, 0.0))])


def test_oracle_all_ray_hits(oracle_lib):
    b = line_of_spheres()
    b["collision_groups"][2] = 2
    o = oracle_of(b)
    r = np.array([[0, 0, 0, 1, 0, 0, 20.0]])
    fr, bo, su, co = o.cast_rays_all(r, 8)
    assert co[0] == 3 and list(bo[0, :3]) == [1, 2, 0]
    np.testing.assert_allclose(fr[0, :3], [2.5 / 20, 5.5 / 20, 8.5 / 20], atol=1e-4)
    fr, bo, su, co = o.cast_rays_all(r, 8, mask=~2 & 0xFFFFFFFF)
    assert co[0] == 2 and list(bo[0, :2]) == [1, 0]


def test_oracle_all_shape_cast_hits(oracle_lib):
    o = oracle_of(line_of_spheres())
    q = np.array([[SPH, 0.25, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 20, 0, 0]], np.float64)
    out, bo, su, co = o.cast_shapes_all(q, 8)
    assert co[0] == 3 and list(bo[0, :3]) == [1, 2, 0] and (su[0, :3] == 0xFFFFFFFF).all()
    np.testing.assert_allclose(out[0, :3, 0], [2.25 / 20, 5.25 / 20, 8.25 / 20], atol=1e-3)


# ---------------------------------------------------------------------------
# the GPU path against the oracle
# ---------------------------------------------------------------------------
@pytest.mark.gpu
def test_gpu_collide_known_answers(gpu_lib, oracle_lib):
    for name, specs, row, ms, pen, axis in COLLIDE_CASES:
        g = gpu_of(static_bodies(specs))
        for mode in (_lib.COLLECT_CLOSEST, _lib.COLLECT_ANY, _lib.COLLECT_ALL):
            h, c = g.collide_shapes(qarray([row]), mode, 4, max_separation_distance=ms)
            if pen is None:
                assert c[0] == 0 and (mode == _lib.COLLECT_ALL or h["body"][0, 0] == -1), name
                continue
            assert c[0] == 1 and h["body"][0, 0] == 0, (name, mode)
            assert abs(float(h["penetration"][0, 0]) - pen) < 1e-3, (name, h["penetration"][0, 0])
            np.testing.assert_allclose(h["axis"][0, 0], axis, atol=1e-3, err_msg=name)


@pytest.mark.gpu
def test_gpu_collide_triangle(gpu_lib, oracle_lib):
    for idx, front in (([0, 1, 2], True), ([0, 2, 1], False)):
        for backfaces in (True, False):
            g = world.GpuWorld(world.standard_settings(), 8)
            g.add_triangle_mesh(TRI, np.array([idx]))
            g.add_bodies(mesh_bodies())
            h, c = g.collide_shapes(qarray([qrow(SPH, (0.5,), (0.2, 0.2, 0.3)),
                                            qrow(BOX, (0.2, 0.2, 0.2, 0.05), (0.3, 0.3, 0.15))]),
                                    _lib.COLLECT_ALL, 4, collide_with_backfaces=backfaces)
            if not front and not backfaces:
                assert (c == 0).all()
                continue
            assert (c == 1).all()
            assert abs(float(h["penetration"][0, 0]) - 0.2) < 1e-5
            assert abs(float(h["penetration"][1, 0]) - 0.05) < 1e-3


def terrain_pile(seed):
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
    return sc, g, o


def random_shapes(rng, n, y_range):
    kinds = rng.integers(0, 3, n)
    params = np.zeros((n, 4))
    params[kinds == 0, 0] = rng.uniform(0.2, 0.6, (kinds == 0).sum())
    params[kinds == 1, 0:3] = rng.uniform(0.2, 0.6, ((kinds == 1).sum(), 3))
    params[kinds == 1, 3] = 0.05
    params[kinds == 2, 0:2] = rng.uniform(0.2, 0.4, ((kinds == 2).sum(), 2))
    pos = np.stack([rng.uniform(-6, 6, n), rng.uniform(*y_range, n), rng.uniform(-6, 6, n)], 1)
    q = scenes.random_quaternions(rng, n)
    return np.concatenate([kinds[:, None], params, pos, q], 1)


def random_cyl_hull(rng, n, y_range, n_hulls):
    """Cylinders and the pile's own hulls as query shapes."""
    kinds = np.where(rng.random(n) < 0.5, _lib.SHAPE_CYLINDER, _lib.SHAPE_CONVEX_HULL)
    params = np.zeros((n, 4))
    cyl = kinds == _lib.SHAPE_CYLINDER
    params[cyl, 0] = rng.uniform(0.2, 0.5, cyl.sum())
    params[cyl, 1] = rng.uniform(0.2, 0.5, cyl.sum())
    params[cyl, 2] = 0.05
    params[~cyl, 0] = rng.integers(0, n_hulls, (~cyl).sum())
    pos = np.stack([rng.uniform(-6, 6, n), rng.uniform(*y_range, n), rng.uniform(-6, 6, n)], 1)
    q = scenes.random_quaternions(rng, n)
    return np.concatenate([kinds[:, None], params, pos, q], 1)


def hit_keys(bodies, subs, count):
    return [(int(b), int(s)) for b, s in zip(bodies[:count], subs[:count])]


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [5, 6])
def test_gpu_collide_shapes_in_terrain_pile(gpu_lib, oracle_lib, seed):
    sc, g, o = terrain_pile(seed)
    rng = np.random.default_rng(seed + 100)
    rows = random_shapes(rng, 1024, (-1.0, 3.0))
    cap = 64
    out, bo, su, co = o.collide_shapes_all(rows, cap)
    h, c = g.collide_shapes(qarray(rows), _lib.COLLECT_ALL, cap)
    assert (co <= cap).all() and co.sum() > 1000 and (co == 0).sum() > 50
    same = np.array([hit_keys(h["body"][k], h["sub_shape_id"][k], c[k]) ==
                     hit_keys(bo[k], su[k], co[k]) for k in range(len(rows))])
    assert same.mean() >= 0.97, same.mean()
    # A box pushed deep through a terrain triangle makes a flat Minkowski difference; EPA stops on
    # a face short of the true depth (a lower bound on both sides: one such case, 0.059 m oracle,
    # 0.095 m device, 0.141 m by the separating axes), and where it stops follows the rounding of
    # fused multiply-adds.  About 3 % of the hits here; 95 % agree to FP64 rounding.
    err = np.concatenate([np.abs(h["penetration"][k, :c[k]] - out[k, :c[k], 0]) for k in np.flatnonzero(same)])
    assert np.quantile(err, 0.95) < 1e-5 and err.max() < 0.1, (np.quantile(err, 0.95), err.max())
    # closest: the deepest of the oracle's list; any: one of the list
    hc, cc = g.collide_shapes(qarray(rows), _lib.COLLECT_CLOSEST, 1)
    ha, ca = g.collide_shapes(qarray(rows), _lib.COLLECT_ANY, 1)
    agree_c, agree_a = 0, 0
    for k in np.flatnonzero(same):
        if co[k] == 0:
            agree_c += cc[k] == 0 and hc["body"][k, 0] == -1
            agree_a += ca[k] == 0
            continue
        deepest = np.max(out[k, :co[k], 0])
        agree_c += cc[k] == 1 and abs(float(hc["penetration"][k, 0]) - deepest) < 0.1
        agree_a += ca[k] == 1 and (int(ha["body"][k, 0]), int(ha["sub_shape_id"][k, 0])) in hit_keys(bo[k], su[k],
                                                                                                       co[k])
    assert agree_c >= 0.99 * same.sum() and agree_a >= 0.99 * same.sum(), (agree_c, agree_a, same.sum())


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [5, 6])
def test_gpu_ray_collectors_in_terrain_pile(gpu_lib, oracle_lib, seed):
    sc, g, o = terrain_pile(seed)
    rng = np.random.default_rng(seed + 200)
    n = 2048
    org = np.stack([rng.uniform(-7, 7, n), rng.uniform(4, 8, n), rng.uniform(-7, 7, n)], 1)
    d = rng.normal(size=(n, 3))
    d[:, 1] = -np.abs(d[:, 1]) - 0.3
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rows = np.concatenate([org, d, rng.uniform(5.0, 30.0, (n, 1))], 1)
    rays = np.zeros(n, _lib.RAY_DTYPE)
    rays["origin"], rays["direction"], rays["length"] = rows[:, 0:3], rows[:, 3:6], rows[:, 6]
    cap = 32
    fr, bo, su, co = o.cast_rays_all(rows, cap)
    h, c = g.cast_rays_collect(rays, _lib.COLLECT_ALL, cap)
    assert (co > 1).sum() > 200  # rays through several bodies or folds of the terrain
    same = np.array([hit_keys(h["body"][k], h["sub_shape_id"][k], c[k]) == hit_keys(bo[k], su[k], co[k])
                     for k in range(n)])
    assert same.mean() >= 0.97, same.mean()
    err = np.concatenate([np.abs(h["fraction"][k, :c[k]] - fr[k, :c[k]]) * rows[k, 6] for k in np.flatnonzero(same)])
    assert np.quantile(err, 0.99) < 2e-3, np.quantile(err, 0.99)
    ha, ca = g.cast_rays_collect(rays, _lib.COLLECT_ANY, 1)
    ok = [(ca[k] == 0) if co[k] == 0 else
          (ca[k] == 1 and (int(ha["body"][k, 0]), int(ha["sub_shape_id"][k, 0])) in hit_keys(bo[k], su[k], co[k]))
          for k in np.flatnonzero(same)]
    assert np.mean(ok) >= 0.99, np.mean(ok)
    # the closest collector through the same entry point equals cc_world_cast_rays
    hc, cc = g.cast_rays_collect(rays, _lib.COLLECT_CLOSEST, 1)
    h0 = g.cast_rays(rays)
    assert (hc["body"][:, 0] == h0["body"]).all() and (hc["fraction"][:, 0] == h0["fraction"]).all()
    assert (cc == (h0["body"] >= 0)).all()
    # too small a list: CC_ERR_CAPACITY
    with pytest.raises(_lib.CCError) as e:
        g.cast_rays_collect(rays, _lib.COLLECT_ALL, 1)
    assert e.value.status == _lib.CC_ERR_CAPACITY


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [5])
def test_gpu_shape_cast_collectors_in_terrain_pile(gpu_lib, oracle_lib, seed):
    sc, g, o = terrain_pile(seed)
    rng = np.random.default_rng(seed + 300)
    n = 512
    rows = random_shapes(rng, n, (7.0, 10.0))
    disp = np.stack([rng.uniform(-2, 2, n), rng.uniform(-14, -10, n), rng.uniform(-2, 2, n)], 1)
    q15 = np.concatenate([rows, disp], 1)
    casts = np.zeros(n, _lib.SHAPE_CAST_DTYPE)
    casts["shape_type"] = rows[:, 0].astype(np.int32)
    casts["shape_params"], casts["position"], casts["quaternion"] = rows[:, 1:5], rows[:, 5:8], rows[:, 8:12]
    casts["displacement"] = disp
    cap = 256
    out, bo, su, co = o.cast_shapes_all(q15, cap)
    h, c = g.cast_shapes_collect(casts, _lib.COLLECT_ALL, cap)
    assert (co <= cap).all() and (co > 1).sum() > 100
    # a swept shape meets many terrain triangles; compare the (body, triangle) sets and the nearest hit
    keys_g = [set(hit_keys(h["body"][k], h["sub_shape_id"][k], c[k])) for k in range(n)]
    keys_o = [set(hit_keys(bo[k], su[k], co[k])) for k in range(n)]
    bodies_same = np.array([{b for b, _ in keys_g[k]} == {b for b, _ in keys_o[k]} for k in range(n)])
    assert bodies_same.mean() >= 0.95, bodies_same.mean()
    overlap = np.array([len(keys_g[k] & keys_o[k]) / max(1, len(keys_g[k] | keys_o[k])) for k in range(n)])
    assert np.quantile(overlap, 0.05) >= 0.9, np.quantile(overlap, 0.05)
    counts_close = np.abs(c - co) <= np.maximum(2, 0.05 * co)
    assert counts_close.mean() >= 0.95, counts_close.mean()
    both = (c > 0) & (co > 0)
    lens = np.linalg.norm(disp, axis=1)
    err = np.abs(h["fraction"][both, 0] - out[both, 0, 0]) * lens[both]
    assert np.quantile(err, 0.99) < 2e-3 and err.max() < 0.1, (np.quantile(err, 0.99), err.max())
    # the closest collector names the same triangle as the oracle's closest cast
    hc = g.cast_shapes(casts)
    oc, ob, osub = o.cast_shapes(q15, with_subs=True)
    mesh = (hc["body"] == ob) & (ob == 0)
    # near-ties between neighbouring triangles may go either way in FP32 (3 of 57 casts once)
    assert mesh.sum() > 30 and (hc["sub_shape_id"][mesh] == osub[mesh]).mean() >= 0.9
    assert (hc["sub_shape_id"][(hc["body"] > 0)] == 0xFFFFFFFF).all()
    ha, ca = g.cast_shapes_collect(casts, _lib.COLLECT_ANY, 1)
    assert ((ca == 1) == (co > 0)).mean() >= 0.99
    hb = ha["body"][:, 0]
    inside = [hb[k] in set(bo[k, :co[k]]) for k in np.flatnonzero((ca == 1) & (co > 0))]
    assert np.mean(inside) >= 0.99


@pytest.mark.gpu
def test_gpu_cylinder_and_hull_queries_in_terrain_pile(gpu_lib, oracle_lib):
    """Cylinders and convex hulls as collide and cast query shapes in a terrain pile: the all-hit
    collide lists and the closest casts against the oracle's, with the bounds of the other tests."""
    sc, g, o = terrain_pile(5)
    rng = np.random.default_rng(400)
    rows = random_cyl_hull(rng, 512, (-1.0, 3.0), len(sc.hull_points))
    cap = 64
    out, bo, su, co = o.collide_shapes_all(rows, cap)
    h, c = g.collide_shapes(qarray(rows), _lib.COLLECT_ALL, cap)
    assert co.sum() > 300
    same = np.array([hit_keys(h["body"][k], h["sub_shape_id"][k], c[k]) == hit_keys(bo[k], su[k], co[k])
                     for k in range(len(rows))])
    assert same.mean() >= 0.97, same.mean()
    up = random_cyl_hull(rng, 512, (7.0, 10.0), len(sc.hull_points))
    disp = np.stack([rng.uniform(-2, 2, 512), rng.uniform(-14, -10, 512), rng.uniform(-2, 2, 512)], 1)
    casts = np.zeros(512, _lib.SHAPE_CAST_DTYPE)
    casts["shape_type"] = up[:, 0].astype(np.int32)
    casts["shape_params"], casts["position"], casts["quaternion"] = up[:, 1:5], up[:, 5:8], up[:, 8:12]
    casts["displacement"] = disp
    hc = g.cast_shapes(casts)
    oc, ob = o.cast_shapes(np.concatenate([up, disp], 1))
    agree = hc["body"] == ob
    assert agree.mean() >= 0.95 and (ob >= 0).mean() > 0.9, agree.mean()
    lens = np.linalg.norm(disp, axis=1)
    hit = agree & (ob >= 0)
    err = np.abs(hc["fraction"][hit] - oc[hit, 0]) * lens[hit]
    assert np.quantile(err, 0.99) < 2e-3, np.quantile(err, 0.99)
    # a hull index the world does not have is refused
    bad = casts[:1].copy()
    bad["shape_type"] = _lib.SHAPE_CONVEX_HULL
    bad["shape_params"][0, 0] = 99.0
    with pytest.raises(_lib.CCError):
        g.cast_shapes(bad)
