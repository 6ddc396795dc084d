"""Compound shapes (src/shapes/compound.ts): convex children at poses in the compound's frame.

The reference's tests build compounds and check their bounds and mass; the oracle's restatement
is pinned by equivalences that follow from the definition:
  * two unit boxes side by side make the 2 x 1 x 1 box: the same mass, centre of mass and
    inertia (massProperties.rotate / translate of each child, compound.ts:177-230), so a free
    compound and the single box fly and spin alike (to 1e-9);
  * dropped on a floor they come to rest alike (the children's hits merge into one manifold of
    the same normal, pruned to the same four corners: within 1e-3 m / 1e-3 rad);
  * a table of five boxes settles upright on its four legs, whose hits join one manifold
    carrying the first leg's sub-shape id (subShape.pushIndex of the child index,
    compound.ts:512-516);
  * queries reach the child: a ray names the child it hits, a point inside a child is inside
    the compound, collide and cast queries report the child's sub-shape id.

GPU tolerances (FP32 device, FP64 oracle): bodies within 2e-3 m of the oracle's while they fall
and settle; queries as in test_query_collectors.py.
"""
import math

import numpy as np
import pytest

from crashcat_gb300 import _lib, scenes, world
from oracle import pyoracle

TWO_BOXES = [("box", (0.5, 0.5, 0.5), (-0.5, 0.0, 0.0)), ("box", (0.5, 0.5, 0.5), (0.5, 0.0, 0.0))]
TABLE = [("box", (1.0, 0.1, 0.6), (0.0, 0.9, 0.0))] + [
    ("box", (0.08, 0.4, 0.08), (sx * 0.85, 0.4, sz * 0.5)) for sx in (-1, 1) for sz in (-1, 1)]


def floor_and(n):
    b = scenes.blank_bodies(n + 1)
    scenes.set_box(b, 0, (20.0, 0.5, 20.0))
    b["motion_type"][0] = _lib.STATIC
    b["object_layer"][0] = scenes.LAYER_NOT_MOVING
    b["position"][0] = (0.0, -0.5, 0.0)
    return b


def oracle_with(bodies, compounds, hulls=()):
    return pyoracle.OracleWorld(world.standard_settings(), bodies, hulls, (), [scenes.compound_children(c)
                                                                              for c in compounds])


def gpu_with(bodies, compounds):
    g = world.GpuWorld(world.standard_settings(), len(bodies) + 8)
    for c in compounds:
        g.add_compound(scenes.compound_children(c))
    g.add_bodies(bodies)
    return g


def pair_scene(compound_first=True, floor=False, spin=True):
    """A compound of two unit boxes and, in a second body slot far away, the 2 x 1 x 1 box."""
    b = floor_and(2) if floor else scenes.blank_bodies(2)
    i0 = 1 if floor else 0
    scenes.set_compound(b, i0, 0)
    scenes.set_box(b, i0 + 1, (1.0, 0.5, 0.5))
    q = np.array([0.1, 0.3, -0.2, 0.9])
    q /= np.linalg.norm(q)
    for k, x in ((i0, -5.0), (i0 + 1, 5.0)):
        b["position"][k] = (x, 2.0, 0.0)
        b["quaternion"][k] = q
        if spin:
            b["linear_velocity"][k] = (0.3, 1.0, -0.2)
            b["angular_velocity"][k] = (0.7, -1.3, 2.1)
    if not floor:
        b["gravity_factor"] = 0.0
    b["linear_damping"] = 0.0
    b["angular_damping"] = 0.0
    return b, i0


# ---------------------------------------------------------------------------
# the oracle (CPU)
# ---------------------------------------------------------------------------
def test_oracle_compound_flies_like_the_single_box(oracle_lib):
    b, i0 = pair_scene()
    o = oracle_with(b, [TWO_BOXES])
    o.step(1.0 / 60.0, 120)
    st = o.state()
    np.testing.assert_allclose(st[i0, 1:13], st[i0 + 1, 1:13], atol=1e-9)
    np.testing.assert_allclose(st[i0, 0] + 10.0, st[i0 + 1, 0], atol=1e-9)


def test_oracle_compound_rests_like_the_single_box(oracle_lib):
    b, i0 = pair_scene(floor=True, spin=False)
    b["quaternion"][1:] = (0.0, 0.0, math.sin(0.15), math.cos(0.15))
    o = oracle_with(b, [TWO_BOXES])
    o.step(1.0 / 60.0, 180)
    st = o.state()
    np.testing.assert_allclose(st[i0, 1:7], st[i0 + 1, 1:7], atol=1e-3)
    assert abs(st[i0, 1] - 0.48) < 5e-3  # its 1 m height resting 2 cm deep (the penetration slop)


def table_scene():
    b = floor_and(1)
    scenes.set_compound(b, 1, 0)
    b["position"][1] = (0.0, 0.3, 0.0)
    b["quaternion"][1] = (0.02, 0.0, 0.03, math.sqrt(1 - 0.02 ** 2 - 0.03 ** 2))
    b["allow_sleeping"] = 0
    return b


def test_oracle_table_settles_on_its_legs(oracle_lib):
    o = oracle_with(table_scene(), [TABLE])
    o.step(1.0 / 60.0, 120)
    st = o.state()
    q = st[1, 3:7]
    assert abs(abs(q[3]) - 1.0) < 1e-3  # upright
    # the legs' feet (0 in the compound's frame) rest on the floor, within the 2 cm penetration slop
    assert -0.025 < st[1, 1] < 0.005, st[1, 1]
    # the four feet share the floor's normal: their hits join one manifold, which keeps the
    # sub-shape ids of its first hit (update.ts:414-449), the first leg (child 1)
    subs = [tuple(int(x) for x in s) for s in o.manifold_sub_shapes()]
    assert subs == [(0xFFFFFFFF, 0xFFFFFFF9)], subs


def test_oracle_compound_queries(oracle_lib):
    b = scenes.blank_bodies(1)
    scenes.set_compound(b, 0, 0)
    b["motion_type"][0] = _lib.STATIC
    b["object_layer"][0] = scenes.LAYER_NOT_MOVING
    o = oracle_with(b, [TWO_BOXES])
    one_bit = 0xFFFFFFFE  # two children: one sub-shape bit
    # a ray down onto the right box names child 1, onto the left child 0
    fr, bo, su = o.cast_rays(np.array([[0.5, 3.0, 0.0, 0, -1, 0, 10.0], [-0.5, 3.0, 0.0, 0, -1, 0, 10.0]]))
    assert list(bo) == [0, 0] and list(su) == [one_bit | 1, one_bit | 0]
    np.testing.assert_allclose(fr, [0.25, 0.25], atol=1e-4)
    co, bo, su = o.collide_points(np.array([[0.7, 0.2, 0.1], [-0.7, 0.2, 0.1], [0.0, 0.7, 0.0]]))
    assert list(co) == [1, 1, 0] and list(su[:2]) == [one_bit | 1, one_bit | 0]
    # a sphere cast down onto the seam: the first child met (ties to the first)
    out, bo, su = o.cast_shapes(np.array([[_lib.SHAPE_SPHERE, 0.25, 0, 0, 0, 0.6, 3.0, 0.0, 0, 0, 0, 1, 0, -4.0, 0]]),
                                with_subs=True)
    assert bo[0] == 0 and su[0] == one_bit | 1 and abs(out[0, 0] - 2.25 / 4.0) < 1e-3
    # a box overlapping both children: one hit per child
    # (0.2 m deep.  Over the seam the reference's EPA is ill-conditioned at some depths: at 0.1 m
    # and 0.12 m a 1e-6 m nudge of the query moves its answer between the true depth and
    # 0.077 m / 0.097 m, where EPA stops early from another starting simplex)
    out, bo, su, co = o.collide_shapes_all(np.array([[_lib.SHAPE_BOX, 0.3, 0.3, 0.3, 0.05, 0.0, 0.6, 0.0, 0, 0, 0, 1]]),
                                           4)
    assert co[0] == 2 and sorted(su[0, :2]) == [one_bit | 0, one_bit | 1]
    np.testing.assert_allclose(out[0, :2, 0], [0.2, 0.2], atol=1e-3)


def test_oracle_refuses_a_cast_compound(oracle_lib):
    b = scenes.blank_bodies(1)
    scenes.set_compound(b, 0, 0)
    b["motion_quality"][0] = 1
    with pytest.raises(AssertionError):
        oracle_with(b, [TWO_BOXES])


# ---------------------------------------------------------------------------
# the GPU path against the oracle
# ---------------------------------------------------------------------------
@pytest.mark.gpu
def test_gpu_compound_flies_like_the_oracle(gpu_lib, oracle_lib):
    b, i0 = pair_scene()
    g, o = gpu_with(b, [TWO_BOXES]), oracle_with(b, [TWO_BOXES])
    g.step(1.0 / 60.0, 120)
    o.step(1.0 / 60.0, 120)
    rows, _ = g.get_state()
    np.testing.assert_allclose(rows[:, 0:13], o.state()[:, 0:13], atol=2e-4)


def compound_pile(n=24, seed=3):
    """Tables, dumbbells (two spheres on a capsule) and L-shapes (two boxes and a cylinder) dropped
    on a floor, on a 3 m grid so that each lands alone."""
    rng = np.random.default_rng(seed)
    b = floor_and(n)
    shapes = [TABLE,
              [("sphere", (0.25,), (-0.6, 0.0, 0.0)), ("sphere", (0.25,), (0.6, 0.0, 0.0)),
               ("capsule", (0.08, 0.5), (0.0, 0.0, 0.0), (0.0, 0.0, math.sin(math.pi / 4), math.cos(math.pi / 4)))],
              [("box", (0.5, 0.1, 0.1), (0.4, 0.0, 0.0)), ("box", (0.1, 0.4, 0.1), (0.0, 0.3, 0.0)),
               ("cylinder", (0.1, 0.2), (0.0, 0.0, 0.3))]]
    for i in range(1, n + 1):
        scenes.set_compound(b, i, int(rng.integers(0, 3)))
        b["position"][i] = (3.0 * ((i - 1) % 5), float(rng.uniform(0.8, 2.0)), 3.0 * ((i - 1) // 5))
        q = rng.normal(size=4)
        b["quaternion"][i] = q / np.linalg.norm(q)
    return b, shapes


@pytest.mark.gpu
def test_gpu_compound_pile_tracks_oracle(gpu_lib, oracle_lib):
    """Compounds of boxes, spheres, capsules and cylinders landing one by one.  Contacts: with the
    GPU's poses handed to the oracle, the same manifolds (bodies and sub-shape ids) and normals
    within 1e-3.  Motion: after 20 steps (most bodies still in the air) the median body within
    2e-3 m of the oracle's; after 120 steps a finite state, nothing below the floor, and the mean
    height of the centres of mass within 3 cm of the oracle's.  Per-body positions are not
    compared once they land: a compound landing on an edge or a corner tips one way or the other
    on the last bits of FP32 against FP64."""
    b, shapes = compound_pile()
    g, o = gpu_with(b, shapes), oracle_with(b, shapes)
    g.step(1.0 / 60.0, 30)
    rows, _ = g.get_state()
    st = o.state()
    st[:, 0:13] = rows[:, 0:13]
    o.set_state(st)
    g.step(0.0, 1)
    o.step(0.0, 1)
    gm, gs = g.get_manifolds(), g.get_manifold_sub_shapes()
    om, os_ = o.manifolds(), o.manifold_sub_shapes()
    gk = {(int(r[0]), int(r[1]), int(s_[0]), int(s_[1])): r for r, s_ in zip(gm, gs)}
    ok = {(int(r[0]), int(r[1]), int(s_[0]), int(s_[1])): r for r, s_ in zip(om, os_)}
    assert len(ok) > 5 and set(gk) == set(ok), set(gk) ^ set(ok)
    for k in ok:
        np.testing.assert_allclose(gk[k][3:6], ok[k][3:6], atol=1e-3)
    b, shapes = compound_pile()
    g, o = gpu_with(b, shapes), oracle_with(b, shapes)
    g.step(1.0 / 60.0, 20)
    o.step(1.0 / 60.0, 20)
    rows, _ = g.get_state()
    err = np.abs(rows[:, 0:3] - o.state()[:, 0:3]).max(axis=1)
    assert np.median(err) < 2e-3, np.sort(err)[-5:]
    g.step(1.0 / 60.0, 100)
    o.step(1.0 / 60.0, 100)
    rows, _ = g.get_state()
    st = o.state()
    assert np.isfinite(rows).all()
    assert rows[1:, 14].min() > -0.02
    assert abs(rows[1:, 14].mean() - st[1:, 14].mean()) < 0.03, (rows[1:, 14].mean(), st[1:, 14].mean())


@pytest.mark.gpu
def test_gpu_table_settles_on_its_legs(gpu_lib):
    g = gpu_with(table_scene(), [TABLE])
    g.step(1.0 / 60.0, 120)
    rows, _ = g.get_state()
    assert abs(abs(rows[1, 6]) - 1.0) < 1e-3 and -0.025 < rows[1, 1] < 0.005
    subs = [tuple(int(x) for x in s) for s in g.get_manifold_sub_shapes()]
    assert subs == [(0xFFFFFFFF, 0xFFFFFFF9)], subs


@pytest.mark.gpu
def test_gpu_compound_on_terrain(gpu_lib, oracle_lib):
    """Compounds dropped on a terrain mesh: the mesh pass collides them child by child (its EPA
    items carry the child); the first contacts' sub-shape ids (child, triangle) as the oracle's."""
    sc = scenes.mesh_drop(n=4, n_cells=12, seed=5, heights=(0.0, 1.0))
    b, shapes = compound_pile(n=12, seed=4)
    b = b[1:]  # no box floor: the terrain (12 m across, centred), the bodies 2.5 m apart inside it
    b["position"][:, 0] = -5.0 + 2.5 * (np.arange(len(b)) % 5)
    b["position"][:, 2] = -3.0 + 2.5 * (np.arange(len(b)) // 5)
    bodies = np.concatenate([sc.bodies[:1], b])
    g = world.GpuWorld(world.standard_settings(), len(bodies) + 8)
    g.add_triangle_mesh(*sc.mesh)
    for c in shapes:
        g.add_compound(scenes.compound_children(c))
    g.add_bodies(bodies)
    o = pyoracle.OracleWorld(world.standard_settings(), bodies, (), [g.get_triangle_mesh(0)],
                             [scenes.compound_children(c) for c in shapes])
    g.step(1.0 / 60.0, 40)
    rows, _ = g.get_state()
    st = o.state()
    st[:, 0:13] = rows[:, 0:13]
    o.set_state(st)
    g.step(0.0, 1)
    o.step(0.0, 1)
    gs = {tuple(int(x) for x in s) for s in g.get_manifold_sub_shapes()}
    os_ = {tuple(int(x) for x in s) for s in o.manifold_sub_shapes()}
    assert len(os_) > 5
    assert len(gs & os_) >= 0.9 * len(gs | os_), (len(gs & os_), len(gs | os_))
    g.step(1.0 / 60.0, 60)
    rows, _ = g.get_state()
    assert np.isfinite(rows).all() and rows[1:, 1].min() > -1.5  # nothing fell through


@pytest.mark.gpu
def test_gpu_compound_queries(gpu_lib, oracle_lib):
    b = scenes.blank_bodies(1)
    scenes.set_compound(b, 0, 0)
    b["motion_type"][0] = _lib.STATIC
    b["object_layer"][0] = scenes.LAYER_NOT_MOVING
    g = gpu_with(b, [TWO_BOXES])
    one_bit = 0xFFFFFFFE
    rays = np.zeros(2, _lib.RAY_DTYPE)
    rays["origin"] = [(0.5, 3.0, 0.0), (-0.5, 3.0, 0.0)]
    rays["direction"] = (0.0, -1.0, 0.0)
    rays["length"] = 10.0
    h = g.cast_rays(rays)
    assert list(h["body"]) == [0, 0] and list(h["sub_shape_id"]) == [one_bit | 1, one_bit | 0]
    np.testing.assert_allclose(h["fraction"], [0.25, 0.25], atol=2e-4)
    ha, c = g.cast_rays_collect(rays[:1], _lib.COLLECT_ALL, 4)
    assert c[0] == 1  # straight down the right box: one child
    p = g.collide_points([[0.7, 0.2, 0.1], [-0.7, 0.2, 0.1], [0.0, 0.7, 0.0]])
    assert list(p["count"]) == [1, 1, 0] and list(p["sub_shape_id"][:2]) == [one_bit | 1, one_bit | 0]
    q = np.zeros(1, _lib.COLLIDE_SHAPE_DTYPE)
    q["shape_type"] = _lib.SHAPE_BOX
    q["shape_params"] = (0.3, 0.3, 0.3, 0.05)
    q["position"] = (0.0, 0.6, 0.0)
    q["quaternion"] = (0.0, 0.0, 0.0, 1.0)
    hc, c = g.collide_shapes(q, _lib.COLLECT_ALL, 4)
    assert c[0] == 2 and sorted(hc["sub_shape_id"][0, :2]) == [one_bit | 0, one_bit | 1]
    np.testing.assert_allclose(hc["penetration"][0, :2], [0.2, 0.2], atol=1e-3)
    cs = np.zeros(1, _lib.SHAPE_CAST_DTYPE)
    cs["shape_type"] = _lib.SHAPE_SPHERE
    cs["shape_params"] = (0.25, 0, 0, 0)
    cs["position"] = (0.6, 3.0, 0.0)
    cs["quaternion"] = (0.0, 0.0, 0.0, 1.0)
    cs["displacement"] = (0.0, -4.0, 0.0)
    hs = g.cast_shapes(cs)
    assert hs["body"][0] == 0 and hs["sub_shape_id"][0] == one_bit | 1 and abs(hs["fraction"][0] - 2.25 / 4) < 1e-3


@pytest.mark.gpu
def test_gpu_compound_refusals(gpu_lib):
    g = world.GpuWorld(world.standard_settings(), 8)
    with pytest.raises(_lib.CCError):
        g.add_compound(scenes.compound_children([("box", (0.5, 0.5, -0.5), (0.0, 0.0, 0.0))]))
    idx = g.add_compound(scenes.compound_children(TWO_BOXES))
    b = scenes.blank_bodies(1)
    scenes.set_compound(b, 0, idx)
    b["motion_quality"][0] = 1  # LINEAR_CAST
    with pytest.raises(_lib.CCError):
        g.add_bodies(b)
    b["motion_quality"][0] = 0
    b["shape_scale"][0] = (2.0, 1.0, 1.0)
    with pytest.raises(_lib.CCError):
        g.add_bodies(b)
