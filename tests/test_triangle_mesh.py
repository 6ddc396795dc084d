"""Triangle meshes (src/shapes/triangle-mesh.ts, utils/triangle-mesh-builder.ts,
utils/triangle-mesh-bvh.ts, collision/active-edges.ts): the construction and the oracle's
active-edge fix against the reference's own tests (CPU), the oracle's mesh contacts against
mechanics (CPU), the GPU path against the oracle.

Known answers (tests/golden/mesh_known_answers.json, transcribed from
tst/shapes/triangle-mesh-builder.test.ts and tst/collision/active-edges.test.ts): triangle counts
after welding and degenerate and duplicate removal, active-edge bits, and which normal fixNormal
keeps.  The BVH is checked structurally: pre-order layout, every triangle in one leaf of at most
8, node bounds that hold their triangles.

GPU tolerances (FP32 device state against the FP64 oracle, the same mesh data on both):
  * broadphase pairs of a terrain drop: bit-exact;
  * mesh contacts of landed bodies (the oracle given the GPU's poses), matched by (bodies,
    triangle sub-shape id): at least 95 % of them, normals within
    1e-3 and depth within 2e-3 m for at least 95 % of the matched (FP32 and FP64 may pick
    another triangle first where hits tie, which regroups a pair's hits);
  * a box and a sphere resting on a flat mesh: within 1e-3 m of the oracle after 60 steps;
  * the terrain drop, 120 steps: nothing below the terrain, mean height within 5 cm of the oracle.
"""
import json
import math
import os

import numpy as np
import pytest

from crashcat_gb300 import _lib, scenes, world
from oracle import pyoracle

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "mesh_known_answers.json")))


# ---------------------------------------------------------------------------
# construction (CPU)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("case", GOLDEN["builder"], ids=[c["name"] for c in GOLDEN["builder"]])
def test_builder_known_answers(gpu_lib, case):
    pos = np.array(case["positions"], np.float64).reshape(-1, 3)
    idx = np.array(case["indices"], np.int64).reshape(-1, 3)
    m = _lib.build_triangle_mesh(pos, idx, case.get("degenerate_tolerance", -1.0))
    assert len(m["triangles"]) == case["count"]
    for t, mask, want in case.get("active", []):
        assert (int(m["triangles"][t, 3]) & mask) == want, (t, mask, m["triangles"])


@pytest.mark.parametrize("case", GOLDEN["fix_normal"], ids=[c["name"] for c in GOLDEN["fix_normal"]])
def test_fix_normal_known_answers(oracle_lib, case):
    t = GOLDEN["fix_normal_triangle"]
    n = case["normal"]
    if isinstance(n, str):  # vec3.normalize(0.001, 1, 0.001)
        v = np.array([0.001, 1.0, 0.001])
        n = v / np.linalg.norm(v)
    got = pyoracle.fix_normal(t["v0"], t["v1"], t["v2"], t["triangle_normal"], case["active"], case["point"], n,
                              case["movement"])
    assert got == case["keeps_normal"]


def check_bvh(m):
    nodes, tris, verts = m["nodes"].astype(np.float64), m["triangles"], m["vertices"].astype(np.float64)
    seen = np.zeros(len(tris), int)

    def walk(k, depth):
        nd = nodes[k]
        lo, hi = nd[0:3], nd[3:6]
        if nd[7] < 0:
            start, count = int(nd[6]), int(-nd[7]) - 1
            assert 1 <= count <= 8 or len(tris) == 0
            for t in range(start, start + count):
                seen[t] += 1
                p = verts[tris[t, :3]]
                assert (p >= lo - 1e-6).all() and (p <= hi + 1e-6).all()
            return k + 1
        left_end = walk(k + 1, depth + 1)
        assert int(nd[6]) == left_end  # the right child follows the left subtree (pre-order)
        for c in (k + 1, left_end):
            assert (nodes[c, 0:3] >= lo - 1e-6).all() and (nodes[c, 3:6] <= hi + 1e-6).all()
        return walk(left_end, depth + 1)

    assert walk(0, 0) == len(nodes)
    assert (seen == 1).all()


@pytest.mark.parametrize("cells", [4, 16, 64])
def test_heightfield_mesh_structure(gpu_lib, cells):
    pos, idx = scenes.heightfield(cells, 1.0, 3.0, seed=cells)
    m = _lib.build_triangle_mesh(pos, idx)
    assert len(m["triangles"]) == 2 * cells * cells and len(m["vertices"]) == (cells + 1) ** 2
    check_bvh(m)
    # normals point up (the winding faces +Y)
    assert (m["normals"][:, 1] > 0).all()


def test_flat_grid_inner_edges_inactive(gpu_lib):
    pos, idx = scenes.heightfield(6, 1.0, 0.0)
    m = _lib.build_triangle_mesh(pos, idx)
    t = m["triangles"]
    v = m["vertices"]
    # an edge is on the boundary when both its ends lie on the grid's border
    border = lambda k: abs(abs(v[k, 0]) - 3.0) < 1e-6 or abs(abs(v[k, 2]) - 3.0) < 1e-6
    for tri in t:
        for e, (i, j) in enumerate(((0, 1), (1, 2), (2, 0))):
            a, b = tri[i], tri[j]
            on_border = border(a) and border(b) and (abs(v[a, 0] - v[b, 0]) < 1e-6 or abs(v[a, 2] - v[b, 2]) < 1e-6)
            assert bool(tri[3] & (1 << e)) == on_border


def test_full_size_terrain_counts(gpu_lib):
    """The mixed workload's terrain: 256 x 256 cells, 66,049 vertices, 131,072 triangles."""
    pos, idx = scenes.heightfield(256, 1.0, 4.0, seed=2)
    m = _lib.build_triangle_mesh(pos, idx)
    assert len(m["vertices"]) == 66049 and len(m["triangles"]) == 131072
    assert m["nodes"][0, 7] >= 0 and len(m["nodes"]) >= 2 * 131072 // 8 - 1


# ---------------------------------------------------------------------------
# the oracle's mesh contacts (CPU)
# ---------------------------------------------------------------------------
def flat_mesh_scene(shape: str, on_mesh: bool):
    """A body resting on a flat 8 x 8 mesh at y = 0, or on a static box whose top is y = 0."""
    b = scenes.blank_bodies(2)
    if on_mesh:
        b["shape_type"][0] = _lib.SHAPE_TRIANGLE_MESH
        b["shape_params"][0] = 0.0
        b["motion_type"][0] = _lib.STATIC
        b["object_layer"][0] = scenes.LAYER_NOT_MOVING
    else:
        scenes.static_floor(b, 0, half=(4.0, 0.5, 4.0))
    b["friction"][0] = 0.5
    if shape == "box":
        scenes.set_box(b, 1, (0.4, 0.3, 0.5))
        b["position"][1] = (0.3, 0.3, -0.2)
    else:
        scenes.set_sphere(b, 1, 0.35)
        b["position"][1] = (0.3, 0.35, -0.2)
    b["friction"][1] = 0.5
    return b


def mesh_oracle(bodies, mesh_arrays, hulls=()):
    return pyoracle.OracleWorld(world.standard_settings(), bodies, hulls, [mesh_arrays])


@pytest.mark.parametrize("shape", ["box", "sphere"])
def test_oracle_flat_mesh_rests_like_a_box_floor(gpu_lib, oracle_lib, shape):
    pos, idx = scenes.heightfield(8, 1.0, 0.0)
    m = _lib.build_triangle_mesh(pos, idx)
    om = mesh_oracle(flat_mesh_scene(shape, True), m)
    ob = pyoracle.OracleWorld(world.standard_settings(), flat_mesh_scene(shape, False))
    om.step(1 / 60, 90)
    ob.step(1 / 60, 90)
    sm, sb = om.state(), ob.state()
    np.testing.assert_allclose(sm[1, 0:3], sb[1, 0:3], atol=2e-3)
    assert np.abs(sm[1, 7:13]).max() < 1e-2


def test_oracle_sphere_rolls_across_inner_edges(gpu_lib, oracle_lib):
    """A sphere rolling over a flat mesh keeps rolling and stays on it.  updateWorld hands the
    active-edge fix A's velocity minus B's in narrowphase order (update.ts:729-733), A being the
    static mesh, and the reversed mesh collide keeps that direction (collide-shape-vs-shape.ts:
    281-354): the fix then keeps the normals of inactive edges ahead of the body and replaces those
    behind it, so the sphere meets the inner edges ahead as small steps (a few millimetres)."""
    pos, idx = scenes.heightfield(12, 0.5, 0.0)
    m = _lib.build_triangle_mesh(pos, idx)
    b = flat_mesh_scene("sphere", True)
    b["position"][1] = (-2.0, 0.35, -0.13)
    b["linear_velocity"][1] = (3.0, 0.0, 0.7)
    b["allow_sleeping"][1] = 0
    o = mesh_oracle(b, m)
    ys = []
    for _ in range(60):
        o.step(1 / 60, 1)
        ys.append(o.state()[1, 1])
    st = o.state()
    assert st[1, 0] > -0.5 and st[1, 7] > 1.0  # still rolling forward
    assert 0.33 < min(ys) and max(ys) < 0.36, (min(ys), max(ys))


# ---------------------------------------------------------------------------
# the GPU path against the oracle
# ---------------------------------------------------------------------------
def gpu_and_oracle_mesh(sc):
    ws = world.standard_settings()
    g = world.GpuWorld(ws, sc.n + 16)
    for p in sc.hull_points or ():
        g.add_convex_hull(p)
    g.add_triangle_mesh(*sc.mesh)
    g.add_bodies(sc.bodies)
    hulls = [g.get_convex_hull(i) for i in range(len(sc.hull_points or ()))]
    o = pyoracle.OracleWorld(ws, sc.bodies, hulls, [g.get_triangle_mesh(0)])
    return g, o


@pytest.mark.gpu
@pytest.mark.parametrize("shape", ["box", "sphere"])
def test_flat_mesh_rest_parity(gpu_lib, oracle_lib, shape):
    pos, idx = scenes.heightfield(8, 1.0, 0.0)
    sc = scenes.Scene("flat", flat_mesh_scene(shape, True), dt=1 / 60, steps=60)
    sc.mesh = (pos, idx)
    g, o = gpu_and_oracle_mesh(sc)
    g.step(sc.dt, 60)
    o.step(sc.dt, 60)
    rows, _ = g.get_state()
    np.testing.assert_allclose(rows[1, 0:3], o.state()[1, 0:3], atol=1e-3)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [5, 6])
def test_terrain_pairs_and_contacts(gpu_lib, oracle_lib, seed):
    sc = scenes.mesh_drop(n=80, n_cells=16, seed=seed, heights=(0.0, 1.0))
    g, o = gpu_and_oracle_mesh(sc)
    # let the bodies land, then hand the oracle the GPU's state: both collide the same poses
    g.step(sc.dt, 50)
    rows, _ = g.get_state()
    st = o.state()
    st[:, 0:13] = rows[:, 0:13]
    o.set_state(st)
    g.step(0.0, 1)
    o.step(0.0, 1)
    gp = {tuple(sorted(p)) for p in g.get_pairs().tolist()}
    op = {tuple(sorted(p)) for p in o.pairs().tolist()}
    assert gp == op
    gm, gs = g.get_manifolds(), g.get_manifold_sub_shapes()
    om, os_ = o.manifolds(), o.manifold_sub_shapes()
    gk = {(int(r[0]), int(r[1]), int(s[0]), int(s[1])): r for r, s in zip(gm, gs)}
    ok = {(int(r[0]), int(r[1]), int(s[0]), int(s[1])): r for r, s in zip(om, os_)}
    mesh_keys = [k for k in ok if k[0] == 0]
    assert len(mesh_keys) > 10
    common = set(gk) & set(ok)
    assert len(common) >= 0.95 * max(len(gk), len(ok)), (len(common), len(gk), len(ok))
    bad = sum(1 for k in common
              if np.abs(gk[k][3:6] - ok[k][3:6]).max() > 1e-3 or abs(gk[k][6] - ok[k][6]) > 2e-3)
    assert bad <= 0.05 * len(common), (bad, len(common))


@pytest.mark.gpu
def test_terrain_drop_settles(gpu_lib, oracle_lib):
    sc = scenes.mesh_drop(n=60, n_cells=16, seed=7)
    g, o = gpu_and_oracle_mesh(sc)
    g.step(sc.dt, 120)
    o.step(sc.dt, 120)
    rows, _ = g.get_state()
    st = o.state()
    assert np.isfinite(rows).all()
    assert rows[1:, 1].min() > -1.5  # the terrain spans +-1 m: nothing fell through
    assert abs(rows[1:, 1].mean() - st[1:, 1].mean()) < 0.05
    assert g.stats()["overflow_flags"] == 0


# ---------------------------------------------------------------------------
# continuous collision against a mesh (castConvexVsTriangleMesh / castSphereVsTriangleMesh)
# ---------------------------------------------------------------------------
def ccd_mesh_scene(shape: str, amplitude: float):
    """A LINEAR_CAST body at 80 m/s straight down onto an 8 x 8 terrain of the given relief."""
    b = scenes.blank_bodies(2)
    b["shape_type"][0] = _lib.SHAPE_TRIANGLE_MESH
    b["motion_type"][0] = _lib.STATIC
    b["object_layer"][0] = scenes.LAYER_NOT_MOVING
    if shape == "box":
        scenes.set_box(b, 1, (0.2, 0.2, 0.2))
    else:
        scenes.set_sphere(b, 1, 0.2)
    b["position"][1] = (0.3, 3.0, 0.2)
    b["linear_velocity"][1] = (0.0, -80.0, 0.0)
    b["motion_quality"][1] = 1
    b["gravity_factor"][1] = 0.0
    return b


CCD_MESH_CASES = [
    # (shape, relief, active-edge cosine, caught by the cast)
    ("box", 3.0, -2.0, True),     # sharp terrain: active edges, the hit registers
    ("box", 0.0, -0.5, True),     # flat, every edge active: the hit registers
    ("box", 0.0, -2.0, False),    # flat, inner edges inactive: fixNormal turns the axis to the
                                  # triangle normal, which faces the body; the collector drops it
    ("sphere", 0.0, -0.5, False), # the sphere cast reports the negated contact normal
                                  # (triangle-mesh.ts:1847-1848): the collector drops it
]


@pytest.mark.parametrize("shape,relief,cos,caught", CCD_MESH_CASES)
def test_oracle_ccd_against_mesh(gpu_lib, oracle_lib, shape, relief, cos, caught):
    """The continuous-collision cast against a mesh as the reference wires it: the visitor casts
    every LINEAR_CAST body against the mesh body (update.ts:1210-1240), and the collector keeps a
    hit only when its penetration axis points along the motion (update.ts:1050-1054)."""
    pos, idx = scenes.heightfield(8, 1.0, relief, seed=3)
    m = _lib.build_triangle_mesh(pos, idx, -1.0, cos)
    o = pyoracle.OracleWorld(world.standard_settings(), ccd_mesh_scene(shape, relief), (), [m])
    hits = 0
    for _ in range(4):
        o.step(1 / 60, 1)
        hits += o.ccd_counts()[1]
    y = o.state()[1, 1]
    if caught:
        assert hits >= 1 and y > -relief / 2 - 0.3, y
    else:
        assert hits == 0 and y < -1.0, y


@pytest.mark.gpu
@pytest.mark.parametrize("shape,relief,cos,caught", CCD_MESH_CASES)
def test_ccd_against_mesh_parity(gpu_lib, oracle_lib, shape, relief, cos, caught):
    pos, idx = scenes.heightfield(8, 1.0, relief, seed=3)
    ws = world.standard_settings()
    g = world.GpuWorld(ws, 8)
    g.add_triangle_mesh(pos, idx, -1.0, cos)
    b = ccd_mesh_scene(shape, relief)
    g.add_bodies(b)
    o = pyoracle.OracleWorld(ws, b, (), [g.get_triangle_mesh(0)])
    for k in range(4):
        g.step(1 / 60, 1)
        o.step(1 / 60, 1)
        s = g.stats()
        assert (s["num_ccd"], s["num_ccd_hits"]) == o.ccd_counts(), k
        rows, _ = g.get_state()
        np.testing.assert_allclose(rows[1, 0:3], o.state()[1, 0:3], atol=5e-3, err_msg=f"step {k}")


# ---------------------------------------------------------------------------
# the reduction collector's pool of 32 manifolds (update.ts:358-361)
# ---------------------------------------------------------------------------
def cone_bowl(sectors: int = 12, radius: float = 3.0, slope_deg: float = 30.0):
    """An inverted cone of `sectors` facets sloping `slope_deg` up from the apex at the origin:
    adjacent facet normals differ by cos = 0.75 + 0.25 cos(360 / sectors), below the manifold
    merge threshold cos 5 degrees, so a body sitting in the apex touches one normal group per
    facet."""
    h = radius * math.tan(math.radians(slope_deg))
    ang = 2.0 * math.pi * np.arange(sectors) / sectors
    pos = np.concatenate([[[0.0, 0.0, 0.0]], np.stack([radius * np.cos(ang), np.full(sectors, h),
                                                        radius * np.sin(ang)], 1)])
    idx = np.array([[0, (i + 1) % sectors + 1, i + 1] for i in range(sectors)])  # facing up
    return pos, idx


@pytest.mark.gpu
@pytest.mark.parametrize("shape", ["sphere", "cylinder"])
def test_bowl_uses_the_32_manifold_pool(gpu_lib, oracle_lib, shape):
    """A sphere (or an upright cylinder, on its rim) settled in the apex of a 12-facet bowl
    touches every facet with its own normal: 12 manifolds for the one pair, as the reference's
    pool of 32 keeps them.  The pair
    overflows the 4-manifold pool of the first passes and is run again with 32 (stats mesh_big);
    no pair outgrows 32 (mesh_reduced 0).  The manifolds match the oracle's at the same poses."""
    b = scenes.blank_bodies(2)
    b["shape_type"][0] = _lib.SHAPE_TRIANGLE_MESH
    b["motion_type"][0] = _lib.STATIC
    b["object_layer"][0] = scenes.LAYER_NOT_MOVING
    if shape == "sphere":
        scenes.set_sphere(b, 1, 1.0)
    else:
        scenes.set_cylinder(b, 1, 0.3, 1.0)
    b["position"][1] = (0.0, 2.5, 0.0)
    sc = scenes.Scene("bowl", b, dt=1 / 60, steps=60)
    sc.mesh = cone_bowl()
    g, o = gpu_and_oracle_mesh(sc)
    g.step(sc.dt, 60)
    rows, _ = g.get_state()
    st = o.state()
    st[:, 0:13] = rows[:, 0:13]
    o.set_state(st)
    g.step(0.0, 1)
    o.step(0.0, 1)
    stats = g.stats()
    assert stats["mesh_big"] == 1 and stats["mesh_reduced"] == 0, stats
    gm, gs = g.get_manifolds(), g.get_manifold_sub_shapes()
    om, os_ = o.manifolds(), o.manifold_sub_shapes()
    assert len(om) > 4 and len(gm) == len(om), (len(gm), len(om))
    gk = {(int(s[0]), int(s[1])): r for r, s in zip(gm, gs)}
    ok = {(int(s[0]), int(s[1])): r for r, s in zip(om, os_)}
    assert set(gk) == set(ok)
    for k in ok:
        np.testing.assert_allclose(gk[k][3:6], ok[k][3:6], atol=1e-3)
        assert abs(gk[k][6] - ok[k][6]) < 2e-3
