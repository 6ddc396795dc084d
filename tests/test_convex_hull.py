"""Convex hull shapes (src/shapes/convex-hull.ts): the host-side construction against exact
geometry (CPU), the oracle's hull bodies against mechanics (CPU), and the GPU path against
the oracle.

The reference's hull tests are not transcribed here (tst/shapes covers box, capsule and
compound); the construction is pinned by exact answers: a cube's six quads, volume and inertia,
a tetrahedron's volume, centre of mass and inertia, Euler's formula and convexity for random
ellipsoid hulls, and the shrunk points inside the hull.

GPU tolerances (FP32 device state against the FP64 oracle, the same hull data on both):
  * broadphase pairs of a mixed pile: bit-exact;
  * contacts: normal within 1e-3, depth within 2e-3 m, for at least 97 % of the manifolds
    (a discrete choice - supporting face, clip side - may flip between FP32 and FP64);
  * a hull dropped on the floor: the first 30 steps within 2e-3 m and 2e-3 rad.
"""
import math

import numpy as np
import pytest

from crashcat_gb300 import _lib, scenes, world
from oracle import pyoracle


def tetra_inertia(v):
    """Unit-density inertia of a tetrahedron about its centroid (Tonon 2004, closed form)."""
    c = v.mean(0)
    a, b, d, e = v - c
    det = abs(np.linalg.det(np.array([b - a, d - a, e - a])))
    vol = det / 6.0
    pts = np.array([a, b, d, e])

    def s(i, j):
        return (sum(pts[k, i] * pts[k, j] for k in range(4)) + sum(pts[:, i]) * sum(pts[:, j])) * det / 120.0

    C = np.array([[s(i, j) for j in range(3)] for i in range(3)])
    return vol, c, np.trace(C) * np.eye(3) - C


# ---------------------------------------------------------------------------
# construction (CPU)
# ---------------------------------------------------------------------------
def test_cube_hull_is_exact(gpu_lib):
    cube = np.array([[x, y, z] for x in (-0.5, 0.5) for y in (-0.5, 0.5) for z in (-0.5, 0.5)], np.float32)
    pts = np.concatenate([cube + (1.0, 2.0, 3.0), [[1.0, 2.0, 3.0], [1.2, 2.1, 2.8]]]).astype(np.float32)
    h = _lib.build_convex_hull(pts, 0.0)
    assert len(h["points"]) == 8 and len(h["faces"]) == 6 and (h["faces"][:, 1] == 4).all()
    assert abs(h["volume"] - 1.0) < 1e-6
    np.testing.assert_allclose(h["com"], (1.0, 2.0, 3.0), atol=1e-6)
    np.testing.assert_allclose(h["inertia"], np.eye(3) / 6.0, atol=1e-7)
    np.testing.assert_allclose(np.abs(h["planes"][:, :3]).max(1), 1.0, atol=1e-7)
    np.testing.assert_allclose(h["planes"][:, 3], -0.5, atol=1e-7)
    # the default convex radius fits; a larger one is cut by the sharp corners: a corner of three
    # orthogonal faces moves sqrt(3) r when its planes move r, so r <= 0.05 / (sqrt(3) - 1)
    # (convex-hull.ts:369-432), well under half the cube's thickness
    assert abs(_lib.build_convex_hull(pts)["convex_radius"] - 0.05) < 1e-7
    assert abs(_lib.build_convex_hull(pts, 0.9)["convex_radius"] - 0.05 / (math.sqrt(3) - 1)) < 1e-6


def test_tetrahedron_mass_properties(gpu_lib):
    v = np.array([[0.1, 0.0, 0.2], [1.3, 0.1, 0.0], [0.2, 1.1, -0.1], [0.3, 0.2, 0.9]])
    h = _lib.build_convex_hull(v.astype(np.float32), 0.0)
    vol, c, I = tetra_inertia(v)
    assert len(h["faces"]) == 4
    assert abs(h["volume"] - vol) < 1e-6
    np.testing.assert_allclose(h["com"], c, atol=1e-6)
    np.testing.assert_allclose(h["inertia"], I, atol=1e-6)


@pytest.mark.parametrize("k", [16, 24, 32])
def test_ellipsoid_hulls_are_closed_and_convex(gpu_lib, k):
    rng = np.random.default_rng(k)
    for _ in range(5):
        p = scenes.ellipsoid_hull_points(rng, k, rng.uniform(0.3, 0.8, 3))
        h = _lib.build_convex_hull(p)
        pts = h["points"].astype(np.float64)
        pl = h["planes"].astype(np.float64)
        V, F, E = len(pts), len(pl), int(h["faces"][:, 1].sum()) // 2
        assert V - E + F == 2
        # every hull point and every input point is on or behind every plane (tolerance 1e-3)
        assert (pts @ pl[:, :3].T + pl[:, 3]).max() < 1e-3
        q = p.astype(np.float64) - h["com"].astype(np.float64)
        assert (q @ pl[:, :3].T + pl[:, 3]).max() < 1e-3
        # the shrunk points lie inside, the convex radius behind the faces that define them
        # (setConvexHullNoConvexSupport convex-hull.ts:732-788; the planes are moved through the
        # point itself, which a merged face holds to within the 1e-3 hull tolerance)
        sd = h["shrunk"].astype(np.float64) @ pl[:, :3].T + pl[:, 3]
        assert sd.max() < 1e-3
        for i, (cnt, f0, f1, f2) in enumerate(h["point_faces"]):
            for f in (f0, f1, f2)[:cnt]:
                assert abs(sd[i, f] + h["convex_radius"]) < 1e-3
        assert 0 < h["convex_radius"] <= 0.05 + 1e-7
        # volume and centre of mass from an independent fan about the hull's first point
        vol = 0.0
        for f0, n in h["faces"]:
            ids = h["face_vertices"][f0:f0 + n]
            for j in range(1, n - 1):
                a, b, c = pts[ids[0]], pts[ids[j]], pts[ids[j + 1]]
                vol += np.dot(a - pts[0], np.cross(b - pts[0], c - pts[0])) / 6.0
        assert abs(vol - h["volume"]) < 1e-5 * max(1.0, h["volume"])


def test_flat_input_is_rejected(gpu_lib):
    with pytest.raises(_lib.CCError):
        _lib.build_convex_hull(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]], np.float32))


# ---------------------------------------------------------------------------
# oracle hull bodies (CPU): a cube-shaped hull rests like the box
# ---------------------------------------------------------------------------
def cube_hull_scene(offset=(0.0, 0.0, 0.0)):
    """A static floor, a box and a hull of the same cube, resting.  The hull's points are
    shifted by offset, so its centre of mass is that far from the body origin.  The reference
    collides a hull at the body position with its points relative to their centre of mass
    (update.ts:755-790 passes body.position; convex-hull.ts:228 stores the points relative to the
    centre of mass), while the dynamics use position + rotation x centre of mass
    (rigid-body.ts:527-536): the geometry rests where the box does and the centre of mass sits
    offset from it."""
    cube = np.array([[x, y, z] for x in (-0.4, 0.4) for y in (-0.4, 0.4) for z in (-0.4, 0.4)], np.float32)
    b = scenes.blank_bodies(3)
    scenes.static_floor(b, 0, half=(20.0, 0.5, 20.0))
    scenes.set_box(b, 1, (0.4, 0.4, 0.4))
    scenes.set_hull(b, 2, 0)
    b["position"][1] = (-2.0, 0.3995, 0.0)
    b["position"][2] = (2.0, 0.3995, 0.0)
    b["friction"] = 0.5
    return scenes.Scene("cube_hull", b, dt=1.0 / 60.0, steps=60, hull_points=[cube + np.float32(offset)])


def test_oracle_cube_hull_rests_like_the_box(gpu_lib, oracle_lib):
    sc = cube_hull_scene(offset=(0.3, -0.2, 0.1))
    hulls = [_lib.build_convex_hull(p) for p in sc.hull_points]
    o = pyoracle.OracleWorld(world.standard_settings(), sc.bodies, hulls)
    o.step(sc.dt, 90)
    st = o.state()
    # the hull's geometry rests where the box does, its centre of mass offset from it
    assert abs(st[2, 1] - st[1, 1]) < 1e-3
    np.testing.assert_allclose(st[2, 13:16] - st[2, 0:3], (0.3, -0.2, 0.1), atol=1e-3)
    assert np.abs(st[1:, 7:13]).max() < 1e-2


# ---------------------------------------------------------------------------
# the GPU path against the oracle
# ---------------------------------------------------------------------------
def gpu_and_oracle(sc, **settings):
    ws = world.standard_settings(velocity_iterations=sc.velocity_iterations,
                                 position_iterations=sc.position_iterations, **settings)
    ws.num_worlds = sc.num_worlds
    g = world.GpuWorld(ws, sc.n + 16)
    for p in sc.hull_points or ():
        g.add_convex_hull(p)
    g.add_bodies(sc.bodies)
    hulls = [g.get_convex_hull(i) for i in range(len(sc.hull_points or ()))]
    o = pyoracle.OracleWorld(ws, sc.bodies, hulls)
    return g, o


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [2, 3])
def test_mixed_pile_pairs_and_contacts(gpu_lib, oracle_lib, seed):
    sc = scenes.mixed_convex_pile(n=300, seed=seed, extent=6.0, heights=(0.5, 3.0))
    g, o = gpu_and_oracle(sc)
    g.step(0.0, 1)
    o.step(0.0, 1)
    gp = {tuple(sorted(p)) for p in g.get_pairs().tolist()}
    op = {tuple(sorted(p)) for p in o.pairs().tolist()}
    assert gp == op
    gm = {(int(r[0]), int(r[1])): r for r in g.get_manifolds()}
    om = {(int(r[0]), int(r[1])): r for r in o.manifolds()}
    common = set(gm) & set(om)
    assert len(common) >= 0.97 * max(len(gm), len(om)) and len(common) > 20
    bad = 0
    for k in common:
        a, b = gm[k], om[k]
        if np.abs(a[3:6] - b[3:6]).max() > 1e-3 or abs(a[6] - b[6]) > 2e-3:
            bad += 1
    assert bad <= 0.03 * len(common), (bad, len(common))


@pytest.mark.gpu
def test_cube_hull_with_offset_com_parity(gpu_lib, oracle_lib):
    sc = cube_hull_scene(offset=(0.3, -0.2, 0.1))
    sc.bodies["quaternion"][2] = (0.0, math.sin(0.2), 0.0, math.cos(0.2))
    sc.bodies["position"][2, 1] += 1.0
    sc.bodies["angular_velocity"][2] = (0.5, 1.0, -0.3)
    g, o = gpu_and_oracle(sc)
    for _ in range(3):
        g.step(sc.dt, 10)
        o.step(sc.dt, 10)
        rows, _ = g.get_state()
        st = o.state()
        np.testing.assert_allclose(rows[:, 0:3], st[:, 0:3], atol=2e-3)
        np.testing.assert_allclose(rows[:, 13:16], st[:, 13:16], atol=2e-3)
        dq = np.minimum(np.abs(rows[:, 3:7] - st[:, 3:7]).max(1), np.abs(rows[:, 3:7] + st[:, 3:7]).max(1))
        assert dq.max() < 2e-3


@pytest.mark.gpu
def test_mixed_pile_settles(gpu_lib, oracle_lib):
    """120 steps of the pile: nothing sinks through the floor and the mean height stays within
    5 cm of the oracle's."""
    sc = scenes.mixed_convex_pile(n=120, seed=4, extent=5.0, heights=(0.5, 4.0))
    g, o = gpu_and_oracle(sc)
    g.step(sc.dt, 120)
    o.step(sc.dt, 120)
    rows, _ = g.get_state()
    st = o.state()
    assert np.isfinite(rows).all()
    assert rows[1:, 14].min() > 0.0
    assert abs(rows[1:, 14].mean() - st[1:, 14].mean()) < 0.05
