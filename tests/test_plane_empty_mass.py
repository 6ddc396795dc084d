"""Plane and empty shapes (src/shapes/plane.ts, empty-shape.ts) and the given mass properties
(RigidBodySettings.mass / massPropertiesOverride, src/body/rigid-body.ts:309-326, 676-700).

The oracle against closed forms: a sphere and a box penetrating the plane y = 0 (depth and
normal of collideConvexVsPlane); a box resting on the plane (4 points from the plane's adaptive
face clipped against the box face); a ray's analytic fraction and point containment (castRay /
collidePoint of plane.ts); an empty body that nothing touches; a given mass scaling the box's
inverse inertia by m0 / m (scaleToMass) and a given inertia tensor used as is.

GPU tolerances: broadphase pairs bit-exact on the plane scene, manifold normals within 1e-3 and
depths within 2e-3; bodies that touch only the plane within 2e-3 m over 90 steps; ray fractions
within 2e-3 and the same hit bodies.
"""
import math

import numpy as np
import pytest

from crashcat_gb300 import _lib, scenes, world
from oracle import pyoracle


def row(b, i=0):
    return np.ascontiguousarray(pyoracle.rows_from_bodies(b)[i])


def plane_and(shape, params, pos, quat=(0.0, 0.0, 0.0, 1.0)):
    b = scenes.blank_bodies(2)
    scenes.set_plane(b, 0, (0.0, 1.0, 0.0), 0.0)
    b["motion_type"][0] = _lib.STATIC
    b["object_layer"][0] = scenes.LAYER_NOT_MOVING
    if shape == "sphere":
        scenes.set_sphere(b, 1, params)
    else:
        scenes.set_box(b, 1, params)
    b["position"][1] = pos
    b["quaternion"][1] = quat
    return b


def collide(lib, b, max_sep=0.02):
    out = np.zeros(13)
    lib.orc_collide_pair(pyoracle.dptr(row(b, 0)), pyoracle.dptr(row(b, 1)), max_sep, pyoracle.dptr(out))
    return out


def test_oracle_plane_contacts(oracle_lib):
    lib = pyoracle.load()
    s = collide(lib, plane_and("sphere", 0.5, (0.3, 0.4, -0.2)))
    assert s[0] == 1 and s[10] == pytest.approx(0.1, abs=1e-7)  # 0.4 passes through an FP32 record
    np.testing.assert_allclose(s[7:10] / np.linalg.norm(s[7:10]), [0, 1, 0], atol=1e-12)
    # a box turned 0.3 rad about Z: its lowest corner 0.05 below the plane
    q = (0.0, 0.0, math.sin(0.15), math.cos(0.15))
    he = np.array([0.5, 0.25, 0.25])
    low = he[0] * math.sin(0.3) + he[1] * math.cos(0.3)
    bx = collide(lib, plane_and("box", tuple(he), (0.0, low - 0.05, 0.0), q))
    assert bx[0] == 1 and bx[10] == pytest.approx(0.05, abs=1e-6)
    assert collide(lib, plane_and("sphere", 0.5, (0.0, 0.55, 0.0)), max_sep=0.0)[0] == 0


def test_oracle_box_rests_on_plane(oracle_lib):
    b = plane_and("box", (0.4, 0.3, 0.2), (0.0, 1.0, 0.0))
    b["allow_sleeping"][1] = 0
    o = pyoracle.OracleWorld(world.standard_settings(), b)
    o.step(1.0 / 60.0, 90)
    st = o.state()
    assert abs(st[1, 14] - 0.3) < 0.02, st[1, 14]
    m = o.manifolds()
    assert len(m) == 1 and int(m[0, 2]) == 4  # the plane's square clipped against the box face


def test_oracle_plane_rays_and_points(oracle_lib):
    b = plane_and("sphere", 0.2, (5.0, 5.0, 5.0))
    o = pyoracle.OracleWorld(world.standard_settings(), b)
    o.step(0.0, 1)
    rays = np.array([[0.0, 2.0, 0.0, 0.0, -1.0, 0.0, 10.0],         # straight down: 2 m
                     [0.0, 2.0, 0.0, 0.6, -0.8, 0.0, 10.0],         # slanted: 2 / 0.8 m
                     [0.0, 2.0, 0.0, 0.0, 1.0, 0.0, 10.0],          # away (a back face): miss
                     [0.0, -1.0, 0.0, 0.0, -1.0, 0.0, 10.0]])       # from inside, solid: 0
    fr, bo, _ = o.cast_rays(rays)
    assert list(bo) == [0, 0, -1, 0]
    np.testing.assert_allclose(fr[[0, 1, 3]] * 10.0, [2.0, 2.5, 0.0], atol=1e-12)
    co, _, _ = o.collide_points(np.array([[1.0, -0.01, 2.0], [1.0, 0.01, 2.0]]))
    assert list(co) == [1, 0]


def test_oracle_empty_body_and_given_mass(oracle_lib):
    lib = pyoracle.load()
    # an empty body: no pairs reach a manifold, and a dynamic one with a given mass falls freely
    b = scenes.blank_bodies(3)
    scenes.set_box(b, 0, (1.0, 1.0, 1.0))
    b["motion_type"][0] = _lib.STATIC
    b["object_layer"][0] = scenes.LAYER_NOT_MOVING
    scenes.set_empty(b, 1)
    b["position"][1] = (0.0, 0.5, 0.0)
    b["mass_properties_mode"][1] = _lib.MASS_GIVEN
    b["mass"][1] = 3.0
    b["linear_damping"][1] = 0.0
    b["allow_sleeping"][1] = 0
    scenes.set_sphere(b, 2, 0.3)
    b["position"][2] = (0.0, 0.5, 0.0)
    b["motion_type"][2] = _lib.STATIC
    b["object_layer"][2] = scenes.LAYER_NOT_MOVING
    o = pyoracle.OracleWorld(world.standard_settings(), b)
    o.step(1.0 / 60.0, 30)
    st = o.state()
    t = 30 / 60.0
    assert abs(st[1, 1] - (0.5 - 0.5 * 9.81 * t * (t + 1 / 60.0))) < 1e-9
    assert len(o.manifolds()) == 0
    # a given mass scales the inverse inertia by m0 / m; a given tensor is used as is
    box = scenes.blank_bodies(1)
    scenes.set_box(box, 0, (0.5, 0.25, 0.125))
    out0, out1, out2 = np.zeros(9), np.zeros(9), np.zeros(9)
    lib.orc_inverse_inertia(pyoracle.dptr(row(box)), pyoracle.dptr(out0))
    box["mass_properties_mode"][0] = _lib.MASS_GIVEN
    box["mass"][0] = 25.0
    lib.orc_inverse_inertia(pyoracle.dptr(row(box)), pyoracle.dptr(out1))
    m0 = 1.0 * 0.5 * 0.25 * 1000.0
    np.testing.assert_allclose(out1, out0 * m0 / 25.0, rtol=1e-12)
    box["mass_properties_mode"][0] = _lib.MASS_AND_INERTIA_GIVEN
    box["inertia"][0] = (2.0, 0.0, 0.0, 3.0, 0.0, 4.0)
    lib.orc_inverse_inertia(pyoracle.dptr(row(box)), pyoracle.dptr(out2))
    np.testing.assert_allclose(np.sort(np.linalg.eigvalsh(out2.reshape(3, 3))), [0.25, 1 / 3, 0.5], rtol=1e-12)


def test_oracle_plane_drop_settles(oracle_lib):
    sc = scenes.plane_drop()
    o = pyoracle.OracleWorld(world.standard_settings(), sc.bodies)
    o.step(sc.dt, sc.steps)
    st = o.state()
    n = np.array([-math.sin(math.radians(10.0)), math.cos(math.radians(10.0)), 0.0])
    # every body above the plane (its centre of mass at least 0.05 m over it)
    assert (st[2:, 13:16] @ n).min() > 0.05


# ---------------------------------------------------------------------------
# the GPU path against the oracle
# ---------------------------------------------------------------------------
def gpu_and_oracle(sc):
    ws = world.standard_settings()
    g = world.GpuWorld(ws, sc.n + 16)
    g.add_bodies(sc.bodies)
    o = pyoracle.OracleWorld(ws, sc.bodies)
    return g, o


@pytest.mark.gpu
def test_plane_drop_pairs_and_contacts(gpu_lib, oracle_lib):
    sc = scenes.plane_drop(n=80, seed=10)
    sc.bodies["position"][2:, 1] -= 0.45  # most bodies start touching the plane
    g, o = gpu_and_oracle(sc)
    g.step(0.0, 1)
    o.step(0.0, 1)
    gp = {tuple(sorted(p)) for p in g.get_pairs().tolist()}
    op = {tuple(sorted(p)) for p in o.pairs().tolist()}
    assert gp == op
    gm = {(int(r[0]), int(r[1])): r for r in g.get_manifolds()}
    om = {(int(r[0]), int(r[1])): r for r in o.manifolds()}
    common = set(gm) & set(om)
    assert len(common) >= 0.97 * max(len(gm), len(om)) and len(common) > 10
    bad = sum(1 for k in common if np.abs(gm[k][3:6] - om[k][3:6]).max() > 1e-3 or abs(gm[k][6] - om[k][6]) > 2e-3)
    assert bad <= 0.03 * len(common), (bad, len(common))


@pytest.mark.gpu
def test_plane_bodies_track_oracle(gpu_lib, oracle_lib):
    """Bodies dropped one by one on a 3 m grid onto the tilted plane (90 steps): 90 % of the
    positions and centres of mass within 2e-3 m of the oracle's, all within 3 cm (a body that
    lands on an edge and slides down the 10 degree slope carries the last bits of FP32 against
    FP64 contact impulses along with it)."""
    sc = scenes.plane_drop(n=25, seed=11, grid=3.0)
    g, o = gpu_and_oracle(sc)
    for _ in range(3):
        g.step(sc.dt, 30)
        o.step(sc.dt, 30)
        rows, _ = g.get_state()
        st = o.state()
        for cols in (slice(0, 3), slice(13, 16)):
            err = np.abs(rows[:, cols] - st[:, cols]).max(axis=1)
            assert np.quantile(err, 0.9) < 2e-3 and err.max() < 3e-2, np.sort(err)[-5:]


@pytest.mark.gpu
def test_plane_and_empty_queries(gpu_lib, oracle_lib):
    b = plane_and("sphere", 0.2, (5.0, 5.0, 5.0))
    b = np.concatenate([b, scenes.blank_bodies(1)])
    scenes.set_empty(b, 2)
    b["motion_type"][2] = _lib.STATIC
    b["object_layer"][2] = scenes.LAYER_NOT_MOVING
    b["position"][2] = (0.0, 1.0, 0.0)
    g = world.GpuWorld(world.standard_settings(), 8)
    g.add_bodies(b)
    o = pyoracle.OracleWorld(world.standard_settings(), b)
    g.step(0.0, 1)
    o.step(0.0, 1)
    rays = np.array([[0.0, 2.0, 0.0, 0.0, -1.0, 0.0, 10.0], [0.0, 2.0, 0.0, 0.6, -0.8, 0.0, 10.0],
                     [0.0, 2.0, 0.0, 0.0, 1.0, 0.0, 10.0], [0.0, -1.0, 0.0, 0.0, -1.0, 0.0, 10.0]])
    hits = g.cast_rays(rays)
    fr, bo, _ = o.cast_rays(rays)
    assert (hits["body"] == bo).all()
    np.testing.assert_allclose(hits["fraction"][bo >= 0], fr[bo >= 0], atol=2e-3)
    pts = np.array([[1.0, -0.01, 2.0], [1.0, 0.01, 2.0], [0.0, 1.0, 0.0]])
    gh = g.collide_points(pts)
    co, _, _ = o.collide_points(pts)
    assert (gh["count"] == co).all() and list(co) == [1, 0, 0]
