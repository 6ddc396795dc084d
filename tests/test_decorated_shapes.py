"""Shape decorators (src/shapes/transformed.ts, scaled.ts, offset-center-of-mass.ts), nested as
OffsetCenterOfMass(Transformed(Scaled(leaf))) in cc_body_desc.

The oracle is pinned by equivalences that follow from the reference's definitions:
  * collideTransformedVsShape passes the inner shape the composed pose (pos + q t, q r), so a
    transformed box collides exactly as a plain box at that pose;
  * a scaled box is a box of |s| times the half extents (setBoxSupport support.ts:343-372) and
    massProperties.scale gives that box's inertia;
  * an offset centre of mass moves no collision geometry, and massProperties.translate adds
    the parallel-axis term m (d.d E - d d^T) to the inertia;
  * a box laid on its side by a transform rests at the same height as the rotated plain box.

GPU tolerances against the oracle: on a pile of 200 decorated bodies broadphase pairs
bit-exact (the decorated local bounds are built in FP64 on both sides), manifold normals within
1e-3 and depths within 2e-3 for 97 % of the pairs; bodies that touch only the floor within
2e-3 m over 90 steps; a colliding pile's mean height within 5 cm after 120 steps.
"""
import math

import numpy as np
import pytest

from crashcat_gb300 import _lib, scenes, world
from oracle import pyoracle


def row(b):
    return np.ascontiguousarray(pyoracle.rows_from_bodies(b)[0])


def one(shape, params, pos=(0.0, 0.0, 0.0), quat=(0.0, 0.0, 0.0, 1.0), **deco):
    b = scenes.blank_bodies(1)
    if shape == "box":
        scenes.set_box(b, 0, params)
    elif shape == "sphere":
        scenes.set_sphere(b, 0, params)
    else:
        scenes.set_capsule(b, 0, *params)
    b["position"][0] = pos
    b["quaternion"][0] = quat
    for k, v in deco.items():
        b[k][0] = v
    return b


def inv_inertia(lib, b):
    out = np.zeros(9)
    lib.orc_inverse_inertia(pyoracle.dptr(row(b)), pyoracle.dptr(out))
    return out.reshape(3, 3)


def collide(lib, ba, bb, max_sep=0.0):
    out = np.zeros(13)
    lib.orc_collide_pair(pyoracle.dptr(row(ba)), pyoracle.dptr(row(bb)), max_sep, pyoracle.dptr(out))
    return out


ROT_Z90 = (0.0, 0.0, math.sin(math.pi / 4), math.cos(math.pi / 4))


def test_oracle_decorated_mass_properties(oracle_lib):
    lib = pyoracle.load()
    # a transform turning the box 90 degrees about Z swaps its X and Y extents
    # (the quaternion passes through an FP32 record: 1e-6)
    t = inv_inertia(lib, one("box", (1.0, 0.5, 0.25), shape_quaternion=ROT_Z90))
    np.testing.assert_allclose(t, inv_inertia(lib, one("box", (0.5, 1.0, 0.25))), rtol=1e-6, atol=1e-9)
    # a scaled box is the box of the scaled extents
    s = inv_inertia(lib, one("box", (0.5, 0.5, 0.5), shape_scale=(2.0, 1.0, 0.5)))
    np.testing.assert_allclose(s, inv_inertia(lib, one("box", (1.0, 0.5, 0.25))), rtol=1e-9, atol=1e-15)
    # a uniformly scaled sphere is the sphere of the scaled radius
    np.testing.assert_allclose(inv_inertia(lib, one("sphere", 0.25, shape_scale=(2.0, 2.0, 2.0))),
                               inv_inertia(lib, one("sphere", 0.5)), rtol=1e-9)
    # the offset centre of mass adds m (d.d E - d d^T)
    d = np.array([0.1, -0.2, 0.05], np.float32).astype(np.float64)  # as the FP32 records hold them
    h = np.array([0.4, 0.3, 0.2], np.float32).astype(np.float64)
    m = 8 * h.prod() * 1000.0
    I = np.diag([(h[1] ** 2 + h[2] ** 2), (h[0] ** 2 + h[2] ** 2), (h[0] ** 2 + h[1] ** 2)]) * (4 * m / 12)
    I = I + m * (d @ d * np.eye(3) - np.outer(d, d))
    np.testing.assert_allclose(inv_inertia(lib, one("box", tuple(h), com_offset=tuple(d))), np.linalg.inv(I),
                               rtol=1e-9, atol=1e-12)


def test_oracle_decorated_collisions(oracle_lib):
    lib = pyoracle.load()
    sphere = one("sphere", 0.5, pos=(0.9, 0.5, 0.1))
    q = np.array([0.1, 0.3, -0.2, 0.9])
    q /= np.linalg.norm(q)
    # a transformed box collides as the plain box at the composed pose
    tq = np.array([0.3, -0.1, 0.2, 0.92])
    tq /= np.linalg.norm(tq)
    tp = np.array([0.4, -0.2, 0.1])

    def qmul(a, b):
        return np.array([a[3] * b[0] + a[0] * b[3] + a[1] * b[2] - a[2] * b[1],
                         a[3] * b[1] - a[0] * b[2] + a[1] * b[3] + a[2] * b[0],
                         a[3] * b[2] + a[0] * b[1] - a[1] * b[0] + a[2] * b[3],
                         a[3] * b[3] - a[0] * b[0] - a[1] * b[1] - a[2] * b[2]])

    def rot(q, v):
        u = q[0:3]
        t = 2.0 * np.cross(u, v)
        return v + q[3] * t + np.cross(u, t)

    pose = np.array([0.2, 0.1, 0.0])
    dec = row(one("box", (0.8, 0.4, 0.3), pos=pose, quat=q, shape_position=tp, shape_quaternion=tq))
    # the plain box's row at the pose composed in FP64 from the record's own FP32 values
    plain = dec.copy()
    plain[7:10] = dec[7:10] + rot(dec[10:14], dec[36:39])
    plain[10:14] = qmul(dec[10:14], dec[39:43])
    plain[33:46] = 0.0
    hd, hp = np.zeros(13), np.zeros(13)
    lib.orc_collide_pair(pyoracle.dptr(dec), pyoracle.dptr(row(sphere)), 0.02, pyoracle.dptr(hd))
    lib.orc_collide_pair(pyoracle.dptr(plain), pyoracle.dptr(row(sphere)), 0.02, pyoracle.dptr(hp))
    assert hd[0] == 1
    np.testing.assert_allclose(hd, hp, rtol=0, atol=1e-12)
    # a scaled box collides as the box of the scaled extents
    # (its convex radius scales too: min(0.05 x 0.625, 0.05))
    sd = collide(lib, one("box", (0.5, 0.5, 0.5), pos=pose, quat=q, shape_scale=(1.25, 0.75, 0.625)), sphere, 0.02)
    plain_box = one("box", (0.625, 0.375, 0.3125), pos=pose, quat=q)
    plain_box["shape_params"][0, 3] = 0.05 * 0.625
    sp = collide(lib, plain_box, sphere, 0.02)
    np.testing.assert_allclose(sd, sp, atol=1e-6)
    # an offset centre of mass moves no geometry
    od = collide(lib, one("box", (0.625, 0.375, 0.3125), pos=pose, quat=q, com_offset=(0.2, 0.1, -0.1)), sphere,
                 0.02)
    np.testing.assert_allclose(od, collide(lib, one("box", (0.625, 0.375, 0.3125), pos=pose, quat=q), sphere, 0.02),
                               atol=1e-12)


def test_oracle_transformed_box_rests_like_the_rotated_box(oracle_lib):
    """A long box laid on its side by its transform comes to rest where the plain box of the
    turned extents does (centre of mass within 0.2 mm: the two runs differ only in rounding,
    the transformed one's support and face arithmetic running in the turned frame)."""
    floor = scenes.blank_bodies(1)
    scenes.set_box(floor, 0, (10.0, 0.5, 10.0))
    floor["motion_type"][0] = _lib.STATIC
    floor["object_layer"][0] = scenes.LAYER_NOT_MOVING
    floor["position"][0] = (0.0, -0.5, 0.0)
    ws = world.standard_settings()
    a = np.concatenate([floor, one("box", (1.0, 0.2, 0.3), pos=(0.0, 1.0, 0.0), shape_quaternion=ROT_Z90)])
    b = np.concatenate([floor, one("box", (0.2, 1.0, 0.3), pos=(0.0, 1.0, 0.0))])
    oa, ob = pyoracle.OracleWorld(ws, a), pyoracle.OracleWorld(ws, b)
    oa.step(1.0 / 60.0, 90)
    ob.step(1.0 / 60.0, 90)
    sa, sb = oa.state(), ob.state()
    np.testing.assert_allclose(sa[1, 13:16], sb[1, 13:16], atol=2e-4)
    assert abs(sa[1, 14] - 1.0) < 0.02  # resting on its 1 m half extent


def test_oracle_offset_com_keeps_geometry(oracle_lib):
    """A box with its centre of mass 0.3 m below its middle rests flat at the box's height:
    the position stays 0.25 m above the floor, the centre of mass 0.3 m lower."""
    floor = scenes.blank_bodies(1)
    scenes.set_box(floor, 0, (10.0, 0.5, 10.0))
    floor["motion_type"][0] = _lib.STATIC
    floor["object_layer"][0] = scenes.LAYER_NOT_MOVING
    floor["position"][0] = (0.0, -0.5, 0.0)
    body = one("box", (0.5, 0.25, 0.5), pos=(0.0, 0.5, 0.0), com_offset=(0.0, -0.3, 0.0))
    o = pyoracle.OracleWorld(world.standard_settings(), np.concatenate([floor, body]))
    o.step(1.0 / 60.0, 120)
    st = o.state()
    assert abs(st[1, 1] - 0.25) < 0.03, st[1, 1]
    assert abs(st[1, 14] - (st[1, 1] - 0.3)) < 1e-4


@pytest.mark.gpu
def test_scaled_hull_is_refused(gpu_lib):
    """A scaled convex hull has no baked form here: cc_world_add_bodies answers
    CC_ERR_UNSUPPORTED."""
    ws = world.standard_settings()
    g = world.GpuWorld(ws, 8)
    idx = g.add_convex_hull(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1]], np.float32) * 0.5)
    b = scenes.blank_bodies(1)
    scenes.set_hull(b, 0, idx)
    b["shape_scale"][0] = (2.0, 1.0, 1.0)
    with pytest.raises(_lib.CCError) as e:
        g.add_bodies(b)
    assert e.value.status == _lib.CC_ERR_UNSUPPORTED


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
def test_decorated_pile_pairs_and_contacts(gpu_lib, oracle_lib):
    sc = scenes.decorated_pile(n=200, seed=7, extent=3.0, heights=(0.3, 2.5))
    g, o = gpu_and_oracle(sc)
    g.step(0.0, 1)
    o.step(0.0, 1)
    gp = {tuple(sorted(p)) for p in g.get_pairs().tolist()}
    op = {tuple(sorted(p)) for p in o.pairs().tolist()}
    assert gp == op and len(gp) > 50
    gm = {(int(r[0]), int(r[1])): r for r in g.get_manifolds()}
    om = {(int(r[0]), int(r[1])): r for r in o.manifolds()}
    common = set(gm) & set(om)
    assert len(common) >= 0.97 * max(len(gm), len(om)) and len(common) > 20
    bad = sum(1 for k in common if np.abs(gm[k][3:6] - om[k][3:6]).max() > 1e-3 or abs(gm[k][6] - om[k][6]) > 2e-3)
    assert bad <= 0.03 * len(common), (bad, len(common))


@pytest.mark.gpu
def test_decorated_bodies_track_oracle(gpu_lib, oracle_lib):
    """Decorated bodies dropped one by one on a 3 m grid (no body touches another) while they
    fall, land, bounce and settle (90 steps): every position and centre of mass within 2e-3 m
    of the oracle's through the fall; after landing, 90 % of the bodies within 2e-3 m and all
    within 3 cm (a body landing on a corner or an edge tips one way or the other on the last
    bits of FP32 against FP64 contact impulses)."""
    sc = scenes.decorated_pile(n=36, seed=8, heights=(0.5, 2.0), grid=3.0)
    g, o = gpu_and_oracle(sc)
    g.step(sc.dt, 8)
    o.step(sc.dt, 8)
    rows, _ = g.get_state()
    st = o.state()
    np.testing.assert_allclose(rows[:, 0:3], st[:, 0:3], atol=2e-3)
    np.testing.assert_allclose(rows[:, 13:16], st[:, 13:16], atol=2e-3)
    for _ in range(3):
        g.step(sc.dt, 30)
        o.step(sc.dt, 30)
        rows, _ = g.get_state()
        st = o.state()
        for cols in (slice(0, 3), slice(13, 16)):
            err = np.abs(rows[:, cols] - st[:, cols]).max(axis=1)
            assert np.quantile(err, 0.9) < 2e-3 and err.max() < 3e-2, np.sort(err)[-5:]


@pytest.mark.gpu
def test_decorated_pile_settles(gpu_lib, oracle_lib):
    """120 steps of a pile of 60: finite state, nothing below the floor, and the mean height of
    the centres of mass within 5 cm of the oracle's (the bodies collide chaotically, so
    per-body positions are not compared)."""
    sc = scenes.decorated_pile(n=60, seed=8, extent=4.0, heights=(0.5, 3.0))
    g, o = gpu_and_oracle(sc)
    g.step(sc.dt, 120)
    o.step(sc.dt, 120)
    rows, _ = g.get_state()
    st = o.state()
    assert np.isfinite(rows).all()
    assert rows[1:, 14].min() > 0.0
    assert abs(rows[1:, 14].mean() - st[1:, 14].mean()) < 0.05
