"""Continuous collision detection for LINEAR_CAST bodies (update.ts:896-1670, ccd.ts): the oracle
against the reference's own tests and against mechanics (CPU), the GPU path against the oracle.

The reference's tst/ccd.test.ts holds two cases, restated here on the oracle and on the GPU:
a 200 m/s bullet ends short of a thin wall, and a bullet that starts against a wall raises an
added-contact event and ends short of the wall.  The oracle is pinned further by what the
algorithm must give: a bullet that tunnels discretely stops at the wall face (radius and the
penetration allowance from it), a restitution of 0.6 returns 0.6 of the normal speed, a body
below the cast threshold moves exactly as a discrete one.

GPU tolerances (FP32 device state against the FP64 oracle, the same scene):
  * cast counts per step: equal;
  * the gallery, every step for the first 8 steps: positions within 5e-3 m, velocities within
    5e-2 m/s (restitution and friction impulses of single iterations).
"""
import math

import numpy as np
import pytest

from crashcat_gb300 import _lib, scenes, world
from oracle import pyoracle


def wall_and_bullet(wall_half, wall_pos, radius, pos, vel, mq=1):
    b = scenes.blank_bodies(2)
    scenes.set_box(b, 0, wall_half)
    b["motion_type"][0] = _lib.STATIC
    b["object_layer"][0] = scenes.LAYER_NOT_MOVING
    b["position"][0] = wall_pos
    scenes.set_sphere(b, 1, radius)
    b["position"][1] = pos
    b["linear_velocity"][1] = vel
    b["motion_quality"][1] = mq
    return b


def reference_case_1(mq=1):
    """tst/ccd.test.ts:7-54: a 0.2 m sphere at 200 m/s from x = -10 toward a static box of half
    extents (5, 5, 0.1) at the origin, one step of 1/60 s."""
    return wall_and_bullet((5.0, 5.0, 0.1), (0.0, 0.0, 0.0), 0.2, (-10.0, 0.0, 0.0), (200.0, 0.0, 0.0), mq)


def reference_case_2():
    """tst/ccd.test.ts:56-108: a 0.3 m sphere at 100 m/s from x = -5 toward a static box of half
    extents (5, 5, 0.5) at the origin."""
    return wall_and_bullet((5.0, 5.0, 0.5), (0.0, 0.0, 0.0), 0.3, (-5.0, 0.0, 0.0), (100.0, 0.0, 0.0))


def thin_wall(mq, v=120.0, restitution=0.0):
    """A 0.2 m sphere at v m/s toward a static wall 10 cm thick at x = 5, no gravity."""
    b = wall_and_bullet((0.05, 2.0, 2.0), (5.0, 2.0, 0.0), 0.2, (0.0, 2.0, 0.0), (v, 0.0, 0.0), mq)
    b["gravity_factor"][1] = 0.0
    b["restitution"][1] = restitution
    return b


def oracle_of(b, hulls=(), num_worlds=1):
    ws = world.standard_settings()
    ws.num_worlds = num_worlds
    return pyoracle.OracleWorld(ws, b, hulls)


# ---------------------------------------------------------------------------
# the oracle (CPU)
# ---------------------------------------------------------------------------
def test_oracle_reference_case_1(oracle_lib):
    o = oracle_of(reference_case_1())
    o.step(1.0 / 60.0, 1)
    st = o.state()
    assert -10.0 < st[1, 0] < 0.5
    assert st[1, 7] != 200.0


def test_oracle_reference_case_2(oracle_lib):
    o = oracle_of(reference_case_2())
    o.step(1.0 / 60.0, 1)
    st = o.state()
    ev = o.contact_events()
    assert any(1 in pair for pair in ev["added"])  # onContactAdded with the bullet
    assert st[1, 0] < 0.5 and abs(st[1, 0]) < 10.0


def test_oracle_stops_at_the_wall_face(oracle_lib):
    # discrete: the sphere passes the wall within two steps; cast: it stops at the face
    od = oracle_of(thin_wall(0))
    oc = oracle_of(thin_wall(1))
    for _ in range(4):
        od.step(1.0 / 60.0, 1)
        oc.step(1.0 / 60.0, 1)
    assert od.state()[1, 0] > 6.0
    st = oc.state()
    # face at 4.95; the centre stops one radius before it plus the allowance min(slop, 0.25 r)
    assert abs(st[1, 0] - (4.95 - 0.2 + 0.02)) < 1e-6, st[1, 0]
    assert abs(st[1, 7]) < 1e-9
    assert oc.ccd_counts() == (0, 0)  # at rest: below the cast threshold


def test_oracle_restitution(oracle_lib):
    o = oracle_of(thin_wall(1, v=120.0, restitution=0.6))
    vx = None
    for k in range(1, 4):
        o.step(1.0 / 60.0, 1)
        if o.ccd_counts()[1]:
            vx = o.state()[1, 7]
            break
    # the speed at the hit: damped once per step so far (accelerationIntegrationUpdate)
    v_in = 120.0 * (1.0 - 0.05 / 60.0) ** k
    # (the cast normal is within the GJK tolerance of the wall normal)
    assert vx is not None and abs(vx - (-0.6 * v_in)) < 1e-4, vx


def test_oracle_below_threshold_is_discrete(oracle_lib):
    sc = scenes.box_stack(height=4)
    a = oracle_of(sc.bodies)
    bq = sc.bodies.copy()
    bq["motion_quality"] = 1
    c = oracle_of(bq)
    for _ in range(40):
        a.step(sc.dt, 1)
        c.step(sc.dt, 1)
        # resting boxes move far less than 0.05 x 0.5 m per step
    np.testing.assert_array_equal(a.state(), c.state())


def test_oracle_gallery_mechanics(gpu_lib, oracle_lib):
    sc = scenes.ccd_gallery()
    hulls = [_lib.build_convex_hull(p) for p in sc.hull_points]
    o = oracle_of(sc.bodies, hulls)
    o.step(sc.dt, sc.steps)
    st = o.state()
    # no bullet went through the wall (x = 8 +- 0.05)
    for i in (2, 3, 4, 5, 6):
        assert st[i, 0] < 8.0, (i, st[i, 0])
    assert st[7, 7] < -50.0  # the bouncing bullet returns
    assert st[8, 7] > 0.5  # the box was pushed
    # the head-on pair: the lower index casts the pair and the impulse stops both; the other
    # record has no hit of its own and still moves its whole displacement (update.ts:1626-1633)
    assert abs(st[10, 7]) < 1.0 and abs(st[11, 7]) < 1.0


# ---------------------------------------------------------------------------
# the GPU path against the oracle
# ---------------------------------------------------------------------------
def gpu_and_oracle(sc):
    ws = world.standard_settings()
    ws.num_worlds = sc.num_worlds
    g = world.GpuWorld(ws, sc.n + 16)
    for p in sc.hull_points or ():
        g.add_convex_hull(p)
    g.add_bodies(sc.bodies)
    hulls = [g.get_convex_hull(i) for i in range(len(sc.hull_points or ()))]
    o = pyoracle.OracleWorld(ws, sc.bodies, hulls)
    return g, o


@pytest.mark.gpu
@pytest.mark.parametrize("case", [reference_case_1, reference_case_2])
def test_reference_cases_gpu(gpu_lib, oracle_lib, case):
    b = case()
    sc = scenes.Scene("case", b, dt=1.0 / 60.0, steps=1)
    g, o = gpu_and_oracle(sc)
    g.step(sc.dt, 1)
    o.step(sc.dt, 1)
    rows, _ = g.get_state()
    st = o.state()
    assert rows[1, 0] < 0.5
    np.testing.assert_allclose(rows[:, 0:3], st[:, 0:3], atol=5e-3)
    np.testing.assert_allclose(rows[:, 7:10], st[:, 7:10], atol=5e-2)


@pytest.mark.gpu
@pytest.mark.parametrize("restitution", [0.0, 0.6])
def test_thin_wall_gpu(gpu_lib, oracle_lib, restitution):
    sc = scenes.Scene("wall", thin_wall(1, restitution=restitution), dt=1.0 / 60.0, steps=4)
    g, o = gpu_and_oracle(sc)
    for _ in range(4):
        g.step(sc.dt, 1)
        o.step(sc.dt, 1)
        s = g.stats()
        assert (s["num_ccd"], s["num_ccd_hits"]) == o.ccd_counts()
        rows, _ = g.get_state()
        st = o.state()
        np.testing.assert_allclose(rows[:, 0:3], st[:, 0:3], atol=5e-3)
        np.testing.assert_allclose(rows[:, 7:10], st[:, 7:10], atol=5e-2)


@pytest.mark.gpu
@pytest.mark.parametrize("num_worlds", [1, 3])
def test_gallery_parity(gpu_lib, oracle_lib, num_worlds):
    """Every world of a batched handle against a single-world oracle of its own bodies (the
    oracle holds one world, as the reference does)."""
    sc = scenes.ccd_gallery(num_worlds=num_worlds)
    ws = world.standard_settings()
    ws.num_worlds = num_worlds
    g = world.GpuWorld(ws, sc.n + 16)
    for p in sc.hull_points:
        g.add_convex_hull(p)
    g.add_bodies(sc.bodies)
    oracles, members = [], []
    for wd in range(num_worlds):
        idx = np.nonzero(sc.bodies["world"] == wd)[0]
        sub = sc.bodies[idx].copy()
        sub["world"] = 0
        sub["shape_params"][sub["shape_type"] == _lib.SHAPE_CONVEX_HULL, 0] = 0.0
        oracles.append(pyoracle.OracleWorld(world.standard_settings(), sub, [g.get_convex_hull(wd)]))
        members.append(idx)
    cast_steps = 0
    for k in range(sc.steps):
        g.step(sc.dt, 1)
        counts = np.zeros(2, dtype=int)
        rows, _ = g.get_state()
        for o, idx in zip(oracles, members):
            o.step(sc.dt, 1)
            counts += o.ccd_counts()
            st = o.state()
            np.testing.assert_allclose(rows[idx, 0:3], st[:, 0:3], atol=5e-3, err_msg=f"step {k}")
            np.testing.assert_allclose(rows[idx, 7:10], st[:, 7:10], atol=5e-2, err_msg=f"step {k}")
        s = g.stats()
        assert (s["num_ccd"], s["num_ccd_hits"]) == tuple(counts), k
        cast_steps += s["num_ccd_hits"] > 0
    assert cast_steps >= 2


@pytest.mark.gpu
def test_sleeping_target_is_woken(gpu_lib, oracle_lib):
    """A bullet that reaches a sleeping box wakes it (resolveCCDContacts update.ts:1664-1667)."""
    b = scenes.blank_bodies(3)
    scenes.static_floor(b, 0)
    scenes.set_box(b, 1, (0.5, 0.5, 0.5))
    b["position"][1] = (0.0, 0.5, 0.0)
    scenes.set_sphere(b, 2, 0.1)
    b["position"][2] = (-200.0, 0.5, 0.0)
    b["linear_velocity"][2] = (180.0, 0.0, 0.0)
    b["gravity_factor"][2] = 0.0
    b["allow_sleeping"][2] = 0
    b["motion_quality"][2] = 1
    sc = scenes.Scene("sleeper", b, dt=1.0 / 60.0, steps=80)
    g, o = gpu_and_oracle(sc)
    slept = False
    for k in range(80):
        g.step(sc.dt, 1)
        o.step(sc.dt, 1)
        _, gs = g.get_state()
        slept = slept or bool(gs[1])
        rows, _ = g.get_state()
        np.testing.assert_allclose(rows[:, 0:3], o.state()[:, 0:3], atol=5e-3, err_msg=f"step {k}")
    assert slept
    rows, gs = g.get_state()
    assert not gs[1] and rows[1, 7] > 0.1
