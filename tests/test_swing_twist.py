"""Swing-twist joints (src/constraints/swing-twist-constraint.ts) and the jointed ragdolls
built from them: the oracle against the limits it must hold (CPU), the GPU path against the
oracle.

The reference ships no swing-twist test with expected values, so the oracle is pinned by
its limits: a cone holds its half angle, a locked twist stays locked, a velocity motor
reaches its target, and ragdolls stay assembled and come to rest.

GPU tolerances (FP32 device state against the FP64 oracle):
  * swing-twist chains, first 15 steps: positions within 2e-3 m; after 90 steps (chaotic)
    the swing and twist angles stay within the same bounds past the limits as the oracle's
    (6 degrees past the cone, 9 degrees past the twist limits);
  * twist motor: angular velocity within 1e-2 rad/s of the oracle;
  * four ragdolls, first 20 steps: positions within 5e-3 m; after 240 steps at rest:
    joint gaps below 3 cm, speeds below 0.5 m/s, mean height within 5 cm of the oracle.
"""
import math

import numpy as np
import pytest

from crashcat_gb300 import _lib, scenes, world
from oracle import pyoracle


def settings_of(sc):
    ws = world.standard_settings(velocity_iterations=sc.velocity_iterations,
                                 position_iterations=sc.position_iterations)
    ws.num_worlds = sc.num_worlds
    return ws


def oracle_of(sc):
    o = pyoracle.OracleWorld(settings_of(sc), sc.bodies)
    for h in sc.hinges if sc.hinges is not None else ():
        o.add_hinge_record(h)
    for h in sc.swings if sc.swings is not None else ():
        o.add_swing_twist_record(h)
    o.set_skip_joint_pairs(sc.skip_joint_pairs)
    return o


def gpu_of(sc):
    g = world.GpuWorld(settings_of(sc), sc.n + 16)
    g.add_bodies(sc.bodies)
    if sc.hinges is not None:
        g.add_hinges(sc.hinges)
    if sc.swings is not None:
        g.add_swing_twists(sc.swings)
    g.set_skip_joint_pairs(sc.skip_joint_pairs)
    return g


def qmul(a, b):
    ax, ay, az, aw = a
    bx, by, bz, bw = b
    return np.array([aw * bx + ax * bw + ay * bz - az * by, aw * by - ax * bz + ay * bw + az * bx,
                     aw * bz + ax * by - ay * bx + az * bw, aw * bw - ax * bx - ay * by - az * bz])


def rotate(q, v):
    u = np.asarray(q[:3], dtype=np.float64)
    t = 2.0 * np.cross(u, v)
    return v + q[3] * t + np.cross(u, t)


def chain_angles(st, chains=4, links=5):
    """Per joint between consecutive links (the anchor joints excluded): the swing angle
    between the links' long axes and the twist about the long axis, degrees."""
    sw, tw = [], []
    for c in range(chains):
        base = c * (links + 1)
        for i in range(1, links):
            qa, qb = st[base + i, 3:7], st[base + 1 + i, 3:7]
            rel = qmul(qa * np.array([-1, -1, -1, 1.0]), qb)  # b relative to a, in a's frame
            if rel[3] < 0:
                rel = -rel
            sw.append(math.degrees(math.acos(np.clip(rotate(rel, np.array([0, 1.0, 0]))[1], -1, 1))))
            tw.append(math.degrees(2 * math.atan2(rel[1], rel[3])))
    return np.array(sw).reshape(chains, links - 1), np.array(tw).reshape(chains, links - 1)


def joint_gaps(sc, st):
    out = []
    for recs, fa, fb in ((sc.hinges, "point_a", "point_b"), (sc.swings, "position_a", "position_b")):
        if recs is None:
            continue
        for h in recs:
            p = []
            for body, f in ((h["body_a"], fa), (h["body_b"], fb)):
                q0 = sc.bodies["quaternion"][body].astype(np.float64)
                local = rotate(q0 * np.array([-1, -1, -1, 1.0]), h[f] - sc.bodies["position"][body])
                p.append(st[body, 0:3] + rotate(st[body, 3:7].astype(np.float64), local))
            out.append(np.linalg.norm(p[0] - p[1]))
    return np.array(out)


def twist_motor_scene():
    b = scenes.blank_bodies(2)
    scenes.set_box(b, 0, (0.1, 0.1, 0.1))
    b["motion_type"][0] = _lib.STATIC
    b["object_layer"][0] = scenes.LAYER_NOT_MOVING
    b["position"][0] = (0.0, 5.0, 0.0)
    scenes.set_box(b, 1, (0.2, 0.6, 0.3))
    b["position"][1] = (0.0, 4.4, 0.0)
    b["allow_sleeping"] = 0
    s = _lib.swing_twist_defaults(1)
    s["body_a"], s["body_b"] = 0, 1
    s["position_a"] = s["position_b"] = (0.0, 5.0, 0.0)
    s["twist_axis_a"] = s["twist_axis_b"] = (0.0, -1.0, 0.0)
    s["plane_axis_a"] = s["plane_axis_b"] = (0.0, 0.0, 1.0)
    s["normal_half_cone_angle"] = s["plane_half_cone_angle"] = math.radians(20.0)
    s["twist_min_angle"], s["twist_max_angle"] = -math.pi, math.pi
    s["twist_motor_state"] = _lib.MOTOR_VELOCITY
    s["target_angular_velocity"] = (2.0, 0.0, 0.0)
    return scenes.Scene("twist_motor", b, dt=1.0 / 60.0, steps=60, swings=s)


# ---------------------------------------------------------------------------
# the oracle against its limits (CPU)
# ---------------------------------------------------------------------------
def test_oracle_cone_and_twist_limits_hold(oracle_lib):
    sc = scenes.swing_twist_chains()
    o = oracle_of(sc)
    worst_sw = np.zeros((4, 4))
    worst_tw = np.zeros((4, 4))
    for _ in range(90):
        o.step(sc.dt, 1)
        sw, tw = chain_angles(o.state())
        worst_sw = np.maximum(worst_sw, sw)
        worst_tw = np.maximum(worst_tw, np.abs(tw))
    # the 30 degree cone engages and holds (a swing into it overshoots by up to a step)
    assert 27.0 < worst_sw[0].max() < 36.0, worst_sw[0]
    # the elliptic cone (20 / 50 degrees) allows more than the 30 degree cone
    assert worst_sw[1].max() > worst_sw[0].max()
    # the +-15 degree twist limits engage and hold (within the same overshoot); the locked
    # twist stays near zero
    assert 15.0 < worst_tw[:3].max() < 24.0, worst_tw
    assert worst_tw[3].max() < 6.0, worst_tw[3]


def test_oracle_twist_motor_reaches_target(oracle_lib):
    sc = twist_motor_scene()
    o = oracle_of(sc)
    o.step(sc.dt, 60)
    st = o.state()
    # twist axis is -Y: the motor drives body B about -Y at 2 rad/s
    assert abs(st[1, 11] - (-2.0)) < 1e-3, st[1, 10:13]


def test_oracle_ragdolls_stay_assembled_and_settle(oracle_lib):
    sc = scenes.ragdolls(num=4, arena=12.0)
    o = oracle_of(sc)
    o.step(sc.dt, 240)
    st = o.state()
    assert joint_gaps(sc, st).max() < 0.03
    assert np.abs(st[6:, 7:10]).max() < 0.5
    assert st[6:, 1].min() > 0.0  # above the floor


# ---------------------------------------------------------------------------
# the GPU path against the oracle
# ---------------------------------------------------------------------------
@pytest.mark.gpu
def test_swing_twist_chains_parity(gpu_lib, oracle_lib):
    sc = scenes.swing_twist_chains()
    g, o = gpu_of(sc), oracle_of(sc)
    g.step(sc.dt, 15)
    o.step(sc.dt, 15)
    rows, _ = g.get_state()
    np.testing.assert_allclose(rows[:, 0:3], o.state()[:, 0:3], atol=2e-3)
    worst = np.zeros((4, 4))
    for _ in range(75):
        g.step(sc.dt, 1)
        sw, tw = chain_angles(g.get_state()[0].astype(np.float64))
        worst = np.maximum(worst, sw)
        assert np.abs(tw[:3]).max() < 24.0 and np.abs(tw[3]).max() < 6.0
    assert worst[0].max() < 36.0


@pytest.mark.gpu
def test_swing_twist_motor_parity(gpu_lib, oracle_lib):
    sc = twist_motor_scene()
    g, o = gpu_of(sc), oracle_of(sc)
    g.step(sc.dt, 60)
    o.step(sc.dt, 60)
    rows, _ = g.get_state()
    np.testing.assert_allclose(rows[1, 10:13], o.state()[1, 10:13], atol=1e-2)


@pytest.mark.gpu
def test_ragdolls_parity(gpu_lib, oracle_lib):
    sc = scenes.ragdolls(num=4, arena=12.0)
    g, o = gpu_of(sc), oracle_of(sc)
    g.step(sc.dt, 20)
    o.step(sc.dt, 20)
    rows, _ = g.get_state()
    np.testing.assert_allclose(rows[:, 0:3], o.state()[:, 0:3], atol=5e-3)
    g.step(sc.dt, 220)
    o.step(sc.dt, 220)
    rows, _ = g.get_state()
    st = o.state()
    assert joint_gaps(sc, rows.astype(np.float64)).max() < 0.03
    assert np.abs(rows[6:, 7:10]).max() < 0.5
    assert abs(rows[6:, 1].mean() - st[6:, 1].mean()) < 0.05


@pytest.mark.gpu
def test_swing_twist_setters(gpu_lib):
    sc = twist_motor_scene()
    g = gpu_of(sc)
    g.step(sc.dt, 30)
    # the motor off and the joint disabled: the body falls freely
    g.set_swing_twist_motor(0, _lib.MOTOR_OFF, _lib.MOTOR_OFF)
    g.set_swing_twist_enabled(0, False)
    rows, _ = g.get_state()
    y0, vy0, t = float(rows[1, 1]), float(rows[1, 8]), 30 * sc.dt
    g.step(sc.dt, 30)
    rows2, _ = g.get_state()
    damp = (1 - 0.05 * sc.dt) ** 30  # default linear damping
    assert rows2[1, 1] < y0 + vy0 * t - 0.5 * 9.81 * t * t * 0.9 * damp
    with pytest.raises(_lib.CCError):
        g.set_swing_twist_limits(5, 0.1, 0.1, -0.1, 0.1)


def test_random_ragdoll_poses_start_inside_their_limits(oracle_lib):
    """Ragdolls spawned at seeded random joint poses (each joint turned inside its limits, the
    joints created in that pose): with gravity off nothing moves over 10 steps, so no hinge or
    swing-twist limit and no contact pushes at spawn, and the joints hold; the pose differs from
    the rest pose."""
    sc = scenes.ragdolls(num=8, arena=12.0, spacing=5.0)
    ws = settings_of(sc)
    ws.gravity_enabled = False
    o = pyoracle.OracleWorld(ws, sc.bodies)
    for h in sc.hinges:
        o.add_hinge_record(h)
    for h in sc.swings:
        o.add_swing_twist_record(h)
    o.set_skip_joint_pairs(True)
    st0 = o.state()
    o.step(sc.dt, 10)
    st = o.state()
    assert np.abs(st[:, 0:3] - st0[:, 0:3]).max() < 1e-5
    assert joint_gaps(sc, st).max() < 1e-4
    rest = scenes.ragdolls(num=8, arena=12.0, spacing=5.0, random_poses=False).bodies["position"]
    moved = np.linalg.norm(rest[6:] - sc.bodies["position"][6:], axis=1)
    assert (moved > 0.05).mean() > 0.5
