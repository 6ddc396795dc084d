"""Hinge joints (src/constraints/hinge-constraint.ts): the oracle's restatement checked
against closed-form mechanics on the CPU, and the GPU path against the oracle.

The reference ships no hinge test with expected values (its tests cover constraint
ids only), so the oracle is pinned by physics: the small-angle period of a hinged
pendulum, hard limits that hold, a velocity motor that reaches its target, and the
joint-pair filter that removes exactly the joined pairs.

GPU tolerances (FP32 device state against the FP64 oracle):
  * motors scene, 90 steps: angular velocity within 2e-2 rad/s, hinge angle within
    5e-3 rad (the position motors settle against gravity; friction and velocity
    motors saturate at their limits);
  * hinge chains, first 20 steps: positions within 2e-3 m; after 60 steps the
    unlimited chains (double pendulums and longer, chaotic) are compared only through
    joint separation (pivot gap below 5 cm, as the oracle's own);
  * broadphase pairs with the joint-pair filter: bit-exact.
"""
import math

import numpy as np
import pytest

from crashcat_gb300 import _lib, scenes, world
from oracle import pyoracle


def oracle_of(sc, **settings):
    ws = world.standard_settings(**settings)
    ws.num_worlds = sc.num_worlds
    o = pyoracle.OracleWorld(ws, sc.bodies)
    for h in sc.hinges:
        o.add_hinge_record(h)
    o.set_skip_joint_pairs(sc.skip_joint_pairs)
    return o


def gpu_of(sc, **settings):
    ws = world.standard_settings(**settings)
    ws.num_worlds = sc.num_worlds
    g = world.GpuWorld(ws, sc.n + 16)
    g.add_bodies(sc.bodies)
    g.add_hinges(sc.hinges)
    g.set_skip_joint_pairs(sc.skip_joint_pairs)
    return g


def rotate(q, v):
    u = q[..., 0:3]
    t = 2.0 * np.cross(u, v)
    return v + q[..., 3:4] * t + np.cross(u, t)


def pivot_gaps(sc, st):
    """World distance between each joint's two attachment points (local points taken from
    the initial poses)."""
    out = []
    b0 = sc.bodies
    for h in sc.hinges:
        pa = []
        for body, p in ((h["body_a"], h["point_a"]), (h["body_b"], h["point_b"])):
            q0 = b0["quaternion"][body].astype(np.float64)
            local = rotate(q0 * np.array([-1, -1, -1, 1.0]), p - b0["position"][body])
            pa.append(st[body, 0:3] + rotate(st[body, 3:7].astype(np.float64), local))
        out.append(np.linalg.norm(pa[0] - pa[1]))
    return np.array(out)


def pendulum(theta0=math.radians(5.0), L=1.0, r=0.1):
    b = scenes.blank_bodies(2)
    scenes.set_box(b, 0, (0.05, 0.05, 0.05))
    b["motion_type"][0] = _lib.STATIC
    b["object_layer"][0] = scenes.LAYER_NOT_MOVING
    b["position"][0] = (0.0, 5.0, 0.0)
    scenes.set_sphere(b, 1, r)
    b["position"][1] = (L * math.sin(theta0), 5.0 - L * math.cos(theta0), 0.0)
    b["linear_damping"] = 0.0
    b["angular_damping"] = 0.0
    b["allow_sleeping"] = 0
    h = _lib.hinge_defaults(1)
    h["body_a"], h["body_b"] = 0, 1
    h["point_a"] = h["point_b"] = (0.0, 5.0, 0.0)
    h["hinge_axis_a"] = h["hinge_axis_b"] = (0.0, 0.0, 1.0)
    h["normal_axis_a"] = h["normal_axis_b"] = (1.0, 0.0, 0.0)
    return scenes.Scene("pendulum", b, dt=1.0 / 240.0, steps=0, hinges=h)


# ---------------------------------------------------------------------------
# the oracle against mechanics (CPU)
# ---------------------------------------------------------------------------
def test_oracle_pendulum_period(oracle_lib):
    """Small-angle period 2 pi sqrt(I_pivot / (m g L)), I_pivot = 2/5 m r^2 + m L^2, within 1 %."""
    L, r = 1.0, 0.1
    sc = pendulum(L=L, r=r)
    o = oracle_of(sc)
    xs = []
    for _ in range(240 * 6):
        o.step(sc.dt, 1)
        xs.append(o.state()[1, 0])
    xs = np.array(xs)
    up = np.nonzero((xs[:-1] < 0) & (xs[1:] >= 0))[0]
    # interpolated upward zero crossings of x
    t = (up + (-xs[up]) / (xs[up + 1] - xs[up])) * sc.dt
    period = np.diff(t).mean()
    expect = 2 * math.pi * math.sqrt((0.4 * r * r + L * L) / (9.81 * L))
    assert abs(period - expect) < 0.01 * expect, (period, expect)
    st = o.state()
    assert abs(np.linalg.norm(st[1, 0:3] - (0.0, 5.0, 0.0)) - L) < 1e-3


def test_oracle_hard_limits_hold(oracle_lib):
    """Of three chains, the middle one has +-40 degree hard limits (the last one's are soft,
    the first is free).  The free chain bends past 60 degrees; the limited one reaches its
    limits and overshoots them by less than 10 degrees.  A limit only engages at setup when
    the angle is already past it (hinge-constraint.ts calculateLimitsConstraintProperties),
    so a joint swinging into it overshoots by up to one step of rotation before the velocity
    and position solves push it back."""
    sc = scenes.hinge_chains(num_chains=3, links=4)
    o = oracle_of(sc)

    def angles(st, hs):
        out = []
        for h in hs:
            qa, qb = st[h["body_a"], 3:7], st[h["body_b"], 3:7]
            za = 2 * math.atan2(qa[2], qa[3]) if h["body_a"] % 5 else 0.0  # anchors are static
            zb = 2 * math.atan2(qb[2], qb[3])
            out.append((zb - za + math.pi) % (2 * math.pi) - math.pi)
        return np.abs(out)

    free = limited = 0.0
    for _ in range(90):
        o.step(sc.dt, 1)
        st = o.state()
        free = max(free, angles(st, sc.hinges[0:4]).max())
        limited = max(limited, angles(st, sc.hinges[4:8]).max())
    assert free > math.radians(60.0)
    assert math.radians(39.0) < limited < math.radians(50.0), math.degrees(limited)


def test_oracle_velocity_motor_reaches_target(oracle_lib):
    sc = scenes.hinge_motors()
    o = oracle_of(sc)
    o.step(sc.dt, 60)
    st = o.state()
    assert abs(st[1, 12] - (-5.0)) < 1e-3  # uncapped velocity motor
    # the capped motor (200 N m) cannot hold the off-balance wing (353 N m of gravity)
    assert st[3, 12] < 0.0


def test_oracle_joint_pair_filter(oracle_lib):
    sc = scenes.hinge_chains(num_chains=1, links=4)
    o_on = oracle_of(sc)
    sc_off = scenes.hinge_chains(num_chains=1, links=4)
    sc_off.skip_joint_pairs = False
    o_off = oracle_of(sc_off)
    o_on.step(0.0, 1)
    o_off.step(0.0, 1)
    joined = {tuple(sorted((int(h["body_a"]), int(h["body_b"])))) for h in sc.hinges}
    on = {tuple(sorted(p)) for p in o_on.pairs().tolist()}
    off = {tuple(sorted(p)) for p in o_off.pairs().tolist()}
    assert joined & off  # neighbouring links overlap within the speculative distance
    assert off - on == joined & off
    assert not (on & joined)


# ---------------------------------------------------------------------------
# the GPU path against the oracle
# ---------------------------------------------------------------------------
@pytest.mark.gpu
def test_hinge_motors_parity(gpu_lib, oracle_lib):
    sc = scenes.hinge_motors()
    g, o = gpu_of(sc), oracle_of(sc)
    for _ in range(3):
        g.step(sc.dt, 30)
        o.step(sc.dt, 30)
        rows, _ = g.get_state()
        st = o.state()
        np.testing.assert_allclose(rows[1::2, 10:13], st[1::2, 10:13], atol=2e-2)
        ang_g = 2 * np.arctan2(rows[1::2, 5], rows[1::2, 6])
        ang_o = 2 * np.arctan2(st[1::2, 5], st[1::2, 6])
        d = (ang_g - ang_o + np.pi) % (2 * np.pi) - np.pi
        assert np.abs(d).max() < 5e-3, d
    # getCurrentAngle: the joint angle relative to the creation pose
    theta = g.hinge_angles(len(sc.hinges))
    ang0 = 2 * np.arctan2(sc.bodies["quaternion"][1::2, 2], sc.bodies["quaternion"][1::2, 3])
    ang = 2 * np.arctan2(rows[1::2, 5], rows[1::2, 6])
    rel = (ang - ang0 + np.pi) % (2 * np.pi) - np.pi
    has_theta = (sc.hinges["motor_state"] != 0) | (sc.hinges["max_friction_torque"] > 0) | \
        (sc.hinges["limits_max"] < np.pi)
    # theta is taken at setup, before this step's solve: one step of rotation behind
    wz = rows[1::2, 12]
    np.testing.assert_allclose(theta[has_theta], (rel - wz * sc.dt)[has_theta], atol=5e-3)


@pytest.mark.gpu
def test_hinge_chains_parity(gpu_lib, oracle_lib):
    sc = scenes.hinge_chains()
    g, o = gpu_of(sc), oracle_of(sc)
    g.step(sc.dt, 20)
    o.step(sc.dt, 20)
    rows, _ = g.get_state()
    st = o.state()
    np.testing.assert_allclose(rows[:, 0:3], st[:, 0:3], atol=2e-3)
    g.step(sc.dt, 40)
    o.step(sc.dt, 40)
    rows, _ = g.get_state()
    st = o.state()
    gaps_g, gaps_o = pivot_gaps(sc, rows.astype(np.float64)), pivot_gaps(sc, st)
    assert gaps_g.max() < 0.05 and gaps_o.max() < 0.05
    # the limited chains stay close to the oracle
    lim_bodies = np.unique(np.concatenate([[h["body_a"], h["body_b"]] for h in sc.hinges if h["limits_max"] < np.pi]))
    assert np.abs(rows[lim_bodies, 0:3] - st[lim_bodies, 0:3]).max() < 0.05


@pytest.mark.gpu
def test_joint_pair_filter_pairs_bit_exact(gpu_lib, oracle_lib):
    sc = scenes.hinge_chains(num_chains=3, links=5)
    g, o = gpu_of(sc), oracle_of(sc)
    g.step(0.0, 1)
    o.step(0.0, 1)
    gp = {tuple(sorted(p)) for p in g.get_pairs().tolist()}
    op = {tuple(sorted(p)) for p in o.pairs().tolist()}
    assert gp == op
    joined = {tuple(sorted((int(h["body_a"]), int(h["body_b"])))) for h in sc.hinges}
    assert not (gp & joined)


@pytest.mark.gpu
def test_hinge_pendulum_matches_oracle_and_setters(gpu_lib, oracle_lib):
    sc = pendulum(theta0=math.radians(30.0))
    g, o = gpu_of(sc), oracle_of(sc)
    g.step(sc.dt, 240)
    o.step(sc.dt, 240)
    rows, _ = g.get_state()
    np.testing.assert_allclose(rows[1, 0:3], o.state()[1, 0:3], atol=2e-3)
    # disabling the joint lets the bob fly freely: y0 + vy0 t - g t^2 / 2 (no damping)
    g.set_hinge_enabled(0, False)
    y0, vy0, t = float(rows[1, 1]), float(rows[1, 8]), 60 * sc.dt
    g.step(sc.dt, 60)
    rows2, _ = g.get_state()
    assert abs(rows2[1, 1] - (y0 + vy0 * t - 0.5 * 9.81 * t * t)) < 1e-2
    assert g.hinge_angles(1).shape == (1,)


@pytest.mark.gpu
def test_batched_worlds_with_joints(gpu_lib, oracle_lib):
    """Two worlds each holding the motors scene step like one world alone."""
    sc = scenes.hinge_motors()
    b = np.concatenate([sc.bodies, sc.bodies])
    b["world"][len(sc.bodies):] = 1
    h = np.concatenate([sc.hinges, sc.hinges])
    h["body_a"][len(sc.hinges):] += len(sc.bodies)
    h["body_b"][len(sc.hinges):] += len(sc.bodies)
    sc2 = scenes.Scene("two", b, dt=sc.dt, steps=0, num_worlds=2, hinges=h)
    g2, g1 = gpu_of(sc2), gpu_of(sc)
    g2.step(sc.dt, 45)
    g1.step(sc.dt, 45)
    r2, _ = g2.get_state()
    r1, _ = g1.get_state()
    np.testing.assert_allclose(r2[: len(sc.bodies)], r1, atol=1e-5)
    np.testing.assert_allclose(r2[len(sc.bodies):], r1, atol=1e-5)
