"""Six-DOF joints (src/constraints/six-dof-constraint.ts): the oracle's restatement checked
against mechanics on the CPU, and the GPU path against the oracle.

The reference's tests for this joint cover creation and ids only, so the oracle is pinned by
physics on one scene of every axis configuration (crashcat_gb300.scenes.six_dof_zoo, 120 steps
at 60 Hz, 10/2 iterations):
  * locked (all six axes fixed): the cantilever keeps its pose within 2 cm / 0.02 rad;
  * ball (rotations free): the pendulum's pivot gap stays below 3 cm;
  * cone of 30 degrees: the swing reaches the limit and overshoots it by less than 3 degrees;
  * pyramid of 20 / 40 degrees: each pushed pendulum reaches its own limit, overshoot < 3
    degrees, and stays inside the other axis' limit;
  * prismatic on a 30 degree incline: rests at its 1 m limit, on its rail within 1 mm, unturned;
  * translation motors: the velocity motor moves at 2 m/s, the position motor settles at 0.5 m;
  * rotation motors: the velocity motor spins at 3 rad/s, the position motor settles at 45
    degrees of twist;
  * friction: 20 N decelerates the 64 kg box by 0.3125 m/s^2;
  * soft limit (2 Hz, damping 0.5): the hanging box settles g / omega^2 = 6.2 cm beyond its
    -0.1 m limit;
  * the free welded pair keeps its relative pose within 3 mm / 3e-3 rad.

GPU tolerances (FP32 device state against the FP64 oracle): each joint's 18 accumulated
impulses after the first step within 1e-3 relative (plus 1e-3 absolute); after 20 steps
positions within 2e-3 m and velocities within 2e-2 m/s; after 120 steps the same mechanical
bounds as the oracle's.
"""
import math

import numpy as np
import pytest

from crashcat_gb300 import _lib, scenes, world
from oracle import pyoracle

SD = _lib.JOINT_SIX_DOF


def oracle_of(sc, **settings):
    o = pyoracle.OracleWorld(world.standard_settings(**settings), sc.bodies)
    for t, recs in sc.joints.items():
        for r in recs:
            o.add_joint_record(t, r)
    o.set_skip_joint_pairs(sc.skip_joint_pairs)
    return o


def gpu_of(sc, **settings):
    g = world.GpuWorld(world.standard_settings(**settings), sc.n + 16)
    g.add_bodies(sc.bodies)
    for t, recs in sc.joints.items():
        idx = g.add_joints(t, recs)
        assert (idx == np.arange(len(recs))).all()
    g.set_skip_joint_pairs(sc.skip_joint_pairs)
    return g


def rotate(q, v):
    q = np.asarray(q, dtype=np.float64)
    u, w = q[:3], q[3]
    v = np.asarray(v, dtype=np.float64)
    return v + 2.0 * np.cross(u, np.cross(u, v) + w * v)


def qangle(q):
    """Rotation angle of a unit quaternion, radians."""
    return 2.0 * math.acos(min(1.0, abs(float(q[3]))))


def run(step, state, sc):
    hist = []
    for _ in range(sc.steps):
        step()
        hist.append(np.asarray(state(), dtype=np.float64).copy())
    return hist


def check_mechanics(sc, hist):
    R = sc.joints[SD]
    st = hist[-1]
    b0 = sc.bodies
    # locked cantilever
    b = R[0]["body_b"]
    assert np.abs(st[b, 0:3] - b0["position"][b]).max() < 2e-2 and qangle(st[b, 3:7]) < 2e-2
    # pendulums: pivot gap, swing angle from hanging straight down
    for k in range(1, 5):
        b = R[k]["body_b"]
        piv = R[k]["position_a"].astype(np.float64)
        gap, ang, sy, sz = 0.0, 0.0, 0.0, 0.0
        for h in hist:
            d = rotate(h[b, 3:7], (0.0, -1.0, 0.0))
            gap = max(gap, np.linalg.norm(h[b, 0:3] - 0.8 * d - piv))
            ang = max(ang, math.degrees(math.acos(np.clip(-d[1], -1.0, 1.0))))
            sz = max(sz, abs(math.degrees(math.atan2(d[0], -d[1]))))  # swing about Z: along world X
            sy = max(sy, abs(math.degrees(math.atan2(d[2], -d[1]))))  # swing about Y: along world Z
        assert gap < 3e-2, (k, gap)
        if k == 1:
            assert ang > 45.0  # the ball joint lets it swing past every limit below
        elif k == 2:
            assert 29.0 < ang < 33.0, ang
        elif k == 3:
            assert 39.0 < sz < 43.0 and sy < 21.0, (sz, sy)
        else:
            assert 19.0 < sy < 23.0 and sz < 41.0, (sy, sz)
    # prismatic at its 1 m limit down the incline
    b = R[5]["body_b"]
    ax = R[5]["axis_x_a"].astype(np.float64)
    u = st[b, 0:3] - b0["position"][b]
    assert abs(u @ ax - 1.0) < 1e-2 and np.linalg.norm(u - (u @ ax) * ax) < 1e-3 and qangle(st[b, 3:7]) < 1e-3
    # translation motors
    b = R[6]["body_b"]
    assert abs(st[b, 7] - 2.0) < 1e-3 and abs(st[b, 0] - b0["position"][b][0] - 2.0 * sc.steps * sc.dt) < 2e-2
    b = R[7]["body_b"]
    assert abs(st[b, 0] - b0["position"][b][0] - 0.5) < 1e-2
    # rotation motors about X
    b = R[8]["body_b"]
    assert abs(st[b, 10] - 3.0) < 1e-2 and abs(st[b, 11]) < 1e-3 and abs(st[b, 12]) < 1e-3
    b = R[9]["body_b"]
    assert abs(math.degrees(2.0 * math.atan2(st[b, 3], st[b, 6])) - 45.0) < 1.0
    # friction: v(t) = 3 - (20 N / 64 kg) t
    b = R[10]["body_b"]
    assert abs(st[b, 7] - (3.0 - 20.0 / 64.0 * sc.steps * sc.dt)) < 2e-2
    # soft limit: settles g / (2 pi 2 Hz)^2 below -0.1 m
    b = R[11]["body_b"]
    sag = -0.1 - 9.81 / (2.0 * math.pi * 2.0) ** 2
    assert abs(st[b, 1] - b0["position"][b][1] - sag) < 1.5e-2
    # free welded pair: relative pose
    a, b = R[12]["body_a"], R[12]["body_b"]
    qa, qb = st[a, 3:7], st[b, 3:7]
    rel0 = np.array([0.5, 0.4, 0.0])
    drift = np.linalg.norm(rotate(qa, rel0) - (st[b, 0:3] - st[a, 0:3]))
    qrel = np.array([qa[3] * qb[0] - qa[0] * qb[3] - qa[1] * qb[2] + qa[2] * qb[1],
                     qa[3] * qb[1] - qa[1] * qb[3] - qa[2] * qb[0] + qa[0] * qb[2],
                     qa[3] * qb[2] - qa[2] * qb[3] - qa[0] * qb[1] + qa[1] * qb[0],
                     qa[3] * qb[3] + qa[0] * qb[0] + qa[1] * qb[1] + qa[2] * qb[2]])  # conj(qa) qb
    assert drift < 3e-3 and qangle(qrel) < 3e-3, (drift, qangle(qrel))


# ---------------------------------------------------------------------------
# the oracle against mechanics (CPU)
# ---------------------------------------------------------------------------
def test_oracle_six_dof_mechanics(oracle_lib):
    sc = scenes.six_dof_zoo()
    o = oracle_of(sc)
    check_mechanics(sc, run(lambda: o.step(sc.dt, 1), o.state, sc))


def test_oracle_six_dof_limits_normalised(oracle_lib):
    """updateTranslationLimits / updateRotationLimits (six-dof-constraint.ts:240-272): a
    translation range given backwards collapses to a fixed axis at 0; a cone's swing limits are
    made symmetric about 0 from the maximum; rotation limits are clamped to [-pi, pi].  Checked
    through motion: the collapsed axis holds the box where it was created."""
    sc = scenes.six_dof_zoo()
    R = sc.joints[SD].copy()
    R[6]["limit_min"][0], R[6]["limit_max"][0] = 1.0, -1.0  # backwards: fixed at 0
    R[6]["motor_state"][0] = 0
    R[2]["limit_min"][4], R[2]["limit_min"][5] = 0.3, 0.3  # cone: mins become -max (+-30 degrees)
    sc.joints[SD] = R
    o = oracle_of(sc)
    hist = run(lambda: o.step(sc.dt, 1), o.state, sc)
    b = R[6]["body_b"]
    assert np.abs(hist[-1][b, 0:3] - sc.bodies["position"][b]).max() < 1e-3
    b = R[2]["body_b"]
    ang = max(math.degrees(math.acos(np.clip(-rotate(h[b, 3:7], (0.0, -1.0, 0.0))[1], -1, 1))) for h in hist)
    assert 29.0 < ang < 33.0


# ---------------------------------------------------------------------------
# the GPU path against the oracle
# ---------------------------------------------------------------------------
@pytest.mark.gpu
def test_six_dof_tracks_oracle(gpu_lib, oracle_lib):
    sc = scenes.six_dof_zoo()
    g, o = gpu_of(sc), oracle_of(sc)
    g.step(sc.dt, 1)
    o.step(sc.dt, 1)
    for i in range(len(sc.joints[SD])):
        lg, lo = g.joint_lambdas(SD, i), o.joint_lambdas(SD, i)
        assert lg.shape == lo.shape == (18,)
        np.testing.assert_allclose(lg, lo, rtol=1e-3, atol=1e-3, err_msg=f"six-DOF joint {i}")
    g.step(sc.dt, 19)
    o.step(sc.dt, 19)
    rows, _ = g.get_state()
    st = o.state()
    np.testing.assert_allclose(rows[:, 0:3], st[:, 0:3], atol=2e-3)
    np.testing.assert_allclose(rows[:, 7:10], st[:, 7:10], atol=2e-2)


@pytest.mark.gpu
def test_six_dof_mechanics_on_gpu(gpu_lib):
    sc = scenes.six_dof_zoo()
    g = gpu_of(sc)
    check_mechanics(sc, run(lambda: g.step(sc.dt, 1), lambda: g.get_state()[0], sc))


@pytest.mark.gpu
def test_six_dof_setters_on_gpu(gpu_lib):
    """setTranslationLimits / setRotationLimits, setMotorState + targets + setMaxFriction and
    enabled, applied between steps: the prismatic box is pulled back inside a tighter limit,
    the velocity motor reverses, the rotation motor's target moves to -30 degrees, and a
    disabled joint lets its box fall freely."""
    sc = scenes.six_dof_zoo()
    R = sc.joints[SD]
    g = gpu_of(sc)
    g.step(sc.dt, 30)
    zero = np.zeros(6)
    g.set_six_dof_limits(5, (-0.5,) + (0.0,) * 5, (0.5,) + (0.0,) * 5)
    g.set_six_dof_motor(6, (1, 0, 0, 0, 0, 0), target_velocity=(-1.0, 0.0, 0.0))
    h = math.radians(-30.0) / 2
    g.set_six_dof_motor(9, (0, 0, 0, 2, 0, 0), target_orientation=(math.sin(h), 0.0, 0.0, math.cos(h)))
    g.set_joint_enabled(SD, 11, False)
    with pytest.raises(_lib.CCError):
        g.set_six_dof_limits(len(R), zero, zero)  # no such six-DOF joint
    with pytest.raises(_lib.CCError):
        g.set_six_dof_motor(0, (3, 0, 0, 0, 0, 0))  # no such motor state
    g.step(sc.dt, 90)
    rows, _ = g.get_state()
    b = R[5]["body_b"]
    ax = R[5]["axis_x_a"].astype(np.float64)
    assert abs((rows[b, 0:3] - sc.bodies["position"][b]) @ ax - 0.5) < 1e-2
    assert abs(rows[R[6]["body_b"], 7] + 1.0) < 1e-3
    b = R[9]["body_b"]
    assert abs(math.degrees(2.0 * math.atan2(rows[b, 3], rows[b, 6])) + 30.0) < 1.0
    assert rows[R[11]["body_b"], 8] < -10.0
