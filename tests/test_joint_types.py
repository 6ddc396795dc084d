"""Point, distance, fixed, cone and slider joints (src/constraints/point-, distance-, fixed-,
cone- and slider-constraint.ts): the oracle's restatement checked against mechanics on the
CPU, and the GPU path against the oracle.

The reference's tests for these joints cover creation and ids only (no expected motion), so
the oracle is pinned by physics on one scene of every configuration
(crashcat_gb300.scenes.joint_zoo, 120 steps at 60 Hz, 10/2 iterations):
  * point chains: pivot gaps stay below 3 cm while the chains swing down;
  * distance: the rigid rod keeps its 1.5 m within 8 mm (its position pass measures the error
    on the attachment points of the last property calculation, taken before this step's
    integration (distance-constraint.ts:428-431), so the rod lags one step of curvature at the
    bottom of the swing: 5 mm at 5.4 m/s); the slack rope goes taut and hangs at its 2 m,
    overshooting by at most one step of travel as it engages; the 2000 N/m spring oscillates
    with the period 2 pi sqrt(m / k) within 3 %;
  * fixed: the welded free pair, thrown spinning, keeps its relative pose within 3 mm /
    3e-3 rad (1.3 mm / 1.2e-3 rad measured), the cantilever sags less than 2 cm;
  * cone: the angle between the twist axes reaches the 30 degree limit and overshoots it by
    less than 3 degrees;
  * slider: the incline rests at its 1 m limit, the velocity motor covers 2 m/s x 2 s, the
    position motor settles at 0.5 m, 20 N of friction decelerates a 64 kg box by
    0.3125 m/s^2, every body stays on its rail within 1 mm and does not turn.

GPU tolerances (FP32 device state against the FP64 oracle): after 20 steps positions within
2e-3 m and velocities within 2e-2 m/s; each joint's accumulated impulses after the first step
within 1e-3 relative (plus 1e-3 absolute); after 120 steps the same mechanical bounds as
the oracle's.
"""
import math

import numpy as np
import pytest

from crashcat_gb300 import _lib, scenes, world
from oracle import pyoracle

P, D, F, CN, S = _lib.JOINT_POINT, _lib.JOINT_DISTANCE, _lib.JOINT_FIXED, _lib.JOINT_CONE, _lib.JOINT_SLIDER


def oracle_of(sc, **settings):
    ws = world.standard_settings(**settings)
    o = pyoracle.OracleWorld(ws, sc.bodies)
    for t, recs in sc.joints.items():
        for r in recs:
            o.add_joint_record(t, r)
    o.set_skip_joint_pairs(sc.skip_joint_pairs)
    return o


def gpu_of(sc, **settings):
    ws = world.standard_settings(**settings)
    g = world.GpuWorld(ws, sc.n + 16)
    g.add_bodies(sc.bodies)
    for t, recs in sc.joints.items():
        idx = g.add_joints(t, recs)
        assert (idx == np.arange(len(recs))).all()
    g.set_skip_joint_pairs(sc.skip_joint_pairs)
    return g


def rotate(q, v):
    u = q[..., 0:3]
    t = 2.0 * np.cross(u, v)
    return v + q[..., 3:4] * t + np.cross(u, t)


def world_point(sc, st, body, p0):
    """Where a point given in world space at creation sits now on its body."""
    b0 = sc.bodies
    q0 = b0["quaternion"][body].astype(np.float64)
    local = rotate(q0 * np.array([-1, -1, -1, 1.0]), np.asarray(p0, np.float64) - b0["position"][body])
    return st[body, 0:3].astype(np.float64) + rotate(st[body, 3:7].astype(np.float64), local)


class Tracker:
    """Mechanical measures of the joint zoo, accumulated step by step from state rows."""

    def __init__(self, sc):
        self.sc = sc
        self.point_gap = 0.0
        self.rod = []
        self.slack = []
        self.spring_y = []
        self.cone = [0.0, 0.0]
        self.rail_off = 0.0
        self.rail_turn = 0.0
        self.chain_low = [np.inf, np.inf]  # lowest height of each chain's last link
        self.st0 = None

    def add(self, st):
        sc, J = self.sc, self.sc.joints
        if self.st0 is None:
            self.st0 = st.copy()
        for c in range(2):
            self.chain_low[c] = min(self.chain_low[c], float(st[J[P][4 * c + 3]["body_b"], 1]))
        for r in J[P]:
            g = np.linalg.norm(world_point(sc, st, r["body_a"], r["point_a"]) -
                               world_point(sc, st, r["body_b"], r["point_b"]))
            self.point_gap = max(self.point_gap, g)
        d = [np.linalg.norm(world_point(sc, st, r["body_a"], r["point_a"]) -
                            world_point(sc, st, r["body_b"], r["point_b"])) for r in J[D]]
        self.rod.append(d[0])
        self.slack.append(d[1])
        self.spring_y.append(st[J[D][2]["body_b"], 1])
        for k, r in enumerate(J[CN]):
            ta = rotate(st[r["body_a"], 3:7].astype(np.float64), np.asarray(r["twist_axis_a"], np.float64))
            q0 = sc.bodies["quaternion"][r["body_b"]].astype(np.float64)
            lt = rotate(q0 * np.array([-1, -1, -1, 1.0]), np.asarray(r["twist_axis_b"], np.float64))
            tb = rotate(st[r["body_b"], 3:7].astype(np.float64), lt)
            ang = math.degrees(math.acos(max(-1.0, min(1.0, float(ta @ tb)))))
            self.cone[k] = max(self.cone[k], ang)
        for r in J[S][:4]:  # bodies on static rails
            b = r["body_b"]
            ax = np.asarray(r["slider_axis_a"], np.float64)
            disp = st[b, 0:3].astype(np.float64) - self.st0[b, 0:3]
            self.rail_off = max(self.rail_off, np.linalg.norm(disp - (disp @ ax) * ax))
            dq = np.abs(np.abs(st[b, 3:7].astype(np.float64) @ self.st0[b, 3:7]) - 1.0)
            self.rail_turn = max(self.rail_turn, dq)

    def spring_period(self):
        y = np.array(self.spring_y)
        m = y - y.mean()
        up = np.nonzero((m[:-1] < 0) & (m[1:] >= 0))[0]
        t = (up + (-m[up]) / (m[up + 1] - m[up])) * self.sc.dt
        return float(np.diff(t).mean())


def welded_drift(sc, st):
    """Relative position and rotation drift of the free welded pair since creation."""
    r = sc.joints[F][1]
    a, b = r["body_a"], r["body_b"]
    b0 = sc.bodies
    def rel(pa, qa, pb, qb):
        qa = qa.astype(np.float64)
        inv = qa * np.array([-1, -1, -1, 1.0])
        return rotate(inv, (pb - pa).astype(np.float64)), qa, qb.astype(np.float64)
    r0, qa0, qb0 = rel(b0["position"][a], b0["quaternion"][a], b0["position"][b], b0["quaternion"][b])
    r1, qa1, qb1 = rel(st[a, 0:3], st[a, 3:7], st[b, 0:3], st[b, 3:7])

    def qmul(p, q):
        return np.array([p[3] * q[0] + p[0] * q[3] + p[1] * q[2] - p[2] * q[1],
                         p[3] * q[1] - p[0] * q[2] + p[1] * q[3] + p[2] * q[0],
                         p[3] * q[2] + p[0] * q[1] - p[1] * q[0] + p[2] * q[3],
                         p[3] * q[3] - p[0] * q[0] - p[1] * q[1] - p[2] * q[2]])
    c = np.array([-1, -1, -1, 1.0])
    rel0, rel1 = qmul(qa0 * c, qb0), qmul(qa1 * c, qb1)
    dq = abs(abs(float(rel0 @ rel1)) - 1.0)
    return float(np.linalg.norm(r1 - r0)), 2.0 * math.sqrt(2.0 * dq)


def check_mechanics(sc, tr, st, slider_pos):
    J = sc.joints
    assert tr.point_gap < 0.03, tr.point_gap
    # the chains swing down: each last link drops well below its release height
    assert max(tr.chain_low) < 5.0, tr.chain_low
    assert np.abs(np.array(tr.rod) - 1.5).max() < 8e-3
    # the rope engages when a step starts past its length: the falling sphere overshoots by at
    # most one step of travel (4.6 m/s x 1/60 s), then hangs at 2 m
    assert max(tr.slack) < 2.08 and abs(tr.slack[-1] - 2.0) < 2e-3, (max(tr.slack), tr.slack[-1])
    m = sc.bodies["density"][J[D][2]["body_b"]] * 4.0 / 3.0 * math.pi * 0.2 ** 3
    expect = 2 * math.pi * math.sqrt(m / 2000.0)
    assert abs(tr.spring_period() - expect) < 0.03 * expect, (tr.spring_period(), expect)
    lin, ang = welded_drift(sc, st)
    assert lin < 3e-3 and ang < 3e-3, (lin, ang)
    tip = world_point(sc, st, J[F][1 - 1]["body_b"], (0.9, 8.0, 12.0))
    assert np.linalg.norm(tip - (0.9, 8.0, 12.0)) < 0.02
    for k in range(2):
        assert 29.0 < tr.cone[k] < 33.0, tr.cone
    np.testing.assert_allclose(slider_pos[:4], [1.0, 4.0, 0.5, 6.0 - 0.5 * (20.0 / 64.0) * 4.0], atol=2e-2)
    assert tr.rail_off < 1e-3 and tr.rail_turn < 1e-6, (tr.rail_off, tr.rail_turn)


# ---------------------------------------------------------------------------
# the oracle against mechanics (CPU)
# ---------------------------------------------------------------------------
def test_oracle_joint_zoo_mechanics(oracle_lib):
    sc = scenes.joint_zoo()
    o = oracle_of(sc)
    tr = Tracker(sc)
    for _ in range(sc.steps):
        o.step(sc.dt, 1)
        tr.add(o.state())
    check_mechanics(sc, tr, o.state(), np.array([o.slider_position(i) for i in range(5)]))


def test_oracle_joint_records_by_type(oracle_lib):
    """Each type has its own index space (the reference's per-type pools), and a disabled
    joint neither links islands nor acts: its body falls freely."""
    sc = scenes.joint_zoo()
    recs = sc.joints[D].copy()
    recs[0]["enabled"] = 0
    sc.joints[D] = recs
    o = oracle_of(sc)
    o.step(sc.dt, 30)
    st = o.state()
    b = recs[0]["body_b"]
    t = 30 * sc.dt
    assert abs(st[b, 1] - (8.0 - 0.5 * 9.81 * t * (t + sc.dt))) < 1e-6 + 1e-2 * t * t


# ---------------------------------------------------------------------------
# the GPU path against the oracle
# ---------------------------------------------------------------------------
@pytest.mark.gpu
def test_joint_zoo_tracks_oracle(gpu_lib, oracle_lib):
    sc = scenes.joint_zoo()
    g, o = gpu_of(sc), oracle_of(sc)
    g.step(sc.dt, 1)
    o.step(sc.dt, 1)
    for t, recs in sc.joints.items():
        for i in range(len(recs)):
            lg, lo = g.joint_lambdas(t, i), o.joint_lambdas(t, i)
            assert lg.shape == lo.shape
            np.testing.assert_allclose(lg, lo, rtol=1e-3, atol=1e-3, err_msg=f"type {t} joint {i}")
    g.step(sc.dt, 19)
    o.step(sc.dt, 19)
    rows, _ = g.get_state()
    st = o.state()
    np.testing.assert_allclose(rows[:, 0:3], st[:, 0:3], atol=2e-3)
    np.testing.assert_allclose(rows[:, 7:10], st[:, 7:10], atol=2e-2)


@pytest.mark.gpu
def test_joint_zoo_mechanics_on_gpu(gpu_lib):
    sc = scenes.joint_zoo()
    g = gpu_of(sc)
    tr = Tracker(sc)
    for _ in range(sc.steps):
        g.step(sc.dt, 1)
        rows, _ = g.get_state()
        tr.add(rows.astype(np.float64))
    rows, _ = g.get_state()
    check_mechanics(sc, tr, rows.astype(np.float64), g.slider_positions(5).astype(np.float64))


@pytest.mark.gpu
def test_joint_setters_on_gpu(gpu_lib, oracle_lib):
    """setDistance / setHalfConeAngle / slider setLimits and setMotorState / enabled, each
    applied between steps on the GPU and checked against the oracle given the same joint from
    creation."""
    sc = scenes.joint_zoo()
    g = gpu_of(sc)
    g.step(sc.dt, 10)
    g.set_joint_enabled(D, 0, False)
    g.set_distance(1, 0.5, 1.2)
    g.set_cone_half_angle(0, math.radians(10.0))
    g.set_slider_limits(0, -0.5, 0.5)
    g.set_slider_motor(1, _lib.MOTOR_VELOCITY, target_velocity=-1.0)
    with pytest.raises(_lib.CCError):
        g.set_distance(5, 1.0, 1.0)  # no such distance joint
    with pytest.raises(_lib.CCError):
        g.set_joint_enabled(7, 0, True)  # no six-DOF joints here
    g.step(sc.dt, 60)
    rows, _ = g.get_state()
    J = sc.joints
    # the disabled rod's sphere falls freely (its speed grew by g t)
    assert rows[J[D][0]["body_b"], 8] < -5.0
    # the slack rope now stops at 1.2 m
    d = np.linalg.norm(world_point(sc, rows, J[D][1]["body_a"], J[D][1]["point_a"]) -
                       world_point(sc, rows, J[D][1]["body_b"], J[D][1]["point_b"]))
    assert d < 1.2 + 5e-3
    pos = g.slider_positions(5)
    assert abs(pos[0] - 0.5) < 1e-2
    assert abs(rows[J[S][1]["body_b"], 7] - (-1.0)) < 1e-3
