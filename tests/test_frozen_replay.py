"""The oracle's frozen-contact replay (oracle/oracle_frozen.h), pinned to the oracle's own
velocity solve, and its dual-number derivative checked against finite differences.

The replay re-runs a taped rollout's warm starts and velocity iterations over fixed contact
rows.  Fed the oracle's own tape, it must reproduce the oracle's post-solve velocities and
final impulses bit for bit (the same FP64 operations in the same order: the restatement of
warmStartVelocityConstraints / solveVelocityConstraintsForIsland, contact-constraints.ts:
906-1053, that the replay carries is the oracle's).  Its dual-number pass must then agree with
central differences of the replay itself (h = 1e-7 in FP64, 1e-5 relative: the friction disc
curves the loss enough that the derivative moves by 1e-5 relative within +-1e-6) and, on the
oracle's own tape, the linearisation at the tape (mode 0) must equal the replay's own
trajectory (mode 1) exactly.  These make the replay a trustworthy FP64 reference for the GPU
adjoint (tests/test_adjoint_frozen.py)."""
import numpy as np
import pytest

from crashcat_gb300 import scenes, world
from oracle import pyoracle


@pytest.fixture(scope="module")
def oracle_tape(oracle_lib):
    sc, targets = scenes.diff_rollout_worlds(num_worlds=2, boxes=64)
    ws = world.standard_settings(velocity_iterations=sc.velocity_iterations,
                                 position_iterations=sc.position_iterations, allow_sleeping=False)
    ws.num_worlds = 2
    o = pyoracle.OracleWorld(ws, sc.bodies)
    tape = pyoracle.FrozenTape(pyoracle.tape_consts(sc.bodies, sc.dt), targets, sc.velocity_iterations, sc.dt)
    v2s, finals = [], []
    for _ in range(30):
        st = o.state()
        b, c, v2, ratio = o.step_taped(sc.dt)
        tape.add_step(b, st[:, 7:13], ratio, c)
        v2s.append(v2)
        f = np.stack([c[:, pyoracle.CON_HEAD + q * pyoracle.POINT_ROW + 14:
                        pyoracle.CON_HEAD + q * pyoracle.POINT_ROW + 17] for q in range(4)], 1)
        finals.append(f)
    final_state = o.state()
    tape.finish(final_state[:, 0:3])
    return sc, targets, tape, np.stack(v2s), np.concatenate(finals), final_state


def test_replay_reproduces_the_oracle_solve(oracle_tape):
    sc, targets, tape, v2s, finals, final_state = oracle_tape
    assert sum(len(c) for c in tape.cons) > 100  # the boxes touch the floor and each other
    loss, _, v2r, lam = tape.replay(0, want_v2=True)
    np.testing.assert_array_equal(v2r, v2s)
    # final impulses of the points in use (unused point slots hold zeros on both sides)
    np.testing.assert_array_equal(lam, finals)
    # the loss at the tape is the rollout's loss
    b = sc.bodies
    want = 0.0
    for wd in range(len(targets)):
        m = (b["world"] == wd) & (b["motion_type"] == 2)
        want += float(((final_state[m, 0:3].mean(0) - targets[wd]) ** 2).sum())
    assert loss == pytest.approx(want, rel=1e-12)


def _directions(n, dyn, seed=5):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(3):
        dv = rng.normal(size=(n, 3)) * dyn[:, None]
        dw = rng.normal(size=(n, 3)) * dyn[:, None] * (k >= 1)
        dm = rng.normal(size=n) * dyn * 0.2 * (k == 2)
        out.append((dv, dw, dm))
    return out


def test_dual_pass_matches_finite_differences(oracle_tape):
    sc, _, tape, *_ = oracle_tape
    dyn = (sc.bodies["motion_type"] == 2).astype(np.float64)
    for dv, dw, dm in _directions(len(sc.bodies), dyn):
        l0, d0 = tape.replay(0, 0.0, dv, dw, dm)
        l1, d1 = tape.replay(1, 0.0, dv, dw, dm)
        # on the oracle's own tape the replay's trajectory is the tape's
        assert l1 == l0 and d1 == d0
        h = 1e-7
        lp, _ = tape.replay(1, h, dv, dw, dm)
        lm, _ = tape.replay(1, -h, dv, dw, dm)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - d0) <= 1e-5 * abs(d0) + 1e-9, (fd, d0)
