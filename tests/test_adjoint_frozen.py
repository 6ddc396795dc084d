"""cc_world_rollout_grad on the differentiable-rollout workload (boxes that slide, spin and
collide on a floor), checked over the model it differentiates: the velocity solve and
integration of each step over that step's fixed contact rows.

The rows come from the GPU itself (cc_world_step_taped, one call per step); the oracle's
frozen-contact replay (oracle/oracle_frozen.h, pinned to the oracle's solver in
tests/test_frozen_replay.py) then gives, in FP64:
  - the replay of each step, which must reproduce the GPU's post-solve velocities (the GPU
    sweeps colour batches, the replay the reference's sequential order; both are the same
    Gauss-Seidel order up to FP32 rounding);
  - the dual-number directional derivative of the loss, linearised at the GPU's trajectory:
    the adjoint's grad . d must match it within 1e-3 relative (FP32 reverse sweep against
    FP64 forward mode on the same rows);
  - central differences (h = 1e-3) of the frozen-contact forward, within 5 % relative:
    the friction disc and the normal clamp switch rows on and off within +-h, which the
    derivative does not see.
"""
import numpy as np
import pytest

from crashcat_gb300 import scenes, world
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def make(bodies, nw, ws_kw):
    ws = world.standard_settings(allow_sleeping=False, **ws_kw)
    ws.num_worlds = nw
    g = world.GpuWorld(ws, len(bodies) + 8)
    g.add_bodies(bodies)
    return g


def gpu_tape(sc, targets, nw, steps):
    """Steps a fresh world `steps` times through cc_world_step_taped; returns the tape and the
    velocities after each step."""
    kw = dict(velocity_iterations=sc.velocity_iterations, position_iterations=sc.position_iterations)
    g = make(sc.bodies, nw, kw)
    tape = pyoracle.FrozenTape(pyoracle.tape_consts(sc.bodies, sc.dt), targets, sc.velocity_iterations, sc.dt)
    after = []
    rows, _ = g.get_state()
    for _ in range(steps):
        tb, tc, ratio, st = g.step_taped(sc.dt)
        assert st == 0
        b, c = pyoracle.tape_rows_from_gpu(tb, tc)
        tape.add_step(b, rows[:, 7:13], ratio, c)
        rows, _ = g.get_state()
        after.append(rows[:, 7:13].astype(np.float64))
    tape.finish(rows[:, 0:3])
    return tape, np.stack(after), kw


def directions(bodies, seed=7):
    rng = np.random.default_rng(seed)
    dyn = (bodies["motion_type"] == 2).astype(np.float64)
    n = len(bodies)
    out = []
    for k in range(3):
        dv = rng.normal(size=(n, 3)) * dyn[:, None]
        dw = rng.normal(size=(n, 3)) * dyn[:, None] * (k >= 1)
        dm = rng.normal(size=n) * dyn * 0.2 * (k == 2)
        out.append((["v", "v+w", "v+w+friction"][k], dv, dw, dm))
    return out


def test_adjoint_matches_dual_and_frozen_fd(gpu_lib, oracle_lib):
    sc, targets = scenes.diff_rollout_worlds(num_worlds=2, boxes=64)
    steps = 20
    tape, after, kw = gpu_tape(sc, targets, 2, steps)
    assert sum(len(c) for c in tape.cons) > 100  # boxes in contact with the floor and each other
    # the FP64 replay of the GPU's rows reproduces the GPU's solve
    _, _, v2, _ = tape.replay(0, want_v2=True)
    dyn = sc.bodies["motion_type"] == 2
    err = np.abs(v2[:, dyn] - after[:, dyn]).max()
    assert err < 2e-4, err
    g = make(sc.bodies, 2, kw)
    loss, gv, gw, gm = g.rollout_grad(sc.dt, steps, targets, checkpoint_every=10)
    l0, _ = tape.replay(0)
    assert abs(l0 - float(loss.sum())) <= 1e-5 * max(1.0, l0)  # the same trajectory
    for name, dv, dw, dm in directions(sc.bodies):
        ad = float((gv * dv).sum() + (gw * dw).sum() + (gm * dm).sum())
        _, dual = tape.replay(0, 0.0, dv, dw, dm)
        assert abs(ad - dual) <= 1e-3 * abs(dual) + 1e-6, (name, ad, dual)
        h = 1e-3
        lp, _ = tape.replay(1, h, dv, dw, dm)
        lm, _ = tape.replay(1, -h, dv, dw, dm)
        fd = (lp - lm) / (2 * h)
        assert abs(ad - fd) <= 0.05 * abs(fd) + 1e-4, (name, ad, fd)
