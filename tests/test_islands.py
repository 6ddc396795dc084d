"""Per-island solver iteration counts (islands.ts:344-386): an island runs the largest
numVelocityStepsOverride / numPositionStepsOverride of its dynamic bodies and joints, raised to
the world's counts when any of them asks for the default (0).

The scenario of the reference's own test (tst/islands.test.ts:70-137): two overlapping spheres,
one with overrides 20 / 15, share an island that runs 20 velocity and 15 position steps against
world counts of 10 / 5; a lone sphere with overrides 8 / 3 runs 8 / 3 (no body of its island uses
0, so the defaults do not apply).  Checked on the oracle (CPU) and on the GPU; on the GPU a stack
whose bodies override the counts also tracks the oracle, step by step."""
import numpy as np
import pytest

from crashcat_gb300 import scenes, world
from oracle import pyoracle


def reference_scene():
    b = scenes.blank_bodies(3)
    scenes.set_sphere(b, [0, 1, 2], 0.5)
    b["position"][0] = (0.0, 0.6, 0.0)   # bodyDefault, overlapping bodyCustom
    b["position"][1] = (0.0, 0.0, 0.0)   # bodyCustom: 20 / 15
    b["position"][2] = (10.0, 0.0, 0.0)  # bodyOther, far away: 8 / 3
    b["num_velocity_steps_override"][1], b["num_position_steps_override"][1] = 20, 15
    b["num_velocity_steps_override"][2], b["num_position_steps_override"][2] = 8, 3
    return b


def reference_settings():
    return world.standard_settings(velocity_iterations=10, position_iterations=5)


EXPECTED = np.array([[20, 15], [20, 15], [8, 3]])


def test_oracle_island_iterations_follow_the_reference(oracle_lib):
    o = pyoracle.OracleWorld(reference_settings(), reference_scene())
    o.step(1.0 / 60.0, 1)
    np.testing.assert_array_equal(o.island_iterations(), EXPECTED)


def overridden_stack(vel, pos):
    sc = scenes.box_stack(height=6)
    b = sc.bodies
    dyn = b["motion_type"] == 2
    b["num_velocity_steps_override"][dyn] = vel
    b["num_position_steps_override"][dyn] = pos
    return sc


def test_oracle_overrides_change_the_solve(oracle_lib):
    """Fewer iterations than the world's leave a different stack state after a few steps."""
    out = []
    for vel, pos in ((0, 0), (2, 1)):
        sc = overridden_stack(vel, pos)
        o = pyoracle.OracleWorld(world.standard_settings(), sc.bodies)
        o.step(sc.dt, 20)
        out.append(o.state())
    assert np.abs(out[0][:, 0:3] - out[1][:, 0:3]).max() > 1e-4


@pytest.mark.gpu
def test_gpu_island_iterations_follow_the_reference(gpu_lib):
    b = reference_scene()
    g = world.GpuWorld(reference_settings(), len(b) + 4)
    g.add_bodies(b)
    g.step(1.0 / 60.0, 1)
    np.testing.assert_array_equal(g.island_iterations(), EXPECTED)


@pytest.mark.gpu
def test_gpu_overridden_stack_tracks_the_oracle(gpu_lib, oracle_lib):
    """A 6-box stack whose bodies ask for 3 velocity and 1 position steps (world: 10 / 2) runs those
    counts on the GPU and tracks the oracle's positions within 2 mm for 30 steps."""
    sc = overridden_stack(3, 1)
    ws = world.standard_settings()
    g = world.GpuWorld(ws, sc.n + 4)
    g.add_bodies(sc.bodies)
    o = pyoracle.OracleWorld(ws, sc.bodies)
    for _ in range(30):
        g.step(sc.dt, 1)
        o.step(sc.dt, 1)
        rows, _ = g.get_state()
        np.testing.assert_allclose(rows[:, 0:3], o.state()[:, 0:3], atol=2e-3)
    it = g.island_iterations()
    dyn = sc.bodies["motion_type"] == 2
    assert (it[dyn] == [3, 1]).all()
    np.testing.assert_array_equal(it, o.island_iterations())
