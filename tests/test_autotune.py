"""cc_world_autotune: the launch-shape tuner leaves the world where it found it (bit for bit),
and the shapes it keeps change results only by the FP32 rounding of the kernel that solves an
island (each island's solve order and each EPA polytope are the same under every shape)."""
import numpy as np
import pytest

from crashcat_gb300 import scenes, world

pytestmark = pytest.mark.gpu


def test_autotune_keeps_the_state_and_the_results(gpu_lib):
    sc = scenes.batched_worlds(num_worlds=96, seed=4)
    ws = world.standard_settings(velocity_iterations=sc.velocity_iterations,
                                 position_iterations=sc.position_iterations)
    ws.num_worlds = sc.num_worlds

    def make():
        g = world.GpuWorld(ws, sc.n + 16)
        g.add_bodies(sc.bodies)
        g.step(sc.dt, 120)
        return g

    tuned, plain = make(), make()
    before, _ = tuned.get_state()
    rep = tuned.autotune(sc.dt, 2)
    after, _ = tuned.get_state()
    np.testing.assert_array_equal(before, after)
    assert rep["trials"] >= 8 and rep["tuned_ms"] > 0 and rep["tuned_ms"] <= rep["default_ms"]
    assert rep["graph_kernels_per_step"] > 10
    tuned.step(sc.dt, 10)
    plain.step(sc.dt, 10)
    d = np.abs(tuned.get_state()[0][:, 0:3] - plain.get_state()[0][:, 0:3]).max(1)
    assert (d < 1e-4).mean() > 0.99 and d.max() < 1e-2
