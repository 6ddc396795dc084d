"""Run-to-run determinism of the GPU step: the same scene stepped in two fresh world handles
ends bit-identical.

The reference steps one JS thread in a fixed order and its contact sort exists so that the
result does not depend on the order pairs were found (contact-constraints.ts:1240-1264).
On the device, pairs, manifolds and EPA items are appended in whatever order threads get
there; every later stage keys on something that does not depend on that order (the cache
by body pair, islands by root, each island's solve order by (sortKey, idA, idB), colours by
rank), and no float is summed with atomics on the step's path.  These tests hold that
property on the batched form, on meshes with hulls and LINEAR_CAST bodies, and on jointed
ragdolls.  The rollout loss and friction gradient sum in fixed point for the same reason
(tests/test_adjoint.py compares checkpoint spacings bit for bit)."""
import numpy as np
import pytest

from crashcat_gb300 import scenes, world

pytestmark = pytest.mark.gpu


def run(sc, steps, ws, hulls=(), mesh=None, joints=False):
    g = world.GpuWorld(ws, sc.n + 16)
    for p in hulls:
        g.add_convex_hull(p)
    if mesh is not None:
        g.add_triangle_mesh(*mesh)
    g.add_bodies(sc.bodies)
    if joints:
        g.add_hinges(sc.hinges)
        g.add_swing_twists(sc.swings)
        g.set_skip_joint_pairs(True)
    out = []
    for _ in range(steps // 20):
        g.step(sc.dt, 20)
        rows, sl = g.get_state()
        out.append((rows.copy(), sl.copy()))
    return out


def assert_same(a, b):
    for (ra, sa), (rb, sb) in zip(a, b):
        np.testing.assert_array_equal(ra, rb)
        np.testing.assert_array_equal(sa, sb)


def test_batched_worlds_step_is_deterministic(gpu_lib):
    sc = scenes.batched_worlds(num_worlds=128, seed=4)
    ws = world.standard_settings(velocity_iterations=sc.velocity_iterations,
                                 position_iterations=sc.position_iterations)
    ws.num_worlds = sc.num_worlds
    assert_same(run(sc, 120, ws), run(sc, 120, ws))


def test_mesh_hull_ccd_step_is_deterministic(gpu_lib):
    sc = scenes.mesh_drop(n=400, n_cells=32, seed=6, heights=(2.0, 10.0), fast_fraction=0.2)
    ws = world.standard_settings(velocity_iterations=8, position_iterations=2)
    a = run(sc, 80, ws, sc.hull_points, sc.mesh)
    b = run(sc, 80, ws, sc.hull_points, sc.mesh)
    assert_same(a, b)


def test_ragdoll_step_is_deterministic(gpu_lib):
    sc = scenes.ragdolls(num=64, arena=20.0)
    ws = world.standard_settings(velocity_iterations=sc.velocity_iterations,
                                 position_iterations=sc.position_iterations)
    assert_same(run(sc, 100, ws, joints=True), run(sc, 100, ws, joints=True))
