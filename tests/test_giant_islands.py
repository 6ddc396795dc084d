"""The solve tiers against one another and against the oracle.

Islands are solved by one thread (the reference's exact order), one warp, one CTA or, past
giant_min constraints, by the whole grid in one cooperative launch.  The colouring of every
tier is greedy in the reference's solve order, so a pile gives the oracle's velocities on its
first step whichever tier runs it.  The launch-shape tunables CRASHCAT_GIANT_MIN and
CRASHCAT_SMALL_JOINTS_MAX move islands between tiers for these tests.

Tolerances: first step of a pyramid 1e-5 m/s (as the per-warp and per-CTA tiers); three
steps against the per-thread order 1e-5 (warm starting sums impulses in colour order rather
than constraint order); ragdolls over 20 steps 5e-3 m, as the ragdoll parity test.
"""
import numpy as np
import pytest

from crashcat_gb300 import scenes, world
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def make(sc, **settings):
    ws = world.standard_settings(velocity_iterations=sc.velocity_iterations,
                                 position_iterations=sc.position_iterations, **settings)
    ws.num_worlds = sc.num_worlds
    g = world.GpuWorld(ws, sc.n + 16)
    g.add_bodies(sc.bodies)
    if sc.hinges is not None:
        g.add_hinges(sc.hinges)
    if sc.swings is not None:
        g.add_swing_twists(sc.swings)
    g.set_skip_joint_pairs(sc.skip_joint_pairs)
    return g


def oracle(sc):
    ws = world.standard_settings(velocity_iterations=sc.velocity_iterations,
                                 position_iterations=sc.position_iterations)
    o = pyoracle.OracleWorld(ws, sc.bodies)
    for h in sc.hinges if sc.hinges is not None else ():
        o.add_hinge_record(h)
    for h in sc.swings if sc.swings is not None else ():
        o.add_swing_twist_record(h)
    o.set_skip_joint_pairs(sc.skip_joint_pairs)
    return o


@pytest.mark.parametrize("base", [9, 14])
def test_giant_tier_pyramid_first_step(gpu_lib, oracle_lib, base, monkeypatch):
    monkeypatch.setenv("CRASHCAT_GIANT_MIN", "64")
    sc = scenes.box_pyramid(base)
    g, o = make(sc), oracle(sc)
    g.step(sc.dt, 1)
    o.step(sc.dt, 1)
    rows, _ = g.get_state()
    st = o.state()
    assert np.abs(rows[:, 7:13] - st[:, 7:13]).max() < 1e-5
    assert np.abs(rows[:, 0:3] - st[:, 0:3]).max() < 1e-6


def test_giant_tier_matches_sequential_order(gpu_lib, monkeypatch):
    sc = scenes.box_pyramid(6)  # 51 contacts
    monkeypatch.setenv("CRASHCAT_SMALL_ISLAND_MAX", "64")
    g_seq = make(sc)
    monkeypatch.delenv("CRASHCAT_SMALL_ISLAND_MAX")
    monkeypatch.setenv("CRASHCAT_GIANT_MIN", "32")
    g_big = make(sc)
    for _ in range(3):
        g_seq.step(sc.dt, 1)
        g_big.step(sc.dt, 1)
    np.testing.assert_allclose(g_big.get_state()[0], g_seq.get_state()[0], atol=1e-5)


@pytest.mark.parametrize("tier", ["cta", "giant"])
def test_ragdolls_on_other_tiers(gpu_lib, oracle_lib, tier, monkeypatch):
    """Single-ragdoll islands forced onto the per-CTA tier (joint colouring) or the grid tier."""
    if tier == "cta":
        monkeypatch.setenv("CRASHCAT_SMALL_JOINTS_MAX", "0")
    else:
        monkeypatch.setenv("CRASHCAT_GIANT_MIN", "8")
    sc = scenes.ragdolls(num=4, arena=12.0)
    g, o = make(sc), oracle(sc)
    g.step(sc.dt, 20)
    o.step(sc.dt, 20)
    rows, _ = g.get_state()
    np.testing.assert_allclose(rows[:, 0:3], o.state()[:, 0:3], atol=5e-3)
    g.step(sc.dt, 100)
    assert np.isfinite(g.get_state()[0]).all()


def test_pile_of_ragdolls_runs_on_the_grid_tier(gpu_lib, monkeypatch):
    """64 ragdolls stacked four high in a 20 m arena fall into piles; with giant_min at 256
    the piles' islands run on the grid tier: the state stays finite, the joints hold and no
    body sinks through the floor."""
    monkeypatch.setenv("CRASHCAT_GIANT_MIN", "256")
    sc = scenes.ragdolls(num=64, arena=20.0)
    g = make(sc)
    g.step(sc.dt, 240)
    rows, _ = g.get_state()
    assert np.isfinite(rows).all()
    assert g.stats()["max_island_constraints"] > 256
    assert rows[6:, 1].min() > -0.2
    from test_swing_twist import joint_gaps
    assert joint_gaps(sc, rows.astype(np.float64)).max() < 0.05
