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

from crashcat_gb300 import _lib, scenes, world
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
        monkeypatch.setenv("CRASHCAT_GIANT_MIN", "8")  # a lone ragdoll's 10 joints and its contacts
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


def test_grid_barrier_wait_runs_out_with_a_status(gpu_lib, monkeypatch):
    """The grid barrier of the whole-grid solve polls a bounded number of times.  With block 0
    withheld from its barriers (CRASHCAT_TEST_WITHHOLD_BARRIER: a flag that nothing sets) the
    other blocks' wait runs out after 20,000 polls: every block leaves, the step returns
    CC_ERR_TIMEOUT with OVF_TIMEOUT in the counters, and the device keeps answering (a world
    without the hook then steps normally)."""
    monkeypatch.setenv("CRASHCAT_GIANT_MIN", "64")
    monkeypatch.setenv("CRASHCAT_TEST_WITHHOLD_BARRIER", "1")
    sc = scenes.box_pyramid(base=12)
    ws = world.standard_settings(device_wait_polls=20000)
    g = world.GpuWorld(ws, sc.n + 8)
    g.add_bodies(sc.bodies)
    with pytest.raises(_lib.CCError) as e:
        g.step(sc.dt, 3)
    assert e.value.status == _lib.CC_ERR_TIMEOUT
    assert g.stats()["num_giant_islands"] >= 1
    assert g.stats()["overflow_flags"] & 64
    monkeypatch.delenv("CRASHCAT_TEST_WITHHOLD_BARRIER")
    ok = world.GpuWorld(world.standard_settings(), sc.n + 8)
    ok.add_bodies(sc.bodies)
    assert ok.step(sc.dt, 3) == _lib.CC_OK
    assert np.isfinite(ok.get_state()[0]).all()


def slab_with_boxes(n_side=8):
    """A dynamic slab resting on the floor, created last (the highest body index, so every link of
    a box on it targets the slab's root), with n_side^2 small boxes resting on it."""
    n = n_side * n_side
    b = scenes.blank_bodies(n + 2)
    scenes.static_floor(b, 0)
    idx = np.arange(1, n + 1)
    scenes.set_box(b, idx, (0.2, 0.2, 0.2))
    g = np.arange(n)
    b["position"][idx] = np.stack([(g % n_side - n_side / 2) * 0.6, np.full(n, 0.5 + 0.2 - 0.005),
                                   (g // n_side - n_side / 2) * 0.6], 1)
    scenes.set_box(b, n + 1, (3.0, 0.25, 3.0))
    b["position"][n + 1] = (0.0, 0.25 - 0.005, 0.0)
    return b


def test_union_find_link_bound_skips_the_solve(gpu_lib):
    """With one compare-and-swap attempt per union-find link, links that lose a race give up: many
    boxes rest on one slab whose root every link targets, so the lanes of a warp race for it.  The
    step reports CC_ERR_CAPACITY with OVF_ISLAND and skips its solve (no body moves), and the device
    keeps answering."""
    b = slab_with_boxes()
    ws = world.standard_settings(island_link_attempts=1)
    g = world.GpuWorld(ws, len(b) + 8)
    g.add_bodies(b)
    before, _ = g.get_state()
    st = g.step(1 / 60, 1)
    assert st == _lib.CC_ERR_CAPACITY
    assert g.stats()["overflow_flags"] & 8
    after, _ = g.get_state()
    np.testing.assert_array_equal(after[:, 0:7], before[:, 0:7])
    ok = world.GpuWorld(world.standard_settings(), len(b) + 8)
    ok.add_bodies(b)
    assert ok.step(1 / 60, 2) == _lib.CC_OK
