"""GPU parity against the FP64 oracle, through the C ABI.

Tolerances (FP32 device state against an FP64 restatement of the reference):
  * broadphase pair sets: bit-exact (the device re-tests candidates in FP64);
  * contacts whose shrunk shapes do not overlap (GJK path): normal within 1e-4,
    depth and points within 1e-4 m + 1e-4 relative;
  * deep contacts (EPA path, depth > 0.05 m): normal within 1e-3, depth within
    1e-3 relative, points within 2e-3 m + 1e-2 x depth (EPA starts from the
    FP32 GJK simplex and stops at the reference's 1e-4 relative tolerance);
  * at most 2 % of contacts may flip a discrete choice (clip plane side,
    prune choice) between FP32 and FP64;
  * free-fall integration over 30 steps: 1e-4 relative;
  * one step of isolated resting contacts and the first 12 steps of a box
    stack: velocities within 1e-4 m/s;
  * 180 steps of the 1,000-box heap: lowest body height within 2 mm, mean
    height within 1 cm of the oracle.
"""
import numpy as np
import pytest

from crashcat_gb300 import scenes, world
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def make_pair(scene, **settings):
    ws = world.standard_settings(velocity_iterations=scene.velocity_iterations,
                                 position_iterations=scene.position_iterations, **settings)
    ws.num_worlds = scene.num_worlds
    g = world.GpuWorld(ws, scene.n + 16)
    g.add_bodies(scene.bodies)
    o = pyoracle.OracleWorld(ws, scene.bodies)
    return g, o


def test_free_fall_integration(gpu_lib, oracle_lib):
    sc = scenes.free_fall(n=256)
    g, o = make_pair(sc)
    for _ in range(3):
        g.step(sc.dt, 10)
        o.step(sc.dt, 10)
    rows, _ = g.get_state()
    st = o.state()
    assert len(g.get_pairs()) == 0 and len(o.pairs()) == 0
    np.testing.assert_allclose(rows[:, 0:3], st[:, 0:3], rtol=1e-4, atol=1e-4)
    np.testing.assert_allclose(rows[:, 7:13], st[:, 7:13], rtol=1e-4, atol=1e-4)
    dq = np.minimum(np.abs(rows[:, 3:7] - st[:, 3:7]).max(1), np.abs(rows[:, 3:7] + st[:, 3:7]).max(1))
    assert dq.max() < 1e-4


def canonical_pairs(p):
    p = np.asarray(p, dtype=np.int64)
    if len(p) == 0:
        return set()
    return set(map(tuple, np.sort(p, axis=1).tolist()))


@pytest.mark.parametrize("seed", [7, 8, 9])
def test_broadphase_pairs_bit_exact(gpu_lib, oracle_lib, seed):
    sc = scenes.random_pairs_scene(n=300, seed=seed)
    g, o = make_pair(sc)
    g.step(0.0, 1)  # dt = 0: broadphase + narrowphase, no solve (update.ts:101)
    o.step(0.0, 1)
    gp, op = g.get_pairs(), o.pairs()
    assert len(gp) == len(op)
    # the query body of each pair is the same body in both (broadphase.ts:126-136)
    assert set(map(tuple, gp.tolist())) == set(map(tuple, op.tolist()))
    assert canonical_pairs(gp) == canonical_pairs(op)


def test_broadphase_pairs_cube_heap_state(gpu_lib, oracle_lib):
    """Pairs of the settled heap (stacked boxes touching within the margin) are bit-exact."""
    sc = scenes.cube_heap()
    o = pyoracle.OracleWorld(world.standard_settings(), sc.bodies)
    o.step(sc.dt, 60)
    st = o.state()
    b = sc.bodies.copy()
    b["position"] = st[:, 0:3].astype(np.float32)
    b["quaternion"] = st[:, 3:7].astype(np.float32)
    g = world.GpuWorld(world.standard_settings(), sc.n + 16)
    g.add_bodies(b)
    o2 = pyoracle.OracleWorld(world.standard_settings(), b)
    g.step(0.0, 1)
    o2.step(0.0, 1)
    assert set(map(tuple, g.get_pairs().tolist())) == set(map(tuple, o2.pairs().tolist()))


def contact_errors(a, b):
    deep = b[6] > 0.05
    n_tol, d_rel = (1e-3, 1e-3) if deep else (1e-4, 1e-4)
    n_ok = np.abs(a[3:6] - b[3:6]).max() < n_tol
    d_ok = abs(a[6] - b[6]) < 1e-4 + d_rel * abs(b[6])
    pg = a[8:8 + 6 * int(a[2])].reshape(-1, 6)
    po = b[8:8 + 6 * int(b[2])].reshape(-1, 6)
    p_tol = (2e-3 + 1e-2 * abs(b[6])) if deep else 1e-4
    p_ok = int(a[2]) == int(b[2]) and all(np.min(np.abs(pg - q).max(1)) < p_tol + 1e-4 * np.abs(q).max() for q in po)
    return n_ok and d_ok and p_ok


@pytest.mark.parametrize("seed", [7, 8])
def test_contact_manifolds(gpu_lib, oracle_lib, seed):
    sc = scenes.random_pairs_scene(n=300, seed=seed)
    g, o = make_pair(sc)
    g.step(0.0, 1)
    o.step(0.0, 1)
    gk = {(int(r[0]), int(r[1])): r for r in g.get_manifolds()}
    ok = {(int(r[0]), int(r[1])): r for r in o.manifolds()}
    assert len(ok) > 20
    common = set(gk) & set(ok)
    assert len(common) >= 0.98 * max(len(gk), len(ok))
    bad = [k for k in common if not contact_errors(gk[k], ok[k])]
    assert len(bad) <= 0.02 * len(common), bad[:5]


def test_contacts_cube_heap_state(gpu_lib, oracle_lib):
    """Resting and stacked box contacts (GJK and box-floor EPA) of the heap after 1 s."""
    sc = scenes.cube_heap()
    o = pyoracle.OracleWorld(world.standard_settings(), sc.bodies)
    o.step(sc.dt, 60)
    st = o.state()
    b = sc.bodies.copy()
    b["position"] = st[:, 0:3].astype(np.float32)
    b["quaternion"] = st[:, 3:7].astype(np.float32)
    g = world.GpuWorld(world.standard_settings(), sc.n + 16)
    g.add_bodies(b)
    o2 = pyoracle.OracleWorld(world.standard_settings(), b)
    g.step(0.0, 1)
    o2.step(0.0, 1)
    gk = {(int(r[0]), int(r[1])): r for r in g.get_manifolds()}
    ok = {(int(r[0]), int(r[1])): r for r in o2.manifolds()}
    assert set(gk) == set(ok)
    bad = [k for k in ok if not contact_errors(gk[k], ok[k])]
    assert len(bad) <= 0.02 * len(ok), bad[:5]


def test_resting_contacts_one_step(gpu_lib, oracle_lib):
    """Isolated boxes on the floor: one contact per island, so the solve order is the
    reference's; post-solve velocities agree within 1e-4 m/s."""
    sc = scenes.resting_boxes(n=64)
    g, o = make_pair(sc)
    for _ in range(5):
        g.step(sc.dt, 1)
        o.step(sc.dt, 1)
        rows, _ = g.get_state()
        st = o.state()
        np.testing.assert_allclose(rows[:, 7:13], st[:, 7:13], atol=1e-4)
        np.testing.assert_allclose(rows[:, 0:3], st[:, 0:3], atol=1e-4)


def test_stack_steps_track_oracle(gpu_lib, oracle_lib):
    """A 10-box column (a chain island: the greedy colouring is fully sequential) tracks
    the oracle step by step, including warm starting from the contact cache."""
    sc = scenes.box_stack(height=10)
    g, o = make_pair(sc)
    for _ in range(12):
        g.step(sc.dt, 1)
        o.step(sc.dt, 1)
        rows, _ = g.get_state()
        st = o.state()
        assert np.abs(rows[:, 7:13] - st[:, 7:13]).max() < 1e-4
        assert np.abs(rows[:, 0:3] - st[:, 0:3]).max() < 1e-5


def test_row_island_colour_parallel(gpu_lib, oracle_lib):
    """A row of touching boxes: colours hold several contacts solved in parallel by one CTA;
    the colouring preserves the reference's order so the result matches."""
    for count in (6, 12):
        sc = scenes.box_row(count)
        g, o = make_pair(sc)
        g.step(sc.dt, 1)
        o.step(sc.dt, 1)
        rows, _ = g.get_state()
        assert np.abs(rows[:, 7:13] - o.state()[:, 7:13]).max() < 1e-4


def test_islands_consistent(gpu_lib):
    """Every contact between two active bodies lies in one island holding both bodies."""
    sc = scenes.cube_heap()
    g = world.GpuWorld(world.standard_settings(), sc.n + 16)
    g.add_bodies(sc.bodies)
    g.step(sc.dt, 40)
    iob, rows = g.debug_islands()
    assert len(rows) > 100
    for a, c, isl in rows:
        ia, ic = iob[a], iob[c]
        if ia >= 0 and ic >= 0:
            assert ia == ic == isl
        else:
            assert isl == max(ia, ic)


def test_cube_heap_drift(gpu_lib, oracle_lib):
    """180 steps of the 1,000-box heap: penetration and heights stay with the oracle's."""
    sc = scenes.cube_heap()
    g, o = make_pair(sc)
    for _ in range(3):
        g.step(sc.dt, 60)
        o.step(sc.dt, 60)
        rows, sl = g.get_state()
        st = o.state()
        assert abs(rows[1:, 1].min() - st[1:, 1].min()) < 2e-3
        assert abs(rows[1:, 1].mean() - st[1:, 1].mean()) < 1e-2
        assert np.isfinite(rows).all()
    assert g.stats()["overflow_flags"] == 0


def test_batched_worlds_are_independent(gpu_lib):
    """Two copies of one world inside one batched handle evolve exactly like the single world."""
    sc = scenes.cube_heap(n_side=4, seed=5)
    b2 = np.concatenate([sc.bodies, sc.bodies])
    b2["world"][sc.n:] = 1
    ws1 = world.standard_settings()
    ws2 = world.standard_settings()
    ws2.num_worlds = 2
    g1 = world.GpuWorld(ws1, sc.n + 8)
    g1.add_bodies(sc.bodies)
    g2 = world.GpuWorld(ws2, 2 * sc.n + 8)
    g2.add_bodies(b2)
    g1.step(sc.dt, 60)
    g2.step(sc.dt, 60)
    r1, _ = g1.get_state()
    r2, _ = g2.get_state()
    # same bodies in the same order: each copy matches the single world (FP32, same order)
    np.testing.assert_allclose(r2[: sc.n], r1, atol=2e-4)
    np.testing.assert_allclose(r2[sc.n:], r1, atol=2e-4)
    # no pair ever crosses worlds
    p = g2.get_pairs()
    assert ((p[:, 0] < sc.n) == (p[:, 1] < sc.n)).all()


@pytest.mark.parametrize("base", [5, 9, 14, 20])
def test_pyramid_island_first_step(gpu_lib, oracle_lib, base):
    """One island per pyramid: base 5 (35 contacts) runs on the per-warp tier's small
    instance, 9 (117) on its large one (sort, colouring and shared-memory sweep), base 14
    (287 contacts) and 20 (590) on one CTA.
    The colouring keeps the reference's order, so the first step matches the
    oracle's velocities.  (Later steps meet prune ties between the pyramid's
    aligned faces, which FP32 and FP64 break differently.)"""
    sc = scenes.box_pyramid(base)
    g, o = make_pair(sc)
    g.step(sc.dt, 1)
    o.step(sc.dt, 1)
    rows, _ = g.get_state()
    st = o.state()
    assert np.abs(rows[:, 7:13] - st[:, 7:13]).max() < 1e-5
    assert np.abs(rows[:, 0:3] - st[:, 0:3]).max() < 1e-6
    assert g.stats()["max_island_constraints"] == len(o.manifolds())


@pytest.mark.parametrize("base", [5, 6])
def test_warp_island_matches_sequential_order(gpu_lib, base, monkeypatch):
    """The per-warp solve (colour sweeps) against the per-thread solve (the
    reference's sequential order, forced by raising the per-thread class limit
    to 64 contacts; base 6 has 51) over 3 steps with warm starting: both give
    the same state."""
    sc = scenes.box_pyramid(base)
    g_warp = world.GpuWorld(world.standard_settings(), sc.n + 16)
    g_warp.add_bodies(sc.bodies)
    monkeypatch.setenv("CRASHCAT_SMALL_ISLAND_MAX", "64")
    g_seq = world.GpuWorld(world.standard_settings(), sc.n + 16)
    g_seq.add_bodies(sc.bodies)
    for _ in range(3):
        g_warp.step(sc.dt, 1)
        g_seq.step(sc.dt, 1)
    r_warp, _ = g_warp.get_state()
    r_seq, _ = g_seq.get_state()
    np.testing.assert_allclose(r_warp, r_seq, atol=1e-6)


def test_epa_fallback_pass_matches_packed_pass(gpu_lib, monkeypatch):
    """EPA items whose polytope outgrows the packed pass's point limit are re-run with
    the reference's limits.  Forcing most items over a limit of 5 points gives the same
    contacts as the packed pass (both run the same FP64 hull code)."""
    sc = scenes.random_pairs_scene(n=300, seed=7)
    ws = world.standard_settings()

    def contacts():
        g = world.GpuWorld(ws, sc.n + 16)
        g.add_bodies(sc.bodies)
        g.step(0.0, 1)
        return g.stats()["num_epa"], {(int(r[0]), int(r[1])): r for r in g.get_manifolds()}

    n_epa, packed = contacts()
    monkeypatch.setenv("CRASHCAT_EPA_PACKED_POINTS", "5")
    _, fallback = contacts()
    assert n_epa > 20
    assert set(packed) == set(fallback)
    for k in packed:
        np.testing.assert_allclose(packed[k][:7], fallback[k][:7], atol=1e-5)
        np.testing.assert_allclose(packed[k][8:], fallback[k][8:], atol=1e-4)


def test_epa_lockstep_rounds_match_the_sequential_pass(gpu_lib, monkeypatch):
    """The packed EPA pass runs a warp's 32 items in lock-step rounds; each lane's polytope sees
    the same operations in the same order as the one-item-per-thread pass (CRASHCAT_EPA_FETCH_WARP
    = 0), so the contacts of a settled batch of worlds, with thousands of EPA items, come out bit
    for bit the same, and so does the state a few steps later."""
    sc = scenes.batched_worlds(num_worlds=64, seed=4)
    ws = world.standard_settings(velocity_iterations=sc.velocity_iterations,
                                 position_iterations=sc.position_iterations)
    ws.num_worlds = sc.num_worlds

    def run():
        g = world.GpuWorld(ws, sc.n + 16)
        g.add_bodies(sc.bodies)
        g.step(sc.dt, 200)
        n_epa = g.stats()["num_epa"]
        m = g.get_manifolds()
        g.step(sc.dt, 5)
        return n_epa, m, g.get_state()[0]

    n_a, m_a, s_a = run()
    monkeypatch.setenv("CRASHCAT_EPA_FETCH_WARP", "0")
    n_b, m_b, s_b = run()
    assert n_a > 500 and n_a == n_b
    np.testing.assert_array_equal(m_a[np.lexsort(m_a[:, 1::-1].T)], m_b[np.lexsort(m_b[:, 1::-1].T)])
    np.testing.assert_array_equal(s_a, s_b)


# ---- capsules ------------------------------------------------------------------------
@pytest.mark.parametrize("seed", [17, 18])
def test_capsule_pairs_and_manifolds(gpu_lib, oracle_lib, seed):
    """Boxes, spheres and capsules (40 %): broadphase pairs bit-exact, contacts within the
    GJK / EPA tolerances of the module docstring."""
    sc = scenes.random_pairs_scene(n=300, seed=seed, capsule_fraction=0.4)
    g, o = make_pair(sc)
    g.step(0.0, 1)
    o.step(0.0, 1)
    assert canonical_pairs(g.get_pairs()) == canonical_pairs(o.pairs())
    gk = {(int(r[0]), int(r[1])): r for r in g.get_manifolds()}
    ok = {(int(r[0]), int(r[1])): r for r in o.manifolds()}
    assert len(ok) > 20
    common = set(gk) & set(ok)
    assert len(common) >= 0.98 * max(len(gk), len(ok))
    bad = [k for k in common if not contact_errors(gk[k], ok[k])]
    assert len(bad) <= 0.02 * len(common), bad[:5]


def test_capsule_edge_clipped_on_box(gpu_lib, oracle_lib):
    """Capsule (body A) lying on a dynamic box: the edge face clipped by clipPolyVsEdge gives
    two points at the cylinder's ends, as in the oracle."""
    import math
    s2 = math.sin(math.pi / 4)
    b = scenes.blank_bodies(2)
    scenes.set_capsule(b, 0, 0.3, 0.6)
    b["position"][0] = (0.0, 0.3 - 0.01, 0.0)
    b["quaternion"][0] = (s2, 0.0, 0.0, s2)
    scenes.set_box(b, 1, (2.0, 0.5, 2.0))
    b["position"][1] = (0.0, -0.5, 0.0)
    sc = scenes.Scene("capsule_on_box", b, dt=1 / 60, steps=1)
    g, o = make_pair(sc)
    g.step(0.0, 1)
    o.step(0.0, 1)
    gm, om = g.get_manifolds(), o.manifolds()
    assert len(gm) == len(om) == 1 and int(gm[0][2]) == int(om[0][2]) == 2
    assert contact_errors(gm[0], om[0])


def test_capsules_on_floor_track_oracle(gpu_lib, oracle_lib):
    """Capsules lying and standing on the floor: 30 steps of velocities and heights."""
    sc = scenes.capsules_on_floor()
    g, o = make_pair(sc)
    for _ in range(3):
        g.step(sc.dt, 10)
        o.step(sc.dt, 10)
        rows, _ = g.get_state()
        st = o.state()
        assert np.abs(rows[:, 1] - st[:, 1]).max() < 2e-3
        assert np.abs(rows[:, 7:10] - st[:, 7:10]).max() < 2e-2
