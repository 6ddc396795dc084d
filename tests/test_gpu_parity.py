"""GPU parity against the FP64 oracle, through the C ABI.

Tolerances (FP32 device state against an FP64 restatement):
  * broadphase pair sets: bit-exact (exact FP64 re-test on the device);
  * contact normals, points and depths: 1e-4 relative (normals: 1e-4 absolute,
    points and depths: 1e-4 m + 1e-4 relative);
  * free-fall integration over 30 steps: 1e-4 relative on positions and velocities;
  * one step of isolated resting contacts: velocities within 2e-3 m/s.
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
    # quaternions up to sign
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


def match_manifolds(gm, om):
    gk = {(int(r[0]), int(r[1])): r for r in gm}
    ok = {(int(r[0]), int(r[1])): r for r in om}
    return gk, ok


@pytest.mark.parametrize("seed", [7, 8])
def test_contact_manifolds(gpu_lib, oracle_lib, seed):
    sc = scenes.random_pairs_scene(n=300, seed=seed)
    g, o = make_pair(sc)
    g.step(0.0, 1)
    o.step(0.0, 1)
    gk, ok = match_manifolds(g.get_manifolds(), o.manifolds())
    assert len(ok) > 20
    # the same body pairs produce contacts, except for pairs within float rounding of the
    # speculative distance; require near-complete agreement
    common = set(gk) & set(ok)
    assert len(common) >= 0.98 * max(len(gk), len(ok))
    bad = []
    for k in common:
        a, b = gk[k], ok[k]
        n_ok = np.abs(a[3:6] - b[3:6]).max() < 1e-4
        d_ok = abs(a[6] - b[6]) < 1e-4 + 1e-4 * abs(b[6])
        # point sets: each oracle point has a GPU point within tolerance
        pg = a[8:8 + 6 * int(a[2])].reshape(-1, 6)
        po = b[8:8 + 6 * int(b[2])].reshape(-1, 6)
        p_ok = int(a[2]) == int(b[2]) and all(
            np.min(np.abs(pg - q).max(1)) < 1e-4 + 1e-4 * np.abs(q).max() for q in po)
        if not (n_ok and d_ok and p_ok):
            bad.append((k, a[2], b[2], a[3:7], b[3:7]))
    assert len(bad) <= 0.01 * len(common), bad[:5]
