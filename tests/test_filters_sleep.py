"""The GPU step's pair filters and sleeping against the oracle.

Filters (filter.ts:159-203, layers.ts:114-124, broadphase.ts:83-138): a scene with three object
layers on two broadphase layers, some layer pairs disabled, and seeded collision groups and masks
on every body; the pair set the GPU step finds (dt = 0: broadphase only, update.ts:101) must be
the oracle's, bit for bit, and so must the manifolds' body pairs after a real step.

Sleeping (sleep.ts:88-117, islands.ts:392-423): boxes settling on a floor and a small stack fall
asleep; the step at which each body falls asleep on the GPU equals the oracle's (the sleep test is
a threshold on motion, so a step of difference is allowed for bodies whose motion sits on the
threshold), and a box dropped onto a sleeping body wakes it on the same step."""
import numpy as np
import pytest

from crashcat_gb300 import scenes, world
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def filtered_settings():
    s = world.create_world_settings()
    bp_moving = world.add_broadphase_layer(s)
    bp_static = world.add_broadphase_layer(s)
    moving = world.add_object_layer(s, bp_moving)
    static = world.add_object_layer(s, bp_static)
    debris = world.add_object_layer(s, bp_moving)
    world.enable_collision(s, moving, moving)
    world.enable_collision(s, moving, static)
    world.enable_collision(s, debris, static)
    world.enable_collision(s, moving, debris)
    world.disable_collision(s, moving, debris)  # on the same broadphase layer, but filtered
    return s, moving, static, debris


def filtered_scene(seed):
    sc = scenes.random_pairs_scene(n=400, seed=seed)
    rng = np.random.default_rng(seed)
    b = sc.bodies
    dyn = b["motion_type"] == 2
    _, moving, static, debris = filtered_settings()
    b["object_layer"][dyn] = np.where(rng.random(dyn.sum()) < 0.3, debris, moving)
    b["collision_groups"][dyn] = rng.integers(1, 16, dyn.sum()).astype(np.uint32)
    b["collision_mask"][dyn] = rng.integers(0, 16, dyn.sum()).astype(np.uint32) | 1
    return sc


def canon(p):
    return sorted(map(tuple, np.sort(np.asarray(p), 1).tolist()))


@pytest.mark.parametrize("seed", [21, 22])
def test_filtered_pairs_match_the_oracle(gpu_lib, oracle_lib, seed):
    sc = filtered_scene(seed)
    ws = filtered_settings()[0]
    g = world.GpuWorld(ws, sc.n + 8)
    g.add_bodies(sc.bodies)
    o = pyoracle.OracleWorld(ws, sc.bodies)
    g.step(0.0, 1)
    o.step(0.0, 1)
    gp, op = canon(g.get_pairs()), canon(o.pairs())
    assert len(op) > 50
    assert gp == op
    # the filters removed pairs that the unfiltered world finds
    ws0 = world.standard_settings()
    b0 = sc.bodies.copy()
    b0["object_layer"][b0["motion_type"] == 2] = 0
    b0["collision_groups"], b0["collision_mask"] = 0xFFFFFFFF, 0xFFFFFFFF
    o0 = pyoracle.OracleWorld(ws0, b0)
    o0.step(0.0, 1)
    assert len(o0.pairs()) > len(op)
    # one real step: the contacts join the same body pairs
    g.step(sc.dt, 1)
    o.step(sc.dt, 1)
    gm = canon(g.get_manifolds()[:, 0:2].astype(int))
    om = canon(o.manifolds()[:, 0:2].astype(int))
    assert len(set(gm) ^ set(om)) <= max(2, len(om) // 50)


def sleep_steps(sleeping):
    """First step at which each body is asleep (-1: never)."""
    s = np.asarray(sleeping)
    first = np.full(s.shape[1], -1)
    for k in range(s.shape[0]):
        new = (first < 0) & (s[k] != 0)
        first[new] = k
    return first


def test_sleep_onset_matches_the_oracle(gpu_lib, oracle_lib):
    sc = scenes.resting_boxes(n=25, seed=3)
    ws = world.standard_settings()
    g = world.GpuWorld(ws, sc.n + 8)
    g.add_bodies(sc.bodies)
    o = pyoracle.OracleWorld(ws, sc.bodies)
    gs, os_ = [], []
    for _ in range(90):
        g.step(sc.dt, 1)
        o.step(sc.dt, 1)
        gs.append(g.get_state()[1].copy())
        os_.append(o.state()[:, 16] != 0)
    fg, fo = sleep_steps(gs), sleep_steps(os_)
    dyn = sc.bodies["motion_type"] == 2
    assert (fo[dyn] >= 0).all()  # every box falls asleep within 1.5 s
    assert np.abs(fg[dyn] - fo[dyn]).max() <= 1


def test_wake_on_impact_matches_the_oracle(gpu_lib, oracle_lib):
    """A box resting on the floor falls asleep; a box dropped from 6 m wakes it on impact, on the
    oracle's step."""
    b = scenes.blank_bodies(3)
    scenes.static_floor(b, 0)
    scenes.set_box(b, [1, 2], (0.5, 0.5, 0.5))
    b["position"][1] = (0.0, 0.49, 0.0)
    b["position"][2] = (0.1, 6.0, 0.0)
    ws = world.standard_settings()
    g = world.GpuWorld(ws, 8)
    g.add_bodies(b)
    o = pyoracle.OracleWorld(ws, b)
    gs, os_ = [], []
    for _ in range(120):
        g.step(1 / 60, 1)
        o.step(1 / 60, 1)
        gs.append(g.get_state()[1][1])
        os_.append(o.state()[1, 16] != 0)
    gs, os_ = np.array(gs, bool), np.array(os_, bool)
    assert os_.any() and gs.any()  # the lower box slept before the impact
    sleep_g, sleep_o = int(np.argmax(gs)), int(np.argmax(os_))
    assert abs(sleep_g - sleep_o) <= 1
    wake_g = sleep_g + int(np.argmax(~gs[sleep_g:]))
    wake_o = sleep_o + int(np.argmax(~os_[sleep_o:]))
    assert not os_[wake_o] and wake_o > sleep_o  # woken by the falling box
    assert abs(wake_g - wake_o) <= 1
