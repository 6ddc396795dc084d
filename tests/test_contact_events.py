"""Contact events (the post-step buffer standing in for Listener.onContactAdded /
onContactPersisted / onContactRemoved) against the oracle's listener call sites
(contact-constraints.ts:494-499, contacts.ts:305-307), step by step over 120 steps of
bouncing spheres.  The trajectories are FP32 against FP64, so a contact near the
speculative distance may start or end one step apart: at most 3 % of the events may
differ, and every kind must occur."""
import numpy as np
import pytest

from crashcat_gb300 import scenes, world
from oracle import pyoracle

pytestmark = pytest.mark.gpu

NAMES = {1: "added", 2: "persisted", 3: "removed"}


def gpu_events(g):
    ev = {v: set() for v in NAMES.values()}
    for t, a, b in g.contact_events().tolist():
        ev[NAMES[t]].add((a, b))
    return ev


def test_contact_events_match_oracle(gpu_lib, oracle_lib):
    sc = scenes.bouncing_spheres()
    ws = world.standard_settings()
    g = world.GpuWorld(ws, sc.n + 8)
    g.add_bodies(sc.bodies)
    o = pyoracle.OracleWorld(ws, sc.bodies)
    total, diff = 0, 0
    seen = {k: 0 for k in NAMES.values()}
    for _ in range(120):
        g.step(sc.dt, 1)
        o.step(sc.dt, 1)
        ge, oe = gpu_events(g), o.contact_events()
        for k in NAMES.values():
            total += len(oe[k])
            diff += len(ge[k] ^ oe[k])
            seen[k] += len(ge[k])
    assert all(v > 50 for v in seen.values()), seen
    assert diff <= 0.03 * total, (diff, total)


def test_update_world_dispatches_listener_events(gpu_lib):
    """update_world(world, listener, dt) calls the listener's contact callbacks after the step."""
    ws = world.standard_settings()
    w = world.create_world(ws)
    world.create_body(w, world.RigidBodySettings(shape=world.Box((10.0, 0.5, 10.0)), object_layer=1,
                                                 motion_type=0, position=(0.0, -0.5, 0.0)))
    ball = world.create_body(w, world.RigidBodySettings(shape=world.Sphere(0.5), object_layer=0,
                                                        position=(0.0, 0.6, 0.0), restitution=0.8))

    class Recorder:
        def __init__(self):
            self.log = []

        def onContactAdded(self, a, b):
            self.log.append(("added", a.index, b.index))

        def onContactPersisted(self, a, b):
            self.log.append(("persisted", a.index, b.index))

        def onContactRemoved(self, a, b):
            self.log.append(("removed", a.index, b.index))

    rec = Recorder()
    for _ in range(90):
        world.update_world(w, rec, 1.0 / 60.0)
    kinds = [k for k, _, _ in rec.log]
    assert kinds[0] == "added" and "removed" in kinds and "persisted" in kinds
    assert all((a, b) == (0, ball.index) for _, a, b in rec.log)

    class Validator:
        def onContactValidate(self, *a):
            return 0

    with pytest.raises(NotImplementedError):
        world.update_world(w, Validator(), 1.0 / 60.0)
