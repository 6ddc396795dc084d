"""cc_world_rollout_grad, the adjoint of the velocity solve and integration over
each step's fixed contact set, against central finite differences (h = 1e-3) of
the full GPU step on scenes whose contact sets stay fixed under the perturbation
(free flight, boxes sliding flat on a floor, a resting box), and the checkpointed
recomputation against itself for several checkpoint spacings.

A directional derivative is checked: FD of L(p + h d) for a seeded direction d
over the initial linear and angular velocities and the per-body friction, against
grad . d from the adjoint; tolerance |fd - ad| <= 0.05 |fd| + 1e-2.  The absolute
term is the FD noise of an FP32 forward: body positions of about 10 m carry about
1e-6 m of rounding, which the division by 2h turns into about 5e-3 on the quotient."""
import numpy as np
import pytest

from crashcat_gb300 import scenes, world

pytestmark = pytest.mark.gpu


def sliders(n=4, air=False, spin=False, seed=3):
    rng = np.random.default_rng(seed)
    b = scenes.blank_bodies(n + 1)
    scenes.static_floor(b, 0, half=(40.0, 0.5, 40.0), friction=0.5)
    idx = np.arange(1, n + 1)
    scenes.set_box(b, idx, (0.4, 0.3, 0.35))
    y = 0.3 + (5.0 if air else 0.0)
    b["position"][idx] = np.stack([np.arange(n) * 4.0, np.full(n, y), np.zeros(n)], 1).astype(np.float32)
    b["linear_velocity"][idx] = np.stack([rng.uniform(1, 3, n), np.zeros(n), rng.uniform(-1, 1, n)], 1).astype(np.float32)
    if spin:
        b["angular_velocity"][idx] = np.stack([np.zeros(n), rng.uniform(-2, 2, n), np.zeros(n)], 1).astype(np.float32)
    b["friction"][idx] = rng.uniform(0.2, 0.8, n).astype(np.float32)
    b["allow_sleeping"][:] = 0
    return b


def make(bodies, nw=1):
    ws = world.standard_settings(allow_sleeping=False)
    ws.num_worlds = nw
    g = world.GpuWorld(ws, len(bodies) + 8)
    g.add_bodies(bodies)
    return g


def host_loss(bodies, targets, dt, steps):
    g = make(bodies)
    g.step(dt, steps)
    rows, _ = g.get_state()
    m = bodies["motion_type"] == 2
    c = rows[m, 0:3].astype(np.float64).mean(0)
    return float(((c - targets[0]) ** 2).sum())


TARGET = np.array([[3.0, 0.2, 1.0]], dtype=np.float32)


@pytest.mark.parametrize("case,steps", [("free_flight", 30), ("flat", 60), ("flat_spin", 60), ("resting", 20)])
def test_adjoint_matches_finite_differences(gpu_lib, case, steps):
    b = {"free_flight": sliders(air=True), "flat": sliders(), "flat_spin": sliders(spin=True),
         "resting": sliders(n=1)}[case]
    dt, h = 1.0 / 60.0, 1e-3
    g = make(b)
    loss, gv, gw, gm = g.rollout_grad(dt, steps, TARGET, checkpoint_every=10)
    assert abs(float(loss[0]) - host_loss(b, TARGET, dt, steps)) < 1e-4 * max(1.0, float(loss[0]))
    rng = np.random.default_rng(11)
    dyn = (b["motion_type"] == 2)[:, None]
    for k in range(3):
        dv = rng.normal(size=(len(b), 3)) * dyn
        dw = rng.normal(size=(len(b), 3)) * dyn * (k >= 1)
        dm = rng.normal(size=len(b)) * dyn[:, 0] * 0.2 * (k == 2)

        def pert(s):
            p = b.copy()
            p["linear_velocity"] = (p["linear_velocity"] + s * h * dv).astype(np.float32)
            p["angular_velocity"] = (p["angular_velocity"] + s * h * dw).astype(np.float32)
            p["friction"] = (p["friction"] + s * h * dm).astype(np.float32)
            return p

        fd = (host_loss(pert(1), TARGET, dt, steps) - host_loss(pert(-1), TARGET, dt, steps)) / (2 * h)
        ad = float((gv * dv).sum() + (gw * dw).sum() + (gm * dm).sum())
        assert abs(fd - ad) <= 0.05 * abs(fd) + 1e-2, (case, k, fd, ad)


def test_checkpoint_spacing_does_not_change_the_gradient(gpu_lib):
    """Recomputing segments from checkpoints reproduces the forward exactly: the step is
    deterministic and the loss and friction gradient sum in fixed point, so spacings 1, 7 and
    40 over a 40-step rollout of colliding boxes give bit-identical losses and gradients."""
    sc, targets = scenes.diff_rollout_worlds(num_worlds=2, boxes=64)
    out = []
    for K in (1, 7, 40):
        g = make(sc.bodies, 2)
        out.append(g.rollout_grad(sc.dt, 40, targets, checkpoint_every=K))
    for o in out[1:]:
        for a, b in zip(out[0], o):
            np.testing.assert_array_equal(a, b)


def test_rollout_leaves_the_forward_state(gpu_lib):
    """After cc_world_rollout_grad the world is where n plain steps would have left it."""
    sc, targets = scenes.diff_rollout_worlds(num_worlds=2, boxes=64)
    g1 = make(sc.bodies, 2)
    g1.rollout_grad(sc.dt, 25, targets, checkpoint_every=10)
    g2 = make(sc.bodies, 2)
    g2.step(sc.dt, 25)
    r1, _ = g1.get_state()
    r2, _ = g2.get_state()
    np.testing.assert_array_equal(r1, r2)
