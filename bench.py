"""Benchmark of the GB300 world step on the batched uneven-worlds workload.

Workload: 4,096 independent worlds whose body counts are drawn log-uniformly
from 8 to 512 (boxes and spheres, each world with its own static floor), dt
1/120 s, 8 velocity / 2 position iterations; a "step" advances every world
once.  Metric: body-steps/s (higher is better).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl gb300 (default): value = bodies x K / device time of K steps (CUDA
events on the library's stream, body state resident in HBM); e2e = the same
metric through cc_world_step_host with the body state rows uploaded from and
read back into pinned host memory every step; roofline of the dominant stage
from the stage profiler; cpu_baseline = the FP64 oracle port timed single
threaded on a bounded sample of the same worlds.

vs_single_world: the same settled worlds stepped through the plain single-world
path (one cc_world handle per world, cc_world_step(handle, dt, 1) world after
world, as a caller without the batched form would) on a spread sample of the
4,096 worlds; both paths run the same kernels and settings, so the tolerance is
the same.  value = sampled bodies x steps / wall time of the sampled worlds'
steps; batched_over_single = the batched value / that value.

adjoint: the differentiable-rollout workload (1,024 worlds x 64 boxes, 120 steps at
dt 1/60, checkpoint every 10 steps).  forward_ms_per_step = the plain rollout (graph-
replayed steps, CUDA events); ms_per_step = cc_world_rollout_grad (forward with
checkpoints, recomputation with tapes, reverse sweep, gradients to the host) / 120;
fd_check: on the first 8 worlds, the adjoint's directional derivative along seeded
directions against the oracle's FP64 dual-number replay of the GPU's per-step solver rows
(the model the adjoint differentiates), against central differences (h = 1e-3 and 1e-5) of
that frozen-contact replay, and against central differences of the full GPU step.

error: the batched workload's first 16 worlds stepped through the settle phase on the GPU and
on the FP64 oracle: penetration, mechanical energy and resting heights on each side, energy
drift, and how far positions diverged.  cube_heap, ragdolls, terrain and adjoint carry the
same report for their workloads.

cube_heap: the plain single-world workload (1,000 boxes dropped on a floor, dt 1/60, 10/2
iterations, 600 steps) through cc_world_step, with its stage roofline; its cpu_baseline is the
oracle on the whole workload (600 steps, one core).

ragdolls: the jointed-ragdoll workload (2,000 ragdolls x 11 capsules with 4 hinges and 6
swing-twist joints each, 600 steps at dt 1/60, 12/4 iterations): GPU body-steps/s over the
whole run with per-phase ms/step (the ragdolls fall, then pile into one giant island solved
by the whole grid); cpu_baseline = the oracle on the same scene for a bounded number of steps
from spawn, against the GPU's value over the same falling phase.

--impl reference: the reference (TypeScript) cannot run on this machine; its FP64
C++ restatement (oracle/) steps a bounded sample of the same worlds on all
host cores (one process per core, worlds split across them).

Under torchrun (N > 1) every rank steps its own 4,096 worlds (weak scaling, no
collective on the data path); timing is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

WORKLOAD = "batched_uneven_worlds"
METRIC = "body-steps/s"
STAGES = ("integrate_forces", "broadphase", "narrowphase", "epa", "contacts_islands", "solve_small_islands",
          "solve_large_islands")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--worlds", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=4)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--adjoint", type=int, default=1, help="measure the rollout adjoint (1) or skip it (0)")
    ap.add_argument("--ragdolls", type=int, default=1, help="measure the jointed-ragdoll workload (1) or skip it (0)")
    ap.add_argument("--terrain", type=int, default=1, help="measure the mixed-shape terrain workload (1) or skip it (0)")
    ap.add_argument("--cube-heap", type=int, default=1, help="measure the plain cube-heap workload (1) or skip it (0)")
    ap.add_argument("--tune", type=int, default=1, help="autotune the launch shapes before the warm-up (1) or not (0)")
    ap.add_argument("--only", default="", choices=["", "cube_heap"],
                    help="run one workload alone and print its report (for profiling)")
    ap.add_argument("--errors", type=int, default=1,
                    help="report the batched workload's error against the FP64 oracle (1) or skip it (0)")
    ap.add_argument("--settle", type=int, default=360,
                    help="untimed steps before the warm-up so the timed steps are contact-rich")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def read_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        import tempfile
        self.gpu = gpu_index
        self.proc = None
        fd, self.path = tempfile.mkstemp(prefix=f"crashcat_clocks_rank{gpu_index}_", suffix=".csv")
        os.close(fd)

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        try:
            os.unlink(self.path)
        except OSError:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def algorithmic_bytes(stage: str, st: dict, n_bodies: int) -> float:
    """Compulsory FP32 bytes of one stage per step (each datum counted once).

    Per awake body 216 B (state read 76, properties 64, state write 52, AABB 24),
    per body 104 B for the tree (AABB 24, key/index 16, node write + read 64),
    per pair 16 B (write + read) plus 72 B of narrowphase input (two transforms
    and shape handles), per manifold (20 + 24 P) B written by the narrowphase,
    (48 + 180 P) B of constraint rows written by the contact setup and read by
    the solver, and 24 P B of impulse cache, P = mean points per manifold.
    """
    na = st["num_awake"]
    npairs = st["num_pairs"]
    nm = max(st["num_manifolds"], 0)
    P = (st["num_contact_points"] / nm) if nm else 0.0
    if stage == "integrate_forces":
        return 148.0 * na
    if stage == "broadphase":
        return 104.0 * n_bodies + 16.0 * npairs
    if stage == "narrowphase":
        return 72.0 * npairs + (20 + 24 * P) * nm
    if stage == "epa":
        ne = st["num_epa"]
        return (72.0 + 20 + 24 * P) * ne
    if stage == "contacts_islands":
        return (20 + 24 * P) * nm + (48 + 180 * P) * nm + 24 * P * nm
    if stage in ("solver", "solve_small_islands", "solve_large_islands"):
        # both solver kernels together move these bytes; each is charged its share of them
        return 216.0 * na + (48 + 180 * P) * nm + 24 * P * nm
    raise ValueError(stage)


# ---------------------------------------------------------------------------
# error against the FP64 oracle, per workload (penetration, energy, resting heights)
# ---------------------------------------------------------------------------
def mass_properties(bodies, hulls=()):
    """Mass and body-frame inertia tensor (about the centre of mass) of every body: solid boxes,
    spheres and capsules (cylinder plus two hemispheres), convex hulls from their built volume and
    unit-density inertia.  Used for the energy figures only."""
    n = len(bodies)
    m = np.zeros(n)
    inertia = np.zeros((n, 3, 3))
    rho = bodies["density"].astype(np.float64)
    prm = bodies["shape_params"].astype(np.float64)
    for i in range(n):
        st = int(bodies["shape_type"][i])
        if st == 1:  # box
            hx, hy, hz = prm[i, 0:3]
            m[i] = rho[i] * 8 * hx * hy * hz
            inertia[i] = np.diag([hy * hy + hz * hz, hx * hx + hz * hz, hx * hx + hy * hy]) * m[i] / 3
        elif st == 0:  # sphere
            r = prm[i, 0]
            m[i] = rho[i] * 4.0 / 3.0 * math.pi * r ** 3
            inertia[i] = np.eye(3) * 0.4 * m[i] * r * r
        elif st == 2:  # capsule along local Y
            r, h = prm[i, 0], prm[i, 1]
            mc, ms = rho[i] * math.pi * r * r * 2 * h, rho[i] * 4.0 / 3.0 * math.pi * r ** 3
            iy = mc * r * r / 2 + ms * 0.4 * r * r
            ix = mc * (r * r / 4 + (2 * h) ** 2 / 12) + ms * (0.4 * r * r + h * h + 0.75 * h * r)
            m[i] = mc + ms
            inertia[i] = np.diag([ix, iy, ix])
        elif st == 3 and hulls:  # convex hull
            hd = hulls[int(prm[i, 0])]
            m[i] = rho[i] * float(hd["volume"])
            inertia[i] = rho[i] * np.asarray(hd["inertia"], dtype=np.float64)
    return m, inertia


def _quat_matrices(q):
    x, y, z, w = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
                     np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
                     np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1)], 1)


def step_metrics(rows, bodies, depths, mass, inertia, g: float = 9.81) -> dict:
    """Mechanical energy (kinetic + rotational + potential m g y of the centre of mass), contact
    penetration (positive manifold depths of the last step) and centre-of-mass heights of the
    dynamic bodies, from state rows (position, quaternion, linear / angular velocity, centre of mass:
    the first 16 columns of both the GPU's and the oracle's rows)."""
    r = np.asarray(rows, dtype=np.float64)
    dyn = bodies["motion_type"] == 2
    v, w, com = r[dyn, 7:10], r[dyn, 10:13], r[dyn, 13:16]
    R = _quat_matrices(r[dyn, 3:7] / np.linalg.norm(r[dyn, 3:7], axis=1, keepdims=True))
    Iw = R @ inertia[dyn] @ np.transpose(R, (0, 2, 1))
    ke = 0.5 * float((mass[dyn] * (v * v).sum(1)).sum()) + 0.5 * float(np.einsum("ni,nij,nj->", w, Iw, w))
    pe = float((mass[dyn] * g * com[:, 1]).sum())
    pen = np.maximum(np.asarray(depths, dtype=np.float64), 0.0)
    return {"energy_j": ke + pe, "kinetic_j": ke, "max_penetration_m": float(pen.max()) if len(pen) else 0.0,
            "mean_penetration_m": float(pen.mean()) if len(pen) else 0.0, "contacts": int(len(pen)),
            "mean_height_m": float(com[:, 1].mean()), "min_height_m": float(com[:, 1].min())}


def error_report(bodies, rows0, gpu_rows, gpu_depths, orc_rows, orc_depths, mass, inertia, steps: int,
                 note: str = "") -> dict:
    """The GPU against the FP64 oracle after `steps` steps from the same start: both sides'
    metrics, their energy drifts from the start, and how far the bodies' positions diverged."""
    s0 = step_metrics(rows0, bodies, [], mass, inertia)
    g = step_metrics(gpu_rows, bodies, gpu_depths, mass, inertia)
    o = step_metrics(orc_rows, bodies, orc_depths, mass, inertia)
    dyn = bodies["motion_type"] == 2
    dp = np.linalg.norm(np.asarray(gpu_rows, np.float64)[dyn, 0:3] - np.asarray(orc_rows, np.float64)[dyn, 0:3], axis=1)
    drift_o = o["energy_j"] - s0["energy_j"]
    return {"steps": steps, "gpu": g, "oracle": o, "initial_energy_j": s0["energy_j"],
            "energy_drift_gpu_j": g["energy_j"] - s0["energy_j"], "energy_drift_oracle_j": drift_o,
            "energy_drift_rel_diff": abs(g["energy_j"] - o["energy_j"]) / max(abs(drift_o), 1e-9),
            "max_penetration_diff_m": g["max_penetration_m"] - o["max_penetration_m"],
            "mean_height_diff_m": g["mean_height_m"] - o["mean_height_m"],
            "position_diff_m": {"median": float(np.median(dp)), "p95": float(np.percentile(dp, 95)),
                                "max": float(dp.max())},
            "note": note}


# ---------------------------------------------------------------------------
# CPU legs (the oracle is test infrastructure: only the baseline legs use it)
# ---------------------------------------------------------------------------
def _cpu_worker(args):
    """Steps a list of worlds with the FP64 oracle; returns seconds for `steps` steps."""
    bodies_list, dt, vel, pos, steps = args
    sys.path.insert(0, ROOT)
    from crashcat_gb300 import world as W
    from oracle import pyoracle
    ws = W.standard_settings(velocity_iterations=vel, position_iterations=pos)
    worlds = [pyoracle.OracleWorld(ws, b) for b in bodies_list]
    t0 = time.perf_counter()
    for _ in range(steps):
        for o in worlds:
            o.step(dt, 1)
    return time.perf_counter() - t0


def _cpu_process(bodies_list, dt, vel, pos, settle, warmup, steps, barrier, out_q, slot):
    """One host core of the reference leg: settle + warm up its worlds, then time `steps`
    steps after every core has reached the barrier."""
    sys.path.insert(0, ROOT)
    from crashcat_gb300 import world as W
    from oracle import pyoracle
    ws = W.standard_settings(velocity_iterations=vel, position_iterations=pos)
    worlds = [pyoracle.OracleWorld(ws, b) for b in bodies_list]
    for o in worlds:
        o.step(dt, settle + warmup)
    barrier.wait()
    t0 = time.perf_counter()
    for _ in range(steps):
        for o in worlds:
            o.step(dt, 1)
    out_q.put((slot, time.perf_counter() - t0))


def split_worlds(scene):
    w = scene.bodies["world"]
    starts = np.flatnonzero(np.r_[True, np.diff(w) != 0])
    ends = np.r_[starts[1:], len(w)]
    return [scene.bodies[s:e].copy() for s, e in zip(starts, ends)]


def cpu_baseline_single(scene, seconds: float, state_rows=None):
    """Single-threaded oracle on the first worlds of the workload, ~`seconds` of work,
    starting from `state_rows` (the GPU's state after its timed steps) when given."""
    from oracle import build as obuild
    obuild.build()
    if state_rows is not None:
        b = scene.bodies.copy()
        b["position"] = state_rows[:, 0:3]
        b["quaternion"] = state_rows[:, 3:7]
        b["linear_velocity"] = state_rows[:, 7:10]
        b["angular_velocity"] = state_rows[:, 10:13]
        scene = type(scene)(**{**scene.__dict__, "bodies": b})
    worlds = split_worlds(scene)
    # calibrate on a handful of worlds
    probe = worlds[:16]
    nb = sum(len(b) for b in probe)
    t = _cpu_worker((probe, scene.dt, scene.velocity_iterations, scene.position_iterations, 2))
    per_body_step = max(t / (2 * nb), 1e-7)
    steps = 10
    target_bodies = int(seconds / (per_body_step * steps))
    sample, tot = [], 0
    for b in worlds:
        if tot >= target_bodies:
            break
        sample.append(b)
        tot += len(b)
    t = _cpu_worker((sample, scene.dt, scene.velocity_iterations, scene.position_iterations, steps))
    return {"value": tot * steps / t, "unit": METRIC, "cores": 1, "kind": "port",
            "sample": f"first {len(sample)} of {len(worlds)} worlds ({tot} bodies), {steps} steps from the "
                      f"GPU's settled state, FP64 oracle, one thread, {t:.1f} s"}


def run_reference(args, rank, world_size):
    if rank != 0:
        return
    import multiprocessing as mp
    from crashcat_gb300 import scenes
    from oracle import build as obuild
    obuild.build()
    scene = scenes.batched_worlds(num_worlds=args.worlds, seed=args.seed)
    worlds = split_worlds(scene)
    cores = os.cpu_count() or 1
    # bounded sample: 32 worlds per host core, stepped in parallel (one process per core)
    sample = worlds[: min(len(worlds), 32 * cores)]
    nb = sum(len(b) for b in sample)
    chunks = [sample[i::cores] for i in range(cores)]
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(cores + 1)
    out_q = ctx.Queue()
    procs = [ctx.Process(target=_cpu_process, args=(c, scene.dt, scene.velocity_iterations,
                                                    scene.position_iterations, args.settle, args.warmup,
                                                    args.steps, barrier, out_q, i)) for i, c in enumerate(chunks)]
    for p in procs:
        p.start()
    barrier.wait()
    t0 = time.perf_counter()
    times = [out_q.get()[1] for _ in procs]
    wall = time.perf_counter() - t0
    for p in procs:
        p.join()
    value = nb * args.steps / wall
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "worlds": args.worlds, "sample_worlds": len(sample),
                   "sample_bodies": nb, "dt": scene.dt, "velocity_iterations": scene.velocity_iterations,
                   "position_iterations": scene.position_iterations, "seed": args.seed,
                   "settle_steps": args.settle},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": cores, "kind": "port",
                         "sample": f"{len(sample)} worlds ({nb} bodies) split over {cores} processes, timed "
                                   f"after {args.settle + args.warmup} untimed steps; the TypeScript reference "
                                   f"cannot run here, its FP64 C++ restatement is timed (slowest process "
                                   f"{max(times):.2f} s)"},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU leg
# ---------------------------------------------------------------------------
def adjoint_measurement(num_worlds: int = 1024, steps: int = 120, checkpoint_every: int = 10):
    """Adjoint ms/step of the differentiable-rollout workload against its forward ms/step."""
    import copy
    from crashcat_gb300 import scenes, world as W
    sc, targets = scenes.diff_rollout_worlds(num_worlds=num_worlds)

    def make(bodies, nw):
        ws = W.standard_settings(velocity_iterations=sc.velocity_iterations,
                                 position_iterations=sc.position_iterations, allow_sleeping=False)
        ws.num_worlds = nw
        g = W.GpuWorld(ws, len(bodies) + 8)
        g.add_bodies(bodies)
        return g

    gf = make(sc.bodies, num_worlds)
    gf.step(sc.dt, 1)
    gf.step(sc.dt, steps - 1)
    fwd_ms = gf.stats()["last_call_ms"] / (steps - 1)
    del gf
    ga = make(sc.bodies, num_worlds)
    loss, gv, gw, gm = ga.rollout_grad(sc.dt, steps, targets, checkpoint_every=checkpoint_every)
    adj_ms = ga.stats()["last_call_ms"] / steps
    del ga
    # finite differences on the first 8 worlds
    nw = 8
    sub = sc.bodies[sc.bodies["world"] < nw].copy()
    tg = targets[:nw]

    def host_loss(b):
        g = make(b, nw)
        g.step(sc.dt, steps)
        rows, _ = g.get_state()
        tot = 0.0
        for k in range(nw):
            m = (b["world"] == k) & (b["motion_type"] == 2)
            tot += float(((rows[m, 0:3].astype(np.float64).mean(0) - tg[k]) ** 2).sum())
        return tot

    g8 = make(sub, nw)
    loss8, gv8, gw8, gm8 = g8.rollout_grad(sc.dt, steps, tg, checkpoint_every=checkpoint_every)
    # the rows of every step of the same rollout (cc_world_step_taped) for the oracle's frozen-contact
    # replay: FP64 central differences through the replay and its FP64 dual-number derivative
    from oracle import build as obuild, pyoracle
    obuild.build()
    gt = make(sub, nw)
    tape = pyoracle.FrozenTape(pyoracle.tape_consts(sub, sc.dt), tg, sc.velocity_iterations, sc.dt)
    rows, _ = gt.get_state()
    for _ in range(steps):
        tb, tc, ratio, _st = gt.step_taped(sc.dt)
        b_rows, c_rows = pyoracle.tape_rows_from_gpu(tb, tc)
        tape.add_step(b_rows, rows[:, 7:13], ratio, c_rows)
        rows, _ = gt.get_state()
    tape.finish(rows[:, 0:3])
    rows_g, depth_g = rows.copy(), gt.get_manifolds()[:, 6]
    del gt
    tape_loss, _ = tape.replay(0)
    # the forward rollout's error against the oracle, one oracle world per world
    import copy as _copy
    ws1 = W.standard_settings(velocity_iterations=sc.velocity_iterations,
                              position_iterations=sc.position_iterations, allow_sleeping=False)
    rows_o, depth_o = [], []
    for k in range(nw):
        bk = _copy.deepcopy(sub[sub["world"] == k])
        bk["world"] = 0
        o = pyoracle.OracleWorld(ws1, bk)
        o.step(sc.dt, steps)
        rows_o.append(o.state())
        depth_o.append(o.manifolds()[:, 6])
    rows_start, _ = make(sub, nw).get_state()
    m8, i8 = mass_properties(sub)
    fwd_err = error_report(sub, rows_start, rows_g, depth_g, np.concatenate(rows_o), np.concatenate(depth_o), m8, i8,
                           steps, f"the first {nw} worlds, {steps} steps from the start")
    rng = np.random.default_rng(5)
    dyn = (sub["motion_type"] == 2)[:, None]
    checks, h = [], 1e-3
    for k in range(3):
        dv = rng.normal(size=(len(sub), 3)) * dyn
        dw = rng.normal(size=(len(sub), 3)) * dyn * (k >= 1)
        dm = rng.normal(size=len(sub)) * dyn[:, 0] * 0.2 * (k == 2)

        def pert(sgn):
            b = copy.deepcopy(sub)
            b["linear_velocity"] = (b["linear_velocity"] + sgn * h * dv).astype(np.float32)
            b["angular_velocity"] = (b["angular_velocity"] + sgn * h * dw).astype(np.float32)
            b["friction"] = (b["friction"] + sgn * h * dm).astype(np.float32)
            return b

        fd = (host_loss(pert(1)) - host_loss(pert(-1))) / (2 * h)
        ad = float((gv8 * dv).sum() + (gw8 * dw).sum() + (gm8 * dm).sum())
        _, dual = tape.replay(0, 0.0, dv, dw, dm)
        lp, _ = tape.replay(1, h, dv, dw, dm)
        lm, _ = tape.replay(1, -h, dv, dw, dm)
        ffd = (lp - lm) / (2 * h)
        lp5, _ = tape.replay(1, 1e-5, dv, dw, dm)
        lm5, _ = tape.replay(1, -1e-5, dv, dw, dm)
        ffd5 = (lp5 - lm5) / 2e-5
        checks.append({"direction": ["v", "v+w", "v+w+friction"][k], "adjoint": ad,
                       "fp64_dual": dual, "rel_err_vs_dual": abs(dual - ad) / max(abs(dual), 1e-12),
                       "frozen_fd": ffd, "rel_err_vs_frozen_fd": abs(ffd - ad) / max(abs(ffd), 1e-12),
                       "frozen_fd_h1e-5": ffd5, "rel_err_vs_frozen_fd_h1e-5": abs(ffd5 - ad) / max(abs(ffd5), 1e-12),
                       "full_step_fd": fd, "rel_err_vs_full_step_fd": abs(fd - ad) / max(abs(fd), 1e-12)})
    return {"workload": "diff_rollout_worlds", "worlds": num_worlds, "bodies": int(sc.n), "steps": steps,
            "checkpoint_every": checkpoint_every, "ms_per_step": adj_ms, "forward_ms_per_step": fwd_ms,
            "adjoint_over_forward": adj_ms / fwd_ms, "loss": float(loss.sum()),
            "grad_norms": {"linvel": float(np.linalg.norm(gv)), "angvel": float(np.linalg.norm(gw)),
                           "friction": float(np.linalg.norm(gm))},
            "error": fwd_err,
            "fd_check": {"worlds": nw, "h": h, "directions": checks,
                         "tape_loss_fp64": tape_loss, "adjoint_loss": float(loss8.sum()),
                         "model": "the adjoint differentiates each step's velocity solve and integration over its "
                                  "fixed contact rows; fp64_dual = the oracle's FP64 dual-number replay of the GPU's "
                                  "rows (cc_world_step_taped), frozen_fd = central differences of that replay "
                                  "(FP64); full_step_fd = central differences of the full GPU step, whose contact "
                                  "set and geometry move with the perturbation"}}


def cube_heap_measurement(peak: float, peak_kind: str, oracle: bool = True):
    """The plain cube heap (1,000 boxes on a 10 x 10 x 10 grid dropped onto a static box floor,
    dt 1/60, 10/2 iterations, 600 steps) on one single-world handle through cc_world_step:
    body-steps/s over all 600 steps (1,001 bodies, the floor included as in the batched figure),
    per phase, with the dominant stage's roofline on the settled heap; the FP64 oracle steps the
    same 600 steps on one host core (the whole workload: it is CPU-runnable), and the error of
    the GPU against it after the 600 steps."""
    from crashcat_gb300 import scenes, world as W
    from oracle import build as obuild, pyoracle
    sc = scenes.cube_heap()
    ws = W.standard_settings(velocity_iterations=sc.velocity_iterations, position_iterations=sc.position_iterations)
    g = W.GpuWorld(ws, sc.n + 8)
    g.add_bodies(sc.bodies)
    rows0, _ = g.get_state()
    phases, total_ms, status = [], 0.0, 0
    for first, count in ((0, 100), (100, 500)):
        status |= g.step(sc.dt, count)
        st = g.stats()
        total_ms += st["last_call_ms"]
        phases.append({"steps": [first, first + count], "ms_per_step": st["last_call_ms"] / count,
                       "awake": st["num_awake"], "manifolds": st["num_manifolds"], "islands": st["num_islands"],
                       "max_island_constraints": st["max_island_constraints"]})
    rows_g, _ = g.get_state()
    depth_g = g.get_manifolds()[:, 6]
    prof = g.profile_steps(sc.dt, 10)
    pst = g.stats()
    dom = max(prof, key=prof.get)
    bytes_dom = algorithmic_bytes(dom, pst, sc.n)
    achieved = bytes_dom / (prof[dom] * 1e-3) / 1e9 if prof[dom] > 0 else 0.0
    del g
    if not oracle:
        return {"workload": "cube_heap", "value": sc.n * 600 / (total_ms * 1e-3), "unit": METRIC,
                "ms_per_step": total_ms / 600, "phases": phases, "stage_ms": prof}
    obuild.build()
    o = pyoracle.OracleWorld(ws, sc.bodies)
    t0 = time.perf_counter()
    o.step(sc.dt, 600)
    cpu_s = time.perf_counter() - t0
    rows_o = o.state()
    depth_o = o.manifolds()[:, 6]
    m, inertia = mass_properties(sc.bodies)
    return {"workload": "cube_heap", "bodies": int(sc.n), "steps": 600, "api": "cc_world_step (one world)",
            "value": sc.n * 600 / (total_ms * 1e-3), "unit": METRIC, "ms_per_step": total_ms / 600,
            "phases": phases, "status": int(status),
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind, "algorithmic_bytes_per_launch": bytes_dom,
                         "stage_ms": prof, "note": "one world of 1,001 bodies: launch and latency bound"},
            "cpu_baseline": {"value": sc.n * 600 / cpu_s, "unit": METRIC, "cores": 1, "kind": "port",
                             "sample": "the whole workload: all 600 steps from the same start, FP64 oracle"},
            "error": error_report(sc.bodies, rows0, rows_g, depth_g, rows_o, depth_o, m, inertia, 600,
                                  "after 600 steps from the same start; the stacks topple chaotically, so "
                                  "per-body positions diverge while heights, energy and penetration agree")}


def batched_error(scene, ws_batched, steps: int = 360, worlds: int = 16) -> dict:
    """The batched workload's error against the oracle: its first `worlds` worlds stepped `steps`
    steps (the settle phase) by a batched GPU handle holding just them and by the oracle, one
    oracle world per world."""
    import copy
    from crashcat_gb300 import world as W
    from oracle import build as obuild, pyoracle
    obuild.build()
    parts = split_worlds(scene)[:worlds]
    bodies = np.concatenate(parts)
    ws = copy.deepcopy(ws_batched)
    ws.num_worlds = worlds
    g = W.GpuWorld(ws, len(bodies) + 8)
    g.add_bodies(bodies)
    rows0, _ = g.get_state()
    g.step(scene.dt, steps)
    rows_g, _ = g.get_state()
    depth_g = g.get_manifolds()[:, 6]
    del g
    ws1 = copy.deepcopy(ws_batched)
    ws1.num_worlds = 1
    rows_o, depth_o = [], []
    t0 = time.perf_counter()
    for b in parts:
        b = b.copy()
        b["world"] = 0
        o = pyoracle.OracleWorld(ws1, b)
        o.step(scene.dt, steps)
        rows_o.append(o.state())
        depth_o.append(o.manifolds()[:, 6])
    cpu_s = time.perf_counter() - t0
    m, inertia = mass_properties(bodies)
    rep = error_report(bodies, rows0, rows_g, depth_g, np.concatenate(rows_o), np.concatenate(depth_o), m, inertia,
                       steps, f"the first {worlds} of the {scene.num_worlds} worlds ({len(bodies)} bodies), the "
                              f"{steps} settle steps from spawn")
    rep["oracle_seconds"] = cpu_s
    return rep


def joint_gaps(sc, rows) -> np.ndarray:
    """Distance between the two bodies' anchor points of every hinge and swing-twist joint at the
    poses in rows (the anchors taken in each body's frame at creation): 0 for a joint that holds."""
    def rot(q, v):
        u = q[..., :3]
        t = 2.0 * np.cross(u, v)
        return v + q[..., 3:4] * t + np.cross(u, t)

    out = []
    b = sc.bodies
    r = np.asarray(rows, dtype=np.float64)
    for recs, fa, fb in ((sc.hinges, "point_a", "point_b"), (sc.swings, "position_a", "position_b")):
        if recs is None or len(recs) == 0:
            continue
        ends = []
        for body_f, f in (("body_a", fa), ("body_b", fb)):
            i = recs[body_f]
            q0 = b["quaternion"][i].astype(np.float64) * np.array([-1, -1, -1, 1.0])
            local = rot(q0, recs[f].astype(np.float64) - b["position"][i].astype(np.float64))
            ends.append(r[i, 0:3] + rot(r[i, 3:7], local))
        out.append(np.linalg.norm(ends[0] - ends[1], axis=1))
    return np.concatenate(out) if out else np.zeros(0)


def _ragdoll_worlds(sc, ws):
    from crashcat_gb300 import world as W
    from oracle import pyoracle
    g = W.GpuWorld(ws, sc.n + 16)
    g.add_bodies(sc.bodies)
    g.add_hinges(sc.hinges)
    g.add_swing_twists(sc.swings)
    g.set_skip_joint_pairs(True)
    o = pyoracle.OracleWorld(ws, sc.bodies)
    for h in sc.hinges:
        o.add_hinge_record(h)
    for h in sc.swings:
        o.add_swing_twist_record(h)
    o.set_skip_joint_pairs(True)
    return g, o


def ragdoll_measurement(cpu_seconds: float = 8.0):
    """The jointed-ragdoll workload (2,000 ragdolls of 11 capsules at seeded random joint poses,
    4 hinges and 6 swing-twist joints each, in a 60 m arena of static walls; dt 1/60, 12/4
    iterations): all 600 steps from spawn on the GPU, timed per phase (falling, piling up,
    resting pile).  The FP64 oracle on one host core: the first steps from spawn (the falling
    phase) and a few steps of the resting pile from the GPU's state after 600 steps.  The error:
    27 ragdolls in a 16 m arena (the same generator), 300 steps on the GPU and on the oracle."""
    from crashcat_gb300 import scenes, world as W
    from oracle import build as obuild
    obuild.build()
    sc = scenes.ragdolls()
    ws = W.standard_settings(velocity_iterations=sc.velocity_iterations, position_iterations=sc.position_iterations)
    g, o = _ragdoll_worlds(sc, ws)
    phases, total_ms, status = [], 0.0, 0
    for first, count in ((0, 100), (100, 400), (500, 100)):
        status |= g.step(sc.dt, count)
        st = g.stats()
        total_ms += st["last_call_ms"]
        phases.append({"steps": [first, first + count], "ms_per_step": st["last_call_ms"] / count,
                       "islands": st["num_islands"], "max_island_constraints": st["max_island_constraints"],
                       "giant_islands": st["num_giant_islands"], "giant_colours": st["giant_colours"],
                       "manifolds": st["num_manifolds"]})
    rows, _ = g.get_state()
    gaps_g = joint_gaps(sc, rows)
    del g
    t0, k = time.perf_counter(), 0
    while time.perf_counter() - t0 < cpu_seconds and k < 100:
        o.step(sc.dt, 1)
        k += 1
    cpu_s = time.perf_counter() - t0
    # the resting pile: the oracle from the GPU's state after the 600 steps (positions, orientations
    # and velocities; its contact cache and joint impulses start empty)
    st = o.state()
    st[:, 0:13] = rows[:, 0:13]
    o.set_state(st)
    t0, kp = time.perf_counter(), 0
    while time.perf_counter() - t0 < cpu_seconds and kp < 20:
        o.step(sc.dt, 1)
        kp += 1
    pile_s = time.perf_counter() - t0
    del o
    # error against the oracle on a small arena of the same generator
    se = scenes.ragdolls(num=27, arena=16.0)
    ge, oe = _ragdoll_worlds(se, ws)
    rows0, _ = ge.get_state()
    ge.step(se.dt, 300)
    oe.step(se.dt, 300)
    rg, _ = ge.get_state()
    ro = oe.state()
    m, inertia = mass_properties(se.bodies)
    err = error_report(se.bodies, rows0, rg, ge.get_manifolds()[:, 6], ro, oe.manifolds()[:, 6], m, inertia, 300,
                       "27 ragdolls in a 16 m arena, 300 steps from spawn")
    jg, jo = joint_gaps(se, rg), joint_gaps(se, ro)
    err["joint_gap_m"] = {"gpu_max": float(jg.max()), "gpu_mean": float(jg.mean()), "oracle_max": float(jo.max()),
                          "oracle_mean": float(jo.mean())}
    gpu_first = phases[0]["ms_per_step"]
    return {"workload": "ragdolls", "ragdolls": 2000, "bodies": int(sc.n), "hinges": int(len(sc.hinges)),
            "swing_twists": int(len(sc.swings)), "steps": 600, "value": sc.n * 600 / (total_ms * 1e-3),
            "unit": METRIC, "ms_per_step": total_ms / 600, "phases": phases, "status": int(status),
            "finite": bool(np.isfinite(rows).all()), "spawn": "seeded random joint poses inside 60 % of the limits",
            "joint_gap_after_600_m": {"max": float(gaps_g.max()), "mean": float(gaps_g.mean())},
            "cpu_baseline": {"value": sc.n * k / cpu_s, "unit": METRIC, "cores": 1, "kind": "port",
                             "sample": f"first {k} steps from spawn (falling phase)",
                             "gpu_same_phase_value": sc.n / (gpu_first * 1e-3)},
            "cpu_baseline_pile": {"value": sc.n * kp / pile_s, "unit": METRIC, "cores": 1, "kind": "port",
                                  "sample": f"{kp} steps of the resting pile from the GPU's state after 600 steps",
                                  "gpu_same_phase_value": sc.n / (phases[2]["ms_per_step"] * 1e-3)},
            "error": err}


def terrain_rays(n: int, half: float, seed: int = 3) -> np.ndarray:
    """Rays from 20-50 m above the terrain, pointing down at random (y component at most -0.5 before
    normalising), 100 m long: a cc_ray array."""
    from crashcat_gb300 import _lib
    rng = np.random.default_rng(seed)
    r = np.zeros(n, _lib.RAY_DTYPE)
    r["origin"] = np.stack([rng.uniform(-half, half, n), rng.uniform(20.0, 50.0, n), rng.uniform(-half, half, n)], 1)
    d = rng.normal(size=(n, 3))
    d[:, 1] = -np.abs(d[:, 1]) - 0.5
    r["direction"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    r["length"] = 100.0
    return r


def ray_query_measurement(g, rays, reps: int = 10):
    """Closest-hit castRay of every ray against the world (cc_world_cast_rays_device on resident
    buffers: the query tree of the current poses, then one thread per ray), and the same through
    cc_world_cast_rays with host arrays (copies in and out inside the timed region)."""
    import ctypes as C
    import torch
    from crashcat_gb300 import _lib
    n = len(rays)
    d_rays = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    d_hits = torch.empty(n * _lib.RAY_HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    f = _lib.QueryFilter(0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF, _lib.CAST_RAY_TREAT_CONVEX_AS_SOLID)

    def call():
        _lib.check(g._lib.cc_world_cast_rays_device(g.handle, d_rays.data_ptr(), n, C.byref(f), d_hits.data_ptr()),
                   "cc_world_cast_rays_device")

    for _ in range(3):
        call()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        call()
    torch.cuda.synchronize()
    dev_s = (time.perf_counter() - t0) / reps
    hits = d_hits.cpu().numpy().view(_lib.RAY_HIT_DTYPE)
    g.cast_rays(rays[:1024])
    t0 = time.perf_counter()
    for _ in range(3):
        h2 = g.cast_rays(rays)
    e2e_s = (time.perf_counter() - t0) / 3
    return {"rays": n, "value": n / dev_s, "unit": "rays/s", "ms_per_batch": dev_s * 1e3,
            "e2e": {"value": n / e2e_s, "unit": "rays/s", "h2d_bytes_per_step": int(rays.nbytes),
                    "d2h_bytes_per_step": int(h2.nbytes)},
            "hit_fraction": float((hits["body"] >= 0).mean()), "terrain_hits": float((hits["body"] == 0).mean()),
            "device_equals_host_api": bool((h2["body"] == hits["body"]).all()), "_bodies": hits["body"].copy()}


def ray_profile(steps: int = 60, rays: int = 1 << 20, reps: int = 3):
    """The terrain workload's queries alone, for a profiler: the scene stepped `steps` times, then
    `reps` batches of `rays` closest-hit rays and of 65,536 shape casts on resident buffers.
    Prints one JSON line."""
    from crashcat_gb300 import scenes, world as W
    sc = scenes.mesh_drop(n=20000, n_cells=256, seed=2, amplitude=4.0, heights=(5.0, 40.0), fast_fraction=0.2)
    g = W.GpuWorld(W.standard_settings(velocity_iterations=8, position_iterations=2), sc.n + 16)
    for p in sc.hull_points:
        g.add_convex_hull(p)
    g.add_triangle_mesh(*sc.mesh)
    g.add_bodies(sc.bodies)
    if steps > 0:
        g.step(sc.dt, steps)
    q = ray_query_measurement(g, terrain_rays(rays, 0.4 * 256), reps=reps)
    q.pop("_bodies")
    c = shape_cast_measurement(g, terrain_casts(1 << 16, 0.4 * 256), reps=reps)
    c.pop("_bodies")
    print(json.dumps({"ray_queries": q, "shape_casts": c}))


def terrain_casts(n: int, half: float, seed: int = 4) -> np.ndarray:
    """Spheres, boxes and capsules (0.1-0.4 m) at random orientations, starting 20-50 m above the
    terrain and swept 40-60 m down with up to 5 m of drift: a cc_shape_cast array."""
    from crashcat_gb300 import _lib, scenes
    rng = np.random.default_rng(seed)
    c = np.zeros(n, _lib.SHAPE_CAST_DTYPE)
    kinds = rng.integers(0, 3, n)
    c["shape_type"] = kinds
    p = np.zeros((n, 4), np.float32)
    p[kinds == 0, 0] = rng.uniform(0.1, 0.4, (kinds == 0).sum())
    p[kinds == 1, 0:3] = rng.uniform(0.1, 0.4, ((kinds == 1).sum(), 3))
    p[kinds == 1, 3] = 0.05
    p[kinds == 2, 0:2] = rng.uniform(0.1, 0.3, ((kinds == 2).sum(), 2))
    c["shape_params"] = p
    c["position"] = np.stack([rng.uniform(-half, half, n), rng.uniform(20.0, 50.0, n), rng.uniform(-half, half, n)], 1)
    c["quaternion"] = scenes.random_quaternions(rng, n)
    c["displacement"] = np.stack([rng.uniform(-5, 5, n), rng.uniform(-60, -40, n), rng.uniform(-5, 5, n)], 1)
    return c


def shape_cast_measurement(g, casts, reps: int = 10):
    """Closest-hit castShape of every sweep (cc_world_cast_shapes_device on resident buffers,
    the query tree rebuilt first), and through cc_world_cast_shapes with host arrays."""
    import ctypes as C
    import torch
    from crashcat_gb300 import _lib
    n = len(casts)
    d_in = torch.from_numpy(casts.view(np.uint8).copy()).cuda()
    d_out = torch.empty(n * _lib.SHAPE_CAST_HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    f = _lib.QueryFilter(0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF, 0)

    def call():
        _lib.check(g._lib.cc_world_cast_shapes_device(g.handle, d_in.data_ptr(), n, C.byref(f), d_out.data_ptr()),
                   "cc_world_cast_shapes_device")

    for _ in range(3):
        call()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        call()
    torch.cuda.synchronize()
    dev_s = (time.perf_counter() - t0) / reps
    hits = d_out.cpu().numpy().view(_lib.SHAPE_CAST_HIT_DTYPE)
    t0 = time.perf_counter()
    for _ in range(3):
        h2 = g.cast_shapes(casts)
    e2e_s = (time.perf_counter() - t0) / 3
    return {"casts": n, "value": n / dev_s, "unit": "casts/s", "ms_per_batch": dev_s * 1e3,
            "e2e": {"value": n / e2e_s, "unit": "casts/s", "h2d_bytes_per_step": int(casts.nbytes),
                    "d2h_bytes_per_step": int(h2.nbytes)},
            "hit_fraction": float((hits["body"] >= 0).mean()), "terrain_hits": float((hits["body"] == 0).mean()),
            "device_equals_host_api": bool((h2["body"] == hits["body"]).all()), "_bodies": hits["body"].copy()}


def terrain_measurement(cpu_seconds: float = 8.0):
    """The mixed-shape terrain workload: 20,000 bodies (spheres, boxes, capsules and convex hulls
    of 16-32 points in the mixed pile's size ranges) dropped from 5-40 m over a 256 x 256-cell
    heightfield mesh (1 m cells, 4 m of relief, 131,072 triangles); 20 % of them start at
    20-60 m/s with LINEAR_CAST motion quality.  dt 1/60, 8/2 iterations, 300 steps from spawn on
    the GPU, timed per phase; the FP64 oracle on the same scene for a bounded number of steps
    from spawn on one host core."""
    from crashcat_gb300 import _lib, scenes, world as W
    from oracle import build as obuild, pyoracle
    sc = scenes.mesh_drop(n=20000, n_cells=256, seed=2, amplitude=4.0, heights=(5.0, 40.0), fast_fraction=0.2)
    ws = W.standard_settings(velocity_iterations=8, position_iterations=2)
    g = W.GpuWorld(ws, sc.n + 16)
    for p in sc.hull_points:
        g.add_convex_hull(p)
    g.add_triangle_mesh(*sc.mesh)
    g.add_bodies(sc.bodies)
    phases, total_ms, status = [], 0.0, 0
    for first, count in ((0, 100), (100, 100), (200, 100)):
        status |= g.step(sc.dt, count)
        st = g.stats()
        total_ms += st["last_call_ms"]
        phases.append({"steps": [first, first + count], "ms_per_step": st["last_call_ms"] / count,
                       "awake": st["num_awake"], "manifolds": st["num_manifolds"], "epa": st["num_epa"],
                       "mesh_pairs": st["num_mesh_pairs"], "mesh_hits": st["num_mesh_hits"],
                       "mesh_big": st["mesh_big"], "mesh_reduced": st["mesh_reduced"],
                       "ccd": st["num_ccd"], "ccd_hits": st["num_ccd_hits"], "islands": st["num_islands"]})
    rows, _ = g.get_state()
    hulls = [g.get_convex_hull(i) for i in range(len(sc.hull_points))]
    mesh = g.get_triangle_mesh(0)
    rays = terrain_rays(1 << 20, 0.4 * 256)
    queries = ray_query_measurement(g, rays)
    casts = terrain_casts(1 << 16, 0.4 * 256)
    sweeps = shape_cast_measurement(g, casts)
    del g
    obuild.build()
    o = pyoracle.OracleWorld(ws, sc.bodies, hulls, [mesh])
    # the oracle's closest-hit ray cast on a sample of the same rays, from the settled poses
    st = o.state()
    st[:, 0:13] = rows[:, 0:13]
    o.set_state(st)
    sample = np.stack([np.concatenate([r["origin"], r["direction"], [r["length"]]]) for r in rays[:2000]])
    t0 = time.perf_counter()
    ofr, obo, _ = o.cast_rays(sample)
    ray_cpu_s = time.perf_counter() - t0
    queries["cpu_baseline"] = {"value": len(sample) / ray_cpu_s, "unit": "rays/s", "cores": 1, "kind": "port",
                               "sample": "first 2,000 of the rays, brute force over the bodies"}
    queries["sample_same_body"] = float((queries.pop("_bodies")[:len(sample)] == obo).mean())
    # the oracle's castShape on a sample of the same sweeps
    cs = casts[:100]
    crow = np.concatenate([cs["shape_type"][:, None], cs["shape_params"], cs["position"], cs["quaternion"],
                           cs["displacement"]], 1).astype(np.float64)
    t0 = time.perf_counter()
    _, cbo = o.cast_shapes(crow)
    cast_cpu_s = time.perf_counter() - t0
    sweeps["cpu_baseline"] = {"value": len(cs) / cast_cpu_s, "unit": "casts/s", "cores": 1, "kind": "port",
                              "sample": "first 100 of the sweeps, every body cast"}
    sweeps["sample_same_body"] = float((sweeps.pop("_bodies")[:len(cs)] == cbo).mean())
    o = pyoracle.OracleWorld(ws, sc.bodies, hulls, [mesh])
    t0, k = time.perf_counter(), 0
    while time.perf_counter() - t0 < cpu_seconds and k < 100:
        o.step(sc.dt, 1)
        k += 1
    cpu_s = time.perf_counter() - t0
    # the settled pile: the oracle from the GPU's state after the 300 steps
    st = o.state()
    st[:, 0:13] = rows[:, 0:13]
    o.set_state(st)
    t0, kp = time.perf_counter(), 0
    while time.perf_counter() - t0 < cpu_seconds and kp < 100:
        o.step(sc.dt, 1)
        kp += 1
    pile_s = time.perf_counter() - t0
    del o
    err = terrain_error(ws)
    return {"workload": "terrain_mixed", "bodies": int(sc.n - 1), "triangles": int(len(mesh["triangles"])),
            "hulls": int(len(hulls)), "linear_cast_bodies": int((sc.bodies["motion_quality"] == 1).sum()),
            "steps": 300, "value": (sc.n - 1) * 300 / (total_ms * 1e-3), "unit": METRIC,
            "ms_per_step": total_ms / 300, "phases": phases, "status": int(status),
            "finite": bool(np.isfinite(rows).all()),
            "below_terrain": int((rows[1:, 1] < -2.5).sum()),
            "ray_queries": queries,
            "shape_casts": sweeps,
            "cpu_baseline": {"value": (sc.n - 1) * k / cpu_s, "unit": METRIC, "cores": 1, "kind": "port",
                             "sample": f"first {k} steps from spawn (falling phase)",
                             "gpu_same_phase_value": (sc.n - 1) / (phases[0]["ms_per_step"] * 1e-3)},
            "cpu_baseline_pile": {"value": (sc.n - 1) * kp / pile_s, "unit": METRIC, "cores": 1, "kind": "port",
                                  "sample": f"{kp} steps of the settled pile from the GPU's state after 300 steps",
                                  "gpu_same_phase_value": (sc.n - 1) / (phases[2]["ms_per_step"] * 1e-3)},
            "error": err}


def terrain_error(ws, n: int = 600, cells: int = 48, steps: int = 200) -> dict:
    """The terrain workload's error against the oracle on a scaled copy of its generator (n bodies
    of every shape over a cells x cells heightfield with the same relief, drop heights and 20 %
    LINEAR_CAST bodies): `steps` steps from spawn on the GPU and on the oracle, with the count of
    bodies that ended below the terrain on each side."""
    from crashcat_gb300 import scenes, world as W
    from oracle import pyoracle
    sc = scenes.mesh_drop(n=n, n_cells=cells, seed=2, amplitude=4.0, heights=(5.0, 40.0), fast_fraction=0.2)
    g = W.GpuWorld(ws, sc.n + 16)
    for p in sc.hull_points:
        g.add_convex_hull(p)
    g.add_triangle_mesh(*sc.mesh)
    g.add_bodies(sc.bodies)
    hulls = [g.get_convex_hull(i) for i in range(len(sc.hull_points))]
    mesh = g.get_triangle_mesh(0)
    rows0, _ = g.get_state()
    g.step(sc.dt, steps)
    rg, _ = g.get_state()
    dg = g.get_manifolds()[:, 6]
    del g
    o = pyoracle.OracleWorld(ws, sc.bodies, hulls, [mesh])
    o.step(sc.dt, steps)
    ro = o.state()
    m, inertia = mass_properties(sc.bodies, hulls)
    rep = error_report(sc.bodies, rows0, rg, dg, ro, o.manifolds()[:, 6], m, inertia, steps,
                       f"{n} bodies over a {cells} x {cells}-cell heightfield (the terrain generator scaled "
                       f"down), {steps} steps from spawn")
    rep["below_terrain"] = {"gpu": int((rg[1:, 1] < -2.5).sum()), "oracle": int((ro[1:, 1] < -2.5).sum()),
                            "bodies": n}
    return rep


def single_world_comparison(scene, ws_batched, settled_rows, dt, steps: int, sample_worlds: int = 48):
    """Steps a spread sample of the workload's worlds through the plain single-world path:
    one handle per world, each stepped once per step with cc_world_step (which blocks until
    the step ends), world after world.  Starts from the batched run's settled state."""
    import copy
    import torch
    from crashcat_gb300 import world as W
    worlds = split_worlds(scene)
    offs = np.cumsum([0] + [len(b) for b in worlds])
    pick = np.unique(np.linspace(0, len(worlds) - 1, sample_worlds).astype(int))
    handles, nb = [], 0
    for k in pick:
        b = worlds[k].copy()
        r = settled_rows[offs[k]:offs[k + 1]]
        b["position"], b["quaternion"] = r[:, 0:3], r[:, 3:7]
        b["linear_velocity"], b["angular_velocity"] = r[:, 7:10], r[:, 10:13]
        b["world"] = 0
        ws = copy.deepcopy(ws_batched)
        ws.num_worlds = 1
        g = W.GpuWorld(ws, len(b) + 8)
        g.add_bodies(b)
        g.step(dt, 2)  # first step (warm-start ratio 0) and the graph capture
        handles.append(g)
        nb += len(b)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        for g in handles:
            g.step(dt, 1)
    t = time.perf_counter() - t0
    del handles
    return {"value": nb * steps / t, "unit": METRIC, "worlds_sampled": int(len(pick)), "bodies_sampled": int(nb),
            "steps": steps, "ms_per_world_step": t * 1e3 / (steps * len(pick)),
            "api": "cc_world_step(handle, dt, 1) per world, one handle per world"}


def run_gpu(args, rank, world_size, local):
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world_size > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from crashcat_gb300 import _lib, build, scenes, world as W
    build.build()
    _lib.load()
    scene = scenes.batched_worlds(num_worlds=args.worlds, seed=args.seed + rank)
    ws = W.standard_settings(velocity_iterations=scene.velocity_iterations,
                             position_iterations=scene.position_iterations)
    ws.num_worlds = scene.num_worlds
    n = scene.n
    g = W.GpuWorld(ws, n + 64)
    g.add_bodies(scene.bodies)
    dt = scene.dt
    if args.settle:
        g.step(dt, args.settle)
    # launch shapes tuned on the settled state (the tuner leaves the state as it found it)
    tune = g.autotune(dt, 3) if args.tune else None
    for _ in range(args.warmup):
        g.step(dt, 1)
    stats_w = g.stats()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    barrier()
    with ClockSampler(local) as clk:
        status = g.step(dt, args.steps)
        barrier()
    dev_ms = g.stats()["last_call_ms"]
    t = torch.tensor([dev_ms], dtype=torch.float64, device="cuda")
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dev_ms = float(t.item())
    stats = g.stats()
    value = n * args.steps * world_size / (dev_ms * 1e-3)

    # end to end through the host-buffer entry point: pinned rows in and out every step
    rows, _ = g.get_state()
    settled_rows = rows.copy()
    h_in = torch.from_numpy(rows.copy()).pin_memory()
    h_out = torch.empty_like(h_in).pin_memory()
    e2e_steps = max(3, min(args.steps, 20))
    lib = _lib.load()
    import ctypes as C
    for _ in range(2):
        lib.cc_world_step_host(g.handle, C.c_float(dt), C.c_void_p(h_in.data_ptr()), C.c_void_p(h_out.data_ptr()))
        h_in, h_out = h_out, h_in
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        st = lib.cc_world_step_host(g.handle, C.c_float(dt), C.c_void_p(h_in.data_ptr()),
                                    C.c_void_p(h_out.data_ptr()))
        if st not in (0, _lib.CC_ERR_CAPACITY):
            _lib.check(st, "cc_world_step_host")
        h_in, h_out = h_out, h_in
    barrier()
    e2e_s = time.perf_counter() - t0
    te = torch.tensor([e2e_s], dtype=torch.float64, device="cuda")
    if dist is not None:
        dist.all_reduce(te, op=dist.ReduceOp.MAX)
    e2e_s = float(te.item())
    row_bytes = n * _lib.STATE_FLOATS * 4

    # stage profile (CUDA events between stages) for the roofline of the dominant stage
    prof = g.profile_steps(dt, max(3, min(args.steps, 10)))
    pst = g.stats()
    dom = max(prof, key=prof.get)
    peak, peak_kind = read_peaks()
    bytes_dom = algorithmic_bytes(dom, pst, n)
    achieved = bytes_dom / (prof[dom] * 1e-3) / 1e9 if prof[dom] > 0 else 0.0
    # DRAM bytes per launch of the dominant stage: the per-unit traffic of the committed ncu
    # capture (profiles/traffic_per_unit.json) times this step's units
    # the dominant stage's issue counters from the committed ncu capture: the stages are latency
    # and issue bound, which the HBM fraction alone does not show
    issue = None
    ipath = os.path.join(ROOT, "profiles", "issue_counters.json")
    if os.path.exists(ipath):
        try:
            issue = json.load(open(ipath)).get(dom)
        except Exception:
            issue = None
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic_per_unit.json")
    if os.path.exists(tpath):
        try:
            t = json.load(open(tpath)).get(dom)
            if t:
                traffic = t["bytes_per_unit"] * pst[t["unit"]]
        except Exception:
            traffic = None

    single = single_world_comparison(scene, ws, settled_rows, dt, steps=max(3, min(args.steps, 10)))
    cube_heap = cube_heap_measurement(peak, peak_kind) if args.cube_heap and rank == 0 else None
    error = batched_error(scene, ws, steps=args.settle or 360) if args.errors and rank == 0 else None
    adjoint = adjoint_measurement() if args.adjoint else None
    ragdolls = ragdoll_measurement() if args.ragdolls and rank == 0 else None
    terrain = terrain_measurement() if args.terrain and rank == 0 else None
    single["batched_over_single"] = value / world_size / single["value"]

    if rank == 0:
        cpu = cpu_baseline_single(scene, args.cpu_seconds, settled_rows)
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world_size, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "worlds": args.worlds, "bodies_per_gpu": n,
                       "dt": dt, "velocity_iterations": scene.velocity_iterations,
                       "position_iterations": scene.position_iterations, "seed": args.seed,
                       "settle_steps": args.settle,
                       "l2": "inputs larger than L2: resident body state and per-step buffers exceed 129 MB",
                       "parallelism": f"{world_size} x independent world batches"},
            "e2e": {"value": n * e2e_steps * world_size / e2e_s, "unit": METRIC,
                    "h2d_bytes_per_step": row_bytes, "d2h_bytes_per_step": row_bytes,
                    "api": "cc_world_step_host (pinned host rows in and out every step)"},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                         "algorithmic_bytes_per_launch": bytes_dom, "stage_ms": prof, "issue": issue},
            "cpu_baseline": cpu,
            "autotune": tune,
            "error": error,
            "vs_single_world": single,
            "cube_heap": cube_heap,
            "adjoint": adjoint,
            "ragdolls": ragdolls,
            "terrain": terrain,
            "clocks": clk.summary(),
            "gpu_launches": stats["gpu_launches_per_step"] * args.steps,
            "counters": {k: stats_w[k] for k in ("num_awake", "num_pairs", "num_manifolds", "num_contact_points",
                                                 "num_epa", "num_islands", "max_island_constraints")},
            "status": _lib.status_string(status),
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


def main():
    args = parse()
    rank, world_size, local = dist_env()
    if args.only == "cube_heap":
        peak, peak_kind = read_peaks()
        print(json.dumps(cube_heap_measurement(peak, peak_kind, oracle=args.cpu_seconds > 0)), flush=True)
        return
    if args.impl == "reference":
        run_reference(args, rank, world_size)
        return
    run_gpu(args, rank, world_size, local)


if __name__ == "__main__":
    main()
