"""cc_penetration_static, the allocation-free penetration query, against the
world step's narrowphase (cc_world_step with dt = 0, then
cc_world_get_manifolds) on the same shape pairs.

Both run the same FP32 GJK and FP64 EPA source, inlined into different
kernels (so the compiler may contract multiply-adds differently).  The
tolerances are the parity suite's: every manifold of the world has a hit in
the query with normal and depth within 1e-4 (GJK path) or within 1e-3 and
1e-3 relative (EPA path, which stops at a 1e-4 relative tolerance), and at
most 1 % of the broadphase pairs differ in whether they hit.  Two
calls in a row, on different scenes, check that the static EPA queue starts
from zero on each call.  This file is collected last so that it also runs
after the rest of the GPU suite in the same process.
"""
import ctypes as C

import numpy as np
import pytest

from crashcat_gb300 import _lib, scenes, world

pytestmark = pytest.mark.gpu


def world_contacts(sc):
    ws = world.standard_settings(velocity_iterations=sc.velocity_iterations,
                                 position_iterations=sc.position_iterations)
    g = world.GpuWorld(ws, sc.n + 16)
    g.add_bodies(sc.bodies)
    g.step(0.0, 1)  # dt = 0: broadphase and narrowphase only (update.ts:101)
    rows, _ = g.get_state()
    return rows, g.get_pairs(), g.get_manifolds(), ws.speculative_contact_distance


def ordered(sc, a, b):
    """The world's A/B order of a pair: lower motion type first, then lower id (update.ts:74)."""
    ma, mb = int(sc.bodies["motion_type"][a]), int(sc.bodies["motion_type"][b])
    if ma > mb or (ma == mb and b < a):
        return b, a
    return a, b


def queries_for(sc, rows, pairs, max_sep):
    q = np.zeros(len(pairs), dtype=_lib.PEN_QUERY_DTYPE)
    for k, (a, b) in enumerate(pairs):
        for side, body in (("a", a), ("b", b)):
            q[side]["shape_type"][k] = sc.bodies["shape_type"][body]
            q[side]["shape_params"][k] = sc.bodies["shape_params"][body]
            q[side]["position"][k] = rows[body, 0:3]
            q[side]["quaternion"][k] = rows[body, 3:7]
    q["max_separation"] = max_sep
    return q


def run_static(lib, q):
    import torch
    qd = torch.from_numpy(q.view(np.uint8).copy()).cuda()
    rd = torch.zeros(len(q) * _lib.PEN_RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    st = lib.cc_penetration_static(C.c_void_p(qd.data_ptr()), len(q), C.c_void_p(rd.data_ptr()),
                                   C.c_float(1e-4), C.c_float(1e-4), C.c_void_p(stream.cuda_stream))
    _lib.check(st, "cc_penetration_static")
    stream.synchronize()
    return rd.cpu().numpy().view(_lib.PEN_RESULT_DTYPE)


def check_against_world(lib, sc):
    rows, pairs, mans, max_sep = world_contacts(sc)
    order = [ordered(sc, int(a), int(b)) for a, b in pairs.tolist()]
    res = run_static(lib, queries_for(sc, rows, order, max_sep))
    by_pair = {p: r for p, r in zip(order, res)}
    assert len(mans) > 20
    assert int(res["used_epa"].sum()) > 0  # the scene exercises the EPA pass
    bad = 0
    for m in mans:
        r = by_pair[(int(m[0]), int(m[1]))]
        tol, rel = (1e-3, 1e-3) if r["used_epa"] else (1e-4, 1e-4)
        ok = (r["hit"] == 1 and np.abs(r["normal"] - m[3:6]).max() < tol
              and abs(float(r["depth"]) - float(m[6])) < tol + rel * abs(float(m[6])))
        bad += not ok
    assert bad <= 0.01 * len(mans)
    assert abs(int(res["hit"].sum()) - len(mans)) <= 0.01 * len(pairs)


def test_static_query_matches_world_twice(gpu_lib):
    check_against_world(gpu_lib, scenes.random_pairs_scene(n=300, seed=7))
    check_against_world(gpu_lib, scenes.random_pairs_scene(n=300, seed=8))


def test_static_query_rejects_oversize(gpu_lib):
    one = C.c_void_p(256)  # never dereferenced: the size check comes first
    st = gpu_lib.cc_penetration_static(one, _lib.STATIC_MAX_QUERIES + 1, one, C.c_float(1e-4), C.c_float(1e-4), None)
    assert st == _lib.CC_ERR_CAPACITY
