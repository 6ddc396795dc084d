"""cc_penetration_static, the allocation-free penetration query, against the
world step's narrowphase (cc_world_step with dt = 0, then
cc_world_get_manifolds) on the same shape pairs, and against the FP64 oracle's
collideConvexVsConvex / collideSphereVsSphere of each pair (hit, normal, depth
and both contact points).

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
from oracle import pyoracle

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


def oracle_hits(sc, rows, order, max_sep):
    """The oracle's pair collide in FP64 on the same (FP32) poses: hit, pa, pb, axis, depth."""
    lib = pyoracle.load()
    b = sc.bodies.copy()
    b["position"] = rows[:, 0:3]
    b["quaternion"] = rows[:, 3:7]
    orows = pyoracle.rows_from_bodies(b)
    out = np.zeros((len(order), 13))
    for k, (a, bb) in enumerate(order):
        ra, rb = np.ascontiguousarray(orows[a]), np.ascontiguousarray(orows[bb])
        o = np.zeros(13)
        lib.orc_collide_pair(pyoracle.dptr(ra), pyoracle.dptr(rb), float(max_sep), pyoracle.dptr(o))
        out[k] = o
    return out


def check_against_oracle(lib, sc):
    """Every pair's hit flag, and for the pairs both hit: the unit normal, the depth and both
    contact points.  GJK contacts within 1e-4 (normal) and 1e-3 m (depth, points); EPA contacts
    within 1e-3 and 5e-3 m, since EPA seeded from an FP32 simplex may settle on another triangle of
    a flat face; at most 2 % of the EPA contacts may put their points elsewhere on such a face."""
    rows, pairs, _, max_sep = world_contacts(sc)
    order = [ordered(sc, int(a), int(b)) for a, b in pairs.tolist()]
    res = run_static(lib, queries_for(sc, rows, order, max_sep))
    orc = oracle_hits(sc, rows, order, max_sep)
    ohit = orc[:, 0] == 1
    ghit = res["hit"] == 1
    assert ohit.sum() > 20
    assert int((ohit != ghit).sum()) <= max(1, int(0.01 * len(order)))
    both = ohit & ghit
    n_o = orc[both, 7:10] / np.linalg.norm(orc[both, 7:10], axis=1, keepdims=True)
    epa = res["used_epa"][both] == 1
    dn = np.abs(res["normal"][both] - n_o).max(1)
    dd = np.abs(res["depth"][both] - orc[both, 10])
    dpa = np.abs(res["point_a"][both] - orc[both, 1:4]).max(1)
    dpb = np.abs(res["point_b"][both] - orc[both, 4:7]).max(1)
    g = ~epa
    assert (dn[g] < 1e-4).all() and (dd[g] < 1e-3).all()
    assert (dpa[g] < 1e-3).all() and (dpb[g] < 1e-3).all()
    assert epa.sum() > 0
    assert (dn[epa] < 1e-3).mean() >= 0.98 and (dd[epa] < 1e-3 + 1e-3 * np.abs(orc[both, 10][epa])).mean() >= 0.98
    assert ((dpa[epa] < 5e-3) & (dpb[epa] < 5e-3)).mean() >= 0.98


def test_static_query_matches_oracle(gpu_lib):
    check_against_oracle(gpu_lib, scenes.random_pairs_scene(n=300, seed=7, capsule_fraction=0.2))
    check_against_oracle(gpu_lib, scenes.random_pairs_scene(n=300, seed=9))


def test_static_query_marks_unsupported_shapes(gpu_lib):
    """A hull, a mesh or a value that names no shape comes back as CC_PENETRATION_UNSUPPORTED;
    the sphere-box query beside them is answered as usual."""
    q = np.zeros(4, dtype=_lib.PEN_QUERY_DTYPE)
    q["a"]["quaternion"] = (0, 0, 0, 1)
    q["b"]["quaternion"] = (0, 0, 0, 1)
    q["a"]["shape_type"] = _lib.SHAPE_SPHERE
    q["a"]["shape_params"] = (0.5, 0, 0, 0)
    q["b"]["shape_params"] = (0.5, 0.5, 0.5, 0.05)
    q["b"]["position"] = (0.0, 0.8, 0.0)
    q["b"]["shape_type"] = (_lib.SHAPE_BOX, _lib.SHAPE_CONVEX_HULL, _lib.SHAPE_TRIANGLE_MESH, 99)
    q["max_separation"] = 0.02
    res = run_static(gpu_lib, q)
    assert res["hit"][0] == 1 and abs(float(res["depth"][0]) - 0.2) < 1e-4
    assert (res["hit"][1:] == _lib.PENETRATION_UNSUPPORTED).all()


def test_static_query_matches_world_twice(gpu_lib):
    check_against_world(gpu_lib, scenes.random_pairs_scene(n=300, seed=7))
    check_against_world(gpu_lib, scenes.random_pairs_scene(n=300, seed=8))


def test_static_query_rejects_oversize(gpu_lib):
    one = C.c_void_p(256)  # never dereferenced: the size check comes first
    st = gpu_lib.cc_penetration_static(one, _lib.STATIC_MAX_QUERIES + 1, one, C.c_float(1e-4), C.c_float(1e-4), None)
    assert st == _lib.CC_ERR_CAPACITY
