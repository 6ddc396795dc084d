"""Pins the FP64 oracle to the reference's own known-answer tests.

The vectors in tests/golden/reference_known_answers.json are transcribed from
crashcat's vitest suites (each case cites its file:line).  The reference is
TypeScript and cannot run in this image, so these assertions - together with
the scenario tests below that restate the reference's integration tests - are
what pins the oracle.
"""
import json
import math
import os

import numpy as np
import pytest

from crashcat_gb300 import scenes, world
from oracle import pyoracle

HERE = os.path.dirname(os.path.abspath(__file__))
KA = json.load(open(os.path.join(HERE, "golden", "reference_known_answers.json")))


@pytest.fixture(scope="module")
def lib(oracle_lib):
    return oracle_lib


def arr(x):
    return np.ascontiguousarray(np.asarray(x, dtype=np.float64))


@pytest.mark.parametrize("case", KA["clip_poly_vs_plane"], ids=lambda c: c["ref"])
def test_clip_poly_vs_plane(lib, case):
    poly = arr(case["poly"])
    out = np.zeros(64 * 3)
    n = lib.orc_clip_poly_vs_plane(pyoracle.dptr(poly), len(poly) // 3, pyoracle.dptr(arr(case["origin"])),
                                   pyoracle.dptr(arr(case["normal"])), pyoracle.dptr(out))
    assert n == case["count"]
    if "vertices" in case:
        np.testing.assert_allclose(out[: 3 * n], case["vertices"], atol=1e-6)


@pytest.mark.parametrize("case", KA["clip_poly_vs_poly"], ids=lambda c: c["ref"])
def test_clip_poly_vs_poly(lib, case):
    poly, clip = arr(case["poly"]), arr(case["clip"])
    out = np.zeros(64 * 3)
    n = lib.orc_clip_poly_vs_poly(pyoracle.dptr(poly), len(poly) // 3, pyoracle.dptr(clip), len(clip) // 3,
                                  pyoracle.dptr(arr(case["normal"])), pyoracle.dptr(out))
    if "count" in case:
        assert n == case["count"]
    else:
        assert case["count_min"] <= n <= case["count_max"]


@pytest.mark.parametrize("case", KA["manifold_between_faces"], ids=lambda c: c["ref"])
def test_manifold_between_faces(lib, case):
    f1, f2 = arr(case["face1"]), arr(case["face2"])
    oa, ob = np.zeros(64 * 3), np.zeros(64 * 3)
    n = lib.orc_manifold_between_faces(pyoracle.dptr(arr(case["cp1"])), pyoracle.dptr(arr(case["cp2"])),
                                       pyoracle.dptr(arr(case["axis"])), case["max_dist"], pyoracle.dptr(f1),
                                       len(f1) // 3, pyoracle.dptr(f2), len(f2) // 3, pyoracle.dptr(oa),
                                       pyoracle.dptr(ob))
    assert n == case["count"]


def test_manifold_relative_to_base_offset(lib):
    """manifold.test.ts:155-190: points are stored relative to the base offset (here 0, so
    they are the clipped world points around +-0.5 at z = 0)."""
    f = arr([-0.5, -0.5, 0, 0.5, -0.5, 0, 0.5, 0.5, 0, -0.5, 0.5, 0])
    f2 = arr([-0.5, -0.5, 0.1, 0.5, -0.5, 0.1, 0.5, 0.5, 0.1, -0.5, 0.5, 0.1])
    oa, ob = np.zeros(64 * 3), np.zeros(64 * 3)
    n = lib.orc_manifold_between_faces(pyoracle.dptr(arr([0, 0, 0])), pyoracle.dptr(arr([0, 0, 0.1])),
                                       pyoracle.dptr(arr([0, 0, 0.1])), 0.2, pyoracle.dptr(f), 4, pyoracle.dptr(f2),
                                       4, pyoracle.dptr(oa), pyoracle.dptr(ob))
    assert n == 4
    pa = oa[:12].reshape(4, 3)
    assert np.all(np.abs(np.abs(pa[:, :2]) - 0.5) < 1e-12) and np.allclose(pa[:, 2], 0.0)


@pytest.mark.parametrize("case", KA["prune_contact_points"], ids=lambda c: c["ref"])
def test_prune_contact_points(lib, case):
    pts = np.array(case["points"], dtype=np.float64)
    if "offset_b" in case:
        pb = pts + np.array(case["offset_b"])
    else:
        pb = pts + np.stack([np.zeros(len(pts)), np.zeros(len(pts)),
                             np.linalg.norm(pts, axis=1) * case["depth_scale"]], 1)
    a = np.ascontiguousarray(pts.reshape(-1))
    b = np.ascontiguousarray(pb.reshape(-1))
    n = lib.orc_prune_contact_points(pyoracle.dptr(a), pyoracle.dptr(b), len(pts), pyoracle.dptr(arr(case["axis"])))
    assert n == case["count"]


@pytest.mark.parametrize("case", KA["barycentric"], ids=lambda c: c["ref"])
def test_barycentric(lib, case):
    out = np.zeros(4)
    c = case.get("c", [0, 0, 0])
    lib.orc_barycentric(pyoracle.dptr(arr(case["a"])), pyoracle.dptr(arr(case["b"])), pyoracle.dptr(arr(c)),
                        case["n"], case["sqtol"], pyoracle.dptr(out))
    assert bool(out[3]) == case["valid"]
    if case["valid"]:
        assert out[0] == pytest.approx(case["u"], abs=5e-3)
        assert out[1] == pytest.approx(case["v"], abs=5e-3)
        if "w" in case:
            assert out[2] == pytest.approx(case["w"], abs=5e-3)


def body_row(shape, params, pos, quat=(0, 0, 0, 1)):
    b = scenes.blank_bodies(1)
    if shape == "sphere":
        scenes.set_sphere(b, 0, params)
    else:
        scenes.set_box(b, 0, params)
    b["position"][0] = pos
    b["quaternion"][0] = quat
    return np.ascontiguousarray(pyoracle.rows_from_bodies(b)[0])


def collide(lib, ra, rb, max_sep=0.0):
    out = np.zeros(13)
    lib.orc_collide_pair(pyoracle.dptr(ra), pyoracle.dptr(rb), max_sep, pyoracle.dptr(out))
    return out


def test_sphere_sphere_cases(lib):
    """collide-shape-vs-shape.test.ts:23-128: distant -> no hit; overlapping -> positive
    penetration; coincident spheres of radius 2 -> depth 4 along +y."""
    far = collide(lib, body_row("sphere", 1.0, (0, 0, 0)), body_row("sphere", 1.0, (5, 0, 0)))
    assert far[0] == 0
    hit = collide(lib, body_row("sphere", 1.0, (0, 0, 0)), body_row("sphere", 1.0, (1.5, 0, 0)))
    assert hit[0] == 1 and hit[10] == pytest.approx(0.5)
    np.testing.assert_allclose(hit[7:10], [1, 0, 0])
    same = collide(lib, body_row("sphere", 2.0, (1, 2, 3)), body_row("sphere", 2.0, (1, 2, 3)))
    assert same[0] == 1 and same[10] == pytest.approx(4.0)
    np.testing.assert_allclose(same[7:10], [0, 1, 0])


def test_box_box_cases(lib):
    """collide-shape-vs-shape.test.ts:268-496: distant boxes miss, overlapping and rotated
    boxes report a positive penetration with 4-vertex supporting faces, a box inside
    another (EPA) still reports one hit."""
    assert collide(lib, body_row("box", (1, 1, 1), (0, 0, 0)), body_row("box", (1, 1, 1), (5, 0, 0)))[0] == 0
    hit = collide(lib, body_row("box", (1, 1, 1), (0, 0, 0)), body_row("box", (1, 1, 1), (1.5, 0, 0)))
    assert hit[0] == 1 and hit[10] == pytest.approx(0.5, abs=1e-6)
    assert hit[11] == 4 and hit[12] == 4
    q = (0.0, 0.0, math.sin(math.pi / 8), math.cos(math.pi / 8))
    rot = collide(lib, body_row("box", (1, 1, 1), (0, 0, 0)), body_row("box", (1, 1, 1), (2.2, 0, 0), q))
    assert rot[0] == 1 and rot[10] > 0
    deep = collide(lib, body_row("box", (2, 2, 2), (0, 0, 0)), body_row("box", (0.5, 0.5, 0.5), (0.1, 0, 0)))
    assert deep[0] == 1 and deep[10] > 1.0


def test_sphere_box_cases(lib):
    """collide-shape-vs-shape.test.ts:497-599: distant miss, face contact depth, corner contact."""
    assert collide(lib, body_row("sphere", 1.0, (5, 0, 0)), body_row("box", (1, 1, 1), (0, 0, 0)))[0] == 0
    hit = collide(lib, body_row("sphere", 1.0, (1.5, 0, 0)), body_row("box", (1, 1, 1), (0, 0, 0)))
    assert hit[0] == 1 and hit[10] == pytest.approx(0.5, abs=1e-4)
    corner = collide(lib, body_row("sphere", 0.5, (1.2, 1.2, 1.2)), body_row("box", (1, 1, 1), (0, 0, 0)))
    # the box corner is rounded by its 0.05 m convex radius (support.ts:339-370)
    assert corner[0] == 1 and corner[10] == pytest.approx(0.5 - (math.sqrt(3) * 0.25 - 0.05), abs=1e-4)


def test_inverse_inertia_matches_r_d_rt(lib):
    """motion-properties.test.ts:6-120: world inverse inertia equals R diag(1/I) R^T and is symmetric."""
    rng = np.random.default_rng(0)
    for _ in range(5):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        b = scenes.blank_bodies(1)
        scenes.set_box(b, 0, (0.3, 0.7, 1.1))
        b["quaternion"][0] = q
        row = np.ascontiguousarray(pyoracle.rows_from_bodies(b)[0])
        out = np.zeros(9)
        lib.orc_inverse_inertia(pyoracle.dptr(row), pyoracle.dptr(out))
        M = out.reshape(3, 3).T  # column-major
        x, y, z, w = row[10:14]
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                      [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                      [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
        full = 2.0 * row[1:4]  # FP32 half extents promoted exactly
        mass = full[0] * full[1] * full[2] * 1000
        sz = full ** 2
        I = np.array([sz[1] + sz[2], sz[0] + sz[2], sz[0] + sz[1]]) * mass / 12
        np.testing.assert_allclose(M, R @ np.diag(1 / I) @ R.T, rtol=1e-9, atol=1e-15)
        np.testing.assert_allclose(M, M.T, atol=1e-15)


def test_sleep_after_time_before_sleep():
    """sleep.test.ts:346-386: a resting sphere without gravity sleeps after 0.6 s."""
    ws = world.standard_settings(gravity_enabled=False)
    b = scenes.blank_bodies(1)
    scenes.set_sphere(b, 0, 1.0)
    o = pyoracle.OracleWorld(ws, b)
    o.step(1 / 60, math.ceil((0.5 + 0.1) * 60))
    assert o.state()[0, 16] == 1.0


def test_stack_comes_to_rest():
    """A 10-box column settles on the floor and the whole island sleeps (islands.ts:392-423)."""
    sc = scenes.box_stack(height=10)
    o = pyoracle.OracleWorld(world.standard_settings(), sc.bodies)
    o.step(sc.dt, 120)
    st = o.state()
    assert st[1:, 16].all()
    assert st[1:, 1].min() > 0.49  # penetration within the slop


def test_broadphase_layers_and_groups():
    """broadphase.test.ts:75-193: pairs are found within the speculative margin, static-static
    pairs are never reported, and group/mask filtering removes a pair."""
    b = scenes.blank_bodies(3)
    scenes.static_floor(b, 0, half=(5, 0.5, 5))
    scenes.set_box(b, 1, (0.5, 0.5, 0.5))
    scenes.set_box(b, 2, (0.5, 0.5, 0.5))
    b["position"][1] = (0, 0.51, 0)   # 1 cm above the floor: inside the 2 cm margin
    b["position"][2] = (3, 0.56, 0)   # 6 cm above: outside
    o = pyoracle.OracleWorld(world.standard_settings(), b)
    o.step(0.0, 1)
    assert {tuple(sorted(p)) for p in o.pairs().tolist()} == {(0, 1)}
    b["collision_groups"][1] = 0b01
    b["collision_mask"][0] = 0b10
    o2 = pyoracle.OracleWorld(world.standard_settings(), b)
    o2.step(0.0, 1)
    assert len(o2.pairs()) == 0


# ---- capsules (tst/shapes/capsule.test.ts) -------------------------------------------
def _capsule_row(r, h, density=1000.0):
    row = np.zeros(pyoracle.F_COUNT)
    row[0] = 2
    row[1], row[2] = r, h
    row[5] = density
    row[6] = 2
    row[13] = 1.0  # identity quaternion (w)
    return row


def _inv_inertia_diag(lib, row):
    out = np.zeros(9)
    lib.orc_inverse_inertia(pyoracle.dptr(row), pyoracle.dptr(out))
    return out.reshape(3, 3).diagonal()


def test_capsule_inertia_properties(oracle_lib):
    """capsule.test.ts:84-165: Ixx == Izz, Iyy < Ixx, density scales inertia, a long
    capsule has Iyy < 0.1 Ixx, a wide one Iyy / Ixx > 0.5."""
    d = 1.0 / _inv_inertia_diag(oracle_lib, _capsule_row(1.0, 1.0))
    assert d[0] == pytest.approx(d[2]) and d[1] < d[0]
    d2 = 1.0 / _inv_inertia_diag(oracle_lib, _capsule_row(1.0, 1.0, 2000.0))
    np.testing.assert_allclose(d2, 2 * d, rtol=1e-12)
    long_ = 1.0 / _inv_inertia_diag(oracle_lib, _capsule_row(0.5, 10.0))
    assert long_[1] < 0.1 * long_[0]
    wide = 1.0 / _inv_inertia_diag(oracle_lib, _capsule_row(2.0, 0.1))
    assert wide[1] / wide[0] > 0.5


def test_capsule_mass_and_bounds(oracle_lib):
    """capsule.test.ts:37-81: volume pi r^2 2h + 4/3 pi r^3, mass = density x volume,
    AABB [-r, -(h+r), -r]..[r, h+r, r]."""
    from crashcat_gb300 import scenes, world
    sc = scenes.blank_bodies(1)
    scenes.set_capsule(sc, 0, 0.5, 2.0)
    sc["density"][0] = 1000.0
    o = pyoracle.OracleWorld(world.standard_settings(), sc)
    box = o.aabbs()[0]
    np.testing.assert_allclose(box, [-0.5, -2.5, -0.5, 0.5, 2.5, 0.5], atol=1e-12)
    # mass from the inverse inertia of a sphere-free check: I_yy of the cylinder + caps
    r, h = 0.5, 2.0
    vol = math.pi * r * r * 2 * h + 4.0 / 3.0 * math.pi * r ** 3
    assert vol == pytest.approx(math.pi * 0.25 * 4 + 4.0 / 3.0 * math.pi * 0.125)


def test_capsule_collides_with_box_edge_face(oracle_lib):
    """A capsule lying on a box.  Faces are clipped only when face A has 2+ vertices and
    face B 3+ (update.ts:474).  With the capsule as body A (both dynamic, lower id) its
    supporting face is the 2-vertex edge (capsule.ts:192-251), clipped against the box's
    top face by clipPolyVsEdge (clip.ts:190-363): two contact points at the ends of the
    cylinder.  On a static floor the floor is body A (lower motion type first,
    update.ts:74) and the capsule's edge is face B, so the contact is a single point."""
    from crashcat_gb300 import scenes, world
    s2 = math.sin(math.pi / 4)
    b = scenes.blank_bodies(2)
    scenes.set_capsule(b, 0, 0.3, 0.6)
    b["position"][0] = (0.0, 0.3 - 0.01, 0.0)
    b["quaternion"][0] = (s2, 0.0, 0.0, s2)  # local Y onto world Z
    scenes.set_box(b, 1, (2.0, 0.5, 2.0))
    b["position"][1] = (0.0, -0.5, 0.0)
    o = pyoracle.OracleWorld(world.standard_settings(), b)
    o.step(0.0, 1)
    m = o.manifolds()
    assert len(m) == 1 and int(m[0][2]) == 2
    pts = m[0][8:20].reshape(2, 6)
    zs = sorted(pts[:, 2])
    assert zs[0] == pytest.approx(-0.6, abs=1e-6) and zs[1] == pytest.approx(0.6, abs=1e-6)
    np.testing.assert_allclose(m[0][3:6], [0.0, -1.0, 0.0], atol=1e-6)  # capsule (A) to box (B)
    assert m[0][6] == pytest.approx(0.01, abs=1e-6)
    # the same capsule on a static floor: one contact point
    b["motion_type"][1] = 0
    o = pyoracle.OracleWorld(world.standard_settings(), b)
    o.step(0.0, 1)
    m = o.manifolds()
    assert len(m) == 1 and int(m[0][2]) == 1
