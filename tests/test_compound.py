"""Compound shapes (src/shapes/compound.ts): convex children at poses in the compound's frame.

The reference's tests build compounds and check their bounds and mass; the oracle's restatement
is pinned by equivalences that follow from the definition:
  * two unit boxes side by side make the 2 x 1 x 1 box: the same mass, centre of mass and
    inertia (massProperties.rotate / translate of each child, compound.ts:177-230), so a free
    compound and the single box fly and spin alike (to 1e-9);
  * dropped on a floor they come to rest alike (the children's hits merge into one manifold of
    the same normal, pruned to the same four corners: within 1e-3 m / 1e-3 rad);
  * a table of five boxes settles upright on its four legs, whose hits join one manifold
    carrying the first leg's sub-shape id (subShape.pushIndex of the child index,
    compound.ts:512-516);
  * queries reach the child: a ray names the child it hits, a point inside a child is inside
    the compound, collide and cast queries report the child's sub-shape id.

GPU tolerances (FP32 device, FP64 oracle): bodies within 2e-3 m of the oracle's while they fall
and settle; queries as in test_query_collectors.py.
"""
import math

import numpy as np
import pytest

from crashcat_gb300 import _lib, scenes, world
from oracle import pyoracle

TWO_BOXES = [("box", (0.5, 0.5, 0.5), (-0.5, 0.0, 0.0)), ("box", (0.5, 0.5, 0.5), (0.5, 0.0, 0.0))]
TABLE = [("box", (1.0, 0.1, 0.6), (0.0, 0.9, 0.0))] + [
    ("box", (0.08, 0.4, 0.08), (sx * 0.85, 0.4, sz * 0.5)) for sx in (-1, 1) for sz in (-1, 1)]


def floor_and(n):
    b = scenes.blank_bodies(n + 1)
    scenes.set_box(b, 0, (20.0, 0.5, 20.0))
    b["motion_type"][0] = _lib.STATIC
    b["object_layer"][0] = scenes.LAYER_NOT_MOVING
    b["position"][0] = (0.0, -0.5, 0.0)
    return b


def oracle_with(bodies, compounds, hulls=()):
    return pyoracle.OracleWorld(world.standard_settings(), bodies, hulls, (), [scenes.compound_children(c)
                                                                              for c in compounds])


def gpu_with(bodies, compounds):
    g = world.GpuWorld(world.standard_settings(), len(bodies) + 8)
    for c in compounds:
        g.add_compound(scenes.compound_children(c))
    g.add_bodies(bodies)
    return g


def pair_scene(compound_first=True, floor=False, spin=True):
    """A compound of two unit boxes and, in a second body slot far away, the 2 x 1 x 1 box."""
    b = floor_and(2) if floor else scenes.blank_bodies(2)
    i0 = 1 if floor else 0
    scenes.set_compound(b, i0, 0)
    scenes.set_box(b, i0 + 1, (1.0, 0.5, 0.5))
    q = np.array([0.1, 0.3, -0.2, 0.9])
    q /= np.linalg.norm(q)
    for k, x in ((i0, -5.0), (i0 + 1, 5.0)):
        b["position"][k] = (x, 2.0, 0.0)
        b["quaternion"][k] = q
        if spin:
            b["linear_velocity"][k] = (0.3, 1.0, -0.2)
            b["angular_velocity"][k] = (0.7, -1.3, 2.1)
    if not floor:
        b["gravity_factor"] = 0.0
    b["linear_damping"] = 0.0
    b["angular_damping"] = 0.0
    return b, i0


# ---------------------------------------------------------------------------
# the oracle (CPU)
# ---------------------------------------------------------------------------
def test_oracle_compound_flies_like_the_single_box(oracle_lib):
    b, i0 = pair_scene()
    o = oracle_with(b, [TWO_BOXES])
    o.step(1.0 / 60.0, 120)
    st = o.state()
    np.testing.assert_allclose(st[i0, 1:13], st[i0 + 1, 1:13], atol=1e-9)
    np.testing.assert_allclose(st[i0, 0] + 10.0, st[i0 + 1, 0], atol=1e-9)


def test_oracle_compound_rests_like_the_single_box(oracle_lib):
    b, i0 = pair_scene(floor=True, spin=False)
    b["quaternion"][1:] = (0.0, 0.0, math.sin(0.15), math.cos(0.15))
    o = oracle_with(b, [TWO_BOXES])
    o.step(1.0 / 60.0, 180)
    st = o.state()
    np.testing.assert_allclose(st[i0, 1:7], st[i0 + 1, 1:7], atol=1e-3)
    assert abs(st[i0, 1] - 0.48) < 5e-3  # its 1 m height resting 2 cm deep (the penetration slop)


def table_scene():
    b = floor_and(1)
    scenes.set_compound(b, 1, 0)
    b["position"][1] = (0.0, 0.3, 0.0)
    b["quaternion"][1] = (0.02, 0.0, 0.03, math.sqrt(1 - 0.02 ** 2 - 0.03 ** 2))
    b["allow_sleeping"] = 0
    return b


def test_oracle_table_settles_on_its_legs(oracle_lib):
    o = oracle_with(table_scene(), [TABLE])
    o.step(1.0 / 60.0, 120)
    st = o.state()
    q = st[1, 3:7]
    assert abs(abs(q[3]) - 1.0) < 1e-3  # upright
    # the legs' feet (0 in the compound's frame) rest on the floor, within the 2 cm penetration slop
    assert -0.025 < st[1, 1] < 0.005, st[1, 1]
    # the four feet share the floor's normal: their hits join one manifold, which keeps the
    # sub-shape ids of its first hit (update.ts:414-449), the first leg (child 1)
    subs = [tuple(int(x) for x in s) for s in o.manifold_sub_shapes()]
    assert subs == [(0xFFFFFFFF, 0xFFFFFFF9)], subs


def test_oracle_compound_queries(oracle_lib):
    b = scenes.blank_bodies(1)
    scenes.set_compound(b, 0, 0)
    b["motion_type"][0] = _lib.STATIC
    b["object_layer"][0] = scenes.LAYER_NOT_MOVING
    o = oracle_with(b, [TWO_BOXES])
    one_bit = 0xFFFFFFFE  # two children: one sub-shape bit
    # a ray down onto the right box names child 1, onto the left child 0
    fr, bo, su = o.cast_rays(np.array([[0.5, 3.0, 0.0, 0, -1, 0, 10.0], [-0.5, 3.0, 0.0, 0, -1, 0, 10.0]]))
    assert list(bo) == [0, 0] and list(su) == [one_bit | 1, one_bit | 0]
    np.testing.assert_allclose(fr, [0.25, 0.25], atol=1e-4)
    co, bo, su = o.collide_points(np.array([[0.7, 0.2, 0.1], [-0.7, 0.2, 0.1], [0.0, 0.7, 0.0]]))
    assert list(co) == [1, 1, 0] and list(su[:2]) == [one_bit | 1, one_bit | 0]
    # a sphere cast down onto the seam: the first child met (ties to the first)
    out, bo, su = o.cast_shapes(np.array([[_lib.SHAPE_SPHERE, 0.25, 0, 0, 0, 0.6, 3.0, 0.0, 0, 0, 0, 1, 0, -4.0, 0]]),
                                with_subs=True)
    assert bo[0] == 0 and su[0] == one_bit | 1 and abs(out[0, 0] - 2.25 / 4.0) < 1e-3
    # a box overlapping both children: one hit per child
    out, bo, su, co = o.collide_shapes_all(np.array([[_lib.SHAPE_BOX, 0.3, 0.3, 0.3, 0.05, 0.0, 0.7, 0.0, 0, 0, 0, 1]]), 4)
    assert co[0] == 2 and sorted(su[0, :2]) == [one_bit | 0, one_bit | 1]
    np.testing.assert_allclose(out[0, :2, 0], [0.1, 0.1], atol=1e-3)


def test_oracle_refuses_a_cast_compound(oracle_lib):
    b = scenes.blank_bodies(1)
    scenes.set_compound(b, 0, 0)
    b["motion_quality"][0] = 1
    with pytest.raises(AssertionError):
        oracle_with(b, [TWO_BOXES])
