"""The C-ABI library builds, loads without a GPU, and exports every entry point
declared in include/crashcat_gpu.h; the host-side mirror validates its input."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from crashcat_gb300 import _lib, build, scenes, world

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    hdr = open(os.path.join(ROOT, "include", "crashcat_gpu.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(cc_[a-z_0-9]+)\s*\(", hdr)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(lib, n), n
        assert n in _lib.EXPORTS, n


def test_status_strings(lib):
    for s in range(7):
        assert lib.cc_status_string(s)
    assert b"overflowed" in lib.cc_status_string(_lib.CC_ERR_CAPACITY)


def test_default_settings_match_reference(lib):
    s = _lib.Settings()
    assert lib.cc_world_settings_default(C.byref(s)) == 0
    ws = world.create_world_settings()
    assert s.speculative_contact_distance == ws.speculative_contact_distance == 0.02
    assert s.velocity_iterations == 10 and s.position_iterations == 2
    assert s.gravity[1] == -9.81 and s.penetration_slop == 0.02 and s.baumgarte_factor == 0.2


def test_invalid_arguments_are_rejected(lib):
    assert lib.cc_world_create(None, None) == _lib.CC_ERR_INVALID
    s = _lib.Settings()
    lib.cc_world_settings_default(C.byref(s))
    s.num_object_layers = 0
    h = C.c_void_p()
    assert lib.cc_world_create(C.byref(s), C.byref(h)) == _lib.CC_ERR_INVALID
    assert lib.cc_world_step(None, C.c_float(0.01), 1) == _lib.CC_ERR_INVALID


def test_record_layouts_match_c(tmp_path):
    """The numpy mirrors of the C records have the C compiler's sizes and field offsets
    (a probe compiled against include/crashcat_gpu.h prints them)."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    recs = {"cc_body_desc": _lib.BODY_DTYPE, "cc_hinge_desc": _lib.HINGE_DTYPE,
            "cc_swing_twist_desc": _lib.SWING_TWIST_DTYPE, "cc_tape_body": _lib.TAPE_BODY_DTYPE,
            "cc_tape_contact": _lib.TAPE_CONTACT_DTYPE, "cc_penetration_query": _lib.PEN_QUERY_DTYPE,
            "cc_penetration_result": _lib.PEN_RESULT_DTYPE, "cc_ray": _lib.RAY_DTYPE,
            "cc_shape_cast": _lib.SHAPE_CAST_DTYPE, "cc_shape_cast_hit": _lib.SHAPE_CAST_HIT_DTYPE,
            "cc_point_desc": _lib.POINT_JOINT_DTYPE, "cc_distance_desc": _lib.DISTANCE_JOINT_DTYPE,
            "cc_fixed_desc": _lib.FIXED_JOINT_DTYPE, "cc_cone_desc": _lib.CONE_JOINT_DTYPE,
            "cc_slider_desc": _lib.SLIDER_JOINT_DTYPE, "cc_six_dof_desc": _lib.SIX_DOF_JOINT_DTYPE,
            "cc_compound_child": _lib.COMPOUND_CHILD_DTYPE, "cc_collide_shape": _lib.COLLIDE_SHAPE_DTYPE,
            "cc_collide_shape_hit": _lib.COLLIDE_SHAPE_HIT_DTYPE}
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{ROOT}/include/crashcat_gpu.h"',
             'int main(void) {']
    for name, dt in recs.items():
        lines.append(f'printf("{name} size %zu\\n", sizeof({name}));')
        for f in dt.names:
            lines.append(f'printf("{name} {f} %zu\\n", offsetof({name}, {f}));')
    lines += ['return 0;', '}']
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-std=c11", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for name, dt in recs.items():
        assert got[(name, "size")] == dt.itemsize, name
        for f in dt.names:
            assert got[(name, f)] == dt.fields[f][1], (name, f)


def test_layer_tables_follow_reference():
    s = world.standard_settings()
    L = s.layers
    # MOVING collides with MOVING and NOT_MOVING; NOT_MOVING only with MOVING (tst/helpers.ts)
    assert L.object_pairs == [0b11, 0b01]
    assert L.broadphase_pairs == [0b11, 0b01]
    assert L.object_vs_broadphase == [0b11, 0b01 | 0b10]


def test_scene_generators_are_seeded():
    a = scenes.cube_heap(seed=1).bodies
    b = scenes.cube_heap(seed=1).bodies
    assert a.tobytes() == b.tobytes()
    c = scenes.batched_worlds(num_worlds=8, seed=4)
    assert c.num_worlds == 8 and (np.diff(c.bodies["world"]) >= 0).all()


def test_static_query_checks_arguments_before_any_cuda_call(lib):
    one = C.c_void_p(256)  # never dereferenced: every check below returns before a launch
    tol = (C.c_float(1e-4), C.c_float(1e-4))
    assert lib.cc_penetration_static(one, _lib.STATIC_MAX_QUERIES + 1, one, *tol, None) == _lib.CC_ERR_CAPACITY
    assert lib.cc_penetration_static(one, -1, one, *tol, None) == _lib.CC_ERR_INVALID
    assert lib.cc_penetration_static(None, 8, one, *tol, None) == _lib.CC_ERR_INVALID
    assert lib.cc_penetration_static(one, 8, one, C.c_float(0.0), tol[1], None) == _lib.CC_ERR_INVALID
    assert lib.cc_penetration_static(None, 0, None, *tol, None) == _lib.CC_OK
    assert _lib.PEN_QUERY_DTYPE.itemsize == 100 and _lib.PEN_RESULT_DTYPE.itemsize == 48


def test_rollout_grad_checks_arguments_before_any_cuda_call(lib):
    t = (C.c_float * 3)()
    assert lib.cc_world_rollout_grad(None, C.c_float(0.01), 10, 5, t, None, None, None, None) == _lib.CC_ERR_INVALID


def test_contact_events_check_arguments(lib):
    cnt = C.c_int32(0)
    assert lib.cc_world_get_contact_events(None, None, 0, C.byref(cnt)) == _lib.CC_ERR_INVALID
