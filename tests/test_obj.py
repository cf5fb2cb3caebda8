"""OBJ input (the reference's Object, optx/object.cxx:23-106): the host parser.

CPU tests: hand-written files (groups, polygons split into fans, negative and
slashed indices, comments), error reporting, and the golden tessellations
written out and read back (with %.9g the float bits survive; with the %f the
reference's sphere writer uses, the result is the float nearest the printed
decimal).  The GPU test checks that an OBJ mesh renders exactly like the same
arrays added directly.
"""
import ctypes
import os

import numpy as np
import pytest

from _helpers import golden_sphere


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_groups_fans_and_index_forms(product, tmp_path):
    R = product
    p = _write(tmp_path, "a.obj", """# comment
mtllib none.mtl
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
vn 0 0 1
vt 0 0
o quad
usemtl x
s off
f 1 2 3 4
g tri
f -4/1/1 -2//1 -1
""")
    shapes = R.obj_parse(p)
    assert len(shapes) == 2
    (v0, i0), (v1, i1) = shapes
    assert np.array_equal(v0, np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32))
    assert np.array_equal(i0, np.array([[0, 1, 2], [0, 2, 3]], np.uint32))       # fan of the quad
    assert np.array_equal(v1, np.array([[0, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32))   # first-reference order
    assert np.array_equal(i1, np.array([[0, 1, 2]], np.uint32))


@pytest.mark.parametrize("text,msg", [
    ("v 0 0 0\nv 1 0 0\nf 1 2 9\n", "out of range"),
    ("v 0 0 0\nv 1 0 0\nf 1 2\n", "at least three"),
    ("v 0 0\n", "three coordinates"),
    ("v 0 0 x\n", "bad coordinate"),
    ("v 0 0 0\nf 1 1 0\n", "index 0"),
])
def test_errors_carry_file_and_line(product, tmp_path, text, msg):
    R = product
    p = _write(tmp_path, "bad.obj", text)
    with pytest.raises(R.RTError) as e:
        R.obj_parse(p)
    assert e.value.status == R.RT_ERR_INVALID_ARG
    assert msg in str(e.value) and "bad.obj:" in str(e.value)


def test_parse_checks_capacity(product, tmp_path):
    """A file that grew between the size query and the fill call does not
    overrun the caller's arrays: the fill call is refused and writes nothing."""
    R = product
    p = _write(tmp_path, "c.obj", "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nf 1 2 3 4\n")
    v = np.full((3, 3), -7.0, np.float32)   # room for 3 of 4 vertices
    i = np.zeros((2, 3), np.uint32)
    nv, ni = ctypes.c_uint(3), ctypes.c_uint(2)
    st = R.lib().rt_obj_parse(p.encode(), 0, ctypes.c_void_p(v.ctypes.data), ctypes.byref(nv),
                              ctypes.c_void_p(i.ctypes.data), ctypes.byref(ni), None)
    assert st == R.RT_ERR_INVALID_ARG and b"vces" in R.lib().rt_last_error_string()
    assert (v == -7.0).all()
    nv.value = 4
    st = R.lib().rt_obj_parse(p.encode(), 0, ctypes.c_void_p(v.ctypes.data), None, None, None, None)
    assert st == R.RT_ERR_INVALID_ARG   # an array without its capacity
    v4 = np.zeros((4, 3), np.float32)
    assert R.lib().rt_obj_parse(p.encode(), 0, ctypes.c_void_p(v4.ctypes.data), ctypes.byref(nv),
                                ctypes.c_void_p(i.ctypes.data), ctypes.byref(ni), None) == R.RT_OK
    assert nv.value == 4 and ni.value == 2 and v4[2].tolist() == [1, 1, 0]


def test_missing_file(product, tmp_path):
    R = product
    with pytest.raises(R.RTError) as e:
        R.obj_parse(str(tmp_path / "none.obj"))
    assert e.value.status == R.RT_ERR_INVALID_ARG


@pytest.mark.parametrize("n", [2, 4])
def test_golden_tessellation_round_trip(product, tmp_path, n):
    R = product
    v, i = golden_sphere(n)
    # exact: %.9g keeps every float32
    lines = ["o sphere"] + ["v %.9g %.9g %.9g" % tuple(x) for x in v.astype(np.float64)]
    lines += ["f %d %d %d" % tuple(t + 1) for t in i]
    p = _write(tmp_path, "s.obj", "\n".join(lines) + "\n")
    (pv, pi), = R.obj_parse(p)
    assert np.array_equal(pv.view(np.uint32), v.view(np.uint32))
    assert np.array_equal(pi, i)
    # the %f text of the reference's writer: the nearest float to each printed decimal
    lines = ["v %f %f %f" % tuple(x) for x in v.astype(np.float64)] + ["f %d %d %d" % tuple(t + 1) for t in i]
    p = _write(tmp_path, "f.obj", "\n".join(lines) + "\n")
    (fv, fi), = R.obj_parse(p)
    want = np.array([[np.float32(float("%f" % c)) for c in x] for x in v.astype(np.float64)], np.float32)
    assert np.array_equal(fv.view(np.uint32), want.view(np.uint32))
    assert np.array_equal(fi, i)


@pytest.mark.gpu
def test_obj_mesh_renders_like_direct_arrays(product, cuda, tmp_path):
    R = product
    v, i = golden_sphere(3)
    lines = ["v %.9g %.9g %.9g" % tuple(x) for x in v.astype(np.float64)] + ["f %d %d %d" % tuple(t + 1) for t in i]
    p = _write(tmp_path, "s.obj", "\n".join(lines) + "\n")
    scenes = []
    for via_obj in (True, False):
        sc = R.Scene()
        mid = sc.add_obj(p)[0] if via_obj else sc.add_mesh(v, i)
        for k, (c, r) in enumerate([((0, 0, 0), 1.0), ((2.2, 0.5, 0), 0.6), ((-2, 0, 1), 0.8)]):
            T = np.array([r, 0, 0, c[0], 0, r, 0, c[1], 0, 0, r, c[2]], np.float32)
            sc.add_thing(R.optics(k % 3, (0.7, 0.5, 0.3), 0.1, 1.5), mid, T)
        sc.add_analytic_sphere((0, -1001, 0), 1000.0, R.optics(0, (0.5, 0.5, 0.5)))
        sc.build()
        scenes.append(sc)
    cam = R.camera_set((0, 1.5, 7), (0, 0, 0), (0, 1, 0), 45, 1.5, 0.0, 7.0)
    params = R.launch_params(96, 64, 4, depth=16, seed=3)
    a, b = (R.render(sc, cam, params) for sc in scenes)
    assert np.array_equal(a["rawRGB"].view(np.uint32), b["rawRGB"].view(np.uint32))
    assert np.array_equal(a["rpp"], b["rpp"])
