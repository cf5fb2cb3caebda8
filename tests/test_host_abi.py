"""CPU: the C ABI library loads, exports every declared symbol, and its
host-side logic (scene recipe, camera, argument checks) matches the oracle."""
import ctypes
import os
import re

import numpy as np
import pytest

from _helpers import golden_scene

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "rt_api.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^(?:rt_status|const char\*)\s+(rt_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(product):
    names = declared_functions()
    assert len(names) >= 30
    lib = product.lib()
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_the_header(product):
    names = set(declared_functions()) - {"rt_last_error_string", "rt_version"}
    assert names <= set(product.SIGNATURES), sorted(names - set(product.SIGNATURES))


def test_version(product):
    assert "sm_103a" in product.version()


@pytest.mark.parametrize("seed", [1, 7])
def test_recipe_glibc_reproduces_reference_scene(product, seed):
    g = golden_scene(seed)
    s = product.rtow_spheres(product.RT_RECIPE_GLIBC, seed, 11)
    assert len(s["radii"]) == len(g)
    assert np.array_equal(s["types"], g[:, 0].astype(np.int32))
    assert np.array_equal(s["centers"], g[:, 1:4].astype(np.float32))
    assert np.array_equal(s["albedos"], g[:, 5:8].astype(np.float32))
    assert np.array_equal(s["fuzz"], g[:, 8].astype(np.float32))
    assert np.array_equal(s["index"], g[:, 9].astype(np.float32))


@pytest.mark.parametrize("kind,seed,H", [(0, 42, 11), (1, 4711, 11), (1, 3, 2), (0, 1, 0)])
def test_recipe_matches_oracle(product, oracle, kind, seed, H):
    a = product.rtow_spheres(kind, seed, H)
    b = oracle.scene_rtow(kind, seed, H)
    for k in ("centers", "radii", "types", "albedos", "fuzz", "index"):
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("w,h", [(1200, 800), (384, 216), (1280, 720), (7, 13)])
def test_camera_set_matches_oracle(product, oracle, w, h):
    a = product.rtow_camera(w, h)
    b = oracle.rtow_camera(w, h)
    for k in ("u", "v", "w", "hvec", "wvec", "dvec"):
        fa = getattr(a, k)
        assert np.array_equal(np.array([fa.x, fa.y, fa.z], np.float32), np.array(getattr(b, k)[:], np.float32)), k


def test_host_errors_are_status_codes(product):
    R = product
    lib = R.lib()
    f = R.f3((0, 0, 0))
    assert lib.rt_camera_set(None, f, f, f, 20.0, 1.0, 0.1, 10.0) == R.RT_ERR_INVALID_ARG
    assert b"NULL" in lib.rt_last_error_string()
    n = ctypes.c_uint()
    assert lib.rt_rtow_spheres(7, 1, 11, 0, None, None, None, ctypes.byref(n)) == R.RT_ERR_INVALID_ARG
    assert lib.rt_rtow_spheres(0, 1, 11, 0, None, None, None, ctypes.byref(n)) == R.RT_OK
    assert lib.rt_last_error_string() == b""
    assert lib.rt_rtow_spheres(0, 1, 11, 3, ctypes.c_void_p(1), None, None, ctypes.byref(n)) == R.RT_ERR_INVALID_ARG
    assert lib.rt_scene_destroy(None) == R.RT_OK
    assert lib.rt_scene_build(None, 60, None) == R.RT_ERR_INVALID_ARG


def test_scene_handle_logic_without_device(product):
    """Ids and transforms are host state: checked before any device work."""
    R = product
    sc = R.Scene()
    st, _ = sc.get_transform(0)
    assert st == R.RT_ERR_INVALID_ARG
    tid = ctypes.c_uint()
    o = R.optics(R.RT_OPTICS_REFLECT, (0.7, 0.6, 0.5), 0.0)
    assert R.lib().rt_scene_add_thing(sc.h, ctypes.byref(o), 0, None, ctypes.byref(tid)) == R.RT_ERR_INVALID_ARG
    assert R.lib().rt_scene_add_analytic_sphere(sc.h, R.f3((0, 0, 0)), -1.0, ctypes.byref(o),
                                                ctypes.byref(tid)) == R.RT_ERR_INVALID_ARG
    bad = R.optics(9)
    assert R.lib().rt_scene_add_analytic_sphere(sc.h, R.f3((0, 0, 0)), 1.0, ctypes.byref(bad),
                                                ctypes.byref(tid)) == R.RT_ERR_INVALID_ARG
    assert sc.add_analytic_sphere((1, 2, 3), 0.5, o) == 0
    st, T = sc.get_transform(0)
    assert st == R.RT_OK and T.tolist() == [0.5, 0, 0, 1, 0, 0.5, 0, 2, 0, 0, 0.5, 3]
    T[3] = 9.0
    assert sc.set_transform(0, T) == R.RT_OK
    assert sc.get_transform(0)[1][3] == 9.0
    sc.close()


def test_add_things_checks_everything_first(product):
    """rt_scene_add_things refuses the whole call for one bad entry (no device needed)."""
    R = product
    sc = R.Scene()
    assert sc.add_analytic_sphere((0, 0, 0), 1.0, R.optics(R.RT_OPTICS_DIFFUSE, (0.5, 0.5, 0.5))) == 0
    T = np.tile(np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], np.float32), (3, 1))
    opts = [R.optics(R.RT_OPTICS_DIFFUSE, (0.1, 0.2, 0.3))] * 3
    with pytest.raises(R.RTError) as e:   # no mesh 0 in this scene
        sc.add_things(opts, [0, 0, 0], T)
    assert e.value.status == R.RT_ERR_INVALID_ARG and b"mesh" in R.lib().rt_last_error_string()
    bad = T.copy()
    bad[1, 0] = np.nan
    with pytest.raises(R.RTError):
        sc.add_things(opts, [0, 0, 0], bad)
    assert sc.add_things([], [], np.zeros((0, 12), np.float32)) == []
    assert sc.add_analytic_sphere((1, 0, 0), 1.0, R.optics(R.RT_OPTICS_DIFFUSE, (0.5, 0.5, 0.5))) == 1
    first = ctypes.c_uint()
    assert R.lib().rt_scene_add_things(sc.h, 2, None, None, None, ctypes.byref(first)) == R.RT_ERR_INVALID_ARG
    sc.close()


def test_accum_host_errors(product):
    """Accumulator calls check their arguments before any device work."""
    R = product
    lib = R.lib()
    h = ctypes.c_void_p()
    assert lib.rt_accum_create(None, 4, 4) == R.RT_ERR_INVALID_ARG
    assert lib.rt_accum_create(ctypes.byref(h), 0, 4) == R.RT_ERR_INVALID_ARG
    assert lib.rt_accum_create(ctypes.byref(h), 1 << 16, 1 << 15) == R.RT_ERR_INVALID_ARG
    n = ctypes.c_ulonglong()
    assert lib.rt_accum_samples(None, ctypes.byref(n)) == R.RT_ERR_INVALID_ARG
    sz = ctypes.c_size_t()
    assert lib.rt_accum_state_size(None, ctypes.byref(sz)) == R.RT_ERR_INVALID_ARG
    assert lib.rt_accum_destroy(None) == R.RT_OK
    assert lib.rt_launch_accum(None, None, None, None, None, None, None) == R.RT_ERR_INVALID_ARG


def test_fail_alloc_hook_without_device(product):
    """The injection hook is host state; a zero switches it off."""
    R = product
    assert R.lib().rt_debug_fail_alloc(3) == R.RT_OK
    assert R.lib().rt_debug_fail_alloc(0) == R.RT_OK
