"""GPU: a destroyed scene's hierarchy arrays go to the next scene built.

rt_scene_destroy keeps the arrays of the scene it destroys for the next scene
the same host thread builds (no cudaFree and cudaMalloc between frames) when
they hold at most about twice its records; otherwise, and on
rt_scene_destroy(NULL), they are freed.  A scene built on arrays handed on
renders exactly as one built on fresh arrays.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _render(R, sc, seed):
    cam = R.rtow_camera(64, 40)
    return R.render(sc, cam, R.launch_params(64, 40, 3, depth=16, seed=seed))


def test_arrays_of_a_destroyed_scene_serve_the_next(product, cuda):
    R = product
    R.free_spare_scene_arrays()
    fresh = R.rtow_scene(4, half_extent=10)       # 400 small spheres, fresh arrays
    ref = _render(R, fresh, 5)
    fresh_bytes = fresh.info().device_bytes
    fresh.close()
    R.free_spare_scene_arrays()

    big = R.rtow_scene(4)                          # 484 small spheres; destroyed: its arrays are kept
    big_bytes = big.info().device_bytes
    big.close()
    again = R.rtow_scene(4, half_extent=10)       # built on the larger scene's arrays
    out = _render(R, again, 5)
    assert again.info().device_bytes == big_bytes > fresh_bytes
    assert np.array_equal(out["rawRGB"].view(np.uint32), ref["rawRGB"].view(np.uint32))
    assert np.array_equal(out["rpp"], ref["rpp"])
    again.close()

    tiny = R.rtow_scene(2, half_extent=4)         # far fewer records: the kept arrays are freed, not taken
    tiny_bytes = tiny.info().device_bytes
    tiny.close()
    R.free_spare_scene_arrays()
    tiny_fresh = R.rtow_scene(2, half_extent=4)
    assert tiny_fresh.info().device_bytes == tiny_bytes < fresh_bytes
    tiny_fresh.close()
    R.free_spare_scene_arrays()
