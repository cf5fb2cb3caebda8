"""GPU: a destroyed scene's hierarchy arrays go to the next scene built.

rt_scene_destroy keeps the arrays of the scene it destroys for the next scene
the same host thread builds (no cudaFree and cudaMalloc between frames);
rt_scene_destroy(NULL) frees them.  A scene built on arrays handed on renders
exactly as one built on fresh arrays, and holds the larger arrays it took.
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
    fresh = R.rtow_scene(2, half_extent=4)        # fresh arrays
    ref = _render(R, fresh, 5)
    fresh_bytes = fresh.info().device_bytes
    fresh.close()
    R.free_spare_scene_arrays()

    big = R.rtow_scene(4)                          # a larger scene, then destroyed: its arrays are kept
    big_bytes = big.info().device_bytes
    _render(R, big, 6)
    big.close()
    small = R.rtow_scene(2, half_extent=4)         # built on the larger scene's arrays
    out = _render(R, small, 5)
    held = small.info().device_bytes   # the larger scene's arrays (its mesh buffers stayed with it)
    assert held >= 0.9 * big_bytes and big_bytes > 10 * fresh_bytes
    assert np.array_equal(out["rawRGB"].view(np.uint32), ref["rawRGB"].view(np.uint32))
    assert np.array_equal(out["rpp"], ref["rpp"])
    small.close()
    R.free_spare_scene_arrays()
    again = R.rtow_scene(2, half_extent=4)        # fresh again after the spare was freed
    assert again.info().device_bytes == fresh_bytes
    again.close()
