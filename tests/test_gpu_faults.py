"""GPU: host-side fault injection -- every device allocation of a scene's
construction, build and render made to fail in turn (rt_debug_fail_alloc).

Each failure must come back as RT_ERR_OUT_OF_MEMORY from the call that
allocated, leave no renderable half-built scene behind, and leave the library
usable: a fresh scene afterwards renders the reference image bit for bit.
No GPU fault is involved: the failing allocation is refused on the host
before cudaMalloc is called.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same(a, b):
    assert np.array_equal(a["rawRGB"].view(np.uint32), b["rawRGB"].view(np.uint32))
    assert np.array_equal(a["rpp"], b["rpp"])


@pytest.mark.parametrize("layout", ["sah", "instanced"])
def test_every_allocation_failure_is_clean(product, cuda, layout):
    R = product
    lay = R.RT_LAYOUT_SAH if layout == "sah" else R.RT_LAYOUT_INSTANCED
    w, h = 48, 32
    cam, params = R.rtow_camera(w, h), R.launch_params(w, h, 2, depth=8, seed=1)
    ref_scene = R.rtow_scene(2, layout=lay)
    ref = R.render(ref_scene, cam, params)
    ref_scene.close()
    failures = 0
    for n in range(1, 200):
        R.lib().rt_debug_fail_alloc(n)
        sc, stage = None, "create"
        try:
            sc = R.Scene()
            stage = "load"
            sc.load_rtow(R.RT_RECIPE_GLIBC, 1, 11, 2)
            stage = "build"
            sc.build(60, layout=lay)
            stage = "render"
            out = R.render(sc, cam, params)
        except R.RTError as e:
            assert e.status == R.RT_ERR_OUT_OF_MEMORY, (stage, str(e))
            assert b"injected" in R.lib().rt_last_error_string()
            failures += 1
            R.lib().rt_debug_fail_alloc(0)
            if stage in ("load", "build"):   # a scene whose construction failed is not renderable
                with pytest.raises(R.RTError) as e2:
                    R.render(sc, cam, params)
                assert e2.value.status == R.RT_ERR_NOT_BUILT
            elif stage == "render":          # the built scene is intact
                _same(R.render(sc, cam, params), ref)
            if sc is not None:
                sc.close()
            fresh = R.rtow_scene(2, layout=lay)
            _same(R.render(fresh, cam, params), ref)
            fresh.close()
            continue
        finally:
            R.lib().rt_debug_fail_alloc(0)
        # the n-th allocation was never reached: every earlier one has failed once
        _same(out, ref)
        sc.close()
        break
    else:
        pytest.fail("more than 199 device allocations for one small scene")
    assert failures >= 5


def test_failed_rebuild_leaves_no_stale_scene(product, cuda):
    R = product
    w, h = 40, 30
    cam, params = R.rtow_camera(w, h), R.launch_params(w, h, 1, depth=8, seed=2)
    sc = R.rtow_scene(2)
    ref = R.render(sc, cam, params)
    R.lib().rt_debug_fail_alloc(1)
    try:
        with pytest.raises(R.RTError) as e:
            sc.build(60, layout=R.RT_LAYOUT_INSTANCED)   # the two-level layout allocates its bottom level
        assert e.value.status == R.RT_ERR_OUT_OF_MEMORY
    finally:
        R.lib().rt_debug_fail_alloc(0)
    with pytest.raises(R.RTError) as e:
        R.render(sc, cam, params)
    assert e.value.status == R.RT_ERR_NOT_BUILT
    sc.build(60, layout=R.RT_LAYOUT_INSTANCED)
    _same(R.render(sc, cam, params), ref)   # layouts give identical images
    sc.close()


def test_copy_bandwidth_probe(product, cuda):
    """The L2 copy probe returns a positive rate and refuses bad sizes."""
    import ctypes
    R = product
    g = ctypes.c_double()
    R.check(R.lib().rt_measure_copy_bandwidth(1 << 20, 4, ctypes.byref(g), None))
    assert g.value > 0
    assert R.lib().rt_measure_copy_bandwidth(100, 4, ctypes.byref(g), None) == R.RT_ERR_INVALID_ARG
