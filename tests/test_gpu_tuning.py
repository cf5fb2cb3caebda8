"""GPU: the launch shape (rt_tuning) changes no image, and the autotuner runs.

Pixel sums are exact integers and hits do not depend on the traversal order,
so every wave size, shading block, persistent grid and refill rule must give
the same colours and rays per pixel bit for bit, in the graph-driven and the
host-driven wave loop, for one scene, an instanced scene and a batch.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [
    {"wave_log2": 16, "shade_block": 128, "extend_blocks_per_sm": 1, "refill_below": 1, "steps_per_check": 1},
    {"wave_log2": 16, "shade_block": 512, "extend_blocks_per_sm": 2, "refill_below": 31, "steps_per_check": 64},
    {"wave_log2": 17, "shade_block": 1024, "extend_blocks_per_sm": 32, "refill_below": 20, "steps_per_check": 5},
    {"wave_log2": 17, "shade_block": 256, "extend_blocks_per_sm": 3, "refill_below": 8, "steps_per_check": 32},
]


@pytest.fixture(autouse=True)
def _reset(product):
    product.tuning_set(None)
    yield
    product.tuning_set(None)


def _same(a, b):
    assert np.array_equal(a["rawRGB"].view(np.uint32), b["rawRGB"].view(np.uint32))
    assert np.array_equal(a["rpp"], b["rpp"])


@pytest.mark.parametrize("layout", ["sah", "instanced"])
@pytest.mark.parametrize("graph", ["1", "0"])
def test_launch_shape_changes_no_image(product, cuda, monkeypatch, layout, graph):
    R = product
    monkeypatch.setenv("RTX_GRAPH", graph)
    lay = R.RT_LAYOUT_SAH if layout == "sah" else R.RT_LAYOUT_INSTANCED
    sc = R.rtow_scene(2, layout=lay)
    w, h = 160, 120
    cam, params = R.rtow_camera(w, h), R.launch_params(w, h, 8, depth=50, seed=5)
    ref = R.render(sc, cam, params)
    assert ref["stats"].waves > 3
    for shape in SHAPES:
        R.tuning_set(shape)
        out = R.render(sc, cam, params)
        _same(out, ref)
        assert out["stats"].wave_capacity == 1 << shape["wave_log2"]
        assert out["stats"].waves > ref["stats"].waves


def test_launch_shape_changes_no_batch_image(product, cuda):
    R, torch = product, cuda
    scenes, bufs, batch = [], [], R.Batch()
    specs = [(40, 30, 3, 2), (64, 48, 5, 3), (33, 17, 2, None)]
    for k, (w, h, spp, level) in enumerate(specs):
        sc = R.Scene()
        sc.load_rtow(R.RT_RECIPE_COUNTER, 50 + k, 3, -1 if level is None else level)
        scenes.append(sc)
        raw = torch.zeros(w * h * 3, dtype=torch.float32, device="cuda")
        rpp = torch.zeros(w * h, dtype=torch.int32, device="cuda")
        bufs.append((raw, rpp))
        fr = R.Frame(ctypes.c_void_p(raw.data_ptr()), ctypes.c_void_p(rpp.data_ptr()), None, None)
        batch.add(sc, R.rtow_camera(w, h), R.launch_params(w, h, spp, depth=16, seed=9 + k), fr)
    batch.build(60)
    batch.launch()
    torch.cuda.synchronize()
    ref = [(a.clone(), b.clone()) for a, b in bufs]
    for shape in SHAPES:
        R.tuning_set(shape)
        for a, b in bufs:
            a.zero_()
            b.zero_()
        batch.launch()
        torch.cuda.synchronize()
        for (a, b), (ra, rb) in zip(bufs, ref):
            assert torch.equal(a.view(torch.int32), ra.view(torch.int32)) and torch.equal(b, rb)
    batch.close()


def test_autotuner_on_a_small_scene(product, cuda, tmp_path):
    R = product
    from rtxplay_gb300 import tune
    sc = R.rtow_scene(2)
    w, h = 128, 96
    cam, params = R.rtow_camera(w, h), R.launch_params(w, h, 4, depth=16, seed=3)
    ref = R.render(sc, cam, params)
    cache = tune.TuneCache(str(tmp_path / "t.json"))
    probe = tune.render_timer(sc, cam, params, repeats=1)
    space = {"shade_block": (256, 128), "refill_below": (12, 8), "wave_log2": (22, 16)}
    t, src = tune.tuned("small", probe, cache=cache, device="gpu", space=space)
    probe.close()
    assert src == "tuned"
    assert t["shade_block"] in (256, 128) and t["refill_below"] in (12, 8) and t["wave_log2"] in (22, 16)
    assert R.tuning_get()["shade_block"] == t["shade_block"]   # applied
    _same(R.render(sc, cam, params), ref)
    assert tune.TuneCache(str(tmp_path / "t.json")).get("gpu", "small")["tuning"] == t
