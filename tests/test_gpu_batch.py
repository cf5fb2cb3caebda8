"""GPU: many scenes in one launch, and the graph-driven wave loop.

A batch builds all scene hierarchies in one segmented pass and renders all
scenes in one wavefront; every scene's image must equal, bit for bit, the
image the single-scene launch renders for it (and the oracle's).
"""
import ctypes

import numpy as np
import pytest

from _helpers import dptr, oracle_camera

pytestmark = pytest.mark.gpu


def _frame(torch, w, h, guides=False):
    n = w * h
    raw = torch.zeros(n * 3, dtype=torch.float32, device="cuda")
    rpp = torch.zeros(n, dtype=torch.int32, device="cuda")
    nrm = torch.zeros(n * 3, dtype=torch.float32, device="cuda") if guides else None
    alb = torch.zeros(n * 3, dtype=torch.float32, device="cuda") if guides else None
    return raw, rpp, nrm, alb


def _frame_struct(R, bufs):
    raw, rpp, nrm, alb = bufs
    return R.Frame(dptr(raw), dptr(rpp), dptr(nrm) if nrm is not None else None,
                   dptr(alb) if alb is not None else None)


SPECS = [  # (level or None, half_extent, w, h, spp, depth, seed, recipe rng, recipe seed)
    (2, 4, 64, 36, 3, 16, 11, 1, 5),
    (None, 11, 48, 48, 2, 50, 12, 0, 1),
    (1, 2, 32, 18, 7, 8, 13, 1, 9),
    (3, 3, 40, 40, 1, 16, 14, 1, 21),
    (0, 6, 56, 32, 4, 4, 15, 0, 3),
]


def _scene(R, spec):
    level, H, w, h, spp, depth, seed, rk, rs = spec
    sc = R.Scene()
    sc.load_rtow(rk, rs, H, -1 if level is None else level)
    return sc


@pytest.mark.parametrize("graph", ["1", "0"])
def test_batch_equals_single_scene_launches(product, oracle, cuda, monkeypatch, graph):
    R, O, torch = product, oracle, cuda
    monkeypatch.setenv("RTX_GRAPH", graph)
    batch = R.Batch()
    scenes, outs = [], []
    for spec in SPECS:
        level, H, w, h, spp, depth, seed, rk, rs = spec
        sc = _scene(R, spec)
        scenes.append(sc)
        bufs = _frame(torch, w, h, guides=True)
        outs.append(bufs)
        batch.add(sc, R.rtow_camera(w, h),
                  R.launch_params(w, h, spp, depth=depth, seed=seed, flags=R.RT_FLAG_GUIDES),
                  _frame_struct(R, bufs))
    batch.build()
    st = batch.launch()
    torch.cuda.synchronize()
    total = 0
    for spec, sc, bufs in zip(SPECS, scenes, outs):
        level, H, w, h, spp, depth, seed, rk, rs = spec
        sc.build()
        one = R.render(sc, R.rtow_camera(w, h),
                       R.launch_params(w, h, spp, depth=depth, seed=seed, flags=R.RT_FLAG_GUIDES), guides=True)
        raw = bufs[0].cpu().numpy().reshape(-1, 3)
        rpp = bufs[1].cpu().numpy().view(np.uint32)
        assert np.array_equal(raw.view(np.uint32), one["rawRGB"].view(np.uint32)), spec
        assert np.array_equal(rpp, one["rpp"]), spec
        assert np.array_equal(bufs[2].cpu().numpy().reshape(-1, 3), one["normals"])
        assert np.array_equal(bufs[3].cpu().numpy().reshape(-1, 3), one["albedos"])
        total += int(rpp.sum())
    assert int(st.rays) == total
    # one scene of the batch against the oracle as well
    level, H, w, h, spp, depth, seed, rk, rs = SPECS[0]
    wd, _ = O.rtow_world(level, rk, rs, H)
    ref = wd.render(oracle_camera(O, R.rtow_camera(w, h)), w, h, spp, depth, seed, guides=False)
    assert np.array_equal(outs[0][0].cpu().numpy().reshape(-1, 3).view(np.uint32), ref["rawRGB"].view(np.uint32))


def test_batch_with_empty_and_single_primitive_scenes(product, cuda):
    R, torch = product, cuda
    empty = R.Scene()
    single = R.Scene()
    single.add_analytic_sphere((0, 0, 0), 1.0, R.optics(R.RT_OPTICS_DIFFUSE, (0.5, 0.5, 0.5)))
    full = _scene(R, SPECS[2])
    batch = R.Batch()
    bufs = []
    cams = [R.rtow_camera(16, 8), R.camera_set((0, 0, 5), (0, 0, 0), (0, 1, 0), 40, 1.0, 0.0, 5.0),
            R.rtow_camera(24, 24)]
    sizes = [(16, 8), (16, 16), (24, 24)]
    for sc, cam, (w, h) in zip((empty, single, full), cams, sizes):
        b = _frame(torch, w, h)
        bufs.append(b)
        batch.add(sc, cam, R.launch_params(w, h, 2, depth=16, seed=3), _frame_struct(R, b))
    batch.build()
    batch.launch()
    torch.cuda.synchronize()
    assert (bufs[0][1].cpu().numpy() == 2).all()           # empty scene: every primary ray misses
    assert bufs[1][1].cpu().numpy().max() > 2              # the sphere is hit
    full.build()
    one = R.render(full, cams[2], R.launch_params(24, 24, 2, depth=16, seed=3))
    assert np.array_equal(bufs[2][0].cpu().numpy().reshape(-1, 3), one["rawRGB"])


def test_graph_and_host_wave_loops_agree(product, cuda, monkeypatch):
    R = product
    sc = R.rtow_scene(2, half_extent=5)
    cam = R.rtow_camera(80, 45)
    params = R.launch_params(80, 45, 6, depth=50, seed=77)
    monkeypatch.setenv("RTX_WAVE", "4096")
    monkeypatch.setenv("RTX_GRAPH", "1")
    a = R.render(sc, cam, params)
    monkeypatch.setenv("RTX_GRAPH", "0")
    b = R.render(sc, cam, params)
    assert np.array_equal(a["rawRGB"], b["rawRGB"]) and np.array_equal(a["rpp"], b["rpp"])
    assert a["stats"].waves == b["stats"].waves > 10


def test_batch_errors(product, cuda):
    R = product
    b = R.Batch()
    with pytest.raises(R.RTError) as e:
        b.launch()
    assert e.value.status == R.RT_ERR_NOT_BUILT
    with pytest.raises(R.RTError) as e:
        b.build()
    assert e.value.status == R.RT_ERR_INVALID_ARG
