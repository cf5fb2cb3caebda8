"""GPU: device memory balance (the reference's check-cudamem target,
optx/Makefile:270-272, balances cudaMalloc against cudaFree by grepping the
sources; here the balance is measured).

Scenes, launchers, batches and accumulators own their device buffers and free
them when destroyed; the per-thread render workspace and build scratch grow
once and are then reused.  After one warm-up cycle, further cycles of
create / build / render / destroy must leave the device's free memory where
it was.
"""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def _cycle(R, torch):
    # images large enough that every per-cycle buffer (launcher images, the
    # accumulator's 5.5 MB of sums, the scenes' hierarchies) spans several MiB
    w, h = 512, 384
    cam = R.rtow_camera(w, h)
    sc = R.rtow_scene(3)
    R.render(sc, cam, R.launch_params(w, h, 1, depth=4, seed=1))
    inst = R.rtow_scene(3, layout=R.RT_LAYOUT_INSTANCED)
    R.render(inst, cam, R.launch_params(w, h, 1, depth=4, seed=1))
    raw = torch.zeros(w * h * 3, dtype=torch.float32, device="cuda")
    rpp = torch.zeros(w * h, dtype=torch.int32, device="cuda")
    fr = R.Frame(ctypes.c_void_p(raw.data_ptr()), ctypes.c_void_p(rpp.data_ptr()), None, None)
    acc = R.Accum(w, h)
    acc.launch(sc, cam, R.launch_params(w, h, 1, depth=4, seed=1), fr)
    acc.close()
    raw2 = torch.zeros(w * h * 3, dtype=torch.float32, device="cuda")
    fr2 = R.Frame(ctypes.c_void_p(raw2.data_ptr()), None, None, None)
    b = R.Batch()
    b.add(sc, cam, R.launch_params(w, h, 1, depth=4, seed=2), fr)
    b.add(inst, cam, R.launch_params(w, h, 1, depth=4, seed=3), fr2)
    b.build(60)
    b.launch()
    b.close()
    inst.close()
    sc.close()
    del raw, rpp, raw2
    torch.cuda.synchronize()


def test_device_memory_returns_to_baseline(product, cuda):
    R, torch = product, cuda
    _cycle(R, torch)   # warm-up: workspace, scratch and the caching allocator settle
    torch.cuda.empty_cache()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(4):
        _cycle(R, torch)
    torch.cuda.empty_cache()
    free1, _ = torch.cuda.mem_get_info()
    assert abs(free0 - free1) <= 2 << 20, (free0, free1)   # within 2 MiB (driver bookkeeping)
