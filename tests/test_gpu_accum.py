"""GPU: progressive rendering with checkpoint and resume (rt_accum).

Sample k of a pixel draws from its own counter-RNG stream and the pixel sums
are exact integers, so chunks of samples rendered into an accumulator, with a
checkpoint to host bytes and a resume into a fresh accumulator in between,
must give the image and rays per pixel of one launch bit for bit.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _frame(R, torch, w, h):
    raw = torch.zeros(w * h * 3, dtype=torch.float32, device="cuda")
    rpp = torch.zeros(w * h, dtype=torch.int32, device="cuda")
    return raw, rpp, R.Frame(ctypes.c_void_p(raw.data_ptr()), ctypes.c_void_p(rpp.data_ptr()), None, None)


def _check(raw, rpp, ref, torch):
    torch.cuda.synchronize()
    assert np.array_equal(raw.cpu().numpy().view(np.uint32), ref["rawRGB"].reshape(-1).view(np.uint32))
    assert np.array_equal(rpp.cpu().numpy().astype(np.int64), ref["rpp"].astype(np.int64))


@pytest.mark.parametrize("level", [None, 2])
def test_chunks_equal_one_launch(product, cuda, level):
    R, torch = product, cuda
    sc = R.rtow_scene(level)
    w, h, seed = 80, 60, 21
    cam = R.rtow_camera(w, h)
    acc = R.Accum(w, h)
    raw, rpp, fr = _frame(R, torch, w, h)
    rays, done = 0, 0
    for spp in (3, 5, 2):
        st = acc.launch(sc, cam, R.launch_params(w, h, spp, depth=50, seed=seed), fr)
        rays += st.rays
        done += spp
        assert acc.samples == done
        _check(raw, rpp, R.render(sc, cam, R.launch_params(w, h, done, depth=50, seed=seed)), torch)
    assert rays == int(R.render(sc, cam, R.launch_params(w, h, 10, depth=50, seed=seed))["rpp"].sum())
    acc.reset()
    assert acc.samples == 0
    acc.launch(sc, cam, R.launch_params(w, h, 4, depth=50, seed=seed), fr)
    _check(raw, rpp, R.render(sc, cam, R.launch_params(w, h, 4, depth=50, seed=seed)), torch)
    acc.close()


def test_checkpoint_and_resume(product, cuda):
    R, torch = product, cuda
    sc = R.rtow_scene(2, layout=R.RT_LAYOUT_INSTANCED)
    w, h, seed = 64, 48, 5
    cam = R.rtow_camera(w, h)
    raw, rpp, fr = _frame(R, torch, w, h)
    a = R.Accum(w, h)
    a.launch(sc, cam, R.launch_params(w, h, 4, depth=16, seed=seed), fr)
    state = a.save()
    a.close()
    b = R.Accum(w, h)   # a new process would start here
    b.load(state)
    assert b.samples == 4
    st = b.launch(sc, cam, R.launch_params(w, h, 7, depth=16, seed=seed), fr)
    assert b.samples == 11
    ref4 = R.render(sc, cam, R.launch_params(w, h, 4, depth=16, seed=seed))
    ref11 = R.render(sc, cam, R.launch_params(w, h, 11, depth=16, seed=seed))
    assert st.rays == int(ref11["rpp"].sum()) - int(ref4["rpp"].sum())
    _check(raw, rpp, R.render(sc, cam, R.launch_params(w, h, 11, depth=16, seed=seed)), torch)
    # wrong size, damaged state, guides and a mismatched image are refused
    c = R.Accum(w + 1, h)
    with pytest.raises(R.RTError):
        c.load(state)
    bad = bytearray(state)
    bad[0] ^= 0xFF
    with pytest.raises(R.RTError):
        b.load(bytes(bad))
    with pytest.raises(R.RTError):
        b.launch(sc, cam, R.launch_params(w, h, 1, depth=16, seed=seed, flags=R.RT_FLAG_GUIDES), fr)
    with pytest.raises(R.RTError):
        c.launch(sc, cam, R.launch_params(w, h, 1, depth=16, seed=seed), fr)
    assert b.samples == 11   # refused calls change nothing
    c.close()
    b.close()
