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


def test_sample_range_split_in_one_process(product, cuda):
    """Samples [0, 4) in one accumulator and [4, 10) in another (first sample
    set to 4), their exact sums added on the device and resolved: the image
    and rays per pixel of one 10-sample launch bit for bit."""
    R, torch = product, cuda
    sc = R.rtow_scene(2, half_extent=4)
    w, h, seed = 72, 40, 13
    cam = R.rtow_camera(w, h)
    a, b = R.Accum(w, h), R.Accum(w, h)
    raw, rpp, fr = _frame(R, torch, w, h)
    sa = a.launch(sc, cam, R.launch_params(w, h, 4, depth=50, seed=seed), fr)
    b.set_first_sample(4)
    sb = b.launch(sc, cam, R.launch_params(w, h, 6, depth=50, seed=seed), fr)
    assert b.samples == 6
    n = w * h

    class _Dev:
        def __init__(self, ptr, typestr):
            self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 3}

    for pa, pb, ts in zip(a.device_sums(), b.device_sums(), ("<i8", "<i8", "<i8", "<i4")):
        ta = torch.as_tensor(_Dev(pa, ts), device="cuda")
        ta += torch.as_tensor(_Dev(pb, ts), device="cuda")
    a.set_range(0, 10, int(sa.rays) + int(sb.rays))
    a.resolve(fr)
    _check(raw, rpp, R.render(sc, cam, R.launch_params(w, h, 10, depth=50, seed=seed)), torch)
    # the state keeps the range; a resumed accumulator continues at sample 10
    c = R.Accum(w, h)
    c.load(a.save())
    assert c.samples == 10
    c.launch(sc, cam, R.launch_params(w, h, 2, depth=50, seed=seed), fr)
    _check(raw, rpp, R.render(sc, cam, R.launch_params(w, h, 12, depth=50, seed=seed)), torch)
    for x in (a, b, c):
        x.close()


def test_sample_range_api_errors(product, cuda):
    R, torch = product, cuda
    sc = R.rtow_scene(1, half_extent=2)
    w, h = 16, 12
    cam = R.rtow_camera(w, h)
    acc = R.Accum(w, h)
    raw, rpp, fr = _frame(R, torch, w, h)
    with pytest.raises(R.RTError) as e:   # nothing to resolve yet
        acc.resolve(fr)
    assert e.value.status == R.RT_ERR_INVALID_ARG
    acc.launch(sc, cam, R.launch_params(w, h, 2, depth=8, seed=1), fr)
    with pytest.raises(R.RTError) as e:   # the first sample of a filled accumulator is fixed
        acc.set_first_sample(5)
    assert e.value.status == R.RT_ERR_INVALID_ARG
    with pytest.raises(R.RTError):
        acc.set_range(0, 1 << 32, 0)
    acc.reset()   # clears the first sample too: the next launch renders samples [0, 3)
    acc.set_first_sample(7)
    acc.reset()
    acc.launch(sc, cam, R.launch_params(w, h, 3, depth=8, seed=1), fr)
    _check(raw, rpp, R.render(sc, cam, R.launch_params(w, h, 3, depth=8, seed=1)), torch)
    acc.close()
