"""GPU: rtow's pixel mapping (RT_FLAG_RTOW_PIXELS) bit for bit against the oracle,
and the product's render against the reference's own renderer, statistically.

The statistical check is the oracle's (tests/test_oracle_rtow_stats.py): the
final scene as analytic spheres at 1280x720, 10 spp, depth 50, gamma-2 8-bit,
16x16 block means against those of the unmodified rtow.cxx, within 6 noise
standard deviations plus 1 % per block and a converged relative RMSE of at
most 1 %.
"""
import ctypes

import numpy as np
import pytest

from _helpers import device_first_hit, oracle_camera, rtow_pair
from test_oracle_rtow_stats import DEPTH, FIXTURE, H, SPP, W, check_against_rtow

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("level", [None, 2])
def test_rtow_pixels_bit_exact_vs_oracle(product, oracle, cuda, level):
    R, O = product, oracle
    sc, wd = rtow_pair(R, O, level)
    w, h, spp = 64, 36, 3
    cam = R.rtow_camera(w, h)
    params = R.launch_params(w, h, spp, depth=50, seed=77, flags=R.RT_FLAG_RTOW_PIXELS)
    out = R.render(sc, cam, params)
    ref = wd.render(oracle_camera(O, cam, rtow_pixels=True), w, h, spp, 50, 77, guides=False)
    assert np.array_equal(out["rawRGB"].view(np.uint32), ref["rawRGB"].view(np.uint32))
    assert np.array_equal(out["rpp"], ref["rpp"])
    plain = R.render(sc, cam, R.launch_params(w, h, spp, depth=50, seed=77))
    assert not np.array_equal(plain["rawRGB"], out["rawRGB"])   # the mapping does change the image
    g = device_first_hit(R, cuda, sc, cam, R.launch_params(w, h, 1, seed=77, flags=R.RT_FLAG_RTOW_PIXELS))
    c = wd.first_hit(oracle_camera(O, cam, rtow_pixels=True), w, h, 77, use_bvh=True)
    assert np.array_equal(g["prim"], c["prim"]) and np.array_equal(g["t"].view(np.uint32), c["t"].view(np.uint32))


def test_rtow_pixels_needs_two_pixels(product, cuda):
    R = product
    sc = R.rtow_scene(None)
    with pytest.raises(R.RTError) as e:
        R.render(sc, R.rtow_camera(1, 8), R.launch_params(1, 8, 1, flags=R.RT_FLAG_RTOW_PIXELS))
    assert e.value.status == R.RT_ERR_INVALID_ARG
    with pytest.raises(R.RTError):
        R.render(sc, R.rtow_camera(8, 8), R.launch_params(8, 8, 1, flags=0x100))   # unknown flag


def _gamma2_top_down(R, torch, raw):
    src = torch.from_numpy(np.ascontiguousarray(raw, np.float32).reshape(-1)).cuda()
    dst = torch.zeros(W * H * 4, dtype=torch.uint8, device="cuda")
    R.check(R.lib().rt_postproc_gamma2(ctypes.c_void_p(src.data_ptr()), ctypes.c_void_p(dst.data_ptr()), W, H,
                                       None))
    torch.cuda.synchronize()
    return dst.cpu().numpy().reshape(H, W, 4)[::-1, :, :3]


def test_product_matches_rtow_statistically(product, cuda):
    R, torch = product, cuda
    f = np.load(FIXTURE)
    sc = R.rtow_scene(None)   # analytic spheres, glibc seed 1: rtow's scene()
    cam = R.rtow_camera(W, H)
    a, b = (_gamma2_top_down(R, torch, R.render(sc, cam, R.launch_params(W, H, SPP, depth=DEPTH, seed=s,
                                                                        flags=R.RT_FLAG_RTOW_PIXELS))["rawRGB"])
            for s in (101, 202))
    rel_rmse, bias = check_against_rtow(a, b, f["blocks"], int(f["block"]))
    assert rel_rmse < 0.01
