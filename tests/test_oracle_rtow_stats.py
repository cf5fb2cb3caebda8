"""CPU: the oracle's render against the reference's own renderer, statistically.

The unmodified rtow.cxx (rand()-driven, FP64) rendered the final scene at
1280x720, 10 spp, depth 50; tests/golden/rtow_1280x720_blocks.npz keeps the
mean of every 16x16 block of its gamma-2 8-bit image (make_rtow_blocks.py).
The oracle renders the same scene, camera and pixel mapping (rtow's, over
w - 1 and h - 1) with its counter RNG, post-processed the same way.  Both
block means estimate the same expectation; the noise of one block mean comes
from two oracle renders with different seeds (their pixel difference cancels
the image structure), plus the 8-bit rounding.

Bounds: every block and channel within 6 noise standard deviations plus 1 %
of its value; the converged relative RMSE over the blocks (the noise variance
subtracted) at most 1 %; per channel, the image means within 0.5 %; and the
noise-normalised squared differences averaging below 1.5 (no structure beyond
noise).  Measured: converged rel-RMSE 0.26 %, the oracle 0.15 % darker.  The
bias is binary32 arithmetic against rtow's FP64: a hit on the r = 1000 ground
sphere is placed up to ~6e-5 inside it, so a few grazing diffuse bounces hit
the ground again beyond t_min (1e-3) and lose half their light; the product
computes in the same binary32 as the oracle, bit for bit.
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "rtow_1280x720_blocks.npz")
W, H, SPP, DEPTH = 1280, 720, 10, 50


def block_stats(a, b, blk):
    """Block means of image a and the variance of one block mean, from a - b."""
    h, w, _ = a.shape
    shape = (h // blk, blk, w // blk, blk, 3)
    m = a.astype(np.float64).reshape(shape).mean(axis=(1, 3))
    d = (a.astype(np.float64) - b.astype(np.float64)).reshape(shape)
    var_pix = d.var(axis=(1, 3), ddof=1) / 2.0 + 1.0 / 12.0   # one render's pixel noise + 8-bit rounding
    return m, var_pix / (blk * blk)


def gamma2_top_down(O, raw):
    img = O.pp("gamma2", raw, W, H)[:, :3].reshape(H, W, 3)
    return img[::-1]   # rows top-down, as rtow writes them


def test_fixture_shape():
    f = np.load(FIXTURE)
    assert int(f["w"]) == W and int(f["h"]) == H and int(f["spp"]) == SPP and int(f["depth"]) == DEPTH
    blk = int(f["block"])
    assert f["blocks"].shape == (H // blk, W // blk, 3)
    assert 0 < f["blocks"].min() and f["blocks"].max() < 256


def test_oracle_matches_rtow_statistically(oracle):
    O = oracle
    f = np.load(FIXTURE)
    ref, blk = f["blocks"], int(f["block"])
    world, _ = O.rtow_world(None, 0, 1, 11)   # analytic spheres, glibc seed 1: rtow's scene()
    cam = O.rtow_camera(W, H)
    cam.rtow_pixels = 1
    a, b = (gamma2_top_down(O, world.render(cam, W, H, SPP, DEPTH, seed, guides=False)["rawRGB"])
            for seed in (101, 202))
    check_against_rtow(a, b, ref, blk)


def check_against_rtow(a, b, ref, blk):
    m, v = block_stats(a, b, blk)
    sd = np.sqrt(2.0 * v)   # both block means carry the noise
    worst = np.abs(m - ref) - (6.0 * sd + 0.01 * ref)
    assert (worst <= 0).all(), np.unravel_index(worst.argmax(), worst.shape)
    rel_rmse = np.sqrt(max(((m - ref) ** 2).mean() - (sd ** 2).mean(), 0.0)) / ref.mean()
    assert rel_rmse <= 0.01, rel_rmse
    bias = m.reshape(-1, 3).mean(axis=0) / ref.reshape(-1, 3).mean(axis=0) - 1.0
    assert (np.abs(bias) <= 0.005).all(), bias
    z = (m - ref) / sd
    assert 0.6 < (z * z).mean() < 1.5
    return rel_rmse, bias
