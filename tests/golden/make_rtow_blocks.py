"""Golden statistics of the reference's own CPU renderer.

Test infrastructure only.  Runs the unmodified ``rtow.cxx`` (compiled by
``oracle/ref_build.sh`` into ``oracle/_ref/rtow``): the final scene of
``scene()`` with glibc ``rand()`` seed 1, 1280x720, 10 samples per pixel,
depth 50, written as a gamma-2 8-bit PPM (rtow.cxx:82-121).  rtow draws its
samples from ``rand()``, so its image can be compared only statistically;
this script keeps, per channel, the mean of every 16x16 pixel block (rows
top-down as in the PPM) in ``rtow_1280x720_blocks.npz``:

    bash oracle/ref_build.sh && python tests/golden/make_rtow_blocks.py

It takes about a minute (rtow is single-threaded).
"""
import os
import subprocess
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
RTOW = os.path.join(ROOT, "oracle", "_ref", "rtow")
OUT = os.path.join(HERE, "rtow_1280x720_blocks.npz")
BLOCK = 16


def parse_ppm(text):
    tok = text.split()
    assert tok[0] == "P3", tok[0]
    w, h, maxval = int(tok[1]), int(tok[2]), int(tok[3])
    vals = np.array(tok[4:4 + w * h * 3], np.int64)
    assert maxval == 255 and vals.size == w * h * 3
    return vals.reshape(h, w, 3)


def block_means(img, b=BLOCK):
    h, w, _ = img.shape
    return img.astype(np.float64).reshape(h // b, b, w // b, b, 3).mean(axis=(1, 3))


def main():
    if not os.path.exists(RTOW):
        raise SystemExit("build oracle/_ref/rtow first: bash oracle/ref_build.sh")
    t0 = time.time()
    r = subprocess.run([RTOW], check=True, capture_output=True, text=True)
    img = parse_ppm(r.stdout)
    np.savez_compressed(OUT, blocks=block_means(img), block=BLOCK, w=img.shape[1], h=img.shape[0], spp=10,
                        depth=50, image_mean=img.reshape(-1, 3).mean(axis=0))
    print(f"wrote {OUT}: {img.shape[1]}x{img.shape[0]}, rtow ran {time.time() - t0:.1f} s")


if __name__ == "__main__":
    main()
