"""Runs the renders of test_gpu_checked.py in a process that loaded the
bounds-checked library (RTX_LIB) and compares them with the normal build's
results saved by the test (npz given as argv[1]).  Prints "checked ok"."""
import ctypes
import sys

import numpy as np

import rtxplay_gb300 as R


def renders():
    """The workloads: name -> dict of arrays (same code in both processes)."""
    out = {}
    w, h = 64, 48
    cam = R.rtow_camera(w, h)
    for name, level, layout in (("sah", 2, R.RT_LAYOUT_SAH), ("inst", 2, R.RT_LAYOUT_INSTANCED),
                                ("grouped", 2, R.RT_LAYOUT_GROUPED), ("flat", 2, R.RT_LAYOUT_FLAT),
                                ("analytic", None, R.RT_LAYOUT_AUTO)):
        sc = R.rtow_scene(level, layout=layout)
        r = R.render(sc, cam, R.launch_params(w, h, 3, depth=50, seed=5))
        out[name + "_raw"] = r["rawRGB"].view(np.uint32)
        out[name + "_rpp"] = r["rpp"]
        sc.close()
    return out


def main():
    assert b"bounds-checked" in R.version().encode(), R.version()
    ref = np.load(sys.argv[1])
    got = renders()
    for k, v in got.items():
        assert np.array_equal(v, ref[k]), k
    print("checked ok")


if __name__ == "__main__":
    main()
