"""GPU: the `rtwo` launcher (C++ over the C ABI, RTWO's command line).

The launcher's P3 image and P2 rays-per-pixel outputs (rows bottom-up, as
RTWO's imgtopnm writes them) must equal the library's own render of the same
scene, camera and parameters through the Python binding, byte for byte; the
statistics line on stderr must count the same rays.
"""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rtwo():
    from rtxplay_gb300 import _build
    if not os.path.exists(_build.RTWO):
        _build.build_rtwo()
    return _build.RTWO


def _pnm_blocks(text):
    """Splits concatenated plain PNMs into (magic, w, h, values)."""
    tok = text.split()
    out, k = [], 0
    while k < len(tok):
        magic, w, h, _maxval = tok[k], int(tok[k + 1]), int(tok[k + 2]), int(tok[k + 3])
        k += 4
        nval = w * h * (3 if magic == "P3" else 1)
        vals = np.array(tok[k:k + nval], np.int64)
        k += nval
        out.append((magic, w, h, vals))
    return out


@pytest.mark.parametrize("scene,level", [("analytic", None), ("tess", 2)])
def test_rtwo_matches_library_render(product, cuda, scene, level):
    R = product
    w, h, spp, seed = 96, 64, 2, 77
    args = [_rtwo(), "-g", f"{w}x{h}", "-s", str(spp), "-d", "50", "--scene", scene, "--seed", str(seed),
            "-A", "RPP", "-S"]
    if level is not None:
        args += ["--level", str(level)]
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    blocks = _pnm_blocks(r.stdout)
    assert [b[0] for b in blocks] == ["P3", "P2"] and all(b[1] == w and b[2] == h for b in blocks)
    img = blocks[0][3].reshape(h, w, 3)[::-1].reshape(-1, 3)   # rows bottom-up
    rpp = blocks[1][3].reshape(h, w)[::-1].reshape(-1)
    sc = R.rtow_scene(level, R.RT_RECIPE_GLIBC, 1, 11)
    out = R.render(sc, R.rtow_camera(w, h), R.launch_params(w, h, spp, depth=50, seed=seed))
    assert np.array_equal(rpp, out["rpp"].astype(np.int64))
    assert np.array_equal(img, out["image"][:, :3].astype(np.int64))
    rays = int(r.stderr.split()[1])
    assert rays == int(out["rpp"].sum())


def test_rtwo_print_args_and_errors(product, cuda):
    exe = _rtwo()
    r = subprocess.run([exe, "--print-args", "-g", "320x200", "-s", "7", "-d", "9"], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 0
    import json
    a = json.loads(r.stdout)
    assert (a["w"], a["h"], a["spp"], a["depth"]) == (320, 200, 7, 9)
    bad = subprocess.run([exe, "--scene", "nosuch"], capture_output=True, text=True, timeout=60)
    assert bad.returncode != 0 and "rtwo:" in bad.stderr


def test_rtwo_checkpoint_and_resume(product, cuda, tmp_path):
    """rtwo -s 3 --checkpoint f, then rtwo -s 4 --resume f: the image and rays per
    pixel of one 7-spp render."""
    R = product
    exe, w, h, seed = _rtwo(), 64, 48, 9
    ck = str(tmp_path / "ck.bin")
    base = [exe, "-g", f"{w}x{h}", "-d", "50", "--scene", "tess", "--level", "2", "--seed", str(seed), "-A", "RPP"]
    r1 = subprocess.run(base + ["-s", "3", "--checkpoint", ck], capture_output=True, text=True, timeout=300)
    assert r1.returncode == 0, r1.stderr
    r2 = subprocess.run(base + ["-s", "4", "--resume", ck, "--checkpoint", ck], capture_output=True, text=True,
                        timeout=300)
    assert r2.returncode == 0, r2.stderr
    blocks = _pnm_blocks(r2.stdout)
    img = blocks[0][3].reshape(h, w, 3)[::-1].reshape(-1, 3)
    rpp = blocks[1][3].reshape(h, w)[::-1].reshape(-1)
    sc = R.rtow_scene(2, R.RT_RECIPE_GLIBC, 1, 11)
    out = R.render(sc, R.rtow_camera(w, h), R.launch_params(w, h, 7, depth=50, seed=seed))
    assert np.array_equal(rpp, out["rpp"].astype(np.int64))
    assert np.array_equal(img, out["image"][:, :3].astype(np.int64))
    # a checkpoint of another image size is refused
    bad = subprocess.run([exe, "-g", "32x32", "-s", "1", "--scene", "tess", "--level", "2", "--resume", ck, "-q"],
                         capture_output=True, text=True, timeout=300)
    assert bad.returncode != 0 and "image size" in bad.stderr
