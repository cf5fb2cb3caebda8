"""Shared helpers of the test suite (device buffers through torch, golden files)."""
import ctypes
import hashlib
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def dptr(t):
    return ctypes.c_void_p(t.data_ptr())


def golden_sphere(n):
    with open(os.path.join(GOLDEN, f"sphere_r1_n{n}.bin"), "rb") as f:
        b = f.read()
    nv, ni = np.frombuffer(b[:8], np.uint32)
    v = np.frombuffer(b[8:8 + 12 * nv], np.float32).reshape(-1, 3)
    i = np.frombuffer(b[8 + 12 * nv:], np.uint32).reshape(-1, 3)
    return v, i


def sphere_hashes():
    with open(os.path.join(GOLDEN, "sphere_hashes.json")) as f:
        return json.load(f)


def mesh_hash(v, i):
    return (hashlib.sha256(np.ascontiguousarray(v, np.float32).tobytes()).hexdigest(),
            hashlib.sha256(np.ascontiguousarray(i, np.uint32).tobytes()).hexdigest())


def golden_scene(seed):
    return np.loadtxt(os.path.join(GOLDEN, f"rtow_scene_seed{seed}.txt"))


def rtow_pair(R, O, level, rng_kind=0, seed=1, half_extent=11, morton_bits=60, layout=0):
    """The same final scene in the product (GPU, any layout) and in the oracle
    (CPU; flat LBVH, with things-grouped keys when the product's layout is
    RT_LAYOUT_GROUPED).  Hits and images do not depend on the trees."""
    sc = R.rtow_scene(level, rng_kind, seed, half_extent, morton_bits, layout=layout)
    w, _ = O.rtow_world(level, rng_kind, seed, half_extent, morton_bits, grouped=layout == 3)
    return sc, w


def device_first_hit(R, torch, sc, cam, params, sample=0):
    n = params.image_w * params.image_h
    prim = torch.empty(n, dtype=torch.int32, device="cuda")
    thing = torch.empty(n, dtype=torch.int32, device="cuda")
    t = torch.empty(n, dtype=torch.float32, device="cuda")
    u = torch.empty(n, dtype=torch.float32, device="cuda")
    v = torch.empty(n, dtype=torch.float32, device="cuda")
    t64 = torch.empty(n, dtype=torch.float64, device="cuda")
    R.check(R.lib().rt_first_hit(sc.h, ctypes.byref(cam), ctypes.byref(params), sample, dptr(prim),
                                 dptr(thing), dptr(t), dptr(u), dptr(v), dptr(t64), None))
    torch.cuda.synchronize()
    return dict(prim=prim.cpu().numpy(), thing=thing.cpu().numpy(), t=t.cpu().numpy(),
                u=u.cpu().numpy(), v=v.cpu().numpy(), t64=t64.cpu().numpy())


def oracle_camera(O, cam, rtow_pixels=False):
    """Oracle camera struct from the product's rt_camera (same float bits); rtow_pixels:
    rtow's pixel mapping, the product's RT_FLAG_RTOW_PIXELS."""
    oc = O._Camera()
    oc.rtow_pixels = 1 if rtow_pixels else 0
    oc.eye[:] = [cam.eye.x, cam.eye.y, cam.eye.z]
    for name in ("u", "v", "w", "hvec", "wvec", "dvec"):
        f = getattr(cam, name)
        getattr(oc, name)[:] = [f.x, f.y, f.z]
    oc.aperture = cam.aperture
    return oc
