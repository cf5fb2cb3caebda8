"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

Bit-exact for integer/index work and for the float path (tessellation,
Morton codes, LBVH topology and boxes, first-hit ids/t/u/v, rendered images,
rays per pixel); hit distances within 1e-5 relative of an FP64 oracle;
sRGB bytes within 1 (powf differs by an ulp between CUDA and glibc).
"""
import ctypes

import numpy as np
import pytest

from _helpers import (device_first_hit, dptr, golden_sphere, mesh_hash, oracle_camera, rtow_pair,
                      sphere_hashes)

pytestmark = pytest.mark.gpu


# ---------------------------------------------------------------- tessellation
@pytest.mark.parametrize("n", [0, 1, 2, 3, 4])
def test_tessellation_bit_exact_vs_reference_golden(product, cuda, n):
    R = product
    sc = R.Scene()
    mid = sc.add_sphere_mesh(1.0, n)
    v, i = sc.get_mesh(mid)
    gv, gi = golden_sphere(n)
    assert v.shape == gv.shape and i.shape == gi.shape
    assert np.array_equal(v.view(np.uint32), gv.view(np.uint32))
    assert np.array_equal(i, gi)


@pytest.mark.parametrize("key", ["r1.0_n5", "r1.0_n6", "r1.0_n7", "r1.0_n8", "r0.2_n6", "r1000.0_n6"])
def test_tessellation_hash_vs_reference_golden(product, cuda, key):
    g = sphere_hashes()[key]
    sc = product.Scene()
    mid = sc.add_sphere_mesh(g["radius"], g["ndiv"])
    v, i = sc.get_mesh(mid)
    assert (len(v), len(i)) == (g["nv"], g["ni"])
    assert mesh_hash(v, i) == (g["vces_sha256"], g["ices_sha256"])


# ------------------------------------------------------------------ radix sort
@pytest.mark.parametrize("bits,n", [(30, 1), (30, 4097), (30, 300000), (60, 123457), (64, 70000), (8, 5000)])
def test_radix_sort_stable_bit_exact(product, cuda, bits, n):
    torch = cuda
    rng = np.random.default_rng(bits * 1000 + n)
    if bits <= 32:
        keys = rng.integers(0, 1 << min(bits, 16), n, dtype=np.uint64).astype(np.uint32)   # many duplicates
        kt = torch.from_numpy(keys.view(np.int32)).cuda()
    else:
        keys = rng.integers(0, 1 << 20, n, dtype=np.uint64) << np.uint64(bits - 20)
        keys |= rng.integers(0, 4, n, dtype=np.uint64)
        kt = torch.from_numpy(keys.view(np.int64)).cuda()
    vals = np.arange(n, dtype=np.uint32)
    vt = torch.from_numpy(vals.view(np.int32)).cuda()
    product.check(product.lib().rt_radix_sort_pairs(dptr(kt), dptr(vt), n, bits, None))
    order = np.argsort(keys, kind="stable")
    got_k = kt.cpu().numpy().view(keys.dtype)
    got_v = vt.cpu().numpy().view(np.uint32)
    assert np.array_equal(got_k, keys[order])
    assert np.array_equal(got_v, vals[order])


# ------------------------------------------------------------------------ LBVH
@pytest.mark.parametrize("bits,layout", [(30, 1), (60, 1), (60, 3)])
@pytest.mark.parametrize("level", [None, 2, 3])
def test_lbvh_bit_exact_vs_oracle_twin(product, oracle, cuda, bits, level, layout):
    """Morton (flat) or things-grouped (grouped) keys, sorted ids, Karras
    children and refit boxes equal the oracle twin's bit for bit."""
    sc, w = rtow_pair(product, oracle, level, morton_bits=bits, layout=layout)
    a, b = sc.lbvh(), w.lbvh()
    assert np.array_equal(a["codes"], b["codes"])
    assert np.array_equal(a["ids"], b["ids"])
    assert np.array_equal(a["left"], b["left"])
    assert np.array_equal(a["right"], b["right"])
    assert np.array_equal(a["boxes"].view(np.uint32), b["boxes"].view(np.uint32))


@pytest.mark.parametrize("layout", [1, 2, 3, 4])
def test_lbvh_topology_is_a_binary_tree(product, cuda, layout):
    sc = product.rtow_scene(3, layout=layout)
    t = sc.lbvh()
    n = len(t["ids"])
    seen_leaf = np.zeros(n, bool)
    seen_int = np.zeros(n - 1, bool)
    kids = np.concatenate([t["left"], t["right"]])
    roots = np.setdiff1d(np.arange(n - 1), kids[kids >= 0])
    assert len(roots) == 1   # the root: the one internal node no node points at
    seen_int[roots[0]] = True
    for c in kids:
        if c < 0:
            assert not seen_leaf[~c]
            seen_leaf[~c] = True
        else:
            assert not seen_int[c]
            seen_int[c] = True
    assert seen_leaf.all() and seen_int.all()
    assert np.array_equal(np.sort(t["ids"]), np.arange(n, dtype=np.uint32))


# ------------------------------------------------------------------- first hit
@pytest.mark.parametrize("layout", [1, 2, 3, 4])
@pytest.mark.parametrize("level,w,h", [(None, 192, 108), (2, 192, 108), (3, 320, 180)])
def test_first_hit_bit_exact_vs_oracle(product, oracle, cuda, level, w, h, layout):
    R, O = product, oracle
    sc, wd = rtow_pair(R, O, level, layout=layout)
    cam = R.rtow_camera(w, h)
    params = R.launch_params(w, h, 1, seed=4711)
    g = device_first_hit(R, cuda, sc, cam, params)
    c = wd.first_hit(oracle_camera(O, cam), w, h, 4711, use_bvh=True)
    assert np.array_equal(g["prim"], c["prim"])
    assert np.array_equal(g["thing"], c["thing"])
    for k in ("t", "u", "v"):
        assert np.array_equal(g[k].view(np.uint32), c[k].view(np.uint32)), k
    assert (g["prim"] >= 0).mean() > 0.5


@pytest.mark.parametrize("layout", [1, 2, 3, 4])
def test_first_hit_equals_brute_force(product, oracle, cuda, layout):
    R, O = product, oracle
    sc, wd = rtow_pair(R, O, 1, half_extent=4, layout=layout)
    cam = R.rtow_camera(96, 64)
    params = R.launch_params(96, 64, 1, seed=7)
    g = device_first_hit(R, cuda, sc, cam, params, sample=3)
    c = wd.first_hit(oracle_camera(O, cam), 96, 64, 7, sample=3, use_bvh=False)
    assert np.array_equal(g["prim"], c["prim"])
    assert np.array_equal(g["t"].view(np.uint32), c["t"].view(np.uint32))


@pytest.mark.parametrize("layout", [1, 2, 3, 4])
def test_first_hit_t_within_1e5_of_fp64(product, oracle, cuda, layout):
    R, O = product, oracle
    sc, wd = rtow_pair(R, O, 3, layout=layout)
    cam = R.rtow_camera(256, 144)
    params = R.launch_params(256, 144, 1, seed=11)
    g = device_first_hit(R, cuda, sc, cam, params)
    c = wd.first_hit(oracle_camera(O, cam), 256, 144, 11, fp64=True)
    hit = g["prim"] >= 0
    assert np.array_equal(hit, np.isfinite(g["t64"]))
    # reported distance: the selected primitive re-evaluated in FP64 (tolerance 1e-5 relative)
    rel64 = np.abs(g["t64"][hit] - c["t64"][hit]) / c["t64"][hit]
    assert rel64.max() <= 1e-5, rel64.max()
    # binary32 selection distance: grazing hits lose digits (error ~ eps / sin(angle))
    rel32 = np.abs(g["t"][hit].astype(np.float64) - c["t64"][hit]) / c["t64"][hit]
    assert np.mean(rel32 <= 1e-5) >= 0.999, np.mean(rel32 <= 1e-5)


def test_picker_matches_first_hit(product, oracle, cuda):
    R, O = product, oracle
    sc, wd = rtow_pair(R, O, 2)
    cam = R.rtow_camera(160, 90)
    params = R.launch_params(160, 90, 1, seed=4711)
    c = wd.first_hit(oracle_camera(O, cam), 160, 90, 4711)
    for (x, y) in [(0, 0), (80, 45), (30, 20), (159, 89), (100, 10)]:
        tid = ctypes.c_uint()
        R.check(R.lib().rt_pick(sc.h, ctypes.byref(cam), ctypes.byref(params), x, y, ctypes.byref(tid), None))
        want = c["thing"][160 * y + x]
        assert tid.value == (0xFFFFFFFF if want < 0 else want)


# ----------------------------------------------------------------------- render
@pytest.mark.parametrize("layout", [1, 2, 3, 4])
@pytest.mark.parametrize("level,w,h,spp,depth", [(None, 64, 36, 4, 50), (2, 64, 36, 3, 50), (3, 48, 32, 2, 8),
                                                 (2, 40, 30, 5, 1)])
def test_render_bit_exact_vs_oracle(product, oracle, cuda, level, w, h, spp, depth, layout):
    R, O = product, oracle
    sc, wd = rtow_pair(R, O, level, layout=layout)
    cam = R.rtow_camera(w, h)
    params = R.launch_params(w, h, spp, depth=depth, seed=4711, flags=R.RT_FLAG_GUIDES)
    out = R.render(sc, cam, params, guides=True)
    ref = wd.render(oracle_camera(O, cam), w, h, spp, depth, 4711)
    assert np.array_equal(out["rpp"], ref["rpp"])
    assert int(out["stats"].rays) == ref["rays"]
    assert np.array_equal(out["rawRGB"].view(np.uint32), ref["rawRGB"].view(np.uint32))
    assert np.array_equal(out["normals"].view(np.uint32), ref["normals"].view(np.uint32))
    assert np.array_equal(out["albedos"].view(np.uint32), ref["albedos"].view(np.uint32))


def test_render_small_waves_match(product, oracle, cuda, monkeypatch):
    """A tiny wave forces many waves and regenerations."""
    R, O = product, oracle
    monkeypatch.setenv("RTX_WAVE", "1000")
    sc, wd = rtow_pair(R, O, 2)
    cam = R.rtow_camera(128, 96)
    params = R.launch_params(128, 96, 21, depth=50, seed=99)
    out = R.render(sc, cam, params)
    ref = wd.render(oracle_camera(O, cam), 128, 96, 21, 50, 99, guides=False)
    assert np.array_equal(out["rawRGB"].view(np.uint32), ref["rawRGB"].view(np.uint32))
    assert np.array_equal(out["rpp"], ref["rpp"])


def test_postproc_vs_oracle(product, oracle, cuda):
    R, O, torch = product, oracle, cuda
    w, h = 64, 48
    rng = np.random.default_rng(5)
    raw = rng.random((w * h, 3), dtype=np.float32)
    raw[:10] = [0.0, 1.0, 0.0031308]
    src = torch.from_numpy(raw).cuda()
    for kind, fn in (("srgb", R.lib().rt_postproc_srgb), ("none", R.lib().rt_postproc_none),
                     ("gamma2", R.lib().rt_postproc_gamma2)):
        dst = torch.empty(w * h * 4, dtype=torch.uint8, device="cuda")
        R.check(fn(dptr(src), dptr(dst), w, h, None))
        got = dst.cpu().numpy().reshape(-1, 4)
        want = O.pp(kind, raw, w, h)
        diff = np.abs(got.astype(int) - want.astype(int))
        if kind == "srgb":
            assert diff.max() <= 1 and (diff > 0).mean() < 1e-2
        else:
            assert diff.max() == 0


# -------------------------------------------------------------- update / refit
@pytest.mark.parametrize("layout", [1, 2, 3, 4])
def test_update_refit_after_transform_edit(product, oracle, cuda, layout):
    R, O = product, oracle
    sc, wd = rtow_pair(R, O, 2, layout=layout)
    moved = {0: None, 5: (1.5, 0.0, -2.0), 100: (0.0, 0.6, 0.3), 486: (-1.0, 0.5, 1.0)}
    for tid, dv in moved.items():
        st, T = sc.get_transform(tid)
        assert st == R.RT_OK
        T = T.copy()
        if dv is None:
            T[0] *= 1.01; T[5] *= 1.01; T[10] *= 1.01
        else:
            T[3] += dv[0]; T[7] += dv[1]; T[11] += dv[2]
        assert sc.set_transform(tid, T) == R.RT_OK
        assert wd.set_transform(tid, T) == 0
    cam = R.rtow_camera(160, 90)
    params = R.launch_params(160, 90, 1, seed=4711)
    sc.update()
    wd.build()
    g = device_first_hit(R, cuda, sc, cam, params)
    c = wd.first_hit(oracle_camera(O, cam), 160, 90, 4711)
    assert np.array_equal(g["prim"], c["prim"])
    assert np.array_equal(g["t"].view(np.uint32), c["t"].view(np.uint32))


def test_errors_are_status_codes(product, cuda):
    R = product
    sc = R.Scene()
    assert sc.set_transform(3, np.zeros(12, np.float32)) == R.RT_ERR_INVALID_ARG
    st, _ = sc.get_transform(0)
    assert st == R.RT_ERR_INVALID_ARG
    cam = R.rtow_camera(8, 8)
    L = R.Launcher(8, 8)
    with pytest.raises(R.RTError) as e:
        L.ignite(sc, cam, R.launch_params(8, 8, 1))
    assert e.value.status == R.RT_ERR_NOT_BUILT
    with pytest.raises(R.RTError) as e:
        R.Scene().add_sphere_mesh(1.0, 11)
    assert e.value.status == R.RT_ERR_INVALID_ARG
    sc.load_rtow(ndiv=1, half_extent=2)
    sc.build()
    with pytest.raises(R.RTError) as e:
        L.ignite(sc, cam, R.launch_params(8, 8, 1, depth=0))
    assert e.value.status == R.RT_ERR_INVALID_ARG
    st, T = sc.get_transform(1)
    sc.set_transform(1, T)
    with pytest.raises(R.RTError) as e:
        L.ignite(sc, cam, R.launch_params(8, 8, 1))
    assert e.value.status == R.RT_ERR_NOT_BUILT   # transforms edited, no update yet
    sc.update()
    L.ignite(sc, cam, R.launch_params(8, 8, 1))


def test_empty_and_single_primitive_scenes(product, cuda):
    R = product
    sc = R.Scene()
    sc.build()
    out = R.render(sc, R.rtow_camera(16, 8), R.launch_params(16, 8, 2))
    assert (out["rpp"] == 2).all()   # every primary ray misses
    sc2 = R.Scene()
    sc2.add_analytic_sphere((0, 0, 0), 1.0, R.optics(R.RT_OPTICS_DIFFUSE, (0.5, 0.5, 0.5)))
    sc2.build()
    out2 = R.render(sc2, R.camera_set((0, 0, 5), (0, 0, 0), (0, 1, 0), 40, 1.0, 0.0, 5.0),
                    R.launch_params(16, 16, 2))
    assert out2["rpp"].max() > 2
