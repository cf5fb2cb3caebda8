"""GPU: the two acceleration-structure layouts give the same hits and images.

A scene mixing analytic spheres, diagonally transformed mesh things
(instanced: one object-space LBVH per mesh under a top level), a negative
scale (instanced, box bounds swap), rotated things and a small mesh (both
flattened to world space) is rendered with RT_LAYOUT_FLAT, RT_LAYOUT_INSTANCED,
RT_LAYOUT_AUTO and RT_LAYOUT_SAH; every image, ray count and first hit must be
identical and equal to the oracle's (which always uses one flat LBVH).
"""
import numpy as np
import pytest

from _helpers import device_first_hit, oracle_camera

pytestmark = pytest.mark.gpu


def _rot_y(a):
    c, s = np.cos(a), np.sin(a)
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]], np.float32)


def _things():
    """(kind, mesh level or None, optics (type, albedo, fuzz, index), transform or (centre, r))"""
    out = []
    out.append(("sphere", None, (0, (0.5, 0.5, 0.5), 0.0, 0.0), ((0, -1000, 0), 1000.0)))
    rng = np.random.default_rng(3)
    for k in range(14):
        r = float(rng.uniform(0.2, 0.6))
        c = (float(rng.uniform(-4, 4)), r, float(rng.uniform(-3, 3)))
        typ = k % 3
        opt = (typ, tuple(float(x) for x in rng.uniform(0.2, 0.9, 3)), 0.2 * (typ == 1), 1.5 if typ == 2 else 0.0)
        if k % 4 == 3:       # rotated: cannot be instanced
            M = _rot_y(0.3 * k) * r
            T = np.array([M[0, 0], M[0, 1], M[0, 2], c[0], M[1, 0], M[1, 1], M[1, 2], c[1],
                          M[2, 0], M[2, 1], M[2, 2], c[2]], np.float32)
            out.append(("mesh", 3, opt, T))
        elif k % 4 == 1:     # small mesh: flattened in AUTO, instanced in INSTANCED
            T = np.array([r, 0, 0, c[0], 0, r, 0, c[1], 0, 0, r, c[2]], np.float32)
            out.append(("mesh", 1, opt, T))
        elif k == 2:         # mirrored: negative scale on x
            T = np.array([-r, 0, 0, c[0], 0, r, 0, c[1], 0, 0, r, c[2]], np.float32)
            out.append(("mesh", 3, opt, T))
        else:
            T = np.array([r, 0, 0, c[0], 0, r, 0, c[1], 0, 0, 1.3 * r, c[2]], np.float32)
            out.append(("mesh", 3, opt, T))
        if k % 5 == 0:
            out.append(("sphere", None, opt, ((c[0], c[1] + 1.2 * r + 0.3, c[2]), 0.3)))
    return out


def _build_pair(R, O, layout):
    sc = R.Scene()
    wd = O.World()
    meshes, omeshes = {}, {}
    for kind, level, opt, geo in _things():
        o = R.optics(opt[0], opt[1], opt[2], opt[3])
        if kind == "sphere":
            sc.add_analytic_sphere(geo[0], geo[1], o)
            wd.add_sphere(opt[0], np.asarray(opt[1], np.float32), opt[2], opt[3], np.asarray(geo[0], np.float32),
                          float(geo[1]))
            continue
        if level not in meshes:
            meshes[level] = sc.add_sphere_mesh(1.0, level)
            v, i = O.tessellate(1.0, level)
            omeshes[level] = wd.add_mesh(v, i)
        sc.add_thing(o, meshes[level], geo)
        wd.add_thing(opt[0], np.asarray(opt[1], np.float32), opt[2], opt[3], omeshes[level], geo)
    sc.build(layout=layout)
    wd.build(60)
    return sc, wd


def test_layout_info(product, oracle, cuda):
    R, O = product, oracle
    flat, _ = _build_pair(R, O, R.RT_LAYOUT_FLAT)
    inst, _ = _build_pair(R, O, R.RT_LAYOUT_INSTANCED)
    auto, _ = _build_pair(R, O, R.RT_LAYOUT_AUTO)
    sah, _ = _build_pair(R, O, R.RT_LAYOUT_SAH)
    fi, ii, ai, si = flat.info(), inst.info(), auto.info(), sah.info()
    assert si.layout == R.RT_LAYOUT_SAH and si.n_top_records == fi.n_top_records and si.n_instances == 0
    assert fi.layout == R.RT_LAYOUT_FLAT and fi.n_instances == 0 and fi.n_bottom_records == 0
    assert ii.layout == R.RT_LAYOUT_INSTANCED and ai.layout == R.RT_LAYOUT_SAH
    assert fi.n_prims == ii.n_prims == ai.n_prims == fi.n_top_records == ai.n_top_records
    assert ai.n_instances == 0 and ai.n_bottom_records == 0
    assert ii.n_instances == 11                           # diagonal things; the rotated ones are flattened
    assert ii.n_bottom_records == 256 + 16                # one bottom level per mesh, shared by its things


@pytest.mark.parametrize("w,h,spp,depth", [(96, 64, 3, 50), (64, 64, 2, 8)])
def test_layouts_render_identically_and_match_oracle(product, oracle, cuda, w, h, spp, depth):
    R, O = product, oracle
    cam = R.camera_set((0, 2.5, 9), (0, 0.3, 0), (0, 1, 0), 40, w / h, 0.05, 9.0)
    params = R.launch_params(w, h, spp, depth=depth, seed=31, flags=R.RT_FLAG_GUIDES)
    outs = []
    for layout in (R.RT_LAYOUT_FLAT, R.RT_LAYOUT_INSTANCED, R.RT_LAYOUT_AUTO, R.RT_LAYOUT_SAH):
        sc, wd = _build_pair(R, O, layout)
        outs.append(R.render(sc, cam, params, guides=True))
    ref = wd.render(oracle_camera(O, cam), w, h, spp, depth, 31)
    for out in outs:
        assert np.array_equal(out["rawRGB"].view(np.uint32), ref["rawRGB"].view(np.uint32))
        assert np.array_equal(out["rpp"], ref["rpp"])
        assert np.array_equal(out["normals"].view(np.uint32), ref["normals"].view(np.uint32))
        assert np.array_equal(out["albedos"].view(np.uint32), ref["albedos"].view(np.uint32))
    assert outs[0]["rpp"].max() > spp   # something is hit


def test_layouts_first_hit_and_fp64_distance(product, oracle, cuda):
    R, O = product, oracle
    w, h = 160, 120
    cam = R.camera_set((0, 2.5, 9), (0, 0.3, 0), (0, 1, 0), 40, w / h, 0.0, 9.0)
    params = R.launch_params(w, h, 1, seed=5)
    for layout in (R.RT_LAYOUT_FLAT, R.RT_LAYOUT_INSTANCED, R.RT_LAYOUT_GROUPED, R.RT_LAYOUT_SAH):
        sc, wd = _build_pair(R, O, layout)
        g = device_first_hit(R, cuda, sc, cam, params)
        c = wd.first_hit(oracle_camera(O, cam), w, h, 5, fp64=True)
        assert np.array_equal(g["prim"], c["prim"])
        assert np.array_equal(g["thing"], c["thing"])
        for k in ("t", "u", "v"):
            assert np.array_equal(g[k].view(np.uint32), c[k].view(np.uint32)), k
        hit = g["prim"] >= 0
        assert np.abs(g["t64"][hit] - c["t64"][hit]).max() <= 1e-5 * c["t64"][hit].max()


def test_update_moves_instances_and_switches_class(product, oracle, cuda):
    """Diagonal edits refit the top level; a diagonal thing turned into a
    rotated one (and a rotated one made diagonal) rebuilds."""
    R, O = product, oracle
    sc, wd = _build_pair(R, O, R.RT_LAYOUT_INSTANCED)
    n0 = sc.info().n_instances
    diag = [k for k, (kind, level, opt, geo) in enumerate(_things())
            if kind == "mesh" and level == 3 and geo[0] > 0 and not np.any(geo[[1, 2, 4, 6, 8, 9]])]
    edits = {}
    st, T = sc.get_transform(diag[0])  # diagonal -> moved
    T = T.copy(); T[3] += 0.7; T[11] -= 0.4
    edits[diag[0]] = T
    st, T = sc.get_transform(diag[1])  # diagonal -> rotated
    M = _rot_y(0.5) * T[0]
    edits[diag[1]] = np.array([M[0, 0], M[0, 1], M[0, 2], T[3], M[1, 0], M[1, 1], M[1, 2], T[7],
                               M[2, 0], M[2, 1], M[2, 2], T[11]], np.float32)
    for tid, T in edits.items():
        assert sc.set_transform(tid, T) == R.RT_OK
        assert wd.set_transform(tid, T) == 0
    sc.update()
    wd.build()
    assert sc.info().n_instances == n0 - 1
    w, h = 128, 96
    cam = R.camera_set((0, 2.5, 9), (0, 0.3, 0), (0, 1, 0), 40, w / h, 0.0, 9.0)
    params = R.launch_params(w, h, 2, depth=16, seed=8)
    out = R.render(sc, cam, params)
    ref = wd.render(oracle_camera(O, cam), w, h, 2, 16, 8, guides=False)
    assert np.array_equal(out["rawRGB"].view(np.uint32), ref["rawRGB"].view(np.uint32))
    assert np.array_equal(out["rpp"], ref["rpp"])


def test_flat_and_instanced_batches_agree(product, cuda):
    R, torch = product, cuda
    from _helpers import dptr
    specs = [(3, 3, 48, 32, 2, 16, 5), (2, 2, 32, 32, 3, 8, 6), (None, 4, 40, 24, 2, 16, 7)]
    imgs = {}
    for layout in (R.RT_LAYOUT_FLAT, R.RT_LAYOUT_INSTANCED, R.RT_LAYOUT_GROUPED, R.RT_LAYOUT_SAH):
        batch = R.Batch()
        bufs = []
        for level, he, w, h, spp, depth, seed in specs:
            sc = R.Scene()
            sc.load_rtow(R.RT_RECIPE_COUNTER, seed, he, -1 if level is None else level)
            raw = torch.zeros(w * h * 3, dtype=torch.float32, device="cuda")
            rpp = torch.zeros(w * h, dtype=torch.int32, device="cuda")
            batch.add(sc, R.rtow_camera(w, h), R.launch_params(w, h, spp, depth=depth, seed=seed),
                      R.Frame(dptr(raw), dptr(rpp), None, None))
            bufs.append((raw, rpp))
        batch.build(layout=layout)
        batch.launch()
        torch.cuda.synchronize()
        imgs[layout] = [(a.cpu().numpy(), b.cpu().numpy()) for a, b in bufs]
    for other in (R.RT_LAYOUT_INSTANCED, R.RT_LAYOUT_GROUPED, R.RT_LAYOUT_SAH):
        for (a, b), (c, d) in zip(imgs[R.RT_LAYOUT_FLAT], imgs[other]):
            assert np.array_equal(a.view(np.uint32), c.view(np.uint32))
            assert np.array_equal(b, d)
