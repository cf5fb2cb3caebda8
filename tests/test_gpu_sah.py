"""GPU: the binned-SAH layout (RT_LAYOUT_SAH).

The hierarchy is checked as a structure (a binary tree over every record
exactly once, every child box the exact union of what lies below it) for
cluster limits from 1 (SAH splits down to single records) to the default, on
one scene and on a batch; its hits and images must equal the oracle's, whose
flat LBVH is a different tree over the same records.
"""
import numpy as np
import pytest

from _helpers import device_first_hit, oracle_camera, rtow_pair

pytestmark = pytest.mark.gpu


@pytest.fixture
def sah_cluster(monkeypatch):
    def set_(n):
        if n is None:
            monkeypatch.delenv("RTX_SAH_CLUSTER", raising=False)
        else:
            monkeypatch.setenv("RTX_SAH_CLUSTER", str(n))
    return set_


def _check_tree(t, tris):
    n = len(t["ids"])
    assert np.array_equal(np.sort(t["ids"]), np.arange(n, dtype=np.uint32))
    left, right, boxes = t["left"], t["right"], t["boxes"]
    kids = np.concatenate([left, right])
    roots = np.setdiff1d(np.arange(n - 1), kids[kids >= 0])
    assert len(roots) == 1
    leaves = kids[kids < 0]
    assert np.array_equal(np.sort(~leaves), np.arange(n))
    internal = kids[kids >= 0]
    assert len(np.unique(internal)) == len(internal) == n - 2
    # every child box is the union of its content
    tb = tris.reshape(-1, 3, 3)
    plo, phi = tb.min(axis=1), tb.max(axis=1)          # record boxes, record-id order
    nlo = np.minimum(boxes[:, 0:3], boxes[:, 6:9])     # node boxes
    nhi = np.maximum(boxes[:, 3:6], boxes[:, 9:12])
    for k, ch in enumerate((left, right)):
        clo, chi = boxes[:, 6 * k:6 * k + 3], boxes[:, 6 * k + 3:6 * k + 6]
        leaf = ch < 0
        rec = t["ids"][~ch[leaf]]
        assert np.array_equal(clo[leaf], plo[rec]) and np.array_equal(chi[leaf], phi[rec])
        inn = ~leaf
        assert np.array_equal(clo[inn], nlo[ch[inn]]) and np.array_equal(chi[inn], nhi[ch[inn]])
    return roots[0]


@pytest.mark.parametrize("cluster", [1, 3, 16, 2048, None])
def test_sah_tree_structure(product, oracle, cuda, sah_cluster, cluster):
    R, O = product, oracle
    sah_cluster(cluster)
    sc, wd = rtow_pair(R, O, 3, layout=R.RT_LAYOUT_SAH)
    assert sc.info().layout == R.RT_LAYOUT_SAH
    _check_tree(sc.lbvh(), wd.triangles())


@pytest.mark.parametrize("cluster", [1, 16, 2048, None])
def test_sah_hits_and_images_match_oracle(product, oracle, cuda, sah_cluster, cluster):
    R, O = product, oracle
    sah_cluster(cluster)
    sc, wd = rtow_pair(R, O, 3, layout=R.RT_LAYOUT_SAH)
    w, h = 240, 160
    cam = R.rtow_camera(w, h)
    g = device_first_hit(R, cuda, sc, cam, R.launch_params(w, h, 1, seed=11))
    c = wd.first_hit(oracle_camera(O, cam), w, h, 11)
    assert np.array_equal(g["prim"], c["prim"]) and np.array_equal(g["thing"], c["thing"])
    for k in ("t", "u", "v"):
        assert np.array_equal(g[k].view(np.uint32), c[k].view(np.uint32)), k
    w, h, spp, depth = 64, 40, 3, 50
    cam = R.rtow_camera(w, h)
    out = R.render(sc, cam, R.launch_params(w, h, spp, depth=depth, seed=12))
    ref = wd.render(oracle_camera(O, cam), w, h, spp, depth, 12, guides=False)
    assert np.array_equal(out["rawRGB"].view(np.uint32), ref["rawRGB"].view(np.uint32))
    assert np.array_equal(out["rpp"], ref["rpp"])


def test_sah_rebuild_is_deterministic(product, cuda):
    R = product
    a = R.rtow_scene(3, layout=R.RT_LAYOUT_SAH).lbvh()
    b = R.rtow_scene(3, layout=R.RT_LAYOUT_SAH).lbvh()
    for k in ("codes", "ids", "left", "right"):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(a["boxes"].view(np.uint32), b["boxes"].view(np.uint32))


def test_sah_fewer_node_visits_than_morton(product, cuda):
    """The point of the layout: on the final scene (level 3) the SAH tree
    visits fewer nodes per ray than the plain and the things-grouped LBVH."""
    R = product
    w, h = 160, 108
    cam = R.rtow_camera(w, h)
    params = R.launch_params(w, h, 4, depth=8, seed=3, flags=R.RT_FLAG_COUNT_VISITS)
    visits = {}
    for layout in (R.RT_LAYOUT_FLAT, R.RT_LAYOUT_GROUPED, R.RT_LAYOUT_SAH):
        sc = R.rtow_scene(3, layout=layout)
        st = R.render(sc, cam, params)["stats"]
        visits[layout] = st.node_visits / st.rays
    print("node visits per ray (flat, grouped, sah):", visits)
    assert visits[R.RT_LAYOUT_SAH] < visits[R.RT_LAYOUT_GROUPED] < visits[R.RT_LAYOUT_FLAT]


@pytest.mark.parametrize("cluster", [2, None])
def test_sah_batch_segments(product, cuda, sah_cluster, cluster):
    """Scenes of a batch get separate SAH trees (small scenes a single
    cluster); every frame equals its single-scene render."""
    R, torch = product, cuda
    from _helpers import dptr
    sah_cluster(cluster)
    specs = [(3, 3, 48, 32, 2, 16, 5), (None, 2, 32, 32, 3, 8, 6), (2, 4, 40, 24, 2, 16, 7), (None, 1, 16, 16, 2, 8, 8)]
    batch = R.Batch()
    bufs, singles = [], []
    for level, he, w, h, spp, depth, seed in specs:
        sc = R.Scene()
        sc.load_rtow(R.RT_RECIPE_COUNTER, seed, he, -1 if level is None else level)
        raw = torch.zeros(w * h * 3, dtype=torch.float32, device="cuda")
        rpp = torch.zeros(w * h, dtype=torch.int32, device="cuda")
        cam, params = R.rtow_camera(w, h), R.launch_params(w, h, spp, depth=depth, seed=seed)
        batch.add(sc, cam, params, R.Frame(dptr(raw), dptr(rpp), None, None))
        bufs.append((raw, rpp))
        s1 = R.Scene()
        s1.load_rtow(R.RT_RECIPE_COUNTER, seed, he, -1 if level is None else level)
        s1.build(layout=R.RT_LAYOUT_FLAT)
        singles.append(R.render(s1, cam, params))
    batch.build(layout=R.RT_LAYOUT_SAH)
    batch.launch()
    torch.cuda.synchronize()
    for (raw, rpp), ref in zip(bufs, singles):
        assert np.array_equal(raw.cpu().numpy().view(np.uint32), ref["rawRGB"].reshape(-1).view(np.uint32))
        assert np.array_equal(rpp.cpu().numpy(), ref["rpp"].reshape(-1))


def _pair_from(R, O, meshes, things, spheres):
    """Product scene (SAH) and oracle world from (vces, ices) meshes,
    (mesh index, transform) things and (centre, radius) analytic spheres."""
    sc, wd = R.Scene(), O.World()
    opt = (0, (0.6, 0.5, 0.4), 0.0, 0.0)
    ro = R.optics(opt[0], opt[1], opt[2], opt[3])
    mids, oids = [], []
    for v, i in meshes:
        mids.append(sc.add_mesh(v, i))
        oids.append(wd.add_mesh(np.ascontiguousarray(v, np.float32), np.ascontiguousarray(i, np.uint32)))
    for m, T in things:
        T = np.asarray(T, np.float32)
        sc.add_thing(ro, mids[m], T)
        wd.add_thing(opt[0], np.asarray(opt[1], np.float32), opt[2], opt[3], oids[m], T)
    for c, r in spheres:
        sc.add_analytic_sphere(c, r, ro)
        wd.add_sphere(opt[0], np.asarray(opt[1], np.float32), opt[2], opt[3], np.asarray(c, np.float32), float(r))
    sc.build(layout=R.RT_LAYOUT_SAH)
    wd.build(60)
    return sc, wd


def _first_hits_match(R, O, cuda, sc, wd, cam, w, h):
    g = device_first_hit(R, cuda, sc, cam, R.launch_params(w, h, 1, seed=21))
    c = wd.first_hit(oracle_camera(O, cam), w, h, 21)
    assert np.array_equal(g["prim"], c["prim"]) and np.array_equal(g["thing"], c["thing"])
    assert np.array_equal(g["t"].view(np.uint32), c["t"].view(np.uint32))
    return g


def test_sah_identical_centroids(product, oracle, cuda):
    """6000 copies of one triangle (one centroid: no border separates them,
    every split is a median split) beside a small sphere mesh."""
    R, O = product, oracle
    tri_v = np.array([[-1, 0, -1], [1, 0, -1], [0, 0, 1]], np.float32)
    tri_i = np.array([[0, 1, 2]] * 6000, np.uint32)
    sv, si = O.tessellate(1.0, 3)
    ident = [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0]
    sc, wd = _pair_from(R, O, [(tri_v, tri_i), (sv, si)], [(0, ident), (1, [0.5, 0, 0, 2, 0, 0.5, 0, 0.6, 0, 0, 0.5, 0])],
                        [])
    assert sc.info().layout == R.RT_LAYOUT_SAH
    _check_tree(sc.lbvh(), wd.triangles())
    cam = R.camera_set((0, 3, 6), (0.5, 0, 0), (0, 1, 0), 40, 1.5, 0.0, 6.0)
    g = _first_hits_match(R, O, cuda, sc, wd, cam, 96, 64)
    assert (g["prim"] >= 0).sum() > 0 and (g["prim"] == 5999).any()   # equal t: the larger id wins


def test_sah_exponential_spacing_hits_level_cap(product, oracle, cuda, sah_cluster):
    """Spheres at x = 1.25^k: binned SAH peels them off one or a few per
    level, past the level cap (64), where the median split takes over."""
    R, O = product, oracle
    sah_cluster(2)
    spheres = [((float(1.25 ** k), 0.0, 0.0), 0.1) for k in range(300)]
    sc, wd = _pair_from(R, O, [], [], spheres)
    t = sc.lbvh()
    n = len(t["ids"])
    assert n == 300 and np.array_equal(np.sort(t["ids"]), np.arange(n, dtype=np.uint32))
    kids = np.concatenate([t["left"], t["right"]])
    assert np.array_equal(np.sort(~kids[kids < 0]), np.arange(n))
    cam = R.camera_set((0.3, 0.0, 40.0), (0.3, 0.0, 0.0), (0, 1, 0), 30, 1.5, 0.0, 40.0)
    _first_hits_match(R, O, cuda, sc, wd, cam, 120, 80)


def test_sah_update_refits_and_rebuilds(product, oracle, cuda):
    """Transform edits under the SAH layout: the refit keeps the tree and the
    hits follow the oracle's rebuilt world."""
    R, O = product, oracle
    sc, wd = rtow_pair(R, O, 2, layout=R.RT_LAYOUT_SAH)
    for tid in (3, 40, 100):
        st, T = sc.get_transform(tid)
        T = T.copy()
        T[3] += 0.4
        T[11] -= 0.3
        assert sc.set_transform(tid, T) == R.RT_OK
        assert wd.set_transform(tid, T) == 0
    sc.update()
    wd.build()
    _check_tree(sc.lbvh(), wd.triangles())
    cam = R.rtow_camera(160, 96)
    _first_hits_match(R, O, cuda, sc, wd, cam, 160, 96)


@pytest.mark.parametrize("level", [None, 2, 3])
@pytest.mark.parametrize("cluster", [1, 16, 2048])
def test_sah_bit_exact_vs_oracle_twin(product, oracle, cuda, sah_cluster, level, cluster):
    """The GPU's binned-SAH hierarchy equals the oracle's restatement node for
    node: cluster-local keys, record order, children and refit boxes."""
    R, O = product, oracle
    sah_cluster(cluster)
    sc = R.rtow_scene(level, layout=R.RT_LAYOUT_SAH)
    wd, _ = O.rtow_world(level, sah_cluster=cluster)
    a, b = sc.lbvh(), wd.lbvh()
    for k in ("codes", "ids", "left", "right"):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(a["boxes"].view(np.uint32), b["boxes"].view(np.uint32))
