"""GPU: randomized scenes against the oracle, every layout.

Each case draws a scene of random meshes (random triangles, some degenerate,
some duplicated), analytic spheres and transforms (rotations, mirrors, tiny
and large scales), a random layout and binned-SAH cluster size, and renders
a small image; colours and rays per pixel must equal the oracle's bit for
bit, and a flattened layout's hierarchy must be a valid tree.
"""
import numpy as np
import pytest

from _helpers import oracle_camera

pytestmark = pytest.mark.gpu


def _rot(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]], np.float32)


def _scene(R, O, rng, layout):
    sc, wd = R.Scene(), O.World()
    meshes = []
    for _ in range(int(rng.integers(1, 4))):
        nv = int(rng.integers(3, 40))
        v = rng.uniform(-1, 1, (nv, 3)).astype(np.float32)
        nt = int(rng.integers(1, 300))
        i = rng.integers(0, nv, (nt, 3)).astype(np.uint32)
        if rng.random() < 0.3:
            i[: nt // 2] = i[0]          # duplicates of one triangle
        meshes.append((sc.add_mesh(v, i), wd.add_mesh(v, i)))
    if rng.random() < 0.5:
        v, i = O.tessellate(1.0, int(rng.integers(0, 4)))
        meshes.append((sc.add_mesh(v, i), wd.add_mesh(v, i)))
    for _ in range(int(rng.integers(1, 25))):
        typ = int(rng.integers(0, 3))
        alb = tuple(float(x) for x in rng.uniform(0.1, 0.95, 3))
        fuzz = float(rng.uniform(0, 0.5)) if typ == 1 else 0.0
        idx = 1.5 if typ == 2 else 0.0
        o = R.optics(typ, alb, fuzz, idx)
        pos = rng.uniform(-4, 4, 3).astype(np.float32)
        if rng.random() < 0.3:
            r = float(10 ** rng.uniform(-2, 0.5))
            sc.add_analytic_sphere(tuple(float(x) for x in pos), r, o)
            wd.add_sphere(typ, np.asarray(alb, np.float32), fuzz, idx, pos, r)
            continue
        s = float(10 ** rng.uniform(-1.5, 0.7))
        if rng.random() < 0.5:
            M = np.diag(rng.choice([-1, 1], 3) * s).astype(np.float32)   # diagonal, may mirror
        else:
            M = (_rot(rng) * s).astype(np.float32)
        T = np.concatenate([M, pos[:, None]], axis=1).astype(np.float32).reshape(-1)
        m = meshes[int(rng.integers(0, len(meshes)))]
        sc.add_thing(o, m[0], T)
        wd.add_thing(typ, np.asarray(alb, np.float32), fuzz, idx, m[1], T)
    sc.build(layout=layout)
    wd.build(60)
    return sc, wd


@pytest.mark.parametrize("case", range(64))
def test_random_scene_matches_oracle(product, oracle, cuda, monkeypatch, case):
    R, O = product, oracle
    rng = np.random.default_rng(1000 + case)
    layout = [R.RT_LAYOUT_FLAT, R.RT_LAYOUT_GROUPED, R.RT_LAYOUT_SAH, R.RT_LAYOUT_INSTANCED][case % 4]
    monkeypatch.setenv("RTX_SAH_CLUSTER", str(int(rng.choice([1, 2, 5, 16, 64, 1000]))))
    sc, wd = _scene(R, O, rng, layout)
    w, h, spp, depth = 40, 30, 2, 8
    eye = tuple(float(x) for x in rng.uniform(-9, 9, 3))
    cam = R.camera_set(eye, (0, 0, 0), (0, 1, 0), float(rng.uniform(20, 70)), w / h, float(rng.uniform(0, 0.2)), 8.0)
    params = R.launch_params(w, h, spp, depth=depth, seed=case)
    out = R.render(sc, cam, params)
    ref = wd.render(oracle_camera(O, cam), w, h, spp, depth, case, guides=False)
    assert np.array_equal(out["rawRGB"].view(np.uint32), ref["rawRGB"].view(np.uint32))
    assert np.array_equal(out["rpp"], ref["rpp"])
    if layout != R.RT_LAYOUT_INSTANCED and sc.info().n_top_records > 1:
        t = sc.lbvh()
        n = len(t["ids"])
        kids = np.concatenate([t["left"], t["right"]])
        assert np.array_equal(np.sort(~kids[kids < 0]), np.arange(n))
        assert len(np.unique(kids[kids >= 0])) == n - 2
