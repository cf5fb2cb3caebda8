"""GPU parity at the benchmark size: the final scene with every sphere
tessellated 6 times (487 x 16384 = 7,979,008 triangles), 1200x800.

All first-hit ids of the full image are compared bit for bit with the CPU
oracle (its own LBVH twin); the render is compared bit for bit on a pixel
subset and through size-independent properties on the whole frame.
"""
import numpy as np
import pytest

from _helpers import device_first_hit, oracle_camera

pytestmark = pytest.mark.gpu

W, H = 1200, 800


@pytest.fixture(scope="module")
def c1(product, oracle):
    sc = product.rtow_scene(6)
    wd, _ = oracle.rtow_world(6)
    return sc, wd


def test_c1_triangle_count(c1):
    sc, wd = c1
    assert sc.info().n_prims == 7979008 == wd.nprims


def test_c1_first_hit_ids_bit_exact(product, oracle, cuda, c1):
    R, O = product, oracle
    sc, wd = c1
    cam = R.rtow_camera(W, H)
    params = R.launch_params(W, H, 1, seed=4711)
    g = device_first_hit(R, cuda, sc, cam, params)
    c = wd.first_hit(oracle_camera(O, cam), W, H, 4711, fp64=True)
    assert np.array_equal(g["prim"], c["prim"])
    assert np.array_equal(g["thing"], c["thing"])
    assert np.array_equal(g["t"].view(np.uint32), c["t"].view(np.uint32))
    hit = g["prim"] >= 0
    rel64 = np.abs(g["t64"][hit] - c["t64"][hit]) / c["t64"][hit]
    assert rel64.max() <= 1e-5, rel64.max()
    rel32 = np.abs(g["t"][hit].astype(np.float64) - c["t64"][hit]) / c["t64"][hit]
    assert np.mean(rel32 <= 1e-5) >= 0.999, np.mean(rel32 <= 1e-5)


def test_c1_lbvh_60bit_matches_twin(c1):
    sc, wd = c1
    a, b = sc.lbvh(), wd.lbvh()
    for k in ("codes", "ids", "left", "right"):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(a["boxes"].view(np.uint32), b["boxes"].view(np.uint32))


def test_c1_render_subset_bit_exact_and_properties(product, oracle, cuda, c1):
    R, O = product, oracle
    sc, wd = c1
    spp = 64
    cam = R.rtow_camera(W, H)
    params = R.launch_params(W, H, spp, depth=50, seed=4711)
    out = R.render(sc, cam, params)
    raw, rpp = out["rawRGB"], out["rpp"]
    # size-independent properties of the whole frame
    assert int(rpp.sum(dtype=np.uint64)) == int(out["stats"].rays)
    assert rpp.min() >= spp and rpp.max() <= spp * 50
    assert np.isfinite(raw).all() and raw.min() >= 0.0 and raw.max() <= 1.0
    # bit-exact on a strided pixel subset
    pix = np.arange(0, W * H, 4999, dtype=np.uint32)
    ref = wd.render(oracle_camera(O, cam), W, H, spp, 50, 4711, pixels=pix, guides=False)
    assert np.array_equal(raw[pix].view(np.uint32), ref["rawRGB"].view(np.uint32))
    assert np.array_equal(rpp[pix], ref["rpp"])
