"""CPU: the oracle pinned against the reference's own outputs and published KATs."""
import json
import os

import numpy as np
import pytest

from _helpers import GOLDEN, golden_scene, golden_sphere, mesh_hash, sphere_hashes


def test_philox_known_answer_vectors(oracle):
    # Philox4x32-10 KAT (Salmon et al., SC'11)
    kat = [
        ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
        ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
        ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
         (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
    ]
    for ctr, key, want in kat:
        assert tuple(int(x) for x in oracle.philox(ctr, key)) == want


def test_u01_is_24_bit_exact(oracle):
    for x in (0, 255, 256, 0xFFFFFFFF, 0x80000000):
        assert oracle.lib().orc_u01(x) == np.float32((x >> 8) / 16777216.0)
    assert oracle.lib().orc_u01(0xFFFFFFFF) < 1.0


def test_glibc_rand_restatement(oracle):
    with open(os.path.join(GOLDEN, "glibc_rand.json")) as f:
        gold = json.load(f)
    for seed, seq in gold.items():
        assert np.array_equal(oracle.glibc_rand(int(seed), len(seq)), np.array(seq, np.int32))


@pytest.mark.parametrize("seed", [1, 7])
def test_scene_recipe_matches_reference_scene(oracle, seed):
    g = golden_scene(seed)
    s = oracle.scene_rtow(0, seed, 11)
    assert len(s["radii"]) == len(g)
    assert np.array_equal(s["types"], g[:, 0].astype(np.int32))
    assert np.array_equal(s["centers"], g[:, 1:4].astype(np.float32))
    assert np.array_equal(s["radii"], g[:, 4].astype(np.float32))
    assert np.array_equal(s["albedos"], g[:, 5:8].astype(np.float32))
    assert np.array_equal(s["fuzz"], g[:, 8].astype(np.float32))
    assert np.array_equal(s["index"], g[:, 9].astype(np.float32))


def test_final_scene_composition(oracle):
    s = oracle.scene_rtow(0, 1, 11)
    assert len(s["radii"]) == 487
    assert np.bincount(s["types"]).tolist() == [394, 64, 29]


@pytest.mark.parametrize("n", [0, 1, 2, 3, 4])
def test_tessellator_bit_exact(oracle, n):
    v, i = oracle.tessellate(1.0, n)
    gv, gi = golden_sphere(n)
    assert np.array_equal(v.view(np.uint32), gv.view(np.uint32))
    assert np.array_equal(i, gi)


@pytest.mark.parametrize("key", sorted(sphere_hashes()))
def test_tessellator_hashes(oracle, key):
    g = sphere_hashes()[key]
    v, i = oracle.tessellate(g["radius"], g["ndiv"])
    assert (len(v), len(i)) == (g["nv"], g["ni"])
    assert mesh_hash(v, i) == (g["vces_sha256"], g["ices_sha256"])


def test_stable_sort_and_karras_topology(oracle):
    rng = np.random.default_rng(0)
    keys = rng.integers(0, 64, 5000).astype(np.uint64)
    k, v = oracle.stable_sort_pairs(keys, np.arange(5000, dtype=np.uint32))
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(k, keys[order]) and np.array_equal(v, order)
    left, right = oracle.karras(k)
    kids = np.concatenate([left, right])
    assert sorted((~kids[kids < 0]).tolist()) == list(range(5000))
    assert sorted(kids[kids >= 0].tolist()) == list(range(1, 4999))


@pytest.mark.parametrize("bits", [30, 60])
@pytest.mark.parametrize("level", [None, 1])
def test_lbvh_closest_hit_equals_brute_force(oracle, bits, level):
    w, _ = oracle.rtow_world(level, half_extent=5, morton_bits=bits)
    cam = oracle.rtow_camera(80, 45)
    a = w.first_hit(cam, 80, 45, 4711, use_bvh=True)
    b = w.first_hit(cam, 80, 45, 4711, use_bvh=False)
    assert np.array_equal(a["prim"], b["prim"])
    assert np.array_equal(a["t"].view(np.uint32), b["t"].view(np.uint32))


def test_render_is_deterministic_and_thread_count_free(oracle):
    w, _ = oracle.rtow_world(None, half_extent=4)
    cam = oracle.rtow_camera(32, 18)
    a = w.render(cam, 32, 18, 3, 50, 1, nthreads=1)
    b = w.render(cam, 32, 18, 3, 50, 1, nthreads=4)
    assert np.array_equal(a["rawRGB"], b["rawRGB"]) and np.array_equal(a["rpp"], b["rpp"])
    assert a["rays"] == int(a["rpp"].sum())


def test_depth_one_is_sky_or_black(oracle):
    w, _ = oracle.rtow_world(None, half_extent=3)
    cam = oracle.rtow_camera(24, 16)
    r = w.render(cam, 24, 16, 1, 1, 1)
    hits = w.first_hit(cam, 24, 16, 1)
    black = (r["rawRGB"] == 0).all(axis=1)
    assert np.array_equal(black, hits["prim"] >= 0)
    assert (r["rpp"] == 1).all()


def test_analytic_render_sanity(oracle):
    """The final scene under a blue sky: blue dominates the mean colour."""
    w, _ = oracle.rtow_world(None)
    cam = oracle.rtow_camera(64, 36)
    r = w.render(cam, 64, 36, 16, 50, 4711)
    mean = r["rawRGB"].mean(axis=0)
    assert 0.3 < mean[2] < 0.9 and mean[2] > mean[0]   # blue-ish sky dominates, as in rtow
