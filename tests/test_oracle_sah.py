"""CPU: the oracle's binned-SAH twin (the GPU layout's restatement).

A binary tree over every record exactly once, child boxes the exact unions
below them, and closest hits equal to brute force over all records (the
slab test is conservative, so no tree changes a hit).
"""
import numpy as np
import pytest


@pytest.mark.parametrize("cluster", [1, 4, 16, 5000])
def test_oracle_sah_tree_and_hits(oracle, cluster):
    O = oracle
    w, _ = O.rtow_world(2, half_extent=4, sah_cluster=cluster)
    t = w.lbvh()
    n = len(t["ids"])
    assert np.array_equal(np.sort(t["ids"]), np.arange(n, dtype=np.uint32))
    kids = np.concatenate([t["left"], t["right"]])
    assert np.array_equal(np.sort(~kids[kids < 0]), np.arange(n))
    internal = kids[kids >= 0]
    assert len(np.unique(internal)) == len(internal) == n - 2
    tb = w.triangles().reshape(-1, 3, 3)
    plo, phi = tb.min(axis=1), tb.max(axis=1)
    boxes = t["boxes"]
    for k, ch in enumerate((t["left"], t["right"])):
        leaf = ch < 0
        rec = t["ids"][~ch[leaf]]
        assert np.array_equal(boxes[leaf, 6 * k:6 * k + 3], plo[rec])
        assert np.array_equal(boxes[leaf, 6 * k + 3:6 * k + 6], phi[rec])
    cam = O.rtow_camera(64, 40)
    a = w.first_hit(cam, 64, 40, 5, use_bvh=True)
    b = w.first_hit(cam, 64, 40, 5, use_bvh=False)
    assert np.array_equal(a["prim"], b["prim"]) and np.array_equal(a["t"].view(np.uint32), b["t"].view(np.uint32))
