"""CPU: which hit the hierarchy returns when a binary32 root leaves its box.

The slab test keeps a box while a hit inside it is in range, and every
ancestor box holds a record's own box, so the closest hit a hierarchy returns
is the closest over the records whose own box passes the test -- whatever the
hierarchy.  For triangles that is brute force (tested on the GPU against all
primitives).  A binary32 sphere root can lie outside the sphere's box: rays
leaving the r = 1000 ground sphere from 4e-5 inside it (the hit points of a
path of the final scene as spheres, 256x256 at 64 spp) get the exit root
1.04e-3, above the box's top at y = 0, while the exact exit (6.9e-4) is below
t_min.  Brute force takes that root; the hierarchy, like the product, does not.
Checked here on the oracle (the product's images equal it bit for bit): the
three recorded rays, 60,000 rays from sphere surfaces, nudged in and out, and
20,000 rays leaving the ground sphere slowly from just inside its top, against
the flat LBVH and the binned-SAH hierarchy.
"""
import numpy as np
import pytest

# rays of the final scene as spheres (glibc seed 1) whose brute-force hit is
# the ground sphere's exit root above its box
ARTEFACT_RAYS = [
    ((0.157554626, -4.0769577e-05, 0.128160715), (0.335184008, 0.0587934256, 0.0435726643)),
    ((0.143372715, -3.66047025e-05, 0.169463813), (0.0619876646, 0.0381976366, -0.26649791)),
    ((0.154655874, -4.05088067e-05, -0.151826531), (-0.0526962429, 0.0491584539, 0.304982752)),
]


@pytest.fixture(scope="module")
def worlds(oracle):
    flat, sc = oracle.rtow_world(None, 0, 1, 11)
    sah, _ = oracle.rtow_world(None, 0, 1, 11, sah_cluster=16)
    return flat, sah, sc


def _rays(sc, n, seed):
    rng = np.random.default_rng(seed)
    c = np.asarray(sc["centers"], np.float32)
    r = np.asarray(sc["radii"], np.float32)
    k = rng.integers(0, len(r), n)
    k[: n // 3] = 0   # a third from the ground sphere (thing 0), near its top
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    top = np.zeros(n, bool)
    top[: n // 3] = True
    xz = rng.uniform(-11, 11, size=(n, 2))
    u[top] = np.stack([xz[top, 0] / 1000.0, np.sqrt(1 - (xz[top] ** 2).sum(1) / 1e6), xz[top, 1] / 1000.0], 1)
    nudge = rng.choice([-1e-4, -4e-5, -1e-5, 0.0, 1e-5, 1e-4], n)
    o = (c[k] + (r[k, None] * (1.0 + nudge[:, None] / np.maximum(r[k, None], 1e-3))) * u).astype(np.float32)
    d = rng.normal(size=(n, 3))
    up = rng.random(n) < 0.5
    d[up, 1] = np.abs(d[up, 1])   # half the rays leave upwards
    z = rng.random(n) < 0.1
    d[z, rng.integers(0, 3, z.sum())] = 0.0   # some with a zero component
    return o, d.astype(np.float32)


def test_recorded_rays_brute_force_takes_the_root_above_the_box(worlds):
    flat, sah, _ = worlds
    o = np.array([a for a, _ in ARTEFACT_RAYS], np.float32)
    d = np.array([b for _, b in ARTEFACT_RAYS], np.float32)
    pb, tb = flat.closest(o, d, "brute")
    assert np.all(pb == 0)                                    # the ground sphere
    assert np.all(o[:, 1] + tb * d[:, 1] > 0.0)               # the root's point is above the box's top (y = 0)
    for w in (flat, sah):
        ph, th = w.closest(o, d, "bvh")
        pr, tr = w.closest(o, d, "boxed")
        assert np.all(ph != 0) and np.array_equal(ph, pr)
        assert np.array_equal(th.view(np.uint32), tr.view(np.uint32))


def _ground_exits(n, seed):
    """Rays leaving the ground sphere (centre (0, -1000, 0), r = 1000) from
    just inside its top, slowly upwards: the exact exit distance straddles
    t_min, where the binary32 root can land above the box."""
    rng = np.random.default_rng(seed)
    xz = rng.uniform(-3, 3, size=(n, 2))
    depth = rng.uniform(1e-5, 8e-5, n)
    y = np.sqrt(1e6 - (xz ** 2).sum(1)) - 1000.0 - depth
    o = np.stack([xz[:, 0], y, xz[:, 1]], 1).astype(np.float32)
    a = rng.uniform(0, 2 * np.pi, n)
    d = np.stack([0.3 * np.cos(a), rng.uniform(0.01, 0.08, n), 0.3 * np.sin(a)], 1).astype(np.float32)
    return o, d


def test_hierarchy_returns_closest_over_records_whose_box_passes(worlds):
    flat, sah, sc = worlds
    o1, d1 = _rays(sc, 60000, 5)
    o2, d2 = _ground_exits(20000, 6)
    o, d = np.concatenate([o1, o2]), np.concatenate([d1, d2])
    pr, tr = flat.closest(o, d, "boxed")
    pb, tb = flat.closest(o, d, "brute")
    for w in (flat, sah):
        ph, th = w.closest(o, d, "bvh")
        assert np.array_equal(ph, pr)
        assert np.array_equal(th.view(np.uint32), tr.view(np.uint32))
    differ = pb != pr
    print(f"brute force differs from the box rule on {int(differ.sum())} of {len(o)} rays")
    assert 0 < differ.sum() < len(o) // 100
    # every difference is the ground sphere's root above its box
    assert np.all(pb[differ] == 0) and np.all(o[differ, 1] + tb[differ] * d[differ, 1] > 0.0)


def test_triangles_hierarchy_equals_brute_force(oracle):
    """The final scene tessellated (level 2): rays leaving random points of the
    triangles, some with a zero direction component -- the flat LBVH and the
    binned-SAH hierarchy return brute force's closest hit, bit for bit."""
    rng = np.random.default_rng(3)
    for cluster in (0, 16):
        wd, _ = oracle.rtow_world(2, 0, 1, 11, sah_cluster=cluster)
        tri = wd.triangles().reshape(-1, 3, 3).astype(np.float64)
        n = 30000
        k = rng.integers(0, len(tri), n)
        u, v = rng.random(n), rng.random(n)
        flip = u + v > 1
        u[flip], v[flip] = 1 - u[flip], 1 - v[flip]
        o = (tri[k, 0] + u[:, None] * (tri[k, 1] - tri[k, 0]) + v[:, None] * (tri[k, 2] - tri[k, 0])).astype(np.float32)
        d = rng.normal(size=(n, 3)).astype(np.float32)
        z = rng.random(n) < 0.1
        d[z, rng.integers(0, 3, z.sum())] = 0.0
        pb, tb = wd.closest(o, d, "brute")
        ph, th = wd.closest(o, d, "bvh")
        assert np.array_equal(ph, pb)
        assert np.array_equal(th.view(np.uint32), tb.view(np.uint32))
