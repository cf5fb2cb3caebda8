"""CPU: the FP64 adjoint of the oracle against finite differences.

Albedo and sky gradients are checked against central differences of whole
renders with common random numbers (paths do not change with these
parameters, so the loss is a polynomial in them).  Fuzz moves directions,
so whole-image differences pick up visibility changes that a replayed
path's derivative does not contain; its derivative is checked per path,
against the central difference of the same path wherever the perturbed paths
keep every hit primitive and branch.
"""
import numpy as np
import pytest

AMB = (0.5, 0.7, 0.95)     # sky colours below 1: no pixel sits on the clamp at 1
WHT = (0.97, 0.98, 0.96)


def _setup(oracle, level, W=20, H=20, spp=6, depth=8, seed=5):
    w, _ = oracle.rtow_world(level, half_extent=3)
    cam = oracle.rtow_camera(W, H)
    I0 = w.render(cam, W, H, spp, depth, seed, ambient=AMB, white=WHT, guides=False)["rawRGB"]
    T = np.clip(I0 + np.random.default_rng(1).normal(0, 0.05, I0.shape).astype(np.float32), 0, 1)
    return w, cam, T, (W, H, spp, depth, seed)


def _loss(w, cam, T, cfg, amb=AMB, wht=WHT):
    W, H, spp, depth, seed = cfg
    I = w.render(cam, W, H, spp, depth, seed, ambient=amb, white=wht, guides=False)["rawRGB"]
    return float(((I.astype(np.float64) - T) ** 2).sum()), I


@pytest.mark.parametrize("level", [None, 2])
def test_albedo_and_sky_gradients_match_finite_differences(oracle, level):
    w, cam, T, cfg = _setup(oracle, level)
    W, H, spp, depth, seed = cfg
    L0, I = _loss(w, cam, T, cfg)
    g = w.adjoint(cam, W, H, spp, depth, seed, I, 2.0 * (I.astype(np.float64) - T), ambient=AMB, white=WHT)
    opt = w.optics()
    h = 1e-3
    checked = 0
    for k in np.argsort(-np.abs(g["albedo"]).sum(1))[:5]:
        if opt["types"][k] == 2:
            continue
        for ch in range(3):
            a = opt["albedos"][k].copy()
            vals = []
            for s in (+h, -h):
                a1 = a.copy()
                a1[ch] += s
                w.set_optics(int(k), int(opt["types"][k]), a1, float(opt["fuzz"][k]), float(opt["index"][k]))
                vals.append(_loss(w, cam, T, cfg)[0])
            w.set_optics(int(k), int(opt["types"][k]), a, float(opt["fuzz"][k]), float(opt["index"][k]))
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(g["albedo"][k, ch] - fd) <= 2e-3 * max(abs(fd), 1e-2), (k, ch, g["albedo"][k, ch], fd)
            checked += 1
    assert checked >= 6
    for j in range(6):
        def L_at(s):
            amb, wht = list(AMB), list(WHT)
            (amb if j < 3 else wht)[j % 3] += s
            return _loss(w, cam, T, cfg, tuple(amb), tuple(wht))[0]
        fd = (L_at(h) - L_at(-h)) / (2 * h)
        assert abs(g["sky"][j] - fd) <= 2e-3 * max(abs(fd), 1e-2), (j, g["sky"][j], fd)


@pytest.mark.parametrize("level", [2, 4])
def test_fuzz_derivative_per_path(oracle, level):
    w, _ = oracle.rtow_world(level, half_extent=3)
    cam = oracle.rtow_camera(32, 32)
    opt = w.optics()
    metals = [k for k in range(w.nthings) if opt["types"][k] == 1]
    total = 0
    for k in metals:
        r = w.fuzz_path_check(cam, 32, 32, 8, 8, 5, k, 1e-3, ambient=AMB, white=WHT)
        if r["compared"] == 0:
            continue
        total += r["compared"]
        assert r["outliers"] == 0, (k, r)
        assert abs(r["sum_adj"] - r["sum_fd"]) <= 2e-3 * max(r["sum_abs_fd"], 1e-3), (k, r)
    assert total > 500


def test_fuzz_gradient_at_image_level_with_visibility_held(oracle):
    """The fuzz tangent against an image-level central difference of the loss
    over double-precision replays that keep every path's primitives and
    branches (the derivative the adjoint forms), final scene as analytic
    spheres at 64x64, 16 spp: the eight metals with the largest gradients."""
    w, _ = oracle.rtow_world(None)
    W = H = 64
    spp, depth, seed = 16, 8, 21
    cam = oracle.rtow_camera(W, H)
    I = w.render(cam, W, H, spp, depth, seed, ambient=AMB, white=WHT, guides=False)["rawRGB"]
    T = np.clip(I + np.random.default_rng(5).normal(0, 0.1, I.shape), 0, 1)
    G = (2.0 * (np.clip(I, 0, 1) - T)).astype(np.float32)
    g = w.adjoint(cam, W, H, spp, depth, seed, I, G, ambient=AMB, white=WHT)
    I64 = I.astype(np.float64)
    mask = (I64 > 0) & (I64 < 1)

    def loss(X):
        return float((((np.clip(X, 0, 1) - T) ** 2) * mask).sum())

    opt = w.optics()
    metals = np.where(opt["types"] == 1)[0]
    h = 1e-7
    for k in metals[np.argsort(-np.abs(g["fuzz"][metals]))][:8]:
        r = w.fuzz_held_delta(cam, W, H, spp, depth, seed, int(k), h, ambient=AMB, white=WHT, image=I, grad_image=G)
        fd = (loss(I64 + r["plus"]) - loss(I64 + r["minus"])) / (2 * h)
        assert r["replayed"] > 0
        assert abs(r["adjoint"] - fd) <= 1e-2 * max(abs(fd), 1e-3), (int(k), r["adjoint"], fd, r)
