"""GPU: the adjoint at the differentiable configuration itself.

The final scene as 488 analytic spheres (glibc seed 1), 256x256, 64 spp,
depth 8, the default sky; the target is the render with every albedo
perturbed by N(0, 0.1) and clamped to [0, 1]; the loss is the pixel L2 of the
clamped image.  Checked:

* the GPU's gradients of every albedo channel, every fuzz and the six sky
  values against the oracle's FP64 adjoint replaying the same paths;
* central finite differences of GPU renders with common random numbers
  (h = 1e-3) on 32 sampled parameters -- 26 albedo channels and the 6 sky
  values -- within 1e-2 relative.  This check renders with sky colours just
  below 1: the default sky's white is exactly 1, so the sky and its mirror
  images sit on the clamp at 1, where the loss has a kink that a central
  step straddles;
* the fuzz gradient at image level for the metals with the largest ones.  A
  whole-image difference of re-renders cannot check it: moving a fuzz moves
  reflected rays across silhouettes, so some paths change their hit
  sequence (the jumps a replay that holds visibility fixed leaves out by
  design), and near a silhouette the derivative of a hit point grows like
  1 / cos of the incidence angle.  The oracle instead replays every path that
  reflects off the metal in double precision along its recorded primitives
  and branches (visibility held fixed) at fuzz f0 and f0 +- h with h small
  enough to follow the steep near-silhouette paths (1e-7), and the image-level
  central difference of the loss is compared with the adjoint's tangent
  evaluated on the same trajectories.  With the GPU's gradients equal to the
  FP64 adjoint's (first check), this pins the GPU fuzz gradient to a
  derivative of images.
"""
import ctypes

import numpy as np
import pytest

from _helpers import dptr, oracle_camera

pytestmark = pytest.mark.gpu

W = H = 256
SPP, DEPTH, SEED = 64, 8, 4711


AMB_FD = (0.5, 0.7, 0.95)   # the finite-difference check's sky: no pixel on the clamp at 1
WHT_FD = (0.97, 0.98, 0.96)


def _setup(R, O, torch, amb=(0.5, 0.7, 1.0), wht=(1.0, 1.0, 1.0)):
    sp = R.rtow_spheres(R.RT_RECIPE_GLIBC, 1, 11)
    sc = R.rtow_scene(None, R.RT_RECIPE_GLIBC, 1, 11)
    n = sc.info().n_things
    cam = R.rtow_camera(W, H)
    params = R.launch_params(W, H, SPP, depth=DEPTH, seed=SEED, ambient=amb, white=wht)

    def set_albedo(alb):
        for k in range(n):
            sc.set_optics(k, R.optics(int(sp["types"][k]), tuple(float(x) for x in alb[k]), float(sp["fuzz"][k]),
                                      float(sp["index"][k])))

    def render():
        raw = torch.zeros(W * H * 3, dtype=torch.float32, device="cuda")
        rpp = torch.zeros(W * H, dtype=torch.int32, device="cuda")
        R.check(R.lib().rt_launch(sc.h, ctypes.byref(cam), ctypes.byref(params),
                                  ctypes.byref(R.Frame(dptr(raw), dptr(rpp), None, None)), None))
        torch.cuda.synchronize()
        return raw

    rng = np.random.default_rng(11)
    set_albedo(np.clip(sp["albedos"] + rng.normal(0, 0.1, sp["albedos"].shape), 0, 1))
    target = render().view(-1, 3).clamp(0, 1)
    set_albedo(sp["albedos"])
    img = render()
    grad_img = (2.0 * (img.view(-1, 3).clamp(0, 1) - target)).reshape(-1).contiguous()
    ga = torch.zeros(n * 3, dtype=torch.float64, device="cuda")
    gf = torch.zeros(n, dtype=torch.float64, device="cuda")
    gs = torch.zeros(6, dtype=torch.float64, device="cuda")
    sc.adjoint(cam, params, dptr(img), dptr(grad_img), dptr(ga), dptr(gf), dptr(gs))
    torch.cuda.synchronize()
    return dict(sp=sp, sc=sc, n=n, cam=cam, ocam=oracle_camera(O, cam), set_albedo=set_albedo, render=render,
                target=target, img=img.cpu().numpy().reshape(-1, 3), grad_img=grad_img.cpu().numpy().reshape(-1, 3),
                albedo=ga.cpu().numpy().reshape(n, 3), fuzz=gf.cpu().numpy(), sky=gs.cpu().numpy())


@pytest.fixture(scope="module")
def c3(product, oracle, cuda):
    d = _setup(product, oracle, cuda)
    d["wd"], _ = oracle.rtow_world(None, 0, 1, 11)
    return d


def _close(a, b, rel):
    scale = max(np.abs(b).max(), 1e-30)
    err = np.abs(a - b).max()
    assert err <= rel * scale, (err, scale)
    return err / scale


def test_c3_image_equals_oracle(c3):
    ref = c3["wd"].render(c3["ocam"], W, H, SPP, DEPTH, SEED, guides=False)
    assert np.array_equal(c3["img"].view(np.uint32), ref["rawRGB"].view(np.uint32))


def test_c3_adjoint_matches_fp64_oracle(c3):
    """All 488 x 3 albedo, 488 fuzz and 6 sky gradients against the FP64 adjoint
    of the same paths (binary32 terms on the GPU: 1e-5 of the largest; the
    binary32 fuzz tangent with two double steps: 2e-4)."""
    ref = c3["wd"].adjoint(c3["ocam"], W, H, SPP, DEPTH, SEED, c3["img"], c3["grad_img"])
    e_a = _close(c3["albedo"], ref["albedo"], 1e-5)
    e_s = _close(c3["sky"], ref["sky"], 1e-5)
    e_f = _close(c3["fuzz"], ref["fuzz"], 2e-4)
    print(f"C3 GPU vs FP64 adjoint: albedo {e_a:.2e}, sky {e_s:.2e}, fuzz {e_f:.2e} of the largest")
    types = c3["sp"]["types"]
    assert np.all(c3["albedo"][types == 2] == 0) and np.all(c3["fuzz"][types != 1] == 0)
    assert np.count_nonzero(c3["fuzz"]) >= 32


def test_c3_albedo_and_sky_against_finite_differences(product, oracle, cuda):
    """26 albedo channels (largest gradients first, channels within 10 h of 0
    left out: a central step there crosses the clamp at 0) and the 6 sky
    values, central differences of GPU renders with common random numbers."""
    R, torch = product, cuda
    c3 = _setup(R, oracle, torch, AMB_FD, WHT_FD)
    sp, sc, n = c3["sp"], c3["sc"], c3["n"]
    h = 1e-3
    target = c3["target"]

    def loss(alb=None, amb=AMB_FD, wht=WHT_FD):
        if alb is not None:
            c3["set_albedo"](alb)
        params = R.launch_params(W, H, SPP, depth=DEPTH, seed=SEED, ambient=amb, white=wht)
        raw = torch.zeros(W * H * 3, dtype=torch.float32, device="cuda")
        rpp = torch.zeros(W * H, dtype=torch.int32, device="cuda")
        R.check(R.lib().rt_launch(sc.h, ctypes.byref(c3["cam"]), ctypes.byref(params),
                                  ctypes.byref(R.Frame(dptr(raw), dptr(rpp), None, None)), None))
        v = float(((raw.view(-1, 3).clamp(0, 1) - target).double() ** 2).sum())
        if alb is not None:
            c3["set_albedo"](sp["albedos"])
        return v

    ga, gs = c3["albedo"], c3["sky"]
    order = np.argsort(-np.abs(ga).max(1))
    cand = [(int(k), c) for k in order[:60] if sp["types"][k] != 2 for c in range(3)
            if sp["albedos"][k, c] > 10 * h]
    worst = 0.0
    for k, c in cand[:26]:
        vals = []
        for sgn in (1, -1):
            a1 = np.array(sp["albedos"], np.float64)
            a1[k, c] += sgn * h
            vals.append(loss(a1))
        fd = (vals[0] - vals[1]) / (2 * h)
        rel = abs(ga[k, c] - fd) / max(abs(fd), 1e-2)
        worst = max(worst, rel)
        assert rel <= 1e-2, (k, c, ga[k, c], fd)
    base = list(AMB_FD) + list(WHT_FD)
    for j in range(6):
        vals = []
        for sgn in (1, -1):
            s = list(base)
            s[j] += sgn * h
            vals.append(loss(None, tuple(s[:3]), tuple(s[3:])))
        fd = (vals[0] - vals[1]) / (2 * h)
        rel = abs(gs[j] - fd) / max(abs(fd), 1e-2)
        worst = max(worst, rel)
        assert rel <= 1e-2, (j, gs[j], fd)
    print(f"C3 finite differences, 32 parameters: worst relative error {worst:.2e}")


def test_c3_fuzz_at_image_level(c3):
    """The six metals with the largest fuzz gradients: image-level central
    difference (h = 1e-7) of the loss over double-precision replays that hold
    every path's visibility fixed, against the adjoint's tangent on the same
    trajectories, within 1e-2 relative."""
    wd, fuzz = c3["wd"], c3["fuzz"]
    types = c3["sp"]["types"]
    I = c3["img"].astype(np.float64)
    T = c3["target"].cpu().numpy().astype(np.float64)
    mask = (I > 0) & (I < 1)

    def loss(X):
        return float((((np.clip(X, 0, 1) - T) ** 2) * mask).sum())

    metals = np.where(types == 1)[0]
    top = metals[np.argsort(-np.abs(fuzz[metals]))][:6]
    h = 1e-7
    rows = []
    for k in top:
        r = wd.fuzz_held_delta(c3["ocam"], W, H, SPP, DEPTH, SEED, int(k), h, image=c3["img"],
                               grad_image=c3["grad_img"])
        fd = (loss(I + r["plus"]) - loss(I + r["minus"])) / (2 * h)
        rel = abs(r["adjoint"] - fd) / max(abs(fd), 1e-3)
        rows.append((int(k), fuzz[k], r["adjoint"], fd, rel, r["replayed"], r["degenerate"], r["changed"]))
        assert r["replayed"] > 0 and rel <= 1e-2, rows[-1]
    for row in rows:
        print("metal %d: GPU %.5g, held-trajectory adjoint %.5g, held FD %.5g (rel %.1e); %d paths, "
              "%d degenerate, %d whose re-render jumps" % row)
