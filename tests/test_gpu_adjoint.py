"""GPU: the adjoint path-replay launch.

Checked three ways: against the FP64 CPU adjoint of the oracle on the same
image and loss gradient (the GPU forms each path's albedo and sky terms in
binary32 and sums them in binary32 per block, double across blocks: 1e-5 of
the largest gradient; the fuzz tangent, binary32 with two double steps: 2e-4);
against central finite
differences of GPU renders with common random numbers (h = 1e-3) for albedo
and sky colours, through a torch.autograd.Function that wraps the forward
launch and the adjoint; and batch against single-scene launches.
"""
import ctypes

import numpy as np
import pytest

from _helpers import dptr, oracle_camera

pytestmark = pytest.mark.gpu

AMB = (0.5, 0.7, 0.95)     # sky colours below 1: no pixel sits on the clamp at 1
WHT = (0.97, 0.98, 0.96)


def _render(R, torch, sc, cam, params):
    n = params.image_w * params.image_h
    raw = torch.zeros(n * 3, dtype=torch.float32, device="cuda")
    rpp = torch.zeros(n, dtype=torch.int32, device="cuda")
    R.check(R.lib().rt_launch(sc.h, ctypes.byref(cam), ctypes.byref(params),
                              ctypes.byref(R.Frame(dptr(raw), dptr(rpp), None, None)), None))
    torch.cuda.synchronize()
    return raw


def _adjoint(R, torch, sc, cam, params, image, grad_image):
    n = sc.info().n_things
    ga = torch.zeros(n * 3, dtype=torch.float64, device="cuda")
    gf = torch.zeros(n, dtype=torch.float64, device="cuda")
    gs = torch.zeros(6, dtype=torch.float64, device="cuda")
    sc.adjoint(cam, params, dptr(image), dptr(grad_image), dptr(ga), dptr(gf), dptr(gs))
    torch.cuda.synchronize()
    return dict(albedo=ga.cpu().numpy().reshape(n, 3), fuzz=gf.cpu().numpy(), sky=gs.cpu().numpy())


def _close(a, b, rel=1e-9):
    scale = max(np.abs(b).max(), 1e-30)
    assert np.abs(a - b).max() <= rel * scale, (np.abs(a - b).max(), scale)


@pytest.mark.parametrize("level,spp,depth,rtow_px", [(None, 8, 8, False), (2, 6, 8, False), (3, 4, 16, False),
                                                     (2, 5, 8, True)])
def test_adjoint_matches_fp64_oracle(product, oracle, cuda, level, spp, depth, rtow_px):
    R, O, torch = product, oracle, cuda
    W, H, seed = 40, 30, 9
    sc = R.rtow_scene(level, R.RT_RECIPE_GLIBC, 1, 3)
    wd, _ = O.rtow_world(level, 0, 1, 3)
    cam = R.rtow_camera(W, H)
    params = R.launch_params(W, H, spp, depth=depth, seed=seed, ambient=AMB, white=WHT,
                             flags=R.RT_FLAG_RTOW_PIXELS if rtow_px else 0)
    img = _render(R, torch, sc, cam, params)
    I = img.cpu().numpy().reshape(-1, 3)
    ocam = oracle_camera(O, cam, rtow_pixels=rtow_px)
    ref_img = wd.render(ocam, W, H, spp, depth, seed, ambient=AMB, white=WHT, guides=False)
    assert np.array_equal(I.view(np.uint32), ref_img["rawRGB"].view(np.uint32))
    rng = np.random.default_rng(3)
    T = np.clip(I + rng.normal(0, 0.05, I.shape), 0, 1).astype(np.float32)
    G = (2.0 * (np.clip(I, 0, 1) - T)).astype(np.float32)
    g_dev = torch.from_numpy(G.reshape(-1)).cuda()
    got = _adjoint(R, torch, sc, cam, params, img, g_dev)
    ref = wd.adjoint(ocam, W, H, spp, depth, seed, I, G, ambient=AMB, white=WHT)
    _close(got["albedo"], ref["albedo"], rel=1e-5)   # binary32 terms against FP64 ones
    _close(got["sky"], ref["sky"], rel=1e-5)
    if np.abs(ref["fuzz"]).max() > 0:
        _close(got["fuzz"], ref["fuzz"], rel=2e-4)   # the fuzz tangent runs in binary32 on the GPU
    # glass has no albedo gradient, only metals have a fuzz gradient
    types = np.array([wd.optics()["types"][k] for k in range(wd.nthings)])
    assert np.all(got["albedo"][types == 2] == 0)
    assert np.all(got["fuzz"][types != 1] == 0)
    assert np.abs(got["albedo"]).sum() > 0 and np.abs(got["sky"]).sum() > 0


class _RenderFn:
    """torch.autograd.Function over (albedo [n,3], sky [6]): forward renders
    with those optics, backward runs the adjoint launch (test harness only)."""

    @staticmethod
    def make(R, torch, sc, cam, params_fn, types, fuzz, index):
        class Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, albedo, sky):
                a = albedo.detach().cpu().numpy()
                for k in range(a.shape[0]):
                    sc.set_optics(k, R.optics(int(types[k]), tuple(float(x) for x in a[k]), float(fuzz[k]),
                                              float(index[k])))
                s = sky.detach().cpu().numpy()
                params = params_fn(tuple(float(x) for x in s[:3]), tuple(float(x) for x in s[3:]))
                img = _render(R, torch, sc, cam, params)
                ctx.save_for_backward(img)
                ctx.params = params
                return img.view(-1, 3)

            @staticmethod
            def backward(ctx, grad_out):
                (img,) = ctx.saved_tensors
                gi = grad_out.contiguous().view(-1).to(torch.float32)
                g = _adjoint(R, torch, sc, cam, ctx.params, img, gi)
                return (torch.from_numpy(g["albedo"]).to(torch.float64),
                        torch.from_numpy(g["sky"]).to(torch.float64))

        return Fn


def test_adjoint_against_finite_differences_through_autograd(product, cuda):
    """Config-0 scene (analytic spheres) at reduced size: 32 sampled
    parameters (albedo channels and the six sky values) against central
    differences with common random numbers, h = 1e-3, 1e-2 relative."""
    R, torch = product, cuda
    W, H, spp, depth = 64, 64, 16, 8
    sc = R.rtow_scene(None, R.RT_RECIPE_GLIBC, 1, 11)
    sp = R.rtow_spheres(R.RT_RECIPE_GLIBC, 1, 11)
    n = sc.info().n_things
    types, fuzz, index = sp["types"], sp["fuzz"], sp["index"]
    cam = R.rtow_camera(W, H)

    def params_fn(amb, wht):
        return R.launch_params(W, H, spp, depth=depth, seed=21, ambient=amb, white=wht)

    Fn = _RenderFn.make(R, torch, sc, cam, params_fn, types, fuzz, index)
    albedo0 = torch.tensor(np.asarray(sp["albedos"], np.float64).reshape(n, 3))
    sky0 = torch.tensor(list(AMB) + list(WHT), dtype=torch.float64)
    with torch.no_grad():
        target = Fn.apply(albedo0, sky0).clamp(0, 1)
        rng = np.random.default_rng(5)
        target = (target + torch.from_numpy(rng.normal(0, 0.1, tuple(target.shape)).astype(np.float32)).cuda()).clamp(0, 1)

    def loss_of(albedo, sky):
        img = Fn.apply(albedo, sky)
        return ((img.clamp(0, 1) - target) ** 2).to(torch.float64).sum()

    a = albedo0.clone().requires_grad_(True)
    s = sky0.clone().requires_grad_(True)
    loss_of(a, s).backward()
    ga, gs = a.grad.numpy(), s.grad.numpy()

    h = 1e-3
    checked = 0
    # largest gradients first; channels whose albedo is within 10 h of 0 are
    # skipped: a central difference there steps to a negative albedo and
    # across the clamp at 0, where the loss has a kink
    order = np.argsort(-np.abs(ga).max(1))
    cand = [(int(k), c) for k in order[:60] if types[k] != 2 for c in range(3) if sp["albedos"][k, c] > 10 * 1e-3]
    with torch.no_grad():
        for k, c in cand[:26]:
            vals = []
            for sgn in (1, -1):
                a1 = albedo0.clone()
                a1[k, c] += sgn * h
                vals.append(float(loss_of(a1, sky0)))
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(ga[k, c] - fd) <= 1e-2 * max(abs(fd), 1e-2), (k, c, ga[k, c], fd)
            checked += 1
        for j in range(6):
            vals = []
            for sgn in (1, -1):
                s1 = sky0.clone()
                s1[j] += sgn * h
                vals.append(float(loss_of(albedo0, s1)))
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(gs[j] - fd) <= 1e-2 * max(abs(fd), 1e-2), (j, gs[j], fd)
            checked += 1
    assert checked == 32
    # optics restored
    for k in range(n):
        sc.set_optics(k, R.optics(int(types[k]), tuple(float(x) for x in sp["albedos"][k]), float(fuzz[k]),
                                  float(index[k])))


def test_batch_adjoint_equals_single_scene_adjoints(product, cuda):
    R, torch = product, cuda
    specs = [(None, 3, 32, 24, 4, 8, 31), (2, 2, 24, 24, 3, 16, 32), (1, 4, 40, 20, 2, 6, 33)]
    batch = R.Batch()
    scenes, bufs = [], []
    for level, he, w, h, spp, depth, seed in specs:
        sc = R.Scene()
        sc.load_rtow(R.RT_RECIPE_COUNTER, seed, he, -1 if level is None else level)
        scenes.append(sc)
        raw = torch.zeros(w * h * 3, dtype=torch.float32, device="cuda")
        rpp = torch.zeros(w * h, dtype=torch.int32, device="cuda")
        params = R.launch_params(w, h, spp, depth=depth, seed=seed, ambient=AMB, white=WHT)
        batch.add(sc, R.rtow_camera(w, h), params, R.Frame(dptr(raw), dptr(rpp), None, None))
        bufs.append((raw, rpp, params))
    batch.build()
    batch.launch()
    torch.cuda.synchronize()
    outs = []
    for k, (sc, (raw, rpp, params)) in enumerate(zip(scenes, bufs)):
        n = sc.info().n_things
        gi = (torch.rand(raw.shape, device="cuda", generator=torch.Generator("cuda").manual_seed(k)) - 0.5)
        o = (gi, torch.zeros(n * 3, dtype=torch.float64, device="cuda"),
             torch.zeros(n, dtype=torch.float64, device="cuda"), torch.zeros(6, dtype=torch.float64, device="cuda"))
        batch.set_adjoint(k, dptr(o[0]), dptr(o[1]), dptr(o[2]), dptr(o[3]))
        outs.append(o)
    batch.adjoint()
    torch.cuda.synchronize()
    for (level, he, w, h, spp, depth, seed), sc, (raw, rpp, params), o in zip(specs, scenes, bufs, outs):
        sc.build()
        cam = R.rtow_camera(w, h)
        img = _render(R, torch, sc, cam, params)
        assert torch.equal(img, raw)
        one = _adjoint(R, torch, sc, cam, params, img, o[0])
        # the same binary32 terms; block sums group the paths differently
        _close(o[1].cpu().numpy().reshape(-1, 3), one["albedo"], rel=1e-5)
        if np.abs(one["fuzz"]).max() > 0:
            _close(o[2].cpu().numpy(), one["fuzz"], rel=1e-5)
        _close(o[3].cpu().numpy(), one["sky"], rel=1e-5)


def test_adjoint_errors(product, cuda):
    R, torch = product, cuda
    sc = R.Scene()
    sc.load_rtow(R.RT_RECIPE_COUNTER, 3, 2, -1)
    cam = R.rtow_camera(8, 8)
    buf = torch.zeros(8 * 8 * 3, dtype=torch.float32, device="cuda")
    with pytest.raises(R.RTError) as e:
        sc.adjoint(cam, R.launch_params(8, 8, 1, depth=8), dptr(buf), dptr(buf), None, None, None)
    assert e.value.status == R.RT_ERR_NOT_BUILT
    sc.build()
    with pytest.raises(R.RTError) as e:
        sc.adjoint(cam, R.launch_params(8, 8, 1, depth=17), dptr(buf), dptr(buf), None, None, None)
    assert e.value.status == R.RT_ERR_INVALID_ARG
    # all outputs NULL is a valid (empty) request
    sc.adjoint(cam, R.launch_params(8, 8, 1, depth=8), dptr(buf), dptr(buf), None, None, None)
