"""GPU: the inverse-rendering pieces and a small batched albedo recovery.

Adam and the L2 loss gradient are checked bit for bit against numpy float32
restatements; device-side albedos against host-side optics (identical
renders); then a few scenes are optimised from albedo 0.5 towards their
recipe albedos, batched and serial, which must agree and reduce the error.
"""
import ctypes

import numpy as np
import pytest

from _helpers import dptr

pytestmark = pytest.mark.gpu


def test_adam_step_matches_float32_restatement(product, cuda):
    R, torch = product, cuda
    rng = np.random.default_rng(0)
    n = 1000
    theta = rng.uniform(0, 1, n).astype(np.float32)
    m = rng.normal(0, 0.1, n).astype(np.float32)
    v = rng.uniform(0, 0.01, n).astype(np.float32)
    g = rng.normal(0, 1, n)
    dt, dm, dv, dg = (torch.from_numpy(x).cuda() for x in (theta, m, v, g))
    lr, b1, b2, eps, step = np.float32(0.01), np.float32(0.9), np.float32(0.999), np.float32(1e-8), 7
    R.adam_step(dptr(dt), dptr(dg), dptr(dm), dptr(dv), n, step, lr=float(lr), beta1=float(b1), beta2=float(b2),
                eps=float(eps), lo=0.0, hi=1.0)
    torch.cuda.synchronize()
    gf = g.astype(np.float32)
    one = np.float32(1)
    mi = b1 * m + (one - b1) * gf
    vi = b2 * v + (one - b2) * (gf * gf)
    bc1 = np.float32(1.0 - float(b1) ** step)
    bc2 = np.float32(1.0 - float(b2) ** step)
    th = theta - lr * (mi / bc1) / (np.sqrt(vi / bc2) + eps)
    th = np.minimum(np.maximum(th, np.float32(0)), np.float32(1))
    assert np.array_equal(dm.cpu().numpy().view(np.uint32), mi.view(np.uint32))
    assert np.array_equal(dv.cpu().numpy().view(np.uint32), vi.view(np.uint32))
    assert np.array_equal(dt.cpu().numpy().view(np.uint32), th.astype(np.float32).view(np.uint32))


def test_l2_loss_grad(product, cuda):
    R, torch = product, cuda
    rng = np.random.default_rng(1)
    n = 5000
    img = rng.uniform(-0.2, 1.3, (n, 3)).astype(np.float32)
    tgt = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    di, dtg = torch.from_numpy(img.reshape(-1)).cuda(), torch.from_numpy(tgt.reshape(-1)).cuda()
    dgr = torch.zeros(n * 3, dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    R.l2_loss_grad(dptr(di), dptr(dtg), dptr(dgr), n, dptr(loss))
    torch.cuda.synchronize()
    e = np.clip(img, 0, 1) - tgt
    assert np.array_equal(dgr.cpu().numpy().reshape(-1, 3).view(np.uint32), (np.float32(2) * e).view(np.uint32))
    assert abs(loss.item() - (e.astype(np.float64) ** 2).sum()) <= 1e-9 * (e.astype(np.float64) ** 2).sum()


def test_device_albedos_render_like_host_optics(product, cuda):
    R, torch = product, cuda
    sc_a = R.rtow_scene(2, R.RT_RECIPE_COUNTER, 3, 3)
    sc_b = R.rtow_scene(2, R.RT_RECIPE_COUNTER, 3, 3)
    sp = R.rtow_spheres(R.RT_RECIPE_COUNTER, 3, 3)
    rng = np.random.default_rng(4)
    alb = rng.uniform(0, 1, sp["albedos"].shape).astype(np.float32)
    for k in range(len(alb)):
        sc_a.set_optics(k, R.optics(int(sp["types"][k]), tuple(float(x) for x in alb[k]), float(sp["fuzz"][k]),
                                    float(sp["index"][k])))
    d = torch.from_numpy(alb.reshape(-1)).cuda()
    sc_b.set_albedos(dptr(d))
    cam = R.rtow_camera(64, 48)
    params = R.launch_params(64, 48, 3, depth=16, seed=5)
    a, b = R.render(sc_a, cam, params), R.render(sc_b, cam, params)
    assert np.array_equal(a["rawRGB"].view(np.uint32), b["rawRGB"].view(np.uint32))


def test_batched_inverse_rendering_recovers_albedos(product, cuda):
    R, torch = product, cuda
    from rtxplay_gb300 import inverse
    specs = inverse.inverse_specs(4, seed=3, level=2, size=64, spp=8, depth=8)
    pb = inverse.InverseProblem(torch, specs)
    ps = inverse.InverseProblem(torch, specs)
    e0 = pb.albedo_error()
    for _ in range(10):
        pb.iterate_batched()
        ps.iterate_serial()
    torch.cuda.synchronize()
    # same renders; adjoint sums differ only in summation order
    assert np.abs(pb.theta.cpu().numpy() - ps.theta.cpu().numpy()).max() <= 1e-4
    l10 = pb.loss.item()
    for _ in range(50):
        pb.iterate_batched()
    torch.cuda.synchronize()
    print("inverse: loss after 10 / 60 iterations", l10, pb.loss.item(), "albedo error", e0, pb.albedo_error())
    assert pb.loss.item() < 0.7 * l10
    assert pb.albedo_error() < e0 - 0.02


def test_adam_step_device_counter(product, cuda):
    """rt_adam_step_device takes step *step + 1 and advances the counter; the
    same update as rt_adam_step within an ulp of the bias corrections."""
    R, torch = product, cuda
    rng = np.random.default_rng(2)
    n = 777
    theta = rng.uniform(0, 1, n).astype(np.float32)
    g = rng.normal(0, 1, n)
    a = [torch.from_numpy(x.copy()).cuda() for x in (theta, np.zeros(n, np.float32), np.zeros(n, np.float32))]
    b = [torch.from_numpy(x.copy()).cuda() for x in (theta, np.zeros(n, np.float32), np.zeros(n, np.float32))]
    dg = torch.from_numpy(g).cuda()
    step = torch.zeros(1, dtype=torch.int32, device="cuda")
    for k in range(1, 4):
        R.adam_step(dptr(a[0]), dptr(dg), dptr(a[1]), dptr(a[2]), n, k)
        R.adam_step_device(dptr(b[0]), dptr(dg), dptr(b[1]), dptr(b[2]), n, dptr(step))
    torch.cuda.synchronize()
    assert int(step.item()) == 3
    assert torch.allclose(a[0], b[0], rtol=1e-6, atol=1e-7)


def test_inverse_iteration_as_one_captured_graph(product, cuda):
    """The batched iteration captured into one CUDA graph (wave loop as a
    conditional node, Adam's step counter on the device) follows the
    call-by-call iteration; the batch reports no error of the captured
    launches; a call that cannot be captured is refused cleanly."""
    R, torch = product, cuda
    from rtxplay_gb300 import inverse
    specs = inverse.inverse_specs(3, seed=5, level=2, size=48, spp=4, depth=8)
    pc = inverse.InverseProblem(torch, specs)
    pg = inverse.InverseProblem(torch, specs)
    for _ in range(6):
        pc.iterate_batched()
    pg.make_graph()          # iteration 1 as calls, then the capture
    for _ in range(5):
        pg.iterate_graph()   # iterations 2..6, one graph launch each
    torch.cuda.synchronize()
    pg.batch.status()
    assert pg.step == pc.step == 6 and int(pg.step_dev.item()) == 6
    # the same renders and adjoints; Adam's bias corrections come from pow on the
    # device against the host's, which may differ in the last bit
    assert torch.allclose(pg.theta, pc.theta, rtol=1e-5, atol=1e-6)
    assert abs(pg.loss.item() - pc.loss.item()) <= 1e-5 * pc.loss.item()
    # stats cannot come out of a capture: refused before anything is enqueued
    g = torch.cuda.CUDAGraph()
    with pytest.raises(R.RTError) as e:
        with torch.cuda.graph(g):
            pg.batch.launch(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), stats=True)
    assert e.value.status == R.RT_ERR_INVALID_ARG
    pg.batch.status()


def test_capture_refuses_what_it_cannot_record(product, cuda):
    """A batch launch inside a capture is refused, before it enqueues anything,
    when host-side optics changed since the last launch (their upload is a host
    copy) and when the batch never ran outside a capture; the batch launches
    normally afterwards and reports no captured error."""
    R, torch = product, cuda
    from rtxplay_gb300 import inverse
    specs = inverse.inverse_specs(2, seed=9, level=1, size=32, spp=2, depth=4)
    p = inverse.InverseProblem(torch, specs)
    p.make_batch()
    side = torch.cuda.Stream()

    def capture_launch():
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=side):
            p.batch.launch(ctypes.c_void_p(side.cuda_stream), stats=False)

    with pytest.raises(R.RTError) as e:   # no launch outside a capture yet
        capture_launch()
    assert e.value.status == R.RT_ERR_INVALID_ARG
    with torch.cuda.stream(side):
        p.batch.launch(ctypes.c_void_p(side.cuda_stream))
    torch.cuda.synchronize()
    sp = p.true[0]
    p.scenes[0].set_optics(0, R.optics(int(sp["types"][0]), (0.3, 0.3, 0.3), float(sp["fuzz"][0]),
                                       float(sp["index"][0])))
    with pytest.raises(R.RTError) as e:   # host optics changed since the last launch
        capture_launch()
    assert e.value.status == R.RT_ERR_INVALID_ARG and b"optics" in R.lib().rt_last_error_string()
    p.batch.launch()
    torch.cuda.synchronize()
    p.batch.status()
