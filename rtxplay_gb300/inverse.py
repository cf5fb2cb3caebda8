"""Batched inverse rendering: recover per-sphere albedos of many final-scene
variants from target images with Adam, every step on the device.

One iteration, batched: ``rt_batch_set_albedos`` (parameters -> optics),
``rt_batch_launch`` (all scenes, one wavefront), ``rt_l2_loss_grad`` over all
frames (one contiguous image buffer), ``rt_batch_adjoint`` (all scenes, one
launch), ``rt_adam_step`` over all parameters.  In graph mode the first
iteration runs as these calls and the same sequence (with the Adam step
counter on the device) is captured into one CUDA graph, which every later
iteration replays with a single launch; errors of the captured launches are
checked with ``rt_batch_status`` at the end.  Serial runs the same steps
scene by scene with the single-scene calls.  The reference has no inverse
rendering; this is the differentiable extension built on its scene recipe
(rtow.cxx:51-80 with the counter RNG).

Device buffers are torch tensors (plumbing only: every computation runs in
the library's kernels).
"""
import ctypes
import time

import numpy as np

import rtxplay_gb300 as R


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def inverse_specs(n, seed=7, level=4, size=256, spp=16, depth=8):
    """n scenes: half-extent U{3..8}, tessellation `level`, size x size, spp, depth."""
    rng = np.random.default_rng(seed)
    return [dict(half=int(rng.integers(3, 9)), level=level, w=size, h=size, spp=spp, depth=depth,
                 scene_seed=5000 + k, seed=9000 + k) for k in range(n)]


class InverseProblem:
    """Scenes, targets (rendered with the recipe's albedos) and Adam state."""

    def __init__(self, torch, specs, init=0.5, stream=None):
        self.torch, self.specs, self.stream = torch, specs, stream
        self.scenes, self.cams, self.params = [], [], []
        self.true = []
        for sp in specs:
            sc = R.Scene()
            sc.load_rtow(R.RT_RECIPE_COUNTER, sp["scene_seed"], sp["half"], sp["level"])
            sc.build()
            self.scenes.append(sc)
            self.cams.append(R.rtow_camera(sp["w"], sp["h"]))
            self.params.append(R.launch_params(sp["w"], sp["h"], sp["spp"], sp["depth"], sp["seed"], 0))
            rs = R.rtow_spheres(R.RT_RECIPE_COUNTER, sp["scene_seed"], sp["half"])
            self.true.append(rs)
        self.nthings = [sc.info().n_things for sc in self.scenes]
        self.toff = np.concatenate([[0], np.cumsum(self.nthings)]).astype(int)
        self.npix = [sp["w"] * sp["h"] for sp in specs]
        self.poff = np.concatenate([[0], np.cumsum(self.npix)]).astype(int)
        T, P = int(self.toff[-1]), int(self.poff[-1])
        dev = "cuda"
        self.image = torch.zeros(P * 3, dtype=torch.float32, device=dev)
        self.rpp = torch.zeros(P, dtype=torch.int32, device=dev)
        self.target = torch.zeros(P * 3, dtype=torch.float32, device=dev)
        self.gimg = torch.zeros(P * 3, dtype=torch.float32, device=dev)
        self.galb = torch.zeros(T * 3, dtype=torch.float64, device=dev)
        self.loss = torch.zeros(1, dtype=torch.float64, device=dev)
        true = np.concatenate([t["albedos"] for t in self.true]).astype(np.float32).reshape(-1)
        self.true_albedo = torch.from_numpy(true).to(dev)
        self.mask = np.concatenate([t["types"] != R.RT_OPTICS_REFRACT for t in self.true])   # glass has no albedo
        self.theta = torch.full((T * 3,), float(init), dtype=torch.float32, device=dev)
        self.m = torch.zeros_like(self.theta)
        self.v = torch.zeros_like(self.theta)
        self.step = 0
        self._frames = []
        for k in range(len(specs)):
            a, b = int(self.poff[k]), int(self.poff[k + 1])
            self._frames.append(R.Frame(_p(self.image[3 * a:3 * b]), _p(self.rpp[a:b]), None, None))
        # targets: render with the recipe's albedos
        for k, sc in enumerate(self.scenes):
            a, b = int(self.toff[k]), int(self.toff[k + 1])
            sc.set_albedos(_p(self.true_albedo[3 * a:3 * b]), stream)
        self._render_serial()
        self.target.copy_(self.image)
        self.batch = None

    def _render_serial(self):
        lib = R.lib()
        for k, sc in enumerate(self.scenes):
            R.check(lib.rt_launch(sc.h, ctypes.byref(self.cams[k]), ctypes.byref(self.params[k]),
                                  ctypes.byref(self._frames[k]), self.stream))

    def make_batch(self):
        b = R.Batch()
        for k, sc in enumerate(self.scenes):
            b.add(sc, self.cams[k], self.params[k], self._frames[k])
        b.build(stream=self.stream)
        for k in range(len(self.scenes)):
            pa, pb = int(self.poff[k]), int(self.poff[k + 1])
            ta, tb = int(self.toff[k]), int(self.toff[k + 1])
            b.set_adjoint(k, _p(self.gimg[3 * pa:3 * pb]), _p(self.galb[3 * ta:3 * tb]), None, None)
        self.batch = b

    def iterate_batched(self, lr=1e-2):
        """One Adam iteration over all scenes with batched launches; returns nothing (loss stays on the device)."""
        if self.batch is None:
            self.make_batch()
        self.step += 1
        s = self.stream
        self.batch.set_albedos(_p(self.theta), s)
        self.batch.launch(s)
        self.loss.zero_()
        R.l2_loss_grad(_p(self.image), _p(self.target), _p(self.gimg), int(self.poff[-1]), _p(self.loss), s)
        self.batch.adjoint(s)
        R.adam_step(_p(self.theta), _p(self.galb), _p(self.m), _p(self.v), self.theta.numel(), self.step, lr=lr,
                    stream=s)

    def _iteration_device(self, s, lr):
        """The batched iteration with the Adam step counter on the device (capturable)."""
        self.batch.set_albedos(_p(self.theta), s)
        self.batch.launch(s, stats=False)
        self.loss.zero_()
        R.l2_loss_grad(_p(self.image), _p(self.target), _p(self.gimg), int(self.poff[-1]), _p(self.loss), s)
        self.batch.adjoint(s)
        R.adam_step_device(_p(self.theta), _p(self.galb), _p(self.m), _p(self.v), self.theta.numel(),
                           _p(self.step_dev), lr=lr, stream=s)

    def make_graph(self, lr=1e-2):
        """Runs one batched iteration with the calls themselves (it sizes the
        batch's buffers and uploads its tables), then captures the same
        iteration into one CUDA graph; iterate_graph replays it."""
        torch = self.torch
        if self.batch is None:
            self.make_batch()
        self.step_dev = torch.tensor([self.step], dtype=torch.int32, device="cuda")
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            self._iteration_device(ctypes.c_void_p(side.cuda_stream), lr)
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        self.step += 1
        self.batch.status()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self._iteration_device(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), lr)

    def iterate_graph(self):
        """One batched iteration: one replay of the captured graph."""
        self.graph.replay()
        self.step += 1

    def iterate_serial(self, lr=1e-2):
        """The same iteration scene by scene (single-scene launches)."""
        self.step += 1
        s = self.stream
        lib = R.lib()
        self.loss.zero_()
        for k, sc in enumerate(self.scenes):
            ta, tb = int(self.toff[k]), int(self.toff[k + 1])
            pa, pb = int(self.poff[k]), int(self.poff[k + 1])
            sc.set_albedos(_p(self.theta[3 * ta:3 * tb]), s)
            R.check(lib.rt_launch(sc.h, ctypes.byref(self.cams[k]), ctypes.byref(self.params[k]),
                                  ctypes.byref(self._frames[k]), s))
            R.l2_loss_grad(_p(self.image[3 * pa:3 * pb]), _p(self.target[3 * pa:3 * pb]),
                           _p(self.gimg[3 * pa:3 * pb]), pb - pa, _p(self.loss), s)
            sc.adjoint(self.cams[k], self.params[k], _p(self.image[3 * pa:3 * pb]), _p(self.gimg[3 * pa:3 * pb]),
                       _p(self.galb[3 * ta:3 * tb]), None, None, s)
            R.adam_step(_p(self.theta[3 * ta:3 * tb]), _p(self.galb[3 * ta:3 * tb]), _p(self.m[3 * ta:3 * tb]),
                        _p(self.v[3 * ta:3 * tb]), 3 * (tb - ta), self.step, lr=lr, stream=s)

    def albedo_error(self):
        """Mean |albedo - recipe albedo| over the non-glass things."""
        th = self.theta.cpu().numpy().reshape(-1, 3)
        tr = self.true_albedo.cpu().numpy().reshape(-1, 3)
        return float(np.abs(th - tr)[self.mask].mean())


def run(torch, specs, iters, batched=True, lr=1e-2, stream=None, graph=False):
    """Optimises from albedo 0.5; returns (initial error, final error, final loss, seconds).
    graph=True (batched only): the first iteration runs as calls and is
    captured, the others replay the captured graph; the capture is timed."""
    prob = InverseProblem(torch, specs, stream=stream)
    if batched:
        prob.make_batch()
    e0 = prob.albedo_error()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    if batched and graph:
        prob.make_graph(lr)
        for _ in range(iters - 1):
            prob.iterate_graph()
        torch.cuda.synchronize()
        prob.batch.status()
    else:
        for _ in range(iters):
            (prob.iterate_batched if batched else prob.iterate_serial)(lr)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    return e0, prob.albedo_error(), float(prob.loss.item()), dt
