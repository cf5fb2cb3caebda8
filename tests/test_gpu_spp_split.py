"""GPU: the spp-split form of the multi-GPU path, with two ranks.

Two processes (gloo, 127.0.0.1; both on the one GPU here, each with its own
context, no kernel of one waiting on the other) render disjoint sample
ranges of the same frame into accumulators: rank r renders samples
[r k, (r + 1) k).  The exact fixed-point sums are summed across the ranks
with all_reduce (on CPU tensors: gloo), written back, declared as samples
[0, 2 k) and resolved: the image and rays per pixel must equal one 2k-sample
launch bit for bit.  This is the one collective of the split (a sum of the
accumulation buffers); the reference renders one frame with a single
optixLaunch (optx/launcher.cxx:60-69).
"""
import os
import socket
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
W, H, K, SEED = 96, 64, 6, 77


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


class _Dev:
    """A device array by address (the accumulator's sums) for torch.as_tensor."""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 3}


def _worker(rank, world, port, q):
    try:
        os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
        sys.path.insert(0, ROOT)
        import ctypes
        import torch
        import torch.distributed as dist
        import rtxplay_gb300 as R
        dist.init_process_group("gloo", rank=rank, world_size=world)
        torch.cuda.init()
        sc = R.rtow_scene(2, half_extent=4)
        cam = R.rtow_camera(W, H)
        acc = R.Accum(W, H)
        raw = torch.zeros(W * H * 3, dtype=torch.float32, device="cuda")
        rpp = torch.zeros(W * H, dtype=torch.int32, device="cuda")
        frame = R.Frame(ctypes.c_void_p(raw.data_ptr()), ctypes.c_void_p(rpp.data_ptr()), None, None)
        acc.set_first_sample(rank * K)
        st = acc.launch(sc, cam, R.launch_params(W, H, K, depth=50, seed=SEED), frame)
        torch.cuda.synchronize()
        n = W * H
        r_p, g_p, b_p, rays_p = acc.device_sums()
        sums = [torch.as_tensor(_Dev(p, n, "<i8"), device="cuda") for p in (r_p, g_p, b_p)]
        sums.append(torch.as_tensor(_Dev(rays_p, n, "<i4"), device="cuda"))
        for t in sums:   # the sum-reduction of the accumulation buffers
            c = t.cpu()
            dist.all_reduce(c)
            t.copy_(c)
        total = torch.tensor([int(st.rays)], dtype=torch.int64)
        dist.all_reduce(total)
        torch.cuda.synchronize()
        acc.set_range(0, world * K, int(total.item()))
        acc.resolve(frame)
        ref = R.render(sc, cam, R.launch_params(W, H, world * K, depth=50, seed=SEED))
        torch.cuda.synchronize()
        same = (np.array_equal(raw.cpu().numpy().view(np.uint32), ref["rawRGB"].reshape(-1).view(np.uint32))
                and np.array_equal(rpp.cpu().numpy().astype(np.int64), ref["rpp"].astype(np.int64)))
        q.put((rank, bool(same), int(total.item()), int(ref["rpp"].sum()), ""))
        acc.close()
        dist.barrier()
        dist.destroy_process_group()
    except Exception as e:   # reported to the parent, which fails the test
        q.put((rank, False, 0, 0, repr(e)))
        raise


def test_two_ranks_split_samples_and_sum_their_accumulators():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(300)
    got = sorted(q.get(timeout=10) for _ in range(2))
    for p in procs:
        assert p.exitcode == 0
    for rank, same, rays, ref_rays, err in got:
        assert err == "" and same, (rank, err)
        assert rays == ref_rays
