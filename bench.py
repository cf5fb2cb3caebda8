"""Benchmark: Mrays/s of the GB300 path tracer on the tessellated final scene.

Workload (one step = one full frame): the RTOW final scene (glibc rand()
seed 1, 487 spheres) with every sphere tessellated 6 times (7,979,008
triangles, LBVH with 60-bit Morton codes), 1200x800 pixels, 500 samples per
pixel, depth 50.  Rays are counted as the reference counts rpp (every
closest-hit query, the final miss included).

  value     Mrays/s with the scene resident in HBM (device-timed, CUDA events on
            the launching stream), max over ranks, summed rays of all ranks.
  e2e       the same metric through the C ABI from host buffers: per step the
            host mesh and things are copied in, the LBVH is built, the frame is
            rendered and post-processed, image and rays-per-pixel are copied out.
  roofline  traversal kernel (k_extend): algorithmic bytes per launch / mean
            launch time against the measured HBM copy bandwidth.
  cpu_baseline  the CPU oracle (a C++ restatement of the reference's path) on a
            bounded pixel sample of the same workload on all host cores.

`--impl reference` times that CPU implementation alone (the reference's GPU
path is OptiX on RT cores and cannot run on this machine).
Multi-GPU runs (torchrun) render independent replicas, one frame per rank per
step: replicas only, no collective on the data path.
"""
import argparse
import ctypes
import json
import os
import re
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s at 1200x800x500spp 8M-tri"
UNIT = "Mrays/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--width", type=int, default=1200)
    p.add_argument("--height", type=int, default=800)
    p.add_argument("--spp", type=int, default=500)
    p.add_argument("--depth", type=int, default=50)
    p.add_argument("--level", type=int, default=6)
    p.add_argument("--morton-bits", type=int, default=60)
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU-baseline sample time")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    p.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    return p.parse_args()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_dram_bytes_per_ray():
    """DRAM bytes per ray of k_extend from the committed ncu summary (one
    capture of full-wave launches), or None."""
    path = os.path.join(ROOT, "profiles", "k_extend_c1.txt")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        m = re.search(r"^dram_bytes_per_ray:\s*([0-9.eE+]+)", f.read(), re.M)
    return float(m.group(1)) if m else None


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        rows = [r.split(",") for r in out.strip().splitlines() if r.count(",") >= 8]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if "Active" in r[5 + k] and "Not" not in r[5 + k]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_oracle_run(args, target_s, threads=None):
    """Oracle (CPU restatement) on a strided pixel sample of the workload."""
    from oracle import oracle as O
    O.build()
    world, _ = O.rtow_world(level=args.level, morton_bits=args.morton_bits)
    cam = O.rtow_camera(args.width, args.height)
    npix = args.width * args.height
    threads = threads or os.cpu_count()
    # calibrate on a small sample, then size the sample for ~target_s
    probe = np.arange(0, npix, max(1, npix // 64), dtype=np.uint32)
    t0 = time.perf_counter()
    r = world.render(cam, args.width, args.height, args.spp, args.depth, 4711, pixels=probe, guides=False,
                     nthreads=threads)
    dt = max(time.perf_counter() - t0, 1e-3)
    want = int(len(probe) * max(1.0, target_s / dt))
    stride = max(1, npix // max(want, 1))
    pix = np.arange(0, npix, stride, dtype=np.uint32)[:want]
    t0 = time.perf_counter()
    r = world.render(cam, args.width, args.height, args.spp, args.depth, 4711, pixels=pix, guides=False,
                     nthreads=threads)
    dt = time.perf_counter() - t0
    return {"value": r["rays"] / dt / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{len(pix)} of {npix} pixels (stride {stride}) x {args.spp} spp, depth {args.depth}, "
                      f"{r['rays']} rays in {dt:.2f} s; LBVH build excluded"}


def run_reference(args, world, rank):
    if world > 1 and rank != 0:
        return
    per_step = max(2.0, min(20.0, 60.0 / max(1, args.steps + args.warmup)))
    for _ in range(args.warmup):
        cpu_oracle_run(args, per_step / 4)
    vals, samples = [], []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        b = cpu_oracle_run(args, per_step)
        vals.append(b["value"])
        samples.append(b)
    wall = time.perf_counter() - t0
    v = float(np.mean(vals))
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (reference scene recipe, glibc rand seed 1)",
            "config": {"workload": "rtow final scene, level-6 tessellation (7,979,008 triangles), "
                                   f"{args.width}x{args.height}, {args.spp} spp, depth {args.depth}",
                       "implementation": "CPU oracle port of rtow/rtwo on all host cores"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": samples[-1]["cores"], "kind": "port",
                             "sample": samples[-1]["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return

    import torch
    import rtxplay_gb300 as R

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    lib = R.lib()
    W, H = args.width, args.height
    npix = W * H
    stream = torch.cuda.current_stream()
    sptr = ctypes.c_void_p(stream.cuda_stream)

    # ---- scene in HBM (build excluded from the timed region, reported apart)
    sc = R.Scene()
    sc.load_rtow(R.RT_RECIPE_GLIBC, 1, 11, args.level)
    sc.build(args.morton_bits, stream=sptr)
    info = sc.info()
    cam = R.rtow_camera(W, H)
    raw = torch.empty(npix * 3, dtype=torch.float32, device="cuda")
    rpp = torch.empty(npix, dtype=torch.int32, device="cuda")
    frame = R.Frame(ctypes.c_void_p(raw.data_ptr()), ctypes.c_void_p(rpp.data_ptr()), None, None)

    def step(seed, flags):
        params = R.launch_params(W, H, args.spp, args.depth, seed, flags)
        st = R.LaunchStats()
        R.check(lib.rt_launch_ex(sc.h, ctypes.byref(cam), ctypes.byref(params), ctypes.byref(frame), sptr,
                                 ctypes.byref(st)))
        return st

    # algorithmic bytes per ray from a counting pass (untimed, reduced spp)
    cnt_params = R.launch_params(W, H, max(1, min(args.spp, 16)), args.depth, 99, R.RT_FLAG_COUNT_VISITS)
    cst = R.LaunchStats()
    R.check(lib.rt_launch_ex(sc.h, ctypes.byref(cam), ctypes.byref(cnt_params), ctypes.byref(frame), sptr,
                             ctypes.byref(cst)))
    nodes_per_ray = cst.node_visits / max(1, cst.rays)
    prims_per_ray = cst.prim_tests / max(1, cst.rays)
    bytes_per_ray = 64.0 * nodes_per_ray + 48.0 * prims_per_ray + 48.0

    for k in range(args.warmup):
        step(1000 + k, 0)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    rays = 0
    ext_ms = 0.0
    ext_launches = 0
    launches = 0
    for k in range(args.steps):
        st = step(4711 + k, R.RT_FLAG_STAGE_TIMING)
        rays += st.rays
        ext_ms += st.extend_ms
        ext_launches += st.extend_launches
        launches += st.kernel_launches
    ev1.record(stream)
    torch.cuda.synchronize()
    elapsed_ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    if dist:
        t = torch.tensor([elapsed_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed_ms = float(t.item())
        r = torch.tensor([float(rays)], device="cuda", dtype=torch.float64)
        dist.all_reduce(r)
        total_rays = float(r.item())
    else:
        total_rays = float(rays)
    value = total_rays / (elapsed_ms * 1e-3) / 1e6

    # ---- end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        from rtxplay_gb300 import _build  # noqa: F401
        mesh_host = None
        m = R.Scene()
        mid = m.add_sphere_mesh(1.0, args.level)
        mesh_host = m.get_mesh(mid)
        m.close()
        spheres = R.rtow_spheres(R.RT_RECIPE_GLIBC, 1, 11)
        img_host = np.empty((npix, 4), np.uint8)
        rpp_host = np.empty(npix, np.uint32)
        L = R.Launcher(W, H)
        h2d = mesh_host[0].nbytes + mesh_host[1].nbytes + len(spheres["radii"]) * (16 + 48 + 20)
        d2h = img_host.nbytes + rpp_host.nbytes
        e2e_rays = 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(args.steps):
            s2 = R.Scene()
            mid = s2.add_mesh(mesh_host[0], mesh_host[1])
            for c, r_, t_, a_, f_, i_ in zip(spheres["centers"], spheres["radii"], spheres["types"],
                                             spheres["albedos"], spheres["fuzz"], spheres["index"]):
                T = np.array([r_, 0, 0, c[0], 0, r_, 0, c[1], 0, 0, r_, c[2]], np.float32)
                s2.add_thing(R.optics(int(t_), a_, float(f_), float(i_)), mid, T)
            s2.build(args.morton_bits)
            params = R.launch_params(W, H, args.spp, args.depth, 4711 + k, 0)
            st = L.ignite(s2, cam, params)
            R.check(lib.rt_launcher_download(L.h, None, ctypes.c_void_p(rpp_host.ctypes.data), None, None,
                                             ctypes.c_void_p(img_host.ctypes.data), None))
            e2e_rays += int(rpp_host.sum(dtype=np.uint64))
            s2.close()
        dt = time.perf_counter() - t0
        L.close()
        e2e = {"value": e2e_rays / dt / 1e6, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h)}
        if dist:
            t = torch.tensor([dt, float(e2e_rays)], device="cuda", dtype=torch.float64)
            dist.all_reduce(t[0:1], op=dist.ReduceOp.MAX)
            dist.all_reduce(t[1:2])
            e2e["value"] = float(t[1].item()) / float(t[0].item()) / 1e6

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_oracle_run(args, args.cpu_seconds)

    peak, peak_src = load_peaks()
    per_launch_ms = ext_ms / max(1, ext_launches)
    rays_per_launch = rays / max(1, ext_launches)
    achieved = bytes_per_ray * rays_per_launch / (per_launch_ms * 1e-3) / 1e9 if per_launch_ms > 0 else None
    dram_per_ray = profile_dram_bytes_per_ray()
    traffic = dram_per_ray * rays_per_launch if dram_per_ray else None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None,
                "traffic": traffic,
                "traffic_note": "ncu dram bytes of full-wave launches (profiles/k_extend_c1.txt), "
                                "per ray, times the rays of a mean launch",
                "kernel": "k_extend (LBVH traversal + ray/triangle tests)",
                "peak_source": f"{peak_src} hbm_gbs",
                "bytes_per_ray": bytes_per_ray, "nodes_per_ray": nodes_per_ray, "prims_per_ray": prims_per_ray,
                "extend_ms_per_launch": per_launch_ms, "extend_share": ext_ms / max(elapsed_ms, 1e-9),
                "rays_per_launch": rays_per_launch}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (reference scene recipe, glibc rand seed 1)",
                "config": {"workload": f"rtow final scene, level-{args.level} tessellation "
                                       f"({info.n_prims} triangles), {W}x{H}, {args.spp} spp, depth {args.depth}",
                           "parallelism": f"replicas x{world}", "morton_bits": info.morton_bits,
                           "l2": "inputs larger than L2 (LBVH + triangles "
                                 f"{info.device_bytes / 2**30:.2f} GiB on device)",
                           "build_ms": info.build_ms},
                "rays_per_step": total_rays / args.steps / world,
                "gpu_launches": launches,
                "clocks": clk, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e}
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
