"""Autotuner of the wavefront's launch shape (``rt_tuning``).

The knobs are the wave-queue size, the shading kernel's block size, the
persistent traversal's blocks per SM and its refill rule (refill a warp when
at most ``refill_below`` lanes are busy, checked every ``steps_per_check``
steps).  None of them changes an image (the pixel sums are exact integers and
the hits do not depend on the traversal order), so any launch of a workload
can time them.

``autotune`` runs coordinate descent from a start point (the built-in
defaults): each knob in turn takes every candidate value with the others
held, and the fastest setting is kept; a tie keeps the current value, so the
search never moves without a gain of at least ``min_gain``.  It stops after a
sweep over all knobs that changed nothing, or after ``max_sweeps`` sweeps.
Every setting is measured once (memoised).

Results live in a JSON cache (``TuneCache``): per device name, per workload
key (``workload_key``), the chosen tuning and its time.  The file shipped in
the package, ``tuning.json``, holds the settings measured for the benchmark
workloads; ``RTX_TUNE_CACHE`` names another file.
"""
import json
import math
import os
import statistics
import tempfile
import time

from . import Launcher, tuning_get, tuning_set

DEFAULT = {"wave_log2": 26, "shade_block": 512, "extend_blocks_per_sm": 0, "refill_below": 12, "steps_per_check": 16}

# candidate values per knob (extend_blocks_per_sm 0: as many as fit)
SPACE = {
    "wave_log2": (20, 21, 22, 23, 24, 25, 26),
    "shade_block": (128, 256, 512, 1024),
    "extend_blocks_per_sm": (0, 4, 3, 2),
    "refill_below": (4, 8, 12, 16, 20),
    "steps_per_check": (8, 16, 32),
}

PACKAGE_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning.json")


def _key_of(t):
    return tuple(sorted(t.items()))


def autotune(measure, space=None, start=None, max_sweeps=3, min_gain=0.01, log=None):
    """Coordinate descent over `space` (knob -> candidate values) from `start`.

    measure(tuning dict) -> seconds (lower is better).  A candidate replaces
    the current value only if it is faster by more than `min_gain` (relative).
    Returns (best tuning, its time, trials) with trials = [(tuning, seconds)]
    in the order measured.
    """
    space = dict(SPACE if space is None else space)
    cur = dict(DEFAULT if start is None else start)
    for k, vals in space.items():
        if not vals:
            raise ValueError(f"no candidates for {k}")
        if cur.get(k) not in vals:
            cur[k] = vals[0]
    seen = {}
    trials = []

    def timed(t):
        key = _key_of(t)
        if key not in seen:
            sec = float(measure(dict(t)))
            if not math.isfinite(sec) or sec < 0:
                raise ValueError(f"measure returned {sec} for {t}")
            seen[key] = sec
            trials.append((dict(t), sec))
            if log:
                log(f"tune {dict(t)}: {sec * 1e3:.3f} ms")
        return seen[key]

    best = timed(cur)
    for _ in range(max_sweeps):
        changed = False
        for k, vals in space.items():
            for v in vals:
                if v == cur[k]:
                    continue
                cand = dict(cur)
                cand[k] = v
                sec = timed(cand)
                if sec < best * (1.0 - min_gain):
                    cur, best, changed = cand, sec, True
        if not changed:
            break
    return cur, best, trials


def workload_key(kind, paths, prims, depth, scenes=1, layout="sah"):
    """Cache key of a workload: kind, scenes, layout, depth and log2 buckets
    of the path and primitive counts (workloads in one bucket share a tuning)."""
    pb = int(round(math.log2(max(1, paths))))
    qb = int(round(math.log2(max(1, prims))))
    return f"{kind}:scenes={scenes}:layout={layout}:depth={depth}:paths~2^{pb}:prims~2^{qb}"


def device_name():
    """Name of CUDA device 0 (through torch when present), else "cuda"."""
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name(0)
    except Exception:
        pass
    return "cuda"


class TuneCache:
    """JSON file {device: {workload key: {"tuning": {...}, "ms": t, ...}}}."""

    def __init__(self, path=None):
        self.path = path or os.environ.get("RTX_TUNE_CACHE") or PACKAGE_CACHE
        self.data = {}
        if os.path.exists(self.path):
            with open(self.path) as f:
                self.data = json.load(f)

    def get(self, device, key):
        e = self.data.get(device, {}).get(key)
        return None if e is None else dict(e)

    def put(self, device, key, tuning, ms, **extra):
        e = {"tuning": {k: int(v) for k, v in tuning.items()}, "ms": float(ms)}
        e.update(extra)
        self.data.setdefault(device, {})[key] = e

    def save(self):
        d = os.path.dirname(os.path.abspath(self.path))
        os.makedirs(d, exist_ok=True)
        fd, tmp = tempfile.mkstemp(dir=d, suffix=".tmp")
        with os.fdopen(fd, "w") as f:
            json.dump(self.data, f, indent=1, sort_keys=True)
            f.write("\n")
        os.replace(tmp, self.path)


def tuned(key, measure=None, cache=None, device=None, retune=False, apply=True, **search):
    """The cached tuning of workload `key` on `device`, else (with a `measure`)
    a fresh autotune stored in the cache; applied with rt_tuning_set when
    `apply`.  Returns (tuning dict, source) with source "cache", "tuned" or
    "default" (no cache entry and no measure)."""
    cache = cache if cache is not None else TuneCache()
    device = device or device_name()
    e = None if retune else cache.get(device, key)
    if e is not None:
        t, src = e["tuning"], "cache"
    elif measure is not None:
        t, sec, trials = autotune(measure, **search)
        cache.put(device, key, t, sec * 1e3, trials=len(trials))
        cache.save()
        src = "tuned"
    else:
        t, src = None, "default"
    if apply:
        tuning_set(t)   # None: the built-in defaults (RTX_WAVE still applies)
    return (dict(DEFAULT) if t is None else t), src


def _median_time(fn, repeats):
    fn()   # warm-up: a new launch shape re-instantiates the wave-loop graph
    ts = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return statistics.median(ts)


def render_timer(scene, cam, params, repeats=3):
    """measure(tuning) for tune(): median wall time of a synchronous launch
    of `scene` (Launcher.ignite) under that tuning; the tuning in effect
    before is restored afterwards."""
    L = Launcher(params.image_w, params.image_h)

    def measure(t):
        before = tuning_get()
        tuning_set(t)
        try:
            return _median_time(lambda: L.ignite(scene, cam, params), repeats)
        finally:
            tuning_set(before)

    measure.close = L.close
    return measure


def batch_timer(batch, repeats=2, stream=None):
    """measure(tuning) for tune(): median wall time of rt_batch_launch."""

    def measure(t):
        before = tuning_get()
        tuning_set(t)
        try:
            return _median_time(lambda: batch.launch(stream), repeats)
        finally:
            tuning_set(before)

    return measure
