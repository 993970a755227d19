"""Autotuner for the tile shape of the mixed-precision direct-sum kernel.

The library compiles ``gh_direct_num_shapes()`` tile shapes of the mixed kernel
(packed f32x2 and scalar FP32 pair loops, 128-512 threads, 2-8 targets per thread)
and picks one by size from a built-in table.  ``tune_direct`` times every shape on
seeded Plummer spheres of the given sizes, for a force and for a fused leapfrog step,
on the current GPU, and installs the winners as rules in the library
(``gh_direct_tune``): from each tuned size on, up to the next one, calls of that kind
use the winner.  Results are cached per GPU name, shape count, kind and size.
"""
from __future__ import annotations

import json
import math
import os
import time

import torch

from . import _capi, engine, ics

KINDS = {"force": 0, "step": 1}


def _cache_path():
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "gravhopper_gb300", "autotune.json")


def _load_cache(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def save_cache(path, cache):
    """Writes the tuning cache: a private file renamed over ``path``, so that ranks of
    one job tuning at the same time never leave a torn file behind (a reader sees the
    old cache or a whole new one).  A cache that cannot be written is skipped."""
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = f"{path}.{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1)
        os.replace(tmp, path)
    except OSError:
        pass


def _time_shape(call, shape, reps):
    _capi.call("gh_direct_set_shape", shape)
    try:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            call()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1) / reps
    finally:
        _capi.call("gh_direct_set_shape", -1)


def tune_direct(sizes=(2048, 8192, 24576, 65536, 262144, 1048576), kinds=("force", "step"), reps=1,
                device=None, use_cache=True, eps=5e-5, dt=0.005):
    """Time every tile shape at each size and kind; install and return the winners.

    Returns {kind: {n: (best_shape, {shape: ms})}}.  Each shape's kernels are loaded by
    an untimed call at a small size first, then timed over ``reps`` calls (CUDA events)
    at the full size.  Sizes between two tuned ones take the shape of the nearer one
    in log scale; sizes down to half the smallest take its shape, and smaller ones keep
    the built-in table.
    """
    dev = device or torch.device("cuda", torch.cuda.current_device())
    lib = _capi.load()
    nshape = int(lib.gh_direct_num_shapes())
    gpu = torch.cuda.get_device_name(dev)
    path = _cache_path()
    cache = _load_cache(path) if use_cache else {}
    sizes = sorted(int(n) for n in sizes)
    out = {}
    warm = ics.plummer(4096, seed=0)
    wx = torch.from_numpy(warm["pos"]).to(dev)
    wv = torch.from_numpy(warm["vel"]).to(dev)
    wm = torch.from_numpy(warm["mass"]).to(dev)
    warmed = set()
    dirty = False
    for kind in kinds:
        fused = KINDS[kind]
        out[kind] = {}
        for n in sizes:
            key = f"{gpu}|direct|{nshape} shapes|{kind}|{n}"
            if key in cache:
                ms = {int(k): v for k, v in cache[key]["ms"].items()}
            else:
                ic = ics.plummer(n, seed=n)
                x = torch.from_numpy(ic["pos"]).to(dev)
                m = torch.from_numpy(ic["mass"]).to(dev)
                if fused:
                    v = torch.from_numpy(ic["vel"]).to(dev)
                    xs, vs = x.clone(), v.clone()
                    call = lambda: engine.run_dkd(xs, vs, m, 1, dt, eps, precision="mixed")  # noqa: E731
                else:
                    call = lambda: engine.direct_force(x, m, eps, precision="mixed")  # noqa: E731
                ms = {}
                for shape in range(nshape):
                    if (kind, shape) not in warmed:  # load this shape's kernels at a small size
                        _capi.call("gh_direct_set_shape", shape)
                        try:
                            if fused:
                                engine.run_dkd(wx.clone(), wv.clone(), wm, 1, dt, eps, precision="mixed")
                            else:
                                engine.direct_force(wx, wm, eps, precision="mixed")
                        finally:
                            _capi.call("gh_direct_set_shape", -1)
                        warmed.add((kind, shape))
                    ms[shape] = _time_shape(call, shape, reps)
                cache[key] = {"ms": ms, "when": time.time()}
                dirty = True
            best = min(ms, key=ms.get)
            out[kind][n] = (best, ms)
        # install: each tuned size's winner from the log-midpoint to the previous size on
        _capi.call("gh_direct_tune", 0, fused, -1)
        for k, n in enumerate(sizes):
            n_min = n // 2 if k == 0 else int(math.sqrt(sizes[k - 1] * n)) + 1
            _capi.call("gh_direct_tune", n_min, fused, out[kind][n][0])
    if use_cache and dirty:
        save_cache(path, cache)
    return out


def clear_direct():
    """Drops the installed rules: the built-in size table applies again."""
    for fused in KINDS.values():
        _capi.call("gh_direct_tune", 0, fused, -1)


def shape_for(n, kind="force"):
    """The tile shape a mixed-precision call of ``n`` particles would use now."""
    return int(_capi.load().gh_direct_shape_for(int(n), KINDS[kind]))
