"""Batched integration of many independent systems on one GPU.

``Ensemble`` packs the systems back to back in device memory and advances all of them
with one persistent kernel launch per step (``gh_ensemble_run``), the step loop
replayed from a CUDA graph.  ``autotune`` times the library's tile shapes on the
actual ensemble and caches the fastest per device and ensemble signature.
``run_one_by_one`` is the comparison: each system integrated on its own with the
single-system mixed-precision path.
"""
from __future__ import annotations

import json
import os
import time

import numpy as np
import torch

from . import _capi, engine


class Ensemble:
    """Systems given as dicts with 'pos' (N,3) [kpc], 'vel' (N,3) [km/s], 'mass' (N)
    [Msun], 'eps' [kpc] and 'dt' [Myr]."""

    def __init__(self, systems, device=None):
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        ns = np.array([len(s["mass"]) for s in systems], dtype=np.int64)
        self.offsets = np.concatenate([[0], np.cumsum(ns)]).astype(np.int64)
        self.eps = np.array([float(s["eps"]) for s in systems], dtype=np.float64)
        self.dt = np.array([float(s["dt"]) for s in systems], dtype=np.float64)
        cat = lambda k: np.ascontiguousarray(np.concatenate([np.asarray(s[k], dtype=np.float64) for s in systems]))
        self.pos = torch.from_numpy(cat("pos")).to(self.device)
        self.vel = torch.from_numpy(cat("vel")).to(self.device)
        self.mass = torch.from_numpy(cat("mass")).to(self.device)
        self.config = -1

    @property
    def nsys(self):
        return len(self.eps)

    @property
    def pairs_per_step(self):
        n = np.diff(self.offsets).astype(np.float64)
        return float(np.sum(n * (n - 1)))

    def signature(self):
        n = np.diff(self.offsets)
        return f"{self.nsys}|{int(self.offsets[-1])}|{int(n.max()) if n.size else 0}"

    def run(self, nsteps, config=None, use_graph=True, stream=None):
        cfg = self.config if config is None else config
        _capi.call("gh_ensemble_run", _capi.ptr(self.pos), _capi.ptr(self.vel), _capi.ptr(self.mass),
                   self.offsets.ctypes.data, self.nsys, self.eps.ctypes.data, self.dt.ctypes.data, int(nsteps),
                   int(cfg), 1 if use_graph else 0, _capi.stream_handle(stream))

    def system(self, k):
        a, b = int(self.offsets[k]), int(self.offsets[k + 1])
        return self.pos[a:b].cpu().numpy(), self.vel[a:b].cpu().numpy()


def _cache_path():
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "gravhopper_gb300", "autotune.json")


def autotune(ens: Ensemble, steps=4, use_cache=True):
    """Pick the fastest tile configuration for ``ens`` by timing each on a copy.

    Returns (best_config, {config: ms_per_step}).  Results are cached per device
    name and ensemble signature.
    """
    nconf = int(_capi.load().gh_ensemble_num_configs())
    key = f"{torch.cuda.get_device_name(ens.device)}|ensemble|{nconf} configs|{ens.signature()}"
    path = _cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            with open(path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
        if key in cache:
            ens.config = int(cache[key]["best"])
            return ens.config, {int(k): v for k, v in cache[key]["ms"].items()}
    saved = (ens.pos.clone(), ens.vel.clone())
    times = {}
    for cfg in range(nconf):
        ens.pos.copy_(saved[0])
        ens.vel.copy_(saved[1])
        ens.run(1, config=cfg, use_graph=False)  # warm-up
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        ens.run(steps, config=cfg, use_graph=False)
        e1.record()
        e1.synchronize()
        times[cfg] = e0.elapsed_time(e1) / steps
    ens.pos.copy_(saved[0])
    ens.vel.copy_(saved[1])
    best = min(times, key=times.get)
    ens.config = best
    if use_cache:
        cache[key] = {"best": best, "ms": times, "when": time.time()}
        from .autotune import save_cache
        save_cache(path, cache)
    return best, times


def run_one_by_one(ens: Ensemble, nsteps, precision="mixed"):
    """Advance each system separately with the single-system path (the baseline)."""
    for k in range(ens.nsys):
        a, b = int(ens.offsets[k]), int(ens.offsets[k + 1])
        x, v = ens.pos[a:b], ens.vel[a:b]
        engine.run_dkd(x, v, ens.mass[a:b], nsteps, float(ens.dt[k]), float(ens.eps[k]), algorithm="direct",
                       precision=precision)
