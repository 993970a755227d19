"""Splitting the force-and-integrate path over several ranks (one GPU each).

Two decompositions:

* Ensembles shard by system: ``partition_systems`` gives each rank a set of whole
  systems, balanced by pair count (longest-processing-time first).  There is no
  exchange at all; each rank runs ``Ensemble`` on its share.
* One direct-sum system shards by target: rank r owns a contiguous slice of particles
  and, each step, all ranks all-gather the half-drifted positions (N*24 bytes) and
  compute the forces on their own slice against every source.  ``sharded_dkd`` is
  that loop; with the FP64 force it is bit-identical to the single-GPU run, because
  the position-mode sum adds an exact zero for a particle's own term.

The Barnes-Hut path would need a distributed tree and is run as replicas only.
"""
from __future__ import annotations

import heapq

import torch

from .units import ACCEL_UNIT, KMS_MYR_TO_KPC


def partition_systems(sizes, world):
    """Assign systems to ranks, balancing sum(n^2); returns one index list per rank."""
    order = sorted(range(len(sizes)), key=lambda k: -int(sizes[k]) ** 2)
    heap = [(0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for k in order:
        load, r = heapq.heappop(heap)
        out[r].append(k)
        heapq.heappush(heap, (load + int(sizes[k]) ** 2, r))
    return [sorted(o) for o in out]


def target_slices(n, world):
    """Contiguous near-equal particle ranges [(start, stop)] for each rank."""
    bounds = [(r * n) // world for r in range(world + 1)]
    return [(bounds[r], bounds[r + 1]) for r in range(world)]


def _gather_rows(t, counts, group):
    """All-gather rank-local (n_r, 3) tensors of different lengths into (sum n_r, 3)."""
    import torch.distributed as dist
    width = max(counts)
    buf = torch.zeros((width, t.shape[1]), dtype=t.dtype, device=t.device)
    buf[: t.shape[0]] = t
    parts = [torch.empty_like(buf) for _ in counts]
    dist.all_gather(parts, buf, group=group)
    return torch.cat([p[:c] for p, c in zip(parts, counts)])


def sharded_dkd(x_local, v_local, mass_all, counts, nsteps, dt, eps, force_fn, group=None):
    """Drift-kick-drift steps of one system split by target over the ranks of ``group``.

    x_local, v_local: this rank's particles (kpc, km/s), updated in place.
    mass_all: all masses in rank order; counts: particles per rank.
    force_fn(sources, masses, eps, targets) -> code-unit accelerations at targets.
    The arithmetic is gravhopper/gravhopper.py:405-416 (as the engine's fused step).
    """
    for _ in range(int(nsteps)):
        xh = x_local + ((0.5 * v_local) * dt) * KMS_MYR_TO_KPC
        xh_all = _gather_rows(xh, counts, group)
        acc = force_fn(xh_all, mass_all, eps, xh) * ACCEL_UNIT
        v_new = v_local + acc * dt
        x_new = xh + ((0.5 * v_new) * dt) * KMS_MYR_TO_KPC
        v_local.copy_(v_new)
        x_local.copy_(x_new)
    return x_local, v_local


def gpu_force_fn(precision="fp64"):
    """Position-mode direct force on the GPU, for ``sharded_dkd``."""
    from . import engine

    def fn(src, mass, eps, tgt):
        return engine.direct_force(src.contiguous(), mass, eps, force_pos=tgt.contiguous(), precision=precision)

    return fn


def counts_of(n, world):
    return [b - a for a, b in target_slices(n, world)]


__all__ = ["partition_systems", "target_slices", "sharded_dkd", "gpu_force_fn", "counts_of"]
