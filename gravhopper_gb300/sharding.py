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
  ``run_dkd_sharded`` is the engine entry: in the mixed form it overlaps the
  all-gather with the force of the rank's own particles, then adds the others'.

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


def run_dkd_sharded(x_local, v_local, mass_all, counts, nsteps, dt, eps, precision="mixed", group=None,
                    force_fn=None):
    """Drift-kick-drift steps of one direct-sum system split by target over the ranks.

    Rank r owns particles [sum(counts[:r]), sum(counts[:r+1])) of the system (x_local,
    v_local in kpc, km/s, updated in place; mass_all all masses in rank order).  Each
    step all-gathers the half-drifted positions (N*24 bytes).

    * ``precision="mixed"``: the all-gather runs asynchronously while this rank sums the
      force of its own particles on its own targets; then the other ranks' particles
      are added.  Each part is a compensated FP32 sum; the two are added in FP64.
    * ``precision="fp64"``: one pass over all sources in ascending order after the
      gather, so the result is the reference's bits (gravhopper/_jbgrav.c:299-353 with
      the self pair's exact zero), the same as ``sharded_dkd``.

    ``force_fn(sources, masses, eps, targets)`` defaults to the GPU direct sum in
    ``precision``.  The step arithmetic is gravhopper/gravhopper.py:405-416.
    """
    import torch.distributed as dist
    force_fn = force_fn or gpu_force_fn(precision)
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    if len(counts) != world:
        raise ValueError("one particle count per rank is needed")
    start = sum(counts[:rank])
    n_local = counts[rank]
    m_local = mass_all[start:start + n_local].contiguous()
    m_remote = torch.cat([mass_all[:start], mass_all[start + n_local:]]).contiguous()
    width = max(counts) if counts else 0
    for _ in range(int(nsteps)):
        xh = x_local + ((0.5 * v_local) * dt) * KMS_MYR_TO_KPC
        if world == 1:
            acc = force_fn(xh, mass_all, eps, xh)
        else:
            buf = torch.zeros((width, 3), dtype=xh.dtype, device=xh.device)
            buf[:n_local] = xh
            parts = [torch.empty_like(buf) for _ in counts]
            work = dist.all_gather(parts, buf, group=group, async_op=True)
            if precision == "fp64":
                work.wait()
                xh_all = torch.cat([p[:c] for p, c in zip(parts, counts)])
                acc = force_fn(xh_all, mass_all, eps, xh)
            else:
                acc = force_fn(xh, m_local, eps, xh)  # overlaps the all-gather
                work.wait()
                others = [p[:c] for r, (p, c) in enumerate(zip(parts, counts)) if r != rank]
                if m_remote.shape[0]:
                    acc = acc + force_fn(torch.cat(others), m_remote, eps, xh)
        acc = acc * ACCEL_UNIT
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


__all__ = ["partition_systems", "target_slices", "sharded_dkd", "run_dkd_sharded", "gpu_force_fn", "counts_of"]
