"""Multi-rank host logic on CPU with gloo (world_size 2): the target-sharded leapfrog
equals the single-process run bit for bit, and the system partition is balanced."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from gravhopper_gb300 import sharding


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _oracle_force(src, mass, eps, tgt):
    from oracle import oracle
    out = oracle.direct_summation_position(src.numpy(), mass.numpy(), tgt.numpy(), eps, nthreads=1)
    return torch.from_numpy(out)


def _worker(rank, world, port, pos, vel, mass, nsteps, out_q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        counts = sharding.counts_of(len(mass), world)
        a, b = sharding.target_slices(len(mass), world)[rank]
        x = torch.from_numpy(pos[a:b].copy())
        v = torch.from_numpy(vel[a:b].copy())
        sharding.sharded_dkd(x, v, torch.from_numpy(mass), counts, nsteps, 0.005, 5e-5, _oracle_force)
        out_q.put((rank, x.numpy(), v.numpy()))
    finally:
        dist.destroy_process_group()


def test_sharded_leapfrog_matches_single_rank():
    from gravhopper_gb300 import ics
    from oracle import oracle
    ic = ics.plummer(301, seed=4)
    nsteps, world = 5, 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, ic["pos"], ic["vel"], ic["mass"], nsteps, q))
             for r in range(world)]
    for p in procs:
        p.start()
    res = dict((r, (x, v)) for r, x, v in (q.get(timeout=120) for _ in range(world)))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    x = np.concatenate([res[r][0] for r in range(world)])
    v = np.concatenate([res[r][1] for r in range(world)])
    rx, rv = oracle.dkd_run(ic["pos"], ic["vel"], ic["mass"], 0.005, 5e-5, nsteps)
    np.testing.assert_array_equal(x, rx)
    np.testing.assert_array_equal(v, rv)


def _engine_worker(rank, world, port, pos, vel, mass, nsteps, precision, out_q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        counts = sharding.counts_of(len(mass), world)
        a, b = sharding.target_slices(len(mass), world)[rank]
        x = torch.from_numpy(pos[a:b].copy())
        v = torch.from_numpy(vel[a:b].copy())
        calls = []

        def force(src, m, eps, tgt):
            calls.append((src.shape[0], tgt.shape[0]))
            return _oracle_force(src, m, eps, tgt)

        sharding.run_dkd_sharded(x, v, torch.from_numpy(mass), counts, nsteps, 0.005, 5e-5, precision=precision,
                                 force_fn=force)
        out_q.put((rank, x.numpy(), v.numpy(), calls))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_engine_sharded_run(precision):
    """run_dkd_sharded on two gloo ranks: the FP64 form takes one ascending pass over
    all sources after the gather and equals the single-process run bit for bit; the
    mixed form first sums the rank's own particles (while the gather is in flight) and
    then the other rank's, which changes only the rounding of the FP64 sum."""
    from gravhopper_gb300 import ics
    from oracle import oracle
    ic = ics.plummer(257, seed=6)
    nsteps, world = 4, 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_engine_worker,
                         args=(r, world, port, ic["pos"], ic["vel"], ic["mass"], nsteps, precision, q))
             for r in range(world)]
    for p in procs:
        p.start()
    res = dict((r, (x, v, c)) for r, x, v, c in (q.get(timeout=120) for _ in range(world)))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    x = np.concatenate([res[r][0] for r in range(world)])
    v = np.concatenate([res[r][1] for r in range(world)])
    rx, rv = oracle.dkd_run(ic["pos"], ic["vel"], ic["mass"], 0.005, 5e-5, nsteps)
    counts = sharding.counts_of(257, world)
    for r in range(world):
        calls = res[r][2]
        if precision == "fp64":
            assert calls == [(257, counts[r])] * nsteps
        else:
            assert calls == [(counts[r], counts[r]), (257 - counts[r], counts[r])] * nsteps
    if precision == "fp64":
        np.testing.assert_array_equal(x, rx)
        np.testing.assert_array_equal(v, rv)
    else:
        np.testing.assert_allclose(x, rx, rtol=0, atol=1e-15)
        np.testing.assert_allclose(v, rv, rtol=1e-11, atol=0)


def test_engine_sharded_run_single_rank():
    """With no process group the entry runs the whole system on this process."""
    from gravhopper_gb300 import ics
    from oracle import oracle
    ic = ics.plummer(100, seed=7)
    x = torch.from_numpy(ic["pos"].copy())
    v = torch.from_numpy(ic["vel"].copy())
    sharding.run_dkd_sharded(x, v, torch.from_numpy(ic["mass"]), [100], 3, 0.005, 5e-5, precision="fp64",
                             force_fn=_oracle_force)
    rx, rv = oracle.dkd_run(ic["pos"], ic["vel"], ic["mass"], 0.005, 5e-5, 3)
    np.testing.assert_array_equal(x.numpy(), rx)
    np.testing.assert_array_equal(v.numpy(), rv)


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_partition_systems_balanced(world):
    rng = np.random.default_rng(world)
    sizes = np.exp(rng.uniform(np.log(256), np.log(8193), size=512)).astype(int)
    parts = sharding.partition_systems(sizes, world)
    assert sorted(k for p in parts for k in p) == list(range(512))
    loads = [sum(int(sizes[k]) ** 2 for k in p) for p in parts]
    assert max(loads) <= 1.02 * (sum(loads) / world) + max(sizes) ** 2


def test_target_slices_cover():
    for n in (0, 1, 7, 1000):
        for w in (1, 2, 5):
            s = sharding.target_slices(n, w)
            assert s[0][0] == 0 and s[-1][1] == n
            assert all(s[i][1] == s[i + 1][0] for i in range(w - 1))
