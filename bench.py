#!/usr/bin/env python3
"""Benchmark of the GravHopper force-and-integrate path on GB300.

Default workload: one drift-kick-drift leapfrog step of an equal-mass Plummer sphere
with N = 1,048,576 particles (b = 1 pc, M = 1e6 Msun, eps = 0.05 pc, dt = 0.005 Myr),
direct-sum force in the mixed form (FP32 pair arithmetic, compensated accumulation,
FP64 state), one fused kernel launch per step.  A step is N*(N-1) pair interactions;
``value`` is pair interactions per second in Gpair/s with the state resident in HBM,
the L2 cache flushed before every timed step.

Also reported on the same line:
* ``e2e``: the same force through the reference-facing C-ABI call with host buffers
  (``gh_direct_host``: pinned host -> device copy, force, device -> host copy),
* ``roofline``: the mixed kernel against the FP32 FMA-pipe peak measured live
  (12 FMA-pipe lane-ops per pair),
* ``secondary``: the mixed form's error against the FP64 form on sampled targets,
  energy drift, the tree, ensemble and adjoint measurements in detail,
* ``tree``: particle-steps/s of tree DKD steps (Hernquist + disk, N = 1,048,576,
  theta 0.7 and 0.5, mixed and FP64 walks) beside the reference tree on the host cores,
* ``fp64``: the precision-matched number, the FP64 form (the reference's operation
  order, bit-identical results) in Gpair/s at N = 262,144, with its FP64-pipe
  fraction and its ratio to ``cpu_baseline``,
* ``cpu_baseline``: the CPU oracle (a restatement of the reference's C loops) on the
  host cores, on a bounded sample of targets.

``--impl reference`` times that CPU implementation alone on the same metric.
Under torchrun with N > 1, every rank runs its own system (replicas; weak scaling);
with ``--shard targets`` the ranks split one system by target and all-gather the
half-drifted positions every step (strong scaling; the mixed form overlaps the gather
with the force of the rank's own particles).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Direct-sum Gpair/s & tree particle-steps/s, mixed vs FP64, 1 GB300 @ <=1e-6 err"
UNIT = "Gpair/s"
PAIR_OPS = 12  # FP32 FMA-pipe lane-ops per pair: 3 sub, 3 fma, 3 mul, 3 fma
PAIR_OPS_EQ = 11  # the same with equal masses: the mass is applied once per target
PAIR_OPS_FP64 = 12  # FP64-pipe ops per pair of the FP64 form: 3 sub, 6 mul, 3 add


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=1 << 20)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--no-secondary", action="store_true")
    ap.add_argument("--shard", default="replicas", choices=["replicas", "targets"],
                    help="N>1: one system per rank (weak scaling) or one system split by target "
                         "over the ranks, positions all-gathered each step (strong scaling)")
    ap.add_argument("--cpu-targets", type=int, default=49152,
                    help="targets in the CPU-baseline sample (each against all N sources)")
    ap.add_argument("--report", choices=["config0", "config1", "config2", "config3", "config4", "config4tangent"],
                    help="print one JSON line of the full measurements for that workload instead")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms in the background."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.rows = []
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.gpu)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows),
                "power_w_max": max((float(r[3]) for r in self.rows
                                    if r[3].replace(".", "").isdigit()), default=None)}


def cpu_baseline(n, targets, seed=0):
    """Oracle direct sum (the reference's loop order, FP64) on a sample of targets."""
    import numpy as np

    from gravhopper_gb300 import ics
    from oracle import oracle
    ic = ics.plummer(n, seed=seed)
    rng = np.random.default_rng(1)
    idx = rng.choice(n, size=min(targets, n), replace=False)
    threads = oracle.default_threads()
    oracle.direct_summation_position(ic["pos"], ic["mass"], ic["pos"][idx[:64]], 5e-5, nthreads=threads)
    t0 = time.perf_counter()
    oracle.direct_summation_position(ic["pos"], ic["mass"], ic["pos"][idx], 5e-5, nthreads=threads)
    dt = time.perf_counter() - t0
    pairs = float(len(idx)) * n
    return {"value": pairs / dt / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{len(idx)} targets x {n} sources (FP64, reference loop order), {dt:.2f} s"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    res = []
    for k in range(args.warmup + args.steps):
        r = cpu_baseline(args.n, max(64, min(args.cpu_targets, 8192) // 2), seed=k)  # ~0.4 s per step
        if k >= args.warmup:
            res.append(r)
    val = statistics.median(r["value"] for r in res)
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(args.n) * (args.n - 1) / (val * 1e9) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": _config(args),
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": res[0]["cores"], "kind": "port",
                             "sample": res[0]["sample"] + " per step; ms_per_step extrapolates to N*(N-1)"},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _config(args, world=1):
    shard = getattr(args, "shard", "replicas") == "targets"
    return {"workload": f"direct-sum DKD leapfrog step, Plummer sphere N={args.n} (b=1 pc, M=1e6 Msun, "
                        f"eps=0.05 pc, dt=0.005 Myr)",
            "precision": args.precision, "n": args.n, "pairs_per_step": args.n * (args.n - 1),
            "l2": "flushed (256 MB write) before every timed step",
            "parallelism": f"targets split over {world} ranks" if shard else "replicas"}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.report:
        import torch
        dev = torch.device("cuda", 0)
        torch.cuda.set_device(0)
        fn = {"config0": report_config0, "config1": report_config1, "config2": report_config2,
              "config3": report_config3, "config4": report_config4,
              "config4tangent": report_config4_tangent}[args.report]
        print(json.dumps({"report": args.report, **fn(dev)}), flush=True)
        return
    import numpy as np
    import torch

    from gravhopper_gb300 import _capi, engine, ics

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    _capi.load()
    n = args.n
    shard = args.shard == "targets"
    ic = ics.plummer(n, seed=0 if shard else rank)
    x = torch.from_numpy(ic["pos"]).to(dev)
    v = torch.from_numpy(ic["vel"]).to(dev)
    m = torch.from_numpy(ic["mass"]).to(dev)
    eps, dt = 5e-5, 0.005
    stream = torch.cuda.current_stream()
    fp32_peak, fp64_peak = _capi.measure_fma_peaks()
    # equal masses (as the Plummer spheres here) run the kernel's equal-mass loop
    equal_mass = bool(np.all(ic["mass"] == ic["mass"][0]) and ic["mass"][0] != 0)
    pair_ops = PAIR_OPS_EQ if equal_mass else PAIR_OPS
    # the pair's instruction mix with operands in registers
    mix_ceiling = _capi.measure_pair_mix(equal_mass=equal_mass)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def step():
        engine.run_dkd(x, v, m, 1, dt, eps, algorithm="direct", precision=args.precision)

    if shard:
        # one system split by target: this rank's slice, all masses, positions gathered per step
        from gravhopper_gb300 import sharding
        counts = sharding.counts_of(n, world)
        lo_, hi_ = sharding.target_slices(n, world)[rank]
        x = x[lo_:hi_].contiguous()
        v = v[lo_:hi_].contiguous()

        def step():  # noqa: F811
            sharding.run_dkd_sharded(x, v, m, counts, 1, dt, eps, precision=args.precision)

    tuned = None
    if args.precision == "mixed" and not shard:
        # the tile shapes of this size's fused step (the timed step) and force (the
        # end-to-end call), picked by timing every shape (untimed here)
        from gravhopper_gb300 import autotune
        res = autotune.tune_direct(sizes=(n,), kinds=("step", "force"), device=dev)
        best, ms = res["step"][n]
        fbest, fms = res["force"][n]
        tuned = {"shape": best, "ms_per_step_by_shape": {k: round(t, 2) for k, t in ms.items()},
                 "force_shape": fbest, "ms_per_force_by_shape": {k: round(t, 2) for k, t in fms.items()}}

    for _ in range(args.warmup):
        step()
    barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    _capi.kernel_timing_collect()
    _capi.kernel_timing(True)
    launches0 = _capi.launch_count()
    with ClockSampler(local) as clocks:
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            step()
            ev[k][1].record(stream)
        barrier()
    launches = _capi.launch_count() - launches0
    _capi.kernel_timing(False)
    kern_ms, kern_n = _capi.kernel_timing_collect()
    step_ms = sum(a.elapsed_time(b) for a, b in ev)
    t = torch.tensor([step_ms], dtype=torch.float64, device=dev)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    step_ms_max = float(t.item())
    pairs = float(n) * (n - 1)
    value = (1 if shard else world) * pairs * args.steps / (step_ms_max * 1e-3) / 1e9

    # End to end through the host-buffer C ABI (pinned host memory, copies timed).
    hp = torch.from_numpy(ic["pos"]).pin_memory()
    hm = torch.from_numpy(ic["mass"]).pin_memory()
    ho = torch.empty((n, 3), dtype=torch.float64).pin_memory()
    prec = _capi.PRECISIONS[args.precision]
    e2e_steps = max(1, min(args.steps, 5))
    _capi.call("gh_direct_host", hp.data_ptr(), hm.data_ptr(), n, None, 0, eps, prec, ho.data_ptr())
    barrier()
    e2e_s = 0.0
    for _ in range(e2e_steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _capi.call("gh_direct_host", hp.data_ptr(), hm.data_ptr(), n, None, 0, eps, prec, ho.data_ptr())
        e2e_s += time.perf_counter() - t0
    e2e = {"value": world * pairs * e2e_steps / e2e_s / 1e9, "unit": UNIT,
           "h2d_bytes_per_step": n * 3 * 8 + n * 8, "d2h_bytes_per_step": n * 3 * 8}
    if tuned is not None:
        from gravhopper_gb300 import autotune
        autotune.clear_direct()  # the other measurements use the library's own size table

    kern_avg_s = kern_ms / max(kern_n, 1) * 1e-3
    # pairs one force launch evaluates (sharded: this rank's targets, own and others' sources)
    achieved = (pairs if not shard else float(x.shape[0]) * n * args.steps / max(kern_n, 1)) / kern_avg_s / 1e9
    mixed = args.precision == "mixed"
    # mixed: 12 FP32 FMA-pipe lane-ops per pair (11 with equal masses); FP64: the 12 of
    # the reference's pair operations that stay on the FP64 pipe (squared distance,
    # division and square root run as exact integer arithmetic)
    peak = (fp32_peak if mixed else fp64_peak) / (pair_ops if mixed else PAIR_OPS_FP64) / 1e9
    # DRAM bytes (read + write) of one launch of the fused DKD kernel at N = 1,048,576,
    # from one single-pass ncu capture (dram__bytes_read.sum 78.47 MB + write 29.32 MB;
    # profiles/direct_mixed_bench_n1048576_launches.md); other sizes: not captured
    traffic = 107.79e6 if (args.precision == "mixed" and n == 1 << 20) else None
    roofline = {"bound": "fp32" if mixed else "fp64",
                "kernel": "direct_mixed_kernel" if mixed else "direct_f64_kernel",
                "achieved": achieved, "peak": peak, "unit": UNIT,
                "frac": achieved / peak, "traffic": traffic,
                "peak_source": (f"measured live: f32x2 FMA chains, {fp32_peak / 1e12:.1f} T lane-op/s "
                                f"/ {pair_ops} lane-ops per pair"
                                + (" (equal masses: no per-pair mass multiply)" if equal_mass else ""))
                               if mixed else
                               (f"measured live: FP64 FMA chains, {fp64_peak / 1e12:.2f} T lane-op/s "
                                f"/ {PAIR_OPS_FP64} FP64-pipe ops per pair"),
                "tflops_20_per_pair": achieved * 20 / 1e3, "kernel_launches_timed": kern_n}
    if mixed:
        # what the same FMA-pipe instructions (12, or 11 with equal masses) and one MUFU
        # per pair reach with every operand in registers (gh_measure_pair_mix): the
        # mix's own ceiling
        roofline["mix_ceiling"] = {"value": mix_ceiling / 1e9, "unit": UNIT, "frac": achieved / (mix_ceiling / 1e9),
                                   "of_fma_peak": mix_ceiling / 1e9 / peak}

    secondary, fp64 = {}, None
    if not args.no_secondary and rank == 0:
        secondary = measure_secondary(ic, dev, fp64_peak)
        fp64 = measure_fp64(dev, fp64_peak)

    if rank == 0:
        # long detail first, the headline extras last (a reader of the line's tail sees them)
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": step_ms_max / args.steps, "higher_is_better": True,
                "scaling": "strong" if shard else "weak", "vs_baseline": None,
                "dtype": "f32" if args.precision == "mixed" else "f64",
                "data": "synthetic", "config": {**_config(args, world), "tile_autotune": tuned},
                "roofline": roofline,
                "clocks": clocks.summary(), "e2e": e2e, "gpu_launches": launches,
                "secondary": _rounded(secondary)}
        if secondary.get("tree"):
            line["tree"] = tree_summary(secondary["tree"])
        cpu = cpu_baseline(n, args.cpu_targets)
        if fp64:
            fp64["vs_cpu_baseline"] = fp64["value"] / cpu["value"]
            if args.precision == "mixed":
                fp64["mixed_over_fp64"] = achieved / fp64["value"]
            line["fp64"] = _rounded(fp64)
        line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def _rounded(obj, digits=4):
    """The same structure with floats rounded to `digits` significant digits."""
    if isinstance(obj, float):
        return float(f"{obj:.{digits}g}")
    if isinstance(obj, dict):
        return {k: _rounded(v, digits) for k, v in obj.items()}
    if isinstance(obj, (list, tuple)):
        return [_rounded(v, digits) for v in obj]
    return obj


def measure_fp64(dev, fp64_peak, n=262144, reps=2):
    """The FP64 form (the reference's per-pair operation order, bit-identical results):
    Gpair/s of the self-force of the N = 262,144 Plummer sphere, kernel-timed over
    `reps` calls after one warm-up, and its fraction of the FP64 pipe measured live
    (12 of the reference's pair operations stay on that pipe)."""
    import torch

    from gravhopper_gb300 import _capi, engine, ics
    s = ics.plummer(n, seed=7)
    xs = torch.from_numpy(s["pos"]).to(dev)
    ms_ = torch.from_numpy(s["mass"]).to(dev)
    engine.direct_force(xs, ms_, 5e-5, precision="fp64")
    torch.cuda.synchronize()
    _capi.kernel_timing_collect()
    _capi.kernel_timing(True)
    for _ in range(reps):
        engine.direct_force(xs, ms_, 5e-5, precision="fp64")
    _capi.kernel_timing(False)
    kms, kn = _capi.kernel_timing_collect()
    sec = kms / max(kn, 1) * 1e-3
    g64 = float(n) * (n - 1) / sec / 1e9
    return {"workload": f"FP64 direct-sum self-force, Plummer sphere N={n} (bit-identical to the reference)",
            "value": g64, "unit": UNIT, "ms_per_force": sec * 1e3, "forces_timed": kn,
            "fp64_pipe_frac": g64 * 1e9 * PAIR_OPS_FP64 / fp64_peak,
            "peak_source": f"measured live: FP64 FMA chains, {fp64_peak / 1e12:.3f} T lane-op/s / "
                           f"{PAIR_OPS_FP64} FP64-pipe ops per pair"}


def tree_summary(tree):
    """Particle-steps/s of the tree steps, with the reference tree on the host cores."""
    out = {"workload": f"tree DKD steps, Hernquist+disk N={tree['n']}", "unit": "particle-steps/s"}
    for key in ("theta_0.7", "theta_0.5"):
        t = tree.get(key, {})
        row = {p: float(f"{t[p]['particle_steps_per_s']:.4g}") for p in ("mixed", "fp64") if p in t}
        if "fp64_pipe_frac" in t.get("fp64", {}):
            row["fp64_walk_pipe_frac"] = float(f"{t['fp64']['fp64_pipe_frac']:.3g}")
        if "cpu_reference_s_per_step" in t:
            row["cpu_reference"] = float(f"{tree['n'] / t['cpu_reference_s_per_step']:.4g}")
            row["cpu_cores"] = t["cpu_reference_cores"]
        out[key] = row
    return out


def measure_secondary(ic, dev, fp64_peak=None):
    """Mixed-form accuracy, energy drift, tree, ensemble and adjoint on this GPU."""
    import numpy as np
    import torch

    from gravhopper_gb300 import engine
    out = {}
    # Mixed-form error against the FP64 form (bit-identical to the oracle) on 4096
    # sampled targets of the N = 1,048,576 system.
    n = ic["pos"].shape[0]
    rng = np.random.default_rng(2)
    idx = torch.from_numpy(rng.choice(n, size=min(4096, n), replace=False)).to(dev)
    x = torch.from_numpy(ic["pos"]).to(dev)
    m = torch.from_numpy(ic["mass"]).to(dev)
    a_mixed = engine.direct_force(x, m, 5e-5, precision="mixed")[idx]
    a64 = engine.direct_force(x, m, 5e-5, force_pos=x[idx].contiguous(), precision="fp64")
    err = torch.linalg.norm(a_mixed - a64, dim=1) / torch.linalg.norm(a64, dim=1)
    out["mixed_rel_err_rms"] = float(torch.sqrt(torch.mean(err * err)))
    out["mixed_rel_err_max"] = float(err.max())
    out["mixed_err_sample"] = f"{idx.numel()} targets of N={n} vs FP64 form"
    del x, m, a_mixed, a64
    out["energy_drift_10_steps"] = measure_energy_drift(dev)
    out["tree"] = measure_tree(dev, fp64_peak=fp64_peak)
    out["ensemble"] = measure_ensemble(dev)
    out["adjoint"] = measure_adjoint(dev)
    return out


def _timed(fn):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fn()
    torch.cuda.synchronize()
    return time.perf_counter() - t0


def measure_energy_drift(dev, n=262144, steps=10):
    """Config-1 energy drift |E(10) - E(0)| / |E(0)| for both forms (FP64 energies)."""
    import torch

    from gravhopper_gb300 import engine, ics
    ic = ics.plummer(n, seed=5)
    m = torch.from_numpy(ic["mass"]).to(dev)
    out = {"n": n, "steps": steps}
    e0 = None
    for prec in ("fp64", "mixed"):
        x = torch.from_numpy(ic["pos"]).to(dev)
        v = torch.from_numpy(ic["vel"]).to(dev)
        if e0 is None:
            e0 = engine.energy(x, v, m, 5e-5)[2]
        engine.run_dkd(x, v, m, steps, 0.005, 5e-5, algorithm="direct", precision=prec)
        out[prec] = abs(engine.energy(x, v, m, 5e-5)[2] - e0) / abs(e0)
    return out


def measure_tree(dev, n=1 << 20, steps=2, fp64_peak=None):
    """Config 2: Hernquist + exponential disk, particle-steps/s of DKD steps with the tree.
    For the FP64 walk also its FP64-pipe fraction: 10 FP64-pipe operations per
    interaction (3 differences, 3 FMAs for r^2, one product, 3 accumulating FMAs) over
    the timed walk, against the FP64 peak measured in the same process."""
    import numpy as np
    import torch

    from gravhopper_gb300 import _capi, engine, ics
    from oracle import oracle
    ic = ics.hernquist_disk(n, seed=1)
    m = torch.from_numpy(ic["mass"]).to(dev)
    l2 = _capi.measure_l2_read()
    out = {"n": n, "workload": "Hernquist (70%) + exponential disk (30%), 1e11 Msun, eps=0.1 kpc, dt=0.5 Myr",
           "l2_read_gbs_measured": l2 / 1e9}
    for theta in (0.7, 0.5):
        key = f"theta_{theta}"
        out[key] = {}
        for prec in ("mixed", "fp64"):
            x = torch.from_numpy(ic["pos"]).to(dev)
            v = torch.from_numpy(ic["vel"]).to(dev)
            # warm-up with the timed call's own step count (every kernel variant loaded)
            engine.run_dkd(x, v, m, steps, 0.5, 0.1, algorithm="tree", theta=theta, precision=prec)
            torch.cuda.synchronize()
            _capi.kernel_timing_collect()
            _capi.kernel_timing(True)
            t = _timed(lambda: engine.run_dkd(x, v, m, steps, 0.5, 0.1, algorithm="tree", theta=theta,
                                              precision=prec))
            _capi.kernel_timing(False)
            walk_ms, walks = _capi.kernel_timing_collect()
            walk_s = walk_ms / max(walks, 1) * 1e-3
            # one more step with the walk counters on (not timed)
            _capi.tree_stats_read()
            _capi.tree_stats(True)
            engine.run_dkd(x, v, m, 1, 0.5, 0.1, algorithm="tree", theta=theta, precision=prec)
            _capi.tree_stats(False)
            c = _capi.tree_stats_read()
            rec_bytes = 48 * c["cell_steps"]  # one 48-byte cell record per warp step
            out[key][prec] = {"particle_steps_per_s": n * steps / t, "ms_per_step": t / steps * 1e3,
                              "walk_ms_per_step": walk_s * 1e3,
                              "build_ms_per_step": t / steps * 1e3 - walk_s * 1e3,
                              "interactions_per_target": c["interactions"] / n,
                              "cells_visited_per_target": c["target_visits"] / n,
                              "exact_tests_per_target": c["exact_tests"] / n,
                              "leaf_interactions_per_target": c["leaf_interactions"] / n,
                              "warp_cell_steps": c["cell_steps"],
                              "single_child_step_frac": c["chain_steps"] / max(c["cell_steps"], 1),
                              "record_bytes_per_walk": rec_bytes,
                              "record_read_gbs": rec_bytes / walk_s / 1e9,
                              "record_read_frac_of_measured_l2": rec_bytes / walk_s / l2,
                              "per_target_record_gbs": 48 * c["target_visits"] / walk_s / 1e9}
            if prec == "fp64" and fp64_peak:
                out[key][prec]["fp64_pipe_frac"] = 10.0 * c["interactions"] / walk_s / fp64_peak
    # CPU reference tree (the oracle restatement of _jbgrav.c) on a sample of targets:
    # its serial build plus the threaded walk of 16384 targets scaled to all N targets
    # (the faster of two calls).
    rng = np.random.default_rng(0)
    idx = rng.choice(n, size=16384, replace=False)
    for theta in (0.7, 0.5):
        best = None
        for _ in range(2):
            tt = [0.0, 0.0]
            oracle.tree_force_position(ic["pos"], ic["mass"], ic["pos"][idx], 0.1, theta,
                                       nthreads=oracle.default_threads(), times=tt)
            best = tt if best is None else [min(best[0], tt[0]), min(best[1], tt[1])]
        out[f"theta_{theta}"]["cpu_reference_s_per_step"] = best[0] + best[1] * n / idx.size
        out[f"theta_{theta}"]["cpu_reference_build_s"] = best[0]
        out[f"theta_{theta}"]["cpu_reference_sample"] = f"build + walk of {idx.size} targets x N / {idx.size}"
        out[f"theta_{theta}"]["cpu_reference_cores"] = oracle.default_threads()
    return out


def measure_ensemble(dev, steps=50, loop_steps=10):
    """Config 3: 512 Plummer spheres, N log-uniform in [256, 8192], one persistent launch
    per step replayed from a CUDA graph, against integrating the systems one by one."""
    from gravhopper_gb300 import ics
    from gravhopper_gb300.ensemble import Ensemble, autotune, run_one_by_one
    systems = ics.plummer_ensemble(512, seed=0)
    e = Ensemble(systems, device=dev)
    best, times = autotune(e, steps=2, use_cache=False)
    e.run(2)
    t = _timed(lambda: e.run(steps, use_graph=True))
    f = Ensemble(systems, device=dev)
    run_one_by_one(f, 1)
    tl = _timed(lambda: run_one_by_one(f, loop_steps))
    pairs = e.pairs_per_step
    return {"systems": 512, "particles": int(e.offsets[-1]), "pairs_per_step": pairs, "tile_config": best,
            "ms_per_step": t / steps * 1e3, "gpair_s": pairs / (t / steps) / 1e9,
            "one_by_one_ms_per_step": tl / loop_steps * 1e3, "speedup_vs_one_by_one": (tl / loop_steps) / (t / steps)}


def measure_adjoint(dev, n=16384, steps=200):
    """Config 4: gradients of a 200-step mixed rollout (checkpoints every 20 steps)
    with respect to x0, v0 and m; backward time over forward time."""
    import numpy as np
    import torch

    from gravhopper_gb300 import engine, ics
    from gravhopper_gb300.adjoint import rollout
    ic = ics.plummer(n, seed=0)
    rng = np.random.default_rng(1)
    x0 = torch.from_numpy(ic["pos"]).to(dev)
    v0 = torch.from_numpy(ic["vel"]).to(dev)
    m = torch.from_numpy(ic["mass"]).to(dev)
    xt = (x0 * torch.from_numpy(1 + 1e-3 * rng.normal(size=ic["pos"].shape)).to(dev)).contiguous()
    vt = (v0 * torch.from_numpy(1 + 1e-3 * rng.normal(size=ic["vel"].shape)).to(dev)).contiguous()
    engine.run_dkd(xt, vt, m, steps, 0.005, 5e-5, precision="mixed")
    out = {"n": n, "steps": steps}
    for k in (20, 1):
        for rep in range(2):  # first repetition warms up
            xa, va, ma = (t.clone().requires_grad_(True) for t in (x0, v0, m))
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            xT, _ = rollout(xa, va, ma, steps, 0.005, 5e-5, checkpoint_every=k, precision="mixed")
            loss = ((xT - xt) ** 2).mean()
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            loss.backward()
            torch.cuda.synchronize()
            t2 = time.perf_counter()
        out[f"checkpoint_{k}"] = {"forward_ms": (t1 - t0) * 1e3, "backward_ms": (t2 - t1) * 1e3,
                                  "backward_over_forward": (t2 - t1) / (t1 - t0)}
    return out


def report_config0(dev):
    """The reference's own example: Plummer N=2000, 400 DKD steps through Simulation.run."""
    import numpy as np

    import gravhopper_gb300 as gh
    from gravhopper_gb300 import ics
    from oracle import oracle
    ic = ics.plummer(2000, b=1e-3, totmass=1e6, seed=0)
    out = {"n": 2000, "steps": 400}
    e0 = oracle.total_energy(ic["pos"], ic["vel"], ic["mass"], 5e-5)
    for prec in ("fp64", "mixed"):
        sim = gh.Simulation(dt=0.005, eps=5e-5, algorithm="direct", precision=prec)
        sim.add_IC(ic)
        sim.run(2)
        sim = gh.Simulation(dt=0.005, eps=5e-5, algorithm="direct", precision=prec)
        sim.add_IC(ic)
        t = _timed(lambda: sim.run(400))
        e1 = oracle.total_energy(sim._pos[400], sim._vel[400], ic["mass"], 5e-5)
        out[prec] = {"run_s": t, "steps_per_s": 400 / t, "energy_drift": (e1 - e0) / abs(e0)}
    t0 = time.perf_counter()
    rx, rv = oracle.dkd_run(ic["pos"], ic["vel"], ic["mass"], 0.005, 5e-5, 400)
    out["cpu_oracle_run_s"] = time.perf_counter() - t0
    out["cpu_oracle_cores"] = oracle.default_threads()
    sim = gh.Simulation(dt=0.005, eps=5e-5, algorithm="direct", precision="fp64")
    sim.add_IC(ic)
    sim.run(400)
    out["fp64_final_state_equals_oracle"] = bool(np.array_equal(sim._pos[400], rx) and
                                                 np.array_equal(sim._vel[400], rv))
    return out


def report_config1(dev):
    """Plummer N = 65,536 / 262,144 / 1,048,576, 10 DKD steps, FP64 and mixed: Gpair/s,
    relative acceleration error (4096 sampled targets against the FP64 form, which is
    bit-identical to the reference) and energy drift (FP64 energies)."""
    import numpy as np
    import torch

    from gravhopper_gb300 import engine, ics
    out = {}
    for n in (65536, 262144, 1 << 20):
        ic = ics.plummer(n, seed=11)
        m = torch.from_numpy(ic["mass"]).to(dev)
        x0 = torch.from_numpy(ic["pos"]).to(dev)
        v0 = torch.from_numpy(ic["vel"]).to(dev)
        rng = np.random.default_rng(3)
        idx = torch.from_numpy(rng.choice(n, size=4096, replace=False)).to(dev)
        a64 = engine.direct_force(x0, m, 5e-5, force_pos=x0[idx].contiguous(), precision="fp64")
        am = engine.direct_force(x0, m, 5e-5, precision="mixed")[idx]
        err = torch.linalg.norm(am - a64, dim=1) / torch.linalg.norm(a64, dim=1)
        e0 = engine.energy(x0, v0, m, 5e-5)[2]
        row = {"rel_err_rms": float(torch.sqrt(torch.mean(err * err))), "rel_err_max": float(err.max())}
        pairs = float(n) * (n - 1)
        for prec in ("mixed", "fp64"):
            steps = 10 if (prec == "mixed" or n <= 262144) else 1
            x, v = x0.clone(), v0.clone()
            t = _timed(lambda: engine.run_dkd(x, v, m, steps, 0.005, 5e-5, precision=prec))
            r = {"steps": steps, "ms_per_step": t / steps * 1e3, "gpair_s": pairs * steps / t / 1e9}
            if steps == 10:
                r["energy_drift_10_steps"] = abs(engine.energy(x, v, m, 5e-5)[2] - e0) / abs(e0)
            row[prec] = r
        row["mixed_over_fp64"] = row["mixed"]["gpair_s"] / row["fp64"]["gpair_s"]
        out[f"n_{n}"] = row
    return out


def report_config2(dev, n=1 << 20, steps=100):
    """Hernquist + exponential disk, N = 1,048,576: 100 DKD steps through
    Simulation.run with the tree at theta 0.7 and 0.5 (mixed and FP64 walks), and the
    force's error against the oracle tree (the reference's algorithm) on 2048 sampled
    targets of the initial state."""
    import numpy as np
    import torch

    import gravhopper_gb300 as gh
    from gravhopper_gb300 import engine, ics
    from oracle import oracle
    ic = ics.hernquist_disk(n, seed=1)
    rng = np.random.default_rng(4)
    idx = rng.choice(n, size=2048, replace=False)
    x = torch.from_numpy(ic["pos"]).to(dev)
    m = torch.from_numpy(ic["mass"]).to(dev)
    out = {"n": n, "steps": steps}
    for theta in (0.7, 0.5):
        ref = oracle.tree_force_position(ic["pos"], ic["mass"], ic["pos"][idx], 0.1, theta)
        row = {}
        for prec in ("mixed", "fp64"):
            got = engine.tree_force(x, m, 0.1, theta, force_pos=x[torch.from_numpy(idx).to(dev)].contiguous(),
                                    precision=prec).cpu().numpy()
            r = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
            sim = gh.Simulation(dt=0.5, eps=0.1, algorithm="tree", theta=theta, precision=prec)
            sim.add_IC(ic)
            t = _timed(lambda: sim.run(steps))
            row[prec] = {"run_s": t, "particle_steps_per_s": n * steps / t, "rel_err_rms": float(np.sqrt(np.mean(r * r))),
                         "rel_err_max": float(r.max())}
        out[f"theta_{theta}"] = row
    return out


def report_config3(dev, steps=1000, loop_steps=20):
    """512 Plummer spheres (N log-uniform in [256, 8192], b in [0.5, 2] pc, eps = 0.05 b,
    dt = 0.005 Myr (b / pc)^1.5): 1000 mixed steps in one persistent launch per step from
    a CUDA graph with the autotuned tiles, against integrating the systems one by one;
    relative energy drift of every system (FP64 energies)."""
    import numpy as np
    import torch

    from gravhopper_gb300 import engine, ics
    from gravhopper_gb300.ensemble import Ensemble, autotune, run_one_by_one
    systems = ics.plummer_ensemble(512, seed=0)
    e = Ensemble(systems, device=dev)

    def energies(ens):
        out = []
        for k in range(ens.nsys):
            a, b = int(ens.offsets[k]), int(ens.offsets[k + 1])
            out.append(engine.energy(ens.pos[a:b].contiguous(), ens.vel[a:b].contiguous(),
                                     ens.mass[a:b].contiguous(), float(ens.eps[k]))[2])
        return np.array(out)

    best, _ = autotune(e, steps=4, use_cache=False)
    e0 = energies(e)
    t = _timed(lambda: e.run(steps, use_graph=True))
    drift = np.abs(energies(e) - e0) / np.abs(e0)
    f = Ensemble(systems, device=dev)
    run_one_by_one(f, 1)
    tl = _timed(lambda: run_one_by_one(f, loop_steps))
    # the same drift measured on 16 of the systems integrated alone in FP64
    sample = np.linspace(0, e.nsys - 1, 16).astype(int)
    d64 = []
    for k in sample:
        sysk = systems[int(k)]
        x = torch.from_numpy(np.ascontiguousarray(sysk["pos"])).to(dev)
        v = torch.from_numpy(np.ascontiguousarray(sysk["vel"])).to(dev)
        m = torch.from_numpy(np.ascontiguousarray(sysk["mass"])).to(dev)
        ea = engine.energy(x, v, m, float(sysk["eps"]))[2]
        engine.run_dkd(x, v, m, steps, float(sysk["dt"]), float(sysk["eps"]), precision="fp64")
        d64.append(abs(engine.energy(x, v, m, float(sysk["eps"]))[2] - ea) / abs(ea))
    pairs = e.pairs_per_step
    return {"systems": e.nsys, "particles": int(e.offsets[-1]), "steps": steps, "tile_config": best,
            "run_s": t, "ms_per_step": t / steps * 1e3, "gpair_s": pairs * steps / t / 1e9,
            "one_by_one_ms_per_step": tl / loop_steps * 1e3, "speedup_vs_one_by_one": (tl / loop_steps) / (t / steps),
            "energy_drift_median": float(np.median(drift)), "energy_drift_max": float(drift.max()),
            "sample_systems": [int(k) for k in sample],
            "sample_drift_ensemble": [float(drift[k]) for k in sample], "sample_drift_fp64_alone": d64}


def report_config4(dev, n=16384):
    """Adjoint gradients with respect to x0 against FP64 central finite differences
    (FP64 rollouts, N = 16,384, 64 random coordinates each): over 20 steps, over 100
    steps with checkpoints every 20, and over the full 200-step rollout with
    checkpoints every 20, where the differences at h = 3e-10, 1e-10, 3e-11 kpc are also
    extrapolated twice (Richardson: the h^2 and h^4 terms cancel)."""
    import numpy as np
    import torch

    from gravhopper_gb300 import engine, ics
    from gravhopper_gb300.adjoint import rollout
    ic = ics.plummer(n, seed=0)
    x0 = torch.from_numpy(ic["pos"]).to(dev)
    v0 = torch.from_numpy(ic["vel"]).to(dev)
    m = torch.from_numpy(ic["mass"]).to(dev)
    out = {"n": n}
    for steps, ncoord, ckpt, hs in ((20, 64, 5, (1e-9,)), (100, 64, 20, (3e-10,)),
                                    (200, 64, 20, (3e-10, 1e-10, 3e-11))):
        rng = np.random.default_rng(1)
        xt = (x0 * torch.from_numpy(1 + 1e-3 * rng.normal(size=ic["pos"].shape)).to(dev)).contiguous()
        vt = (v0 * torch.from_numpy(1 + 1e-3 * rng.normal(size=ic["vel"].shape)).to(dev)).contiguous()
        engine.run_dkd(xt, vt, m, steps, 0.005, 5e-5, precision="fp64")
        xa = x0.clone().requires_grad_(True)
        xT, _ = rollout(xa, v0, m, steps, 0.005, 5e-5, checkpoint_every=ckpt, precision="fp64")
        ((xT - xt) ** 2).mean().backward()
        g = xa.grad.reshape(-1).cpu().numpy()

        def loss_at(xp):
            x, v = xp.reshape(-1, 3).clone(), v0.clone()
            engine.run_dkd(x, v, m, steps, 0.005, 5e-5, precision="fp64")
            return float(((x - xt) ** 2).mean())

        idx = rng.choice(3 * n, size=ncoord, replace=False)
        flat = x0.reshape(-1)
        row = {"coordinates": ncoord, "checkpoint_every": ckpt}
        den = np.maximum(np.abs(g[idx]), 1e-3 * np.abs(g).max())
        fds = []
        for h in hs:
            fd = []
            for i in idx:
                xp, xm = flat.clone(), flat.clone()
                xp[i] += h
                xm[i] -= h
                fd.append((loss_at(xp) - loss_at(xm)) / (2 * h))
            fd = np.array(fd)
            fds.append(fd)
            rel = np.abs(fd - g[idx]) / den
            row[f"h_{h:g}"] = {"rel_err_max": float(rel.max()), "rel_err_median": float(np.median(rel))}
        if len(hs) == 3:
            r = hs[0] / hs[1]
            r1 = [(r * r * fds[k + 1] - fds[k]) / (r * r - 1) for k in range(2)]
            r2 = (r ** 4 * r1[1] - r1[0]) / (r ** 4 - 1)
            rel = np.abs(r2 - g[idx]) / den
            row["richardson_2"] = {"rel_err_max": float(rel.max()), "rel_err_median": float(np.median(rel)),
                                   "rel_err_per_coordinate": [float(f"{e:.3g}") for e in rel]}
        out[f"steps_{steps}"] = row
    return out


def report_config4_tangent(dev, n=16384, steps=200, ncoord=64):
    """Adjoint gradients with respect to x0 (FP64, checkpoints every 20) over the full
    200-step rollout against exact directional derivatives of the same FP64 trajectory
    from forward-mode tangent rollouts (``adjoint.tangent_rollout``), on the 64 random
    coordinates of ``report_config4``; relative to the larger of |g_i| and 1e-3 max |g|."""
    import numpy as np
    import torch

    from gravhopper_gb300 import engine, ics
    from gravhopper_gb300.adjoint import rollout, tangent_rollout
    ic = ics.plummer(n, seed=0)
    x0 = torch.from_numpy(ic["pos"]).to(dev)
    v0 = torch.from_numpy(ic["vel"]).to(dev)
    m = torch.from_numpy(ic["mass"]).to(dev)
    rng = np.random.default_rng(1)
    xt = (x0 * torch.from_numpy(1 + 1e-3 * rng.normal(size=ic["pos"].shape)).to(dev)).contiguous()
    vt = (v0 * torch.from_numpy(1 + 1e-3 * rng.normal(size=ic["vel"].shape)).to(dev)).contiguous()
    engine.run_dkd(xt, vt, m, steps, 0.005, 5e-5, precision="fp64")
    xa = x0.clone().requires_grad_(True)
    xT, _ = rollout(xa, v0, m, steps, 0.005, 5e-5, checkpoint_every=20, precision="fp64")
    ((xT - xt) ** 2).mean().backward()
    g = xa.grad.reshape(-1)
    idx = rng.choice(3 * n, size=ncoord, replace=False)
    gmax = float(g.abs().max())
    rel, same = [], True
    t0 = time.perf_counter()
    for i in idx:
        u = torch.zeros(3 * n, dtype=torch.float64, device=dev)
        u[int(i)] = 1.0
        xT2, _, txT, _ = tangent_rollout(x0, v0, m, steps, 0.005, 5e-5, u.reshape(-1, 3), precision="fp64")
        same = same and bool(torch.equal(xT2, xT.detach()))
        d = float(2.0 * ((xT2 - xt) * txT).sum() / xt.numel())
        gi = float(g[int(i)])
        rel.append(abs(d - gi) / max(abs(gi), 1e-3 * gmax))
    rel = np.array(rel)
    return {"n": n, "steps": steps, "checkpoint_every": 20, "coordinates": ncoord,
            "rel_err_max": float(rel.max()), "rel_err_median": float(np.median(rel)),
            "final_state_bit_identical": same, "seconds": time.perf_counter() - t0}


if __name__ == "__main__":
    main()
