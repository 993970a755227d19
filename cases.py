"""Run one engine workload a few times and print its timing (for profiling).

    python cases.py direct   --n 131072 --reps 2   # mixed direct force
    python cases.py direct64 --n 65536  --reps 1   # FP64 direct force
    python cases.py dkd      --n 1048576 --reps 1  # mixed DKD step
    python cases.py tree     --n 65536  --theta 0.7 --precision fp64
    python cases.py ensemble --systems 64
    python cases.py vjp      --n 16384
    python cases.py external --n 1048576 --reps 6 --ext device   # tree run with an external force

Each case builds seeded inputs (Plummer spheres; Hernquist plus disk for the tree),
runs one warm-up call and ``--reps`` timed calls on cuda:0, and prints one line of
milliseconds per call.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["direct", "direct64", "dkd", "tree", "ensemble", "vjp", "external"])
    ap.add_argument("--n", type=int, default=131072)
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--theta", type=float, default=0.7)
    ap.add_argument("--systems", type=int, default=64)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"], help="tree and vjp cases")
    ap.add_argument("--shape", type=int, default=-1, help="direct: mixed kernel tile shape (-1 auto)")
    ap.add_argument("--fp64-form", type=int, default=-1, choices=[-1, 0, 1],
                    help="direct64: FP64 kernel (0 thread per target, 1 ordered CTA-wide terms, -1 auto)")
    ap.add_argument("--ext", default="device", choices=["none", "device", "host"],
                    help="external: a Plummer-halo pull as a device force, a host function or none")
    a = ap.parse_args(argv)
    if a.case == "external":
        return external(a)

    import torch

    from gravhopper_gb300 import _capi, engine, ics
    dev = torch.device("cuda", 0)
    _capi.load()
    _capi.call("gh_direct_set_fp64_form", a.fp64_form)
    _capi.call("gh_direct_set_shape", a.shape)
    if a.case in ("direct", "direct64", "dkd", "vjp"):
        ic = ics.plummer(a.n, seed=0)
    elif a.case == "tree":
        ic = ics.hernquist_disk(a.n, seed=1)
    if a.case == "ensemble":
        from gravhopper_gb300.ensemble import Ensemble
        e = Ensemble(ics.plummer_ensemble(a.systems, seed=0), device=dev)
        call = lambda: e.run(1, use_graph=False)  # noqa: E731
    else:
        x = torch.from_numpy(ic["pos"]).to(dev)
        m = torch.from_numpy(ic["mass"]).to(dev)
        if a.case == "direct":
            call = lambda: engine.direct_force(x, m, 5e-5, precision="mixed")  # noqa: E731
        elif a.case == "dkd":  # one leapfrog step with the mixed direct sum (the bench's step)
            v = torch.from_numpy(ic["vel"]).to(dev)
            call = lambda: engine.run_dkd(x, v, m, 1, 0.005, 5e-5, precision="mixed")  # noqa: E731
        elif a.case == "direct64":
            call = lambda: engine.direct_force(x, m, 5e-5, precision="fp64")  # noqa: E731
        elif a.case == "tree":
            call = lambda: engine.tree_force(x, m, 0.1, a.theta, precision=a.precision)  # noqa: E731
        else:
            lam = torch.ones_like(x)
            call = lambda: engine.direct_vjp(x, m, 5e-5, lam, precision=a.precision)  # noqa: E731
    call()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(a.reps):
        call()
    torch.cuda.synchronize()
    print(f"{a.case} n={a.n} reps={a.reps}: {(time.perf_counter() - t0) / max(a.reps, 1) * 1e3:.3f} ms per call")


def external(a):
    """Simulation.run steps (mixed tree, theta as given, history kept) of the Hernquist
    + disk system with a Plummer-halo pull registered as a device force, as a host
    function, or no external force; one warm-up step, then --reps steps."""
    import numpy as np
    import torch

    import gravhopper_gb300 as gh
    from gravhopper_gb300 import ics

    def halo(pos, args):
        xp = np if isinstance(pos, np.ndarray) else torch
        r2 = pos[:, 0] * pos[:, 0] + pos[:, 1] * pos[:, 1] + pos[:, 2] * pos[:, 2]
        s = r2 + args["b"] * args["b"]
        return -args["k"] * pos / (s * xp.sqrt(s))[:, None]

    sim = gh.Simulation(dt=0.5, eps=0.1, algorithm="tree", precision="mixed", theta=a.theta)
    sim.add_IC(ics.hernquist_disk(a.n, seed=1))
    if a.ext != "none":
        sim.add_external_force(halo, {"k": 1e3, "b": 5.0}, device=a.ext == "device")
    sim.run(1)
    t0 = time.perf_counter()
    sim.run(a.reps)
    print(f"external ({a.ext}) n={a.n} reps={a.reps}: {(time.perf_counter() - t0) / max(a.reps, 1) * 1e3:.3f} ms per step")


if __name__ == "__main__":
    main()
