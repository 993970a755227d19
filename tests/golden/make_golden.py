"""Generates tests/golden/*.npz from the reference extension compiled from source.

Run here (where the reference source exists):

    make -C oracle ref && python tests/golden/make_golden.py

Every output in the fixtures comes from the reference's own ``_jbgrav`` functions
(gravhopper/_jbgrav.c) on seeded inputs stored alongside.  Trajectories use those
forces inside the NumPy restatement of Simulation.perform_timestep
(gravhopper/gravhopper.py:405-416) in ``oracle/oracle.py``, since the reference's
Python layer needs astropy, which is not installed.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from gravhopper_gb300 import ics  # noqa: E402
from oracle import oracle  # noqa: E402


def main():
    ref = oracle.reference_module()
    if ref is None:
        raise SystemExit("reference extension not built: run `make -C oracle ref` first")
    rng = np.random.default_rng(20261203)
    out = {}

    # --- direct_summation: small random systems and edge sizes -----------------
    for n in (0, 1, 2, 3, 64, 333):
        pos = rng.normal(size=(n, 3)) * 1e-3
        mass = rng.uniform(0.5, 2.0, size=n) * 1e3
        for tag, eps in (("eps", 5e-5), ("eps0", 0.0)):
            if tag == "eps0" and n > 3:
                continue
            out[f"direct_{n}_{tag}_pos"] = pos
            out[f"direct_{n}_{tag}_mass"] = mass
            out[f"direct_{n}_{tag}_eps"] = np.array(eps)
            out[f"direct_{n}_{tag}_out"] = ref.direct_summation(pos, mass, eps)

    # --- direct_summation_position: coincident targets with eps = 0 ------------
    pos = rng.normal(size=(200, 3)) * 1e-3
    mass = rng.uniform(0.5, 2.0, size=200) * 1e3
    fpos = np.concatenate([pos[:7], rng.normal(size=(41, 3)) * 2e-3])
    for tag, eps in (("eps", 5e-5), ("eps0", 0.0)):
        out[f"dpos_{tag}_pos"] = pos
        out[f"dpos_{tag}_mass"] = mass
        out[f"dpos_{tag}_fpos"] = fpos
        out[f"dpos_{tag}_eps"] = np.array(eps)
        out[f"dpos_{tag}_out"] = ref.direct_summation_position(pos, mass, fpos, eps)

    # --- config-0 Plummer sphere: force at t=0 and a 400-step trajectory ---------
    ic = ics.plummer(2000, b=1e-3, totmass=1e6, seed=0)
    out["plummer_pos"], out["plummer_vel"], out["plummer_mass"] = ic["pos"], ic["vel"], ic["mass"]
    out["plummer_force"] = ref.direct_summation(ic["pos"], ic["mass"], 5e-5)
    x, v, snaps = oracle.dkd_run(ic["pos"], ic["vel"], ic["mass"], 0.005, 5e-5, 400,
                                 force=ref.direct_summation, snap_every=100)
    for k, (sx, sv) in enumerate(snaps):
        out[f"traj_direct_x_{(k + 1) * 100}"] = sx
        out[f"traj_direct_v_{(k + 1) * 100}"] = sv

    # --- tree_force / tree_force_position ----------------------------------------
    tic = ics.plummer(500, b=1e-3, totmass=1e6, seed=5)
    out["tree_pos"], out["tree_mass"] = tic["pos"], tic["mass"]
    tfp = np.concatenate([tic["pos"][:9], rng.normal(size=(30, 3)) * 3e-3])
    out["tree_fpos"] = tfp
    for th in (0.0, 0.5, 0.7, 1.0):
        key = str(th).replace(".", "p")
        out[f"tree_{key}_out"] = ref.tree_force(tic["pos"], tic["mass"], 5e-5, th)
        out[f"treepos_{key}_out"] = ref.tree_force_position(tic["pos"], tic["mass"], tfp, 0.0, th)
    for n in (1, 2, 3):
        p = rng.normal(size=(n, 3))
        m = rng.uniform(1.0, 2.0, size=n)
        out[f"tree_small_{n}_pos"], out[f"tree_small_{n}_mass"] = p, m
        out[f"tree_small_{n}_out"] = ref.tree_force(p, m, 0.01, 0.7)
    # Hernquist-plus-disk sample (wide dynamic range, deep tree)
    hic = ics.hernquist_disk(4000, seed=11)
    out["hq_pos"], out["hq_mass"] = hic["pos"], hic["mass"]
    for th in (0.5, 0.7):
        key = str(th).replace(".", "p")
        out[f"hq_{key}_out"] = ref.tree_force(hic["pos"], hic["mass"], 0.1, th)
    # Tree-driven trajectory: 20 DKD steps of the 2000-particle Plummer sphere
    tx, tv = oracle.dkd_run(ic["pos"], ic["vel"], ic["mass"], 0.005, 5e-5, 20,
                            force=lambda p, m, e: ref.tree_force(p, m, e, 0.7))
    out["traj_tree_x_20"], out["traj_tree_v_20"] = tx, tv

    path = os.path.join(HERE, "reference_vectors.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}: {len(out)} arrays, {os.path.getsize(path) / 1e3:.0f} kB")


if __name__ == "__main__":
    main()
