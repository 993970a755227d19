"""CPU oracle for the GravHopper force-and-integrate path.  TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
import this module, and only as the checker.  The engine in ``gravhopper_gb300`` never
imports it.

Contents
--------
* ``direct_summation`` / ``direct_summation_position`` / ``tree_force`` /
  ``tree_force_position``: the four functions of the reference extension
  ``gravhopper._jbgrav`` (gravhopper/_jbgrav.c:25-31), computed by the C restatement
  in ``oracle/gh_oracle.c`` (same operation order, O(N) memory, threaded over targets).
* ``dkd_run``: a NumPy restatement of ``Simulation.perform_timestep``
  (gravhopper/gravhopper.py:405-416) in the internal units kpc, km/s, Msun, Myr, with
  the factors astropy applies (gravhopper/jbgrav.py:37-48).
* ``reference_module()``: the reference extension itself, compiled unchanged from its
  source by ``make -C oracle ref`` where that source exists (absent on hosts without it).

Parity pins: ``tests/golden/*.npz`` hold outputs of the compiled reference on seeded
inputs (generated by ``tests/golden/make_golden.py``); ``tests/test_oracle.py`` checks
this restatement against them bit for bit.
"""
from __future__ import annotations

import ctypes
import glob
import importlib.util
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libghoracle.so")

# Unit factors (gravhopper/jbgrav.py:38-48 and the astropy conversions in
# gravhopper/gravhopper.py:409-416), derived from G=6.6743e-11, GM_sun=1.3271244e20,
# pc = au / 1 arcsec, Julian year.
ACCEL_UNIT = 4.398600412921223e-09       # G*Msun/kpc^2 in km/s/Myr
KMS_MYR_TO_KPC = 1.022712165045695e-03   # (km/s)*Myr in kpc
G_KPC_KMS2_MSUN = 4.30091727003628e-06   # G in kpc (km/s)^2 / Msun

_lib = None


def build() -> str:
    """Compile the C restatement (``make -C oracle``) and return the .so path."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        lib = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        lib.ghor_direct.argtypes = [dp, dp, ctypes.c_int64, dp, ctypes.c_int64, ctypes.c_double,
                                    ctypes.c_int, dp, ctypes.c_int]
        lib.ghor_direct.restype = ctypes.c_int
        lib.ghor_tree.argtypes = [dp, dp, ctypes.c_int64, dp, ctypes.c_int64, ctypes.c_double,
                                  ctypes.c_double, dp, ctypes.c_int, ctypes.c_int,
                                  ctypes.POINTER(ctypes.c_int64), dp]
        lib.ghor_tree.restype = ctypes.c_int
        lib.ghor_potential.argtypes = [dp, dp, ctypes.c_int64, ctypes.c_double, dp]
        lib.ghor_potential.restype = ctypes.c_int
        _lib = lib
    return _lib


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _as_f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def default_threads() -> int:
    return max(1, len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count() or 1)


def direct_summation(pos, mass, eps, nthreads=None):
    """Oracle for ``_jbgrav.direct_summation`` (gravhopper/_jbgrav.c:68-193)."""
    pos = _as_f64(pos)
    mass = _as_f64(mass)
    out = np.empty((pos.shape[0], 3))
    rc = _load().ghor_direct(_dptr(pos), _dptr(mass), pos.shape[0], _dptr(pos), pos.shape[0],
                             float(eps), 1, _dptr(out), nthreads or default_threads())
    if rc:
        raise RuntimeError(f"oracle direct failed ({rc})")
    return out


def direct_summation_position(pos, mass, force_pos, eps, nthreads=None):
    """Oracle for ``_jbgrav.direct_summation_position`` (gravhopper/_jbgrav.c:200-353)."""
    pos = _as_f64(pos)
    mass = _as_f64(mass)
    fp = _as_f64(force_pos)
    out = np.empty((fp.shape[0], 3))
    rc = _load().ghor_direct(_dptr(pos), _dptr(mass), pos.shape[0], _dptr(fp), fp.shape[0],
                             float(eps), 0, _dptr(out), nthreads or default_threads())
    if rc:
        raise RuntimeError(f"oracle direct_position failed ({rc})")
    return out


def tree_force_position(pos, mass, force_pos, eps, theta=0.7, nthreads=None, maxdepth=4096,
                        return_nodes=False, times=None):
    """Oracle for ``_jbgrav.tree_force_position`` (gravhopper/_jbgrav.c:634-806).

    ``times``: optional list that receives [build seconds, walk seconds]."""
    pos = _as_f64(pos)
    mass = _as_f64(mass)
    fp = _as_f64(force_pos)
    out = np.empty((fp.shape[0], 3))
    nn = ctypes.c_int64(0)
    tt = np.zeros(2)
    rc = _load().ghor_tree(_dptr(pos), _dptr(mass), pos.shape[0], _dptr(fp), fp.shape[0],
                           float(eps), float(theta), _dptr(out), nthreads or default_threads(),
                           int(maxdepth), ctypes.byref(nn), _dptr(tt))
    if times is not None:
        times[:] = [float(tt[0]), float(tt[1])]
    if rc == 3:
        raise RuntimeError("oracle tree: depth limit exceeded (coincident particles?)")
    if rc:
        raise RuntimeError(f"oracle tree failed ({rc})")
    return (out, nn.value) if return_nodes else out


def tree_force(pos, mass, eps, theta=0.7, nthreads=None, maxdepth=4096, return_nodes=False):
    """Oracle for ``_jbgrav.tree_force`` (gravhopper/_jbgrav.c:564-630)."""
    return tree_force_position(pos, mass, pos, eps, theta, nthreads, maxdepth, return_nodes)


def potential_energy(pos, mass, eps):
    """Softened potential energy in code units (G=1, kpc, Msun)."""
    pos = _as_f64(pos)
    mass = _as_f64(mass)
    phi = ctypes.c_double(0.0)
    _load().ghor_potential(_dptr(pos), _dptr(mass), pos.shape[0], float(eps), ctypes.byref(phi))
    return phi.value


def total_energy(pos, vel, mass, eps):
    """Kinetic + potential energy in Msun (km/s)^2."""
    mass = _as_f64(mass)
    vel = _as_f64(vel)
    ke = 0.5 * float(np.sum(mass * np.sum(vel * vel, axis=1)))
    return ke + G_KPC_KMS2_MSUN * potential_energy(pos, mass, eps)


def dkd_step(pos, vel, mass, dt, eps, force):
    """One ``Simulation.perform_timestep`` (gravhopper/gravhopper.py:405-416).

    pos [kpc], vel [km/s], dt [Myr], eps [kpc]; ``force(pos, mass, eps)`` returns the
    code-unit acceleration.  The drift multiplies ``(0.5*v)*dt`` by the km*Myr/s -> kpc
    factor as astropy does when adding to a kpc array; the kick uses
    ``acc[code] * ACCEL_UNIT`` (jbgrav.py:48) times dt.
    """
    half = (0.5 * vel) * dt
    xh = pos + half * KMS_MYR_TO_KPC
    if pos.shape[0] > 1:
        acc = force(xh, mass, eps) * ACCEL_UNIT
    else:
        acc = np.zeros_like(pos)
    v1 = vel + acc * dt
    x1 = xh + ((0.5 * v1) * dt) * KMS_MYR_TO_KPC
    return x1, v1


def dkd_run(pos, vel, mass, dt, eps, nsteps, force=None, snap_every=0):
    """Run ``nsteps`` DKD steps; returns final (pos, vel) and optional snapshots."""
    force = force or direct_summation
    x = _as_f64(pos).copy()
    v = _as_f64(vel).copy()
    m = _as_f64(mass)
    snaps = []
    for k in range(nsteps):
        x, v = dkd_step(x, v, m, dt, eps, force)
        if snap_every and (k + 1) % snap_every == 0:
            snaps.append((x.copy(), v.copy()))
    return (x, v, snaps) if snap_every else (x, v)


def reference_module():
    """The reference extension compiled from source into ``oracle/_ref`` (or None)."""
    cands = glob.glob(os.path.join(HERE, "_ref", "_jbgrav*.so"))
    if not cands:
        return None
    spec = importlib.util.spec_from_file_location("_jbgrav", cands[0])
    mod = importlib.util.module_from_spec(spec)
    try:
        spec.loader.exec_module(mod)
    except ImportError:
        return None
    return mod
