"""Drop-in for the reference extension module ``gravhopper._jbgrav``.

Same four functions, arguments, return shapes and ``RuntimeError`` messages as
gravhopper/_jbgrav.c:25-31, 68-135, 200-294, 564-727; the arithmetic runs on the GPU
through the C ABI (``gh_direct_summation``, ``gh_direct_summation_position``,
``gh_tree_force``, ``gh_tree_force_position``).  Inputs are converted like
``PyArray_FROM_OTF(obj, NPY_DOUBLE, NPY_ARRAY_IN_ARRAY)``: any array-like is cast to a
C-contiguous float64 array.  Outputs are new (N,3) float64 arrays in code units
(G=1, kpc, Msun).
"""
from __future__ import annotations

import numpy as np

from . import _capi


def _f64(obj):
    return np.ascontiguousarray(obj, dtype=np.float64)


def _mass_vector(mass, n, msg):
    # The reference reads mass[j] through PyArray_GETPTR1 after checking only
    # PyArray_DIM(mass, 0) == np (_jbgrav.c:103); trailing dimensions are ignored.
    if mass.ndim == 0 or mass.shape[0] != n:
        raise RuntimeError(msg)
    if mass.ndim > 1:
        mass = np.ascontiguousarray(mass.reshape(n, -1)[:, 0])
    return mass


def _check_pos(pos, prefix):
    if pos.ndim != 2:
        raise RuntimeError(f"{prefix} array does not have 2 dimensions.")
    if pos.shape[1] != 3:
        raise RuntimeError(f"{prefix} array is not Nx3.")


def direct_summation(pos, mass, eps):
    """Acceleration on every particle from every other particle by direct summation.

    Mirrors ``_jbgrav.direct_summation`` (gravhopper/_jbgrav.c:68-193); FP64,
    bit-identical to the reference's operation order.
    """
    pos = _f64(pos)
    mass = _f64(mass)
    _check_pos(pos, "Position")
    n = pos.shape[0]
    mass = _mass_vector(mass, n, "Mass array and position array contain different numbers of particles.")
    out = np.empty_like(pos)
    _capi.call("gh_direct_summation", _capi.ptr(pos), _capi.ptr(mass), n, float(eps), _capi.ptr(out))
    return out


def direct_summation_position(pos, mass, force_pos, eps):
    """Acceleration at arbitrary points by direct summation.

    Mirrors ``_jbgrav.direct_summation_position`` (gravhopper/_jbgrav.c:200-353): a
    point that coincides with a particle gets no term from it when eps == 0.
    """
    pos = _f64(pos)
    mass = _f64(mass)
    fpos = _f64(force_pos)
    _check_pos(pos, "Particle position")
    n = pos.shape[0]
    mass = _mass_vector(mass, n,
                        "Mass array and particle position array contain different numbers of particles.")
    _check_pos(fpos, "Force position")
    out = np.empty_like(fpos)
    _capi.call("gh_direct_summation_position", _capi.ptr(pos), _capi.ptr(mass), n, _capi.ptr(fpos),
               fpos.shape[0], float(eps), _capi.ptr(out))
    return out


def tree_force(pos, mass, eps, theta):
    """Acceleration on every particle from a Barnes-Hut octree.

    Mirrors ``_jbgrav.tree_force`` (gravhopper/_jbgrav.c:564-630, 737-806).
    """
    pos = _f64(pos)
    mass = _f64(mass)
    _check_pos(pos, "Position")
    n = pos.shape[0]
    mass = _mass_vector(mass, n, "Mass array and position array contain different numbers of particles.")
    out = np.empty_like(pos)
    _capi.call("gh_tree_force", _capi.ptr(pos), _capi.ptr(mass), n, float(eps), float(theta),
               _capi.ptr(out))
    return out


def tree_force_position(pos, mass, force_pos, eps, theta):
    """Acceleration at arbitrary points from a Barnes-Hut octree.

    Mirrors ``_jbgrav.tree_force_position`` (gravhopper/_jbgrav.c:634-727).
    """
    pos = _f64(pos)
    mass = _f64(mass)
    fpos = _f64(force_pos)
    _check_pos(pos, "Particle position")
    n = pos.shape[0]
    mass = _mass_vector(mass, n,
                        "Mass array and particle position array contain different numbers of particles.")
    _check_pos(fpos, "Force position")
    out = np.empty_like(fpos)
    _capi.call("gh_tree_force_position", _capi.ptr(pos), _capi.ptr(mass), n, _capi.ptr(fpos),
               fpos.shape[0], float(eps), float(theta), _capi.ptr(out))
    return out


def direct_summation_mixed(pos, mass, eps, force_pos=None):
    """Direct sum with FP32 pair arithmetic and compensated accumulation (engine extension).

    ``force_pos=None`` computes the self-consistent force (self term skipped).
    """
    pos = _f64(pos)
    mass = _f64(mass)
    _check_pos(pos, "Position")
    n = pos.shape[0]
    mass = _mass_vector(mass, n, "Mass array and position array contain different numbers of particles.")
    if force_pos is None:
        out = np.empty_like(pos)
        _capi.call("gh_direct_host", _capi.ptr(pos), _capi.ptr(mass), n, None, 0, float(eps),
                   _capi.GH_PREC_MIXED, _capi.ptr(out))
        return out
    fpos = _f64(force_pos)
    _check_pos(fpos, "Force position")
    out = np.empty_like(fpos)
    _capi.call("gh_direct_host", _capi.ptr(pos), _capi.ptr(mass), n, _capi.ptr(fpos), fpos.shape[0],
               float(eps), _capi.GH_PREC_MIXED, _capi.ptr(out))
    return out
