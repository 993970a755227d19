"""Drop-in for ``gravhopper.jbgrav`` (gravhopper/jbgrav.py:14-177).

Same names and signatures: ``direct_summation(snap, eps)``,
``tree_force(snap, eps, theta=0.7)``, ``direct_summation_position(snap, force_pos, eps)``
and ``tree_force_position(snap, force_pos, eps, theta=0.7)``.  ``snap`` is a dict with
``'pos'`` (Np,3) and ``'mass'`` (Np).  Results are accelerations in km/s/Myr: the
code-unit result times G*Msun/kpc^2 (jbgrav.py:40-48).  With astropy present the
inputs may be Quantities and the result is a Quantity; otherwise inputs are plain
numbers in kpc and Msun.

Extension: ``precision='mixed'`` selects the FP32-pair / compensated form for the
direct sum.
"""
from __future__ import annotations

import numpy as np

from . import _jbgrav
from . import units as U

__all__ = ["direct_summation", "direct_summation_position", "tree_force", "tree_force_position"]


def _strip(snap, eps):
    pos = U.value(snap["pos"], U.LENGTH, "pos")
    mass = U.value(snap["mass"], U.MASS, "mass")
    e = U.value(eps, U.LENGTH, "eps")
    return pos, mass, float(e)


def _finish(code_accel):
    return U.quantity(np.asarray(code_accel) * U.ACCEL_UNIT, U.ACCEL)


def direct_summation(snap, eps, precision="fp64"):
    """Acceleration on every particle of ``snap`` by direct summation."""
    pos, mass, e = _strip(snap, eps)
    if precision == "mixed":
        return _finish(_jbgrav.direct_summation_mixed(pos, mass, e))
    return _finish(_jbgrav.direct_summation(pos, mass, e))


def tree_force(snap, eps, theta=0.7):
    """Acceleration on every particle of ``snap`` from a Barnes-Hut tree."""
    pos, mass, e = _strip(snap, eps)
    return _finish(_jbgrav.tree_force(pos, mass, e, theta))


def direct_summation_position(snap, force_pos, eps, precision="fp64"):
    """Acceleration at ``force_pos`` from every particle of ``snap`` (direct sum)."""
    pos, mass, e = _strip(snap, eps)
    fp = U.value(force_pos, U.LENGTH, "force_pos")
    if precision == "mixed":
        return _finish(_jbgrav.direct_summation_mixed(pos, mass, e, force_pos=fp))
    return _finish(_jbgrav.direct_summation_position(pos, mass, fp, e))


def tree_force_position(snap, force_pos, eps, theta=0.7):
    """Acceleration at ``force_pos`` from a Barnes-Hut tree of ``snap``."""
    pos, mass, e = _strip(snap, eps)
    fp = U.value(force_pos, U.LENGTH, "force_pos")
    return _finish(_jbgrav.tree_force_position(pos, mass, fp, e, theta))
