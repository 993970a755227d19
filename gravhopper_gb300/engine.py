"""Device-level API over the C ABI, on torch CUDA tensors.

All tensors are CUDA float64, C-contiguous: positions/velocities (N,3), masses (N).
Work is enqueued on the given torch stream (the current stream by default).  Forces
are in code units (G=1, kpc, Msun); leapfrog state is kpc, km/s, Msun, Myr.
"""
from __future__ import annotations

import torch

from . import _capi


def _check(t, name, shape_tail=None):
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch tensor")
    if not t.is_cuda or t.dtype != torch.float64 or not t.is_contiguous():
        raise ValueError(f"{name} must be a contiguous CUDA float64 tensor")
    if shape_tail is not None and (t.dim() != 2 or t.shape[1] != shape_tail):
        raise ValueError(f"{name} must have shape (N,{shape_tail})")


def direct_force(pos, mass, eps, force_pos=None, precision="fp64", out=None, stream=None):
    """Direct-sum acceleration (code units).  ``force_pos=None``: self-force, j != i."""
    _check(pos, "pos", 3)
    _check(mass, "mass")
    if mass.shape[0] != pos.shape[0]:
        raise ValueError("mass and pos have different lengths")
    if force_pos is not None:
        _check(force_pos, "force_pos", 3)
    n_out = pos.shape[0] if force_pos is None else force_pos.shape[0]
    if out is None:
        out = torch.empty((n_out, 3), dtype=torch.float64, device=pos.device)
    _capi.call("gh_direct_dev", _capi.ptr(pos), _capi.ptr(mass), pos.shape[0], _capi.ptr(force_pos),
               0 if force_pos is None else force_pos.shape[0], float(eps),
               _capi.PRECISIONS[precision], _capi.ptr(out), _capi.stream_handle(stream))
    return out


def tree_force(pos, mass, eps, theta=0.7, force_pos=None, out=None, stream=None, precision="fp64"):
    """Barnes-Hut acceleration (code units) with the reference's opening decisions.

    ``precision='mixed'`` evaluates accepted cells in FP32 (compensated sums)."""
    _check(pos, "pos", 3)
    _check(mass, "mass")
    if mass.shape[0] != pos.shape[0]:
        raise ValueError("mass and pos have different lengths")
    if force_pos is not None:
        _check(force_pos, "force_pos", 3)
    n_out = pos.shape[0] if force_pos is None else force_pos.shape[0]
    if out is None:
        out = torch.empty((n_out, 3), dtype=torch.float64, device=pos.device)
    _capi.call("gh_tree_dev", _capi.ptr(pos), _capi.ptr(mass), pos.shape[0], _capi.ptr(force_pos),
               0 if force_pos is None else force_pos.shape[0], float(eps), float(theta),
               _capi.PRECISIONS[precision], _capi.ptr(out), _capi.stream_handle(stream))
    return out


def run_dkd(pos, vel, mass, nsteps, dt, eps, algorithm="direct", precision="fp64", theta=0.7,
            hist_stride=0, stream=None):
    """Advance (pos, vel) in place by ``nsteps`` drift-kick-drift steps on the device.

    Returns ``(hist_pos, hist_vel)`` of shape (nsteps // hist_stride, N, 3) when
    ``hist_stride > 0``, else None.
    """
    _check(pos, "pos", 3)
    _check(vel, "vel", 3)
    _check(mass, "mass")
    n = pos.shape[0]
    if vel.shape[0] != n or mass.shape[0] != n:
        raise ValueError("pos, vel and mass have different lengths")
    hp = hv = None
    if hist_stride > 0:
        ns = nsteps // hist_stride
        hp = torch.empty((ns, n, 3), dtype=torch.float64, device=pos.device)
        hv = torch.empty((ns, n, 3), dtype=torch.float64, device=pos.device)
    _capi.call("gh_run_dkd", _capi.ptr(pos), _capi.ptr(vel), _capi.ptr(mass), n, int(nsteps), float(dt),
               float(eps), _capi.ALGORITHMS[algorithm], _capi.PRECISIONS[precision], float(theta),
               _capi.ptr(hp), _capi.ptr(hv), int(hist_stride), _capi.stream_handle(stream))
    return (hp, hv) if hist_stride > 0 else None


def dkd_drift(pos, vel, dt, out=None, stream=None):
    """First drift of a leapfrog step: ``pos + ((0.5 vel) dt) F`` (kpc; F = km Myr/s
    in kpc), into ``out`` (a new tensor by default; may be ``pos``)."""
    _check(pos, "pos", 3)
    _check(vel, "vel", 3)
    if vel.shape[0] != pos.shape[0]:
        raise ValueError("pos and vel have different lengths")
    if out is None:
        out = torch.empty_like(pos)
    _check(out, "out", 3)
    _capi.call("gh_dkd_drift", _capi.ptr(pos), _capi.ptr(vel), pos.shape[0], float(dt), _capi.ptr(out),
               _capi.stream_handle(stream))
    return out


def dkd_kick_drift(pos_half, vel, acc, acc_ext, dt, out=None, stream=None):
    """Kick and second drift of a leapfrog step: ``vel += ((acc ACC) + acc_ext) dt`` in
    place, then ``out = pos_half + ((0.5 vel) dt) F``.  ``acc`` is the N-body
    acceleration in code units or None (no N-body force); ``acc_ext`` the external
    acceleration in km/s/Myr or None."""
    _check(pos_half, "pos_half", 3)
    _check(vel, "vel", 3)
    n = pos_half.shape[0]
    for t, name in ((acc, "acc"), (acc_ext, "acc_ext")):
        if t is not None:
            _check(t, name, 3)
            if t.shape[0] != n:
                raise ValueError(f"{name} and pos_half have different lengths")
    if vel.shape[0] != n:
        raise ValueError("pos_half and vel have different lengths")
    if out is None:
        out = torch.empty_like(pos_half)
    _check(out, "out", 3)
    _capi.call("gh_dkd_kick_drift", _capi.ptr(pos_half), _capi.ptr(vel), _capi.ptr(acc), _capi.ptr(acc_ext), n,
               float(dt), _capi.ptr(out), _capi.stream_handle(stream))
    return out


def direct_vjp(pos, mass, eps, cot, precision="fp64", grad_pos=None, grad_mass=None, stream=None):
    """Vector-Jacobian product of the direct-sum self-acceleration (code units).

    Returns (grad_pos (N,3), grad_mass (N)) = (cot . da/dx, cot . da/dm).
    """
    _check(pos, "pos", 3)
    _check(mass, "mass")
    _check(cot, "cot", 3)
    n = pos.shape[0]
    if grad_pos is None:
        grad_pos = torch.empty((n, 3), dtype=torch.float64, device=pos.device)
    if grad_mass is None:
        grad_mass = torch.empty(n, dtype=torch.float64, device=pos.device)
    _capi.call("gh_direct_vjp_dev", _capi.ptr(pos), _capi.ptr(mass), n, float(eps), _capi.ptr(cot),
               _capi.PRECISIONS[precision], _capi.ptr(grad_pos), _capi.ptr(grad_mass), _capi.stream_handle(stream))
    return grad_pos, grad_mass


def potential(pos, mass, eps, out=None, stream=None):
    """Per-particle softened potential -sum_{j!=k} m_j / sqrt(r^2+eps^2) (G=1), FP64."""
    _check(pos, "pos", 3)
    _check(mass, "mass")
    n = pos.shape[0]
    if out is None:
        out = torch.empty(n, dtype=torch.float64, device=pos.device)
    _capi.call("gh_potential_dev", _capi.ptr(pos), _capi.ptr(mass), n, float(eps), _capi.ptr(out),
               _capi.stream_handle(stream))
    return out


def energy(pos, vel, mass, eps):
    """(kinetic, potential, total) energy in Msun (km/s)^2, on the device in FP64."""
    from .units import G_KPC_KMS2_MSUN
    ke = 0.5 * float(torch.sum(mass * torch.sum(vel * vel, dim=1)))
    pe = 0.5 * G_KPC_KMS2_MSUN * float(torch.sum(mass * potential(pos, mass, eps)))
    return ke, pe, ke + pe


def momentum(pos, vel, mass):
    """Total linear momentum (3,) in Msun km/s and angular momentum about the origin
    (3,) in Msun kpc km/s, FP64 sums on the device."""
    _check(pos, "pos", 3)
    _check(vel, "vel", 3)
    _check(mass, "mass")
    p = torch.sum(mass[:, None] * vel, dim=0)
    lm = torch.sum(mass[:, None] * torch.linalg.cross(pos, vel, dim=1), dim=0)
    return p, lm
