"""Differentiable leapfrog rollout with the hand-written direct-sum adjoint.

``rollout(x0, v0, m, nsteps, dt, eps)`` is a ``torch.autograd.Function``: the forward
pass runs the drift-kick-drift leapfrog on the GPU (gravhopper/gravhopper.py:405-416
arithmetic), keeping the state every ``checkpoint_every`` steps; the backward pass
hands all checkpoints to ``gh_dkd_backward_chain_dev``, which walks the segments in
reverse, recomputing each segment's states from its checkpoint (on a second stream,
while the following segment back-propagates) and back-propagating step by step:

    forward:  xh = x + c v,  a = A F(xh, m),  v' = v + dt a,  x' = xh + c v'
    backward: w = v'bar + c x'bar,  lam = A dt w,  (gx, gm) = VJP of F at xh with lam,
              xhbar = x'bar + gx,  xbar = xhbar,  vbar = w + c xhbar,  mbar += gm

with c = 0.5 dt (km*Myr/s -> kpc), A = G*Msun/kpc^2 in km/s/Myr, F the code-unit
direct sum and its VJP the ``gh_direct_vjp_dev`` kernel (softened tidal tensor
contracted with the cotangent, plus the mass gradient).
"""
from __future__ import annotations

import ctypes

import torch

from . import _capi, engine


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x0, v0, m, nsteps, dt, eps, checkpoint_every, precision):
        x = x0.detach().clone().contiguous()
        v = v0.detach().clone().contiguous()
        md = m.detach().contiguous()
        k = max(1, int(checkpoint_every))
        segs = [min(k, nsteps - s0) for s0 in range(0, nsteps, k)]
        cx = torch.empty((len(segs),) + tuple(x.shape), dtype=x.dtype, device=x.device)
        cv = torch.empty_like(cx)
        for q, seg in enumerate(segs):
            cx[q].copy_(x)
            cv[q].copy_(v)
            engine.run_dkd(x, v, md, seg, dt, eps, algorithm="direct", precision=precision)
        ctx.ckpts = (cx, cv, segs)
        ctx.params = (dt, eps, precision)
        ctx.save_for_backward(md)
        return x, v

    @staticmethod
    def backward(ctx, gx, gv):
        (m,) = ctx.saved_tensors
        dt, eps, precision = ctx.params
        n = m.shape[0]
        xb = gx.contiguous().clone() if gx is not None else torch.zeros((n, 3), dtype=torch.float64, device=m.device)
        vb = gv.contiguous().clone() if gv is not None else torch.zeros_like(xb)
        mb = torch.zeros_like(m)
        cx, cv, segs = ctx.ckpts
        if segs:
            seg_arr = (ctypes.c_int64 * len(segs))(*segs)
            _capi.call("gh_dkd_backward_chain_dev", _capi.ptr(cx), _capi.ptr(cv), ctypes.addressof(seg_arr),
                       len(segs), _capi.ptr(m), n, float(dt), float(eps), _capi.PRECISIONS[precision],
                       _capi.ptr(xb), _capi.ptr(vb), _capi.ptr(mb), _capi.stream_handle())
        ctx.ckpts = None
        return xb, vb, mb, None, None, None, None, None


def rollout(x0, v0, m, nsteps, dt, eps, checkpoint_every=20, precision="mixed"):
    """Differentiable ``nsteps`` leapfrog steps; returns (x_T, v_T)."""
    return _Rollout.apply(x0, v0, m, int(nsteps), float(dt), float(eps), int(checkpoint_every), precision)


def tangent_rollout(x0, v0, m, nsteps, dt, eps, dx0, dv0=None, precision="fp64"):
    """Forward-mode derivative of ``nsteps`` leapfrog steps along (dx0, dv0), masses
    held fixed: returns (x_T, v_T, dx_T, dv_T).

    The state advances by the engine's split step (first drift, direct-sum force, kick
    and second drift; the fused step's operations, so the same bits as ``rollout``'s
    forward pass), and the tangent by the same two linear step kernels with the
    force's Jacobian-vector product J u = VJP(m u) / m: the direct sum's Jacobian
    blocks are m_k M(x_k - x_i) (M the symmetric, even softened tidal tensor) and
    -sum_j m_j M(x_j - x_i) on the diagonal, so the VJP kernel applied to the cotangent
    m u gives m_i (J u)_i.  Every mass must be nonzero.  Costs one force and one VJP
    per step; where ``rollout``'s adjoint gives the whole gradient of a scalar loss,
    this gives the exact directional derivative of the same computed trajectory."""
    md = m.detach().contiguous()
    if bool((md == 0).any()):
        raise ValueError("tangent_rollout: every mass must be nonzero")
    x = x0.detach().clone().contiguous()
    v = v0.detach().clone().contiguous()
    tx = dx0.detach().clone().contiguous()
    tv = torch.zeros_like(v) if dv0 is None else dv0.detach().clone().contiguous()
    mm = md[:, None]
    xh, txh, acc, cot, g, ta = (torch.empty_like(x) for _ in range(6))
    gm = torch.empty_like(md)
    for _ in range(int(nsteps)):
        engine.dkd_drift(x, v, dt, out=xh)
        engine.direct_force(xh, md, eps, precision=precision, out=acc)
        engine.dkd_kick_drift(xh, v, acc, None, dt, out=x)
        engine.dkd_drift(tx, tv, dt, out=txh)
        torch.mul(txh, mm, out=cot)
        engine.direct_vjp(xh, md, eps, cot, precision=precision, grad_pos=g, grad_mass=gm)
        torch.div(g, mm, out=ta)
        engine.dkd_kick_drift(txh, tv, ta, None, dt, out=tx)
    return x, v, tx, tv

