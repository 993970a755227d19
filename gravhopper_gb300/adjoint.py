"""Differentiable leapfrog rollout with the hand-written direct-sum adjoint.

``rollout(x0, v0, m, nsteps, dt, eps)`` is a ``torch.autograd.Function``: the forward
pass runs the drift-kick-drift leapfrog on the GPU (gravhopper/gravhopper.py:405-416
arithmetic), keeping the state every ``checkpoint_every`` steps; the backward pass
walks the segments in reverse, recomputes each segment's states from its checkpoint,
and back-propagates step by step:

    forward:  xh = x + c v,  a = A F(xh, m),  v' = v + dt a,  x' = xh + c v'
    backward: w = v'bar + c x'bar,  lam = A dt w,  (gx, gm) = VJP of F at xh with lam,
              xhbar = x'bar + gx,  xbar = xhbar,  vbar = w + c xhbar,  mbar += gm

with c = 0.5 dt (km*Myr/s -> kpc), A = G*Msun/kpc^2 in km/s/Myr, F the code-unit
direct sum and its VJP the ``gh_direct_vjp_dev`` kernel (softened tidal tensor
contracted with the cotangent, plus the mass gradient).
"""
from __future__ import annotations

import torch

from . import engine
from .units import ACCEL_UNIT, KMS_MYR_TO_KPC


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x0, v0, m, nsteps, dt, eps, checkpoint_every, precision):
        x = x0.detach().clone().contiguous()
        v = v0.detach().clone().contiguous()
        md = m.detach().contiguous()
        k = max(1, int(checkpoint_every))
        ckpts = []
        done = 0
        while done < nsteps:
            seg = min(k, nsteps - done)
            ckpts.append((x.clone(), v.clone(), seg))
            engine.run_dkd(x, v, md, seg, dt, eps, algorithm="direct", precision=precision)
            done += seg
        ctx.ckpts = ckpts
        ctx.params = (dt, eps, precision)
        ctx.save_for_backward(md)
        return x, v

    @staticmethod
    def backward(ctx, gx, gv):
        (m,) = ctx.saved_tensors
        dt, eps, precision = ctx.params
        c = 0.5 * dt * KMS_MYR_TO_KPC
        n = m.shape[0]
        xb = gx.contiguous().clone() if gx is not None else torch.zeros((n, 3), dtype=torch.float64, device=m.device)
        vb = gv.contiguous().clone() if gv is not None else torch.zeros_like(xb)
        mb = torch.zeros_like(m)
        gpos = torch.empty_like(xb)
        gmass = torch.empty_like(m)
        for xs, vs, seg in reversed(ctx.ckpts):
            states = [(xs, vs)]
            if seg > 1:
                x = xs.clone()
                v = vs.clone()
                hp, hv = engine.run_dkd(x, v, m, seg - 1, dt, eps, algorithm="direct", precision=precision,
                                        hist_stride=1)
                states += [(hp[j], hv[j]) for j in range(seg - 1)]
            for xj, vj in reversed(states):
                xh = xj + ((0.5 * vj) * dt) * KMS_MYR_TO_KPC
                w = vb + c * xb
                lam = (ACCEL_UNIT * dt) * w
                engine.direct_vjp(xh.contiguous(), m, eps, lam.contiguous(), precision=precision,
                                  grad_pos=gpos, grad_mass=gmass)
                xhb = xb + gpos
                mb += gmass
                vb = w + c * xhb
                xb = xhb
        ctx.ckpts = None
        return xb, vb, mb, None, None, None, None, None


def rollout(x0, v0, m, nsteps, dt, eps, checkpoint_every=20, precision="mixed"):
    """Differentiable ``nsteps`` leapfrog steps; returns (x_T, v_T)."""
    return _Rollout.apply(x0, v0, m, int(nsteps), float(dt), float(eps), int(checkpoint_every), precision)
