"""Seeded initial-condition generators for the engine's workloads.

Units: kpc, km/s, Msun (the reference's internal units, gravhopper/gravhopper.py:146-151).
These are this project's own samplers of the published distributions; the reference's
generators (gravhopper/gravhopper.py:1327-1785) need astropy and are not run here.

* ``plummer``: Plummer sphere (Plummer 1911; Aarseth, Henon & Wielen 1974):
  r = b / sqrt(u^(-2/3) - 1), v = q sqrt(2GM/b) (1 + r^2/b^2)^(-1/4) with q drawn by
  rejection from q^2 (1-q^2)^(7/2); isotropic directions; centred (force_centers,
  gravhopper/gravhopper.py:1740-1785).
* ``hernquist_disk``: 70 % Hernquist sphere (Hernquist 1990) with r = a sqrt(u)/(1-sqrt(u))
  and Gaussian velocities of the closed-form isotropic Jeans dispersion, plus a 30 %
  exponential disk (R ~ Gamma(2, Rd), sech^2(z/z0) vertical profile, circular speed of
  the combined enclosed mass, 10 % Gaussian dispersion).
* ``plummer_ensemble``: many Plummer spheres of uneven N for batched integration.
"""
from __future__ import annotations

import numpy as np

from .units import G_KPC_KMS2_MSUN as G


def _isotropic(rng, n):
    cth = rng.uniform(-1.0, 1.0, size=n)
    phi = rng.uniform(0.0, 2.0 * np.pi, size=n)
    sth = np.sqrt(1.0 - cth * cth)
    return np.stack([sth * np.cos(phi), sth * np.sin(phi), cth], axis=1)


def _centre(pos, vel, mass):
    mtot = mass.sum()
    pos = pos - (mass[:, None] * pos).sum(0) / mtot
    vel = vel - (mass[:, None] * vel).sum(0) / mtot
    return pos, vel


def plummer(n, b=1e-3, totmass=1e6, seed=0):
    """Plummer sphere of ``n`` equal-mass particles (b in kpc, totmass in Msun)."""
    rng = np.random.default_rng(seed)
    u = rng.uniform(0.0, 1.0, size=n)
    u = np.clip(u, 1e-300, 1.0 - 1e-16)
    r = b / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
    pos = r[:, None] * _isotropic(rng, n)
    # q from g(q) = q^2 (1-q^2)^(7/2) by rejection; g peaks at q^2 = 2/9.
    gmax = (2.0 / 9.0) * (7.0 / 9.0) ** 3.5
    q = np.empty(n)
    filled = 0
    while filled < n:
        k = max(2 * (n - filled), 64)
        qq = rng.uniform(0.0, 1.0, size=k)
        yy = rng.uniform(0.0, gmax, size=k)
        acc = qq[yy < qq * qq * (1.0 - qq * qq) ** 3.5]
        take = min(n - filled, acc.size)
        q[filled:filled + take] = acc[:take]
        filled += take
    speed = q * np.sqrt(2.0 * G * totmass / b) * (1.0 + (r / b) ** 2) ** (-0.25)
    vel = speed[:, None] * _isotropic(rng, n)
    mass = np.full(n, totmass / n)
    pos, vel = _centre(pos, vel, mass)
    return {"pos": pos, "vel": vel, "mass": mass}


def hernquist_sigma2(r, a, m):
    """Isotropic Jeans radial dispersion^2 of a Hernquist sphere [(km/s)^2] (Hernquist 1990 eq. 10)."""
    r = np.asarray(r, dtype=np.float64)
    x = r / a
    out = np.empty_like(x)
    small = x < 50.0
    xs = np.maximum(x[small], 1e-300)
    t = (12.0 * xs * (1.0 + xs) ** 3 * np.log1p(1.0 / xs)
         - xs / (1.0 + xs) * (25.0 + 52.0 * xs + 42.0 * xs ** 2 + 12.0 * xs ** 3))
    out[small] = G * m / (12.0 * a) * t
    # Large-r series of the bracket in y = a/r (the closed form cancels
    # catastrophically in FP64 there): 12/5 y - 14/5 y^2 + 102/35 y^3 - 207/70 y^4
    # + 125/42 y^5 - 209/70 y^6 + 329/110 y^7 + O(y^8).
    y = 1.0 / x[~small]
    coef = [329.0 / 110, -209.0 / 70, 125.0 / 42, -207.0 / 70, 102.0 / 35, -14.0 / 5, 12.0 / 5, 0.0]
    out[~small] = G * m / (12.0 * a) * np.polyval(coef, y)
    return np.maximum(out, 0.0)


def hernquist_disk(n, totmass=1e11, bulge_frac=0.7, a=1.0, rd=3.0, z0=0.3, disp=0.1, seed=0):
    """Hernquist spheroid plus exponential disk, ``n`` equal-mass particles."""
    rng = np.random.default_rng(seed)
    nh = int(round(bulge_frac * n))
    nd = n - nh
    mh = totmass * nh / n
    md = totmass - mh
    # Hernquist sphere
    u = rng.uniform(0.0, 1.0, size=nh)
    su = np.sqrt(np.clip(u, 0.0, 1.0 - 1e-16))
    r = a * su / (1.0 - su)
    ph = r[:, None] * _isotropic(rng, nh)
    sig = np.sqrt(hernquist_sigma2(r, a, mh))
    vh = sig[:, None] * rng.normal(size=(nh, 3))
    # Exponential disk
    R = rng.gamma(2.0, rd, size=nd)
    phi = rng.uniform(0.0, 2.0 * np.pi, size=nd)
    z = z0 * np.arctanh(np.clip(2.0 * rng.uniform(0.0, 1.0, size=nd) - 1.0, -1 + 1e-16, 1 - 1e-16))
    pd = np.stack([R * np.cos(phi), R * np.sin(phi), z], axis=1)
    m_enc = mh * R * R / (R + a) ** 2 + md * (1.0 - (1.0 + R / rd) * np.exp(-R / rd))
    vc = np.sqrt(G * m_enc / np.maximum(R, 1e-12))
    vd = np.stack([-vc * np.sin(phi), vc * np.cos(phi), np.zeros(nd)], axis=1)
    vd = vd + (disp * vc)[:, None] * rng.normal(size=(nd, 3))
    pos = np.concatenate([ph, pd])
    vel = np.concatenate([vh, vd])
    mass = np.full(n, totmass / n)
    pos, vel = _centre(pos, vel, mass)
    return {"pos": pos, "vel": vel, "mass": mass}


def plummer_ensemble(n_systems=512, nmin=256, nmax=8192, totmass=1e6, seed=0):
    """Independent Plummer spheres with log-uniform N, b ~ U(0.5, 2) pc.

    Each system gets eps = 0.05 b and dt = 0.005 Myr * (b / 1 pc)^1.5.
    Returns a list of dicts with pos, vel, mass, eps, dt.
    """
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(nmin), np.log(nmax + 1), size=n_systems)).astype(np.int64)
    ns = np.clip(ns, nmin, nmax)
    bs = rng.uniform(0.5e-3, 2.0e-3, size=n_systems)
    out = []
    for k in range(n_systems):
        s = plummer(int(ns[k]), b=float(bs[k]), totmass=totmass, seed=int(rng.integers(1 << 62)))
        s["eps"] = 0.05 * float(bs[k])
        s["dt"] = 0.005 * (float(bs[k]) / 1e-3) ** 1.5
        out.append(s)
    return out
