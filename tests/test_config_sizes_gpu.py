"""Parity at the sizes the benchmark workloads run, on sampled targets.

The direct-sum scaling workload runs Plummer spheres of N = 262,144 and 1,048,576
particles and the Barnes-Hut workload a Hernquist sphere plus exponential disk of
N = 1,048,576 at theta 0.5 and 0.7.  The kernels, tile shapes and key widths chosen
at those sizes differ from the ones the smaller tests reach: the thread-per-target
FP64 kernel (the default above ~311,000 targets), the 384 x 6 scalar tile of the
fused leapfrog step (N >= 131,072), the 512 x 4 tile of the mixed force, two-word
octree keys with the full multi-word sort.  Each test computes every particle on the
GPU through the C ABI and checks a seeded sample of targets against the oracle's
target-point forms (gravhopper/_jbgrav.c:299-353 for the direct sum, :634-806 for the
tree), whose result for a target that is one of the particles equals the self-force
(the self pair contributes +0.0).

Tolerances, as elsewhere: FP64 direct sum bit-exact; mixed direct sum rms relative
error <= 1e-6 and max <= 1e-3; FP64 tree rms <= 1e-12, max <= 1e-9; mixed tree rms
<= 1e-6, max <= 1e-3.
"""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu

EPS_PLUMMER = 5e-5   # 0.05 pc
DT_PLUMMER = 0.005   # Myr
EPS_TREE = 0.1       # kpc
SAMPLE = 4096
TREE_SAMPLE = 2048


def rel_err(a, ref):
    num = np.linalg.norm(a - ref, axis=1)
    den = np.linalg.norm(ref, axis=1)
    r = num / np.where(den > 0, den, 1.0)
    return float(np.sqrt(np.mean(r * r))), float(r.max())


def sample(n, k, seed):
    return np.sort(np.random.default_rng(seed).choice(n, size=k, replace=False))


_IC = {}


def plummer(n):
    from gravhopper_gb300 import ics
    if ("p", n) not in _IC:
        _IC[("p", n)] = ics.plummer(n, seed=n + 1)
    return _IC[("p", n)]


def hernquist_disk(n):
    from gravhopper_gb300 import ics
    if ("h", n) not in _IC:
        _IC[("h", n)] = ics.hernquist_disk(n, seed=n + 2)
    return _IC[("h", n)]


@pytest.mark.parametrize("form", [0, 1])
def test_fp64_direct_262144_bitexact(lib, cuda, form):
    """FP64 self-force at N = 262,144, both FP64 kernels: thread per target (form 0,
    what N above ~311,000 selects) and CTA-wide ordered sums (form 1, the default
    here), bit for bit against the oracle on 4096 sampled targets."""
    import torch

    from gravhopper_gb300 import _capi, engine
    n = 262144
    ic = plummer(n)
    x = torch.from_numpy(ic["pos"]).to(cuda)
    m = torch.from_numpy(ic["mass"]).to(cuda)
    idx = sample(n, SAMPLE, 11)
    _capi.call("gh_direct_set_fp64_form", form)
    try:
        got = engine.direct_force(x, m, EPS_PLUMMER, precision="fp64").cpu().numpy()[idx]
    finally:
        _capi.call("gh_direct_set_fp64_form", -1)
    ref = oracle.direct_summation_position(ic["pos"], ic["mass"], ic["pos"][idx], EPS_PLUMMER)
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("n", [262144, 1048576])
def test_mixed_direct_force_config_sizes(lib, cuda, n):
    import torch

    from gravhopper_gb300 import engine
    ic = plummer(n)
    x = torch.from_numpy(ic["pos"]).to(cuda)
    m = torch.from_numpy(ic["mass"]).to(cuda)
    idx = sample(n, SAMPLE, 12)
    got = engine.direct_force(x, m, EPS_PLUMMER, precision="mixed").cpu().numpy()[idx]
    ref = oracle.direct_summation_position(ic["pos"], ic["mass"], ic["pos"][idx], EPS_PLUMMER)
    rms, mx = rel_err(got, ref)
    assert rms <= 1e-6 and mx <= 1e-3, (n, rms, mx)


@pytest.mark.parametrize("n", [262144, 1048576])
def test_mixed_dkd_step_config_sizes(lib, cuda, n):
    """One fused mixed leapfrog step (384 x 6 tile).  The kick of each sampled particle,
    v1 - v, is checked against the oracle's FP64 force at the half-drifted positions
    (Simulation.perform_timestep, gravhopper/gravhopper.py:405-416) to the mixed
    tolerance; the final drift, FP64 in the epilogue, reproduces the host's
    uncontracted formula bit for bit from the GPU's new velocity."""
    import torch

    from gravhopper_gb300 import engine
    K = oracle.KMS_MYR_TO_KPC
    ic = plummer(n)
    x = torch.from_numpy(ic["pos"]).to(cuda)
    v = torch.from_numpy(ic["vel"]).to(cuda)
    m = torch.from_numpy(ic["mass"]).to(cuda)
    engine.run_dkd(x, v, m, 1, DT_PLUMMER, EPS_PLUMMER, algorithm="direct", precision="mixed")
    idx = sample(n, SAMPLE, 13)
    x1 = x.cpu().numpy()[idx]
    v1 = v.cpu().numpy()[idx]
    xh = ic["pos"] + ((0.5 * ic["vel"]) * DT_PLUMMER) * K
    acc = oracle.direct_summation_position(xh, ic["mass"], xh[idx], EPS_PLUMMER) * oracle.ACCEL_UNIT
    kick_ref = acc * DT_PLUMMER
    rms, mx = rel_err(v1 - ic["vel"][idx], kick_ref)
    assert rms <= 1e-6 and mx <= 1e-3, (n, rms, mx)
    np.testing.assert_array_equal(x1, xh[idx] + ((0.5 * v1) * DT_PLUMMER) * K)


_TREE_REF = {}


def tree_ref(theta):
    n = 1048576
    if theta not in _TREE_REF:
        ic = hernquist_disk(n)
        idx = sample(n, TREE_SAMPLE, 14)
        _TREE_REF[theta] = (idx, oracle.tree_force_position(ic["pos"], ic["mass"], ic["pos"][idx], EPS_TREE, theta))
    return _TREE_REF[theta]


@pytest.mark.parametrize("precision,rms_tol,max_tol", [("fp64", 1e-12, 1e-9), ("mixed", 1e-6, 1e-3)])
@pytest.mark.parametrize("theta", [0.5, 0.7])
def test_tree_hernquist_disk_1m(lib, cuda, theta, precision, rms_tol, max_tol):
    """Barnes-Hut self-force of the 1,048,576-particle Hernquist sphere plus disk:
    its outliers make the root cell ~10^6 kpc wide, so the core needs two-word keys
    and the full multi-word sort."""
    import torch

    from gravhopper_gb300 import engine
    ic = hernquist_disk(1048576)
    x = torch.from_numpy(ic["pos"]).to(cuda)
    m = torch.from_numpy(ic["mass"]).to(cuda)
    idx, ref = tree_ref(theta)
    got = engine.tree_force(x, m, EPS_TREE, theta, precision=precision).cpu().numpy()[idx]
    rms, mx = rel_err(got, ref)
    assert rms <= rms_tol and mx <= max_tol, (theta, precision, rms, mx)
