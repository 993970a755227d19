"""The target-sharded run entry on the GPU, one process.

The sharded leapfrog's FP64 form is bit-identical to one process only if the
position-mode direct sum over all particles, evaluated at the particles themselves,
gives each particle's own term as an exact +0.0 (the reference's position workhorse,
gravhopper/_jbgrav.c:299-353, and its self-force workhorse, :140-193, then agree bit
for bit).  Checked here through the GPU kernels for both FP64 forms, with and without
softening, and the entry itself (sharding.run_dkd_sharded, with the GPU force) against
the engine's fused leapfrog (gravhopper/gravhopper.py:405-416): FP64 bit for bit,
mixed within the mixed tolerance (rms 1e-6 of the velocity change)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("form", [0, 1])
@pytest.mark.parametrize("eps", [5e-5, 0.0])
def test_position_mode_self_term_is_exact_zero(lib, cuda, form, eps):
    import torch

    from gravhopper_gb300 import _capi, engine, ics
    ic = ics.plummer(3001, seed=41)
    x = torch.from_numpy(ic["pos"]).to(cuda)
    m = torch.from_numpy(ic["mass"]).to(cuda)
    _capi.call("gh_direct_set_fp64_form", form)
    try:
        a_self = engine.direct_force(x, m, eps, precision="fp64").cpu().numpy()
        a_pos = engine.direct_force(x, m, eps, force_pos=x, precision="fp64").cpu().numpy()
    finally:
        _capi.call("gh_direct_set_fp64_form", -1)
    np.testing.assert_array_equal(a_pos, a_self)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sharded_entry_single_process_matches_fused_leapfrog(lib, cuda, precision):
    import torch

    from gravhopper_gb300 import engine, ics, sharding
    n, steps, dt, eps = 5000, 3, 0.005, 5e-5
    ic = ics.plummer(n, seed=42)
    m = torch.from_numpy(ic["mass"]).to(cuda)
    x1 = torch.from_numpy(ic["pos"]).to(cuda)
    v1 = torch.from_numpy(ic["vel"]).to(cuda)
    sharding.run_dkd_sharded(x1, v1, m, [n], steps, dt, eps, precision=precision)
    x2 = torch.from_numpy(ic["pos"]).to(cuda)
    v2 = torch.from_numpy(ic["vel"]).to(cuda)
    engine.run_dkd(x2, v2, m, steps, dt, eps, algorithm="direct", precision=precision)
    if precision == "fp64":
        assert torch.equal(x1, x2) and torch.equal(v1, v2)
    else:
        dv1 = (v1 - torch.from_numpy(ic["vel"]).to(cuda)).cpu().numpy()
        dv2 = (v2 - torch.from_numpy(ic["vel"]).to(cuda)).cpu().numpy()
        r = np.linalg.norm(dv1 - dv2, axis=1) / np.linalg.norm(dv2, axis=1)
        assert np.sqrt(np.mean(r * r)) <= 1e-6
