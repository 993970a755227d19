"""The identity behind adjoint.tangent_rollout, on the CPU with dense PyTorch FP64:
for the softened direct-sum acceleration a(x) (the reference's pair law,
gravhopper/_jbgrav.c:155-185), the Jacobian-vector product equals the
vector-Jacobian product of the mass-weighted vector divided by the masses,
J u = (J^T (m u)) / m, for unequal masses too."""
import numpy as np
import pytest


def _accel(torch, x, m, eps):
    d = x[None, :, :] - x[:, None, :]
    eye = torch.eye(x.shape[0], dtype=x.dtype)
    s = (d * d).sum(-1) + eps * eps + eye  # the self pair (d = 0) gets s = 1, then no term
    inv = s ** -1.5 * (1.0 - eye)
    return (m[None, :, None] * d * inv[..., None]).sum(1)


@pytest.mark.parametrize("eps", [1e-2, 0.0])
def test_jvp_equals_mass_weighted_vjp(eps):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    n = 64
    x = torch.from_numpy(rng.normal(size=(n, 3)))
    m = torch.from_numpy(rng.uniform(0.2, 3.0, size=n))
    u = torch.from_numpy(rng.normal(size=(n, 3)))
    _, jvp = torch.func.jvp(lambda y: _accel(torch, y, m, eps), (x,), (u,))
    _, vjp_fn = torch.func.vjp(lambda y: _accel(torch, y, m, eps), x)
    (vjp,) = vjp_fn(m[:, None] * u)
    assert torch.isfinite(jvp).all()
    np.testing.assert_allclose((vjp / m[:, None]).numpy(), jvp.numpy(), rtol=1e-12, atol=1e-12 * float(jvp.abs().max()))


def test_tangent_rollout_refuses_zero_mass():
    """The identity divides by the masses: a zero mass is refused before any work."""
    torch = pytest.importorskip("torch")
    from gravhopper_gb300.adjoint import tangent_rollout
    x = torch.zeros((4, 3), dtype=torch.float64)
    m = torch.tensor([1.0, 0.0, 1.0, 1.0], dtype=torch.float64)
    with pytest.raises(ValueError, match="nonzero"):
        tangent_rollout(x, x, m, 1, 0.005, 5e-5, x)
