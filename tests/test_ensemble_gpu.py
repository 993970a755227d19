"""Batched ensemble on the GPU: every system matches its own FP64 oracle trajectory,
graph replay equals plain launches bit for bit, every tile configuration agrees."""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


def _systems(k=10, seed=0):
    from gravhopper_gb300 import ics
    return ics.plummer_ensemble(k, nmin=40, nmax=900, seed=seed)


def test_ensemble_matches_oracle_per_system(lib, cuda):
    # Few steps: close encounters in these small systems amplify any FP32 force error
    # (a float32 CPU emulation of system 1 drifts 1.5e-7 kpc from FP64 by step 12).
    from gravhopper_gb300.ensemble import Ensemble
    systems = _systems()
    ens = Ensemble(systems, device=cuda)
    ens.run(4, use_graph=True)
    for k, s in enumerate(systems):
        rx, rv = oracle.dkd_run(s["pos"], s["vel"], s["mass"], s["dt"], s["eps"], 4)
        x, v = ens.system(k)
        # float32 CPU emulation of these systems deviates by up to 5.5e-8 relative
        assert np.abs(x - rx).max() <= 1e-6 * np.abs(rx).max(), k
        assert np.abs(v - rv).max() <= 1e-5 * np.abs(rv).max(), k


def test_ensemble_equal_and_unequal_masses(lib, cuda):
    """Systems whose masses are all equal take the equal-mass loop (the mass applied
    once per target), the others the general loop, in the same launch; each matches its
    own FP64 oracle trajectory as in test_ensemble_matches_oracle_per_system."""
    from gravhopper_gb300.ensemble import Ensemble
    systems = _systems(8, seed=5)
    rng = np.random.default_rng(6)
    for k in (1, 4, 6):
        s = systems[k]
        s["mass"] = s["mass"] * rng.uniform(0.5, 1.5, size=s["mass"].shape)
    ens = Ensemble(systems, device=cuda)
    ens.run(4, use_graph=False)
    for k, s in enumerate(systems):
        rx, rv = oracle.dkd_run(s["pos"], s["vel"], s["mass"], s["dt"], s["eps"], 4)
        x, v = ens.system(k)
        assert np.abs(x - rx).max() <= 1e-6 * np.abs(rx).max(), k
        assert np.abs(v - rv).max() <= 1e-5 * np.abs(rv).max(), k


def test_graph_replay_is_bitwise_plain(lib, cuda):
    from gravhopper_gb300.ensemble import Ensemble
    systems = _systems(7, seed=3)
    a = Ensemble(systems, device=cuda)
    b = Ensemble(systems, device=cuda)
    a.run(70, use_graph=True)   # one 64-step graph replay + 6 plain steps
    b.run(70, use_graph=False)
    assert (a.pos == b.pos).all() and (a.vel == b.vel).all()


def test_all_tile_configs_agree(lib, cuda):
    from gravhopper_gb300 import _capi
    from gravhopper_gb300.ensemble import Ensemble
    systems = _systems(5, seed=9)
    ref = None
    for cfg in range(_capi.load().gh_ensemble_num_configs()):
        e = Ensemble(systems, device=cuda)
        e.run(5, config=cfg, use_graph=False)
        x = e.pos.cpu().numpy()
        if ref is None:
            ref = x
        else:
            # each configuration sums the pairs in its own chunks; a close pair amplifies
            # that rounding over 5 steps, so they agree as each agrees with the FP64
            # oracle (test_ensemble_matches_oracle_per_system)
            np.testing.assert_allclose(x, ref, rtol=0, atol=1e-6 * np.abs(ref).max())


def test_autotune_and_one_by_one(lib, cuda, tmp_path, monkeypatch):
    monkeypatch.setenv("XDG_CACHE_HOME", str(tmp_path))
    from gravhopper_gb300.ensemble import Ensemble, autotune, run_one_by_one
    systems = _systems(6, seed=4)
    e = Ensemble(systems, device=cuda)
    best, times = autotune(e, steps=2)
    assert best in times and all(t > 0 for t in times.values())
    assert autotune(e, steps=2)[0] == best  # cached
    e.run(4)
    f = Ensemble(systems, device=cuda)
    run_one_by_one(f, 4)
    np.testing.assert_allclose(e.pos.cpu().numpy(), f.pos.cpu().numpy(), rtol=0, atol=1e-9)


def test_ensemble_edge_systems(lib, cuda):
    """Systems of 0, 1 and 2 particles and one with eps = 0 (the variant that gives a
    coincident pair no term) in one ensemble beside ordinary ones: each matches its
    own FP64 oracle trajectory (one particle drifts at constant velocity, as
    Simulation.calculate_acceleration gives Np <= 1 no force, gravhopper.py:419-459)."""
    from gravhopper_gb300.ensemble import Ensemble
    systems = _systems(4, seed=5)
    rng = np.random.default_rng(6)
    one = {"pos": rng.normal(size=(1, 3)) * 1e-3, "vel": rng.normal(size=(1, 3)), "mass": np.ones(1) * 1e3,
           "eps": 5e-5, "dt": 0.005}
    empty = {"pos": np.zeros((0, 3)), "vel": np.zeros((0, 3)), "mass": np.zeros(0), "eps": 5e-5, "dt": 0.005}
    two = {"pos": np.array([[0.0, 0.0, 0.0], [1e-3, 2e-4, 0.0]]), "vel": np.array([[0.0, 5.0, 0.0], [0.0, -5.0, 1.0]]),
           "mass": np.array([1e4, 3e3]), "eps": 5e-5, "dt": 0.005}
    zero_eps = dict(systems[0])
    zero_eps["eps"] = 0.0
    systems = [systems[1], one, empty, two, zero_eps, systems[2]]
    ens = Ensemble(systems, device=cuda)
    ens.run(3, use_graph=False)
    for k, s in enumerate(systems):
        x, v = ens.system(k)
        if len(s["mass"]) == 0:
            assert x.shape == (0, 3)
            continue
        rx, rv = oracle.dkd_run(s["pos"], s["vel"], s["mass"], s["dt"], s["eps"], 3)
        assert np.isfinite(x).all() and np.isfinite(v).all(), k
        assert np.abs(x - rx).max() <= 1e-6 * np.abs(rx).max(), k
        assert np.abs(v - rv).max() <= 1e-5 * max(np.abs(rv).max(), 1e-30), k
