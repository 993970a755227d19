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
            np.testing.assert_allclose(x, ref, rtol=0, atol=1e-9)


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
