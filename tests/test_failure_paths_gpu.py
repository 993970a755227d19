"""Error paths on the GPU, made to fire without faulting or hanging the device.

* Out of memory: host-side injection makes a workspace reservation fail as a failed
  cudaMalloc would (GH_ERR_OOM, with a message); the next call works and gives the
  oracle's result.  The reference calls exit() there (gravhopper/_jbgrav.c:364, 779).
* Bounded waits: the radix sort's decoupled look-back waits for a tile that is never
  published and gives up after a short limit (GH_ERR_TIMEOUT, context still usable);
  a tree build that finds its sort's wait given up reports GH_ERR_TIMEOUT.
* Non-finite input: the direct sum propagates NaN and infinity exactly as the
  reference's arithmetic does (gravhopper/_jbgrav.c:155-185); the tree refuses NaN or
  infinite particles with GH_ERR_ARG, where the reference's insert never terminates
  (its "p > center" test is false at every level, _jbgrav.c:401-413, 441-450), and
  gives NaN for NaN target points, as the reference's walk does.
"""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


def test_allocation_failure_is_reported_and_recovers(lib, cuda):
    from gravhopper_gb300 import _capi, _jbgrav, ics
    ic = ics.plummer(3000, seed=21)
    ref_d = oracle.direct_summation(ic["pos"], ic["mass"], 5e-5)
    ref_t = oracle.tree_force(ic["pos"], ic["mass"], 5e-5, 0.7)
    calls = [
        (lambda: _jbgrav.direct_summation(ic["pos"], ic["mass"], 5e-5), ref_d, 0.0),
        (lambda: _jbgrav.direct_summation_mixed(ic["pos"], ic["mass"], 5e-5), ref_d, 1e-6),
        (lambda: _jbgrav.tree_force(ic["pos"], ic["mass"], 5e-5, 0.7), ref_t, 1e-12),
    ]
    try:
        for fn, ref, tol in calls:
            for k in (1, 3):  # the first reservation of the call, and a later one
                _capi.inject(_capi.GH_INJECT_ALLOC, k)
                failed = False
                try:
                    fn()
                except _capi.EngineError as e:
                    failed = True
                    assert e.code == _capi.GH_ERR_OOM
                    assert "out of memory" in str(e)
                _capi.inject(_capi.GH_INJECT_ALLOC, 0)
                if k == 1:
                    assert failed
                got = fn()
                if tol == 0.0:
                    np.testing.assert_array_equal(got, ref)
                else:
                    r = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
                    assert np.sqrt(np.mean(r * r)) <= tol
    finally:
        _capi.inject(_capi.GH_INJECT_ALLOC, 0)


def test_ensemble_allocation_failure_recovers(lib, cuda):
    import torch

    from gravhopper_gb300 import _capi, ics
    from gravhopper_gb300.ensemble import Ensemble
    systems = ics.plummer_ensemble(6, seed=3)
    e_ref = Ensemble(systems, device=cuda)
    e_ref.run(4, use_graph=False)
    e = Ensemble(systems, device=cuda)
    _capi.inject(_capi.GH_INJECT_ALLOC, 1)
    try:
        with pytest.raises(_capi.EngineError) as err:
            e.run(4, use_graph=False)
        assert err.value.code == _capi.GH_ERR_OOM
    finally:
        _capi.inject(_capi.GH_INJECT_ALLOC, 0)
    torch.cuda.synchronize()
    e.run(4, use_graph=False)  # the failed call advanced nothing
    torch.cuda.synchronize()
    assert torch.equal(e.pos, e_ref.pos) and torch.equal(e.vel, e_ref.vel)


def test_sort_lookback_wait_gives_up(lib, cuda):
    """The only CTA waits on a predecessor tile that never publishes; after 2 ms of the
    GPU's timer the wait gives up and the call reports GH_ERR_TIMEOUT."""
    from gravhopper_gb300 import _capi, _jbgrav, ics
    rc, ns = _capi.sort_stall(2_000_000)
    assert rc == _capi.GH_ERR_TIMEOUT, rc
    assert b"gave up" in _capi.load().gh_last_error()
    assert 2_000_000 <= ns < 5_000_000_000
    # the context is still usable
    ic = ics.plummer(2000, seed=22)
    got = _jbgrav.tree_force(ic["pos"], ic["mass"], 5e-5, 0.7)
    ref = oracle.tree_force(ic["pos"], ic["mass"], 5e-5, 0.7)
    r = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert np.sqrt(np.mean(r * r)) <= 1e-12


def test_tree_reports_sort_timeout(lib, cuda):
    from gravhopper_gb300 import _capi, _jbgrav, ics
    ic = ics.plummer(2000, seed=23)
    _capi.inject(_capi.GH_INJECT_TREE_WAIT, 1)
    try:
        with pytest.raises(_capi.EngineError) as err:
            _jbgrav.tree_force(ic["pos"], ic["mass"], 5e-5, 0.7)
        assert err.value.code == _capi.GH_ERR_TIMEOUT
    finally:
        _capi.inject(_capi.GH_INJECT_TREE_WAIT, 0)
    got = _jbgrav.tree_force(ic["pos"], ic["mass"], 5e-5, 0.7)
    assert np.isfinite(got).all()


def _nonfinite_cases(n=700, seed=24):
    rng = np.random.default_rng(seed)
    pos = rng.normal(size=(n, 3)) * 1e-3
    mass = rng.uniform(0.5, 2.0, size=n)
    cases = []
    for what, val in (("pos", np.nan), ("pos", np.inf), ("pos", -np.inf), ("mass", np.nan)):
        p, m = pos.copy(), mass.copy()
        k = int(rng.integers(n))
        if what == "pos":
            p[k, int(rng.integers(3))] = val
        else:
            m[k] = val
        cases.append((what, val, k, p, m))
    return cases


@pytest.mark.parametrize("form", [0, 1])
def test_nonfinite_direct_fp64_matches_reference(lib, cuda, form):
    from gravhopper_gb300 import _capi, _jbgrav
    _capi.call("gh_direct_set_fp64_form", form)
    try:
        for what, val, k, p, m in _nonfinite_cases():
            for eps in (5e-5, 0.0):
                got = _jbgrav.direct_summation(p, m, eps)
                ref = oracle.direct_summation(p, m, eps)
                assert np.array_equal(got, ref, equal_nan=True), (what, val, eps)
            fp = p[:50]
            got = _jbgrav.direct_summation_position(p, m, fp, 0.0)
            assert np.array_equal(got, oracle.direct_summation_position(p, m, fp, 0.0), equal_nan=True)
    finally:
        _capi.call("gh_direct_set_fp64_form", -1)


def test_nonfinite_direct_mixed_propagates(lib, cuda):
    """The mixed form is non-finite exactly where the reference is, and within its
    tolerance elsewhere.  One documented difference: it evaluates the self pair as a
    zero-offset term, m_k (x_k - x_k), which is NaN when m_k is NaN or a coordinate of
    x_k is infinite, so that particle's own row is NaN in every component where the
    reference (which skips the self pair) has finite components."""
    from gravhopper_gb300 import _jbgrav
    for what, val, k, p, m in _nonfinite_cases():
        got = _jbgrav.direct_summation_mixed(p, m, 5e-5)
        ref = oracle.direct_summation(p, m, 5e-5)
        bad_ref = ~np.isfinite(ref)
        bad_ref[k] = True
        np.testing.assert_array_equal(~np.isfinite(got), bad_ref, err_msg=f"{what} {val}")
        rows = np.isfinite(ref).all(axis=1) & np.isfinite(got).all(axis=1)
        if rows.any():
            r = np.linalg.norm(got[rows] - ref[rows], axis=1) / np.linalg.norm(ref[rows], axis=1)
            assert np.sqrt(np.mean(r * r)) <= 1e-6


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nonfinite_tree_sources_refused(lib, cuda, precision):
    import torch

    from gravhopper_gb300 import _capi, engine
    for what, val, k, p, m in _nonfinite_cases():
        x = torch.from_numpy(p).to(cuda)
        mm = torch.from_numpy(m).to(cuda)
        with pytest.raises(_capi.EngineError) as err:
            engine.tree_force(x, mm, 5e-5, 0.7, precision=precision)
        assert err.value.code == _capi.GH_ERR_ARG, (what, val)
        assert "finite" in str(err.value)
    # the library is usable afterwards
    _, _, _, p, m = _nonfinite_cases()[0]
    p = np.nan_to_num(p)
    x = torch.from_numpy(p).to(cuda)
    got = engine.tree_force(x, torch.from_numpy(m).to(cuda), 5e-5, 0.7, precision=precision).cpu().numpy()
    ref = oracle.tree_force(p, m, 5e-5, 0.7)
    r = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert np.sqrt(np.mean(r * r)) <= (1e-12 if precision == "fp64" else 1e-6)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nan_target_points_give_nan(lib, cuda, precision):
    import torch

    from gravhopper_gb300 import engine, ics
    ic = ics.plummer(3000, seed=25)
    rng = np.random.default_rng(3)
    fp = rng.normal(size=(200, 3)) * 1e-3
    fp[[3, 77, 150], [0, 1, 2]] = np.nan
    x = torch.from_numpy(ic["pos"]).to(cuda)
    m = torch.from_numpy(ic["mass"]).to(cuda)
    got = engine.tree_force(x, m, 5e-5, 0.7, force_pos=torch.from_numpy(fp).to(cuda),
                            precision=precision).cpu().numpy()
    ref = oracle.tree_force_position(ic["pos"], ic["mass"], fp, 5e-5, 0.7)
    np.testing.assert_array_equal(np.isnan(got), np.isnan(ref))
    ok = ~np.isnan(ref).any(axis=1)
    r = np.linalg.norm(got[ok] - ref[ok], axis=1) / np.linalg.norm(ref[ok], axis=1)
    assert np.sqrt(np.mean(r * r)) <= (1e-12 if precision == "fp64" else 1e-6)
