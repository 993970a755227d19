"""Barnes-Hut parity on the GPU against the reference tree.

The GPU tree has the reference's cells and takes the reference's opening decisions
exactly; internal-cell moments are summed in a different order and the interaction
uses a Newton-refined reciprocal square root, so forces agree to rounding.  Stated
tolerance, per particle, |a_gpu - a_ref| / |a_ref|: rms <= 1e-12, max <= 1e-9.
"""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu

TREE_RMS_TOL = 1e-12
TREE_MAX_TOL = 1e-9


def check(got, ref, rms_tol=TREE_RMS_TOL, max_tol=TREE_MAX_TOL):
    num = np.linalg.norm(got - ref, axis=1)
    den = np.linalg.norm(ref, axis=1)
    zero = den == 0
    assert np.all(num[zero] == 0), "nonzero force where the reference has exactly zero"
    r = num[~zero] / den[~zero]
    if r.size:
        rms = float(np.sqrt(np.mean(r * r)))
        assert rms <= rms_tol and r.max() <= max_tol, (rms, float(r.max()))


@pytest.mark.parametrize("theta", [0.0, 0.5, 0.7, 1.0])
def test_tree_matches_reference_golden(golden, lib, cuda, theta):
    from gravhopper_gb300 import _jbgrav
    key = str(theta).replace(".", "p")
    got = _jbgrav.tree_force(golden["tree_pos"], golden["tree_mass"], 5e-5, theta)
    check(got, golden[f"tree_{key}_out"])
    got = _jbgrav.tree_force_position(golden["tree_pos"], golden["tree_mass"], golden["tree_fpos"], 0.0, theta)
    check(got, golden[f"treepos_{key}_out"])


def test_tree_small_and_hernquist_golden(golden, lib, cuda):
    from gravhopper_gb300 import _jbgrav
    for n in (1, 2, 3):
        k = f"tree_small_{n}"
        check(_jbgrav.tree_force(golden[k + "_pos"], golden[k + "_mass"], 0.01, 0.7), golden[k + "_out"])
    for th in (0.5, 0.7):
        key = str(th).replace(".", "p")
        check(_jbgrav.tree_force(golden["hq_pos"], golden["hq_mass"], 0.1, th), golden[f"hq_{key}_out"])


@pytest.mark.parametrize("theta", [0.5, 0.7])
def test_tree_matches_oracle_hernquist_disk(lib, cuda, theta):
    from gravhopper_gb300 import _jbgrav, ics
    ic = ics.hernquist_disk(30000, seed=3)
    got = _jbgrav.tree_force(ic["pos"], ic["mass"], 0.1, theta)
    check(got, oracle.tree_force(ic["pos"], ic["mass"], 0.1, theta))


def test_tree_deep_levels_widen_keys(lib, cuda):
    # pairs separated by ~1e-13 in a unit box need ~45 octree levels (> 2 key words)
    from gravhopper_gb300 import _jbgrav
    rng = np.random.default_rng(5)
    base = rng.uniform(-1, 1, size=(50, 3))
    pos = np.concatenate([base, base + 1e-13 * rng.normal(size=base.shape)])
    m = rng.uniform(1, 2, size=100)
    check(_jbgrav.tree_force(pos, m, 1e-3, 0.6), oracle.tree_force(pos, m, 1e-3, 0.6))


@pytest.mark.parametrize("clumps,per_clump", [(30, 100), (1, 2000)])
def test_tree_dense_clumps(lib, cuda, clumps, per_clump):
    """Clumps of side 1e-8 in a unit box share their first 21 levels: runs of up to
    256 equal first key words are ordered in place, a longer run takes the full
    multi-word sort.  At theta = 0 (every leaf, no internal monopole) the forces and
    the number of cells match the reference tree tightly.  At theta > 0 the internal
    monopoles, summed in another order, differ from the reference's by ~1e-16 of the
    clump's distance from the origin, i.e. ~1e-8 of the clump's own size, and the
    forces inside a clump by as much: rms <= 1e-7, max <= 1e-6 there."""
    from gravhopper_gb300 import _capi, _jbgrav
    rng = np.random.default_rng(6)
    centres = rng.uniform(-1, 1, size=(clumps, 1, 3))
    pos = (centres + 1e-8 * rng.uniform(0, 1, size=(clumps, per_clump, 3))).reshape(-1, 3)
    pos = np.concatenate([pos, rng.uniform(-1, 1, size=(200, 3))])
    m = rng.uniform(1, 2, size=len(pos))
    ref, ncells = oracle.tree_force(pos, m, 1e-10, 0.0, return_nodes=True)
    _capi.tree_stats_read()
    _capi.tree_stats(True)
    try:
        got = _jbgrav.tree_force(pos, m, 1e-10, 0.0)
        c = _capi.tree_stats_read()
    finally:
        _capi.tree_stats(False)
    check(got, ref)
    assert c["target_visits"] == len(pos) * ncells
    for theta in (0.5, 0.7):
        check(_jbgrav.tree_force(pos, m, 1e-10, theta), oracle.tree_force(pos, m, 1e-10, theta),
              rms_tol=1e-7, max_tol=1e-6)


def test_tree_lattice_on_cell_centres(lib, cuda):
    """A lattice puts particles exactly on cell centres and faces, where the octant
    test's ties go low (_jbgrav.c:441-450) and the keys take the FP64 recurrence."""
    from gravhopper_gb300 import _capi, _jbgrav
    g = np.arange(12) / 8.0
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    m = np.ones(len(pos))
    ref, ncells = oracle.tree_force(pos, m, 0.01, 0.0, return_nodes=True)
    _capi.tree_stats_read()
    _capi.tree_stats(True)
    try:
        got = _jbgrav.tree_force(pos, m, 0.01, 0.0)
        c = _capi.tree_stats_read()
    finally:
        _capi.tree_stats(False)
    check(got, ref)
    assert c["target_visits"] == len(pos) * ncells
    for theta in (0.5, 0.7):
        check(_jbgrav.tree_force(pos, m, 0.01, theta), oracle.tree_force(pos, m, 0.01, theta))


def test_tree_coincident_particles_error(lib, cuda):
    from gravhopper_gb300 import _capi, _jbgrav
    pos = np.array([[0.0, 0.0, 0.0], [1.0, 2.0, 3.0], [1.0, 2.0, 3.0]])
    with pytest.raises(_capi.EngineError) as e:
        _jbgrav.tree_force(pos, np.ones(3), 0.01, 0.7)
    assert e.value.code == _capi.GH_ERR_DEPTH
    # the library stays usable afterwards
    ok = _jbgrav.tree_force(pos[:2], np.ones(2), 0.01, 0.7)
    assert np.isfinite(ok).all()


def test_tree_empty_sources_and_targets(lib, cuda):
    from gravhopper_gb300 import _jbgrav
    assert _jbgrav.tree_force(np.zeros((0, 3)), np.zeros(0), 0.1, 0.7).shape == (0, 3)
    out = _jbgrav.tree_force_position(np.zeros((0, 3)), np.zeros(0), np.ones((3, 3)), 0.1, 0.7)
    np.testing.assert_array_equal(out, np.zeros((3, 3)))
    out = _jbgrav.tree_force_position(np.ones((4, 3)) * np.arange(4)[:, None], np.ones(4), np.zeros((0, 3)),
                                      0.1, 0.7)
    assert out.shape == (0, 3)


def test_tree_run_matches_reference_trajectory(golden, lib, cuda):
    import torch

    from gravhopper_gb300 import engine
    x = torch.from_numpy(golden["plummer_pos"].copy()).to(cuda)
    v = torch.from_numpy(golden["plummer_vel"].copy()).to(cuda)
    m = torch.from_numpy(golden["plummer_mass"].copy()).to(cuda)
    engine.run_dkd(x, v, m, 20, 0.005, 5e-5, algorithm="tree", theta=0.7)
    np.testing.assert_allclose(x.cpu().numpy(), golden["traj_tree_x_20"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(v.cpu().numpy(), golden["traj_tree_v_20"], rtol=1e-9, atol=1e-9)


MIXED_TREE_RMS_TOL = 1e-6
MIXED_TREE_MAX_TOL = 1e-3


@pytest.mark.parametrize("theta", [0.5, 0.7])
def test_mixed_tree_against_reference_golden(golden, lib, cuda, theta):
    """Mixed walk: same opening decisions, FP32 interactions with compensated sums."""
    import torch

    from gravhopper_gb300 import engine
    key = str(theta).replace(".", "p")
    for pos, mass, eps, ref in ((golden["tree_pos"], golden["tree_mass"], 5e-5, golden[f"tree_{key}_out"]),
                                (golden["hq_pos"], golden["hq_mass"], 0.1, golden[f"hq_{key}_out"])):
        x = torch.from_numpy(pos).to(cuda)
        m = torch.from_numpy(mass).to(cuda)
        got = engine.tree_force(x, m, eps, theta, precision="mixed").cpu().numpy()
        check(got, ref, MIXED_TREE_RMS_TOL, MIXED_TREE_MAX_TOL)


@pytest.mark.parametrize("theta", [0.5, 0.7])
def test_mixed_tree_zero_softening_and_targets(golden, lib, cuda, theta):
    """Mixed walk with eps = 0 (a target on a particle gets no term from it, as the
    reference's r^2 + eps^2 == 0 rule) at target points."""
    import torch

    from gravhopper_gb300 import engine
    key = str(theta).replace(".", "p")
    x = torch.from_numpy(golden["tree_pos"]).to(cuda)
    m = torch.from_numpy(golden["tree_mass"]).to(cuda)
    fp = torch.from_numpy(golden["tree_fpos"]).to(cuda)
    got = engine.tree_force(x, m, 0.0, theta, force_pos=fp, precision="mixed").cpu().numpy()
    assert np.isfinite(got).all()
    check(got, golden[f"treepos_{key}_out"], MIXED_TREE_RMS_TOL, MIXED_TREE_MAX_TOL)


def test_mixed_tree_large_against_oracle(lib, cuda):
    import torch

    from gravhopper_gb300 import engine, ics
    ic = ics.hernquist_disk(200000, seed=9)
    x = torch.from_numpy(ic["pos"]).to(cuda)
    m = torch.from_numpy(ic["mass"]).to(cuda)
    idx = np.random.default_rng(0).choice(200000, size=3000, replace=False)
    got = engine.tree_force(x, m, 0.1, 0.7, precision="mixed").cpu().numpy()[idx]
    ref = oracle.tree_force_position(ic["pos"], ic["mass"], ic["pos"][idx], 0.1, 0.7)
    check(got, ref, MIXED_TREE_RMS_TOL, MIXED_TREE_MAX_TOL)


def test_mixed_tree_run_tracks_reference(golden, lib, cuda):
    import torch

    from gravhopper_gb300 import engine
    x = torch.from_numpy(golden["plummer_pos"].copy()).to(cuda)
    v = torch.from_numpy(golden["plummer_vel"].copy()).to(cuda)
    m = torch.from_numpy(golden["plummer_mass"].copy()).to(cuda)
    engine.run_dkd(x, v, m, 20, 0.005, 5e-5, algorithm="tree", precision="mixed", theta=0.7)
    # close pairs amplify FP32 force errors over 20 steps (2 of 6000 coordinates > 1e-9 kpc)
    np.testing.assert_allclose(x.cpu().numpy(), golden["traj_tree_x_20"], rtol=0, atol=1e-8)


def test_simulation_default_tree(golden, lib, cuda):
    import gravhopper_gb300 as gh
    sim = gh.Simulation(dt=0.005, eps=5e-5)  # algorithm='tree' by default, theta 0.7
    sim.add_IC({"pos": golden["plummer_pos"], "vel": golden["plummer_vel"], "mass": golden["plummer_mass"]})
    sim.run(20)
    np.testing.assert_allclose(sim.positions[20], golden["traj_tree_x_20"], rtol=0, atol=1e-12)


def test_tree_walk_counters(lib, cuda):
    """theta = 0 opens every internal cell, so each target visits every cell once and
    interacts with every leaf (one per particle); each warp steps through all cells."""
    from gravhopper_gb300 import _capi, _jbgrav, ics
    n = 5000
    ic = ics.plummer(n, seed=8)
    _capi.tree_stats_read()
    _capi.tree_stats(True)
    try:
        _jbgrav.tree_force(ic["pos"], ic["mass"], 5e-5, 0.0)
        c0 = _capi.tree_stats_read()
        _jbgrav.tree_force(ic["pos"], ic["mass"], 5e-5, 0.7)
        c7 = _capi.tree_stats_read()
    finally:
        _capi.tree_stats(False)
    assert c0["walks"] == 1 and c0["interactions"] == n * n
    _, ncells = oracle.tree_force(ic["pos"], ic["mass"], 5e-5, 0.0, return_nodes=True)
    assert c0["target_visits"] == n * ncells
    assert c0["cell_steps"] == (n + 31) // 32 * ncells
    assert c7["walks"] == 1
    assert 0 < c7["interactions"] < c7["target_visits"] < c0["target_visits"]
    assert c7["cell_steps"] * 32 >= c7["target_visits"] and c7["exact_tests"] <= c7["target_visits"]
    assert _capi.tree_stats_read()["walks"] == 0


@pytest.mark.parametrize("eps", [0.1, 0.0])
@pytest.mark.parametrize("precision,rms_tol,max_tol", [("fp64", TREE_RMS_TOL, TREE_MAX_TOL),
                                                        ("mixed", MIXED_TREE_RMS_TOL, MIXED_TREE_MAX_TOL)])
def test_tree_many_target_points_any_order(lib, cuda, precision, rms_tol, max_tol, eps):
    """From 8192 target points on, the walk takes the targets in octant-key order (a
    radix sort of their keys in the sources' root cell; points outside it clamped to
    its faces) and writes each force to the target's own slot.  20,000 targets in
    random order, some outside the sources' box and some on particles, against the
    reference tree's target-point form (gravhopper/_jbgrav.c:634-727), with softening
    and with eps = 0 (a point on a particle gets no term from it)."""
    import torch

    from gravhopper_gb300 import engine, ics
    ic = ics.hernquist_disk(30000, seed=15)
    rng = np.random.default_rng(16)
    fp = np.concatenate([rng.normal(size=(17000, 3)) * 3.0, rng.uniform(-300, 300, size=(2000, 3)),
                         ic["pos"][rng.choice(30000, 1000, replace=False)]])
    fp = fp[rng.permutation(len(fp))]
    x = torch.from_numpy(ic["pos"]).to(cuda)
    m = torch.from_numpy(ic["mass"]).to(cuda)
    got = engine.tree_force(x, m, eps, 0.7, force_pos=torch.from_numpy(fp).to(cuda),
                            precision=precision).cpu().numpy()
    assert np.isfinite(got).all()
    check(got, oracle.tree_force_position(ic["pos"], ic["mass"], fp, eps, 0.7), rms_tol, max_tol)


def _validate(pos, m, eps):
    import torch

    from gravhopper_gb300 import _capi
    d = torch.device("cuda:0")
    return _capi.tree_validate(torch.as_tensor(np.ascontiguousarray(pos), dtype=torch.float64, device=d),
                               torch.as_tensor(np.ascontiguousarray(m), dtype=torch.float64, device=d), eps)


def _tree_cases():
    from gravhopper_gb300 import ics
    rng = np.random.default_rng(21)
    g = np.arange(12) / 8.0
    lattice = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    base = rng.uniform(-1, 1, size=(50, 3))
    deep = np.concatenate([base, base + 1e-13 * rng.normal(size=base.shape)])
    clumps = (rng.uniform(-1, 1, size=(30, 1, 3)) + 1e-8 * rng.uniform(0, 1, size=(30, 100, 3))).reshape(-1, 3)
    pl = ics.plummer(5000, seed=8)
    return {"one": (np.array([[0.5, -1.0, 2.0]]), np.array([3.0])),
            "two": (np.array([[0.0, 0.0, 0.0], [1.0, 2.0, 3.0]]), np.array([1.0, 2.0])),
            "lattice": (lattice, np.ones(len(lattice))),
            "deep": (deep, rng.uniform(1, 2, size=len(deep))),
            "clumps": (clumps, rng.uniform(1, 2, size=len(clumps))),
            "plummer": (pl["pos"], pl["mass"])}


@pytest.mark.parametrize("case", ["one", "two", "lattice", "deep", "clumps", "plummer"])
def test_tree_invariants_match_reference_cell_count(lib, cuda, case):
    """gh_tree_validate on trees the reference builds too: one leaf per particle, skip
    indices that tile every cell's subtree with at most 8 children, cell masses equal
    to their children's sums, every child's centre of mass inside its cell, walk
    records equal to the FP64 cells, and as many cells as the reference's tree, which
    inserts one particle at a time (gravoct_add_particle, _jbgrav.c:387-439)."""
    pos, m = _tree_cases()[case]
    v = _validate(pos, m, 1e-3)
    _, ncells = oracle.tree_force(pos, m, 1e-3, 0.0, return_nodes=True)
    assert v["leaves"] == len(m) and v["cells"] == ncells, v
    assert all(v[k] == 0 for k in v if k not in ("cells", "leaves")), v


def test_tree_invariants_large(lib, cuda):
    """The same invariants at 1M particles of a Hernquist disk (the tree-force bench
    workload) and with target points sorted into the build."""
    from gravhopper_gb300 import ics
    ic = ics.hernquist_disk(1 << 20, seed=1)
    v = _validate(ic["pos"], ic["mass"], 5e-5)
    assert v["leaves"] == 1 << 20 and v["cells"] > 1 << 20, v
    assert all(v[k] == 0 for k in v if k not in ("cells", "leaves")), v
