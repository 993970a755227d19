"""The oracle is pinned to the reference: bit-exact against the golden vectors made by
the compiled reference extension, and against that extension directly where it exists."""
import numpy as np
import pytest

from oracle import oracle


def test_direct_matches_golden(golden):
    keys = sorted(k[:-4] for k in golden if k.startswith("direct_") and k.endswith("_out"))
    assert len(keys) >= 8
    for k in keys:
        pos, mass, eps = golden[k + "_pos"], golden[k + "_mass"], float(golden[k + "_eps"])
        np.testing.assert_array_equal(oracle.direct_summation(pos, mass, eps), golden[k + "_out"],
                                      err_msg=k)


def test_direct_position_matches_golden(golden):
    for tag in ("eps", "eps0"):
        k = f"dpos_{tag}"
        got = oracle.direct_summation_position(golden[k + "_pos"], golden[k + "_mass"],
                                               golden[k + "_fpos"], float(golden[k + "_eps"]))
        np.testing.assert_array_equal(got, golden[k + "_out"])


def test_plummer_force_matches_golden(golden):
    got = oracle.direct_summation(golden["plummer_pos"], golden["plummer_mass"], 5e-5)
    np.testing.assert_array_equal(got, golden["plummer_force"])


@pytest.mark.parametrize("theta", [0.0, 0.5, 0.7, 1.0])
def test_tree_matches_golden(golden, theta):
    key = str(theta).replace(".", "p")
    got = oracle.tree_force(golden["tree_pos"], golden["tree_mass"], 5e-5, theta)
    np.testing.assert_array_equal(got, golden[f"tree_{key}_out"])
    got = oracle.tree_force_position(golden["tree_pos"], golden["tree_mass"], golden["tree_fpos"], 0.0,
                                     theta)
    np.testing.assert_array_equal(got, golden[f"treepos_{key}_out"])


def test_tree_small_and_hernquist_match_golden(golden):
    for n in (1, 2, 3):
        k = f"tree_small_{n}"
        got = oracle.tree_force(golden[k + "_pos"], golden[k + "_mass"], 0.01, 0.7)
        np.testing.assert_array_equal(got, golden[k + "_out"])
    for th in (0.5, 0.7):
        key = str(th).replace(".", "p")
        got = oracle.tree_force(golden["hq_pos"], golden["hq_mass"], 0.1, th)
        np.testing.assert_array_equal(got, golden[f"hq_{key}_out"])


def test_dkd_trajectory_matches_golden(golden):
    x, v, snaps = oracle.dkd_run(golden["plummer_pos"], golden["plummer_vel"], golden["plummer_mass"],
                                 0.005, 5e-5, 100, snap_every=100)
    np.testing.assert_array_equal(x, golden["traj_direct_x_100"])
    np.testing.assert_array_equal(v, golden["traj_direct_v_100"])


def test_tree_trajectory_matches_golden(golden):
    x, v = oracle.dkd_run(golden["plummer_pos"], golden["plummer_vel"], golden["plummer_mass"], 0.005,
                          5e-5, 20, force=lambda p, m, e: oracle.tree_force(p, m, e, 0.7))
    np.testing.assert_array_equal(x, golden["traj_tree_x_20"])
    np.testing.assert_array_equal(v, golden["traj_tree_v_20"])


def test_thread_count_does_not_change_results():
    rng = np.random.default_rng(3)
    pos = rng.normal(size=(301, 3))
    m = rng.uniform(1, 2, size=301)
    a1 = oracle.direct_summation(pos, m, 0.01, nthreads=1)
    a7 = oracle.direct_summation(pos, m, 0.01, nthreads=7)
    np.testing.assert_array_equal(a1, a7)
    t1 = oracle.tree_force(pos, m, 0.01, 0.6, nthreads=1)
    t5 = oracle.tree_force(pos, m, 0.01, 0.6, nthreads=5)
    np.testing.assert_array_equal(t1, t5)


def test_duplicate_particles_give_depth_error():
    pos = np.array([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0], [1.0, 1.0, 1.0]])
    with pytest.raises(RuntimeError, match="depth"):
        oracle.tree_force(pos, np.ones(3), 0.01, 0.7)


def test_oracle_against_compiled_reference():
    ref = oracle.reference_module()
    if ref is None:
        pytest.skip("reference extension not built here (make -C oracle ref)")
    rng = np.random.default_rng(17)
    for n in (5, 129, 700):
        pos = rng.standard_cauchy(size=(n, 3))
        m = rng.uniform(0.1, 3.0, size=n)
        fp = np.concatenate([pos[:3], rng.normal(size=(20, 3))])
        np.testing.assert_array_equal(oracle.direct_summation(pos, m, 0.02), ref.direct_summation(pos, m, 0.02))
        np.testing.assert_array_equal(oracle.direct_summation_position(pos, m, fp, 0.0),
                                      ref.direct_summation_position(pos, m, fp, 0.0))
        for th in (0.3, 0.7):
            np.testing.assert_array_equal(oracle.tree_force(pos, m, 0.02, th), ref.tree_force(pos, m, 0.02, th))
            np.testing.assert_array_equal(oracle.tree_force_position(pos, m, fp, 0.0, th),
                                          ref.tree_force_position(pos, m, fp, 0.0, th))
