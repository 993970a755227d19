"""Host-side logic that needs no GPU: argument checks and errors of the reference
interface, parameter validation, IC handling, and the stream-K work partition."""
import numpy as np
import pytest

import gravhopper_gb300 as gh
from gravhopper_gb300 import _jbgrav, ics


@pytest.mark.parametrize("fn,args,msg", [
    (_jbgrav.direct_summation, (np.zeros(3), np.ones(1), 0.1), "Position array does not have 2 dimensions."),
    (_jbgrav.direct_summation, (np.zeros((4, 2)), np.ones(4), 0.1), "Position array is not Nx3."),
    (_jbgrav.direct_summation, (np.zeros((4, 3)), np.ones(5), 0.1),
     "Mass array and position array contain different numbers of particles."),
    (_jbgrav.tree_force, (np.zeros((4, 3)), np.ones(3), 0.1, 0.7),
     "Mass array and position array contain different numbers of particles."),
    (_jbgrav.direct_summation_position, (np.zeros((4, 3, 1)), np.ones(4), np.zeros((2, 3)), 0.1),
     "Particle position array does not have 2 dimensions."),
    (_jbgrav.direct_summation_position, (np.zeros((4, 3)), np.ones(3), np.zeros((2, 3)), 0.1),
     "Mass array and particle position array contain different numbers of particles."),
    (_jbgrav.direct_summation_position, (np.zeros((4, 3)), np.ones(4), np.zeros(3), 0.1),
     "Force position array does not have 2 dimensions."),
    (_jbgrav.tree_force_position, (np.zeros((4, 3)), np.ones(4), np.zeros((2, 4)), 0.1, 0.7),
     "Force position array is not Nx3."),
])
def test_reference_error_messages(fn, args, msg):
    # _jbgrav.c:88-108, 223-262, 584-604, 657-696: RuntimeError with these exact texts.
    with pytest.raises(RuntimeError) as e:
        fn(*args)
    assert str(e.value) == msg


def test_simulation_parameter_validation():
    sim = gh.Simulation(dt=0.005, eps=5e-5, algorithm="direct")
    assert sim.get_algorithm() == "direct" and sim.get_theta() == 0.7
    with pytest.raises(ValueError):
        sim.set_algorithm("fmm")
    with pytest.raises(ValueError):
        sim.set_precision("fp16")
    with pytest.raises(gh.UninitializedSimulationException):
        sim.run(1)


def test_add_ic_checks_and_stacking():
    sim = gh.Simulation(dt=0.01, eps=0.01)
    with pytest.raises(gh.ICException):
        sim.add_IC({"pos": np.zeros((2, 3)), "vel": np.zeros((2, 3))})
    with pytest.raises(gh.ICException):
        sim.add_IC({"pos": np.zeros((2, 3)), "vel": np.zeros((3, 3)), "mass": np.ones(2)})
    sim.add_IC({"pos": np.zeros((2, 3)), "vel": np.zeros((2, 3)), "mass": np.ones(2)})
    sim.add_IC({"pos": np.ones((3, 3)), "vel": np.zeros((3, 3)), "mass": np.ones(3)})
    assert sim.ICarrays["pos"].shape == (5, 3) and sim.ICarrays["mass"].shape == (5,)
    sim.init_run(4)
    assert sim.positions.shape == (5, 5, 3) and sim.times.shape == (5,)


def test_plummer_generator_is_seeded_and_centred():
    a = ics.plummer(4096, seed=3)
    b = ics.plummer(4096, seed=3)
    np.testing.assert_array_equal(a["pos"], b["pos"])
    np.testing.assert_allclose(a["pos"].mean(0), 0.0, atol=1e-15)
    np.testing.assert_allclose(a["vel"].mean(0), 0.0, atol=1e-10)
    r = np.linalg.norm(a["pos"], axis=1)
    # Plummer half-mass radius ~1.305 b
    assert 1.15e-3 < np.median(r) < 1.45e-3
    assert np.isclose(a["mass"].sum(), 1e6)


def test_ic_class_plummer_and_hernquist_disk():
    p = gh.IC.Plummer(N=1000, b=1e-3, totmass=1e6, seed=1)
    assert p["pos"].shape == (1000, 3)
    h = ics.hernquist_disk(10000, seed=2)
    assert np.isfinite(h["vel"]).all() and np.isclose(h["mass"].sum(), 1e11)
    # large-r series of the Jeans dispersion joins the closed form smoothly
    s = ics.hernquist_sigma2(np.array([49.99999, 50.00001]), 1.0, 1e10)
    assert abs(s[0] / s[1] - 1) < 1e-6


def _sk(n_tiles, chunks, grid):
    units = n_tiles * chunks
    grid = min(grid, units)
    start = lambda g: (g * units) // grid
    owner = lambda u: ((u + 1) * grid + units - 1) // units - 1
    return units, grid, start, owner


@pytest.mark.parametrize("n_tiles,chunks,grid", [(1, 8, 304), (8, 8, 304), (1024, 4096, 304),
                                                  (3, 5, 7), (977, 13, 456), (2, 1, 456)])
def test_streamk_partition(n_tiles, chunks, grid):
    # Python restatement of sk_start / sk_owner in csrc/direct.cuh.
    units, grid, start, owner = _sk(n_tiles, chunks, grid)
    assert start(0) == 0 and start(grid) == units
    for g in range(grid):
        assert start(g) <= start(g + 1)
    for u in list(range(min(units, 5000))) + [units - 1]:
        g = owner(u)
        assert start(g) <= u < start(g + 1)
    # each tile's contributors are contiguous and use slot 0 only for their first tile
    for t in range(min(n_tiles, 200)):
        gf, gl = owner(t * chunks), owner(t * chunks + chunks - 1)
        for g in range(gf, gl + 1):
            first_tile = start(g) // chunks
            last_tile = (start(g + 1) - 1) // chunks
            assert first_tile <= t <= last_tile
