"""Pins the FP64 CPU oracle against the known-answer vectors of ReaDDy's own unit tests.

These run without a GPU.  They establish that the oracle restates the reference before any CUDA
result is compared with it.
"""
import numpy as np
import pytest

import oracle
from tests.golden import known_answers as ka


def _oracle_from_case(case, seed=1, n_threads=1):
    n_types = max(len(case.get("diffusion", (1.0,))), max(case.get("types", [0])) + 1)
    diff = list(case.get("diffusion", (1.0,))) + [1.0] * (n_types - len(case.get("diffusion", (1.0,))))
    s = oracle.OracleSystem(case["box"], case["periodic"], 1.0, diff, seed=seed, n_threads=n_threads)
    for kind, t1, t2, p in case.get("potentials", []):
        if kind == "harmonic_repulsion":
            s.add_harmonic_repulsion(t1, t2, p["k"], p["d"])
        elif kind == "lennard_jones":
            s.add_lennard_jones(t1, t2, p["m"], p["n"], p["cutoff"], p["shift"], p["epsilon"], p["sigma"])
        elif kind == "screened_electrostatics":
            s.add_screened_electrostatics(t1, t2, p["C"], p["kappa"], p["D"], p["sigma"], p["exponent"],
                                          p["cutoff"])
        elif kind == "weak_interaction_piecewise_harmonic":
            s.add_weak_interaction_piecewise_harmonic(t1, t2, p["k"], p["desired"], p["depth"], p["cutoff"])
    return s


@pytest.mark.parametrize("case", ka.PAIR_CASES, ids=lambda c: c["name"])
def test_pair_potential_known_answers(case):
    s = _oracle_from_case(case)
    s.add_particles(np.array(case["positions"], float), np.array(case["types"]))
    s.nl_setup(s.calculate_max_cutoff())
    e1 = s.calculate_forces()
    e2 = s.calculate_forces()  # calculating twice must not accumulate (TestStateModel.cpp:80-81)
    assert e1 == e2
    rtol = case.get("energy_rtol", 1e-12)
    assert e1 == pytest.approx(case["energy"], rel=max(rtol, 1e-12))
    _, _, ids, f, _ = s.particles()
    exp = np.array(ka.per_particle_forces(case))
    order = np.argsort(ids)
    np.testing.assert_allclose(f[order], exp, rtol=0, atol=case["force_atol"] + 1e-12)


@pytest.mark.parametrize("case", ka.EXTERNAL_CASES, ids=lambda c: c["name"])
def test_external_potential_known_answers(case):
    n_types = max(case["types"]) + 1
    s = oracle.OracleSystem(case["box"], case["periodic"], 1.0, (1.0,) * n_types)
    for kind, t, args in case["potentials"]:
        getattr(s, "add_" + kind)(t, *args)
    s.add_particles(np.array(case["positions"], float), np.array(case["types"]))
    e = s.calculate_forces()
    assert e == pytest.approx(case["energy"], rel=1e-9)
    _, _, ids, f, _ = s.particles()
    np.testing.assert_allclose(f[np.argsort(ids)], np.array(case["forces"]), rtol=0, atol=case["force_atol"])


def test_spherical_barrier_rejects_a_width_above_its_radius():
    s = oracle.OracleSystem((10., 10., 10.), (1, 1, 1), 1.0, (1.0,))
    with pytest.raises(RuntimeError, match="radius larger than its width"):
        s.add_spherical_barrier(0, 1.0, 2.0, (0., 0., 0.), 1.0)


@pytest.mark.parametrize("case", ka.BONDED_CASES, ids=lambda c: c["name"])
def test_bonded_known_answers(case):
    s = oracle.OracleSystem(case["box"], case["periodic"], 1.0, (1.0,), seed=1)
    s.add_particles(np.array(case["positions"], float), 0)
    for idx, k, l0 in case["bonds"]:
        s.add_harmonic_bonds([idx], k, l0)
    for idx, k, th in case["angles"]:
        s.add_harmonic_angles([idx], k, th)
    for idx, k, mult, phi0 in case["dihedrals"]:
        s.add_cosine_dihedrals([idx], k, mult, phi0)
    e = s.calculate_forces()
    assert e == pytest.approx(case["energy"], rel=case["energy_rtol"], abs=1e-14)
    _, _, _, f, _ = s.particles()
    np.testing.assert_allclose(f, np.array(case["forces"], float), rtol=0, atol=case["force_atol"] + 1e-14)


def _oracle_reaction_case(case, seed):
    s = oracle.OracleSystem(case["box"], case["periodic"], 1.0, case["diffusion"], seed=seed)
    for kind, p in case["reactions"]:
        assert kind == "fusion"
        s.add_fusion(p["a"], p["b"], p["c"], p["rate"], p["educt_distance"])
    s.add_particles(np.array(case["positions"], float), np.array(case.get("types", [0] * len(case["positions"]))))
    return s


@pytest.mark.parametrize("handler", [oracle.UNCONTROLLED_APPROXIMATION, oracle.GILLESPIE])
@pytest.mark.parametrize("case", ka.REACTION_CASES, ids=lambda c: c["name"])
def test_reaction_known_answers(case, handler):
    for seed in range(5):
        s = _oracle_reaction_case(case, seed)
        s.nl_setup(s.calculate_max_cutoff())
        (s.gillespie if handler == oracle.GILLESPIE else s.uncontrolled_approximation)(1.0)
        pos, types, _, _, _ = s.particles()
        assert len(pos) == case["expect_n"]
        if "expect_positions" in case:
            np.testing.assert_allclose(pos, np.array(case["expect_positions"]), rtol=case["pos_rtol"])
        else:
            got = sorted((int(t), tuple(np.round(p, 6))) for t, p in zip(types, pos))
            exp = sorted((t, tuple(np.round(np.array(p, float), 6))) for t, p in case["expect_particles"])
            assert [g[0] for g in got] == [e[0] for e in exp]
            np.testing.assert_allclose(np.array([g[1] for g in got]), np.array([e[1] for e in exp]),
                                       atol=case["pos_atol"])


@pytest.mark.parametrize("handler", [oracle.UNCONTROLLED_APPROXIMATION, oracle.GILLESPIE])
def test_fission_near_boundary(handler):
    """readdy/test/TestReactions.cpp:191-213: products straddle the periodic boundary."""
    for seed in range(10):
        s = oracle.OracleSystem((10., 10., 10.), (True,) * 3, 1.0, (0.,), seed=seed)
        s.add_fission(0, 0, 0, 1e16, 2.0)
        s.add_particles([(-4.9999999, 0, 0)], 0)
        s.nl_setup(1.0)
        (s.gillespie if handler == oracle.GILLESPIE else s.uncontrolled_approximation)(1.0)
        pos, _, _, _, _ = s.particles()
        assert len(pos) == 2
        assert (pos[0, 0] <= 0) != (pos[1, 0] <= 0)
        assert np.all(pos >= -5.0) and np.all(pos < 5.0)


@pytest.mark.parametrize("box,pbc", [((10, 10, 10), (1, 1, 1)), ((10, 10, 10), (0, 0, 0)),
                                     ((5, 12, 7), (1, 0, 1)), ((3.3, 3.3, 3.3), (1, 1, 1)),
                                     ((2.5, 8, 2.5), (1, 1, 0)), ((20, 4, 4), (1, 1, 1)),
                                     ((6, 6, 30), (0, 1, 1))])
@pytest.mark.parametrize("radius", [1, 2])
def test_cell_list_pairs_match_brute_force(box, pbc, radius):
    """kernels/cpu/test/TestNeighborList.cpp:267-362: cell-list pair set == brute-force pair set."""
    rng = np.random.default_rng(7)
    s = oracle.OracleSystem(box, pbc, 1.0, (1.0, 1.0), seed=3, cll_radius=radius)
    s.add_harmonic_repulsion(0, 1, 1.0, 1.2)
    s.add_harmonic_repulsion(0, 0, 1.0, 0.9)
    n = 400
    pos = (rng.random((n, 3)) - 0.5) * np.array(box, float)
    s.add_particles(pos, rng.integers(0, 2, n))
    s.nl_setup(s.calculate_max_cutoff())
    for step in range(3):
        a = s.nl_pairs(1.2)
        b = s.brute_force_pairs(1.2)
        assert len(a) > 0
        np.testing.assert_array_equal(a, b)
        s.euler_bd(0.01)
        s.nl_update()


def test_multithreaded_forces_match_serial():
    rng = np.random.default_rng(11)
    pos = (rng.random((3000, 3)) - 0.5) * 15.0
    types = rng.integers(0, 3, 3000)
    out = []
    for nt in (1, 4):
        s = oracle.OracleSystem((15., 15., 15.), (1, 1, 1), 1.0, (1., .5, .2), seed=1, n_threads=nt)
        s.add_lennard_jones(0, 0, 12, 6, 2.5, True, 1.0, 1.0)
        s.add_weak_interaction_piecewise_harmonic(1, 1, 10.0, 1.0, 0.5, 1.5)
        s.add_harmonic_repulsion(0, 1, 10.0, 1.0)
        s.add_harmonic_repulsion(0, 2, 10.0, 1.0)
        s.add_harmonic_repulsion(1, 2, 10.0, 1.0)
        s.add_harmonic_repulsion(2, 2, 10.0, 1.0)
        s.add_particles(pos, types)
        s.nl_setup(s.calculate_max_cutoff())
        e = s.calculate_forces()
        out.append((e, s.particles()[3]))
    assert out[0][0] == pytest.approx(out[1][0], rel=1e-12)
    np.testing.assert_allclose(out[0][1], out[1][1], rtol=1e-12, atol=1e-12)


def test_brownian_msd_matches_6Dt():
    """Free diffusion: <|dx|^2> = 6 D t, 60k samples give a 3-sigma band of 1 %."""
    rng = np.random.default_rng(5)
    n, steps, dt, D = 20000, 30, 1e-3, 1.0
    s = oracle.OracleSystem((1000., 1000., 1000.), (1, 1, 1), 1.0, (D,), seed=9, n_threads=2)
    p0 = (rng.random((n, 3)) - 0.5) * 100.0
    s.add_particles(p0, 0)
    for _ in range(steps):
        s.euler_bd(dt)
    p1 = s.particles()[0]
    msd = np.mean(np.sum((p1 - p0) ** 2, axis=1))
    assert abs(msd / (6 * D * dt * steps) - 1) < 0.01


@pytest.mark.slow
@pytest.mark.parametrize("handler", [oracle.UNCONTROLLED_APPROXIMATION, oracle.GILLESPIE])
def test_michaelis_menten_time_averaged_substrate(handler):
    """readdy/test/IntegrationTests.cpp:30-106: the substrate count averaged over 37501 observations
    lies within 3 % of 665.2 for both reaction handlers."""
    mm = ka.MICHAELIS_MENTEN
    rng = np.random.default_rng(2024)
    L = mm["box"][0]
    n = mm["n_e"] + mm["n_s"]
    pos = (rng.random((n, 3)) - 0.5) * L
    types = np.array([0] * mm["n_e"] + [1] * mm["n_s"])
    o = oracle.OracleSystem(mm["box"], mm["periodic"], 1.0, mm["diffusion"], seed=7, n_threads=4)
    o.add_fusion(0, 1, 2, mm["k_fwd"], mm["educt_distance"])
    o.add_fission(2, 0, 1, mm["k_back"], mm["product_distance"])
    o.add_fission(2, 0, 3, mm["k_prod"], mm["product_distance"])
    o.add_particles(pos, types)
    c = o.run(mm["n_steps"], mm["dt"], handler=handler, count_stride=1)
    assert abs(c[:, 1].mean() - mm["mean_s"]) < mm["rel_band"] * mm["mean_s"]


def test_virial_of_one_pair():
    """HR k=1, d=2, particles 1.8 apart along z (the pair of TestStateModel.cpp:57-99): the force on the
    first is -0.2 z, x_01 = 1.8 z, so the virial outer(-x_01, f_0) has zz = 0.36 and nothing else."""
    s = oracle.OracleSystem((10., 10., 10.), (1, 1, 1), 1.0, (1.0,))
    s.set_record_virial(True)
    s.add_harmonic_repulsion(0, 0, 1.0, 2.0)
    s.add_particles(np.array([[0., 0., 0.], [0., 0., 1.8]]), np.array([0, 0]))
    s.nl_setup(2.0)
    s.calculate_forces()
    expect = np.zeros((3, 3))
    expect[2, 2] = 0.36
    np.testing.assert_allclose(s.virial(), expect, atol=1e-12)


def test_radial_distribution_of_one_pair():
    """The reference's radial-distribution scenario (readdy/tests/test_observables_io.py:201-239): A at
    (-2.5, 0, 0) and B at the origin in a periodic 10^3 box, bins of 0.01 up to 5, from A to B at density
    1/1000: one count, in the bin of 2.5, normalised by its shell volume."""
    s = oracle.OracleSystem((10., 10., 10.), (1, 1, 1), 2.0, (0.2, 0.2))
    s.add_harmonic_repulsion(0, 1, 10.0, 2.0)
    s.add_particles(np.array([[-2.5, 0., 0.], [0., 0., 0.]]), np.array([0, 1], np.int32))
    borders = np.arange(0, 5, .01)
    counts, dist = s.radial_distribution(borders, [0], [1], 1. / 1000.)
    k = np.searchsorted(borders, 2.5, side="right") - 1  # std::upper_bound - 1
    expected = np.zeros(len(borders) - 1)
    expected[k] = 1.0
    np.testing.assert_array_equal(counts, expected)
    shell = 4. / 3. * np.pi * (borders[k + 1] ** 3 - borders[k] ** 3)
    assert dist[k] == pytest.approx(1.0 / (shell * 1 * 1e-3), rel=1e-12)
    assert np.count_nonzero(dist) == 1
    # from B to A and from both to both count the reverse pair as well
    c2, _ = s.radial_distribution(borders, [0, 1], [0, 1], 1. / 1000.)
    assert c2[k] == 2.0 and c2.sum() == 2.0


def test_histogram_along_axis_counts_like_the_cpu_kernel():
    """HistogramAlongAxis of the CPU kernel (CPUObservables.cpp:85-146): a coordinate equal to a border
    counts into the bin above it (upper_bound), only listed types count, and the last bin is never filled."""
    s = oracle.OracleSystem((10., 10., 10.), (1, 1, 1), 1.0, (1.0, 1.0))
    xs = [-4.0, -3.5, -3.0, -1.0, 0.0, 0.5, 3.9, 4.5, 2.0]
    ts = [0, 0, 0, 0, 0, 0, 0, 0, 1]
    s.add_particles(np.array([[x, 0., 0.] for x in xs]), np.array(ts, np.int32))
    borders = np.array([-4.0, -3.0, 0.0, 1.0, 4.0, 5.0])
    h = s.histogram_along_axis(borders, [0], 0)
    # bins [-4,-3): -4, -3.5; [-3,0): -3, -1; [0,1): 0, 0.5; [1,4): 3.9; [4,5): 4.5 -> never counted
    np.testing.assert_array_equal(h, [2., 2., 2., 1., 0.])
    np.testing.assert_array_equal(s.histogram_along_axis(borders, [1], 0), [0., 0., 0., 1., 0.])
