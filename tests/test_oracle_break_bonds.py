"""The oracle's topology graphs and BreakBonds against the reference's known answers
(readdy/test/TestBreakingBonds.cpp) and against its own explicit bonded terms."""
import numpy as np
import pytest

import oracle
from tests.golden import known_answers as ka


def break_bonds_oracle(case, seed=1):
    s = oracle.OracleSystem([10.0, 10.0, 10.0], (True, True, True), 1.0, (1.0, 1.0, 1.0), seed=seed)
    for t in range(3):
        s.set_particle_flavor(t, 1)  # TOPOLOGY
    for a, b in case["bonds"]:
        s.configure_harmonic_bond(a, b, 1.0, 1.0)
    for top in case["topologies"]:
        s.add_topology(np.asarray(top["positions"], float), np.asarray(top["types"], np.int32), top["edges"])
    return s


@pytest.mark.parametrize("case", ka.BREAK_BONDS_CASES, ids=lambda c: c["name"])
def test_oracle_break_bonds_known_answers(case):
    s = break_bonds_oracle(case)
    pos0, t0, ids0, _, _ = s.particles()
    for rnd in case["rounds"]:
        s.break_bonds(1.0, rnd)
    tops = s.topologies()
    assert sorted(len(ids) for _, ids in tops) == case["after"]
    assert all(tt == 0 for tt, _ in tops)  # the pieces keep the topology type
    pos, t, ids, _, _ = s.particles()
    np.testing.assert_array_equal(ids, ids0)
    np.testing.assert_array_equal(pos, pos0)  # particles stay where they are
    if "partners" in case:
        two = [ids for _, ids in tops if len(ids) == 2][0]
        types = {int(i): int(tt) for i, tt in zip(ids, t)}
        assert sorted(types[int(i)] for i in two) == sorted(case["partners"])


def test_oracle_one_particle_pieces_of_normal_flavor_leave_the_topologies():
    """include/readdy/model/actions/Utils.h:59-79: a piece that is a single particle of NORMAL flavor is
    no topology any more; a TOPOLOGY-flavored one stays a one-particle topology."""
    case = ka.BREAK_BONDS_CASES[2]  # trimer A-A-B, the A-B bond breaks
    s = break_bonds_oracle(case)
    s.set_particle_flavor(1, 0)  # B: NORMAL
    s.break_bonds(1.0, case["rounds"][0])
    assert sorted(len(ids) for _, ids in s.topologies()) == [2]
    assert s.n_particles == 3


def chain_system(chains, seed=0):
    L = 30.0
    s = oracle.OracleSystem([L, L, L], (True, True, True), 1.0, (1.0,), seed=seed)
    return s


def test_oracle_configured_terms_equal_explicit_terms():
    """GraphTopology::configure over chain graphs gives the chain's bonds, angles and dihedrals: forces
    equal those of the same terms given explicitly."""
    rng = np.random.default_rng(3)
    n_chains, n = 20, 12
    steps = rng.normal(size=(n_chains, n, 3))
    steps /= np.linalg.norm(steps, axis=2, keepdims=True)
    pos = (np.cumsum(steps, axis=1) + rng.uniform(-10, 10, (n_chains, 1, 3))).reshape(-1, 3)
    pos = (pos + 15.0) % 30.0 - 15.0
    a = chain_system(None)
    b = chain_system(None)
    for s in (a, b):
        s.configure_harmonic_bond(0, 0, 50.0, 1.0)
        s.configure_harmonic_angle(0, 0, 0, 5.0, 2.5)
        s.configure_cosine_dihedral(0, 0, 0, 0, 1.0, 3.0, 0.3)
    for c in range(n_chains):
        a.add_topology(pos[c * n:(c + 1) * n], np.zeros(n, np.int32), [(i, i + 1) for i in range(n - 1)])
    b.add_particles(pos, np.zeros(len(pos), np.int32))
    idx = np.arange(len(pos)).reshape(n_chains, n)
    b.add_harmonic_bonds(np.stack([idx[:, :-1].ravel(), idx[:, 1:].ravel()], 1), 50.0, 1.0)
    b.add_harmonic_angles(np.stack([idx[:, :-2].ravel(), idx[:, 1:-1].ravel(), idx[:, 2:].ravel()], 1), 5.0, 2.5)
    b.add_cosine_dihedrals(np.stack([idx[:, :-3].ravel(), idx[:, 1:-2].ravel(), idx[:, 2:-1].ravel(),
                                     idx[:, 3:].ravel()], 1), 1.0, 3.0, 0.3)
    ea, eb = a.calculate_forces(), b.calculate_forces()
    fa, fb = a.particles()[3], b.particles()[3]
    np.testing.assert_allclose(ea, eb, rtol=1e-12)
    np.testing.assert_allclose(fa, fb, rtol=1e-10, atol=1e-10)


def test_oracle_break_rate_matches_the_coin_probability():
    """Dimers stretched above the threshold break with probability 1 - exp(-rate dt), the others never."""
    n = 4000
    rng = np.random.default_rng(5)
    s = oracle.OracleSystem([200.0, 200.0, 200.0], (True, True, True), 1.0, (1.0,), seed=11)
    s.set_particle_flavor(0, 1)
    s.configure_harmonic_bond(0, 0, 1.0, 1.0)
    centers = rng.uniform(-90, 90, (n, 3))
    stretched = np.arange(n) % 2 == 0
    length = np.where(stretched, 2.0, 1.5)  # energies 1 and 0.25 against a threshold of 0.5
    for c, l in zip(centers, length):
        s.add_topology(np.array([c, c + (0, 0, l)]), np.zeros(2, np.int32), [(0, 1)])
    rate, dt = 0.5, 1.0
    nb = s.break_bonds(dt, [(0, 0, 0.5, rate)])
    p = 1 - np.exp(-rate * dt)
    m = stretched.sum()
    assert abs(nb - p * m) < 4 * np.sqrt(m * p * (1 - p))
    sizes = [len(ids) for _, ids in s.topologies()]
    assert sizes.count(1) == 2 * nb and sizes.count(2) == n - nb
