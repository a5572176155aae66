"""BreakBonds on the device (rdc_break_bonds) against the reference's known answers
(readdy/test/TestBreakingBonds.cpp), the coin probability, and the oracle's restatement: which
topologies remain, their edges, and the bonded forces of the terms derived again from them."""
import numpy as np
import pytest

import oracle
from tests.golden import known_answers as ka
from tests.helpers import f32

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rg():
    import readdy_gb300
    readdy_gb300.load()
    return readdy_gb300


def known_answer_kernel(rg, case, normal_types=()):
    ctx = rg.Context((10.0, 10.0, 10.0), (True, True, True), 1.0, (1.0, 1.0, 1.0))
    for t in range(3):
        ctx.set_particle_flavor(t, ctx.NORMAL if t in normal_types else ctx.TOPOLOGY)
    for a, b in case["bonds"]:
        ctx.configure_harmonic_bond(a, b, 1.0, 1.0)
    k = rg.CUDAKernel(ctx, seed=3)
    for top in case["topologies"]:
        k.add_topology(np.asarray(top["positions"], float), np.asarray(top["types"], np.int32), top["edges"],
                       topology_type=2)
    return k


@pytest.mark.parametrize("with_neighbor_list", [False, True])
@pytest.mark.parametrize("case", ka.BREAK_BONDS_CASES, ids=lambda c: c["name"])
def test_break_bonds_known_answers(rg, case, with_neighbor_list):
    k = known_answer_kernel(rg, case)
    if with_neighbor_list:
        k.create_neighbor_list(1.0)
    pos0, t0, ids0 = k.get_particles()
    for rnd in case["rounds"]:
        k.break_bonds(1.0, rnd)
    tops = k.get_topologies()
    assert sorted(len(ids) for _, ids in tops) == case["after"]
    assert all(tt == 2 for tt, _ in tops)  # the pieces keep the topology type
    pos, t, ids = k.get_particles()
    o0, o = np.argsort(ids0), np.argsort(ids)
    np.testing.assert_array_equal(ids[o], ids0[o0])
    np.testing.assert_array_equal(pos[o], pos0[o0])  # the particles stay where they are
    if "partners" in case:
        two = [ids for _, ids in tops if len(ids) == 2][0]
        types = {int(i): int(tt) for i, tt in zip(ids, t)}
        assert sorted(types[int(i)] for i in two) == sorted(case["partners"])
    edges = k.get_topology_edges()
    assert sum(len(e) for e in edges) == sum(len(ids) for _, ids in tops) - len(tops)  # pieces stay trees


def test_break_bonds_one_particle_pieces_of_normal_flavor_leave(rg):
    case = ka.BREAK_BONDS_CASES[2]  # trimer A-A-B, the A-B bond breaks
    k = known_answer_kernel(rg, case, normal_types=(1,))
    assert k.break_bonds(1.0, case["rounds"][0]) == 1
    assert sorted(len(ids) for _, ids in k.get_topologies()) == [2]
    assert k.n_particles == 3


def test_break_bonds_rejects_bad_input(rg):
    k = known_answer_kernel(rg, ka.BREAK_BONDS_CASES[0])
    with pytest.raises(ValueError):
        k.break_bonds(1.0, [(0, 5, 0.5, 1.0)])
    with pytest.raises(ValueError):
        k.break_bonds(1.0, [(0, 0, 0.5, -1.0)])
    with pytest.raises(ValueError):
        k.break_bonds(0.0, [(0, 0, 0.5, 1.0)])
    assert sorted(len(ids) for _, ids in k.get_topologies()) == [2]


def test_break_rate_matches_the_coin_probability(rg):
    """20000 dimers, half of them stretched above the threshold: those break with probability
    1 - exp(-rate dt), the others never."""
    n = 20000
    rng = np.random.default_rng(8)
    ctx = rg.Context((400.0, 400.0, 400.0), (True, True, True), 1.0, (1.0,))
    ctx.set_particle_flavor(0, ctx.TOPOLOGY)
    ctx.configure_harmonic_bond(0, 0, 1.0, 1.0)
    k = rg.CUDAKernel(ctx, seed=21)
    centers = rng.uniform(-190, 190, (n, 3))
    stretched = np.arange(n) % 2 == 0
    length = np.where(stretched, 2.0, 1.5)  # energies 1 and 0.25 against a threshold of 0.5
    pos = np.stack([centers, centers + np.stack([np.zeros(n), np.zeros(n), length], 1)], 1).reshape(-1, 3)
    ids = []
    for d in range(n):
        ids.append(k.add_topology(pos[2 * d:2 * d + 2], np.zeros(2, np.int32), [(0, 1)]))
    rate, dt = 0.5, 1.0
    nb = k.break_bonds(dt, [(0, 0, 0.5, rate)])
    p = 1 - np.exp(-rate * dt)
    m = stretched.sum()
    assert abs(nb - p * m) < 4 * np.sqrt(m * p * (1 - p)), (nb, p * m)
    tops = k.get_topologies()
    sizes = [len(t) for _, t in tops]
    assert sizes.count(1) == 2 * nb and sizes.count(2) == n - nb
    # no relaxed dimer broke
    pieces = {frozenset(int(i) for i in t) for _, t in tops}
    for d in np.flatnonzero(~stretched):
        assert frozenset(int(i) for i in ids[d]) in pieces
    # a second call draws fresh coins: about p of the remaining stretched dimers break
    nb2 = k.break_bonds(dt, [(0, 0, 0.5, rate)])
    m2 = m - nb
    assert abs(nb2 - p * m2) < 4 * np.sqrt(m2 * p * (1 - p)), (nb2, p * m2)


def stretched_chains(n_chains, n, seed):
    """Random-walk chains whose steps are 1.0 or 1.8 long (bond energies 0 and 0.64 for k = 1, l0 = 1),
    held in FP32."""
    rng = np.random.default_rng(seed)
    steps = rng.normal(size=(n_chains, n, 3))
    steps /= np.linalg.norm(steps, axis=2, keepdims=True)
    steps *= np.where(rng.random((n_chains, n, 1)) < 0.15, 1.8, 1.0)
    steps[:, 0] = 0
    starts = rng.uniform(-60, 60, (n_chains, 1, 3))
    return f32(np.cumsum(steps, axis=1) + starts)


@pytest.mark.parametrize("with_neighbor_list", [False, True])
def test_break_bonds_matches_oracle_topologies_and_forces(rg, with_neighbor_list):
    """Chains with bonds, angles and dihedrals; every stretched bond breaks (certain coin).  The GPU
    and the oracle keep the same pieces with the same edges, and the bonded forces of the terms derived
    from the remaining graphs agree (1e-5 relative, floor 1e-5 of the largest force)."""
    n_chains, n = 120, 20
    chains = stretched_chains(n_chains, n, seed=4)
    box = (160.0, 160.0, 160.0)
    ctx = rg.Context(box, (True, True, True), 1.0, (1.0,))
    o = oracle.OracleSystem(list(box), (True, True, True), 1.0, (1.0,), seed=1)
    ctx.set_particle_flavor(0, ctx.TOPOLOGY)
    o.set_particle_flavor(0, 1)
    for sys_ in (ctx, o):
        sys_.configure_harmonic_bond(0, 0, 1.0, 1.0)
        sys_.configure_harmonic_angle(0, 0, 0, 2.0, 2.6)
        sys_.configure_cosine_dihedral(0, 0, 0, 0, 0.5, 3.0, 0.2)
    k = rg.CUDAKernel(ctx, seed=5)
    edges = [(i, i + 1) for i in range(n - 1)]
    for c in chains:
        ig = k.add_topology(c, np.zeros(n, np.int32), edges)
        io = o.add_topology(c, np.zeros(n, np.int32), edges)
        np.testing.assert_array_equal(ig, io)
    if with_neighbor_list:
        k.create_neighbor_list(1.0)
    nb_g = k.break_bonds(1.0, [(0, 0, 0.3, 1e10)])
    nb_o = o.break_bonds(1.0, [(0, 0, 0.3, 1e10)])
    assert nb_g == nb_o > 0
    tops_g = {frozenset(int(i) for i in t) for _, t in k.get_topologies()}
    tops_o = {frozenset(int(i) for i in t) for _, t in o.topologies()}
    assert tops_g == tops_o
    edges_g = {frozenset((int(a), int(b))) for e in k.get_topology_edges() for a, b in e}
    edges_o = {frozenset((int(a), int(b))) for e in o.topology_edges() for a, b in e}
    assert edges_g == edges_o
    if not with_neighbor_list:
        k.create_neighbor_list(1.0)
    k.calculate_forces()
    e_o = o.calculate_forces()
    fg, ig = k.get_forces()
    _, _, io, fo, _ = o.particles()
    fg, = [fg[np.argsort(ig)]]
    fo, = [fo[np.argsort(io)]]
    scale = np.abs(fo).max()
    err = np.linalg.norm(fg - fo, axis=1) / np.maximum(np.linalg.norm(fo, axis=1), 1e-5 * scale)
    assert err.max() < 1e-5, err.max()
    np.testing.assert_allclose(k.energy, e_o, rtol=1e-5)


def test_break_then_run(rg):
    """A run after breaking uses the derived terms: the bonded energy of the pieces stays finite and the
    pieces keep their edges."""
    chains = stretched_chains(50, 20, seed=9)
    ctx = rg.Context((160.0, 160.0, 160.0), (True, True, True), 1.0, (1.0,))
    ctx.set_particle_flavor(0, ctx.TOPOLOGY)
    ctx.configure_harmonic_bond(0, 0, 1.0, 1.0)
    ctx.configure_harmonic_angle(0, 0, 0, 2.0, 2.6)
    k = rg.CUDAKernel(ctx, seed=5)
    for c in chains:
        k.add_topology(c, np.zeros(20, np.int32), [(i, i + 1) for i in range(19)])
    k.create_neighbor_list(1.0)
    k.break_bonds(1.0, [(0, 0, 0.3, 1e10)])
    before = k.get_topology_edges()
    k.run(200, 1e-3)
    assert np.isfinite(k.energy)
    after = k.get_topology_edges()
    assert [len(e) for e in before] == [len(e) for e in after]
