"""Spatial topology reactions on the device (rdc_evaluate_topology_reactions, and rdc_run with them) against
the reference's known answers (readdy/test/TestTopologyReactions.cpp, TestTopologyReactionsExternal.cpp), the
coin probability, and the oracle: the same topologies, edges and bonded forces after merges and attachments
whose outcome is certain."""
import numpy as np
import pytest

import oracle
from tests.golden import known_answers as ka
from tests.helpers import check_topology_case, f32, topology_case_system

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rg():
    import readdy_gb300
    readdy_gb300.load()
    return readdy_gb300


@pytest.mark.parametrize("case", ka.TOPOLOGY_REACTION_CASES, ids=lambda c: c["name"])
def test_topology_reaction_known_answers(rg, case):
    k, _ = topology_case_system(case, rg)
    k.run(case["steps"], case["dt"])
    pos, t, ids = k.get_particles()
    types_by_id = {int(i): int(tt) for i, tt in zip(ids, t)}
    pos_by_id = {int(i): p for i, p in zip(ids, pos)}
    check_topology_case(case, k.get_topologies(), types_by_id, pos_by_id, k.get_topology_edges())


def isolated_pairs(n_pairs, spacing=6.0):
    side = int(np.ceil(n_pairs ** (1 / 3)))
    L = side * spacing
    g = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n_pairs]
    c = (g + 0.5) * spacing - L / 2
    return L, c, c + (0.0, 0.0, 0.5)


def test_topology_fusion_rate_matches_the_coin_probability(rg):
    """20000 isolated X1 + X2 pairs of single-particle topologies fuse with probability 1 - exp(-rate dt);
    a second evaluation draws fresh clocks and coins."""
    n = 20000
    L, a, b = isolated_pairs(n)
    ctx = rg.Context((L, L, L), (True, True, True), 1.0, (0.0,) * 4)
    for t in range(4):
        ctx.set_particle_flavor(t, ctx.TOPOLOGY)
    ctx.configure_harmonic_bond(2, 3, 1.0, 0.5)
    ctx.add_spatial_topology_reaction(ctx.TT_FUSION, (0, 0), (1, 0), (2, 1), (3, 1), 0.7, 1.0)
    k = rg.CUDAKernel(ctx, seed=4)
    for i in range(n):
        k.add_topology(a[i:i + 1], [0], [])
        k.add_topology(b[i:i + 1], [1], [])
    k.create_neighbor_list(ctx.calculate_max_cutoff())
    done = k.evaluate_topology_reactions(1.0)
    p = 1 - np.exp(-0.7)
    assert abs(done - p * n) < 4 * np.sqrt(n * p * (1 - p)), (done, p * n)
    sizes = [len(i) for _, i in k.get_topologies()]
    assert sizes.count(2) == done and sizes.count(1) == 2 * (n - done)
    done2 = k.evaluate_topology_reactions(1.0)
    m = n - done
    assert abs(done2 - p * m) < 4 * np.sqrt(m * p * (1 - p)), (done2, p * m)
    assert list(k.topology_reaction_counts()) == [done + done2]
    # the fused pairs carry the Y--Z bond: types and edges
    pos, t, ids = k.get_particles()
    types = dict(zip(ids.tolist(), t.tolist()))
    for tt, tids in k.get_topologies():
        if len(tids) == 2:
            assert tt == 1 and sorted(types[int(i)] for i in tids) == [2, 3]


def chain_pairs(n_pairs, n=5, seed=0):
    """Pairs of nearly straight chains (end, middle..., end) along x whose facing ends are about 0.8 apart
    (within the reaction radius 1 for any jitter drawn); pairs 8 apart."""
    rng = np.random.default_rng(seed)
    side = int(np.ceil(n_pairs ** (1 / 3)))
    spacing = 2 * n + 8.0
    L = side * spacing
    chains = []
    for q in range(n_pairs):
        c = (np.array(np.unravel_index(q, (side,) * 3)) + 0.5) * spacing - L / 2
        tilt = rng.normal(scale=0.02, size=(n, 3))
        x0 = np.stack([np.arange(n) * 1.0, np.zeros(n), np.zeros(n)], 1) + tilt
        chains.append(f32(c + x0 - (n - 1 + 0.4, 0, 0)))
        chains.append(f32(c + x0 + (0.4, 0, 0)))
    return L, chains


def build_pair_systems(rg, mode_tp=False, n_pairs=60, n=5):
    """GPU and oracle systems: TOPOLOGY types middle 0, end 1; bonds, angles, dihedrals; end + end fusion
    (or, mode_tp, end + free A(2, NORMAL) attachment) with a certain coin."""
    L, chains = chain_pairs(n_pairs, n)
    box = (L, L, L)
    ctx = rg.Context(box, (True, True, True), 1.0, (0.0,) * 4)
    o = oracle.OracleSystem(list(box), (True, True, True), 1.0, (0.0,) * 4, seed=3)
    for t, fl in ((0, 1), (1, 1), (2, 0), (3, 1)):
        ctx.set_particle_flavor(t, fl)
        o.set_particle_flavor(t, fl)
    for sys_ in (ctx, o):
        for a, b in ((0, 0), (0, 1), (1, 1), (0, 3), (1, 3)):
            sys_.configure_harmonic_bond(a, b, 10.0, 1.0)
        sys_.configure_harmonic_angle(0, 0, 0, 5.0, np.pi)
        sys_.configure_harmonic_angle(1, 0, 0, 5.0, np.pi)
        sys_.configure_cosine_dihedral(0, 0, 0, 0, 1.0, 3.0, 0.0)
        if mode_tp:  # end(TA) + A -> middle(TA) -- end(TA): A joins as the new end
            sys_.add_spatial_topology_reaction(4, (1, 0), (2, None), (0, 0), (1, None), 1e10, 1.0)
        else:
            sys_.add_spatial_topology_reaction(1, (1, 0), (1, 0), (0, 0), (0, 0), 1e10, 1.0)
    k = rg.CUDAKernel(ctx, seed=6)
    types = np.array([1] + [0] * (n - 2) + [1], np.int32)
    edges = [(i, i + 1) for i in range(n - 1)]
    free = []
    for c_idx, c in enumerate(chains):
        if mode_tp and c_idx % 2 == 1:
            free.append(c[0])  # the partner chain's first bead becomes a free A facing the first chain's end
            continue
        ig = k.add_topology(c, types, edges)
        io = o.add_topology(c, types, edges)
        np.testing.assert_array_equal(ig, io)
    if mode_tp:
        fp = np.asarray(free)
        ig = k.add_particles(fp, np.full(len(fp), 2, np.int32))
        o.add_particles(fp, np.full(len(fp), 2, np.int32))
    return k, o


@pytest.mark.parametrize("mode_tp", [False, True], ids=["topology_fusion", "particle_attachment"])
def test_topology_reactions_match_oracle_topologies_and_forces(rg, mode_tp):
    """Chain pairs whose facing ends fuse (or chains that take up a free particle at one end), each pair
    isolated and the coin certain: the device and the oracle end with the same topologies, edges and
    particle types, and the bonded forces of the terms derived from the new graphs agree at 1e-5."""
    k, o = build_pair_systems(rg, mode_tp)
    cut = max(1.0, k.context.calculate_max_cutoff())
    k.create_neighbor_list(cut)
    o.nl_setup(cut)
    ng = k.evaluate_topology_reactions(1e-3)
    no = o.evaluate_topology_reactions(1e-3)
    assert ng == no == 60
    tops_g = {(tt, frozenset(int(i) for i in ids)) for tt, ids in k.get_topologies()}
    tops_o = {(tt, frozenset(int(i) for i in ids)) for tt, ids in o.topologies()}
    assert tops_g == tops_o
    eg = {frozenset((int(a), int(b))) for e in k.get_topology_edges() for a, b in e}
    eo = {frozenset((int(a), int(b))) for e in o.topology_edges() for a, b in e}
    assert eg == eo
    pg, tg, ig = k.get_particles()
    po, to, io, _, _ = o.particles()
    np.testing.assert_array_equal(tg[np.argsort(ig)], to[np.argsort(io)])
    k.calculate_forces()
    e_o = o.calculate_forces()
    fg, ig = k.get_forces()
    _, _, io, fo, _ = o.particles()
    fg, fo = fg[np.argsort(ig)], fo[np.argsort(io)]
    scale = np.abs(fo).max()
    err = np.linalg.norm(fg - fo, axis=1) / np.maximum(np.linalg.norm(fo, axis=1), 1e-5 * scale)
    assert err.max() < 1e-5, err.max()
    np.testing.assert_allclose(k.energy, e_o, rtol=1e-5)


def test_normal_enzymatic_reaction_with_a_topology_catalyst(rg):
    """readdy/test/TestTopologyReactionsExternal.cpp:70-116: a topology particle catalyses A -> B."""
    ctx = rg.Context((10.0, 10.0, 10.0), (True, True, True), 1.0, (1.0, 1.0, 1.0))
    ctx.set_particle_flavor(0, ctx.TOPOLOGY)
    ctx.add_enzymatic(0, 1, 2, 1e16, 1.0)
    k = rg.CUDAKernel(ctx, seed=2)
    k.add_topology(np.zeros((1, 3)), [0], [])
    k.add_particles(np.zeros((1, 3)), [1])
    k.create_neighbor_list(1.0)
    k.uncontrolled_approximation(1.0)
    _, t, _ = k.get_particles()
    assert sorted(t.tolist()) == [0, 2]
    assert len(k.get_topologies()) == 1


def _tops(tops):
    return {(int(tt), frozenset(int(i) for i in ids)) for tt, ids in tops}


def test_spatial_rate_function_matches_oracle(rg):
    """A rate function of the two topologies (SpatialTopologyReaction.h:179-191), certain for pairs of single
    particles and zero for pairs of chains: exactly the single-particle pairs fuse, on the device as in the
    oracle, topology for topology."""
    from tests.helpers import only_singles, rate_function_system
    k = rate_function_system(rg, only_singles, n_pairs=40)
    o = rate_function_system("oracle", only_singles, n_pairs=40)
    assert k.evaluate_topology_reactions(1e-3) == o.evaluate_topology_reactions(1e-3) == 20
    assert _tops(k.get_topologies()) == _tops(o.topologies())
    assert sorted((tt, len(ids)) for tt, ids in k.get_topologies()) == [(0, 2)] * 40 + [(1, 2)] * 20


def test_spatial_rate_function_equal_to_the_constant_rate(rg):
    """A rate function that returns the constant draws the same clocks and coins as the constant rate."""
    from tests.helpers import rate_function_system
    a = rate_function_system(rg, 700.0, n_pairs=60, seed=4)
    b = rate_function_system(rg, lambda x, y: 700.0, n_pairs=60, seed=4)
    na, nb = a.evaluate_topology_reactions(1e-3), b.evaluate_topology_reactions(1e-3)
    assert na == nb and 0 < na < 60
    assert _tops(a.get_topologies()) == _tops(b.get_topologies())


def test_spatial_rate_function_errors(rg):
    """A rate below 0 raises; an exception of the function reaches the caller; topology-particle reactions
    take constant rates only."""
    from tests.helpers import rate_function_system
    k = rate_function_system(rg, lambda x, y: -1.0, n_pairs=8)
    with pytest.raises(RuntimeError):
        k.evaluate_topology_reactions(1e-3)

    def bad(x, y):
        raise KeyError("rate failed")

    k = rate_function_system(rg, bad, n_pairs=8)
    with pytest.raises(KeyError):
        k.evaluate_topology_reactions(1e-3)
    ctx = rg.Context((10.0, 10.0, 10.0), (True, True, True), 1.0, (0.0,) * 3)
    with pytest.raises(ValueError):
        ctx.add_spatial_topology_reaction(4, (0, 0), (1, None), (0, 0), (2, None), lambda x, y: 1.0, 1.0)
