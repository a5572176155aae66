"""The oracle's spatial topology reactions against the reference's known answers
(readdy/test/TestTopologyReactions.cpp, TestTopologyReactionsExternal.cpp) and the coin probability."""
import numpy as np
import pytest

import oracle
from tests.golden import known_answers as ka
from tests.helpers import check_topology_case, topology_case_system


@pytest.mark.parametrize("case", ka.TOPOLOGY_REACTION_CASES, ids=lambda c: c["name"])
def test_oracle_topology_reaction_known_answers(case):
    s, _ = topology_case_system(case, "oracle")
    s.run(case["steps"], case["dt"])
    pos, t, ids, _, _ = s.particles()
    types_by_id = {int(i): int(tt) for i, tt in zip(ids, t)}
    pos_by_id = {int(i): p for i, p in zip(ids, pos)}
    check_topology_case(case, s.topologies(), types_by_id, pos_by_id, s.topology_edges())


def isolated_pairs(n_pairs, spacing=6.0):
    """Single-particle topologies X1 (type 0) and X2 (type 1) in isolated pairs 0.5 apart on a lattice."""
    side = int(np.ceil(n_pairs ** (1 / 3)))
    L = side * spacing
    g = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n_pairs]
    c = (g + 0.5) * spacing - L / 2
    return L, c, c + (0.0, 0.0, 0.5)


def test_oracle_topology_fusion_rate_matches_the_coin_probability():
    """Isolated X1 + X2 pairs of single-particle topologies fuse with probability 1 - exp(-rate dt)."""
    n = 3000
    L, a, b = isolated_pairs(n)
    s = oracle.OracleSystem([L, L, L], (True, True, True), 1.0, (0.0,) * 4, seed=9)
    for t in range(4):
        s.set_particle_flavor(t, 1)
    s.configure_harmonic_bond(2, 3, 1.0, 0.5)
    s.add_spatial_topology_reaction(1, (0, 0), (1, 0), (2, 1), (3, 1), 0.7, 1.0)
    for k in range(n):
        s.add_topology(a[k:k + 1], [0], [])
        s.add_topology(b[k:k + 1], [1], [])
    s.nl_setup(s.calculate_max_cutoff())
    done = s.evaluate_topology_reactions(1.0)
    p = 1 - np.exp(-0.7)
    assert abs(done - p * n) < 4 * np.sqrt(n * p * (1 - p)), (done, p * n)
    sizes = [len(i) for _, i in s.topologies()]
    assert sizes.count(2) == done and sizes.count(1) == 2 * (n - done)
    assert list(s.topology_reaction_counts()) == [done]


def _tops(s):
    return sorted((int(tt), tuple(sorted(int(i) for i in ids))) for tt, ids in s.topologies())


def test_oracle_spatial_rate_function():
    """SpatialTopologyReaction's rate function (SpatialTopologyReaction.h:179-191) called with the two
    topologies of each candidate (CPUEvaluateTopologyReactions.cpp:296-303): certain for pairs of single
    particles and zero for pairs of chains, so exactly the single-particle pairs fuse."""
    from tests.helpers import only_singles, rate_function_system
    s = rate_function_system("oracle", only_singles, n_pairs=40)
    assert s.evaluate_topology_reactions(1e-3) == 20
    tops = s.topologies()
    assert len(tops) == 20 + 40
    assert sorted((int(tt), len(ids)) for tt, ids in tops) == [(0, 2)] * 40 + [(1, 2)] * 20


def test_oracle_spatial_rate_function_equal_to_the_constant_rate():
    """A rate function that returns the constant gives the constant rate's result, event for event."""
    from tests.helpers import rate_function_system
    a = rate_function_system("oracle", 700.0, n_pairs=60, seed=4)
    b = rate_function_system("oracle", lambda x, y: 700.0, n_pairs=60, seed=4)
    na, nb = a.evaluate_topology_reactions(1e-3), b.evaluate_topology_reactions(1e-3)
    assert na == nb and 0 < na < 60
    assert _tops(a) == _tops(b)


def test_oracle_spatial_rate_function_errors():
    from tests.helpers import rate_function_system
    s = rate_function_system("oracle", lambda x, y: -1.0, n_pairs=8)
    with pytest.raises(RuntimeError):
        s.evaluate_topology_reactions(1e-3)

    def bad(x, y):
        raise KeyError("rate failed")

    s = rate_function_system("oracle", bad, n_pairs=8)
    with pytest.raises(KeyError):
        s.evaluate_topology_reactions(1e-3)
    o = oracle.OracleSystem([10.0] * 3, (True, True, True), 1.0, (0.0,) * 3)
    with pytest.raises(RuntimeError):  # topology-particle reactions take constant rates
        o.add_spatial_topology_reaction(4, (0, 0), (1, None), (0, 0), (2, None), lambda x, y: 1.0, 1.0)
