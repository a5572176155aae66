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
