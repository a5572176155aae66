"""The oracle's structural topology reactions against the reference's known answers
(readdy/test/TestTopologyReactions.cpp:116-323)."""
import numpy as np
import pytest

from tests.helpers import structural_system


def test_oracle_structural_change_particle_type():
    s = structural_system("oracle")
    s.add_structural_topology_reaction(0, lambda v: 1e10, lambda v: [("change_particle_type", 0, 1)])
    assert s.evaluate_topology_reactions(1.0) == 1
    v = s.topology(0)
    assert v.types.tolist() == [1, 0, 0]


def test_oracle_structural_add_edge():
    s = structural_system("oracle")
    s.add_structural_topology_reaction(0, lambda v: 1e10, lambda v: [("add_edge", 0, v.n_particles - 1)])
    s.evaluate_topology_reactions(1.0)
    (v,) = [s.topology(0)]
    assert {frozenset(e) for e in v.edges.tolist()} == {frozenset((0, 1)), frozenset((1, 2)), frozenset((0, 2))}


def test_oracle_structural_remove_edge_creates_children():
    s = structural_system("oracle")
    ids = s.topology(0).ids.tolist()
    s.add_structural_topology_reaction(0, lambda v: 1e10, lambda v: [("remove_edge", 0, 1)], expect_connected=False)
    s.evaluate_topology_reactions(1.0)
    tops = sorted((ids_.tolist() for _, ids_ in s.topologies()), key=len)
    assert tops == [ids[:1], ids[1:]]
    two = [s.topology(k) for k in range(2) if s.topology(k).n_particles == 2][0]
    assert two.edges.tolist() == [[0, 1]]


def test_oracle_structural_expect_connected_raises():
    s = structural_system("oracle")
    s.add_structural_topology_reaction(0, lambda v: 1e10, lambda v: [("remove_edge", 0, 1)], expect_connected=True)
    with pytest.raises(RuntimeError):
        s.evaluate_topology_reactions(1.0)


def split_rate(view):
    """the reference's rate function: n / 50 for a topology of n > 1 particles (TestTopologyReactions.cpp:289-291)"""
    return view.n_particles / 50.0 if view.n_particles > 1 else 0.0


def split_reaction(rng):
    """the reference's reaction function: remove the edge between vertices i and i + 1, i uniform in
    [0, n - 2] (TestTopologyReactions.cpp:272-288)"""
    def fn(view):
        if view.n_particles < 2:
            return []
        i = int(rng.integers(0, view.n_particles - 1))
        return [("remove_edge", i, i + 1)]
    return fn


def test_oracle_chain_split_up():
    """A chain of 50 splits at a random edge at rate n/50 until only single particles are left."""
    s = structural_system("oracle", n_small=0, chain=50)
    s.add_structural_topology_reaction(0, split_rate, split_reaction(np.random.default_rng(0)),
                                       expect_connected=False)
    s.run(500, 1.0)
    assert len(s.topologies()) == 50 and all(len(ids) == 1 for _, ids in s.topologies())


def test_oracle_one_structural_event_per_evaluation():
    """Structural events are all mutually dependent in the reference (eventsDependent with the default second
    particle index): certain coins on 40 topologies still give one event per evaluation."""
    s = structural_system("oracle", n_small=40)
    s.add_structural_topology_reaction(0, lambda v: 1e10 if v.types[0] == 0 else 0.0,
                                       lambda v: [("change_particle_type", 0, 1)])
    for k in range(10):
        assert s.evaluate_topology_reactions(1.0) == 1
    changed = sum(1 for k in range(40) if s.topology(k).types[0] == 1)
    assert changed == 10 and list(s.structural_reaction_counts()) == [10]


def test_oracle_structural_append_and_move():
    """Recipe steps that add a particle (joined to vertices 0 and 2) and move one."""
    s = structural_system("oracle")
    s.add_structural_topology_reaction(0, lambda v: 1e10 if v.n_particles == 3 else 0.0,
                                       lambda v: [("append_particle", [0, 2], 1, (1.0, 2.0, 3.0)),
                                                  ("change_particle_position", 1, (6.0, 0.5, -0.5))])
    s.evaluate_topology_reactions(1.0)
    v = s.topology(0)
    assert v.n_particles == 4 and v.types.tolist() == [0, 0, 0, 1]
    assert {frozenset(e) for e in v.edges.tolist()} == {frozenset(x) for x in ((0, 1), (1, 2), (0, 3), (2, 3))}
    np.testing.assert_allclose(v.positions[3], (1.0, 2.0, 3.0))
    np.testing.assert_allclose(v.positions[1], (-4.0, 0.5, -0.5))  # wrapped into the box
    assert s.n_particles == 4
