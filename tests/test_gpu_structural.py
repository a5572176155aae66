"""Structural topology reactions on the device path (rdc_add_structural_topology_reaction with the functions of
the caller, evaluated by rdc_evaluate_topology_reactions and rdc_run) against the reference's known answers
(readdy/test/TestTopologyReactions.cpp:116-323) and the oracle: the same pieces, edges, types and bonded
forces after a recipe."""
import numpy as np
import pytest

import oracle
from tests.helpers import f32, structural_system

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rg():
    import readdy_gb300
    readdy_gb300.load()
    return readdy_gb300


def test_structural_change_particle_type(rg):
    k = structural_system(rg)
    k.add_structural_topology_reaction(0, lambda v: 1e10, lambda v: [("change_particle_type", 0, 1)])
    assert k.evaluate_topology_reactions(1.0) == 1
    v = k.get_topology(0)
    assert v.types.tolist() == [1, 0, 0]
    _, t, ids = k.get_particles()
    assert dict(zip(ids.tolist(), t.tolist()))[int(v.ids[0])] == 1  # the device's particle changed too


def test_structural_add_edge(rg):
    k = structural_system(rg)
    k.add_structural_topology_reaction(0, lambda v: 1e10, lambda v: [("add_edge", 0, v.n_particles - 1)])
    k.evaluate_topology_reactions(1.0)
    v = k.get_topology(0)
    assert {frozenset(e) for e in v.edges.tolist()} == {frozenset((0, 1)), frozenset((1, 2)), frozenset((0, 2))}


def test_structural_remove_edge_creates_children(rg):
    k = structural_system(rg)
    ids = k.get_topology(0).ids.tolist()
    k.add_structural_topology_reaction(0, lambda v: 1e10, lambda v: [("remove_edge", 0, 1)], expect_connected=False)
    k.evaluate_topology_reactions(1.0)
    tops = sorted((i.tolist() for _, i in k.get_topologies()), key=len)
    assert tops == [ids[:1], ids[1:]]
    two = [k.get_topology(j) for j in range(2) if k.get_topology(j).n_particles == 2][0]
    assert two.edges.tolist() == [[0, 1]]


def test_structural_expect_connected_raises(rg):
    k = structural_system(rg)
    k.add_structural_topology_reaction(0, lambda v: 1e10, lambda v: [("remove_edge", 0, 1)], expect_connected=True)
    with pytest.raises(RuntimeError):
        k.evaluate_topology_reactions(1.0)


def test_structural_function_errors_reach_the_caller(rg):
    k = structural_system(rg)

    def bad(view):
        raise KeyError("recipe failed")

    k.add_structural_topology_reaction(0, lambda v: 1e10, bad)
    with pytest.raises(KeyError):
        k.evaluate_topology_reactions(1.0)


def test_chain_split_up(rg):
    """TestTopologyReactions.cpp:247-323: a chain of 50 splits at a random edge at rate n/50 until only single
    particles are left, through rdc_run."""
    from tests.test_oracle_structural import split_rate, split_reaction
    k = structural_system(rg, n_small=0, chain=50)
    k.add_structural_topology_reaction(0, split_rate, split_reaction(np.random.default_rng(0)), expect_connected=False)
    k.run(500, 1.0)
    tops = k.get_topologies()
    assert len(tops) == 50 and all(len(i) == 1 for _, i in tops)
    assert k.structural_reaction_counts()[0] == 49


def test_one_structural_event_per_evaluation(rg):
    """The reference takes any two structural events as dependent: one per evaluation, as the oracle."""
    k = structural_system(rg, n_small=40)
    k.add_structural_topology_reaction(0, lambda v: 1e10 if v.types[0] == 0 else 0.0,
                                       lambda v: [("change_particle_type", 0, 1)])
    for _ in range(10):
        assert k.evaluate_topology_reactions(1.0) == 1
    assert sum(1 for j in range(40) if k.get_topology(j).types[0] == 1) == 10
    assert list(k.structural_reaction_counts()) == [10]


def test_structural_recipe_matches_oracle_topologies_and_forces(rg):
    """One chain of 12 with bonds and angles: a recipe removes the edge 5-6, changes vertex 0 to Topology B and
    adds the edge 7-9.  The device and the oracle keep the same pieces, edges and types, and the bonded forces
    derived from the new graphs agree at 1e-5."""
    rng = np.random.default_rng(2)
    n = 12
    steps = rng.normal(size=(n, 3))
    steps /= np.linalg.norm(steps, axis=1, keepdims=True)
    pos = f32(np.cumsum(steps, axis=0) * 0.3)
    box = (10.0, 10.0, 10.0)
    ctx = rg.Context(box, (True, True, True), 1.0, (0.0,) * 4)
    o = oracle.OracleSystem(list(box), (True, True, True), 1.0, (0.0,) * 4, seed=3)
    for sys_ in (ctx, o):
        for t, fl in ((0, 1), (1, 1), (2, 1), (3, 0)):
            sys_.set_particle_flavor(t, fl)
        for a, b in ((0, 0), (0, 1), (1, 1)):
            sys_.configure_harmonic_bond(a, b, 10.0, 0.3)
        sys_.configure_harmonic_angle(0, 0, 0, 2.0, 2.5)
        sys_.configure_harmonic_angle(1, 0, 0, 2.0, 2.5)
    k = rg.CUDAKernel(ctx, seed=5)
    edges = [(i, i + 1) for i in range(n - 1)]
    np.testing.assert_array_equal(k.add_topology(pos, np.zeros(n, np.int32), edges),
                                  o.add_topology(pos, np.zeros(n, np.int32), edges))
    recipe = [("remove_edge", 5, 6), ("change_particle_type", 0, 1), ("add_edge", 7, 9)]
    for sys_ in (k, o):
        sys_.add_structural_topology_reaction(0, lambda v: 1e10 if v.n_particles == n else 0.0,
                                              lambda v: recipe, expect_connected=False)
    k.create_neighbor_list(1.0)
    o.nl_setup(1.0)
    assert k.evaluate_topology_reactions(1e-3) == o.evaluate_topology_reactions(1e-3) == 1
    tops_g = {(tt, frozenset(int(i) for i in ids)) for tt, ids in k.get_topologies()}
    tops_o = {(tt, frozenset(int(i) for i in ids)) for tt, ids in o.topologies()}
    assert tops_g == tops_o and len(tops_g) == 2
    eg = {frozenset((int(a), int(b))) for e in k.get_topology_edges() for a, b in e}
    eo = {frozenset((int(a), int(b))) for e in o.topology_edges() for a, b in e}
    assert eg == eo
    k.calculate_forces()
    e_o = o.calculate_forces()
    fg, ig = k.get_forces()
    _, to, io, fo, _ = o.particles()
    _, tg, ig2 = k.get_particles()
    np.testing.assert_array_equal(tg[np.argsort(ig2)], to[np.argsort(io)])
    fg, fo = fg[np.argsort(ig)], fo[np.argsort(io)]
    scale = np.abs(fo).max()
    err = np.linalg.norm(fg - fo, axis=1) / np.maximum(np.linalg.norm(fo, axis=1), 1e-5 * scale)
    assert err.max() < 1e-5, err.max()
    np.testing.assert_allclose(k.energy, e_o, rtol=1e-5)


def test_structural_append_and_move(rg):
    """Recipe steps that add a particle (joined to vertices 0 and 2) and move one, with and without a
    neighbour list; the new particle is on the device with its id, type and position."""
    for with_nl in (False, True):
        k = structural_system(rg)
        if with_nl:
            k.create_neighbor_list(1.0)
        k.add_structural_topology_reaction(0, lambda v: 1e10 if v.n_particles == 3 else 0.0,
                                           lambda v: [("append_particle", [0, 2], 1, (1.0, 2.0, 3.0)),
                                                      ("change_particle_position", 1, (6.0, 0.5, -0.5))])
        k.evaluate_topology_reactions(1.0)
        v = k.get_topology(0)
        assert v.n_particles == 4 and v.types.tolist() == [0, 0, 0, 1]
        assert {frozenset(e) for e in v.edges.tolist()} == {frozenset(x) for x in ((0, 1), (1, 2), (0, 3), (2, 3))}
        np.testing.assert_allclose(v.positions[3], (1.0, 2.0, 3.0))
        np.testing.assert_allclose(v.positions[1], (-4.0, 0.5, -0.5))  # wrapped into the box
        pos, t, ids = k.get_particles()
        assert k.n_particles == 4 and int(v.ids[3]) in ids.tolist()
        k.create_neighbor_list(1.0)
        k.calculate_forces()
        assert np.isfinite(k.energy)


def test_structural_append_matches_oracle_forces(rg):
    """A chain of 6: the recipe appends a particle joined to the last vertex and moves vertex 2; pieces, edges,
    positions and bonded forces agree with the oracle's (1e-5)."""
    rng = np.random.default_rng(4)
    n = 6
    steps = rng.normal(size=(n, 3))
    steps /= np.linalg.norm(steps, axis=1, keepdims=True)
    pos = f32(np.cumsum(steps, axis=0) * 0.3)
    new_at = tuple(f32(pos[-1] + (0.25, 0.1, 0.0)))
    moved_to = tuple(f32(pos[2] + (0.05, -0.05, 0.02)))
    box = (10.0, 10.0, 10.0)
    ctx = rg.Context(box, (True, True, True), 1.0, (0.0,) * 4)
    o = oracle.OracleSystem(list(box), (True, True, True), 1.0, (0.0,) * 4, seed=3)
    for sys_ in (ctx, o):
        for t, fl in ((0, 1), (1, 1), (2, 1), (3, 0)):
            sys_.set_particle_flavor(t, fl)
        for a, b in ((0, 0), (0, 1), (1, 1)):
            sys_.configure_harmonic_bond(a, b, 10.0, 0.3)
        sys_.configure_harmonic_angle(0, 0, 1, 2.0, 2.5)
    k = rg.CUDAKernel(ctx, seed=5)
    edges = [(i, i + 1) for i in range(n - 1)]
    k.add_topology(pos, np.zeros(n, np.int32), edges)
    o.add_topology(pos, np.zeros(n, np.int32), edges)
    recipe = [("append_particle", [n - 1], 1, new_at), ("change_particle_position", 2, moved_to)]
    for sys_ in (k, o):
        sys_.add_structural_topology_reaction(0, lambda v: 1e10 if v.n_particles == n else 0.0, lambda v: recipe)
    k.create_neighbor_list(1.0)
    o.nl_setup(1.0)
    assert k.evaluate_topology_reactions(1e-3) == o.evaluate_topology_reactions(1e-3) == 1
    vg, vo = k.get_topology(0), o.topology(0)
    np.testing.assert_array_equal(vg.ids, vo.ids)
    np.testing.assert_array_equal(vg.types, vo.types)
    assert {frozenset(e) for e in vg.edges.tolist()} == {frozenset(e) for e in vo.edges.tolist()}
    np.testing.assert_allclose(vg.positions, vo.positions, atol=1e-6)
    o.nl_update()
    k.calculate_forces()
    e_o = o.calculate_forces()
    fg, ig = k.get_forces()
    _, _, io, fo, _ = o.particles()
    fg, fo = fg[np.argsort(ig)], fo[np.argsort(io)]
    scale = np.abs(fo).max()
    err = np.linalg.norm(fg - fo, axis=1) / np.maximum(np.linalg.norm(fo, axis=1), 1e-5 * scale)
    assert err.max() < 1e-5, err.max()
    np.testing.assert_allclose(k.energy, e_o, rtol=1e-5)
