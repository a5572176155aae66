"""Builds the same system on the CUDA kernel and on the FP64 oracle from one description."""
import numpy as np
import pytest

import oracle


def _pot_args(kind, p):
    if kind == "harmonic_repulsion":
        return (p["k"], p["d"])
    if kind == "weak_interaction_piecewise_harmonic":
        return (p["k"], p["desired"], p["depth"], p["cutoff"])
    if kind == "lennard_jones":
        return (p["m"], p["n"], p["cutoff"], p["shift"], p["epsilon"], p["sigma"])
    if kind == "screened_electrostatics":
        return (p["C"], p["kappa"], p["D"], p["sigma"], p["exponent"], p["cutoff"])
    raise KeyError(kind)


def make_context(spec):
    import readdy_gb300 as rg
    ctx = rg.Context(spec["box"], spec.get("periodic", (True, True, True)), spec.get("kbt", 1.0),
                     spec["diffusion"])
    for kind, t1, t2, p in spec.get("potentials", []):
        getattr(ctx, "add_" + kind)(t1, t2, *_pot_args(kind, p))
    for kind, t, args in spec.get("externals", []):
        getattr(ctx, "add_" + kind)(t, *args)
    for kind, p in spec.get("reactions", []):
        if kind == "fusion":
            ctx.add_fusion(p["a"], p["b"], p["c"], p["rate"], p["educt_distance"], p.get("w1", .5), p.get("w2", .5))
        elif kind == "fission":
            ctx.add_fission(p["a"], p["b"], p["c"], p["rate"], p["product_distance"], p.get("w1", .5),
                            p.get("w2", .5))
        elif kind == "conversion":
            ctx.add_conversion(p["a"], p["b"], p["rate"])
        elif kind == "decay":
            ctx.add_decay(p["a"], p["rate"])
        elif kind == "enzymatic":
            ctx.add_enzymatic(p["catalyst"], p["a"], p["b"], p["rate"], p["educt_distance"])
    return ctx


def make_oracle(spec, seed=1, n_threads=1, cll_radius=1):
    box = [float(np.float32(b)) for b in spec["box"]]
    s = oracle.OracleSystem(box, spec.get("periodic", (True, True, True)), spec.get("kbt", 1.0),
                            spec["diffusion"], seed=seed, n_threads=n_threads, cll_radius=cll_radius)
    for kind, t1, t2, p in spec.get("potentials", []):
        getattr(s, "add_" + kind)(t1, t2, *_pot_args(kind, p))
    for kind, t, args in spec.get("externals", []):
        getattr(s, "add_" + kind)(t, *args)
    for kind, p in spec.get("reactions", []):
        if kind == "fusion":
            s.add_fusion(p["a"], p["b"], p["c"], p["rate"], p["educt_distance"], p.get("w1", .5), p.get("w2", .5))
        elif kind == "fission":
            s.add_fission(p["a"], p["b"], p["c"], p["rate"], p["product_distance"], p.get("w1", .5), p.get("w2", .5))
        elif kind == "conversion":
            s.add_conversion(p["a"], p["b"], p["rate"])
        elif kind == "decay":
            s.add_decay(p["a"], p["rate"])
        elif kind == "enzymatic":
            s.add_enzymatic(p["catalyst"], p["a"], p["b"], p["rate"], p["educt_distance"])
    return s


def f32(a):
    """Values as the device holds them (FP32), widened back to FP64."""
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def by_id(ids, *arrays):
    o = np.argsort(ids)
    return [np.asarray(a)[o] for a in arrays]


def crowded_spec(n=20000, density=0.2, seed=0):
    """The three-species crowded chemistry of the 200k-particle benchmark at a smaller size."""
    L = float(np.float32((n / density) ** (1 / 3)))
    rng = np.random.default_rng(seed)
    pos = (rng.random((n, 3)) - 0.5) * L
    types = rng.choice(3, size=n, p=[0.5, 0.3, 0.2])
    spec = dict(
        box=(L, L, L), periodic=(True, True, True), diffusion=(1.0, 0.5, 0.2),
        potentials=[("lennard_jones", 0, 0, dict(m=12, n=6, cutoff=2.5, shift=True, epsilon=1.0, sigma=1.0)),
                    ("weak_interaction_piecewise_harmonic", 1, 1, dict(k=10.0, desired=1.0, depth=0.5,
                                                                       cutoff=1.5)),
                    ("harmonic_repulsion", 0, 1, dict(k=10.0, d=1.0)),
                    ("harmonic_repulsion", 0, 2, dict(k=10.0, d=1.0)),
                    ("harmonic_repulsion", 1, 2, dict(k=10.0, d=1.0)),
                    ("harmonic_repulsion", 2, 2, dict(k=10.0, d=1.0))],
        reactions=[("conversion", dict(a=0, b=1, rate=0.01))],
    )
    return spec, pos, types


def abc_spec(n=2000, box=20.0, seed=0):
    """A + B <-> C with harmonic repulsion between all species (the 1000 A + 1000 B workload)."""
    rng = np.random.default_rng(seed)
    pos = (rng.random((n, 3)) - 0.5) * box
    types = np.array([0] * (n // 2) + [1] * (n - n // 2))
    pots = [("harmonic_repulsion", a, b, dict(k=10.0, d=1.0)) for a in range(3) for b in range(a, 3)]
    spec = dict(box=(box, box, box), periodic=(True, True, True), diffusion=(1.0, 1.0, 0.5), potentials=pots,
                reactions=[("fusion", dict(a=0, b=1, c=2, rate=1.0, educt_distance=1.0)),
                           ("fission", dict(a=2, b=0, c=1, rate=0.1, product_distance=1.0))])
    return spec, pos, types


def polymer_spec(n_chains=200, chain_len=50, n_solvent=10000, box=30.0, seed=0):
    """Linear chains as random walks of step 1.0 in solvent with harmonic repulsion between all pairs
    (the polymer-in-solvent chemistry at a smaller size).  Type 0 = bead, 1 = solvent."""
    rng = np.random.default_rng(seed)
    chains = []
    for c in range(n_chains):
        start = (rng.random(3) - 0.5) * box
        steps = rng.normal(size=(chain_len - 1, 3))
        steps /= np.linalg.norm(steps, axis=1)[:, None]
        p = np.vstack([start, start + np.cumsum(steps, axis=0)])
        p = (p + box / 2) % box - box / 2
        chains.append(p)
    solvent = (rng.random((n_solvent, 3)) - 0.5) * box
    spec = dict(box=(box, box, box), periodic=(True, True, True), diffusion=(0.1, 1.0),
                potentials=[("harmonic_repulsion", a, b, dict(k=10.0, d=1.0)) for a, b in [(0, 0), (0, 1), (1, 1)]],
                bond=dict(k=100.0, l0=1.0), angle=dict(k=10.0, theta0=np.pi),
                dihedral=dict(k=1.0, n=3, phi0=0.0))
    return spec, chains, solvent


def externals_spec(n=4000, box=20.0, seed=0, pair=False):
    """Eight species, each under one order-1 potential (box in/out, sphere in/out, capsule in/out,
    spherical barrier, cylinder in/out), particles uniform in a periodic box."""
    rng = np.random.default_rng(seed)
    pos = (rng.random((n, 3)) - 0.5) * box
    types = rng.integers(0, 9, n)
    ext = [("box", 0, (10.0, (-3., -4., -5.), (6., 8., 7.), True)),
           ("box", 1, (10.0, (-3., -4., -5.), (6., 8., 7.), False)),
           ("sphere", 2, (5.0, (1., -1., 0.5), 4.0, True)),
           ("sphere", 3, (5.0, (1., -1., 0.5), 4.0, False)),
           ("capsule", 4, (3.0, (0.5, 0., 0.), (1., 2., -1.), 6.0, 2.5, True)),
           ("capsule", 5, (3.0, (0.5, 0., 0.), (1., 2., -1.), 6.0, 2.5, False)),
           ("spherical_barrier", 6, (3.0, 2.0, (-1., 2., 0.), 6.0)),
           ("cylinder", 7, (4.0, (1., -2., 3.), (0.3, 0.1, 1.), 3.5, True)),
           ("cylinder", 8, (4.0, (1., -2., 3.), (0.3, 0.1, 1.), 3.5, False))]
    pots = [("harmonic_repulsion", a, b, dict(k=10.0, d=1.0)) for a in range(9) for b in range(a, 9)] if pair else []
    spec = dict(box=(box, box, box), periodic=(True, True, True), diffusion=(1.0,) * 9, potentials=pots,
                externals=ext)
    return spec, pos, types


def topology_case_system(case, make, seed=1):
    """Builds a spatial topology reaction case (tests/golden/known_answers.py TOPOLOGY_REACTION_CASES) on the
    oracle (make = "oracle") or on the device (make = a readdy_gb300 module); returns (system, ids per topology
    as added)."""
    n = case["n_types"]
    if make == "oracle":
        s = oracle.OracleSystem(list(case["box"]), (True, True, True), 1.0, (0.0,) * n, seed=seed)
        target = s
    else:
        ctx = make.Context(case["box"], (True, True, True), 1.0, (0.0,) * n)
        target = ctx
    for t in range(n):
        target.set_particle_flavor(t, 1)
    for a, b, k, l0 in case["bonds"]:
        target.configure_harmonic_bond(a, b, k, l0)
    for mode, e1, e2, p1, p2, rate, radius, dmin in case["reactions"]:
        target.add_spatial_topology_reaction(mode, e1, e2, p1, p2, rate, radius, dmin)
    if make != "oracle":
        s = make.CUDAKernel(ctx, seed=seed)
    ids = []
    for tt, pos, types, edges in case["topologies"]:
        ids.append(s.add_topology(np.asarray(pos, float), np.asarray(types, np.int32), edges, topology_type=tt))
    return s, ids


def check_topology_case(case, tops, types_by_id, pos_by_id, edges):
    """Asserts the reference test's expectations on the topologies [(type, ids)], the particle types and
    positions by id and the edges per topology [(m, 2) ids]."""
    exp = case["expect"]
    assert sorted(len(i) for _, i in tops) == exp["sizes"], [len(i) for _, i in tops]
    if "types_of_topologies" in exp:
        assert sorted(t for t, _ in tops) == exp["types_of_topologies"]
    if "particle_types" in exp:
        got = sorted(sorted(types_by_id[int(i)] for i in ids) for _, ids in tops)
        assert got == sorted(exp["particle_types"]), got
    if "links" in exp:
        assert sum(1 for _, ids in tops for i in ids if types_by_id[int(i)] == 3) == exp["links"]
    if exp.get("linear"):
        (_, ids), = tops
        deg = {int(i): 0 for i in ids}
        for a, b in edges[0]:
            deg[int(a)] += 1
            deg[int(b)] += 1
        assert max(deg.values()) <= 2 and len(edges[0]) == len(ids) - 1
        ends = sorted(i for i, d in deg.items() if d == 1)
        assert all(types_by_id[i] == 1 for i in ends)
        assert sorted(pos_by_id[i][0] for i in ends) == pytest.approx(exp["end_x"])


def structural_system(make, n_small=1, chain=None, seed=1):
    """The fixture of readdy/test/TestTopologyReactions.cpp:82-95 on the oracle (make = "oracle") or the device
    (make = a readdy_gb300 module): Topology A 0, Topology B 1, Topology Invalid Type 2 (TOPOLOGY flavor),
    A 3 (NORMAL), bonds k = 10, l0 = 10 among the topology types, box 10.  Diffusion is 0: the cases test
    the topology structure only.  Adds n_small copies of setUpSmallTopology (:55-67; three particles at
    the origin, edges 0-1, 1-2) or, with `chain`, one chain of that many particles along x (:247-270)."""
    box = (10.0, 10.0, 10.0)
    if make == "oracle":
        s = oracle.OracleSystem(list(box), (True, True, True), 1.0, (0.0,) * 4, seed=seed)
        target = s
    else:
        ctx = make.Context(box, (True, True, True), 1.0, (0.0,) * 4)
        target = ctx
    for t, fl in ((0, 1), (1, 1), (2, 1), (3, 0)):
        target.set_particle_flavor(t, fl)
    for a, b in ((0, 0), (0, 1), (1, 1)):
        target.configure_harmonic_bond(a, b, 10.0, 10.0)
    if make != "oracle":
        s = make.CUDAKernel(ctx, seed=seed)
    if chain:
        pos = np.stack([-5 + np.arange(chain) * 10.0 / chain, np.zeros(chain), np.zeros(chain)], 1)
        s.add_topology(pos, np.zeros(chain, np.int32), [(i, i + 1) for i in range(chain - 1)])
    for _ in range(n_small):
        s.add_topology(np.zeros((3, 3)), np.zeros(3, np.int32), [(0, 1), (1, 2)])
    return s


def rate_function_system(make, rate, n_pairs=40, seed=1, spacing=6.0):
    """Isolated pairs of topologies facing each other, for spatial reactions with a rate function: even pairs
    are single-particle topologies X1 (type 0) and X2 (type 1) 0.5 apart, odd pairs chains X1-X1 and X2-X2 whose
    facing ends are 0.5 apart (their other particles 1.0 further out, beyond the radius).  All four types are
    TOPOLOGY flavored; X1 (topology type 0) + X2 (topology type 0) fuse into 2--3 of topology type 1 within
    1.0 at `rate` (a number or a function of two topology views).  make: rg (the CUDA package) or "oracle".
    Returns the system (kernel or oracle) with its neighbour list set up."""
    side = int(np.ceil(n_pairs ** (1 / 3)))
    L = side * spacing
    g = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n_pairs]
    centres = (g + 0.5) * spacing - L / 2
    box = (L, L, L)
    if make == "oracle":
        s = oracle.OracleSystem(list(box), (True, True, True), 1.0, (0.0,) * 4, seed=seed)
        conf = s
    else:
        conf = make.Context(box, (True, True, True), 1.0, (0.0,) * 4)
    for t in range(4):
        conf.set_particle_flavor(t, 1)
    for a, b, l0 in ((0, 0, 1.0), (1, 1, 1.0), (2, 3, 0.5), (0, 2, 1.0), (1, 3, 1.0)):
        conf.configure_harmonic_bond(a, b, 1.0, l0)
    conf.add_spatial_topology_reaction(1, (0, 0), (1, 0), (2, 1), (3, 1), rate, 1.0)
    if make != "oracle":
        s = make.CUDAKernel(conf, seed=seed)
    for k, c in enumerate(centres):
        if k % 2 == 0:
            s.add_topology(f32(c[None, :]), np.array([0], np.int32), [])
            s.add_topology(f32(c[None, :] + (0.0, 0.0, 0.5)), np.array([1], np.int32), [])
        else:
            s.add_topology(f32(np.stack([c - (0.0, 0.0, 1.0), c])), np.array([0, 0], np.int32), [(0, 1)])
            s.add_topology(f32(np.stack([c + (0.0, 0.0, 0.5), c + (0.0, 0.0, 1.5)])), np.array([1, 1], np.int32),
                           [(0, 1)])
    if make == "oracle":
        s.nl_setup(1.0)
    else:
        s.create_neighbor_list(1.0)
    return s


def only_singles(a, b):
    """A symmetric rate function: certain for two single-particle topologies, zero otherwise."""
    return 1e10 if len(a.ids) + len(b.ids) == 2 else 0.0
