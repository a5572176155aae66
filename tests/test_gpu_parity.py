"""Parity of the CUDA kernel with the FP64 oracle and with the reference's known answers.

Tolerances (FP32 device arithmetic against FP64):
  * neighbour pair sets: bit-exact;
  * forces: |F_gpu - F_ref| <= 1e-5 * max(|F_ref|, 0.1 * S) per particle, where S is the sum of the
    magnitudes of the force terms acting on the particle (from the oracle).  The floor covers
    particles whose net force cancels: FP32 rounds every term at ~6e-8 of its own size, so the error
    of a cancelling sum scales with S, not with the net force; energies: relative 1e-5;
  * known-answer vectors: the reference test's own tolerance or 1e-5 relative, whichever is looser.
"""
import numpy as np
import pytest

import oracle
from tests.golden import known_answers as ka
from tests.helpers import abc_spec, by_id, crowded_spec, f32, make_context, make_oracle

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-5
ENERGY_RTOL = 1e-5


@pytest.fixture(scope="module")
def rg():
    import readdy_gb300
    readdy_gb300.load()
    return readdy_gb300


def gpu_system(rg, spec, pos, types, seed=1):
    ctx = make_context(spec)
    k = rg.CUDAKernel(ctx, seed=seed)
    k.add_particles(pos, types)
    return ctx, k


FLOOR = 0.1


def force_error(f_gpu, f_ref, scale):
    """Per-particle |dF| / max(|F|, FLOOR * S) and the plain relative error of the well-conditioned
    particles (|F| >= FLOOR * S)."""
    fn = np.linalg.norm(f_ref, axis=1)
    denom = np.maximum(fn, FLOOR * scale)
    denom = np.where(denom > 0, denom, 1.0)
    d = np.linalg.norm(f_gpu - f_ref, axis=1)
    good = (fn >= FLOOR * scale) & (fn > 0)
    return d / denom, (d[good] / fn[good]) if good.any() else np.zeros(1)


@pytest.mark.parametrize("case", ka.PAIR_CASES, ids=lambda c: c["name"])
def test_pair_potential_known_answers(rg, case):
    spec = dict(box=case["box"], periodic=case["periodic"], diffusion=case["diffusion"],
                potentials=[(k, a, b, p) for k, a, b, p in case["potentials"]])
    ctx, k = gpu_system(rg, spec, np.array(case["positions"], float), np.array(case["types"]))
    k.create_neighbor_list(ctx.calculate_max_cutoff())
    k.calculate_forces()
    k.calculate_forces()  # must not accumulate (TestStateModel.cpp:80-81)
    e = k.energy
    assert e == pytest.approx(case["energy"], rel=max(case.get("energy_rtol", 0), ENERGY_RTOL))
    f, ids = k.get_forces()
    (f,) = by_id(ids, f)
    exp = np.array(ka.per_particle_forces(case))
    scale = max(np.abs(exp).max(), 1e-12)
    np.testing.assert_allclose(f, exp, rtol=0, atol=max(case["force_atol"], FORCE_RTOL * scale))
    # the per-particle shares of the energy sum to it
    pe, _ = k.get_particle_energies()
    assert pe.sum() == pytest.approx(e, rel=1e-6, abs=1e-12)


@pytest.mark.parametrize("case", ka.BONDED_CASES, ids=lambda c: c["name"])
def test_bonded_known_answers(rg, case):
    ctx = rg.Context(case["box"], case["periodic"], 1.0, (1.0,))
    for idx, kf, l0 in case["bonds"]:
        ctx.configure_harmonic_bond(0, 0, kf, l0)
    for idx, kf, th in case["angles"]:
        ctx.configure_harmonic_angle(0, 0, 0, kf, th)
    for idx, kf, mult, phi0 in case["dihedrals"]:
        ctx.configure_cosine_dihedral(0, 0, 0, 0, kf, mult, phi0)
    n = len(case["positions"])
    edges = [(i, i + 1) for i in range(n - 1)]
    if not case["bonds"]:
        # every edge needs a bond configuration (GraphTopology.cpp:89-99); k = 0 bonds are skipped
        ctx.configure_harmonic_bond(0, 0, 0.0, 1.0)
    k = rg.CUDAKernel(ctx)
    k.add_topology(np.array(case["positions"], float), np.zeros(n, np.int32), edges)
    k.calculate_forces()
    e = k.energy
    assert e == pytest.approx(case["energy"], rel=max(case["energy_rtol"], ENERGY_RTOL), abs=1e-6)
    f, ids = k.get_forces()
    (f,) = by_id(ids, f)
    exp = np.array(case["forces"], float)
    np.testing.assert_allclose(f, exp, rtol=0, atol=max(case["force_atol"], 2e-5 * np.abs(exp).max()))


NL_BOXES = [((10, 10, 10), (1, 1, 1)), ((10, 10, 10), (0, 0, 0)), ((5, 12, 7), (1, 0, 1)),
            ((3.3, 3.3, 3.3), (1, 1, 1)), ((2.5, 8, 2.5), (1, 1, 0)), ((20, 4, 4), (1, 1, 1)),
            ((6, 6, 30), (0, 1, 1))]


@pytest.mark.parametrize("box,pbc", NL_BOXES)
@pytest.mark.parametrize("radius", [1, 2])
def test_neighbor_pairs_bit_exact(rg, box, pbc, radius):
    """kernels/cpu/test/TestNeighborList.cpp:267-362 on the device: the pair set equals the oracle's."""
    rng = np.random.default_rng(17)
    spec = dict(box=box, periodic=pbc, diffusion=(1.0, 1.0),
                potentials=[("harmonic_repulsion", 0, 1, dict(k=1.0, d=1.2)),
                            ("harmonic_repulsion", 0, 0, dict(k=1.0, d=0.9))])
    n = 600
    pos = (rng.random((n, 3)) - 0.5) * np.array(box, float)
    types = rng.integers(0, 2, n)
    ctx, k = gpu_system(rg, spec, pos, types)
    k.set_cell_radius(radius)
    k.create_neighbor_list(1.2)
    for step in range(3):
        p, t, ids = k.get_particles()
        o = make_oracle(spec)
        (p, t, ids) = by_id(ids, p, t, ids)
        o.add_particles(p, t)  # oracle ids 0..n-1 follow the id order of the device
        ref = o.brute_force_pairs(1.2)
        got = k.neighbor_pairs(1.2)
        id_of = ids.astype(np.uint64)
        ref_ids = np.sort(np.stack([id_of[ref[:, 0].astype(int)], id_of[ref[:, 1].astype(int)]], 1), axis=1)
        ref_ids = ref_ids[np.lexsort((ref_ids[:, 1], ref_ids[:, 0]))]
        assert len(got) > 0
        np.testing.assert_array_equal(got, ref_ids)
        k.euler_bd_integrator(0.01)
        k.update_neighbor_list()


def test_neighbor_pairs_at_the_cutoff(rg):
    """Pairs placed within a few ulp of the cutoff are decided exactly like the FP64 reference."""
    L = 50.0
    rc = 1.0
    pts, types = [], []
    rng = np.random.default_rng(3)
    for i in range(400):
        a = (rng.random(3) - 0.5) * (L - 4)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        r = np.float64(rc) * (1 + rng.integers(-4, 5) * 2.0 ** -24)
        b = a + r * d
        pts += [a, b]
        types += [0, 0]
    # pairs straddling the periodic boundary
    for i in range(100):
        a = np.array([L / 2 - 0.3, (rng.random() - 0.5) * L, (rng.random() - 0.5) * L])
        b = a + np.array([rc * (1 + rng.integers(-4, 5) * 2.0 ** -24), 0, 0])
        b[0] -= L
        pts += [a, b]
        types += [0, 0]
    pos = f32(np.array(pts))
    spec = dict(box=(L, L, L), periodic=(1, 1, 1), diffusion=(1.0,),
                potentials=[("harmonic_repulsion", 0, 0, dict(k=1.0, d=rc))])
    ctx, k = gpu_system(rg, spec, pos, np.array(types))
    k.create_neighbor_list(rc)
    p, t, ids = k.get_particles()
    (p, t, ids) = by_id(ids, p, t, ids)
    o = make_oracle(spec)
    o.add_particles(p, t)
    ref = o.brute_force_pairs(rc)
    got = k.neighbor_pairs(rc)
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("case", ka.EXTERNAL_CASES, ids=lambda c: c["name"])
def test_external_potential_known_answers(rg, case):
    n_types = max(case["types"]) + 1
    ctx = rg.Context(case["box"], case["periodic"], 1.0, (1.0,) * n_types)
    for kind, t, args in case["potentials"]:
        getattr(ctx, "add_" + kind)(t, *args)
    k = rg.CUDAKernel(ctx, seed=1)
    k.add_particles(np.array(case["positions"], float), np.array(case["types"]))
    k.calculate_forces()
    k.calculate_forces()  # must not accumulate
    assert k.energy == pytest.approx(case["energy"], rel=ENERGY_RTOL)
    f, ids = k.get_forces()
    (f,) = by_id(ids, f)
    exp = np.array(case["forces"])
    scale = max(np.abs(exp).max(), 1e-12)
    np.testing.assert_allclose(f, exp, rtol=0, atol=max(case["force_atol"], FORCE_RTOL * scale))


def _run_reference_loop(k, ctx, dt, n_steps, check):
    """run() of readdy/test/TestPotentials.cpp:56-73: forces, Euler BD and neighbour-list update for
    200 steps, with the positions checked after every step."""
    cutoff = ctx.calculate_max_cutoff()
    if cutoff > 0:
        k.create_neighbor_list(cutoff)
    for _ in range(n_steps):
        k.calculate_forces()
        k.euler_bd_integrator(dt)
        if cutoff > 0:
            k.update_neighbor_list()
        p, _, _ = k.get_particles()
        check(p)


def test_box_potential_confines_particles(rg):
    """TestPotentials.cpp:80-125: 10 A (D = 1) and 10 B (D = 0.1) near the origin of a non-periodic
    1^3 box, each under a harmonic box of k = 10 spanning [-1, 1]^3, A-B repulsion k = 0.01 d = 0.11:
    over 200 steps of 0.005 every particle stays within [-2.5, 2.5]^3 (most of them outside the
    simulation box, where only the external potential acts on them)."""
    rng = np.random.default_rng(12)
    ctx = rg.Context((1., 1., 1.), (False, False, False), 1.0, (1.0, 0.1))
    ctx.add_harmonic_repulsion(0, 1, 0.01, 0.11)
    for t in (0, 1):
        ctx.add_box(t, 10.0, (-1., -1., -1.), (2., 2., 2.))
    k = rg.CUDAKernel(ctx, seed=3)
    k.add_particles(rng.normal(size=(20, 3)), [0] * 10 + [1] * 10)

    def check(p):
        assert np.all(np.abs(p) <= 2.5), np.abs(p).max()
    _run_reference_loop(k, ctx, 0.005, 200, check)


def test_spherical_inclusion_confines_particles(rg):
    """TestPotentials.cpp:126-166: spherical inclusion of radius 3 (k = 20) in a non-periodic 10^3 box:
    every particle stays within distance 4 of the origin for 200 steps of 0.005."""
    rng = np.random.default_rng(13)
    ctx = rg.Context((10., 10., 10.), (False, False, False), 1.0, (1.0, 0.1))
    for t in (0, 1):
        ctx.add_sphere(t, 20.0, (0., 0., 0.), 3.0, True)
    k = rg.CUDAKernel(ctx, seed=4)
    k.add_particles(rng.normal(size=(20, 3)), [0] * 10 + [1] * 10)

    def check(p):
        assert np.all((p * p).sum(1) < 16.0)
    _run_reference_loop(k, ctx, 0.005, 200, check)


@pytest.mark.parametrize("pair", [False, True], ids=["external_only", "with_pairs"])
def test_external_potentials_match_oracle(rg, pair):
    """All eight order-1 forms on random positions, alone (each particle's force is one term, so the
    1e-5 bound is plain relative error, also next to the surfaces) and together with pair repulsion."""
    from tests.helpers import externals_spec
    spec, pos, types = externals_spec(n=4000, seed=3, pair=pair)
    pos = f32(pos)
    ctx, k = gpu_system(rg, spec, pos, types)
    if pair:
        k.create_neighbor_list(ctx.calculate_max_cutoff())
    k.calculate_forces()
    e_gpu = k.energy
    f_gpu, ids = k.get_forces()
    (f_gpu,) = by_id(ids, f_gpu)
    o = make_oracle(spec, n_threads=4)
    o.add_particles(pos, types)
    if pair:
        o.nl_setup(o.calculate_max_cutoff())
    e_ref = o.calculate_forces()
    _, _, oid, f_ref, _ = o.particles()
    sc = o.force_scales()
    (f_ref, sc) = by_id(oid, f_ref, sc)
    err, _ = force_error(f_gpu, f_ref, sc)
    for t in range(9):
        m = types == t
        print(f"type {t} ({spec['externals'][t][0]}): max err {err[m].max():.3e}")
    assert err.max() <= FORCE_RTOL
    assert abs(e_gpu - e_ref) <= ENERGY_RTOL * abs(e_ref)


def test_virial_matches_oracle(rg):
    """Pair virial of the crowded three-species chemistry (LJ, WIPH, HR) against the FP64 oracle: each
    entry within 1e-5 of the largest entry."""
    spec, pos, types = crowded_spec(n=20000, density=0.2, seed=5)
    pos = f32(pos)
    ctx = make_context(spec)
    ctx.record_virial = True
    k = rg.CUDAKernel(ctx, seed=1)
    k.add_particles(pos, types)
    k.create_neighbor_list(ctx.calculate_max_cutoff())
    k.calculate_forces()
    v_gpu = k.virial()
    p, t, ids = k.get_particles()
    (p, t) = by_id(ids, p, t)
    o = make_oracle(spec, n_threads=4)
    o.set_record_virial(True)
    o.add_particles(p, t)
    o.nl_setup(o.calculate_max_cutoff())
    o.calculate_forces()
    v_ref = o.virial()
    print("virial gpu", v_gpu.ravel(), "ref", v_ref.ravel())
    np.testing.assert_allclose(v_gpu, v_ref, rtol=0, atol=1e-5 * np.abs(v_ref).max())
    # without the flag the virial stays zero and forces are unchanged
    k2 = rg.CUDAKernel(make_context(spec), seed=1)
    k2.add_particles(pos, types)
    k2.create_neighbor_list(ctx.calculate_max_cutoff())
    k2.calculate_forces()
    f_off, _ = k2.get_forces()
    assert np.all(k2.virial() == 0)
    # switched on for the system as it is (rdc_set_record_virial: ReaDDy's Virial observable sets the flag
    # after particles may have been added), the next force calculation records it; the forces are those of
    # the walk that also sums the virial (each potential's force through a per-pair temporary), equal to the
    # plain walk's within 1e-5 of the largest force
    k2.set_record_virial(True)
    k2.calculate_forces()
    f_on, _ = k2.get_forces()
    np.testing.assert_allclose(f_on, f_off, rtol=0, atol=1e-5 * np.abs(f_off).max())
    np.testing.assert_allclose(k2.virial(), v_ref, rtol=0, atol=1e-5 * np.abs(v_ref).max())
    # and through a run's captured graph, and off again
    k2.run(2, 1e-4, handler=rg.UNCONTROLLED_APPROXIMATION)
    assert np.abs(k2.virial()).max() > 0
    k2.set_record_virial(False)
    k2.calculate_forces()
    assert np.all(k2.virial() == 0)


def _compare_forces(rg, spec, pos, types, label):
    ctx, k = gpu_system(rg, spec, pos, types)
    k.create_neighbor_list(ctx.calculate_max_cutoff())
    k.calculate_forces()
    e_gpu = k.energy
    f_gpu, ids = k.get_forces()
    p, t, ids2 = k.get_particles()
    (f_gpu,) = by_id(ids, f_gpu)
    (p, t) = by_id(ids2, p, t)
    o = make_oracle(spec, n_threads=8)
    o.add_particles(p, t)
    o.nl_setup(o.calculate_max_cutoff())
    e_ref = o.calculate_forces()
    _, _, oid, f_ref, _ = o.particles()
    sc = o.force_scales()
    (f_ref, sc) = by_id(oid, f_ref, sc)
    err, rel_good = force_error(f_gpu, f_ref, sc)
    print(f"{label}: n={len(p)} max err (floored) {err.max():.3e} (p99.9 {np.quantile(err, .999):.3e}); "
          f"max rel err of well-conditioned {rel_good.max():.3e} ({len(rel_good)} particles); "
          f"energy {e_gpu:.9g} vs {e_ref:.9g} rel {abs(e_gpu - e_ref) / max(abs(e_ref), 1e-30):.3e}")
    return err, e_gpu, e_ref


@pytest.mark.parametrize("n", [20000, 200000], ids=["20k", "200k"])
@pytest.mark.parametrize("which", ["lennard_jones", "weak_interaction_piecewise_harmonic", "harmonic_repulsion",
                                   "all"])
def test_forces_match_oracle_crowded(rg, which, n):
    """The crowded three-species chemistry, per potential type and combined: at 20k particles and at the
    full 200k-particle size (100^3 box, density 0.2)."""
    spec, pos, types = crowded_spec(n=n, density=0.2, seed=4)
    if which != "all":
        spec["potentials"] = [p for p in spec["potentials"] if p[0] == which]
    spec["reactions"] = []
    err, e_gpu, e_ref = _compare_forces(rg, spec, f32(pos), types, which)
    assert err.max() <= FORCE_RTOL
    assert abs(e_gpu - e_ref) <= ENERGY_RTOL * abs(e_ref)


def test_forces_match_oracle_screened_electrostatics(rg):
    rng = np.random.default_rng(8)
    n, L = 3000, 20.0
    pos = f32((rng.random((n, 3)) - 0.5) * L)
    spec = dict(box=(L, L, L), periodic=(1, 1, 1), diffusion=(1.0,),
                potentials=[("screened_electrostatics", 0, 0,
                             dict(C=-1.0, kappa=1.0, D=1.0, sigma=1.0, exponent=6, cutoff=3.0))])
    err, e_gpu, e_ref = _compare_forces(rg, spec, pos, np.zeros(n, int), "screened_electrostatics")
    assert err.max() <= FORCE_RTOL
    assert abs(e_gpu - e_ref) <= ENERGY_RTOL * abs(e_ref)


def _reaction_case_system(rg, case, seed):
    spec = dict(box=case["box"], periodic=case["periodic"], diffusion=case["diffusion"],
                reactions=[(kind, dict(p)) for kind, p in case["reactions"]])
    return gpu_system(rg, spec, np.array(case["positions"], float),
                      np.array(case.get("types", [0] * len(case["positions"]))), seed=seed)


@pytest.mark.parametrize("handler", ["uncontrolled_approximation", "gillespie"])
@pytest.mark.parametrize("case", ka.REACTION_CASES, ids=lambda c: c["name"])
def test_reaction_known_answers(rg, case, handler):
    for seed in range(5):
        ctx, k = _reaction_case_system(rg, case, seed)
        k.create_neighbor_list(ctx.calculate_max_cutoff())
        getattr(k, handler)(1.0)
        pos, types, _ = k.get_particles()
        assert len(pos) == case["expect_n"]
        if "expect_positions" in case:
            np.testing.assert_allclose(pos, np.array(case["expect_positions"]), rtol=case["pos_rtol"])
        else:
            got = sorted((int(t), tuple(np.round(p, 5))) for t, p in zip(types, pos))
            exp = sorted((t, tuple(np.round(np.array(p, float), 5))) for t, p in case["expect_particles"])
            assert [g[0] for g in got] == [e[0] for e in exp]
            np.testing.assert_allclose(np.array([g[1] for g in got]), np.array([e[1] for e in exp]),
                                       atol=case["pos_atol"])


@pytest.mark.parametrize("handler", ["uncontrolled_approximation", "gillespie"])
def test_fission_near_boundary(rg, handler):
    """readdy/test/TestReactions.cpp:191-213."""
    for seed in range(10):
        ctx = rg.Context((10., 10., 10.), (1, 1, 1), 1.0, (0.,))
        ctx.add_fission(0, 0, 0, 1e16, 2.0)
        k = rg.CUDAKernel(ctx, seed=seed)
        k.add_particles([(-4.9999999, 0, 0)], [0])
        k.create_neighbor_list(1.0)
        getattr(k, handler)(1.0)
        pos, _, _ = k.get_particles()
        assert len(pos) == 2
        assert (pos[0, 0] <= 0) != (pos[1, 0] <= 0)
        assert np.all(pos >= -5.0) and np.all(pos < 5.0)


def test_brownian_msd_matches_6Dt(rg):
    """Free diffusion: <|dx|^2> within 1 % of 6 D t with 60k displacement samples."""
    rng = np.random.default_rng(5)
    n, steps, dt, D = 60000, 30, 1e-3, 1.0
    ctx = rg.Context((1000., 1000., 1000.), (1, 1, 1), 1.0, (D,))
    k = rg.CUDAKernel(ctx, seed=11)
    p0 = f32((rng.random((n, 3)) - 0.5) * 100.0)
    ids = k.add_particles(p0, np.zeros(n, np.int32))
    for _ in range(steps):
        k.euler_bd_integrator(dt)
    p1, _, ids1 = k.get_particles()
    (p1,) = by_id(ids1, p1)
    msd = np.mean(np.sum((p1 - p0) ** 2, axis=1))
    assert abs(msd / (6 * D * dt * steps) - 1) < 0.01


def test_run_conserves_a_plus_b_c(rg):
    """A + B <-> C: A + C and B + C are conserved over a run (counts every 10 steps)."""
    spec, pos, types = abc_spec(n=2000, box=20.0, seed=2)
    ctx, k = gpu_system(rg, spec, pos, types, seed=3)
    counts = k.run(200, 1e-3, handler=rg.UNCONTROLLED_APPROXIMATION, count_stride=10)
    assert counts.shape == (21, 3)
    assert np.all(counts[:, 0] + counts[:, 2] == 1000)
    assert np.all(counts[:, 1] + counts[:, 2] == 1000)
    assert counts[-1, 2] > 0
    k.synchronize()


@pytest.mark.parametrize("external", [False, True], ids=["pairs", "pairs_and_external"])
@pytest.mark.parametrize("handler", [0, 1])
def test_batch_replica_equals_plain_run(rg, handler, external):
    """A replica advanced inside a batch follows the same trajectory as the same system run alone
    through the per-system path with the replica's seed (also under order-1 potentials)."""
    from readdy_gb300.batch import ReplicaBatch, replica_seed
    rng = np.random.default_rng(9)
    sizes = [200, 900, 2000, 450]
    specs = []
    poss, typess, boxes = [], [], []
    for n in sizes:
        L = float(np.float32((n / 0.25) ** (1 / 3)))
        spec, pos, types = abc_spec(n=n, box=L, seed=int(rng.integers(1 << 30)))
        if external:
            spec["externals"] = [("sphere", 0, (2.0, (0., 0., 0.), 3.0, True)),
                                 ("cylinder", 2, (1.0, (0.5, 0., 0.), (0., 1., 1.), 2.0, False))]
        specs.append(spec)
        poss.append(f32(pos))
        typess.append(types)
        boxes.append((L, L, L))
    ctx = make_context(specs[0])
    b = ReplicaBatch(ctx, boxes, [2 * n for n in sizes], seed=77)
    b.set_particles(poss, typess)
    b.configure(handler=handler, dt=1e-3, cell_width_scale=1.0, threads_per_block=256)
    steps = 100
    b.step(steps)
    b.synchronize()
    for r, n in enumerate(sizes):
        ctx_r = make_context(specs[r])
        k = rg.CUDAKernel(ctx_r, seed=replica_seed(77, r))
        k.add_particles(poss[r], typess[r])
        k.run(steps, 1e-3, handler=handler)
        pa, ta, ia = k.get_particles()
        pb, tb, ib = b.get_particles(r)
        (pa, ta, ia) = by_id(ia, pa, ta, ia)
        (pb, tb, ib) = by_id(ib, pb, tb, ib)
        assert len(pa) == len(pb)
        np.testing.assert_array_equal(ia, ib)
        np.testing.assert_array_equal(ta, tb)
        np.testing.assert_allclose(pa, pb, rtol=0, atol=1e-5)


def _reactive_batch(rg, periodic, dense, carry):
    """Six replicas of four species under harmonic repulsion with fast fusion, fission, conversion,
    decay and enzymatic reactions (capacity twice the initial count)."""
    from readdy_gb300.batch import ReplicaBatch
    rng = np.random.default_rng(31)
    density, reach = (1.0, 2.0) if dense else (0.25, 1.0)
    sizes = [200, 700, 1500, 3000, 450, 5000]
    boxes, poss, typess = [], [], []
    for n in sizes:
        L = float(np.float32((n / density) ** (1 / 3)))
        boxes.append((L, L, L))
        poss.append(f32((rng.random((n, 3)) - 0.5) * L))
        typess.append(rng.integers(0, 4, n).astype(np.int32))
    ctx = rg.Context(boxes[0], (periodic,) * 3, 1.0, (1.0, 1.0, 0.5, 0.8))
    for a in range(4):
        for b in range(a, 4):
            ctx.add_harmonic_repulsion(a, b, 10.0, 1.0)
    ctx.add_fusion(0, 1, 2, 5.0, reach)
    ctx.add_fission(2, 0, 1, 2.0, 1.0)
    ctx.add_conversion(0, 3, 0.5)
    ctx.add_decay(3, 0.5)
    ctx.add_enzymatic(2, 1, 0, 1.0, reach)
    b = ReplicaBatch(ctx, boxes, [2 * n for n in sizes], seed=5)
    b.set_particles(poss, typess)
    b.configure(handler=rg.UNCONTROLLED_APPROXIMATION, dt=1e-3, cell_width_scale=1.0, threads_per_block=256)
    b.set_carry_forces(carry)
    return b, sizes


@pytest.mark.parametrize("dense", [False, True], ids=["sparse", "dense"])
@pytest.mark.parametrize("periodic", [True, False], ids=["periodic", "walls"])
def test_batch_carried_forces_bitwise(rg, periodic, dense):
    """Pair forces carried from each step's event walk to the next step, with the particles near a
    reaction walking again, give the trajectory of forces summed at the start of every step bit for
    bit.  Dense replicas have particles with more reaction partners than the walk keeps in registers
    and more tuples than the tuple list holds; without walls particles leave the box."""
    a, sizes = _reactive_batch(rg, periodic, dense, carry=True)
    b, _ = _reactive_batch(rg, periodic, dense, carry=False)
    c0 = a.count_types()
    a.step(150)
    b.step(150)
    a.synchronize()
    b.synchronize()
    ca, cb = a.count_types(), b.count_types()
    np.testing.assert_array_equal(ca, cb)
    assert np.any(ca != c0)
    na = a.n_particles()
    for r in range(len(sizes)):
        pa, ta, ia = a.get_particles(r)
        pb, tb, ib = b.get_particles(r)
        assert na[r] == len(pa) == ca[r].sum()  # live particles of a state with removed slots in place
        (pa, ta, ia) = by_id(ia, pa, ta, ia)
        (pb, tb, ib) = by_id(ib, pb, tb, ib)
        np.testing.assert_array_equal(ia, ib)
        np.testing.assert_array_equal(ta, tb)
        np.testing.assert_array_equal(pa, pb)


def test_batch_flat_upload_equals_list_upload(rg):
    """rdc_batch_set_particles (one flat array with offsets) and rdc_batch_set_particles_list (one array per
    replica) give the same batch, and both reject a type out of range."""
    import ctypes as C
    from readdy_gb300 import _native as N
    b1, sizes = _reactive_batch(rg, True, False, carry=True)
    rng = np.random.default_rng(31)
    boxes, poss, typess = [], [], []
    for n in sizes:  # the draws of _reactive_batch
        L = float(np.float32((n / 0.25) ** (1 / 3)))
        boxes.append((L, L, L))
        poss.append(f32((rng.random((n, 3)) - 0.5) * L))
        typess.append(rng.integers(0, 4, n).astype(np.int32))
    b2, _ = _reactive_batch(rg, True, False, carry=True)
    offs = np.zeros(len(sizes) + 1, np.int64)
    offs[1:] = np.cumsum(sizes)
    flat = np.ascontiguousarray(np.concatenate(poss), np.float64)
    ty = np.ascontiguousarray(np.concatenate(typess), np.int32)
    lib = N.load()
    lib.rdc_batch_set_particles.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    assert lib.rdc_batch_set_particles(b2._h, offs.ctypes.data, flat.ctypes.data, ty.ctypes.data) == 0
    b2.configure(handler=rg.UNCONTROLLED_APPROXIMATION, dt=1e-3, cell_width_scale=1.0, threads_per_block=256)
    b1.step(20)
    b2.step(20)
    b1.synchronize()
    b2.synchronize()
    for r in range(len(sizes)):
        p1, t1, i1 = b1.get_particles(r)
        p2, t2, i2 = b2.get_particles(r)
        np.testing.assert_array_equal(i1, i2)
        np.testing.assert_array_equal(t1, t2)
        np.testing.assert_array_equal(p1, p2)
    bad = [t.copy() for t in typess]
    bad[2][5] = 7
    with pytest.raises(ValueError):
        b1.set_particles(poss, bad)


POLYMER_SIZES = {
    # 200 chains of 50 beads in 10k solvent, 30^3 box
    "small": dict(n_chains=200, chain_len=50, n_solvent=10000, box=30.0),
    # the full polymer workload: 2000 chains of 50 beads in 100k solvent, 120^3 box
    "full": dict(n_chains=2000, chain_len=50, n_solvent=100000, box=120.0),
}


def dihedral_near_zero_force_switch(pos, quads, box, band=2e-6):
    """Per particle: whether it belongs to a dihedral whose FP64 |cos phi| (the reference's m.n / (|m||n|),
    TorsionPotential.cpp:80-93) lies within `band` of the 1e-4 below which the reference sets the force
    to zero, so that FP32 rounding may put it on either side."""
    L = np.asarray(box, float)

    def d(a, b):  # minimum image b - a
        v = pos[b] - pos[a]
        return v - L * np.round(v / L)

    x_ji = d(quads[:, 1], quads[:, 0])
    x_kj = d(quads[:, 2], quads[:, 1])
    x_kl = d(quads[:, 2], quads[:, 3])
    m = np.cross(x_ji, x_kj)
    n = np.cross(x_kl, -x_kj)
    mm = np.maximum((m * m).sum(1), 1e-4)
    nn = np.maximum((n * n).sum(1), 1e-4)
    cos_phi = (m * n).sum(1) / np.maximum(np.sqrt(mm) * np.sqrt(nn), 1e-4)
    near = np.abs(np.abs(cos_phi) - 1e-4) < band
    flag = np.zeros(len(pos), bool)
    flag[quads[near].ravel()] = True
    return flag


@pytest.mark.parametrize("size", list(POLYMER_SIZES))
@pytest.mark.parametrize("terms", ["bond", "angle", "dihedral", "all"])
def test_polymer_forces_match_oracle(rg, terms, size):
    """Random-walk chains (step 1.0) with bond/angle/dihedral terms in solvent, per term type, at a small
    size and at the full polymer-in-solvent size."""
    from tests.helpers import polymer_spec
    spec, chains, solvent = polymer_spec(**POLYMER_SIZES[size], seed=6)
    use = {"bond", "angle", "dihedral"} if terms == "all" else {terms}
    ctx = make_context(dict(spec, potentials=spec["potentials"] if terms == "all" else []))
    ctx.configure_harmonic_bond(0, 0, spec["bond"]["k"] if "bond" in use else 0.0, spec["bond"]["l0"])
    if "angle" in use:
        ctx.configure_harmonic_angle(0, 0, 0, spec["angle"]["k"], spec["angle"]["theta0"])
    if "dihedral" in use:
        d = spec["dihedral"]
        ctx.configure_cosine_dihedral(0, 0, 0, 0, d["k"], d["n"], d["phi0"])
    k = rg.CUDAKernel(ctx, seed=1)
    L = len(chains[0])
    for c in chains:
        k.add_topology(f32(c), np.zeros(L, np.int32), [(i, i + 1) for i in range(L - 1)])
    k.add_particles(f32(solvent), np.ones(len(solvent), np.int32))
    k.create_neighbor_list(1.0)
    k.calculate_forces()
    f_gpu, ids = k.get_forces()
    p, t, ids2 = k.get_particles()
    (f_gpu,) = by_id(ids, f_gpu)
    (p, t) = by_id(ids2, p, t)
    o = make_oracle(dict(spec, potentials=spec["potentials"] if terms == "all" else []), n_threads=8)
    o.add_particles(p, t)
    nb = len(chains) * L
    idx = np.arange(nb).reshape(len(chains), L)
    if "bond" in use:
        o.add_harmonic_bonds(np.stack([idx[:, :-1].ravel(), idx[:, 1:].ravel()], 1), spec["bond"]["k"],
                             spec["bond"]["l0"])
    if "angle" in use:
        o.add_harmonic_angles(np.stack([idx[:, :-2].ravel(), idx[:, 1:-1].ravel(), idx[:, 2:].ravel()], 1),
                              spec["angle"]["k"], spec["angle"]["theta0"])
    quads = np.stack([idx[:, :-3].ravel(), idx[:, 1:-2].ravel(), idx[:, 2:-1].ravel(), idx[:, 3:].ravel()], 1)
    if "dihedral" in use:
        d = spec["dihedral"]
        o.add_cosine_dihedrals(quads, d["k"], d["n"], d["phi0"])
    o.nl_setup(1.0)
    e_ref = o.calculate_forces()
    _, _, oid, f_ref, _ = o.particles()
    sc = o.force_scales()
    (f_ref, sc) = by_id(oid, f_ref, sc)
    err, rel_good = force_error(f_gpu, f_ref, sc)
    e_gpu = k.energy
    print(f"polymer {terms}: max err (floored) {err.max():.3e} p99.9 {np.quantile(err, .999):.3e} "
          f"well-conditioned max {rel_good.max():.3e}; energy {e_gpu:.9g} vs {e_ref:.9g}")
    # a particle above the tolerance must sit on a dihedral within FP32 rounding of the |cos phi| < 1e-4
    # zero-force switch (TorsionPotential.cpp:91-93); any other is a failure
    bad = err > FORCE_RTOL
    if bad.any():
        assert "dihedral" in use, np.sort(err)[-8:]
        excused = dihedral_near_zero_force_switch(p[:nb], quads, spec["box"])
        excused = np.concatenate([excused, np.zeros(len(err) - nb, bool)])
        print(f"{bad.sum()} particles above tolerance, all on dihedrals at the zero-force switch")
        assert np.all(excused[bad]), (np.flatnonzero(bad & ~excused), err[bad & ~excused])
    assert abs(e_gpu - e_ref) <= ENERGY_RTOL * abs(e_ref)


def _observable_case(case):
    """(box, periodic, positions, types, borders for the histogram and the RDF, steps to run first)."""
    rng = np.random.default_rng(41)
    if case == "lattice":  # pair distances and coordinates on the bin borders
        g = np.arange(-4.0, 4.0)
        pos = np.array([[x, y, z] for x in g for y in g for z in g])
        types = rng.integers(0, 3, len(pos)).astype(np.int32)
        return (8., 8., 8.), (1, 1, 1), pos, types, np.arange(-4.0, 4.01, 1.0), np.arange(0., 4.01, 0.5), 0
    if case == "walls":  # particles on both sides of the walls of a closed box
        pos = (rng.random((3000, 3)) - 0.5) * 12.0
        types = rng.integers(0, 3, len(pos)).astype(np.int32)
        return (10., 10., 10.), (0, 0, 0), pos, types, np.linspace(-6., 6., 97), np.linspace(0., 7., 141), 0
    pos = (rng.random((4000, 3)) - 0.5) * 16.0
    types = rng.integers(0, 3, len(pos)).astype(np.int32)
    return (16., 16., 16.), (1, 1, 1), pos, types, np.linspace(-8., 8., 257), np.linspace(0., 7.5, 301), 20


@pytest.mark.parametrize("case", ["random", "lattice", "walls"])
def test_observables_match_oracle(rg, case):
    """HistogramAlongAxis and RadialDistribution on the device equal the FP64 restatement of the reference's
    observables bit for bit (counts and normalised distribution), on the state left by the GPU's dynamics:
    exact ties of coordinates and distances with the borders, particles outside a closed box, and a
    bin set too large for the per-block shared-memory histogram."""
    box, pbc, pos, types, hb, rb = _observable_case(case)[:6]
    steps = _observable_case(case)[6]
    ctx = rg.Context(box, pbc, 1.0, (1.0, 0.5, 0.2))
    for a in range(3):
        for b in range(a, 3):
            ctx.add_harmonic_repulsion(a, b, 10.0, 1.0)
    k = rg.CUDAKernel(ctx, seed=3)
    k.add_particles(f32(pos), types)
    if steps:
        k.run(steps, 1e-3)
    p, t, _ = k.get_particles()
    o = oracle.OracleSystem([float(np.float32(x)) for x in box], pbc, 1.0, (1.0, 0.5, 0.2))
    o.add_particles(np.asarray(p, np.float64), np.asarray(t, np.int32))
    for axis in range(3):
        for sel in ([0], [1, 2], [0, 1, 2]):
            np.testing.assert_array_equal(k.histogram_along_axis(hb, sel, axis), o.histogram_along_axis(hb, sel, axis))
    for frm, to in (([0], [1]), ([1, 2], [0, 1, 2]), ([0, 1, 2], [0, 1, 2])):
        _, dist, counts = k.radial_distribution(rb, frm, to, 0.25)
        oc, od = o.radial_distribution(rb, frm, to, 0.25)
        np.testing.assert_array_equal(counts, oc)
        np.testing.assert_array_equal(dist, od)
        assert counts.sum() > 0
    # more bins than the shared-memory histogram holds: counts go straight to global memory
    fine = np.linspace(0., 7.5, 5001)
    np.testing.assert_array_equal(k.radial_distribution(fine, [0], [1, 2], 0.25)[2],
                                  o.radial_distribution(fine, [0], [1, 2], 0.25)[0])


@pytest.mark.parametrize("steps", [0, 20], ids=["initial", "after_20_steps"])
@pytest.mark.parametrize("name", ["crowded_200k", "polymer_200k"])
def test_forces_match_oracle_on_the_benchmarked_single_systems(rg, name, steps):
    """The inputs that bench.py times through the per-system path (the 200k crowded system on its jittered
    lattice; 2000 chains of 50 beads in 100k solvent), at the start and after 20 steps of their own
    dynamics: forces and energy of the state the GPU holds against the oracle."""
    import bench
    w = bench.single_system(name)
    k = bench._gpu_system(w, seed=3)
    if steps:
        k.run(steps, w["dt"], handler=rg.GILLESPIE if w["handler"] == "gillespie" else rg.UNCONTROLLED_APPROXIMATION)
    cutoff = k.context.calculate_max_cutoff()
    k.create_neighbor_list(cutoff)
    k.calculate_forces()
    f_gpu, ids = k.get_forces()
    p, t, ids2 = k.get_particles()
    (f_gpu,) = by_id(ids, f_gpu)
    (p, t) = by_id(ids2, p, t)
    nb = 0
    w2 = dict(w, pos=p, types=t)
    if w["chains"] is not None:
        L = len(w["chains"][0])
        nb = L * len(w["chains"])
        w2 = dict(w, chains=list(p[:nb].reshape(-1, L, 3)), pos=p[nb:], types=t[nb:])
    o = bench._oracle_system(w2, seed=3, threads=8)
    o.nl_setup(cutoff)
    e_ref = o.calculate_forces()
    _, _, oid, f_ref, _ = o.particles()
    sc = o.force_scales()
    (f_ref, sc) = by_id(oid, f_ref, sc)
    err, rel_good = force_error(f_gpu, f_ref, sc)
    e_gpu = k.energy
    print(f"{name} after {steps} steps: max err (floored) {err.max():.3e} p99.9 {np.quantile(err, .999):.3e}; "
          f"energy {e_gpu:.9g} vs {e_ref:.9g}")
    bad = err > FORCE_RTOL
    if bad.any():
        assert nb > 0, np.sort(err)[-8:]
        idx = np.arange(nb).reshape(len(w["chains"]), -1)
        quads = np.stack([idx[:, :-3].ravel(), idx[:, 1:-2].ravel(), idx[:, 2:-1].ravel(), idx[:, 3:].ravel()], 1)
        excused = np.concatenate([dihedral_near_zero_force_switch(p[:nb], quads, w["box"]),
                                  np.zeros(len(err) - nb, bool)])
        assert np.all(excused[bad]), (np.flatnonzero(bad & ~excused), err[bad & ~excused])
    assert abs(e_gpu - e_ref) <= ENERGY_RTOL * abs(e_ref)
