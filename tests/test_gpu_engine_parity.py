"""Parity of the fused replica engine (the batched form behind the throughput figure) with the FP64
oracle and with the per-system path, including the replicas whose cell grid is widened to fit the
shared-memory cell array (above ~11.7k particles at density 0.25) and replicas whose cell starts stay
in global memory (capacity of 65536 particles or more).

Tolerances: forces |dF| <= 1e-5 * max(|F|, 0.1 * S) per particle (S: sum of the magnitudes of the pair
terms, from the oracle); trajectories through the batch and through the per-system path share ids and
types exactly and positions within 1e-5; ensemble means of counts within 3 sigma of oracle ensembles.
"""
import concurrent.futures as cf
import functools

import numpy as np
import pytest

import oracle
from tests.helpers import abc_spec, by_id, f32, make_context, make_oracle

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-5
FLOOR = 0.1


@pytest.fixture(scope="module")
def rg():
    import readdy_gb300
    readdy_gb300.load()
    return readdy_gb300


def _box(n, density=0.25):
    return float(np.float32((n / density) ** (1 / 3)))


def _natural_dims(L, cutoff=1.0):
    return int(np.floor(L / (cutoff + L * 2.0 ** -19 + 1e-6 * cutoff)))


@pytest.mark.parametrize("handler", [0, 1], ids=["uncontrolled_approximation", "gillespie"])
def test_widened_replicas_equal_plain_runs(rg, handler):
    """Replicas of 13k, 16k and 20k particles run on widened cells (their natural grid does not fit the
    shared-memory cell array) and one of 30k particles with capacity above 65535 keeps int starts in
    global memory; each follows the trajectory of the same system run alone through the per-system
    path with the replica's seed, next to small replicas, with forces carried between steps."""
    from readdy_gb300.batch import ReplicaBatch, replica_seed
    rng = np.random.default_rng(19)
    sizes = [13000, 600, 16000, 2500, 20000, 30000]
    caps = [2 * n if n < 30000 else 70000 for n in sizes]
    specs, poss, typess, boxes = [], [], [], []
    for n in sizes:
        L = _box(n)
        spec, pos, types = abc_spec(n=n, box=L, seed=int(rng.integers(1 << 30)))
        specs.append(spec)
        poss.append(f32(pos))
        typess.append(types)
        boxes.append((L, L, L))
    b = ReplicaBatch(make_context(specs[0]), boxes, caps, seed=123)
    b.set_particles(poss, typess)
    b.configure(handler=handler, dt=1e-3, cell_width_scale=1.0, threads_per_block=512)
    for r, n in enumerate(sizes):
        dims, shared = b.replica_grid(r)
        nat = _natural_dims(boxes[r][0])
        if n >= 13000 and caps[r] < 65536:
            assert shared and dims[0] < nat, (n, dims, nat)  # widened to fit shared memory
        elif caps[r] >= 65536:
            assert not shared and dims[0] == nat, (n, dims, nat)  # int starts in global memory
    steps = 60
    b.step(steps)
    b.synchronize()
    counts = b.reaction_counts()
    assert counts[:, 0].min() > 0  # every replica performed fusions
    for r, n in enumerate(sizes):
        k = rg.CUDAKernel(make_context(specs[r]), seed=replica_seed(123, r))
        k.add_particles(poss[r], typess[r])
        k.run(steps, 1e-3, handler=handler)
        pa, ta, ia = k.get_particles()
        pb, tb, ib = b.get_particles(r)
        (pa, ta, ia) = by_id(ia, pa, ta, ia)
        (pb, tb, ib) = by_id(ib, pb, tb, ib)
        assert len(pa) == len(pb), (n, len(pa), len(pb))
        np.testing.assert_array_equal(ia, ib)
        np.testing.assert_array_equal(ta, tb)
        np.testing.assert_allclose(pa, pb, rtol=0, atol=1e-5)
        np.testing.assert_array_equal(k.reaction_counts()[:2], counts[r, :2])


def _oracle_forces(spec, box, pos, types):
    o = make_oracle(dict(spec, box=box, reactions=[]), n_threads=8)
    o.add_particles(pos, types)
    o.nl_setup(o.calculate_max_cutoff())
    o.calculate_forces()
    _, _, oid, f_ref, _ = o.particles()
    sc = o.force_scales()
    return by_id(oid, f_ref, sc)


@pytest.mark.parametrize("handler", [0, 1], ids=["uncontrolled_approximation", "gillespie"])
def test_carried_forces_of_widened_replicas_match_oracle(rg, handler):
    """After a few steps with fast reactions, the pair forces a replica carries into its next step (summed
    in the event walk over its sorted state, and walked again over the unsorted state for the particles
    near a reaction) equal the oracle's FP64 forces on the same positions, on widened cells, on the
    natural grid and with int starts in global memory."""
    from readdy_gb300.batch import ReplicaBatch
    rng = np.random.default_rng(23)
    sizes = [18000, 3000, 14000, 25000]
    caps = [2 * sizes[0], 2 * sizes[1], 2 * sizes[2], 70000]
    specs, poss, typess, boxes = [], [], [], []
    for n in sizes:
        L = _box(n)
        spec, pos, types = abc_spec(n=n, box=L, seed=int(rng.integers(1 << 30)))
        spec["reactions"] = [("fusion", dict(a=0, b=1, c=2, rate=20.0, educt_distance=1.0)),
                             ("fission", dict(a=2, b=0, c=1, rate=5.0, product_distance=1.0))]
        specs.append(spec)
        poss.append(f32(pos))
        typess.append(types)
        boxes.append((L, L, L))
    b = ReplicaBatch(make_context(specs[0]), boxes, caps, seed=7)
    b.set_particles(poss, typess)
    b.configure(handler=handler, dt=1e-3, cell_width_scale=1.0, threads_per_block=512)
    grids = [b.replica_grid(r) for r in range(len(sizes))]
    assert grids[0][1] and grids[0][0][0] < _natural_dims(boxes[0][0])   # widened, shared memory
    assert not grids[3][1]                                               # global-memory starts
    b.step(8)
    b.synchronize()
    rc = b.reaction_counts()
    assert rc[:, 0].min() > 0 and rc[:, 1].sum() > 0  # fusions in every replica, fissions
    for r in range(len(sizes)):
        p, t, ids = b.get_particles(r)
        f, fids = b.get_forces(r)
        np.testing.assert_array_equal(ids, fids)
        (p, t, f) = by_id(ids, p, t, f)
        f_ref, sc = _oracle_forces(specs[r], boxes[r], p, t)
        fn = np.linalg.norm(f_ref, axis=1)
        err = np.linalg.norm(f - f_ref, axis=1) / np.maximum(np.maximum(fn, FLOOR * sc), 1e-30)
        print(f"replica {r} ({len(p)} particles, grid {grids[r]}): max force err {err.max():.3e}")
        assert err.max() <= FORCE_RTOL


def test_streamed_count_records_equal_the_per_system_records(rg):
    """Count records streamed from a batch (switched on after 7 steps, polled twice while steps continue)
    equal, record for record, the counts of the same replicas run alone through the per-system path, and
    carry the time steps of ReaDDy's time series."""
    from readdy_gb300.batch import ReplicaBatch, replica_seed
    from readdy_gb300 import io
    rng = np.random.default_rng(41)
    sizes = [300, 1200, 2500]
    specs, poss, typess, boxes = [], [], [], []
    for n in sizes:
        L = _box(n)
        spec, pos, types = abc_spec(n=n, box=L, seed=int(rng.integers(1 << 30)))
        specs.append(spec)
        poss.append(f32(pos))
        typess.append(types)
        boxes.append((L, L, L))
    b = ReplicaBatch(make_context(specs[0]), boxes, [2 * n for n in sizes], seed=55)
    b.set_particles(poss, typess)
    b.configure(handler=1, dt=1e-3, cell_width_scale=1.0, threads_per_block=256)
    b.step(7)
    b.record_counts(stride=10, max_records=16)
    b.step(23)
    s1, c1 = b.poll_count_records()
    b.step(40)
    s2, c2 = b.poll_count_records()
    steps, counts = np.concatenate([s1, s2]), np.concatenate([c1, c2])
    np.testing.assert_array_equal(steps, [7, 10, 20, 30, 40, 50, 60, 70])
    np.testing.assert_array_equal(counts[-1], b.count_types())
    lay = io.batch_n_particles_layout(steps, counts)
    for r, n in enumerate(sizes):
        k = rg.CUDAKernel(make_context(specs[r]), seed=replica_seed(55, r))
        k.add_particles(poss[r], typess[r])
        ref = k.run(70, 1e-3, handler=1, count_stride=10)  # t = 0, 10, ..., 70
        np.testing.assert_array_equal(counts[1:, r, :], ref[1:])
        np.testing.assert_array_equal(lay[f"readdy/observables/n_particles/replica_{r}/data"][1:], ref[1:])


def test_batch_virial_matches_oracle(rg):
    """The Virial observable of replicas of the batch (forces summed over the sorted state, carried forces
    off), after a few steps of dynamics with reactions, against the oracle's virial of the same positions:
    each entry within 1e-5 of the largest entry; a batch that carries its forces refuses."""
    from readdy_gb300.batch import ReplicaBatch
    rng = np.random.default_rng(29)
    sizes = [3000, 800, 14000, 25000]
    caps = [2 * n if n < 25000 else 70000 for n in sizes]
    specs, poss, typess, boxes = [], [], [], []
    for n in sizes:
        L = _box(n)
        spec, pos, types = abc_spec(n=n, box=L, seed=int(rng.integers(1 << 30)))
        specs.append(spec)
        poss.append(f32(pos))
        typess.append(types)
        boxes.append((L, L, L))
    b = ReplicaBatch(make_context(specs[0]), boxes, caps, seed=3)
    b.set_particles(poss, typess)
    b.configure(handler=1, dt=1e-3, cell_width_scale=1.0, threads_per_block=512)
    with pytest.raises(RuntimeError):
        b.virial()
    b.set_carry_forces(False)
    b.step(10)
    b.synchronize()
    vir = b.virial()
    for r in range(len(sizes)):
        p, t, ids = b.get_particles(r)
        (p, t) = by_id(ids, p, t)
        o = make_oracle(dict(specs[r], box=boxes[r], reactions=[]), n_threads=8)
        o.set_record_virial(True)
        o.add_particles(p, t)
        o.nl_setup(o.calculate_max_cutoff())
        o.calculate_forces()
        v_ref = o.virial()
        np.testing.assert_allclose(vir[r], v_ref, rtol=0, atol=1e-5 * np.abs(v_ref).max())


# ---- ensembles through the batch against ensembles of oracle runs ----------------------------------

SYSTEMS = {
    # 100 A + 100 B in a 10^3 box, 2000 steps of 5e-3
    "small": dict(n=200, box=10.0, steps=2000, dt=5e-3, seed=1),
    # 1000 A + 1000 B in a 20^3 box, 1000 steps of 1e-3 (the reference's plain A+B<->C workload)
    "abc2000": dict(n=2000, box=20.0, steps=1000, dt=1e-3, seed=1),
}
N_RUNS = 48


@functools.lru_cache(maxsize=None)
def oracle_ensemble(system, handler):
    """(final C, fusions, fissions) of N_RUNS oracle runs from one initial configuration, run on host
    threads (each run is one call into the oracle library, which releases the interpreter lock)."""
    s = SYSTEMS[system]
    spec, pos, types = abc_spec(n=s["n"], box=s["box"], seed=s["seed"])
    h = oracle.GILLESPIE if handler == 1 else oracle.UNCONTROLLED_APPROXIMATION

    def one(r):
        o = make_oracle(spec, seed=5000 + r)
        o.add_particles(f32(pos), types)
        c = o.run(s["steps"], s["dt"], handler=h, count_stride=s["steps"])
        return [c[-1, 2], *o.reaction_counts(2)]

    with cf.ThreadPoolExecutor(max_workers=16) as ex:
        return np.array(list(ex.map(one, range(N_RUNS))), float)


def _within_3_sigma(gpu, orc, what):
    for q, name in enumerate(["final C", "fusions", "fissions"]):
        diff = gpu[:, q].mean() - orc[:, q].mean()
        sigma = np.sqrt(gpu[:, q].var(ddof=1) / len(gpu) + orc[:, q].var(ddof=1) / len(orc))
        print(f"{what} {name}: GPU {gpu[:, q].mean():.2f} oracle {orc[:, q].mean():.2f} sigma {sigma:.2f}")
        assert abs(diff) <= 3 * sigma, f"{what} {name}: GPU {gpu[:, q].mean():.2f} vs oracle {orc[:, q].mean():.2f}"


@pytest.mark.parametrize("system", list(SYSTEMS))
@pytest.mark.parametrize("handler", [0, 1], ids=["uncontrolled_approximation", "gillespie"])
def test_batch_ensemble_matches_oracle_ensemble(rg, system, handler):
    """N_RUNS replicas of one A + B <-> C system in one batch (each replica its own random streams): the
    ensemble means of the final C count and of the per-replica fusion and fission counts agree with
    N_RUNS oracle runs within 3 sigma."""
    from readdy_gb300.batch import ReplicaBatch
    s = SYSTEMS[system]
    spec, pos, types = abc_spec(n=s["n"], box=s["box"], seed=s["seed"])
    L = s["box"]
    b = ReplicaBatch(make_context(spec), [(L, L, L)] * N_RUNS, [2 * s["n"]] * N_RUNS, seed=2024 + handler)
    b.set_particles([f32(pos)] * N_RUNS, [types] * N_RUNS)
    b.configure(handler=handler, dt=s["dt"], cell_width_scale=1.0, threads_per_block=512)
    b.step(s["steps"])
    b.synchronize()
    c = b.count_types()
    rc = b.reaction_counts()
    assert np.all(c[:, 0] + c[:, 2] == s["n"] // 2) and np.all(c[:, 1] + c[:, 2] == s["n"] - s["n"] // 2)
    gpu = np.stack([c[:, 2], rc[:, 0], rc[:, 1]], 1).astype(float)
    _within_3_sigma(gpu, oracle_ensemble(system, handler), f"batch {system}")


@pytest.mark.parametrize("handler", [0, 1], ids=["uncontrolled_approximation", "gillespie"])
def test_plain_path_abc2000_ensemble_matches_oracle_ensemble(rg, handler):
    """The 2000-particle A + B <-> C workload over 1000 steps of 1e-3 through the per-system path
    (one rdc_run per member): ensemble means within 3 sigma of the oracle ensemble."""
    s = SYSTEMS["abc2000"]
    spec, pos, types = abc_spec(n=s["n"], box=s["box"], seed=s["seed"])
    gpu = []
    for r in range(N_RUNS):
        k = rg.CUDAKernel(make_context(spec), seed=9000 + r)
        k.add_particles(f32(pos), types)
        c = k.run(s["steps"], s["dt"], handler=handler, count_stride=s["steps"])
        gpu.append([c[-1, 2], *k.reaction_counts()[:2]])
    _within_3_sigma(np.array(gpu, float), oracle_ensemble("abc2000", handler), "plain abc2000")


def test_streamed_trajectory_equals_the_particles_at_the_same_steps(rg):
    """Trajectory frames streamed from a batch (switched on after 7 steps, polled twice while steps
    continue) equal the particles of an identical batch read at the same steps, and fill ReaDDy's
    FlatTrajectory layout."""
    from readdy_gb300.batch import ReplicaBatch
    from readdy_gb300 import io
    rng = np.random.default_rng(43)
    sizes = [300, 1500, 14000]  # the last replica runs on widened cells
    poss, typess, boxes = [], [], []
    spec = None
    for n in sizes:
        L = _box(n)
        s_, pos, types = abc_spec(n=n, box=L, seed=int(rng.integers(1 << 30)))
        spec = spec or s_
        poss.append(f32(pos))
        typess.append(types)
        boxes.append((L, L, L))

    def batch():
        b = ReplicaBatch(make_context(spec), boxes, [2 * n for n in sizes], seed=77)
        b.set_particles(poss, typess)
        b.configure(handler=1, dt=1e-3, cell_width_scale=1.0, threads_per_block=256)
        return b

    a, ref = batch(), batch()
    sel = [0, 2]
    a.step(7)
    a.record_trajectory(sel, stride=10, max_frames=8)
    a.step(23)
    s1, f1 = a.poll_trajectory()
    a.step(20)
    s2, f2 = a.poll_trajectory()
    steps, frames = np.concatenate([s1, s2]), f1 + f2
    np.testing.assert_array_equal(steps, [7, 10, 20, 30, 40, 50])
    at = 0
    for s, fr in zip(steps, frames):
        ref.step(int(s) - at)
        at = int(s)
        for k, r in enumerate(sel):
            pr, tr, ir = ref.get_particles(r)
            pg, tg, ig = fr[k]
            og, orr = np.argsort(ig), np.argsort(ir)
            np.testing.assert_array_equal(ig[og], ir[orr])
            np.testing.assert_array_equal(tg[og], tr[orr])
            np.testing.assert_array_equal(pg[og], pr[orr])
    lay = io.batch_trajectory_layout(steps, frames, sel)
    for k, r in enumerate(sel):
        g = f"readdy/trajectory/replica_{r}"
        lim = lay[f"{g}/limits"]
        assert len(lim) == len(steps) and lim[0, 0] == 0 and lim[-1, 1] == len(lay[f"{g}/records"])
        np.testing.assert_array_equal(lim[:, 1] - lim[:, 0], [len(fr[k][2]) for fr in frames])
        np.testing.assert_array_equal(lay[f"{g}/time"], steps)
    a.record_trajectory([], 1, 1)  # off
    with pytest.raises(RuntimeError):
        a.poll_trajectory()
