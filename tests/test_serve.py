"""Served form on the GPU: a request's result is the same alone, in a mix of requests and through the
per-system path; admission respects the device-memory budget and the submit order."""
import numpy as np
import pytest

from readdy_gb300.serve import serving_workload

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rg():
    import readdy_gb300
    readdy_gb300.load()
    return readdy_gb300


def small_stream(n_requests=6, seed=11):
    """Requests of the serving workload at test size: N in [300, 3000], 100-400 steps, counts every 50."""
    specs = serving_workload(seed=seed, n_requests=n_requests, n_range=(300, 3000), steps=(100, 400))
    for s in specs:
        s.count_stride = 50
    return specs


def run_all(specs, budget=1 << 30, plain_threshold=1 << 30, max_steps=64, **kw):
    from readdy_gb300.serve import Server
    srv = Server(budget, plain_threshold=plain_threshold, **kw)
    ids = {srv.submit(s.context(), s.positions, s.types, s.n_steps, s.dt, s.count_stride, s.seed): k
           for k, s in enumerate(specs)}
    out, trace = {}, []
    while len(out) < len(specs):
        srv.progress(max_steps)
        trace.append(srv.stats())
        for rid in srv.poll():
            out[ids[rid]] = srv.result(rid)
    return out, trace


def test_engine_request_equals_per_system_run(rg):
    s = small_stream(1, seed=5)[0]
    res, _ = run_all([s])
    k = rg.CUDAKernel(s.context(), seed=s.seed)
    k.add_particles(s.positions, s.types)
    ref = k.run(s.n_steps, s.dt, handler=rg.GILLESPIE, count_stride=s.count_stride)
    assert res[0]["status"] == 0
    np.testing.assert_array_equal(res[0]["counts"], ref)


def test_results_are_the_same_alone_and_in_the_mix(rg):
    specs = small_stream(6, seed=11)
    # the largest request takes the per-system leg, the others share the fused engine
    thr = sorted(len(s.positions) for s in specs)[-2]
    mix, _ = run_all(specs, plain_threshold=thr)
    for k, s in enumerate(specs):
        alone, _ = run_all([s], plain_threshold=thr)
        assert mix[k]["status"] == 0 and alone[0]["status"] == 0
        np.testing.assert_array_equal(mix[k]["counts"], alone[0]["counts"], err_msg=f"request {k}")
        assert len(mix[k]["counts"]) == s.n_steps // s.count_stride + 1


def test_admission_respects_the_budget_and_the_submit_order(rg):
    from readdy_gb300.serve import Server
    specs = small_stream(6, seed=23)
    sizes = [Server.request_bytes(s.context(), len(s.positions), s.n_steps, s.count_stride)[0] for s in specs]
    budget = int(2.2 * max(sizes))  # room for two of the largest at a time
    res, trace = run_all(specs, budget=budget)
    assert all(t["bytes_in_use"] <= budget for t in trace)
    assert max(t["active"] for t in trace) <= budget // min(sizes)
    admits = [res[k]["admit"] for k in range(len(specs))]
    assert admits == sorted(admits)  # first come, first served
    for k, s in enumerate(specs):
        c = res[k]["counts"]
        assert res[k]["status"] == 0
        mass = c @ np.asarray(s.mass)
        assert np.all(mass == len(s.positions))  # the network conserves mass units
        assert res[k]["finish"] >= res[k]["admit"] >= res[k]["submit"]


def test_particle_steps_are_counted_on_the_device_in_both_legs(rg):
    """Requests whose networks only convert species keep their particle count, so the particle-steps the
    server reports (engine leg and per-system leg, both counted on the device) are the sum of N x steps."""
    from readdy_gb300.serve import Server, RequestSpec
    rng = np.random.default_rng(3)
    specs = []
    for n, steps in [(400, 120), (900, 80), (5000, 60), (6000, 50)]:
        L = float(np.float32((n / 0.3) ** (1 / 3)))
        specs.append(RequestSpec(arrival=0.0, n_types=2, diffusion=[1.0, 0.5], box=L,
                                 reactions=[("conversion", (0, 1, 0.5)), ("conversion", (1, 0, 0.5))],
                                 positions=(rng.random((n, 3)) - 0.5) * L, types=np.zeros(n, np.int32),
                                 n_steps=steps, seed=int(rng.integers(1 << 40)), count_stride=10, mass=[1, 1]))
    srv = Server(1 << 32, plain_threshold=4096)  # the two larger requests take the per-system leg
    for s in specs:
        srv.submit(s.context(), s.positions, s.types, s.n_steps, s.dt, s.count_stride, s.seed)
    done = 0
    while done < len(specs):
        srv.progress(32)
        done += len(srv.poll())
    assert srv.stats()["particle_steps"] == sum(len(s.positions) * s.n_steps for s in specs)


def test_records_stream_while_requests_run(rg):
    """rdc_server_peek_records: while requests run, their records so far are a prefix of the final ones, in
    the engine leg (after each progress call) and in the per-system leg (after each chunk of its run); a
    per-system request run in chunks gives the records of one uninterrupted run."""
    from readdy_gb300.serve import Server
    specs = sorted(small_stream(2, seed=31), key=lambda s: len(s.positions))
    specs[0].n_steps, specs[0].count_stride = 1000, 50    # engine leg
    specs[1].n_steps, specs[1].count_stride = 4500, 100   # per-system leg, three chunks
    thr = len(specs[1].positions)
    assert len(specs[0].positions) < thr
    srv = Server(1 << 30, plain_threshold=thr)
    ids = [srv.submit(s.context(), s.positions, s.types, s.n_steps, s.dt, s.count_stride, s.seed) for s in specs]
    peeks = {rid: [] for rid in ids}
    done = {}
    while len(done) < len(ids):
        srv.progress(64)
        for rid in ids:
            if rid not in done:
                peeks[rid].append(srv.peek_records(rid))
        for rid in srv.poll():
            done[rid] = srv.result(rid)
    for rid, s in zip(ids, specs):
        final = done[rid]["counts"]
        assert done[rid]["status"] == 0 and len(final) == s.n_steps // s.count_stride + 1
        for p in peeks[rid]:
            np.testing.assert_array_equal(p, final[:len(p)])
        np.testing.assert_array_equal(srv.peek_records(rid), final)
    assert any(0 < len(p) < len(done[ids[0]]["counts"]) for p in peeks[ids[0]])
    k = rg.CUDAKernel(specs[1].context(), seed=specs[1].seed)
    k.add_particles(specs[1].positions, specs[1].types)
    ref = k.run(specs[1].n_steps, specs[1].dt, handler=rg.GILLESPIE, count_stride=specs[1].count_stride)
    np.testing.assert_array_equal(done[ids[1]]["counts"], ref)


def test_small_engine_requests_take_more_steps_per_launch(rg):
    """In one engine launch a request takes as many steps as fit into one step of the largest active engine
    request, by the cost model of a replica-step (a fixed part worth 740 particles plus its particles):
    after one launch a 200-particle request beside a 6000-particle one has taken (740 + 6000) // (740 + 200)
    = 7 steps, the large one 1; both end with their results alone."""
    from readdy_gb300.serve import Server, RequestSpec
    rng = np.random.default_rng(8)
    specs = []
    for n in (6000, 200):
        L = float(np.float32((n / 0.3) ** (1 / 3)))
        specs.append(RequestSpec(arrival=0.0, n_types=2, diffusion=[1.0, 0.5], box=L,
                                 reactions=[("conversion", (0, 1, 0.5)), ("conversion", (1, 0, 0.5))],
                                 positions=(rng.random((n, 3)) - 0.5) * L, types=np.zeros(n, np.int32),
                                 n_steps=40, seed=int(rng.integers(1 << 40)), count_stride=1, mass=[1, 1]))
    srv = Server(1 << 32, plain_threshold=1 << 30)
    ids = [srv.submit(s.context(), s.positions, s.types, s.n_steps, s.dt, s.count_stride, s.seed) for s in specs]
    srv.progress(1)
    assert len(srv.peek_records(ids[0])) == 1 + 1
    assert len(srv.peek_records(ids[1])) == 1 + 7
    done = {}
    while len(done) < 2:
        srv.progress(64)
        for rid in srv.poll():
            done[rid] = srv.result(rid)
    for rid, s in zip(ids, specs):
        alone, _ = run_all([s])
        np.testing.assert_array_equal(done[rid]["counts"], alone[0]["counts"])
