"""Served form: a request loop over independent simulations (rdc_server_* in include/readdy_cuda.h), and
the seeded request stream of the serving workload.

A request is one complete simulation -- its own species, diffusion constants, potentials, reactions,
box, particles, step count, time step, count stride and seed.  The server admits requests first come,
first served while their device bytes fit the budget, keeps their particle state resident on the
device, runs the small ones together in the fused replica engine (one launch per step) and the large
ones as per-system simulations, and reports per-type count records with submit/admit/finish times.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from .kernel import Context

_M64 = (1 << 64) - 1


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class Server:
    def __init__(self, budget_bytes: int, max_active: int = 1024, handler: int = N.GILLESPIE,
                 plain_threshold: int = 32768, plain_workers: int = 24):
        self._lib = N.load()
        h = C.c_void_p()
        N.check(self._lib.rdc_server_create(C.byref(h), int(budget_bytes), int(max_active), int(handler),
                                            int(plain_threshold)))
        self._h = h
        N.check(self._lib.rdc_server_set_plain_workers(h, int(plain_workers)))
        self.plain_workers = int(plain_workers)
        self.budget_bytes = int(budget_bytes)
        self.plain_threshold = int(plain_threshold)
        self.handler = handler
        self._types = {}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.rdc_server_destroy(h)
            self._h = None

    @staticmethod
    def request_bytes(context: Context, n: int, n_steps: int, count_stride: int, plain_threshold: int = 32768):
        """(device bytes, takes the per-system leg) of a request; host arithmetic only."""
        lib = N.load()
        b = C.c_uint64()
        p = C.c_int()
        N.check(lib.rdc_server_request_bytes(context.handle, int(n), int(n_steps), int(count_stride),
                                             int(plain_threshold), C.byref(b), C.byref(p)))
        return int(b.value), bool(p.value)

    def submit(self, context: Context, positions, types, n_steps: int, dt: float = 1e-3, count_stride: int = 100,
               seed: int = 0) -> int:
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        t = np.ascontiguousarray(np.broadcast_to(np.asarray(types, dtype=np.int32), (len(pos),)))
        rid = C.c_int64()
        N.check(self._lib.rdc_server_submit(self._h, context.handle, len(pos), _p(pos, C.c_double), _p(t, C.c_int),
                                            int(n_steps), float(dt), int(count_stride), int(seed) & _M64,
                                            C.byref(rid)))
        self._types[rid.value] = context.n_types
        return rid.value

    def progress(self, max_steps: int = 100) -> int:
        n = C.c_int64()
        N.check(self._lib.rdc_server_progress(self._h, int(max_steps), C.byref(n)))
        return n.value

    def poll(self, capacity: int = 4096):
        ids = np.zeros(capacity, np.int64)
        n = C.c_int64()
        N.check(self._lib.rdc_server_poll(self._h, capacity, _p(ids, C.c_int64), C.byref(n)))
        return [int(x) for x in ids[:n.value]]

    def result(self, request_id: int):
        """dict(counts=(n_records, n_types) int64, status=int, submit/admit/finish=seconds)."""
        nrec = C.c_int64()
        st = C.c_int()
        times = np.zeros(3)
        N.check(self._lib.rdc_server_result(self._h, int(request_id), 0, None, C.byref(nrec), C.byref(st),
                                            _p(times, C.c_double)))
        T = self._types[request_id]
        counts = np.zeros((nrec.value, T), np.int64)
        if nrec.value:
            N.check(self._lib.rdc_server_result(self._h, int(request_id), counts.size, _p(counts, C.c_int64),
                                                C.byref(nrec), C.byref(st), None))
        return dict(counts=counts, status=st.value, submit=times[0], admit=times[1], finish=times[2])

    def peek_records(self, request_id: int):
        """The count records the request has written so far, (n_records, n_types) int64, while it runs."""
        nrec = C.c_int64()
        N.check(self._lib.rdc_server_peek_records(self._h, int(request_id), 0, None, C.byref(nrec)))
        T = self._types[request_id]
        counts = np.zeros((nrec.value, T), np.int64)
        if nrec.value:
            N.check(self._lib.rdc_server_peek_records(self._h, int(request_id), counts.size, _p(counts, C.c_int64),
                                                      C.byref(nrec)))
        return counts[:nrec.value]

    def release(self, request_id: int):
        N.check(self._lib.rdc_server_release(self._h, int(request_id)))
        self._types.pop(request_id, None)

    def stats(self):
        ps = C.c_uint64()
        b = C.c_uint64()
        a = C.c_int64()
        p = C.c_int64()
        N.check(self._lib.rdc_server_stats(self._h, C.byref(ps), C.byref(b), C.byref(a), C.byref(p)))
        return dict(particle_steps=int(ps.value), bytes_in_use=int(b.value), active=int(a.value),
                    pending=int(p.value))


# ---- the serving workload ------------------------------------------------------------------------

@dataclass
class RequestSpec:
    """One seeded request of the serving workload."""
    arrival: float                 # seconds after the stream starts
    n_types: int
    diffusion: list
    box: float
    reactions: list                # (kind, args) in Context.add_<kind> argument order
    positions: np.ndarray
    types: np.ndarray
    n_steps: int
    seed: int
    dt: float = 1e-3
    count_stride: int = 100
    mass: list = field(default_factory=list)  # mass units per species (conserved by the network)

    def context(self) -> Context:
        L = self.box
        ctx = Context((L, L, L), (True, True, True), 1.0, tuple(self.diffusion))
        for a in range(self.n_types):
            for b in range(a, self.n_types):
                ctx.add_harmonic_repulsion(a, b, 10.0, 1.0)
        for kind, args in self.reactions:
            getattr(ctx, "add_" + kind)(*args)
        return ctx


def reaction_network(rng, n_types):
    """Seeded mass-conserving network over n_types species.  Species 0 has one mass unit.  Each later
    species k is either the fusion product of two earlier species i + j -> k (with its fission k -> i + j)
    or a conversion partner of one earlier species of the same mass (i -> k and k -> i).  Every reaction
    conserves mass units, so a system that starts from species 0 never holds more particles than it
    started with.  Rates are log-uniform in [1e-3, 1]; educt and product distances are 1."""
    def rate():
        return float(np.exp(rng.uniform(np.log(1e-3), np.log(1.0))))
    mass = [1]
    reactions = []
    for k in range(1, n_types):
        if rng.random() < 0.5:
            i, j = (int(x) for x in rng.integers(0, k, 2))
            mass.append(mass[i] + mass[j])
            reactions.append(("fusion", (i, j, k, rate(), 1.0)))
            reactions.append(("fission", (k, i, j, rate(), 1.0)))
        else:
            i = int(rng.integers(0, k))
            mass.append(mass[i])
            reactions.append(("conversion", (i, k, rate())))
            reactions.append(("conversion", (k, i, rate())))
    return reactions, mass


def serving_workload(seed=7, n_requests=2000, rate=20.0, n_range=(500, 200000), density=(0.1, 0.5),
                     steps=(1000, 100000), step_scale=1.0):
    """The seeded request stream: Poisson arrivals at `rate` per second; 2-6 species; N log-uniform in
    n_range at a density uniform in `density`; D uniform in [0.1, 2]; first- and second-order rates
    log-uniform in [1e-3, 1]; harmonic repulsion k = 10 (distance 1) between all species; steps
    log-uniform in `steps` (times step_scale), dt = 1e-3; per-type counts every 100 steps.  All
    particles start as species 0, uniformly in the box."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for q in range(n_requests):
        t += float(rng.exponential(1.0 / rate))
        T = int(rng.integers(2, 7))
        n = int(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1]))))
        rho = float(rng.uniform(*density))
        L = float(np.float32((n / rho) ** (1.0 / 3.0)))
        D = [float(x) for x in rng.uniform(0.1, 2.0, T)]
        reactions, mass = reaction_network(rng, T)
        st = int(np.exp(rng.uniform(np.log(steps[0]), np.log(steps[1]))) * step_scale)
        pos = (rng.random((n, 3)) - 0.5) * L
        out.append(RequestSpec(arrival=t, n_types=T, diffusion=D, box=L, reactions=reactions, positions=pos,
                               types=np.zeros(n, np.int32), n_steps=max(st, 1), seed=int(rng.integers(0, 2**63)),
                               mass=mass))
    return out


def run_stream(server: Server, specs, max_steps: int = 100, time_limit: float = None):
    """Replays the stream in wall-clock time: each request is submitted at its arrival time, the server
    progresses in chunks of up to max_steps, finished requests are collected.  Returns
    (results by stream index, wall seconds, particle-steps)."""
    t0 = time.perf_counter()
    ps0 = server.stats()["particle_steps"]
    order = sorted(range(len(specs)), key=lambda k: specs[k].arrival)
    nxt = 0
    ids = {}
    results = {}
    while len(results) < len(specs):
        now = time.perf_counter() - t0
        if time_limit is not None and now > time_limit:
            break
        while nxt < len(order) and specs[order[nxt]].arrival <= now:
            s = specs[order[nxt]]
            ids[server.submit(s.context(), s.positions, s.types, s.n_steps, s.dt, s.count_stride, s.seed)] = order[nxt]
            nxt += 1
        st = server.stats()
        if st["active"] == 0 and st["pending"] == 0:
            if nxt < len(order):
                time.sleep(max(0.0, min(0.01, specs[order[nxt]].arrival - now)))
            continue
        server.progress(max_steps)
        for rid in server.poll():
            results[ids[rid]] = server.result(rid)
            server.release(rid)
    wall = time.perf_counter() - t0
    return results, wall, server.stats()["particle_steps"] - ps0
