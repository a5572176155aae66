#!/usr/bin/env python3
"""Benchmark of the batched uneven ensemble on one GB300.

Workload (the batched-replica configuration of the ReaDDy hot path): 4096 independent replicas of the
A + B <-> C chemistry (fusion A + B -> C, rate 1, educt distance 1; fission C -> A + B, rate 0.1,
product distance 1; harmonic repulsion k = 10, distance 1 between all species; D = 1, 1, 0.5;
kBT = 1).  Replica particle counts are log-uniform in [200, 20000] from a seed, half A and half B,
placed uniformly in a periodic cubic box whose edge holds the number density at 0.25.  Gillespie
handler, dt = 1e-3.  Inputs are synthetic and seeded.

Metric: particle-steps/s (particles advanced per step, summed over replicas and steps, over the device
time of the timed steps).  Every step is one persistent fused launch over all replicas replayed from
a CUDA graph.  The same replicas advanced one at a time through the per-system GPU path are timed on
a random sample and reported beside it, as is the FP64 CPU restatement of the reference kernel on the
host cores (a bounded sample).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "particle-steps/s batched vs one-at-a-time on GB300; p50/p99 solve latency"
UNIT = "particle-steps/s"
DENSITY = 0.25
N_MIN, N_MAX = 200, 20000
# DRAM bytes per particle of one fused step (dram__bytes_read.sum + dram__bytes_write.sum of one ncu
# capture of k_engine_step on the first 512 replicas of the ensemble, divided by its particles), and the
# same capture's warp instructions per particle-step and issue activity: the bound that applies to this
# kernel is the instruction stream, not DRAM bandwidth.
DRAM_BYTES_PER_PARTICLE = (99.62e6 + 104.93e6) / 2097522
WARP_INST_PER_PARTICLE = 304.89e6 / 2097522
ISSUE_ACTIVE_PCT = 52.8
# algorithmic bytes of one fused step per particle: the particle state (float4 position with the type,
# uint32 id) read once and written once (the pair forces carried between steps, 2 x 16 bytes, are a
# choice of the implementation and count as traffic, not as algorithmic bytes)
ALG_BYTES_PER_PARTICLE = 2 * (16 + 4)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--replicas", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--cpu-seconds", type=float, default=60.0,
                    help="time budget of the CPU legs: no further sampled replica starts once it is spent")
    ap.add_argument("--serve-requests", type=int, default=200, help="requests of the served-stream sample (0: skip)")
    ap.add_argument("--serve-seconds", type=float, default=120.0, help="wall-time limit of the served-stream sample")
    ap.add_argument("--single-systems", type=int, default=1, help="time the three single-system workloads (0: skip)")
    ap.add_argument("--plain-threshold", type=int, default=32768,
                    help="requests above this many particles take the per-system leg of the server")
    ap.add_argument("--plain-workers", type=int, default=24,
                    help="per-system requests the server runs at once, each on its own stream")
    ap.add_argument("--profile-system", choices=["abc_2k", "crowded_200k", "polymer_200k"], default=None,
                    help="only run one single-system workload through the per-system path (--warmup then "
                         "--steps steps; for profiler captures of its kernels)")
    return ap.parse_args()


def ensemble(seed: int, n_replicas: int):
    """Particle counts, boxes, positions and types of the uneven ensemble."""
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(N_MIN), np.log(N_MAX), n_replicas)).astype(np.int64)
    boxes, pos, types = [], [], []
    for n in ns:
        L = float(np.float32((n / DENSITY) ** (1.0 / 3.0)))
        boxes.append((L, L, L))
        pos.append((rng.random((n, 3)) - 0.5) * L)
        t = np.zeros(n, np.int32)
        t[n // 2:] = 1
        types.append(t)
    return ns, np.array(boxes), pos, types


def chemistry(box=(10.0, 10.0, 10.0)):
    import readdy_gb300 as rg
    ctx = rg.Context(box, (True, True, True), 1.0, (1.0, 1.0, 0.5))
    for a in range(3):
        for b in range(a, 3):
            ctx.add_harmonic_repulsion(a, b, 10.0, 1.0)
    ctx.add_fusion(0, 1, 2, 1.0, 1.0)
    ctx.add_fission(2, 0, 1, 0.1, 1.0)
    return ctx


def oracle_system(box, pos, types, seed, n_threads):
    import oracle
    o = oracle.OracleSystem(box, (True, True, True), 1.0, (1.0, 1.0, 0.5), seed=seed, n_threads=n_threads)
    for a in range(3):
        for b in range(a, 3):
            o.add_harmonic_repulsion(a, b, 10.0, 1.0)
    o.add_fusion(0, 1, 2, 1.0, 1.0)
    o.add_fission(2, 0, 1, 0.1, 1.0)
    o.add_particles(pos, types)
    return o


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while the timed region runs."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.proc = None
        self.path = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200", "-f", self.path],
                                         stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        loaded = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


CPU_SAMPLE = 16  # replicas of the ensemble that the CPU legs advance


def reference_cpu(ns, boxes, pos, types, seed, steps, warmup, budget_s=60.0):
    """The reference path on the host cores, on a fixed random sample of CPU_SAMPLE replicas of the ensemble:
    the reference's own pthread CPU kernel (kernels/cpu built from the reference sources into
    oracle/_ref; SimulationLoop::run with Gillespie) when it could be built, otherwise the FP64 oracle
    restatement.  Every sampled replica runs `warmup` untimed steps, then `steps` timed steps with all host
    threads; no further replica starts once budget_s is spent.  The reference kernel's own default thread count
    (4 x cores when READDY_N_CORES is unset, include/readdy/common/common.h:80-95) is timed beside it on the
    same replicas.  Returns (particle-steps/s, particles of the replicas run, cpu_baseline description).  The in-run baseline of the GPU arm and the reference arm call
    this with the same sample, step counts and budget."""
    import oracle
    from oracle import ref_build, reference_kernel
    cores = os.cpu_count() or 1
    sample = np.random.default_rng(seed + 5).choice(len(ns), size=min(CPU_SAMPLE, len(ns)), replace=False)
    use_ref = reference_kernel.available()
    spent, done, ran = 0.0, 0, []
    spent_default = 0.0  # the same replicas and steps at the reference's default thread count
    for r in sample:
        if ran and spent > budget_s:
            break
        ran.append(int(r))
        box = tuple(float(x) for x in boxes[r])
        if use_ref:
            def timed(n_threads):
                k = reference_kernel.ReferenceKernel(box, (True, True, True), 1.0, (1.0, 1.0, 0.5),
                                                     n_threads=n_threads)
                for a in range(3):
                    for b in range(a, 3):
                        k.add_harmonic_repulsion(a, b, 10.0, 1.0)
                k.add_fusion(0, 1, 2, 1.0, 1.0)
                k.add_fission(2, 0, 1, 0.1, 1.0)
                k.add_particles(pos[r], types[r])
                if warmup:
                    k.run(warmup, 1e-3, handler=reference_kernel.GILLESPIE)
                return k.run(steps, 1e-3, handler=reference_kernel.GILLESPIE)[1]
            sec = timed(cores)
            spent_default += timed(4 * cores)
        else:
            oracle.build()
            o = oracle_system(box, pos[r], types[r], seed + int(r), cores)
            if warmup:
                o.run(warmup, 1e-3, handler=oracle.GILLESPIE)
            t0 = time.perf_counter()
            o.run(steps, 1e-3, handler=oracle.GILLESPIE)
            sec = time.perf_counter() - t0
        spent += sec
        done += int(ns[r]) * steps
    what = ("the reference's pthread CPU kernel (kernels/cpu, compiled from the reference sources, "
            "SimulationLoop::run, Gillespie)" if use_ref else
            "the FP64 restatement of the reference CPU kernel (reference build unavailable: "
            f"{ref_build.unavailable_reason()})")
    v = done / spent
    n_run = int(ns[ran].sum())
    return v, n_run, {"value": v, "unit": UNIT, "cores": cores, "kind": "reference" if use_ref else "port",
               "threads": cores, "reference_default_threads": 4 * cores,
               "value_at_default_threads": (done / spent_default) if use_ref and spent_default > 0 else None,
               "sample": f"{len(ran)} random replicas of the ensemble ({n_run} particles) x "
                         f"{steps} steps after {warmup} warm-up steps, {what}, {cores} threads per replica; "
                         f"{done} particle-steps in {spent:.1f} s"}


def one_at_a_time(ns, boxes, pos, types, seed, n_sample, steps, rng_pick):
    """The same replicas through the per-system GPU path (rdc_run, graph-replayed), one after another,
    on a random sample of the ensemble."""
    import readdy_gb300 as rg
    from readdy_gb300.batch import replica_seed
    pick = rng_pick.choice(len(ns), size=min(n_sample, len(ns)), replace=False)
    total_ps, total_t = 0, 0.0
    for r in pick:
        ctx = chemistry(tuple(boxes[r]))
        k = rg.CUDAKernel(ctx, seed=replica_seed(seed, int(r)))
        k.add_particles(pos[r], types[r])
        k.run(2, 1e-3, handler=rg.GILLESPIE)
        t0 = time.perf_counter()
        k.run(steps, 1e-3, handler=rg.GILLESPIE)
        total_t += time.perf_counter() - t0
        total_ps += int(ns[r]) * steps
    return {"value": total_ps / total_t, "unit": UNIT, "sample": f"{len(pick)} random replicas x {steps} steps, "
            "each through the per-system path (CUDA-graph replay of the SimulationLoop step), run sequentially"}


# ---- single systems through the per-system path (the drop-in for one ReaDDy simulation) ----------

def single_system(name, seed=11):
    """(context arguments, particles, topologies, run settings) of the three single-system workloads:
    A+B<->C with 2000 particles in a 20^3 box; 200k crowded particles of three species (LJ, weak
    piecewise harmonic, harmonic repulsion) in 100^3 on a jittered lattice; 2000 chains of 50 beads
    with bonds, angles and dihedrals in 100k solvent in 120^3."""
    rng = np.random.default_rng(seed)
    if name == "abc_2k":
        L = 20.0
        pos = (rng.random((2000, 3)) - 0.5) * L
        types = np.array([0] * 1000 + [1] * 1000, np.int32)
        pots = [("harmonic_repulsion", a, b, (10.0, 1.0)) for a in range(3) for b in range(a, 3)]
        rx = [("fusion", (0, 1, 2, 1.0, 1.0)), ("fission", (2, 0, 1, 0.1, 1.0))]
        return dict(box=(L, L, L), D=(1.0, 1.0, 0.5), pots=pots, rx=rx, pos=pos, types=types, chains=None,
                    dt=1e-3, handler="ua")
    if name == "crowded_200k":
        L = 100.0
        n = 200000
        # jittered cubic lattice: uniformly random positions overlap at this density, and the
        # Lennard-Jones forces of overlapping pairs (~1e12 at r = 0.1) blow the Euler step up
        side = int(np.ceil(n ** (1.0 / 3.0)))
        a = L / side
        sites = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)
        sites = sites[rng.permutation(len(sites))[:n]]
        pos = (sites + 0.5 + rng.uniform(-0.25, 0.25, (n, 3))) * a - L / 2
        types = rng.choice(3, size=n, p=[0.5, 0.3, 0.2]).astype(np.int32)
        pots = [("lennard_jones", 0, 0, (12, 6, 2.5, True, 1.0, 1.0)),
                ("weak_interaction_piecewise_harmonic", 1, 1, (10.0, 1.0, 0.5, 1.5)),
                ("harmonic_repulsion", 0, 1, (10.0, 1.0)), ("harmonic_repulsion", 0, 2, (10.0, 1.0)),
                ("harmonic_repulsion", 1, 2, (10.0, 1.0)), ("harmonic_repulsion", 2, 2, (10.0, 1.0))]
        rx = [("conversion", (0, 1, 0.01))]
        # uncontrolled approximation: the reference's Gillespie selection is serial and quadratic in the
        # event count, and every species-0 particle carries a conversion event here
        return dict(box=(L, L, L), D=(1.0, 0.5, 0.2), pots=pots, rx=rx, pos=pos, types=types, chains=None,
                    dt=1e-4, handler="ua")
    if name == "polymer_200k":
        L = 120.0
        chains = []
        for c in range(2000):
            start = (rng.random(3) - 0.5) * L
            steps = rng.normal(size=(49, 3))
            steps /= np.linalg.norm(steps, axis=1)[:, None]
            p = np.vstack([start, start + np.cumsum(steps, axis=0)])
            chains.append((p + L / 2) % L - L / 2)
        pos = (rng.random((100000, 3)) - 0.5) * L
        pots = [("harmonic_repulsion", a, b, (10.0, 1.0)) for a, b in [(0, 0), (0, 1), (1, 1)]]
        return dict(box=(L, L, L), D=(0.1, 1.0), pots=pots, rx=[], pos=pos, types=np.ones(100000, np.int32),
                    chains=chains, dt=1e-4, handler="gillespie")
    raise KeyError(name)


def _gpu_system(w, seed):
    import readdy_gb300 as rg
    ctx = rg.Context(w["box"], (True, True, True), 1.0, w["D"])
    for kind, a, b, args in w["pots"]:
        getattr(ctx, "add_" + kind)(a, b, *args)
    for kind, args in w["rx"]:
        getattr(ctx, "add_" + kind)(*args)
    if w["chains"] is not None:
        ctx.configure_harmonic_bond(0, 0, 100.0, 1.0)
        ctx.configure_harmonic_angle(0, 0, 0, 10.0, np.pi)
        ctx.configure_cosine_dihedral(0, 0, 0, 0, 1.0, 3, 0.0)
    k = rg.CUDAKernel(ctx, seed=seed)
    if w["chains"] is not None:
        for c in w["chains"]:
            k.add_topology(c, np.zeros(len(c), np.int32), [(i, i + 1) for i in range(len(c) - 1)])
    k.add_particles(w["pos"], w["types"])
    return k


def _oracle_system(w, seed, threads):
    import oracle
    o = oracle.OracleSystem(w["box"], (True, True, True), 1.0, w["D"], seed=seed, n_threads=threads)
    for kind, a, b, args in w["pots"]:
        getattr(o, "add_" + kind)(a, b, *args)
    for kind, args in w["rx"]:
        getattr(o, "add_" + kind)(*args)
    if w["chains"] is not None:
        nb = sum(len(c) for c in w["chains"])
        o.add_particles(np.vstack(w["chains"]), np.zeros(nb, np.int32))
        idx = np.arange(nb).reshape(len(w["chains"]), -1)
        o.add_harmonic_bonds(np.stack([idx[:, :-1].ravel(), idx[:, 1:].ravel()], 1), 100.0, 1.0)
        o.add_harmonic_angles(np.stack([idx[:, :-2].ravel(), idx[:, 1:-1].ravel(), idx[:, 2:].ravel()], 1),
                              10.0, np.pi)
        o.add_cosine_dihedrals(np.stack([idx[:, :-3].ravel(), idx[:, 1:-2].ravel(), idx[:, 2:-1].ravel(),
                                         idx[:, 3:].ravel()], 1), 1.0, 3, 0.0)
    o.add_particles(w["pos"], w["types"])
    return o


def single_systems(gpu_steps=200, cpu_steps=3):
    """Time per step of each single-system workload through rdc_run (per-system kernels replayed from
    a CUDA graph) and through the FP64 oracle on all host cores."""
    import oracle
    import readdy_gb300 as rg
    oracle.build()
    cores = os.cpu_count() or 1
    out = {}
    for name in ("abc_2k", "crowded_200k", "polymer_200k"):
        w = single_system(name)
        n = len(w["pos"]) + (sum(len(c) for c in w["chains"]) if w["chains"] is not None else 0)
        h_gpu = rg.GILLESPIE if w["handler"] == "gillespie" else rg.UNCONTROLLED_APPROXIMATION
        k = _gpu_system(w, seed=3)
        k.run(5, w["dt"], handler=h_gpu)
        k.synchronize()
        t0 = time.perf_counter()
        k.run(gpu_steps, w["dt"], handler=h_gpu)
        k.synchronize()
        g = (time.perf_counter() - t0) / gpu_steps
        o = _oracle_system(w, seed=3, threads=cores)
        h_orc = oracle.GILLESPIE if w["handler"] == "gillespie" else oracle.UNCONTROLLED_APPROXIMATION
        t0 = time.perf_counter()
        o.run(cpu_steps, w["dt"], handler=h_orc)
        c = (time.perf_counter() - t0) / cpu_steps
        out[name] = {"particles": int(n), "gpu_ms_per_step": g * 1e3, "cpu_ms_per_step": c * 1e3,
                     "gpu_particle_steps_per_s": n / g, "cpu_particle_steps_per_s": n / c, "cpu_cores": cores,
                     "gpu_steps": gpu_steps, "cpu_steps": cpu_steps,
                     "timing": "wall clock around rdc_run (graph replays, one sync) / oracle run, same inputs"}
    return out


def profile_system(name, warmup, steps):
    """One single-system workload through rdc_run: `warmup` steps, then `steps` steps timed by wall
    clock (the command that profiler captures of the per-system kernels run)."""
    import readdy_gb300 as rg
    w = single_system(name)
    h = rg.GILLESPIE if w["handler"] == "gillespie" else rg.UNCONTROLLED_APPROXIMATION
    k = _gpu_system(w, seed=3)
    k.run(warmup, w["dt"], handler=h)
    k.synchronize()
    t0 = time.perf_counter()
    k.run(steps, w["dt"], handler=h)
    k.synchronize()
    dt = (time.perf_counter() - t0) / max(steps, 1)
    n = len(w["pos"]) + (sum(len(c) for c in w["chains"]) if w["chains"] is not None else 0)
    return {"profile_system": name, "particles": int(n), "steps": steps, "ms_per_step": dt * 1e3}


def serving(n_requests, time_limit, plain_threshold, seed=7, plain_workers=24):
    """The served form on the first n_requests of the seeded serving stream (Poisson arrivals at 20/s;
    2-6 species; N log-uniform in [500, 200000] at density 0.1-0.5; 1k-100k steps; counts every 100
    steps), replayed in wall-clock time against a 150 GB device-memory budget."""
    from readdy_gb300.serve import Server, run_stream, serving_workload
    specs = serving_workload(seed=seed, n_requests=n_requests)
    srv = Server(150 << 30, plain_threshold=plain_threshold, plain_workers=plain_workers)
    res, wall, ps = run_stream(srv, specs, max_steps=100, time_limit=time_limit)
    lat = np.array(sorted(r["finish"] - r["submit"] for r in res.values()))
    queue = np.array(sorted(r["admit"] - r["submit"] for r in res.values()))
    done_ps = float(sum(len(specs[k].positions) * specs[k].n_steps for k in res))
    return {"p50_latency_s": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_latency_s": float(np.percentile(lat, 99)) if len(lat) else None,
            "p50_queueing_s": float(np.percentile(queue, 50)) if len(queue) else None,
            "particle_steps_per_s": ps / wall, "completed": len(res), "requests": n_requests,
            "wall_s": wall, "time_limit_s": time_limit,
            "offered_particle_steps": float(sum(len(s.positions) * s.n_steps for s in specs)),
            "completed_particle_steps": done_ps,
            "failed": int(sum(r["status"] != 0 for r in res.values())),
            "plain_threshold": plain_threshold, "plain_workers": plain_workers,
            "particle_steps": "counted on the device in both legs (engine counter, per-system integrator counter)",
            "sample": f"first {n_requests} requests of the seeded 2000-request stream (seed {seed}), arrivals at "
                      f"20/s replayed in wall-clock time, 150 GB budget, stopped after {time_limit:.0f} s; latency "
                      "= finish - submit over the completed requests"}


def run_gb300(args, rank, world):
    import readdy_gb300 as rg
    from readdy_gb300.batch import ReplicaBatch
    rg.load()
    seed = rank_seed(args.seed, rank)
    ns, boxes, pos, types = ensemble(seed, args.replicas)
    caps = ns + 64
    ctx = chemistry()
    b = ReplicaBatch(ctx, boxes, caps, seed=seed)
    b.set_particles(pos, types)
    from readdy_gb300.batch import autotune_inplace
    tuned, tune_table = autotune_inplace(b)  # cell width x threads per block, on these replicas
    cws, tpb = tuned["cell_width_scale"], tuned["threads_per_block"]
    b.step(args.warmup)
    b.synchronize()
    barrier(world)
    ps0 = b.particle_steps()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clocks:
        ms = b.step_timed(args.steps)
    b.synchronize()
    ps1 = b.particle_steps()
    ms_max = allreduce_max(ms, world)
    ps_sum = allreduce_sum(ps1 - ps0, world)
    value = ps_sum / (ms_max / 1e3)

    # end to end through the public API: host arrays in, counts out
    t0 = time.perf_counter()
    e = ReplicaBatch(ctx, boxes, caps, seed=seed + 7)
    e.set_particles(pos, types)
    e.configure(handler=rg.GILLESPIE, dt=1e-3, cell_width_scale=cws, threads_per_block=tpb)
    e.step(args.steps)
    counts = e.count_types()
    e2e_t = time.perf_counter() - t0
    e2e_ps = e.particle_steps()
    del e
    # float4 particles; per replica its descriptor (256 B), state (40 B), LPT order slot (4 B) and two
    # unpacking offsets (16 B); one set of potential/reaction tables (36752 B)
    h2d = int(sum(len(p) for p in pos) * 16 + len(ns) * (256 + 40 + 4 + 16) + 36752)
    d2h = int(counts.nbytes)

    result = None
    if rank == 0:
        pick = np.random.default_rng(args.seed + 99)
        oat = one_at_a_time(ns, boxes, pos, types, seed, 64, 50, pick)
        _, _, cpu = reference_cpu(ns, boxes, pos, types, args.seed, args.steps, args.warmup, args.cpu_seconds)
        served = (serving(args.serve_requests, args.serve_seconds, args.plain_threshold, plain_workers=args.plain_workers)
                  if args.serve_requests else None)
        singles = single_systems() if args.single_systems else None
        peak, peak_kind = measured_peaks()
        n_avg = (ps1 - ps0) / args.steps
        launch_ms = ms / args.steps
        achieved = ALG_BYTES_PER_PARTICLE * n_avg / (launch_ms / 1e3) / 1e9
        result = {
            "metric": METRIC,
            "value": value,
            "unit": UNIT,
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms_max / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic (seeded uneven ensemble)",
            "config": {
                "workload": "batched uneven ensemble: 4096 replicas of A+B<->C, N log-uniform in [200, 20000], "
                            "density 0.25, HR k=10 d=1, Gillespie, dt=1e-3",
                "replicas": int(args.replicas), "particles": int(ns.sum()),
                "launch": "one persistent fused launch per step (k_engine_step), CUDA graph",
                "cell_width_scale": cws, "threads_per_block": tpb,
                "autotune": {"chosen": tuned, "table": tune_table},
                "l2": "inputs larger than L2 (particle state %.0f MB > 129 MB)" % (ns.sum() * 40 / 1e6),
                "parallelism": f"replicas only, {world} rank(s), one ensemble per GPU",
            },
            "one_at_a_time": oat,
            "batched_over_one_at_a_time": value / world / oat["value"],
            "e2e": {"value": e2e_ps / e2e_t, "unit": UNIT, "h2d_bytes_per_step": h2d // max(args.steps, 1),
                    "d2h_bytes_per_step": d2h // max(args.steps, 1),
                    "timed": "ReplicaBatch create + set_particles (host arrays) + configure + steps + count_types"},
            "roofline": {"bound": "hbm", "kernel": "k_engine_step", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                         "algorithmic_bytes_per_launch": ALG_BYTES_PER_PARTICLE * n_avg,
                         "traffic": DRAM_BYTES_PER_PARTICLE * n_avg if DRAM_BYTES_PER_PARTICLE else None,
                         "traffic_source": "ncu capture of a smaller ensemble scaled by particles",
                         "issue": {"warp_instructions_per_particle_step": WARP_INST_PER_PARTICLE,
                                   "warp_instructions_per_launch": WARP_INST_PER_PARTICLE * n_avg,
                                   "issue_active_pct": ISSUE_ACTIVE_PCT,
                                   "source": "ncu capture of the first 512 replicas (768 threads), scaled by particles"}},
            "cpu_baseline": cpu,
            "clocks": clocks.summary(),
            "gpu_launches": 2 * args.steps,
            "serving": served,
            "single_systems": singles,
        }
    return result


def run_reference(args):
    """The reference arm: the reference path on the host cores (reference_cpu), on this arm's config,
    metric and unit."""
    ns, boxes, pos, types = ensemble(args.seed, args.replicas)
    v, n_run, cpu = reference_cpu(ns, boxes, pos, types, args.seed, args.steps, args.warmup, args.cpu_seconds)
    ms = n_run / v * 1e3  # one step of every sampled replica
    return {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded uneven ensemble)", "impl": "reference",
            "config": {"workload": "batched uneven ensemble: 4096 replicas of A+B<->C, N log-uniform in [200, 20000], "
                                   "density 0.25, HR k=10 d=1, Gillespie, dt=1e-3",
                       "sample": cpu["sample"]},
            "cpu_baseline": cpu,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ---- minimal distributed helpers (torch.distributed only when launched with several ranks) ----
_dist = None


_dist_device = "cpu"


def rank_seed(seed: int, rank: int) -> int:
    """Seed of a rank's ensemble: every rank advances its own, disjoint set of replicas."""
    return seed + 1000003 * rank


def init_dist():
    """One process per GPU under torchrun (NCCL); gloo on machines without CUDA.  The only collectives
    are the barrier around the timed region and the reductions of its time (max) and particle-steps
    (sum): replicas are independent, so the data path has no exchange."""
    global _dist, _dist_device
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
            dist.init_process_group("nccl")
            _dist_device = "cuda"
        else:
            dist.init_process_group("gloo")
            _dist_device = "cpu"
        _dist = dist
    return rank, world


def barrier(world):
    if world > 1 and _dist is not None:
        _dist.barrier()


def _allreduce(v, world, op):
    if world <= 1 or _dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64, device=_dist_device)
    _dist.all_reduce(t, op=op)
    return float(t.item())


def allreduce_max(v, world):
    return _allreduce(v, world, _dist.ReduceOp.MAX if _dist else None)


def allreduce_sum(v, world):
    return _allreduce(v, world, _dist.ReduceOp.SUM if _dist else None)


def main():
    args = parse()
    rank, world = init_dist()
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)), flush=True)
        return
    if args.profile_system:
        if rank == 0:
            print(json.dumps(profile_system(args.profile_system, args.warmup, args.steps)), flush=True)
        return
    if world > 1:
        # the library creates its streams and buffers on the rank's own GPU
        from readdy_gb300 import _native
        _native.check(_native.load().rdc_set_device(int(os.environ.get("LOCAL_RANK", "0"))))
    res = run_gb300(args, rank, world)
    if rank == 0 and res is not None:
        print(json.dumps(res), flush=True)
    if world > 1 and _dist is not None:
        _dist.destroy_process_group()


if __name__ == "__main__":
    main()
