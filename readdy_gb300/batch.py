"""Batched replicas: thousands of independent copies of one Context advanced by one fused launch per
step (rdc_batch_* in include/readdy_cuda.h), and the autotuner that picks its launch knobs.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import _native as N
from .kernel import Context

_M64 = (1 << 64) - 1


def _splitmix64(x: int) -> int:
    x = (x + 0x9E3779B97F4A7C15) & _M64
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & _M64
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & _M64
    return x ^ (x >> 31)


def replica_seed(seed: int, replica: int) -> int:
    """Seed of replica `replica` inside a batch created with `seed`; a CUDAKernel created with this
    seed runs the same random streams as that replica."""
    return _splitmix64((seed ^ ((0x5DEECE66D * (replica + 1)) & _M64)) & _M64)


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class ReplicaBatch:
    def __init__(self, context: Context, boxes, capacities, seed: int = 0):
        self._lib = N.load()
        self.context = context
        boxes = np.ascontiguousarray(boxes, dtype=np.float64).reshape(-1, 3)
        caps = np.ascontiguousarray(capacities, dtype=np.int64)
        assert len(caps) == len(boxes)
        self.n_replicas = len(boxes)
        h = C.c_void_p()
        N.check(self._lib.rdc_batch_create(C.byref(h), context.handle, self.n_replicas, _p(boxes, C.c_double),
                                           _p(caps, C.c_int64), int(seed) & _M64))
        self._h = h
        self.seed = seed
        self.boxes = boxes
        self.capacities = caps

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.rdc_batch_destroy(h)
            self._h = None

    def set_particles(self, positions_per_replica, types_per_replica):
        """Initial particles, one (n, 3) position array and one type array per replica; the arrays are
        read where they lie (no concatenated copy)."""
        if len(positions_per_replica) != self.n_replicas or len(types_per_replica) != self.n_replicas:
            raise ValueError("one position and one type array per replica")
        pos = [np.ascontiguousarray(np.asarray(p, np.float64).reshape(-1, 3)) for p in positions_per_replica]
        types = [np.ascontiguousarray(np.asarray(t, np.int32).reshape(-1)) for t in types_per_replica]
        counts = np.array([len(p) for p in pos], np.int64)
        if any(len(t) != len(p) for p, t in zip(pos, types)):
            raise ValueError("positions and types differ in length")
        pp = (C.c_void_p * self.n_replicas)(*[p.ctypes.data for p in pos])
        tp = (C.c_void_p * self.n_replicas)(*[t.ctypes.data for t in types])
        N.check(self._lib.rdc_batch_set_particles_list(self._h, _p(counts, C.c_int64), C.cast(pp, C.c_void_p),
                                                       C.cast(tp, C.c_void_p)))

    def configure(self, handler=N.GILLESPIE, dt=1e-3, cell_width_scale=1.0, threads_per_block=256):
        N.check(self._lib.rdc_batch_configure(self._h, int(handler), float(dt), float(cell_width_scale),
                                              int(threads_per_block)))
        self.handler, self.dt = handler, dt
        self.cell_width_scale, self.threads_per_block = cell_width_scale, threads_per_block

    def set_carry_forces(self, on=True):
        """Pair forces carried from each step's event walk to the next step (default) or summed at
        the start of every step; the trajectories are bitwise the same."""
        N.check(self._lib.rdc_batch_set_carry_forces(self._h, 1 if on else 0))

    def step(self, n_steps=1):
        N.check(self._lib.rdc_batch_step(self._h, int(n_steps)))

    def step_timed(self, n_steps=1):
        """Advances n_steps and returns the device time in ms (CUDA events on the batch's stream)."""
        ms = C.c_double()
        N.check(self._lib.rdc_batch_step_timed(self._h, int(n_steps), C.byref(ms)))
        return ms.value

    def particle_steps(self):
        v = C.c_uint64()
        N.check(self._lib.rdc_batch_particle_steps(self._h, C.byref(v)))
        return int(v.value)

    def synchronize(self):
        N.check(self._lib.rdc_batch_synchronize(self._h))

    def count_types(self):
        out = np.zeros((self.n_replicas, self.context.n_types), np.int64)
        N.check(self._lib.rdc_batch_count_types(self._h, _p(out, C.c_int64)))
        return out

    def n_particles(self):
        out = np.zeros(self.n_replicas, np.int64)
        N.check(self._lib.rdc_batch_n_particles(self._h, _p(out, C.c_int64)))
        return out

    def get_forces(self, replica):
        """(forces (n, 3), ids) of one replica's live particles, in the order of get_particles: the force
        its next step applies (pair forces carried or summed, plus order-1 potentials)."""
        n = int(self.n_particles()[replica])
        f = np.zeros((n, 3)); ids = np.zeros(n, np.uint64)
        got = C.c_int64()
        N.check(self._lib.rdc_batch_get_forces(self._h, int(replica), n, _p(f, C.c_double), _p(ids, C.c_uint64),
                                               C.byref(got)))
        return f[:got.value], ids[:got.value]

    def record_counts(self, stride: int, max_records: int):
        """From now on every replica records its per-type counts every `stride` steps (record 0 now)."""
        N.check(self._lib.rdc_batch_record_counts(self._h, int(stride), int(max_records)))
        self._max_records = int(max_records)

    def poll_count_records(self):
        """(steps (k,), counts (k, n_replicas, n_types)) of the records written since the last poll."""
        cap = getattr(self, "_max_records", 0)
        steps = np.zeros(max(cap, 1), np.int64)
        counts = np.zeros((max(cap, 1), self.n_replicas, self.context.n_types), np.int64)
        n = C.c_int64()
        N.check(self._lib.rdc_batch_poll_count_records(self._h, cap, _p(steps, C.c_int64), _p(counts, C.c_int64),
                                                       C.byref(n)))
        return steps[:n.value], counts[:n.value]

    def record_trajectory(self, replicas, stride: int, max_frames: int):
        """From now on a frame of the given replicas' particles is taken every `stride` steps (frame 0 now),
        up to max_frames frames kept on the device until polled; replicas=[] switches it off."""
        sel = np.ascontiguousarray(replicas, dtype=np.int32).reshape(-1)
        N.check(self._lib.rdc_batch_record_trajectory(self._h, len(sel), _p(sel, C.c_int), int(stride),
                                                      int(max_frames)))
        self._traj_sel = sel.copy()
        self._traj_max = int(max_frames)

    def poll_trajectory(self):
        """The frames taken since the last poll: (steps (f,), frames) with frames[f][k] = (positions (n, 3),
        types (n,), ids (n,)) of the k-th recorded replica."""
        sel = getattr(self, "_traj_sel", np.zeros(0, np.int32))
        nf_cap = max(getattr(self, "_traj_max", 0), 1)
        cap = int(self.capacities[sel].sum()) * nf_cap if len(sel) else 1
        steps = np.zeros(nf_cap, np.int64)
        counts = np.zeros((nf_cap, max(len(sel), 1)), np.int64)
        pos = np.zeros((cap, 3)); types = np.zeros(cap, np.int32); ids = np.zeros(cap, np.uint64)
        nf, ne = C.c_int64(), C.c_int64()
        N.check(self._lib.rdc_batch_poll_trajectory(self._h, nf_cap, cap, _p(steps, C.c_int64), _p(counts, C.c_int64),
                                                    _p(pos, C.c_double), _p(types, C.c_int), _p(ids, C.c_uint64),
                                                    C.byref(nf), C.byref(ne)))
        frames, at = [], 0
        for f in range(nf.value):
            per = []
            for k in range(len(sel)):
                c = int(counts[f, k])
                per.append((pos[at:at + c], types[at:at + c], ids[at:at + c]))
                at += c
            frames.append(per)
        return steps[:nf.value], frames

    def virial(self):
        """Pair virial of every replica's current state, (n_replicas, 3, 3); needs carried forces off."""
        out = np.zeros((self.n_replicas, 3, 3))
        N.check(self._lib.rdc_batch_get_virial(self._h, _p(out, C.c_double)))
        return out

    def reaction_counts(self):
        """Performed events per replica and reaction id, (n_replicas, n_reactions)."""
        n = self.context.n_reactions
        out = np.zeros((self.n_replicas, max(n, 1)), np.int64)
        N.check(self._lib.rdc_batch_reaction_counts(self._h, n, _p(out, C.c_int64)))
        return out[:, :n]

    def replica_grid(self, replica):
        """(cells per axis, cell starts in shared memory during a step) of one replica."""
        dims = np.zeros(3, np.int32)
        sh = C.c_int()
        N.check(self._lib.rdc_batch_replica_grid(self._h, int(replica), _p(dims, C.c_int), C.byref(sh)))
        return tuple(int(x) for x in dims), bool(sh.value)

    def get_particles(self, replica):
        n = int(self.n_particles()[replica])
        pos = np.zeros((n, 3)); t = np.zeros(n, np.int32); ids = np.zeros(n, np.uint64)
        got = C.c_int64()
        N.check(self._lib.rdc_batch_get_particles(self._h, int(replica), n, _p(pos, C.c_double), _p(t, C.c_int),
                                                  _p(ids, C.c_uint64), C.byref(got)))
        return pos[:got.value], t[:got.value], ids[:got.value]


def autotune(make_batch, steps=20, scales=(1.0, 1.5, 2.0), threads=(512, 768), handler=N.GILLESPIE, dt=1e-3):
    """Times short runs of freshly made batches over cell width scale x threads per block and returns
    the fastest setting as a dict.  `make_batch()` must return a batch with its particles set."""
    best = None
    for r in scales:
        for t in threads:
            b = make_batch()
            b.configure(handler=handler, dt=dt, cell_width_scale=r, threads_per_block=t)
            b.step(2)
            b.synchronize()
            t0 = time.perf_counter()
            b.step(steps)
            b.synchronize()
            dtm = (time.perf_counter() - t0) / steps
            if best is None or dtm < best["s_per_step"]:
                best = dict(cell_width_scale=r, threads_per_block=t, s_per_step=dtm)
            del b
    return best


def autotune_inplace(batch: ReplicaBatch, scales=(1.0, 1.15, 1.3), threads=(512, 640, 768), steps=5,
                     handler=N.GILLESPIE, dt=1e-3):
    """Autotunes a batch on its own replicas: for every cell width scale x threads per block it
    reconfigures the batch, runs two untimed steps and `steps` steps timed with CUDA events on the
    batch's stream, then leaves the batch configured with the fastest setting.  The replicas advance
    by all these steps.  Returns the fastest setting and the table of timings (ms per step)."""
    table = []
    for r in scales:
        for t in threads:
            batch.configure(handler=handler, dt=dt, cell_width_scale=r, threads_per_block=t)
            batch.step(2)
            table.append(dict(cell_width_scale=r, threads_per_block=t, ms_per_step=batch.step_timed(steps) / steps))
    best = min(table, key=lambda x: x["ms_per_step"])
    batch.configure(handler=handler, dt=dt, cell_width_scale=best["cell_width_scale"],
                    threads_per_block=best["threads_per_block"])
    return best, table
