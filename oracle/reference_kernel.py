"""TEST INFRASTRUCTURE ONLY: ctypes front end of oracle/_ref/libreaddy_ref.so, the reference's own pthread
CPU kernel built by oracle/ref_build.py (see there).  Used to cross-check the oracle restatement against
the reference itself and as the CPU baseline of bench.py; never on the product path."""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np

from . import ref_build

UNCONTROLLED_APPROXIMATION = 0
GILLESPIE = 1

_lib = None
_lock = threading.Lock()


def available() -> bool:
    return ref_build.build() is not None


def _load():
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = ref_build.build()
        if path is None:
            raise RuntimeError("reference CPU kernel unavailable: " + str(ref_build.unavailable_reason()))
        lib = C.CDLL(path)
        d, i, i64, vp = C.c_double, C.c_int, C.c_int64, C.c_void_p
        P = C.POINTER
        lib.refk_last_error.restype = C.c_char_p
        lib.refk_create.restype = vp
        lib.refk_create.argtypes = [P(d), P(i), d, i, P(d), i]
        lib.refk_destroy.argtypes = [vp]
        for name, args in [("refk_add_harmonic_repulsion", [vp, i, i, d, d]),
                           ("refk_add_weak_interaction_piecewise_harmonic", [vp, i, i, d, d, d, d]),
                           ("refk_add_lennard_jones", [vp, i, i, C.c_uint, C.c_uint, d, i, d, d]),
                           ("refk_add_fusion", [vp, i, i, i, d, d]),
                           ("refk_add_fission", [vp, i, i, i, d, d]),
                           ("refk_add_particles", [vp, i64, vp, vp]),
                           ("refk_calculate_forces", [vp, i64, vp, vp, P(i64), P(d)]),
                           ("refk_run", [vp, i64, d, i, vp, P(d)])]:
            f = getattr(lib, name)
            f.restype = i
            f.argtypes = args
        _lib = lib
        return lib


class ReferenceKernel:
    """One readdy::kernel::cpu::CPUKernel with species T0..T{n-1}."""

    def __init__(self, box, periodic=(True, True, True), kbt=1.0, diffusion=(1.0,), n_threads=0):
        self._lib = _load()
        b = (C.c_double * 3)(*box)
        p = (C.c_int * 3)(*[int(bool(x)) for x in periodic])
        D = (C.c_double * len(diffusion))(*diffusion)
        self.n_types = len(diffusion)
        self._h = self._lib.refk_create(b, p, float(kbt), len(diffusion), D, int(n_threads))
        if not self._h:
            raise RuntimeError(self._lib.refk_last_error().decode())

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.refk_destroy(h)
            self._h = None

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(self._lib.refk_last_error().decode())

    def add_harmonic_repulsion(self, t1, t2, k, d):
        self._check(self._lib.refk_add_harmonic_repulsion(self._h, t1, t2, k, d))

    def add_weak_interaction_piecewise_harmonic(self, t1, t2, k, desired, depth, cutoff):
        self._check(self._lib.refk_add_weak_interaction_piecewise_harmonic(self._h, t1, t2, k, desired, depth, cutoff))

    def add_lennard_jones(self, t1, t2, m, n, cutoff, shift, epsilon, sigma):
        self._check(self._lib.refk_add_lennard_jones(self._h, t1, t2, m, n, cutoff, int(bool(shift)), epsilon, sigma))

    def add_fusion(self, a, b, c, rate, educt_distance):
        self._check(self._lib.refk_add_fusion(self._h, a, b, c, rate, educt_distance))

    def add_fission(self, a, b, c, rate, product_distance):
        self._check(self._lib.refk_add_fission(self._h, a, b, c, rate, product_distance))

    def add_particles(self, positions, types):
        pos = np.ascontiguousarray(positions, np.float64).reshape(-1, 3)
        t = np.ascontiguousarray(types, np.int32)
        self._check(self._lib.refk_add_particles(self._h, len(pos), pos.ctypes.data, t.ctypes.data))

    def calculate_forces(self, n_particles):
        """(ids, forces (n, 3), energy) of the reference's CalculateForces on the current particles."""
        ids = np.zeros(n_particles, np.uint64)
        f = np.zeros((n_particles, 3))
        n = C.c_int64()
        e = C.c_double()
        self._check(self._lib.refk_calculate_forces(self._h, n_particles, ids.ctypes.data, f.ctypes.data,
                                                    C.byref(n), C.byref(e)))
        return ids[:n.value], f[:n.value], e.value

    def run(self, n_steps, dt, handler=GILLESPIE):
        """SimulationLoop::run(n_steps); returns (final per-type counts, wall seconds of the loop)."""
        counts = np.zeros(self.n_types, np.int64)
        sec = C.c_double()
        self._check(self._lib.refk_run(self._h, int(n_steps), float(dt), int(handler), counts.ctypes.data,
                                       C.byref(sec)))
        return counts, sec.value
