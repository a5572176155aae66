"""TEST INFRASTRUCTURE ONLY -- the FP64 CPU oracle for the ReaDDy hot path.

ctypes front end of ``readdy_oracle.cpp``, an FP64 restatement of ReaDDy's CPU kernel
(kernels/cpu/src: cell-linked list, forces, Euler BD, uncontrolled approximation, Gillespie).
Only the tests, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of ``bench.py`` may
use it, and only as the checker; the product path never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libreaddy_oracle.so")
_lib = None
_lock = threading.Lock()

UNCONTROLLED_APPROXIMATION = 0
GILLESPIE = 1


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++, a few seconds; make skips an up-to-date library)."""
    subprocess.run(["make", "-s", "-C", _HERE] + (["-B"] if force else []), check=True)
    return _LIB_PATH


def _load():
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        build()
        lib = C.CDLL(_LIB_PATH)
        d, i, u64, vp = C.c_double, C.c_int, C.c_uint64, C.c_void_p
        i64 = C.c_int64
        P = C.POINTER
        sig = {
            "orc_create": (vp, [P(d), P(i), d, i, P(d), u64, i, i]),
            "orc_destroy": (None, [vp]),
            "orc_last_error": (C.c_char_p, []),
            "orc_set_record_virial": (i, [vp, i]),
            "orc_get_virial": (i, [vp, P(d)]),
            "orc_add_box": (i, [vp, i, d, P(d), P(d), i]),
            "orc_add_sphere": (i, [vp, i, d, P(d), d, i]),
            "orc_add_capsule": (i, [vp, i, d, P(d), P(d), d, d, i]),
            "orc_add_spherical_barrier": (i, [vp, i, d, d, P(d), d]),
            "orc_add_cylinder": (i, [vp, i, d, P(d), P(d), d, i]),
            "orc_add_harmonic_repulsion": (i, [vp, i, i, d, d]),
            "orc_add_weak_interaction_piecewise_harmonic": (i, [vp, i, i, d, d, d, d]),
            "orc_add_lennard_jones": (i, [vp, i, i, C.c_uint, C.c_uint, d, i, d, d]),
            "orc_add_screened_electrostatics": (i, [vp, i, i, d, d, d, d, C.c_uint, d]),
            "orc_add_conversion": (i, [vp, i, i, d]),
            "orc_add_decay": (i, [vp, i, d]),
            "orc_add_fusion": (i, [vp, i, i, i, d, d, d, d]),
            "orc_add_fission": (i, [vp, i, i, i, d, d, d, d]),
            "orc_add_enzymatic": (i, [vp, i, i, i, d, d]),
            "orc_add_harmonic_bonds": (i, [vp, i, P(i), P(d), P(d)]),
            "orc_add_harmonic_angles": (i, [vp, i, P(i), P(d), P(d)]),
            "orc_add_cosine_dihedrals": (i, [vp, i, P(i), P(d), P(d), P(d)]),
            "orc_set_particle_flavor": (i, [vp, i, i]),
            "orc_configure_harmonic_bond": (i, [vp, i, i, d, d]),
            "orc_configure_harmonic_angle": (i, [vp, i, i, i, d, d]),
            "orc_configure_cosine_dihedral": (i, [vp, i, i, i, i, d, d, d]),
            "orc_add_topology": (i, [vp, i, i, P(d), P(i), i, P(i), P(u64)]),
            "orc_break_bonds": (i, [vp, d, i, P(i), P(i), P(d), P(d), P(i64)]),
            "orc_get_topologies": (i, [vp, P(i), P(i64), P(u64), P(i64), P(i64)]),
            "orc_get_topology_edges": (i, [vp, P(i64), P(u64), P(i64)]),
            "orc_add_spatial_topology_reaction": (i, [vp, i, i, i, i, i, i, i, i, i, d, d, i]),
            "orc_set_legacy_topology_self_fusion": (i, [vp, i]),
            "orc_evaluate_topology_reactions": (i, [vp, d, P(i64)]),
            "orc_topology_reaction_counts": (i, [vp, P(i64), i]),
            "orc_add_structural_topology_reaction": (i, [vp, i, RATE_FN, RECIPE_FN, vp, i]),
            "orc_set_spatial_topology_rate_function": (i, [vp, i, SPATIAL_RATE_FN, vp]),
            "orc_structural_reaction_counts": (i, [vp, P(i64), i]),
            "orc_recipe_change_particle_type": (i, [vp, i64, i]),
            "orc_recipe_add_edge": (i, [vp, i64, i64]),
            "orc_recipe_remove_edge": (i, [vp, i64, i64]),
            "orc_recipe_separate_vertex": (i, [vp, i64]),
            "orc_recipe_change_topology_type": (i, [vp, i]),
            "orc_recipe_append_particle": (i, [vp, i64, P(i64), i, P(d)]),
            "orc_recipe_change_particle_position": (i, [vp, i64, P(d)]),
            "orc_get_topology": (i, [vp, i64, P(i), P(u64), P(i), P(d), P(i64), P(i64), P(i64)]),
            "orc_add_particles": (i, [vp, i, P(d), P(i)]),
            "orc_n_particles": (i, [vp]),
            "orc_n_entries": (i, [vp]),
            "orc_get_particles": (i, [vp, P(d), P(i), P(u64), P(d), P(i)]),
            "orc_calculate_max_cutoff": (d, [vp]),
            "orc_get_force_scales": (i, [vp, P(d)]),
            "orc_nl_setup": (i, [vp, d]),
            "orc_nl_update": (i, [vp]),
            "orc_nl_pairs": (i64, [vp, d, i64, P(u64)]),
            "orc_brute_force_pairs": (i64, [vp, d, i64, P(u64)]),
            "orc_calculate_forces": (d, [vp]),
            "orc_energy": (d, [vp]),
            "orc_euler_bd": (i, [vp, d]),
            "orc_uncontrolled_approximation": (i, [vp, d]),
            "orc_gillespie": (i, [vp, d]),
            "orc_run": (i, [vp, i64, d, i, i, P(i64), i64]),
            "orc_reaction_counts": (i, [vp, P(i64), i]),
            "orc_histogram_along_axis": (i, [vp, i, P(d), i, P(i), i, P(d)]),
            "orc_radial_distribution": (i, [vp, i, P(d), i, P(i), i, P(i), d, P(d), P(d)]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
        return lib


RATE_FN = C.CFUNCTYPE(C.c_double, C.c_void_p, C.c_void_p, C.c_int64)
SPATIAL_RATE_FN = C.CFUNCTYPE(C.c_double, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64)
RECIPE_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p)


class TopologyView:
    """One oracle topology as structural reaction functions see it: index, type, ids, types and positions by
    local vertex, edges as local vertex pairs."""

    def __init__(self, lib, h, index):
        self.index = int(index)
        tt, nv, ne = C.c_int(), C.c_int64(), C.c_int64()
        lib.orc_get_topology(h, self.index, C.byref(tt), None, None, None, C.byref(nv), None, C.byref(ne))
        self.type = tt.value
        self.ids = np.zeros(nv.value, np.uint64)
        self.types = np.zeros(nv.value, np.int32)
        self.positions = np.zeros((nv.value, 3))
        self.edges = np.zeros((ne.value, 2), np.int64)
        lib.orc_get_topology(h, self.index, None, _ptr(self.ids, C.c_uint64), _ptr(self.types, C.c_int),
                             _ptr(self.positions, C.c_double), C.byref(nv), _ptr(self.edges, C.c_int64), C.byref(ne))

    @property
    def n_particles(self):
        return len(self.ids)


def _ptr(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


class OracleSystem:
    """One FP64 CPU system with the reference's CPU-kernel semantics."""

    def __init__(self, box, periodic=(True, True, True), kbt=1.0, diffusion=(1.0,), seed=0,
                 n_threads=1, cll_radius=1):
        self._lib = _load()
        b = np.ascontiguousarray(box, dtype=np.float64)
        p = np.ascontiguousarray([int(bool(x)) for x in periodic], dtype=np.int32)
        D = np.ascontiguousarray(diffusion, dtype=np.float64)
        self.n_types = len(D)
        self._h = self._lib.orc_create(_ptr(b, C.c_double), _ptr(p, C.c_int), float(kbt), self.n_types,
                                       _ptr(D, C.c_double), int(seed) & (2**64 - 1), int(n_threads),
                                       int(cll_radius))
        if not self._h:
            raise ValueError(self._lib.orc_last_error().decode())

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.orc_destroy(h)
            self._h = None

    def _check(self, rc):
        if rc < 0:
            raise RuntimeError(self._lib.orc_last_error().decode())
        return rc

    def set_record_virial(self, record=True):
        self._lib.orc_set_record_virial(self._h, int(bool(record)))

    def virial(self):
        out = np.zeros(9)
        self._lib.orc_get_virial(self._h, _ptr(out, C.c_double))
        return out.reshape(3, 3)

    # order-1 (external) potentials
    @staticmethod
    def _v3(v):
        return np.ascontiguousarray(v, dtype=np.float64).reshape(3)

    def add_box(self, t, force_constant, origin, extent, inclusion=True):
        o, e = self._v3(origin), self._v3(extent)
        return self._check(self._lib.orc_add_box(self._h, t, force_constant, _ptr(o, C.c_double),
                                                 _ptr(e, C.c_double), int(bool(inclusion))))

    def add_sphere(self, t, force_constant, origin, radius, inclusion):
        o = self._v3(origin)
        return self._check(self._lib.orc_add_sphere(self._h, t, force_constant, _ptr(o, C.c_double), radius,
                                                    int(bool(inclusion))))

    def add_capsule(self, t, force_constant, center, direction, length, radius, inclusion=True):
        c, v = self._v3(center), self._v3(direction)
        return self._check(self._lib.orc_add_capsule(self._h, t, force_constant, _ptr(c, C.c_double),
                                                     _ptr(v, C.c_double), length, radius, int(bool(inclusion))))

    def add_spherical_barrier(self, t, height, width, origin, radius):
        o = self._v3(origin)
        return self._check(self._lib.orc_add_spherical_barrier(self._h, t, height, width, _ptr(o, C.c_double),
                                                               radius))

    def add_cylinder(self, t, force_constant, origin, normal, radius, inclusion):
        o, n = self._v3(origin), self._v3(normal)
        return self._check(self._lib.orc_add_cylinder(self._h, t, force_constant, _ptr(o, C.c_double),
                                                      _ptr(n, C.c_double), radius, int(bool(inclusion))))

    # potentials
    def add_harmonic_repulsion(self, t1, t2, k, d):
        return self._check(self._lib.orc_add_harmonic_repulsion(self._h, t1, t2, k, d))

    def add_weak_interaction_piecewise_harmonic(self, t1, t2, k, desired, depth, cutoff):
        return self._check(self._lib.orc_add_weak_interaction_piecewise_harmonic(self._h, t1, t2, k, desired,
                                                                                 depth, cutoff))

    def add_lennard_jones(self, t1, t2, m, n, cutoff, shift, epsilon, sigma):
        return self._check(self._lib.orc_add_lennard_jones(self._h, t1, t2, m, n, cutoff, int(shift),
                                                           epsilon, sigma))

    def add_screened_electrostatics(self, t1, t2, C_, kappa, D_, sigma, exponent, cutoff):
        return self._check(self._lib.orc_add_screened_electrostatics(self._h, t1, t2, C_, kappa, D_, sigma,
                                                                     exponent, cutoff))

    # reactions
    def add_conversion(self, a, b, rate):
        return self._check(self._lib.orc_add_conversion(self._h, a, b, rate))

    def add_decay(self, a, rate):
        return self._check(self._lib.orc_add_decay(self._h, a, rate))

    def add_fusion(self, a, b, c, rate, educt_distance, w1=0.5, w2=0.5):
        return self._check(self._lib.orc_add_fusion(self._h, a, b, c, rate, educt_distance, w1, w2))

    def add_fission(self, a, b, c, rate, product_distance, w1=0.5, w2=0.5):
        return self._check(self._lib.orc_add_fission(self._h, a, b, c, rate, product_distance, w1, w2))

    def add_enzymatic(self, catalyst, a, b, rate, educt_distance):
        return self._check(self._lib.orc_add_enzymatic(self._h, catalyst, a, b, rate, educt_distance))

    # bonded
    def add_harmonic_bonds(self, idx, k, l0):
        idx = np.ascontiguousarray(idx, dtype=np.int32).reshape(-1, 2)
        n = len(idx)
        k = np.ascontiguousarray(np.broadcast_to(k, (n,)), dtype=np.float64)
        l0 = np.ascontiguousarray(np.broadcast_to(l0, (n,)), dtype=np.float64)
        return self._check(self._lib.orc_add_harmonic_bonds(self._h, n, _ptr(idx, C.c_int), _ptr(k, C.c_double),
                                                            _ptr(l0, C.c_double)))

    def add_harmonic_angles(self, idx, k, theta0):
        idx = np.ascontiguousarray(idx, dtype=np.int32).reshape(-1, 3)
        n = len(idx)
        k = np.ascontiguousarray(np.broadcast_to(k, (n,)), dtype=np.float64)
        t = np.ascontiguousarray(np.broadcast_to(theta0, (n,)), dtype=np.float64)
        return self._check(self._lib.orc_add_harmonic_angles(self._h, n, _ptr(idx, C.c_int), _ptr(k, C.c_double),
                                                             _ptr(t, C.c_double)))

    def add_cosine_dihedrals(self, idx, k, multiplicity, phi0):
        idx = np.ascontiguousarray(idx, dtype=np.int32).reshape(-1, 4)
        n = len(idx)
        k = np.ascontiguousarray(np.broadcast_to(k, (n,)), dtype=np.float64)
        m = np.ascontiguousarray(np.broadcast_to(multiplicity, (n,)), dtype=np.float64)
        p = np.ascontiguousarray(np.broadcast_to(phi0, (n,)), dtype=np.float64)
        return self._check(self._lib.orc_add_cosine_dihedrals(self._h, n, _ptr(idx, C.c_int), _ptr(k, C.c_double),
                                                              _ptr(m, C.c_double), _ptr(p, C.c_double)))

    # topology registry, flavors, topologies, BreakBonds
    def set_particle_flavor(self, t, flavor):
        return self._check(self._lib.orc_set_particle_flavor(self._h, t, flavor))

    def configure_harmonic_bond(self, t1, t2, k, l0):
        return self._check(self._lib.orc_configure_harmonic_bond(self._h, t1, t2, k, l0))

    def configure_harmonic_angle(self, t1, t2, t3, k, theta0):
        return self._check(self._lib.orc_configure_harmonic_angle(self._h, t1, t2, t3, k, theta0))

    def configure_cosine_dihedral(self, t1, t2, t3, t4, k, multiplicity, phi0):
        return self._check(self._lib.orc_configure_cosine_dihedral(self._h, t1, t2, t3, t4, k, multiplicity, phi0))

    def add_topology(self, positions, types, edges, topology_type=0):
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        t = np.ascontiguousarray(np.broadcast_to(types, (len(pos),)), dtype=np.int32)
        e = np.ascontiguousarray(np.asarray(edges, dtype=np.int32).reshape(-1, 2))
        ids = np.zeros(len(pos), np.uint64)
        self._check(self._lib.orc_add_topology(self._h, topology_type, len(pos), _ptr(pos, C.c_double),
                                               _ptr(t, C.c_int), len(e), _ptr(e, C.c_int), _ptr(ids, C.c_uint64)))
        return ids

    def break_bonds(self, dt, breakable_pairs):
        pairs = list(breakable_pairs)
        t1 = np.ascontiguousarray([p[0] for p in pairs], dtype=np.int32)
        t2 = np.ascontiguousarray([p[1] for p in pairs], dtype=np.int32)
        thr = np.ascontiguousarray([p[2] for p in pairs], dtype=np.float64)
        rate = np.ascontiguousarray([p[3] for p in pairs], dtype=np.float64)
        nb = C.c_int64()
        self._check(self._lib.orc_break_bonds(self._h, dt, len(pairs), _ptr(t1, C.c_int), _ptr(t2, C.c_int),
                                              _ptr(thr, C.c_double), _ptr(rate, C.c_double), C.byref(nb)))
        return nb.value

    def add_spatial_topology_reaction(self, mode, educt1, educt2, product1, product2, rate, radius,
                                      min_graph_distance=0):
        tt2 = -1 if educt2[1] is None else int(educt2[1])
        tto2 = -1 if product2[1] is None else int(product2[1])
        self._n_spatial = getattr(self, "_n_spatial", 0) + 1
        rid = self._check(self._lib.orc_add_spatial_topology_reaction(
            self._h, mode, educt1[0], educt1[1], educt2[0], tt2, product1[0], product1[1], product2[0], tto2,
            1.0 if callable(rate) else rate, radius, min_graph_distance))
        if callable(rate):  # rate(view1, view2) of the two topologies
            lib, h = self._lib, self._h

            def rate_cb(_u, _s, g1, g2):
                try:
                    return float(rate(TopologyView(lib, h, g1), TopologyView(lib, h, g2)))
                except BaseException as e:
                    self._callback_error = getattr(self, "_callback_error", None) or e
                    return float("nan")

            cb = SPATIAL_RATE_FN(rate_cb)
            self._callbacks = getattr(self, "_callbacks", []) + [cb]
            self._check(self._lib.orc_set_spatial_topology_rate_function(self._h, rid, cb, None))
        return rid

    def set_legacy_topology_self_fusion(self, legacy):
        return self._check(self._lib.orc_set_legacy_topology_self_fusion(self._h, int(bool(legacy))))

    def evaluate_topology_reactions(self, dt):
        n = C.c_int64()
        rc = self._lib.orc_evaluate_topology_reactions(self._h, dt, C.byref(n))
        err, self._callback_error = getattr(self, "_callback_error", None), None
        if err is not None:
            raise err
        self._check(rc)
        return n.value

    def topology_reaction_counts(self):
        n = getattr(self, "_n_spatial", 0)
        out = np.zeros(max(n, 1), np.int64)
        self._lib.orc_topology_reaction_counts(self._h, _ptr(out, C.c_int64), n)
        return out[:n]

    def add_structural_topology_reaction(self, topology_type, rate_function, reaction_function,
                                         expect_connected=True):
        lib, h = self._lib, self._h

        def rate_cb(_u, _s, k):
            try:
                return float(rate_function(TopologyView(lib, h, k)))
            except BaseException as e:
                self._callback_error = getattr(self, "_callback_error", None) or e
                return 0.0

        def recipe_cb(_u, _s, k, recipe):
            try:
                for step in reaction_function(TopologyView(lib, h, k)) or ():
                    if step[0] == "append_particle":
                        nb = np.ascontiguousarray(step[1], dtype=np.int64)
                        pos = np.ascontiguousarray(step[3], dtype=np.float64)
                        lib.orc_recipe_append_particle(recipe, len(nb), _ptr(nb, C.c_int64), int(step[2]),
                                                       _ptr(pos, C.c_double))
                    elif step[0] == "change_particle_position":
                        pos = np.ascontiguousarray(step[2], dtype=np.float64)
                        lib.orc_recipe_change_particle_position(recipe, int(step[1]), _ptr(pos, C.c_double))
                    else:
                        getattr(lib, "orc_recipe_" + step[0])(recipe, *[int(a) for a in step[1:]])
            except BaseException as e:
                self._callback_error = getattr(self, "_callback_error", None) or e
                lib.orc_recipe_change_particle_type(recipe, -1, 0)

        cbs = (RATE_FN(rate_cb), RECIPE_FN(recipe_cb))
        self._callbacks = getattr(self, "_callbacks", []) + [cbs]
        self._n_structural = getattr(self, "_n_structural", 0) + 1
        return self._check(lib.orc_add_structural_topology_reaction(h, topology_type, cbs[0], cbs[1], None,
                                                                    int(bool(expect_connected))))

    def structural_reaction_counts(self):
        n = getattr(self, "_n_structural", 0)
        out = np.zeros(max(n, 1), np.int64)
        self._lib.orc_structural_reaction_counts(self._h, _ptr(out, C.c_int64), n)
        return out[:n]

    def topology(self, index):
        return TopologyView(self._lib, self._h, index)

    def topologies(self):
        """[(topology type, particle ids[] uint64)]"""
        nt, ni = C.c_int64(), C.c_int64()
        self._lib.orc_get_topologies(self._h, None, None, None, C.byref(nt), C.byref(ni))
        types = np.zeros(nt.value, np.int32); off = np.zeros(nt.value + 1, np.int64); ids = np.zeros(ni.value, np.uint64)
        self._lib.orc_get_topologies(self._h, _ptr(types, C.c_int), _ptr(off, C.c_int64), _ptr(ids, C.c_uint64),
                                     C.byref(nt), C.byref(ni))
        return [(int(types[k]), ids[off[k]:off[k + 1]]) for k in range(nt.value)]

    def topology_edges(self):
        """[(m, 2) particle-id pairs] per topology, in the order of topologies()"""
        ne = C.c_int64()
        nt = len(self.topologies())
        self._lib.orc_get_topology_edges(self._h, None, None, C.byref(ne))
        off = np.zeros(nt + 1, np.int64); e = np.zeros((ne.value, 2), np.uint64)
        self._lib.orc_get_topology_edges(self._h, _ptr(off, C.c_int64), _ptr(e, C.c_uint64), C.byref(ne))
        return [e[off[k]:off[k + 1]] for k in range(nt)]

    # particles
    def add_particles(self, positions, types):
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        t = np.ascontiguousarray(np.broadcast_to(types, (len(pos),)), dtype=np.int32)
        return self._check(self._lib.orc_add_particles(self._h, len(pos), _ptr(pos, C.c_double),
                                                       _ptr(t, C.c_int)))

    @property
    def n_particles(self):
        return self._lib.orc_n_particles(self._h)

    def particles(self):
        """(positions[n,3], types[n], ids[n], forces[n,3], storage_index[n]) of active particles."""
        n = self.n_particles
        pos = np.zeros((n, 3)); f = np.zeros((n, 3))
        t = np.zeros(n, np.int32); ids = np.zeros(n, np.uint64); si = np.zeros(n, np.int32)
        self._lib.orc_get_particles(self._h, _ptr(pos, C.c_double), _ptr(t, C.c_int), _ptr(ids, C.c_uint64),
                                    _ptr(f, C.c_double), _ptr(si, C.c_int))
        return pos, t, ids, f, si

    def force_scales(self):
        """Per active particle: sum of the magnitudes of its force terms (same order as particles())."""
        out = np.zeros(self.n_particles)
        self._lib.orc_get_force_scales(self._h, _ptr(out, C.c_double))
        return out

    def calculate_max_cutoff(self):
        return self._lib.orc_calculate_max_cutoff(self._h)

    def nl_setup(self, cutoff):
        return self._check(self._lib.orc_nl_setup(self._h, cutoff))

    def nl_update(self):
        return self._check(self._lib.orc_nl_update(self._h))

    def _pairs(self, fn, cutoff):
        cap = max(1024, 64 * self.n_particles)
        while True:
            out = np.zeros((cap, 2), np.uint64)
            n = fn(self._h, cutoff, cap, _ptr(out, C.c_uint64))
            if n >= 0:
                return out[:n].copy()
            cap *= 4

    def nl_pairs(self, cutoff):
        return self._pairs(self._lib.orc_nl_pairs, cutoff)

    def brute_force_pairs(self, cutoff):
        return self._pairs(self._lib.orc_brute_force_pairs, cutoff)

    def calculate_forces(self):
        e = self._lib.orc_calculate_forces(self._h)
        if e != e:
            err = self._lib.orc_last_error().decode()
            if err:
                raise RuntimeError(err)
        return e

    @property
    def energy(self):
        return self._lib.orc_energy(self._h)

    def euler_bd(self, dt):
        return self._check(self._lib.orc_euler_bd(self._h, dt))

    def uncontrolled_approximation(self, dt):
        return self._check(self._lib.orc_uncontrolled_approximation(self._h, dt))

    def gillespie(self, dt):
        return self._check(self._lib.orc_gillespie(self._h, dt))

    def run(self, n_steps, dt, handler=UNCONTROLLED_APPROXIMATION, count_stride=0):
        """SimulationLoop::run; returns per-type counts every count_stride steps (incl. t=0)."""
        nrec = (n_steps // count_stride + 1) if count_stride > 0 else 0
        counts = np.zeros((max(nrec, 1), self.n_types), np.int64)
        r = self._check(self._lib.orc_run(self._h, n_steps, dt, handler, count_stride,
                                          _ptr(counts, C.c_int64), nrec))
        return counts[:r]

    def reaction_counts(self, n):
        out = np.zeros(n, np.int64)
        k = self._lib.orc_reaction_counts(self._h, _ptr(out, C.c_int64), n)
        return out[:k]

    def histogram_along_axis(self, borders, types, axis):
        """HistogramAlongAxis of the CPU kernel (CPUObservables.cpp:85-146); n_borders - 1 counts."""
        b = np.ascontiguousarray(borders, np.float64)
        t = np.ascontiguousarray(types, np.int32)
        out = np.zeros(max(len(b) - 1, 1), np.float64)
        if self._lib.orc_histogram_along_axis(self._h, len(b), _ptr(b, C.c_double), len(t), _ptr(t, C.c_int),
                                              int(axis), _ptr(out, C.c_double)) < 0:
            raise ValueError("need at least two borders and an axis in 0..2")
        return out

    def radial_distribution(self, borders, from_types, to_types, particle_to_density):
        """RadialDistribution (RadialDistribution.cpp:75-128): (counts, distribution)."""
        b = np.ascontiguousarray(borders, np.float64)
        f = np.ascontiguousarray(from_types, np.int32)
        t = np.ascontiguousarray(to_types, np.int32)
        counts = np.zeros(max(len(b) - 1, 1), np.float64)
        dist = np.zeros_like(counts)
        if self._lib.orc_radial_distribution(self._h, len(b), _ptr(b, C.c_double), len(f), _ptr(f, C.c_int), len(t),
                                             _ptr(t, C.c_int), float(particle_to_density), _ptr(counts, C.c_double),
                                             _ptr(dist, C.c_double)) < 0:
            raise ValueError("need at least two borders")
        return counts, dist
