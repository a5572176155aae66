"""The "CUDA" kernel: a ReaDDy model::Kernel over the C ABI.

``Context`` mirrors model::Context (box, periodicity, kBT, species, potential, reaction and topology
registries) and ``CUDAKernel`` mirrors a kernel instance with its state model and action factory
(include/readdy/model/Kernel.h:71-235, StateModel.h:53-118, actions/ActionFactory.h:56-129).
Every method is one call into libreaddy_cuda_core.so; nothing runs on the CPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N

KERNEL_NAME = "CUDA"


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class Context:
    """Physical description of a system (include/readdy/model/Context.h)."""

    def __init__(self, box_size, periodic_boundary_conditions=(True, True, True), kbt=1.0,
                 diffusion_constants=(1.0,)):
        self._lib = N.load()
        box = np.ascontiguousarray(box_size, dtype=np.float64)
        pbc = np.ascontiguousarray([int(bool(x)) for x in periodic_boundary_conditions], dtype=np.int32)
        D = np.ascontiguousarray(diffusion_constants, dtype=np.float64)
        h = C.c_void_p()
        N.check(self._lib.rdc_context_create(C.byref(h), _p(box, C.c_double), _p(pbc, C.c_int), float(kbt),
                                             len(D), _p(D, C.c_double)))
        self._h = h
        self.box_size = tuple(float(np.float32(x)) for x in box)
        self.periodic_boundary_conditions = tuple(bool(x) for x in pbc)
        self.kbt = float(kbt)
        self.diffusion_constants = tuple(float(x) for x in D)
        self.n_types = len(D)
        self.n_reactions = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.rdc_context_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def calculate_max_cutoff(self) -> float:
        c = C.c_double()
        N.check(self._lib.rdc_context_max_cutoff(self._h, C.byref(c)))
        return c.value

    @property
    def record_virial(self) -> bool:
        return getattr(self, "_record_virial", False)

    @record_virial.setter
    def record_virial(self, value: bool):
        N.check(self._lib.rdc_context_set_record_virial(self._h, int(bool(value))))
        self._record_virial = bool(value)

    # particle flavors of ParticleTypeRegistry::add (ParticleTypeRegistry.h:58-63)
    NORMAL, TOPOLOGY, MEMBRANE = 0, 1, 2

    def set_particle_flavor(self, particle_type, flavor):
        """The flavor of a species (NORMAL by default); BreakBonds drops one-particle pieces of NORMAL types
        from the topologies."""
        N.check(self._lib.rdc_context_set_particle_flavor(self._h, particle_type, flavor))

    # TopologyRegistry spatial reactions (SpatialTopologyReaction.h:64-191), modes in STRMode order
    TT_ENZYMATIC, TT_FUSION, TT_FUSION_ALLOW_SELF, TP_ENZYMATIC, TP_FUSION = 0, 1, 2, 3, 4

    def add_spatial_topology_reaction(self, mode, educt1, educt2, product1, product2, rate, radius,
                                      min_graph_distance=0):
        """TopologyRegistry::addSpatialReaction with the parsed descriptor: educt1/product1 are
        (particle type, topology type), educt2/product2 the same or (particle type, None) for a free
        particle (topology-particle modes).  A fusion's result takes product1's topology type; a self
        fusion (TT_FUSION_ALLOW_SELF) needs more than min_graph_distance edges between the two.  rate is a
        number, or for topology-topology modes a function rate(view1, view2) of the TopologyViews of the
        topologies that take the first and second educt, called for every candidate pair at every
        evaluation.  Returns the reaction's index."""
        tt2 = -1 if educt2[1] is None else int(educt2[1])
        tto2 = -1 if product2[1] is None else int(product2[1])
        rid = C.c_int()
        N.check(self._lib.rdc_context_add_spatial_topology_reaction(
            self._h, int(mode), int(educt1[0]), int(educt1[1]), int(educt2[0]), tt2, int(product1[0]),
            int(product1[1]), int(product2[0]), tto2, 1.0 if callable(rate) else float(rate), float(radius),
            int(min_graph_distance), C.byref(rid)))
        self._n_spatial = getattr(self, "_n_spatial", 0) + 1
        if callable(rate):
            lib = self._lib

            def rate_cb(_user, sys, g1, g2):
                try:
                    return float(rate(TopologyView(lib, sys, g1), TopologyView(lib, sys, g2)))
                except BaseException as e:  # reported by the call that ran the function
                    self._callback_error = getattr(self, "_callback_error", None) or e
                    return float("nan")

            cb = N.SPATIAL_RATE_FN(rate_cb)
            self._callbacks = getattr(self, "_callbacks", []) + [cb]
            N.check(lib.rdc_context_set_spatial_topology_rate_function(self._h, rid.value, cb, None))
        return rid.value

    @property
    def n_spatial_topology_reactions(self) -> int:
        return getattr(self, "_n_spatial", 0)

    def set_legacy_topology_self_fusion(self, legacy: bool):
        N.check(self._lib.rdc_context_set_legacy_topology_self_fusion(self._h, int(bool(legacy))))

    # PotentialRegistry
    def add_harmonic_repulsion(self, t1, t2, force_constant, interaction_distance):
        N.check(self._lib.rdc_context_add_harmonic_repulsion(self._h, t1, t2, force_constant, interaction_distance))

    def add_weak_interaction_piecewise_harmonic(self, t1, t2, force_constant, desired_distance, depth,
                                                no_interaction_distance):
        N.check(self._lib.rdc_context_add_weak_interaction_piecewise_harmonic(
            self._h, t1, t2, force_constant, desired_distance, depth, no_interaction_distance))

    def add_lennard_jones(self, t1, t2, m, n, cutoff, shift, epsilon, sigma):
        N.check(self._lib.rdc_context_add_lennard_jones(self._h, t1, t2, m, n, cutoff, int(bool(shift)),
                                                        epsilon, sigma))

    def add_screened_electrostatics(self, t1, t2, electrostatic_strength, inverse_screening_depth,
                                    repulsion_strength, repulsion_distance, exponent, cutoff):
        N.check(self._lib.rdc_context_add_screened_electrostatics(
            self._h, t1, t2, electrostatic_strength, inverse_screening_depth, repulsion_strength,
            repulsion_distance, exponent, cutoff))

    # order-1 (external) potentials, names and argument order of api/registry/potentials.py
    @staticmethod
    def _v3(v):
        return (C.c_double * 3)(*[float(x) for x in v])

    def add_box(self, particle_type, force_constant, origin, extent, inclusion=True):
        N.check(self._lib.rdc_context_add_box(self._h, particle_type, force_constant, self._v3(origin),
                                              self._v3(extent), int(bool(inclusion))))

    def add_sphere(self, particle_type, force_constant, origin, radius, inclusion):
        N.check(self._lib.rdc_context_add_sphere(self._h, particle_type, force_constant, self._v3(origin), radius,
                                                 int(bool(inclusion))))

    def add_capsule(self, particle_type, force_constant, center, direction, length, radius, inclusion=True):
        N.check(self._lib.rdc_context_add_capsule(self._h, particle_type, force_constant, self._v3(center),
                                                  self._v3(direction), length, radius, int(bool(inclusion))))

    def add_spherical_barrier(self, particle_type, height, width, origin, radius):
        N.check(self._lib.rdc_context_add_spherical_barrier(self._h, particle_type, height, width,
                                                            self._v3(origin), radius))

    def add_cylinder(self, particle_type, force_constant, origin, normal, radius, inclusion):
        N.check(self._lib.rdc_context_add_cylinder(self._h, particle_type, force_constant, self._v3(origin),
                                                   self._v3(normal), radius, int(bool(inclusion))))

    # ReactionRegistry
    def _rid(self, rc, rid):
        N.check(rc)
        self.n_reactions = max(self.n_reactions, rid.value + 1)
        return rid.value

    def add_conversion(self, type_from, type_to, rate):
        rid = C.c_int()
        return self._rid(self._lib.rdc_context_add_conversion(self._h, type_from, type_to, rate, C.byref(rid)), rid)

    def add_decay(self, type_from, rate):
        rid = C.c_int()
        return self._rid(self._lib.rdc_context_add_decay(self._h, type_from, rate, C.byref(rid)), rid)

    def add_fusion(self, type_from1, type_from2, type_to, rate, educt_distance, weight1=0.5, weight2=0.5):
        rid = C.c_int()
        return self._rid(self._lib.rdc_context_add_fusion(self._h, type_from1, type_from2, type_to, rate,
                                                          educt_distance, weight1, weight2, C.byref(rid)), rid)

    def add_fission(self, type_from, type_to1, type_to2, rate, product_distance, weight1=0.5, weight2=0.5):
        rid = C.c_int()
        return self._rid(self._lib.rdc_context_add_fission(self._h, type_from, type_to1, type_to2, rate,
                                                           product_distance, weight1, weight2, C.byref(rid)), rid)

    def add_enzymatic(self, type_catalyst, type_from, type_to, rate, educt_distance):
        rid = C.c_int()
        return self._rid(self._lib.rdc_context_add_enzymatic(self._h, type_catalyst, type_from, type_to, rate,
                                                             educt_distance, C.byref(rid)), rid)

    # TopologyRegistry potential configuration
    def configure_harmonic_bond(self, t1, t2, force_constant=1.0, length=1.0):
        N.check(self._lib.rdc_context_configure_harmonic_bond(self._h, t1, t2, force_constant, length))

    def configure_harmonic_angle(self, t1, t2, t3, force_constant=1.0, equilibrium_angle=0.0):
        N.check(self._lib.rdc_context_configure_harmonic_angle(self._h, t1, t2, t3, force_constant,
                                                               equilibrium_angle))

    def configure_cosine_dihedral(self, t1, t2, t3, t4, force_constant=1.0, multiplicity=1, phi0=0.0):
        N.check(self._lib.rdc_context_configure_cosine_dihedral(self._h, t1, t2, t3, t4, force_constant,
                                                                float(multiplicity), phi0))


class TopologyView:
    """One topology as a structural reaction's functions see it (GraphTopology): its index, its type, the ids
    and types of its particles by local vertex, its edges as local vertex pairs, and on request the
    positions."""

    def __init__(self, lib, handle, index):
        self._lib, self._h, self.index = lib, handle, int(index)
        tt, nv, ne = C.c_int(), C.c_int64(), C.c_int64()
        N.check(lib.rdc_get_topology(handle, self.index, C.byref(tt), 0, None, None, C.byref(nv), 0, None,
                                     C.byref(ne)))
        self.type = tt.value
        self.ids = np.zeros(nv.value, np.uint64)
        self.types = np.zeros(nv.value, np.int32)
        edges = np.zeros((ne.value, 2), np.int64)
        N.check(lib.rdc_get_topology(handle, self.index, None, nv.value, _p(self.ids, C.c_uint64),
                                     _p(self.types, C.c_int), C.byref(nv), ne.value, _p(edges, C.c_int64),
                                     C.byref(ne)))
        self.edges = edges

    @property
    def n_particles(self) -> int:
        return len(self.ids)

    @property
    def positions(self):
        out = np.zeros((len(self.ids), 3))
        N.check(self._lib.rdc_get_topology_positions(self._h, self.index, len(self.ids), _p(out, C.c_double)))
        return out


# recipe steps (Recipe.h:74-110) as the reaction function returns them: ("change_particle_type", v, type),
# ("add_edge", v1, v2), ("remove_edge", v1, v2), ("separate_vertex", v), ("change_topology_type", type),
# ("append_particle", [neighbour vertices], type, (x, y, z)), ("change_particle_position", v, (x, y, z))
RECIPE_STEPS = ("change_particle_type", "add_edge", "remove_edge", "separate_vertex", "change_topology_type",
                "append_particle", "change_particle_position")


def _apply_recipe(lib, recipe, steps):
    for step in steps or ():
        name = step[0]
        if name not in RECIPE_STEPS:
            raise ValueError(f"unknown recipe step {name!r}")
        if name == "append_particle":
            nb = np.ascontiguousarray(step[1], dtype=np.int64)
            pos = np.ascontiguousarray(step[3], dtype=np.float64)
            N.check(lib.rdc_recipe_append_particle(recipe, len(nb), _p(nb, C.c_int64), int(step[2]),
                                                   _p(pos, C.c_double)))
        elif name == "change_particle_position":
            pos = np.ascontiguousarray(step[2], dtype=np.float64)
            N.check(lib.rdc_recipe_change_particle_position(recipe, int(step[1]), _p(pos, C.c_double)))
        else:
            N.check(getattr(lib, "rdc_recipe_" + name)(recipe, *[int(a) for a in step[1:]]))


class CUDAKernel:
    """One simulation on the GPU: state model plus the ActionFactory's actions."""

    name = KERNEL_NAME

    def __init__(self, context: Context, seed: int = 0):
        self._lib = N.load()
        self.context = context
        h = C.c_void_p()
        N.check(self._lib.rdc_system_create(C.byref(h), context.handle, int(seed) & (2 ** 64 - 1)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.rdc_system_destroy(h)
            self._h = None

    # ---- StateModel ----
    def add_particles(self, positions, types):
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        t = np.ascontiguousarray(np.broadcast_to(np.asarray(types, dtype=np.int32), (len(pos),)))
        ids = np.zeros(len(pos), np.uint64)
        N.check(self._lib.rdc_add_particles(self._h, len(pos), _p(pos, C.c_double), _p(t, C.c_int),
                                            _p(ids, C.c_uint64)))
        return ids

    def add_topology(self, positions, types, edges, topology_type=0):
        """StateModel::addTopology with the graph's edges (local vertex indices); returns the particle ids."""
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        t = np.ascontiguousarray(np.broadcast_to(np.asarray(types, dtype=np.int32), (len(pos),)))
        e = np.ascontiguousarray(np.asarray(edges, dtype=np.int64).reshape(-1, 2))
        ids = np.zeros(len(pos), np.uint64)
        N.check(self._lib.rdc_add_topology_typed(self._h, int(topology_type), len(pos), _p(pos, C.c_double),
                                                 _p(t, C.c_int), len(e), _p(e, C.c_int64), _p(ids, C.c_uint64)))
        return ids

    def break_bonds(self, time_step, breakable_pairs):
        """BreakBonds (Actions.h:190-290) with a BreakConfig of (type1, type2, threshold_energy, rate)
        entries; returns the number of edges removed."""
        pairs = list(breakable_pairs)
        t1 = np.ascontiguousarray([p[0] for p in pairs], dtype=np.int32)
        t2 = np.ascontiguousarray([p[1] for p in pairs], dtype=np.int32)
        thr = np.ascontiguousarray([p[2] for p in pairs], dtype=np.float64)
        rate = np.ascontiguousarray([p[3] for p in pairs], dtype=np.float64)
        nb = C.c_int64()
        N.check(self._lib.rdc_break_bonds(self._h, float(time_step), len(pairs), _p(t1, C.c_int), _p(t2, C.c_int),
                                          _p(thr, C.c_double), _p(rate, C.c_double), C.byref(nb)))
        return nb.value

    def _check_callbacks(self, rc):
        """Status of a call that may run reaction functions (structural ones of this kernel, spatial rate
        functions of its context): their own exception first."""
        err = getattr(self, "_callback_error", None) or getattr(self.context, "_callback_error", None)
        self._callback_error = None
        self.context._callback_error = None
        if err is not None:
            raise err
        N.check(rc)

    def add_structural_topology_reaction(self, topology_type, rate_function, reaction_function,
                                         expect_connected=True):
        """StructuralTopologyReaction on topologies of topology_type: rate_function(view) -> rate,
        reaction_function(view) -> recipe steps, e.g. [("remove_edge", 3, 4), ("change_particle_type", 0, 2)]
        (RECIPE_STEPS; vertices by local index of the view).  Without expect_connected a topology that falls
        apart becomes its pieces.  Returns the reaction's index."""
        lib = self._lib

        def rate_cb(_user, _sys, k):
            try:
                return float(rate_function(TopologyView(lib, self._h, k)))
            except BaseException as e:  # reported by the call that ran the function
                self._callback_error = getattr(self, "_callback_error", None) or e
                return float("nan")

        def recipe_cb(_user, _sys, k, recipe):
            try:
                _apply_recipe(lib, recipe, reaction_function(TopologyView(lib, self._h, k)))
            except BaseException as e:
                self._callback_error = getattr(self, "_callback_error", None) or e
                lib.rdc_recipe_change_particle_type(recipe, -1, 0)  # makes the evaluation fail

        cbs = (N.TOPOLOGY_RATE_FN(rate_cb), N.TOPOLOGY_RECIPE_FN(recipe_cb))
        self._callbacks = getattr(self, "_callbacks", []) + [cbs]
        rid = C.c_int()
        N.check(lib.rdc_add_structural_topology_reaction(self._h, int(topology_type), cbs[0], cbs[1], None,
                                                        int(bool(expect_connected)), C.byref(rid)))
        self._n_structural = getattr(self, "_n_structural", 0) + 1
        return rid.value

    def structural_reaction_counts(self):
        n = getattr(self, "_n_structural", 0)
        out = np.zeros(max(n, 1), np.int64)
        N.check(self._lib.rdc_get_structural_reaction_counts(self._h, n, _p(out, C.c_int64)))
        return out[:n]

    def get_topology(self, index):
        """TopologyView of the topology with this index (the order of get_topologies)."""
        return TopologyView(self._lib, self._h, index)

    def evaluate_topology_reactions(self, time_step):
        """EvaluateTopologyReactions (structural and spatial); returns the number of events performed."""
        n = C.c_int64()
        self._check_callbacks(self._lib.rdc_evaluate_topology_reactions(self._h, float(time_step), C.byref(n)))
        return n.value

    def topology_reaction_counts(self):
        """Performed events per spatial topology reaction since creation."""
        n = self.context.n_spatial_topology_reactions
        out = np.zeros(max(n, 1), np.int64)
        N.check(self._lib.rdc_get_topology_reaction_counts(self._h, n, _p(out, C.c_int64)))
        return out[:n]

    def get_topologies(self):
        """StateModel::getTopologies: a list of (topology type, particle ids[] uint64)."""
        nt, nid = C.c_int64(), C.c_int64()
        st = self._lib.rdc_get_topologies(self._h, 0, None, None, 0, None, C.byref(nt), C.byref(nid))
        if st not in (N.RDC_OK, N.RDC_ERR_CAPACITY):
            N.check(st)
        types = np.zeros(nt.value, np.int32)
        off = np.zeros(nt.value + 1, np.int64)
        ids = np.zeros(nid.value, np.uint64)
        N.check(self._lib.rdc_get_topologies(self._h, nt.value, _p(types, C.c_int), _p(off, C.c_int64), nid.value,
                                             _p(ids, C.c_uint64), C.byref(nt), C.byref(nid)))
        return [(int(types[k]), ids[off[k]:off[k + 1]]) for k in range(nt.value)]

    def get_topology_edges(self):
        """The graph edges of every topology, in the order of get_topologies: a list of (m, 2) id arrays."""
        nt, ne = C.c_int64(), C.c_int64()
        st = self._lib.rdc_get_topology_edges(self._h, 0, None, 0, None, C.byref(nt), C.byref(ne))
        if st not in (N.RDC_OK, N.RDC_ERR_CAPACITY):
            N.check(st)
        off = np.zeros(nt.value + 1, np.int64)
        edges = np.zeros((ne.value, 2), np.uint64)
        N.check(self._lib.rdc_get_topology_edges(self._h, nt.value, _p(off, C.c_int64), ne.value,
                                                 _p(edges, C.c_uint64), C.byref(nt), C.byref(ne)))
        return [edges[off[k]:off[k + 1]] for k in range(nt.value)]

    @property
    def n_particles(self) -> int:
        n = C.c_int64()
        N.check(self._lib.rdc_get_n_particles(self._h, C.byref(n)))
        return n.value

    def get_particles(self):
        """(positions[n,3] float64, types[n] int32, ids[n] uint64) in device storage order."""
        n = self.n_particles
        pos = np.zeros((n, 3)); t = np.zeros(n, np.int32); ids = np.zeros(n, np.uint64)
        got = C.c_int64()
        N.check(self._lib.rdc_get_particles(self._h, n, _p(pos, C.c_double), _p(t, C.c_int),
                                            _p(ids, C.c_uint64), C.byref(got)))
        return pos[:got.value], t[:got.value], ids[:got.value]

    def get_forces(self):
        n = self.n_particles
        f = np.zeros((n, 3)); ids = np.zeros(n, np.uint64)
        got = C.c_int64()
        N.check(self._lib.rdc_get_forces(self._h, n, _p(f, C.c_double), _p(ids, C.c_uint64), C.byref(got)))
        return f[:got.value], ids[:got.value]

    def get_particle_energies(self):
        """(energies[n], ids[n]): each particle's share of the last force calculation's energy."""
        n = self.n_particles
        e = np.zeros(n); ids = np.zeros(n, np.uint64)
        got = C.c_int64()
        N.check(self._lib.rdc_get_particle_energies(self._h, n, _p(e, C.c_double), _p(ids, C.c_uint64),
                                                    C.byref(got)))
        return e[:got.value], ids[:got.value]

    @property
    def energy(self) -> float:
        e = C.c_double()
        N.check(self._lib.rdc_get_energy(self._h, C.byref(e)))
        return e.value

    def set_record_virial(self, record: bool = True):
        """Context::recordVirial for this system as it is (rdc_set_record_virial): the next force calculation
        records the virial, or stops recording it."""
        N.check(self._lib.rdc_set_record_virial(self._h, int(bool(record))))

    def virial(self):
        """StateModel::virial() of the last force calculation, 3x3."""
        out = np.zeros(9)
        N.check(self._lib.rdc_get_virial(self._h, _p(out, C.c_double)))
        return out.reshape(3, 3)

    def count_types(self):
        out = np.zeros(self.context.n_types, np.int64)
        N.check(self._lib.rdc_count_types(self._h, _p(out, C.c_int64)))
        return out

    def particle_steps(self) -> int:
        """Particles advanced by the integrator since creation, summed over steps."""
        v = C.c_uint64()
        N.check(self._lib.rdc_get_particle_steps(self._h, C.byref(v)))
        return int(v.value)

    def reaction_counts(self):
        n = max(self.context.n_reactions, 1)
        out = np.zeros(n, np.int64)
        N.check(self._lib.rdc_get_reaction_counts(self._h, n, _p(out, C.c_int64)))
        return out[:self.context.n_reactions]

    def histogram_along_axis(self, bin_borders, types, axis):
        """HistogramAlongAxis observable (CPUObservables.cpp:85-146): counts of the listed types' particles
        along `axis` in the bins between ascending borders (the CPU kernel never fills the last bin)."""
        b = np.ascontiguousarray(bin_borders, np.float64)
        t = np.ascontiguousarray(types, np.int32)
        out = np.zeros(max(len(b) - 1, 1), np.float64)
        N.check(self._lib.rdc_histogram_along_axis(self._h, len(b), _p(b, C.c_double), len(t), _p(t, C.c_int),
                                                   int(axis), _p(out, C.c_double)))
        return out[:len(b) - 1]

    def radial_distribution(self, bin_borders, from_types, to_types, particle_to_density):
        """RadialDistribution observable (RadialDistribution.cpp:75-128): (bin centers, distribution, counts)."""
        b = np.ascontiguousarray(bin_borders, np.float64)
        f = np.ascontiguousarray(from_types, np.int32)
        t = np.ascontiguousarray(to_types, np.int32)
        counts = np.zeros(max(len(b) - 1, 1), np.float64)
        dist = np.zeros_like(counts)
        N.check(self._lib.rdc_radial_distribution(self._h, len(b), _p(b, C.c_double), len(f), _p(f, C.c_int), len(t),
                                                  _p(t, C.c_int), float(particle_to_density), _p(counts, C.c_double),
                                                  _p(dist, C.c_double)))
        centers = (b[:-1] + b[1:]) / 2
        return centers, dist[:len(b) - 1], counts[:len(b) - 1]

    def reserve(self, capacity):
        N.check(self._lib.rdc_reserve(self._h, int(capacity)))

    def set_cell_radius(self, radius):
        N.check(self._lib.rdc_set_cell_radius(self._h, int(radius)))

    # ---- actions ----
    def initialize(self):
        N.check(self._lib.rdc_initialize(self._h))

    def create_neighbor_list(self, cutoff):
        N.check(self._lib.rdc_nl_create(self._h, float(cutoff)))

    def update_neighbor_list(self):
        N.check(self._lib.rdc_nl_update(self._h))

    def clear_neighbor_list(self):
        N.check(self._lib.rdc_nl_clear(self._h))

    def calculate_forces(self):
        N.check(self._lib.rdc_calculate_forces(self._h))

    def euler_bd_integrator(self, dt):
        N.check(self._lib.rdc_euler_bd_integrate(self._h, float(dt)))

    def uncontrolled_approximation(self, dt):
        N.check(self._lib.rdc_uncontrolled_approximation(self._h, float(dt)))

    def gillespie(self, dt):
        N.check(self._lib.rdc_gillespie(self._h, float(dt)))

    def run(self, n_steps, dt, handler=N.UNCONTROLLED_APPROXIMATION, count_stride=0):
        """SimulationLoop::run on the device; returns per-type counts every count_stride steps."""
        nrec = (n_steps // count_stride + 1) if count_stride > 0 else 0
        counts = np.zeros((max(nrec, 1), self.context.n_types), np.int64)
        got = C.c_int64()
        self._check_callbacks(self._lib.rdc_run(self._h, int(n_steps), float(dt), int(handler), int(count_stride),
                                                _p(counts, C.c_int64) if nrec else None, nrec, C.byref(got)))
        return counts[:got.value]

    def neighbor_pairs(self, cutoff):
        """Sorted (min id, max id) pairs with d^2 < cutoff^2 from the current cell list."""
        cap = max(1024, 64 * self.n_particles)
        while True:
            out = np.zeros((cap, 2), np.uint64)
            n = C.c_int64()
            rc = self._lib.rdc_nl_pairs(self._h, float(cutoff), cap, _p(out, C.c_uint64), C.byref(n))
            if rc == N.RDC_ERR_CAPACITY and n.value > cap:
                cap = int(n.value) + 16
                continue
            N.check(rc)
            return out[:n.value].copy()

    def synchronize(self):
        N.check(self._lib.rdc_synchronize(self._h))
