"""ctypes binding of libreaddy_cuda_core.so (the C ABI declared in include/readdy_cuda.h).

There is no CPU fallback: if the library cannot be built or loaded, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

RDC_OK = 0
RDC_ERR_INVALID_ARGUMENT = 1
RDC_ERR_LOGIC = 2
RDC_ERR_RUNTIME = 3
RDC_ERR_CUDA = 4
RDC_ERR_CAPACITY = 5

UNCONTROLLED_APPROXIMATION = 0
GILLESPIE = 1

_lib = None
_lock = threading.Lock()


class CudaKernelError(RuntimeError):
    """A CUDA runtime failure or a device-side capacity/status error."""


class CapacityError(CudaKernelError):
    pass


# structural topology reaction functions (include/readdy_cuda.h: rdc_topology_rate_fn, rdc_topology_recipe_fn)
TOPOLOGY_RATE_FN = C.CFUNCTYPE(C.c_double, C.c_void_p, C.c_void_p, C.c_int64)
TOPOLOGY_RECIPE_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p)
# spatial topology reaction rate from two topologies (include/readdy_cuda.h: rdc_spatial_rate_fn)
SPATIAL_RATE_FN = C.CFUNCTYPE(C.c_double, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64)


def _sig(lib):
    d, i, u64, i64, vp = C.c_double, C.c_int, C.c_uint64, C.c_int64, C.c_void_p
    P = C.POINTER
    vpp = P(vp)
    table = {
        "rdc_last_error": (C.c_char_p, []),
        "rdc_version": (i, []),
        "rdc_kernel_name": (C.c_char_p, []),
        "rdc_set_device": (i, [i]),
        "rdc_context_create": (i, [vpp, P(d), P(i), d, i, P(d)]),
        "rdc_context_destroy": (i, [vp]),
        "rdc_context_max_cutoff": (i, [vp, P(d)]),
        "rdc_context_set_record_virial": (i, [vp, i]),
        "rdc_context_set_particle_flavor": (i, [vp, i, i]),
        "rdc_context_add_spatial_topology_reaction": (i, [vp, i, i, i, i, i, i, i, i, i, d, d, i, P(i)]),
        "rdc_context_set_legacy_topology_self_fusion": (i, [vp, i]),
        "rdc_context_set_spatial_topology_rate_function": (i, [vp, i, SPATIAL_RATE_FN, vp]),
        "rdc_get_virial": (i, [vp, P(d)]),
        "rdc_set_record_virial": (i, [vp, i]),
        "rdc_context_add_harmonic_repulsion": (i, [vp, i, i, d, d]),
        "rdc_context_add_weak_interaction_piecewise_harmonic": (i, [vp, i, i, d, d, d, d]),
        "rdc_context_add_lennard_jones": (i, [vp, i, i, C.c_uint, C.c_uint, d, i, d, d]),
        "rdc_context_add_screened_electrostatics": (i, [vp, i, i, d, d, d, d, C.c_uint, d]),
        "rdc_context_add_box": (i, [vp, i, d, P(d), P(d), i]),
        "rdc_context_add_sphere": (i, [vp, i, d, P(d), d, i]),
        "rdc_context_add_capsule": (i, [vp, i, d, P(d), P(d), d, d, i]),
        "rdc_context_add_spherical_barrier": (i, [vp, i, d, d, P(d), d]),
        "rdc_context_add_cylinder": (i, [vp, i, d, P(d), P(d), d, i]),
        "rdc_context_add_conversion": (i, [vp, i, i, d, P(i)]),
        "rdc_context_add_decay": (i, [vp, i, d, P(i)]),
        "rdc_context_add_fusion": (i, [vp, i, i, i, d, d, d, d, P(i)]),
        "rdc_context_add_fission": (i, [vp, i, i, i, d, d, d, d, P(i)]),
        "rdc_context_add_enzymatic": (i, [vp, i, i, i, d, d, P(i)]),
        "rdc_context_configure_harmonic_bond": (i, [vp, i, i, d, d]),
        "rdc_context_configure_harmonic_angle": (i, [vp, i, i, i, d, d]),
        "rdc_context_configure_cosine_dihedral": (i, [vp, i, i, i, i, d, d, d]),
        "rdc_system_create": (i, [vpp, vp, u64]),
        "rdc_system_destroy": (i, [vp]),
        "rdc_add_particles": (i, [vp, i64, P(d), P(i), P(u64)]),
        "rdc_add_topology": (i, [vp, i64, P(d), P(i), i64, P(i64), P(u64)]),
        "rdc_add_topology_typed": (i, [vp, i, i64, P(d), P(i), i64, P(i64), P(u64)]),
        "rdc_break_bonds": (i, [vp, d, i, P(i), P(i), P(d), P(d), P(i64)]),
        "rdc_get_topologies": (i, [vp, i64, P(i), P(i64), i64, P(u64), P(i64), P(i64)]),
        "rdc_evaluate_topology_reactions": (i, [vp, d, P(i64)]),
        "rdc_get_topology_reaction_counts": (i, [vp, i, P(i64)]),
        "rdc_add_structural_topology_reaction": (i, [vp, i, TOPOLOGY_RATE_FN, TOPOLOGY_RECIPE_FN, vp, i, P(i)]),
        "rdc_get_structural_reaction_counts": (i, [vp, i, P(i64)]),
        "rdc_recipe_change_particle_type": (i, [vp, i64, i]),
        "rdc_recipe_add_edge": (i, [vp, i64, i64]),
        "rdc_recipe_remove_edge": (i, [vp, i64, i64]),
        "rdc_recipe_separate_vertex": (i, [vp, i64]),
        "rdc_recipe_change_topology_type": (i, [vp, i]),
        "rdc_recipe_append_particle": (i, [vp, i64, P(i64), i, P(d)]),
        "rdc_recipe_change_particle_position": (i, [vp, i64, P(d)]),
        "rdc_get_topology": (i, [vp, i64, P(i), i64, P(u64), P(i), P(i64), i64, P(i64), P(i64)]),
        "rdc_get_topology_positions": (i, [vp, i64, i64, P(d)]),
        "rdc_get_topology_edges": (i, [vp, i64, P(i64), i64, P(u64), P(i64), P(i64)]),
        "rdc_get_n_particles": (i, [vp, P(i64)]),
        "rdc_get_particles": (i, [vp, i64, P(d), P(i), P(u64), P(i64)]),
        "rdc_get_forces": (i, [vp, i64, P(d), P(u64), P(i64)]),
        "rdc_get_particle_energies": (i, [vp, i64, P(d), P(u64), P(i64)]),
        "rdc_get_energy": (i, [vp, P(d)]),
        "rdc_count_types": (i, [vp, P(i64)]),
        "rdc_get_particle_steps": (i, [vp, P(u64)]),
        "rdc_get_reaction_counts": (i, [vp, i, P(i64)]),
        "rdc_histogram_along_axis": (i, [vp, i, P(d), i, P(i), i, P(d)]),
        "rdc_radial_distribution": (i, [vp, i, P(d), i, P(i), i, P(i), d, P(d), P(d)]),
        "rdc_reserve": (i, [vp, i64]),
        "rdc_set_cell_radius": (i, [vp, i]),
        "rdc_initialize": (i, [vp]),
        "rdc_nl_create": (i, [vp, d]),
        "rdc_nl_update": (i, [vp]),
        "rdc_nl_clear": (i, [vp]),
        "rdc_calculate_forces": (i, [vp]),
        "rdc_euler_bd_integrate": (i, [vp, d]),
        "rdc_uncontrolled_approximation": (i, [vp, d]),
        "rdc_gillespie": (i, [vp, d]),
        "rdc_run": (i, [vp, i64, d, i, i64, P(i64), i64, P(i64)]),
        "rdc_nl_pairs": (i, [vp, d, i64, P(u64), P(i64)]),
        "rdc_synchronize": (i, [vp]),
        "rdc_batch_create": (i, [vpp, vp, i, P(d), P(i64), u64]),
        "rdc_batch_destroy": (i, [vp]),
        "rdc_batch_set_particles": (i, [vp, P(i64), P(d), P(i)]),
        "rdc_batch_configure": (i, [vp, i, d, d, i]),
        "rdc_batch_set_carry_forces": (i, [vp, i]),
        "rdc_batch_set_particles_list": (i, [vp, vp, vp, vp]),
        "rdc_batch_step": (i, [vp, i64]),
        "rdc_batch_step_timed": (i, [vp, i64, P(d)]),
        "rdc_batch_particle_steps": (i, [vp, P(u64)]),
        "rdc_batch_count_types": (i, [vp, P(i64)]),
        "rdc_batch_n_particles": (i, [vp, P(i64)]),
        "rdc_batch_get_particles": (i, [vp, i, i64, P(d), P(i), P(u64), P(i64)]),
        "rdc_batch_get_forces": (i, [vp, i, i64, P(d), P(u64), P(i64)]),
        "rdc_batch_reaction_counts": (i, [vp, i, P(i64)]),
        "rdc_batch_get_virial": (i, [vp, P(d)]),
        "rdc_batch_record_counts": (i, [vp, i64, i64]),
        "rdc_batch_record_trajectory": (i, [vp, i, P(i), i64, i64]),
        "rdc_batch_poll_trajectory": (i, [vp, i64, i64, P(i64), P(i64), P(d), P(i), P(u64), P(i64), P(i64)]),
        "rdc_batch_poll_count_records": (i, [vp, i64, P(i64), P(i64), P(i64)]),
        "rdc_batch_replica_grid": (i, [vp, i, P(i), P(i)]),
        "rdc_batch_synchronize": (i, [vp]),
        "rdc_server_create": (i, [vpp, u64, i, i, i64]),
        "rdc_server_destroy": (i, [vp]),
        "rdc_server_set_plain_workers": (i, [vp, i]),
        "rdc_server_request_bytes": (i, [vp, i64, i64, i64, i64, P(u64), P(i)]),
        "rdc_server_submit": (i, [vp, vp, i64, P(d), P(i), i64, d, i64, u64, P(i64)]),
        "rdc_server_progress": (i, [vp, i64, P(i64)]),
        "rdc_server_poll": (i, [vp, i64, P(i64), P(i64)]),
        "rdc_server_result": (i, [vp, i64, i64, P(i64), P(i64), P(i), P(d)]),
        "rdc_server_peek_records": (i, [vp, i64, i64, P(i64), P(i64)]),
        "rdc_server_release": (i, [vp, i64]),
        "rdc_server_stats": (i, [vp, P(u64), P(u64), P(i64), P(i64)]),
        "rdc_forces_noalloc": (i, [vp, i64, vp, vp, vp, vp, vp]),
    }
    for name, (res, args) in table.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


EXPORTED = None  # filled from the header by tests


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load the CUDA core, building it in-tree first if needed (nvcc for sm_103a)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing:
            _build.build()
        if not os.path.exists(path):
            raise CudaKernelError(f"CUDA core library missing: {path} (run readdy_gb300.build.build())")
        _lib = _sig(C.CDLL(path))
        return _lib


def check(rc: int):
    if rc == RDC_OK:
        return
    msg = _lib.rdc_last_error().decode() if _lib is not None else "unknown error"
    if rc == RDC_ERR_INVALID_ARGUMENT:
        raise ValueError(msg)
    if rc == RDC_ERR_LOGIC:
        raise RuntimeError(msg)
    if rc == RDC_ERR_CAPACITY:
        raise CapacityError(msg)
    raise CudaKernelError(msg)
