"""The C ABI library builds, loads and exports every entry point include/*.h declares.

No compute call is made here: these run on machines without a GPU.
"""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(rdc_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "rdc_system_create" in names and "rdc_batch_step" in names
    assert len(names) >= 40


def test_library_exports_every_declared_symbol():
    from readdy_gb300 import _native
    lib = _native.load()
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_kernel_name_and_version_without_gpu():
    from readdy_gb300 import _native
    lib = _native.load()
    assert lib.rdc_kernel_name().decode() == "CUDA"
    assert lib.rdc_version() >= 1000


def test_context_registries_validate_like_the_reference():
    """Argument checks of the registries need no device (Potentials.cpp:163-201, TorsionPotential.h:63-67)."""
    import readdy_gb300 as rg
    ctx = rg.Context((10, 10, 10), diffusion_constants=(1.0, 0.5))
    with pytest.raises(ValueError, match="not greater than the second exponent"):
        ctx.add_lennard_jones(0, 0, 6, 12, 2.5, True, 1.0, 1.0)
    with pytest.raises(ValueError, match="inverse screening depth"):
        ctx.add_screened_electrostatics(0, 0, -1.0, -1.0, 1.0, 1.0, 6, 8.0)
    with pytest.raises(ValueError, match="equilibrium angle"):
        ctx.configure_cosine_dihedral(0, 0, 0, 0, 1.0, 3, 4.0)
    with pytest.raises(ValueError, match="type out of range"):
        ctx.add_harmonic_repulsion(0, 5, 1.0, 1.0)
    with pytest.raises(ValueError, match="radius larger than its width"):
        ctx.add_spherical_barrier(0, 2.0, 3.0, (0, 0, 0), 1.0)
    with pytest.raises(ValueError, match="normal must be nonzero"):
        ctx.add_cylinder(0, 1.0, (0, 0, 0), (0, 0, 0), 1.0, True)
    ctx.add_box(1, 10.0, (-1, -1, -1), (2, 2, 2))
    ctx.add_harmonic_repulsion(0, 1, 10.0, 1.0)
    ctx.add_fusion(0, 1, 1, 1.0, 1.5)
    assert ctx.calculate_max_cutoff() == pytest.approx(1.5)
    assert ctx.add_fission(1, 0, 1, 0.1, 1.0) == 1


def test_null_arguments_are_rejected_before_any_device_call():
    """The entry points added for observables, uploads and the force switch check their pointers first, so a
    caller's mistake is an RDC_ERR_INVALID_ARGUMENT (1) with a message, on any machine."""
    from readdy_gb300 import _native
    lib = _native.load()
    v = ctypes.c_void_p
    for name, nargs in (("rdc_histogram_along_axis", 7), ("rdc_radial_distribution", 10),
                        ("rdc_batch_set_particles_list", 4), ("rdc_batch_set_carry_forces", 2)):
        f = getattr(lib, name)
        f.restype = ctypes.c_int
        args = [None] * nargs
        if name == "rdc_histogram_along_axis":
            f.argtypes = [v, ctypes.c_int, v, ctypes.c_int, v, ctypes.c_int, v]
            args = [None, 2, None, 0, None, 0, None]
        elif name == "rdc_radial_distribution":
            f.argtypes = [v, ctypes.c_int, v, ctypes.c_int, v, ctypes.c_int, v, ctypes.c_double, v, v]
            args = [None, 2, None, 0, None, 0, None, 1.0, None, None]
        elif name == "rdc_batch_set_carry_forces":
            f.argtypes = [v, ctypes.c_int]
            args = [None, 1]
        else:
            f.argtypes = [v] * nargs
        assert f(*args) == 1, name
        assert "null argument" in lib.rdc_last_error().decode()


def test_topology_registries_validate_like_the_reference():
    """Spatial topology reactions and flavors are checked without a device (SpatialTopologyReaction.h:88-91,
    TopologyRegistry.cpp:238-242, ParticleTypeRegistry.h:58-63); their radius counts in the largest cutoff
    (Context::calculateMaxCutoff)."""
    import readdy_gb300 as rg
    ctx = rg.Context((10, 10, 10), diffusion_constants=(1.0, 1.0, 1.0))
    with pytest.raises(ValueError, match="flavor"):
        ctx.set_particle_flavor(0, 7)
    with pytest.raises(ValueError, match="rate"):
        ctx.add_spatial_topology_reaction(ctx.TT_FUSION, (0, 0), (1, 0), (2, 1), (2, 1), 0.0, 1.0)
    with pytest.raises(ValueError, match="radius"):
        ctx.add_spatial_topology_reaction(ctx.TT_FUSION, (0, 0), (1, 0), (2, 1), (2, 1), 1.0, -1.0)
    with pytest.raises(ValueError, match="mode"):
        ctx.add_spatial_topology_reaction(9, (0, 0), (1, 0), (2, 1), (2, 1), 1.0, 1.0)
    with pytest.raises(ValueError, match="topology_type2"):  # a topology-particle mode with two topologies
        ctx.add_spatial_topology_reaction(ctx.TP_FUSION, (0, 0), (1, 0), (2, 1), (2, None), 1.0, 1.0)
    with pytest.raises(ValueError, match="type out of range"):
        ctx.add_spatial_topology_reaction(ctx.TT_FUSION, (0, 0), (5, 0), (2, 1), (2, 1), 1.0, 1.0)
    assert ctx.add_spatial_topology_reaction(ctx.TP_FUSION, (0, 0), (1, None), (2, 0), (2, None), 1.0, 2.5) == 0
    assert ctx.calculate_max_cutoff() == pytest.approx(2.5)
    ctx.set_legacy_topology_self_fusion(True)


def test_recipe_steps_reject_null_arguments():
    from readdy_gb300 import _native
    lib = _native.load()
    assert lib.rdc_recipe_add_edge(None, 0, 1) == 1
    assert lib.rdc_recipe_append_particle(None, 0, None, 0, None) == 1
    assert lib.rdc_recipe_change_particle_position(None, 0, None) == 1
