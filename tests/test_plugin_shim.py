"""The ReaDDy plugin (readdy_gb300/plugin/CUDAKernel.cpp) compiles against the reference's own headers and
exports the two C symbols the plugin loader reads (include/readdy/kernel/cpu/CPUKernel.h:150-152,
readdy/main/plugin/KernelProvider.cpp:135-175), under a file name the loader accepts (:123-133).

The reference tree and a C++20 compiler are needed: the test is skipped where the reference sources are
absent.  spdlog, nlohmann-json and h5rd/HDF5, which ReaDDy's headers include and this image lacks, come
from the stand-ins in oracle/shim_include; {fmt} comes from the one PyTorch installs.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_INCLUDE = "/root/reference/include"
LIB_NAME = "libreaddy_kernel_cuda.so"


def _fmt_include():
    try:
        import torch
    except ImportError:
        return None
    inc = os.path.join(os.path.dirname(torch.__file__), "include")
    return inc if os.path.exists(os.path.join(inc, "fmt", "format.h")) else None


def loader_accepts(path):
    """KernelProvider::isSharedLibrary (readdy/main/plugin/KernelProvider.cpp:123-133), restated."""
    return ((".dll" in path or ".so" in path or ".dylib" in path) and
            not any(s in path for s in (".lib", ".exp", ".pdb", ".manifest", ".rsp", ".obj", ".a")))


def test_library_name_passes_the_loader_filter():
    assert loader_accepts("/opt/readdy/plugins/" + LIB_NAME)
    assert not loader_accepts("/opt/readdy/plugins/libreaddy_kernel_cuda.a")


@pytest.mark.skipif(not os.path.isdir(REF_INCLUDE), reason="reference headers not present")
def test_plugin_compiles_against_reference_headers_and_exports_name_and_create_kernel(tmp_path):
    cxx = shutil.which("g++")
    fmt = _fmt_include()
    if cxx is None or fmt is None:
        pytest.skip("g++ or the {fmt} headers are missing")
    obj = tmp_path / "CUDAKernel.o"
    cmd = [cxx, "-std=c++20", "-fPIC", "-Wall", "-DFMT_HEADER_ONLY", "-c",
           "-I", os.path.join(ROOT, "oracle", "shim_include"), "-I", REF_INCLUDE, "-I", os.path.join(ROOT, "include"),
           "-I", fmt, os.path.join(ROOT, "readdy_gb300", "plugin", "CUDAKernel.cpp"), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    syms = subprocess.run(["nm", "-g", "--defined-only", str(obj)], capture_output=True, text=True).stdout.split()
    assert "name" in syms and "createKernel" in syms


EXPECTED_STRUCTURAL_LOG = """ids A=0 B=1 T1=0 T2=1
register type=0 expect_connected=1
register type=0 expect_connected=0
rate 36
change_particle_type 0 1
add_edge 0 2
remove_edge 0 1
remove_edge 1 0
remove_edge 1 2
append_particle 2 0 type 1 at 4 5 6
change_particle_position 1 7 8 9
change_topology_type 1
rate 2.5
change_particle_type 2 1"""


@pytest.fixture(scope="module")
def harness_objects(tmp_path_factory):
    """The plugin and the stand-in C ABI (tests/plugin_harness/fake_abi.cpp) compiled once, with stubs that return
    RDC_OK for the plugin's other calls, and ReaDDy's model library from the reference build (oracle/_ref)."""
    if not os.path.isdir(REF_INCLUDE):
        pytest.skip("reference headers not present")
    import oracle.ref_build as rb
    cxx, gcc = shutil.which("g++"), shutil.which("gcc")
    fmt = _fmt_include()
    if cxx is None or gcc is None or fmt is None:
        pytest.skip("g++, gcc or the {fmt} headers are missing")
    lib = rb.build()
    if lib is None:
        pytest.skip(rb.unavailable_reason())
    out = tmp_path_factory.mktemp("plugin_harness")
    flags = ["-std=c++20", "-fPIC", "-DFMT_HEADER_ONLY", "-w", "-I", os.path.join(ROOT, "oracle", "shim_include"),
             "-I", REF_INCLUDE, "-I", os.path.join(ROOT, "include"), "-I", fmt]
    srcs = {"plugin": os.path.join(ROOT, "readdy_gb300", "plugin", "CUDAKernel.cpp"),
            "fake": os.path.join(ROOT, "tests", "plugin_harness", "fake_abi.cpp")}
    objs = {}
    for name, src in srcs.items():
        objs[name] = str(out / (name + ".o"))
        r = subprocess.run([cxx, *flags, "-c", src, "-o", objs[name]], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-4000:]

    def rdc_symbols(obj, opt):
        text = subprocess.run(["nm", opt, obj], capture_output=True, text=True).stdout
        return {w for line in text.splitlines() for w in line.split() if w.startswith("rdc_")}

    rest = sorted(rdc_symbols(objs["plugin"], "-u") - rdc_symbols(objs["fake"], "--defined-only"))
    stubs = out / "stubs.c"
    stubs.write_text("".join(f"int {s}() {{ return 0; }}\n" for s in rest))
    objs["stubs"] = str(out / "stubs.o")
    r = subprocess.run([gcc, "-std=gnu17", "-c", str(stubs), "-o", objs["stubs"]], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return {"cxx": cxx, "flags": flags, "objs": objs, "libdir": os.path.dirname(lib)}


def _harness(h, tmp_path, main_name):
    """Links tests/plugin_harness/<main_name> with the objects of harness_objects, runs it and returns its
    stdout lines."""
    main_obj = str(tmp_path / "main.o")
    r = subprocess.run([h["cxx"], *h["flags"], "-c", os.path.join(ROOT, "tests", "plugin_harness", main_name), "-o",
                        main_obj], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    exe = str(tmp_path / "harness")
    r = subprocess.run([h["cxx"], main_obj, *h["objs"].values(), "-L", h["libdir"], "-lreaddy_ref",
                        "-Wl,-rpath," + h["libdir"], "-pthread", "-ldl", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr[-2000:]
    return r.stdout.strip().splitlines()


def test_plugin_structural_reactions_drive_the_recipe_abi(harness_objects, tmp_path):
    """The plugin registers every structural reaction of ReaDDy's topology registry and runs its rate and
    reaction functions on the topology the C ABI describes: ReaDDy's own Recipe (Recipe.h, Recipe.cpp:55-69,
    with separateVertex's edge removals) becomes the rdc_recipe_* calls step by step, the rate function reads
    the topology's particles through the plugin's state model, and an exception of a reaction's function
    reaches the caller of the EvaluateTopologyReactions action.  A spatial reaction's rate function
    (SpatialTopologyReaction.h:77-99) is bound the same way and called with the two topologies."""
    lines = _harness(harness_objects, tmp_path, "structural_main.cpp")
    assert "\n".join(lines[:14]) == EXPECTED_STRUCTURAL_LOG
    # the spatial reaction's rate function on the two topologies (the stand-in passes its one topology as
    # both): 100 x 3 vertices + x = 1 + 2 + 3 of the second, read through the plugin's state model
    assert lines[14] == "spatial rate 306"
    assert lines[-1] == "caught rate failed"


# ids A=0 B=1 C=2 D=3 (C, D TOPOLOGY flavored), topology types T1=0 T2=1; the values of context_main.cpp
EXPECTED_CONTEXT_CALLS = """context box (10 12 14) pbc 1 1 0 kbt 1.5 D 1 0.5 0.25 2
flavor 0 0
flavor 1 0
flavor 2 1
flavor 3 1
spatial mode 1 2/0 + 3/0 -> 2/1 + 3/-1 rate 2 radius 1.5 distance 0
spatial mode 1 2/1 + 3/1 -> 2/0 + 3/-1 rate 1 radius 0.75 distance 0
spatial rate function of mode 1 2/1 + 3/1 -> 2/0 + 3/-1 rate 1 radius 0.75 distance 0
legacy self fusion 0
harmonic repulsion 0 1 k 10 d 1.1
weak interaction 1 1 k 5 desired 0.7 depth 0.3 cutoff 1.9
lennard jones 0 0 m 12 n 6 cutoff 2.5 shift 1 epsilon 1.25 sigma 0.9
screened electrostatics 0 2 strength -1 kappa 0.8 repulsion 1.2 sigma 0.6 exponent 6 cutoff 3.5
box 0 k 2 origin (-4 -5 -6) extent (8 10 12) inclusion 1
sphere 1 k 3 origin (0.5 0.25 -0.5) radius 4 inclusion 1
sphere 1 k 3.5 origin (0 0 0) radius 2 inclusion 0
capsule 2 k 4 center (0 1 0) direction (1 0 0) length 3 radius 1.5 inclusion 1
spherical barrier 3 height 2.5 width 0.5 origin (1 1 1) radius 2
cylinder 0 k 1.5 origin (0 0 0) normal (0 0 1) radius 3 inclusion 1
conversion 0 -> 1 rate 0.1
decay 1 rate 0.02
fusion 0 + 1 -> 2 rate 1 distance 1.2 weights 0.25 0.75
fission 2 -> 0 + 1 rate 0.5 distance 0.8 weights 0.5 0.5
enzymatic catalyst 3 0 -> 1 rate 0.7 distance 1.1
bond 2 3 k 10 length 1
angle 2 3 2 k 2 theta0 3
dihedral 2 3 3 2 k 1 n 3 phi0 0.5
record virial 0"""


def test_plugin_translates_the_context_into_the_abi(harness_objects, tmp_path):
    """Kernel::initialize turns a model::Context built through ReaDDy's own registries into rdc_context_* calls
    with exactly the values given: box, periodicity, kBT, diffusion constants and flavors; the four pair
    potentials (the parameters ReaDDy keeps without getters, read through member pointers and describe()); the
    five order-1 potentials, inclusion and exclusion; the five reactions with their normalised weights
    (Fusion.h:62-68); the bonded terms of the topology registry and its spatial reaction (descriptor parsed by
    ReaDDy).  The calls are compared as a set: the registries are hash maps."""
    lines = _harness(harness_objects, tmp_path, "context_main.cpp")
    assert lines[0] == "ids A=0 B=1 C=2 D=3 T1=0 T2=1"
    calls = lines[1:]
    assert len(calls) == len(set(calls))
    assert set(calls) == set(EXPECTED_CONTEXT_CALLS.splitlines())


EXPECTED_SYSTEM_CALLS = """add particle (0.5 1.5 -2.5) type 0
add particle (1 2 3) type 0
topology particles pending: (0 0 0)/1 (1 0 0)/1 (2 0 0.25)/1
pending vertex 2 type 1 x 2
system record virial 1
add topology type 0: (0 0 0)/1 (1 0 0)/1 (2 0 0.25)/1 edges 0-1 1-2
system record virial 1
initialize
neighbor list create 2.5
calculate forces
euler bd 0.01
neighbor list update
uncontrolled approximation 0.02
gillespie 0.03
break bonds dt 0.04 1-1 threshold 2 rate 0.5
same topology object after reload 1
topology particles uploaded: (0 0 0)/1 (1 0 0)/1 (2 0 0.25)/1
neighbor list clear
get virial
get reaction counts
reaction counts fus 101 conv 100
force of A 100 -100 0.5
force of A 101 -101 0.5
position of T 0 0 0
position of T 1 0 0
position of T 2 0 0.25
particles 5: 0/100 0/101 1/102 1/103 1/104
energy 42.5
count types
histogram axis 2 borders 0 1 2.5 types 1
radial distribution borders 0 0.5 1 2 from 0 to 0 1 density 0.25
topology record type 0 particles 2 3 4 edges 0-1 1-2
system create
add particle (0.5 1.5 -2.5) type 0
add particle (1 2 3) type 0
add topology type 0: (0 0 0)/1 (1 0 0)/1 (2 0 0.25)/1 edges 0-1 1-2
initialize
after initialize: 5 particles, 1 topologies, 3 vertices, 2 edges
after removeAllParticles: 0 particles, 0 topologies
virial 1 5 9
n particles 7 8
histogram 0 1
radial distribution centers 0.25 0.75 1.5 values 0 0.5 1"""


def test_plugin_state_model_actions_and_observables_reach_the_abi(harness_objects, tmp_path):
    """The state model, the actions in SimulationLoop's order and the binning observables, driven through
    ReaDDy's own interfaces: particles are uploaded at once, a topology with the edges added after addTopology
    returned is uploaded at the first action, every action passes its time step or cutoff, BreakBonds its
    configuration's pairs, and the observables their bins and type selections; the observables' results are
    the ABI's (the RadialDistribution bin centres are ReaDDy's midpoints); ReaDDy's own Topologies observable
    sees the topology with dense particle indices and local edges.  ReactionCounts maps ReaDDy's reaction ids
    (registration order: fusion 0, conversion 1) onto the device's (order-1 reactions first: conversion 0,
    fusion 1), whose counts the stand-in gives as 100 + device id.  Forces and Positions keep the selected
    types' particles, Particles all of them with types and ids, Energy the system's energy.  A Virial observable registered
    after the system holds particles switches the live system's virial on, and InitializeKernel applies the
    context's flag again, as CPUMiscActions.h:80-89 re-reads the context.  After BreakBonds reads the
    topologies back, the topology object the caller got from addTopology is still the state model's, and
    getParticlesForTopology gives its particles before and after the upload (before it, the vertices hold
    placeholder indices that GraphTopology::particleForVertex resolves too).  Kernel::initialize moves the free
    particles and the topology, with its edges, to a new system (CPUKernel.cpp:63-83 keeps them), and
    removeAllParticles leaves none."""
    assert _harness(harness_objects, tmp_path, "actions_main.cpp") == EXPECTED_SYSTEM_CALLS.splitlines()


EXPECTED_LOOP_CALLS = """supports topologies 1
add topology type 0: (0 0 0)/1 (1 0 0)/1 edges 0-1
system record virial 0
initialize
neighbor list create 2
calculate forces
euler bd 0.01
neighbor list update
gillespie 0.01
evaluate topology reactions 0.01
neighbor list update
calculate forces
euler bd 0.01
neighbor list update
gillespie 0.01
evaluate topology reactions 0.01
neighbor list update
calculate forces
neighbor list clear"""


def test_readdy_simulation_loop_drives_the_plugin(harness_objects, tmp_path):
    """ReaDDy's own SimulationLoop (SimulationLoop.h:256-306) runs two steps through the plugin: ReaDDy sees
    topology support (Kernel::supportsTopologies, which gates Simulation::addTopology and the loop's topology
    reactions), and the loop's actions reach the ABI in its order; the neighbour list takes the cutoff the loop
    holds when it runs: the context's largest (the pair potential's 1.5 over the topology reaction's radius
    1.0) plus the skin of 0.5 set through SimulationLoop::neighborListCutoff()."""
    lines = [l for l in _harness(harness_objects, tmp_path, "loop_main.cpp") if not l.startswith("[console]")]
    assert lines == EXPECTED_LOOP_CALLS.splitlines()


EXPECTED_PROVIDER_RUN = """CUDA kernel available 1
selected CUDA supports topologies 1
system create
initialize
add particle (0.5 0.5 0.5) type 0
add topology type 0: (0 0 0)/1 (1 0 0)/1 edges 0-1
system record virial 0
initialize
neighbor list create 1.5
calculate forces
count types
observed 7 particles of A
euler bd 0.01
neighbor list update
gillespie 0.01
neighbor list update
calculate forces
count types
observed 7 particles of A
euler bd 0.01
neighbor list update
gillespie 0.01
neighbor list update
calculate forces
count types
observed 7 particles of A
neighbor list clear"""


def test_kernel_provider_loads_the_plugin_and_a_simulation_runs(harness_objects, tmp_path):
    """The plugin built as libreaddy_kernel_cuda.so (with the stand-in C ABI inside) in a plugin directory:
    ReaDDy's KernelProvider loads it (KernelProvider.cpp:99-175), readdy::Simulation("CUDA", context) creates
    the kernel, adds a particle and a topology, registers an NParticles observable and runs two steps; the
    stand-in's log shows the calls in SimulationLoop's order and the observable evaluated at every step."""
    h = harness_objects
    plugins = tmp_path / "plugins"
    plugins.mkdir()
    lib = plugins / LIB_NAME
    assert loader_accepts(str(lib))
    r = subprocess.run([h["cxx"], "-shared", "-o", str(lib), h["objs"]["plugin"], h["objs"]["fake"], h["objs"]["stubs"],
                        "-L", h["libdir"], "-lreaddy_ref", "-Wl,-rpath," + h["libdir"]], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    main_obj, exe = str(tmp_path / "provider.o"), str(tmp_path / "provider")
    r = subprocess.run([h["cxx"], *h["flags"], "-c", os.path.join(ROOT, "tests", "plugin_harness", "provider_main.cpp"),
                        "-o", main_obj], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    r = subprocess.run([h["cxx"], main_obj, "-L", h["libdir"], "-lreaddy_ref", "-Wl,-rpath," + h["libdir"], "-pthread",
                        "-ldl", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    r = subprocess.run([exe, str(plugins)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-2000:])
    lines = [l for l in r.stdout.strip().splitlines() if not l.startswith("[console]")]
    assert lines == EXPECTED_PROVIDER_RUN.splitlines()
