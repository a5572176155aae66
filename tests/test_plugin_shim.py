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


@pytest.mark.skipif(not os.path.isdir(REF_INCLUDE), reason="reference headers not present")
def test_plugin_structural_reactions_drive_the_recipe_abi(tmp_path):
    """The plugin registers every structural reaction of ReaDDy's topology registry and runs its rate and
    reaction functions on the topology the C ABI describes: ReaDDy's own Recipe (Recipe.h, Recipe.cpp:55-69,
    with separateVertex's edge removals) becomes the rdc_recipe_* calls step by step, the rate function reads
    the topology's particles through the plugin's state model, and an exception of a reaction's function
    reaches the caller of the EvaluateTopologyReactions action.  ReaDDy's model library comes from the
    reference build (oracle/_ref); the C ABI is the host-side stand-in tests/plugin_harness/fake_abi.cpp."""
    import oracle.ref_build as rb
    cxx, gcc = shutil.which("g++"), shutil.which("gcc")
    fmt = _fmt_include()
    if cxx is None or gcc is None or fmt is None:
        pytest.skip("g++, gcc or the {fmt} headers are missing")
    lib = rb.build()
    if lib is None:
        pytest.skip(rb.unavailable_reason())
    flags = ["-std=c++20", "-fPIC", "-DFMT_HEADER_ONLY", "-w", "-I", os.path.join(ROOT, "oracle", "shim_include"),
             "-I", REF_INCLUDE, "-I", os.path.join(ROOT, "include"), "-I", fmt]
    harness = os.path.join(ROOT, "tests", "plugin_harness")
    srcs = {"plugin": os.path.join(ROOT, "readdy_gb300", "plugin", "CUDAKernel.cpp"),
            "fake": os.path.join(harness, "fake_abi.cpp"), "main": os.path.join(harness, "structural_main.cpp")}
    objs = {}
    for name, src in srcs.items():
        objs[name] = str(tmp_path / (name + ".o"))
        r = subprocess.run([cxx, *flags, "-c", src, "-o", objs[name]], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-4000:]

    def rdc_symbols(obj, opt):
        out = subprocess.run(["nm", opt, obj], capture_output=True, text=True).stdout
        return {w for line in out.splitlines() for w in line.split() if w.startswith("rdc_")}

    # the plugin's other C-ABI calls: stubs that return RDC_OK
    rest = sorted(rdc_symbols(objs["plugin"], "-u") - rdc_symbols(objs["fake"], "--defined-only"))
    stubs = tmp_path / "stubs.c"
    stubs.write_text("".join(f"int {s}() {{ return 0; }}\n" for s in rest))
    r = subprocess.run([gcc, "-std=gnu17", "-c", str(stubs), "-o", str(tmp_path / "stubs.o")], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    exe = str(tmp_path / "harness")
    libdir = os.path.dirname(lib)
    r = subprocess.run([cxx, *objs.values(), str(tmp_path / "stubs.o"), "-L", libdir, "-lreaddy_ref",
                        "-Wl,-rpath," + libdir, "-pthread", "-ldl", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = r.stdout.strip().splitlines()
    assert "\n".join(lines[:14]) == EXPECTED_STRUCTURAL_LOG
    assert lines[-1] == "caught rate failed"
