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
