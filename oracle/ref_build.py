"""TEST INFRASTRUCTURE ONLY: builds the reference's own pthread CPU kernel (kernels/cpu with readdy/main and
kernels/singlecpu) into oracle/_ref/libreaddy_ref.so, together with oracle/ref_driver.cpp, the C ABI that
bench.py's reference arm and the oracle's cross-check tests call through ctypes.

The reference tree is read where it lies when it is present.  Its sources needed for the build (ReaDDy's
headers with the vendored graphs and h5rd, readdy/main, kernels/cpu, kernels/singlecpu) are also staged
under oracle/_ref/src, which git ignores, so that a machine without the reference tree -- the Arm GPU
host, where binaries built here do not run -- builds the same library from the staged copy.  Nothing of
the reference is committed.  Third-party headers the reference includes and this image lacks (spdlog,
nlohmann-json, h5rd's HDF5 backend) come from the stand-ins in oracle/shim_include; {fmt} comes from the
copy PyTorch installs.  Flags follow the reference's Release build: -O3 -DNDEBUG (CMakeLists.txt:110).
The HDF5 compression filter (readdy/main/io/BloscFilter.cpp) needs the blosc library and is replaced by
stand-in definitions in ref_driver.cpp; no file is written.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF = "/root/reference"
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")
LIB = os.path.join(OUT, "libreaddy_ref.so")
STAGED = ["include", "readdy/main", "kernels/cpu/src", "kernels/cpu/include", "kernels/singlecpu/src",
          "kernels/singlecpu/include"]
SKIP = {"readdy/main/io/BloscFilter.cpp"}


def _fmt_include():
    try:
        import torch
    except ImportError:
        return None
    inc = os.path.join(os.path.dirname(torch.__file__), "include")
    return inc if os.path.exists(os.path.join(inc, "fmt", "format.h")) else None


def _stage() -> str | None:
    """Root of the reference sources to build from: the reference tree (staged under oracle/_ref/src on the
    way), or an earlier staged copy."""
    if os.path.isdir(REF):
        for d in STAGED:
            src, dst = os.path.join(REF, d), os.path.join(SRC, d)
            if os.path.isdir(src):
                shutil.copytree(src, dst, dirs_exist_ok=True)
        return SRC
    return SRC if os.path.isdir(os.path.join(SRC, "readdy", "main")) else None


def unavailable_reason() -> str | None:
    if _stage() is None:
        return "the reference sources are absent (neither the reference tree nor a staged copy)"
    if shutil.which("g++") is None:
        return "g++ is missing"
    if _fmt_include() is None:
        return "the {fmt} headers are missing"
    return None


def build(force: bool = False, jobs: int | None = None) -> str | None:
    """Compile and link the library (in parallel, a minute or so); returns its path, or None when it cannot
    be built here (see unavailable_reason())."""
    if not force and os.path.exists(LIB):
        return LIB
    if unavailable_reason() is not None:
        return None
    root = SRC
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    sources = []
    for d in ("readdy/main", "kernels/cpu/src", "kernels/singlecpu/src"):
        for dirpath, _, files in os.walk(os.path.join(root, d)):
            for f in files:
                rel = os.path.relpath(os.path.join(dirpath, f), root)
                if f.endswith(".cpp") and rel not in SKIP:
                    sources.append(os.path.join(root, rel))
    sources.append(os.path.join(HERE, "ref_driver.cpp"))
    flags = ["-std=c++20", "-O3", "-DNDEBUG", "-fPIC", "-DFMT_HEADER_ONLY", "-w",
             "-I", os.path.join(HERE, "shim_include"), "-I", os.path.join(root, "include"),
             "-I", os.path.join(root, "kernels", "cpu", "include"),
             "-I", os.path.join(root, "kernels", "singlecpu", "include"), "-I", _fmt_include()]

    def compile_one(src):
        obj = os.path.join(objdir, os.path.relpath(src, root if src.startswith(root) else HERE).replace("/", "_") + ".o")
        r = subprocess.run(["g++", *flags, "-c", src, "-o", obj], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compiling {src} failed:\n{r.stderr[-3000:]}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        objs = list(ex.map(compile_one, sources))
    tmp = LIB + ".tmp"
    r = subprocess.run(["g++", "-shared", "-o", tmp, *objs, "-pthread", "-ldl"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("linking the reference CPU kernel failed:\n" + r.stderr[-3000:])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv) or unavailable_reason())
