"""Build libcwa.so in-tree: nvcc for the sm_103a kernels, g++ for host-only
sources, translation units compiled in parallel, then one shared link.

No cmake.  Objects go to coupledwateranimation_gb300/_build/, the library to
coupledwateranimation_gb300/libcwa.so (both git-ignored).  The CUDA runtime
is linked statically, so the library needs only the driver at run time.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
OBJDIR = PKG / "_build"
LIB = PKG / "libcwa.so"
# the index-checked build (CWA_DEBUG_CHECKS): separate objects and library
OBJDIR_DEBUG = PKG / "_build_debug"
LIB_DEBUG = PKG / "libcwa_debug.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = ["-O3", "-fPIC", "-ffp-contract=off", "-fno-fast-math"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcwa")


def _cuda_include(nvcc: str) -> str:
    return str(Path(nvcc).resolve().parent.parent / "include")


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _stale(src: Path, obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *deps, Path(__file__)])


def _compile(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(force: bool = False, verbose: bool = False, debug: bool = False) -> Path:
    """Compile and link libcwa.so; with debug=True, libcwa_debug.so, the same
    sources with the device index checks of CWA_DEBUG_CHECKS compiled in."""
    nvcc = _nvcc()
    objdir, lib_out = (OBJDIR_DEBUG, LIB_DEBUG) if debug else (OBJDIR, LIB)
    defs = ["-DCWA_DEBUG_CHECKS"] if debug else []
    objdir.mkdir(exist_ok=True)
    deps = _headers()
    jobs = []
    objs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = objdir / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(src, obj, deps):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", *defs, "-Xcompiler",
                         ",".join(HOST_FLAGS), "-c", str(src), "-o", str(obj)])
    cxx = os.environ.get("CXX", "g++")
    for src in sorted(CSRC.glob("*.cpp")):
        obj = objdir / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(src, obj, deps):
            jobs.append([cxx, *HOST_FLAGS, "-std=c++17", *defs, "-I", _cuda_include(nvcc), "-c", str(src),
                         "-o", str(obj)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(_compile, jobs))
    if force or jobs or not lib_out.exists():
        tmp = lib_out.with_suffix(".so.tmp")
        _compile([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-Xcompiler", "-fPIC"])
        os.replace(tmp, lib_out)
    if verbose:
        print(f"built {lib_out}")
    return lib_out


if __name__ == "__main__":
    build(verbose=True)
