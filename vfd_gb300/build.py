"""Builds libvfd_dfsph.so, the CUDA library behind include/vfd_dfsph.h.

Each .cu file under csrc/ is compiled for sm_103a in parallel and linked into
an in-tree shared library (vfd_gb300/libvfd_dfsph.so). Host code is compiled
with -ffp-contract=off so that the SPH kernel table is built with the same
float operations as the reference's host code; device code keeps nvcc's
default contraction. No cmake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libvfd_dfsph.so")
# The bounds-checked variant (-DVFD_BOUNDS_CHECK): device index checks that record a
# failure in the status word instead of faulting; a debugging build, never the default.
BUILD_CHECKED = os.path.join(HERE, "_build_checked")
LIB_CHECKED = os.path.join(HERE, "libvfd_dfsph_checked.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-Xptxas", "-O3", "-I", INCLUDE]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps() -> list[str]:
    out = [os.path.join(INCLUDE, "vfd_dfsph.h")]
    out += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return out


def _stale(target: str, inputs: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(p) > t for p in inputs)


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None,
          bounds_check: bool = False) -> str:
    """Compile (if needed) and return the library path (the bounds-checked variant
    with bounds_check=True)."""
    build_dir, lib_path = (BUILD_CHECKED, LIB_CHECKED) if bounds_check else (BUILD, LIB)
    os.makedirs(build_dir, exist_ok=True)
    cc = nvcc()
    flags = ARCH + NVCC_FLAGS + (extra_flags or []) + (["-DVFD_BOUNDS_CHECK"] if bounds_check else [])
    deps = _deps()
    jobs = []
    objs = []
    for src in sources():
        obj = os.path.join(build_dir, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + deps):
            jobs.append([cc, *flags, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, file=sys.stderr)
        return r

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _stale(lib_path, objs):
        tmp = lib_path + ".tmp"
        run([cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
        os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, bounds_check="--bounds-check" in sys.argv))
