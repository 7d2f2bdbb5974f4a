"""Build libtetragpu.so in tree with nvcc for sm_103a (GB300).

The translation units compile in parallel; a rebuild happens only when a
source or header is newer than the library.  No CMake, no torch extension
machinery: the library is plain CUDA C++ behind the C ABI in
include/tetragpu.h.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libtetragpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "--expt-relaxed-constexpr",
           "-I" + INCLUDE, "-I" + CSRC]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libtetragpu.so")


def sources() -> list:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _stale(target: str, deps: list) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, defines: dict | None = None,
          out_dir: str | None = None) -> str:
    """Compile every csrc/*.cu and link libtetragpu.so.  defines: extra -D
    NAME=value (the tuning sweep's candidates), built under out_dir (its own
    objects and library) instead of the package."""
    nvcc = _nvcc()
    build_dir = os.path.join(out_dir, "obj") if out_dir else BUILD
    lib = os.path.join(out_dir, "libtetragpu.so") if out_dir else LIB
    dflags = [f"-D{k}={v}" for k, v in sorted((defines or {}).items())]
    os.makedirs(build_dir, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    objs = []
    jobs = []
    for src in sources():
        obj = os.path.join(build_dir, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc, *ARCH, *NVFLAGS, *dflags, "-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            results = list(ex.map(lambda cmd: subprocess.run(cmd, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, results):
            if verbose and r.stdout:
                print(r.stdout)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stderr)
    if force or jobs or _stale(lib, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", lib, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + " ".join(cmd) + "\n" + r.stderr)
    return lib


if __name__ == "__main__":
    print(build(verbose=True))
