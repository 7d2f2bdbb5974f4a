"""The C++ drop-in layer for the reference's cuda_extraction.h entry points
(include/tetragpu_compat.h): its signatures against the reference's own
headers (CPU, where the reference tree exists), and a C++ caller that follows
the reference's per-relation test flow against the CPU oracle (GPU)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from tetragpu_gb300 import meshgen

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.join(ROOT, "tests", "compat")


def _nvcc():
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    pytest.skip("nvcc not available")


def test_signatures_match_reference_headers(tmp_path):
    """The reference's datatypes.h + cuda_extraction.h and tetragpu_compat.h
    compile together (same signatures) and every entry point links."""
    from oracle import oracle as O
    if O.build_reference() is None or O.reference_root() is None:
        pytest.skip("reference source tree not present (TG_REFERENCE_ROOT)")
    from tetragpu_gb300 import _build
    _build.build()
    out = tmp_path / "sig"
    cmd = [_nvcc(), "-std=c++17", "-I", os.path.join(ROOT, "oracle", "_ref", "include"),
           "-I", os.path.join(O.reference_root(), "include"), "-I", os.path.join(ROOT, "include"),
           os.path.join(HERE, "signatures.cu"), "-o", str(out),
           "-L", os.path.dirname(_build.LIB), "-ltetragpu",
           "-Xlinker", "-rpath=" + os.path.dirname(_build.LIB)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


@pytest.mark.gpu
@pytest.mark.parametrize("dims,frac,seed", [(5, 0.3, 3), ((9, 7, 6), 0.2, 4)])
def test_compat_driver_against_oracle(gpu_lib, tmp_path, dims, frac, seed):
    from oracle import oracle as O
    O.build()
    from tetragpu_gb300 import _build
    exe = tmp_path / "compat_driver"
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "oracle"), "-I", "/usr/local/cuda/include",
           os.path.join(HERE, "compat_driver.cpp"), "-o", str(exe),
           "-L", os.path.dirname(_build.LIB), "-ltetragpu",
           "-Xlinker", "-rpath=" + os.path.dirname(_build.LIB),
           os.path.join(ROOT, "oracle", "liboracle.so"),
           "-Xlinker", "-rpath=" + os.path.join(ROOT, "oracle"),
           "-L", "/usr/local/cuda/lib64", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    m = meshgen.kuhn_mesh(dims, frac, seed=seed)
    path = tmp_path / "mesh.bin"
    with open(path, "wb") as f:
        f.write(np.int64(m.n_cells).tobytes())
        f.write(np.int64(m.n_verts).tobytes())
        f.write(np.ascontiguousarray(m.tv, np.int32).tobytes())
    r = subprocess.run([str(exe), str(path)], capture_output=True, text=True)
    assert r.returncode == 0 and "compat OK" in r.stdout, r.stdout + r.stderr
