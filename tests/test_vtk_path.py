"""The reference's VTK path behind the C ABI: its TV_Data holds vtkIdType
(int64) cells, as get_TV_from_VTK (src/vtk_load.cu:46-298) fills them from a
.vtu.  tg_tv_narrow_i64 narrows them to int32, slots in their order, and
refuses ids that do not narrow (host code: runs without a GPU);
tg_mesh_create_i64 builds the mesh from them (GPU).  The VTK-gated driver
(tetragpu_gb300/vtk/tg_vtk_classify.cpp) compiles against the reference's own
headers where the reference tree is present; VTK itself is not installed
here, so the loader's declaration stands in for its header."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from tetragpu_gb300 import meshgen

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TG_ERR_INVALID_MESH, TG_ERR_UNSUPPORTED = 2, 5


def _narrow(lib, tv64, n_points):
    tv64 = np.ascontiguousarray(tv64, dtype=np.int64)
    out = np.full(tv64.shape, -7, dtype=np.int32)
    rc = lib.tg_tv_narrow_i64(tv64.ctypes.data, tv64.shape[0], n_points, out.ctypes.data)
    return rc, out


def _lib():
    from tetragpu_gb300 import _build
    import tetragpu_gb300 as tg
    _build.build()
    return tg.load()


def test_narrowing_keeps_ids_and_slot_order():
    lib = _lib()
    m = meshgen.kuhn_mesh(3, 0.3, seed=4)          # slots shuffled, ids permuted
    rc, out = _narrow(lib, m.tv.astype(np.int64), m.n_verts)
    assert rc == 0 and np.array_equal(out, m.tv)
    big = np.array([[0, 1, 2, (1 << 31) - 2]], np.int64)   # the largest id that narrows
    rc, out = _narrow(lib, big, (1 << 31) - 1)
    assert rc == 0 and out[0, 3] == (1 << 31) - 2


@pytest.mark.parametrize("bad", [[[0, 1, 2, 5]], [[0, -1, 2, 3]], [[0, 1, 2, 1 << 32]]])
def test_narrowing_refuses_ids_outside_the_mesh(bad):
    lib = _lib()
    tv = np.array([[0, 1, 2, 3]] + bad, np.int64)
    rc, _ = _narrow(lib, tv, 5)
    assert rc == TG_ERR_INVALID_MESH
    assert b"cell 1" in lib.tg_last_error_string()


def test_narrowing_refuses_point_counts_beyond_int32():
    lib = _lib()
    rc, _ = _narrow(lib, np.array([[0, 1, 2, 3]], np.int64), 1 << 31)
    assert rc == TG_ERR_UNSUPPORTED


def test_vtk_driver_compiles_against_reference_headers(tmp_path):
    from oracle import oracle as O
    if O.build_reference() is None or O.reference_root() is None:
        pytest.skip("reference source tree not present (TG_REFERENCE_ROOT)")
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    # VTK is not installed: the loader's declaration stands in for vtk_load.h
    (tmp_path / "vtk_load.h").write_text(
        "#include <memory>\n#include \"datatypes.h\"\n"
        "std::shared_ptr<TV_Data> get_TV_from_VTK(const runtime_arguments args);\n")
    cuda_inc = "/usr/local/cuda/include"
    cmd = [cxx, "-std=c++17", "-fsyntax-only", "-DTG_WITH_VTK", "-I", str(tmp_path),
           "-I", os.path.join(ROOT, "oracle", "_ref", "include"),
           "-I", os.path.join(O.reference_root(), "include"), "-I", os.path.join(ROOT, "include"),
           "-I", cuda_inc, os.path.join(ROOT, "tetragpu_gb300", "vtk", "tg_vtk_classify.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


@pytest.mark.gpu
def test_mesh_from_int64_tv_equals_int32_path(gpu_lib):
    m = meshgen.kuhn_mesh((5, 4, 3), 0.3, seed=6)
    lib = gpu_lib.load()
    tv64 = np.ascontiguousarray(m.tv, dtype=np.int64)
    h = C.c_void_p()
    assert lib.tg_mesh_create_i64(tv64.ctypes.data, m.n_cells, m.n_verts, None, C.byref(h)) == 0
    try:
        mask = gpu_lib.mask_of(["TE", "TF", "VV"])
        gpu_lib._lib.check(lib.tg_extract(h, mask, 0, None))
        with gpu_lib.Mesh(m.tv, m.n_verts) as g:
            g.extract(["TE", "TF", "VV"])
            for name in ("TE", "TF"):
                d = g.device_relation(name)
                want = g.relation(name)
                ent = np.empty(d["n_entries"], np.int32)
                gpu_lib._lib.check(lib.tg_copy_relation(h, gpu_lib.REL[name], None,
                                                        ent.ctypes.data, None))
                assert np.array_equal(ent.reshape(want.shape), want), name
        bad = np.array([[0, 1, 2, 9]], np.int64)
        h2 = C.c_void_p()
        assert lib.tg_mesh_create_i64(bad.ctypes.data, 1, 4, None, C.byref(h2)) == TG_ERR_INVALID_MESH
    finally:
        lib.tg_mesh_destroy(h)
