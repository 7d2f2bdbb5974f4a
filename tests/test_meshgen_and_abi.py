"""Workload generators (sizes and determinism) and the C-ABI library
(builds, loads without a GPU, exports every function include/tetragpu.h
declares)."""
import os
import re

import numpy as np
import pytest

from tetragpu_gb300 import meshgen

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_small_workload_sizes(oracle):
    m = meshgen.workload_small()
    assert (m.n_verts, m.n_cells) == (4913, 24576)
    r = oracle.extract(oracle.canonicalize(m.tv, m.n_verts), m.n_verts, mask=1 << 1 | 1 << 4)
    assert r["counts"] == (4913, 31024, 50688, 24576)


def test_irregular_workload_sizes():
    m = meshgen.workload_irregular()
    assert (m.n_verts, m.n_cells) == (327054, 1887438)
    assert m.field.dtype == np.float32 and m.field.shape == (m.n_verts,)


def test_generator_is_deterministic():
    a = meshgen.kuhn_mesh(4, 0.3, seed=99)
    b = meshgen.kuhn_mesh(4, 0.3, seed=99)
    assert np.array_equal(a.tv, b.tv) and np.array_equal(a.coords, b.coords)
    assert not np.array_equal(a.tv, meshgen.kuhn_mesh(4, 0.3, seed=98).tv)


def test_coned_mesh_is_conforming(oracle):
    """Every face lies in at most two cells (the oracle rejects otherwise) and
    the mesh is a ball (Euler characteristic 1)."""
    m = meshgen.kuhn_mesh((5, 4, 3), 0.5, seed=7)
    r = oracle.extract(oracle.canonicalize(m.tv, m.n_verts), m.n_verts, mask=1 << 1 | 1 << 4 | 1 << 7)
    V, E, F, T = r["counts"]
    assert V - E + F - T == 1


def _declared_functions():
    with open(os.path.join(ROOT, "include", "tetragpu.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(tg_[a-z_0-9]+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    import ctypes
    from tetragpu_gb300 import _build
    _build.build()
    lib = ctypes.CDLL(_build.LIB)
    names = _declared_functions()
    assert len(names) >= 12
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_constants_match_the_header():
    # relation bits, options and field types as the header defines them
    from tetragpu_gb300 import _lib
    with open(os.path.join(ROOT, "include", "tetragpu.h")) as f:
        src = f.read()
    defs = {}
    for name, val in re.findall(r"^#define (TG_[A-Z0-9_]+) (.+?)\s*(?:/\*.*)?$", src, re.M):
        m = re.fullmatch(r"\(1u? << (\d+)\)", val)
        defs[name] = 1 << int(m.group(1)) if m else int(val.rstrip("u"), 0)
    for i, name in enumerate(_lib.RELATIONS[1:], start=1):
        assert defs[f"TG_{name}"] == 1 << i, name
        assert _lib.REL[name] == i
    assert defs["TG_ALL_RELATIONS"] == _lib.ALL_RELATIONS
    assert defs["TG_OPT_TT_VERTEX_SHARING"] == _lib.OPT_TT_VERTEX_SHARING
    assert defs["TG_OPT_LINK_ADJACENCY"] == _lib.OPT_LINK_ADJACENCY
    assert (defs["TG_FIELD_F32"], defs["TG_FIELD_F64"]) == (_lib.FIELD_F32, _lib.FIELD_F64)


def test_library_loads_and_reports_without_gpu():
    import tetragpu_gb300 as tg
    assert "sm_103a" in tg.version()
    assert tg.kernel_launch_count() >= 0


def test_no_cpu_fallback_when_library_missing(tmp_path):
    from tetragpu_gb300 import _lib
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib._lib_backup = _lib._lib
        try:
            _lib._lib = None
            _lib.load(str(tmp_path / "libtetragpu.so"))
        finally:
            _lib._lib = _lib._lib_backup


def test_class_report_matches_the_reference_wording(tmp_path):
    """tg_export_classes (host only): the reference's totals, with its swapped
    labels, and the per-vertex lines its verifier reads."""
    import tetragpu_gb300 as tg
    from tetragpu_gb300 import _build
    if not os.path.exists(_build.LIB):
        pytest.skip("library not built")
    # (lower-link components, upper-link components, code)
    cls = np.array([[1, 0, 2],      # only lower neighbours: code 2, a true maximum
                    [0, 1, 1],      # code 1, a true minimum
                    [1, 1, 3],
                    [2, 2, 4],
                    [0, 0, 4],
                    [0, 1, 3]],     # disagrees with its counts: reported, still counted
                   dtype=np.uint32)
    path = tmp_path / "classes.txt"
    counts = tg.export_classes(cls, str(path), per_vertex_lines=True)
    assert counts == [0, 1, 1, 2, 2]
    lines = path.read_text().splitlines()
    assert lines[:6] == ["A 0 2", "A 1 1", "A 2 3", "A 3 4", "A 4 4", "A 5 3"]
    assert lines[6:] == ["Total number of minima:  1", "Total number of maxima:  1",
                         "Total number of saddles: 2", "Total number of regular: 2",
                         "Total number of voids:   0"]
