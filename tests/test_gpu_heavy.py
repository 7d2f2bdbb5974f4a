"""Vertices beyond the fast paths' 64-bit masks, against the CPU oracle
through the C ABI: stars of more than 64 cells (tg_heavy.cu's share of the
star passes), more than 64 neighbours (heavy EE rows and critical points),
an edge in more than 255 cells (the widened ET / EF row lengths), several
heavy vertices sharing edges, inside larger meshes and in a batch.  The
reference's CPU path has no such bounds (src/cpu_extraction.cpp:259-289);
its critPoints kernel sizes blocks by the largest VV row
(src/cuda_extraction.cu:1160-1178)."""
import numpy as np
import pytest

from helpers import RELS, assert_relations_equal
from tetragpu_gb300 import meshgen

pytestmark = pytest.mark.gpu


def _ring(k, rng):
    # k cells around the axis (0, 1): both axis vertices in k cells with k + 1
    # neighbours, the axis edge in k cells; ids permuted, slots shuffled
    tv = np.array([[0, 1, 2 + i, 2 + (i + 1) % k] for i in range(k)], np.int64)
    n = k + 2
    perm = rng.permutation(n)
    tv = rng.permuted(perm[tv], axis=1)
    return tv.astype(np.int32), n


def _mesh(tv, n, name):
    return meshgen.Mesh(tv=tv, n_verts=n, coords=np.zeros((n, 3), np.float32), name=name)


def _union(parts, rng):
    """Disjoint union of (tv, n) parts, vertex ids permuted over the whole."""
    tvs, off = [], 0
    for tv, n in parts:
        tvs.append(tv + off)
        off += n
    perm = rng.permutation(off).astype(np.int32)
    return perm[np.concatenate(tvs)], off


def _check(tg, oracle, tv, n, seed):
    tvs = oracle.canonicalize(tv, n)
    ref = oracle.extract(tvs, n)
    field = np.random.default_rng(seed).standard_normal(n).astype(np.float32)
    ref_cp = oracle.critical_points(tvs, n, field)
    with tg.Mesh(tv, n) as g:
        g.extract(tg.ALL_RELATIONS, options=tg.OPT_LINK_ADJACENCY)
        assert g.counts() == ref["counts"]
        assert_relations_equal({r: g.relation(r) for r in RELS}, ref)
        assert np.array_equal(g.critical_points(field), ref_cp)
        f64 = -field.astype(np.float64)
        assert np.array_equal(g.critical_points(f64), oracle.critical_points(tvs, n, f64))
    return ref


@pytest.mark.parametrize("k", [65, 100, 300])
def test_heavy_ring(gpu_lib, oracle, k):
    rng = np.random.default_rng(k)
    tv, n = _ring(k, rng)
    ref = _check(gpu_lib, oracle, tv, n, k)
    et_off, _ = ref["ET"]
    assert np.diff(et_off).max() == k          # the axis edge lies in all k cells


def test_heavy_vertices_inside_a_grid(gpu_lib, oracle):
    """Heavy rings and fans next to a coned grid in one mesh: the star order
    puts the heavy vertices last, the windows of the light ones stop before
    them, the ids interleave."""
    rng = np.random.default_rng(7)
    grid = meshgen.kuhn_mesh((6, 5, 4), 0.3, seed=8)
    fan = np.array([[0, 3 * i + 1, 3 * i + 2, 3 * i + 3] for i in range(80)], np.int32)
    coned = meshgen.kuhn_mesh(3, 1.0, seed=9)
    parts = [(grid.tv, grid.n_verts), _ring(90, rng), (fan, 241), _ring(40, rng),
             (coned.tv, coned.n_verts)]
    tv, n = _union(parts, rng)
    # cells interleaved too: heavy stars' cells spread over the whole cell range
    tv = tv[rng.permutation(tv.shape[0])]
    _check(gpu_lib, oracle, tv, n, 11)


def test_heavy_in_batch_equals_alone(gpu_lib):
    rng = np.random.default_rng(12)
    meshes = [meshgen.kuhn_mesh(3, 0.2, seed=1), None, meshgen.kuhn_mesh(2, 0.5, seed=2)]
    tv, n = _ring(120, rng)
    meshes[1] = _mesh(tv, n, "ring120")
    fields = [np.random.default_rng(20 + i).standard_normal(m.n_verts).astype(np.float32)
              for i, m in enumerate(meshes)]
    with gpu_lib.Batch([m.tv for m in meshes], [m.n_verts for m in meshes]) as b:
        b.extract(gpu_lib.ALL_RELATIONS, options=gpu_lib.OPT_LINK_ADJACENCY)
        cp = b.critical_points(np.concatenate(fields))
        v0 = 0
        for i, m in enumerate(meshes):
            with gpu_lib.Mesh(m.tv, m.n_verts) as g:
                g.extract(gpu_lib.ALL_RELATIONS)
                for r in RELS:
                    got, want = b.relation(i, r), g.relation(r)
                    if isinstance(want, tuple):
                        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
                    else:
                        assert np.array_equal(got, want), (i, r)
                assert np.array_equal(cp[v0:v0 + m.n_verts], g.critical_points(fields[i]))
            v0 += m.n_verts
