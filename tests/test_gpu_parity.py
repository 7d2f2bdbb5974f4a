"""CUDA path (through the C ABI) against the CPU oracle: bit-exact on every
relation and on the critical-point classes."""
import numpy as np
import pytest

from helpers import RELS, assert_relations_equal, gpu_extract_all
from tetragpu_gb300 import meshgen

pytestmark = pytest.mark.gpu


def _check_mesh(tg, oracle, m, options=0):
    tvs = oracle.canonicalize(m.tv, m.n_verts)
    ref = oracle.extract(tvs, m.n_verts, options=options)
    got = gpu_extract_all(tg, m.tv, m.n_verts, options=options)
    assert got["counts"] == ref["counts"]
    assert_relations_equal(got, ref)
    return ref


@pytest.mark.parametrize("name", ["two_tets", "kuhn_cube", "coned_cube"])
def test_tiny_known_answers(gpu_lib, oracle, name):
    m, counts = meshgen.tiny_meshes()[name]
    ref = _check_mesh(gpu_lib, oracle, m)
    assert ref["counts"] == counts


def test_small_kuhn16(gpu_lib, oracle):
    _check_mesh(gpu_lib, oracle, meshgen.workload_small())


@pytest.mark.parametrize("seed,frac", [(3, 0.0), (4, 0.2), (5, 1.0)])
def test_coned_grids(gpu_lib, oracle, seed, frac):
    _check_mesh(gpu_lib, oracle, meshgen.kuhn_mesh((7, 5, 9), frac, seed=seed))


def test_tt_vertex_sharing(gpu_lib, oracle):
    m = meshgen.kuhn_mesh(5, 0.3, seed=9)
    tvs = oracle.canonicalize(m.tv, m.n_verts)
    ref = oracle.extract(tvs, m.n_verts, mask=1 << 10, options=1)
    with gpu_lib.Mesh(m.tv, m.n_verts) as g:
        g.extract(["TT"], options=gpu_lib.OPT_TT_VERTEX_SHARING)
        got = g.relation("TT")
    assert np.array_equal(got[0], ref["TT"][0]) and np.array_equal(got[1], ref["TT"][1])


def test_unsorted_rows_and_isolated_vertices(gpu_lib, oracle):
    # slots shuffled, plus 5 vertex ids that no cell uses
    m = meshgen.kuhn_mesh(3, 0.5, seed=21)
    m.n_verts += 5
    _check_mesh(gpu_lib, oracle, m)


def test_empty_mesh(gpu_lib):
    with gpu_lib.Mesh(np.zeros((0, 4), np.int32), 7) as g:
        g.extract(gpu_lib.ALL_RELATIONS)
        assert g.counts() == (7, 0, 0, 0)
        off, ent = g.relation("VV")
        assert np.array_equal(off, np.zeros(8, np.int64)) and ent.size == 0
        cp = g.critical_points(np.arange(7, dtype=np.float32))
        assert (cp[:, 2] == 4).all()
    with gpu_lib.Mesh(np.zeros((0, 4), np.int32), 7) as g:
        g.extract(gpu_lib.ALL_RELATIONS, options=gpu_lib.OPT_LINK_ADJACENCY)
        cp = g.critical_points(np.arange(7, dtype=np.float32))
        assert (cp[:, 2] == 4).all()


@pytest.mark.parametrize("bad,code", [([[0, 1, 2, 9]], 2), ([[0, 1, 1, 2]], 2), ([[0, -1, 2, 3]], 2)])
def test_invalid_meshes_rejected(gpu_lib, bad, code):
    with pytest.raises(gpu_lib.TetraGPUError) as ei:
        gpu_lib.Mesh(np.array(bad, np.int32), 4)
    assert ei.value.code == code


def test_nonmanifold_face_rejected(gpu_lib):
    tv = np.array([[0, 1, 2, 3], [0, 1, 2, 4], [0, 1, 2, 5]], np.int32)
    with gpu_lib.Mesh(tv, 6) as g:
        with pytest.raises(gpu_lib.TetraGPUError) as ei:
            g.extract(["TF"])
        assert ei.value.code == 2


def test_nonmanifold_vertex_star(gpu_lib, oracle):
    # two tets touching at one vertex: 6 neighbours around a 2-cell star,
    # beyond the manifold bound (cells + 2); the wide summary takes over
    tv = np.array([[0, 1, 2, 3], [0, 4, 5, 6]], np.int32)
    ref = oracle.extract(tv, 7)
    got = gpu_extract_all(gpu_lib, tv, 7)
    assert_relations_equal(got, ref)


def test_critical_points_small(gpu_lib, oracle):
    m = meshgen.workload_small()
    tvs = oracle.canonicalize(m.tv, m.n_verts)
    ref = oracle.critical_points(tvs, m.n_verts, m.field)
    with gpu_lib.Mesh(m.tv, m.n_verts) as g:
        got = g.critical_points(m.field)
        # second field on the same mesh reuses the cached link adjacency
        f2 = meshgen.sine_field(m.coords, seed=3)
        got2 = g.critical_points(f2.astype(np.float64))
    assert np.array_equal(got, ref)
    assert np.array_equal(got2, oracle.critical_points(tvs, m.n_verts, f2.astype(np.float64)))


def test_critical_points_ties_broken_by_id(gpu_lib, oracle):
    m = meshgen.kuhn_mesh(4, 0.25, seed=2)
    field = np.round(meshgen.gaussian_mixture_field(m.coords, n_gauss=4, seed=5) * 4) / 4
    tvs = oracle.canonicalize(m.tv, m.n_verts)
    with gpu_lib.Mesh(m.tv, m.n_verts) as g:
        got = g.critical_points(field.astype(np.float32))
    assert np.array_equal(got, oracle.critical_points(tvs, m.n_verts, field.astype(np.float32)))


@pytest.mark.parametrize("mesh", ["coned", "wide"])
def test_link_adjacency_prepared_during_extraction(gpu_lib, oracle, mesh):
    # the field-independent half of critical points built beside the last
    # extraction kernels (a side stream) gives the same relations and classes
    if mesh == "coned":
        m = meshgen.kuhn_mesh(10, 0.3, seed=11)
        tv, nv = m.tv, m.n_verts
        field = meshgen.gaussian_mixture_field(m.coords, n_gauss=6, seed=12).astype(np.float32)
    else:   # stars and VV rows beyond 32: the 64-bit masks
        rng = np.random.default_rng(13)
        tv, nv = _ring(40, rng=rng)
        field = rng.standard_normal(nv).astype(np.float32)
    tvs = oracle.canonicalize(tv, nv)
    ref = oracle.extract(tvs, nv)
    with gpu_lib.Mesh(tv, nv) as g:
        g.extract(gpu_lib.ALL_RELATIONS, options=gpu_lib.OPT_LINK_ADJACENCY)
        assert_relations_equal({n: g.relation(n) for n in RELS}, ref)
        got = g.critical_points(field)
        got2 = g.critical_points(-field)   # the prepared adjacency serves a second field
    assert np.array_equal(got, oracle.critical_points(tvs, nv, field))
    assert np.array_equal(got2, oracle.critical_points(tvs, nv, -field))


def test_irregular_full(gpu_lib, oracle):
    """The 64^3, 20%-coned workload: all 13 relations and critical points."""
    m = meshgen.workload_irregular()
    tvs = oracle.canonicalize(m.tv, m.n_verts)
    ref = oracle.extract(tvs, m.n_verts)
    ref_cp = oracle.critical_points(tvs, m.n_verts, m.field)
    with gpu_lib.Mesh(m.tv, m.n_verts) as g:
        g.extract(gpu_lib.ALL_RELATIONS)
        assert g.counts() == ref["counts"]
        for n in RELS:
            got = g.relation(n)
            want = ref[n]
            if isinstance(want, tuple):
                assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1]), n
            else:
                assert np.array_equal(got, want), n
        assert np.array_equal(g.critical_points(m.field), ref_cp)


def _fan(n_tets):
    # n_tets tets sharing only vertex 0 (faces all distinct: a valid mesh)
    tv = np.array([[0, 3 * i + 1, 3 * i + 2, 3 * i + 3] for i in range(n_tets)], np.int32)
    return tv, 3 * n_tets + 1


@pytest.mark.parametrize("n_tets", [70, 30])
def test_beyond_fast_path_limits_bit_exact(gpu_lib, oracle, n_tets):
    """70 cells around a vertex exceed the star passes' 64-cell masks (the
    heavy-star path takes it); 30 give 90 neighbours, beyond the 64 a link
    mask holds (the heavy EE and critical-point paths).  Every relation and
    the classes against the oracle, alone and inside a coned grid (the
    reference has no such bound, src/cpu_extraction.cpp:259-289)."""
    tv, nv = _fan(n_tets)
    rng = np.random.default_rng(n_tets)
    m = meshgen.Mesh(tv=tv, n_verts=nv, coords=np.zeros((nv, 3), np.float32), name="fan")
    _check_mesh(gpu_lib, oracle, m)
    grid = meshgen.kuhn_mesh(4, 0.3, seed=3)
    perm = rng.permutation(grid.n_verts + nv).astype(np.int32)
    both_tv = perm[np.concatenate([tv + grid.n_verts, grid.tv])]
    both = meshgen.Mesh(tv=both_tv, n_verts=grid.n_verts + nv,
                        coords=np.zeros((grid.n_verts + nv, 3), np.float32), name="fan+grid")
    _check_mesh(gpu_lib, oracle, both)
    field = rng.standard_normal(both.n_verts).astype(np.float32)
    tvs = oracle.canonicalize(both.tv, both.n_verts)
    with gpu_lib.Mesh(both.tv, both.n_verts) as g:
        assert np.array_equal(g.critical_points(field),
                              oracle.critical_points(tvs, both.n_verts, field))
    with gpu_lib.Mesh(both.tv, both.n_verts) as g:   # adjacency built during the extraction
        g.extract(gpu_lib.ALL_RELATIONS, options=gpu_lib.OPT_LINK_ADJACENCY)
        assert np.array_equal(g.critical_points(-field),
                              oracle.critical_points(tvs, both.n_verts, -field))


def test_large_mesh_properties(gpu_lib):
    """The 128^3 workload (12.6M tets): counts, size identities, sorted rows,
    symmetric VV and critical-point codes, checked without the oracle."""
    m = meshgen.workload_large()
    T, V = m.n_cells, m.n_verts
    with gpu_lib.Mesh(m.tv, V) as g:
        g.extract(gpu_lib.ALL_RELATIONS)
        v, e, f, t = g.counts()
        assert (v, e, f, t) == (2146689, 14827904, 25264128, 12582912)
        assert v - e + f - t == 1                      # a solid cube
        et_off, et = g.relation("ET")
        ef_off, _ = g.relation("EF")
        assert et_off[-1] == 6 * T and ef_off[-1] == 3 * f
        vt_off, vt = g.relation("VT")
        assert vt_off[-1] == 4 * T
        vv_off, vv = g.relation("VV")
        assert vv_off[-1] == 2 * e
        # rows ascending
        for off, ent in ((vv_off, vv), (vt_off, vt), (et_off, et)):
            d = np.diff(ent.astype(np.int64))
            starts = np.zeros(ent.size, bool)
            starts[off[1:-1][off[1:-1] < ent.size]] = True
            assert (d[~starts[1:]] > 0).all()
        # VV symmetric: (v, u) present iff (u, v)
        rows = np.repeat(np.arange(V, dtype=np.int64), np.diff(vv_off))
        fwd = rows * V + vv
        bwd = vv.astype(np.int64) * V + rows
        assert np.array_equal(np.sort(fwd), np.sort(bwd))
        te = g.relation("TE")
        assert te.min() == 0 and te.max() == e - 1
        ft = g.relation("FT")
        n_bnd = int((ft[:, 1] < 0).sum())
        assert n_bnd == 6 * 2 * 128 * 128              # two triangles per boundary square
        tt_off, _ = g.relation("TT")
        assert tt_off[-1] == 4 * T - n_bnd
        cp = g.critical_points(m.field)
        assert set(np.unique(cp[:, 2])) <= {1, 2, 3, 4}
        regular = cp[:, 2] == 3
        assert ((cp[regular, 0] == 1) & (cp[regular, 1] == 1)).all()


def test_int32_offset_copies_match(gpu_lib):
    """tg_copy_relation_i32: every CSR relation's offsets narrowed to int32
    equal the int64 ones, entries identical; fixed-width relations refused by
    the Python helper."""
    m = meshgen.kuhn_mesh((5, 4, 6), 0.3, seed=77)
    with gpu_lib.Mesh(m.tv, m.n_verts) as g:
        g.extract(gpu_lib.ALL_RELATIONS)
        for name in ("ET", "EF", "VT", "TT", "FF", "EE", "VV"):
            off64, ent64 = g.relation(name)
            off32, ent32 = g.relation_i32(name)
            assert off32.dtype == np.int32 and np.array_equal(off32.astype(np.int64), off64), name
            assert np.array_equal(ent32, ent64), name
        with pytest.raises(ValueError):
            g.relation_i32("TE")


def test_relations_copied_at_once_with_int32_offsets(gpu_lib):
    """tg_copy_relations_async_i32: all 13 relations in one call (one
    narrowing launch, then the copies) equal the per-relation int64 copies."""
    import ctypes as C
    import torch
    from tetragpu_gb300._lib import check
    m = meshgen.kuhn_mesh((4, 6, 5), 0.25, seed=78)
    with gpu_lib.Mesh(m.tv, m.n_verts) as g:
        g.extract(gpu_lib.ALL_RELATIONS)
        offs, ents = (C.c_void_p * 14)(), (C.c_void_p * 14)()
        got, mask = {}, 0
        for name in RELS:
            d = g.device_relation(name)
            r = gpu_lib.REL[name]
            mask |= 1 << r
            ent = np.empty(max(d["n_entries"], 1), dtype=np.int32)
            ents[r] = ent.ctypes.data
            off = None
            if d["width"] == 0:
                off = np.empty(d["rows"] + 1, dtype=np.int32)
                offs[r] = off.ctypes.data
            got[name] = (off, ent, d)
        check(g._lib.tg_copy_relations_async_i32(g._h, mask, offs, ents, None))
        torch.cuda.synchronize()
        for name, (off, ent, d) in got.items():
            want = g.relation(name)
            if d["width"] > 0:
                assert np.array_equal(ent[:d["n_entries"]].reshape(d["rows"], d["width"]), want), name
            else:
                assert np.array_equal(off.astype(np.int64), want[0]), name
                assert np.array_equal(ent[:d["n_entries"]], want[1]), name


def _ring(k, offset=0, rng=None):
    # k cells around the axis (v, c): cells (v, c, r_i, r_i+1), ring closed.
    # v and c lie in k cells with k + 1 neighbours each, the ring vertices in
    # two cells with four neighbours.  Vertex ids permuted when rng is given.
    v, c = 0, 1
    tv = np.array([[v, c, 2 + i, 2 + (i + 1) % k] for i in range(k)], np.int64)
    n = k + 2
    if rng is not None:
        perm = rng.permutation(n)
        tv = perm[tv]
        tv = rng.permuted(tv, axis=1)   # slots unsorted too
    return (tv + offset).astype(np.int32), n


@pytest.mark.parametrize("k", [33, 40, 63])
def test_wide_stars_and_long_rows(gpu_lib, oracle, k):
    """Stars of more than 32 cells and VV rows of more than 32 neighbours take
    the 64-bit star-position and link masks (narrower windows of the same
    mesh the 32-bit ones): every relation and the classes against the oracle,
    alone and next to a coned grid in one mesh."""
    rng = np.random.default_rng(k)
    tv, n = _ring(k, rng=rng)
    m = meshgen.Mesh(tv=tv, n_verts=n, coords=np.zeros((n, 3), np.float32), name=f"ring{k}")
    _check_mesh(gpu_lib, oracle, m)
    grid = meshgen.kuhn_mesh(3, 0.4, seed=k)
    tv2 = np.concatenate([grid.tv, tv + grid.n_verts])
    both = meshgen.Mesh(tv=tv2, n_verts=grid.n_verts + n,
                        coords=np.zeros((grid.n_verts + n, 3), np.float32), name="grid+ring")
    _check_mesh(gpu_lib, oracle, both)
    field = rng.standard_normal(both.n_verts).astype(np.float32)
    tvs = oracle.canonicalize(both.tv, both.n_verts)
    with gpu_lib.Mesh(both.tv, both.n_verts) as g:
        assert np.array_equal(g.critical_points(field),
                              oracle.critical_points(tvs, both.n_verts, field))
