"""Batches of meshes (their disjoint union through one pipeline run) against
the same meshes one at a time: every relation and the critical-point classes
bit-exact per mesh, with each mesh's own ids."""
import numpy as np
import pytest

from helpers import RELS, assert_relations_equal, gpu_extract_all, same
from tetragpu_gb300 import meshgen

pytestmark = pytest.mark.gpu


def _meshes():
    out = [m for m, _ in meshgen.tiny_meshes().values()]
    out.append(meshgen.kuhn_mesh((4, 3, 5), 0.3, seed=11))
    out.append(meshgen.kuhn_mesh(6, 0.0, seed=12))
    iso = meshgen.kuhn_mesh(3, 0.5, seed=13)
    iso.n_verts += 4                       # vertices no cell uses
    out.append(iso)
    out.append(meshgen.Mesh(tv=np.zeros((0, 4), np.int32), n_verts=3,
                            coords=np.zeros((3, 3), np.float32), name="empty"))
    out.append(meshgen.kuhn_mesh((2, 7, 3), 1.0, seed=14))
    rng = np.random.default_rng(5)
    for m in out:
        m.field = rng.standard_normal(m.n_verts).astype(np.float32)
    return out


def test_batch_matches_single_meshes(gpu_lib):
    meshes = _meshes()
    with gpu_lib.Batch([m.tv for m in meshes], [m.n_verts for m in meshes]) as b:
        b.extract(gpu_lib.ALL_RELATIONS)
        classes = b.critical_points(np.concatenate([m.field for m in meshes]))
        v0 = 0
        for i, m in enumerate(meshes):
            want = gpu_extract_all(gpu_lib, m.tv, m.n_verts)
            got = {n: b.relation(i, n) for n in RELS}
            assert b.counts(i) == want["counts"], m.name
            assert_relations_equal(got, want)
            with gpu_lib.Mesh(m.tv, m.n_verts) as g:
                cp = g.critical_points(m.field)
            assert np.array_equal(classes[v0:v0 + m.n_verts], cp), m.name
            v0 += m.n_verts


def test_batch_against_oracle(gpu_lib, oracle):
    meshes = [meshgen.kuhn_mesh((5, 4, 3), 0.25, seed=31), meshgen.workload_small()]
    with gpu_lib.Batch([m.tv for m in meshes], [m.n_verts for m in meshes]) as b:
        b.extract(gpu_lib.ALL_RELATIONS)
        for i, m in enumerate(meshes):
            tvs = oracle.canonicalize(m.tv, m.n_verts)
            ref = oracle.extract(tvs, m.n_verts)
            got = {n: b.relation(i, n) for n in RELS}
            assert b.counts(i) == ref["counts"]
            assert_relations_equal(got, ref)


def test_batch_offsets_are_the_union_ids(gpu_lib):
    meshes = _meshes()[:4]
    with gpu_lib.Batch([m.tv for m in meshes], [m.n_verts for m in meshes]) as b:
        b.extract(["TE", "TF"])
        e_prev = f_prev = 0
        for i, m in enumerate(meshes):
            v0, e0, f0, c0 = b.offsets(i)
            assert (e0, f0) == (e_prev, f_prev)
            _, ne, nf, _ = b.counts(i)
            e_prev, f_prev = e0 + ne, f0 + nf
            te = b.relation(i, "TE")
            assert te.size == 0 or (te.min() == 0 and te.max() == ne - 1)


def test_batch_vertex_sharing_tt(gpu_lib):
    meshes = [meshgen.kuhn_mesh(3, 0.3, seed=41), meshgen.kuhn_mesh((2, 3, 2), 0.0, seed=42)]
    with gpu_lib.Batch([m.tv for m in meshes], [m.n_verts for m in meshes]) as b:
        b.extract(["TT"], options=gpu_lib.OPT_TT_VERTEX_SHARING)
        for i, m in enumerate(meshes):
            with gpu_lib.Mesh(m.tv, m.n_verts) as g:
                g.extract(["TT"], options=gpu_lib.OPT_TT_VERTEX_SHARING)
                assert same(b.relation(i, "TT"), g.relation("TT"))


def test_batch_rejects_an_id_outside_its_mesh(gpu_lib):
    a = meshgen.kuhn_mesh(2, 0.0, seed=51)
    bad = meshgen.kuhn_mesh(2, 0.0, seed=52)
    bad.tv = bad.tv.copy()
    bad.tv[3, 1] = bad.n_verts            # valid in the union, not in its mesh
    with pytest.raises(gpu_lib.TetraGPUError) as ei:
        gpu_lib.Batch([a.tv, bad.tv], [a.n_verts, bad.n_verts])
    assert ei.value.code == 2


def test_batch_of_nothing(gpu_lib):
    with gpu_lib.Batch([], []) as b:
        b.extract(gpu_lib.ALL_RELATIONS)
        assert b.n_meshes == 0


def test_uneven_batch_matches_meshes_alone(gpu_lib):
    """Forty meshes from the uneven-batch generator (sizes log-uniform, 0-30%
    coned, ids permuted): every mesh's relations and classes from the batch
    equal the mesh processed alone, compared by digest."""
    from helpers import digest
    meshes = meshgen.workload_batch(n_meshes=40, lo=2000, hi=60000, seed=91)
    field = np.concatenate([m.field for m in meshes])
    with gpu_lib.Batch([m.tv for m in meshes], [m.n_verts for m in meshes]) as b:
        b.extract(gpu_lib.ALL_RELATIONS)
        classes = b.critical_points(field)
        v0 = 0
        for i, m in enumerate(meshes):
            with gpu_lib.Mesh(m.tv, m.n_verts) as g:
                g.extract(gpu_lib.ALL_RELATIONS)
                for n in RELS:
                    assert digest(b.relation(i, n)) == digest(g.relation(n)), (i, n)
                assert np.array_equal(classes[v0:v0 + m.n_verts], g.critical_points(m.field))
            v0 += m.n_verts
