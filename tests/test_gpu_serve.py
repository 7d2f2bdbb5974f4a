"""The serving loop (tg_server_*): requests that overlap on the device and
share batches give the same results as each mesh processed alone."""
import threading
import time

import numpy as np
import pytest

from helpers import RELS, same
from tetragpu_gb300 import meshgen

pytestmark = pytest.mark.gpu


def _mesh_pool(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        dims = tuple(int(x) for x in rng.integers(1, 7, size=3))
        m = meshgen.kuhn_mesh(dims, float(rng.uniform(0, 0.4)), seed=seed * 100 + i)
        m.field = rng.standard_normal(m.n_verts).astype(np.float32)
        out.append(m)
    return out


def _alone(gpu_lib, m, field):
    with gpu_lib.Mesh(m.tv, m.n_verts) as g:
        return g.critical_points(field)


def test_serve_mix_matches_alone(gpu_lib):
    meshes = _mesh_pool(24, 3)
    rng = np.random.default_rng(7)
    extra = {}  # request id -> (mesh index, field)
    submitted = []
    with gpu_lib.Server(n_slots=4, batch_cells=2000) as srv:
        def producer():
            for i, m in enumerate(meshes):
                rid, mid = srv.submit_mesh(m.tv, m.n_verts, m.field)
                submitted.append((rid, i, m.field, mid))
                if i % 3 == 2:  # a new field on an earlier mesh
                    j = int(rng.integers(0, i + 1))
                    f = rng.standard_normal(meshes[j].n_verts).astype(np.float32)
                    r2 = srv.submit_field(submitted[j][3], f)
                    extra[r2] = (j, f)
                time.sleep(float(rng.uniform(0, 0.002)))

        t = threading.Thread(target=producer)
        t.start()
        t.join()
        for rid, i, f, mid in submitted:
            cls, lat = srv.wait(rid)
            assert lat >= 0
            assert np.array_equal(cls, _alone(gpu_lib, meshes[i], f)), f"mesh {i}"
        for rid, (j, f) in extra.items():
            cls, _ = srv.wait(rid)
            assert np.array_equal(cls, _alone(gpu_lib, meshes[j], f)), f"field on mesh {j}"
        # relations of resident meshes, with each mesh's own ids
        for rid, i, f, mid in submitted[:4]:
            m = meshes[i]
            with gpu_lib.Mesh(m.tv, m.n_verts) as g:
                g.extract(RELS)
                for n in RELS:
                    assert same(srv.relation(mid, n), g.relation(n)), (i, n)
        st = srv.stats()
        assert st["completed"] == len(submitted) + len(extra) and st["failed"] == 0
        assert st["resident_meshes"] == len(meshes)


def test_serve_eviction_rebuilds(gpu_lib):
    meshes = _mesh_pool(6, 5)
    # a budget below any mesh: every finished batch is evicted by the next
    with gpu_lib.Server(n_slots=2, hbm_budget_bytes=1) as srv:
        ids = [srv.submit_mesh(m.tv, m.n_verts, m.field) for m in meshes]
        for (rid, _), m in zip(ids, meshes):
            cls, _ = srv.wait(rid)
            assert np.array_equal(cls, _alone(gpu_lib, m, m.field))
        rng = np.random.default_rng(9)
        for (rid, mid), m in zip(ids, meshes):
            f = rng.standard_normal(m.n_verts).astype(np.float32)
            cls, _ = srv.wait(srv.submit_field(mid, f))
            assert np.array_equal(cls, _alone(gpu_lib, m, f))
        st = srv.stats()
        assert st["evictions"] > 0 and st["meshes_built"] > len(meshes)


def test_serve_invalid_mesh_fails_alone(gpu_lib):
    good = _mesh_pool(2, 11)
    bad = meshgen.kuhn_mesh(2, 0.0, seed=12)
    bad.tv = bad.tv.copy()
    bad.tv[0, 0] = bad.n_verts + 5
    with gpu_lib.Server(n_slots=1) as srv:
        r0, _ = srv.submit_mesh(good[0].tv, good[0].n_verts, good[0].field)
        rb, _ = srv.submit_mesh(bad.tv, bad.n_verts, np.zeros(bad.n_verts, np.float32))
        r1, _ = srv.submit_mesh(good[1].tv, good[1].n_verts, good[1].field)
        assert np.array_equal(srv.wait(r0)[0], _alone(gpu_lib, good[0], good[0].field))
        with pytest.raises(gpu_lib.TetraGPUError) as ei:
            srv.wait(rb)
        assert ei.value.code == 2
        assert np.array_equal(srv.wait(r1)[0], _alone(gpu_lib, good[1], good[1].field))


def test_serve_released_mesh(gpu_lib):
    m = _mesh_pool(1, 13)[0]
    with gpu_lib.Server(n_slots=1) as srv:
        rid, mid = srv.submit_mesh(m.tv, m.n_verts, m.field)
        srv.wait(rid)
        srv.release(mid)
        with pytest.raises(gpu_lib.TetraGPUError):
            srv.submit_field(mid, m.field)
        assert srv.stats()["resident_meshes"] == 0
