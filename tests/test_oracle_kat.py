"""Hand-derived known answers for the CPU oracle, including the relations the
reference has no CPU code for (FE, FT, EF, TT, FF, EE), and its edge cases."""
import numpy as np
import pytest

from tetragpu_gb300 import meshgen


def rows(csr):
    off, ent = csr
    return [ent[off[i]:off[i + 1]].tolist() for i in range(len(off) - 1)]


@pytest.fixture(scope="module")
def two(oracle):
    tv = np.array([[0, 1, 2, 3], [1, 2, 3, 4]], np.int32)
    return oracle.extract(oracle.canonicalize(tv, 5), 5)


def test_two_tets_ids(two):
    # edges by first occurrence, pairs (0,1),(0,2),(0,3),(1,2),(1,3),(2,3)
    assert two["TE"].tolist() == [[0, 1, 2, 3, 4, 5], [3, 4, 6, 5, 7, 8]]
    assert two["EV"].tolist() == [[0, 1], [0, 2], [0, 3], [1, 2], [1, 3], [2, 3], [1, 4], [2, 4], [3, 4]]
    # faces visited with skip = 3,2,1,0: TF column order
    assert two["TF"].tolist() == [[0, 1, 2, 3], [3, 4, 5, 6]]
    assert two["FV"].tolist() == [[0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3], [1, 2, 4], [1, 3, 4], [2, 3, 4]]


def test_two_tets_restated_relations(two):
    # FE: edges (a,b), (a,c), (b,c) of face (a,b,c)
    assert two["FE"][3].tolist() == [3, 4, 5]       # face (1,2,3)
    assert two["FE"][0].tolist() == [0, 1, 3]       # face (0,1,2)
    assert two["FT"].tolist() == [[0, -1], [0, -1], [0, -1], [0, 1], [1, -1], [1, -1], [1, -1]]
    assert rows(two["TT"]) == [[1], [0]]
    assert rows(two["FF"])[3] == [0, 1, 2, 4, 5, 6]
    assert rows(two["FF"])[0] == [1, 2, 3]
    assert rows(two["EF"])[3] == [0, 3, 4]          # edge (1,2): faces (0,1,2),(1,2,3),(1,2,4)
    assert rows(two["ET"])[3] == [0, 1]
    assert rows(two["EE"])[0] == [1, 2, 3, 4, 6]    # edge (0,1)
    assert rows(two["VV"]) == [[1, 2, 3], [0, 2, 3, 4], [0, 1, 3, 4], [0, 1, 2, 4], [1, 2, 3]]
    assert rows(two["VT"]) == [[0], [0, 1], [0, 1], [0, 1], [1]]


def test_tt_vertex_sharing(oracle):
    tv = np.array([[0, 1, 2, 3], [1, 2, 3, 4], [4, 5, 6, 7], [8, 9, 10, 11]], np.int32)
    r = oracle.extract(tv, 12, mask=1 << 10, options=1)
    assert rows(r["TT"]) == [[1], [0, 2], [1], []]
    r = oracle.extract(tv, 12, mask=1 << 10, options=0)
    assert rows(r["TT"]) == [[1], [0], [], []]


def test_canonicalize_rejects(oracle):
    with pytest.raises(RuntimeError):
        oracle.canonicalize(np.array([[0, 1, 2, 9]], np.int32), 4)
    with pytest.raises(RuntimeError):
        oracle.canonicalize(np.array([[0, 1, 1, 2]], np.int32), 4)
    with pytest.raises(RuntimeError):
        oracle.canonicalize(np.array([[0, -1, 2, 3]], np.int32), 4)


def test_nonmanifold_face_rejected(oracle):
    tv = np.array([[0, 1, 2, 3], [0, 1, 2, 4], [0, 1, 2, 5]], np.int32)
    with pytest.raises(RuntimeError):
        oracle.extract(tv, 6)


def test_empty_and_isolated(oracle):
    r = oracle.extract(np.zeros((0, 4), np.int32), 3)
    assert r["counts"] == (3, 0, 0, 0)
    assert rows(r["VV"]) == [[], [], []]
    cp = oracle.critical_points(np.zeros((0, 4), np.int32), 3, np.zeros(3, np.float32))
    assert cp[:, 2].tolist() == [4, 4, 4]


@pytest.mark.parametrize("name", ["two_tets", "kuhn_cube", "coned_cube"])
def test_tiny_counts(oracle, name):
    m, counts = meshgen.tiny_meshes()[name]
    r = oracle.extract(oracle.canonicalize(m.tv, m.n_verts), m.n_verts, mask=1 << 1 | 1 << 4)
    assert r["counts"] == counts


def test_relation_identities(oracle):
    """Size identities every tetrahedral mesh satisfies."""
    m = meshgen.kuhn_mesh((4, 3, 5), 0.4, seed=17)
    r = oracle.extract(oracle.canonicalize(m.tv, m.n_verts), m.n_verts)
    V, E, F, T = r["counts"]
    assert V - E + F - T == 1                        # a ball
    assert r["ET"][0][-1] == 6 * T and r["VT"][0][-1] == 4 * T
    assert r["EF"][0][-1] == 3 * F and r["VV"][0][-1] == 2 * E
    interior = int((r["FT"][:, 1] >= 0).sum())
    assert r["TT"][0][-1] == 2 * interior
    assert r["FF"][0][-1] == 3 * (F + interior)
    deg = np.diff(r["VV"][0])
    assert r["EE"][0][-1] == int((deg[r["EV"][:, 0]] + deg[r["EV"][:, 1]] - 2).sum())
