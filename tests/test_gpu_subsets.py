"""Relations requested alone or in small groups (through the C ABI) against
the CPU oracle: each relation's internal inputs (FV and FE read off TF and FT,
EF off ET and TF, the FF offsets computed with the FF rows, EE from the
id-sorted incident edges) are made as temporaries when only it is asked for,
and the result matches the full extraction bit for bit.  A mesh with heavy
stars takes the slow paths for the same subsets.  TE, EV, ET, TF, FV, VT and
VV follow the reference's own CPU code (oracle pinned to its build); FE, FT,
EF, TT, FF and EE are parity against the restatement (the reference has no
code for them)."""
import pytest

from helpers import RELS, assert_relations_equal
from tetragpu_gb300 import meshgen

pytestmark = pytest.mark.gpu

GROUPS = [[n] for n in RELS] + [["FV", "FF"], ["FE", "EF"], ["TE", "FT", "EE"],
                                ["EV", "TT", "VV"], ["ET", "FV", "FE"]]


def _heavy_mesh():
    """A coned grid plus a fan of 70 cells around one vertex (more than the
    64 cells a star takes on the fast path)."""
    import numpy as np
    m = meshgen.kuhn_mesh((5, 4, 6), 0.3, seed=21)
    n0 = m.n_verts
    hub, ring = n0, [n0 + 1 + i for i in range(71)]
    fan = [[hub, ring[i], ring[i + 1], n0 + 72] for i in range(70)]
    tv = np.concatenate([m.tv, np.array(fan, dtype=np.int32)])
    return tv, n0 + 73


@pytest.fixture(scope="module")
def meshes(oracle):
    out = []
    m = meshgen.kuhn_mesh((6, 5, 7), 0.25, seed=17)
    out.append((m.tv, m.n_verts))
    out.append(_heavy_mesh())
    return [(tv, nv, oracle.extract(oracle.canonicalize(tv, nv), nv)) for tv, nv in out]


@pytest.mark.parametrize("names", GROUPS, ids=["+".join(g) for g in GROUPS])
def test_subset_matches_oracle(gpu_lib, meshes, names):
    for tv, nv, ref in meshes:
        with gpu_lib.Mesh(tv, nv) as g:
            g.extract(names)
            got = {n: g.relation(n) for n in names}
        assert_relations_equal(got, ref, names)
