"""The CPU oracle (oracle/tg_oracle.c) pinned against the reference's own CPU
code: live, against oracle/_ref/libtgref.so compiled from the reference tree
(skipped where that tree is absent), and always against the golden digests
in tests/golden/ that the reference build produced."""
import json
import os

import numpy as np
import pytest

from helpers import digest
from tetragpu_gb300 import meshgen

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
PINNED = ["TE", "EV", "ET", "TF", "FV", "VT", "VV"]


def _ref():
    from oracle.oracle import Reference, REF_LIB
    if not Reference.available():
        from oracle import oracle as O
        if O.build_reference() is None:
            pytest.skip("reference source tree not present")
    return Reference()


def _compare_live(oracle, ref, tv, n_verts):
    from oracle.oracle import sort_rows
    tvs = oracle.canonicalize(tv, n_verts)
    a = oracle.extract(tvs, n_verts)
    b = ref.extract(tvs, n_verts)
    assert a["counts"] == b["counts"]
    for k in ("TE", "TF", "EV", "FV"):
        assert np.array_equal(a[k], b[k]), k
    for k in ("ET", "VT"):
        assert np.array_equal(a[k][0], b[k][0]) and np.array_equal(a[k][1], b[k][1]), k
    # VV: the reference keeps first-encounter order; compare row-sorted
    assert np.array_equal(a["VV"][0], b["VV"][0])
    assert np.array_equal(a["VV"][1], sort_rows(*b["VV"]))
    return tvs, a


@pytest.mark.parametrize("name", ["two_tets", "kuhn_cube", "coned_cube"])
def test_tiny_against_reference(oracle, name):
    m, counts = meshgen.tiny_meshes()[name]
    ref = _ref()
    _, a = _compare_live(oracle, ref, m.tv, m.n_verts)
    assert a["counts"] == counts


@pytest.mark.parametrize("seed,frac,dims", [(1, 0.0, 6), (2, 0.2, (5, 7, 4)), (3, 1.0, 3)])
def test_grids_against_reference(oracle, seed, frac, dims):
    m = meshgen.kuhn_mesh(dims, frac, seed=seed)
    _compare_live(oracle, _ref(), m.tv, m.n_verts)


def test_reference_validators_accept_oracle(oracle):
    """The reference's validate.cpp comparators (TE, EV, TF, FV, VV, with
    VV sizes made strict) pass the oracle's relations."""
    m = meshgen.kuhn_mesh(4, 0.3, seed=8)
    ref = _ref()
    tvs, a = _compare_live(oracle, ref, m.tv, m.n_verts)
    assert ref.validate(tvs, m.n_verts, a) == 0


def test_reference_validators_catch_a_planted_error(oracle):
    m = meshgen.kuhn_mesh(3, 0.0, seed=8)
    ref = _ref()
    tvs = oracle.canonicalize(m.tv, m.n_verts)
    a = oracle.extract(tvs, m.n_verts)
    a["TE"] = a["TE"].copy()
    a["TE"][5, 2] = a["TE"][5, 3]          # plant a wrong edge id in the oracle output
    assert ref.validate(tvs, m.n_verts, a) & (1 << 1)


def test_unsorted_rows_break_reference_face_ids():
    """Why both paths sort rows first: the reference CPU face numbering on
    the same two tets with slots in another order mints an extra face."""
    ref = _ref()
    sorted_tv = np.array([[0, 1, 2, 3], [1, 2, 3, 4]], np.int32)
    shuffled = np.array([[0, 1, 2, 3], [3, 2, 4, 1]], np.int32)
    assert ref.extract(sorted_tv, 5)["counts"][2] == 7
    assert ref.extract(shuffled, 5)["counts"][2] == 8


def _golden_cases():
    with open(os.path.join(GOLDEN, "reference_digests.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("case", sorted(_golden_cases()))
def test_oracle_matches_golden_digests(oracle, case):
    g = _golden_cases()[case]
    d = np.load(os.path.join(GOLDEN, g["mesh"]))
    tv, n_verts = d["tv"], int(d["n_verts"])
    tvs = oracle.canonicalize(tv, n_verts)
    a = oracle.extract(tvs, n_verts)
    assert list(a["counts"]) == g["counts"]
    for k in PINNED:
        assert digest(a[k]) == g["digests"][k], k
