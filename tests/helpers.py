"""Shared comparison helpers for the test-suite."""
from __future__ import annotations

import hashlib

import numpy as np

RELS = ["TE", "EV", "ET", "TF", "FV", "FE", "FT", "EF", "VT", "TT", "FF", "EE", "VV"]


def same(a, b) -> bool:
    if isinstance(a, tuple) or isinstance(b, tuple):
        return (isinstance(a, tuple) and isinstance(b, tuple) and np.array_equal(a[0], b[0])
                and np.array_equal(a[1], b[1]))
    return np.array_equal(a, b)


def digest(x) -> str:
    """sha256 of a relation's canonical bytes (offsets int64 then entries int32)."""
    h = hashlib.sha256()
    if isinstance(x, tuple):
        h.update(np.ascontiguousarray(x[0], dtype=np.int64).tobytes())
        h.update(np.ascontiguousarray(x[1], dtype=np.int32).tobytes())
    else:
        h.update(np.ascontiguousarray(x, dtype=np.int32).tobytes())
    return h.hexdigest()


def assert_relations_equal(got: dict, want: dict, names=RELS):
    bad = [n for n in names if n in want and not same(got[n], want[n])]
    assert not bad, f"relations differ: {bad}"


def gpu_extract_all(tg, tv, n_verts, options=0, names=RELS):
    with tg.Mesh(tv, n_verts) as g:
        g.extract(names, options=options)
        out = {n: g.relation(n) for n in names}
        out["counts"] = g.counts()
    return out
