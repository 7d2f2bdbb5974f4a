#!/usr/bin/env python3
"""Generate the golden fixtures in this directory from the reference's own CPU
code (src/cpu_extraction.cpp of tlranda/TetraGPU, compiled from the reference
source tree by oracle/build_ref.sh).

For every case it stores the mesh (row-sorted int32 TV + vertex count) as a
compressed .npz, and in reference_digests.json the reference's edge/face
counts and the sha256 of each relation it computes (TE, EV, ET, TF, FV, VT,
and VV with rows sorted), over canonical bytes: fixed-width relations as
int32 row-major; CSR relations as int64 offsets followed by int32 entries.

Run from the repository root:  python tests/golden/make_golden.py [REF_ROOT]
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from helpers import digest  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tetragpu_gb300 import meshgen  # noqa: E402


def cases():
    out = {}
    for name, (m, _) in meshgen.tiny_meshes().items():
        out[name] = m
    out["kuhn16"] = meshgen.workload_small()
    out["kuhn_6x5x4_coned25"] = meshgen.kuhn_mesh((6, 5, 4), 0.25, seed=31)
    out["kuhn_3_coned100"] = meshgen.kuhn_mesh(3, 1.0, seed=32)
    return out


def main():
    # the reference tree: argv[1], else TG_REFERENCE_ROOT, else build_ref.sh's default
    ref_root = sys.argv[1] if len(sys.argv) > 1 else None
    if O.build_reference(ref_root) is None:
        sys.exit("reference source tree not found (pass it or set TG_REFERENCE_ROOT)")
    O.build()
    orc = O.Oracle()
    ref = O.Reference()
    digests = {}
    for name, m in cases().items():
        tvs = orc.canonicalize(m.tv, m.n_verts)
        fname = f"{name}.npz"
        np.savez_compressed(os.path.join(HERE, fname), tv=tvs, n_verts=np.int64(m.n_verts))
        r = ref.extract(tvs, m.n_verts)
        r["VV"] = (r["VV"][0], O.sort_rows(*r["VV"]))
        digests[name] = {
            "mesh": fname,
            "counts": [int(x) for x in r["counts"]],
            "digests": {k: digest(r[k]) for k in ("TE", "EV", "ET", "TF", "FV", "VT", "VV")},
        }
        print(name, r["counts"])
    with open(os.path.join(HERE, "reference_digests.json"), "w") as f:
        json.dump(digests, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
