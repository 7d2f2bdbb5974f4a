"""Per-size-bucket tuning of the kernels' tile parameters.

    python -m tetragpu_gb300.tune [--apply] [--steps K]

The tile constants of the kernels (star-pass windows, block sizes of the
VT sort and the link adjacency, EE lanes per edge, slots per thread of the
edge-offset pass) are compile-time constants.  For every candidate setting
(the default and one change at a time from it) this builds a variant of
libtetragpu.so with -D overrides under tetragpu_gb300/_build/variants/, loads
it, and times the batched pipeline (tg_batch create + all 13 relations with
the link adjacency + critical points + destroy; CUDA events, L2 flushed
before every step) on each size bucket of the uneven 512-mesh batch (its
meshes grouped by tet count, each bucket run as a batch of its own) and on
the whole batch.  It records every time in tetragpu_gb300/tuning.json
together with the best setting of each bucket and the setting it selects:
the one with the smallest total over the buckets, with its margin to each
bucket's best.  --apply merges the selected change into the TUNED block of
csrc/tg_tuning.h (the settings the default build compiles in).

The batch runs as one disjoint-union mesh, so every kernel launches once per
batch with one setting; a setting per bucket applies to batches whose
members fall in one bucket, which is what the per-bucket rows measure.
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import _build

PKG = os.path.dirname(os.path.abspath(__file__))
VARIANTS = os.path.join(PKG, "_build", "variants")
TUNING_JSON = os.path.join(PKG, "tuning.json")
TUNING_H = os.path.join(PKG, "csrc", "tg_tuning.h")

# the setting compiled in now ("default": the TUNED block of csrc/tg_tuning.h
# over the defaults there) and one change at a time from it
CANDIDATES = [
    ("default", {}),
    ("star_b_win_192", {"TG_STAR_WIN_B": 192}),
    ("star_b_win_240", {"TG_STAR_WIN_B": 240}),
    ("star_b_win_256", {"TG_STAR_WIN_B": 256}),
    ("star_a_win_192", {"TG_STAR_WIN": 192}),
    ("efa_lanes_1", {"TG_EFA_LANES": 1}),
    ("ee_group_8", {"TG_EE_GROUP": 8}),
    ("adj_threads_64", {"TG_ADJ_THREADS": 64}),
    ("adj_threads_256", {"TG_ADJ_THREADS": 256}),
    ("vt_sort_threads_32", {"TG_VTS_THREADS": 32}),
    ("vt_sort_threads_128", {"TG_VTS_THREADS": 128}),
    ("edge_items_16", {"TG_EDGE_ITEMS": 16}),
]
# tet-count buckets of the batch's meshes: [lo, hi)
BUCKETS = [(2000, 20000), (20000, 100000), (100000, 400001)]


def bucket_batches():
    """The 512-mesh batch, and its meshes grouped by size bucket."""
    from . import meshgen
    meshes = meshgen.workload_batch()
    groups = [[m for m in meshes if lo <= m.n_cells < hi] for lo, hi in BUCKETS]
    return [("all", meshes)] + [(f"{lo}-{hi - 1}", g) for (lo, hi), g in zip(BUCKETS, groups)]


def _device_batch(torch, meshes):
    nc = np.array([m.n_cells for m in meshes], np.int64)
    nv = np.array([m.n_verts for m in meshes], np.int64)
    tv = torch.from_numpy(np.concatenate([m.tv for m in meshes])).cuda()
    f = torch.from_numpy(np.concatenate([m.field for m in meshes]).astype(np.float32)).cuda()
    cls = torch.empty(3 * int(nv.sum()), dtype=torch.int32, device="cuda")
    return nc, nv, tv, f, cls


def time_variant(torch, tg, batches, steps: int, warmup: int = 3) -> list:
    """ms per batched step, one value per batch."""
    stream = torch.cuda.Stream()
    s = stream.cuda_stream
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    out = []
    for _, (nc, nv, tv, f, cls) in batches:
        def step():
            with tg.Batch(tv.data_ptr(), nv, n_cells=nc, on_device=True, stream=s) as b:
                b.extract(tg.ALL_RELATIONS, options=tg.OPT_LINK_ADJACENCY, stream=s)
                b.critical_points(f.data_ptr(), on_device=True, out_ptr=cls.data_ptr(), stream=s)
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                step()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        with torch.cuda.stream(stream):
            for k in range(steps):
                flush.fill_(k & 0xff)
                ev[k][0].record(stream)
                step()
                ev[k][1].record(stream)
        torch.cuda.synchronize()
        out.append(sorted(a.elapsed_time(b) for a, b in ev)[steps // 2])   # median
    return out


def tuned_defines(path: str = TUNING_H) -> dict:
    """The settings the TUNED block of csrc/tg_tuning.h holds now."""
    with open(path) as fh:
        text = fh.read()
    block = text.split("// BEGIN TUNED\n", 1)[1].split("// END TUNED\n", 1)[0]
    out = {}
    for line in block.splitlines():
        parts = line.split()
        if len(parts) == 3 and parts[0] == "#define":
            out[parts[1]] = int(parts[2])
    return out


def write_header(defines: dict, path: str = TUNING_H):
    with open(path) as fh:
        text = fh.read()
    head, rest = text.split("// BEGIN TUNED\n", 1)
    _, tail = rest.split("// END TUNED\n", 1)
    body = "".join(f"#ifndef {k}\n#define {k} {v}\n#endif\n" for k, v in sorted(defines.items()))
    with open(path, "w") as fh:
        fh.write(head + "// BEGIN TUNED\n" + body + "// END TUNED\n" + tail)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--apply", action="store_true",
                    help="write the selected setting into csrc/tg_tuning.h")
    ap.add_argument("--only", default="", help="comma-separated candidate names")
    args = ap.parse_args(argv)
    import torch
    from . import _lib
    import tetragpu_gb300 as tg

    cands = [c for c in CANDIDATES if not args.only or c[0] in args.only.split(",")]
    t0 = time.time()
    built = {}
    for name, defs in cands:
        built[name] = _build.build(defines=defs, out_dir=os.path.join(VARIANTS, name))
    t_build = time.time() - t0
    groups = bucket_batches()
    batches = [(name, _device_batch(torch, ms)) for name, ms in groups if ms]
    results = {}
    for name, defs in cands:
        _lib._lib = None   # the next load() opens this variant's library
        _lib.load(built[name])
        results[name] = [round(x, 4) for x in time_variant(torch, tg, batches, args.steps)]
        print(name, results[name], flush=True)
    labels = [b[0] for b in batches]
    bucket_idx = [i for i, lab in enumerate(labels) if lab != "all"]
    best = {labels[i]: min(results, key=lambda n: results[n][i]) for i in range(len(labels))}
    selected = min(results, key=lambda n: sum(results[n][i] for i in bucket_idx))
    margin = {labels[i]: round(100.0 * (results[selected][i] / results[best[labels[i]]][i] - 1.0), 2)
              for i in range(len(labels))}
    rec = {
        "what": "ms per batched step (median of the timed steps): tg_batch create + all 13 "
                "relations with the link adjacency + critical points + destroy",
        "buckets": labels,
        "bucket_meshes": {name: len(ms) for name, ms in groups},
        "bucket_cells": {name: int(sum(m.n_cells for m in ms)) for name, ms in groups},
        "candidates": {name: defs for name, defs in cands},
        "results_ms": results,
        "best_per_bucket": best,
        "selected": selected,
        "selected_defines": dict(cands)[selected],
        "selected_margin_pct": margin,
        "steps": args.steps,
        "build_s": round(t_build, 1),
        "device": torch.cuda.get_device_name(0),
    }
    with open(TUNING_JSON, "w") as fh:
        json.dump(rec, fh, indent=1, sort_keys=True)
    print(json.dumps({"selected": selected, "margin_pct": margin, "best": best}))
    if args.apply:
        # every candidate is one change from the settings compiled in now (the
        # TUNED block; "default" is those settings): keep them, apply the change
        write_header({**tuned_defines(), **rec["selected_defines"]})
    return rec


if __name__ == "__main__":
    main()
