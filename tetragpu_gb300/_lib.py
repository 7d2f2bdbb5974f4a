"""ctypes binding of libtetragpu.so (the C ABI in include/tetragpu.h).

There is no CPU fallback: if the library is missing or fails to load, every
call raises.  Build it with ``tetragpu_gb300._build.build()`` (nvcc,
sm_103a).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _build

RELATIONS = ["validate", "TE", "EV", "ET", "TF", "FV", "FE", "FT", "EF", "VT",
             "TT", "FF", "EE", "VV"]
REL = {name: i for i, name in enumerate(RELATIONS)}
ALL_RELATIONS = 0x3FFE
OPT_TT_VERTEX_SHARING = 0x1
OPT_LINK_ADJACENCY = 0x2
FIELD_F32, FIELD_F64 = 0, 1

STATUS = {0: "TG_OK", 1: "TG_ERR_INVALID_ARGUMENT", 2: "TG_ERR_INVALID_MESH", 3: "TG_ERR_CUDA",
          4: "TG_ERR_OUT_OF_MEMORY", 5: "TG_ERR_UNSUPPORTED", 6: "TG_ERR_NOT_COMPUTED",
          7: "TG_ERR_TIMEOUT"}


class TetraGPUError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


_lib = None


def mask_of(names) -> int:
    m = 0
    for n in names:
        m |= 1 << REL[n]
    return m


def load(path: str | None = None) -> C.CDLL:
    """Load libtetragpu.so from the package directory (raises if absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or _build.LIB
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with tetragpu_gb300._build.build() "
                           "(there is no CPU fallback)")
    lib = C.CDLL(path)
    vp, i64, i32, u32 = C.c_void_p, C.c_int64, C.c_int32, C.c_uint32
    P = C.POINTER
    sig = {
        "tg_version": (C.c_char_p, []),
        "tg_last_error_string": (C.c_char_p, []),
        "tg_mesh_create": (C.c_int, [vp, i64, i64, C.c_int, vp, P(vp)]),
        "tg_mesh_destroy": (C.c_int, [vp]),
        "tg_extract": (C.c_int, [vp, u32, u32, vp]),
        "tg_mesh_counts": (C.c_int, [vp, P(i64), P(i64), P(i64), P(i64)]),
        "tg_get_relation": (C.c_int, [vp, C.c_int, P(vp), P(vp), P(i64), P(i64), P(i32)]),
        "tg_copy_relation": (C.c_int, [vp, C.c_int, vp, vp, vp]),
        "tg_copy_relation_async": (C.c_int, [vp, C.c_int, vp, vp, vp]),
        "tg_copy_relation_async_i32": (C.c_int, [vp, C.c_int, vp, vp, vp]),
        "tg_copy_relation_i32": (C.c_int, [vp, C.c_int, vp, vp, vp]),
        "tg_copy_relations_async_i32": (C.c_int, [vp, u32, vp, vp, vp]),
        "tg_get_tv": (C.c_int, [vp, P(vp)]),
        "tg_export_relation_i64": (C.c_int, [vp, C.c_int, vp, vp, C.c_int, vp]),
        "tg_export_rows_padded": (C.c_int, [vp, C.c_int, i32, vp, vp, vp]),
        "tg_critical_points": (C.c_int, [vp, vp, C.c_int, C.c_int, vp, C.c_int, vp]),
        "tg_mesh_device_bytes": (i64, [vp]),
        "tg_kernel_launch_count": (i64, []),
        "tg_tuning_info": (C.c_char_p, []),
        "tg_tv_narrow_i64": (C.c_int, [vp, i64, i64, vp]),
        "tg_mesh_create_i64": (C.c_int, [vp, i64, i64, vp, P(vp)]),
        "tg_smooth_field": (C.c_int, [vp, vp, vp, C.c_int, vp, vp]),
        "tg_get_device_mesh": (C.c_int, [vp, vp]),
        "tg_profile_kernel": (C.c_int, [C.c_char_p]),
        "tg_profile_read": (C.c_int, [P(C.c_double), P(i64), C.c_int]),
        "tg_batch_create": (C.c_int, [vp, vp, vp, i64, C.c_int, vp, P(vp)]),
        "tg_batch_destroy": (C.c_int, [vp]),
        "tg_batch_extract": (C.c_int, [vp, u32, u32, vp]),
        "tg_batch_critical_points": (C.c_int, [vp, vp, C.c_int, C.c_int, vp, C.c_int, vp]),
        "tg_batch_mesh_counts": (C.c_int, [vp, i64, P(i64), P(i64), P(i64), P(i64)]),
        "tg_batch_mesh_offsets": (C.c_int, [vp, i64, P(i64), P(i64), P(i64), P(i64)]),
        "tg_batch_relation_size": (C.c_int, [vp, i64, C.c_int, P(i64), P(i64), P(i32)]),
        "tg_batch_copy_relation": (C.c_int, [vp, i64, C.c_int, vp, vp, vp]),
        "tg_batch_union": (vp, [vp]),
        "tg_export_classes": (C.c_int, [vp, i64, C.c_char_p, C.c_int, P(i64)]),
        "tg_server_create": (C.c_int, [C.c_int, vp, P(vp)]),
        "tg_server_destroy": (C.c_int, [vp]),
        "tg_server_submit_mesh": (C.c_int, [vp, vp, i64, i64, vp, C.c_int, P(i64), P(i64)]),
        "tg_server_submit_field": (C.c_int, [vp, i64, vp, C.c_int, P(i64)]),
        "tg_server_wait": (C.c_int, [vp, i64, i64, vp, P(C.c_double)]),
        "tg_server_relation_size": (C.c_int, [vp, i64, C.c_int, P(i64), P(i64), P(i32)]),
        "tg_server_copy_relation": (C.c_int, [vp, i64, C.c_int, vp, vp]),
        "tg_server_release_mesh": (C.c_int, [vp, i64]),
        "tg_server_get_stats": (C.c_int, [vp, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int):
    if rc != 0:
        raise TetraGPUError(rc, load().tg_last_error_string().decode())


def _stream(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return int(getattr(stream, "cuda_stream", stream))


class Mesh:
    """A mesh resident on the current CUDA device.

    ``tv`` is an int32 [n_cells, 4] numpy array (host) or a device pointer
    (int) with ``on_device=True``.
    """

    def __init__(self, tv, n_verts: int, n_cells: int | None = None, on_device: bool = False,
                 stream=None):
        lib = load()
        self._lib = lib
        self._h = C.c_void_p()
        if on_device:
            ptr = int(tv)
            assert n_cells is not None, "n_cells is required for a device pointer"
            keep = None
        else:
            keep = np.ascontiguousarray(tv, dtype=np.int32).reshape(-1, 4)
            ptr = keep.ctypes.data if keep.size else None
            n_cells = keep.shape[0]
        self.n_cells = int(n_cells)
        self.n_verts = int(n_verts)
        check(lib.tg_mesh_create(ptr, self.n_cells, self.n_verts, int(bool(on_device)),
                                 _stream(stream), C.byref(self._h)))

    def close(self):
        if self._h:
            self._lib.tg_mesh_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def extract(self, relations=ALL_RELATIONS, options: int = 0, stream=None):
        mask = relations if isinstance(relations, int) else mask_of(relations)
        check(self._lib.tg_extract(self._h, mask, options, _stream(stream)))
        return self

    def counts(self) -> tuple:
        v, e, f, t = (C.c_int64() for _ in range(4))
        check(self._lib.tg_mesh_counts(self._h, C.byref(v), C.byref(e), C.byref(f), C.byref(t)))
        return v.value, e.value, f.value, t.value

    def device_relation(self, name: str) -> dict:
        off, ent = C.c_void_p(), C.c_void_p()
        rows, n, width = C.c_int64(), C.c_int64(), C.c_int32()
        check(self._lib.tg_get_relation(self._h, REL[name], C.byref(off), C.byref(ent),
                                        C.byref(rows), C.byref(n), C.byref(width)))
        return {"offsets": off.value, "entries": ent.value, "rows": rows.value,
                "n_entries": n.value, "width": width.value}

    def relation(self, name: str, stream=None):
        """Host copy: [rows, width] array, or (offsets int64, entries int32)."""
        d = self.device_relation(name)
        ent = np.empty(d["n_entries"], dtype=np.int32)
        if d["width"] > 0:
            check(self._lib.tg_copy_relation(self._h, REL[name], None,
                                             ent.ctypes.data if ent.size else None, _stream(stream)))
            return ent.reshape(d["rows"], d["width"])
        off = np.empty(d["rows"] + 1, dtype=np.int64)
        check(self._lib.tg_copy_relation(self._h, REL[name], off.ctypes.data,
                                         ent.ctypes.data if ent.size else None, _stream(stream)))
        return off, ent

    def relation_i32(self, name: str):
        """Host copy of a CSR relation with int32 offsets (narrowed on the
        device): (offsets int32, entries int32)."""
        d = self.device_relation(name)
        if d["width"] > 0:
            raise ValueError(f"{name} is fixed-width: use relation()")
        off = np.empty(d["rows"] + 1, dtype=np.int32)
        ent = np.empty(d["n_entries"], dtype=np.int32)
        check(self._lib.tg_copy_relation_i32(self._h, REL[name], off.ctypes.data,
                                             ent.ctypes.data if ent.size else None, None))
        return off, ent

    def tv_sorted_ptr(self) -> int:
        p = C.c_void_p()
        check(self._lib.tg_get_tv(self._h, C.byref(p)))
        return p.value

    def critical_points(self, field, on_device: bool = False, out_ptr: int | None = None,
                        field_type: int | None = None, stream=None):
        """uint32 [V, 3] (lower comps, upper comps, class code); with
        ``out_ptr`` the result goes to device memory and None is returned."""
        if on_device:
            fptr = int(field)
            ftype = FIELD_F32 if field_type is None else field_type
        else:
            arr = np.ascontiguousarray(field)
            if arr.dtype == np.float64:
                ftype = FIELD_F64
            else:
                arr = arr.astype(np.float32, copy=False)
                ftype = FIELD_F32
            fptr = arr.ctypes.data
        if out_ptr is not None:
            check(self._lib.tg_critical_points(self._h, fptr, ftype, int(bool(on_device)),
                                               int(out_ptr), 1, _stream(stream)))
            return None
        out = np.empty((self.n_verts, 3), dtype=np.uint32)
        check(self._lib.tg_critical_points(self._h, fptr, ftype, int(bool(on_device)),
                                           out.ctypes.data, 0, _stream(stream)))
        return out

    def smooth_field(self, in_ptr: int, out_ptr: int, iterations: int = 1,
                     scratch_ptr: int | None = None, stream=None):
        """Laplacian smoothing over VV of a float32 device field
        (tg_smooth_field): device pointers in, out and (iterations > 1)
        scratch, n_verts floats each."""
        check(self._lib.tg_smooth_field(self._h, in_ptr, out_ptr, iterations, scratch_ptr,
                                        _stream(stream)))

    def device_bytes(self) -> int:
        return int(self._lib.tg_mesh_device_bytes(self._h))


class Batch:
    """Independent meshes processed as one (their disjoint union).

    ``tvs`` is a list of int32 [n_cells_i, 4] arrays, each with its own
    vertex ids 0 .. n_verts[i] - 1; or, with ``n_cells`` given, every cell
    back to back as one host int32 array, a host pointer (int), or with
    ``on_device=True`` a device pointer.
    """

    def __init__(self, tvs, n_verts, n_cells=None, on_device: bool = False, stream=None):
        lib = load()
        self._lib = lib
        self._h = C.c_void_p()
        nv = np.ascontiguousarray(n_verts, dtype=np.int64)
        if on_device or n_cells is not None:
            # all cells back to back: a device pointer, a host pointer, or a
            # host int32 array
            nc = np.ascontiguousarray(n_cells, dtype=np.int64)
            if isinstance(tvs, int):
                ptr = tvs
                keep = None
            else:
                keep = np.ascontiguousarray(tvs, dtype=np.int32)
                ptr = keep.ctypes.data if keep.size else None
        else:
            parts = [np.ascontiguousarray(t, dtype=np.int32).reshape(-1, 4) for t in tvs]
            nc = np.array([p.shape[0] for p in parts], dtype=np.int64)
            keep = np.concatenate(parts) if parts else np.zeros((0, 4), np.int32)
            ptr = keep.ctypes.data if keep.size else None
        assert nc.shape == nv.shape
        self.n_meshes = int(nv.shape[0])
        self.n_verts = nv
        self.n_cells = nc
        check(lib.tg_batch_create(ptr, nc.ctypes.data, nv.ctypes.data, self.n_meshes,
                                  int(bool(on_device)), _stream(stream), C.byref(self._h)))

    def close(self):
        if self._h:
            self._lib.tg_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def extract(self, relations=ALL_RELATIONS, options: int = 0, stream=None):
        mask = relations if isinstance(relations, int) else mask_of(relations)
        check(self._lib.tg_batch_extract(self._h, mask, options, _stream(stream)))
        return self

    def counts(self, i: int) -> tuple:
        v, e, f, t = (C.c_int64() for _ in range(4))
        check(self._lib.tg_batch_mesh_counts(self._h, i, C.byref(v), C.byref(e), C.byref(f),
                                             C.byref(t)))
        return v.value, e.value, f.value, t.value

    def offsets(self, i: int) -> tuple:
        """First (vertex, edge, face, cell) id of mesh i in the union."""
        v, e, f, t = (C.c_int64() for _ in range(4))
        check(self._lib.tg_batch_mesh_offsets(self._h, i, C.byref(v), C.byref(e), C.byref(f),
                                              C.byref(t)))
        return v.value, e.value, f.value, t.value

    def relation(self, i: int, name: str, stream=None):
        """Mesh i's relation with its own ids: [rows, width], or (offsets, entries)."""
        r = REL[name]
        rows, n, width = C.c_int64(), C.c_int64(), C.c_int32()
        check(self._lib.tg_batch_relation_size(self._h, i, r, C.byref(rows), C.byref(n),
                                               C.byref(width)))
        ent = np.empty(n.value, dtype=np.int32)
        if width.value > 0:
            check(self._lib.tg_batch_copy_relation(self._h, i, r, None,
                                                   ent.ctypes.data if ent.size else None,
                                                   _stream(stream)))
            return ent.reshape(rows.value, width.value)
        off = np.empty(rows.value + 1, dtype=np.int64)
        check(self._lib.tg_batch_copy_relation(self._h, i, r, off.ctypes.data,
                                               ent.ctypes.data if ent.size else None,
                                               _stream(stream)))
        return off, ent

    def critical_points(self, field, on_device: bool = False, out_ptr: int | None = None,
                        field_type: int | None = None, stream=None):
        """All meshes' classes back to back, uint32 [sum n_verts, 3]."""
        if on_device:
            fptr = int(field)
            ftype = FIELD_F32 if field_type is None else field_type
        else:
            arr = np.ascontiguousarray(field)
            if arr.dtype == np.float64:
                ftype = FIELD_F64
            else:
                arr = arr.astype(np.float32, copy=False)
                ftype = FIELD_F32
            fptr = arr.ctypes.data
        if out_ptr is not None:
            check(self._lib.tg_batch_critical_points(self._h, fptr, ftype, int(bool(on_device)),
                                                     int(out_ptr), 1, _stream(stream)))
            return None
        out = np.empty((int(self.n_verts.sum()), 3), dtype=np.uint32)
        check(self._lib.tg_batch_critical_points(self._h, fptr, ftype, int(bool(on_device)),
                                                 out.ctypes.data, 0, _stream(stream)))
        return out


class _ServerConfig(C.Structure):
    _fields_ = [("n_slots", C.c_int32), ("hbm_budget_bytes", C.c_int64),
                ("batch_cells", C.c_int64), ("relation_mask", C.c_uint32)]


class _ServerStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("submitted", "completed", "failed", "batches",
                                         "meshes_built", "evictions", "resident_meshes",
                                         "resident_bytes", "peak_bytes")]


class Server:
    """Request loop with continuous batching on one device (tg_server_*)."""

    def __init__(self, device: int = 0, n_slots: int = 4, hbm_budget_bytes: int = 150 * 10**9,
                 batch_cells: int = 4 * 1024 * 1024, relations=ALL_RELATIONS):
        lib = load()
        self._lib = lib
        self._h = C.c_void_p()
        mask = relations if isinstance(relations, int) else mask_of(relations)
        cfg = _ServerConfig(n_slots, hbm_budget_bytes, batch_cells, mask)
        check(lib.tg_server_create(device, C.byref(cfg), C.byref(self._h)))
        self._nv = {}

    def close(self):
        if self._h:
            self._lib.tg_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @staticmethod
    def _field(field):
        arr = np.ascontiguousarray(field)
        if arr.dtype != np.float64:
            arr = arr.astype(np.float32, copy=False)
        return arr, (FIELD_F64 if arr.dtype == np.float64 else FIELD_F32)

    def submit_mesh(self, tv, n_verts: int, field) -> tuple:
        """(request id, mesh id); TV and field are copied before returning."""
        tv = np.ascontiguousarray(tv, dtype=np.int32).reshape(-1, 4)
        f, ft = self._field(field)
        rid, mid = C.c_int64(), C.c_int64()
        check(self._lib.tg_server_submit_mesh(self._h, tv.ctypes.data if tv.size else None,
                                              tv.shape[0], int(n_verts),
                                              f.ctypes.data if f.size else None, ft,
                                              C.byref(rid), C.byref(mid)))
        self._nv[rid.value] = int(n_verts)
        self._nv[("mesh", mid.value)] = int(n_verts)
        return rid.value, mid.value

    def submit_field(self, mesh_id: int, field) -> int:
        f, ft = self._field(field)
        rid = C.c_int64()
        check(self._lib.tg_server_submit_field(self._h, mesh_id, f.ctypes.data if f.size else None,
                                               ft, C.byref(rid)))
        self._nv[rid.value] = self._nv.get(("mesh", mesh_id), f.shape[0])
        return rid.value

    def wait(self, request_id: int, timeout_ms: int = -1) -> tuple:
        """(classes uint32 [V, 3], latency ms)."""
        nv = self._nv.pop(request_id, 0)
        out = np.empty((nv, 3), dtype=np.uint32)
        lat = C.c_double()
        check(self._lib.tg_server_wait(self._h, request_id, timeout_ms,
                                       out.ctypes.data if out.size else None, C.byref(lat)))
        return out, lat.value

    def relation(self, mesh_id: int, name: str):
        r = REL[name]
        rows, n, width = C.c_int64(), C.c_int64(), C.c_int32()
        check(self._lib.tg_server_relation_size(self._h, mesh_id, r, C.byref(rows), C.byref(n),
                                                C.byref(width)))
        ent = np.empty(n.value, dtype=np.int32)
        if width.value > 0:
            check(self._lib.tg_server_copy_relation(self._h, mesh_id, r, None,
                                                    ent.ctypes.data if ent.size else None))
            return ent.reshape(rows.value, width.value)
        off = np.empty(rows.value + 1, dtype=np.int64)
        check(self._lib.tg_server_copy_relation(self._h, mesh_id, r, off.ctypes.data,
                                                ent.ctypes.data if ent.size else None))
        return off, ent

    def release(self, mesh_id: int):
        check(self._lib.tg_server_release_mesh(self._h, mesh_id))
        self._nv.pop(("mesh", mesh_id), None)

    def stats(self) -> dict:
        st = _ServerStats()
        check(self._lib.tg_server_get_stats(self._h, C.byref(st)))
        return {n: getattr(st, n) for n, _ in _ServerStats._fields_}


def export_classes(classes, path: str | None = None, per_vertex_lines: bool = False) -> list:
    """The reference's class report (see tg_export_classes); returns the
    vertex count per code 0..4."""
    cls = np.ascontiguousarray(classes, dtype=np.uint32).reshape(-1, 3)
    counts = (C.c_int64 * 5)()
    check(load().tg_export_classes(cls.ctypes.data if cls.size else None, cls.shape[0],
                                   path.encode() if path else None, int(per_vertex_lines), counts))
    return list(counts)


def kernel_launch_count() -> int:
    return int(load().tg_kernel_launch_count())


def profile_kernel(name: str | None):
    """Time every launch of the named kernel with CUDA events."""
    check(load().tg_profile_kernel(name.encode() if name else None))


def profile_read(reset: bool = True) -> tuple:
    """(total milliseconds, number of timed launches) since the last reset."""
    ms, n = C.c_double(), C.c_int64()
    check(load().tg_profile_read(C.byref(ms), C.byref(n), int(reset)))
    return ms.value, n.value


def tuning_info() -> dict:
    """The tile parameters the kernels use (tg_tuning_info)."""
    import json
    return json.loads(load().tg_tuning_info().decode())


def batch_tuning() -> dict:
    """How the batched path is tuned: the tile parameters compiled in, and the
    sweep that chose them (tetragpu_gb300/tuning.json, written by
    python -m tetragpu_gb300.tune) when it exists."""
    import json
    d = {"compiled": tuning_info()}
    p = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning.json")
    if os.path.exists(p):
        with open(p) as f:
            rec = json.load(f)
        d.update({"sweep": "tetragpu_gb300/tuning.json", "selected": rec.get("selected"),
                  "selected_defines": rec.get("selected_defines"),
                  "best_per_bucket": rec.get("best_per_bucket"),
                  "selected_margin_pct": rec.get("selected_margin_pct")})
    else:
        d["sweep"] = None
    return d


def version() -> str:
    return load().tg_version().decode()
