"""ctypes bindings for the CPU oracle.  TEST INFRASTRUCTURE ONLY.

* ``Oracle`` wraps liboracle.so, the C restatement in tg_oracle.c.
* ``Reference`` wraps _ref/libtgref.so, the reference's own CPU relation code
  compiled from its source tree by build_ref.sh (only where that tree exists).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline legs of bench.py
use this module, always as the checker or the timed CPU baseline, never as a
step of the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libtgref.so")

RELATIONS = ["validate", "TE", "EV", "ET", "TF", "FV", "FE", "FT", "EF", "VT",
             "TT", "FF", "EE", "VV"]
BIT = {name: i for i, name in enumerate(RELATIONS)}
ALL_MASK = sum(1 << i for i in range(1, 14))
FIXED_WIDTH = {"TE": 6, "EV": 2, "TF": 4, "FV": 3, "FE": 3, "FT": 2}
OPT_TT_VERTEX_SHARING = 0x1


class _Rel(C.Structure):
    _fields_ = [("n_rows", C.c_int64), ("n_entries", C.c_int64), ("width", C.c_int32),
                ("off", C.POINTER(C.c_int64)), ("ent", C.POINTER(C.c_int32))]


class _Result(C.Structure):
    _fields_ = [("n_verts", C.c_int64), ("n_edges", C.c_int64), ("n_faces", C.c_int64),
                ("n_cells", C.c_int64), ("rel", _Rel * 14)]


class _RefResult(C.Structure):
    _fields_ = [("n_edges", C.c_int64), ("n_faces", C.c_int64),
                ("te", C.POINTER(C.c_int32)), ("tf", C.POINTER(C.c_int32)),
                ("ev", C.POINTER(C.c_int32)), ("fv", C.POINTER(C.c_int32)),
                ("et_off", C.POINTER(C.c_int64)), ("vt_off", C.POINTER(C.c_int64)),
                ("vv_off", C.POINTER(C.c_int64)),
                ("et", C.POINTER(C.c_int32)), ("vt", C.POINTER(C.c_int32)),
                ("vv", C.POINTER(C.c_int32)), ("seconds", C.c_double)]


def build(force: bool = False) -> str:
    """Compile liboracle.so in place (gcc, a second or two)."""
    src = os.path.join(HERE, "tg_oracle.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])
    return LIB


def build_reference(ref_root: str | None = None) -> str | None:
    """Compile the reference's CPU code if its source tree is present.

    The tree is ``ref_root`` when given, else the ``TG_REFERENCE_ROOT``
    environment variable, else build_ref.sh's own default.  Returns None when
    no tree is found (the tests that need it skip)."""
    cmd = [os.path.join(HERE, "build_ref.sh")]
    if ref_root:
        cmd.append(ref_root)
    r = subprocess.run(cmd, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True)
    if r.returncode == 2:
        return None
    if r.returncode != 0:
        raise RuntimeError("build_ref.sh failed:\n" + r.stderr)
    return REF_LIB


def reference_root() -> str | None:
    """The reference source tree the last build_reference() compiled, if any."""
    p = os.path.join(HERE, "_ref", "reference_root")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        root = f.read().strip()
    return root if os.path.isdir(root) else None


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _copy(ptr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


class Oracle:
    def __init__(self, path: str = LIB):
        if not os.path.exists(path):
            build()
        lib = C.CDLL(path)
        lib.og_canonicalize.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p]
        lib.og_extract.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_uint32, C.c_uint32,
                                   C.POINTER(_Result)]
        lib.og_free.argtypes = [C.POINTER(_Result)]
        lib.og_critical_points.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p]
        lib.og_critical_points_f32.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p]
        lib.og_last_error.restype = C.c_char_p
        self.lib = lib

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(f"oracle error {rc}: {self.lib.og_last_error().decode()}")

    def canonicalize(self, tv: np.ndarray, n_verts: int) -> np.ndarray:
        tv = _i32(tv).reshape(-1, 4)
        out = np.empty_like(tv)
        self._check(self.lib.og_canonicalize(tv.ctypes.data, tv.shape[0], n_verts, out.ctypes.data))
        return out

    def extract(self, tvs: np.ndarray, n_verts: int, mask: int = ALL_MASK,
                options: int = 0) -> dict:
        """Relations of a row-sorted TV.  Returns {'counts': (V, E, F, T),
        name: array (fixed width, shape [rows, width]) or (offsets, entries)}."""
        tvs = _i32(tvs).reshape(-1, 4)
        res = _Result()
        self._check(self.lib.og_extract(tvs.ctypes.data, tvs.shape[0], n_verts, mask, options,
                                        C.byref(res)))
        try:
            out = {"counts": (res.n_verts, res.n_edges, res.n_faces, res.n_cells)}
            for i in range(1, 14):
                if not (mask >> i) & 1:
                    continue
                r = res.rel[i]
                ent = _copy(r.ent, r.n_entries, np.int32)
                if r.width > 0:
                    out[RELATIONS[i]] = ent.reshape(r.n_rows, r.width)
                else:
                    out[RELATIONS[i]] = (_copy(r.off, r.n_rows + 1, np.int64), ent)
            return out
        finally:
            self.lib.og_free(C.byref(res))

    def critical_points(self, tvs: np.ndarray, n_verts: int, field: np.ndarray) -> np.ndarray:
        """uint32 [V, 3]: (lower components, upper components, class code)."""
        tvs = _i32(tvs).reshape(-1, 4)
        out = np.zeros((n_verts, 3), dtype=np.uint32)
        if field.dtype == np.float32:
            f = np.ascontiguousarray(field, dtype=np.float32)
            rc = self.lib.og_critical_points_f32(tvs.ctypes.data, tvs.shape[0], n_verts,
                                                 f.ctypes.data, out.ctypes.data)
        else:
            f = np.ascontiguousarray(field, dtype=np.float64)
            rc = self.lib.og_critical_points(tvs.ctypes.data, tvs.shape[0], n_verts,
                                             f.ctypes.data, out.ctypes.data)
        self._check(rc)
        return out


class Reference:
    """The reference's own CPU path (cpu_extraction.cpp, validate.cpp)."""

    def __init__(self, path: str = REF_LIB):
        lib = C.CDLL(path)
        lib.ref_extract.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.POINTER(_RefResult)]
        lib.ref_free.argtypes = [C.POINTER(_RefResult)]
        lib.ref_validate.restype = C.c_uint32
        lib.ref_validate.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                                     C.c_void_p, C.c_void_p]
        self.lib = lib

    @staticmethod
    def available(path: str = REF_LIB) -> bool:
        return os.path.exists(path)

    def extract(self, tvs: np.ndarray, n_verts: int) -> dict:
        tvs = _i32(tvs).reshape(-1, 4)
        T = tvs.shape[0]
        r = _RefResult()
        self.lib.ref_extract(tvs.ctypes.data, T, n_verts, C.byref(r))
        try:
            E, F = r.n_edges, r.n_faces
            out = {
                "counts": (n_verts, E, F, T),
                "seconds": r.seconds,
                "TE": _copy(r.te, 6 * T, np.int32).reshape(T, 6),
                "TF": _copy(r.tf, 4 * T, np.int32).reshape(T, 4),
                "EV": _copy(r.ev, 2 * E, np.int32).reshape(E, 2),
                "FV": _copy(r.fv, 3 * F, np.int32).reshape(F, 3),
            }
            for name, off, ent, rows in (("ET", r.et_off, r.et, E), ("VT", r.vt_off, r.vt, n_verts),
                                         ("VV", r.vv_off, r.vv, n_verts)):
                o = _copy(off, rows + 1, np.int64)
                out[name] = (o, _copy(ent, int(o[-1]), np.int32))
            return out
        finally:
            self.lib.ref_free(C.byref(r))

    def validate(self, tvs, n_verts, rel: dict) -> int:
        """Run the reference's validate.cpp comparators on ``rel``; returns
        the bitmask of relations that failed (0 = all agree)."""
        tvs = _i32(tvs).reshape(-1, 4)
        te, tf, ev, fv = (_i32(rel[k]) for k in ("TE", "TF", "EV", "FV"))
        vo = np.ascontiguousarray(rel["VV"][0], dtype=np.int64)
        vv = _i32(rel["VV"][1])
        return int(self.lib.ref_validate(tvs.ctypes.data, tvs.shape[0], n_verts,
                                         te.ctypes.data, tf.ctypes.data, ev.ctypes.data,
                                         ev.shape[0], fv.ctypes.data, fv.shape[0],
                                         vo.ctypes.data, vv.ctypes.data))


def sort_rows(off: np.ndarray, ent: np.ndarray) -> np.ndarray:
    """Entries with every CSR row sorted ascending (vectorised)."""
    n = off.shape[0] - 1
    row = np.repeat(np.arange(n, dtype=np.int64), np.diff(off))
    order = np.lexsort((ent, row))
    return ent[order]
