"""tg_critical_points_noalloc, the entry point for callers that cannot
allocate device memory (code running during stream capture, hosts that give
the library a fixed memory budget, real-time loops), called through the C
ABI.  Its classes must equal those of tg_critical_points, the allocating
entry point, bit for bit, on two calls in a row (the second call reuses the
shared scratch the first one left behind), and VV larger than its fixed
scratch must be rejected with TG_ERR_UNSUPPORTED before anything runs."""
import ctypes as C

import numpy as np
import pytest

from tetragpu_gb300 import meshgen

pytestmark = pytest.mark.gpu

TG_ERR_UNSUPPORTED = 5
MAX_VV_ENTRIES = 1 << 23


def _noalloc(lib):
    fn = lib.tg_critical_points_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_int,
                   C.c_void_p, C.c_void_p]
    return fn


def test_noalloc_matches_allocating_entry_point(gpu_lib):
    import torch
    m = meshgen.kuhn_mesh(12, 0.25, seed=41)
    fields = [meshgen.gaussian_mixture_field(m.coords, n_gauss=12, seed=42),
              meshgen.sine_field(m.coords, seed=43)]
    lib = gpu_lib.load()
    fn = _noalloc(lib)
    with gpu_lib.Mesh(m.tv, m.n_verts) as g:
        g.extract(["VV"])
        vv = g.device_relation("VV")
        out = torch.empty(3 * m.n_verts, dtype=torch.int32, device="cuda")
        for field in fields:
            want = g.critical_points(field)
            d_field = torch.from_numpy(field).cuda()
            torch.cuda.synchronize()
            rc = fn(vv["offsets"], vv["entries"], m.n_verts, vv["n_entries"],
                    d_field.data_ptr(), gpu_lib.FIELD_F32, out.data_ptr(), None)
            assert rc == 0, lib.tg_last_error_string().decode()
            got = out.cpu().numpy().view(np.uint32).reshape(-1, 3)
            assert np.array_equal(got, want)


def test_noalloc_rejects_vv_beyond_its_scratch(gpu_lib):
    import torch
    lib = gpu_lib.load()
    fn = _noalloc(lib)
    buf = torch.zeros(16, dtype=torch.int64, device="cuda")
    rc = fn(buf.data_ptr(), buf.data_ptr(), 1, MAX_VV_ENTRIES + 1, buf.data_ptr(),
            gpu_lib.FIELD_F32, buf.data_ptr(), None)
    assert rc == TG_ERR_UNSUPPORTED
    assert b"at most" in lib.tg_last_error_string()
