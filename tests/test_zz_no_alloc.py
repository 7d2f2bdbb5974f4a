"""tg_critical_points_noalloc, the entry point for callers that cannot
allocate device memory when they classify (a host that gave the library a
fixed device-memory budget at start-up, a real-time loop that forbids
allocator calls once it runs), called through the C ABI.  Its classes must
equal those of tg_critical_points, the allocating entry point, bit for bit,
on two calls in a row (the second call reuses the shared scratch the first
one left behind), for float32 and float64 fields, on the legacy default
stream and on a stream of the caller's; VV larger than its fixed scratch
must be rejected with TG_ERR_UNSUPPORTED before anything runs, and so must a
vertex with more than 64 neighbours (its link masks do not fit)."""
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


@pytest.mark.parametrize("dtype,use_stream", [(np.float32, False), (np.float64, True)])
def test_noalloc_matches_allocating_entry_point(gpu_lib, dtype, use_stream):
    import torch
    m = meshgen.kuhn_mesh(12, 0.25, seed=41)
    fields = [meshgen.gaussian_mixture_field(m.coords, n_gauss=12, seed=42),
              meshgen.sine_field(m.coords, seed=43)]
    lib = gpu_lib.load()
    fn = _noalloc(lib)
    ftype = gpu_lib.FIELD_F32 if dtype == np.float32 else gpu_lib.FIELD_F64
    stream = torch.cuda.Stream() if use_stream else None
    handle = stream.cuda_stream if use_stream else None
    with gpu_lib.Mesh(m.tv, m.n_verts) as g:
        g.extract(["VV"])
        vv = g.device_relation("VV")
        out = torch.empty(3 * m.n_verts, dtype=torch.int32, device="cuda")
        for field in fields:
            field = field.astype(dtype)
            want = g.critical_points(field)
            d_field = torch.from_numpy(field).cuda()
            out.fill_(-1)
            torch.cuda.synchronize()
            rc = fn(vv["offsets"], vv["entries"], m.n_verts, vv["n_entries"],
                    d_field.data_ptr(), ftype, out.data_ptr(), handle)
            assert rc == 0, lib.tg_last_error_string().decode()
            torch.cuda.synchronize()
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


def test_noalloc_rejects_more_than_64_neighbours(gpu_lib):
    """A fan of 30 tets around vertex 0: 90 neighbours, beyond a 64-bit link
    mask.  The call reports it; a following call on a valid VV still works."""
    import torch
    lib = gpu_lib.load()
    fn = _noalloc(lib)
    k = 30
    n = 3 * k + 1
    rows = [list(range(1, n))]
    for i in range(k):
        a, b, c = 3 * i + 1, 3 * i + 2, 3 * i + 3
        rows += [[0, b, c], [0, a, c], [0, a, b]]
    off = np.concatenate([[0], np.cumsum([len(r) for r in rows])]).astype(np.int64)
    ent = np.concatenate([np.array(r, np.int32) for r in rows])
    d_off, d_ent = torch.from_numpy(off).cuda(), torch.from_numpy(ent).cuda()
    d_f = torch.from_numpy(np.arange(n, dtype=np.float32)).cuda()
    out = torch.empty(3 * n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = fn(d_off.data_ptr(), d_ent.data_ptr(), n, int(off[-1]), d_f.data_ptr(),
            gpu_lib.FIELD_F32, out.data_ptr(), None)
    assert rc == TG_ERR_UNSUPPORTED
    assert b"64 neighbours" in lib.tg_last_error_string()
    # the device and the scratch stay usable
    m = meshgen.kuhn_mesh(4, 0.3, seed=5)
    field = meshgen.gaussian_mixture_field(m.coords, n_gauss=4, seed=6)
    with gpu_lib.Mesh(m.tv, m.n_verts) as g:
        g.extract(["VV"])
        vv = g.device_relation("VV")
        want = g.critical_points(field)
        d_field = torch.from_numpy(field).cuda()
        out = torch.empty(3 * m.n_verts, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rc = fn(vv["offsets"], vv["entries"], m.n_verts, vv["n_entries"], d_field.data_ptr(),
                gpu_lib.FIELD_F32, out.data_ptr(), None)
        assert rc == 0, lib.tg_last_error_string().decode()
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy().view(np.uint32).reshape(-1, 3), want)
