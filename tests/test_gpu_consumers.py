"""Relations read in place by an algorithm kernel (include/tetragpu_device.h,
the reference's aim in src/cuda_extraction.cu:16-22): tg_smooth_field walks
the resident VV rows through the device accessors.  Checked against the same
smoothing computed on the host from the oracle's VV, and the device mesh's
pointers against tg_get_relation."""
import ctypes as C

import numpy as np
import pytest

from tetragpu_gb300 import meshgen

pytestmark = pytest.mark.gpu


class _Csr(C.Structure):
    _fields_ = [("off", C.c_void_p), ("ent", C.c_void_p), ("rows", C.c_int64)]


class _Fixed(C.Structure):
    _fields_ = [("ent", C.c_void_p), ("rows", C.c_int64), ("width", C.c_int32)]


class _DeviceMesh(C.Structure):
    _fields_ = [("n_verts", C.c_int64), ("n_edges", C.c_int64), ("n_faces", C.c_int64),
                ("n_cells", C.c_int64), ("tv", C.c_void_p),
                ("te", _Fixed), ("ev", _Fixed), ("tf", _Fixed), ("fv", _Fixed), ("fe", _Fixed),
                ("ft", _Fixed),
                ("et", _Csr), ("ef", _Csr), ("vt", _Csr), ("tt", _Csr), ("ff", _Csr),
                ("ee", _Csr), ("vv", _Csr)]


def _smooth_host(off, ent, f, iterations):
    deg = np.diff(off)
    rows = np.repeat(np.arange(len(deg)), deg)
    for _ in range(iterations):
        s = f.astype(np.float32).copy()
        np.add.at(s, rows, f[ent])
        f = (s / (deg + 1).astype(np.float32)).astype(np.float32)
    return f


@pytest.mark.parametrize("iterations", [1, 4])
def test_smooth_field_reads_vv_in_place(gpu_lib, oracle, iterations):
    import torch
    m = meshgen.kuhn_mesh((6, 5, 4), 0.3, seed=15)
    f = meshgen.gaussian_mixture_field(m.coords, n_gauss=5, seed=16).astype(np.float32)
    tvs = oracle.canonicalize(m.tv, m.n_verts)
    off, ent = oracle.extract(tvs, m.n_verts, mask=1 << 13)["VV"]
    want = _smooth_host(off, ent, f, iterations)
    d_in = torch.from_numpy(f).cuda()
    d_out = torch.empty_like(d_in)
    d_tmp = torch.empty_like(d_in)
    with gpu_lib.Mesh(m.tv, m.n_verts) as g:
        g.smooth_field(d_in.data_ptr(), d_out.data_ptr(), iterations, d_tmp.data_ptr())
        torch.cuda.synchronize()
    # the same sums in a possibly different order: float32 rounding only
    np.testing.assert_allclose(d_out.cpu().numpy(), want, rtol=1e-5, atol=1e-6)


def test_device_mesh_points_at_resident_relations(gpu_lib):
    m = meshgen.kuhn_mesh(4, 0.2, seed=17)
    with gpu_lib.Mesh(m.tv, m.n_verts) as g:
        g.extract(["TE", "VV", "ET"])
        dm = _DeviceMesh()
        gpu_lib._lib.check(g._lib.tg_get_device_mesh(g._h, C.byref(dm)))
        assert (dm.n_verts, dm.n_edges, dm.n_faces, dm.n_cells) == g.counts()
        assert dm.te.ent == g.device_relation("TE")["entries"] and dm.te.width == 6
        vv = g.device_relation("VV")
        assert dm.vv.off == vv["offsets"] and dm.vv.ent == vv["entries"]
        assert dm.vv.rows == m.n_verts
        assert dm.ff.off is None and dm.ff.ent is None      # not extracted
        assert dm.tv == g.tv_sorted_ptr()
