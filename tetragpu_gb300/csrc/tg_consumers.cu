// tg_consumers.cu -- algorithm kernels that read resident relations in place
// through include/tetragpu_device.h, as a caller's own kernels would (the
// reference's aim for its relation kernels, src/cuda_extraction.cu:16-22).
//
//   tg_get_device_mesh  every resident relation's device pointers
//   tg_smooth_field     Laplacian smoothing of a vertex field over VV: each
//                       step replaces f[v] by the mean of f[v] and its
//                       neighbours' values (ping-pong between two buffers)
#include <algorithm>

#include "tetragpu.h"
#include "tetragpu_device.h"
#include "tg_internal.h"

namespace tg {
namespace {

__global__ void __launch_bounds__(256)
k_smooth(tg_device_mesh m, const float *__restrict__ in, float *__restrict__ out)
{
    griddep_wait();
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= m.n_verts) return;
    const int32_t n = tg_row_size(m.vv, v);
    const int32_t *nb = tg_row(m.vv, v);
    float s = in[v];
    for (int32_t i = 0; i < n; i++) s += in[nb[i]];
    out[v] = s / (float)(n + 1);
}

}  // namespace
}  // namespace tg

using namespace tg;

extern "C" tg_status tg_get_device_mesh(const tg_mesh *mesh, tg_device_mesh *out)
{
    if (!mesh || !out) {
        set_last_error("NULL argument");
        return TG_ERR_INVALID_ARGUMENT;
    }
    tg_device_mesh m{};
    tg_mesh_counts(mesh, &m.n_verts, &m.n_edges, &m.n_faces, &m.n_cells);
    tg_get_tv(mesh, &m.tv);
    auto fixed = [&](int r, tg_fixed_view &v) {
        const int64_t *off;
        const int32_t *ent;
        int64_t rows, n;
        int32_t w;
        if (tg_get_relation(mesh, r, &off, &ent, &rows, &n, &w) == TG_OK) v = {ent, rows, w};
    };
    auto csr = [&](int r, tg_csr_view &v) {
        const int64_t *off;
        const int32_t *ent;
        int64_t rows, n;
        int32_t w;
        if (tg_get_relation(mesh, r, &off, &ent, &rows, &n, &w) == TG_OK) v = {off, ent, rows};
    };
    fixed(TG_REL_TE, m.te);
    fixed(TG_REL_EV, m.ev);
    fixed(TG_REL_TF, m.tf);
    fixed(TG_REL_FV, m.fv);
    fixed(TG_REL_FE, m.fe);
    fixed(TG_REL_FT, m.ft);
    csr(TG_REL_ET, m.et);
    csr(TG_REL_EF, m.ef);
    csr(TG_REL_VT, m.vt);
    csr(TG_REL_TT, m.tt);
    csr(TG_REL_FF, m.ff);
    csr(TG_REL_EE, m.ee);
    csr(TG_REL_VV, m.vv);
    set_last_error("");   // relations not extracted are NULL, not an error
    *out = m;
    return TG_OK;
}

extern "C" tg_status tg_smooth_field(tg_mesh *mesh, const float *in, float *out, int iterations,
                                     float *scratch, void *stream)
{
    if (!mesh || !in || !out || iterations < 0 || (iterations > 1 && !scratch)) {
        set_last_error("NULL argument, negative iterations, or no scratch for more than one");
        return TG_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t s = (cudaStream_t)stream;
    tg_status st = tg_extract(mesh, TG_VV, 0, stream);   // no-op when VV is resident
    if (st != TG_OK) return st;
    tg_device_mesh m;
    tg_get_device_mesh(mesh, &m);
    const unsigned grid = (unsigned)std::max<int64_t>((m.n_verts + 255) / 256, 1);
    if (iterations == 0) {
        if (cudaMemcpyAsync(out, in, (size_t)m.n_verts * 4, cudaMemcpyDeviceToDevice, s) !=
            cudaSuccess) {
            (void)cudaGetLastError();
            set_last_error("cudaMemcpyAsync failed");
            return TG_ERR_CUDA;
        }
        return TG_OK;
    }
    // steps alternate between out and scratch so that the last one lands in out
    const float *src = in;
    for (int k = 0; k < iterations; k++) {
        float *dst = ((iterations - 1 - k) % 2 == 0) ? out : scratch;
        if (m.n_verts > 0) {
            Launch L("k_smooth", s);
            launch_pdl(k_smooth, grid, 256, 0, s, m, src, dst);
        }
        src = dst;
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(cudaGetErrorString(e));
        return TG_ERR_CUDA;
    }
    return TG_OK;
}
