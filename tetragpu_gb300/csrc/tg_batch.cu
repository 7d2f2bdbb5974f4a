// tg_batch.cu -- batches of independent meshes as one disjoint union.
//
// The union of meshes with disjoint vertex ranges is itself a mesh, and the
// relation ids are ranks of first occurrences in cell order, so with mesh i's
// cells contiguous at [c0_i, c1_i) and its vertices renumbered to
// [v0_i, v1_i), the union's relations restricted to mesh i are mesh i's own
// relations shifted by (v0_i, e0_i, f0_i, c0_i): its edges are ids
// [e0_i, e1_i) with e0_i the rank of the first occurrence slot 6 * c0_i, and
// likewise for faces.  One run of the pipeline then serves every mesh: each
// kernel launches once over all of them.  Per-mesh results are cut out and
// shifted back on the way out.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "tg_internal.h"

namespace tg {
namespace {

// add each cell's mesh vertex offset; a local id outside the mesh becomes -1
// (which mesh creation rejects as out of range)
__global__ void __launch_bounds__(256)
k_batch_shift(const int4 *__restrict__ tv, int64_t T, const int64_t *__restrict__ seg_c,
              const int64_t *__restrict__ seg_v, int64_t n, int4 *__restrict__ out)
{
    griddep_wait();
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= T) return;
    int64_t lo = 0, hi = n;  // last i with seg_c[i] <= c
    while (hi - lo > 1) {
        const int64_t mid = (lo + hi) >> 1;
        if (seg_c[mid] <= c) lo = mid; else hi = mid;
    }
    const int64_t v0 = seg_v[lo], nv = seg_v[lo + 1] - v0;
    int4 w = tv[c];
    w.x = (w.x >= 0 && w.x < nv) ? (int)(w.x + v0) : -1;
    w.y = (w.y >= 0 && w.y < nv) ? (int)(w.y + v0) : -1;
    w.z = (w.z >= 0 && w.z < nv) ? (int)(w.z + v0) : -1;
    w.w = (w.w >= 0 && w.w < nv) ? (int)(w.w + v0) : -1;
    out[c] = w;
}

// dst = src - shift, negative entries (FT's missing second cell) kept
__global__ void __launch_bounds__(256)
k_rebase32(const int *__restrict__ src, int64_t n, int shift, int *__restrict__ dst)
{
    griddep_wait();
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int x = src[k];
    dst[k] = x < 0 ? x : x - shift;
}

__global__ void __launch_bounds__(256)
k_rebase64(const int64_t *__restrict__ src, int64_t n, int64_t shift, int64_t *__restrict__ dst)
{
    griddep_wait();
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    dst[k] = src[k] - shift;
}

unsigned blocks(int64_t n) { return (unsigned)((n + 255) / 256); }

}  // namespace
}  // namespace tg

using namespace tg;

struct tg_batch {
    tg_mesh *u = nullptr;
    int device = 0;
    int64_t n = 0;
    std::vector<int64_t> c0, v0;  // n + 1 cell / vertex starts
    std::vector<int64_t> e0, f0;  // n + 1 edge / face starts, once read back
    bool ids_read = false;
    cudaStream_t s = nullptr;     // stream of the last extraction
    std::mutex mu;
};

namespace {

tg_status bfail(tg_status code, const char *msg)
{
    set_last_error(msg);
    return code;
}

#define TRY_B(call)                                                                 \
    do {                                                                            \
        tg_status t_ = (call);                                                      \
        if (t_ != TG_OK) return t_;                                                 \
    } while (0)

#define BCK(call)                                                                   \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess) {                                                    \
            set_last_error(cudaGetErrorString(e_));                                 \
            return TG_ERR_CUDA;                                                     \
        }                                                                           \
    } while (0)

// rows and value spaces of each relation: 0 vertices, 1 edges, 2 faces, 3 cells
const int kRowSpace[14] = {0, 3, 1, 1, 3, 2, 2, 2, 1, 0, 3, 2, 1, 0};
const int kValSpace[14] = {0, 1, 0, 3, 2, 0, 1, 3, 2, 3, 3, 2, 1, 0};

// first edge / face ids of every mesh, read back once per extraction
tg_status ensure_ids(tg_batch *b)
{
    if (b->ids_read) return TG_OK;
    int64_t E = -1;
    tg_mesh_counts(b->u, nullptr, &E, nullptr, nullptr);
    const int64_t *d = mesh_segment_ids(b->u);
    if (E < 0 || !d) return bfail(TG_ERR_NOT_COMPUTED, "the batch's edges have not been extracted");
    std::vector<int64_t> h(2 * (b->n + 1));
    BCK(cudaMemcpyAsync(h.data(), d, h.size() * 8, cudaMemcpyDeviceToHost, b->s));
    BCK(cudaStreamSynchronize(b->s));
    b->e0.assign(h.begin(), h.begin() + b->n + 1);
    b->f0.assign(h.begin() + b->n + 1, h.end());
    b->ids_read = true;
    return TG_OK;
}

bool uses_ids(int r)
{
    return kRowSpace[r] == 1 || kRowSpace[r] == 2 || kValSpace[r] == 1 || kValSpace[r] == 2;
}

const std::vector<int64_t> &space(const tg_batch *b, int sp)
{
    return sp == 0 ? b->v0 : (sp == 1 ? b->e0 : (sp == 2 ? b->f0 : b->c0));
}

}  // namespace

extern "C" {

tg_status tg_batch_create(const int32_t *tv, const int64_t *n_cells, const int64_t *n_verts,
                          int64_t n_meshes, int tv_on_device, void *stream, tg_batch **out)
{
    if (!out) return bfail(TG_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (n_meshes < 0 || (n_meshes > 0 && (!n_cells || !n_verts)))
        return bfail(TG_ERR_INVALID_ARGUMENT, "bad mesh count or NULL count arrays");
    cudaStream_t s = (cudaStream_t)stream;
    tg_batch *b = new tg_batch;
    b->n = n_meshes;
    b->s = s;
    b->c0.assign(n_meshes + 1, 0);
    b->v0.assign(n_meshes + 1, 0);
    for (int64_t i = 0; i < n_meshes; i++) {
        if (n_cells[i] < 0 || n_verts[i] < 0) {
            delete b;
            return bfail(TG_ERR_INVALID_ARGUMENT, "negative mesh size in the batch");
        }
        b->c0[i + 1] = b->c0[i] + n_cells[i];
        b->v0[i + 1] = b->v0[i] + n_verts[i];
    }
    const int64_t T = b->c0[n_meshes], V = b->v0[n_meshes];
    if (V > 0x7fffffffLL) {
        delete b;
        return bfail(TG_ERR_UNSUPPORTED, "the batch has more than 2^31 - 1 vertices");
    }
    cudaGetDevice(&b->device);
    if (T > 0 && !tv) {
        delete b;
        return bfail(TG_ERR_INVALID_ARGUMENT, "NULL TV");
    }
    // union TV with global vertex ids
    int4 *d_in = nullptr, *d_tv = nullptr;
    int64_t *d_seg = nullptr;
    auto cleanup = [&]() {
        if (d_in && d_in != reinterpret_cast<const int4 *>(tv)) cudaFreeAsync(d_in, s);
        if (d_tv) cudaFreeAsync(d_tv, s);
        if (d_seg) cudaFreeAsync(d_seg, s);
    };
    cudaError_t e = cudaSuccess;
    if (T > 0) {
        if (tv_on_device) {
            d_in = const_cast<int4 *>(reinterpret_cast<const int4 *>(tv));
        } else {
            e = cudaMallocAsync(&d_in, (size_t)T * 16, s);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(d_in, tv, (size_t)T * 16, cudaMemcpyHostToDevice, s);
        }
        if (e == cudaSuccess) e = cudaMallocAsync(&d_tv, (size_t)T * 16, s);
        if (e == cudaSuccess) e = cudaMallocAsync(&d_seg, (size_t)(n_meshes + 1) * 16, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_seg, b->c0.data(), (size_t)(n_meshes + 1) * 8,
                                cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_seg + n_meshes + 1, b->v0.data(), (size_t)(n_meshes + 1) * 8,
                                cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) {
            Launch L("k_batch_shift", s);
            launch_pdl(k_batch_shift, blocks(T), 256, 0, s, d_in, T, d_seg, d_seg + n_meshes + 1,
                                                    n_meshes, d_tv);
            e = cudaGetLastError();
        }
        if (e != cudaSuccess) {
            cleanup();
            delete b;
            set_last_error(cudaGetErrorString(e));
            return TG_ERR_CUDA;
        }
    }
    tg_status st = tg_mesh_create(reinterpret_cast<const int32_t *>(d_tv), T, V, 1, stream, &b->u);
    cleanup();
    if (st != TG_OK) {
        delete b;
        return st;
    }
    st = mesh_set_segments(b->u, b->c0.data(), n_meshes, s);
    if (st != TG_OK) {
        tg_mesh_destroy(b->u);
        delete b;
        return st;
    }
    *out = b;
    return TG_OK;
}

tg_status tg_batch_destroy(tg_batch *b)
{
    if (!b) return TG_OK;
    tg_status st = tg_mesh_destroy(b->u);
    delete b;
    return st;
}

tg_status tg_batch_extract(tg_batch *b, uint32_t mask, uint32_t options, void *stream)
{
    if (!b) return bfail(TG_ERR_INVALID_ARGUMENT, "batch is NULL");
    std::lock_guard<std::mutex> g(b->mu);
    b->s = (cudaStream_t)stream;
    b->ids_read = false;
    return tg_extract(b->u, mask, options, stream);
}

tg_status tg_batch_critical_points(tg_batch *b, const void *field, int field_type,
                                   int field_on_device, uint32_t *classes_out, int out_on_device,
                                   void *stream)
{
    if (!b) return bfail(TG_ERR_INVALID_ARGUMENT, "batch is NULL");
    return tg_critical_points(b->u, field, field_type, field_on_device, classes_out,
                              out_on_device, stream);
}

tg_status tg_batch_mesh_offsets(tg_batch *b, int64_t i, int64_t *vert0, int64_t *edge0,
                                int64_t *face0, int64_t *cell0)
{
    if (!b || i < 0 || i >= b->n) return bfail(TG_ERR_INVALID_ARGUMENT, "bad batch or mesh index");
    std::lock_guard<std::mutex> g(b->mu);
    int64_t E = -1;
    tg_mesh_counts(b->u, nullptr, &E, nullptr, nullptr);
    if (E >= 0) TRY_B(ensure_ids(b));
    if (vert0) *vert0 = b->v0[i];
    if (cell0) *cell0 = b->c0[i];
    if (edge0) *edge0 = b->ids_read ? b->e0[i] : -1;
    if (face0) *face0 = b->ids_read ? b->f0[i] : -1;
    return TG_OK;
}

tg_status tg_batch_mesh_counts(tg_batch *b, int64_t i, int64_t *nv, int64_t *ne, int64_t *nf,
                               int64_t *nc)
{
    int64_t v0, e0, f0, c0;
    tg_status st = tg_batch_mesh_offsets(b, i, &v0, &e0, &f0, &c0);
    if (st != TG_OK) return st;
    if (nv) *nv = b->v0[i + 1] - v0;
    if (nc) *nc = b->c0[i + 1] - c0;
    if (ne) *ne = b->ids_read ? b->e0[i + 1] - e0 : -1;
    if (nf) *nf = b->ids_read ? b->f0[i + 1] - f0 : -1;
    return TG_OK;
}

tg_status tg_batch_relation_size(tg_batch *b, int64_t i, int r, int64_t *rows, int64_t *entries,
                                 int32_t *width)
{
    if (!b || i < 0 || i >= b->n || r < 1 || r > 13)
        return bfail(TG_ERR_INVALID_ARGUMENT, "bad batch, mesh index or relation");
    const int64_t *off;
    int64_t urows, uent;
    int32_t w;
    TRY_B(tg_get_relation(b->u, r, &off, nullptr, &urows, &uent, &w));
    std::lock_guard<std::mutex> g(b->mu);
    if (uses_ids(r)) TRY_B(ensure_ids(b));
    const std::vector<int64_t> &rs = space(b, kRowSpace[r]);
    const int64_t r0 = rs[i], r1 = rs[i + 1];
    if (rows) *rows = r1 - r0;
    if (width) *width = w;
    if (entries) {
        if (w > 0) {
            *entries = (r1 - r0) * w;
        } else {
            int64_t h[2] = {0, 0};
            BCK(cudaMemcpyAsync(&h[0], off + r0, 8, cudaMemcpyDeviceToHost, b->s));
            BCK(cudaMemcpyAsync(&h[1], off + r1, 8, cudaMemcpyDeviceToHost, b->s));
            BCK(cudaStreamSynchronize(b->s));
            *entries = h[1] - h[0];
        }
    }
    return TG_OK;
}

tg_status tg_batch_copy_relation(tg_batch *b, int64_t i, int r, int64_t *off_host,
                                 int32_t *ent_host, void *stream)
{
    if (!b || i < 0 || i >= b->n || r < 1 || r > 13)
        return bfail(TG_ERR_INVALID_ARGUMENT, "bad batch, mesh index or relation");
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t *off;
    const int32_t *ent;
    int64_t urows, uent;
    int32_t w;
    TRY_B(tg_get_relation(b->u, r, &off, &ent, &urows, &uent, &w));
    std::lock_guard<std::mutex> g(b->mu);
    if (uses_ids(r)) TRY_B(ensure_ids(b));
    const std::vector<int64_t> &rs = space(b, kRowSpace[r]);
    const int64_t r0 = rs[i], r1 = rs[i + 1];
    const int64_t shift = space(b, kValSpace[r])[i];
    int64_t e_lo, e_hi;
    if (w > 0) {
        e_lo = r0 * w;
        e_hi = r1 * w;
    } else {
        int64_t h[2];
        BCK(cudaMemcpyAsync(&h[0], off + r0, 8, cudaMemcpyDeviceToHost, s));
        BCK(cudaMemcpyAsync(&h[1], off + r1, 8, cudaMemcpyDeviceToHost, s));
        BCK(cudaStreamSynchronize(s));
        e_lo = h[0];
        e_hi = h[1];
    }
    const int64_t n_ent = e_hi - e_lo, n_off = w > 0 ? 0 : r1 - r0 + 1;
    int32_t *d_ent = nullptr;
    int64_t *d_off = nullptr;
    cudaError_t e = cudaSuccess;
    if (n_ent > 0 && ent_host) {
        e = cudaMallocAsync(&d_ent, (size_t)n_ent * 4, s);
        if (e == cudaSuccess) {
            Launch L("k_rebase32", s);
            launch_pdl(k_rebase32, blocks(n_ent), 256, 0, s, ent + e_lo, n_ent, (int)shift, d_ent);
            e = cudaMemcpyAsync(ent_host, d_ent, (size_t)n_ent * 4, cudaMemcpyDeviceToHost, s);
        }
    }
    if (e == cudaSuccess && n_off > 0 && off_host) {
        e = cudaMallocAsync(&d_off, (size_t)n_off * 8, s);
        if (e == cudaSuccess) {
            Launch L("k_rebase64", s);
            launch_pdl(k_rebase64, blocks(n_off), 256, 0, s, off + r0, n_off, e_lo, d_off);
            e = cudaMemcpyAsync(off_host, d_off, (size_t)n_off * 8, cudaMemcpyDeviceToHost, s);
        }
    }
    if (d_ent) cudaFreeAsync(d_ent, s);
    if (d_off) cudaFreeAsync(d_off, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_last_error(cudaGetErrorString(e));
        return TG_ERR_CUDA;
    }
    return TG_OK;
}

tg_mesh *tg_batch_union(tg_batch *b) { return b ? b->u : nullptr; }

}  // extern "C"
