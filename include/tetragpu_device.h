/*
 * tetragpu_device.h -- reading relations in place, inside the caller's own
 * CUDA kernels.
 *
 * The reference's stated aim was that its relation kernels could be "tied
 * together (perhaps as inlines) to make a device-contained relationship remap
 * fit within the algorithm kernel with great locality"
 * (src/cuda_extraction.cu:16-22 of tlranda/TetraGPU).  Relations extracted by
 * tg_extract stay resident in device memory; tg_get_device_mesh (declared in
 * tetragpu.h) fills a tg_device_mesh with their pointers, and the inline
 * accessors below read rows straight from them in device code: no copies, no
 * padding, rows sorted ascending.  A relation that was not extracted has NULL
 * pointers.  The pointers stay valid until the mesh is destroyed or the
 * relation is extracted again with other options.
 */
#ifndef TETRAGPU_DEVICE_H
#define TETRAGPU_DEVICE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* a variable-width relation: row r is ent[off[r] .. off[r + 1]) */
typedef struct {
    const int64_t *off;
    const int32_t *ent;
    int64_t rows;
} tg_csr_view;

/* a fixed-width relation: row r is ent[r * width .. (r + 1) * width) */
typedef struct {
    const int32_t *ent;
    int64_t rows;
    int32_t width;
} tg_fixed_view;

/* Every relation of a mesh, by the reference's names; TV is the row-sorted
 * cell array the ids refer to (4 per cell). */
typedef struct {
    int64_t n_verts, n_edges, n_faces, n_cells;
    const int32_t *tv;
    tg_fixed_view te, ev, tf, fv, fe, ft;
    tg_csr_view et, ef, vt, tt, ff, ee, vv;
} tg_device_mesh;

#ifdef __cplusplus
}
#endif

#ifdef __CUDACC__
/* number of entries of row r */
__device__ __forceinline__ int32_t tg_row_size(const tg_csr_view &v, int64_t r)
{
    return (int32_t)(v.off[r + 1] - v.off[r]);
}
/* first entry of row r */
__device__ __forceinline__ const int32_t *tg_row(const tg_csr_view &v, int64_t r)
{
    return v.ent + v.off[r];
}
__device__ __forceinline__ const int32_t *tg_row(const tg_fixed_view &v, int64_t r)
{
    return v.ent + r * v.width;
}
/* the 4 vertices of cell c, ascending */
__device__ __forceinline__ int4 tg_cell(const tg_device_mesh &m, int64_t c)
{
    return reinterpret_cast<const int4 *>(m.tv)[c];
}
/* whether x is in row r (rows are sorted: a binary search) */
__device__ __forceinline__ bool tg_row_contains(const tg_csr_view &v, int64_t r, int32_t x)
{
    int64_t lo = v.off[r], hi = v.off[r + 1];
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (v.ent[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return lo < v.off[r + 1] && v.ent[lo] == x;
}
#endif

#endif
