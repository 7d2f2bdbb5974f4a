/*
 * tetragpu.h -- C ABI of the GB300-native (sm_103a) relation-extraction and
 * critical-point library, libtetragpu.so.
 *
 * This is the drop-in boundary for TetraGPU's hot path.  It replaces the
 * reference's C++ entry points in include/cuda_extraction.h (tlranda/TetraGPU)
 * and the critPoints kernel launch in src/alg/critPoints.cu; each function
 * below names the reference interface it stands in for.  Plain C: pointers,
 * sizes and integer status codes only.  A CUDA stream is passed as void* (a
 * cudaStream_t cast); NULL means the legacy default stream.
 *
 * Data model (the reference's TV-in / CSR-out layout, kept as is):
 *   - TV is int32 [n_cells x 4].  The library sorts every row ascending
 *     before numbering (the reference CPU face numbering is only consistent
 *     on sorted rows, src/cpu_extraction.cpp:136-153); TE and TF columns refer
 *     to the sorted row.
 *   - Edge ids and face ids are the reference CPU ids: the rank of each
 *     edge's / face's first occurrence when cells are scanned in order,
 *     edges of a cell in pair order (0,1),(0,2),(0,3),(1,2),(1,3),(2,3)
 *     (src/cpu_extraction.cpp:28-62), faces visited with skip (the omitted
 *     slot) = 3,2,1,0, which is TF column order 0..3 (column = 3 - skip,
 *     src/cpu_extraction.cpp:122-174).
 *   - Fixed-width relations (TE 6, EV 2, TF 4, FV 3, FE 3, FT 2) are dense
 *     row-major int32.  FT pads a boundary face's missing cell with -1.
 *   - Variable-width relations (ET, EF, VT, TT, FF, EE, VV) are CSR: int64
 *     offsets [n_rows + 1] and int32 entries, each row sorted ascending.
 *     Exact size: no padding, no duplicates.
 *   - Relations live in device memory owned by the mesh handle until
 *     tg_mesh_destroy (the reference returned raw device pointers the caller
 *     had to cudaFree, src/cuda_extraction.cu:3-22).
 *
 * Errors are status codes (the reference exit()s, include/cuda_safety.h:19-27);
 * tg_last_error_string() describes the last failure on the calling thread.
 * Handles are independent: one mesh per thread needs no locking (the
 * reference keeps its device inputs in file-scope globals,
 * src/cuda_extraction.cu:62,82-84,158-160).
 */
#ifndef TETRAGPU_H
#define TETRAGPU_H

#include <stdint.h>

#include "tetragpu_device.h"   /* tg_device_mesh (plain C structs) */

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    TG_OK = 0,
    TG_ERR_INVALID_ARGUMENT = 1,
    TG_ERR_INVALID_MESH = 2,    /* id out of range, repeated vertex, face in >2 cells */
    TG_ERR_CUDA = 3,
    TG_ERR_OUT_OF_MEMORY = 4,
    TG_ERR_UNSUPPORTED = 5,     /* a limit of this build was exceeded (message says which) */
    TG_ERR_NOT_COMPUTED = 6,    /* relation not extracted yet */
    TG_ERR_TIMEOUT = 7
} tg_status;

/* Relation bits: the reference's arg_flags bit positions
 * (include/datatypes.h.in:164-197, set by --build_XX in src/argparse.cu:82-94).
 * Bit 0 (validate) is accepted and ignored: validation is the test suite's
 * job, against the CPU oracle. */
#define TG_VALIDATE (1u << 0)
#define TG_TE (1u << 1)
#define TG_EV (1u << 2)
#define TG_ET (1u << 3)
#define TG_TF (1u << 4)
#define TG_FV (1u << 5)
#define TG_FE (1u << 6)
#define TG_FT (1u << 7)
#define TG_EF (1u << 8)
#define TG_VT (1u << 9)
#define TG_TT (1u << 10)
#define TG_FF (1u << 11)
#define TG_EE (1u << 12)
#define TG_VV (1u << 13)
#define TG_ALL_RELATIONS 0x3FFEu

/* relation index = bit position */
enum {
    TG_REL_TE = 1, TG_REL_EV = 2, TG_REL_ET = 3, TG_REL_TF = 4, TG_REL_FV = 5,
    TG_REL_FE = 6, TG_REL_FT = 7, TG_REL_EF = 8, TG_REL_VT = 9, TG_REL_TT = 10,
    TG_REL_FF = 11, TG_REL_EE = 12, TG_REL_VV = 13
};

/* tg_extract options */
#define TG_OPT_TT_VERTEX_SHARING 0x1u /* TT = cells sharing >= 1 vertex (default: sharing a face) */
/* Also build the field-independent half of tg_critical_points (the link
 * adjacency over VV, kept on the mesh) during the extraction, beside its last
 * kernels, for a caller that classifies fields next.  Needs VV in the mask. */
#define TG_OPT_LINK_ADJACENCY 0x2u

/* critical-point field types */
#define TG_FIELD_F32 0
#define TG_FIELD_F64 1

typedef struct tg_mesh tg_mesh;

/* Library version string. */
const char *tg_version(void);

/* The tile parameters this build's kernels use (star-pass windows, block
 * sizes, lanes per edge; the values tetragpu_gb300/tune.py selects), as a
 * JSON object. */
const char *tg_tuning_info(void);

/* Description of the last error on this thread ("" if none). */
const char *tg_last_error_string(void);

/* Create a mesh from TV (int32 [n_cells x 4]) in host memory (tv_on_device =
 * 0) or device memory (1) of the current device.  Sorts rows, validates ids
 * and builds VT.  Replaces make_TV_for_GPU (src/cuda_extraction.cu:62-80),
 * without its single-use global and its int/vtkIdType size mix-up (:71). */
tg_status tg_mesh_create(const int32_t *tv, int64_t n_cells, int64_t n_verts,
                         int tv_on_device, void *stream, tg_mesh **out);

/* The reference's cells are vtkIdType (int64; TV_Data::cells,
 * include/datatypes.h.in:63-101, as its VTK loader get_TV_from_VTK in
 * src/vtk_load.cu:46-298 fills them).  tg_tv_narrow_i64 copies 4 * n_cells
 * such ids into int32, slots in their order (tg_mesh_create sorts rows), and
 * refuses what does not narrow: TG_ERR_INVALID_MESH for an id outside
 * [0, n_points) (the message names the cell), TG_ERR_UNSUPPORTED for more
 * than 2^31 - 1 points.  Host only; needs no GPU. */
tg_status tg_tv_narrow_i64(const int64_t *cells, int64_t n_cells, int64_t n_points, int32_t *out);

/* tg_mesh_create from the reference's int64 host TV (tg_tv_narrow_i64, then
 * tg_mesh_create with tv_on_device = 0). */
tg_status tg_mesh_create_i64(const int64_t *tv, int64_t n_cells, int64_t n_verts, void *stream,
                             tg_mesh **out);

/* Frees the mesh's device memory, ordered on the stream of its last call and
 * waiting for that stream: destroy a mesh before the stream it last used. */
tg_status tg_mesh_destroy(tg_mesh *mesh);

/* Extract every relation whose bit is set (plus what they depend on) and keep
 * them resident.  Replaces the make_X_GPU_return family
 * (include/cuda_extraction.h:27-138) and the CPU id minting they depended on
 * (make_TE_and_VE / make_TF_and_VF, src/cpu_extraction.cpp:28-174).
 * Returns after the work is enqueued and the sizes are known (it
 * synchronises the stream a few times to size the outputs). */
tg_status tg_extract(tg_mesh *mesh, uint32_t relation_mask, uint32_t options,
                     void *stream);

/* Counts: vertices, edges (-1 until edges are numbered), faces (-1 until
 * faces are numbered), cells. */
tg_status tg_mesh_counts(const tg_mesh *mesh, int64_t *n_verts, int64_t *n_edges,
                         int64_t *n_faces, int64_t *n_cells);

/* Device pointers of an extracted relation.  Fixed-width relations return
 * offsets == NULL and *row_width = width; CSR relations *row_width = 0.
 * Pointers stay valid until the mesh is destroyed or the relation is
 * re-extracted with different options. */
tg_status tg_get_relation(const tg_mesh *mesh, int relation, const int64_t **offsets,
                          const int32_t **entries, int64_t *n_rows, int64_t *n_entries,
                          int32_t *row_width);

/* Copy a relation to host buffers (offsets may be NULL for fixed width, or
 * to skip them).  Synchronous with respect to the host. */
tg_status tg_copy_relation(const tg_mesh *mesh, int relation, int64_t *offsets_host,
                           int32_t *entries_host, void *stream);
/* The same copies issued on `stream` without waiting for them: a caller that
 * processes many meshes overlaps one mesh's copies with the next one's
 * extraction (pinned host buffers; destroy the mesh, which waits for its last
 * stream, or synchronise the stream before reading the buffers). */
tg_status tg_copy_relation_async(tg_mesh *mesh, int relation, int64_t *offsets_host,
                                 int32_t *entries_host, void *stream);
/* tg_copy_relation_async with a CSR relation's offsets narrowed to int32 on
 * the device first: half the offset bytes over the host link (the
 * reference's device_VV row index is 32-bit as well,
 * src/cuda_extraction.cu:1180-1274).  A relation of 2^31 or more entries is
 * refused with TG_ERR_UNSUPPORTED; fixed-width relations copy their entries
 * only. */
tg_status tg_copy_relation_async_i32(tg_mesh *mesh, int relation, int32_t *offsets_host,
                                     int32_t *entries_host, void *stream);
/* The same, synchronous with respect to the host. */
tg_status tg_copy_relation_i32(tg_mesh *mesh, int relation, int32_t *offsets_host,
                               int32_t *entries_host, void *stream);
/* Every relation in relation_mask (TG_TE | TG_EV | ...) at once, as
 * tg_copy_relation_async_i32 does one: offsets_host[r] and entries_host[r]
 * (arrays of 14 pointers indexed by relation, NULL to skip one) receive
 * relation r.  The offsets of all requested CSR relations are narrowed by one
 * launch before any copy is issued, so the copies follow one another on the
 * copy engine without waiting for kernels between them. */
tg_status tg_copy_relations_async_i32(tg_mesh *mesh, uint32_t relation_mask,
                                      int32_t *const *offsets_host,
                                      int32_t *const *entries_host, void *stream);

/* A relation's entries widened to int64 (the reference's vtkIdType) and its
 * int64 offsets (CSR only; may be NULL), into caller memory on the device
 * (out_on_device = 1, stream-ordered) or the host (0, synchronous).  Serves
 * callers of the make_X_GPU_return functions, which returned vtkIdType device
 * arrays (include/cuda_extraction.h:27-138). */
tg_status tg_export_relation_i64(const tg_mesh *mesh, int relation, int64_t *entries_out,
                                 int64_t *offsets_out, int out_on_device, void *stream);

/* A CSR relation in the reference's padded device_VV layout
 * (src/cuda_extraction.cu:1180-1274, read by the critPoints kernel): row r at
 * padded_out[r * width], int64 entries, unused slots -1, and row lengths in
 * counts_out (may be NULL).  Device memory, stream-ordered.  Rows longer than
 * width are truncated: size width from the mesh (e.g. the largest VV row). */
tg_status tg_export_rows_padded(const tg_mesh *mesh, int relation, int32_t width,
                                int64_t *padded_out, uint32_t *counts_out, void *stream);

/* Device pointer of the canonical (row-sorted) TV, int32 [n_cells x 4]. */
tg_status tg_get_tv(const tg_mesh *mesh, const int32_t **tv_sorted);

/* Classify every vertex of a scalar field (float32 or float64, host or
 * device, n_verts values).  Writes uint32 [n_verts x 3] in the reference
 * layout of critPoints (src/alg/critPoints.cu:275-331): [3v] lower-link
 * components, [3v+1] upper-link components, [3v+2] class code with the
 * reference's numeric values: 1 minimum, 2 maximum, 3 regular, 4 saddle.
 * A neighbour u of v is lower when f[u] < f[v], or f[u] == f[v] and u < v;
 * two neighbours are linked when the mesh has an edge between them (the
 * reference's VV test, critPoints.cu:172-202).  classes_out is host memory
 * (out_on_device = 0, synchronous) or device memory (1, stream-ordered).
 * Extracts VV if needed.  The field-independent part (the link adjacency) is
 * cached on the mesh, so a second field costs only the classification. */
tg_status tg_critical_points(tg_mesh *mesh, const void *field, int field_type,
                             int field_on_device, uint32_t *classes_out,
                             int out_on_device, void *stream);

/* The reference's class report (export_classes, src/alg/critPoints.cu:340-453)
 * for classes in host memory (the tg_critical_points layout): the five
 * "Total number of ..." lines with the reference's wording and numbers (its
 * labels are swapped: "minima" counts code 2, the true maxima), preceded, if
 * per_vertex_lines, by one "A <vertex> <code>" line per classified vertex
 * (the form its verifier script parses).  path NULL writes to stdout.
 * counts_out (may be NULL): vertices per code 0..4.  Host only. */
tg_status tg_export_classes(const uint32_t *classes, int64_t n_verts, const char *path,
                            int per_vertex_lines, int64_t *counts_out);

/* ---- reading resident relations in place ----------------------------------
 * tetragpu_device.h declares tg_device_mesh and inline accessors for device
 * code; tg_get_device_mesh fills one with the mesh's resident relations
 * (NULL where a relation was not extracted).  Serves the reference's aim of
 * algorithm kernels reading relations where they lie
 * (src/cuda_extraction.cu:16-22). */
tg_status tg_get_device_mesh(const tg_mesh *mesh, tg_device_mesh *out);

/* An algorithm kernel built that way (a downstream consumer of VV): Laplacian
 * smoothing of a float32 vertex field on the device, each of `iterations`
 * steps replacing f[v] by the mean of f[v] and its neighbours' values.  in,
 * out and scratch (needed when iterations > 1) are device arrays of n_verts
 * floats, in may not alias out or scratch; extracts VV if needed.
 * Stream-ordered. */
tg_status tg_smooth_field(tg_mesh *mesh, const float *in, float *out, int iterations,
                          float *scratch, void *stream);

/* Bytes of device memory the mesh currently holds. */
int64_t tg_mesh_device_bytes(const tg_mesh *mesh);

/* Number of kernel launches this library has issued in this process. */
int64_t tg_kernel_launch_count(void);

/* Critical points for callers that cannot allocate device memory when they
 * classify: a host application that gives this library a fixed device-memory
 * budget at start-up and accounts for every byte afterwards, or a real-time
 * loop whose rules forbid allocator calls (and the synchronisation they can
 * bring) once it runs.  No counterpart in the reference.  Inputs and output
 * are device memory the caller owns: VV as CSR (vv_off [n_verts + 1], vv
 * [n_vv_entries], rows sorted, as tg_get_relation returns it), the field
 * (TG_FIELD_F32/F64, n_verts values) and classes_out (uint32 [n_verts x 3],
 * the layout of tg_critical_points).  The link adjacency goes to a fixed
 * device array of TG_NOALLOC_MAX_VV_ENTRIES 64-bit masks (64 MiB, plus a
 * 128 KiB window table) that every GPU loading the library holds until the
 * process exits; larger VV is rejected with TG_ERR_UNSUPPORTED before
 * anything runs, and so is a vertex with more than 64 neighbours (after the
 * kernels ran: classes_out is then not valid).  The first call on a device
 * looks up that array's device address.  Calls share the array and keep the
 * last call's contents in it: calls that overlap on the GPU race, so
 * serialise them.  The call reads the kernels' status word back, so it
 * waits for its stream before returning.  Nothing is allocated (no
 * cudaMalloc, cudaFree or allocating library routine). */
#define TG_NOALLOC_MAX_VV_ENTRIES (1 << 23)
tg_status tg_critical_points_noalloc(const int64_t *vv_off, const int32_t *vv, int64_t n_verts,
                                     int64_t n_vv_entries, const void *field, int field_type,
                                     uint32_t *classes_out, void *stream);

/* ---- batches of independent meshes ---------------------------------------
 * Many meshes processed as one: their disjoint union is a mesh, so every
 * kernel of the path runs once over all of them (no per-mesh launches,
 * allocations or synchronisations).  A mesh's relations are the union's
 * restricted to its rows, minus its first vertex / edge / face / cell id, and
 * are identical to what that mesh alone gives (ids are ranks of first
 * occurrences in cell order and a mesh's cells are contiguous).  No
 * counterpart in the reference, which runs one mesh per process. */
typedef struct tg_batch tg_batch;

/* tv: the meshes' cells back to back, int32 [sum n_cells x 4], each mesh
 * with its own vertex ids 0 .. n_verts[i] - 1 (an id outside that range is
 * TG_ERR_INVALID_MESH).  n_cells / n_verts: host arrays of n_meshes. */
tg_status tg_batch_create(const int32_t *tv, const int64_t *n_cells, const int64_t *n_verts,
                          int64_t n_meshes, int tv_on_device, void *stream, tg_batch **out);
tg_status tg_batch_destroy(tg_batch *batch);
/* tg_extract over the whole batch. */
tg_status tg_batch_extract(tg_batch *batch, uint32_t relation_mask, uint32_t options,
                           void *stream);
/* tg_critical_points over the whole batch: field holds every mesh's values
 * back to back (sum n_verts), classes_out uint32 [sum n_verts x 3]. */
tg_status tg_batch_critical_points(tg_batch *batch, const void *field, int field_type,
                                   int field_on_device, uint32_t *classes_out,
                                   int out_on_device, void *stream);
/* Counts of mesh i (E and F once extracted, else -1).  Synchronous on first
 * use after an extraction. */
tg_status tg_batch_mesh_counts(tg_batch *batch, int64_t i, int64_t *n_verts, int64_t *n_edges,
                               int64_t *n_faces, int64_t *n_cells);
/* Mesh i's relation with that mesh's own ids, copied to host memory:
 * offsets_out (CSR: rows + 1, starting at 0; NULL for fixed width or not
 * wanted) and entries_out.  Sizes from tg_batch_relation_size.  Synchronous. */
tg_status tg_batch_relation_size(tg_batch *batch, int64_t i, int relation, int64_t *rows,
                                 int64_t *entries, int32_t *width);
tg_status tg_batch_copy_relation(tg_batch *batch, int64_t i, int relation, int64_t *offsets_out,
                                 int32_t *entries_out, void *stream);
/* The union mesh (ids of the whole batch), e.g. for tg_get_relation. */
tg_mesh *tg_batch_union(tg_batch *batch);
/* First vertex, edge, face and cell id of mesh i in the union (E and F once
 * extracted). */
tg_status tg_batch_mesh_offsets(tg_batch *batch, int64_t i, int64_t *vert0, int64_t *edge0,
                                int64_t *face0, int64_t *cell0);

/* ---- serving -------------------------------------------------------------
 * A request loop over one device: new meshes (with a field) and new fields on
 * meshes already resident.  Worker slots (a thread and a CUDA stream each) run
 * concurrently; when a slot frees, the new-mesh requests waiting at the head
 * of the queue are merged into one batch (tg_batch_*) up to batch_cells cells
 * and up to the device-memory budget, so requests that arrive while others are
 * on the GPU join the next batch and overlap on the device.  Meshes stay
 * resident (their relations and link adjacency) for later fields; when memory
 * runs short, idle resident batches are evicted least-recently-used first and
 * a later field on an evicted mesh rebuilds it from the host copy of its TV.
 * Results are identical to the mesh processed alone.  No counterpart in the
 * reference. */
typedef struct tg_server tg_server;
typedef struct {
    int32_t n_slots;          /* concurrent work slots; 0 = 4 */
    int64_t hbm_budget_bytes; /* device memory for resident meshes and work in flight; 0 = 150e9 */
    int64_t batch_cells;      /* most cells merged into one batch; 0 = 4,194,304 */
    uint32_t relation_mask;   /* relations extracted for every new mesh (VV always added) */
} tg_server_config;
typedef struct {
    int64_t submitted, completed, failed;
    int64_t batches;          /* pipeline runs for new meshes */
    int64_t meshes_built;     /* meshes created, rebuilt ones included */
    int64_t evictions;        /* resident batches evicted for memory */
    int64_t resident_meshes, resident_bytes, peak_bytes;
} tg_server_stats;

/* device: CUDA device index; cfg may be NULL (defaults). */
tg_status tg_server_create(int device, const tg_server_config *cfg, tg_server **out);
/* Waits for every request in flight, then frees everything. */
tg_status tg_server_destroy(tg_server *server);
/* A new mesh and a field on it.  TV (int32 [n_cells x 4], host) and the field
 * (n_verts values, host) are copied before returning.  request_id names the
 * request for tg_server_wait; mesh_id names the resident mesh. */
tg_status tg_server_submit_mesh(tg_server *server, const int32_t *tv, int64_t n_cells,
                                int64_t n_verts, const void *field, int field_type,
                                int64_t *request_id, int64_t *mesh_id);
/* A new field on a resident mesh (copied before returning). */
tg_status tg_server_submit_field(tg_server *server, int64_t mesh_id, const void *field,
                                 int field_type, int64_t *request_id);
/* Waits for a request (timeout_ms < 0: no limit; TG_ERR_TIMEOUT when it runs
 * out) and hands back its classes (host uint32 [n_verts x 3], may be NULL)
 * and its latency from submission to completion.  A request can be waited
 * for once; its record is then dropped. */
tg_status tg_server_wait(tg_server *server, int64_t request_id, int64_t timeout_ms,
                         uint32_t *classes_out, double *latency_ms);
/* Relation of a resident mesh with its own ids (extracted if needed), like
 * tg_batch_relation_size / tg_batch_copy_relation.  Synchronous. */
tg_status tg_server_relation_size(tg_server *server, int64_t mesh_id, int relation,
                                  int64_t *rows, int64_t *entries, int32_t *width);
tg_status tg_server_copy_relation(tg_server *server, int64_t mesh_id, int relation,
                                  int64_t *offsets_out, int32_t *entries_out);
/* The mesh is no longer needed; its memory goes once its batch is unused. */
tg_status tg_server_release_mesh(tg_server *server, int64_t mesh_id);
tg_status tg_server_get_stats(tg_server *server, tg_server_stats *out);

/* Time every launch of one kernel (by name, e.g. "k_star_b") with CUDA
 * events recorded on the stream it is launched on; NULL or "" turns timing
 * off.  For measurement tools; the reference's analogue is its Timer class
 * (src/metrics.cpp).  Not thread-safe against concurrent extractions. */
tg_status tg_profile_kernel(const char *name);

/* Sum of the timed launches' durations (waits for them), their number, and
 * optionally forget them. */
tg_status tg_profile_read(double *total_ms, int64_t *launches, int reset);

#ifdef __cplusplus
}
#endif
#endif
