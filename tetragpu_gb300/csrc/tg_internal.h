// tg_internal.h -- declarations shared by the host orchestration (tg_api.cu)
// and the kernel translation units.  Not part of the public ABI.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace tg {

// Device-side status word, written by kernels with atomics, read back by the
// host at the synchronisation points of tg_extract.
struct DevStatus {
    unsigned int flags;
    int bad_cell;      // lowest offending cell (atomicMin), INT_MAX if none
    int bad_vertex;    // lowest offending vertex (atomicMin), INT_MAX if none
    int max_star;      // largest number of cells around a vertex
    int max_deg;       // largest number of neighbours of a vertex
    int pad[3];
};

enum StatusFlag : unsigned int {
    ST_BAD_ID = 1u,            // vertex id outside [0, n_verts)
    ST_DUP_VERTEX = 2u,        // a cell repeats a vertex
    ST_HEAVY_STAR = 4u,        // a vertex lies in more cells than the star kernels hold
    ST_STAR_OVERFLOW = 8u,     // more neighbours than the summary slot holds
    ST_NONMANIFOLD_FACE = 16u, // a face lies in more than two cells
    ST_HASH_FULL = 32u,        // per-vertex neighbour table overflowed
    ST_HEAVY_DEG = 64u         // a vertex has more neighbours than the kernels hold
};

// Largest star (cells around one vertex) and neighbourhood handled on the
// fast path: star positions and neighbours are bits of a 64-bit mask.
constexpr int kMaxStar = 64;
constexpr int kMaxDeg = 64;

// ---- scans (tg_scan.cu) ----
enum ScanKind : int {
    SCAN_COUNT_I32 = 0,  // in: int32 counts, out: int64 offsets [n + 1]
    SCAN_POPC_U32 = 1    // in: uint32 bit words, out: int32 prefix of popcounts [n + 1]
};
struct ScanJob {
    const void *in;
    void *out;
    int64_t n;
    int kind;
    int pad;
};
constexpr int kMaxScanJobs = 8;
// Exclusive scans of up to kMaxScanJobs arrays in three launches.  `scratch`
// must hold scan_scratch_bytes(max n) bytes per job.
size_t scan_scratch_bytes(int64_t n);
void scan_batch(const ScanJob *jobs, int n_jobs, void *scratch, cudaStream_t s);

// ---- pipeline kernels (tg_kernels.cu) ----
struct Sizes {
    int64_t V, T;
};

void launch_canon(const int32_t *tv_in, int64_t T, int64_t V, int4 *tvs, int32_t *deg_t,
                  DevStatus *st, cudaStream_t s);
void launch_vt_fill(const int4 *tvs, int64_t T, const int64_t *vt_off, int32_t *cursor,
                    int32_t *vt, cudaStream_t s);
void launch_sort_rows(const int64_t *off, int32_t *ent, int64_t n_rows, cudaStream_t s);

struct StarA {
    const int64_t *vt_off;
    const int32_t *vt;
    const int4 *tvs;
    int64_t V;
    int32_t *deg;          // [V] out
    int32_t *sum_nb;       // padded summary, base vt_off[v] + 2v
    uint64_t *sum_mask;
    uint32_t *eflag;       // bit per edge occurrence 6c+j
    uint32_t *fflag;       // bit per face occurrence 4c+k
    DevStatus *st;
    int wide;              // summary capacity 3D per vertex instead of D + 2
};
void launch_star_a(const StarA &a, cudaStream_t s);

void launch_vv_finalize(const int64_t *vt_off, const int32_t *sum_nb, const uint64_t *sum_mask,
                        const int64_t *vv_off, int64_t V, int wide, int32_t *vv,
                        uint64_t *vvmask, cudaStream_t s);

struct StarB {
    const int64_t *vt_off;
    const int32_t *vt;
    const int4 *tvs;
    const int64_t *vv_off;
    const int32_t *vv;
    const uint64_t *vvmask;
    const uint32_t *eflag;
    const int32_t *epre;
    const uint32_t *fflag;
    const int32_t *fpre;
    int64_t V;
    int32_t *eidv;     // [2E] edge id of every VV entry
    int32_t *ev;       // [2E] or null
    int32_t *te;       // [6T] or null
    int32_t *tf;       // [4T] or null
    int32_t *fv;       // [3F] or null
    int32_t *ft;       // [2F] or null
    int32_t *et_cnt;   // [E] or null
    int32_t *ef_cnt;   // [E] or null
    int32_t *ee_cnt;   // [E] or null
    int32_t *ff_cnt;   // [F] or null
    int32_t *tt_cnt;   // [T] or null (atomic adds; zeroed by the caller)
    DevStatus *st;
};
void launch_star_b(const StarB &b, cudaStream_t s);

struct StarC {
    const int64_t *vt_off;
    const int32_t *vt;
    const int4 *tvs;
    const int64_t *vv_off;
    const int32_t *vv;
    const uint64_t *vvmask;
    const int32_t *eidv;
    const uint32_t *fflag;
    const int32_t *fpre;
    int64_t V;
    const int64_t *et_off;
    int32_t *et;       // or null
    const int64_t *ef_off;
    int32_t *ef;       // or null
};
void launch_star_c(const StarC &c, cudaStream_t s);

void launch_cell_fe_tt(const int4 *tvs, int64_t T, const int32_t *te, const int32_t *tf,
                       const int32_t *ft, int32_t *fe, const int64_t *tt_off, int32_t *tt,
                       cudaStream_t s);
void launch_ff_fill(const int32_t *ft, const int32_t *tf, int64_t F, const int64_t *ff_off,
                    int32_t *ff, cudaStream_t s);
void launch_ee_fill(const int32_t *ev, int64_t E, const int64_t *vv_off, const int32_t *eid_sorted,
                    const int64_t *ee_off, int32_t *ee, cudaStream_t s);
void launch_tt_vertex_count(const int4 *tvs, int64_t T, const int64_t *vt_off, const int32_t *vt,
                            int32_t *cnt, cudaStream_t s);
void launch_tt_vertex_fill(const int4 *tvs, int64_t T, const int64_t *vt_off, const int32_t *vt,
                           const int64_t *tt_off, int32_t *tt, cudaStream_t s);

// critical points (tg_crit.cu)
void launch_crit_adj(const int64_t *vv_off, const int32_t *vv, int64_t V, uint64_t *adj,
                     DevStatus *st, cudaStream_t s);
void launch_crit_classify(const int64_t *vv_off, const int32_t *vv, const uint64_t *adj,
                          const void *field, int field_type, int64_t V, uint32_t *classes3,
                          cudaStream_t s);

// launch accounting and optional CUDA-event timing of one named kernel
void count_launch(int n = 1);
void prof_begin(const char *name, cudaStream_t s);
void prof_end(const char *name, cudaStream_t s);

// RAII wrapper around every launch: counts it and, when the kernel is the
// one selected with tg_profile_kernel, brackets it with CUDA events.
struct Launch {
    const char *name;
    cudaStream_t s;
    Launch(const char *n, cudaStream_t st) : name(n), s(st) { prof_begin(name, s); }
    ~Launch()
    {
        prof_end(name, s);
        count_launch();
    }
};

}  // namespace tg
