// tg_internal.h -- declarations shared by the host orchestration (tg_api.cu)
// and the kernel translation units.  Not part of the public ABI.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <utility>

#include "tetragpu.h"
#include "tg_tuning.h"

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
    ST_HEAVY_DEG = 64u,        // a vertex has more neighbours than the kernels hold
    ST_SCAN_STALLED = 128u     // a scan tile gave up waiting for the tiles before it
};

// Largest star (cells around one vertex) and neighbourhood handled on the
// fast path: star positions and neighbours are bits of a 64-bit mask.
constexpr int kMaxStar = 64;
constexpr int kMaxDeg = 64;

// VV entries per window of the link-adjacency kernel (tg_crit.cu): its
// window table has n_vv / kAdjWin + 2 entries
constexpr int kAdjWin = TG_ADJ_WIN;
static_assert(kAdjWin >= 64 && kAdjWin <= 4096, "link-adjacency window size");

// ---- scans (tg_scan.cu) ----
enum ScanKind : int {
    SCAN_COUNT_I32 = 0,  // in: int32 counts, out: int64 offsets [n + 1]
    SCAN_POPC_RANK = 1,  // in: uint32 bit words, out: uint2 {word, popcount prefix} [n + 1],
                         //     out[n] = {0, total}: rank of bit p = one 8-byte load
    SCAN_SQUARE_I32 = 2  // in: int32 x, out: int64 prefix of x*x [n + 1]
};
struct ScanJob {
    const void *in;
    void *out;
    int64_t n;
    int kind;
    int pad;
};
constexpr int kMaxScanJobs = 8;
// Exclusive scans of up to kMaxScanJobs arrays in one launch, over a
// workspace of two buffers of kMaxScanJobs * job_words words (zeroed once when
// made): a scan uses one buffer and zeroes the other for the next scan, so no
// scan needs a memset.  A scan issued on another stream than the last one
// waits for the last one first (event `done`).  A stalled scan sets
// ST_SCAN_STALLED in st.
struct ScanWorkspace {
    unsigned long long *buf = nullptr;   // 2 * kMaxScanJobs * job_words words
    int64_t job_words = 0;               // tile words + ticket of the longest array
    int cur = 0;
    cudaEvent_t done = nullptr;
    cudaStream_t last = nullptr;
    bool used = false;
};
int64_t scan_job_words(int64_t max_n);
void scan_batch(const ScanJob *jobs, int n_jobs, ScanWorkspace &ws, DevStatus *st, cudaStream_t s);
// For another single-pass kernel on the workspace: the buffer to use now
// (kMaxScanJobs * job_words words, zero), the one to zero for the next user;
// scan_ws_end after the launch.
void scan_ws_begin(ScanWorkspace &ws, cudaStream_t s, unsigned long long **cur,
                   unsigned long long **next, int64_t *next_words);
void scan_ws_end(ScanWorkspace &ws, cudaStream_t s);

#ifdef __CUDACC__
// Single-pass scan step (decoupled look-back, Merrill and Garland), called by
// one whole warp: publish tile `tile`'s sum in w[tile] (sum << 2 | 1), add
// the published sums of the tiles before it, 32 at a time (lane i reads the
// i-th tile back), until one holds an inclusive prefix (sum << 2 | 2); then
// publish its own inclusive prefix.  Returns the sum of the tiles before it
// (in every lane).  Tiles are numbered in block start order, so the tiles
// waited for are running; after kLookbackPolls polls the wait gives up and
// sets ST_SCAN_STALLED.
constexpr unsigned kLookbackPolls = 1u << 16;
__device__ __forceinline__ long long look_back(unsigned long long *w, long long tile, long long sum,
                                               unsigned *err)
{
    const int lane = threadIdx.x & 31;
    if (tile == 0) {
        if (lane == 0) atomicExch(w, ((unsigned long long)sum << 2) | 2ull);
        return 0;
    }
    if (lane == 0) atomicExch(w + tile, ((unsigned long long)sum << 2) | 1ull);
    long long prefix = 0;
    long long k = tile - 1;   // the window: tiles k - 31 .. k
    unsigned polls = 0;
    while (true) {
        const long long t = k - lane;
        const unsigned long long x =
            t >= 0 ? *reinterpret_cast<volatile unsigned long long *>(w + t) : 0ull;
        const unsigned f = (unsigned)(x & 3ull);
        const unsigned pre = __ballot_sync(0xffffffffu, f == 2);
        const int first = pre ? __ffs(pre) - 1 : 31;   // nearest inclusive prefix, or all
        const unsigned need = first >= 31 ? 0xffffffffu : (2u << first) - 1u;
        if (__ballot_sync(0xffffffffu, f == 0) & need) {   // a tile has not published yet
            if (++polls > kLookbackPolls) {
                if (lane == 0) atomicOr(err, ST_SCAN_STALLED);
                break;
            }
            __nanosleep(32);
            continue;
        }
        long long v = lane <= first ? (long long)(x >> 2) : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        prefix += v;
        if (pre) break;
        k -= 32;
    }
    if (lane == 0) atomicExch(w + tile, ((unsigned long long)(prefix + sum) << 2) | 2ull);
    return prefix;
}
#endif

// ---- pipeline kernels (tg_kernels.cu) ----
struct Sizes {
    int64_t V, T;
};

void launch_reset_status(DevStatus *st, cudaStream_t s);
// Status word and up to 8 sizes (int64, or int32 sign-extended) stored by a
// kernel into device-mapped pinned host memory (no copy engine involved)
struct PublishArgs {
    DevStatus *st;           // reset once copied
    const void *src[8];
    int wide[8];
    int n;
    DevStatus *h_st;
    int64_t *h_sz;
};
void launch_publish(const PublishArgs &a, cudaStream_t s);
void launch_widen(const int32_t *src, int64_t *dst, int64_t n, cudaStream_t s);
void launch_narrow(const int64_t *src, int32_t *dst, int64_t n, cudaStream_t s);
// up to 16 int64 arrays narrowed into one int32 array, back to back
struct NarrowJobs {
    const int64_t *src[16];
    int64_t start[17];   // start[k]: first output element of array k; start[n] = total
    int n;
    int32_t *dst;
};
void launch_narrow_multi(const NarrowJobs &j, cudaStream_t s);
void launch_pad_rows(const int64_t *off, const int32_t *ent, int64_t rows, int width,
                     int64_t *out, uint32_t *counts, cudaStream_t s);
// sort each TV row, validate ids, count cells per vertex; occ[c] = the
// cell's place in each of its vertices' (unsorted) VT rows
void launch_canon(const int32_t *tv_in, int64_t T, int64_t V, int4 *tvs, int32_t *deg_t,
                  int4 *occ, DevStatus *st, cudaStream_t s);
void launch_vt_fill(const int4 *tvs, int64_t T, const int64_t *vt_off, const int4 *occ,
                    int32_t *vt, cudaStream_t s);
void launch_sort_rows(const int64_t *off, int32_t *ent, int64_t n_rows, cudaStream_t s);
// Windows of win_size entries over a CSR: win[w] = first row starting at or
// after entry win_size * w (w = 0 .. window_count), win[window_count] = rows;
// wbase[w] (when given) = that row's first entry, off[win[w]] (below 2^31).
int64_t window_count(int64_t n_entries, int win_size);
void launch_window_starts(const int64_t *off, int64_t rows, int64_t n_entries, int win_size,
                          int32_t *win, cudaStream_t s, int win_size2 = 0,
                          int32_t *win2 = nullptr, int32_t *wbase = nullptr,
                          int32_t *wbase2 = nullptr);
int star_window();    // the window size of star pass A over VT
int star_window_b();  // the window size of star pass B
// sort every VT row (tg_star.cu): window-staged, coalesced.  Also marks each
// vertex's star-order key 4 * (lowest cell) + (slot in it) in vflag (4T bits,
// zeroed by the caller) and stores it in vkey[v]; rows with no cells are left
// alone.
void launch_vt_sort(const int64_t *vt_off, const int32_t *win, int32_t *vt, int64_t V,
                    int64_t nvt, const int4 *tvs, uint32_t *vflag, int64_t *vkey, int32_t *heavy_cnt,
                    cudaStream_t s);
// Star processing order (vertices by first cell): vorder[pos] = vertex and
// dcount[pos] = its row length, pos = rank of its key; vtp = VT rows in that
// order, pofs = its offsets (rows with no cells last, length 0)
void launch_vorder_place(const int64_t *vt_off, int64_t V, const int64_t *vkey,
                         const uint2 *vrank, int64_t nwk, const int32_t *heavy_cnt, int32_t *vorder,
                         int32_t *dcount, cudaStream_t s);
void launch_vtp_fill(const int32_t *vorder, const int64_t *pofs, int64_t V, const int64_t *vt_off,
                     const int32_t *vt, int32_t *vtp, cudaStream_t s);

struct StarA {
    const int64_t *pofs;       // VT offsets in star processing order (rows + 1)
    const int32_t *win;        // window table over pofs
    const int32_t *wbase;      // first entry of each window
    const int32_t *vorder;     // vertex at each processing position
    const int32_t *vtp;        // VT rows in processing order
    const int4 *tvs;
    int64_t V;
    int64_t nvt;               // VT entries (4 * cells)
    int32_t *deg;              // [V] neighbour counts (zeroed by the caller)
    uint32_t *ecnt;            // [6T] ET | EF << 16 row lengths at owned edges' first slots
    uint32_t *eflag;           // bit per edge occurrence 6c+j (first occurrences)
    uint32_t *fflag;           // bit per face occurrence 4c+k (first occurrences)
    uint32_t *fbnd;            // bit per face occurrence: first and only (boundary face)
    DevStatus *st;
    uint32_t *emask;           // [3][nvt] star positions holding each entry's candidates
                               // (the low 32 of a star's up to 64 positions)
    uint32_t *emask_hi;        // [3][nvt] the high 32, written only for stars of more
                               // than 32 cells; null when the mesh has none
    bool narrow;               // no star holds more than 32 cells (emask_hi is null)
    int64_t light_end;         // entries of the light stars (they come first): 4T - heavy entries
};
void launch_star_a(const StarA &a, cudaStream_t s);
// seg_ef[i] = first edge id and seg_ef[n + 1 + i] = first face id of the
// cells from seg_c[i] on (i = 0 .. n; seg_c[n] = T gives the totals)
void launch_seg_ranks(const int64_t *seg_c, int64_t n, const uint2 *erank, const uint2 *frank,
                      int64_t *seg_ef, cudaStream_t s);

// ET / EF / EE offsets in edge-id order from one scan over the 6T edge slots
// ET/EF/EE offsets in edge-id order in one pass (also EV when ev is given;
// len: E scratch words); edge_offsets_words = the tile words it needs in the
// scan workspace
int64_t edge_offsets_words(int64_t n_slots);
void launch_edge_offsets(const uint32_t *eflag, const uint32_t *ecnt, const int4 *tvs,
                         const int32_t *deg, const uint2 *erank, int64_t n_slots, int64_t E,
                         int64_t *et_off, int64_t *ef_off, int64_t *ee_off, int32_t *ev,
                         uint2 *len, ScanWorkspace &ws, DevStatus *st, cudaStream_t s);

struct StarB {
    const int64_t *pofs;       // as in StarA
    const int32_t *win;        // window table over pofs with star_window_b()
    const int32_t *wbase;      // first entry of each window
    const int32_t *vorder;
    const int32_t *vtp;
    const int4 *tvs;
    int64_t V;
    int64_t nvt;
    const int64_t *vv_off;
    const uint2 *erank;        // {bits, prefix} per 32 edge occurrences
    const uint2 *frank;        // same for face occurrences
    const uint2 *brank;        // same for boundary-face occurrences
    const uint32_t *emask;     // [3][nvt] from pass A, as in StarA
    const uint32_t *emask_hi;
    bool narrow;               // as in StarA
    int32_t *vv;               // [2E] VV rows
    int32_t *eid_sorted;       // [2E] incident edge ids sorted by id, or null
    int32_t *te;               // [6T] or null
    int32_t *tf;               // [4T] or null
    int32_t *ft;               // [2F] or null
    const int64_t *et_off;
    int32_t *et;               // or null
    DevStatus *st;
};
void launch_star_b(const StarB &b, cudaStream_t s);

// A face at its first cell c (occurrence q = 4c + TF column), c2 its
// second cell or -1: its id is the rank of q among first occurrences; its
// FT row and its TF entry in c are written here, the caller writes TF in c2.
// Pass B and the heavy-star pass call it, once per face (FV and FE follow
// and the FF offset in k_face_fill).
__device__ __forceinline__ int face_at_first(const uint2 *__restrict__ frank, int32_t *tf,
                                             int32_t *ft, long long q, int c, int c2)
{
    const uint2 w = __ldg(frank + (q >> 5));
    const int fid = (int)w.y + __popc(w.x & ((1u << (q & 31)) - 1u));
    if (tf) tf[q] = fid;
    if (ft) *reinterpret_cast<int2 *>(ft + 2LL * fid) = make_int2(c, c2);
    return fid;
}

// TT offsets (4c - boundary faces before cell c), TT rows (or null), and the
// closing TT and FF offsets.
void launch_cell_tt(int64_t T, int64_t F, const int32_t *tf, const int32_t *ft, const uint2 *brank,
                    int64_t *tt_off, int32_t *tt, int64_t *ff_off, cudaStream_t s);
// EF rows (one thread per edge) from ET, the sorted TV and TF
void launch_ef_fill(const int32_t *ev, int64_t E, const int64_t *et_off, const int32_t *et,
                    const int4 *tvs, const int32_t *tf, const int64_t *ef_off, int32_t *ef,
                    cudaStream_t s);
// per face (each may be null): FV, FE, FF offsets (but the closing one) and
// FF rows (ff_off and ff together)
void launch_face_fill(const int32_t *ft, const int32_t *tf, const int4 *tvs, const int32_t *te,
                      const uint2 *brank, int64_t F, int32_t *fv, int32_t *fe, int64_t *ff_off,
                      int32_t *ff, cudaStream_t s);
void launch_ee_fill(const int32_t *ev, int64_t E, const int64_t *vv_off, const int32_t *eid_sorted,
                    const int64_t *ee_off, int32_t *ee, cudaStream_t s);
void launch_tt_vertex_count(const int4 *tvs, int64_t T, const int64_t *vt_off, const int32_t *vt,
                            int32_t *cnt, cudaStream_t s);
void launch_tt_vertex_fill(const int4 *tvs, int64_t T, const int64_t *vt_off, const int32_t *vt,
                           const int64_t *tt_off, int32_t *tt, cudaStream_t s);

// ---- heavy vertices (tg_heavy.cu) ----
// Stars of more than kMaxStar cells: they follow every other vertex with
// cells in the star processing order (positions n_light .. n_light +
// n_heavy - 1), and these kernels do their share of star passes A and B.
struct HeavyStars {
    int64_t n_light, n_heavy;
    const int64_t *pofs;
    const int32_t *vorder;
    const int32_t *vtp;
    const int4 *tvs;
    int2 *pairs;               // 3 per heavy star entry: (neighbour, position), sorted by pass A
    int32_t *ids;              // 6 per heavy star entry (pass B scratch)
    DevStatus *st;
    // pass A
    int32_t *deg;
    uint32_t *ecnt, *eflag, *fflag, *fbnd;
    // pass B
    const int64_t *vv_off;
    const uint2 *erank, *frank;
    int32_t *vv, *eid_sorted, *te, *tf, *ft, *et;
    const int64_t *et_off;
};
void launch_heavy_a(const HeavyStars &h, cudaStream_t s);
void launch_heavy_b(const HeavyStars &h, cudaStream_t s);
// EE rows of edges with an endpoint of more than kMaxDeg neighbours
void launch_ee_heavy(const int32_t *ev, int64_t E, const int64_t *vv_off, const int32_t *eid,
                     const int64_t *ee_off, int32_t *ee, cudaStream_t s);
// classes of the vertices in [v0, v0 + nv) with more than kMaxDeg neighbours
// (at most max_listed of them): list (capacity max_listed) and n_list (one
// int, zeroed by the caller) are scratch, scratch holds one int per VV entry
void launch_crit_heavy(const int64_t *vv_off, const int32_t *vv, int64_t v0, int64_t nv,
                       int64_t max_listed, const void *field, int field_type, uint32_t *classes3,
                       int32_t *list, int32_t *n_list, int32_t *scratch, cudaStream_t s);

// critical points (tg_crit.cu)
// vv_win: window table of VV (launch_window_starts over vv_off, crit_window())
int crit_window();
// heavy: 0 no row longer than kMaxDeg, 1 such rows get the heavy path
// (masks of their light neighbours computed from the light side), 2 report
// them with ST_HEAVY_DEG
// order / ooff / ostart: visit the rows in this vertex order (ooff: the row
// lengths' prefix in it, V + 1 entries; ostart: each row's start in VV;
// vv_win a window table over ooff), or null for id order (vv_win over vv_off)
void launch_crit_adj(const int64_t *vv_off, const int32_t *vv, const int32_t *order,
                     const int64_t *ooff, const int64_t *ostart, const int32_t *vv_win,
                     int64_t V, int64_t n_vv, uint64_t *adj, DevStatus *st, int heavy,
                     cudaStream_t s);
// len[i] = length and start[i] = first entry of VV row order[i] (0 from
// n_with_cells on)
void launch_vv_lengths_in_order(const int64_t *vv_off, const int32_t *order, int64_t V,
                                int64_t n_with_cells, int32_t *len, int64_t *start,
                                cudaStream_t s);
// classify rows [v0, v0 + nv): field and classes3 hold nv values / rows from v0
void launch_crit_classify(const int64_t *vv_off, const int32_t *vv, const uint64_t *adj,
                          const void *field, int field_type, int64_t v0, int64_t nv,
                          uint32_t *classes3, cudaStream_t s);

// the message tg_last_error_string returns on this thread
void set_last_error(const char *msg);
// Cell segments of a mesh (the meshes of a batch, tg_batch.cu): seg_c_host
// holds n + 1 cell starts; each extraction then fills n + 1 first edge ids
// followed by n + 1 first face ids (device, read by mesh_segment_ids).
tg_status mesh_set_segments(tg_mesh *m, const int64_t *seg_c_host, int64_t n, cudaStream_t s);
const int64_t *mesh_segment_ids(const tg_mesh *m);
// tg_critical_points restricted to the vertices [v0, v0 + nv), which must
// hold every neighbour of their vertices (a whole mesh of a batch): field
// holds their nv values, classes_out their nv rows
tg_status critical_points_rows(tg_mesh *m, int64_t v0, int64_t nv, const void *field,
                               int field_type, int field_on_device, uint32_t *classes_out,
                               int out_on_device, cudaStream_t s);

// launch accounting and optional CUDA-event timing of one named kernel
void count_launch(int n = 1);
void prof_begin(const char *name, cudaStream_t s);
void prof_end(const char *name, cudaStream_t s);

// RAII wrapper around every launch: counts it and, when the kernel is the
// one selected with tg_profile_kernel, brackets it with CUDA events.
#ifdef __CUDACC__
// Programmatic dependent launch.  Kernels go out with programmatic stream
// serialisation allowed, so a kernel's launch is processed while the kernel
// before it on the stream runs.  Every kernel starts with griddep_wait(),
// which returns once the grids it depends on have completed and their memory
// is visible (at once when it was not launched that way).  The kernels do not
// signal their dependents early: blocks of the next kernel waiting on SMs
// cost the running one more than the earlier start saves.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Asynchronous global -> shared copies (cp.async): no register holds the
// data in flight, so a kernel can put many dependent-load chains' loads in
// flight at once.  A thread sees its own copies after cp_async_wait(); other
// threads' after that and a barrier.
template <int B>
__device__ __forceinline__ void cp_async(void *smem, const void *gmem)
{
    static_assert(B == 4 || B == 8 || B == 16, "cp.async copies 4, 8 or 16 bytes");
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem);
    if constexpr (B == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gmem) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(d), "l"(gmem), "n"(B)
                     : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_all;" ::: "memory"); }
template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                       Args &&...args)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}
#endif

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
