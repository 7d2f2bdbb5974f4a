// tg_api.cu -- host orchestration of the relation pipeline behind the C ABI
// declared in include/tetragpu.h.
//
// One tg_mesh owns its device buffers.  Memory comes from the device's
// stream-ordered pool (cudaMallocAsync) with an unlimited release threshold,
// so repeated extractions reuse blocks instead of returning them to the
// driver.  tg_extract synchronises the stream at two points, to learn the
// edge/face/neighbour counts and then the CSR totals that size the outputs;
// everything between those points is asynchronous on the caller's stream.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "tetragpu.h"
#include "tg_internal.h"

namespace tg {
static std::atomic<long long> g_launches{0};
void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// Optional timing of one named kernel with CUDA events on its own stream
// (tg_profile_kernel / tg_profile_read).  Off unless a name is set.
namespace {
std::mutex g_prof_mu;
std::string g_prof_name;
std::atomic<bool> g_prof_on{false};
struct EvPair {
    cudaEvent_t a, b;
};
std::vector<EvPair> g_prof_events;
std::vector<cudaEvent_t> g_prof_pool;
cudaEvent_t g_prof_open = nullptr;

cudaEvent_t prof_event()
{
    if (!g_prof_pool.empty()) {
        cudaEvent_t e = g_prof_pool.back();
        g_prof_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}
}  // namespace

void prof_begin(const char *name, cudaStream_t s)
{
    if (!g_prof_on.load(std::memory_order_relaxed)) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    if (g_prof_name != name) return;
    g_prof_open = prof_event();
    cudaEventRecord(g_prof_open, s);
}

void prof_end(const char *name, cudaStream_t s)
{
    if (!g_prof_on.load(std::memory_order_relaxed)) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    if (g_prof_name != name || !g_prof_open) return;
    cudaEvent_t b = prof_event();
    cudaEventRecord(b, s);
    g_prof_events.push_back({g_prof_open, b});
    g_prof_open = nullptr;
}
}  // namespace tg

using namespace tg;

namespace {

thread_local std::string g_err;

tg_status fail(tg_status code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

tg_status cuda_fail(cudaError_t e, const char *what, int line)
{
    (void)cudaGetLastError();
    return fail(e == cudaErrorMemoryAllocation ? TG_ERR_OUT_OF_MEMORY : TG_ERR_CUDA,
                "%s (%s) at tg_api.cu:%d: %s", cudaGetErrorName(e), cudaGetErrorString(e), line,
                what);
}

#define CK(call)                                                        \
    do {                                                                \
        cudaError_t _e = (call);                                        \
        if (_e != cudaSuccess) return cuda_fail(_e, #call, __LINE__);   \
    } while (0)

#define TRY(expr)                                   \
    do {                                            \
        tg_status _s = (expr);                      \
        if (_s != TG_OK) return _s;                 \
    } while (0)

constexpr int64_t kMaxCells = 357913941LL;  // 6 * cells must fit in 31 bits

std::mutex g_pool_mu;
bool g_pool_ready[64];

void setup_pool(int dev)
{
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (dev < 0 || dev >= 64 || g_pool_ready[dev]) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    (void)cudaGetLastError();
    g_pool_ready[dev] = true;
}

// Pinned, device-mapped host slots for the status word and the sizes read
// back at the synchronisation points: a kernel stores them there directly,
// so a read-back never queues behind large copies in flight on the copy
// engines (a caller draining an earlier mesh's relations).  Pinned
// allocation is slow, so slots come from a process-wide pool of 4 KiB
// chunks and are recycled.
struct PinnedPool {
    std::mutex mu;
    std::vector<void *> free_slots;
    void *get()
    {
        std::lock_guard<std::mutex> lk(mu);
        if (free_slots.empty()) {
            char *chunk = nullptr;
            if (cudaHostAlloc((void **)&chunk, 4096, cudaHostAllocMapped) != cudaSuccess)
                return nullptr;
            for (int i = 0; i < 16; i++) free_slots.push_back(chunk + 256 * i);
        }
        void *p = free_slots.back();
        free_slots.pop_back();
        return p;
    }
    void put(void *p)
    {
        if (!p) return;
        std::lock_guard<std::mutex> lk(mu);
        free_slots.push_back(p);
    }
};
PinnedPool g_pinned;

// Side streams for kernels of one extraction that need nothing from each
// other (EF, TT, the per-face rows and the link adjacency beside EE):
// a stream and its fork / join events, kept per device and reused, so that a
// mesh built per request creates none.
struct SideLane {
    int device = 0;
    cudaStream_t s = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};
struct SidePool {
    std::mutex mu;
    std::vector<SideLane *> free_lanes;
    SideLane *get(int device)
    {
        {
            std::lock_guard<std::mutex> lk(mu);
            for (size_t i = 0; i < free_lanes.size(); i++)
                if (free_lanes[i]->device == device) {
                    SideLane *l = free_lanes[i];
                    free_lanes.erase(free_lanes.begin() + (std::ptrdiff_t)i);
                    return l;
                }
        }
        SideLane *l = new SideLane();
        l->device = device;
        if (cudaStreamCreateWithFlags(&l->s, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&l->fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&l->join, cudaEventDisableTiming) != cudaSuccess) {
            (void)cudaGetLastError();
            if (l->s) cudaStreamDestroy(l->s);
            if (l->fork) cudaEventDestroy(l->fork);
            delete l;
            return nullptr;
        }
        return l;
    }
    void put(SideLane *l)
    {
        if (!l) return;
        std::lock_guard<std::mutex> lk(mu);
        free_lanes.push_back(l);
    }
};
SidePool g_side;

// One fork of an extraction's stream: the stream fork() returns runs what it
// is given after everything enqueued on the main stream before the call;
// join() makes the main stream wait for that work.  The destructor joins, so
// declared after the extraction's temporaries it orders their frees after
// the side work, on every return path.  Without a side stream (none could
// be made) fork() returns the main stream itself.
struct Fork {
    cudaStream_t main;
    int device;
    SideLane *lane = nullptr;
    bool open = false;
    Fork(cudaStream_t s, int dev) : main(s), device(dev) {}
    cudaStream_t fork()
    {
        join();
        if (!lane) lane = g_side.get(device);
        if (!lane) return main;
        if (cudaEventRecord(lane->fork, main) != cudaSuccess ||
            cudaStreamWaitEvent(lane->s, lane->fork, 0) != cudaSuccess) {
            (void)cudaGetLastError();
            return main;
        }
        open = true;
        return lane->s;
    }
    void join()
    {
        if (!open) return;
        open = false;
        if (cudaEventRecord(lane->join, lane->s) != cudaSuccess ||
            cudaStreamWaitEvent(main, lane->join, 0) != cudaSuccess) {
            // the main stream cannot be ordered after the side stream: wait
            // for it from the host instead
            (void)cudaGetLastError();
            cudaStreamSynchronize(lane->s);
        }
    }
    ~Fork()
    {
        join();
        g_side.put(lane);
    }
};

struct Rel {
    int64_t rows = 0, entries = 0;
    int width = 0;
    int64_t *off = nullptr;
    int32_t *ent = nullptr;
    bool ready = false;
    uint32_t opts = 0;
};

const int kWidth[14] = {0, 6, 2, 0, 4, 3, 3, 2, 0, 0, 0, 0, 0, 0};
const char *kName[14] = {"validate", "TE", "EV", "ET", "TF", "FV", "FE",
                         "FT",       "EF", "VT", "TT", "FF", "EE", "VV"};

// Scoped list of stream-ordered temporaries, freed when the stage ends.
struct Temps {
    cudaStream_t s;
    void *p[64];
    int n = 0;
    explicit Temps(cudaStream_t st) : s(st) {}
    ~Temps()
    {
        for (int i = 0; i < n; i++)
            if (p[i]) cudaFreeAsync(p[i], s);
    }
    template <class T>
    tg_status alloc(T **out, int64_t count, bool zero = false)
    {
        size_t b = (size_t)std::max<int64_t>(count, 1) * sizeof(T);
        if (n >= 64) return fail(TG_ERR_UNSUPPORTED, "too many temporaries in one stage");
        void *q = nullptr;
        cudaError_t e = cudaMallocAsync(&q, b, s);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMallocAsync (temporary)", __LINE__);
        if (zero) {
            e = cudaMemsetAsync(q, 0, b, s);
            if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync", __LINE__);
        }
        p[n++] = q;
        *out = (T *)q;
        return TG_OK;
    }
    // free q with the others if the stage fails (list sized for every path)
    void track(void *q) { p[n++] = q; }
    // hand a temporary over to the caller (it is not freed here)
    void keep(void *q)
    {
        for (int i = 0; i < n; i++)
            if (p[i] == q) p[i] = nullptr;
    }
};

template <class T>
tg_status dalloc(T **out, int64_t count, cudaStream_t s)
{
    size_t b = (size_t)std::max<int64_t>(count, 1) * sizeof(T);
    void *q = nullptr;
    cudaError_t e = cudaMallocAsync(&q, b, s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMallocAsync", __LINE__);
    *out = (T *)q;
    return TG_OK;
}

// Offsets of several arrays in one allocation (each on a 256-byte boundary),
// so that arrays zeroed together cost one memset.
struct Carve {
    size_t bytes = 0;
    template <class T>
    size_t add(int64_t n)
    {
        const size_t off = bytes;
        bytes += ((size_t)std::max<int64_t>(n, 1) * sizeof(T) + 255) & ~size_t(255);
        return off;
    }
};

}  // namespace

void tg::set_last_error(const char *msg) { g_err = msg; }

struct tg_mesh {
    int device = 0;
    cudaStream_t last_stream = nullptr;  // stream of the last call, used to free asynchronously
    int64_t V = 0, T = 0, E = -1, F = -1;
    int4 *tvs = nullptr;
    int32_t *vt_win = nullptr;          // VT window table (window_count + 1 entries)
    // star processing order: vertices by first cell (see tg_star.cu)
    int32_t *vorder = nullptr;          // [V] vertex at each position (cell-less ones last)
    int64_t *pofs = nullptr;            // [V + 1] VT offsets in that order
    int32_t *vtp = nullptr;             // [4T] VT rows in that order
    int32_t *st_win = nullptr;          // window table over pofs (star pass A)
    int32_t *st_win_b = nullptr;        // the same for star pass B's windows
    int32_t *st_wbase = nullptr;        // first entry of each pass A window
    int32_t *st_wbase_b = nullptr;      // first entry of each pass B window
    ScanWorkspace scan;                 // every prefix scan of the mesh (tg_scan.cu)
    // segments of cells (the meshes of a batch): cell starts, and after each
    // extraction their first edge and face ids (device, n_seg + 1 each)
    int64_t n_seg = 0;
    int64_t *seg_c = nullptr;
    int64_t *seg_ef = nullptr;
    Rel rel[14];
    // stars of more than kMaxStar cells (tg_heavy.cu): processing positions
    // n_light .. n_light + n_heavy - 1, heavy_entries VT entries in all
    int64_t n_light = 0, n_heavy = 0, heavy_entries = 0;
    bool wide_stars = false;    // a light star holds more than 32 cells (64-bit star masks)
    int max_deg = 0;            // largest degree above kMaxDeg seen by the extraction, else 0
    uint64_t *cadj = nullptr;   // link adjacency for critical points, aligned with VV
    DevStatus *st = nullptr;    // device
    DevStatus *st_host = nullptr;
    int64_t *sz_host = nullptr; // pinned slots for sizes read back at sync points
};

namespace {

void free_rel(Rel &r, cudaStream_t s = nullptr, bool async = false)
{
    if (async) {
        if (r.off) cudaFreeAsync(r.off, s);
        if (r.ent) cudaFreeAsync(r.ent, s);
    } else {
        if (r.off) cudaFree(r.off);
        if (r.ent) cudaFree(r.ent);
    }
    r = Rel();
}

tg_status reset_status(tg_mesh *m, cudaStream_t s)
{
    launch_reset_status(m->st, s);
    return TG_OK;
}

// Read the status word plus up to 8 device scalars (int64 if `wide[i]`,
// else int32) into m->sz_host, synchronously.
tg_status sync_read(tg_mesh *m, cudaStream_t s, int n, const void *const *src, const bool *wide)
{
    PublishArgs a{};
    a.st = m->st;
    a.n = n;
    for (int i = 0; i < n; i++) {
        a.src[i] = src[i];
        a.wide[i] = wide[i] ? 1 : 0;
    }
    CK(cudaHostGetDevicePointer((void **)&a.h_st, m->st_host, 0));
    CK(cudaHostGetDevicePointer((void **)&a.h_sz, m->sz_host, 0));
    launch_publish(a, s);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s));
    return TG_OK;
}

tg_status check_flags(const tg_mesh *m, unsigned mask_ok = 0)
{
    const DevStatus &h = *m->st_host;
    const unsigned f = h.flags & ~mask_ok;
    if (!f) return TG_OK;
    if (f & ST_BAD_ID)
        return fail(TG_ERR_INVALID_MESH, "cell %d has a vertex id outside [0, %lld)", h.bad_cell,
                    (long long)m->V);
    if (f & ST_DUP_VERTEX)
        return fail(TG_ERR_INVALID_MESH, "cell %d repeats a vertex", h.bad_cell);
    if (f & ST_NONMANIFOLD_FACE)
        return fail(TG_ERR_INVALID_MESH, "a face of cell %d lies in more than two cells",
                    h.bad_cell);
    if (f & ST_HEAVY_STAR)
        return fail(TG_ERR_UNSUPPORTED,
                    "vertex %d lies in more than %d cells (largest star this build handles)",
                    h.bad_vertex, kMaxStar);
    if (f & ST_HEAVY_DEG)
        return fail(TG_ERR_UNSUPPORTED,
                    "a vertex has %d neighbours (more than %d, the largest this build handles)",
                    h.max_deg, kMaxDeg);
    if (f & ST_HASH_FULL)
        return fail(TG_ERR_UNSUPPORTED, "vertex %d: neighbour table overflow", h.bad_vertex);
    if (f & ST_STAR_OVERFLOW)
        return fail(TG_ERR_UNSUPPORTED, "vertex %d: neighbour summary overflow", h.bad_vertex);
    if (f & ST_SCAN_STALLED)
        return fail(TG_ERR_CUDA, "a prefix scan gave up waiting for a preceding tile");
    return fail(TG_ERR_CUDA, "unexpected device status 0x%x", f);
}

inline uint32_t bit(int r) { return 1u << r; }

tg_status set_fixed(tg_mesh *m, int r, int32_t *ent, int64_t rows)
{
    free_rel(m->rel[r]);
    Rel &x = m->rel[r];
    x.rows = rows;
    x.width = kWidth[r];
    x.entries = rows * kWidth[r];
    x.ent = ent;
    x.ready = true;
    return TG_OK;
}

void set_csr(tg_mesh *m, int r, int64_t *off, int32_t *ent, int64_t rows, int64_t entries,
             uint32_t opts = 0)
{
    free_rel(m->rel[r]);
    Rel &x = m->rel[r];
    x.rows = rows;
    x.entries = entries;
    x.width = 0;
    x.off = off;
    x.ent = ent;
    x.ready = true;
    x.opts = opts;
}

// The link adjacency of critical points into m->cadj (allocated by the
// caller), on stream s: VV's rows visited in the star processing order, so
// that the neighbours' rows a window reads were read by the windows just
// before it (in L2); the order's row lengths, their prefix and its window
// table are temporaries of tmp.
tg_status build_link_adjacency(tg_mesh *m, const int64_t *vv_off, const int32_t *vv, int64_t nvv,
                               Temps &tmp, cudaStream_t s)
{
    const int64_t V = m->V;
    int32_t *len, *win;
    int64_t *ooff, *ostart;
    TRY(tmp.alloc(&len, V));
    TRY(tmp.alloc(&ooff, V + 1));
    TRY(tmp.alloc(&ostart, V));
    TRY(tmp.alloc(&win, window_count(nvv, crit_window()) + 1));
    launch_vv_lengths_in_order(vv_off, m->vorder, V, m->n_light + m->n_heavy, len, ostart, s);
    ScanJob job{len, ooff, V, SCAN_COUNT_I32, 0};
    scan_batch(&job, 1, m->scan, m->st, s);
    launch_window_starts(ooff, V, nvv, crit_window(), win, s);
    launch_crit_adj(vv_off, vv, m->vorder, ooff, ostart, win, V, nvv, m->cadj, m->st,
                    m->max_deg ? 1 : 0, s);
    return TG_OK;
}

tg_status run_extract(tg_mesh *m, uint32_t mask, uint32_t opts, cudaStream_t s)
{
    const int64_t V = m->V, T = m->T, NVT = 4 * T;
    const bool tt_vertex = (opts & TG_OPT_TT_VERTEX_SHARING) != 0;
    const bool want_tt_face = (mask & TG_TT) && !tt_vertex;
    const uint32_t star_rel = TG_TE | TG_EV | TG_ET | TG_TF | TG_FV | TG_FE | TG_FT | TG_EF |
                              TG_FF | TG_EE | TG_VV;
    const bool want_star = (mask & star_rel) || want_tt_face;
    const int64_t *vt_off = m->rel[TG_REL_VT].off;
    const int32_t *vt = m->rel[TG_REL_VT].ent;
    Temps tmp(s);
    Fork side(s, m->device);   // after tmp: joined before its frees

    if (want_star) {
        // the status is clean: the read-back that ended the last call reset it
        // ---- pass A: first occurrences, neighbour counts, ET/EF row lengths ----
        const int64_t nwe = (6 * T + 31) / 32, nwf = (4 * T + 31) / 32;
        uint32_t *eflag, *fflag, *fbnd;
        uint2 *erank, *frank, *brank;
        uint32_t *ecnt = nullptr;
        int32_t *deg;
        int64_t *vv_off;
        const bool need_ecnt = mask & (TG_ET | TG_EF | TG_EE);
        {
            // the bitmaps pass A sets bits in and the neighbour counts: one
            // zeroed allocation (the row lengths are read only where pass A
            // wrote them: no zeroing)
            Carve c;
            const size_t o_e = c.add<uint32_t>(nwe), o_f = c.add<uint32_t>(nwf),
                         o_b = c.add<uint32_t>(nwf), o_d = c.add<int32_t>(V);
            char *z;
            TRY(tmp.alloc(&z, (int64_t)c.bytes, true));
            eflag = (uint32_t *)(z + o_e);
            fflag = (uint32_t *)(z + o_f);
            fbnd = (uint32_t *)(z + o_b);
            deg = (int32_t *)(z + o_d);
        }
        TRY(tmp.alloc(&erank, nwe + 1));
        TRY(tmp.alloc(&frank, nwf + 1));
        TRY(tmp.alloc(&brank, nwf + 1));
        if (need_ecnt) TRY(tmp.alloc(&ecnt, 6 * T));
        TRY(dalloc(&vv_off, V + 1, s));
        tmp.track(vv_off);  // owned by the VV relation once it is ready
        int64_t *deg_sq;  // prefix of deg^2: its total sizes EE (sum deg^2 - 2E)
        TRY(tmp.alloc(&deg_sq, V + 1));
        // pass A's candidate masks, pass B's input: their low 32 bits for
        // every entry, the high 32 for the entries of stars of more than 32
        // cells (an array only when the mesh has such stars; only their
        // entries of it are touched)
        const bool narrow = !m->wide_stars;
        uint32_t *emask, *emask_hi = nullptr;
        TRY(tmp.alloc(&emask, 3 * NVT));
        if (!narrow) TRY(tmp.alloc(&emask_hi, 3 * NVT));
        StarA a{m->pofs, m->st_win, m->st_wbase, m->vorder, m->vtp, m->tvs, V, NVT, deg, ecnt,
                eflag, fflag, fbnd, m->st, emask, emask_hi, narrow, NVT - m->heavy_entries};
        if (!ecnt) {
            // pass A always records row lengths; give it a throwaway buffer
            TRY(tmp.alloc(&ecnt, 6 * T));
            a.ecnt = ecnt;
        }
        launch_star_a(a, s);
        HeavyStars hv{};
        if (m->n_heavy > 0) {
            hv.n_light = m->n_light;
            hv.n_heavy = m->n_heavy;
            hv.pofs = m->pofs;
            hv.vorder = m->vorder;
            hv.vtp = m->vtp;
            hv.tvs = m->tvs;
            hv.st = m->st;
            TRY(tmp.alloc(&hv.pairs, 3 * m->heavy_entries));
            TRY(tmp.alloc(&hv.ids, 6 * m->heavy_entries));
            hv.deg = deg;
            hv.ecnt = a.ecnt;
            hv.eflag = eflag;
            hv.fflag = fflag;
            hv.fbnd = fbnd;
            launch_heavy_a(hv, s);
        }
        ScanJob jobs[5] = {{deg, vv_off, V, SCAN_COUNT_I32, 0},
                           {eflag, erank, nwe, SCAN_POPC_RANK, 0},
                           {fflag, frank, nwf, SCAN_POPC_RANK, 0},
                           {fbnd, brank, nwf, SCAN_POPC_RANK, 0},
                           {deg, deg_sq, V, SCAN_SQUARE_I32, 0}};
        scan_batch(jobs, 5, m->scan, m->st, s);

        // ---- the one synchronisation: edge, face, neighbour and boundary
        // counts size every output from here on ----
        {
            const void *src[5] = {vv_off + V, &erank[nwe].y, &frank[nwf].y, &brank[nwf].y,
                                  deg_sq + V};
            const bool w8[5] = {true, false, false, false, true};
            TRY(sync_read(m, s, 5, src, w8));
        }
        if (m->st_host->flags) return check_flags(m);
        m->max_deg = m->st_host->max_deg > kMaxDeg ? m->st_host->max_deg : 0;
        const int64_t nvv = m->sz_host[0];
        const int64_t E = m->sz_host[1], F = m->sz_host[2];
        const int64_t n_bnd = m->sz_host[3];  // boundary faces
        const int64_t sum_deg_sq = m->sz_host[4];
        m->E = E;
        m->F = F;
        if (m->seg_c) launch_seg_ranks(m->seg_c, m->n_seg, erank, frank, m->seg_ef, s);
        int64_t *et_off = nullptr, *ef_off = nullptr, *ee_off = nullptr;
        // EF rows are read off ET rows and TF (k_ef_fill): ET, TF and EV are
        // made for EF too
        const bool need_et = mask & (TG_ET | TG_EF);
        if (need_et) TRY(dalloc(&et_off, E + 1, s));
        if (mask & TG_EF) TRY(dalloc(&ef_off, E + 1, s));
        if (mask & TG_EE) TRY(dalloc(&ee_off, E + 1, s));
        if (et_off) tmp.track(et_off);
        if (ef_off) tmp.track(ef_off);
        if (ee_off) tmp.track(ee_off);
        // ---- pass B: ids, VV, fixed-width relations, ET rows ----
        const bool need_ev = mask & (TG_EV | TG_EE | TG_EF);
        const bool need_te = mask & (TG_TE | TG_FE);
        // FV and FE are read off each face's first cell (k_face_fill), which
        // the face's FT row and the cell's TF row tell
        const bool need_tf = (mask & (TG_TF | TG_FV | TG_FE | TG_FF | TG_EF)) || want_tt_face;
        const bool need_ft = (mask & (TG_FT | TG_FV | TG_FE | TG_FF)) || want_tt_face;
        int32_t *vv, *eid_sorted = nullptr;
        int32_t *ev = nullptr, *te = nullptr, *tf = nullptr, *fv = nullptr, *ft = nullptr;
        int64_t *ff_off = nullptr;
        // each kernel goes out once its own buffers exist; the later
        // allocations are made while it runs
        if (need_ev) TRY(tmp.alloc(&ev, 2 * E));
        if (et_off || ef_off || ee_off || ev) {
            uint2 *len;
            TRY(tmp.alloc(&len, E));
            launch_edge_offsets(eflag, ecnt, m->tvs, deg, erank, 6 * T, E, et_off, ef_off, ee_off,
                                ev, len, m->scan, m->st, s);
        }
        TRY(dalloc(&vv, nvv, s));
        tmp.track(vv);
        if (mask & TG_EE) TRY(tmp.alloc(&eid_sorted, nvv));
        if (need_te) TRY(tmp.alloc(&te, 6 * T));
        if (need_tf) TRY(tmp.alloc(&tf, 4 * T));
        if (mask & TG_FV) TRY(tmp.alloc(&fv, 3 * F));
        if (need_ft) TRY(tmp.alloc(&ft, 2 * F));
        if (mask & TG_FF) TRY(tmp.alloc(&ff_off, F + 1));
        // CSR totals: ET = 6T, EF = 3F always; EE from the scan (read back
        // only when EE is wanted); TT and FF from the boundary-face count
        int32_t *et = nullptr, *ef = nullptr, *ee = nullptr, *ff = nullptr, *tt = nullptr,
                *fe = nullptr;
        int64_t *tt_off = nullptr;
        const int64_t n_et = 6 * T, n_ef = 3 * F;
        const int64_t n_tt = 4 * T - n_bnd, n_ff = 3 * (2 * F - n_bnd);
        if (et_off) TRY(dalloc(&et, n_et, s));
        if (ef_off) TRY(dalloc(&ef, n_ef, s));
        if (et && !(mask & TG_ET)) tmp.track(et);   // a temporary for EF (et_off is tracked)
        if (mask & TG_FE) TRY(dalloc(&fe, 3 * F, s));
        if (want_tt_face) {
            TRY(dalloc(&tt_off, T + 1, s));
            TRY(dalloc(&tt, n_tt, s));
            if (T == 0) CK(cudaMemsetAsync(tt_off, 0, 8, s));
        }
        if (mask & TG_FF) {
            TRY(dalloc(&ff, n_ff, s));
            if (T == 0) CK(cudaMemsetAsync(ff_off, 0, 8, s));
        }
        StarB b{};
        b.pofs = m->pofs; b.win = m->st_win_b; b.wbase = m->st_wbase_b; b.vorder = m->vorder;
        b.vtp = m->vtp;
        b.tvs = m->tvs; b.V = V; b.nvt = NVT;
        b.vv_off = vv_off; b.erank = erank; b.frank = frank; b.brank = brank;
        b.emask = emask; b.emask_hi = emask_hi; b.narrow = narrow; b.vv = vv; b.eid_sorted = eid_sorted;
        b.te = te; b.tf = tf; b.ft = ft;
        b.et_off = et_off; b.et = et; b.st = m->st;
        launch_star_b(b, s);
        if (m->n_heavy > 0) {
            hv.vv_off = vv_off;
            hv.erank = erank;
            hv.frank = frank;
            hv.vv = vv;
            hv.eid_sorted = eid_sorted;
            hv.te = te;
            hv.tf = tf;
            hv.ft = ft;
            hv.et = et;
            hv.et_off = et_off;
            launch_heavy_b(hv, s);
        }
        tmp.keep(vv);
        tmp.keep(vv_off);
        set_csr(m, TG_REL_VV, vv_off, vv, V, nvv);
        if (m->cadj) {
            cudaFreeAsync(m->cadj, s);
            m->cadj = nullptr;
        }

        // EF, the per-cell TT rows, the per-face FV / FE / FF rows and on
        // request the link adjacency of critical points, on a side stream
        // beside EE (each reads only what pass B and the passes before it
        // wrote)
        const int64_t n_ee = sum_deg_sq - 2 * E;   // deg(a) + deg(b) - 2 per edge (a,b)
        if (ee_off) TRY(dalloc(&ee, n_ee, s));
        const bool prep_adj = (opts & TG_OPT_LINK_ADJACENCY) && (mask & TG_VV);
        if (prep_adj) TRY(dalloc(&m->cadj, nvv, s));
        if (fv || fe || tt || ff_off || ff || ef || prep_adj) {
            const cudaStream_t s2 = side.fork();
            if (ef) launch_ef_fill(ev, E, et_off, et, m->tvs, tf, ef_off, ef, s2);
            if (tt || ff_off) launch_cell_tt(T, F, tf, ft, brank, tt_off, tt, ff_off, s2);
            if (fv || fe || ff) launch_face_fill(ft, tf, m->tvs, te, brank, F, fv, fe, ff_off, ff, s2);
            if (prep_adj) TRY(build_link_adjacency(m, vv_off, vv, nvv, tmp, s2));
        }
        if (ee_off) {
            launch_ee_fill(ev, E, vv_off, eid_sorted, ee_off, ee, s);
            if (m->max_deg) launch_ee_heavy(ev, E, vv_off, eid_sorted, ee_off, ee, s);
        }
        side.join();
        CK(cudaGetLastError());

        auto give_fixed = [&](int r, int32_t *p, int64_t rows) {
            tmp.keep(p);
            set_fixed(m, r, p, rows);
        };
        if (mask & TG_EV) give_fixed(TG_REL_EV, ev, E);
        if (mask & TG_TE) give_fixed(TG_REL_TE, te, T);
        if (mask & TG_TF) give_fixed(TG_REL_TF, tf, T);
        if (mask & TG_FV) give_fixed(TG_REL_FV, fv, F);
        if (mask & TG_FT) give_fixed(TG_REL_FT, ft, F);
        if (fe) set_fixed(m, TG_REL_FE, fe, F);
        if (et && (mask & TG_ET)) {
            tmp.keep(et_off);
            tmp.keep(et);
            set_csr(m, TG_REL_ET, et_off, et, E, n_et);
        }
        if (ef) {
            tmp.keep(ef_off);
            set_csr(m, TG_REL_EF, ef_off, ef, E, n_ef);
        }
        if (ee) {
            tmp.keep(ee_off);
            set_csr(m, TG_REL_EE, ee_off, ee, E, n_ee);
        }
        if (ff) {
            tmp.keep(ff_off);
            set_csr(m, TG_REL_FF, ff_off, ff, F, n_ff);
        }
        if (tt) set_csr(m, TG_REL_TT, tt_off, tt, T, n_tt, 0);
    }

    if ((mask & TG_TT) && tt_vertex) {
        int32_t *cnt;
        int64_t *tt_off;
        TRY(tmp.alloc(&cnt, T));
        TRY(dalloc(&tt_off, T + 1, s));
        launch_tt_vertex_count(m->tvs, T, vt_off, vt, cnt, s);
        ScanJob job{cnt, tt_off, T, SCAN_COUNT_I32, 0};
        scan_batch(&job, 1, m->scan, m->st, s);
        const void *src[1] = {tt_off + T};
        const bool w8[1] = {true};
        TRY(sync_read(m, s, 1, src, w8));
        int32_t *tt;
        TRY(dalloc(&tt, m->sz_host[0], s));
        launch_tt_vertex_fill(m->tvs, T, vt_off, vt, tt_off, tt, s);
        set_csr(m, TG_REL_TT, tt_off, tt, T, m->sz_host[0], TG_OPT_TT_VERTEX_SHARING);
    }
    CK(cudaGetLastError());
    return TG_OK;
}

}  // namespace

tg_status tg::critical_points_rows(tg_mesh *m, int64_t v0, int64_t nv, const void *field,
                                   int field_type, int field_on_device, uint32_t *classes_out,
                                   int out_on_device, cudaStream_t s)
{
    if (!m || !field || !classes_out) return fail(TG_ERR_INVALID_ARGUMENT, "NULL argument");
    if (field_type != TG_FIELD_F32 && field_type != TG_FIELD_F64)
        return fail(TG_ERR_INVALID_ARGUMENT, "field_type must be TG_FIELD_F32 or TG_FIELD_F64");
    if (v0 < 0 || nv < 0 || v0 + nv > m->V) return fail(TG_ERR_INVALID_ARGUMENT, "bad vertex range");
    m->last_stream = s;
    if (!m->rel[TG_REL_VV].ready) TRY(tg_extract(m, TG_VV, 0, s));
    const int64_t V = m->V;
    const Rel &vv = m->rel[TG_REL_VV];
    if (!m->cadj) {
        TRY(dalloc(&m->cadj, vv.entries, s));
        // VV rows longer than the adjacency masks take the heavy path of the
        // classification, so no status read-back here
        Temps adj_tmp(s);
        TRY(build_link_adjacency(m, vv.off, vv.ent, vv.entries, adj_tmp, s));
    }
    Temps tmp(s);
    const size_t esz = field_type == TG_FIELD_F64 ? 8 : 4;
    const void *f = field;
    if (!field_on_device) {
        char *d;
        TRY(tmp.alloc(&d, (int64_t)(nv * esz)));
        CK(cudaMemcpyAsync(d, field, nv * esz, cudaMemcpyHostToDevice, s));
        f = d;
    }
    uint32_t *out = classes_out;
    if (!out_on_device) TRY(tmp.alloc(&out, 3 * nv));
    launch_crit_classify(vv.off, vv.ent, m->cadj, f, field_type, v0, nv, out, s);
    if (m->max_deg) {
        // vertices of more than kMaxDeg neighbours: at most one per
        // kMaxDeg + 1 VV entries
        const int64_t max_listed = std::min<int64_t>(nv, vv.entries / (kMaxDeg + 1) + 1);
        int32_t *list, *n_list, *scratch;
        TRY(tmp.alloc(&list, max_listed));
        TRY(tmp.alloc(&n_list, 1, true));
        TRY(tmp.alloc(&scratch, vv.entries));
        launch_crit_heavy(vv.off, vv.ent, v0, nv, max_listed, f, field_type, out, list, n_list,
                          scratch, s);
    }
    CK(cudaGetLastError());
    if (!out_on_device) {
        CK(cudaMemcpyAsync(classes_out, out, (size_t)nv * 12, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
    return TG_OK;
}

extern "C" {

const char *tg_version(void) { return "tetragpu-gb300 1.1 (sm_103a)"; }

const char *tg_tuning_info(void)
{
    static std::string info;
    static std::once_flag once;
    std::call_once(once, [] {
        char buf[512];
        snprintf(buf, sizeof buf,
                 "{\"TG_STAR_WIN\": %d, \"TG_STAR_WIN_B\": %d, \"TG_STAR_THREADS\": %d, "
                 "\"TG_EFA_LANES\": %d, \"TG_VTS_THREADS\": %d, \"TG_EDGE_ITEMS\": %d, "
                 "\"TG_ADJ_WIN\": %d, \"TG_ADJ_THREADS\": %d, \"TG_EE_GROUP\": %d}",
                 TG_STAR_WIN, TG_STAR_WIN_B, TG_STAR_THREADS, TG_EFA_LANES, TG_VTS_THREADS,
                 TG_EDGE_ITEMS, TG_ADJ_WIN, TG_ADJ_THREADS, TG_EE_GROUP);
        info = buf;
    });
    return info.c_str();
}

const char *tg_last_error_string(void) { return g_err.c_str(); }

int64_t tg_kernel_launch_count(void) { return tg::g_launches.load(); }

tg_status tg_mesh_destroy(tg_mesh *m)
{
    if (!m) return TG_OK;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(m->device);
    // stream-ordered frees on the stream the mesh was last used on, then one
    // wait for that stream (no device-wide synchronisation)
    cudaStream_t s = m->last_stream;
    for (auto &r : m->rel) free_rel(r, s, true);
    if (m->tvs) cudaFreeAsync(m->tvs, s);
    if (m->vt_win) cudaFreeAsync(m->vt_win, s);
    if (m->vorder) cudaFreeAsync(m->vorder, s);
    if (m->pofs) cudaFreeAsync(m->pofs, s);
    if (m->vtp) cudaFreeAsync(m->vtp, s);
    if (m->st_win) cudaFreeAsync(m->st_win, s);
    if (m->st_win_b) cudaFreeAsync(m->st_win_b, s);
    if (m->st_wbase) cudaFreeAsync(m->st_wbase, s);
    if (m->st_wbase_b) cudaFreeAsync(m->st_wbase_b, s);
    if (m->seg_c) cudaFreeAsync(m->seg_c, s);
    if (m->seg_ef) cudaFreeAsync(m->seg_ef, s);
    if (m->cadj) cudaFreeAsync(m->cadj, s);
    if (m->st) cudaFreeAsync(m->st, s);
    if (m->scan.buf) {
        // after the last scan, whichever stream it ran on
        if (m->scan.used && m->scan.last != s) cudaStreamWaitEvent(s, m->scan.done, 0);
        cudaFreeAsync(m->scan.buf, s);
    }
    cudaStreamSynchronize(s);  // no copy into the pinned slots is still in flight
    if (m->scan.done) cudaEventDestroy(m->scan.done);
    g_pinned.put(m->st_host);
    g_pinned.put(m->sz_host);
    cudaSetDevice(cur);
    (void)cudaGetLastError();
    delete m;
    return TG_OK;
}

static tg_status mesh_create_impl(const int32_t *tv, int64_t T, int64_t V, int on_device,
                                  cudaStream_t s, tg_mesh *m)
{
    CK(cudaGetDevice(&m->device));
    setup_pool(m->device);
    m->st_host = (DevStatus *)g_pinned.get();
    m->sz_host = (int64_t *)g_pinned.get();
    if (!m->st_host || !m->sz_host) return fail(TG_ERR_OUT_OF_MEMORY, "pinned host memory");
    TRY(dalloc(&m->st, 1, s));
    TRY(reset_status(m, s));
    TRY(dalloc(&m->tvs, T, s));
    const int32_t *src = tv;
    if (!on_device && T > 0) {
        CK(cudaMemcpyAsync(m->tvs, tv, (size_t)T * 16, cudaMemcpyHostToDevice, s));
        src = reinterpret_cast<const int32_t *>(m->tvs);
    }
    // the scan workspace of every later scan on the mesh, zeroed once
    m->scan.job_words = std::max(scan_job_words(std::max(std::max(V, T), (6 * T + 31) / 32)),
                                 (edge_offsets_words(6 * T) + kMaxScanJobs - 1) / kMaxScanJobs);
    const size_t ws_bytes = (size_t)2 * kMaxScanJobs * m->scan.job_words * 8;
    CK(cudaMallocAsync((void **)&m->scan.buf, ws_bytes, s));
    CK(cudaMemsetAsync(m->scan.buf, 0, ws_bytes, s));
    CK(cudaEventCreateWithFlags(&m->scan.done, cudaEventDisableTiming));
    Temps tmp(s);
    // the per-vertex cell counts and the first-cell bitmap: one zeroed
    // allocation
    const int64_t nwk = (4 * T + 31) / 32;
    int32_t *deg_t, *heavy_cnt;
    uint32_t *vflag;
    {
        Carve c;
        const size_t o_d = c.add<int32_t>(V), o_f = c.add<uint32_t>(nwk), o_h = c.add<int32_t>(3);
        char *z;
        TRY(tmp.alloc(&z, (int64_t)c.bytes, true));
        deg_t = (int32_t *)(z + o_d);
        vflag = (uint32_t *)(z + o_f);
        heavy_cnt = (int32_t *)(z + o_h);
    }
    int4 *occ;
    TRY(tmp.alloc(&occ, T));
    launch_canon(src, T, V, m->tvs, deg_t, occ, m->st, s);
    int64_t *vt_off;
    int32_t *vt;
    TRY(dalloc(&vt_off, V + 1, s));
    ScanJob job{deg_t, vt_off, V, SCAN_COUNT_I32, 0};
    scan_batch(&job, 1, m->scan, m->st, s);
    TRY(dalloc(&vt, 4 * T, s));
    launch_vt_fill(m->tvs, T, vt_off, occ, vt, s);
    TRY(dalloc(&m->vt_win, window_count(4 * T, star_window()) + 1, s));
    launch_window_starts(vt_off, V, 4 * T, star_window(), m->vt_win, s);
    // VT row sort, which also marks each vertex's star-order key; then the
    // star processing order: positions, row lengths, offsets, rows, windows
    uint2 *vrank;
    int64_t *vkey;
    int32_t *dcount;
    TRY(tmp.alloc(&vrank, nwk + 1));
    TRY(tmp.alloc(&vkey, V));
    TRY(tmp.alloc(&dcount, V));
    launch_vt_sort(vt_off, m->vt_win, vt, V, 4 * T, m->tvs, vflag, vkey, heavy_cnt, s);
    {
        ScanJob jf{vflag, vrank, nwk, SCAN_POPC_RANK, 0};
        scan_batch(&jf, 1, m->scan, m->st, s);
        TRY(dalloc(&m->vorder, V, s));
        launch_vorder_place(vt_off, V, vkey, vrank, nwk, heavy_cnt, m->vorder, dcount, s);
        TRY(dalloc(&m->pofs, V + 1, s));
        ScanJob jd{dcount, m->pofs, V, SCAN_COUNT_I32, 0};
        scan_batch(&jd, 1, m->scan, m->st, s);
        TRY(dalloc(&m->vtp, 4 * T, s));
        launch_vtp_fill(m->vorder, m->pofs, V, vt_off, vt, m->vtp, s);
        TRY(dalloc(&m->st_win, window_count(4 * T, star_window()) + 1, s));
        TRY(dalloc(&m->st_win_b, window_count(4 * T, star_window_b()) + 1, s));
        TRY(dalloc(&m->st_wbase, window_count(4 * T, star_window()) + 1, s));
        TRY(dalloc(&m->st_wbase_b, window_count(4 * T, star_window_b()) + 1, s));
        launch_window_starts(m->pofs, V, 4 * T, star_window(), m->st_win, s, star_window_b(),
                             m->st_win_b, m->st_wbase, m->st_wbase_b);
    }
    CK(cudaGetLastError());
    set_csr(m, TG_REL_VT, vt_off, vt, V, 4 * T);
    // vertices with light stars, heavy ones, the heavy stars' entries and
    // whether a light star holds more than 32 cells
    const void *rd[4] = {&vrank[nwk].y, heavy_cnt, heavy_cnt + 1, heavy_cnt + 2};
    const bool w8[4] = {false, false, false, false};
    TRY(sync_read(m, s, 4, rd, w8));
    m->n_light = T ? m->sz_host[0] : 0;
    m->n_heavy = T ? m->sz_host[1] : 0;
    m->heavy_entries = T ? m->sz_host[2] : 0;
    m->wide_stars = T ? m->sz_host[3] != 0 : false;
    return check_flags(m);
}

tg_status tg_mesh_create(const int32_t *tv, int64_t n_cells, int64_t n_verts, int tv_on_device,
                         void *stream, tg_mesh **out)
{
    if (!out) return fail(TG_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (n_cells < 0 || n_verts < 0 || (n_cells > 0 && !tv))
        return fail(TG_ERR_INVALID_ARGUMENT, "bad mesh sizes or NULL TV");
    if (n_cells > kMaxCells)
        return fail(TG_ERR_UNSUPPORTED, "more than %lld cells (occurrence ids use 31 bits)",
                    (long long)kMaxCells);
    if (n_verts > INT_MAX) return fail(TG_ERR_UNSUPPORTED, "more than 2^31-1 vertices");
    tg_mesh *m = new tg_mesh();
    m->V = n_verts;
    m->T = n_cells;
    m->last_stream = (cudaStream_t)stream;
    tg_status st = mesh_create_impl(tv, n_cells, n_verts, tv_on_device, (cudaStream_t)stream, m);
    if (st != TG_OK) {
        std::string keep = g_err;
        tg_mesh_destroy(m);
        g_err = keep;
        return st;
    }
    *out = m;
    return TG_OK;
}

tg_status tg_tv_narrow_i64(const int64_t *cells, int64_t n_cells, int64_t n_points, int32_t *out)
{
    if (n_cells < 0 || n_points < 0 || (n_cells > 0 && (!cells || !out)))
        return fail(TG_ERR_INVALID_ARGUMENT, "bad sizes or NULL pointer");
    if (n_points > INT_MAX)
        return fail(TG_ERR_UNSUPPORTED, "%lld points: ids must fit int32 (at most 2^31-1 points)",
                    (long long)n_points);
    for (int64_t i = 0; i < 4 * n_cells; i++) {
        const int64_t x = cells[i];
        if (x < 0 || x >= n_points)
            return fail(TG_ERR_INVALID_MESH, "cell %lld has vertex id %lld, outside [0, %lld)",
                        (long long)(i / 4), (long long)x, (long long)n_points);
        out[i] = (int32_t)x;
    }
    return TG_OK;
}

tg_status tg_mesh_create_i64(const int64_t *tv, int64_t n_cells, int64_t n_verts, void *stream,
                             tg_mesh **out)
{
    if (!out) return fail(TG_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (n_cells < 0 || n_cells > kMaxCells)
        return fail(n_cells < 0 ? TG_ERR_INVALID_ARGUMENT : TG_ERR_UNSUPPORTED,
                    "bad cell count %lld", (long long)n_cells);
    std::vector<int32_t> tv32((size_t)(4 * n_cells));
    TRY(tg_tv_narrow_i64(tv, n_cells, n_verts, tv32.data()));
    return tg_mesh_create(tv32.data(), n_cells, n_verts, 0, stream, out);
}

tg_status tg_extract(tg_mesh *m, uint32_t mask, uint32_t options, void *stream)
{
    if (!m) return fail(TG_ERR_INVALID_ARGUMENT, "mesh is NULL");
    mask &= TG_ALL_RELATIONS;
    bool all_ready = true;
    for (int r = 1; r < 14; r++)
        if ((mask & bit(r)) && !(m->rel[r].ready && (r != TG_REL_TT || m->rel[r].opts ==
                                                     (options & TG_OPT_TT_VERTEX_SHARING))))
            all_ready = false;
    if (all_ready) return TG_OK;
    int cur = 0;
    cudaGetDevice(&cur);
    if (cur != m->device) CK(cudaSetDevice(m->device));
    m->last_stream = (cudaStream_t)stream;
    tg_status st = run_extract(m, mask, options, (cudaStream_t)stream);
    if (cur != m->device) cudaSetDevice(cur);
    return st;
}

tg_status tg_mesh_counts(const tg_mesh *m, int64_t *nv, int64_t *ne, int64_t *nf, int64_t *nc)
{
    if (!m) return fail(TG_ERR_INVALID_ARGUMENT, "mesh is NULL");
    if (nv) *nv = m->V;
    if (ne) *ne = m->E;
    if (nf) *nf = m->F;
    if (nc) *nc = m->T;
    return TG_OK;
}

tg_status tg_get_relation(const tg_mesh *m, int r, const int64_t **off, const int32_t **ent,
                          int64_t *rows, int64_t *entries, int32_t *width)
{
    if (!m || r < 1 || r > 13) return fail(TG_ERR_INVALID_ARGUMENT, "bad mesh or relation index");
    const Rel &x = m->rel[r];
    if (!x.ready) return fail(TG_ERR_NOT_COMPUTED, "relation %s has not been extracted", kName[r]);
    if (off) *off = x.off;
    if (ent) *ent = x.ent;
    if (rows) *rows = x.rows;
    if (entries) *entries = x.entries;
    if (width) *width = x.width;
    return TG_OK;
}

tg_status tg_copy_relation(const tg_mesh *m, int r, int64_t *off_host, int32_t *ent_host,
                           void *stream)
{
    if (!m || r < 1 || r > 13) return fail(TG_ERR_INVALID_ARGUMENT, "bad mesh or relation index");
    const Rel &x = m->rel[r];
    if (!x.ready) return fail(TG_ERR_NOT_COMPUTED, "relation %s has not been extracted", kName[r]);
    cudaStream_t s = (cudaStream_t)stream;
    if (off_host && x.off)
        CK(cudaMemcpyAsync(off_host, x.off, (size_t)(x.rows + 1) * 8, cudaMemcpyDeviceToHost, s));
    if (ent_host && x.entries)
        CK(cudaMemcpyAsync(ent_host, x.ent, (size_t)x.entries * 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return TG_OK;
}

tg_status tg_copy_relation_async(tg_mesh *m, int r, int64_t *off_host, int32_t *ent_host,
                                 void *stream)
{
    if (!m || r < 1 || r > 13) return fail(TG_ERR_INVALID_ARGUMENT, "bad mesh or relation index");
    const Rel &x = m->rel[r];
    if (!x.ready) return fail(TG_ERR_NOT_COMPUTED, "relation %s has not been extracted", kName[r]);
    cudaStream_t s = (cudaStream_t)stream;
    m->last_stream = s;
    if (off_host && x.off)
        CK(cudaMemcpyAsync(off_host, x.off, (size_t)(x.rows + 1) * 8, cudaMemcpyDeviceToHost, s));
    if (ent_host && x.entries)
        CK(cudaMemcpyAsync(ent_host, x.ent, (size_t)x.entries * 4, cudaMemcpyDeviceToHost, s));
    return TG_OK;
}

tg_status tg_copy_relation_async_i32(tg_mesh *m, int r, int32_t *off_host, int32_t *ent_host,
                                     void *stream)
{
    if (!m || r < 1 || r > 13) return fail(TG_ERR_INVALID_ARGUMENT, "bad mesh or relation index");
    const Rel &x = m->rel[r];
    if (!x.ready) return fail(TG_ERR_NOT_COMPUTED, "relation %s has not been extracted", kName[r]);
    cudaStream_t s = (cudaStream_t)stream;
    m->last_stream = s;
    if (off_host && x.off) {
        if (x.entries > INT32_MAX)
            return fail(TG_ERR_UNSUPPORTED, "relation %s has %lld entries: its offsets need int64",
                        kName[r], (long long)x.entries);
        int32_t *d = nullptr;
        const size_t b = (size_t)(x.rows + 1) * 4;
        CK(cudaMallocAsync(&d, b, s));
        launch_narrow(x.off, d, x.rows + 1, s);
        const cudaError_t e = cudaMemcpyAsync(off_host, d, b, cudaMemcpyDeviceToHost, s);
        cudaFreeAsync(d, s);   // stream-ordered: after the copy
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync (offsets)", __LINE__);
    }
    if (ent_host && x.entries)
        CK(cudaMemcpyAsync(ent_host, x.ent, (size_t)x.entries * 4, cudaMemcpyDeviceToHost, s));
    return TG_OK;
}

tg_status tg_copy_relations_async_i32(tg_mesh *m, uint32_t mask, int32_t *const *off_host,
                                      int32_t *const *ent_host, void *stream)
{
    if (!m || !off_host || !ent_host) return fail(TG_ERR_INVALID_ARGUMENT, "NULL argument");
    mask &= TG_ALL_RELATIONS;
    cudaStream_t s = (cudaStream_t)stream;
    m->last_stream = s;
    NarrowJobs j{};
    int64_t at[14] = {};
    for (int r = 1; r < 14; r++) {
        if (!(mask & bit(r))) continue;
        const Rel &x = m->rel[r];
        if (!x.ready)
            return fail(TG_ERR_NOT_COMPUTED, "relation %s has not been extracted", kName[r]);
        if (!off_host[r] || !x.off) continue;
        if (x.entries > INT32_MAX)
            return fail(TG_ERR_UNSUPPORTED, "relation %s has %lld entries: its offsets need int64",
                        kName[r], (long long)x.entries);
        at[r] = j.start[j.n];
        j.src[j.n] = x.off;
        j.start[j.n + 1] = j.start[j.n] + x.rows + 1;
        j.n++;
    }
    int32_t *d = nullptr;
    if (j.n > 0) {
        CK(cudaMallocAsync(&d, (size_t)j.start[j.n] * 4, s));
        j.dst = d;
        launch_narrow_multi(j, s);
    }
    cudaError_t e = cudaSuccess;
    for (int r = 1; r < 14 && e == cudaSuccess; r++) {
        if (!(mask & bit(r))) continue;
        const Rel &x = m->rel[r];
        if (off_host[r] && x.off)
            e = cudaMemcpyAsync(off_host[r], d + at[r], (size_t)(x.rows + 1) * 4,
                                cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && ent_host[r] && x.entries)
            e = cudaMemcpyAsync(ent_host[r], x.ent, (size_t)x.entries * 4, cudaMemcpyDeviceToHost,
                                s);
    }
    if (d) cudaFreeAsync(d, s);   // stream-ordered: after the copies
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync (relations)", __LINE__);
    return TG_OK;
}

tg_status tg_copy_relation_i32(tg_mesh *m, int r, int32_t *off_host, int32_t *ent_host,
                               void *stream)
{
    TRY(tg_copy_relation_async_i32(m, r, off_host, ent_host, stream));
    CK(cudaStreamSynchronize((cudaStream_t)stream));
    return TG_OK;
}

tg_status tg_export_relation_i64(const tg_mesh *m, int r, int64_t *entries_out,
                                 int64_t *offsets_out, int out_on_device, void *stream)
{
    if (!m || r < 1 || r > 13) return fail(TG_ERR_INVALID_ARGUMENT, "bad mesh or relation index");
    const Rel &x = m->rel[r];
    if (!x.ready) return fail(TG_ERR_NOT_COMPUTED, "relation %s has not been extracted", kName[r]);
    cudaStream_t s = (cudaStream_t)stream;
    if (entries_out && x.entries) {
        int64_t *dst = entries_out;
        Temps tmp(s);
        if (!out_on_device) TRY(tmp.alloc(&dst, x.entries));
        launch_widen(x.ent, dst, x.entries, s);
        if (!out_on_device)
            CK(cudaMemcpyAsync(entries_out, dst, (size_t)x.entries * 8, cudaMemcpyDeviceToHost, s));
        CK(cudaGetLastError());
    }
    if (offsets_out && x.off)
        CK(cudaMemcpyAsync(offsets_out, x.off, (size_t)(x.rows + 1) * 8,
                           out_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
    if (!out_on_device) CK(cudaStreamSynchronize(s));
    return TG_OK;
}

tg_status tg_export_rows_padded(const tg_mesh *m, int r, int32_t width, int64_t *padded_out,
                                uint32_t *counts_out, void *stream)
{
    if (!m || r < 1 || r > 13 || width < 0 || !padded_out)
        return fail(TG_ERR_INVALID_ARGUMENT, "bad mesh, relation index, width or output");
    const Rel &x = m->rel[r];
    if (!x.ready) return fail(TG_ERR_NOT_COMPUTED, "relation %s has not been extracted", kName[r]);
    if (!x.off) return fail(TG_ERR_INVALID_ARGUMENT, "relation %s is fixed width", kName[r]);
    cudaStream_t s = (cudaStream_t)stream;
    launch_pad_rows(x.off, x.ent, x.rows, width, padded_out, counts_out, s);
    CK(cudaGetLastError());
    return TG_OK;
}

tg_status tg_get_tv(const tg_mesh *m, const int32_t **tv)
{
    if (!m || !tv) return fail(TG_ERR_INVALID_ARGUMENT, "NULL argument");
    *tv = reinterpret_cast<const int32_t *>(m->tvs);
    return TG_OK;
}

tg_status tg_critical_points(tg_mesh *m, const void *field, int field_type, int field_on_device,
                             uint32_t *classes_out, int out_on_device, void *stream)
{
    if (!m) return fail(TG_ERR_INVALID_ARGUMENT, "NULL argument");
    return critical_points_rows(m, 0, m->V, field, field_type, field_on_device, classes_out,
                                out_on_device, (cudaStream_t)stream);
}

tg_status tg_profile_kernel(const char *name)
{
    std::lock_guard<std::mutex> lk(tg::g_prof_mu);
    tg::g_prof_name = name ? name : "";
    tg::g_prof_on.store(!tg::g_prof_name.empty());
    return TG_OK;
}

tg_status tg_profile_read(double *total_ms, int64_t *launches, int reset)
{
    std::lock_guard<std::mutex> lk(tg::g_prof_mu);
    double ms = 0.0;
    for (auto &p : tg::g_prof_events) {
        CK(cudaEventSynchronize(p.b));
        float x = 0.f;
        CK(cudaEventElapsedTime(&x, p.a, p.b));
        ms += x;
    }
    if (total_ms) *total_ms = ms;
    if (launches) *launches = (int64_t)tg::g_prof_events.size();
    if (reset) {
        for (auto &p : tg::g_prof_events) {
            tg::g_prof_pool.push_back(p.a);
            tg::g_prof_pool.push_back(p.b);
        }
        tg::g_prof_events.clear();
    }
    return TG_OK;
}

int64_t tg_mesh_device_bytes(const tg_mesh *m)
{
    if (!m) return 0;
    int64_t b = m->T * 16;
    for (int r = 1; r < 14; r++) {
        const Rel &x = m->rel[r];
        if (!x.ready) continue;
        b += x.entries * 4;
        if (x.off) b += (x.rows + 1) * 8;
    }
    if (m->cadj) b += m->rel[TG_REL_VV].entries * 8;
    return b;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// internal: segments (tg_batch.cu)
tg_status tg::mesh_set_segments(tg_mesh *m, const int64_t *seg_c_host, int64_t n, cudaStream_t s)
{
    if (m->seg_c) cudaFreeAsync(m->seg_c, s);
    if (m->seg_ef) cudaFreeAsync(m->seg_ef, s);
    m->seg_c = m->seg_ef = nullptr;
    m->n_seg = n;
    TRY(dalloc(&m->seg_c, n + 1, s));
    TRY(dalloc(&m->seg_ef, 2 * (n + 1), s));
    CK(cudaMemcpyAsync(m->seg_c, seg_c_host, (size_t)(n + 1) * 8, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));  // the host array may go away
    return TG_OK;
}

const int64_t *tg::mesh_segment_ids(const tg_mesh *m) { return m->seg_ef; }
