// tg_noalloc.cu -- critical-point classification that allocates no memory.
//
// tg_critical_points builds the link adjacency of every vertex (one 64-bit
// mask per VV entry) in memory it allocates and caches on the mesh.  Some
// callers cannot allocate device memory when they classify: a host
// application that hands this library a fixed device-memory budget at
// start-up and accounts for every byte afterwards, or a real-time loop whose
// rules forbid allocator calls (and the synchronisation they can cause) once
// it runs.  tg_critical_points_noalloc serves them: the caller passes VV
// (device CSR), the field and the output, and the adjacency lives in
// file-scope device arrays of fixed size, TG_NOALLOC_MAX_VV_ENTRIES masks
// (64 MiB) plus their window table (128 KiB), which every GPU that loads
// this library holds until the process exits.  The call reads the kernels'
// status word back and waits for its stream to do so.
#include <climits>
#include <cstdio>
#include <mutex>

#include "tetragpu.h"
#include "tg_internal.h"

namespace {

// Scratch shared by every call on a device: the adjacency masks and a status
// word for the kernels.  Calls that overlap on the GPU (two streams at once)
// race on it; serialise them.
static __device__ __align__(256) unsigned long long g_noalloc_adj[TG_NOALLOC_MAX_VV_ENTRIES];
// (the window table of the adjacency kernel: kAdjWin-entry windows over VV)
static __device__ __align__(256) int g_noalloc_win[TG_NOALLOC_MAX_VV_ENTRIES / tg::kAdjWin + 2];
static __device__ __align__(256) tg::DevStatus g_noalloc_status;

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_adj_ptr[kMaxDevices];
void *g_win_ptr[kMaxDevices];
void *g_status_ptr[kMaxDevices];

tg_status fail(tg_status code, const char *msg, cudaError_t e = cudaSuccess)
{
    char buf[256];
    if (e != cudaSuccess)
        snprintf(buf, sizeof buf, "%s: %s", msg, cudaGetErrorString(e));
    else
        snprintf(buf, sizeof buf, "%s", msg);
    tg::set_last_error(buf);
    return code;
}

// Device addresses of the scratch arrays for the current device, looked up
// once per device (the array names are host-side stand-ins, not addresses).
tg_status scratch_for_current_device(void **adj, void **win, void **status)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(TG_ERR_CUDA, "cudaGetDevice", e);
    if (dev < 0 || dev >= kMaxDevices) return fail(TG_ERR_UNSUPPORTED, "device ordinal too large");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_adj_ptr[dev]) {
        void *a = nullptr, *w = nullptr, *s = nullptr;
        e = cudaGetSymbolAddress(&a, g_noalloc_adj);
        if (e != cudaSuccess) return fail(TG_ERR_CUDA, "cudaGetSymbolAddress(adjacency scratch)", e);
        e = cudaGetSymbolAddress(&w, g_noalloc_win);
        if (e != cudaSuccess) return fail(TG_ERR_CUDA, "cudaGetSymbolAddress(window scratch)", e);
        e = cudaGetSymbolAddress(&s, g_noalloc_status);
        if (e != cudaSuccess) return fail(TG_ERR_CUDA, "cudaGetSymbolAddress(status scratch)", e);
        g_adj_ptr[dev] = a;
        g_win_ptr[dev] = w;
        g_status_ptr[dev] = s;
    }
    *adj = g_adj_ptr[dev];
    *win = g_win_ptr[dev];
    *status = g_status_ptr[dev];
    return TG_OK;
}

}  // namespace

extern "C" tg_status tg_critical_points_noalloc(const int64_t *vv_off, const int32_t *vv,
                                                int64_t n_verts, int64_t n_vv_entries,
                                                const void *field, int field_type,
                                                uint32_t *classes_out, void *stream)
{
    if (!vv_off || (n_vv_entries > 0 && !vv) || !field || !classes_out || n_verts < 0 ||
        n_vv_entries < 0)
        return fail(TG_ERR_INVALID_ARGUMENT, "NULL pointer or negative size");
    if (field_type != TG_FIELD_F32 && field_type != TG_FIELD_F64)
        return fail(TG_ERR_INVALID_ARGUMENT, "field_type must be TG_FIELD_F32 or TG_FIELD_F64");
    if (n_vv_entries > TG_NOALLOC_MAX_VV_ENTRIES) {
        char buf[200];
        snprintf(buf, sizeof buf,
                 "VV has %lld entries; the no-allocation scratch holds at most %d "
                 "(use tg_critical_points)",
                 (long long)n_vv_entries, TG_NOALLOC_MAX_VV_ENTRIES);
        return fail(TG_ERR_UNSUPPORTED, buf);
    }
    if (n_verts > INT_MAX) return fail(TG_ERR_UNSUPPORTED, "more than 2^31-1 vertices");
    void *adj = nullptr, *win = nullptr, *status = nullptr;
    tg_status st = scratch_for_current_device(&adj, &win, &status);
    if (st != TG_OK) return st;
    static_assert(tg::kAdjWin >= 1, "window size");
    cudaStream_t s = (cudaStream_t)stream;
    // an error left by an earlier, unrelated call would be reported as this
    // call's: clear it (sticky errors come back from the calls below)
    (void)cudaGetLastError();
    // the status word keeps the previous call's contents: clear it; the
    // window table and every adjacency mask are rewritten before they are read
    cudaError_t e = cudaMemsetAsync(status, 0, sizeof(tg::DevStatus), s);
    if (e != cudaSuccess) return fail(TG_ERR_CUDA, "clearing the status word", e);
    tg::launch_window_starts(vv_off, n_verts, n_vv_entries, tg::crit_window(), (int32_t *)win, s);
    tg::launch_crit_adj(vv_off, vv, nullptr, nullptr, nullptr, (const int32_t *)win, n_verts,
                        n_vv_entries, (uint64_t *)adj, (tg::DevStatus *)status, 2, s);
    tg::launch_crit_classify(vv_off, vv, (const uint64_t *)adj, field, field_type, 0, n_verts,
                             classes_out, s);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TG_ERR_CUDA, "launching the critical-point kernels", e);
    tg::DevStatus out{};
    e = cudaMemcpyAsync(&out, status, sizeof out, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return fail(TG_ERR_CUDA, "critical-point kernels", e);
    }
    // a row longer than the 64-bit link masks hold: its masks were not
    // written, so the classes of that call are not valid
    if (out.flags & tg::ST_HEAVY_DEG)
        return fail(TG_ERR_UNSUPPORTED,
                    "a vertex has more than 64 neighbours (tg_critical_points handles it)");
    return TG_OK;
}
