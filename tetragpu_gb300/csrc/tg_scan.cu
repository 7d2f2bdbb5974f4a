// tg_scan.cu -- batched exclusive scans in one pass (decoupled look-back).
//
// Every CSR offset array and every bit-rank prefix of the pipeline comes out
// of here.  Up to kMaxScanJobs independent arrays are scanned by one launch
// (blockIdx.y selects the array), reading each input once.  A block takes the
// next tile of its array in start order (a ticket), sums the tile, publishes
// the sum, and adds the published sums of the tiles before it until it meets
// one whose inclusive prefix is already known (Merrill and Garland's
// single-pass scan).  A block waits only on tiles whose blocks started before
// it, so every wait ends; it is bounded all the same: after kLookbackPolls
// polls the block records ST_SCAN_STALLED in the mesh status (reported at the
// next status read-back) and goes on.
#include "tg_internal.h"

namespace tg {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;  // 2048 elements per tile

struct ScanParams {
    ScanJob job[kMaxScanJobs];
    // per array: one word per tile (sum << 2 | 1 once the tile's sum is
    // published, inclusive prefix << 2 | 2 once that is known, 0 before),
    // then the ticket counter; zeroed before the launch
    unsigned long long *tiles[kMaxScanJobs];
    unsigned long long *next;   // the other buffer, zeroed here for the next scan
    int64_t next_words;
    unsigned *err;
    int n_jobs;
};

__device__ __forceinline__ int64_t load_value(const ScanJob &j, int64_t i)
{
    if (j.kind == SCAN_COUNT_I32) return (int64_t)__ldg((const int32_t *)j.in + i);
    if (j.kind == SCAN_SQUARE_I32) {
        const int64_t x = __ldg((const int32_t *)j.in + i);
        return x * x;
    }
    return (int64_t)__popc(__ldg((const uint32_t *)j.in + i));
}

__device__ __forceinline__ void store_value(const ScanJob &j, int64_t i, int64_t v)
{
    if (j.kind != SCAN_POPC_RANK) ((int64_t *)j.out)[i] = v;
    else ((uint2 *)j.out)[i] = make_uint2(i < j.n ? __ldg((const uint32_t *)j.in + i) : 0u,
                                          (unsigned)v);
}

// Block-wide exclusive scan of one int64 per thread; returns the block total.
template <int NT>
__device__ __forceinline__ int64_t block_exclusive_scan(int64_t x, int64_t &excl, int64_t *sm)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) sm[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int64_t w = (lane < NT / 32) ? sm[lane] : 0;
        int64_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        if (lane < NT / 32) sm[lane] = wi - w;  // exclusive warp offsets
        if (lane == NT / 32 - 1) sm[NT / 32] = wi;
    }
    __syncthreads();
    excl = sm[warp] + incl - x;
    int64_t total = sm[NT / 32];
    __syncthreads();
    return total;
}

__global__ void __launch_bounds__(kThreads) k_scan(ScanParams p)
{
    griddep_wait();
    const int jb = blockIdx.y;
    if (jb >= p.n_jobs) return;
    const ScanJob &j = p.job[jb];
    const int64_t ntiles = (j.n + kTile - 1) / kTile;
    unsigned long long *w = p.tiles[jb];
    {
        const int64_t nthreads = (int64_t)gridDim.x * gridDim.y * blockDim.x;
        const int64_t t0 = ((int64_t)blockIdx.y * gridDim.x + blockIdx.x) * blockDim.x + threadIdx.x;
        for (int64_t i = t0; i < p.next_words; i += nthreads) p.next[i] = 0ull;
    }
    __shared__ int64_t sm[kThreads / 32 + 1];
    __shared__ int64_t s_tile, s_prefix;
    if (threadIdx.x == 0) s_tile = (int64_t)atomicAdd(w + ntiles, 1ull);   // the ticket
    __syncthreads();
    const int64_t tile = s_tile;
    if (ntiles == 0) {   // an empty array: its total alone
        if (tile == 0 && threadIdx.x == 0) store_value(j, 0, 0);
        return;
    }
    if (tile >= ntiles) return;   // a surplus block of a shorter array
    const int64_t base = tile * kTile + (int64_t)threadIdx.x * kItems;
    int64_t v[kItems];
    int64_t s = 0;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        v[k] = (base + k < j.n) ? load_value(j, base + k) : 0;
        s += v[k];
    }
    int64_t excl;
    const int64_t total = block_exclusive_scan<kThreads>(s, excl, sm);
    if (threadIdx.x < 32) {   // warp 0
        const int64_t pre = look_back(w, tile, total, p.err);
        if (threadIdx.x == 0) s_prefix = pre;
    }
    __syncthreads();
    int64_t run = s_prefix + excl;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        if (base + k < j.n) store_value(j, base + k, run);
        run += v[k];
    }
    if (tile == ntiles - 1 && threadIdx.x == 0) store_value(j, j.n, s_prefix + total);
}

}  // namespace

int64_t scan_job_words(int64_t max_n)
{
    return (max_n + kTile - 1) / kTile + 1;
}

void scan_batch(const ScanJob *jobs, int n_jobs, ScanWorkspace &ws, DevStatus *st, cudaStream_t s)
{
    if (n_jobs <= 0) return;
    ScanParams p{};
    p.n_jobs = n_jobs;
    p.err = &st->flags;
    int64_t max_tiles = 1;
    unsigned long long *cur;
    scan_ws_begin(ws, s, &cur, &p.next, &p.next_words);
    for (int i = 0; i < n_jobs; i++) {
        p.job[i] = jobs[i];
        p.tiles[i] = cur + (int64_t)i * ws.job_words;
        const int64_t t = (jobs[i].n + kTile - 1) / kTile;
        if (t > max_tiles) max_tiles = t;
    }
    dim3 grid((unsigned)max_tiles, n_jobs);
    {
        Launch L("k_scan", s);
        launch_pdl(k_scan, grid, kThreads, 0, s, p);
    }
    scan_ws_end(ws, s);
}

void scan_ws_begin(ScanWorkspace &ws, cudaStream_t s, unsigned long long **cur,
                   unsigned long long **next, int64_t *next_words)
{
    const int64_t words = (int64_t)kMaxScanJobs * ws.job_words;
    *cur = ws.buf + (int64_t)ws.cur * words;
    *next = ws.buf + (int64_t)(ws.cur ^ 1) * words;
    *next_words = words;
    if (ws.used && ws.last != s) cudaStreamWaitEvent(s, ws.done, 0);
}

void scan_ws_end(ScanWorkspace &ws, cudaStream_t s)
{
    cudaEventRecord(ws.done, s);
    ws.last = s;
    ws.used = true;
    ws.cur ^= 1;
}

}  // namespace tg
