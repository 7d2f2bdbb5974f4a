// tg_scan.cu -- batched exclusive scans (reduce, scan partials, downsweep).
//
// Every CSR offset array and every bit-rank prefix of the pipeline comes out
// of here.  Up to kMaxScanJobs independent arrays are scanned by the same
// three launches (blockIdx.y selects the array), so a stage that produces
// five count arrays pays three launches, not fifteen.  No spin-waits: the
// partial sums go through global memory between launches.
#include "tg_internal.h"

namespace tg {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;  // 2048 elements per tile

struct ScanParams {
    ScanJob job[kMaxScanJobs];
    int64_t *partials[kMaxScanJobs];
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

__global__ void __launch_bounds__(kThreads) k_scan_reduce(ScanParams p)
{
    const int jb = blockIdx.y;
    if (jb >= p.n_jobs) return;
    const ScanJob &j = p.job[jb];
    const int64_t ntiles = (j.n + kTile - 1) / kTile;
    const int64_t tile = blockIdx.x;
    if (tile >= ntiles) return;
    const int64_t base = tile * kTile + (int64_t)threadIdx.x * kItems;
    int64_t s = 0;
#pragma unroll
    for (int k = 0; k < kItems; k++)
        if (base + k < j.n) s += load_value(j, base + k);
    __shared__ int64_t sm[kThreads / 32 + 1];
    int64_t excl;
    int64_t total = block_exclusive_scan<kThreads>(s, excl, sm);
    if (threadIdx.x == 0) p.partials[jb][tile] = total;
}

__global__ void __launch_bounds__(1024) k_scan_partials(ScanParams p)
{
    const int jb = blockIdx.x;
    if (jb >= p.n_jobs) return;
    const ScanJob &j = p.job[jb];
    const int64_t ntiles = (j.n + kTile - 1) / kTile;
    int64_t *part = p.partials[jb];
    __shared__ int64_t sm[1024 / 32 + 1];
    // chunks of 8192 tiles: a thread loads eight consecutive partials at
    // once, one block-wide scan of the thread sums per chunk
    constexpr int kPer = 8;
    int64_t carry = 0;
    for (int64_t b = 0; b < ntiles; b += 1024 * kPer) {
        const int64_t i0 = b + (int64_t)threadIdx.x * kPer;
        int64_t v[kPer], x = 0;
#pragma unroll
        for (int k = 0; k < kPer; k++) {
            v[k] = i0 + k < ntiles ? part[i0 + k] : 0;
            x += v[k];
        }
        int64_t run;
        const int64_t tot = block_exclusive_scan<1024>(x, run, sm);
        run += carry;
#pragma unroll
        for (int k = 0; k < kPer; k++) {
            if (i0 + k < ntiles) part[i0 + k] = run;
            run += v[k];
        }
        carry += tot;
    }
    const int64_t total = carry;
    if (threadIdx.x == 0) store_value(j, j.n, total);
}

__global__ void __launch_bounds__(kThreads) k_scan_down(ScanParams p)
{
    const int jb = blockIdx.y;
    if (jb >= p.n_jobs) return;
    const ScanJob &j = p.job[jb];
    const int64_t ntiles = (j.n + kTile - 1) / kTile;
    const int64_t tile = blockIdx.x;
    if (tile >= ntiles) return;
    const int64_t base = tile * kTile + (int64_t)threadIdx.x * kItems;
    int64_t v[kItems];
    int64_t s = 0;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        v[k] = (base + k < j.n) ? load_value(j, base + k) : 0;
        s += v[k];
    }
    __shared__ int64_t sm[kThreads / 32 + 1];
    int64_t excl;
    block_exclusive_scan<kThreads>(s, excl, sm);
    int64_t run = p.partials[jb][tile] + excl;
#pragma unroll
    for (int k = 0; k < kItems; k++) {
        if (base + k < j.n) store_value(j, base + k, run);
        run += v[k];
    }
}

}  // namespace

size_t scan_scratch_bytes(int64_t n)
{
    int64_t ntiles = (n + kTile - 1) / kTile;
    return (size_t)(ntiles + 1) * sizeof(int64_t);
}

void scan_batch(const ScanJob *jobs, int n_jobs, void *scratch, cudaStream_t s)
{
    if (n_jobs <= 0) return;
    ScanParams p{};
    p.n_jobs = n_jobs;
    int64_t max_tiles = 0;
    size_t stride = 0;
    for (int i = 0; i < n_jobs; i++) {
        size_t b = scan_scratch_bytes(jobs[i].n);
        if (b > stride) stride = b;
    }
    stride = (stride + 255) & ~size_t(255);
    for (int i = 0; i < n_jobs; i++) {
        p.job[i] = jobs[i];
        p.partials[i] = (int64_t *)((char *)scratch + stride * i);
        int64_t t = (jobs[i].n + kTile - 1) / kTile;
        if (t > max_tiles) max_tiles = t;
    }
    if (max_tiles > 0) {
        dim3 grid((unsigned)max_tiles, n_jobs);
        Launch L("k_scan_reduce", s);
        k_scan_reduce<<<grid, kThreads, 0, s>>>(p);
    }
    {
        Launch L("k_scan_partials", s);
        k_scan_partials<<<n_jobs, 1024, 0, s>>>(p);
    }
    if (max_tiles > 0) {
        dim3 grid((unsigned)max_tiles, n_jobs);
        Launch L("k_scan_down", s);
        k_scan_down<<<grid, kThreads, 0, s>>>(p);
    }
}

}  // namespace tg
