// tg_crit.cu -- critical-point classification of a vertex scalar field.
//
// Semantics of the reference critPoints kernel (tlranda/TetraGPU,
// src/alg/critPoints.cu:49-331), restated on an exact VV:
//   * neighbour u of v is lower when f[u] < f[v], or f[u] == f[v] and u < v
//     (:136-140);
//   * two neighbours of the same kind are joined when the mesh has the edge
//     between them, i.e. w is in VV[u] (:172-202), not only edges in v's star;
//   * the lower-link and upper-link component counts go to classes[3v] and
//     classes[3v+1] (:275-284) and the code to classes[3v+2]: (>=1, 0) -> 2,
//     (0, >=1) -> 1, (1, 1) -> 3, anything else -> 4 (:303-330).
//
// Two kernels, so that a second field on the same mesh reuses the first:
//   k_crit_adj       field-independent: for every VV entry (v, u), the bitmask
//                    of v's neighbours adjacent to u.  Thread per edge (both
//                    of its entries), v's row staged in shared memory.
//   k_crit_classify  field-dependent: lower/upper split, then the components
//                    of each kind counted by a bitmask search over the
//                    adjacency masks of same-kind neighbours.
#include "tg_internal.h"

namespace tg {
namespace {

// Link adjacency: for every VV entry (v, u), bit j of the mask is set when
// v's j-th neighbour is also a neighbour of u.  The common neighbours of v
// and u give both entries (v, u) and (u, v), so one thread takes each edge
// once, from its lower end v: it scans u's row from global memory, finds each
// w in v's row (staged in shared memory) by binary search, and sets bit j in
// (v, u)'s mask and bit i (w's place in u's row) in (u, v)'s, which sits at
// v's place in u's row.  A block takes the vertices whose VV rows start in a
// 256-entry window (win); the entries it owns (u > v) form a work list.
constexpr int kAdjCap = kAdjWin + kMaxDeg;
constexpr int kAdjThreads = TG_ADJ_THREADS;

// u's row (urow, un entries; read four at a time from 16-byte boundaries
// when the array is aligned: i from i0 = -(ub mod 4), one load instruction
// per four entries; else one entry at a time) against v's row (row, d
// entries, shared memory, padded with INT_MAX to top = the power of two at or
// above d): each w found at position lo of v's row sets bit lo of bits_v and
// bit i of bits_u; pv = v's place in u's row.  The search takes the steps
// top / 2, .. 1 (those above top / 2 skipped by a per-thread predicate, so
// the lanes of a warp stay together) and needs no bound: every probe lies in
// the padded row.
template <typename M, int TOP>
__device__ __forceinline__ void adj_scan(const int *row, int d, int top,
                                         const int *__restrict__ urow, int i0, int un, int lim,
                                         bool vec, int v, M &bits_v, M &bits_u, int &pv)
{
    // the next four entries are loaded while the current four are searched
    auto load4 = [&](int j) -> int4 {
        if (vec && j + 4 <= lim) return __ldg(reinterpret_cast<const int4 *>(urow + j));
        int4 x;
        x.x = j < lim && j < un ? __ldg(urow + j) : 0;
        x.y = j + 1 < lim && j + 1 < un ? __ldg(urow + j + 1) : 0;
        x.z = j + 2 < lim && j + 2 < un ? __ldg(urow + j + 2) : 0;
        x.w = j + 3 < lim && j + 3 < un ? __ldg(urow + j + 3) : 0;
        return x;
    };
    int4 nxt = i0 < un ? load4(i0) : make_int4(0, 0, 0, 0);
    for (; i0 < un; i0 += 4) {
        const int4 cur = nxt;
        if (i0 + 4 < un) nxt = load4(i0 + 4);
        const int q[4] = {cur.x, cur.y, cur.z, cur.w};
        // four searches in lock step (independent shared-memory loads in
        // flight together); entries outside [0, un) search harmlessly and
        // set nothing
        int lo[4] = {0, 0, 0, 0};
#pragma unroll
        for (int step = TOP / 2; step > 0; step >>= 1) {
            if (2 * step > top) continue;
#pragma unroll
            for (int t = 0; t < 4; t++)
                lo[t] += row[lo[t] + step - 1] < q[t] ? step : 0;
        }
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const int i = i0 + t;
            const bool valid = i >= 0 && i < un;
            if (valid && q[t] == v) pv = i;
            const bool hit = valid && q[t] != v && row[lo[t]] == q[t];
            bits_v |= (M)hit << lo[t];
            bits_u |= (M)hit << (i & (8 * (int)sizeof(M) - 1));
        }
    }
}

// Rows longer than kMaxDeg (vertices whose classes tg_heavy.cu computes) are
// not staged and get no masks; with heavy = 1 an entry (v, u) of a light v
// whose neighbour u is such a vertex is computed from v's side whichever end
// is lower (u computes nothing); heavy = 2 reports them instead
// (ST_HEAVY_DEG) for callers without the heavy path.  Light rows start
// below kAdjWin in their window and end below kAdjCap, so they always fit.
//
// Windows run over the rows in `order` (the star processing order: vertices
// by first cell, so consecutive windows share neighbours and the neighbours'
// rows stay in L2; ooff = the row lengths' prefix in that order, ostart =
// each row's start in VV, read beside ooff instead of after the vertex), or
// in id order when order is null (ooff = vv_off).  A staged row keeps its
// global start in gst[row start].
__global__ void __launch_bounds__(kAdjThreads)
k_crit_adj(const int64_t *__restrict__ vv_off, const int *__restrict__ vv, int64_t n_vv,
           const int *__restrict__ order, const int64_t *__restrict__ ooff,
           const int64_t *__restrict__ ostart, const int *__restrict__ win,
           unsigned long long *__restrict__ adj, DevStatus *st, int heavy)
{
    griddep_wait();
    __shared__ int nb[kAdjCap];
    __shared__ int prow[2 * kAdjCap];   // the row starting at rs at 2 rs, INT_MAX to 2 rs + 2 d
    __shared__ int meta[kAdjCap];   // row start | row length << 16; -1: no light row there
    __shared__ int vid[kAdjCap];
    __shared__ int own[kAdjCap];
    __shared__ long long gst[kAdjCap];   // at a row start: the row's first entry in VV
    __shared__ int n_own;
    // every thread reads the window's bounds itself (the same words: one
    // transaction each), so the block needs no barrier before the rows
    // unless the heavy modes mark the slots of rows they leave out
    const int s_vlo = win[blockIdx.x], s_vhi = win[blockIdx.x + 1];
    const long long s_base = ooff[s_vlo];
    const int s_n = (int)(ooff[s_vhi] - s_base);
    if (threadIdx.x == 0) n_own = 0;
    if (heavy) {
        for (int e = threadIdx.x; e < kAdjCap; e += blockDim.x) meta[e] = -1;
        __syncthreads();
    }
    const int n = min(s_n, kAdjCap);
    const long long base = s_base;
    if (heavy == 2 && s_n > kAdjCap) {  // a row longer than kMaxDeg lies in this window
        if (threadIdx.x == 0) {
            atomicOr(&st->flags, ST_HEAVY_DEG);
            atomicMin(&st->bad_vertex, order ? order[s_vlo] : s_vlo);
        }
        return;
    }
    for (int i = s_vlo + threadIdx.x; i < s_vhi; i += blockDim.x) {
        const int rs = (int)(ooff[i] - base);
        const int d = (int)(ooff[i + 1] - ooff[i]);
        if (d == 0) continue;
        const int v = order ? order[i] : i;
        if (d > kMaxDeg) {
            if (heavy == 2) {
                atomicOr(&st->flags, ST_HEAVY_DEG);
                atomicMin(&st->bad_vertex, v);
            }
            continue;
        }
        const long long g0 = order ? ostart[i] : base + rs;
        gst[rs] = g0;
        // the row's entries are copied asynchronously as soon as its start
        // is known
        for (int k = 0; k < d; k++) {
            meta[rs + k] = rs | (d << 16);
            vid[rs + k] = v;
            cp_async<4>(&nb[rs + k], vv + g0 + k);
        }
    }
    cp_async_commit();
    cp_async_wait();
    __syncthreads();
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        const int m = meta[e];
        if (m < 0) continue;
        const int rs = m & 0xffff, d = m >> 16;
        prow[rs + e] = nb[e];            // 2 rs + (e - rs)
        prow[rs + e + d] = INT_MAX;
        bool mine = nb[e] > vid[e];
        if (!mine && heavy == 1) {       // a heavy lower end computes nothing
            const int u = nb[e];
            mine = __ldg(vv_off + u + 1) - __ldg(vv_off + u) > kMaxDeg;
        }
        if (mine) own[atomicAdd(&n_own, 1)] = e;
    }
    __syncthreads();
    const int no = n_own;
    const bool vec = (reinterpret_cast<uintptr_t>(vv) & 15) == 0;
    for (int k = threadIdx.x; k < no; k += blockDim.x) {
        const int e = own[k];
        const int m = meta[e], rs = m & 0xffff, d = m >> 16;
        const int v = vid[e], u = nb[e];
        const int64_t ub = vv_off[u];
        const int un = (int)(vv_off[u + 1] - ub);
        if (un > kMaxDeg && heavy != 1) continue;  // reported by u's own block
        // entries of u's row at or past the array's end are not loaded
        const int lim = (int)min(n_vv - ub, (int64_t)INT_MAX);
        int pv = -1;
        unsigned long long bv, bu;
        const int top = d <= 1 ? 1 : 1 << (32 - __clz(d - 1));
        if (d <= 32 && un <= 32) {   // both masks fit 32 bits (the common case)
            unsigned bv32 = 0u, bu32 = 0u;
            adj_scan<unsigned, 32>(prow + 2 * rs, d, top, vv + ub, vec ? -(int)(ub & 3) : 0, un,
                                   lim, vec, v, bv32, bu32, pv);
            bv = bv32;
            bu = bu32;
        } else {
            bv = bu = 0ull;
            adj_scan<unsigned long long, 64>(prow + 2 * rs, d, top, vv + ub,
                                             vec ? -(int)(ub & 3) : 0, un, lim, vec, v, bv, bu,
                                             pv);
        }
        adj[gst[rs] + (e - rs)] = bv;
        // u's mask is u's to keep only when u's row is light (else it has none)
        if (pv >= 0 && un <= kMaxDeg) adj[ub + pv] = bu;
    }
}

constexpr int kClassifyThreads = 128;

// Components of the lower and upper link subgraphs by bitmask search: a
// component grows from its lowest unvisited member, each member reached
// once adding its same-kind neighbours (its adjacency mask) to the frontier.
// Every neighbour is visited exactly once, so a vertex costs deg iterations
// whatever the link's shape (no data-dependent find loops).
template <typename F>
__global__ void __launch_bounds__(kClassifyThreads)
k_crit_classify(const int64_t *__restrict__ vv_off, const int *__restrict__ vv,
                const unsigned long long *__restrict__ adj, const F *__restrict__ field_v0,
                int64_t v0, int64_t nv, unsigned *__restrict__ classes3_v0)
{
    griddep_wait();
    // rows [v0, v0 + nv); field and classes indexed from v0 (a vertex range
    // holds every neighbour of its vertices when it is a whole mesh of a batch)
    const int64_t v = v0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= v0 + nv) return;
    const F *field = field_v0 - v0;
    unsigned *classes3 = classes3_v0 - 3 * v0;
    const int64_t b = vv_off[v];
    const int n = (int)(vv_off[v + 1] - b);
    if (n > kMaxDeg) return;   // tg_heavy.cu classifies it
    unsigned lo = 0, up = 0;
    {
        const F fv = field[v];
        unsigned long long lower = 0ull;
        for (int k = 0; k < n; k++) {
            const int u = __ldg(vv + b + k);
            const F fu = __ldg(field + u);
            const bool is_lower = (fu == fv) ? (u < (int)v) : (fu < fv);
            lower |= (unsigned long long)is_lower << k;
        }
        const unsigned long long all = n == 64 ? ~0ull : (1ull << n) - 1ull;
        unsigned long long rem = all;
        while (rem) {
            const int s = __ffsll((long long)rem) - 1;
            const bool is_lo = (lower >> s) & 1ull;
            const unsigned long long kind = is_lo ? lower : (all & ~lower);
            unsigned long long comp = 1ull << s, frontier = comp;
            while (frontier) {
                const int j = __ffsll((long long)frontier) - 1;
                frontier &= frontier - 1;
                const unsigned long long nb = __ldg(adj + b + j) & kind & ~comp;
                comp |= nb;
                frontier |= nb;
            }
            rem &= ~comp;
            if (is_lo) lo++; else up++;
        }
    }
    unsigned code;
    if (lo >= 1 && up == 0) code = 2;
    else if (lo == 0 && up >= 1) code = 1;
    else if (lo == 1 && up == 1) code = 3;
    else code = 4;
    classes3[3 * v] = lo;
    classes3[3 * v + 1] = up;
    classes3[3 * v + 2] = code;
}

}  // namespace

int crit_window() { return kAdjWin; }

void launch_crit_adj(const int64_t *vv_off, const int32_t *vv, const int32_t *order,
                     const int64_t *ooff, const int64_t *ostart, const int32_t *vv_win,
                     int64_t V, int64_t n_vv, uint64_t *adj, DevStatus *st, int heavy,
                     cudaStream_t s)
{
    if (V == 0) return;
    Launch L("k_crit_adj", s);
    launch_pdl(k_crit_adj, (unsigned)window_count(n_vv, kAdjWin), kAdjThreads, 0, s,
        vv_off, vv, n_vv, order, order ? ooff : vv_off, ostart, vv_win,
        reinterpret_cast<unsigned long long *>(adj), st, heavy);
}

namespace {
// row lengths and row starts of VV in the star processing order (positions
// past the vertices with cells hold placeholders: length 0)
__global__ void __launch_bounds__(256)
k_vv_lengths_in_order(const int64_t *__restrict__ vv_off, const int *__restrict__ order,
                      int64_t V, int64_t n_with_cells, int *__restrict__ len,
                      int64_t *__restrict__ start)
{
    griddep_wait();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    int d = 0;
    int64_t b = 0;
    if (i < n_with_cells) {
        const int v = order[i];
        b = vv_off[v];
        d = (int)(vv_off[v + 1] - b);
    }
    len[i] = d;
    start[i] = b;
}
}  // namespace

void launch_vv_lengths_in_order(const int64_t *vv_off, const int32_t *order, int64_t V,
                                int64_t n_with_cells, int32_t *len, int64_t *start, cudaStream_t s)
{
    if (V == 0) return;
    Launch L("k_vv_lengths_in_order", s);
    launch_pdl(k_vv_lengths_in_order, (unsigned)((V + 255) / 256), 256, 0, s, vv_off, order, V,
               n_with_cells, len, start);
}

void launch_crit_classify(const int64_t *vv_off, const int32_t *vv, const uint64_t *adj,
                          const void *field, int field_type, int64_t v0, int64_t nv,
                          uint32_t *classes3, cudaStream_t s)
{
    if (nv == 0) return;
    const unsigned grid = (unsigned)((nv + kClassifyThreads - 1) / kClassifyThreads);
    const auto *a = reinterpret_cast<const unsigned long long *>(adj);
    Launch L("k_crit_classify", s);
    if (field_type == 1)
        launch_pdl(k_crit_classify<double>, grid, kClassifyThreads, 0, s,
            vv_off, vv, a, (const double *)field, v0, nv, classes3);
    else
        launch_pdl(k_crit_classify<float>, grid, kClassifyThreads, 0, s,
            vv_off, vv, a, (const float *)field, v0, nv, classes3);
}

}  // namespace tg
