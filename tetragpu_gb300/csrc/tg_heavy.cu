// tg_heavy.cu -- the slow path for vertices the star windows do not hold.
//
// The star passes (tg_star.cu) keep a vertex's star positions as bits of a
// 64-bit mask, so they take stars of at most kMaxStar = 64 cells.  A vertex
// in more cells ("heavy") is placed after every other vertex in the star
// processing order, the windows stop where the heavy rows begin, and the
// kernels here do that vertex's share of both passes, one thread per heavy
// vertex, serially over its star.  They write exactly what the star passes
// would: the reference CPU path has no bound on a star
// (src/cpu_extraction.cpp:259-289), and neither has this one.
//
// A heavy vertex v with star cells c_0 < c_1 < ... (its sorted VT row, star
// positions j) lists every (neighbour u, position j) pair of its star and
// sorts them by neighbour, then position.  A neighbour's run is the list of
// positions holding it, ascending, so
//   * the run's first position is the first occurrence of edge (v, u)
//     (its cell and pair slot give the id, as in the star passes),
//   * the run is the ET row of (v, u) when v is the low end,
//   * the first common position of the runs of x and y is the first
//     occurrence of face (v, x, y), the second its other cell.
//
// Beside them: the EE rows of edges with an endpoint of more than kMaxDeg
// neighbours (a serial merge per edge), and the critical-point classes of
// such vertices (a union-find over the neighbours, the link subgraph taken
// from VV as in the reference, src/alg/critPoints.cu:160-266).
#include <algorithm>
#include <climits>

#include "tg_internal.h"

namespace tg {
namespace {

__device__ __forceinline__ int get4(const int4 &w, int i)
{
    return i == 0 ? w.x : (i == 1 ? w.y : (i == 2 ? w.z : w.w));
}
__device__ __forceinline__ int slot_of(const int4 &w, int u)
{
    return (w.x < u) + (w.y < u) + (w.z < u) + (w.w < u);
}
__device__ __forceinline__ int pair_slot(int s, int t)  // s < t, reference TE order
{
    return s == 0 ? t - 1 : (s == 1 ? t + 1 : 5);
}
__device__ __forceinline__ bool holds(const int4 &w, int x)
{
    return w.x == x || w.y == x || w.z == x || w.w == x;
}
__device__ __forceinline__ int omitted_slot(const int4 &w, int a, int b, int c)
{
    if (w.x != a && w.x != b && w.x != c) return 0;
    if (w.y != a && w.y != b && w.y != c) return 1;
    if (w.z != a && w.z != b && w.z != c) return 2;
    return 3;
}
__device__ __forceinline__ int rank_of(const uint2 *__restrict__ rk, long long p)
{
    const uint2 w = rk[p >> 5];
    return (int)w.y + __popc(w.x & ((1u << (p & 31)) - 1u));
}
__device__ __forceinline__ void set_bit(uint32_t *bits, long long p)
{
    atomicOr(bits + (p >> 5), 1u << (p & 31));
}

// (neighbour, position) pairs: by neighbour, then position
__device__ __forceinline__ bool pair_less(int2 a, int2 b)
{
    return a.x < b.x || (a.x == b.x && a.y < b.y);
}

template <typename T, typename Less>
__device__ void sift_down(T *a, int root, int n, Less less)
{
    while (true) {
        int child = 2 * root + 1;
        if (child >= n) return;
        if (child + 1 < n && less(a[child], a[child + 1])) child++;
        if (!less(a[root], a[child])) return;
        const T t = a[root];
        a[root] = a[child];
        a[child] = t;
        root = child;
    }
}

// heapsort: O(n log n) whatever the input, no recursion, no extra memory
template <typename T, typename Less>
__device__ void heap_sort(T *a, int n, Less less)
{
    for (int start = n / 2 - 1; start >= 0; start--) sift_down(a, start, n, less);
    for (int end = n - 1; end > 0; end--) {
        const T t = a[0];
        a[0] = a[end];
        a[end] = t;
        sift_down(a, 0, end, less);
    }
}

// the run [lo, hi) of neighbour x in the sorted pairs (empty when absent)
__device__ void run_of(const int2 *a, int n, int x, int &lo, int &hi)
{
    int l = 0, r = n;
    while (l < r) {
        const int m = (l + r) >> 1;
        if (a[m].x < x) l = m + 1;
        else r = m;
    }
    lo = l;
    r = n;
    while (l < r) {
        const int m = (l + r) >> 1;
        if (a[m].x <= x) l = m + 1;
        else r = m;
    }
    hi = l;
}

// positions common to two runs: how many, the first and the second (-1)
__device__ int common_positions(const int2 *a, int x0, int x1, int y0, int y1, int &first,
                                int &second)
{
    int cnt = 0;
    first = second = -1;
    while (x0 < x1 && y0 < y1) {
        const int px = a[x0].y, py = a[y0].y;
        if (px < py) {
            x0++;
        } else if (py < px) {
            y0++;
        } else {
            if (cnt == 0) first = px;
            else if (cnt == 1) second = px;
            cnt++;
            x0++;
            y0++;
        }
    }
    return cnt;
}

// The two vertices of a face of w that contains w[sv], omitting slot o.
__device__ __forceinline__ void face_others(const int4 &w, int sv, int o, int &x, int &y)
{
    x = -1;
    y = -1;
#pragma unroll
    for (int t = 0; t < 4; t++)
        if (t != sv && t != o) {
            if (x < 0) x = get4(w, t);
            else y = get4(w, t);
        }
}

// Is position r of run [s0, ...) the first cell of face (v, u, x)?  True
// when no earlier cell of the run holds x.
__device__ __forceinline__ bool first_with(const HeavyStars &h, const int *cells, const int2 *a,
                                           int s0, int r, int x)
{
    for (int r2 = s0; r2 < r; r2++)
        if (holds(h.tvs[cells[a[r2].y]], x)) return false;
    return true;
}

struct Star {
    int v, D;
    const int *cells;
    int2 *pairs;
    int *ids;   // 6 per star entry: edge id at each run's first pair, then the ids sorted
};

__device__ Star heavy_star(const HeavyStars &h, int k)
{
    Star s;
    const int64_t n_light = h.n_light;
    const int64_t heavy_base = h.pofs[n_light];
    const int64_t i = n_light + k;
    const int64_t b0 = h.pofs[i];
    s.v = h.vorder[i];
    s.D = (int)(h.pofs[i + 1] - b0);
    s.cells = h.vtp + b0;
    s.pairs = h.pairs + 3 * (b0 - heavy_base);
    s.ids = h.ids ? h.ids + 6 * (b0 - heavy_base) : nullptr;
    return s;
}

// Pass A's share: neighbour count, first-occurrence flags and the ET / EF row
// lengths of the edges v owns, the first-occurrence and boundary flags of the
// faces whose lowest vertex is v.
__global__ void __launch_bounds__(64) k_heavy_a(HeavyStars h)
{
    griddep_wait();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= h.n_heavy) return;
    const Star s = heavy_star(h, k);
    const int v = s.v;
    int2 *a = s.pairs;
    int n = 0;
    for (int j = 0; j < s.D; j++) {
        const int4 w = h.tvs[s.cells[j]];
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const int x = get4(w, t);
            if (x != v) a[n++] = make_int2(x, j);
        }
    }
    heap_sort(a, n, pair_less);
    int deg = 0;
    for (int s0 = 0; s0 < n;) {
        const int u = a[s0].x;
        int s1 = s0 + 1;
        while (s1 < n && a[s1].x == u) s1++;
        deg++;
        if (u > v) {   // v owns the edge
            const int c0 = s.cells[a[s0].y];
            const int4 w0 = h.tvs[c0];
            const long long p = 6LL * c0 + pair_slot(slot_of(w0, v), slot_of(w0, u));
            const int n_et = s1 - s0;
            int n_ef = 0;
            for (int r = s0; r < s1; r++) {
                const int4 w = h.tvs[s.cells[a[r].y]];
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    const int x = get4(w, t);
                    if (x != v && x != u) n_ef += first_with(h, s.cells, a, s0, r, x);
                }
            }
            if (n_et > 0xffff || n_ef > 0xffff) {
                atomicOr(&h.st->flags, ST_STAR_OVERFLOW);
                atomicMin(&h.st->bad_vertex, v);
            }
            set_bit(h.eflag, p);
            h.ecnt[p] = (uint32_t)n_et | ((uint32_t)n_ef << 16);
        }
        s0 = s1;
    }
    h.deg[v] = deg;
    if (deg > kMaxDeg) atomicMax(&h.st->max_deg, deg);
    // faces whose lowest vertex is v: v in slot 0 (omit 1, 2 or 3) or in
    // slot 1 (omit 0)
    for (int j = 0; j < s.D; j++) {
        const int c = s.cells[j];
        const int4 w = h.tvs[c];
        const int sv = slot_of(w, v);
        if (sv > 1) continue;
        const int o_lo = sv == 0 ? 1 : 0, o_hi = sv == 0 ? 3 : 0;
        for (int o = o_lo; o <= o_hi; o++) {
            int x, y, x0, x1, y0, y1, f1, f2;
            face_others(w, sv, o, x, y);
            run_of(a, n, x, x0, x1);
            run_of(a, n, y, y0, y1);
            const int cnt = common_positions(a, x0, x1, y0, y1, f1, f2);
            if (f1 != j) continue;
            const long long q = 4LL * c + (3 - o);
            set_bit(h.fflag, q);
            if (cnt == 1) set_bit(h.fbnd, q);
            if (cnt > 2) {
                atomicOr(&h.st->flags, ST_NONMANIFOLD_FACE);
                atomicMin(&h.st->bad_cell, c);
            }
        }
    }
}

// Pass B's share (the pairs stay sorted from pass A): VV row, edge ids and
// the id-sorted incident edges, TE of the pairs v is the low end of, TF and
// FT of the faces whose lowest vertex is v, ET rows of the edges v owns (EF
// rows come from k_ef_fill, as for every edge).
__global__ void __launch_bounds__(64) k_heavy_b(HeavyStars h)
{
    griddep_wait();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= h.n_heavy) return;
    const Star s = heavy_star(h, k);
    const int v = s.v;
    const int2 *a = s.pairs;
    const int n = 3 * s.D;
    int *id_at = s.ids;               // id at each run's first pair
    int *id_sorted = s.ids + n;       // ids in run order, then sorted
    const int64_t vb = h.vv_off[v];
    int r = 0;
    for (int s0 = 0; s0 < n;) {
        const int u = a[s0].x;
        int s1 = s0 + 1;
        while (s1 < n && a[s1].x == u) s1++;
        const int c0 = s.cells[a[s0].y];
        const int4 w0 = h.tvs[c0];
        const int sv = slot_of(w0, v), su = slot_of(w0, u);
        const int id = rank_of(h.erank, 6LL * c0 + pair_slot(min(sv, su), max(sv, su)));
        if (h.vv) h.vv[vb + r] = u;
        id_at[s0] = id;
        id_sorted[r] = id;
        if (u > v && h.et) {
            const int64_t o = h.et_off[id];
            for (int q = s0; q < s1; q++) h.et[o + (q - s0)] = s.cells[a[q].y];
        }
        r++;
        s0 = s1;
    }
    const int deg = r;
    if (h.eid_sorted) {
        heap_sort(id_sorted, deg, [](int x, int y) { return x < y; });
        for (int q = 0; q < deg; q++) h.eid_sorted[vb + q] = id_sorted[q];
    }
    for (int j = 0; j < s.D; j++) {
        const int c = s.cells[j];
        const int4 w = h.tvs[c];
        const int sv = slot_of(w, v);
        if (h.te) {
            for (int t = sv + 1; t < 4; t++) {
                int lo, hi;
                run_of(a, n, get4(w, t), lo, hi);
                h.te[6LL * c + pair_slot(sv, t)] = id_at[lo];
            }
        }
        if (sv > 1 || (!h.tf && !h.ft)) continue;
        const int o_lo = sv == 0 ? 1 : 0, o_hi = sv == 0 ? 3 : 0;
        for (int o = o_lo; o <= o_hi; o++) {
            int x, y, x0, x1, y0, y1, f1, f2;
            face_others(w, sv, o, x, y);
            run_of(a, n, x, x0, x1);
            run_of(a, n, y, y0, y1);
            common_positions(a, x0, x1, y0, y1, f1, f2);
            if (f1 != j) continue;
            const long long q = 4LL * c + (3 - o);
            const int c2 = f2 < 0 ? -1 : s.cells[f2];
            const int fid = face_at_first(h.frank, h.tf, h.ft, q, c, c2);
            if (c2 >= 0 && h.tf) h.tf[4LL * c2 + (3 - omitted_slot(h.tvs[c2], v, x, y))] = fid;
        }
    }
}

// EE rows of the edges that k_ee_fill leaves (an endpoint with more than
// kMaxDeg neighbours): the two sorted incident-edge rows merged, the edge
// itself (in both) dropped.
__global__ void __launch_bounds__(256)
k_ee_heavy(const int *__restrict__ ev, int64_t E, const int64_t *__restrict__ vv_off,
           const int *__restrict__ eid, const int64_t *__restrict__ ee_off, int *__restrict__ ee)
{
    griddep_wait();
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int2 ab = reinterpret_cast<const int2 *>(ev)[e];
        const int64_t ra = vv_off[ab.x], rb = vv_off[ab.y];
        const int na = (int)(vv_off[ab.x + 1] - ra), nb = (int)(vv_off[ab.y + 1] - rb);
        if (max(na, nb) <= kMaxDeg) continue;
        int64_t o = ee_off[e];
        int i = 0, j = 0;
        while (i < na || j < nb) {
            int x;
            if (j >= nb || (i < na && eid[ra + i] < eid[rb + j])) x = eid[ra + i++];
            else x = eid[rb + j++];
            if (x != (int)e) ee[o++] = x;
        }
    }
}

// vertices with more than kMaxDeg neighbours, listed (count in *n)
__global__ void __launch_bounds__(256)
k_list_heavy_deg(const int64_t *__restrict__ vv_off, int64_t v0, int64_t nv, int *list, int *n)
{
    griddep_wait();
    const int64_t v = v0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= v0 + nv) return;
    if (vv_off[v + 1] - vv_off[v] > kMaxDeg) list[atomicAdd(n, 1)] = (int)v;
}

__device__ int uf_find(int *p, int i)
{
    while (p[i] != i) {
        p[i] = p[p[i]];   // path halving
        i = p[i];
    }
    return i;
}

// Critical-point class of a listed vertex v: its neighbours split into lower
// and upper (ties by id), joined when the mesh has an edge between them (w in
// VV[u]), components counted per kind by a union-find with path halving in
// scratch (one int per VV entry of v).
template <typename F>
__global__ void __launch_bounds__(64)
k_crit_heavy(const int64_t *__restrict__ vv_off, const int *__restrict__ vv,
             const int *__restrict__ list, const int *__restrict__ n_list,
             const F *__restrict__ field_v0, int64_t v0, unsigned *__restrict__ classes3_v0,
             int *__restrict__ scratch)
{
    griddep_wait();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= *n_list) return;
    const int v = list[k];
    const F *field = field_v0 - v0;
    unsigned *classes3 = classes3_v0 - 3 * v0;
    const int64_t b = vv_off[v];
    const int d = (int)(vv_off[v + 1] - b);
    const int *row = vv + b;
    int *p = scratch + b;
    const F fv = field[v];
    auto is_lower = [&](int u) {
        const F fu = field[u];
        return (fu == fv) ? (u < v) : (fu < fv);
    };
    for (int i = 0; i < d; i++) p[i] = i;
    for (int i = 0; i < d; i++) {
        const int u = row[i];
        const bool li = is_lower(u);
        const int64_t ub = vv_off[u];
        const int un = (int)(vv_off[u + 1] - ub);
        for (int q = 0; q < un; q++) {
            const int x = vv[ub + q];
            if (x <= u) continue;   // each pair once, from its lower member
            int l = 0, r = d;       // x's place in v's row
            while (l < r) {
                const int m = (l + r) >> 1;
                if (row[m] < x) l = m + 1;
                else r = m;
            }
            if (l == d || row[l] != x || is_lower(x) != li) continue;
            const int ri = uf_find(p, i), rl = uf_find(p, l);
            if (ri != rl) p[max(ri, rl)] = min(ri, rl);
        }
    }
    unsigned lo = 0, up = 0;
    for (int i = 0; i < d; i++)
        if (uf_find(p, i) == i) {
            if (is_lower(row[i])) lo++;
            else up++;
        }
    unsigned code;
    if (lo >= 1 && up == 0) code = 2;
    else if (lo == 0 && up >= 1) code = 1;
    else if (lo == 1 && up == 1) code = 3;
    else code = 4;
    classes3[3LL * v] = lo;
    classes3[3LL * v + 1] = up;
    classes3[3LL * v + 2] = code;
}

}  // namespace

void launch_heavy_a(const HeavyStars &h, cudaStream_t s)
{
    if (h.n_heavy == 0) return;
    Launch L("k_heavy_a", s);
    launch_pdl(k_heavy_a, (unsigned)((h.n_heavy + 63) / 64), 64, 0, s, h);
}

void launch_heavy_b(const HeavyStars &h, cudaStream_t s)
{
    if (h.n_heavy == 0) return;
    Launch L("k_heavy_b", s);
    launch_pdl(k_heavy_b, (unsigned)((h.n_heavy + 63) / 64), 64, 0, s, h);
}

void launch_ee_heavy(const int32_t *ev, int64_t E, const int64_t *vv_off, const int32_t *eid,
                     const int64_t *ee_off, int32_t *ee, cudaStream_t s)
{
    if (E == 0) return;
    Launch L("k_ee_heavy", s);
    const int64_t blocks = std::min<int64_t>((E + 255) / 256, 152 * 16);
    launch_pdl(k_ee_heavy, (unsigned)blocks, 256, 0, s, ev, E, vv_off, eid, ee_off, ee);
}

void launch_crit_heavy(const int64_t *vv_off, const int32_t *vv, int64_t v0, int64_t nv,
                       int64_t max_listed, const void *field, int field_type, uint32_t *classes3,
                       int32_t *list, int32_t *n_list, int32_t *scratch, cudaStream_t s)
{
    if (nv == 0 || max_listed == 0) return;
    {
        Launch L("k_list_heavy_deg", s);
        launch_pdl(k_list_heavy_deg, (unsigned)((nv + 255) / 256), 256, 0, s, vv_off, v0, nv, list,
                   n_list);
    }
    // one thread per listed vertex (at most max_listed of them; threads past
    // the list's end return at once)
    const unsigned grid = (unsigned)((max_listed + 63) / 64);
    Launch L("k_crit_heavy", s);
    if (field_type == 1)
        launch_pdl(k_crit_heavy<double>, grid, 64, 0, s, vv_off, vv, (const int *)list,
                   (const int *)n_list, (const double *)field, v0, classes3, scratch);
    else
        launch_pdl(k_crit_heavy<float>, grid, 64, 0, s, vv_off, vv, (const int *)list,
                   (const int *)n_list, (const float *)field, v0, classes3, scratch);
}

}  // namespace tg
