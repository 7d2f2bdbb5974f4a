// tg_kernels.cu -- the relation-extraction pipeline for sm_103a.
//
// Id rules reproduced (reference tlranda/TetraGPU, src/cpu_extraction.cpp):
//   edge id = rank of the edge's first occurrence p = 6*cell + j, pairs j in
//             order (0,1),(0,2),(0,3),(1,2),(1,3),(2,3)         (:28-62)
//   face id = rank of the face's first occurrence q = 4*cell + k, faces
//             visited with skip = 3,2,1,0 (:145) and k = TF column = 3 - skip,
//             skip being the omitted slot                        (:122-174)
// on row-sorted TV.  Instead of the reference's serial table scans, the
// first occurrences are found per vertex: the cells around a vertex v (its
// star, the sorted VT row) contain every cell holding any edge or face at v,
// so the lowest star position holding a neighbour u is the first occurrence
// of edge (v,u), and the lowest holding both x and y is the first occurrence
// of face (v,x,y).  First occurrences are marked in bitmaps over all
// occurrence slots; a popcount prefix turns any occurrence into its id.
//
// Kernels, in pipeline order (one thread per cell/face/edge unless noted):
//   k_canon        sort TV rows, validate ids, count cells per vertex
//   k_vt_fill      scatter cells into VT rows (atomic cursors)
//   k_sort_rows    sort each CSR row in place (VT, incident-edge rows)
//   k_star_a       warp per vertex: distinct neighbours and the star positions
//                  holding each (a 64-bit mask), via __match_any_sync and a
//                  shared-memory hash; marks first occurrences of the edges
//                  and faces the vertex owns (owner = lowest vertex)
//   k_vv_finalize  thread per vertex: sort neighbours -> VV and masks
//   k_star_b       warp per vertex: edge ids of all incident edges; EV, TE,
//                  TF, FV, FT and the row counts of ET, EF, EE, FF, TT
//   k_star_c       warp per vertex: ET and EF rows of owned edges
//   k_cell_fe_tt   FE (from TE of a face's first cell) and face-sharing TT
//   k_ff_fill      FF;  k_ee_fill  EE;  k_tt_vertex_*  vertex-sharing TT
#include <climits>

#include "tg_internal.h"

namespace tg {
namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ int get4(const int4 &w, int i)
{
    return i == 0 ? w.x : (i == 1 ? w.y : (i == 2 ? w.z : w.w));
}

// position of u in a sorted row that contains it
__device__ __forceinline__ int slot_of(const int4 &w, int u)
{
    return (w.x < u) + (w.y < u) + (w.z < u) + (w.w < u);
}

// index of the vertex pair (s, t), s < t, in the reference TE order
__device__ __forceinline__ int pair_slot(int s, int t)
{
    return s == 0 ? t - 1 : (s == 1 ? t + 1 : 5);
}

// slot of the one vertex of sorted row w that is none of a, b, c
__device__ __forceinline__ int omitted_slot(const int4 &w, int a, int b, int c)
{
    if (w.x != a && w.x != b && w.x != c) return 0;
    if (w.y != a && w.y != b && w.y != c) return 1;
    if (w.z != a && w.z != b && w.z != c) return 2;
    return 3;
}

// rank of occurrence p among the set bits of flag (ids are ranks)
__device__ __forceinline__ int bit_rank(const uint32_t *__restrict__ flag,
                                        const int32_t *__restrict__ pre, long long p)
{
    const long long wd = p >> 5;
    const uint32_t bits = __ldg(flag + wd);
    return __ldg(pre + wd) + __popc(bits & ((1u << (p & 31)) - 1u));
}

__device__ __forceinline__ int lower_bound_sm(const int *a, int n, int key)
{
    int lo = 0, hi = n;
    while (lo < hi) {
        int m = (lo + hi) >> 1;
        if (a[m] < key) lo = m + 1; else hi = m;
    }
    return lo;
}

#define TG_CSWAP(x, y) \
    if ((x) > (y)) { int _t = (x); (x) = (y); (y) = _t; }

// ---------------------------------------------------------------------------
// k_canon
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
k_canon(const int32_t *tv, int64_t T, int V, int4 *tvs, int *deg_t, DevStatus *st, int aligned)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= T) return;
    int a, b, d, e;
    if (aligned) {
        int4 w = reinterpret_cast<const int4 *>(tv)[c];
        a = w.x; b = w.y; d = w.z; e = w.w;
    } else {
        a = tv[4 * c]; b = tv[4 * c + 1]; d = tv[4 * c + 2]; e = tv[4 * c + 3];
    }
    if ((unsigned)a >= (unsigned)V || (unsigned)b >= (unsigned)V ||
        (unsigned)d >= (unsigned)V || (unsigned)e >= (unsigned)V) {
        atomicOr(&st->flags, ST_BAD_ID);
        atomicMin(&st->bad_cell, (int)c);
        return;
    }
    TG_CSWAP(a, b);
    TG_CSWAP(d, e);
    TG_CSWAP(a, d);
    TG_CSWAP(b, e);
    TG_CSWAP(b, d);
    if (a == b || b == d || d == e) {
        atomicOr(&st->flags, ST_DUP_VERTEX);
        atomicMin(&st->bad_cell, (int)c);
        return;
    }
    tvs[c] = make_int4(a, b, d, e);
    atomicAdd(deg_t + a, 1);
    atomicAdd(deg_t + b, 1);
    atomicAdd(deg_t + d, 1);
    atomicAdd(deg_t + e, 1);
}

// ---------------------------------------------------------------------------
// k_vt_fill / k_sort_rows
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
k_vt_fill(const int4 *__restrict__ tvs, int64_t T, const int64_t *__restrict__ vt_off,
          int *__restrict__ cursor, int *__restrict__ vt)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= T) return;
    const int4 w = tvs[c];
    vt[vt_off[w.x] + atomicAdd(cursor + w.x, 1)] = (int)c;
    vt[vt_off[w.y] + atomicAdd(cursor + w.y, 1)] = (int)c;
    vt[vt_off[w.z] + atomicAdd(cursor + w.z, 1)] = (int)c;
    vt[vt_off[w.w] + atomicAdd(cursor + w.w, 1)] = (int)c;
}

__global__ void __launch_bounds__(256)
k_sort_rows(const int64_t *__restrict__ off, int *__restrict__ ent, int64_t n_rows)
{
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n_rows) {
        const int64_t b = off[r], e = off[r + 1];
        for (int64_t i = b + 1; i < e; i++) {
            const int x = ent[i];
            int64_t j = i - 1;
            while (j >= b && ent[j] > x) {
                ent[j + 1] = ent[j];
                j--;
            }
            ent[j + 1] = x;
        }
    }
}

// ---------------------------------------------------------------------------
// Star kernels: one warp per vertex, star positions in shared memory
// ---------------------------------------------------------------------------
constexpr int kWarps = 8;
constexpr int kHash = 128;  // neighbour table slots per warp (>= 2 * kMaxDeg)

struct StarTile {
    int cell[kMaxStar];
    int4 tv[kMaxStar];
    signed char sv[kMaxStar];
};

__device__ __forceinline__ unsigned hash_slot(int u)
{
    return ((unsigned)u * 2654435761u) >> (32 - 7);
}

// Load the sorted star of v into shared memory (lanes stride positions).
__device__ __forceinline__ void load_star(StarTile &t, const int *__restrict__ vt, int64_t b0, int D,
                                          const int4 *__restrict__ tvs, int v, int lane)
{
    for (int i = lane; i < D; i += 32) {
        const int c = __ldg(vt + b0 + i);
        const int4 w = __ldg(tvs + c);
        t.cell[i] = c;
        t.tv[i] = w;
        t.sv[i] = (signed char)slot_of(w, v);
    }
}

struct SmemA {
    StarTile t;
    int hkey[kHash];
    unsigned long long hmask[kHash];
};

__device__ __forceinline__ bool h_insert(int *hkey, unsigned long long *hmask, int u,
                                         unsigned long long bits)
{
    unsigned h = hash_slot(u);
    for (int probe = 0; probe < kHash; probe++) {
        const int old = atomicCAS(hkey + h, -1, u);
        if (old == -1 || old == u) {
            atomicOr(hmask + h, bits);
            return true;
        }
        h = (h + 1) & (kHash - 1);
    }
    return false;
}

__device__ __forceinline__ unsigned long long h_lookup(const int *hkey,
                                                       const unsigned long long *hmask, int u)
{
    unsigned h = hash_slot(u);
    for (int probe = 0; probe < kHash; probe++) {
        const int k = hkey[h];
        if (k == u) return hmask[h];
        if (k == -1) return 0ull;
        h = (h + 1) & (kHash - 1);
    }
    return 0ull;
}

__global__ void __launch_bounds__(kWarps * 32) k_star_a(StarA a)
{
    __shared__ SmemA sm_all[kWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t v64 = (int64_t)blockIdx.x * kWarps + warp;
    if (v64 >= a.V) return;
    const int v = (int)v64;
    SmemA &sm = sm_all[warp];
    const int64_t b0 = a.vt_off[v];
    const int D = (int)(a.vt_off[v + 1] - b0);
    if (D > kMaxStar) {
        if (lane == 0) {
            atomicOr(&a.st->flags, ST_HEAVY_STAR);
            atomicMin(&a.st->bad_vertex, v);
            a.deg[v] = 0;
        }
        return;
    }
    for (int h = lane; h < kHash; h += 32) {
        sm.hkey[h] = -1;
        sm.hmask[h] = 0ull;
    }
    load_star(sm.t, a.vt, b0, D, a.tvs, v, lane);
    __syncwarp();

    // Distinct neighbours with the star positions holding them.  Lanes that
    // hold the same neighbour in the same column are merged by
    // __match_any_sync first, so one lane per group touches the table.
    bool full = false;
    for (int base = 0; base < D; base += 32) {
        const int i = base + lane;
        const bool act = i < D;
        const unsigned amask = __ballot_sync(kFull, act);
        if (act) {
            const int4 w = sm.t.tv[i];
            const int s = sm.t.sv[i];
#pragma unroll
            for (int jj = 0; jj < 3; jj++) {
                const int t = jj + (jj >= s);
                const int u = get4(w, t);
                const unsigned grp = __match_any_sync(amask, u);
                if (lane == __ffs(grp) - 1)
                    full |= !h_insert(sm.hkey, sm.hmask, u, (unsigned long long)grp << base);
            }
        }
    }
    __syncwarp();
    if (__any_sync(kFull, full)) {
        if (lane == 0) {
            atomicOr(&a.st->flags, ST_HASH_FULL);
            atomicMin(&a.st->bad_vertex, v);
            a.deg[v] = 0;
        }
        return;
    }

    // Compact the table into the padded per-vertex summary: capacity D + 2,
    // enough for any vertex whose link is a triangulated sphere or disk, or
    // 3D (always enough) when a.wide is set after an overflow.
    const int64_t sbase = a.wide ? 3 * b0 : b0 + 2 * v64;
    const int cap = a.wide ? 3 * D : D + 2;
    int cnt = 0;
    for (int s0 = 0; s0 < kHash; s0 += 32) {
        const int k = sm.hkey[s0 + lane];
        const bool valid = k >= 0;
        const unsigned bal = __ballot_sync(kFull, valid);
        const int pos = cnt + __popc(bal & ((1u << lane) - 1u));
        if (valid && pos < cap) {
            a.sum_nb[sbase + pos] = k;
            a.sum_mask[sbase + pos] = sm.hmask[s0 + lane];
        }
        cnt += __popc(bal);
    }
    if (lane == 0) {
        a.deg[v] = cnt <= cap ? cnt : 0;
        if (cnt > cap) {
            atomicOr(&a.st->flags, ST_STAR_OVERFLOW);
            atomicMin(&a.st->bad_vertex, v);
        }
        if (cnt > kMaxDeg) {
            atomicOr(&a.st->flags, ST_HEAVY_DEG);
            atomicMax(&a.st->max_deg, cnt);
        }
    }
    if (cnt > cap) return;

    // First occurrences of the edges v owns (v is the low end).
    for (int h = lane; h < kHash; h += 32) {
        const int u = sm.hkey[h];
        if (u > v) {
            const unsigned long long m = sm.hmask[h];
            const int i = __ffsll((long long)m) - 1;
            const int4 w = sm.t.tv[i];
            const int s = sm.t.sv[i], su = slot_of(w, u);
            const long long p = 6LL * sm.t.cell[i] + pair_slot(min(s, su), max(s, su));
            atomicOr(a.eflag + (p >> 5), 1u << (p & 31));
        }
    }
    // First occurrences of the faces v owns: in a cell where v sits in slot
    // 0 it is the low vertex of the faces omitting slots 1, 2, 3; in slot 1,
    // of the face omitting slot 0.
    for (int i = lane; i < D; i += 32) {
        const int s = sm.t.sv[i];
        if (s > 1) continue;
        const int4 w = sm.t.tv[i];
        const int o_lo = (s == 0) ? 1 : 0, o_hi = (s == 0) ? 3 : 0;
        for (int o = o_lo; o <= o_hi; o++) {
            int x = -1, y = -1;
#pragma unroll
            for (int t = 0; t < 4; t++)
                if (t != s && t != o) {
                    if (x < 0) x = get4(w, t); else y = get4(w, t);
                }
            const unsigned long long m = h_lookup(sm.hkey, sm.hmask, x) & h_lookup(sm.hkey, sm.hmask, y);
            if (__popcll(m) > 2) {
                atomicOr(&a.st->flags, ST_NONMANIFOLD_FACE);
                atomicMin(&a.st->bad_cell, sm.t.cell[i]);
            }
            if (__ffsll((long long)m) - 1 == i) {
                const long long q = 4LL * sm.t.cell[i] + (3 - o);
                atomicOr(a.fflag + (q >> 5), 1u << (q & 31));
            }
        }
    }
}

__global__ void __launch_bounds__(256)
k_vv_finalize(const int64_t *__restrict__ vt_off, const int *__restrict__ sum_nb,
              const unsigned long long *__restrict__ sum_mask, const int64_t *__restrict__ vv_off,
              int64_t V, int wide, int *__restrict__ vv, unsigned long long *__restrict__ vvmask)
{
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const int64_t sb = wide ? 3 * vt_off[v] : vt_off[v] + 2 * v;
    const int64_t ob = vv_off[v];
    const int n = (int)(vv_off[v + 1] - ob);
    for (int k = 0; k < n; k++) {
        const int x = sum_nb[sb + k];
        const unsigned long long mx = sum_mask[sb + k];
        int j = k - 1;
        while (j >= 0 && vv[ob + j] > x) {
            vv[ob + j + 1] = vv[ob + j];
            vvmask[ob + j + 1] = vvmask[ob + j];
            j--;
        }
        vv[ob + j + 1] = x;
        vvmask[ob + j + 1] = mx;
    }
}

struct SmemB {
    StarTile t;
    int nb[kMaxDeg];
    unsigned long long nmask[kMaxDeg];
    int nid[kMaxDeg];
};

// Load star + sorted neighbours (+ edge ids when eidv is given).
__device__ __forceinline__ bool load_vertex(SmemB &sm, int v, int lane, const int64_t *vt_off,
                                            const int *vt, const int4 *tvs, const int64_t *vv_off,
                                            const int *vv, const unsigned long long *vvmask,
                                            const int *eidv, int &D, int &deg, int64_t &vb)
{
    const int64_t b0 = vt_off[v];
    D = (int)(vt_off[v + 1] - b0);
    vb = vv_off[v];
    deg = (int)(vv_off[v + 1] - vb);
    if (D > kMaxStar || deg > kMaxDeg) return false;
    load_star(sm.t, vt, b0, D, tvs, v, lane);
    for (int k = lane; k < deg; k += 32) {
        sm.nb[k] = __ldg(vv + vb + k);
        sm.nmask[k] = __ldg(vvmask + vb + k);
        if (eidv) sm.nid[k] = __ldg(eidv + vb + k);
    }
    __syncwarp();
    return true;
}

__global__ void __launch_bounds__(kWarps * 32) k_star_b(StarB b)
{
    __shared__ SmemB sm_all[kWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t v64 = (int64_t)blockIdx.x * kWarps + warp;
    if (v64 >= b.V) return;
    const int v = (int)v64;
    SmemB &sm = sm_all[warp];
    int D, deg;
    int64_t vb;
    if (!load_vertex(sm, v, lane, b.vt_off, b.vt, b.tvs, b.vv_off, b.vv,
                     reinterpret_cast<const unsigned long long *>(b.vvmask), nullptr, D, deg, vb))
        return;

    // 1. id of every incident edge (first occurrence -> rank)
    for (int k = lane; k < deg; k += 32) {
        const int u = sm.nb[k];
        const unsigned long long m = sm.nmask[k];
        const int i = __ffsll((long long)m) - 1;
        const int4 w = sm.t.tv[i];
        const int s = sm.t.sv[i], su = slot_of(w, u);
        const long long p = 6LL * sm.t.cell[i] + pair_slot(min(s, su), max(s, su));
        const int id = bit_rank(b.eflag, b.epre, p);
        sm.nid[k] = id;
        b.eidv[vb + k] = id;
        if (u > v) {
            if (b.ev) reinterpret_cast<int2 *>(b.ev)[id] = make_int2(v, u);
            if (b.et_cnt) b.et_cnt[id] = __popcll(m);
            if (b.ef_cnt) {
                int c = 0;
                for (int kk = 0; kk < deg; kk++) c += (kk != k) && (sm.nmask[kk] & m);
                b.ef_cnt[id] = c;
            }
            if (b.ee_cnt) b.ee_cnt[id] = deg + (int)(b.vv_off[u + 1] - b.vv_off[u]) - 2;
        }
    }
    __syncwarp();

    // 2. TE entries of the pairs whose low end is v
    if (b.te) {
        for (int i = lane; i < D; i += 32) {
            const int s = sm.t.sv[i];
            const int4 w = sm.t.tv[i];
            int *row = b.te + 6LL * sm.t.cell[i];
            for (int t = s + 1; t < 4; t++) {
                const int k = lower_bound_sm(sm.nb, deg, get4(w, t));
                row[pair_slot(s, t)] = sm.nid[k];
            }
        }
    }

    // 3. faces v owns: TF entries of every occurrence; FV, FT and counts once
    const bool faces = b.tf || b.fv || b.ft || b.ff_cnt || b.tt_cnt;
    if (faces) {
        for (int i = lane; i < D; i += 32) {
            const int s = sm.t.sv[i];
            if (s > 1) continue;
            const int4 w = sm.t.tv[i];
            const int c = sm.t.cell[i];
            const int o_lo = (s == 0) ? 1 : 0, o_hi = (s == 0) ? 3 : 0;
            for (int o = o_lo; o <= o_hi; o++) {
                int x = -1, y = -1;
#pragma unroll
                for (int t = 0; t < 4; t++)
                    if (t != s && t != o) {
                        if (x < 0) x = get4(w, t); else y = get4(w, t);
                    }
                const int kx = lower_bound_sm(sm.nb, deg, x), ky = lower_bound_sm(sm.nb, deg, y);
                const unsigned long long m = sm.nmask[kx] & sm.nmask[ky];
                const int f = __ffsll((long long)m) - 1;
                const int of = (f == i) ? o : omitted_slot(sm.t.tv[f], v, x, y);
                const long long q = 4LL * sm.t.cell[f] + (3 - of);
                const int fid = bit_rank(b.fflag, b.fpre, q);
                if (b.tf) b.tf[4LL * c + (3 - o)] = fid;
                if (f == i) {
                    const unsigned long long m2 = m & (m - 1);
                    const int c2 = m2 ? sm.t.cell[__ffsll((long long)m2) - 1] : -1;
                    if (b.fv) {
                        b.fv[3LL * fid] = v;
                        b.fv[3LL * fid + 1] = x;
                        b.fv[3LL * fid + 2] = y;
                    }
                    if (b.ft) reinterpret_cast<int2 *>(b.ft)[fid] = make_int2(c, c2);
                    if (b.ff_cnt) b.ff_cnt[fid] = 3 * __popcll(m);
                    if (b.tt_cnt && c2 >= 0) {
                        atomicAdd(b.tt_cnt + c, 1);
                        atomicAdd(b.tt_cnt + c2, 1);
                    }
                }
            }
        }
    }
}

__global__ void __launch_bounds__(kWarps * 32) k_star_c(StarC p)
{
    __shared__ SmemB sm_all[kWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t v64 = (int64_t)blockIdx.x * kWarps + warp;
    if (v64 >= p.V) return;
    const int v = (int)v64;
    SmemB &sm = sm_all[warp];
    int D, deg;
    int64_t vb;
    if (!load_vertex(sm, v, lane, p.vt_off, p.vt, p.tvs, p.vv_off, p.vv,
                     reinterpret_cast<const unsigned long long *>(p.vvmask), p.eidv, D, deg, vb))
        return;
    for (int k = lane; k < deg; k += 32) {
        const int u = sm.nb[k];
        if (u <= v) continue;
        const int id = sm.nid[k];
        const unsigned long long m = sm.nmask[k];
        if (p.et) {
            int64_t pos = p.et_off[id];
            unsigned long long mm = m;
            while (mm) {
                const int i = __ffsll((long long)mm) - 1;
                mm &= mm - 1;
                p.et[pos++] = sm.t.cell[i];
            }
        }
        if (p.ef) {
            const int64_t pos0 = p.ef_off[id];
            int n = 0;
            for (int kk = 0; kk < deg; kk++) {
                if (kk == k) continue;
                const unsigned long long mm = m & sm.nmask[kk];
                if (!mm) continue;
                const int f = __ffsll((long long)mm) - 1;
                const int of = omitted_slot(sm.t.tv[f], v, u, sm.nb[kk]);
                const long long q = 4LL * sm.t.cell[f] + (3 - of);
                const int fid = bit_rank(p.fflag, p.fpre, q);
                int64_t j = pos0 + n - 1;
                while (j >= pos0 && p.ef[j] > fid) {
                    p.ef[j + 1] = p.ef[j];
                    j--;
                }
                p.ef[j + 1] = fid;
                n++;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Cell, face and edge fills
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
k_cell_fe_tt(const int4 *__restrict__ tvs, int64_t T, const int *__restrict__ te,
             const int *__restrict__ tf, const int *__restrict__ ft, int *__restrict__ fe,
             const int64_t *__restrict__ tt_off, int *__restrict__ tt)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= T) return;
    const int4 f4 = reinterpret_cast<const int4 *>(tf)[c];
    int nbr[4];
    int n = 0;
#pragma unroll
    for (int col = 0; col < 4; col++) {
        const int f = get4(f4, col);
        const int2 cells = reinterpret_cast<const int2 *>(ft)[f];
        if (fe && cells.x == (int)c) {
            const int omit = 3 - col;
            int sl[3], k = 0;
#pragma unroll
            for (int t = 0; t < 4; t++)
                if (t != omit) sl[k++] = t;
            const int *row = te + 6 * c;
            fe[3LL * f] = row[pair_slot(sl[0], sl[1])];
            fe[3LL * f + 1] = row[pair_slot(sl[0], sl[2])];
            fe[3LL * f + 2] = row[pair_slot(sl[1], sl[2])];
        }
        const int o = (cells.x == (int)c) ? cells.y : cells.x;
        if (o >= 0) nbr[n++] = o;
    }
    if (tt) {
        for (int i = 1; i < n; i++) {
            const int x = nbr[i];
            int j = i - 1;
            while (j >= 0 && nbr[j] > x) { nbr[j + 1] = nbr[j]; j--; }
            nbr[j + 1] = x;
        }
        int *row = tt + tt_off[c];
        for (int i = 0; i < n; i++) row[i] = nbr[i];
    }
}

__global__ void __launch_bounds__(256)
k_ff_fill(const int *__restrict__ ft, const int *__restrict__ tf, int64_t F,
          const int64_t *__restrict__ ff_off, int *__restrict__ ff)
{
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    const int2 cells = reinterpret_cast<const int2 *>(ft)[f];
    int r[6];
    int n = 0;
    for (int s = 0; s < 2; s++) {
        const int c = s ? cells.y : cells.x;
        if (c < 0) continue;
        const int4 w = reinterpret_cast<const int4 *>(tf)[c];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int g = get4(w, k);
            if (g != (int)f) r[n++] = g;
        }
    }
    for (int i = 1; i < n; i++) {
        const int x = r[i];
        int j = i - 1;
        while (j >= 0 && r[j] > x) { r[j + 1] = r[j]; j--; }
        r[j + 1] = x;
    }
    int *row = ff + ff_off[f];
    for (int i = 0; i < n; i++) row[i] = r[i];
}

__global__ void __launch_bounds__(256)
k_ee_fill(const int *__restrict__ ev, int64_t E, const int64_t *__restrict__ vv_off,
          const int *__restrict__ eid, const int64_t *__restrict__ ee_off, int *__restrict__ ee)
{
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const int2 ab = reinterpret_cast<const int2 *>(ev)[e];
    const int *A = eid + vv_off[ab.x];
    const int *B = eid + vv_off[ab.y];
    const int na = (int)(vv_off[ab.x + 1] - vv_off[ab.x]);
    const int nb = (int)(vv_off[ab.y + 1] - vv_off[ab.y]);
    int *out = ee + ee_off[e];
    int i = 0, j = 0, p = 0;
    while (i < na || j < nb) {
        int x;
        if (j >= nb || (i < na && A[i] < B[j])) x = A[i++];
        else if (i >= na || B[j] < A[i]) x = B[j++];
        else { x = A[i++]; j++; }
        if (x != (int)e) out[p++] = x;
    }
}

// Vertex-sharing TT: the union of the VT rows of the cell's four vertices,
// minus the cell itself, by a four-way merge of sorted rows.
template <bool FILL>
__global__ void __launch_bounds__(256)
k_tt_vertex(const int4 *__restrict__ tvs, int64_t T, const int64_t *__restrict__ vt_off,
            const int *__restrict__ vt, int *__restrict__ cnt, const int64_t *__restrict__ tt_off,
            int *__restrict__ tt)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= T) return;
    const int4 w = tvs[c];
    int64_t pos[4], end[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int v = get4(w, k);
        pos[k] = vt_off[v];
        end[k] = vt_off[v + 1];
    }
    int n = 0;
    int *out = FILL ? tt + tt_off[c] : nullptr;
    while (true) {
        int m = INT_MAX;
#pragma unroll
        for (int k = 0; k < 4; k++)
            if (pos[k] < end[k]) m = min(m, vt[pos[k]]);
        if (m == INT_MAX) break;
#pragma unroll
        for (int k = 0; k < 4; k++)
            if (pos[k] < end[k] && vt[pos[k]] == m) pos[k]++;
        if (m != (int)c) {
            if (FILL) out[n] = m;
            n++;
        }
    }
    if (!FILL) cnt[c] = n;
}

inline unsigned blocks_for(int64_t n, int threads)
{
    return (unsigned)((n + threads - 1) / threads);
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
void launch_canon(const int32_t *tv_in, int64_t T, int64_t V, int4 *tvs, int32_t *deg_t,
                  DevStatus *st, cudaStream_t s)
{
    if (T == 0) return;
    const int aligned = ((uintptr_t)tv_in & 15) == 0;
    {
        Launch L("k_canon", s);
        k_canon<<<blocks_for(T, 256), 256, 0, s>>>(tv_in, T, (int)V, tvs, deg_t, st, aligned);
    }
}

void launch_vt_fill(const int4 *tvs, int64_t T, const int64_t *vt_off, int32_t *cursor, int32_t *vt,
                    cudaStream_t s)
{
    if (T == 0) return;
    {
        Launch L("k_vt_fill", s);
        k_vt_fill<<<blocks_for(T, 256), 256, 0, s>>>(tvs, T, vt_off, cursor, vt);
    }
}

void launch_sort_rows(const int64_t *off, int32_t *ent, int64_t n_rows, cudaStream_t s)
{
    if (n_rows == 0) return;
    {
        Launch L("k_sort_rows", s);
        k_sort_rows<<<blocks_for(n_rows, 256), 256, 0, s>>>(off, ent, n_rows);
    }
}

void launch_star_a(const StarA &a, cudaStream_t s)
{
    if (a.V == 0) return;
    {
        Launch L("k_star_a", s);
        k_star_a<<<blocks_for(a.V, kWarps), kWarps * 32, 0, s>>>(a);
    }
}

void launch_vv_finalize(const int64_t *vt_off, const int32_t *sum_nb, const uint64_t *sum_mask,
                        const int64_t *vv_off, int64_t V, int wide, int32_t *vv, uint64_t *vvmask,
                        cudaStream_t s)
{
    if (V == 0) return;
    {
        Launch L("k_vv_finalize", s);
        k_vv_finalize<<<blocks_for(V, 256), 256, 0, s>>>(
            vt_off, sum_nb, reinterpret_cast<const unsigned long long *>(sum_mask), vv_off, V, wide, vv,
            reinterpret_cast<unsigned long long *>(vvmask));
    }
}

void launch_star_b(const StarB &b, cudaStream_t s)
{
    if (b.V == 0) return;
    {
        Launch L("k_star_b", s);
        k_star_b<<<blocks_for(b.V, kWarps), kWarps * 32, 0, s>>>(b);
    }
}

void launch_star_c(const StarC &c, cudaStream_t s)
{
    if (c.V == 0) return;
    {
        Launch L("k_star_c", s);
        k_star_c<<<blocks_for(c.V, kWarps), kWarps * 32, 0, s>>>(c);
    }
}

void launch_cell_fe_tt(const int4 *tvs, int64_t T, const int32_t *te, const int32_t *tf,
                       const int32_t *ft, int32_t *fe, const int64_t *tt_off, int32_t *tt,
                       cudaStream_t s)
{
    if (T == 0) return;
    {
        Launch L("k_cell_fe_tt", s);
        k_cell_fe_tt<<<blocks_for(T, 256), 256, 0, s>>>(tvs, T, te, tf, ft, fe, tt_off, tt);
    }
}

void launch_ff_fill(const int32_t *ft, const int32_t *tf, int64_t F, const int64_t *ff_off,
                    int32_t *ff, cudaStream_t s)
{
    if (F == 0) return;
    {
        Launch L("k_ff_fill", s);
        k_ff_fill<<<blocks_for(F, 256), 256, 0, s>>>(ft, tf, F, ff_off, ff);
    }
}

void launch_ee_fill(const int32_t *ev, int64_t E, const int64_t *vv_off, const int32_t *eid_sorted,
                    const int64_t *ee_off, int32_t *ee, cudaStream_t s)
{
    if (E == 0) return;
    {
        Launch L("k_ee_fill", s);
        k_ee_fill<<<blocks_for(E, 256), 256, 0, s>>>(ev, E, vv_off, eid_sorted, ee_off, ee);
    }
}

void launch_tt_vertex_count(const int4 *tvs, int64_t T, const int64_t *vt_off, const int32_t *vt,
                            int32_t *cnt, cudaStream_t s)
{
    if (T == 0) return;
    {
        Launch L("k_tt_vertex", s);
        k_tt_vertex<false><<<blocks_for(T, 256), 256, 0, s>>>(tvs, T, vt_off, vt, cnt, nullptr, nullptr);
    }
}

void launch_tt_vertex_fill(const int4 *tvs, int64_t T, const int64_t *vt_off, const int32_t *vt,
                           const int64_t *tt_off, int32_t *tt, cudaStream_t s)
{
    if (T == 0) return;
    {
        Launch L("k_tt_vertex", s);
        k_tt_vertex<true><<<blocks_for(T, 256), 256, 0, s>>>(tvs, T, vt_off, vt, nullptr, tt_off, tt);
    }
}

}  // namespace tg
