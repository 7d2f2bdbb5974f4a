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
//   k_star_a/b/c   the per-vertex star passes (tg_star.cu)
//   k_cell_tt      face-sharing TT
//   k_face_fill    FV, FE (from TE of a face's first cell), FF
//   k_ef_fill      EF from ET and TF;  k_ee_fill  EE;
//   k_tt_vertex_*  vertex-sharing TT
#include <algorithm>
#include <climits>

#include "tg_internal.h"

namespace tg {
namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ int get4(const int4 &w, int i)
{
    return i == 0 ? w.x : (i == 1 ? w.y : (i == 2 ? w.z : w.w));
}

// index of the vertex pair (s, t), s < t, in the reference TE order
__device__ __forceinline__ int pair_slot(int s, int t)
{
    return s == 0 ? t - 1 : (s == 1 ? t + 1 : 5);
}

#define TG_CSWAP(x, y) \
    if ((x) > (y)) { int _t = (x); (x) = (y); (y) = _t; }

// one comparator of a sorting network: (x, y) <- (min, max)
__device__ __forceinline__ void cswap(int &x, int &y)
{
    const int lo = min(x, y);
    y = max(x, y);
    x = lo;
}

// ---------------------------------------------------------------------------
// k_canon
// ---------------------------------------------------------------------------
// A block's 1024 (cell, slot) pairs name far fewer distinct vertices on
// meshes whose cells come in spatial order (a run of cubes shares its
// corners): the block counts them in a shared-memory hash (vertex -> count;
// each pair's place is its local rank there) and makes one global atomic per
// distinct vertex, whose return value is the block's base in that vertex's
// VT row.
constexpr int kCanonHash = 2048;   // twice the block's pairs: never full

__global__ void __launch_bounds__(256)
k_canon(const int32_t *tv, int64_t T, int V, int4 *tvs, int *deg_t, int4 *occ, DevStatus *st,
        int aligned)
{
    griddep_wait();
    __shared__ int hkey[kCanonHash], hcnt[kCanonHash];
    for (int i = threadIdx.x; i < kCanonHash; i += blockDim.x) {
        hkey[i] = -1;
        hcnt[i] = 0;
    }
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int q[4];
    bool ok = false;
    if (c < T) {
        int a, b, d, e;
        if (aligned) {
            int4 w = reinterpret_cast<const int4 *>(tv)[c];
            a = w.x; b = w.y; d = w.z; e = w.w;
        } else {
            a = tv[4 * c]; b = tv[4 * c + 1]; d = tv[4 * c + 2]; e = tv[4 * c + 3];
        }
        // A rejected cell is overwritten with -1s (the input may alias tvs)
        // and takes no part in the counts; every later kernel skips it, and
        // the host reports the error before anything reads the mesh again.
        if ((unsigned)a >= (unsigned)V || (unsigned)b >= (unsigned)V ||
            (unsigned)d >= (unsigned)V || (unsigned)e >= (unsigned)V) {
            atomicOr(&st->flags, ST_BAD_ID);
            atomicMin(&st->bad_cell, (int)c);
            tvs[c] = make_int4(-1, -1, -1, -1);
        } else {
            TG_CSWAP(a, b);
            TG_CSWAP(d, e);
            TG_CSWAP(a, d);
            TG_CSWAP(b, e);
            TG_CSWAP(b, d);
            if (a == b || b == d || d == e) {
                atomicOr(&st->flags, ST_DUP_VERTEX);
                atomicMin(&st->bad_cell, (int)c);
                tvs[c] = make_int4(-1, -1, -1, -1);
            } else {
                tvs[c] = make_int4(a, b, d, e);
                q[0] = a; q[1] = b; q[2] = d; q[3] = e;
                ok = true;
            }
        }
    }
    __syncthreads();
    int hs[4], rk[4];
    if (ok) {
#pragma unroll
        for (int k = 0; k < 4; k++) {
            unsigned h = ((unsigned)q[k] * 0x9E3779B1u) >> 21;   // 11 bits
            hs[k] = 0;
            rk[k] = 0;
            for (int probe = 0; probe < kCanonHash; probe++) {
                const int old = atomicCAS(&hkey[h], -1, q[k]);
                if (old == -1 || old == q[k]) {
                    hs[k] = (int)h;
                    rk[k] = atomicAdd(&hcnt[h], 1);
                    break;
                }
                h = (h + 1) & (kCanonHash - 1);
            }
        }
    }
    __syncthreads();
    // the count so far is the block's place in each vertex's VT row (rows
    // are sorted afterwards)
    for (int i = threadIdx.x; i < kCanonHash; i += blockDim.x) {
        const int n = hcnt[i];
        if (n) hcnt[i] = atomicAdd(deg_t + hkey[i], n);
    }
    __syncthreads();
    if (ok)
        occ[c] = make_int4(hcnt[hs[0]] + rk[0], hcnt[hs[1]] + rk[1], hcnt[hs[2]] + rk[2],
                           hcnt[hs[3]] + rk[3]);
}

// ---------------------------------------------------------------------------
// k_vt_fill / k_sort_rows
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
k_vt_fill(const int4 *__restrict__ tvs, int64_t T, const int64_t *__restrict__ vt_off,
          const int4 *__restrict__ occ, int *__restrict__ vt)
{
    griddep_wait();
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= T) return;
    const int4 w = tvs[c];
    if (w.x < 0) return;  // rejected by k_canon
    const int4 o = occ[c];
    vt[vt_off[w.x] + o.x] = (int)c;
    vt[vt_off[w.y] + o.y] = (int)c;
    vt[vt_off[w.z] + o.z] = (int)c;
    vt[vt_off[w.w] + o.w] = (int)c;
}

__global__ void __launch_bounds__(256)
k_sort_rows(const int64_t *__restrict__ off, int *__restrict__ ent, int64_t n_rows)
{
    griddep_wait();
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
// Cell, face and edge fills
// ---------------------------------------------------------------------------
__device__ __forceinline__ int rank_of(const uint2 *__restrict__ rk, long long p)
{
    const uint2 w = __ldg(rk + (p >> 5));
    return (int)w.y + __popc(w.x & ((1u << (p & 31)) - 1u));
}

// Face-sharing TT rows at offset 4c - (boundary faces in cells before c),
// since a cell's TT row holds one entry per interior face (the cell across
// each face from FT, sorted); the closing offsets of TT and FF.
__global__ void __launch_bounds__(256)
k_cell_tt(int64_t T, int64_t F, const int *__restrict__ tf, const int *__restrict__ ft,
          const uint2 *__restrict__ brank, int64_t *__restrict__ tt_off, int *__restrict__ tt,
          int64_t *__restrict__ ff_off)
{
    griddep_wait();
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= T) return;
    if (c == T - 1) {
        const int64_t nb = rank_of(brank, 4 * T);
        if (tt_off) tt_off[T] = 4 * T - nb;
        if (ff_off) ff_off[F] = 3 * (2 * F - nb);
    }
    if (!tt) return;
    const int4 f4 = reinterpret_cast<const int4 *>(tf)[c];
    int nbr[4];
    int n = 0;
#pragma unroll
    for (int col = 0; col < 4; col++) {
        const int2 cells = reinterpret_cast<const int2 *>(ft)[get4(f4, col)];
        const int o = (cells.x == (int)c) ? cells.y : cells.x;
        nbr[col] = o >= 0 ? o : INT_MAX;   // no cell across a boundary face
        n += o >= 0;
    }
    // a sorting network (no data-dependent loops); the missing neighbours
    // sort last
    cswap(nbr[0], nbr[1]);
    cswap(nbr[2], nbr[3]);
    cswap(nbr[0], nbr[2]);
    cswap(nbr[1], nbr[3]);
    cswap(nbr[1], nbr[2]);
    const int64_t off = 4 * c - rank_of(brank, 4 * c);
    tt_off[c] = off;
    int *row = tt + off;
#pragma unroll
    for (int i = 0; i < 4; i++)
        if (i < n) row[i] = nbr[i];
}

// EF rows, a thread per edge e = (a, b): walk its ET row (cells ascending)
// and take at each cell the two faces holding a and b (the columns omitting
// one of the other two slots), smaller id first, keeping an id only when it
// exceeds the last one kept.  A face's id is the rank of its first
// occurrence (4 * cell + column), so a face first met at this cell has a
// larger id than every face met before, and a face met again (its second
// cell) has an id no larger than the last kept: the row comes out ascending
// with each face once.
__global__ void __launch_bounds__(256)
k_ef_fill(const int2 *__restrict__ ev, int64_t E, const int64_t *__restrict__ et_off,
          const int *__restrict__ et, const int4 *__restrict__ tvs, const int *__restrict__ tf,
          const int64_t *__restrict__ ef_off, int *__restrict__ ef)
{
    griddep_wait();
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const int2 ab = __ldg(ev + e);
    const int64_t r0 = __ldg(et_off + e), r1 = __ldg(et_off + e + 1);
    int *out = ef + __ldg(ef_off + e);
    int last = -1, n = 0;
    for (int64_t r = r0; r < r1; r++) {
        const int c = __ldg(et + r);
        const int4 w = __ldg(tvs + c);
        // the slots of a and b (rows sorted, a < b), the other two t1 < t2
        const int sa = (w.x < ab.x) + (w.y < ab.x) + (w.z < ab.x) + (w.w < ab.x);
        const int sb = (w.x < ab.y) + (w.y < ab.y) + (w.z < ab.y) + (w.w < ab.y);
        const int t1 = sa == 0 ? (sb == 1 ? 2 : 1) : 0;
        const int t2 = 6 - sa - sb - t1;
        // face omitting t: column 3 - t (t1 < t2: column 3 - t2 first)
        const int f2 = __ldg(tf + 4LL * c + (3 - t2)), f1 = __ldg(tf + 4LL * c + (3 - t1));
        const int lo = min(f1, f2), hi = max(f1, f2);
        if (lo > last) {
            out[n++] = lo;
            last = lo;
        }
        if (hi > last) {
            out[n++] = hi;
            last = hi;
        }
    }
}

// Thread per face f (consecutive threads write consecutive rows): its first
// cell c (FT[f][0]) and its column in c's TF row give the face's occurrence
// slot q = 4c + column and its vertices (c's sorted slots but 3 - column);
// FV from c's vertices, FE from c's TE row, the FF offset 3 * (2f - boundary
// faces before f, counted over occurrence slots up to q) and the FF row (the
// faces of both cells, f itself (once in each row) and a missing second
// cell as INT_MAX, sorted by a 19-comparator network: the first 6 (interior)
// or 3 (boundary) are the row).
__global__ void __launch_bounds__(256)
k_face_fill(const int *__restrict__ ft, const int *__restrict__ tf, const int4 *__restrict__ tvs,
            const int *__restrict__ te, const uint2 *__restrict__ brank, int64_t F,
            int *__restrict__ fv, int *__restrict__ fe, int64_t *__restrict__ ff_off,
            int *__restrict__ ff)
{
    griddep_wait();
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    const int2 cells = reinterpret_cast<const int2 *>(ft)[f];
    const int4 w0 = reinterpret_cast<const int4 *>(tf)[cells.x];
    const int col = w0.x == (int)f ? 0 : (w0.y == (int)f ? 1 : (w0.z == (int)f ? 2 : 3));
    if (fv || fe) {
        // the face's slots in its first cell: all but 3 - col
        const int omit = 3 - col;
        const int s0 = omit == 0 ? 1 : 0, s1 = omit <= 1 ? 2 : 1, s2 = omit <= 2 ? 3 : 2;
        if (fv) {
            const int4 w = tvs[cells.x];
            fv[3 * f] = get4(w, s0);
            fv[3 * f + 1] = get4(w, s1);
            fv[3 * f + 2] = get4(w, s2);
        }
        if (fe) {
            const int *row = te + 6LL * cells.x;
            fe[3 * f] = row[pair_slot(s0, s1)];
            fe[3 * f + 1] = row[pair_slot(s0, s2)];
            fe[3 * f + 2] = row[pair_slot(s1, s2)];
        }
    }
    if (!ff) return;
    const int64_t off = 3 * (2 * f - rank_of(brank, 4LL * cells.x + col));
    ff_off[f] = off;
    const int4 w1 = cells.y >= 0 ? reinterpret_cast<const int4 *>(tf)[cells.y]
                                 : make_int4((int)f, (int)f, (int)f, (int)f);
    int r[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
#pragma unroll
    for (int k = 0; k < 8; k++)
        if (r[k] == (int)f) r[k] = INT_MAX;
    cswap(r[0], r[2]); cswap(r[1], r[3]); cswap(r[4], r[6]); cswap(r[5], r[7]);
    cswap(r[0], r[4]); cswap(r[1], r[5]); cswap(r[2], r[6]); cswap(r[3], r[7]);
    cswap(r[0], r[1]); cswap(r[2], r[3]); cswap(r[4], r[5]); cswap(r[6], r[7]);
    cswap(r[2], r[4]); cswap(r[3], r[5]);
    cswap(r[1], r[4]); cswap(r[3], r[6]);
    cswap(r[1], r[2]); cswap(r[3], r[4]); cswap(r[5], r[6]);
    const int n = cells.y >= 0 ? 6 : 3;
    int *row = ff + off;
#pragma unroll
    for (int i = 0; i < 6; i++)
        if (i < n) row[i] = r[i];
}

// EE: a warp takes 32 consecutive edges (each lane fetches one edge's
// endpoints and offsets), then merges them one at a time.  For e = (a, b) the
// sorted incident-edge rows of a and b (at most kMaxDeg = 64 each) form one
// bitonic sequence over 32 * R positions (lane l holds positions l + 32 r):
// a's row ascending in the first half, b's row descending in the second, both
// padded with INT_MAX towards the middle.  One bitonic merge sorts it; e sits
// twice at adjacent positions (it is in both rows, and the rows share nothing
// else), so dropping both copies leaves e's EE row.  R = 1, 2 or 4 by the
// longer row (16, 32, 64 entries).
constexpr int kEeWarps = 8;

template <int R>
__device__ __forceinline__ void ee_merge_one(const int *__restrict__ eid, int64_t ra, int na,
                                             int64_t rb, int nb, int ei, int *__restrict__ out,
                                             int lane)
{
    constexpr int N = 32 * R, H = N / 2;
    int x[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int p = lane + 32 * r;
        if (p < H) {
            x[r] = p < na ? __ldg(eid + ra + p) : INT_MAX;
        } else {
            const int j = N - 1 - p;
            x[r] = j < nb ? __ldg(eid + rb + j) : INT_MAX;
        }
    }
    // strides >= 32: between registers
#pragma unroll
    for (int sr = R / 2; sr >= 1; sr >>= 1) {
#pragma unroll
        for (int r = 0; r < R; r++) {
            if (r & sr) continue;
            const int lo = min(x[r], x[r + sr]), hi = max(x[r], x[r + sr]);
            x[r] = lo;
            x[r + sr] = hi;
        }
    }
    // strides 16 .. 1: between lanes
#pragma unroll
    for (int sl = 16; sl >= 1; sl >>= 1) {
        const bool upper = lane & sl;
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int y = __shfl_xor_sync(kFull, x[r], sl);
            x[r] = upper ? max(x[r], y) : min(x[r], y);
        }
    }
    // the row is sorted: an entry above e follows both copies of e
    const int n = na + nb;
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int p = lane + 32 * r;
        if (p < n && x[r] != ei) out[p - (x[r] > ei ? 2 : 0)] = x[r];
    }
}

// Rows of at most 16 entries each (the common case: 14 neighbours inside a
// Kuhn grid) go 32 / G edges at a time, G lanes to an edge, 32 / G registers
// to a lane (position gl + G r): the same bitonic merge over 32 positions,
// the strides of G and more between registers, the smaller ones between the
// group's lanes.
constexpr int kEeGroup = TG_EE_GROUP;
static_assert(kEeGroup == 4 || kEeGroup == 8, "lanes per edge: 4 or 8");

template <int G>
__device__ __forceinline__ void ee_merge_group(const int *__restrict__ eid, int64_t ra, int na,
                                               int64_t rb, int nb, int ei, int *__restrict__ out,
                                               int gl)
{
    constexpr int R = 32 / G;
    int x[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int p = gl + G * r;
        if (p < 16) {
            x[r] = p < na ? __ldg(eid + ra + p) : INT_MAX;
        } else {
            const int j = 31 - p;
            x[r] = j < nb ? __ldg(eid + rb + j) : INT_MAX;
        }
    }
    // strides 16 .. G: between registers (register stride sr = stride / G)
#pragma unroll
    for (int sr = 16 / G; sr >= 1; sr >>= 1) {
#pragma unroll
        for (int r = 0; r < R; r++) {
            if (r & sr) continue;
            const int lo = min(x[r], x[r + sr]), hi = max(x[r], x[r + sr]);
            x[r] = lo;
            x[r + sr] = hi;
        }
    }
    // strides G / 2 .. 1: lanes of the group
#pragma unroll
    for (int sl = G / 2; sl >= 1; sl >>= 1) {
        const bool upper = gl & sl;
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int y = __shfl_xor_sync(kFull, x[r], sl);
            x[r] = upper ? max(x[r], y) : min(x[r], y);
        }
    }
    // the row is sorted: an entry above e follows both copies of e
    const int n = na + nb;
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int p = gl + G * r;
        if (p < n && x[r] != ei) out[p - (x[r] > ei ? 2 : 0)] = x[r];
    }
}

__global__ void __launch_bounds__(kEeWarps * 32)
k_ee_fill(const int *__restrict__ ev, int64_t E, const int64_t *__restrict__ vv_off,
          const int *__restrict__ eid, const int64_t *__restrict__ ee_off, int *__restrict__ ee)
{
    griddep_wait();
    const int lane = threadIdx.x & 31;
    const int64_t e0 = ((int64_t)blockIdx.x * kEeWarps + (threadIdx.x >> 5)) * 32;
    if (e0 >= E) return;  // warp-uniform
    const int cnt = E - e0 < 32 ? (int)(E - e0) : 32;
    int64_t my_ra = 0, my_rb = 0, my_out = 0;
    int my_na = 0, my_nb = 0;
    if (lane < cnt) {
        const int2 ab = __ldg(reinterpret_cast<const int2 *>(ev) + e0 + lane);
        my_ra = __ldg(vv_off + ab.x);
        my_rb = __ldg(vv_off + ab.y);
        my_na = (int)(__ldg(vv_off + ab.x + 1) - my_ra);
        my_nb = (int)(__ldg(vv_off + ab.y + 1) - my_rb);
        my_out = __ldg(ee_off + e0 + lane);
    }
    const unsigned small = __ballot_sync(kFull, lane < cnt && max(my_na, my_nb) <= 16);
    // rows longer than kMaxDeg: the heavy path's (k_ee_heavy)
    const unsigned big = __ballot_sync(kFull, lane < cnt && max(my_na, my_nb) <= kMaxDeg) & ~small;
    // small edges, 32 / G per round (group g takes the (k + g)-th one)
    constexpr int G = kEeGroup;
    const int g = lane / G, gl = lane % G;
    const int n_small = __popc(small);
    const bool all_small = small == 0xffffffffu;   // no lanes to skip (the common case)
    for (int k = 0; k < n_small; k += 32 / G) {
        const int which = k + g;
        const int src = all_small ? which : (which < n_small ? (int)__fns(small, 0, which + 1) : 0);
        const int64_t ra = __shfl_sync(kFull, my_ra, src), rb = __shfl_sync(kFull, my_rb, src);
        int na = __shfl_sync(kFull, my_na, src), nb = __shfl_sync(kFull, my_nb, src);
        const int64_t o = __shfl_sync(kFull, my_out, src);
        if (which >= n_small) na = nb = 0;  // an idle group: nothing to write
        ee_merge_group<G>(eid, ra, na, rb, nb, (int)(e0 + src), ee + o, gl);
    }
    // longer rows one edge at a time over the whole warp
    for (unsigned rest = big; rest; rest &= rest - 1) {
        const int j = __ffs(rest) - 1;
        const int64_t ra = __shfl_sync(kFull, my_ra, j), rb = __shfl_sync(kFull, my_rb, j);
        const int na = __shfl_sync(kFull, my_na, j), nb = __shfl_sync(kFull, my_nb, j);
        int *out = ee + __shfl_sync(kFull, my_out, j);
        const int ei = (int)(e0 + j);
        if (max(na, nb) <= 32)
            ee_merge_one<2>(eid, ra, na, rb, nb, ei, out, lane);
        else
            ee_merge_one<4>(eid, ra, na, rb, nb, ei, out, lane);
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
    griddep_wait();
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

// int32 -> int64 (the reference's vtkIdType) copy
__global__ void __launch_bounds__(256)
k_widen(const int *__restrict__ src, long long *__restrict__ dst, int64_t n)
{
    griddep_wait();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

// int64 -> int32 copy (CSR offsets of a relation below 2^31 entries)
__global__ void __launch_bounds__(256)
k_narrow(const int64_t *__restrict__ src, int *__restrict__ dst, int64_t n)
{
    griddep_wait();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = (int)src[i];
}

__global__ void __launch_bounds__(256) k_narrow_multi(NarrowJobs j)
{
    griddep_wait();
    const int64_t total = j.start[j.n];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        int k = 0;
        while (i >= j.start[k + 1]) k++;
        j.dst[i] = (int)j.src[k][i - j.start[k]];
    }
}

// CSR rows -> the reference's padded device_VV layout: row v at v * width,
// unused slots -1, plus the row lengths
__global__ void __launch_bounds__(256)
k_pad_rows(const int64_t *__restrict__ off, const int *__restrict__ ent, int64_t rows, int width,
           long long *__restrict__ out, unsigned *__restrict__ counts)
{
    griddep_wait();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * width) return;
    const int64_t r = i / width;
    const int k = (int)(i - r * width);
    const int64_t b = off[r];
    const int n = (int)(off[r + 1] - b);
    out[i] = k < n ? (long long)ent[b + k] : -1ll;
    if (k == 0 && counts) counts[r] = (unsigned)n;
}

__global__ void k_reset_status(DevStatus *st)
{
    griddep_wait();
    st->flags = 0;
    st->bad_cell = INT_MAX;
    st->bad_vertex = INT_MAX;
    st->max_star = 0;
    st->max_deg = 0;
}

inline unsigned blocks_for(int64_t n, int threads)
{
    return (unsigned)((n + threads - 1) / threads);
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
void launch_widen(const int32_t *src, int64_t *dst, int64_t n, cudaStream_t s)
{
    if (n == 0) return;
    Launch L("k_widen", s);
    const int64_t blocks = std::min<int64_t>((n + 255) / 256, 152 * 32);
    launch_pdl(k_widen, (unsigned)blocks, 256, 0, s, src, reinterpret_cast<long long *>(dst), n);
}

void launch_narrow(const int64_t *src, int32_t *dst, int64_t n, cudaStream_t s)
{
    if (n == 0) return;
    Launch L("k_narrow", s);
    const int64_t blocks = std::min<int64_t>((n + 255) / 256, 152 * 32);
    launch_pdl(k_narrow, (unsigned)blocks, 256, 0, s, src, dst, n);
}

void launch_narrow_multi(const NarrowJobs &j, cudaStream_t s)
{
    const int64_t n = j.start[j.n];
    if (n == 0) return;
    Launch L("k_narrow_multi", s);
    const int64_t blocks = std::min<int64_t>((n + 255) / 256, 152 * 32);
    launch_pdl(k_narrow_multi, (unsigned)blocks, 256, 0, s, j);
}

void launch_pad_rows(const int64_t *off, const int32_t *ent, int64_t rows, int width,
                     int64_t *out, uint32_t *counts, cudaStream_t s)
{
    if (rows == 0 || width == 0) return;
    Launch L("k_pad_rows", s);
    launch_pdl(k_pad_rows, blocks_for(rows * width, 256), 256, 0, s, off, ent, rows, width,
                                                            reinterpret_cast<long long *>(out), counts);
}

// copies the status and the sizes to mapped host memory, then resets the
// status for the next call on the mesh (the host has consumed it)
__global__ void k_publish(PublishArgs a)
{
    griddep_wait();
    if (threadIdx.x != 0) return;
    *a.h_st = *a.st;
    for (int i = 0; i < a.n; i++)
        a.h_sz[i] = a.wide[i] ? *(const int64_t *)a.src[i] : (int64_t) * (const int32_t *)a.src[i];
    __threadfence_system();
    a.st->flags = 0;
    a.st->bad_cell = INT_MAX;
    a.st->bad_vertex = INT_MAX;
    a.st->max_star = 0;
    a.st->max_deg = 0;
}

void launch_publish(const PublishArgs &a, cudaStream_t s)
{
    Launch L("k_publish", s);
    launch_pdl(k_publish, 1, 32, 0, s, a);
}

void launch_reset_status(DevStatus *st, cudaStream_t s)
{
    Launch L("k_reset_status", s);
    launch_pdl(k_reset_status, 1, 1, 0, s, st);
}

void launch_canon(const int32_t *tv_in, int64_t T, int64_t V, int4 *tvs, int32_t *deg_t,
                  int4 *occ, DevStatus *st, cudaStream_t s)
{
    if (T == 0) return;
    const int aligned = ((uintptr_t)tv_in & 15) == 0;
    {
        Launch L("k_canon", s);
        launch_pdl(k_canon, blocks_for(T, 256), 256, 0, s, tv_in, T, (int)V, tvs, deg_t, occ, st, aligned);
    }
}

void launch_vt_fill(const int4 *tvs, int64_t T, const int64_t *vt_off, const int4 *occ, int32_t *vt,
                    cudaStream_t s)
{
    if (T == 0) return;
    {
        Launch L("k_vt_fill", s);
        launch_pdl(k_vt_fill, blocks_for(T, 256), 256, 0, s, tvs, T, vt_off, occ, vt);
    }
}

void launch_sort_rows(const int64_t *off, int32_t *ent, int64_t n_rows, cudaStream_t s)
{
    if (n_rows == 0) return;
    {
        Launch L("k_sort_rows", s);
        launch_pdl(k_sort_rows, blocks_for(n_rows, 256), 256, 0, s, off, ent, n_rows);
    }
}





void launch_cell_tt(int64_t T, int64_t F, const int32_t *tf, const int32_t *ft, const uint2 *brank,
                    int64_t *tt_off, int32_t *tt, int64_t *ff_off, cudaStream_t s)
{
    if (T == 0) return;
    {
        Launch L("k_cell_tt", s);
        launch_pdl(k_cell_tt, blocks_for(T, 256), 256, 0, s, T, F, tf, ft, brank, tt_off, tt,
                   ff_off);
    }
}

void launch_ef_fill(const int32_t *ev, int64_t E, const int64_t *et_off, const int32_t *et,
                    const int4 *tvs, const int32_t *tf, const int64_t *ef_off, int32_t *ef,
                    cudaStream_t s)
{
    if (E == 0) return;
    Launch L("k_ef_fill", s);
    launch_pdl(k_ef_fill, blocks_for(E, 256), 256, 0, s, reinterpret_cast<const int2 *>(ev), E,
               et_off, et, tvs, tf, ef_off, ef);
}

void launch_face_fill(const int32_t *ft, const int32_t *tf, const int4 *tvs, const int32_t *te,
                      const uint2 *brank, int64_t F, int32_t *fv, int32_t *fe, int64_t *ff_off,
                      int32_t *ff, cudaStream_t s)
{
    if (F == 0) return;
    {
        Launch L("k_face_fill", s);
        launch_pdl(k_face_fill, blocks_for(F, 256), 256, 0, s, ft, tf, tvs, te, brank, F, fv, fe,
                   ff_off, ff);
    }
}

void launch_ee_fill(const int32_t *ev, int64_t E, const int64_t *vv_off, const int32_t *eid_sorted,
                    const int64_t *ee_off, int32_t *ee, cudaStream_t s)
{
    if (E == 0) return;
    {
        Launch L("k_ee_fill", s);
        launch_pdl(k_ee_fill, blocks_for((E + 31) / 32, kEeWarps), kEeWarps * 32, 0, s, ev, E, vv_off, eid_sorted,
                                                                   ee_off, ee);
    }
}

void launch_tt_vertex_count(const int4 *tvs, int64_t T, const int64_t *vt_off, const int32_t *vt,
                            int32_t *cnt, cudaStream_t s)
{
    if (T == 0) return;
    {
        Launch L("k_tt_vertex", s);
        launch_pdl(k_tt_vertex<false>, blocks_for(T, 256), 256, 0, s, tvs, T, vt_off, vt, cnt, nullptr, nullptr);
    }
}

void launch_tt_vertex_fill(const int4 *tvs, int64_t T, const int64_t *vt_off, const int32_t *vt,
                           const int64_t *tt_off, int32_t *tt, cudaStream_t s)
{
    if (T == 0) return;
    {
        Launch L("k_tt_vertex", s);
        launch_pdl(k_tt_vertex<true>, blocks_for(T, 256), 256, 0, s, tvs, T, vt_off, vt, nullptr, tt_off, tt);
    }
}

}  // namespace tg
