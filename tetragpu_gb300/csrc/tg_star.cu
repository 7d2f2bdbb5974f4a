// tg_star.cu -- the per-vertex "star" passes of the relation pipeline.
//
// The star of a vertex v is its VT row: the cells around v, ascending.  Every
// cell that holds an edge or a face at v is in it, so within the star
//   * the first position holding a neighbour u is the first occurrence of
//     edge (v,u) in the reference's cell-order scan, and
//   * the first position holding both x and y is the first occurrence of
//     face (v,x,y),
// which is what the reference CPU ids are ranks of (src/cpu_extraction.cpp:
// 28-62 edges, 122-174 faces).
//
// Work decomposition: the VT rows, in star processing order (vertices by
// first cell, see k_vorder_place), are cut into windows of kWin entries (kWinB
// for pass B).  A block owns the vertices whose rows START in its window (at
// most kWin + kMaxStar - 1 entries), stages their cells and the cells' sorted
// TV rows in shared memory (all gathers in flight at once), and gives one
// thread to each (vertex, star cell) entry.  In pass A a shared-memory hash
// keyed by (vertex, neighbour) holds, per neighbour, the mask of star
// positions whose cell contains it (32-bit in a window whose stars have at
// most 32 cells, else 64-bit); lanes holding the same key are merged by
// __match_any_sync first, so one lane per group touches the table.  Pass A
// leaves every entry's three candidate masks in global memory (their low 32
// bits for every entry, the high 32 in a second array for the entries of
// stars of more than 32 cells) and pass B stages them instead of rebuilding
// the table.  With the masks, "first
// position holding u" is a count-trailing-zeros and "first position holding
// x and y" a ctz of an AND.
//
//   k_star_a  first-occurrence bitmaps (edges owned by v = v is the low end,
//             faces owned by v = v is the lowest vertex, boundary faces), the
//             ET / EF row lengths at each owned edge's first-occurrence slot,
//             neighbour counts, the candidate masks
//   k_star_b  ids (ranks of first occurrences), sorted VV rows, id-sorted
//             incident edge ids, TE, TF, ET rows, and at each face's first
//             cell its FT row
//   k_edge_offsets  the id-ordered pass over edge occurrence slots: ET / EF /
//             EE offsets and EV (one pass with a look-back scan)
#include "tg_internal.h"

namespace tg {
namespace {

constexpr int kWin = TG_STAR_WIN;         // VT entries per block window
constexpr int kCap = kWin + kMaxStar;     // staged entries (rows starting in the window)
// pass B keeps more per entry (neighbour lists, ids, work lists; no table),
// and its windows are sized so that eight of its blocks share an SM
constexpr int kWinB = TG_STAR_WIN_B;
constexpr int kEfLanesA = TG_EFA_LANES;   // lanes per owned edge for its EF count (pass A)
constexpr int kCapB = kWinB + kMaxStar;
constexpr int kThreads = TG_STAR_THREADS;
constexpr int kHashBits = TG_STAR_HASH_BITS;
constexpr int kHash = 1 << kHashBits;     // (vertex, neighbour) slots per block, >= 3 * kCap
constexpr unsigned long long kEmpty = ~0ull;

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
__device__ __forceinline__ int omitted_slot(const int4 &w, int a, int b, int c)
{
    if (w.x != a && w.x != b && w.x != c) return 0;
    if (w.y != a && w.y != b && w.y != c) return 1;
    if (w.z != a && w.z != b && w.z != c) return 2;
    return 3;
}
// id of occurrence p: the set bits of the first-occurrence bitmap below p
__device__ __forceinline__ int rank_of(const uint2 *__restrict__ rk, long long p)
{
    const uint2 w = __ldg(rk + (p >> 5));
    return (int)w.y + __popc(w.x & ((1u << (p & 31)) - 1u));
}
// Star-position masks: bit j = position j of a vertex's star.  A block
// whose window holds only stars of at most 32 cells works with 32-bit masks
// (the GPU's integer operations are 32-bit: a 64-bit and, shift or
// find-first-set costs several instructions), any other with 64-bit ones
// (stars of at most kMaxStar = 64 cells).  Both run the same templated code;
// the masks in global memory are 64-bit either way.
__device__ __forceinline__ int mctz(unsigned m) { return __ffs((int)m) - 1; }
__device__ __forceinline__ int mctz(unsigned long long m) { return __ffsll((long long)m) - 1; }
__device__ __forceinline__ int mpopc(unsigned m) { return __popc(m); }
__device__ __forceinline__ int mpopc(unsigned long long m) { return __popcll(m); }
constexpr int kNarrowStar = 32;   // the most cells a star may have for 32-bit masks

// pass A's row-start metadata word, above the row start, length and slot
// fields: the row's neighbour count (bits 22-29; at most 3 * kMaxStar = 192)
// and whether v has a boundary face (bit 30)
constexpr int kRowCount = 1 << 22;
constexpr int kRowBoundary = 1 << 30;
static_assert(3 * kMaxStar < 256, "the neighbour count must fit its 8 bits");

// Pass A's shared memory: the fields that do not depend on the mask width
// first (staged before the width is chosen), the masks last.
struct StageBaseA {
    int cell[kCap];
    int4 tv[kCap];
    int vid[kCap];
    int meta[kCap];                     // row start | D << 10 | slot of v << 20
    unsigned long long hkey[kHash];     // (row start << 32) | neighbour, kEmpty if free
    short cslot[kCap][3];               // hash slot of each entry's 3 candidates (other vertices)
    int n, vlo, vhi, full;
    long long base;
};
template <typename M>
struct Stage : StageBaseA {
    M hmask[kHash];                     // star positions whose cell holds the neighbour
};

// static shared memory is capped at 48 KiB per block
static_assert(sizeof(Stage<unsigned long long>) <= 48 * 1024,
              "star stage exceeds the static shared-memory limit");
static_assert(offsetof(StageBaseA, tv) % 16 == 0, "staged rows must be 16-byte aligned for cp.async");

// Pass B stages the same window without a hash: pass A leaves every VT
// entry's three candidate masks in global memory.  It also lists each
// vertex's neighbours (at 3 * row start, the most a row of D cells can have
// is 3D) with their edge ids.
struct StageBaseB {
    int cell[kCapB];
    int4 tv[kCapB];
    int vid[kCapB];
    int meta[kCapB];                     // row start | D << 10 | slot of v << 20
    int hv[kCapB][3];                    // at first sightings: list index, then edge id
    int cnt[kCapB];
    int list_u[3 * kCapB];               // neighbours, then (after pass 2) their edge ids
    int work[3 * kCapB];                 // first sightings (list index << 11 | entry << 2 |
                                        // candidate): n_owned
                                        // owned ones (u > v) from the front, n_work others
                                        // from the back
    unsigned head[kCapB / 32 + 1];      // bit rs: a row starts at entry rs
    int n, vlo, vhi, n_work, n_owned, wide;
    int n_pairs, n_faces;               // the last phase's work lists
    long long base;
};
template <typename M>
struct StageM : StageBaseB {
    M cm[kCapB][3];                      // star positions holding each candidate
    // with 32-bit masks, room for each listed neighbour's first occurrence
    // (6 cell + pair slot): phase 2 then ranks a first sighting among the
    // row's edge ids (the order of their first occurrences) together with
    // its VV rank, with no pass rewriting the lists as ids
    int lkey[sizeof(M) == 4 ? 3 * kCapB : 1];
};
static_assert(sizeof(StageM<unsigned long long>) <= 48 * 1024,
              "star stage B exceeds the static shared-memory limit");
static_assert(offsetof(StageBaseB, tv) % 16 == 0, "staged rows must be 16-byte aligned for cp.async");

__device__ __forceinline__ int m_rs(int m) { return m & 1023; }
__device__ __forceinline__ int m_D(int m) { return (m >> 10) & 1023; }
__device__ __forceinline__ int m_sv(int m) { return (m >> 20) & 3; }

__device__ __forceinline__ unsigned hslot(unsigned long long key)
{
    return (unsigned)((key * 0x9E3779B97F4A7C15ull) >> (64 - kHashBits));
}

template <typename M>
__device__ __forceinline__ int h_insert(Stage<M> &S, unsigned long long key, M bits)
{
    unsigned h = hslot(key);
    for (int probe = 0; probe < kHash; probe++) {
        const unsigned long long old = atomicCAS(&S.hkey[h], kEmpty, key);
        if (old == kEmpty || old == key) {
            atomicOr(&S.hmask[h], bits);
            return (int)h;
        }
        h = (h + 1) & (kHash - 1);
    }
    return -1;
}

__device__ __forceinline__ unsigned long long hk(int rs, int u)
{
    return ((unsigned long long)(unsigned)rs << 32) | (unsigned)u;
}

// Pass B's rows: the row starts are marked in a bitmap (head), and an
// entry's row start is the nearest mark at or below it (rows hold at most
// kMaxStar entries, so the search looks at most three words back).  Only
// the row starts' vid / meta are written by the rows; the other entries copy
// theirs, all threads at once.
__device__ __forceinline__ void fill_rows(const unsigned *head, int *vid, int *meta, int n)
{
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        int w = e >> 5;
        unsigned bits = head[w] & (0xffffffffu >> (31 - (e & 31)));
        for (int k = 0; k < 3 && !bits && w > 0; k++) bits = head[--w];
        const int rs = 32 * w + 31 - __clz(bits | 1u);
        if (rs != e) {
            vid[e] = vid[rs];
            meta[e] = meta[rs];
        }
    }
}

// The staging in one barrier: the window ends at the next window's first
// entry or at the first heavy star's (light_end: heavy stars come after every
// light one), each row's thread writes its entries' row metadata itself, the
// table's keys and masks are cleared beside the row loads (as G, the widest
// masks this launch uses: 64-bit ones cover the 32-bit layout too), and
// whether a star of the window holds more than kNarrowStar cells (returned,
// block-uniform) comes from the barrier itself.
template <typename G>
__device__ int stage_rows_a1(StageBaseA &S, const StarA &a)
{
    const int plo = __ldg(a.win + blockIdx.x), phi = __ldg(a.win + blockIdx.x + 1);
    const int base = __ldg(a.wbase + blockIdx.x);
    const int n = (int)(min((int64_t)__ldg(a.wbase + blockIdx.x + 1), a.light_end) - base);
    for (int e = threadIdx.x; e < n; e += blockDim.x) cp_async<4>(&S.cell[e], a.vtp + base + e);
    cp_async_commit();
    if (threadIdx.x == 0) {
        S.vlo = plo;
        S.vhi = phi;
        S.base = base;
        S.n = n;
        S.full = 0;
    }
    G *hm = reinterpret_cast<Stage<G> &>(S).hmask;
    for (int h = threadIdx.x; h < kHash; h += blockDim.x) {
        S.hkey[h] = kEmpty;
        hm[h] = 0;
    }
    int wide = 0;
    for (int i = plo + threadIdx.x; i < phi; i += blockDim.x) {
        const int rs = (int)(a.pofs[i] - base);
        const int D = (int)(a.pofs[i + 1] - a.pofs[i]);
        if (D == 0 || rs >= n) continue;   // a heavy star's row: tg_heavy.cu's
        wide |= D > kNarrowStar;
        const int v = a.vorder[i];
        for (int k = 0; k < D; k++) {
            S.vid[rs + k] = v;
            S.meta[rs + k] = rs | (D << 10);
        }
    }
    cp_async_wait();
    for (int e = threadIdx.x; e < n; e += blockDim.x) cp_async<16>(&S.tv[e], a.tvs + S.cell[e]);
    cp_async_commit();
    cp_async_wait();
    return __syncthreads_or(wide);
}

// Fill the (vertex, neighbour) table from the staged cells.  Returns
// false (block-uniformly) when the table overflows.
// Z: the table's masks were cleared by the staging (stage_rows_a1)
template <typename M, bool Z>
__device__ bool stage_cells_and_hash(Stage<M> &S, const int *__restrict__ vorder, DevStatus *st)
{
    const int n = S.n;
    if constexpr (!Z) {
        for (int h = threadIdx.x; h < kHash; h += blockDim.x) S.hmask[h] = 0;
        __syncthreads();
    }
    // insert the 3 other vertices of every staged cell, keyed by the row
    for (int e0 = 0; e0 < n; e0 += blockDim.x) {
        const int e = e0 + threadIdx.x;
        const bool act = e < n;
        const unsigned amask = __ballot_sync(0xffffffffu, act);
        if (!act) continue;
        const int v = S.vid[e];
        const int m = S.meta[e];
        const int rs = m_rs(m);
        const int4 w = S.tv[e];
        const int sv = slot_of(w, v);
        S.meta[e] = m | (sv << 20);
        const int ewarp = e - (threadIdx.x & 31);  // entry of lane 0 of this warp
        const int shift = ewarp - rs;               // lane l sits at row position l + shift
        // the lanes holding this row's entries are contiguous: match on the
        // neighbour alone and keep those lanes
        const int lo = max(-shift, 0), hi = min(-shift + m_D(m), 32);
        const unsigned rowmask = (hi >= 32 ? 0xffffffffu : ((1u << hi) - 1u)) & ~((1u << lo) - 1u);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const int t = k + (k >= sv);
            const int u = get4(w, t);
            const unsigned long long key = hk(rs, u);
            const unsigned grp = __match_any_sync(amask, u) & rowmask;
            const int leader = __ffs(grp) - 1;
            int h = 0;
            if ((int)(threadIdx.x & 31) == leader) {
                // the group's row positions (below the star's size, so
                // within the mask's width)
                const M bits = shift >= 0 ? (M)grp << shift : (M)grp >> -shift;
                h = h_insert(S, key, bits);
                if (h < 0) {
                    S.full = 1;
                    h = 0;
                }
            }
            S.cslot[e][k] = (short)__shfl_sync(amask, h, leader);
        }
    }
    __syncthreads();
    if (S.full) {
        if (threadIdx.x == 0) {
            atomicOr(&st->flags, ST_HASH_FULL);
            atomicMin(&st->bad_vertex, vorder[S.vlo]);
        }
        return false;
    }
    return true;
}

// Occurrence indices (6 cell + pair, 4 cell + column) fit 31 bits (at most
// kMaxCells cells): pass A computes them in 32-bit arithmetic (in pass B the
// 64-bit forms keep its register allocation free of spills).
__device__ __forceinline__ void set_bit(uint32_t *bits, int p)
{
    atomicOr(bits + (p >> 5), 1u << (p & 31));
}

// candidate index (0..2) of slot t in a cell where v sits in slot sv (t != sv)
__device__ __forceinline__ int cand_of(int t, int sv) { return t - (t > sv); }

// The two vertices of a face owned by the vertex in slot sv with slot o omitted.
__device__ __forceinline__ void face_others(const int4 &w, int sv, int o, int &x, int &y)
{
    x = -1;
    y = -1;
#pragma unroll
    for (int t = 0; t < 4; t++)
        if (t != sv && t != o) {
            if (x < 0) x = get4(w, t); else y = get4(w, t);
        }
}

// ---------------------------------------------------------------------------
template <typename M>
__device__ __forceinline__ void star_a_body(Stage<M> &S, const StarA &a, int &n_work)
{
    // in the hash keys' space once the table is built (only its masks are
    // read after that): the first sightings of owned edges (entry << 2 |
    // candidate); each row's neighbour count and boundary flag live in the
    // high bits of its row start's metadata word (kRowCount, kRowBoundary),
    // zero since the staging wrote it
    static_assert(sizeof(S.hkey) >= 3 * kCap * sizeof(int), "work list does not fit the keys");
    int *work = reinterpret_cast<int *>(S.hkey);
    if (!stage_cells_and_hash<M, true>(S, a.vorder, a.st)) return;
    const int n = S.n;
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        const int v = S.vid[e], m = S.meta[e];
        const int rs = m_rs(m), sv = m_sv(m), pos = e - rs;
        const int4 w = S.tv[e];
        const int c = S.cell[e];
        M cm[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            cm[k] = S.hmask[S.cslot[e][k]];
            a.emask[k * a.nvt + S.base + e] = (uint32_t)cm[k];
            if constexpr (sizeof(M) == 8)
                if (m_D(m) > kNarrowStar) a.emask_hi[k * a.nvt + S.base + e] = (uint32_t)(cm[k] >> 32);
        }
#pragma unroll
        for (int k = 0; k < 3; k++) {
            if (mctz(cm[k]) != pos) continue;                  // not the first sighting
            atomicAdd(&S.meta[rs], kRowCount);
            if (get4(w, k + (k >= sv)) > v) work[atomicAdd(&n_work, 1)] = (e << 2) | k;
        }
        // a face at v held by this cell alone (the AND of its two other
        // vertices' masks is this position's bit): v is on the boundary
        const M bit = (M)1 << pos;
        if ((cm[0] & cm[1]) == bit || (cm[0] & cm[2]) == bit || (cm[1] & cm[2]) == bit)
            atomicOr(&S.meta[rs], kRowBoundary);
        if (sv <= 1) {
            // faces whose lowest vertex is v: omit slot 1, 2, 3 when v is in
            // slot 0; omit slot 0 when v is in slot 1.  The face's other two
            // vertices are two of this entry's candidates.
            const int o_lo = sv == 0 ? 1 : 0, o_hi = sv == 0 ? 3 : 0;
            for (int o = o_lo; o <= o_hi; o++) {
                const int ko = cand_of(o, sv);      // the omitted candidate
                const M mf = ko == 0 ? cm[1] & cm[2] : (ko == 1 ? cm[0] & cm[2] : cm[0] & cm[1]);
                if (mctz(mf) != pos) continue;
                const int q = 4 * c + (3 - o);
                set_bit(a.fflag, q);
                const int ncell = mpopc(mf);
                if (ncell == 1) set_bit(a.fbnd, q);
                if (ncell > 2) {
                    atomicOr(&a.st->flags, ST_NONMANIFOLD_FACE);
                    atomicMin(&a.st->bad_cell, c);
                }
            }
        }
    }
    __syncthreads();
    // the edges v owns, kEfLanesA lanes to an edge: flag the first
    // occurrence and record the ET and EF row lengths at that occurrence
    // slot.  At a vertex with no boundary face every face (v,u,x) lies in
    // two cells of the edge's star and every cell holds two of them, so an
    // edge has as many faces as cells; at a boundary vertex each lane takes
    // every kEfLanesA-th cell of the edge's star and counts the faces (v,u,x)
    // whose first cell it is.
    const int nw = n_work;
    constexpr int L = kEfLanesA;
    const int span = ((nw * L + (int)blockDim.x - 1) / (int)blockDim.x) * (int)blockDim.x;
    for (int tt = threadIdx.x; tt < span; tt += blockDim.x) {   // block-uniform trip count
        const int i = tt / L, sub = tt % L;
        int n_ef = 0;
        M mu = 0;
        int p = 0;
        if (i < nw) {
            const int e = work[i] >> 2, k = work[i] & 3;
            const int m = S.meta[e];
            const int rs = m_rs(m), sv = m_sv(m);
            const int t = k + (k >= sv);
            const int u = get4(S.tv[e], t);
            mu = S.hmask[S.cslot[e][k]];
            p = 6 * S.cell[e] + pair_slot(sv, t);
            M mm = (S.meta[rs] & kRowBoundary) ? mu : 0;
            if (!mm && sub == 0) n_ef = mpopc(mu);
            for (int q = 0; q < sub; q++) mm &= mm - 1;
            while (mm) {
                const int j = mctz(mm);
                const int ej = rs + j;
                const int ku = cand_of(slot_of(S.tv[ej], u), m_sv(S.meta[ej]));
#pragma unroll
                for (int kk = 0; kk < 3; kk++) {
                    if (kk == ku) continue;
                    n_ef += mctz(mu & S.hmask[S.cslot[ej][kk]]) == j;
                }
#pragma unroll
                for (int q = 0; q < L; q++) mm &= mm - 1;
            }
        }
#pragma unroll
        for (int off = 1; off < L; off <<= 1) n_ef += __shfl_xor_sync(0xffffffffu, n_ef, off);
        if (i < nw && sub == 0) {
            set_bit(a.eflag, p);
            a.ecnt[p] = (uint32_t)mpopc(mu) | ((uint32_t)n_ef << 16);
        }
    }
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        const int m = S.meta[e];
        if (m_rs(m) != e) continue;
        const int d = (m >> 22) & 255;
        a.deg[S.vid[e]] = d;
        // vertices of more than kMaxDeg neighbours take the heavy paths of
        // EE and critical points (tg_heavy.cu); the largest degree tells the
        // host whether to launch them
        if (d > kMaxDeg) atomicMax(&a.st->max_deg, d);
    }
}

// G: the widest candidate masks the launch keeps in shared memory (32-bit
// when no star of the mesh holds more than kNarrowStar cells, so that no
// window is wide; else 64-bit for the windows holding such a star)
template <typename G>
__global__ void __launch_bounds__(kThreads, 8) k_star_a(StarA a)
{
    griddep_wait();
    // sized for the widest masks this instantiation uses (32-bit ones leave
    // room for larger windows at eight blocks per SM)
    __shared__ __align__(16) unsigned char raw[sizeof(Stage<G>)];
    __shared__ int n_work;
    StageBaseA &S = *reinterpret_cast<StageBaseA *>(raw);
    if (threadIdx.x == 0) n_work = 0;   // ordered before its use by the staging's barrier
    const int wide = stage_rows_a1<G>(S, a);

    if constexpr (sizeof(G) == 8) {
        if (wide) {   // block-uniform
            star_a_body(*reinterpret_cast<Stage<unsigned long long> *>(raw), a, n_work);
            return;
        }
    }
    star_a_body(*reinterpret_cast<Stage<unsigned> *>(raw), a, n_work);
}

// ---------------------------------------------------------------------------
// Stage pass B's window: cells (copied asynchronously, issued first), rows
// (and whether a star has more than kNarrowStar cells), then the cells'
// vertices and the candidate masks pass A computed, copied asynchronously
// as soon as this thread's cells have landed.  Pass A has already rejected
// every window this cannot hold, so nothing here fails.  Cells are staged up
// to the window's end before heavy rows clip it (at most kCapB entries).
// The candidate masks into shared memory: 32-bit in a window whose stars
// hold at most kNarrowStar cells (the low halves), else 64-bit, the high
// half copied for the entries of stars of more than kNarrowStar cells and
// zero for the others (which is what their high half is).  The wide form
// reads each entry's row length, so its rows must be filled in.
__device__ __forceinline__ void copy_masks(StageM<unsigned> &S, const StarB &b, int base, int nst)
{
    for (int e = threadIdx.x; e < nst; e += blockDim.x)
#pragma unroll
        for (int k = 0; k < 3; k++) cp_async<4>(&S.cm[e][k], b.emask + k * b.nvt + base + e);
}
__device__ __forceinline__ void copy_masks(StageM<unsigned long long> &S, const StarB &b, int base,
                                           int nst)
{
    for (int e = threadIdx.x; e < nst; e += blockDim.x) {
        const bool hi = m_D(S.meta[e]) > kNarrowStar;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            unsigned *half = reinterpret_cast<unsigned *>(&S.cm[e][k]);   // little-endian
            cp_async<4>(half, b.emask + k * b.nvt + base + e);
            if (hi)
                cp_async<4>(half + 1, b.emask_hi + k * b.nvt + base + e);
            else
                half[1] = 0u;
        }
    }
}

template <typename G>
__device__ void stage_rows_b(unsigned char *raw, const StarB &b)
{
    StageBaseB &S = *reinterpret_cast<StageBaseB *>(raw);
    const int plo = __ldg(b.win + blockIdx.x), phi = __ldg(b.win + blockIdx.x + 1);
    const int base = __ldg(b.wbase + blockIdx.x);
    const int nst = min(__ldg(b.wbase + blockIdx.x + 1) - base, kCapB);
    for (int e = threadIdx.x; e < nst; e += blockDim.x) cp_async<4>(&S.cell[e], b.vtp + base + e);
    cp_async_commit();
    if (threadIdx.x == 0) {
        S.vlo = plo;
        S.vhi = phi;
        S.base = base;
        S.n = __ldg(b.wbase + blockIdx.x + 1) - base;
        S.n_work = 0;
        S.n_owned = 0;
        S.n_pairs = 0;
        S.n_faces = 0;
        S.wide = 0;
    }
    for (int w = threadIdx.x; w < kCapB / 32 + 1; w += blockDim.x) S.head[w] = 0u;
    __syncthreads();
    for (int i = plo + threadIdx.x; i < phi; i += blockDim.x) {
        const int rs = (int)(b.pofs[i] - base);
        const int D = (int)(b.pofs[i + 1] - b.pofs[i]);
        if (D == 0) continue;
        if (D > kMaxStar) {   // heavy rows (all after this one) are tg_heavy.cu's
            atomicMin(&S.n, rs);
            continue;
        }
        if (D > kNarrowStar) S.wide = 1;
        S.vid[rs] = b.vorder[i];
        S.meta[rs] = rs | (D << 10);
        S.cnt[rs] = 0;
        atomicOr(&S.head[rs >> 5], 1u << (rs & 31));
    }
    cp_async_wait();
    for (int e = threadIdx.x; e < nst; e += blockDim.x) cp_async<16>(&S.tv[e], b.tvs + S.cell[e]);
    // with 32-bit masks in global memory every window is narrow; else the
    // width is known once the rows are in
    if constexpr (sizeof(G) == 4)
        copy_masks(*reinterpret_cast<StageM<unsigned> *>(raw), b, base, nst);
    cp_async_commit();
    __syncthreads();
    fill_rows(S.head, S.vid, S.meta, S.n);
    if constexpr (sizeof(G) == 8) {
        // each thread's own entries: their rows were filled in just above
        if (S.wide)
            copy_masks(*reinterpret_cast<StageM<unsigned long long> *>(raw), b, base, nst);
        else
            copy_masks(*reinterpret_cast<StageM<unsigned> *>(raw), b, base, nst);
        cp_async_commit();
    }
    cp_async_wait();
    __syncthreads();
}

// flat index (entry * 3 + candidate) of candidate u of entry e's first sighting
template <typename M>
__device__ __forceinline__ int first_slot(const StageM<M> &S, int e, int k, int rs, int u)
{
    const int f = rs + mctz(S.cm[e][k]);
    if (f == e) return 3 * e + k;
    return 3 * f + cand_of(slot_of(S.tv[f], u), m_sv(S.meta[f]));
}

// hv entry of candidate u of entry e: the one at u's first sighting in e's row
template <typename M>
__device__ __forceinline__ int hv_of(const StageM<M> &S, int e, int k, int rs, int u)
{
    const int f = rs + mctz(S.cm[e][k]);
    if (f == e) return S.hv[e][k];
    return S.hv[f][cand_of(slot_of(S.tv[f], u), m_sv(S.meta[f]))];
}

template <typename M>
__device__ __forceinline__ void star_b_body(StageM<M> &S, const StarB &b)
{
    const int n = S.n;

    // 1. list every vertex's neighbours (each at its first sighting); the
    //    first sightings form one work list, owned edges (u > v) from the
    //    front, the others from the back
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        const int v = S.vid[e], m = S.meta[e];
        const int rs = m_rs(m), pos = e - rs;
        const int4 w = S.tv[e];
        const int sv = slot_of(w, v);
        S.meta[e] = m | (sv << 20);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            if (mctz(S.cm[e][k]) != pos) continue;
            const int t = k + (k >= sv);
            const int u = get4(w, t);
            const int li = atomicAdd(&S.cnt[rs], 1);
            S.list_u[3 * rs + li] = u;
            if constexpr (sizeof(M) == 4)
                S.lkey[3 * rs + li] = 6 * S.cell[e] + pair_slot(min(sv, t), max(sv, t));
            S.hv[e][k] = li;
            const int item = (li << 11) | (e << 2) | k;
            if (u > v)
                S.work[atomicAdd(&S.n_owned, 1)] = item;
            else
                S.work[3 * kCapB - 1 - atomicAdd(&S.n_work, 1)] = item;
        }
    }
    __syncthreads();
    const int n_owned = S.n_owned, n_first = n_owned + S.n_work;
    auto first_item = [&](int i) {
        return i < n_owned ? S.work[i] : S.work[3 * kCapB - 1 - (i - n_owned)];
    };

    // 2. every first sighting: edge id and VV position (with 32-bit masks also
    //    its place among v's incident edge ids, for EE)
    if constexpr (sizeof(M) == 4) {
        for (int i = threadIdx.x; i < n_first; i += blockDim.x) {
            const int it = first_item(i);
            const int e = (it >> 2) & 511, k = it & 3;
            const int v = S.vid[e], rs = m_rs(S.meta[e]);
            const int u = S.list_u[3 * rs + (it >> 11)], p = S.lkey[3 * rs + (it >> 11)];
            const int deg = S.cnt[rs];
            const int *lu = S.list_u + 3 * rs, *lk = S.lkey + 3 * rs;
            int rank = 0, er = 0;
            for (int j = 0; j < deg; j++) {
                rank += lu[j] < u;
                er += lk[j] < p;
            }
            const int id = rank_of(b.erank, p);
            S.hv[e][k] = id;
            const long long vb = b.vv_off[v];
            if (b.vv) b.vv[vb + rank] = u;
            if (b.eid_sorted) b.eid_sorted[vb + er] = id;
        }
        __syncthreads();
    } else {
    for (int i = threadIdx.x; i < n_first; i += blockDim.x) {
        const int it = first_item(i);
        const int e = (it >> 2) & 511, k = it & 3;
        const int v = S.vid[e], m = S.meta[e];
        const int rs = m_rs(m), sv = m_sv(m);
        const int t = k + (k >= sv);
        const int u = get4(S.tv[e], t);
        const int deg = S.cnt[rs];
        const int *lu = S.list_u + 3 * rs;
        int rank = 0;
        for (int j = 0; j < deg; j++) rank += lu[j] < u;
        S.hv[e][k] = rank_of(b.erank, 6LL * S.cell[e] + pair_slot(min(sv, t), max(sv, t)));
        if (b.vv) b.vv[b.vv_off[v] + rank] = u;
    }
    __syncthreads();
    // the neighbour lists become edge-id lists (for the id order of EE)
    if (b.eid_sorted) {
        for (int i = threadIdx.x; i < n_first; i += blockDim.x) {
            const int it = first_item(i);
            const int e = (it >> 2) & 511, k = it & 3;
            S.list_u[3 * m_rs(S.meta[e]) + (it >> 11)] = S.hv[e][k];
        }
        __syncthreads();
    }

    // 3a. each first sighting's place among v's incident edge ids (for EE)
    if (b.eid_sorted) {
        for (int i = threadIdx.x; i < n_first; i += blockDim.x) {
            const int it = first_item(i);
            const int e = (it >> 2) & 511, k = it & 3;
            const int rs = m_rs(S.meta[e]);
            const int id = S.hv[e][k];
            const int deg = S.cnt[rs];
            const int *li = S.list_u + 3 * rs;
            int r = 0;
            for (int j = 0; j < deg; j++) r += li[j] < id;
            b.eid_sorted[b.vv_off[S.vid[e]] + r] = id;
        }
        __syncthreads();
    }
    }
    // 3b. the ET offsets of the edges v owns, once per edge, at its first
    //     sighting (in the neighbour lists' space, free from here on; ET
    //     offsets are below 6T < 2^31)
    int *eto = S.list_u;
    if (b.et) {
        for (int i = threadIdx.x; i < n_owned; i += blockDim.x) {
            const int it = S.work[i];
            const int e = (it >> 2) & 511, k = it & 3;
            eto[3 * e + k] = (int)b.et_off[S.hv[e][k]];
        }
        // with 32-bit masks the pair list below goes to the spent first
        // occurrences, not over the owned edges this loop reads: no barrier
        // between the two (the ET offsets' loads stay in flight meanwhile)
        if constexpr (sizeof(M) != 4) __syncthreads();
    }
    // 3c. TE of the pairs v is the low end of and the entry's cell in those
    //     edges' ET rows (its place: the star positions below it holding the
    //     other end); TF / FT's second cell of the faces v owns, handled at
    //     their first cell.  An entry holds 3 - sv such pairs and, at sv <= 1,
    //     up to three faces, so a loop over entries would leave most lanes
    //     idle; the pairs (entry << 2 | other slot) and the faces (entry << 2
    //     | omitted slot) are listed first, in the spent first occurrences (or
    //     first-sighting list) and row counts, and the lists run with every
    //     lane busy.  A window
    //     with more first-cell faces than the face list holds handles its
    //     faces entry by entry.
    const bool do_pairs = b.te || b.et, do_faces = b.tf || b.ft;
    int *pairs = sizeof(M) == 4 ? S.lkey : S.work;   // <= 3 per entry
    int *faces = S.cnt;    // <= kCapB, else the fallback below
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        const int m = S.meta[e];
        const int rs = m_rs(m), sv = m_sv(m), pos = e - rs;
        if (do_pairs && sv < 3) {
            const int p0 = atomicAdd(&S.n_pairs, 3 - sv);
            for (int t = sv + 1; t < 4; t++) pairs[p0 + t - sv - 1] = (e << 2) | t;
        }
        if (do_faces && sv <= 1) {
            const int o_lo = sv == 0 ? 1 : 0, o_hi = sv == 0 ? 3 : 0;
            for (int o = o_lo; o <= o_hi; o++) {
                const int ko = cand_of(o, sv);
                const int ka = ko == 0 ? 1 : 0, kb = ko == 2 ? 1 : 2;
                if (mctz(S.cm[e][ka] & S.cm[e][kb]) != pos) continue;
                const int q = atomicAdd(&S.n_faces, 1);
                if (q < kCapB) faces[q] = (e << 2) | o;
            }
        }
    }
    __syncthreads();
    const int n_pairs = S.n_pairs, n_faces = S.n_faces;
    for (int i = threadIdx.x; i < n_pairs; i += blockDim.x) {
        const int it = pairs[i];
        const int e = it >> 2, t = it & 3, k = t - 1;   // cand_of(t, sv) for t > sv
        const int m = S.meta[e];
        const int rs = m_rs(m), sv = m_sv(m), pos = e - rs;
        const int c = S.cell[e];
        const int fs = first_slot(S, e, k, rs, get4(S.tv[e], t));
        if (b.te) b.te[6LL * c + pair_slot(sv, t)] = (&S.hv[0][0])[fs];
        if (b.et) b.et[(long long)eto[fs] + mpopc(S.cm[e][k] & (((M)1 << pos) - (M)1))] = c;
    }
    auto face = [&](int e, int o) {
        const int m = S.meta[e];
        const int rs = m_rs(m), sv = m_sv(m);
        const int c = S.cell[e];
        const int ko = cand_of(o, sv);
        const int ka = ko == 0 ? 1 : 0, kb = ko == 2 ? 1 : 2;
        const M mf = S.cm[e][ka] & S.cm[e][kb];
        const M m2 = mf & (mf - 1);
        const int j2 = m2 ? rs + mctz(m2) : -1;
        const int c2 = m2 ? S.cell[j2] : -1;
        const int fid = face_at_first(b.frank, b.tf, b.ft, 4LL * c + (3 - o), c, c2);
        if (m2 && b.tf) {
            int x, y;
            face_others(S.tv[e], sv, o, x, y);
            b.tf[4LL * c2 + (3 - omitted_slot(S.tv[j2], S.vid[e], x, y))] = fid;
        }
    };
    if (n_faces <= kCapB) {
        for (int i = threadIdx.x; i < n_faces; i += blockDim.x) face(faces[i] >> 2, faces[i] & 3);
    } else {
        for (int e = threadIdx.x; e < n; e += blockDim.x) {
            const int m = S.meta[e];
            const int rs = m_rs(m), sv = m_sv(m), pos = e - rs;
            if (sv > 1) continue;
            const int o_lo = sv == 0 ? 1 : 0, o_hi = sv == 0 ? 3 : 0;
            for (int o = o_lo; o <= o_hi; o++) {
                const int ko = cand_of(o, sv);
                const int ka = ko == 0 ? 1 : 0, kb = ko == 2 ? 1 : 2;
                if (mctz(S.cm[e][ka] & S.cm[e][kb]) == pos) face(e, o);
            }
        }
    }
}

template <typename G>
__global__ void __launch_bounds__(kThreads, 8) k_star_b(StarB b)
{
    griddep_wait();
    __shared__ __align__(16) unsigned char raw[sizeof(StageM<G>)];
    StageBaseB &S = *reinterpret_cast<StageBaseB *>(raw);
    stage_rows_b<G>(raw, b);
    if constexpr (sizeof(G) == 8) {
        if (S.wide) {   // block-uniform
            star_b_body(*reinterpret_cast<StageM<unsigned long long> *>(raw), b);
            return;
        }
    }
    star_b_body(*reinterpret_cast<StageM<unsigned> *>(raw), b);
}

// ---------------------------------------------------------------------------
// Star processing order (see k_vorder_place): vertex v with first cell c in
// slot k has key 4c + k; its bit in vflag marks it, its rank is v's position.
// A vertex whose star holds more than kMaxStar cells is heavy: it takes no
// key and is numbered among the heavy vertices instead (vkey = -1 - index),
// which follow every other vertex with cells in the processing order, so
// the star passes' windows never mix them with the rest (tg_heavy.cu
// processes them).
__device__ __forceinline__ void mark_first(const int4 *__restrict__ tvs, uint32_t *vflag,
                                           int64_t *vkey, int *heavy_cnt, int v, int c, int64_t D)
{
    if (D > kMaxStar) {   // heavy_cnt[0]: heavy vertices, [1]: their star entries
        vkey[v] = -1 - (long long)atomicAdd(heavy_cnt, 1);
        atomicAdd(heavy_cnt + 1, (int)D);
        return;
    }
    // heavy_cnt[2]: some light star holds more than kNarrowStar cells (the
    // star passes then keep their candidate masks 64-bit in global memory)
    if (D > kNarrowStar) heavy_cnt[2] = 1;
    const int4 w = __ldg(tvs + c);
    const long long key = 4LL * c + (w.x == v ? 0 : (w.y == v ? 1 : (w.z == v ? 2 : 3)));
    vkey[v] = key;
    atomicOr(vflag + (key >> 5), 1u << (key & 31));
}

// Sort every VT row ascending.  Rows starting in a window are staged in
// shared memory and each entry lands at its rank in its row (cells in a row
// are distinct); windows holding more than kCap entries fall back to an
// insertion sort per row in global memory.  A block's time is mostly a chain
// of dependent loads (window, offsets, cells, first cells): small blocks put
// more chains in flight per SM.
constexpr int kVtsThreads = TG_VTS_THREADS;
__global__ void __launch_bounds__(kVtsThreads)
k_vt_sort(const int64_t *__restrict__ vt_off, const int *__restrict__ win, int *__restrict__ vt,
          const int4 *__restrict__ tvs, uint32_t *__restrict__ vflag, int64_t *__restrict__ vkey,
          int *__restrict__ heavy_cnt)
{
    griddep_wait();
    __shared__ int cell[kCap], out[kCap], meta[kCap];
    // every thread reads the window's bounds itself (the same words)
    const int s_vlo = win[blockIdx.x], s_vhi = win[blockIdx.x + 1];
    const long long base = vt_off[s_vlo];
    const int n = (int)(vt_off[s_vhi] - base);
    if (n > kCap) {
        for (int v = s_vlo + threadIdx.x; v < s_vhi; v += blockDim.x) {
            const int64_t b = vt_off[v], e = vt_off[v + 1];
            for (int64_t i = b + 1; i < e; i++) {
                const int x = vt[i];
                int64_t j = i - 1;
                while (j >= b && vt[j] > x) {
                    vt[j + 1] = vt[j];
                    j--;
                }
                vt[j + 1] = x;
            }
            if (e > b) mark_first(tvs, vflag, vkey, heavy_cnt, v, vt[b], e - b);
        }
        return;
    }
    for (int v = s_vlo + threadIdx.x; v < s_vhi; v += blockDim.x) {
        const int rs = (int)(vt_off[v] - base);
        const int D = (int)(vt_off[v + 1] - vt_off[v]);
        for (int i = 0; i < D; i++) meta[rs + i] = rs | (D << 10);
    }
    for (int e = threadIdx.x; e < n; e += blockDim.x) cell[e] = vt[base + e];
    __syncthreads();
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        const int m = meta[e], rs = m_rs(m), D = m_D(m), x = cell[e];
        int r = 0;
        for (int j = rs; j < rs + D; j++) r += cell[j] < x;
        out[rs + r] = x;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n; e += blockDim.x) vt[base + e] = out[e];
    for (int v = s_vlo + threadIdx.x; v < s_vhi; v += blockDim.x) {
        const int64_t b = vt_off[v];
        if (vt_off[v + 1] > b)
            mark_first(tvs, vflag, vkey, heavy_cnt, v, out[b - base], vt_off[v + 1] - b);
    }
}

// ---------------------------------------------------------------------------
// ET / EF / EE offsets in edge-id order.  Edge ids are ranks of first
// occurrences, so scanning the 6T edge-occurrence slots in order visits the
// edges in id order: a slot holding a first occurrence contributes the ET
// and EF row lengths k_star_a left there and deg(a) + deg(b) - 2 for EE.
// One pass: a block takes a tile of slots (in start order), gathers each of
// its edges' row lengths (packed in one word by id) and EV, scans the three
// sums with a look-back over the tiles before it, then writes the offsets of
// its edges from the packed words it just wrote.
constexpr int kEdgeThreads = 256;
constexpr int kEdgeItems = TG_EDGE_ITEMS;             // slots per thread: 8, 16 or 32
constexpr int kEdgeTile = kEdgeItems * kEdgeThreads;  // slots per tile
static_assert(kEdgeItems == 8 || kEdgeItems == 16 || kEdgeItems == 32, "slots per thread");

struct EdgeOffsets {
    const uint32_t *eflag;
    const uint32_t *ecnt;
    const int4 *tvs;
    const int32_t *deg;
    const uint2 *erank;
    int64_t n_slots, n_tiles;
    unsigned long long *tiles;   // 3 * n_tiles tile words (ET, EF, EE), then the ticket
    unsigned long long *next;    // the workspace buffer zeroed for the next user
    int64_t next_words;
    unsigned *err;
    uint2 *len;          // [E]: {ET | EF << 16, EE}
    int64_t *et_off, *ef_off, *ee_off;
    int32_t *ev;         // [2E] or null: the edge's two vertices, ascending
    int64_t E;
};

template <int NT>
__device__ __forceinline__ void block_scan3(long long x[3], long long excl[3], long long tot[3])
{
    static_assert(NT % 32 == 0 && NT <= 1024, "block of whole warps");
    __shared__ long long sm[3][NT / 32 + 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < 3; q++) {
        long long incl = x[q];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) sm[q][warp] = incl;
        excl[q] = incl - x[q];
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const long long w = lane < NT / 32 ? sm[q][lane] : 0;
            long long wi = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const long long y = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) wi += y;
            }
            if (lane < NT / 32) sm[q][lane] = wi - w;
            if (lane == NT / 32 - 1) sm[q][NT / 32] = wi;
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 3; q++) {
        excl[q] += sm[q][warp];
        tot[q] = sm[q][NT / 32];
    }
    __syncthreads();
}

__device__ __forceinline__ uint32_t slot_bits(const EdgeOffsets &p, long long s0)
{
    // kEdgeItems consecutive slots starting at a multiple of kEdgeItems lie
    // in one 32-bit word
    if (s0 >= p.n_slots) return 0u;
    const uint32_t w = p.eflag[s0 >> 5];
    return kEdgeItems == 32 ? w : (w >> (s0 & 31)) & ((1u << kEdgeItems) - 1u);
}

// eight blocks per SM (32 registers): the extra resident blocks hide the
// gathers' latency better than the few spilled registers cost
__global__ void __launch_bounds__(kEdgeThreads, TG_EDGE_MINB) k_edge_offsets(EdgeOffsets p)
{
    griddep_wait();
    {
        const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < p.next_words;
             i += nthreads)
            p.next[i] = 0ull;
    }
    __shared__ long long s_tile, s_pre[3];
    if (threadIdx.x == 0) s_tile = (long long)atomicAdd(p.tiles + 3 * p.n_tiles, 1ull);
    __syncthreads();
    const long long tile = s_tile;
    if (p.n_tiles == 0) {   // no slots: the totals alone
        if (tile == 0 && threadIdx.x == 0) {
            if (p.et_off) p.et_off[p.E] = 0;
            if (p.ef_off) p.ef_off[p.E] = 0;
            if (p.ee_off) p.ee_off[p.E] = 0;
        }
        return;
    }
    if (tile >= p.n_tiles) return;
    const long long s0 = tile * kEdgeTile + threadIdx.x * kEdgeItems;
    long long x[3] = {0, 0, 0};
    const uint32_t bits = slot_bits(p, s0);
    const int id0 = bits ? rank_of(p.erank, s0) : 0;
    int id = id0;
    for (uint32_t m = bits; m; m &= m - 1) {
        const int i = __ffs(m) - 1;
        const long long s = s0 + i;
        if (s >= p.n_slots) break;
        const long long cell = s / 6;
        const int j = (int)(s - 6 * cell);
        const int4 w = __ldg(p.tvs + cell);
        const int a = get4(w, j < 3 ? 0 : (j < 5 ? 1 : 2));
        const int b = get4(w, j < 3 ? j + 1 : (j == 3 ? 2 : 3));
        const uint32_t c = p.ecnt[s];
        const int et = c & 0xffff, ef = c >> 16;
        const int ee = p.ee_off ? __ldg(p.deg + a) + __ldg(p.deg + b) - 2 : 0;
        x[0] += et;
        x[1] += ef;
        x[2] += ee;
        p.len[id] = make_uint2(c, (uint32_t)ee);
        if (p.ev) reinterpret_cast<int2 *>(p.ev)[id] = make_int2(a, b);
        id++;
    }
    long long excl[3], tot[3];
    block_scan3<kEdgeThreads>(x, excl, tot);
    if (threadIdx.x < 96) {   // one look-back per sum, warps 0-2 at once
        const int q = threadIdx.x >> 5;
        const long long t = q == 0 ? tot[0] : (q == 1 ? tot[1] : tot[2]);
        const long long pre = look_back(p.tiles + q * p.n_tiles, tile, t, p.err);
        if ((threadIdx.x & 31) == 0) s_pre[q] = pre;
    }
    __syncthreads();
    long long run[3];
#pragma unroll
    for (int q = 0; q < 3; q++) run[q] = s_pre[q] + excl[q];
    // this thread's packed words again (it wrote them: cache hits)
    for (int k = id0; k < id; k++) {
        const uint2 w = p.len[k];
        if (p.et_off) p.et_off[k] = run[0];
        if (p.ef_off) p.ef_off[k] = run[1];
        if (p.ee_off) p.ee_off[k] = run[2];
        run[0] += w.x & 0xffff;
        run[1] += w.x >> 16;
        run[2] += w.y;
    }
    if (tile == p.n_tiles - 1 && threadIdx.x == 0) {
        if (p.et_off) p.et_off[p.E] = s_pre[0] + tot[0];
        if (p.ef_off) p.ef_off[p.E] = s_pre[1] + tot[1];
        if (p.ee_off) p.ee_off[p.E] = s_pre[2] + tot[2];
    }
}

// win[w] = first vertex whose row starts at or after entry kWin * w, for
// w in [0, n_win], with win[n_win] = V.  Vertex v owns the windows w with
// off[v-1] < kWin * w <= off[v].  A second table over the same offsets with
// another window size (win2, or null) comes from the same launch.
__device__ __forceinline__ void window_owner(const long long lo, const long long hi, int64_t v,
                                             int64_t n_win, int win_size, int *win, int *wbase,
                                             long long base_v)
{
    long long w = lo < 0 ? 0 : lo / win_size + 1;
    const long long w_hi = hi / win_size;
    for (; w <= w_hi && w <= n_win; w++) {
        win[w] = (int)v;
        if (wbase) wbase[w] = (int)base_v;
    }
}

__global__ void __launch_bounds__(256)
k_window_starts(const int64_t *__restrict__ off, int64_t V, int64_t n_win, int win_size,
                int *__restrict__ win, int64_t n_win2, int win_size2, int *__restrict__ win2,
                int *__restrict__ wbase, int *__restrict__ wbase2)
{
    griddep_wait();
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v > V) return;
    const long long lo = v == 0 ? -1 : off[v - 1];
    const long long base_v = off[v];   // off[V] = the entry count
    window_owner(lo, v == V ? (long long)win_size * n_win : off[v], v, n_win, win_size, win, wbase,
                 base_v);
    if (win2)
        window_owner(lo, v == V ? (long long)win_size2 * n_win2 : off[v], v, n_win2, win_size2,
                     win2, wbase2, base_v);
}

// ---------------------------------------------------------------------------
// Star processing order.  Vertex ids need not carry locality (meshes are
// often renumbered; the workloads here permute them) while cell order usually
// does (generators and partitioners emit cells in space-filling order).  The
// star passes therefore visit vertices by first cell, the head of the sorted
// VT row, ties by slot: consecutive vertices then share cells, so a block's
// cell gathers hit L2 and the output sectors of cell- and id-ordered
// relations it writes are completed by blocks running at the same time.
// k_vt_sort marks each vertex's key 4 * first cell + slot in a bitmap over
// the 4T cell slots; the key's rank is the vertex's position.  Heavy vertices
// (vkey < 0) follow at n_light + their index; vertices without cells come
// last.
__global__ void __launch_bounds__(256)
k_vorder_place(const int64_t *__restrict__ vt_off, int64_t V, const int64_t *__restrict__ vkey,
               const uint2 *__restrict__ vrank, int64_t nwk, const int *__restrict__ heavy_cnt,
               int *__restrict__ vorder, int *__restrict__ dcount)
{
    griddep_wait();
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const int64_t n_light = (int64_t)__ldg(&vrank[nwk].y);
    // the positions past the vertices with cells (their rows are empty)
    if (v >= n_light + *heavy_cnt) {
        vorder[v] = 0;
        dcount[v] = 0;
    }
    const int D = (int)(vt_off[v + 1] - vt_off[v]);
    if (D == 0) return;
    const long long key = vkey[v];
    int64_t pos;
    if (key < 0) {
        pos = n_light + (-1 - key);
    } else {
        const uint2 r = __ldg(vrank + (key >> 5));
        pos = (int64_t)r.y + __popc(r.x & ((1u << (key & 31)) - 1u));
    }
    vorder[pos] = (int)v;
    dcount[pos] = D;
}

// VT rows copied into processing order: a warp fetches 32 rows' positions
// and sources at once, then copies them one after another, lanes across the
// row
constexpr int kVtpRows = TG_VTP_ROWS;
__global__ void __launch_bounds__(256, TG_VTP_MINB)
k_vtp_fill(const int *__restrict__ vorder, const int64_t *__restrict__ pofs, int64_t V,
           const int64_t *__restrict__ vt_off, const int *__restrict__ vt, int *__restrict__ vtp)
{
    griddep_wait();
    const int64_t r0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32;
    const int lane = threadIdx.x & 31;
    if (r0 >= V) return;  // warp-uniform
    const int64_t r = r0 + lane;
    long long dst = 0, src = 0;
    int D = 0;
    if (r < V) {
        dst = pofs[r];
        D = (int)(pofs[r + 1] - dst);
        if (D > 0) src = __ldg(vt_off + __ldg(vorder + r));
    }
    // kVtpRows rows at a time: their loads are in flight together (lane k
    // takes entry k; entries past 32 of a longer row follow)
    constexpr int R = kVtpRows;
    for (int j = 0; j < 32; j += R) {
        int x[R], Dj[R];
        long long dj[R], sj[R];
#pragma unroll
        for (int t = 0; t < R; t++) {
            Dj[t] = __shfl_sync(0xffffffffu, D, j + t);
            dj[t] = __shfl_sync(0xffffffffu, dst, j + t);
            sj[t] = __shfl_sync(0xffffffffu, src, j + t);
            x[t] = lane < Dj[t] ? __ldg(vt + sj[t] + lane) : 0;
        }
#pragma unroll
        for (int t = 0; t < R; t++) {
            if (lane < Dj[t]) vtp[dj[t] + lane] = x[t];
            for (int k = lane + 32; k < Dj[t]; k += 32) vtp[dj[t] + k] = __ldg(vt + sj[t] + k);
        }
    }
}

// First edge and face id of each segment of cells (a mesh of a batch):
// ids are ranks of first occurrences in cell order, so segment i's ids start
// at the rank of its first cell's first occurrence slot.
__global__ void __launch_bounds__(256)
k_seg_ranks(const int64_t *__restrict__ seg_c, int64_t n, const uint2 *__restrict__ erank,
            const uint2 *__restrict__ frank, int64_t *__restrict__ seg_ef)
{
    griddep_wait();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    seg_ef[i] = rank_of(erank, 6LL * seg_c[i]);
    seg_ef[n + 1 + i] = rank_of(frank, 4LL * seg_c[i]);
}

inline unsigned n_windows(int64_t nvt) { return (unsigned)(nvt / kWin + 1); }
inline unsigned n_windows_b(int64_t nvt) { return (unsigned)(nvt / kWinB + 1); }

}  // namespace

int star_window() { return kWin; }
int star_window_b() { return kWinB; }

int64_t window_count(int64_t n_entries, int win_size) { return n_entries / win_size + 1; }

void launch_window_starts(const int64_t *off, int64_t V, int64_t n_entries, int win_size,
                          int32_t *win, cudaStream_t s, int win_size2, int32_t *win2,
                          int32_t *wbase, int32_t *wbase2)
{
    Launch L("k_window_starts", s);
    launch_pdl(k_window_starts, (unsigned)((V + 1 + 255) / 256), 256, 0, s,
        off, V, window_count(n_entries, win_size), win_size, win,
        win2 ? window_count(n_entries, win_size2) : 0, win_size2, win2, wbase, wbase2);
}

int64_t edge_offsets_words(int64_t n_slots)
{
    return 3 * ((n_slots + kEdgeTile - 1) / kEdgeTile) + 1;
}

void launch_edge_offsets(const uint32_t *eflag, const uint32_t *ecnt, const int4 *tvs,
                         const int32_t *deg, const uint2 *erank, int64_t n_slots, int64_t E,
                         int64_t *et_off, int64_t *ef_off, int64_t *ee_off, int32_t *ev,
                         uint2 *len, ScanWorkspace &ws, DevStatus *st, cudaStream_t s)
{
    const int64_t tiles = (n_slots + kEdgeTile - 1) / kEdgeTile;
    EdgeOffsets p{};
    p.eflag = eflag;
    p.ecnt = ecnt;
    p.tvs = tvs;
    p.deg = deg;
    p.erank = erank;
    p.n_slots = n_slots;
    p.n_tiles = tiles;
    p.err = &st->flags;
    p.len = len;
    p.et_off = et_off;
    p.ef_off = ef_off;
    p.ee_off = ee_off;
    p.ev = ev;
    p.E = E;
    scan_ws_begin(ws, s, &p.tiles, &p.next, &p.next_words);
    {
        Launch L("k_edge_offsets", s);
        launch_pdl(k_edge_offsets, (unsigned)std::max<int64_t>(tiles, 1), kEdgeThreads, 0, s, p);
    }
    scan_ws_end(ws, s);
}

void launch_star_a(const StarA &a, cudaStream_t s)
{
    if (a.V == 0) return;
    Launch L("k_star_a", s);
    if (a.narrow)
        launch_pdl(k_star_a<uint32_t>, n_windows(a.nvt), kThreads, 0, s, a);
    else
        launch_pdl(k_star_a<uint64_t>, n_windows(a.nvt), kThreads, 0, s, a);
}

void launch_star_b(const StarB &b, cudaStream_t s)
{
    if (b.V == 0) return;
    Launch L("k_star_b", s);
    if (b.narrow)
        launch_pdl(k_star_b<uint32_t>, n_windows_b(b.nvt), kThreads, 0, s, b);
    else
        launch_pdl(k_star_b<uint64_t>, n_windows_b(b.nvt), kThreads, 0, s, b);
}

void launch_vt_sort(const int64_t *vt_off, const int32_t *win, int32_t *vt, int64_t V,
                    int64_t nvt, const int4 *tvs, uint32_t *vflag, int64_t *vkey, int32_t *heavy_cnt,
                    cudaStream_t s)
{
    if (V == 0) return;
    Launch L("k_vt_sort", s);
    launch_pdl(k_vt_sort, n_windows(nvt), kVtsThreads, 0, s, vt_off, win, vt, tvs, vflag, vkey,
               heavy_cnt);
}


void launch_vorder_place(const int64_t *vt_off, int64_t V, const int64_t *vkey,
                         const uint2 *vrank, int64_t nwk, const int32_t *heavy_cnt, int32_t *vorder,
                         int32_t *dcount, cudaStream_t s)
{
    if (V == 0) return;
    Launch L("k_vorder_place", s);
    launch_pdl(k_vorder_place, (unsigned)((V + 255) / 256), 256, 0, s, vt_off, V, vkey, vrank, nwk,
               heavy_cnt, vorder, dcount);
}

void launch_vtp_fill(const int32_t *vorder, const int64_t *pofs, int64_t V, const int64_t *vt_off,
                     const int32_t *vt, int32_t *vtp, cudaStream_t s)
{
    if (V == 0) return;
    Launch L("k_vtp_fill", s);
    launch_pdl(k_vtp_fill, (unsigned)((V + 255) / 256), 256, 0, s, vorder, pofs, V, vt_off, vt, vtp);
}


void launch_seg_ranks(const int64_t *seg_c, int64_t n, const uint2 *erank, const uint2 *frank,
                      int64_t *seg_ef, cudaStream_t s)
{
    Launch L("k_seg_ranks", s);
    launch_pdl(k_seg_ranks, (unsigned)((n + 1 + 255) / 256), 256, 0, s, seg_c, n, erank, frank, seg_ef);
}

}  // namespace tg
