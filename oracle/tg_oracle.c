/*
 * tg_oracle.c -- CPU restatement of TetraGPU's relation-extraction and
 * critical-point path.  TEST INFRASTRUCTURE ONLY (see tg_oracle.h).
 *
 * Each routine names the reference code it restates, by path:line within the
 * reference project (tlranda/TetraGPU).  The reference keeps per-vertex
 * std::vector tables searched with std::find_if; this file keeps the same
 * tables as per-vertex singly linked lists searched front to back.  Ids are
 * minted in exactly the same order (first occurrence while scanning cells in
 * order), because a search in an unordered list of unique keys finds the same
 * key whatever the list order.
 *
 * Plain C99, single-threaded, no dependencies.
 */
#include "tg_oracle.h"

#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static __thread char g_err[256];

static int fail(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return code;
}

const char *og_last_error(void) { return g_err; }

#define XMALLOC(p, n)                                                        \
    do {                                                                     \
        size_t _n = (size_t)(n) * sizeof(*(p));                              \
        (p) = malloc(_n ? _n : 1);                                           \
        if (!(p)) { rc = fail(OG_ERR_NOMEM, "out of memory"); goto done; }   \
    } while (0)

/* ---------------------------------------------------------------------- */
/* Canonicalisation                                                        */
/* ---------------------------------------------------------------------- */

/* The reference CPU face numbering picks low/mid/high by slot position
 * (cpu_extraction.cpp:151-153) and is only consistent on ascending rows, as
 * its own comment at :137 assumes; the reference mesh writer emits sorted
 * tets (make_mesh.py:56).  Both paths therefore sort every row first. */
int og_canonicalize(const int32_t *tv, int64_t n_cells, int64_t n_verts,
                    int32_t *out)
{
    if (n_cells < 0 || n_verts < 0 || (n_cells > 0 && (!tv || !out)))
        return fail(OG_ERR_ARG, "bad arguments");
    if (n_cells > 357913941LL || n_verts > 2147483647LL)
        return fail(OG_ERR_ARG, "mesh too large for 32-bit ids");
    for (int64_t c = 0; c < n_cells; c++) {
        int32_t w[4];
        for (int k = 0; k < 4; k++) {
            w[k] = tv[4 * c + k];
            if (w[k] < 0 || w[k] >= n_verts)
                return fail(OG_ERR_MESH, "cell %lld has vertex id %d outside [0,%lld)",
                            (long long)c, w[k], (long long)n_verts);
        }
        for (int i = 1; i < 4; i++) {
            int32_t x = w[i];
            int j = i - 1;
            while (j >= 0 && w[j] > x) { w[j + 1] = w[j]; j--; }
            w[j + 1] = x;
        }
        for (int k = 0; k < 3; k++)
            if (w[k] == w[k + 1])
                return fail(OG_ERR_MESH, "cell %lld repeats vertex %d",
                            (long long)c, w[k]);
        memcpy(out + 4 * c, w, sizeof w);
    }
    return OG_OK;
}

/* ---------------------------------------------------------------------- */
/* Helpers                                                                 */
/* ---------------------------------------------------------------------- */

static int cmp_i32(const void *a, const void *b)
{
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

static void sort_rows(int64_t *off, int32_t *ent, int64_t n_rows)
{
    for (int64_t r = 0; r < n_rows; r++) {
        int64_t n = off[r + 1] - off[r];
        if (n > 1) qsort(ent + off[r], (size_t)n, sizeof(int32_t), cmp_i32);
    }
}

/* Build CSR offsets from counts (exclusive scan). */
static void scan_counts(const int64_t *cnt, int64_t n, int64_t *off)
{
    off[0] = 0;
    for (int64_t i = 0; i < n; i++) off[i + 1] = off[i] + cnt[i];
}

/* TE pair order of the reference CPU path, cpu_extraction.cpp:37-39:
 * {0-1},{0-2},{0-3},{1-2},{1-3},{2-3}. */
static const int PJ[6] = {0, 0, 0, 1, 1, 2};
static const int PK[6] = {1, 2, 3, 2, 3, 3};

typedef struct {
    int64_t n;         /* number of edges */
    int32_t *head;     /* [V] first edge in the low vertex's list, -1 none */
    int32_t *next;     /* [E] */
    int32_t *lo, *hi;  /* [E] */
} edge_table;

typedef struct {
    int64_t n;
    int32_t *head;
    int32_t *next;
    int32_t *lo, *mid, *hi;
} face_table;

static int32_t find_edge(const edge_table *t, int32_t a, int32_t b)
{
    if (a > b) { int32_t s = a; a = b; b = s; }
    for (int32_t e = t->head[a]; e >= 0; e = t->next[e])
        if (t->hi[e] == b) return e;
    return -1;
}

/* Restates make_TE_and_VE, cpu_extraction.cpp:28-62: scan cells in order,
 * pairs in slot order, swap each pair to (low, high) (:44), search the low
 * vertex's table for the high vertex (:48-49); a miss mints the next edge id
 * (:50-53). */
static int number_edges(const int32_t *tvs, int64_t T, int64_t V,
                        int32_t *te, edge_table *t)
{
    int rc = OG_OK;
    memset(t, 0, sizeof *t);
    XMALLOC(t->head, V);
    XMALLOC(t->next, 6 * T);
    XMALLOC(t->lo, 6 * T);
    XMALLOC(t->hi, 6 * T);
    for (int64_t v = 0; v < V; v++) t->head[v] = -1;
    int32_t n = 0;
    for (int64_t c = 0; c < T; c++) {
        const int32_t *w = tvs + 4 * c;
        for (int j = 0; j < 6; j++) {
            int32_t a = w[PJ[j]], b = w[PK[j]];
            if (a > b) { int32_t s = a; a = b; b = s; }
            int32_t e;
            for (e = t->head[a]; e >= 0; e = t->next[e])
                if (t->hi[e] == b) break;
            if (e < 0) {
                e = n++;
                t->lo[e] = a;
                t->hi[e] = b;
                t->next[e] = t->head[a];
                t->head[a] = e;
            }
            if (te) te[6 * c + j] = e;
        }
    }
    t->n = n;
done:
    return rc;
}

/* Restates make_TF_and_VF, cpu_extraction.cpp:122-174: faces are visited with
 * skip_id = 3,2,1,0 (the decrementing loop at :145; the comment at :146-150
 * lists them in another order), low/mid/high picked by slot (:151-153), looked
 * up in the low vertex's table by (mid, high) (:155-160), new ids minted on a
 * miss (:161-168), and written to TF column 3-skip (:166,170). */
static int number_faces(const int32_t *tvs, int64_t T, int64_t V,
                        int32_t *tf, face_table *t)
{
    int rc = OG_OK;
    memset(t, 0, sizeof *t);
    XMALLOC(t->head, V);
    XMALLOC(t->next, 4 * T);
    XMALLOC(t->lo, 4 * T);
    XMALLOC(t->mid, 4 * T);
    XMALLOC(t->hi, 4 * T);
    for (int64_t v = 0; v < V; v++) t->head[v] = -1;
    int32_t n = 0;
    for (int64_t c = 0; c < T; c++) {
        const int32_t *w = tvs + 4 * c;
        for (int skip = 3; skip >= 0; skip--) {
            int lo = (skip > 0) ? 0 : 1;
            int mid = (skip > 1) ? 1 : 2;
            int hi = (skip == 3) ? 2 : 3;
            int32_t a = w[lo], b = w[mid], d = w[hi];
            int32_t f;
            for (f = t->head[a]; f >= 0; f = t->next[f])
                if (t->mid[f] == b && t->hi[f] == d) break;
            if (f < 0) {
                f = n++;
                t->lo[f] = a;
                t->mid[f] = b;
                t->hi[f] = d;
                t->next[f] = t->head[a];
                t->head[a] = f;
            }
            if (tf) tf[4 * c + 3 - skip] = f;
        }
    }
    t->n = n;
done:
    return rc;
}

static void free_edges(edge_table *t)
{
    free(t->head); free(t->next); free(t->lo); free(t->hi);
    memset(t, 0, sizeof *t);
}

static void free_faces(face_table *t)
{
    free(t->head); free(t->next); free(t->lo); free(t->mid); free(t->hi);
    memset(t, 0, sizeof *t);
}

static int alloc_fixed(og_rel *r, int64_t rows, int32_t width)
{
    r->n_rows = rows;
    r->width = width;
    r->n_entries = rows * width;
    r->off = NULL;
    r->ent = malloc((size_t)(r->n_entries ? r->n_entries : 1) * sizeof(int32_t));
    return r->ent ? OG_OK : fail(OG_ERR_NOMEM, "out of memory");
}

static int alloc_csr(og_rel *r, int64_t rows, const int64_t *cnt)
{
    r->n_rows = rows;
    r->width = 0;
    r->off = malloc((size_t)(rows + 1) * sizeof(int64_t));
    if (!r->off) return fail(OG_ERR_NOMEM, "out of memory");
    scan_counts(cnt, rows, r->off);
    r->n_entries = r->off[rows];
    r->ent = malloc((size_t)(r->n_entries ? r->n_entries : 1) * sizeof(int32_t));
    return r->ent ? OG_OK : fail(OG_ERR_NOMEM, "out of memory");
}

/* Restates elective_make_VT, cpu_extraction.cpp:291-342: every cell appends
 * itself to the row of each of its vertices, so rows come out ascending. */
static int build_vt(const int32_t *tvs, int64_t T, int64_t V, og_rel *r)
{
    int rc = OG_OK;
    int64_t *cnt = NULL;
    XMALLOC(cnt, V);
    memset(cnt, 0, (size_t)V * sizeof(int64_t));
    for (int64_t i = 0; i < 4 * T; i++) cnt[tvs[i]]++;
    if ((rc = alloc_csr(r, V, cnt))) goto done;
    for (int64_t v = 0; v < V; v++) cnt[v] = r->off[v];
    for (int64_t c = 0; c < T; c++)
        for (int k = 0; k < 4; k++) r->ent[cnt[tvs[4 * c + k]]++] = (int32_t)c;
done:
    free(cnt);
    return rc;
}

/* Restates elective_make_VV, cpu_extraction.cpp:259-289: for every cell and
 * every ordered pair of distinct slots, append the destination vertex to the
 * source vertex's list unless std::find already sees it (:271-277).  The
 * reference keeps first-encounter order; rows are sorted afterwards because
 * both paths are compared row-sorted. */
static int build_vv(const int32_t *tvs, int64_t T, int64_t V, og_rel *r)
{
    int rc = OG_OK;
    int64_t *cap = NULL, *len = NULL, *base = NULL;
    int32_t *buf = NULL;
    XMALLOC(cap, V);
    XMALLOC(len, V);
    XMALLOC(base, V + 1);
    memset(cap, 0, (size_t)V * sizeof(int64_t));
    for (int64_t i = 0; i < 4 * T; i++) cap[tvs[i]] += 3;  /* upper bound */
    scan_counts(cap, V, base);
    XMALLOC(buf, base[V]);
    memset(len, 0, (size_t)V * sizeof(int64_t));
    for (int64_t c = 0; c < T; c++) {
        const int32_t *w = tvs + 4 * c;
        for (int i = 0; i < 4; i++) {
            int32_t src = w[i];
            int32_t *row = buf + base[src];
            for (int j = 0; j < 4; j++) {
                if (i == j) continue;
                int32_t dst = w[j];
                int64_t k;
                for (k = 0; k < len[src]; k++)
                    if (row[k] == dst) break;
                if (k == len[src]) row[len[src]++] = dst;
            }
        }
    }
    if ((rc = alloc_csr(r, V, len))) goto done;
    for (int64_t v = 0; v < V; v++)
        memcpy(r->ent + r->off[v], buf + base[v], (size_t)len[v] * sizeof(int32_t));
    sort_rows(r->off, r->ent, V);
done:
    free(cap); free(len); free(base); free(buf);
    return rc;
}

/* ---------------------------------------------------------------------- */
/* Extraction                                                              */
/* ---------------------------------------------------------------------- */

#define BIT(x) (1u << (x))
enum { R_TE = 1, R_EV, R_ET, R_TF, R_FV, R_FE, R_FT, R_EF, R_VT, R_TT, R_FF,
       R_EE, R_VV };

int og_extract(const int32_t *tvs, int64_t T, int64_t V, uint32_t mask,
               uint32_t options, og_result *res)
{
    int rc = OG_OK;
    edge_table et = {0};
    face_table ft = {0};
    int32_t *te = NULL, *tf = NULL, *fe = NULL, *ftab = NULL;
    int64_t *cnt = NULL;
    og_rel vt = {0};
    int keep_vt = 0;

    if (!res || T < 0 || V < 0 || (T > 0 && !tvs))
        return fail(OG_ERR_ARG, "bad arguments");
    memset(res, 0, sizeof *res);
    res->n_verts = V;
    res->n_cells = T;
    for (int64_t c = 0; c < T; c++) {
        const int32_t *w = tvs + 4 * c;
        if (w[0] < 0 || w[3] >= V || !(w[0] < w[1] && w[1] < w[2] && w[2] < w[3]))
            return fail(OG_ERR_MESH, "cell %lld is not a sorted row of distinct ids in range",
                        (long long)c);
    }

    const uint32_t need_edges = BIT(R_TE) | BIT(R_EV) | BIT(R_ET) | BIT(R_FE) |
                                BIT(R_EF) | BIT(R_EE);
    const uint32_t need_faces = BIT(R_TF) | BIT(R_FV) | BIT(R_FE) | BIT(R_FT) |
                                BIT(R_EF) | BIT(R_FF) |
                                ((options & OG_OPT_TT_VERTEX_SHARING) ? 0 : BIT(R_TT));

    if (mask & need_edges) {
        XMALLOC(te, 6 * T);
        if ((rc = number_edges(tvs, T, V, te, &et))) goto done;
        res->n_edges = et.n;
    }
    if (mask & need_faces) {
        XMALLOC(tf, 4 * T);
        if ((rc = number_faces(tvs, T, V, tf, &ft))) goto done;
        res->n_faces = ft.n;
    }
    const int64_t E = res->n_edges, F = res->n_faces;

    /* FT: restated.  FT_Data is array<vtkIdType,2> (datatypes.h.in:143):
     * the ascending cells containing the face, -1 when the face is on the
     * boundary.  A face in more than two cells is not a tetrahedral mesh. */
    if ((mask & need_faces) &
        (BIT(R_FT) | BIT(R_FF) |
         ((options & OG_OPT_TT_VERTEX_SHARING) ? 0 : BIT(R_TT)))) {
        XMALLOC(ftab, 2 * F);
        for (int64_t i = 0; i < 2 * F; i++) ftab[i] = -1;
        for (int64_t c = 0; c < T; c++)
            for (int k = 0; k < 4; k++) {
                int32_t f = tf[4 * c + k];
                if (ftab[2 * f] < 0) ftab[2 * f] = (int32_t)c;
                else if (ftab[2 * f + 1] < 0) ftab[2 * f + 1] = (int32_t)c;
                else { rc = fail(OG_ERR_MESH, "face %d lies in more than two cells", f); goto done; }
            }
    }

    /* FE: restated.  FE_Data is three edges per face (datatypes.h.in:142);
     * for face (a<b<c) they are listed as (a,b), (a,c), (b,c). */
    if (mask & (BIT(R_FE) | BIT(R_EF))) {
        XMALLOC(fe, 3 * F);
        for (int64_t f = 0; f < F; f++) {
            int32_t a = ft.lo[f], b = ft.mid[f], c = ft.hi[f];
            fe[3 * f + 0] = find_edge(&et, a, b);
            fe[3 * f + 1] = find_edge(&et, a, c);
            fe[3 * f + 2] = find_edge(&et, b, c);
        }
    }

    if (mask & BIT(R_TE)) {
        og_rel *r = &res->rel[R_TE];
        if ((rc = alloc_fixed(r, T, 6))) goto done;
        memcpy(r->ent, te, (size_t)(6 * T) * sizeof(int32_t));
    }
    /* Restates elective_make_EV, cpu_extraction.cpp:95-107: EV[id] = {low,
     * high}. */
    if (mask & BIT(R_EV)) {
        og_rel *r = &res->rel[R_EV];
        if ((rc = alloc_fixed(r, E, 2))) goto done;
        for (int64_t e = 0; e < E; e++) {
            r->ent[2 * e] = et.lo[e];
            r->ent[2 * e + 1] = et.hi[e];
        }
    }
    /* Restates elective_make_ET, cpu_extraction.cpp:109-120: each cell
     * appends itself to the row of each of its 6 edges (ascending rows). */
    if (mask & BIT(R_ET)) {
        og_rel *r = &res->rel[R_ET];
        XMALLOC(cnt, E > V ? E : V);
        memset(cnt, 0, (size_t)E * sizeof(int64_t));
        for (int64_t i = 0; i < 6 * T; i++) cnt[te[i]]++;
        if ((rc = alloc_csr(r, E, cnt))) goto done;
        for (int64_t e = 0; e < E; e++) cnt[e] = r->off[e];
        for (int64_t c = 0; c < T; c++)
            for (int j = 0; j < 6; j++) r->ent[cnt[te[6 * c + j]]++] = (int32_t)c;
        free(cnt); cnt = NULL;
    }
    if (mask & BIT(R_TF)) {
        og_rel *r = &res->rel[R_TF];
        if ((rc = alloc_fixed(r, T, 4))) goto done;
        memcpy(r->ent, tf, (size_t)(4 * T) * sizeof(int32_t));
    }
    /* Restates elective_make_FV, cpu_extraction.cpp:225-243: FV[id] holds the
     * face's low, middle and high vertex. */
    if (mask & BIT(R_FV)) {
        og_rel *r = &res->rel[R_FV];
        if ((rc = alloc_fixed(r, F, 3))) goto done;
        for (int64_t f = 0; f < F; f++) {
            r->ent[3 * f] = ft.lo[f];
            r->ent[3 * f + 1] = ft.mid[f];
            r->ent[3 * f + 2] = ft.hi[f];
        }
    }
    if (mask & BIT(R_FE)) {
        og_rel *r = &res->rel[R_FE];
        if ((rc = alloc_fixed(r, F, 3))) goto done;
        memcpy(r->ent, fe, (size_t)(3 * F) * sizeof(int32_t));
    }
    if (mask & BIT(R_FT)) {
        og_rel *r = &res->rel[R_FT];
        if ((rc = alloc_fixed(r, F, 2))) goto done;
        memcpy(r->ent, ftab, (size_t)(2 * F) * sizeof(int32_t));
    }
    /* EF: restated from the driver's definition EF = (TV x VE)'
     * (test_driver.cu:311-314): the faces containing each edge, ascending. */
    if (mask & BIT(R_EF)) {
        og_rel *r = &res->rel[R_EF];
        XMALLOC(cnt, E);
        memset(cnt, 0, (size_t)E * sizeof(int64_t));
        for (int64_t i = 0; i < 3 * F; i++) cnt[fe[i]]++;
        if ((rc = alloc_csr(r, E, cnt))) goto done;
        for (int64_t e = 0; e < E; e++) cnt[e] = r->off[e];
        for (int64_t f = 0; f < F; f++)
            for (int k = 0; k < 3; k++) r->ent[cnt[fe[3 * f + k]]++] = (int32_t)f;
        free(cnt); cnt = NULL;
    }
    if (mask & (BIT(R_VT) | ((options & OG_OPT_TT_VERTEX_SHARING) ? BIT(R_TT) : 0))) {
        if ((rc = build_vt(tvs, T, V, &vt))) goto done;
        keep_vt = 1;
    }
    if (mask & BIT(R_VT)) {
        res->rel[R_VT] = vt;
        keep_vt = 0;
    }
    /* TT: restated from TT = TV x TV' (test_driver.cu:323-326).  Default:
     * cells sharing a face; with OG_OPT_TT_VERTEX_SHARING, cells sharing at
     * least one vertex (the literal product).  Self excluded, rows ascending. */
    if (mask & BIT(R_TT)) {
        og_rel *r = &res->rel[R_TT];
        XMALLOC(cnt, T);
        if (!(options & OG_OPT_TT_VERTEX_SHARING)) {
            for (int64_t c = 0; c < T; c++) {
                int64_t n = 0;
                for (int k = 0; k < 4; k++) {
                    int32_t f = tf[4 * c + k];
                    int32_t o = ftab[2 * f] == c ? ftab[2 * f + 1] : ftab[2 * f];
                    n += (o >= 0);
                }
                cnt[c] = n;
            }
            if ((rc = alloc_csr(r, T, cnt))) goto done;
            for (int64_t c = 0; c < T; c++) {
                int64_t p = r->off[c];
                for (int k = 0; k < 4; k++) {
                    int32_t f = tf[4 * c + k];
                    int32_t o = ftab[2 * f] == c ? ftab[2 * f + 1] : ftab[2 * f];
                    if (o >= 0) r->ent[p++] = o;
                }
            }
        } else {
            /* count with a stamp array, then fill */
            int32_t *stamp = NULL;
            XMALLOC(stamp, T);
            for (int64_t c = 0; c < T; c++) stamp[c] = -1;
            for (int pass = 0; pass < 2; pass++) {
                if (pass == 1) {
                    if ((rc = alloc_csr(r, T, cnt))) { free(stamp); goto done; }
                    for (int64_t c = 0; c < T; c++) stamp[c] = -1;
                }
                for (int64_t c = 0; c < T; c++) {
                    int64_t n = 0;
                    for (int k = 0; k < 4; k++) {
                        int32_t v = tvs[4 * c + k];
                        for (int64_t i = vt.off[v]; i < vt.off[v + 1]; i++) {
                            int32_t o = vt.ent[i];
                            if (o == c || stamp[o] == (int32_t)c) continue;
                            stamp[o] = (int32_t)c;
                            if (pass == 1) r->ent[r->off[c] + n] = o;
                            n++;
                        }
                    }
                    if (pass == 0) cnt[c] = n;
                }
            }
            free(stamp);
        }
        sort_rows(r->off, r->ent, T);
        free(cnt); cnt = NULL;
    }
    /* FF: restated from FF = TF' x TF (test_driver.cu:328-331): faces sharing
     * a cell with the face, self excluded, rows ascending. */
    if (mask & BIT(R_FF)) {
        og_rel *r = &res->rel[R_FF];
        XMALLOC(cnt, F);
        for (int64_t f = 0; f < F; f++)
            cnt[f] = 3 * ((ftab[2 * f] >= 0) + (ftab[2 * f + 1] >= 0));
        if ((rc = alloc_csr(r, F, cnt))) goto done;
        for (int64_t f = 0; f < F; f++) {
            int64_t p = r->off[f];
            for (int s = 0; s < 2; s++) {
                int32_t c = ftab[2 * f + s];
                if (c < 0) continue;
                for (int k = 0; k < 4; k++)
                    if (tf[4 * c + k] != f) r->ent[p++] = tf[4 * c + k];
            }
        }
        sort_rows(r->off, r->ent, F);
        free(cnt); cnt = NULL;
    }
    /* EE: restated from EE = EV' x VE (test_driver.cu:333-336): edges sharing
     * a vertex with the edge, self excluded, rows ascending. */
    if (mask & BIT(R_EE)) {
        og_rel *r = &res->rel[R_EE];
        og_rel inc = {0};
        XMALLOC(cnt, E > V ? E : V);
        memset(cnt, 0, (size_t)V * sizeof(int64_t));
        for (int64_t e = 0; e < E; e++) { cnt[et.lo[e]]++; cnt[et.hi[e]]++; }
        if ((rc = alloc_csr(&inc, V, cnt))) goto done;
        for (int64_t v = 0; v < V; v++) cnt[v] = inc.off[v];
        for (int64_t e = 0; e < E; e++) {
            inc.ent[cnt[et.lo[e]]++] = (int32_t)e;
            inc.ent[cnt[et.hi[e]]++] = (int32_t)e;
        }
        for (int64_t e = 0; e < E; e++)
            cnt[e] = (inc.off[et.lo[e] + 1] - inc.off[et.lo[e]]) +
                     (inc.off[et.hi[e] + 1] - inc.off[et.hi[e]]) - 2;
        if ((rc = alloc_csr(r, E, cnt))) { free(inc.off); free(inc.ent); goto done; }
        for (int64_t e = 0; e < E; e++) {
            /* merge two ascending rows, skipping e itself */
            const int32_t *A = inc.ent + inc.off[et.lo[e]], *B = inc.ent + inc.off[et.hi[e]];
            int64_t na = inc.off[et.lo[e] + 1] - inc.off[et.lo[e]];
            int64_t nb = inc.off[et.hi[e] + 1] - inc.off[et.hi[e]];
            int64_t i = 0, j = 0, p = r->off[e];
            while (i < na || j < nb) {
                int32_t x;
                if (j >= nb || (i < na && A[i] < B[j])) x = A[i++];
                else if (i >= na || B[j] < A[i]) x = B[j++];
                else { x = A[i++]; j++; }
                if (x != e) r->ent[p++] = x;
            }
            if (p != r->off[e + 1]) {
                free(inc.off); free(inc.ent);
                rc = fail(OG_ERR_MESH, "edge %lld: inconsistent incidence", (long long)e);
                goto done;
            }
        }
        free(inc.off); free(inc.ent);
        free(cnt); cnt = NULL;
    }
    if (mask & BIT(R_VV)) {
        if ((rc = build_vv(tvs, T, V, &res->rel[R_VV]))) goto done;
    }

done:
    free_edges(&et);
    free_faces(&ft);
    free(te); free(tf); free(fe); free(ftab); free(cnt);
    if (keep_vt) { free(vt.off); free(vt.ent); }
    if (rc) og_free(res);
    return rc;
}

void og_free(og_result *res)
{
    if (!res) return;
    for (int i = 0; i < 14; i++) {
        free(res->rel[i].off);
        free(res->rel[i].ent);
        res->rel[i].off = NULL;
        res->rel[i].ent = NULL;
    }
}

/* ---------------------------------------------------------------------- */
/* Critical points                                                         */
/* ---------------------------------------------------------------------- */

static int32_t uf_find(int32_t *parent, int32_t x)
{
    while (parent[x] != x) {
        parent[x] = parent[parent[x]];
        x = parent[x];
    }
    return x;
}

static int64_t lower_bound_i32(const int32_t *a, int64_t n, int32_t key)
{
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t m = (lo + hi) >> 1;
        if (a[m] < key) lo = m + 1; else hi = m;
    }
    return lo;
}

/* Restates the critPoints kernel, src/alg/critPoints.cu:49-331, on an exact
 * (duplicate-free) VV:
 *   - a neighbour u of v is "lower" (class -1) when s[u] < s[v], or when
 *     s[u] == s[v] and u < v; otherwise "upper" (+1) (:136-140);
 *   - two same-class neighbours u, w are joined when w is in VV[u], i.e. the
 *     mesh has edge (u,w) (:172-202), not only when the edge lies in v's star;
 *   - the kernel's min-label propagation (:170-266) leaves exactly one root
 *     per connected component; union-find counts the same components;
 *   - classes[3v + (class+1)/2] counts the roots of each class (:275-284), so
 *     slot 0 holds the lower components and slot 1 the upper ones;
 *   - the code (:303-330): slot0 >= 1 && slot1 == 0 -> 2; slot0 == 0 &&
 *     slot1 >= 1 -> 1; slot0 == 1 && slot1 == 1 -> 3; otherwise 4.  A vertex
 *     with only lower neighbours is a maximum, so 1 = minimum, 2 = maximum,
 *     3 = regular, 4 = saddle (including a vertex with no neighbours). */
static int crit_common(const int32_t *tvs, int64_t T, int64_t V,
                       const double *fd, const float *ff, uint32_t *classes3)
{
    int rc = OG_OK;
    og_rel vv = {0};
    int32_t *parent = NULL;
    int8_t *cls = NULL;
    if (!classes3 || (!fd && !ff)) return fail(OG_ERR_ARG, "bad arguments");
    if ((rc = build_vv(tvs, T, V, &vv))) return rc;
    int64_t maxdeg = 0;
    for (int64_t v = 0; v < V; v++)
        if (vv.off[v + 1] - vv.off[v] > maxdeg) maxdeg = vv.off[v + 1] - vv.off[v];
    XMALLOC(parent, maxdeg);
    XMALLOC(cls, maxdeg);
    for (int64_t v = 0; v < V; v++) {
        const int32_t *nb = vv.ent + vv.off[v];
        int64_t n = vv.off[v + 1] - vv.off[v];
        double sv = fd ? fd[v] : (double)ff[v];
        for (int64_t k = 0; k < n; k++) {
            int32_t u = nb[k];
            double su = fd ? fd[u] : (double)ff[u];
            int lower = (su == sv) ? (u < v) : (su < sv);
            cls[k] = lower ? -1 : 1;
            parent[k] = (int32_t)k;
        }
        for (int64_t k = 0; k < n; k++) {
            int32_t u = nb[k];
            const int32_t *row = vv.ent + vv.off[u];
            int64_t m = vv.off[u + 1] - vv.off[u];
            for (int64_t i = 0; i < m; i++) {
                int64_t j = lower_bound_i32(nb, n, row[i]);
                if (j < n && nb[j] == row[i] && cls[j] == cls[k]) {
                    int32_t a = uf_find(parent, (int32_t)k), b = uf_find(parent, (int32_t)j);
                    if (a != b) parent[a < b ? b : a] = a < b ? a : b;
                }
            }
        }
        uint32_t lo = 0, up = 0;
        for (int64_t k = 0; k < n; k++)
            if (uf_find(parent, (int32_t)k) == k) {
                if (cls[k] < 0) lo++; else up++;
            }
        uint32_t code;
        if (lo >= 1 && up == 0) code = 2;
        else if (lo == 0 && up >= 1) code = 1;
        else if (lo == 1 && up == 1) code = 3;
        else code = 4;
        classes3[3 * v] = lo;
        classes3[3 * v + 1] = up;
        classes3[3 * v + 2] = code;
    }
done:
    free(parent); free(cls);
    free(vv.off); free(vv.ent);
    return rc;
}

int og_critical_points(const int32_t *tvs, int64_t n_cells, int64_t n_verts,
                       const double *field, uint32_t *classes3)
{
    return crit_common(tvs, n_cells, n_verts, field, NULL, classes3);
}

int og_critical_points_f32(const int32_t *tvs, int64_t n_cells,
                           int64_t n_verts, const float *field,
                           uint32_t *classes3)
{
    return crit_common(tvs, n_cells, n_verts, NULL, field, classes3);
}
