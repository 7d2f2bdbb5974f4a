/*
 * ref_driver.cpp -- a C entry point around the reference's own CPU relation
 * code (src/cpu_extraction.cpp, src/validate.cpp of tlranda/TetraGPU),
 * compiled unmodified from the reference source tree by oracle/build_ref.sh
 * into oracle/_ref/libtgref.so.  TEST INFRASTRUCTURE ONLY: it pins the CPU
 * restatement in tg_oracle.c and generates golden digests.  It is only built
 * where the reference source tree exists; nothing in the product links it.
 *
 * The driver follows the reference's own per-relation flow
 * (src/alg/test_driver.cu:70-77, 193-205, 357-372): make_TE_and_VE and
 * make_TF_and_VF mint the ids, elective_make_{EV,ET,FV,VV,VT} derive the
 * rest, and results are returned as flat arrays (VV in the reference's
 * first-encounter order; the comparison sorts rows).
 */
#include <chrono>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <sstream>
#include <vector>

#include "cpu_extraction.h"
#include "validate.h"

struct ref_result {
    int64_t n_edges, n_faces;
    int32_t *te, *tf, *ev, *fv;            /* fixed width */
    int64_t *et_off, *vt_off, *vv_off;     /* CSR, n_rows + 1 */
    int32_t *et, *vt, *vv;
    double seconds;                        /* the reference functions alone (steady_clock) */
};

static int32_t *alloc_i32(size_t n) { return (int32_t *)malloc((n ? n : 1) * sizeof(int32_t)); }
static int64_t *alloc_i64(size_t n) { return (int64_t *)malloc((n ? n : 1) * sizeof(int64_t)); }

template <class Rows>
static void flatten(const Rows &rows, int64_t **off, int32_t **ent)
{
    size_t n = 0;
    for (const auto &r : rows) n += r.size();
    *off = alloc_i64(rows.size() + 1);
    *ent = alloc_i32(n);
    size_t p = 0, i = 0;
    (*off)[0] = 0;
    for (const auto &r : rows) {
        for (auto x : r) (*ent)[p++] = (int32_t)x;
        (*off)[++i] = (int64_t)p;
    }
}

extern "C" {

/* Run the reference CPU path on a row-sorted int32 TV. */
int ref_extract(const int32_t *tvs, int64_t n_cells, int64_t n_verts, ref_result *out)
{
    std::memset(out, 0, sizeof *out);
    TV_Data tv(n_verts, n_cells);
    for (int64_t i = 0; i < 4 * n_cells; i++) tv.cells[i] = tvs[i];

    // cout noise from the reference is silenced for the duration
    std::streambuf *saved_out = std::cout.rdbuf(), *saved_err = std::cerr.rdbuf();
    std::ostringstream sink;
    std::cout.rdbuf(sink.rdbuf());
    std::cerr.rdbuf(sink.rdbuf());

    const auto t0 = std::chrono::steady_clock::now();
    TE_Data te(n_cells);
    VE_Data ve(n_verts);
    vtkIdType n_edges = make_TE_and_VE(tv, te, ve);
    TF_Data tf(n_cells);
    VF_Data vf(n_verts);
    vtkIdType n_faces = make_TF_and_VF(tv, tf, vf);
    std::unique_ptr<EV_Data> ev = elective_make_EV(ve, n_verts, n_edges);
    std::unique_ptr<ET_Data> et = elective_make_ET(te, n_edges);
    std::unique_ptr<FV_Data> fv = elective_make_FV(vf, n_faces);
    std::unique_ptr<VV_Data> vv = elective_make_VV(tv, n_verts);
    std::unique_ptr<VT_Data> vt = elective_make_VT(tv);
    out->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

    std::cout.rdbuf(saved_out);
    std::cerr.rdbuf(saved_err);

    out->n_edges = n_edges;
    out->n_faces = n_faces;
    out->te = alloc_i32(6 * (size_t)n_cells);
    out->tf = alloc_i32(4 * (size_t)n_cells);
    for (int64_t c = 0; c < n_cells; c++) {
        for (int j = 0; j < 6; j++) out->te[6 * c + j] = (int32_t)te[c][j];
        for (int j = 0; j < 4; j++) out->tf[4 * c + j] = (int32_t)tf[c][j];
    }
    out->ev = alloc_i32(2 * (size_t)n_edges);
    for (int64_t e = 0; e < n_edges; e++) {
        out->ev[2 * e] = (int32_t)(*ev)[e][0];
        out->ev[2 * e + 1] = (int32_t)(*ev)[e][1];
    }
    /* FaceData for FV holds {middleVert, highVert, id = low vertex}
       (cpu_extraction.cpp:236-238); flattened here as (low, middle, high). */
    out->fv = alloc_i32(3 * (size_t)n_faces);
    for (int64_t f = 0; f < n_faces; f++) {
        out->fv[3 * f] = (int32_t)(*fv)[f].id;
        out->fv[3 * f + 1] = (int32_t)(*fv)[f].middleVert;
        out->fv[3 * f + 2] = (int32_t)(*fv)[f].highVert;
    }
    flatten(*et, &out->et_off, &out->et);
    flatten(*vt, &out->vt_off, &out->vt);
    flatten(*vv, &out->vv_off, &out->vv);
    return 0;
}

void ref_free(ref_result *r)
{
    free(r->te); free(r->tf); free(r->ev); free(r->fv);
    free(r->et_off); free(r->vt_off); free(r->vv_off);
    free(r->et); free(r->vt); free(r->vv);
    std::memset(r, 0, sizeof *r);
}

/* Run the reference validators (validate.cpp) on a candidate result against
 * the reference's own CPU result for the same mesh.  Returns a bitmask of
 * relations that FAILED (bit = arg_flags position): TE 1, EV 2, TF 4, FV 5,
 * VV 13.  These comparators are O(N^2); call them on small meshes only. */
uint32_t ref_validate(const int32_t *tvs, int64_t n_cells, int64_t n_verts,
                      const int32_t *te, const int32_t *tf, const int32_t *ev,
                      int64_t n_edges, const int32_t *fv, int64_t n_faces,
                      const int64_t *vv_off, const int32_t *vv)
{
    TV_Data tv(n_verts, n_cells);
    for (int64_t i = 0; i < 4 * n_cells; i++) tv.cells[i] = tvs[i];
    std::streambuf *saved_out = std::cout.rdbuf(), *saved_err = std::cerr.rdbuf();
    std::ostringstream sink;
    std::cout.rdbuf(sink.rdbuf());
    std::cerr.rdbuf(sink.rdbuf());

    TE_Data hte(n_cells);
    VE_Data ve(n_verts);
    vtkIdType ne = make_TE_and_VE(tv, hte, ve);
    TF_Data htf(n_cells);
    VF_Data vf(n_verts);
    vtkIdType nf = make_TF_and_VF(tv, htf, vf);
    std::unique_ptr<EV_Data> hev = elective_make_EV(ve, n_verts, ne);
    std::unique_ptr<FV_Data> hfv = elective_make_FV(vf, nf);
    std::unique_ptr<VV_Data> hvv = elective_make_VV(tv, n_verts);

    TE_Data dte(n_cells);
    TF_Data dtf(n_cells);
    for (int64_t c = 0; c < n_cells; c++) {
        for (int j = 0; j < 6; j++) dte[c][j] = te[6 * c + j];
        for (int j = 0; j < 4; j++) dtf[c][j] = tf[4 * c + j];
    }
    EV_Data dev(n_edges);
    for (int64_t e = 0; e < n_edges; e++) dev[e] = {ev[2 * e], ev[2 * e + 1]};
    FV_Data dfv(n_faces);
    for (int64_t f = 0; f < n_faces; f++)
        dfv[f] = FaceData(fv[3 * f + 1], fv[3 * f + 2], fv[3 * f]);
    VV_Data dvv(n_verts);
    for (int64_t v = 0; v < n_verts; v++)
        for (int64_t i = vv_off[v]; i < vv_off[v + 1]; i++) dvv[v].push_back(vv[i]);

    uint32_t failed = 0;
    if (!check_host_vs_device_TE(hte, dte)) failed |= 1u << 1;
    if (!check_host_vs_device_EV(*hev, dev)) failed |= 1u << 2;
    if (!check_host_vs_device_TF(htf, dtf)) failed |= 1u << 4;
    if (!check_host_vs_device_FV(*hfv, dfv)) failed |= 1u << 5;
    if (!check_host_vs_device_VV(*hvv, dvv)) failed |= 1u << 13;
    /* the reference VV comparator tolerates extra entries; demand equal sizes */
    for (int64_t v = 0; v < n_verts; v++)
        if ((*hvv)[v].size() != dvv[v].size()) failed |= 1u << 13;

    std::cout.rdbuf(saved_out);
    std::cerr.rdbuf(saved_err);
    return failed;
}

}  // extern "C"
