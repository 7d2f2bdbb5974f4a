/*
 * tg_oracle.h -- CPU restatement of TetraGPU's relation-extraction and
 * critical-point path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path in
 * tetragpu_gb300/csrc.  Only tests/, __graft_entry__.smoke() and the CPU
 * baseline legs of bench.py may load it.  The product never calls it and has
 * no CPU fallback.
 *
 * Pinning: the seven relations that have reference CPU code (TE, EV, ET, TF,
 * FV, VV, VT) are checked against the reference's own cpu_extraction.cpp,
 * compiled unmodified from its source tree by oracle/build_ref.sh (see
 * tests/test_oracle_pin.py), and against golden digests generated from that
 * build (tests/golden/).  FE, FT, EF, TT, FF, EE and critical points have no
 * reference CPU code; they are restated here from the reference's definitions
 * and from its GPU kernel, and cross-checked against a literal simulation of
 * the reference critPoints kernel (tests/test_oracle_crit.py).
 *
 * Conventions (shared with the CUDA path):
 *   - TV is int32 [n_cells x 4].  og_canonicalize sorts each row ascending;
 *     every other entry point expects sorted rows (the reference CPU face
 *     numbering is only consistent on sorted rows: cpu_extraction.cpp:136-153).
 *   - Relation indices and mask bits are the reference arg_flags bit
 *     positions (include/datatypes.h.in:164-197): 1 TE, 2 EV, 3 ET, 4 TF,
 *     5 FV, 6 FE, 7 FT, 8 EF, 9 VT, 10 TT, 11 FF, 12 EE, 13 VV.
 *   - Fixed-width relations (TE 6, EV 2, TF 4, FV 3, FE 3, FT 2) are dense
 *     row-major int32; FT pads a boundary face's missing cell with -1.
 *   - Variable-width relations (ET, EF, VT, TT, FF, EE, VV) are CSR with int64
 *     offsets [n_rows + 1] and int32 entries, every row sorted ascending.
 */
#ifndef TG_ORACLE_H
#define TG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    OG_OK = 0,
    OG_ERR_ARG = 1,
    OG_ERR_MESH = 2,
    OG_ERR_NOMEM = 4
};

/* extraction options */
#define OG_OPT_TT_VERTEX_SHARING 0x1u  /* TT = cells sharing >= 1 vertex */

typedef struct {
    int64_t n_rows;
    int64_t n_entries;
    int32_t width;     /* > 0: fixed width, off == NULL; 0: CSR */
    int64_t *off;
    int32_t *ent;
} og_rel;

typedef struct {
    int64_t n_verts, n_edges, n_faces, n_cells;
    og_rel rel[14];    /* index = relation bit position */
} og_result;

/* Sort each tet's 4 vertex slots ascending and validate ids (in range,
 * distinct within a tet).  out may alias tv. */
int og_canonicalize(const int32_t *tv, int64_t n_cells, int64_t n_verts,
                    int32_t *out);

/* Build every relation whose bit is set in mask from row-sorted TV. */
int og_extract(const int32_t *tvs, int64_t n_cells, int64_t n_verts,
               uint32_t mask, uint32_t options, og_result *res);
void og_free(og_result *res);

/* Critical-point classes in the reference layout: classes3[3v+0] = number of
 * components among neighbours below v, [3v+1] = among neighbours above v,
 * [3v+2] = class code (1 minimum, 2 maximum, 3 regular, 4 saddle). */
int og_critical_points(const int32_t *tvs, int64_t n_cells, int64_t n_verts,
                       const double *field, uint32_t *classes3);
int og_critical_points_f32(const int32_t *tvs, int64_t n_cells,
                           int64_t n_verts, const float *field,
                           uint32_t *classes3);

const char *og_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
