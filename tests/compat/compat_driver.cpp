// A caller of the reference's cuda_extraction.h entry points, following the
// per-relation flow of the reference's src/alg/test_driver.cu (TV in, ids from
// the CPU tables, one make_X_GPU per relation, compare against the CPU), built
// against tetragpu_compat.h and libtetragpu.so.  The CPU answers come from the
// oracle (oracle/tg_oracle.h).  Usage: compat_driver mesh.bin
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "tetragpu_compat.h"
#include "tg_oracle.h"

static int failures = 0;
#define EXPECT(cond, what)                                  \
    do {                                                    \
        if (!(cond)) {                                      \
            fprintf(stderr, "MISMATCH %s\n", what);         \
            failures++;                                     \
        } else {                                            \
            printf("ok %s\n", what);                        \
        }                                                   \
    } while (0)

static std::vector<std::vector<vtkIdType>> rows_of(const og_rel &r)
{
    std::vector<std::vector<vtkIdType>> out((size_t)r.n_rows);
    for (int64_t i = 0; i < r.n_rows; i++) out[i].assign(r.ent + r.off[i], r.ent + r.off[i + 1]);
    return out;
}

int main(int argc, char **argv)
{
    if (argc < 2) return 2;
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 2;
    int64_t T, V;
    if (fread(&T, 8, 1, f) != 1 || fread(&V, 8, 1, f) != 1) return 2;
    std::vector<int32_t> tv32((size_t)(4 * T));
    if (fread(tv32.data(), 4, tv32.size(), f) != tv32.size()) return 2;
    fclose(f);

    // reference side: TV_Data with vtkIdType cells, slots as loaded
    TV_Data tv(V, T);
    for (size_t i = 0; i < tv32.size(); i++) tv.cells[i] = tv32[i];

    // CPU answers (row-sorted TV, like the reference CPU path expects)
    std::vector<int32_t> tvs(tv32.size());
    if (og_canonicalize(tv32.data(), T, V, tvs.data()) != 0) return 3;
    og_result ref;
    if (og_extract(tvs.data(), T, V, 0x3FFEu, 0, &ref) != 0) return 3;
    const int64_t E = ref.n_edges, F = ref.n_faces;

    // the CPU tables the reference passes along (VE, VF): from EV and FV
    VE_Data ve((size_t)V);
    for (int64_t e = 0; e < E; e++)
        ve[ref.rel[2].ent[2 * e]].push_back(EdgeData(ref.rel[2].ent[2 * e + 1], e));
    VF_Data vf((size_t)V);
    for (int64_t g = 0; g < F; g++)
        vf[ref.rel[5].ent[3 * g]].push_back(
            FaceData(ref.rel[5].ent[3 * g + 1], ref.rel[5].ent[3 * g + 2], g));

    make_TV_for_GPU(tv);
    make_VE_for_GPU(ve, E, V);
    make_VF_for_GPU(vf, V, F);

    auto te = make_TE_GPU(tv, ve, V, E, T, false);
    bool ok = (int64_t)te->size() == T;
    for (int64_t c = 0; ok && c < T; c++)
        for (int k = 0; k < 6; k++) ok &= (*te)[c][k] == ref.rel[1].ent[6 * c + k];
    EXPECT(ok, "TE");

    auto ev = make_EV_GPU(ve, V, E, false);
    ok = (int64_t)ev->size() == E;
    for (int64_t e = 0; ok && e < E; e++)
        ok &= (*ev)[e][0] == ref.rel[2].ent[2 * e] && (*ev)[e][1] == ref.rel[2].ent[2 * e + 1];
    EXPECT(ok, "EV");

    auto tf = make_TF_GPU(tv, vf, V, F, T, false);
    ok = (int64_t)tf->size() == T;
    for (int64_t c = 0; ok && c < T; c++)
        for (int k = 0; k < 4; k++) ok &= (*tf)[c][k] == ref.rel[4].ent[4 * c + k];
    EXPECT(ok, "TF");

    auto fv = make_FV_GPU(vf, V, F, false);
    ok = (int64_t)fv->size() == F;
    for (int64_t g = 0; ok && g < F; g++)
        ok &= (*fv)[g].middleVert == ref.rel[5].ent[3 * g] &&
              (*fv)[g].highVert == ref.rel[5].ent[3 * g + 1] &&
              (*fv)[g].id == ref.rel[5].ent[3 * g + 2];
    EXPECT(ok, "FV");

    auto fe = make_FE_GPU(vf, ve, V, E, F, false);
    ok = (int64_t)fe->size() == F;
    for (int64_t g = 0; ok && g < F; g++)
        for (int k = 0; k < 3; k++) ok &= (*fe)[g][k].id == ref.rel[6].ent[3 * g + k];
    EXPECT(ok, "FE");

    // device arrays the caller frees, as with the reference
    vtkIdType *dte = make_TE_GPU_return(tv, ve, V, E, T, false);
    std::vector<vtkIdType> hte((size_t)(6 * T));
    cudaMemcpy(hte.data(), dte, hte.size() * 8, cudaMemcpyDeviceToHost);
    cudaFree(dte);
    ok = true;
    for (size_t i = 0; i < hte.size(); i++) ok &= hte[i] == ref.rel[1].ent[i];
    EXPECT(ok, "TE device (vtkIdType)");

    EXPECT(*make_VV_GPU(tv, (int)T, (int)V, false) == rows_of(ref.rel[13]), "VV");
    const int width = get_approx_max_VV(tv, V, 0);
    device_VV *dvv = make_VV_GPU_return(tv, (int)T, (int)V, width, false);
    std::vector<vtkIdType> pad((size_t)V * width);
    std::vector<unsigned> idx((size_t)V);
    cudaMemcpy(pad.data(), dvv->computed, pad.size() * 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(idx.data(), dvv->index, idx.size() * 4, cudaMemcpyDeviceToHost);
    cudaFree(dvv->computed);
    cudaFree(dvv->index);
    delete dvv;
    auto vv = rows_of(ref.rel[13]);
    ok = true;
    for (int64_t v = 0; v < V; v++) {
        ok &= idx[v] == vv[v].size();
        for (int k = 0; k < width; k++)
            ok &= pad[(size_t)v * width + k] == (k < (int)vv[v].size() ? vv[v][k] : -1);
    }
    EXPECT(ok, "VV padded device_VV");

    device_VT *dvt = make_VT_GPU_return(tv);
    std::vector<vtkIdType> hvt((size_t)(4 * T));
    cudaMemcpy(hvt.data(), dvt->computed, hvt.size() * 8, cudaMemcpyDeviceToHost);
    cudaFree(dvt->computed);
    cudaFree(dvt->index);
    delete dvt;
    ok = true;
    for (size_t i = 0; i < hvt.size(); i++) ok &= hvt[i] == ref.rel[9].ent[i];
    EXPECT(ok, "VT device");

    EXPECT(*make_ET_GPU(tv) == rows_of(ref.rel[3]), "ET");
    EXPECT(*make_EF_GPU(tv) == rows_of(ref.rel[8]), "EF");
    EXPECT(*make_TT_GPU(tv) == rows_of(ref.rel[10]), "TT");
    EXPECT(*make_FF_GPU(tv) == rows_of(ref.rel[11]), "FF");
    EXPECT(*make_EE_GPU(tv) == rows_of(ref.rel[12]), "EE");
    auto ft = make_FT_GPU(tv);
    ok = (int64_t)ft->size() == F;
    for (int64_t g = 0; ok && g < F; g++)
        ok &= (*ft)[g][0] == ref.rel[7].ent[2 * g] && (*ft)[g][1] == ref.rel[7].ent[2 * g + 1];
    EXPECT(ok, "FT");

    tetragpu_compat_release();
    og_free(&ref);
    printf(failures ? "compat FAILED\n" : "compat OK\n");
    return failures ? 1 : 0;
}
