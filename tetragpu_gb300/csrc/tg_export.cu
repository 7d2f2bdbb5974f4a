// tg_export.cu -- the critical-point class report of the reference
// (export_classes, src/alg/critPoints.cu:340-453), host code.
//
// The report keeps the reference's wording and numbers exactly, including its
// swapped labels: the line "Total number of minima" counts code 2 vertices
// (MINIMUM_CLASS, which the kernel assigns to true maxima) and "maxima" code
// 1.  The optional per-vertex lines "A <vertex> <code>" are the short form
// the reference's verifier script reads (it skips lines starting "Total").
#include <cstdint>
#include <cstdio>

#include "tetragpu.h"
#include "tg_internal.h"

extern "C" tg_status tg_export_classes(const uint32_t *classes, int64_t n_verts, const char *path,
                                       int per_vertex_lines, int64_t *counts_out)
{
    if ((n_verts > 0 && !classes) || n_verts < 0) {
        tg::set_last_error("bad classes or vertex count");
        return TG_ERR_INVALID_ARGUMENT;
    }
    // codes as the reference names them (critPoints.cu:18-21)
    const unsigned kMax = 1, kMin = 2, kRegular = 3, kSaddle = 4;
    int64_t n[5] = {0, 0, 0, 0, 0}, insane = 0;
    FILE *f = path ? fopen(path, "w") : stdout;
    if (!f) {
        tg::set_last_error("cannot open the export file");
        return TG_ERR_INVALID_ARGUMENT;
    }
    for (int64_t i = 0; i < n_verts; i++) {
        // slot 0 holds what the reference calls the upper count (F7)
        const unsigned up = classes[3 * i], lo = classes[3 * i + 1], c = classes[3 * i + 2];
        if ((up >= 1 && lo == 0 && c != kMin) || (up == 0 && lo >= 1 && c != kMax) ||
            (up == 1 && lo == 1 && c != kRegular) || (up > 1 && lo > 1 && c != kSaddle))
            insane++;
        if (c <= 4) n[c]++;
        if (per_vertex_lines && c > 0) fprintf(f, "A %lld %u\n", (long long)i, c);
    }
    if (insane > 0)
        fprintf(stderr, "Insanity detected; GPU did not agree on its own answers for %lld points.\n",
                (long long)insane);
    fprintf(f, "Total number of minima:  %lld\n", (long long)n[kMin]);
    fprintf(f, "Total number of maxima:  %lld\n", (long long)n[kMax]);
    fprintf(f, "Total number of saddles: %lld\n", (long long)n[kSaddle]);
    fprintf(f, "Total number of regular: %lld\n", (long long)n[kRegular]);
    fprintf(f, "Total number of voids:   %lld\n", (long long)n[0]);
    if (path) fclose(f); else fflush(f);
    if (counts_out)
        for (int k = 0; k < 5; k++) counts_out[k] = n[k];
    return TG_OK;
}
