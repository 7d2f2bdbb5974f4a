// tg_vtk_classify.cpp -- the reference's VTK loader, unchanged, feeding the C
// ABI: read a .vtu with get_TV_from_VTK (src/vtk_load.cu:46-298 of
// tlranda/TetraGPU, compiled from the reference tree as it is), build the mesh
// on one GPU from its int64 TV (tg_mesh_create_i64: ids narrowed to int32 with
// range checks, rows sorted on the device), extract the relations the flags
// ask for, classify the vertex attribute it loaded and print the reference's
// class report (export_classes' wording, src/alg/critPoints.cu:340-453).  The
// single-GPU path of the reference's critPoints driver
// (src/alg/critPoints.cu:1359-1514) without its partitioning.
//
// Built only where VTK is installed: `make -C tetragpu_gb300/vtk` with
// TG_REFERENCE_ROOT (the reference tree) and VTK_PREFIX set (see the
// Makefile).  Without TG_WITH_VTK this file compiles to nothing.
#ifdef TG_WITH_VTK
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <vector>

#include "argparse.h"   // the reference's runtime_arguments and parse()
#include "tetragpu.h"
#include "vtk_load.h"   // get_TV_from_VTK, unchanged

static int check(tg_status st, const char *what)
{
    if (st == TG_OK) return 0;
    std::fprintf(stderr, "tetragpu: %s: %s\n", what, tg_last_error_string());
    return 1;
}

int main(int argc, char **argv)
{
    runtime_arguments args;
    parse(argc, argv, args);   // the reference's CLI: -i file.vtu, -a array, -e export, flags
    std::shared_ptr<TV_Data> tv = get_TV_from_VTK(args);
    if (!tv) return 1;
    tg_mesh *mesh = nullptr;
    if (check(tg_mesh_create_i64(reinterpret_cast<const int64_t *>(tv->cells), tv->nCells,
                                 tv->nPoints, nullptr, &mesh),
              "mesh"))
        return 1;
    // the relation flags the reference's --build_XX options set (bit 0 is
    // validation, which this path leaves to the test suite)
    const uint32_t mask = (uint32_t)args.arg_flags.to_ulong() & TG_ALL_RELATIONS;
    int rc = 0;
    if (mask) rc |= check(tg_extract(mesh, mask, 0, nullptr), "extract");
    if (!rc && tv->vertexAttributes) {
        std::vector<uint32_t> classes((size_t)tv->nPoints * 3);
        rc |= check(tg_critical_points(mesh, tv->vertexAttributes, TG_FIELD_F64, 0, classes.data(),
                                       0, nullptr),
                    "critical points");
        if (!rc)
            rc |= check(tg_export_classes(classes.data(), tv->nPoints,
                                          args.export_.empty() ? nullptr : args.export_.c_str(),
                                          0, nullptr),
                        "class report");
    }
    tg_mesh_destroy(mesh);
    return rc;
}
#endif
