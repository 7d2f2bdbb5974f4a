/*
 * tetragpu_compat.h -- the reference's C++ GPU entry points
 * (include/cuda_extraction.h of tlranda/TetraGPU, lines 10-138) with the same
 * names, signatures and return conventions, implemented in libtetragpu.so
 * over the C ABI of tetragpu.h.  A caller of the reference swaps its
 * cuda_extraction.h include for this header and links libtetragpu.so.
 *
 * Types: when the caller's own datatypes.h (the reference's, guard
 * TETRA_DATA_TYPES) is included first, its definitions are used.  Otherwise
 * this header declares layout-compatible restatements of the types the entry
 * points take (vtkIdType, EdgeData, FaceData, TV_Data, device_VV, device_VT,
 * the *_Data containers; include/datatypes.h.in:44-151).
 *
 * Behaviour, per entry point:
 *   - make_TV_for_GPU registers the mesh (the reference copied TV to a global
 *     and exit()ed on a second call; here a second call with the same TV
 *     reuses it, another TV replaces it).  Every function that takes a
 *     TV_Data registers it the same way.
 *   - make_VE_for_GPU / make_VF_for_GPU are accepted and do nothing: edge and
 *     face ids are minted on the GPU (identical to the reference CPU tables
 *     on row-sorted TV).  Functions that take only VE/VF (EV, FV, FE) use the
 *     registered mesh and check the counts they are given.
 *   - make_X_GPU_return returns a cudaMalloc'd device array of vtkIdType the
 *     caller must cudaFree (as before); make_X_GPU returns host containers.
 *     TE / TF columns follow the reference CPU column order.
 *   - make_VV_GPU_return returns the reference's padded device_VV (rows of
 *     max_VV_guess entries, -1 padding, row lengths in index); rows are exact
 *     and sorted, without the reference's duplicates.
 *   - free_transients releases the registered mesh after the call.
 *   - Errors print to stderr and return nullptr / empty containers (the
 *     reference exit()ed); tg_last_error_string() has the detail.
 * The relations the reference declared but never implemented on the GPU (ET,
 * FT, EF, TT, FF, EE) are added as make_X_GPU(const TV_Data &).
 */
#ifndef TETRAGPU_COMPAT_H
#define TETRAGPU_COMPAT_H

#include <array>
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "tetragpu.h"

#ifndef TETRA_DATA_TYPES
#define TETRA_DATA_TYPES
typedef long long vtkIdType;

const int nbVertsInCell = 4;
const int nbVertsInFace = 3;
const int nbVertsInEdge = 2;
const int nbEdgesInCell = 6;
const int nbEdgesInFace = 3;
const int nbFacesInCell = 4;

struct EdgeData {
    vtkIdType highVert = 0, id = 0;
    EdgeData(vtkIdType hv, vtkIdType i) : highVert{hv}, id{i} {}
    EdgeData() {}
};
struct FaceData {
    vtkIdType middleVert = 0, highVert = 0, id = 0;  // id: face id, or the low vertex in FV
    FaceData(vtkIdType mv, vtkIdType hv, vtkIdType i) : middleVert{mv}, highVert{hv}, id{i} {}
    FaceData() {}
    bool operator==(const FaceData &o) const
    {
        return id == o.id && middleVert == o.middleVert && highVert == o.highVert;
    }
};
struct TV_Data {
    vtkIdType nPoints, nCells;
    int n_partitions;
    vtkIdType *cells;
    double *vertexAttributes;
    int *partitionIDs, *n_per_partition, *partitionCells;
    TV_Data(vtkIdType points, vtkIdType cells_)
        : nPoints(points), nCells(cells_), n_partitions(1), cells(new vtkIdType[4 * cells_]),
          vertexAttributes(nullptr), partitionIDs(nullptr), n_per_partition(nullptr),
          partitionCells(nullptr)
    {
    }
    ~TV_Data()
    {
        delete[] cells;
        delete[] vertexAttributes;
        delete[] partitionIDs;
        delete[] n_per_partition;
        delete[] partitionCells;
    }
    TV_Data(const TV_Data &) = delete;
    TV_Data &operator=(const TV_Data &) = delete;
};
typedef struct deviceVV {
    vtkIdType *computed = nullptr;
    unsigned int *index = nullptr;
    deviceVV() {}
    deviceVV(vtkIdType *c, unsigned int *i) : computed(c), index(i) {}
} device_VV;
typedef struct deviceVT {
    vtkIdType *computed = nullptr;
    unsigned long long *index = nullptr;
    deviceVT() {}
    deviceVT(vtkIdType *c, unsigned long long *i) : computed(c), index(i) {}
} device_VT;

typedef std::vector<std::array<vtkIdType, nbEdgesInCell>> TE_Data;
typedef std::vector<std::vector<EdgeData>> VE_Data;
typedef std::vector<std::array<vtkIdType, nbFacesInCell>> TF_Data;
typedef std::vector<std::vector<FaceData>> VF_Data;
typedef std::vector<std::array<vtkIdType, nbVertsInEdge>> EV_Data;
typedef std::vector<std::vector<vtkIdType>> ET_Data;
typedef std::vector<FaceData> FV_Data;
typedef std::vector<std::array<EdgeData, nbEdgesInFace>> FE_Data;
typedef std::vector<std::array<vtkIdType, 2>> FT_Data;
typedef std::vector<std::vector<vtkIdType>> EF_Data;
typedef std::vector<std::vector<vtkIdType>> VT_Data;
typedef std::vector<std::vector<vtkIdType>> VV_Data;
typedef std::vector<std::vector<vtkIdType>> EE_Data;
typedef std::vector<std::vector<vtkIdType>> FF_Data;
typedef std::vector<std::vector<vtkIdType>> TT_Data;
#endif  // TETRA_DATA_TYPES

// marshalling (include/cuda_extraction.h:10-23)
void make_TV_for_GPU(const TV_Data &tv_relationship);
void make_VE_for_GPU(const VE_Data &ve_relationship, const vtkIdType n_edges,
                     const vtkIdType n_verts);
void make_VF_for_GPU(const VF_Data &vf_relationship, const vtkIdType n_verts,
                     const vtkIdType n_faces);

// relations (include/cuda_extraction.h:25-138)
vtkIdType *make_EV_GPU_return(const VE_Data &edgeTable, const vtkIdType n_points,
                              const vtkIdType n_edges, const bool free_transients);
std::unique_ptr<EV_Data> make_EV_GPU(const VE_Data &edgeTable, const vtkIdType n_points,
                                     const vtkIdType n_edges, const bool free_transients);
vtkIdType *make_TF_GPU_return(const TV_Data &TV, const VF_Data &VF, const vtkIdType n_points,
                              const vtkIdType n_faces, const vtkIdType n_cells,
                              const bool free_transients);
std::unique_ptr<TF_Data> make_TF_GPU(const TV_Data &TV, const VF_Data &VF,
                                     const vtkIdType n_points, const vtkIdType n_faces,
                                     const vtkIdType n_cells, const bool free_transients);
vtkIdType *make_TE_GPU_return(const TV_Data &TV, const VE_Data &VE, const vtkIdType n_points,
                              const vtkIdType n_edges, const vtkIdType n_cells,
                              const bool free_transients);
std::unique_ptr<TE_Data> make_TE_GPU(const TV_Data &TV, const VE_Data &VE,
                                     const vtkIdType n_points, const vtkIdType n_edges,
                                     const vtkIdType n_cells, const bool free_transients);
vtkIdType *make_FV_GPU_return(const VF_Data &VF, const vtkIdType n_points,
                              const vtkIdType n_faces, const bool free_transients);
std::unique_ptr<FV_Data> make_FV_GPU(const VF_Data &VF, const vtkIdType n_points,
                                     const vtkIdType n_faces, const bool free_transients);
vtkIdType *make_FE_GPU_return(const VF_Data &VF, const VE_Data &VE, const vtkIdType n_points,
                              const vtkIdType n_edges, const vtkIdType n_faces,
                              const bool free_transients);
std::unique_ptr<FE_Data> make_FE_GPU(const VF_Data &VF, const VE_Data &VE,
                                     const vtkIdType n_points, const vtkIdType n_edges,
                                     const vtkIdType n_faces, const bool free_transients);
int get_approx_max_VV(const TV_Data &TV, const vtkIdType n_points, const int debug);
device_VV *make_VV_GPU_return(const TV_Data &TV, const int n_cells, const int n_points,
                              const int max_VV_guess, const bool free_transients);
std::unique_ptr<VV_Data> make_VV_GPU(const TV_Data &TV, const int n_cells, const int n_points,
                                     const bool free_transients);
device_VT *make_VT_GPU_return(const TV_Data &TV);
device_VT *make_VT_GPU_return(const VT_Data &VT);

// relations the reference declared but did not implement on the GPU
std::unique_ptr<ET_Data> make_ET_GPU(const TV_Data &TV);
std::unique_ptr<FT_Data> make_FT_GPU(const TV_Data &TV);
std::unique_ptr<EF_Data> make_EF_GPU(const TV_Data &TV);
std::unique_ptr<TT_Data> make_TT_GPU(const TV_Data &TV);
std::unique_ptr<FF_Data> make_FF_GPU(const TV_Data &TV);
std::unique_ptr<EE_Data> make_EE_GPU(const TV_Data &TV);

// the registered mesh (nullptr if none), e.g. for tg_critical_points
tg_mesh *tetragpu_compat_mesh(void);
// release the registered mesh
void tetragpu_compat_release(void);

#endif
