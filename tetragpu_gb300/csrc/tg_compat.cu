// tg_compat.cu -- the reference's cuda_extraction.h entry points over the C
// ABI (declarations and behaviour in include/tetragpu_compat.h).  Host code
// only: every relation comes from tg_extract on the GPU; this file marshals
// between the reference's containers and the library's CSR buffers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <mutex>

#include "tetragpu_compat.h"

static_assert(sizeof(vtkIdType) == sizeof(int64_t), "vtkIdType is 64-bit");

namespace {

std::mutex g_mu;
tg_mesh *g_mesh = nullptr;       // the registered mesh
const vtkIdType *g_cells = nullptr;
vtkIdType g_ncells = -1, g_npoints = -1;

void report(const char *where)
{
    fprintf(stderr, "tetragpu: %s: %s\n", where, tg_last_error_string());
}

void release_locked()
{
    if (g_mesh) tg_mesh_destroy(g_mesh);
    g_mesh = nullptr;
    g_cells = nullptr;
    g_ncells = g_npoints = -1;
}

// Register TV (narrowed to int32) unless it is the registered mesh already.
tg_mesh *register_tv(const TV_Data &tv)
{
    if (g_mesh && g_cells == tv.cells && g_ncells == tv.nCells && g_npoints == tv.nPoints)
        return g_mesh;
    release_locked();
    // the library's TV is int32: ids that do not narrow are refused (the
    // reference's vtkIdType is 64-bit)
    tg_mesh *m = nullptr;
    if (tg_mesh_create_i64(reinterpret_cast<const int64_t *>(tv.cells), tv.nCells, tv.nPoints,
                           nullptr, &m) != TG_OK) {
        report("mesh");
        return nullptr;
    }
    g_mesh = m;
    g_cells = tv.cells;
    g_ncells = tv.nCells;
    g_npoints = tv.nPoints;
    return m;
}

bool extract(tg_mesh *m, uint32_t mask)
{
    if (!m) return false;
    if (tg_extract(m, mask, 0, nullptr) != TG_OK) {
        report("extract");
        return false;
    }
    return true;
}

bool check_count(tg_mesh *m, int which, vtkIdType expected, const char *what)
{
    int64_t v, e, f, c;
    tg_mesh_counts(m, &v, &e, &f, &c);
    const int64_t got = which == 0 ? e : f;
    if (expected >= 0 && got != expected) {
        fprintf(stderr, "tetragpu: %s: the mesh has %lld, the caller passed %lld "
                        "(ids follow the reference CPU numbering on row-sorted TV)\n",
                what, (long long)got, (long long)expected);
        return false;
    }
    return true;
}

// a relation as a cudaMalloc'd vtkIdType array the caller frees
vtkIdType *device_i64(tg_mesh *m, int rel)
{
    int64_t rows, n;
    int32_t width;
    if (tg_get_relation(m, rel, nullptr, nullptr, &rows, &n, &width) != TG_OK) return nullptr;
    vtkIdType *out = nullptr;
    if (cudaMalloc((void **)&out, (size_t)std::max<int64_t>(n, 1) * sizeof(vtkIdType)) !=
        cudaSuccess)
        return nullptr;
    if (tg_export_relation_i64(m, rel, (int64_t *)out, nullptr, 1, nullptr) != TG_OK) {
        report("export");
        cudaFree(out);
        return nullptr;
    }
    cudaDeviceSynchronize();
    return out;
}

// host copy of a relation (entries int32, offsets for CSR)
bool host_copy(tg_mesh *m, int rel, std::vector<int64_t> &off, std::vector<int32_t> &ent,
               int32_t &width)
{
    int64_t rows, n;
    if (tg_get_relation(m, rel, nullptr, nullptr, &rows, &n, &width) != TG_OK) return false;
    ent.resize((size_t)n);
    off.resize(width ? 0 : (size_t)(rows + 1));
    return tg_copy_relation(m, rel, width ? nullptr : off.data(), n ? ent.data() : nullptr,
                            nullptr) == TG_OK;
}

template <class Rows>
std::unique_ptr<Rows> csr_rows(tg_mesh *m, int rel)
{
    std::vector<int64_t> off;
    std::vector<int32_t> ent;
    int32_t width;
    auto out = std::make_unique<Rows>();
    if (!host_copy(m, rel, off, ent, width) || width) return out;
    out->resize(off.size() - 1);
    for (size_t r = 0; r + 1 < off.size(); r++)
        (*out)[r].assign(ent.begin() + off[r], ent.begin() + off[r + 1]);
    return out;
}

template <class Rows, int W>
std::unique_ptr<Rows> fixed_rows(tg_mesh *m, int rel)
{
    std::vector<int64_t> off;
    std::vector<int32_t> ent;
    int32_t width;
    auto out = std::make_unique<Rows>();
    if (!host_copy(m, rel, off, ent, width) || width != W) return out;
    out->resize(ent.size() / W);
    for (size_t r = 0; r < out->size(); r++)
        for (int k = 0; k < W; k++) (*out)[r][k] = ent[W * r + k];
    return out;
}

void maybe_release(bool free_transients)
{
    if (free_transients) release_locked();
}

}  // namespace

void make_TV_for_GPU(const TV_Data &tv)
{
    std::lock_guard<std::mutex> lk(g_mu);
    register_tv(tv);
}

void make_VE_for_GPU(const VE_Data &, const vtkIdType, const vtkIdType) {}
void make_VF_for_GPU(const VF_Data &, const vtkIdType, const vtkIdType) {}

vtkIdType *make_EV_GPU_return(const VE_Data &, const vtkIdType, const vtkIdType n_edges,
                              const bool free_transients)
{
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_mesh) {
        fprintf(stderr, "tetragpu: make_EV_GPU_return needs a registered mesh (make_TV_for_GPU)\n");
        return nullptr;
    }
    if (!extract(g_mesh, TG_EV) || !check_count(g_mesh, 0, n_edges, "EV")) return nullptr;
    vtkIdType *out = device_i64(g_mesh, TG_REL_EV);
    maybe_release(free_transients);
    return out;
}

std::unique_ptr<EV_Data> make_EV_GPU(const VE_Data &, const vtkIdType, const vtkIdType n_edges,
                                     const bool free_transients)
{
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_mesh || !extract(g_mesh, TG_EV) || !check_count(g_mesh, 0, n_edges, "EV"))
        return std::make_unique<EV_Data>();
    auto out = fixed_rows<EV_Data, 2>(g_mesh, TG_REL_EV);
    maybe_release(free_transients);
    return out;
}

vtkIdType *make_TF_GPU_return(const TV_Data &TV, const VF_Data &, const vtkIdType,
                              const vtkIdType n_faces, const vtkIdType, const bool free_transients)
{
    std::lock_guard<std::mutex> lk(g_mu);
    tg_mesh *m = register_tv(TV);
    if (!extract(m, TG_TF) || !check_count(m, 1, n_faces, "TF")) return nullptr;
    vtkIdType *out = device_i64(m, TG_REL_TF);
    maybe_release(free_transients);
    return out;
}

std::unique_ptr<TF_Data> make_TF_GPU(const TV_Data &TV, const VF_Data &, const vtkIdType,
                                     const vtkIdType n_faces, const vtkIdType,
                                     const bool free_transients)
{
    std::lock_guard<std::mutex> lk(g_mu);
    tg_mesh *m = register_tv(TV);
    if (!extract(m, TG_TF) || !check_count(m, 1, n_faces, "TF")) return std::make_unique<TF_Data>();
    auto out = fixed_rows<TF_Data, 4>(m, TG_REL_TF);
    maybe_release(free_transients);
    return out;
}

vtkIdType *make_TE_GPU_return(const TV_Data &TV, const VE_Data &, const vtkIdType,
                              const vtkIdType n_edges, const vtkIdType, const bool free_transients)
{
    std::lock_guard<std::mutex> lk(g_mu);
    tg_mesh *m = register_tv(TV);
    if (!extract(m, TG_TE) || !check_count(m, 0, n_edges, "TE")) return nullptr;
    vtkIdType *out = device_i64(m, TG_REL_TE);
    maybe_release(free_transients);
    return out;
}

std::unique_ptr<TE_Data> make_TE_GPU(const TV_Data &TV, const VE_Data &, const vtkIdType,
                                     const vtkIdType n_edges, const vtkIdType,
                                     const bool free_transients)
{
    std::lock_guard<std::mutex> lk(g_mu);
    tg_mesh *m = register_tv(TV);
    if (!extract(m, TG_TE) || !check_count(m, 0, n_edges, "TE")) return std::make_unique<TE_Data>();
    auto out = fixed_rows<TE_Data, 6>(m, TG_REL_TE);
    maybe_release(free_transients);
    return out;
}

vtkIdType *make_FV_GPU_return(const VF_Data &, const vtkIdType, const vtkIdType n_faces,
                              const bool free_transients)
{
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_mesh) {
        fprintf(stderr, "tetragpu: make_FV_GPU_return needs a registered mesh (make_TV_for_GPU)\n");
        return nullptr;
    }
    if (!extract(g_mesh, TG_FV) || !check_count(g_mesh, 1, n_faces, "FV")) return nullptr;
    vtkIdType *out = device_i64(g_mesh, TG_REL_FV);
    maybe_release(free_transients);
    return out;
}

std::unique_ptr<FV_Data> make_FV_GPU(const VF_Data &, const vtkIdType, const vtkIdType n_faces,
                                     const bool free_transients)
{
    std::lock_guard<std::mutex> lk(g_mu);
    auto out = std::make_unique<FV_Data>();
    if (!g_mesh || !extract(g_mesh, TG_FV) || !check_count(g_mesh, 1, n_faces, "FV")) return out;
    std::vector<int64_t> off;
    std::vector<int32_t> ent;
    int32_t width;
    if (!host_copy(g_mesh, TG_REL_FV, off, ent, width)) return out;
    // the reference's make_FV_GPU packs the three device values in order into
    // FaceData(middleVert, highVert, id) (src/cuda_extraction.cu:830-833)
    out->reserve(ent.size() / 3);
    for (size_t f = 0; f < ent.size() / 3; f++)
        out->emplace_back(FaceData(ent[3 * f], ent[3 * f + 1], ent[3 * f + 2]));
    maybe_release(free_transients);
    return out;
}

vtkIdType *make_FE_GPU_return(const VF_Data &, const VE_Data &, const vtkIdType, const vtkIdType,
                              const vtkIdType n_faces, const bool free_transients)
{
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_mesh) {
        fprintf(stderr, "tetragpu: make_FE_GPU_return needs a registered mesh (make_TV_for_GPU)\n");
        return nullptr;
    }
    if (!extract(g_mesh, TG_FE) || !check_count(g_mesh, 1, n_faces, "FE")) return nullptr;
    vtkIdType *out = device_i64(g_mesh, TG_REL_FE);
    maybe_release(free_transients);
    return out;
}

std::unique_ptr<FE_Data> make_FE_GPU(const VF_Data &, const VE_Data &, const vtkIdType,
                                     const vtkIdType, const vtkIdType n_faces,
                                     const bool free_transients)
{
    std::lock_guard<std::mutex> lk(g_mu);
    auto out = std::make_unique<FE_Data>();
    if (!g_mesh || !extract(g_mesh, TG_FE | TG_EV) || !check_count(g_mesh, 1, n_faces, "FE"))
        return out;
    std::vector<int64_t> off;
    std::vector<int32_t> fe, ev;
    int32_t w1, w2;
    if (!host_copy(g_mesh, TG_REL_FE, off, fe, w1) || !host_copy(g_mesh, TG_REL_EV, off, ev, w2))
        return out;
    // FE_Data holds EdgeData{high vertex, edge id} per edge of the face
    out->resize(fe.size() / 3);
    for (size_t f = 0; f < out->size(); f++)
        for (int k = 0; k < 3; k++) {
            const int32_t e = fe[3 * f + k];
            (*out)[f][k] = EdgeData(ev[2 * (size_t)e + 1], e);
        }
    maybe_release(free_transients);
    return out;
}

int get_approx_max_VV(const TV_Data &TV, const vtkIdType, const int)
{
    // the reference's sizing rule (src/cuda_extraction.cu:1160-1178): three
    // neighbours per cell around the busiest vertex, rounded up to 32
    std::lock_guard<std::mutex> lk(g_mu);
    tg_mesh *m = register_tv(TV);
    if (!m) return 32;
    std::vector<int64_t> off((size_t)TV.nPoints + 1);
    const int64_t *doff;
    if (tg_get_relation(m, TG_REL_VT, &doff, nullptr, nullptr, nullptr, nullptr) != TG_OK ||
        cudaMemcpy(off.data(), doff, off.size() * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
        return 32;
    int64_t most = 0;
    for (size_t v = 0; v + 1 < off.size(); v++) most = std::max(most, off[v + 1] - off[v]);
    return (int)(((3 * most + 31) / 32) * 32);
}

device_VV *make_VV_GPU_return(const TV_Data &TV, const int, const int n_points,
                              const int max_VV_guess, const bool free_transients)
{
    std::lock_guard<std::mutex> lk(g_mu);
    tg_mesh *m = register_tv(TV);
    if (!extract(m, TG_VV)) return nullptr;
    vtkIdType *computed = nullptr;
    unsigned int *index = nullptr;
    const size_t cells = (size_t)std::max(n_points, 1) * (size_t)std::max(max_VV_guess, 1);
    if (cudaMalloc((void **)&computed, cells * sizeof(vtkIdType)) != cudaSuccess ||
        cudaMalloc((void **)&index, (size_t)std::max(n_points, 1) * sizeof(unsigned)) !=
            cudaSuccess) {
        cudaFree(computed);
        return nullptr;
    }
    if (tg_export_rows_padded(m, TG_REL_VV, max_VV_guess, (int64_t *)computed, index, nullptr) !=
        TG_OK) {
        report("VV");
        cudaFree(computed);
        cudaFree(index);
        return nullptr;
    }
    cudaDeviceSynchronize();
    maybe_release(free_transients);
    return new device_VV(computed, index);
}

std::unique_ptr<VV_Data> make_VV_GPU(const TV_Data &TV, const int, const int,
                                     const bool free_transients)
{
    std::lock_guard<std::mutex> lk(g_mu);
    tg_mesh *m = register_tv(TV);
    if (!extract(m, TG_VV)) return std::make_unique<VV_Data>();
    auto out = csr_rows<VV_Data>(m, TG_REL_VV);
    maybe_release(free_transients);
    return out;
}

device_VT *make_VT_GPU_return(const TV_Data &TV)
{
    std::lock_guard<std::mutex> lk(g_mu);
    tg_mesh *m = register_tv(TV);
    if (!extract(m, TG_VT)) return nullptr;
    int64_t rows, n;
    int32_t width;
    tg_get_relation(m, TG_REL_VT, nullptr, nullptr, &rows, &n, &width);
    vtkIdType *computed = nullptr;
    unsigned long long *index = nullptr;
    if (cudaMalloc((void **)&computed, (size_t)std::max<int64_t>(n, 1) * 8) != cudaSuccess ||
        cudaMalloc((void **)&index, (size_t)(rows + 1) * 8) != cudaSuccess) {
        cudaFree(computed);
        return nullptr;
    }
    if (tg_export_relation_i64(m, TG_REL_VT, (int64_t *)computed, (int64_t *)index, 1, nullptr) !=
        TG_OK) {
        report("VT");
        cudaFree(computed);
        cudaFree(index);
        return nullptr;
    }
    cudaDeviceSynchronize();
    return new device_VT(computed, index);
}

device_VT *make_VT_GPU_return(const VT_Data &VT)
{
    // the reference uploads a host-built VT as CSR (src/cuda_extraction.cu:1282-1318)
    std::vector<vtkIdType> flat;
    std::vector<unsigned long long> index(VT.size() + 1);
    for (size_t v = 0; v < VT.size(); v++) {
        index[v] = flat.size();
        flat.insert(flat.end(), VT[v].begin(), VT[v].end());
    }
    index[VT.size()] = flat.size();
    vtkIdType *computed = nullptr;
    unsigned long long *dindex = nullptr;
    if (cudaMalloc((void **)&computed, std::max<size_t>(flat.size(), 1) * 8) != cudaSuccess ||
        cudaMalloc((void **)&dindex, index.size() * 8) != cudaSuccess) {
        cudaFree(computed);
        return nullptr;
    }
    cudaMemcpy(computed, flat.data(), flat.size() * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(dindex, index.data(), index.size() * 8, cudaMemcpyHostToDevice);
    return new device_VT(computed, dindex);
}

#define TG_COMPAT_CSR(NAME, TYPE, BIT, REL)                         \
    std::unique_ptr<TYPE> NAME(const TV_Data &TV)                    \
    {                                                                \
        std::lock_guard<std::mutex> lk(g_mu);                        \
        tg_mesh *m = register_tv(TV);                                \
        if (!extract(m, BIT)) return std::make_unique<TYPE>();       \
        return csr_rows<TYPE>(m, REL);                               \
    }

TG_COMPAT_CSR(make_ET_GPU, ET_Data, TG_ET, TG_REL_ET)
TG_COMPAT_CSR(make_EF_GPU, EF_Data, TG_EF, TG_REL_EF)
TG_COMPAT_CSR(make_TT_GPU, TT_Data, TG_TT, TG_REL_TT)
TG_COMPAT_CSR(make_FF_GPU, FF_Data, TG_FF, TG_REL_FF)
TG_COMPAT_CSR(make_EE_GPU, EE_Data, TG_EE, TG_REL_EE)

std::unique_ptr<FT_Data> make_FT_GPU(const TV_Data &TV)
{
    std::lock_guard<std::mutex> lk(g_mu);
    tg_mesh *m = register_tv(TV);
    if (!extract(m, TG_FT)) return std::make_unique<FT_Data>();
    return fixed_rows<FT_Data, 2>(m, TG_REL_FT);
}

tg_mesh *tetragpu_compat_mesh(void)
{
    std::lock_guard<std::mutex> lk(g_mu);
    return g_mesh;
}

void tetragpu_compat_release(void)
{
    std::lock_guard<std::mutex> lk(g_mu);
    release_locked();
}
