// tg_crit.cu -- critical-point classification of a vertex scalar field.
//
// Semantics of the reference critPoints kernel (tlranda/TetraGPU,
// src/alg/critPoints.cu:49-331), restated on an exact VV:
//   * neighbour u of v is lower when f[u] < f[v], or f[u] == f[v] and u < v
//     (:136-140);
//   * two neighbours of the same kind are joined when the mesh has the edge
//     between them, i.e. w is in VV[u] (:172-202), not only edges in v's star;
//   * the lower-link and upper-link component counts go to classes[3v] and
//     classes[3v+1] (:275-284) and the code to classes[3v+2]: (>=1, 0) -> 2,
//     (0, >=1) -> 1, (1, 1) -> 3, anything else -> 4 (:303-330).
//
// Two kernels, so that a second field on the same mesh reuses the first:
//   k_crit_adj       field-independent: for every VV entry (v, u), the bitmask
//                    of v's neighbours adjacent to u (merge of two sorted
//                    rows).  Thread per vertex.
//   k_crit_classify  field-dependent: lower/upper split, then a union-find
//                    with path halving in shared memory over the adjacency
//                    bits of same-kind neighbours; roots are counted.
#include "tg_internal.h"

namespace tg {
namespace {

__global__ void __launch_bounds__(128)
k_crit_adj(const int64_t *__restrict__ vv_off, const int *__restrict__ vv, int64_t V,
           unsigned long long *__restrict__ adj, DevStatus *st)
{
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const int64_t b = vv_off[v];
    const int n = (int)(vv_off[v + 1] - b);
    if (n > kMaxDeg) {
        atomicOr(&st->flags, ST_HEAVY_DEG);
        atomicMin(&st->bad_vertex, (int)v);
        return;
    }
    const int *row = vv + b;
    for (int k = 0; k < n; k++) {
        const int u = __ldg(row + k);
        const int64_t ub = vv_off[u];
        const int un = (int)(vv_off[u + 1] - ub);
        const int *urow = vv + ub;
        unsigned long long bits = 0ull;
        int i = 0, j = 0;
        while (i < un && j < n) {
            const int x = __ldg(urow + i), y = __ldg(row + j);
            if (x < y) i++;
            else if (x > y) j++;
            else {
                bits |= 1ull << j;
                i++;
                j++;
            }
        }
        adj[b + k] = bits;
    }
}

constexpr int kClassifyThreads = 128;

__device__ __forceinline__ int uf_find(unsigned char *p, int stride, int x)
{
    // path halving: every visited node skips to its grandparent
    while (true) {
        const int px = p[x * stride];
        if (px == x) return x;
        const int gx = p[px * stride];
        p[x * stride] = (unsigned char)gx;
        x = gx;
    }
}

template <typename F>
__global__ void __launch_bounds__(kClassifyThreads)
k_crit_classify(const int64_t *__restrict__ vv_off, const int *__restrict__ vv,
                const unsigned long long *__restrict__ adj, const F *__restrict__ field, int64_t V,
                unsigned *__restrict__ classes3)
{
    __shared__ unsigned char parent_all[kMaxDeg * kClassifyThreads];
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    unsigned char *parent = parent_all + threadIdx.x;  // parent[k * stride]
    const int stride = kClassifyThreads;
    const int64_t b = vv_off[v];
    const int n = (int)(vv_off[v + 1] - b);
    unsigned lo = 0, up = 0;
    if (n <= kMaxDeg) {
        const F fv = field[v];
        unsigned long long lower = 0ull;
        for (int k = 0; k < n; k++) {
            const int u = __ldg(vv + b + k);
            const F fu = __ldg(field + u);
            const bool is_lower = (fu == fv) ? (u < (int)v) : (fu < fv);
            lower |= (unsigned long long)is_lower << k;
            parent[k * stride] = (unsigned char)k;
        }
        for (int k = 0; k < n; k++) {
            const unsigned long long same = ((lower >> k) & 1ull) ? lower : ~lower;
            // partners above k of the same kind
            unsigned long long m = __ldg(adj + b + k) & same & (~0ull << k) & ~(1ull << k);
            while (m) {
                const int j = __ffsll((long long)m) - 1;
                m &= m - 1;
                const int ra = uf_find(parent, stride, k), rb = uf_find(parent, stride, j);
                if (ra != rb) {
                    if (ra < rb) parent[rb * stride] = (unsigned char)ra;
                    else parent[ra * stride] = (unsigned char)rb;
                }
            }
        }
        for (int k = 0; k < n; k++)
            if (parent[k * stride] == k) {
                if ((lower >> k) & 1ull) lo++; else up++;
            }
    }
    unsigned code;
    if (lo >= 1 && up == 0) code = 2;
    else if (lo == 0 && up >= 1) code = 1;
    else if (lo == 1 && up == 1) code = 3;
    else code = 4;
    classes3[3 * v] = lo;
    classes3[3 * v + 1] = up;
    classes3[3 * v + 2] = code;
}

}  // namespace

void launch_crit_adj(const int64_t *vv_off, const int32_t *vv, int64_t V, uint64_t *adj,
                     DevStatus *st, cudaStream_t s)
{
    if (V == 0) return;
    {
        Launch L("k_crit_adj", s);
        k_crit_adj<<<(unsigned)((V + 127) / 128), 128, 0, s>>>(
            vv_off, vv, V, reinterpret_cast<unsigned long long *>(adj), st);
    }
}

void launch_crit_classify(const int64_t *vv_off, const int32_t *vv, const uint64_t *adj,
                          const void *field, int field_type, int64_t V, uint32_t *classes3,
                          cudaStream_t s)
{
    if (V == 0) return;
    const unsigned grid = (unsigned)((V + kClassifyThreads - 1) / kClassifyThreads);
    const auto *a = reinterpret_cast<const unsigned long long *>(adj);
    Launch L("k_crit_classify", s);
    if (field_type == 1)
        k_crit_classify<double><<<grid, kClassifyThreads, 0, s>>>(
            vv_off, vv, a, (const double *)field, V, classes3);
    else
        k_crit_classify<float><<<grid, kClassifyThreads, 0, s>>>(
            vv_off, vv, a, (const float *)field, V, classes3);
}

}  // namespace tg
