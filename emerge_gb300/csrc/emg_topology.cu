// Mesh topology and the Nedelec-2 DOF map on the GPU.
//
// The reference derives the edge/face topology of a tetrahedral mesh in
// Mesh3D.update (fem/mesh3d.py:224-355) with Python loops and dicts over the
// tets, and the DOF map in Nedelec2.__init__ (fem/elements/nedelec2.py:32-62).
// At millions of tets those loops take minutes.  This file builds the same
// arrays with sorts:
//
//  * edges: one 64-bit key (lo << 32 | hi) per (tet, edge slot), slot pairs
//    (0,1),(0,2),(0,3),(1,2),(3,1),(2,3) (fem/mesh3d.py:290-292); a stable radix
//    sort of the keys carrying the slot index; run heads get consecutive ids, so
//    edges are numbered in ascending (lo, hi) order.
//  * faces: the sorted triple (a <= b <= c) of every (tet, face slot), slots
//    (0,1,2),(0,2,3),(0,3,1),(1,2,3) (fem/mesh3d.py:296); sorted by (b, c), then
//    stably by a, which gives ascending (a, b, c) order for any vertex count.
//  * tri_to_edge: (v0,v1), (v1,v2), (v0,v2) of each sorted triple
//    (fem/mesh3d.py:331-335), by binary search in the sorted unique edge keys.
//  * tri_to_tet: the (at most two) tets of each face, ascending, -1 if one.
//  * tet_to_field (20, nT): edge ids, face ids + nE, edge ids + nE + nTri,
//    face ids + 2 nE + nTri (fem/elements/nedelec2.py:46-50).
//  * edge lengths: sqrt(dx*dx + dy*dy + dz*dz) rounded step by step
//    (fem/mesh3d.py:351).
//
// The numbering is the ascending vertex-tuple order (the reference numbers in
// CPython set order, which no other program reproduces); every array is
// bitwise equal to the host builder's (emerge_gb300/mesh.py).
#include <cub/device/device_radix_sort.cuh>

#include "emg_common.cuh"

namespace emg {
namespace topo {

__constant__ int8_t c_eslot[2][6] = {{0, 0, 0, 1, 3, 2}, {1, 2, 3, 2, 1, 3}};
__constant__ int8_t c_fslot[3][4] = {{0, 0, 0, 1}, {1, 2, 3, 2}, {2, 3, 1, 3}};

#define TOPO_ERR_VERTEX 1
#define TOPO_ERR_FACE 2
#define TOPO_ERR_EDGE 4

__device__ __forceinline__ void sort3(int32_t& a, int32_t& b, int32_t& c) {
    int32_t t;
    if (a > b) { t = a; a = b; b = t; }
    if (b > c) { t = b; b = c; c = t; }
    if (a > b) { t = a; a = b; b = t; }
}

__device__ __forceinline__ void face_of(const int32_t* __restrict__ tets, int64_t nT, int64_t i, int32_t& a,
                                        int32_t& b, int32_t& c) {
    const int f = (int)(i / nT);
    const int64_t t = i - (int64_t)f * nT;
    a = tets[c_fslot[0][f] * nT + t];
    b = tets[c_fslot[1][f] * nT + t];
    c = tets[c_fslot[2][f] * nT + t];
    sort3(a, b, c);
}

// i = slot * nT + t over the (6, nT) edge slots.
__global__ void k_edge_keys(const int32_t* __restrict__ tets, int64_t nT, int64_t nN, uint64_t* keys,
                            int32_t* vals, int* err) {
    const int64_t n = 6 * nT;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int e = (int)(i / nT);
        const int64_t t = i - (int64_t)e * nT;
        const int32_t a = tets[c_eslot[0][e] * nT + t], b = tets[c_eslot[1][e] * nT + t];
        if (a < 0 || b < 0 || a >= nN || b >= nN) atomicOr(err, TOPO_ERR_VERTEX);
        const uint32_t lo = (uint32_t)min(a, b), hi = (uint32_t)max(a, b);
        keys[i] = ((uint64_t)lo << 32) | hi;
        vals[i] = (int32_t)i;
    }
}

// heads[i] = 1 where a run of equal keys starts
template <typename K>
__global__ void k_heads(const K* __restrict__ keys, int64_t n, int64_t* heads) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        heads[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

__global__ void k_edge_scatter(const uint64_t* __restrict__ keys, const int32_t* __restrict__ vals, int64_t n,
                               const int64_t* __restrict__ hscan, int64_t nE, int32_t* t2e, int32_t* edges,
                               uint64_t* ukeys) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const bool head = (hscan[i + 1] - hscan[i]) != 0;
        const int64_t id = hscan[i + 1] - 1;
        t2e[vals[i]] = (int32_t)id;
        if (head) {
            const uint64_t k = keys[i];
            edges[id] = (int32_t)(k >> 32);
            edges[nE + id] = (int32_t)(k & 0xffffffffu);
            ukeys[id] = k;
        }
    }
}

// first sort key of the faces: (b << 32 | c) of the sorted triple
__global__ void k_face_keys(const int32_t* __restrict__ tets, int64_t nT, uint64_t* keys, int32_t* vals) {
    const int64_t n = 4 * nT;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t a, b, c;
        face_of(tets, nT, i, a, b, c);
        keys[i] = ((uint64_t)(uint32_t)b << 32) | (uint32_t)c;
        vals[i] = (int32_t)i;
    }
}

// second sort key: a, in the order of the first sort
__global__ void k_face_keys_a(const int32_t* __restrict__ tets, int64_t nT, const int32_t* __restrict__ vals,
                              uint32_t* keys) {
    const int64_t n = 4 * nT;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t a, b, c;
        face_of(tets, nT, vals[i], a, b, c);
        keys[i] = (uint32_t)a;
    }
}

// full (a, b, c) triple of each sorted position (a 3 x 32-bit key, compared field by field)
__global__ void k_face_heads(const int32_t* __restrict__ tets, int64_t nT, const int32_t* __restrict__ vals,
                             int64_t* heads) {
    const int64_t n = 4 * nT;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (i == 0) { heads[i] = 1; continue; }
        int32_t a, b, c, a0, b0, c0;
        face_of(tets, nT, vals[i], a, b, c);
        face_of(tets, nT, vals[i - 1], a0, b0, c0);
        heads[i] = (a != a0 || b != b0 || c != c0) ? 1 : 0;
    }
}

__device__ __forceinline__ int64_t find_edge(const uint64_t* __restrict__ ukeys, int64_t nE, uint64_t k) {
    int64_t lo = 0, hi = nE - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (ukeys[mid] < k) lo = mid + 1; else hi = mid;
    }
    return (nE > 0 && ukeys[lo] == k) ? lo : -1;
}

__global__ void k_face_scatter(const int32_t* __restrict__ tets, int64_t nT, const int32_t* __restrict__ vals,
                               int64_t n, const int64_t* __restrict__ hscan, int64_t nTri, const uint64_t* ukeys,
                               int64_t nE, int32_t* t2t, int32_t* tris, int32_t* tri2e, int32_t* tri2tet, int* err) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const bool head = (hscan[i + 1] - hscan[i]) != 0;
        const int64_t id = hscan[i + 1] - 1;
        const int32_t v = vals[i];
        t2t[v] = (int32_t)id;
        if (!head) continue;
        int32_t a, b, c;
        face_of(tets, nT, v, a, b, c);
        tris[id] = a;
        tris[nTri + id] = b;
        tris[2 * nTri + id] = c;
        const int64_t e0 = find_edge(ukeys, nE, ((uint64_t)(uint32_t)a << 32) | (uint32_t)b);
        const int64_t e1 = find_edge(ukeys, nE, ((uint64_t)(uint32_t)b << 32) | (uint32_t)c);
        const int64_t e2 = find_edge(ukeys, nE, ((uint64_t)(uint32_t)a << 32) | (uint32_t)c);
        if (e0 < 0 || e1 < 0 || e2 < 0) atomicOr(err, TOPO_ERR_EDGE);
        tri2e[id] = (int32_t)e0;
        tri2e[nTri + id] = (int32_t)e1;
        tri2e[2 * nTri + id] = (int32_t)e2;
        // the run of this face: one or two (tet, slot) entries
        const int64_t t0 = v % nT;
        int64_t t1 = -1;
        if (i + 1 < n && hscan[i + 2] == hscan[i + 1]) {
            t1 = vals[i + 1] % nT;
            if (i + 2 < n && hscan[i + 3] == hscan[i + 2]) atomicOr(err, TOPO_ERR_FACE);
        }
        tri2tet[id] = (int32_t)(t1 >= 0 ? min(t0, t1) : t0);
        tri2tet[nTri + id] = (int32_t)(t1 >= 0 ? max(t0, t1) : -1);
    }
}

__global__ void k_dof_map(const int32_t* __restrict__ t2e, const int32_t* __restrict__ t2t, int64_t nT, int64_t nE,
                          int64_t nTri, int32_t* t2f) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nT; t += (int64_t)gridDim.x * blockDim.x) {
        for (int e = 0; e < 6; ++e) {
            const int32_t id = t2e[e * nT + t];
            t2f[e * nT + t] = id;
            t2f[(10 + e) * nT + t] = (int32_t)(id + nE + nTri);
        }
        for (int f = 0; f < 4; ++f) {
            const int32_t id = t2t[f * nT + t];
            t2f[(6 + f) * nT + t] = (int32_t)(id + nE);
            t2f[(16 + f) * nT + t] = (int32_t)(id + 2 * nE + nTri);
        }
    }
}

__global__ void k_edge_len(const double* __restrict__ nodes, int64_t nN, const int32_t* __restrict__ edges,
                           int64_t nE, double* len) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nE; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t a = edges[i], b = edges[nE + i];
        const double dx = __dsub_rn(nodes[a], nodes[b]);
        const double dy = __dsub_rn(nodes[nN + a], nodes[nN + b]);
        const double dz = __dsub_rn(nodes[2 * nN + a], nodes[2 * nN + b]);
        len[i] = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
    }
}

}  // namespace topo
}  // namespace emg

struct emg_topology {
    int64_t nN = 0, nT = 0, nE = 0, nTri = 0;
    int32_t* edges = nullptr;      // (2, nE)
    int32_t* tris = nullptr;       // (3, nTri)
    int32_t* t2e = nullptr;        // (6, nT)
    int32_t* t2t = nullptr;        // (4, nT)
    int32_t* tri2e = nullptr;      // (3, nTri)
    int32_t* tri2tet = nullptr;    // (2, nTri)
    int32_t* t2f = nullptr;        // (20, nT)
};

namespace {

void free_topo(emg_topology* p) {
    if (!p) return;
    emg::dfree(p->edges);
    emg::dfree(p->tris);
    emg::dfree(p->t2e);
    emg::dfree(p->t2t);
    emg::dfree(p->tri2e);
    emg::dfree(p->tri2tet);
    emg::dfree(p->t2f);
    delete p;
}

}  // namespace

extern "C" int emg_topology_create(int64_t n_nodes, int64_t n_tets, const int32_t* tets, void* stream,
                                   emg_topology** out) {
    using namespace emg;
    using namespace emg::topo;
    EMG_CHECK_ARG(out != nullptr, "emg_topology_create: output pointer is NULL");
    *out = nullptr;
    EMG_CHECK_ARG(n_nodes >= 0 && n_tets >= 0, "emg_topology_create: negative size");
    EMG_CHECK_ARG(n_tets == 0 || tets != nullptr, "emg_topology_create: NULL tets");
    EMG_CHECK_ARG(6 * n_tets < (int64_t)INT32_MAX && n_nodes < (int64_t)INT32_MAX,
                  "emg_topology_create: 6 * n_tets and n_nodes must fit int32");
    cudaStream_t s = (cudaStream_t)stream;
    emg_topology* p = new emg_topology();
    p->nN = n_nodes;
    p->nT = n_tets;
    const int64_t nT = n_tets;
    const int64_t ne_slots = 6 * nT, nf_slots = 4 * nT;
    uint64_t *k1 = nullptr, *k2 = nullptr, *ukeys = nullptr;
    uint32_t *a1 = nullptr, *a2 = nullptr;          // 32-bit key views into k1 (not allocated)
    int32_t *v1 = nullptr, *v2 = nullptr;
    int64_t *heads = nullptr, *hscan = nullptr, *scratch = nullptr;
    int* d_err = nullptr;
    void* tmp = nullptr;
    auto fail = [&](int code) {
        dfree(k1); dfree(k2); dfree(ukeys); dfree(v1); dfree(v2);
        dfree(heads); dfree(hscan); dfree(scratch); dfree(d_err);
        if (tmp) cudaFree(tmp);
        free_topo(p);
        return code;
    };
#define TRY(x) do { int _r = (x); if (_r) return fail(_r); } while (0)
#define TRYC(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) return fail(cuda_status(_e, #x)); } while (0)
    if (nT == 0) {
        *out = p;
        return EMG_OK;
    }
    const int64_t nmax = ne_slots;
    TRY(dalloc(&k1, nmax, "topology keys"));
    TRY(dalloc(&k2, nmax, "topology keys"));
    TRY(dalloc(&v1, nmax, "topology values"));
    TRY(dalloc(&v2, nmax, "topology values"));
    TRY(dalloc(&heads, nmax + 1, "topology heads"));
    TRY(dalloc(&hscan, nmax + 1, "topology scan"));
    TRY(dalloc(&scratch, scan_scratch_elems(nmax + 1) + 1, "topology scan scratch"));
    TRY(dalloc(&d_err, 1, "topology error flag"));
    TRY(dalloc(&p->t2e, ne_slots, "tet_to_edge"));
    TRY(dalloc(&p->t2t, nf_slots, "tet_to_tri"));
    TRY(dalloc(&p->t2f, 20 * nT, "tet_to_field"));
    TRYC(cudaMemsetAsync(d_err, 0, sizeof(int), s));
    // temp storage for the largest sort (64-bit keys over the edge slots)
    size_t tmp_bytes = 0, need = 0;
    TRYC(cub::DeviceRadixSort::SortPairs(nullptr, need, k1, k2, v1, v2, (int)ne_slots, 0, 64, s));
    tmp_bytes = need;
    TRYC(cub::DeviceRadixSort::SortPairs(nullptr, need, a1, a2, v1, v2, (int)nf_slots, 0, 32, s));
    tmp_bytes = tmp_bytes > need ? tmp_bytes : need;
    TRYC(cudaMalloc(&tmp, tmp_bytes));
    const int T = 256;
    // ---- edges
    k_edge_keys<<<grid_for(ne_slots, T), T, 0, s>>>(tets, nT, n_nodes, k1, v1, d_err);
    TRYC(cudaGetLastError());
    TRYC(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, k1, k2, v1, v2, (int)ne_slots, 0, 64, s));
    k_heads<uint64_t><<<grid_for(ne_slots, T), T, 0, s>>>(k2, ne_slots, heads);
    TRYC(cudaGetLastError());
    TRY(scan_exclusive_i64(heads, hscan, ne_slots, scratch, s));
    TRYC(cudaMemcpyAsync(&p->nE, hscan + ne_slots, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    TRYC(cudaStreamSynchronize(s));
    TRY(dalloc(&p->edges, 2 * p->nE, "edges"));
    TRY(dalloc(&ukeys, p->nE, "unique edge keys"));
    k_edge_scatter<<<grid_for(ne_slots, T), T, 0, s>>>(k2, v2, ne_slots, hscan, p->nE, p->t2e, p->edges, ukeys);
    TRYC(cudaGetLastError());
    // ---- faces: (b, c) first, then stably by a
    k_face_keys<<<grid_for(nf_slots, T), T, 0, s>>>(tets, nT, k1, v1);
    TRYC(cudaGetLastError());
    TRYC(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, k1, k2, v1, v2, (int)nf_slots, 0, 64, s));
    a1 = reinterpret_cast<uint32_t*>(k1);          // k1 is free again: reuse as 32-bit keys
    a2 = reinterpret_cast<uint32_t*>(k1) + nf_slots;
    k_face_keys_a<<<grid_for(nf_slots, T), T, 0, s>>>(tets, nT, v2, a1);
    TRYC(cudaGetLastError());
    TRYC(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, a1, a2, v2, v1, (int)nf_slots, 0, 32, s));
    a1 = a2 = nullptr;                              // views of k1, not allocations
    k_face_heads<<<grid_for(nf_slots, T), T, 0, s>>>(tets, nT, v1, heads);
    TRYC(cudaGetLastError());
    TRY(scan_exclusive_i64(heads, hscan, nf_slots, scratch, s));
    TRYC(cudaMemcpyAsync(&p->nTri, hscan + nf_slots, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    TRYC(cudaStreamSynchronize(s));
    TRY(dalloc(&p->tris, 3 * p->nTri, "tris"));
    TRY(dalloc(&p->tri2e, 3 * p->nTri, "tri_to_edge"));
    TRY(dalloc(&p->tri2tet, 2 * p->nTri, "tri_to_tet"));
    k_face_scatter<<<grid_for(nf_slots, T), T, 0, s>>>(tets, nT, v1, nf_slots, hscan, p->nTri, ukeys, p->nE, p->t2t,
                                                       p->tris, p->tri2e, p->tri2tet, d_err);
    TRYC(cudaGetLastError());
    k_dof_map<<<grid_for(nT, T), T, 0, s>>>(p->t2e, p->t2t, nT, p->nE, p->nTri, p->t2f);
    TRYC(cudaGetLastError());
    int h_err = 0;
    TRYC(cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    TRYC(cudaStreamSynchronize(s));
    if (h_err) {
        std::string m = "emg_topology_create: invalid mesh:";
        if (h_err & TOPO_ERR_VERTEX) m += " a tet vertex index outside [0, n_nodes);";
        if (h_err & TOPO_ERR_FACE) m += " a face shared by more than two tets;";
        if (h_err & TOPO_ERR_EDGE) m += " a face edge missing from the edge list;";
        set_error(m);
        return fail(EMG_ERR_MESH);
    }
    if (2 * p->nE + 2 * p->nTri >= (int64_t)INT32_MAX) {
        set_error("emg_topology_create: n_field = 2 nE + 2 nTri must fit int32");
        return fail(EMG_ERR_LIMIT);
    }
    dfree(k1); dfree(k2); dfree(ukeys); dfree(v1); dfree(v2);
    dfree(heads); dfree(hscan); dfree(scratch); dfree(d_err);
    cudaFree(tmp);
#undef TRY
#undef TRYC
    *out = p;
    return EMG_OK;
}

extern "C" int emg_topology_sizes(const emg_topology* p, int64_t* n_edges, int64_t* n_tris) {
    EMG_CHECK_ARG(p && n_edges && n_tris, "emg_topology_sizes: NULL argument");
    *n_edges = p->nE;
    *n_tris = p->nTri;
    return EMG_OK;
}

extern "C" int emg_topology_get(const emg_topology* p, int32_t* edges, int32_t* tris, int32_t* tet_to_edge,
                                int32_t* tet_to_tri, int32_t* tri_to_edge, int32_t* tri_to_tet,
                                int32_t* tet_to_field, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(p != nullptr, "emg_topology_get: NULL topology");
    cudaStream_t s = (cudaStream_t)stream;
    auto cp = [&](int32_t* dst, const int32_t* src, int64_t n) -> int {
        if (dst == nullptr || n == 0) return EMG_OK;
        EMG_CUDA(cudaMemcpyAsync(dst, src, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s));
        return EMG_OK;
    };
    int rc;
    if ((rc = cp(edges, p->edges, 2 * p->nE))) return rc;
    if ((rc = cp(tris, p->tris, 3 * p->nTri))) return rc;
    if ((rc = cp(tet_to_edge, p->t2e, 6 * p->nT))) return rc;
    if ((rc = cp(tet_to_tri, p->t2t, 4 * p->nT))) return rc;
    if ((rc = cp(tri_to_edge, p->tri2e, 3 * p->nTri))) return rc;
    if ((rc = cp(tri_to_tet, p->tri2tet, 2 * p->nTri))) return rc;
    return cp(tet_to_field, p->t2f, 20 * p->nT);
}

extern "C" void emg_topology_destroy(emg_topology* p) { free_topo(p); }

extern "C" int emg_edge_lengths(int64_t n_nodes, const double* nodes, int64_t n_edges, const int32_t* edges,
                                double* lengths, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(n_nodes >= 0 && n_edges >= 0, "emg_edge_lengths: negative size");
    EMG_CHECK_ARG(n_edges == 0 || (nodes && edges && lengths), "emg_edge_lengths: NULL array");
    if (n_edges == 0) return EMG_OK;
    topo::k_edge_len<<<grid_for(n_edges, 256), 256, 0, (cudaStream_t)stream>>>(nodes, n_nodes, edges, n_edges, lengths);
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}
