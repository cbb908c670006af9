// Float-float fill of the tet assembly (emg_fill_df.cu): plan-side data and entry points.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace emg {

constexpr int kDfMaxInc = 12;    // incident tets per edge entity handled by the fast fill
constexpr int kDfMaxCols = 128;  // CSR columns per entity handled by the fast fill

// Device arrays of the fast fill, owned by the assembly plan.
struct DfPlan {
    void* recs = nullptr;        // per-tet normalised float-float invariants (448 B/tet; general meshes)
    double2* gscale = nullptr;   // per-tet FP64 scales of the curl-curl and mass blocks
    float4* tscale = nullptr;    // per-tet complex material scales (written by each fill)
    // canonical-frame fill (every tet's orientations follow one vertex order): per-tet
    // invariants (43 x nT float pairs), DOF ids in canonical slot order (nT x 20),
    // incidences with canonical slots and their CSR positions, entity descriptors, and
    // the staging buffer of the element blocks
    bool canon = false;
    float2* inv = nullptr;
    int32_t* dofc = nullptr;
    int64_t* inc_c = nullptr;
    uint8_t* ipos = nullptr;     // CSR position of each incidence's 20 columns in its entity's row
    void* edesc = nullptr;       // per fast-fill entity: CSR row offsets, first incidence, sizes
    float4* st = nullptr;        // staged element blocks: 32 B per (tet, row pair, column), tets interleaved by 8
    int* mu_flag = nullptr;      // set by a fill whose mu^-1 has an imaginary part
    int2* groups = nullptr;      // warp work units: (first index into gents, entity count)
    int32_t* gents = nullptr;    // fast-fill entities ordered by class (2 edges / 1 edge / 6 faces per unit)
    int32_t* slow = nullptr;     // entities outside the fast-fill limits (FP64 fill)
    int64_t n_groups = 0;
    int64_t n_slow = 0;
};

int df_plan_build(const double* nodes, int64_t nN, const int32_t* tets, int64_t nT, const int32_t* edges, int64_t nE,
                  const int32_t* tris, int64_t nTri, const int32_t* t2f, const int32_t* t2e, const double* edge_len,
                  const int32_t* ent_list, int64_t n_ent, const int32_t* partner, const int64_t* inc_ptr,
                  const int64_t* inc, int64_t n_inc, const int64_t* indptr, const int32_t* indices, DfPlan* p,
                  cudaStream_t s);

int df_fill(const DfPlan& p, int64_t nT, const int32_t* partner, const int64_t* inc_ptr, const int64_t* inc,
            const int64_t* indptr, const int32_t* indices, const double* eps, const double* mu_inv, double* E,
            double* B, cudaStream_t s);

void df_plan_free(DfPlan* p);

}  // namespace emg
