// Second-order Nedelec tetrahedral assembly on GB300 (sm_103a).
//
// Replaces the reference's Numba assembler:
//   tet_mass_stiffness_matrices  fem/physics/edm/optimized_assembly.py:43-64
//   _matrix_builder              fem/physics/edm/optimized_assembly.py:66-116
//   ned2_tet_stiff_mass          fem/mth/tet.py:854-1088
//   tet_coefficients_bcd         fem/mth/optimized.py:343-369
//
// Design (entity-owner, deterministic, write-once):
//  * A DOF "entity" is an edge or a face: its two DOFs (mode 1 row r1, mode 2
//    row r2) have the same CSR column set, the union of the DOFs of the tets
//    that contain the entity.  The 20x20 element matrix of a tet is 10x10
//    blocks of 2x2 (entity x entity, mode x mode).  Block-row s of tet t
//    belongs to the entity in slot s of t.
//  * Plan (once per mesh): incidence lists entity -> (tet, slot) sorted by tet,
//    the CSR pattern (sorted unique columns per entity, written to both rows),
//    and a per-tet geometry record (TetRec).
//  * Fill: one warp owns one entity; it walks the entity's incident tets in
//    ascending tet order, computes that tet's 2x10 block-row, and adds it into
//    the entity's two CSR rows.  No two warps write the same row, so no
//    atomics are needed and the summation order is fixed (bitwise repeatable).
//
// Rounding parity: the volume and the gradient cofactors are evaluated with the
// reference's expanded formulas, term by term, with no fused multiply-add, so
// they round exactly like the reference.  This matters: on a unit-cube mesh
// with h = 1/80 the expanded 6V sum cancels ~5 orders of magnitude, and any
// other (more accurate) formula would differ from the reference by ~1e-10
// relative in 1/(6V)^4.
#include <algorithm>
#include <vector>

#include "emg_common.cuh"
#include "emg_fill_df.cuh"

namespace emg {
namespace {

// ---------------------------------------------------------------- tables ---
// Vertex pairs in "pair index" order (also the order of TetRec::ds).
__constant__ int8_t c_pidx[4][4] = {{-1, 0, 1, 2}, {0, -1, 3, 4}, {1, 3, -1, 5}, {2, 4, 5, -1}};
__constant__ int8_t c_gidx[4][4] = {{0, 1, 2, 3}, {1, 4, 5, 6}, {2, 5, 7, 8}, {3, 6, 8, 9}};

// Expanded-determinant terms of 6V (fem/mth/optimized.py:352): sign, x-, y-, z-vertex.
__constant__ int8_t c_vol_terms[24][4] = {
    {-1, 0, 1, 2}, {+1, 0, 1, 3}, {+1, 0, 2, 1}, {-1, 0, 2, 3}, {-1, 0, 3, 1}, {+1, 0, 3, 2},
    {+1, 1, 0, 2}, {-1, 1, 0, 3}, {-1, 1, 2, 0}, {+1, 1, 2, 3}, {+1, 1, 3, 0}, {-1, 1, 3, 2},
    {-1, 2, 0, 1}, {+1, 2, 0, 3}, {+1, 2, 1, 0}, {-1, 2, 1, 3}, {-1, 2, 3, 0}, {+1, 2, 3, 1},
    {+1, 3, 0, 1}, {-1, 3, 0, 2}, {-1, 3, 1, 0}, {+1, 3, 1, 2}, {+1, 3, 2, 0}, {-1, 3, 2, 1}};
// Cofactor sums (fem/mth/optimized.py:354-365): sign, u-vertex, v-vertex for b_i
// (u,v = y,z); d_i uses the same terms with (x,y); c_i the negated terms with (x,z).
__constant__ int8_t c_cof_terms[4][6][3] = {
    {{-1, 1, 2}, {+1, 1, 3}, {+1, 2, 1}, {-1, 2, 3}, {-1, 3, 1}, {+1, 3, 2}},
    {{+1, 0, 2}, {-1, 0, 3}, {-1, 2, 0}, {+1, 2, 3}, {+1, 3, 0}, {-1, 3, 2}},
    {{-1, 0, 1}, {+1, 0, 3}, {+1, 1, 0}, {-1, 1, 3}, {-1, 3, 0}, {+1, 3, 1}},
    {{+1, 0, 1}, {-1, 0, 2}, {-1, 1, 0}, {+1, 1, 2}, {+1, 2, 0}, {-1, 2, 1}}};

// Simplex monomial integrals prod(k_v!)/(sum k + 3)! indexed by vertex letters
// 0..4 (0 = absent), fem/mth/optimized.py:251-260; filled from the host.
__constant__ double c_vcoef[625];

// Per-tet geometry record written by the plan, read by the fill (AoS: one
// tet's record is read by several lanes at once).
struct __align__(16) TetRec {
    double gram[10];   // G_p . G_q, p <= q (G_p = (b_p, c_p, d_p) = 6V grad(lambda_p))
    double cdot[21];   // (G_a x G_b) . (G_c x G_d) over vertex pairs P <= R
    double ds[6];      // vertex distances, pair order
    double len[6];     // mesh edge lengths of edge slots 0..5
    double kd;         // 6V * 1/(6V)^4  (curl-curl scale)
    double kf;         // 6V * 1/(6V)^2  (mass scale)
    uint64_t lmap;     // local maps: edge slot e -> bits 4e (first vertex), 4e+2 (second);
                       // face slot f -> bits 24+6f, +2, +4 (tri vertices 0,1,2)
    int32_t dof[20];   // tet_to_field column
    double G[12];      // cofactor vectors G_p = (b_p, c_p, d_p), p-major (tensor materials)
};

// Material-weighted invariants of one tet for tensor materials, one real part
// (re or im) of the complex values: gram[p*4+q] = G_p . (Mm G_q) and
// cdot[P*6+R] = X_P . (Ms X_R), X_P = G_a x G_b for vertex pair P = (a < b).
constexpr int kTInv = 52;
struct TView {
    const double* len;
    const double* ds;
    uint64_t lmap;
    const double* inv;
};

constexpr int kFillWarps = 4;
constexpr int kCandCap = 1280;   // per-entity column candidates (64 incident tets x 20)

__device__ __forceinline__ int gi(int p, int q) { return c_gidx[p][q]; }
__device__ __forceinline__ int cidx(int P, int R) {
    if (P > R) { int t = P; P = R; R = t; }
    return P * 6 - (P * (P - 1)) / 2 + (R - P);
}
// (G_p x G_q) . (G_r x G_s) from the record's pair table.
__device__ __forceinline__ double ccv(const TetRec& r, int p, int q, int s1, int s2) {
    if (p == q || s1 == s2) return 0.0;
    int P = c_pidx[p][q], R = c_pidx[s1][s2];
    double sg = ((p < q) == (s1 < s2)) ? 1.0 : -1.0;
    return sg * r.cdot[cidx(P, R)];
}
__device__ __forceinline__ double gv(const TetRec& r, int p, int q) { return r.gram[gi(p, q)]; }
__device__ __forceinline__ double dsv(const TetRec& r, int p, int q) { return r.ds[c_pidx[p][q]]; }
// The same accessors over ordered (row vertex, column vertex) tensor invariants.
__device__ __forceinline__ double ccv(const TView& r, int p, int q, int s1, int s2) {
    if (p == q || s1 == s2) return 0.0;
    const int P = c_pidx[p][q], R = c_pidx[s1][s2];
    const double sg = ((p < q) == (s1 < s2)) ? 1.0 : -1.0;
    return sg * r.inv[16 + P * 6 + R];
}
__device__ __forceinline__ double gv(const TView& r, int p, int q) { return r.inv[p * 4 + q]; }
__device__ __forceinline__ double dsv(const TView& r, int p, int q) { return r.ds[c_pidx[p][q]]; }
// volume coefficient of letters (0-based vertices; -1 = absent)
__device__ __forceinline__ double v4(const double* vt, int a, int b, int c, int d) {
    return vt[(((a + 1) * 5 + (b + 1)) * 5 + (c + 1)) * 5 + (d + 1)];
}
__device__ __forceinline__ double v2(const double* vt, int a, int b) { return vt[((a + 1) * 5 + (b + 1)) * 25]; }

__device__ __forceinline__ void edge_verts(uint64_t m, int e, int& a, int& b) {
    a = (int)((m >> (4 * e)) & 3);
    b = (int)((m >> (4 * e + 2)) & 3);
}
__device__ __forceinline__ void face_verts(uint64_t m, int f, int& a, int& b, int& c) {
    a = (int)((m >> (24 + 6 * f)) & 3);
    b = (int)((m >> (24 + 6 * f + 2)) & 3);
    c = (int)((m >> (24 + 6 * f + 4)) & 3);
}

// Edge x edge block (fem/mth/tet.py:887-939).
template <class Rec>
__device__ void block_ee(const Rec& r, const double* vt, int e, int j, double D[2][2], double F[2][2]) {
    int A, B, C, Dl;
    edge_verts(r.lmap, e, A, B);
    edge_verts(r.lmap, j, C, Dl);
    const double Q2 = r.len[e] * r.len[j];
    const double Q = Q2 * 9.0 * ccv(r, A, B, C, Dl);
    D[0][0] = Q * v2(vt, A, C);
    D[0][1] = Q * v2(vt, A, Dl);
    D[1][0] = Q * v2(vt, B, C);
    D[1][1] = Q * v2(vt, B, Dl);
    const double gAC = gv(r, A, C), gAD = gv(r, A, Dl), gBC = gv(r, B, C), gBD = gv(r, B, Dl);
    F[0][0] = Q2 * (v4(vt, A, B, C, Dl) * gAC - v4(vt, A, B, C, C) * gAD - v4(vt, A, A, C, Dl) * gBC + v4(vt, A, A, C, C) * gBD);
    F[0][1] = Q2 * (v4(vt, A, B, Dl, Dl) * gAC - v4(vt, A, B, C, Dl) * gAD - v4(vt, A, A, Dl, Dl) * gBC + v4(vt, A, A, C, Dl) * gBD);
    F[1][0] = Q2 * (v4(vt, B, B, C, Dl) * gAC - v4(vt, B, B, C, C) * gAD - v4(vt, A, B, C, Dl) * gBC + v4(vt, A, B, C, C) * gBD);
    F[1][1] = Q2 * (v4(vt, B, B, Dl, Dl) * gAC - v4(vt, B, B, C, Dl) * gAD - v4(vt, A, B, Dl, Dl) * gBC + v4(vt, A, B, C, Dl) * gBD);
}

// Edge (rows) x face (columns) block (fem/mth/tet.py:941-993).
template <class Rec>
__device__ void block_ef(const Rec& r, const double* vt, int e, int f, double D[2][2], double F[2][2]) {
    int A, B, C, Dl, Fl;
    edge_verts(r.lmap, e, A, B);
    face_verts(r.lmap, f, C, Dl, Fl);
    const double L1 = r.len[e];
    const double Lab2 = dsv(r, C, Dl), Lac2 = dsv(r, C, Fl);
    const double AI = ccv(r, A, B, C, Fl), AJ = ccv(r, A, B, Dl, Fl), AK = ccv(r, A, B, C, Dl);
    const double gAF = gv(r, A, Fl), gAC = gv(r, A, C), gBF = gv(r, B, Fl), gBC = gv(r, B, C);
    const double gAD = gv(r, A, Dl), gBD = gv(r, B, Dl);
    const double c0 = L1 * Lac2, c1 = L1 * Lab2;
    D[0][0] = c0 * (-6.0 * v2(vt, A, Dl) * AI - 3.0 * v2(vt, A, C) * AJ - 3.0 * v2(vt, A, Fl) * AK);
    D[0][1] = c1 * (6.0 * v2(vt, A, Fl) * AK + 3.0 * v2(vt, A, Dl) * AI - 3.0 * v2(vt, A, C) * AJ);
    D[1][0] = c0 * (-6.0 * v2(vt, B, Dl) * AI - 3.0 * v2(vt, B, C) * AJ - 3.0 * v2(vt, B, Fl) * AK);
    D[1][1] = c1 * (6.0 * v2(vt, B, Fl) * AK + 3.0 * v2(vt, B, Dl) * AI - 3.0 * v2(vt, B, C) * AJ);
    F[0][0] = c0 * (v4(vt, A, B, C, Dl) * gAF - v4(vt, A, B, Dl, Fl) * gAC - v4(vt, A, A, C, Dl) * gBF + v4(vt, A, A, Dl, Fl) * gBC);
    F[0][1] = c1 * (v4(vt, A, B, Dl, Fl) * gAC - v4(vt, A, B, Fl, C) * gAD - v4(vt, A, A, Dl, Fl) * gBC + v4(vt, A, A, C, Fl) * gBD);
    F[1][0] = c0 * (v4(vt, B, B, C, Dl) * gAF - v4(vt, B, B, Dl, Fl) * gAC - v4(vt, A, B, C, Dl) * gBF + v4(vt, A, B, Dl, Fl) * gBC);
    F[1][1] = c1 * (v4(vt, B, B, Dl, Fl) * gAC - v4(vt, B, B, Fl, C) * gAD - v4(vt, A, B, Dl, Fl) * gBC + v4(vt, A, B, Fl, C) * gBD);
}

// Face x face block (fem/mth/tet.py:1006-1083), including the reference's
// choice of coefficient letters in the asymmetric mass terms.
template <class Rec>
__device__ void block_ff(const Rec& r, const double* vt, int fi, int fj, double D[2][2], double F[2][2]) {
    int A, B, E, C, Dl, Fl;
    face_verts(r.lmap, fi, A, B, E);
    face_verts(r.lmap, fj, C, Dl, Fl);
    const double Lac1 = dsv(r, A, E), Lab1 = dsv(r, A, B);
    const double Lac2 = dsv(r, C, Fl), Lab2 = dsv(r, C, Dl);
    const double AK = ccv(r, A, E, C, Fl), AL = ccv(r, A, E, Dl, Fl), AM = ccv(r, A, E, C, Dl);
    const double AN = ccv(r, B, E, C, Fl), AO = ccv(r, B, E, Dl, Fl), AP = ccv(r, B, E, C, Dl);
    const double AQ = ccv(r, A, B, C, Fl), AR = ccv(r, A, B, Dl, Fl), AS = ccv(r, A, B, C, Dl);
    const double gEF = gv(r, E, Fl), gEC = gv(r, E, C), gAF = gv(r, A, Fl), gAC = gv(r, A, C);
    const double gED = gv(r, E, Dl), gAD = gv(r, A, Dl), gBF = gv(r, B, Fl), gBC = gv(r, B, C), gBD = gv(r, B, Dl);
    const double vAD = v2(vt, A, Dl), vAC = v2(vt, A, C), vAF = v2(vt, A, Fl);
    const double vBF = v2(vt, B, Fl), vBC = v2(vt, B, C), vBD = v2(vt, B, Dl);
    const double vDE = v2(vt, E, Dl), vEF = v2(vt, E, Fl), vCE = v2(vt, E, C);
    const double vABCD = v4(vt, A, B, C, Dl), vABDF = v4(vt, A, B, Dl, Fl), vACEF = v4(vt, A, C, E, Fl);
    const double vABCF = v4(vt, A, B, Fl, C), vBCDX = v4(vt, B, C, Dl, Fl), vBDEF = v4(vt, B, E, Dl, Fl);
    const double vACDE = v4(vt, E, A, C, Dl), vBCEF = v4(vt, B, E, Fl, C), vADEF = v4(vt, E, A, Dl, Fl);
    const double Q1 = 2.0 * vAD * AN + vAC * AO + vAF * AP;
    const double Q2 = -2.0 * vAF * AP - vAD * AN + vAC * AO;
    D[0][0] = Lac1 * Lac2 * (4.0 * vBD * AK + 2.0 * vBC * AL + 2.0 * vBF * AM + Q1 + 2.0 * vDE * AQ + vCE * AR + vEF * AS);
    D[0][1] = Lac1 * Lab2 * (-4.0 * vBF * AM - 2.0 * vBD * AK + 2.0 * vBC * AL + Q2 - 2.0 * vEF * AS - vDE * AQ + vCE * AR);
    D[1][0] = Lab1 * Lac2 * (-4.0 * vDE * AQ - 2.0 * vCE * AR - 2.0 * vEF * AS - 2.0 * vBD * AK - vBC * AL - vBF * AM + Q1);
    D[1][1] = Lab1 * Lab2 * (4.0 * vEF * AS + 2.0 * vDE * AQ - 2.0 * vCE * AR + 2.0 * vBF * AM + vBD * AK - vBC * AL + Q2);
    F[0][0] = Lac1 * Lac2 * (vABCD * gEF - vABDF * gEC - vBCDX * gAF + vBDEF * gAC);
    F[0][1] = Lac1 * Lab2 * (vABDF * gEC - vABCF * gED - vBDEF * gAC + vBCEF * gAD);
    F[1][0] = Lab1 * Lac2 * (vBCDX * gAF - vBDEF * gAC - vACDE * gBF + vADEF * gBC);
    F[1][1] = Lab1 * Lab2 * (vBDEF * gAC - vBCEF * gAD - vADEF * gBC + vACEF * gBD);
}

// Block (row entity slot s, column entity slot j) of a tet, geometric part
// (without the material scale and without kd / kf).
template <class Rec>
__device__ __forceinline__ void tet_block(const Rec& r, const double* vt, int s, int j, double D[2][2],
                                          double F[2][2]) {
    if (s < 6) {
        if (j < 6) block_ee(r, vt, s, j, D, F);
        else block_ef(r, vt, s, j - 6, D, F);
    } else if (j < 6) {
        // face rows x edge columns are the transpose of the edge x face block
        double Dt[2][2], Ft[2][2];
        block_ef(r, vt, j, s - 6, Dt, Ft);
        D[0][0] = Dt[0][0]; D[0][1] = Dt[1][0]; D[1][0] = Dt[0][1]; D[1][1] = Dt[1][1];
        F[0][0] = Ft[0][0]; F[0][1] = Ft[1][0]; F[1][0] = Ft[0][1]; F[1][1] = Ft[1][1];
    } else {
        block_ff(r, vt, s - 6, j - 6, D, F);
    }
}

// ------------------------------------------------------------ plan kernels ---
#define ERR_LOCALMAP 1
#define ERR_PARTNER 2
#define ERR_ROLE 4
#define ERR_CANDCAP 8
#define ERR_DOFRANGE 16

__global__ void k_incidence_count(const int32_t* __restrict__ t2f, int64_t nT, int64_t N, int32_t* partner,
                                  int32_t* role, int64_t* inc_cnt, int* err) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nT * 10; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = i / 10;
        const int s = (int)(i % 10);
        const int32_t r1 = t2f[s * nT + t], r2 = t2f[(s + 10) * nT + t];
        if (r1 < 0 || r1 >= N || r2 < 0 || r2 >= N) { atomicOr(err, ERR_DOFRANGE); continue; }
        atomicAdd(reinterpret_cast<unsigned long long*>(&inc_cnt[r1]), 1ull);
        const int32_t old = atomicCAS(&partner[r1], -1, r2);
        if (old != -1 && old != r2) atomicOr(err, ERR_PARTNER);
        atomicOr(&role[r1], 1);
        atomicOr(&role[r2], 2);
    }
}

__global__ void k_check_roles(const int32_t* role, int64_t N, const int64_t* inc_cnt, int64_t* ent_flag, int* err) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x) {
        if (role[r] == 3) atomicOr(err, ERR_ROLE);
        ent_flag[r] = inc_cnt[r] > 0 ? 1 : 0;
    }
}

__global__ void k_compact(const int64_t* flag_scan, const int64_t* inc_cnt, int64_t N, int32_t* ent_list) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x)
        if (inc_cnt[r] > 0) ent_list[flag_scan[r]] = (int32_t)r;
}

__global__ void k_incidence_fill(const int32_t* __restrict__ t2f, int64_t nT, const int64_t* inc_ptr,
                                 int32_t* cursor, int64_t* inc) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nT * 10; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = i / 10;
        const int s = (int)(i % 10);
        const int32_t r1 = t2f[s * nT + t];
        const int32_t k = atomicAdd(&cursor[r1], 1);
        inc[inc_ptr[r1] + k] = (t << 4) | s;
    }
}

// Sort each entity's incidences by tet id (keys are unique per entity).
__global__ void k_incidence_sort(const int32_t* ent_list, int64_t n_ent, const int64_t* inc_ptr, int64_t* inc) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_ent; e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r1 = ent_list[e];
        int64_t* a = inc + inc_ptr[r1];
        const int64_t n = inc_ptr[r1 + 1] - inc_ptr[r1];
        for (int64_t i = 1; i < n; ++i) {
            const int64_t v = a[i];
            int64_t j = i - 1;
            while (j >= 0 && a[j] > v) { a[j + 1] = a[j]; --j; }
            a[j + 1] = v;
        }
    }
}

// Warp per entity: sorted unique columns of the union of the incident tets'
// DOFs.  mode 0 writes row lengths; mode 1 writes the columns of both rows.
__global__ void __launch_bounds__(32 * kFillWarps) k_pattern(const int32_t* __restrict__ t2f, int64_t nT,
                                                              const int32_t* ent_list, int64_t n_ent,
                                                              const int32_t* partner, const int64_t* inc_ptr,
                                                              const int64_t* inc, int mode, int64_t* row_len,
                                                              const int64_t* indptr, int32_t* indices, int* err) {
    __shared__ int32_t cand[kFillWarps][kCandCap];
    __shared__ uint8_t first[kFillWarps][kCandCap];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int32_t* cw = cand[w];
    uint8_t* fw = first[w];
    for (int64_t e = blockIdx.x * (int64_t)kFillWarps + w; e < n_ent; e += (int64_t)gridDim.x * kFillWarps) {
        const int32_t r1 = ent_list[e];
        const int32_t r2 = partner[r1];
        const int64_t i0 = inc_ptr[r1], k = inc_ptr[r1 + 1] - i0;
        const int n = (int)(k * 20);
        if (n > kCandCap) {
            if (lane == 0) atomicOr(err, ERR_CANDCAP);
            continue;
        }
        for (int c = lane; c < n; c += 32) {
            const int64_t t = inc[i0 + c / 20] >> 4;
            cw[c] = t2f[(int64_t)(c % 20) * nT + t];
        }
        __syncwarp();
        for (int c = lane; c < n; c += 32) {
            const int32_t x = cw[c];
            bool f = true;
            for (int q = 0; q < c; ++q) if (cw[q] == x) { f = false; break; }
            fw[c] = f;
        }
        __syncwarp();
        int cnt = 0;
        for (int c = lane; c < n; c += 32) cnt += fw[c];
        for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        if (mode == 0) {
            if (lane == 0) { row_len[r1] = cnt; row_len[r2] = cnt; }
        } else {
            const int64_t b1 = indptr[r1], b2 = indptr[r2];
            for (int c = lane; c < n; c += 32) {
                if (!fw[c]) continue;
                const int32_t x = cw[c];
                int rank = 0;
                for (int q = 0; q < n; ++q) rank += (fw[q] && cw[q] < x);
                indices[b1 + rank] = x;
                indices[b2 + rank] = x;
            }
        }
        __syncwarp();
    }
}

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }

// Thread per tet: geometry record with the reference's rounding of V and the cofactors.
__global__ void k_tet_prep(const double* __restrict__ nodes, int64_t nN, const int32_t* __restrict__ tets,
                           int64_t nT, const int32_t* __restrict__ edges, int64_t nE, const int32_t* __restrict__ tris,
                           int64_t nTri, const int32_t* __restrict__ t2f, const int32_t* __restrict__ t2e,
                           const double* __restrict__ edge_len, TetRec* __restrict__ recs, int* err) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nT; t += (int64_t)gridDim.x * blockDim.x) {
        int32_t vid[4];
        double x[4], y[4], z[4];
        for (int k = 0; k < 4; ++k) {
            vid[k] = tets[k * nT + t];
            x[k] = nodes[vid[k]];
            y[k] = nodes[nN + vid[k]];
            z[k] = nodes[2 * nN + vid[k]];
        }
        double s = 0.0;
        for (int k = 0; k < 24; ++k) {
            const double term = __ddiv_rn(dm(dm(x[c_vol_terms[k][1]], y[c_vol_terms[k][2]]), z[c_vol_terms[k][3]]), 6.0);
            s = c_vol_terms[k][0] > 0 ? __dadd_rn(s, term) : __dsub_rn(s, term);
        }
        const double V = fabs(s);
        double G[4][3];
        for (int i = 0; i < 4; ++i) {
            double sb = 0.0, sc = 0.0, sd = 0.0;
            for (int k = 0; k < 6; ++k) {
                const int sg = c_cof_terms[i][k][0], a = c_cof_terms[i][k][1], b = c_cof_terms[i][k][2];
                const double pb = dm(y[a], z[b]), pc = dm(x[a], z[b]), pd = dm(x[a], y[b]);
                sb = sg > 0 ? __dadd_rn(sb, pb) : __dsub_rn(sb, pb);
                sc = sg > 0 ? __dsub_rn(sc, pc) : __dadd_rn(sc, pc);
                sd = sg > 0 ? __dadd_rn(sd, pd) : __dsub_rn(sd, pd);
            }
            G[i][0] = sb; G[i][1] = sc; G[i][2] = sd;
        }
        TetRec r;
        for (int i = 0; i < 4; ++i)
            for (int k = 0; k < 3; ++k) r.G[i * 3 + k] = G[i][k];
        for (int p = 0; p < 4; ++p)
            for (int q = p; q < 4; ++q) r.gram[c_gidx[p][q]] = G[p][0] * G[q][0] + G[p][1] * G[q][1] + G[p][2] * G[q][2];
        double X[6][3];
        const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {1, 2, 3, 2, 3, 3};
        for (int P = 0; P < 6; ++P) {
            const double* u = G[pa[P]];
            const double* v = G[pb[P]];
            X[P][0] = u[1] * v[2] - u[2] * v[1];
            X[P][1] = u[2] * v[0] - u[0] * v[2];
            X[P][2] = u[0] * v[1] - u[1] * v[0];
            const double dx = x[pa[P]] - x[pb[P]], dy = y[pa[P]] - y[pb[P]], dz = z[pa[P]] - z[pb[P]];
            r.ds[P] = sqrt(dx * dx + dy * dy + dz * dz);
        }
        for (int P = 0; P < 6; ++P)
            for (int R = P; R < 6; ++R)
                r.cdot[cidx(P, R)] = X[P][0] * X[R][0] + X[P][1] * X[R][1] + X[P][2] * X[R][2];
        const double V6 = 6.0 * V;
        const double V6sq = V6 * V6;
        r.kd = V6 * (1.0 / (V6sq * V6sq));
        r.kf = V6 * (1.0 / V6sq);
        uint64_t lm = 0;
        bool ok = true;
        for (int e = 0; e < 6; ++e) {
            const int32_t eid = t2f[e * nT + t];
            r.len[e] = edge_len[t2e[e * nT + t]];
            if (eid < 0 || eid >= nE) { ok = false; continue; }
            for (int j = 0; j < 2; ++j) {
                const int32_t g = edges[j * nE + eid];
                int loc = -1;
                for (int k = 0; k < 4; ++k) if (vid[k] == g) { loc = k; break; }
                if (loc < 0) { ok = false; loc = 0; }
                lm |= (uint64_t)loc << (4 * e + 2 * j);
            }
        }
        for (int f = 0; f < 4; ++f) {
            const int64_t tri = (int64_t)t2f[(6 + f) * nT + t] - nE;
            if (tri < 0 || tri >= nTri) { ok = false; continue; }
            for (int j = 0; j < 3; ++j) {
                const int32_t g = tris[j * nTri + tri];
                int loc = -1;
                for (int k = 0; k < 4; ++k) if (vid[k] == g) { loc = k; break; }
                if (loc < 0) { ok = false; loc = 0; }
                lm |= (uint64_t)loc << (24 + 6 * f + 2 * j);
            }
        }
        if (!ok) atomicOr(err, ERR_LOCALMAP);
        r.lmap = lm;
        for (int k = 0; k < 20; ++k) r.dof[k] = t2f[k * nT + t];
        recs[t] = r;
    }
}

// -------------------------------------------------------------- fill kernel ---
__device__ __forceinline__ int find_col(const int32_t* __restrict__ cols, int n, int32_t c) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(cols + mid) < c) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// Warp per entity (see file header).  eps / mu_inv: complex per tet.
__global__ void __launch_bounds__(32 * kFillWarps) k_fill(const TetRec* __restrict__ recs, const int32_t* ent_list,
                                                           int64_t n_ent, const int32_t* __restrict__ partner,
                                                           const int64_t* __restrict__ inc_ptr,
                                                           const int64_t* __restrict__ inc,
                                                           const int64_t* __restrict__ indptr,
                                                           const int32_t* __restrict__ indices,
                                                           const double2* __restrict__ eps,
                                                           const double2* __restrict__ mu_inv, double2* E,
                                                           double2* B) {
    __shared__ double vt[625];
    for (int i = threadIdx.x; i < 625; i += blockDim.x) vt[i] = c_vcoef[i];
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int64_t e = blockIdx.x * (int64_t)kFillWarps + w; e < n_ent; e += (int64_t)gridDim.x * kFillWarps) {
        const int32_t r1 = ent_list[e];
        const int32_t r2 = partner[r1];
        const int64_t b1 = indptr[r1], b2 = indptr[r2];
        const int n = (int)(indptr[r1 + 1] - b1);
        for (int c = lane; c < n; c += 32) {
            E[b1 + c] = make_double2(0.0, 0.0);
            E[b2 + c] = make_double2(0.0, 0.0);
            B[b1 + c] = make_double2(0.0, 0.0);
            B[b2 + c] = make_double2(0.0, 0.0);
        }
        __syncwarp();
        const int32_t* cols = indices + b1;
        const int64_t i0 = inc_ptr[r1], i1 = inc_ptr[r1 + 1];
        for (int64_t i = i0; i < i1; ++i) {
            const int64_t code = inc[i];
            const int64_t t = code >> 4;
            const int s = (int)(code & 15);
            if (lane < 10) {
                const TetRec& r = recs[t];
                double D[2][2], F[2][2];
                tet_block(r, vt, s, lane, D, F);
                const double2 me = mu_inv[t], ep = eps[t];
                const double kd = r.kd, kf = r.kf;
                const double2 sE = make_double2(me.x * kd, me.y * kd);
                const double2 sB = make_double2(ep.x * kf, ep.y * kf);
                const int p[2] = {find_col(cols, n, r.dof[lane]), find_col(cols, n, r.dof[lane + 10])};
                const int64_t rb[2] = {b1, b2};
#pragma unroll
                for (int a = 0; a < 2; ++a)
#pragma unroll
                    for (int b = 0; b < 2; ++b) {
                        const int64_t o = rb[a] + p[b];
                        double2 ve = E[o], vb = B[o];
                        ve.x += sE.x * D[a][b];
                        ve.y += sE.y * D[a][b];
                        vb.x += sB.x * F[a][b];
                        vb.y += sB.y * F[a][b];
                        E[o] = ve;
                        B[o] = vb;
                    }
            }
            __syncwarp();
        }
    }
}

// Tensor materials (the reference's full (3,3) er / matinv(ur) per tet): thread per
// tet, invariants in the reference's evaluation order (matmul(M, v) row by row, then
// dot_c; fem/mth/tet.py:35-40,918-925,967-982), with no fused multiply-add.  The
// imaginary part of G and X is zero, so every complex product splits into a real
// and an imaginary evaluation of the same real expression.
__global__ void k_tensor_prep(const TetRec* __restrict__ recs, int64_t nT, const double2* __restrict__ eps9,
                              const double2* __restrict__ muinv9, double* __restrict__ tinv) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nT; t += (int64_t)gridDim.x * blockDim.x) {
        double G[4][3];
        for (int i = 0; i < 12; ++i) G[i / 3][i % 3] = recs[t].G[i];
        double X[6][3];
        const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {1, 2, 3, 2, 3, 3};
        for (int P = 0; P < 6; ++P) {
            const double* u = G[pa[P]];
            const double* v = G[pb[P]];
            X[P][0] = __dsub_rn(__dmul_rn(u[1], v[2]), __dmul_rn(u[2], v[1]));
            X[P][1] = __dsub_rn(__dmul_rn(u[2], v[0]), __dmul_rn(u[0], v[2]));
            X[P][2] = __dsub_rn(__dmul_rn(u[0], v[1]), __dmul_rn(u[1], v[0]));
        }
        double* out = tinv + t * (2 * kTInv);
        for (int part = 0; part < 2; ++part) {
            double Mm[9], Ms[9];
            for (int i = 0; i < 9; ++i) {
                const double2 a = eps9[i * nT + t], b = muinv9[i * nT + t];
                Mm[i] = part ? a.y : a.x;
                Ms[i] = part ? b.y : b.x;
            }
            double* o = out + part * kTInv;
            for (int q = 0; q < 4; ++q) {
                double w[3];
                for (int k = 0; k < 3; ++k)
                    w[k] = __dadd_rn(__dadd_rn(__dmul_rn(Mm[3 * k], G[q][0]), __dmul_rn(Mm[3 * k + 1], G[q][1])),
                                     __dmul_rn(Mm[3 * k + 2], G[q][2]));
                for (int p = 0; p < 4; ++p)
                    o[p * 4 + q] = __dadd_rn(__dadd_rn(__dmul_rn(G[p][0], w[0]), __dmul_rn(G[p][1], w[1])),
                                             __dmul_rn(G[p][2], w[2]));
            }
            for (int R = 0; R < 6; ++R) {
                double w[3];
                for (int k = 0; k < 3; ++k)
                    w[k] = __dadd_rn(__dadd_rn(__dmul_rn(Ms[3 * k], X[R][0]), __dmul_rn(Ms[3 * k + 1], X[R][1])),
                                     __dmul_rn(Ms[3 * k + 2], X[R][2]));
                for (int P = 0; P < 6; ++P)
                    o[16 + P * 6 + R] = __dadd_rn(__dadd_rn(__dmul_rn(X[P][0], w[0]), __dmul_rn(X[P][1], w[1])),
                                                  __dmul_rn(X[P][2], w[2]));
            }
        }
    }
}

// Entity-owner FP64 fill for tensor materials: as k_fill, with the block formulas
// evaluated once on the real and once on the imaginary invariants (both are linear
// in them) and scaled by the geometric factors only.
__global__ void __launch_bounds__(32 * kFillWarps) k_fill_tensor(const TetRec* __restrict__ recs,
                                                                  const double* __restrict__ tinv,
                                                                  const int32_t* ent_list, int64_t n_ent,
                                                                  const int32_t* __restrict__ partner,
                                                                  const int64_t* __restrict__ inc_ptr,
                                                                  const int64_t* __restrict__ inc,
                                                                  const int64_t* __restrict__ indptr,
                                                                  const int32_t* __restrict__ indices, double2* E,
                                                                  double2* B) {
    __shared__ double vt[625];
    for (int i = threadIdx.x; i < 625; i += blockDim.x) vt[i] = c_vcoef[i];
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int64_t e = blockIdx.x * (int64_t)kFillWarps + w; e < n_ent; e += (int64_t)gridDim.x * kFillWarps) {
        const int32_t r1 = ent_list[e];
        const int32_t r2 = partner[r1];
        const int64_t b1 = indptr[r1], b2 = indptr[r2];
        const int n = (int)(indptr[r1 + 1] - b1);
        for (int c = lane; c < n; c += 32) {
            E[b1 + c] = make_double2(0.0, 0.0);
            E[b2 + c] = make_double2(0.0, 0.0);
            B[b1 + c] = make_double2(0.0, 0.0);
            B[b2 + c] = make_double2(0.0, 0.0);
        }
        __syncwarp();
        const int32_t* cols = indices + b1;
        const int64_t i0 = inc_ptr[r1], i1 = inc_ptr[r1 + 1];
        for (int64_t i = i0; i < i1; ++i) {
            const int64_t code = inc[i];
            const int64_t t = code >> 4;
            const int s = (int)(code & 15);
            if (lane < 10) {
                const TetRec& r = recs[t];
                const TView vre{r.len, r.ds, r.lmap, tinv + t * (2 * kTInv)};
                const TView vim{r.len, r.ds, r.lmap, tinv + t * (2 * kTInv) + kTInv};
                double Dr[2][2], Fr[2][2], Di[2][2], Fi[2][2];
                tet_block(vre, vt, s, lane, Dr, Fr);
                tet_block(vim, vt, s, lane, Di, Fi);
                const double kd = r.kd, kf = r.kf;
                const int p[2] = {find_col(cols, n, r.dof[lane]), find_col(cols, n, r.dof[lane + 10])};
                const int64_t rb[2] = {b1, b2};
#pragma unroll
                for (int a = 0; a < 2; ++a)
#pragma unroll
                    for (int b = 0; b < 2; ++b) {
                        const int64_t o = rb[a] + p[b];
                        double2 ve = E[o], vb = B[o];
                        ve.x += kd * Dr[a][b];
                        ve.y += kd * Di[a][b];
                        vb.x += kf * Fr[a][b];
                        vb.y += kf * Fi[a][b];
                        E[o] = ve;
                        B[o] = vb;
                    }
            }
            __syncwarp();
        }
    }
}

}  // namespace
}  // namespace emg

// ------------------------------------------------------------------ C ABI ---
struct emg_plan {
    int64_t nT = 0, N = 0, nnz = 0, n_ent = 0;
    emg::TetRec* recs = nullptr;
    int32_t* ent_list = nullptr;
    int32_t* partner = nullptr;
    int64_t* inc_ptr = nullptr;
    int64_t* inc = nullptr;
    int64_t* indptr = nullptr;
    int32_t* indices = nullptr;
    double* eps_dev = nullptr;     // staging for the host entry point
    double* mu_dev = nullptr;
    double* E_dev = nullptr;
    double* B_dev = nullptr;
    double* tinv = nullptr;        // tensor-material invariants (2 x 52 per tet), on first use
    double* eps9_dev = nullptr;    // staging for the tensor host entry point
    double* mu9_dev = nullptr;
    emg::DfPlan df;                // float-float fast fill (emg_fill_df.cu)
};

namespace {

void free_plan(emg_plan* p) {
    if (!p) return;
    emg::dfree(p->recs);
    emg::df_plan_free(&p->df);
    emg::dfree(p->ent_list);
    emg::dfree(p->partner);
    emg::dfree(p->inc_ptr);
    emg::dfree(p->inc);
    emg::dfree(p->indptr);
    emg::dfree(p->indices);
    emg::dfree(p->eps_dev);
    emg::dfree(p->mu_dev);
    emg::dfree(p->E_dev);
    emg::dfree(p->B_dev);
    emg::dfree(p->tinv);
    emg::dfree(p->eps9_dev);
    emg::dfree(p->mu9_dev);
    delete p;
}

// __constant__ memory is per device: the table is uploaded once for every device used
bool g_vcoef_ready[64] = {false};

int upload_vcoef() {
    int dev = 0;
    EMG_CUDA(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64 && g_vcoef_ready[dev]) return EMG_OK;
    static const double fact[10] = {1, 1, 2, 6, 24, 120, 720, 5040, 40320, 362880};
    double h[625];
    for (int a = 0; a < 5; ++a)
        for (int b = 0; b < 5; ++b)
            for (int c = 0; c < 5; ++c)
                for (int d = 0; d < 5; ++d) {
                    int k[5] = {0, 0, 0, 0, 0};
                    k[a]++; k[b]++; k[c]++; k[d]++;
                    const double num = fact[k[1]] * fact[k[2]] * fact[k[3]] * fact[k[4]];
                    h[((a * 5 + b) * 5 + c) * 5 + d] = num / fact[k[1] + k[2] + k[3] + k[4] + 3];
                }
    EMG_CUDA(cudaMemcpyToSymbol(emg::c_vcoef, h, sizeof(h)));
    if (dev >= 0 && dev < 64) g_vcoef_ready[dev] = true;
    return EMG_OK;
}

int check_err_flag(int* d_err, cudaStream_t s) {
    int h = 0;
    EMG_CUDA(cudaMemcpyAsync(&h, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    EMG_CUDA(cudaStreamSynchronize(s));
    if (h == 0) return EMG_OK;
    std::string m = "mesh check failed:";
    if (h & ERR_LOCALMAP) m += " an edge/face vertex is not a vertex of its tet;";
    if (h & ERR_PARTNER) m += " a mode-1 DOF pairs with two different mode-2 DOFs;";
    if (h & ERR_ROLE) m += " a DOF is used both as mode-1 and mode-2;";
    if (h & ERR_DOFRANGE) m += " tet_to_field value outside [0, n_field);";
    if (h & ERR_CANDCAP) {
        emg::set_error("an edge or face is shared by more than 64 tetrahedra (limit of the pattern builder)");
        return EMG_ERR_LIMIT;
    }
    emg::set_error(m);
    return EMG_ERR_MESH;
}

}  // namespace

extern "C" int emg_plan_create(int64_t n_nodes, int64_t n_tets, int64_t n_edges, int64_t n_tris, int64_t n_field,
                               const double* nodes, const int32_t* tets, const int32_t* edges, const int32_t* tris,
                               const int32_t* tet_to_field, const int32_t* tet_to_edge, const double* edge_lengths,
                               void* stream, emg_plan** out) {
    using namespace emg;
    EMG_CHECK_ARG(out != nullptr, "emg_plan_create: plan output pointer is NULL");
    *out = nullptr;
    EMG_CHECK_ARG(n_nodes >= 0 && n_tets >= 0 && n_edges >= 0 && n_tris >= 0 && n_field >= 0,
                  "emg_plan_create: negative size");
    EMG_CHECK_ARG(n_field == 2 * n_edges + 2 * n_tris, "emg_plan_create: n_field != 2*n_edges + 2*n_tris");
    EMG_CHECK_ARG(n_field < (int64_t)INT32_MAX && n_tets < ((int64_t)1 << 59),
                  "emg_plan_create: n_field must fit int32");
    EMG_CHECK_ARG(n_tets == 0 || (nodes && tets && edges && tris && tet_to_field && tet_to_edge && edge_lengths),
                  "emg_plan_create: NULL input array");
    cudaStream_t s = (cudaStream_t)stream;
    int rc = upload_vcoef();
    if (rc) return rc;
    emg_plan* p = new emg_plan();
    p->nT = n_tets;
    p->N = n_field;
    const int64_t N = n_field;
    int* d_err = nullptr;
    int32_t *role = nullptr, *cursor = nullptr;
    int64_t *inc_cnt = nullptr, *flag = nullptr, *flag_scan = nullptr, *row_len = nullptr, *scratch = nullptr;
    auto fail = [&](int code) {
        dfree(d_err); dfree(role); dfree(cursor); dfree(inc_cnt); dfree(flag); dfree(flag_scan);
        dfree(row_len); dfree(scratch);
        free_plan(p);
        return code;
    };
#define TRY(x) do { int _r = (x); if (_r) return fail(_r); } while (0)
#define TRYC(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) return fail(cuda_status(_e, #x)); } while (0)
    TRY(dalloc(&d_err, 1, "plan err"));
    TRY(dalloc(&p->partner, N, "partner"));
    TRY(dalloc(&role, N, "role"));
    TRY(dalloc(&inc_cnt, N + 1, "inc_cnt"));
    TRY(dalloc(&flag, N + 1, "flag"));
    TRY(dalloc(&flag_scan, N + 1, "flag_scan"));
    TRY(dalloc(&p->inc_ptr, N + 1, "inc_ptr"));
    TRY(dalloc(&cursor, N, "cursor"));
    TRY(dalloc(&row_len, N + 1, "row_len"));
    TRY(dalloc(&p->indptr, N + 1, "indptr"));
    TRY(dalloc(&scratch, scan_scratch_elems(N + 1) + 1, "scan scratch"));
    TRY(dalloc(&p->inc, n_tets * 10, "incidences"));
    TRYC(cudaMemsetAsync(d_err, 0, sizeof(int), s));
    if (N > 0) {
        TRYC(cudaMemsetAsync(p->partner, 0xff, sizeof(int32_t) * N, s));
        TRYC(cudaMemsetAsync(role, 0, sizeof(int32_t) * N, s));
        TRYC(cudaMemsetAsync(inc_cnt, 0, sizeof(int64_t) * (N + 1), s));
        TRYC(cudaMemsetAsync(cursor, 0, sizeof(int32_t) * N, s));
        TRYC(cudaMemsetAsync(row_len, 0, sizeof(int64_t) * (N + 1), s));
    }
    const int T = 256;
    if (n_tets > 0) {
        k_incidence_count<<<grid_for(n_tets * 10, T), T, 0, s>>>(tet_to_field, n_tets, N, p->partner, role, inc_cnt, d_err);
        TRYC(cudaGetLastError());
        TRY(check_err_flag(d_err, s));
    }
    if (N > 0) {
        k_check_roles<<<grid_for(N, T), T, 0, s>>>(role, N, inc_cnt, flag, d_err);
        TRYC(cudaGetLastError());
    }
    TRY(scan_exclusive_i64(flag, flag_scan, N, scratch, s));
    TRY(scan_exclusive_i64(inc_cnt, p->inc_ptr, N, scratch, s));
    TRYC(cudaMemcpyAsync(&p->n_ent, flag_scan + N, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    TRYC(cudaStreamSynchronize(s));
    TRY(check_err_flag(d_err, s));
    TRY(dalloc(&p->ent_list, p->n_ent, "entity list"));
    if (p->n_ent > 0) {
        k_compact<<<grid_for(N, T), T, 0, s>>>(flag_scan, inc_cnt, N, p->ent_list);
        k_incidence_fill<<<grid_for(n_tets * 10, T), T, 0, s>>>(tet_to_field, n_tets, p->inc_ptr, cursor, p->inc);
        k_incidence_sort<<<grid_for(p->n_ent, T), T, 0, s>>>(p->ent_list, p->n_ent, p->inc_ptr, p->inc);
        const unsigned gp = grid_for(p->n_ent, kFillWarps, 152u * 32u);
        k_pattern<<<gp, 32 * kFillWarps, 0, s>>>(tet_to_field, n_tets, p->ent_list, p->n_ent, p->partner, p->inc_ptr,
                                                 p->inc, 0, row_len, nullptr, nullptr, d_err);
        TRYC(cudaGetLastError());
    }
    TRY(scan_exclusive_i64(row_len, p->indptr, N, scratch, s));
    TRYC(cudaMemcpyAsync(&p->nnz, p->indptr + N, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    TRYC(cudaStreamSynchronize(s));
    TRY(check_err_flag(d_err, s));
    TRY(dalloc(&p->indices, p->nnz, "indices"));
    if (p->n_ent > 0) {
        const unsigned gp = grid_for(p->n_ent, kFillWarps, 152u * 32u);
        k_pattern<<<gp, 32 * kFillWarps, 0, s>>>(tet_to_field, n_tets, p->ent_list, p->n_ent, p->partner, p->inc_ptr,
                                                 p->inc, 1, nullptr, p->indptr, p->indices, d_err);
        TRYC(cudaGetLastError());
    }
    TRY(check_err_flag(d_err, s));
    // fast fill: float-float blocks for entities within its limits
    TRY(df_plan_build(nodes, n_nodes, tets, n_tets, edges, n_edges, tris, n_tris, tet_to_field, tet_to_edge,
                      edge_lengths, p->ent_list, p->n_ent, p->partner, p->inc_ptr, p->inc, 10 * n_tets, p->indptr,
                      p->indices, &p->df, s));
    // FP64 records: the fill of entities outside the fast-fill limits and of tensor materials
    if (n_tets > 0) {
        TRY(dalloc(&p->recs, n_tets, "tet records"));
        k_tet_prep<<<grid_for(n_tets, T), T, 0, s>>>(nodes, n_nodes, tets, n_tets, edges, n_edges, tris, n_tris,
                                                     tet_to_field, tet_to_edge, edge_lengths, p->recs, d_err);
        TRYC(cudaGetLastError());
        TRY(check_err_flag(d_err, s));
    }
    dfree(d_err); dfree(role); dfree(cursor); dfree(inc_cnt); dfree(flag); dfree(flag_scan);
    dfree(row_len); dfree(scratch);
#undef TRY
#undef TRYC
    *out = p;
    return EMG_OK;
}

extern "C" int64_t emg_plan_nnz(const emg_plan* p) { return p ? p->nnz : -1; }

extern "C" int emg_plan_pattern(const emg_plan* p, int64_t* indptr, int32_t* indices, void* stream) {
    EMG_CHECK_ARG(p && indptr && (indices || p->nnz == 0), "emg_plan_pattern: NULL argument");
    cudaStream_t s = (cudaStream_t)stream;
    EMG_CUDA(cudaMemcpyAsync(indptr, p->indptr, sizeof(int64_t) * (p->N + 1), cudaMemcpyDeviceToDevice, s));
    if (p->nnz > 0)
        EMG_CUDA(cudaMemcpyAsync(indices, p->indices, sizeof(int32_t) * p->nnz, cudaMemcpyDeviceToDevice, s));
    return EMG_OK;
}

extern "C" int emg_assemble_tet(emg_plan* p, const double* eps, const double* mu_inv, double* E_data, double* B_data,
                                void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(p != nullptr, "emg_assemble_tet: NULL plan");
    EMG_CHECK_ARG(p->nnz == 0 || (eps && mu_inv && E_data && B_data), "emg_assemble_tet: NULL array");
    if (p->n_ent == 0) return EMG_OK;
    cudaStream_t s = (cudaStream_t)stream;
    int rc = df_fill(p->df, p->nT, p->partner, p->inc_ptr, p->inc, p->indptr, p->indices, eps, mu_inv, E_data, B_data, s);
    if (rc) return rc;
    if (p->df.n_slow > 0) {
        const unsigned g = grid_for(p->df.n_slow, kFillWarps, 152u * 16u);
        k_fill<<<g, 32 * kFillWarps, 0, s>>>(p->recs, p->df.slow, p->df.n_slow, p->partner, p->inc_ptr, p->inc,
                                             p->indptr, p->indices, reinterpret_cast<const double2*>(eps),
                                             reinterpret_cast<const double2*>(mu_inv),
                                             reinterpret_cast<double2*>(E_data), reinterpret_cast<double2*>(B_data));
        EMG_CUDA(cudaGetLastError());
    }
    return EMG_OK;
}

namespace {
// Device address of ``n`` bytes of page-locked host memory at ``h`` (cudaHostAlloc'd or
// registered, mapped into the device's address space), or nullptr when either end of
// the range is not page-locked host memory.
void* mapped_host_range(void* h, size_t n) {
    cudaPointerAttributes a0, a1;
    if (cudaPointerGetAttributes(&a0, h) != cudaSuccess ||
        cudaPointerGetAttributes(&a1, static_cast<char*>(h) + (n - 1)) != cudaSuccess) {
        cudaGetLastError();   // an unknown pointer: clear the error for later calls
        return nullptr;
    }
    if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer || !a1.devicePointer)
        return nullptr;
    if (static_cast<char*>(a1.devicePointer) - static_cast<char*>(a0.devicePointer) != (ptrdiff_t)(n - 1))
        return nullptr;
    return a0.devicePointer;
}
}  // namespace

extern "C" int emg_assemble_tet_host(emg_plan* p, const double* eps, const double* mu_inv, double* E_data,
                                     double* B_data, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(p != nullptr, "emg_assemble_tet_host: NULL plan");
    EMG_CHECK_ARG(p->nnz == 0 || (eps && mu_inv && E_data && B_data), "emg_assemble_tet_host: NULL array");
    cudaStream_t s = (cudaStream_t)stream;
    // Page-locked outputs: the fill stores its write-once values straight into them
    // over the host link, so the element arithmetic overlaps the transfer (the link,
    // not HBM, bounds this call).  Pageable outputs: fill into device staging, then copy.
    const size_t vbytes = sizeof(double) * 2 * (size_t)p->nnz;
    double* Ed = p->nnz > 0 ? static_cast<double*>(mapped_host_range(E_data, vbytes)) : nullptr;
    double* Bd = p->nnz > 0 ? static_cast<double*>(mapped_host_range(B_data, vbytes)) : nullptr;
    const bool direct = Ed && Bd;
    {
        int rc;
        if (!p->eps_dev && (rc = dalloc(&p->eps_dev, 2 * p->nT, "eps staging"))) return rc;
        if (!p->mu_dev && (rc = dalloc(&p->mu_dev, 2 * p->nT, "mu staging"))) return rc;
        if (!direct && !p->E_dev && (rc = dalloc(&p->E_dev, 2 * p->nnz, "E staging"))) return rc;
        if (!direct && !p->B_dev && (rc = dalloc(&p->B_dev, 2 * p->nnz, "B staging"))) return rc;
    }
    if (p->nT > 0) {
        EMG_CUDA(cudaMemcpyAsync(p->eps_dev, eps, sizeof(double) * 2 * p->nT, cudaMemcpyHostToDevice, s));
        EMG_CUDA(cudaMemcpyAsync(p->mu_dev, mu_inv, sizeof(double) * 2 * p->nT, cudaMemcpyHostToDevice, s));
    }
    int rc = emg_assemble_tet(p, p->eps_dev, p->mu_dev, direct ? Ed : p->E_dev, direct ? Bd : p->B_dev, stream);
    if (rc) return rc;
    if (!direct && p->nnz > 0) {
        EMG_CUDA(cudaMemcpyAsync(E_data, p->E_dev, vbytes, cudaMemcpyDeviceToHost, s));
        EMG_CUDA(cudaMemcpyAsync(B_data, p->B_dev, vbytes, cudaMemcpyDeviceToHost, s));
    }
    EMG_CUDA(cudaStreamSynchronize(s));
    return EMG_OK;
}

extern "C" int emg_assemble_tet_tensor(emg_plan* p, const double* eps9, const double* mu_inv9, double* E_data,
                                       double* B_data, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(p != nullptr, "emg_assemble_tet_tensor: NULL plan");
    EMG_CHECK_ARG(p->nnz == 0 || (eps9 && mu_inv9 && E_data && B_data), "emg_assemble_tet_tensor: NULL array");
    if (p->n_ent == 0) return EMG_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (!p->tinv) {
        int rc = dalloc(&p->tinv, p->nT * 2 * kTInv, "tensor invariants");
        if (rc) return rc;
    }
    k_tensor_prep<<<grid_for(p->nT, 128), 128, 0, s>>>(p->recs, p->nT, reinterpret_cast<const double2*>(eps9),
                                                       reinterpret_cast<const double2*>(mu_inv9), p->tinv);
    EMG_CUDA(cudaGetLastError());
    const unsigned g = grid_for(p->n_ent, kFillWarps, 152u * 16u);
    k_fill_tensor<<<g, 32 * kFillWarps, 0, s>>>(p->recs, p->tinv, p->ent_list, p->n_ent, p->partner, p->inc_ptr,
                                                p->inc, p->indptr, p->indices, reinterpret_cast<double2*>(E_data),
                                                reinterpret_cast<double2*>(B_data));
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}

extern "C" int emg_assemble_tet_tensor_host(emg_plan* p, const double* eps9, const double* mu_inv9, double* E_data,
                                            double* B_data, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(p != nullptr, "emg_assemble_tet_tensor_host: NULL plan");
    EMG_CHECK_ARG(p->nnz == 0 || (eps9 && mu_inv9 && E_data && B_data), "emg_assemble_tet_tensor_host: NULL array");
    cudaStream_t s = (cudaStream_t)stream;
    int rc;
    if (!p->eps9_dev && (rc = dalloc(&p->eps9_dev, 18 * p->nT, "eps tensor staging"))) return rc;
    if (!p->mu9_dev && (rc = dalloc(&p->mu9_dev, 18 * p->nT, "mu tensor staging"))) return rc;
    if (!p->E_dev && (rc = dalloc(&p->E_dev, 2 * p->nnz, "E staging"))) return rc;
    if (!p->B_dev && (rc = dalloc(&p->B_dev, 2 * p->nnz, "B staging"))) return rc;
    if (p->nT > 0) {
        EMG_CUDA(cudaMemcpyAsync(p->eps9_dev, eps9, sizeof(double) * 18 * p->nT, cudaMemcpyHostToDevice, s));
        EMG_CUDA(cudaMemcpyAsync(p->mu9_dev, mu_inv9, sizeof(double) * 18 * p->nT, cudaMemcpyHostToDevice, s));
    }
    if ((rc = emg_assemble_tet_tensor(p, p->eps9_dev, p->mu9_dev, p->E_dev, p->B_dev, stream))) return rc;
    if (p->nnz > 0) {
        EMG_CUDA(cudaMemcpyAsync(E_data, p->E_dev, sizeof(double) * 2 * p->nnz, cudaMemcpyDeviceToHost, s));
        EMG_CUDA(cudaMemcpyAsync(B_data, p->B_dev, sizeof(double) * 2 * p->nnz, cudaMemcpyDeviceToHost, s));
    }
    EMG_CUDA(cudaStreamSynchronize(s));
    return EMG_OK;
}

extern "C" void emg_plan_destroy(emg_plan* p) { free_plan(p); }

// ------------------------------------------------- pattern without allocation ---
// emg_csr_pattern_noalloc: the CSR pattern builder of emg_plan_create for callers
// that cannot allocate device memory.  All of its scratch lives in one file-scope
// device array of fixed size, so the entry point calls no cudaMalloc/cudaFree.
#include <mutex>

namespace emg {
namespace {

constexpr int64_t kNoAllocMaxTets = 8192;
constexpr int64_t kNoAllocMaxField = 65536;

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
// byte offsets of the scratch arrays inside g_noalloc_scratch
constexpr size_t kOffErr = 0;
constexpr size_t kOffPartner = align256(kOffErr + sizeof(int));
constexpr size_t kOffRole = align256(kOffPartner + sizeof(int32_t) * kNoAllocMaxField);
constexpr size_t kOffCursor = align256(kOffRole + sizeof(int32_t) * kNoAllocMaxField);
constexpr size_t kOffEntList = align256(kOffCursor + sizeof(int32_t) * kNoAllocMaxField);
constexpr size_t kOffIncCnt = align256(kOffEntList + sizeof(int32_t) * kNoAllocMaxField);
constexpr size_t kOffFlag = align256(kOffIncCnt + sizeof(int64_t) * (kNoAllocMaxField + 1));
constexpr size_t kOffFlagScan = align256(kOffFlag + sizeof(int64_t) * (kNoAllocMaxField + 1));
constexpr size_t kOffIncPtr = align256(kOffFlagScan + sizeof(int64_t) * (kNoAllocMaxField + 1));
constexpr size_t kOffRowLen = align256(kOffIncPtr + sizeof(int64_t) * (kNoAllocMaxField + 1));
constexpr size_t kOffScan = align256(kOffRowLen + sizeof(int64_t) * (kNoAllocMaxField + 1));
constexpr size_t kScanElems = (kNoAllocMaxField + 1 + 4095) / 4096 + 2;
constexpr size_t kOffInc = align256(kOffScan + sizeof(int64_t) * kScanElems);
constexpr size_t kNoAllocBytes = align256(kOffInc + sizeof(int64_t) * 10 * kNoAllocMaxTets);  // ~4.9 MB

// Shared by every call on a device; holds the last call's contents.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mutex;
void* g_noalloc_addr[64] = {nullptr};

// Device address of g_noalloc_scratch on the current device (looked up once per device).
int noalloc_scratch(unsigned char** out) {
    int dev = 0;
    EMG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error("emg_csr_pattern_noalloc: device ordinal >= 64");
        return EMG_ERR_LIMIT;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (g_noalloc_addr[dev] == nullptr) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_noalloc_addr[dev] = p;
    }
    *out = static_cast<unsigned char*>(g_noalloc_addr[dev]);
    return EMG_OK;
}

}  // namespace
}  // namespace emg

extern "C" int emg_csr_pattern_noalloc(int64_t n_tets, int64_t n_field, const int32_t* tet_to_field,
                                       int64_t* indptr, int32_t* indices, int64_t indices_capacity,
                                       int64_t* nnz_out, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(nnz_out != nullptr && indptr != nullptr, "emg_csr_pattern_noalloc: NULL output pointer");
    EMG_CHECK_ARG(n_tets >= 0 && n_field >= 0 && indices_capacity >= 0, "emg_csr_pattern_noalloc: negative size");
    if (n_tets > kNoAllocMaxTets || n_field > kNoAllocMaxField) {
        set_error("emg_csr_pattern_noalloc: mesh too large for the fixed scratch (at most 8192 tets and 65536 "
                  "DOFs); use emg_plan_create");
        return EMG_ERR_LIMIT;
    }
    EMG_CHECK_ARG(n_tets == 0 || tet_to_field != nullptr, "emg_csr_pattern_noalloc: NULL tet_to_field");
    *nnz_out = 0;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char* base = nullptr;
    int rc = noalloc_scratch(&base);
    if (rc) return rc;
    const int64_t N = n_field;
    int* d_err = reinterpret_cast<int*>(base + kOffErr);
    int32_t* partner = reinterpret_cast<int32_t*>(base + kOffPartner);
    int32_t* role = reinterpret_cast<int32_t*>(base + kOffRole);
    int32_t* cursor = reinterpret_cast<int32_t*>(base + kOffCursor);
    int32_t* ent_list = reinterpret_cast<int32_t*>(base + kOffEntList);
    int64_t* inc_cnt = reinterpret_cast<int64_t*>(base + kOffIncCnt);
    int64_t* flag = reinterpret_cast<int64_t*>(base + kOffFlag);
    int64_t* flag_scan = reinterpret_cast<int64_t*>(base + kOffFlagScan);
    int64_t* inc_ptr = reinterpret_cast<int64_t*>(base + kOffIncPtr);
    int64_t* row_len = reinterpret_cast<int64_t*>(base + kOffRowLen);
    int64_t* scan_tmp = reinterpret_cast<int64_t*>(base + kOffScan);
    int64_t* inc = reinterpret_cast<int64_t*>(base + kOffInc);
    // the previous call's contents are still there: reset what the build accumulates into
    EMG_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), s));
    if (N > 0) {
        EMG_CUDA(cudaMemsetAsync(partner, 0xff, sizeof(int32_t) * N, s));
        EMG_CUDA(cudaMemsetAsync(role, 0, sizeof(int32_t) * N, s));
        EMG_CUDA(cudaMemsetAsync(cursor, 0, sizeof(int32_t) * N, s));
        EMG_CUDA(cudaMemsetAsync(inc_cnt, 0, sizeof(int64_t) * (N + 1), s));
        EMG_CUDA(cudaMemsetAsync(row_len, 0, sizeof(int64_t) * (N + 1), s));
    }
    const int T = 256;
    if (n_tets > 0) {
        k_incidence_count<<<grid_for(n_tets * 10, T), T, 0, s>>>(tet_to_field, n_tets, N, partner, role, inc_cnt, d_err);
        EMG_CUDA(cudaGetLastError());
        if ((rc = check_err_flag(d_err, s))) return rc;
    }
    if (N > 0) {
        k_check_roles<<<grid_for(N, T), T, 0, s>>>(role, N, inc_cnt, flag, d_err);
        EMG_CUDA(cudaGetLastError());
    }
    if ((rc = scan_exclusive_i64(flag, flag_scan, N, scan_tmp, s))) return rc;
    if ((rc = scan_exclusive_i64(inc_cnt, inc_ptr, N, scan_tmp, s))) return rc;
    int64_t n_ent = 0;
    EMG_CUDA(cudaMemcpyAsync(&n_ent, flag_scan + N, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    EMG_CUDA(cudaStreamSynchronize(s));
    if ((rc = check_err_flag(d_err, s))) return rc;
    if (n_ent > 0) {
        k_compact<<<grid_for(N, T), T, 0, s>>>(flag_scan, inc_cnt, N, ent_list);
        k_incidence_fill<<<grid_for(n_tets * 10, T), T, 0, s>>>(tet_to_field, n_tets, inc_ptr, cursor, inc);
        k_incidence_sort<<<grid_for(n_ent, T), T, 0, s>>>(ent_list, n_ent, inc_ptr, inc);
        k_pattern<<<grid_for(n_ent, kFillWarps, 152u * 32u), 32 * kFillWarps, 0, s>>>(
            tet_to_field, n_tets, ent_list, n_ent, partner, inc_ptr, inc, 0, row_len, nullptr, nullptr, d_err);
        EMG_CUDA(cudaGetLastError());
    }
    if ((rc = scan_exclusive_i64(row_len, indptr, N, scan_tmp, s))) return rc;
    int64_t nnz = 0;
    EMG_CUDA(cudaMemcpyAsync(&nnz, indptr + N, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    EMG_CUDA(cudaStreamSynchronize(s));
    if ((rc = check_err_flag(d_err, s))) return rc;
    *nnz_out = nnz;
    if (nnz > indices_capacity || (nnz > 0 && indices == nullptr)) {
        set_error("emg_csr_pattern_noalloc: indices capacity " + std::to_string(indices_capacity) +
                  " is smaller than nnz " + std::to_string(nnz));
        return EMG_ERR_LIMIT;
    }
    if (n_ent > 0) {
        k_pattern<<<grid_for(n_ent, kFillWarps, 152u * 32u), 32 * kFillWarps, 0, s>>>(
            tet_to_field, n_tets, ent_list, n_ent, partner, inc_ptr, inc, 1, nullptr, indptr, indices, d_err);
        EMG_CUDA(cudaGetLastError());
    }
    return check_err_flag(d_err, s);
}

// ------------------------------------------------------------ materials ---
namespace emg {
namespace {
__device__ __forceinline__ double2 cmul2(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 csub2(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cadd2(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 crecip(double2 z) {
    const double d = z.x * z.x + z.y * z.y;
    return make_double2(z.x / d, -z.y / d);
}

// matinv (fem/mth/optimized.py:440-461) per tet, thread per tet: a tensor whose six
// off-diagonal entries are all zero gets its reciprocal diagonal; any other gets the
// reference's adj(s) * det(s) (it multiplies by the determinant instead of dividing).
// ncomp 9: s, out are complex (9, n) = the reference's (3,3,n) C order; ncomp 1: complex
// scalars (isotropic tensors s * I), out = 1 / s.
__global__ void k_matinv(int64_t n, int ncomp, const double2* __restrict__ s9, double2* __restrict__ o9) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        if (ncomp == 1) {
            o9[t] = crecip(s9[t]);
            continue;
        }
        double2 a[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) a[i][j] = s9[(i * 3 + j) * n + t];
        bool diag = true;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                if (i != j && (a[i][j].x != 0.0 || a[i][j].y != 0.0)) diag = false;
        double2 o[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) o[i][j] = make_double2(0.0, 0.0);
        if (diag) {
            for (int i = 0; i < 3; ++i) o[i][i] = crecip(a[i][i]);
        } else {
            // det and adjugate in the reference's term order
            double2 det = cmul2(cmul2(a[0][0], a[1][1]), a[2][2]);
            det = csub2(det, cmul2(cmul2(a[0][0], a[1][2]), a[2][1]));
            det = csub2(det, cmul2(cmul2(a[0][1], a[1][0]), a[2][2]));
            det = cadd2(det, cmul2(cmul2(a[0][1], a[1][2]), a[2][0]));
            det = cadd2(det, cmul2(cmul2(a[0][2], a[1][0]), a[2][1]));
            det = csub2(det, cmul2(cmul2(a[0][2], a[1][1]), a[2][0]));
            const double2 neg = make_double2(-1.0, 0.0);
            o[0][0] = csub2(cmul2(a[1][1], a[2][2]), cmul2(a[1][2], a[2][1]));
            o[0][1] = cadd2(cmul2(cmul2(neg, a[0][1]), a[2][2]), cmul2(a[0][2], a[2][1]));
            o[0][2] = csub2(cmul2(a[0][1], a[1][2]), cmul2(a[0][2], a[1][1]));
            o[1][0] = cadd2(cmul2(cmul2(neg, a[1][0]), a[2][2]), cmul2(a[1][2], a[2][0]));
            o[1][1] = csub2(cmul2(a[0][0], a[2][2]), cmul2(a[0][2], a[2][0]));
            o[1][2] = cadd2(cmul2(cmul2(neg, a[0][0]), a[1][2]), cmul2(a[0][2], a[1][0]));
            o[2][0] = csub2(cmul2(a[1][0], a[2][1]), cmul2(a[1][1], a[2][0]));
            o[2][1] = cadd2(cmul2(cmul2(neg, a[0][0]), a[2][1]), cmul2(a[0][1], a[2][0]));
            o[2][2] = csub2(cmul2(a[0][0], a[1][1]), cmul2(a[0][1], a[1][0]));
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) o[i][j] = cmul2(o[i][j], det);
        }
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) o9[(i * 3 + j) * n + t] = o[i][j];
    }
}
}  // namespace
}  // namespace emg

extern "C" int emg_matinv(int64_t n_tets, int ncomp, const double* s, double* out, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(n_tets >= 0 && (ncomp == 1 || ncomp == 9), "emg_matinv: bad size or ncomp (1 or 9)");
    if (n_tets == 0) return EMG_OK;
    EMG_CHECK_ARG(s != nullptr && out != nullptr, "emg_matinv: NULL array");
    k_matinv<<<grid_for(n_tets, 256), 256, 0, (cudaStream_t)stream>>>(n_tets, ncomp, reinterpret_cast<const double2*>(s),
                                                                      reinterpret_cast<double2*>(out));
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}
