// Restricted system plan and the preconditioner-generic GMRES driver shared by
// the ILU(0) path (emg_krylov.cu) and the slab factorization (emg_slab.cu).
#pragma once

#include <vector>

#include "emg_common.cuh"

struct emg_rplan {
    int64_t N = 0, ns = 0, nnz = 0, nnz_full = 0;
    int64_t* sid = nullptr;       // solve ids (ns)
    int32_t* map = nullptr;       // full -> restricted (N), -1 if removed
    int64_t* rptr = nullptr;      // (ns+1)
    int32_t* rind = nullptr;      // (nnz)
    int64_t* rsrc = nullptr;      // (nnz) positions in the full pattern
    int64_t* rdiag = nullptr;     // (ns)
    int64_t* uptr = nullptr;      // (ns+1) factorization update lists
    int64_t* ulist = nullptr;     // pairs (kk_local << 32 | pos in row k, target pos)
    int32_t* lrows = nullptr;     // rows by forward level
    int32_t* urows = nullptr;     // rows by backward level
    std::vector<int64_t> lptr, uptr_lv;   // level boundaries (host)
    // GMRES workspace (grown on demand)
    size_t ws_bytes = 0;
    void* ws = nullptr;
    // private stream for graph capture of the Arnoldi step (the caller's stream may be
    // the legacy default stream, which cannot be captured)
    cudaStream_t gs = nullptr;
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
};

namespace emg {

// Right preconditioner M^-1 applied to Bc columns (vectors [n][Bc], complex
// double).  prepare() runs before any stream capture and does every allocation;
// apply() is captured into CUDA graphs, so it may only enqueue work on ``s``.
struct Precond {
    virtual ~Precond() = default;
    virtual int prepare(int64_t Bc) { (void)Bc; return EMG_OK; }
    virtual int apply(const double2* in, double2* out, cudaStream_t s) = 0;   // in and out do not alias
};

// The operator of column c: either stored matrix cmat[c] of A ([nnz][Bm]), or a
// matrix family sum_a coef[c][a] fam[a] (fam: [nfam][nnz], coef: [Bc][nfam], device)
// formed on the fly inside the product, e.g. A(k) = E - k^2 B + sum_p gamma_p P_p.
constexpr int kMaxFamily = 8;
struct MatArg {
    const double2* A = nullptr;
    int64_t Bm = 0;
    const int32_t* cmat = nullptr;
    int nfam = 0;
    const double2* fam = nullptr;
    const double2* coef = nullptr;
};

// Y = A X, or Y = Bv - A X when Bv is not NULL (vectors [n][Bc]).
void spmv_op(const emg_rplan* p, int64_t Bc, const MatArg& A, const double2* X, const double2* Bv, double2* Y,
             cudaStream_t s);

// Restarted GMRES(restart) with CGS2 over Bc lockstep columns.  flexible: keep
// z_j = M^-1 v_j and update x with them (FGMRES, required when M^-1 is not an exact
// fixed linear map, e.g. a reduced-precision factorization); otherwise
// x += M^-1 (V y).
int gmres_run(emg_rplan* p, int64_t Bc, const MatArg& A, const double2* rhs, double2* x, int restart, int max_iter,
              double tol, int32_t* iters_out, double* resid_out, cudaStream_t caller, Precond& M, bool flexible);

// Complex slab product on the tcgen05 tensor cores (TF32 products, FP32 accumulation;
// emg_tc.cu): Out[row0 + r, cols of group] = alpha S_g[r, :] Y[row0 + :, cols] + beta
// Out for the 16-byte group records {factor, col0, ncol, pad}; status (device) set
// to 1 if a bounded wait ran out.
int tc_slab_product(int64_t w, int64_t row0, int64_t Bc, const void* groups, int G, int maxcol, const float2* Sinv,
                    int64_t totD, int64_t offD, const float2* Y, float alpha, int beta, float2* Out, int32_t* status,
                    cudaStream_t st);

// Rank-64 update of Gauss-Jordan step k on the tcgen05 tensor cores in FP32-equivalent
// precision (split-TF32 products, FP32 accumulation; emg_tc.cu): M[r, c] -= M[r, K]
// M[K, c] for the F complex64 w x w blocks Sinv + f totD + offD, rows and columns of
// tile k excluded, tile (la, la) excluded when la >= 0; status (device) set to 1 if a
// bounded wait ran out.
int tc_gj_update(int64_t w, int k, int la, int64_t F, float2* Sinv, int64_t totD, int64_t offD, int32_t* status,
                 cudaStream_t st);

// Preconditioner on FP32 vectors (the inner solves of the mixed-precision refinement).
struct Precond32 {
    virtual ~Precond32() = default;
    virtual int prepare(int64_t Bc) { (void)Bc; return EMG_OK; }
    virtual int apply(const float2* in, float2* out, cudaStream_t s) = 0;   // in and out do not alias
};

// Mixed-precision solve: FP64 iterative refinement around inner FGMRES(restart)
// iterations on FP32 vectors with the FP32 copy A32 of the stored matrices (same
// [nnz][Bm] layout and cmat).  Each refinement step forms the true residual in
// FP64, scales each column to unit norm, solves A32 d = r to ``inner_tol`` in FP32
// and adds ||r|| d to x.  iters_out: inner iterations summed over the steps.
int ir_run(emg_rplan* p, int64_t Bc, const MatArg& A, const float2* A32, const double2* rhs, double2* x, int restart,
           int max_iter, double tol, double inner_tol, int32_t* iters_out, double* resid_out, int32_t* steps_out,
           cudaStream_t caller, Precond32& M);

}  // namespace emg
