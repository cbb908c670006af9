// Restricted frequency-domain systems and a batched ILU(0)-preconditioned GMRES.
//
// Replaces the solve behind SolveRoutine.solve (fem/solver.py:405-469):
//   A[ix_(solve_ids, solve_ids)] restriction (solver.py:434-435), the linear
//   solve itself (SuperLU/PARDISO/GMRES, solver.py:220-309), and the scatter of
//   the solution back to all DOFs with zeros on PEC DOFs (solver.py:465).
//
// Batching: B right-hand-side columns are solved in lockstep; column c uses
// matrix cmat[c] of Bm stored matrices.  A frequency sweep stores one matrix per
// frequency, A(k) = E - k^2 B + sum_p gamma_p(k) P_p, formed from the volume
// matrices and unit port matrices (every Robin block is linear in gamma), with
// one column per (frequency, port).  Layouts put the batch index innermost so
// that threads of a warp handle neighbouring columns of the same row and all
// loads are coalesced: matrices [nnz][Bm], vectors [n][B] (complex double2).
//
// ILU(0) is level-scheduled: row i of L depends on the rows j < i it references,
// so the rows of one level are factored/solved in parallel, one launch per
// level.  The factorization update lists (which entries of row i row k of U
// updates) are built once per pattern on the host.
#include <algorithm>
#include <vector>

#include "emg_krylov.cuh"

namespace emg {
namespace kry {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) { return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x); }  // conj(a)*b
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
    const double d = b.x * b.x + b.y * b.y;
    return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }

// restricted pattern: count kept entries of each kept row
__global__ void k_rcount(int64_t ns, const int64_t* __restrict__ sid, const int64_t* __restrict__ indptr,
                         const int32_t* __restrict__ indices, const int32_t* __restrict__ map, int64_t* cnt) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < ns; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = sid[r];
        int64_t c = 0;
        for (int64_t k = indptr[row]; k < indptr[row + 1]; ++k) c += map[indices[k]] >= 0;
        cnt[r] = c;
    }
}

__global__ void k_rwrite(int64_t ns, const int64_t* __restrict__ sid, const int64_t* __restrict__ indptr,
                         const int32_t* __restrict__ indices, const int32_t* __restrict__ map,
                         const int64_t* __restrict__ rptr, int32_t* rind, int64_t* rsrc, int64_t* rdiag) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < ns; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = sid[r];
        int64_t o = rptr[r];
        rdiag[r] = -1;
        for (int64_t k = indptr[row]; k < indptr[row + 1]; ++k) {
            const int32_t m = map[indices[k]];
            if (m < 0) continue;
            rind[o] = m;
            rsrc[o] = k;
            if (m == r) rdiag[r] = o;
            ++o;
        }
    }
}

__global__ void k_map(int64_t ns, const int64_t* __restrict__ sid, int32_t* map) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < ns; r += (int64_t)gridDim.x * blockDim.x)
        map[sid[r]] = (int32_t)r;
}

// A[k][m] = E[s] - k2[m] B[s] + sum_p gam[p][m] P[p][s],  s = src[k]
__global__ void k_form(int64_t nnz_r, int64_t Bm, const int64_t* __restrict__ src, const double2* __restrict__ E,
                       const double2* __restrict__ B, const double* __restrict__ k2, int64_t n_ports,
                       const double2* __restrict__ P, int64_t nnz_full, const double2* __restrict__ gam,
                       double2* __restrict__ A) {
    const int64_t total = nnz_r * Bm;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = t / Bm, m = t % Bm;
        const int64_t s = src[k];
        const double2 e = E[s], b = B[s];
        double2 v = make_double2(e.x - k2[m] * b.x, e.y - k2[m] * b.y);
        for (int64_t p = 0; p < n_ports; ++p) v = cadd(v, cmul(gam[p * Bm + m], P[p * nnz_full + s]));
        A[t] = v;
    }
}

// ILU(0) of the rows of one level, thread per (row, matrix).  For row i, in column
// order: a_ik /= a_kk for each k < i, then a_ij -= a_ik a_kj over the update list.
__global__ void k_ilu_level(int64_t nrows, const int32_t* __restrict__ rows, int64_t Bm,
                            const int64_t* __restrict__ rptr, const int32_t* __restrict__ rind,
                            const int64_t* __restrict__ rdiag, const int64_t* __restrict__ uptr,
                            const int64_t* __restrict__ ulist, double2* __restrict__ LU) {
    const int64_t total = nrows * Bm;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = rows[t / Bm], m = t % Bm;
        int64_t u = uptr[i];
        for (int64_t kk = rptr[i]; kk < rdiag[i]; ++kk) {
            const int32_t k = rind[kk];
            const double2 l = cdiv(LU[kk * Bm + m], LU[rdiag[k] * Bm + m]);
            LU[kk * Bm + m] = l;
            // update list entries for this kk: pairs (source position in row k, target in row i)
            while (u < uptr[i + 1] && ulist[2 * u] >> 32 == kk - rptr[i]) {
                const int64_t sk = ulist[2 * u] & 0xffffffffll, ti = ulist[2 * u + 1];
                LU[ti * Bm + m] = csub(LU[ti * Bm + m], cmul(l, LU[sk * Bm + m]));
                ++u;
            }
        }
    }
}

// Level of forward (L) or backward (U) substitution: thread per (row, column).
__global__ void k_trsv_level(int64_t nrows, const int32_t* __restrict__ rows, int64_t Bc, const int32_t* __restrict__ cmat,
                             int64_t Bm, const int64_t* __restrict__ rptr, const int32_t* __restrict__ rind,
                             const int64_t* __restrict__ rdiag, const double2* __restrict__ LU, int upper,
                             double2* __restrict__ X) {
    const int64_t total = nrows * Bc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = rows[t / Bc], c = t % Bc;
        const int64_t m = cmat[c];
        double2 s = X[i * Bc + c];
        if (!upper) {
            for (int64_t k = rptr[i]; k < rdiag[i]; ++k) s = csub(s, cmul(LU[k * Bm + m], X[(int64_t)rind[k] * Bc + c]));
            X[i * Bc + c] = s;
        } else {
            for (int64_t k = rdiag[i] + 1; k < rptr[i + 1]; ++k) s = csub(s, cmul(LU[k * Bm + m], X[(int64_t)rind[k] * Bc + c]));
            X[i * Bc + c] = cdiv(s, LU[rdiag[i] * Bm + m]);
        }
    }
}

// Small batches (Bc <= kSmallBc): warp per row, lanes over the row's nonzeros.
constexpr int kSmallBc = 8;
__global__ void k_trsv_level_w(int64_t nrows, const int32_t* __restrict__ rows, int64_t Bc,
                               const int32_t* __restrict__ cmat, int64_t Bm, const int64_t* __restrict__ rptr,
                               const int32_t* __restrict__ rind, const int64_t* __restrict__ rdiag,
                               const double2* __restrict__ LU, int upper, double2* __restrict__ X) {
    const int64_t wid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (wid >= nrows) return;
    const int64_t i = rows[wid];
    const int64_t k0 = upper ? rdiag[i] + 1 : rptr[i], k1 = upper ? rptr[i + 1] : rdiag[i];
    double2 acc[kSmallBc];
#pragma unroll
    for (int c = 0; c < kSmallBc; ++c) acc[c] = make_double2(0.0, 0.0);
    for (int64_t k = k0 + lane; k < k1; k += 32) {
        const int64_t col = rind[k];
#pragma unroll
        for (int c = 0; c < kSmallBc; ++c)
            if (c < Bc) acc[c] = cadd(acc[c], cmul(LU[k * Bm + cmat[c]], X[col * Bc + c]));
    }
#pragma unroll
    for (int c = 0; c < kSmallBc; ++c) {
        if (c >= Bc) break;
        double2 v = acc[c];
        for (int o = 16; o > 0; o >>= 1) {
            v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
            v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
        }
        if (lane == 0) {
            const double2 s = csub(X[i * Bc + c], v);
            X[i * Bc + c] = upper ? cdiv(s, LU[rdiag[i] * Bm + cmat[c]]) : s;
        }
    }
}

__global__ void k_spmv_w(int64_t n, int64_t Bc, const int32_t* __restrict__ cmat, int64_t Bm,
                         const int64_t* __restrict__ rptr, const int32_t* __restrict__ rind, const double2* __restrict__ A,
                         const double2* __restrict__ X, const double2* __restrict__ Bv, double2* __restrict__ Y) {
    const int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= n) return;
    double2 acc[kSmallBc];
#pragma unroll
    for (int c = 0; c < kSmallBc; ++c) acc[c] = make_double2(0.0, 0.0);
    for (int64_t k = rptr[i] + lane; k < rptr[i + 1]; k += 32) {
        const int64_t col = rind[k];
#pragma unroll
        for (int c = 0; c < kSmallBc; ++c)
            if (c < Bc) acc[c] = cadd(acc[c], cmul(A[k * Bm + cmat[c]], X[col * Bc + c]));
    }
#pragma unroll
    for (int c = 0; c < kSmallBc; ++c) {
        if (c >= Bc) break;
        double2 v = acc[c];
        for (int o = 16; o > 0; o >>= 1) {
            v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
            v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
        }
        if (lane == 0) Y[i * Bc + c] = Bv ? csub(Bv[i * Bc + c], v) : v;
    }
}

// Y = A X (batched, thread per (row, column)); alpha*A X + beta*Y when add.
__global__ void k_spmv(int64_t n, int64_t Bc, const int32_t* __restrict__ cmat, int64_t Bm,
                       const int64_t* __restrict__ rptr, const int32_t* __restrict__ rind, const double2* __restrict__ A,
                       const double2* __restrict__ X, const double2* __restrict__ Bv, double2* __restrict__ Y) {
    const int64_t total = n * Bc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / Bc, c = t % Bc;
        const int64_t m = cmat[c];
        double2 s = make_double2(0.0, 0.0);
        for (int64_t k = rptr[i]; k < rptr[i + 1]; ++k) s = cadd(s, cmul(A[k * Bm + m], X[(int64_t)rind[k] * Bc + c]));
        // Bv != nullptr: Y = Bv - A X (residual)
        Y[t] = Bv ? csub(Bv[t], s) : s;
    }
}

// Y = A_c X with A_c = sum_a coef[c][a] fam[a] formed on the fly (thread per (row,
// column); the family values of a row are shared by the warp's columns).
__global__ void k_spmv_fam(int64_t n, int64_t nnz, int64_t Bc, int nfam, const double2* __restrict__ fam,
                           const double2* __restrict__ coef, const int64_t* __restrict__ rptr,
                           const int32_t* __restrict__ rind, const double2* __restrict__ X,
                           const double2* __restrict__ Bv, double2* __restrict__ Y) {
    const int64_t total = n * Bc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / Bc, c = t % Bc;
        double2 cf[kMaxFamily];
#pragma unroll
        for (int a = 0; a < kMaxFamily; ++a) cf[a] = a < nfam ? coef[c * nfam + a] : make_double2(0.0, 0.0);
        double2 s = make_double2(0.0, 0.0);
        for (int64_t k = rptr[i]; k < rptr[i + 1]; ++k) {
            double2 v = make_double2(0.0, 0.0);
#pragma unroll
            for (int a = 0; a < kMaxFamily; ++a)
                if (a < nfam) v = cadd(v, cmul(cf[a], fam[a * nnz + k]));
            s = cadd(s, cmul(v, X[(int64_t)rind[k] * Bc + c]));
        }
        Y[t] = Bv ? csub(Bv[t], s) : s;
    }
}

// Column-wise partial dots: part[blk][j][c] = sum_{rows in blk} conj(V_j[r,c]) W[r,c], j < nj.
constexpr int kDotRows = 1024;
constexpr int kMaxRestart = 256;
__global__ void k_dots_partial(int64_t n, int64_t Bc, int nj, const double2* __restrict__ V, int64_t vstride,
                               const double2* __restrict__ W, double2* __restrict__ part) {
    const int64_t c = blockIdx.y * (int64_t)blockDim.x + threadIdx.x;
    if (c >= Bc) return;
    const int64_t r0 = (int64_t)blockIdx.x * kDotRows, r1 = min(n, r0 + kDotRows);
    for (int j = 0; j < nj; ++j) {
        double2 s = make_double2(0.0, 0.0);
        const double2* Vj = V + j * vstride;
        for (int64_t r = r0; r < r1; ++r) s = cadd(s, cmulc(Vj[r * Bc + c], W[r * Bc + c]));
        part[((int64_t)blockIdx.x * nj + j) * Bc + c] = s;
    }
}

// Small batches (Bc < 32): warp per (vector j, column c) pair, lanes over rows.
__global__ void k_dots_partial_small(int64_t n, int64_t Bc, int nj, const double2* __restrict__ V, int64_t vstride,
                                     const double2* __restrict__ W, double2* __restrict__ part) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int64_t r0 = (int64_t)blockIdx.x * kDotRows, r1 = min(n, r0 + kDotRows);
    for (int64_t pr = warp; pr < (int64_t)nj * Bc; pr += nw) {
        const int64_t j = pr / Bc, c = pr % Bc;
        const double2* Vj = V + j * vstride;
        double2 s = make_double2(0.0, 0.0);
        for (int64_t r = r0 + lane; r < r1; r += 32) s = cadd(s, cmulc(Vj[r * Bc + c], W[r * Bc + c]));
        for (int o = 16; o > 0; o >>= 1) {
            s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
            s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
        }
        if (lane == 0) part[((int64_t)blockIdx.x * nj + j) * Bc + c] = s;
    }
}

__global__ void k_dots_final(int64_t nblk, int64_t Bc, int nj, const double2* __restrict__ part, double2* __restrict__ out) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)nj * Bc) return;
    const int64_t j = t / Bc, c = t % Bc;
    double2 s = make_double2(0.0, 0.0);
    for (int64_t b = 0; b < nblk; ++b) s = cadd(s, part[(b * nj + j) * Bc + c]);
    out[t] = s;
}

// W[r,c] -= sum_j h[j][c] V_j[r,c]   (masked columns untouched)
__global__ void k_orth_update(int64_t n, int64_t Bc, int nj, const double2* __restrict__ V, int64_t vstride,
                              const double2* __restrict__ h, const int32_t* __restrict__ active, double2* __restrict__ W) {
    const int64_t total = n * Bc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = t % Bc;
        if (!active[c]) continue;
        double2 w = W[t];
        for (int j = 0; j < nj; ++j) w = csub(w, cmul(h[(int64_t)j * Bc + c], V[j * vstride + t]));
        W[t] = w;
    }
}

// V_out[r,c] = W[r,c] * scale[c]
__global__ void k_scale_cols(int64_t n, int64_t Bc, const double* __restrict__ scale, const double2* __restrict__ W,
                             double2* __restrict__ Vout) {
    const int64_t total = n * Bc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const double s = scale[t % Bc];
        const double2 w = W[t];
        Vout[t] = make_double2(w.x * s, w.y * s);
    }
}

// X[r,c] += sum_j y[j][c] Z_j[r,c]   (masked by ``has``: columns with a nonzero update length)
__global__ void k_combine_basis(int64_t n, int64_t Bc, int nj, const double2* __restrict__ Z, int64_t zstride,
                                const double2* __restrict__ y, double2* __restrict__ X) {
    const int64_t total = n * Bc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = t % Bc;
        double2 x = X[t];
        for (int j = 0; j < nj; ++j) x = cadd(x, cmul(y[(int64_t)j * Bc + c], Z[j * zstride + t]));
        X[t] = x;
    }
}

// Per column Arnoldi step bookkeeping (thread per column): append column j of H
// (h[0..j] from two Gram-Schmidt passes, hn = ||w||), apply the stored Givens
// rotations, make the new one, update g, decide convergence.
__global__ void k_arnoldi_col(int64_t Bc, int j, int m, const double2* __restrict__ h1, const double2* __restrict__ h2,
                              const double* __restrict__ wnorm2, double2* __restrict__ H, double2* __restrict__ cs,
                              double2* __restrict__ sn, double2* __restrict__ g, const double* __restrict__ bnorm,
                              double tol, int32_t* active, int32_t* len, double* vscale, double* resid) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= Bc) return;
    if (!active[c]) { vscale[c] = 0.0; return; }
    // column j of H: entries 0..j, then the subdiagonal
    double2 col[kMaxRestart + 1];
    for (int i = 0; i <= j; ++i) col[i] = cadd(h1[(int64_t)i * Bc + c], h2[(int64_t)i * Bc + c]);
    const double hn = sqrt(fmax(wnorm2[c], 0.0));
    col[j + 1] = make_double2(hn, 0.0);
    for (int i = 0; i < j; ++i) {
        const double2 ci = cs[(int64_t)i * Bc + c], si = sn[(int64_t)i * Bc + c];
        // [c  s; -conj(s) c] with real-valued c stored in .x
        const double2 a = col[i], b = col[i + 1];
        col[i] = cadd(make_double2(ci.x * a.x, ci.x * a.y), cmul(si, b));
        col[i + 1] = csub(make_double2(ci.x * b.x, ci.x * b.y), cmulc(si, a));
    }
    const double2 a = col[j], b = col[j + 1];
    const double na = sqrt(a.x * a.x + a.y * a.y), nb = sqrt(b.x * b.x + b.y * b.y);
    double cr;
    double2 s;
    if (nb == 0.0) { cr = 1.0; s = make_double2(0.0, 0.0); }
    else if (na == 0.0) { cr = 0.0; s = make_double2(1.0, 0.0); }
    else {
        const double nr = sqrt(na * na + nb * nb);
        cr = na / nr;
        // s = (a/|a|) * conj(b) / nr
        const double2 ua = make_double2(a.x / na, a.y / na);
        s = cmul(ua, make_double2(b.x / nr, -b.y / nr));
    }
    cs[(int64_t)j * Bc + c] = make_double2(cr, 0.0);
    sn[(int64_t)j * Bc + c] = s;
    col[j] = cadd(make_double2(cr * a.x, cr * a.y), cmul(s, b));
    col[j + 1] = make_double2(0.0, 0.0);
    for (int i = 0; i <= j; ++i) H[((int64_t)i * m + j) * Bc + c] = col[i];
    const double2 gj = g[(int64_t)j * Bc + c];
    g[(int64_t)j * Bc + c] = make_double2(cr * gj.x, cr * gj.y);
    g[(int64_t)(j + 1) * Bc + c] = make_double2(-(s.x * gj.x + s.y * gj.y), -(s.x * gj.y - s.y * gj.x));  // -conj(s)*g
    const double2 gn = g[(int64_t)(j + 1) * Bc + c];
    const double rn = sqrt(gn.x * gn.x + gn.y * gn.y);
    resid[c] = rn / bnorm[c];
    len[c] = j + 1;
    vscale[c] = hn > 0.0 ? 1.0 / hn : 0.0;
    if (rn <= tol * bnorm[c] || hn == 0.0) active[c] = 0;
}

// Back substitution H y = g per column (thread per column), lengths len[c].
__global__ void k_backsolve(int64_t Bc, int m, const double2* __restrict__ H, const double2* __restrict__ g,
                            const int32_t* __restrict__ len, double2* __restrict__ y, int nmax) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= Bc) return;
    const int L = len[c];
    for (int i = nmax - 1; i >= 0; --i) {
        if (i >= L) { y[(int64_t)i * Bc + c] = make_double2(0.0, 0.0); continue; }
        double2 s = g[(int64_t)i * Bc + c];
        for (int k = i + 1; k < L; ++k) s = csub(s, cmul(H[((int64_t)i * m + k) * Bc + c], y[(int64_t)k * Bc + c]));
        y[(int64_t)i * Bc + c] = cdiv(s, H[((int64_t)i * m + i) * Bc + c]);
    }
}

// Per column: norms from the dots (|.|^2 sums), set up a restart: bnorm, g0, V0 scale, active.
__global__ void k_restart_cols(int64_t Bc, const double2* __restrict__ rr, const double* __restrict__ bnorm, double tol,
                               double2* __restrict__ g, double* __restrict__ vscale, int32_t* active, int32_t* len,
                               double* resid, int64_t gstride) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= Bc) return;
    const double rn = sqrt(fmax(rr[c].x, 0.0));
    resid[c] = bnorm[c] > 0 ? rn / bnorm[c] : 0.0;
    len[c] = 0;
    const bool act = rn > tol * bnorm[c] && bnorm[c] > 0;
    active[c] = act ? 1 : 0;
    g[c] = make_double2(rn, 0.0);
    for (int64_t i = 1; i < gstride; ++i) g[i * Bc + c] = make_double2(0.0, 0.0);
    vscale[c] = act ? 1.0 / rn : 0.0;
}

__global__ void k_gather_rhs(int64_t ns, int64_t Bc, const int64_t* __restrict__ sid, int64_t N,
                             const double2* __restrict__ full, double2* __restrict__ out) {
    const int64_t total = ns * Bc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / Bc, c = t % Bc;
        out[t] = full[c * N + sid[i]];
    }
}

__global__ void k_scatter_sol(int64_t ns, int64_t Bc, const int64_t* __restrict__ sid, int64_t N,
                              const double2* __restrict__ x, double2* __restrict__ full) {
    const int64_t total = ns * Bc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / Bc, c = t % Bc;
        full[c * N + sid[i]] = x[t];
    }
}

__global__ void k_axpy1(int64_t nv, const double2* __restrict__ d, double2* __restrict__ x) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nv; t += (int64_t)gridDim.x * blockDim.x)
        x[t] = cadd(x[t], d[t]);
}

__global__ void k_real(int64_t Bc, const double2* __restrict__ in, double* __restrict__ out) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c < Bc) out[c] = in[c].x;
}

__global__ void k_sqrt_real(int64_t Bc, const double2* __restrict__ in, double* __restrict__ out) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c < Bc) out[c] = sqrt(fmax(in[c].x, 0.0));
}

// ---- FP32-vector kernels for the inner solves of the mixed-precision refinement ----
__device__ __forceinline__ float2 fmulc(float2 a, float2 b) { return make_float2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x); }
__device__ __forceinline__ void ffma(float2& acc, float2 a, float2 b) {
    acc.x = fmaf(a.x, b.x, acc.x);
    acc.x = fmaf(-a.y, b.y, acc.x);
    acc.y = fmaf(a.x, b.y, acc.y);
    acc.y = fmaf(a.y, b.x, acc.y);
}

__global__ void k_spmv32(int64_t n, int64_t Bc, const int32_t* __restrict__ cmat, int64_t Bm,
                         const int64_t* __restrict__ rptr, const int32_t* __restrict__ rind, const float2* __restrict__ A,
                         const float2* __restrict__ X, const float2* __restrict__ Bv, float2* __restrict__ Y) {
    const int64_t total = n * Bc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / Bc, c = t % Bc;
        const int64_t m = cmat[c];
        float2 s = make_float2(0.f, 0.f);
        for (int64_t k = rptr[i]; k < rptr[i + 1]; ++k) ffma(s, A[k * Bm + m], X[(int64_t)rind[k] * Bc + c]);
        Y[t] = Bv ? make_float2(Bv[t].x - s.x, Bv[t].y - s.y) : s;
    }
}

__global__ void k_spmv32_w(int64_t n, int64_t Bc, const int32_t* __restrict__ cmat, int64_t Bm,
                           const int64_t* __restrict__ rptr, const int32_t* __restrict__ rind, const float2* __restrict__ A,
                           const float2* __restrict__ X, const float2* __restrict__ Bv, float2* __restrict__ Y) {
    const int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= n) return;
    float2 acc[kSmallBc];
#pragma unroll
    for (int c = 0; c < kSmallBc; ++c) acc[c] = make_float2(0.f, 0.f);
    for (int64_t k = rptr[i] + lane; k < rptr[i + 1]; k += 32) {
        const int64_t col = rind[k];
#pragma unroll
        for (int c = 0; c < kSmallBc; ++c)
            if (c < Bc) ffma(acc[c], A[k * Bm + cmat[c]], X[col * Bc + c]);
    }
#pragma unroll
    for (int c = 0; c < kSmallBc; ++c) {
        if (c >= Bc) break;
        float2 v = acc[c];
        for (int o = 16; o > 0; o >>= 1) {
            v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
            v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
        }
        if (lane == 0) Y[i * Bc + c] = Bv ? make_float2(Bv[i * Bc + c].x - v.x, Bv[i * Bc + c].y - v.y) : v;
    }
}

// partial dots over kDotRows rows: FP32 products and running sums, FP64 block partials
__global__ void k_dots32(int64_t n, int64_t Bc, int nj, const float2* __restrict__ V, int64_t vstride,
                         const float2* __restrict__ W, double2* __restrict__ part) {
    const int64_t c = blockIdx.y * (int64_t)blockDim.x + threadIdx.x;
    if (c >= Bc) return;
    const int64_t r0 = (int64_t)blockIdx.x * kDotRows, r1 = min(n, r0 + kDotRows);
    for (int j = 0; j < nj; ++j) {
        float2 s = make_float2(0.f, 0.f);
        const float2* Vj = V + j * vstride;
        for (int64_t r = r0; r < r1; ++r) {
            const float2 p = fmulc(Vj[r * Bc + c], W[r * Bc + c]);
            s.x += p.x;
            s.y += p.y;
        }
        part[((int64_t)blockIdx.x * nj + j) * Bc + c] = make_double2(s.x, s.y);
    }
}

__global__ void k_dots32_small(int64_t n, int64_t Bc, int nj, const float2* __restrict__ V, int64_t vstride,
                               const float2* __restrict__ W, double2* __restrict__ part) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int64_t r0 = (int64_t)blockIdx.x * kDotRows, r1 = min(n, r0 + kDotRows);
    for (int64_t pr = warp; pr < (int64_t)nj * Bc; pr += nw) {
        const int64_t j = pr / Bc, c = pr % Bc;
        const float2* Vj = V + j * vstride;
        float2 s = make_float2(0.f, 0.f);
        for (int64_t r = r0 + lane; r < r1; r += 32) {
            const float2 p = fmulc(Vj[r * Bc + c], W[r * Bc + c]);
            s.x += p.x;
            s.y += p.y;
        }
        for (int o = 16; o > 0; o >>= 1) {
            s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
            s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
        }
        if (lane == 0) part[((int64_t)blockIdx.x * nj + j) * Bc + c] = make_double2(s.x, s.y);
    }
}

__global__ void k_orth32(int64_t n, int64_t Bc, int nj, const float2* __restrict__ V, int64_t vstride,
                         const double2* __restrict__ h, const int32_t* __restrict__ active, float2* __restrict__ W) {
    const int64_t total = n * Bc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = t % Bc;
        if (!active[c]) continue;
        float2 w = W[t];
        for (int j = 0; j < nj; ++j) {
            const double2 hj = h[(int64_t)j * Bc + c];
            ffma(w, make_float2(-(float)hj.x, -(float)hj.y), V[j * vstride + t]);
        }
        W[t] = w;
    }
}

__global__ void k_scale32(int64_t n, int64_t Bc, const double* __restrict__ scale, const float2* __restrict__ W,
                          float2* __restrict__ Vout) {
    const int64_t total = n * Bc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const float sc = (float)scale[t % Bc];
        const float2 w = W[t];
        Vout[t] = make_float2(w.x * sc, w.y * sc);
    }
}

__global__ void k_combine32(int64_t n, int64_t Bc, int nj, const float2* __restrict__ Z, int64_t zstride,
                            const double2* __restrict__ y, float2* __restrict__ X) {
    const int64_t total = n * Bc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = t % Bc;
        float2 x = X[t];
        for (int j = 0; j < nj; ++j) {
            const double2 yj = y[(int64_t)j * Bc + c];
            ffma(x, make_float2((float)yj.x, (float)yj.y), Z[j * zstride + t]);
        }
        X[t] = x;
    }
}

// out = r * scale[c] in FP32; x += scale[c] * d in FP64; FP64 -> FP32 copy of matrix values
__global__ void k_to32_scaled(int64_t n, int64_t Bc, const double2* __restrict__ r, const double* __restrict__ scale,
                              float2* __restrict__ out) {
    const int64_t total = n * Bc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const double sc = scale[t % Bc];
        out[t] = make_float2((float)(r[t].x * sc), (float)(r[t].y * sc));
    }
}

__global__ void k_axpy_from32(int64_t n, int64_t Bc, const float2* __restrict__ d, const double* __restrict__ scale,
                              double2* __restrict__ x) {
    const int64_t total = n * Bc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const double sc = scale[t % Bc];
        x[t].x += sc * (double)d[t].x;
        x[t].y += sc * (double)d[t].y;
    }
}

__global__ void k_to32(int64_t nv, const double2* __restrict__ in, float2* __restrict__ out) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nv; t += (int64_t)gridDim.x * blockDim.x)
        out[t] = make_float2((float)in[t].x, (float)in[t].y);
}

}  // namespace kry
}  // namespace emg

// ------------------------------------------------------------------ plan ---
namespace {
using namespace emg;

void rplan_free(emg_rplan* p) {
    if (!p) return;
    dfree(p->sid); dfree(p->map); dfree(p->rptr); dfree(p->rind); dfree(p->rsrc); dfree(p->rdiag);
    dfree(p->uptr); dfree(p->ulist); dfree(p->lrows); dfree(p->urows);
    if (p->ws) cudaFree(p->ws);
    if (p->ev_in) cudaEventDestroy(p->ev_in);
    if (p->ev_out) cudaEventDestroy(p->ev_out);
    if (p->gs) cudaStreamDestroy(p->gs);
    delete p;
}
}  // namespace

extern "C" int emg_rplan_create(int64_t N, const int64_t* indptr, const int32_t* indices, int64_t nnz_full,
                                int64_t n_solve, const int64_t* solve_ids, void* stream, emg_rplan** out) {
    using namespace emg;
    EMG_CHECK_ARG(out && indptr && indices && (solve_ids || n_solve == 0), "emg_rplan_create: NULL argument");
    EMG_CHECK_ARG(N >= 0 && n_solve >= 0 && n_solve <= N, "emg_rplan_create: bad size");
    cudaStream_t s = (cudaStream_t)stream;
    emg_rplan* p = new emg_rplan();
    p->N = N;
    p->ns = n_solve;
    p->nnz_full = nnz_full;
    const int64_t ns = n_solve;
    int64_t* cnt = nullptr;
    int64_t* tmp = nullptr;
    auto fail = [&](int code) { dfree(cnt); dfree(tmp); rplan_free(p); return code; };
#define TRY(x) do { int _r = (x); if (_r) return fail(_r); } while (0)
#define TRYC(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) return fail(cuda_status(_e, #x)); } while (0)
    TRY(dalloc(&p->sid, ns + 1, "solve ids"));
    TRY(dalloc(&p->map, N + 1, "dof map"));
    TRY(dalloc(&p->rptr, ns + 1, "restricted indptr"));
    TRY(dalloc(&p->rdiag, ns + 1, "restricted diag"));
    TRY(dalloc(&cnt, ns + 1, "row counts"));
    TRY(dalloc(&tmp, scan_scratch_elems(ns + 1) + 1, "scan scratch"));
    if (ns > 0) TRYC(cudaMemcpyAsync(p->sid, solve_ids, sizeof(int64_t) * ns, cudaMemcpyDeviceToDevice, s));
    if (N > 0) TRYC(cudaMemsetAsync(p->map, 0xff, sizeof(int32_t) * N, s));
    const int T = 256;
    if (ns > 0) {
        kry::k_map<<<grid_for(ns, T), T, 0, s>>>(ns, p->sid, p->map);
        kry::k_rcount<<<grid_for(ns, T), T, 0, s>>>(ns, p->sid, indptr, indices, p->map, cnt);
        TRYC(cudaGetLastError());
    }
    TRY(scan_exclusive_i64(cnt, p->rptr, ns, tmp, s));
    TRYC(cudaMemcpyAsync(&p->nnz, p->rptr + ns, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    TRYC(cudaStreamSynchronize(s));
    TRY(dalloc(&p->rind, p->nnz + 1, "restricted indices"));
    TRY(dalloc(&p->rsrc, p->nnz + 1, "restricted sources"));
    if (ns > 0) {
        kry::k_rwrite<<<grid_for(ns, T), T, 0, s>>>(ns, p->sid, indptr, indices, p->map, p->rptr, p->rind, p->rsrc,
                                                    p->rdiag);
        TRYC(cudaGetLastError());
    }
    // host: levels and factorization update lists
    std::vector<int64_t> rptr(ns + 1), rdiag(ns);
    std::vector<int32_t> rind(p->nnz);
    TRYC(cudaMemcpyAsync(rptr.data(), p->rptr, sizeof(int64_t) * (ns + 1), cudaMemcpyDeviceToHost, s));
    if (ns > 0) TRYC(cudaMemcpyAsync(rdiag.data(), p->rdiag, sizeof(int64_t) * ns, cudaMemcpyDeviceToHost, s));
    if (p->nnz > 0) TRYC(cudaMemcpyAsync(rind.data(), p->rind, sizeof(int32_t) * p->nnz, cudaMemcpyDeviceToHost, s));
    TRYC(cudaStreamSynchronize(s));
    for (int64_t i = 0; i < ns; ++i)
        if (rdiag[i] < 0) {
            set_error("emg_rplan_create: restricted row " + std::to_string(i) + " has no diagonal entry");
            return fail(EMG_ERR_MESH);
        }
    std::vector<int32_t> lev(ns, 0), ulev(ns, 0);
    int32_t nl = 0, nu = 0;
    for (int64_t i = 0; i < ns; ++i) {
        int32_t l = 0;
        for (int64_t k = rptr[i]; k < rdiag[i]; ++k) l = std::max(l, lev[rind[k]] + 1);
        lev[i] = l;
        nl = std::max(nl, l + 1);
    }
    for (int64_t i = ns - 1; i >= 0; --i) {
        int32_t l = 0;
        for (int64_t k = rdiag[i] + 1; k < rptr[i + 1]; ++k) l = std::max(l, ulev[rind[k]] + 1);
        ulev[i] = l;
        nu = std::max(nu, l + 1);
    }
    auto bucket = [&](const std::vector<int32_t>& lv, int32_t nlev, std::vector<int64_t>& ptr, std::vector<int32_t>& rows) {
        ptr.assign(nlev + 1, 0);
        for (int64_t i = 0; i < ns; ++i) ptr[lv[i] + 1]++;
        for (int32_t l = 0; l < nlev; ++l) ptr[l + 1] += ptr[l];
        rows.resize(ns);
        std::vector<int64_t> pos(ptr.begin(), ptr.end() - 1);
        for (int64_t i = 0; i < ns; ++i) rows[pos[lv[i]]++] = (int32_t)i;
    };
    std::vector<int32_t> lrows, urows;
    bucket(lev, nl, p->lptr, lrows);
    bucket(ulev, nu, p->uptr_lv, urows);
    // update lists: for row i, each kk in its L part (column k), each entry of row k's U
    // part whose column is in row i: (kk local index << 32 | source pos, target pos)
    std::vector<int64_t> uptr(ns + 1, 0), ulist;
    ulist.reserve((size_t)p->nnz * 8);
    std::vector<int64_t> where(ns, -1);
    for (int64_t i = 0; i < ns; ++i) {
        for (int64_t k = rptr[i]; k < rptr[i + 1]; ++k) where[rind[k]] = k;
        for (int64_t kk = rptr[i]; kk < rdiag[i]; ++kk) {
            const int32_t k = rind[kk];
            for (int64_t jj = rdiag[k] + 1; jj < rptr[k + 1]; ++jj) {
                const int64_t t = where[rind[jj]];
                if (t < 0) continue;
                ulist.push_back(((kk - rptr[i]) << 32) | jj);
                ulist.push_back(t);
            }
        }
        for (int64_t k = rptr[i]; k < rptr[i + 1]; ++k) where[rind[k]] = -1;
        uptr[i + 1] = (int64_t)ulist.size() / 2;
    }
    TRY(dalloc(&p->uptr, ns + 1, "ilu update ptr"));
    TRY(dalloc(&p->ulist, (int64_t)ulist.size() + 2, "ilu update list"));
    TRY(dalloc(&p->lrows, ns + 1, "L level rows"));
    TRY(dalloc(&p->urows, ns + 1, "U level rows"));
    TRYC(cudaMemcpyAsync(p->uptr, uptr.data(), sizeof(int64_t) * (ns + 1), cudaMemcpyHostToDevice, s));
    if (!ulist.empty())
        TRYC(cudaMemcpyAsync(p->ulist, ulist.data(), sizeof(int64_t) * ulist.size(), cudaMemcpyHostToDevice, s));
    if (ns > 0) {
        TRYC(cudaMemcpyAsync(p->lrows, lrows.data(), sizeof(int32_t) * ns, cudaMemcpyHostToDevice, s));
        TRYC(cudaMemcpyAsync(p->urows, urows.data(), sizeof(int32_t) * ns, cudaMemcpyHostToDevice, s));
    }
    TRYC(cudaStreamSynchronize(s));
    TRYC(cudaStreamCreateWithFlags(&p->gs, cudaStreamNonBlocking));
    TRYC(cudaEventCreateWithFlags(&p->ev_in, cudaEventDisableTiming));
    TRYC(cudaEventCreateWithFlags(&p->ev_out, cudaEventDisableTiming));
    dfree(cnt);
    dfree(tmp);
#undef TRY
#undef TRYC
    *out = p;
    return EMG_OK;
}

extern "C" int64_t emg_rplan_n(const emg_rplan* p) { return p ? p->ns : -1; }
extern "C" int64_t emg_rplan_nnz(const emg_rplan* p) { return p ? p->nnz : -1; }
extern "C" int64_t emg_rplan_levels(const emg_rplan* p) { return p ? (int64_t)p->lptr.size() - 1 : -1; }
extern "C" void emg_rplan_destroy(emg_rplan* p) { rplan_free(p); }

extern "C" int emg_rplan_pattern(const emg_rplan* p, int64_t* indptr_out, int32_t* indices_out) {
    using namespace emg;
    EMG_CHECK_ARG(p && indptr_out && indices_out, "emg_rplan_pattern: NULL argument");
    EMG_CUDA(cudaMemcpy(indptr_out, p->rptr, sizeof(int64_t) * (p->ns + 1), cudaMemcpyDeviceToHost));
    if (p->nnz) EMG_CUDA(cudaMemcpy(indices_out, p->rind, sizeof(int32_t) * p->nnz, cudaMemcpyDeviceToHost));
    return EMG_OK;
}

extern "C" int emg_rplan_form(const emg_rplan* p, int64_t Bm, const double* E, const double* B, const double* k2,
                              int64_t n_ports, const double* P, const double* gam, double* A, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(p && E && B && k2 && A && Bm > 0 && n_ports >= 0 && (n_ports == 0 || (P && gam)),
                  "emg_rplan_form: bad argument");
    if (p->nnz == 0) return EMG_OK;
    kry::k_form<<<grid_for(p->nnz * Bm, 256), 256, 0, (cudaStream_t)stream>>>(
        p->nnz, Bm, p->rsrc, reinterpret_cast<const double2*>(E), reinterpret_cast<const double2*>(B), k2, n_ports,
        reinterpret_cast<const double2*>(P), p->nnz_full, reinterpret_cast<const double2*>(gam),
        reinterpret_cast<double2*>(A));
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}

extern "C" int emg_ilu0(const emg_rplan* p, int64_t Bm, double* LU, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(p && LU && Bm > 0, "emg_ilu0: bad argument");
    cudaStream_t s = (cudaStream_t)stream;
    for (size_t l = 0; l + 1 < p->lptr.size(); ++l) {
        const int64_t r0 = p->lptr[l], nr = p->lptr[l + 1] - r0;
        kry::k_ilu_level<<<grid_for(nr * Bm, 128), 128, 0, s>>>(nr, p->lrows + r0, Bm, p->rptr, p->rind, p->rdiag,
                                                                p->uptr, p->ulist, reinterpret_cast<double2*>(LU));
    }
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}

namespace {
int trsv(const emg_rplan* p, int64_t Bc, const int32_t* cmat, int64_t Bm, const double2* LU, double2* X, cudaStream_t s) {
    const bool small = Bc <= kry::kSmallBc;
    for (int up = 0; up < 2; ++up) {
        const std::vector<int64_t>& lv = up ? p->uptr_lv : p->lptr;
        const int32_t* rows = up ? p->urows : p->lrows;
        for (size_t l = 0; l + 1 < lv.size(); ++l) {
            const int64_t r0 = lv[l], nr = lv[l + 1] - r0;
            if (small)
                kry::k_trsv_level_w<<<(unsigned)((nr * 32 + 127) / 128), 128, 0, s>>>(nr, rows + r0, Bc, cmat, Bm, p->rptr,
                                                                                     p->rind, p->rdiag, LU, up, X);
            else
                kry::k_trsv_level<<<grid_for(nr * Bc, 128), 128, 0, s>>>(nr, rows + r0, Bc, cmat, Bm, p->rptr, p->rind,
                                                                         p->rdiag, LU, up, X);
        }
    }
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}
}  // namespace

extern "C" int emg_ilu_apply(const emg_rplan* p, int64_t Bc, const int32_t* cmat, int64_t Bm, const double* LU,
                             double* X, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(p && cmat && LU && X && Bc > 0 && Bm > 0, "emg_ilu_apply: bad argument");
    return trsv(p, Bc, cmat, Bm, reinterpret_cast<const double2*>(LU), reinterpret_cast<double2*>(X),
                (cudaStream_t)stream);
}

extern "C" int emg_spmv(const emg_rplan* p, int64_t Bc, const int32_t* cmat, int64_t Bm, const double* A,
                        const double* X, const double* Bv, double* Y, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(p && cmat && A && X && Y && Bc > 0 && Bm > 0, "emg_spmv: bad argument");
    if (p->ns == 0) return EMG_OK;
    kry::k_spmv<<<grid_for(p->ns * Bc, 256), 256, 0, (cudaStream_t)stream>>>(
        p->ns, Bc, cmat, Bm, p->rptr, p->rind, reinterpret_cast<const double2*>(A), reinterpret_cast<const double2*>(X),
        reinterpret_cast<const double2*>(Bv), reinterpret_cast<double2*>(Y));
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}

extern "C" int emg_spmv_family(const emg_rplan* p, int64_t Bc, int nfam, const double* fam, const double* coef,
                               const double* X, const double* Bv, double* Y, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(p && fam && coef && X && Y && Bc > 0 && nfam >= 1 && nfam <= kMaxFamily,
                  "emg_spmv_family: bad argument");
    if (p->ns == 0) return EMG_OK;
    MatArg A;
    A.nfam = nfam;
    A.fam = reinterpret_cast<const double2*>(fam);
    A.coef = reinterpret_cast<const double2*>(coef);
    spmv_op(p, Bc, A, reinterpret_cast<const double2*>(X), reinterpret_cast<const double2*>(Bv),
            reinterpret_cast<double2*>(Y), (cudaStream_t)stream);
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}

extern "C" int emg_rplan_gather(const emg_rplan* p, int64_t Bc, const double* full, double* out, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(p && full && out && Bc > 0, "emg_rplan_gather: bad argument");
    if (p->ns == 0) return EMG_OK;
    kry::k_gather_rhs<<<grid_for(p->ns * Bc, 256), 256, 0, (cudaStream_t)stream>>>(
        p->ns, Bc, p->sid, p->N, reinterpret_cast<const double2*>(full), reinterpret_cast<double2*>(out));
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}

extern "C" int emg_rplan_scatter(const emg_rplan* p, int64_t Bc, const double* x, double* full, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(p && x && full && Bc > 0, "emg_rplan_scatter: bad argument");
    cudaStream_t s = (cudaStream_t)stream;
    EMG_CUDA(cudaMemsetAsync(full, 0, sizeof(double) * 2 * p->N * Bc, s));
    if (p->ns == 0) return EMG_OK;
    kry::k_scatter_sol<<<grid_for(p->ns * Bc, 256), 256, 0, s>>>(p->ns, Bc, p->sid, p->N,
                                                                reinterpret_cast<const double2*>(x),
                                                                reinterpret_cast<double2*>(full));
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}

// ------------------------------------------------------------------ GMRES ---
// Right-preconditioned restarted GMRES(m) with classical Gram-Schmidt applied
// twice (CGS2), all columns in lockstep; a column stops updating once its
// implicit residual reaches tol * ||b||.  The final residual is recomputed
// explicitly in FP64 (resid_out) after every restart.
namespace {
void spmv(const emg_rplan* p, int64_t Bc, const int32_t* cmat, int64_t Bm, const double2* A, const double2* X,
          const double2* Bv, double2* Y, cudaStream_t s) {
    const int64_t n = p->ns;
    if (Bc <= kry::kSmallBc)
        kry::k_spmv_w<<<(unsigned)((n * 32 + 127) / 128), 128, 0, s>>>(n, Bc, cmat, Bm, p->rptr, p->rind, A, X, Bv, Y);
    else
        kry::k_spmv<<<grid_for(n * Bc, 256), 256, 0, s>>>(n, Bc, cmat, Bm, p->rptr, p->rind, A, X, Bv, Y);
}

void dots(int64_t n, int64_t Bc, int nj, const double2* V, int64_t vstride, const double2* W, double2* part,
          int64_t nblk, cudaStream_t s) {
    if (Bc < 32) {
        kry::k_dots_partial_small<<<(unsigned)nblk, 256, 0, s>>>(n, Bc, nj, V, vstride, W, part);
    } else {
        const dim3 g((unsigned)nblk, (unsigned)((Bc + 127) / 128));
        kry::k_dots_partial<<<g, 128, 0, s>>>(n, Bc, nj, V, vstride, W, part);
    }
}
}  // namespace

namespace emg {
void spmv_op(const emg_rplan* p, int64_t Bc, const MatArg& A, const double2* X, const double2* Bv, double2* Y,
             cudaStream_t s) {
    if (A.nfam > 0)
        kry::k_spmv_fam<<<grid_for(p->ns * Bc, 256), 256, 0, s>>>(p->ns, p->nnz, Bc, A.nfam, A.fam, A.coef, p->rptr,
                                                                  p->rind, X, Bv, Y);
    else
        spmv(p, Bc, A.cmat, A.Bm, A.A, X, Bv, Y, s);
}
}  // namespace emg

namespace emg {
int gmres_run(emg_rplan* p, int64_t Bc, const MatArg& A, const double2* rhs, double2* x, int restart, int max_iter,
              double tol, int32_t* iters_out, double* resid_out, cudaStream_t caller, Precond& M, bool flexible) {
    const int64_t n = p->ns;
    if (n == 0) return EMG_OK;
    {
        const int rc = M.prepare(Bc);
        if (rc) return rc;
    }
    EMG_CUDA(cudaEventRecord(p->ev_in, caller));
    EMG_CUDA(cudaStreamWaitEvent(p->gs, p->ev_in, 0));
    cudaStream_t s = p->gs;
    const int m = restart;
    const int64_t vec = n * Bc;
    const int64_t nblk = (n + kry::kDotRows - 1) / kry::kDotRows;
    // workspace layout
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = (off + bytes + 255) & ~(size_t)255; return o; };
    const size_t oV = take(sizeof(double2) * vec * (m + 1));
    const size_t oZ = flexible ? take(sizeof(double2) * vec * m) : 0;
    const size_t oW = take(sizeof(double2) * vec);
    const size_t oT = take(sizeof(double2) * vec);
    const size_t oPart = take(sizeof(double2) * nblk * (m + 1) * Bc);
    const size_t oH1 = take(sizeof(double2) * (m + 1) * Bc);
    const size_t oH2 = take(sizeof(double2) * (m + 1) * Bc);
    const size_t oH = take(sizeof(double2) * m * m * Bc);
    const size_t oCs = take(sizeof(double2) * m * Bc);
    const size_t oSn = take(sizeof(double2) * m * Bc);
    const size_t oG = take(sizeof(double2) * (m + 1) * Bc);
    const size_t oY = take(sizeof(double2) * m * Bc);
    const size_t oBn = take(sizeof(double) * Bc);
    const size_t oVs = take(sizeof(double) * Bc);
    const size_t oWn = take(sizeof(double) * Bc);
    const size_t oAct = take(sizeof(int32_t) * Bc);
    const size_t oLen = take(sizeof(int32_t) * Bc);
    const size_t oRes = take(sizeof(double) * Bc);
    const size_t oIt = take(sizeof(int32_t) * Bc);
    if (off > p->ws_bytes) {
        if (p->ws) cudaFree(p->ws);
        p->ws = nullptr;
        p->ws_bytes = 0;
        EMG_CUDA(cudaMalloc(&p->ws, off));
        p->ws_bytes = off;
    }
    char* base = static_cast<char*>(p->ws);
    auto* V = reinterpret_cast<double2*>(base + oV);
    auto* Z = flexible ? reinterpret_cast<double2*>(base + oZ) : nullptr;
    auto* W = reinterpret_cast<double2*>(base + oW);
    auto* Tv = reinterpret_cast<double2*>(base + oT);
    auto* part = reinterpret_cast<double2*>(base + oPart);
    auto* h1 = reinterpret_cast<double2*>(base + oH1);
    auto* h2 = reinterpret_cast<double2*>(base + oH2);
    auto* H = reinterpret_cast<double2*>(base + oH);
    auto* cs = reinterpret_cast<double2*>(base + oCs);
    auto* sn = reinterpret_cast<double2*>(base + oSn);
    auto* g = reinterpret_cast<double2*>(base + oG);
    auto* y = reinterpret_cast<double2*>(base + oY);
    auto* bn = reinterpret_cast<double*>(base + oBn);
    auto* vs = reinterpret_cast<double*>(base + oVs);
    auto* wn = reinterpret_cast<double*>(base + oWn);
    auto* act = reinterpret_cast<int32_t*>(base + oAct);
    auto* len = reinterpret_cast<int32_t*>(base + oLen);
    auto* res = reinterpret_cast<double*>(base + oRes);
    auto* its = reinterpret_cast<int32_t*>(base + oIt);
    const int T = 256;
    const dim3 dgrid((unsigned)nblk, (unsigned)((Bc + 127) / 128));
    const unsigned cgrid = (unsigned)((Bc + 127) / 128);
    auto norms2 = [&](const double2* Vv) {   // h1[c] = ||Vv[:,c]||^2 (real part)
        dots(n, Bc, 1, Vv, vec, Vv, part, nblk, s);
        kry::k_dots_final<<<cgrid, 128, 0, s>>>(nblk, Bc, 1, part, h1);
        return h1;
    };
    kry::k_sqrt_real<<<cgrid, 128, 0, s>>>(Bc, norms2(rhs), bn);
    EMG_CUDA(cudaMemsetAsync(its, 0, sizeof(int32_t) * Bc, s));
    // one Arnoldi step for Krylov index j (from the first restart on, captured once
    // per j into a CUDA graph)
    auto step = [&](int j) -> int {
        double2* Vj = V + (int64_t)j * vec;
        double2* Mv = flexible ? Z + (int64_t)j * vec : Tv;
        int rc = M.apply(Vj, Mv, s);
        if (rc) return rc;
        spmv_op(p, Bc, A, Mv, nullptr, W, s);
        // CGS2: two passes of h = V^H w, w -= V h
        const unsigned hgrid = (unsigned)(((int64_t)(j + 1) * Bc + 127) / 128);
        dots(n, Bc, j + 1, V, vec, W, part, nblk, s);
        kry::k_dots_final<<<hgrid, 128, 0, s>>>(nblk, Bc, j + 1, part, h1);
        kry::k_orth_update<<<grid_for(vec, T), T, 0, s>>>(n, Bc, j + 1, V, vec, h1, act, W);
        dots(n, Bc, j + 1, V, vec, W, part, nblk, s);
        kry::k_dots_final<<<hgrid, 128, 0, s>>>(nblk, Bc, j + 1, part, h2);
        kry::k_orth_update<<<grid_for(vec, T), T, 0, s>>>(n, Bc, j + 1, V, vec, h2, act, W);
        dots(n, Bc, 1, W, vec, W, part, nblk, s);
        kry::k_dots_final<<<cgrid, 128, 0, s>>>(nblk, Bc, 1, part, y);
        kry::k_real<<<cgrid, 128, 0, s>>>(Bc, y, wn);
        kry::k_arnoldi_col<<<cgrid, 128, 0, s>>>(Bc, j, m, h1, h2, wn, H, cs, sn, g, bn, tol, act, len, vs, res);
        kry::k_scale_cols<<<grid_for(vec, T), T, 0, s>>>(n, Bc, vs, W, V + (int64_t)(j + 1) * vec);
        EMG_CUDA(cudaGetLastError());
        return EMG_OK;
    };
    std::vector<cudaGraphExec_t> graphs(m, nullptr);
    struct GraphGuard {
        std::vector<cudaGraphExec_t>* g;
        ~GraphGuard() { for (auto& e : *g) if (e) cudaGraphExecDestroy(e); }
    } guard{&graphs};
    int total = 0;
    std::vector<int32_t> hact(Bc), hprev(Bc), hits(Bc, 0);
    for (int cycle = 0; total < max_iter; ++cycle) {
        // r = b - A x ; V0 = r / ||r||
        spmv_op(p, Bc, A, x, rhs, W, s);
        double2* rr = norms2(W);
        kry::k_restart_cols<<<cgrid, 128, 0, s>>>(Bc, rr, bn, tol, g, vs, act, len, res, m + 1);
        kry::k_scale_cols<<<grid_for(vec, T), T, 0, s>>>(n, Bc, vs, W, V);
        EMG_CUDA(cudaGetLastError());
        EMG_CUDA(cudaMemcpyAsync(hact.data(), act, sizeof(int32_t) * Bc, cudaMemcpyDeviceToHost, s));
        EMG_CUDA(cudaStreamSynchronize(s));
        bool any = false;
        for (int64_t c = 0; c < Bc; ++c) any |= hact[c] != 0;
        if (!any) break;
        int j = 0;
        while (j < m && total < max_iter) {
            hprev = hact;
            if (cycle == 0) {
                // first cycle: direct launches (a graph would be instantiated for one use)
                const int rc = step(j);
                if (rc) return rc;
            } else {
                // restarted cycles replay each Arnoldi step's graph
                if (!graphs[j]) {
                    cudaGraph_t gr = nullptr;
                    EMG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
                    const int rc = step(j);
                    const cudaError_t ec = cudaStreamEndCapture(s, &gr);
                    if (rc) { if (gr) cudaGraphDestroy(gr); return rc; }
                    if (ec != cudaSuccess) return cuda_status(ec, "cudaStreamEndCapture");
                    const cudaError_t ei = cudaGraphInstantiate(&graphs[j], gr, 0);
                    cudaGraphDestroy(gr);
                    if (ei != cudaSuccess) return cuda_status(ei, "cudaGraphInstantiate");
                }
                EMG_CUDA(cudaGraphLaunch(graphs[j], s));
            }
            ++j;
            ++total;
            EMG_CUDA(cudaMemcpyAsync(hact.data(), act, sizeof(int32_t) * Bc, cudaMemcpyDeviceToHost, s));
            EMG_CUDA(cudaStreamSynchronize(s));
            bool any2 = false;
            for (int64_t c = 0; c < Bc; ++c) {
                if (hprev[c]) hits[c] = total;
                any2 |= hact[c] != 0;
            }
            if (!any2) break;
        }
        // x += Z y (flexible) or x += M^-1 (V y)   (y from back substitution over each
        // column's Krylov length)
        kry::k_backsolve<<<cgrid, 128, 0, s>>>(Bc, m, H, g, len, y, j);
        if (flexible) {
            EMG_CUDA(cudaMemsetAsync(Tv, 0, sizeof(double2) * vec, s));
            kry::k_combine_basis<<<grid_for(vec, T), T, 0, s>>>(n, Bc, j, Z, vec, y, Tv);
        } else {
            EMG_CUDA(cudaMemsetAsync(W, 0, sizeof(double2) * vec, s));
            kry::k_combine_basis<<<grid_for(vec, T), T, 0, s>>>(n, Bc, j, V, vec, y, W);
            const int rc = M.apply(W, Tv, s);
            if (rc) return rc;
        }
        kry::k_axpy1<<<grid_for(vec, T), T, 0, s>>>(vec, Tv, x);
        EMG_CUDA(cudaGetLastError());
    }
    // explicit final residual
    spmv_op(p, Bc, A, x, rhs, W, s);
    double2* rr = norms2(W);
    std::vector<double2> hr(Bc);
    std::vector<double> hb(Bc), hres(Bc);
    EMG_CUDA(cudaMemcpyAsync(hr.data(), rr, sizeof(double2) * Bc, cudaMemcpyDeviceToHost, s));
    EMG_CUDA(cudaMemcpyAsync(hb.data(), bn, sizeof(double) * Bc, cudaMemcpyDeviceToHost, s));
    EMG_CUDA(cudaStreamSynchronize(s));
    for (int64_t c = 0; c < Bc; ++c) hres[c] = hb[c] > 0 ? sqrt(std::max(hr[c].x, 0.0)) / hb[c] : 0.0;
    EMG_CUDA(cudaMemcpyAsync(resid_out, hres.data(), sizeof(double) * Bc, cudaMemcpyHostToDevice, s));
    EMG_CUDA(cudaMemcpyAsync(iters_out, hits.data(), sizeof(int32_t) * Bc, cudaMemcpyHostToDevice, s));
    EMG_CUDA(cudaStreamSynchronize(s));
    EMG_CUDA(cudaEventRecord(p->ev_out, s));
    EMG_CUDA(cudaStreamWaitEvent(caller, p->ev_out, 0));
    return EMG_OK;
}
}  // namespace emg

namespace emg {
namespace {
void spmv32(const emg_rplan* p, int64_t Bc, const int32_t* cmat, int64_t Bm, const float2* A, const float2* X,
            const float2* Bv, float2* Y, cudaStream_t s) {
    const int64_t n = p->ns;
    if (Bc <= kry::kSmallBc)
        kry::k_spmv32_w<<<(unsigned)((n * 32 + 127) / 128), 128, 0, s>>>(n, Bc, cmat, Bm, p->rptr, p->rind, A, X, Bv,
                                                                           Y);
    else
        kry::k_spmv32<<<grid_for(n * Bc, 256), 256, 0, s>>>(n, Bc, cmat, Bm, p->rptr, p->rind, A, X, Bv, Y);
}

void dots32(int64_t n, int64_t Bc, int nj, const float2* V, int64_t vstride, const float2* W, double2* part,
            int64_t nblk, cudaStream_t s) {
    if (Bc < 32) {
        kry::k_dots32_small<<<(unsigned)nblk, 256, 0, s>>>(n, Bc, nj, V, vstride, W, part);
    } else {
        const dim3 g((unsigned)nblk, (unsigned)((Bc + 127) / 128));
        kry::k_dots32<<<g, 128, 0, s>>>(n, Bc, nj, V, vstride, W, part);
    }
}

// Workspace of the inner FP32 FGMRES (carved once per ir_run, reused by every step
// so the captured Arnoldi-step graphs stay valid across refinement steps).
struct Inner32 {
    int m = 0;
    int64_t vec = 0, nblk = 0;
    float2 *V = nullptr, *Z = nullptr, *W = nullptr;
    double2 *part = nullptr, *h1 = nullptr, *h2 = nullptr, *H = nullptr, *cs = nullptr, *sn = nullptr, *g = nullptr,
            *y = nullptr;
    double *bn = nullptr, *vs = nullptr, *wn = nullptr, *res = nullptr;
    int32_t *act = nullptr, *len = nullptr;
    int cycles = 0;                      // Arnoldi cycles run so far (graphs from the second on)
    std::vector<cudaGraphExec_t> graphs;
    ~Inner32() {
        for (auto& e : graphs)
            if (e) cudaGraphExecDestroy(e);
    }
};

// FGMRES(m) on FP32 vectors from x = 0; hits[c] = iterations of column c.
int gmres32(emg_rplan* p, int64_t Bc, const int32_t* cmat, int64_t Bm, const float2* A32, const float2* rhs,
            float2* x, int max_iter, double tol, Inner32& w, std::vector<int32_t>& hits, cudaStream_t s,
            Precond32& M) {
    const int64_t n = p->ns, vec = w.vec, nblk = w.nblk;
    const int m = w.m, T = 256;
    const unsigned cgrid = (unsigned)((Bc + 127) / 128);
    auto norms2 = [&](const float2* Vv) {
        dots32(n, Bc, 1, Vv, vec, Vv, w.part, nblk, s);
        kry::k_dots_final<<<cgrid, 128, 0, s>>>(nblk, Bc, 1, w.part, w.h1);
        return w.h1;
    };
    kry::k_sqrt_real<<<cgrid, 128, 0, s>>>(Bc, norms2(rhs), w.bn);
    auto step = [&](int j) -> int {
        float2* Vj = w.V + (int64_t)j * vec;
        float2* Zj = w.Z + (int64_t)j * vec;
        int rc = M.apply(Vj, Zj, s);
        if (rc) return rc;
        spmv32(p, Bc, cmat, Bm, A32, Zj, nullptr, w.W, s);
        const unsigned hgrid = (unsigned)(((int64_t)(j + 1) * Bc + 127) / 128);
        dots32(n, Bc, j + 1, w.V, vec, w.W, w.part, nblk, s);
        kry::k_dots_final<<<hgrid, 128, 0, s>>>(nblk, Bc, j + 1, w.part, w.h1);
        kry::k_orth32<<<grid_for(vec, T), T, 0, s>>>(n, Bc, j + 1, w.V, vec, w.h1, w.act, w.W);
        dots32(n, Bc, j + 1, w.V, vec, w.W, w.part, nblk, s);
        kry::k_dots_final<<<hgrid, 128, 0, s>>>(nblk, Bc, j + 1, w.part, w.h2);
        kry::k_orth32<<<grid_for(vec, T), T, 0, s>>>(n, Bc, j + 1, w.V, vec, w.h2, w.act, w.W);
        dots32(n, Bc, 1, w.W, vec, w.W, w.part, nblk, s);
        kry::k_dots_final<<<cgrid, 128, 0, s>>>(nblk, Bc, 1, w.part, w.y);
        kry::k_real<<<cgrid, 128, 0, s>>>(Bc, w.y, w.wn);
        kry::k_arnoldi_col<<<cgrid, 128, 0, s>>>(Bc, j, m, w.h1, w.h2, w.wn, w.H, w.cs, w.sn, w.g, w.bn, tol, w.act,
                                                 w.len, w.vs, w.res);
        kry::k_scale32<<<grid_for(vec, T), T, 0, s>>>(n, Bc, w.vs, w.W, w.V + (int64_t)(j + 1) * vec);
        EMG_CUDA(cudaGetLastError());
        return EMG_OK;
    };
    hits.assign(Bc, 0);
    std::vector<int32_t> hact(Bc), hprev(Bc);
    int total = 0;
    while (total < max_iter) {
        spmv32(p, Bc, cmat, Bm, A32, x, rhs, w.W, s);   // W = rhs - A32 x
        double2* rr = norms2(w.W);
        kry::k_restart_cols<<<cgrid, 128, 0, s>>>(Bc, rr, w.bn, tol, w.g, w.vs, w.act, w.len, w.res, m + 1);
        kry::k_scale32<<<grid_for(vec, T), T, 0, s>>>(n, Bc, w.vs, w.W, w.V);
        EMG_CUDA(cudaGetLastError());
        EMG_CUDA(cudaMemcpyAsync(hact.data(), w.act, sizeof(int32_t) * Bc, cudaMemcpyDeviceToHost, s));
        EMG_CUDA(cudaStreamSynchronize(s));
        bool any = false;
        for (int64_t c = 0; c < Bc; ++c) any |= hact[c] != 0;
        if (!any) break;
        int j = 0;
        while (j < m && total < max_iter) {
            hprev = hact;
            if (w.cycles == 0) {
                const int rc = step(j);
                if (rc) return rc;
            } else {
                if (!w.graphs[j]) {
                    cudaGraph_t gr = nullptr;
                    EMG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
                    const int rc = step(j);
                    const cudaError_t ec = cudaStreamEndCapture(s, &gr);
                    if (rc) { if (gr) cudaGraphDestroy(gr); return rc; }
                    if (ec != cudaSuccess) return cuda_status(ec, "cudaStreamEndCapture");
                    const cudaError_t ei = cudaGraphInstantiate(&w.graphs[j], gr, 0);
                    cudaGraphDestroy(gr);
                    if (ei != cudaSuccess) return cuda_status(ei, "cudaGraphInstantiate");
                }
                EMG_CUDA(cudaGraphLaunch(w.graphs[j], s));
            }
            ++j;
            ++total;
            EMG_CUDA(cudaMemcpyAsync(hact.data(), w.act, sizeof(int32_t) * Bc, cudaMemcpyDeviceToHost, s));
            EMG_CUDA(cudaStreamSynchronize(s));
            bool any2 = false;
            for (int64_t c = 0; c < Bc; ++c) {
                if (hprev[c]) hits[c] = total;
                any2 |= hact[c] != 0;
            }
            if (!any2) break;
        }
        kry::k_backsolve<<<cgrid, 128, 0, s>>>(Bc, m, w.H, w.g, w.len, w.y, j);
        kry::k_combine32<<<grid_for(vec, T), T, 0, s>>>(n, Bc, j, w.Z, vec, w.y, x);
        EMG_CUDA(cudaGetLastError());
        ++w.cycles;
    }
    return EMG_OK;
}
}  // namespace

int ir_run(emg_rplan* p, int64_t Bc, const MatArg& A, const float2* A32, const double2* rhs, double2* x, int restart,
           int max_iter, double tol, double inner_tol, int32_t* iters_out, double* resid_out, int32_t* steps_out,
           cudaStream_t caller, Precond32& M) {
    const int64_t n = p->ns;
    if (n == 0) return EMG_OK;
    {
        const int rc = M.prepare(Bc);
        if (rc) return rc;
    }
    EMG_CUDA(cudaEventRecord(p->ev_in, caller));
    EMG_CUDA(cudaStreamWaitEvent(p->gs, p->ev_in, 0));
    cudaStream_t s = p->gs;
    const int m = restart, T = 256;
    const int64_t vec = n * Bc, nblk = (n + kry::kDotRows - 1) / kry::kDotRows;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = (off + bytes + 255) & ~(size_t)255; return o; };
    const size_t oR64 = take(sizeof(double2) * vec), oR32 = take(sizeof(float2) * vec), oD32 = take(sizeof(float2) * vec);
    const size_t oV = take(sizeof(float2) * vec * (m + 1)), oZ = take(sizeof(float2) * vec * m);
    const size_t oW = take(sizeof(float2) * vec);
    const size_t oPart = take(sizeof(double2) * nblk * (m + 1) * Bc);
    const size_t oH1 = take(sizeof(double2) * (m + 1) * Bc), oH2 = take(sizeof(double2) * (m + 1) * Bc);
    const size_t oH = take(sizeof(double2) * m * m * Bc), oCs = take(sizeof(double2) * m * Bc);
    const size_t oSn = take(sizeof(double2) * m * Bc), oG = take(sizeof(double2) * (m + 1) * Bc);
    const size_t oY = take(sizeof(double2) * (m + 1) * Bc);
    const size_t oBn = take(sizeof(double) * Bc), oVs = take(sizeof(double) * Bc), oWn = take(sizeof(double) * Bc);
    const size_t oRes = take(sizeof(double) * Bc), oAct = take(sizeof(int32_t) * Bc), oLen = take(sizeof(int32_t) * Bc);
    const size_t oBn64 = take(sizeof(double) * Bc), oRn = take(sizeof(double) * Bc), oSc = take(sizeof(double) * Bc);
    if (off > p->ws_bytes) {
        if (p->ws) cudaFree(p->ws);
        p->ws = nullptr;
        p->ws_bytes = 0;
        EMG_CUDA(cudaMalloc(&p->ws, off));
        p->ws_bytes = off;
    }
    char* base = static_cast<char*>(p->ws);
    auto* r64 = reinterpret_cast<double2*>(base + oR64);
    auto* r32 = reinterpret_cast<float2*>(base + oR32);
    auto* d32 = reinterpret_cast<float2*>(base + oD32);
    Inner32 w;
    w.m = m;
    w.vec = vec;
    w.nblk = nblk;
    w.V = reinterpret_cast<float2*>(base + oV);
    w.Z = reinterpret_cast<float2*>(base + oZ);
    w.W = reinterpret_cast<float2*>(base + oW);
    w.part = reinterpret_cast<double2*>(base + oPart);
    w.h1 = reinterpret_cast<double2*>(base + oH1);
    w.h2 = reinterpret_cast<double2*>(base + oH2);
    w.H = reinterpret_cast<double2*>(base + oH);
    w.cs = reinterpret_cast<double2*>(base + oCs);
    w.sn = reinterpret_cast<double2*>(base + oSn);
    w.g = reinterpret_cast<double2*>(base + oG);
    w.y = reinterpret_cast<double2*>(base + oY);
    w.bn = reinterpret_cast<double*>(base + oBn);
    w.vs = reinterpret_cast<double*>(base + oVs);
    w.wn = reinterpret_cast<double*>(base + oWn);
    w.res = reinterpret_cast<double*>(base + oRes);
    w.act = reinterpret_cast<int32_t*>(base + oAct);
    w.len = reinterpret_cast<int32_t*>(base + oLen);
    w.graphs.assign(m, nullptr);
    auto* bn64 = reinterpret_cast<double*>(base + oBn64);
    auto* rn = reinterpret_cast<double*>(base + oRn);
    auto* sc = reinterpret_cast<double*>(base + oSc);
    const unsigned cgrid = (unsigned)((Bc + 127) / 128);
    // ||b|| in FP64
    dots(n, Bc, 1, rhs, vec, rhs, w.part, nblk, s);
    kry::k_dots_final<<<cgrid, 128, 0, s>>>(nblk, Bc, 1, w.part, w.h1);
    kry::k_sqrt_real<<<cgrid, 128, 0, s>>>(Bc, w.h1, bn64);
    std::vector<double> hb(Bc), hr(Bc), hs(Bc), rel(Bc);
    EMG_CUDA(cudaMemcpyAsync(hb.data(), bn64, sizeof(double) * Bc, cudaMemcpyDeviceToHost, s));
    std::vector<int32_t> tot(Bc, 0), hits;
    int steps = 0, used = 0;
    constexpr int kMaxSteps = 12;
    for (;;) {
        // true residual in FP64
        spmv_op(p, Bc, A, x, rhs, r64, s);
        dots(n, Bc, 1, r64, vec, r64, w.part, nblk, s);
        kry::k_dots_final<<<cgrid, 128, 0, s>>>(nblk, Bc, 1, w.part, w.h1);
        kry::k_sqrt_real<<<cgrid, 128, 0, s>>>(Bc, w.h1, rn);
        EMG_CUDA(cudaGetLastError());
        EMG_CUDA(cudaMemcpyAsync(hr.data(), rn, sizeof(double) * Bc, cudaMemcpyDeviceToHost, s));
        EMG_CUDA(cudaStreamSynchronize(s));
        bool all = true;
        for (int64_t c = 0; c < Bc; ++c) {
            rel[c] = hb[c] > 0 ? hr[c] / hb[c] : 0.0;
            all &= rel[c] <= tol;
        }
        if (all || steps >= kMaxSteps || used >= max_iter) break;
        // inner solve of A d = r / ||r|| for the unconverged columns
        for (int64_t c = 0; c < Bc; ++c) hs[c] = rel[c] > tol ? 1.0 / hr[c] : 0.0;
        EMG_CUDA(cudaMemcpyAsync(sc, hs.data(), sizeof(double) * Bc, cudaMemcpyHostToDevice, s));
        kry::k_to32_scaled<<<grid_for(vec, T), T, 0, s>>>(n, Bc, r64, sc, r32);
        EMG_CUDA(cudaMemsetAsync(d32, 0, sizeof(float2) * vec, s));
        const int rc = gmres32(p, Bc, A.cmat, A.Bm, A32, r32, d32, max_iter - used, inner_tol, w, hits, s, M);
        if (rc) return rc;
        int mx = 0;
        for (int64_t c = 0; c < Bc; ++c) {
            tot[c] += hits[c];
            mx = std::max(mx, (int)hits[c]);
            hs[c] = rel[c] > tol ? hr[c] : 0.0;
        }
        used += std::max(mx, 1);
        EMG_CUDA(cudaMemcpyAsync(sc, hs.data(), sizeof(double) * Bc, cudaMemcpyHostToDevice, s));
        kry::k_axpy_from32<<<grid_for(vec, T), T, 0, s>>>(n, Bc, d32, sc, x);
        EMG_CUDA(cudaGetLastError());
        ++steps;
    }
    EMG_CUDA(cudaMemcpyAsync(resid_out, rel.data(), sizeof(double) * Bc, cudaMemcpyHostToDevice, s));
    EMG_CUDA(cudaMemcpyAsync(iters_out, tot.data(), sizeof(int32_t) * Bc, cudaMemcpyHostToDevice, s));
    EMG_CUDA(cudaStreamSynchronize(s));
    if (steps_out) *steps_out = steps;
    EMG_CUDA(cudaEventRecord(p->ev_out, s));
    EMG_CUDA(cudaStreamWaitEvent(caller, p->ev_out, 0));
    return EMG_OK;
}
}  // namespace emg

namespace {
// ILU(0) factors as the preconditioner: out = (LU)^-1 in.
struct IluPrecond : emg::Precond {
    const emg_rplan* p;
    int64_t Bc, Bm;
    const int32_t* cmat;
    const double2* LU;
    IluPrecond(const emg_rplan* p_, int64_t Bc_, const int32_t* cmat_, int64_t Bm_, const double2* LU_)
        : p(p_), Bc(Bc_), Bm(Bm_), cmat(cmat_), LU(LU_) {}
    int apply(const double2* in, double2* out, cudaStream_t s) override {
        EMG_CUDA(cudaMemcpyAsync(out, in, sizeof(double2) * p->ns * Bc, cudaMemcpyDeviceToDevice, s));
        return trsv(p, Bc, cmat, Bm, LU, out, s);
    }
};
}  // namespace

extern "C" int emg_gmres(const emg_rplan* pc, int64_t Bc, const int32_t* cmat, int64_t Bm, const double* A_,
                         const double* LU_, const double* rhs_, double* x_, int restart, int max_iter, double tol,
                         int32_t* iters_out, double* resid_out, void* stream) {
    using namespace emg;
    emg_rplan* p = const_cast<emg_rplan*>(pc);
    EMG_CHECK_ARG(p && cmat && A_ && LU_ && rhs_ && x_ && iters_out && resid_out && Bc > 0 && Bm > 0,
                  "emg_gmres: bad argument");
    EMG_CHECK_ARG(restart >= 1 && restart <= kry::kMaxRestart && max_iter >= 1 && tol > 0,
                  "emg_gmres: restart must be in [1, 256]");
    IluPrecond M(p, Bc, cmat, Bm, reinterpret_cast<const double2*>(LU_));
    MatArg A;
    A.A = reinterpret_cast<const double2*>(A_);
    A.Bm = Bm;
    A.cmat = cmat;
    return gmres_run(p, Bc, A, reinterpret_cast<const double2*>(rhs_), reinterpret_cast<double2*>(x_), restart,
                     max_iter, tol, iters_out, resid_out, (cudaStream_t)stream, M, false);
}
