// Slab factorization: a direct block-tridiagonal solver for the restricted
// frequency-domain system, used as the preconditioner of a flexible GMRES.
//
// Replaces the direct sparse solve of SolveRoutine (SuperLU / PARDISO / UMFPACK,
// fem/solver.py:220-309, 405-469) for guided-wave structures.  The level-scheduled
// ILU(0) of emg_krylov.cu does not converge on resonant structures (iris filters),
// so a sweep needs a factorization that is exact up to rounding.
//
// Structure.  A breadth-first search from a pseudo-peripheral DOF splits the
// restricted DOFs into level sets ("slabs"); every matrix entry couples DOFs of the
// same slab or of neighbouring slabs, so A is block tridiagonal:
//     A = tridiag(C_i, D_i, U_i),  C_i = A[L_i, L_{i-1}],  U_i = A[L_i, L_{i+1}].
// On a waveguide the slabs are cross-sections and their widths stay near the DOF
// count of one cross-section.  Block elimination gives
//     S_0 = D_0,  S_i = D_i - C_i S_{i-1}^-1 U_{i-1}
// and the factor stores the dense inverses S_i^-1 (complex FP32 or FP64), plus
// the sparse couplings C_i, U_i.  A solve is then, per slab, a sparse product and
// one dense matrix x block-of-vectors product forward, the same backward:
//     z_i = S_i^-1 (b_i - C_i z_{i-1}),   x_i = z_i - S_i^-1 U_i x_{i+1}.
//
// Kernels.  S_i - C_i S_{i-1}^-1 U_{i-1} is one launch per slab: a CTA owns a few
// rows, builds R = C S^-1 for them in shared memory from coalesced rows of S^-1,
// then multiplies by the sparse U columns.  S_i^-1 is computed in place by blocked
// Gauss-Jordan with 64 x 64 tiles: the pivot tile is inverted by one CTA with
// partial pivoting inside the tile (a pivot below a relative threshold is replaced
// by the threshold and counted), the pivot row panel is multiplied by it, every
// other tile gets a rank-64 update (the bulk of the flops: for FP32 factors on the
// tcgen05 tensor cores with split-TF32 products, emg_tc.cu; for FP64 a tiled complex
// GEMM on the FP64 pipes), and the pivot column panel is multiplied by minus it.  The
// next pivot tile is updated first and inverted on a side stream while the rest of
// the step runs (one-step lookahead).  Several factorizations (anchor frequencies) run
// in the same launches (grid z), each with its own values.
#include <algorithm>
#include <cmath>
#include <vector>

#include "emg_krylov.cuh"

namespace emg {
namespace slab {

template <typename R> struct C2;
template <> struct C2<float> { using T = float2; };
template <> struct C2<double> { using T = double2; };

__device__ __forceinline__ float2 mk(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ double2 mk(double a, double b) { return make_double2(a, b); }
template <typename T> __device__ __forceinline__ T czero() { T z; z.x = 0; z.y = 0; return z; }
template <typename T> __device__ __forceinline__ void cfma(T& acc, T a, T b) {   // acc += a b
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}
template <typename T> __device__ __forceinline__ T cmul(T a, T b) { return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
template <typename T> __device__ __forceinline__ T cvt(double2 v);
template <> __device__ __forceinline__ float2 cvt<float2>(double2 v) { return make_float2((float)v.x, (float)v.y); }
template <> __device__ __forceinline__ double2 cvt<double2>(double2 v) { return v; }
__device__ __forceinline__ double2 to_d(float2 v) { return make_double2(v.x, v.y); }
__device__ __forceinline__ double2 to_d(double2 v) { return v; }

constexpr int kTile = 64;          // Gauss-Jordan tile and GEMM output tile
constexpr int kThreads = 256;
constexpr int kDiagThreads = 256;   // pivot-tile inversion: a 4 x 4 block per thread
constexpr int kMaxRows = 16;       // rows per CTA in the Schur-complement kernel
constexpr int kSchurSmem = 200 * 1024;
constexpr int64_t kMaxWidth = 12288;

template <typename R> struct Tile {
    using T = typename C2<R>::T;
    static constexpr int BK = sizeof(R) == 4 ? 16 : 8;
    static constexpr int LA = kTile * BK / kThreads;   // A elements per thread and chunk
    T a[2][BK][kTile + 1];
    T b[2][BK][kTile];
};

// acc[i][j] (row ty+16i, column tx+16j of the 64 x 64 output tile) += A B with
// A (M x K, row-major lda) and B (K x N, row-major ldb), M, N <= 64.  Zero fill
// outside.  Double-buffered through shared memory, one barrier per K chunk.
template <typename R>
__device__ __forceinline__ void tile_mac(typename C2<R>::T (&acc)[4][4], const typename C2<R>::T* __restrict__ A,
                                         int64_t lda, const typename C2<R>::T* __restrict__ B, int64_t ldb, int M,
                                         int N, int64_t K, Tile<R>& sm) {
    using T = typename C2<R>::T;
    constexpr int BK = Tile<R>::BK, LA = Tile<R>::LA;
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    T ra[LA], rb[LA];
    auto load = [&](int64_t k0) {
#pragma unroll
        for (int q = 0; q < LA; ++q) {
            const int idx = tid + kThreads * q;
            const int r = idx / BK, kk = idx % BK;
            ra[q] = (r < M && k0 + kk < K) ? A[(int64_t)r * lda + k0 + kk] : czero<T>();
            const int kb = idx / kTile, c = idx % kTile;
            rb[q] = (c < N && k0 + kb < K) ? B[(k0 + kb) * ldb + c] : czero<T>();
        }
    };
    auto store = [&](int buf) {
#pragma unroll
        for (int q = 0; q < LA; ++q) {
            const int idx = tid + kThreads * q;
            sm.a[buf][idx % BK][idx / BK] = ra[q];
            sm.b[buf][idx / kTile][idx % kTile] = rb[q];
        }
    };
    load(0);
    store(0);
    __syncthreads();
    int buf = 0;
    for (int64_t k0 = 0; k0 < K; k0 += BK) {
        const bool more = k0 + BK < K;
        if (more) load(k0 + BK);
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            T av[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) av[i] = sm.a[buf][kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) bv[j] = sm.b[buf][kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) cfma(acc[i][j], av[i], bv[j]);
        }
        if (more) store(buf ^ 1);
        __syncthreads();
        buf ^= 1;
    }
}

// ------------------------------------------------------------ factorization ---
// Dense blocks D_i and the sparse couplings of F matrices: column amat[f] of A
// ([nnz][Bm]) goes to factor f.
template <typename R>
__global__ void k_values(int64_t nnz, int64_t Bm, int64_t F, const int32_t* __restrict__ amat,
                         const double2* __restrict__ A, const int64_t* __restrict__ dmap, int64_t totD,
                         typename C2<R>::T* __restrict__ D) {
    using T = typename C2<R>::T;
    const int64_t total = nnz * F;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = t / F, f = t % F;
        const int64_t d = dmap[e];
        if (d >= 0) D[f * totD + d] = cvt<T>(A[e * Bm + amat[f]]);
    }
}

template <typename R>
__global__ void k_offvals(int64_t nn, int64_t Bm, int64_t F, const int32_t* __restrict__ amat,
                          const double2* __restrict__ A, const int64_t* __restrict__ src,
                          typename C2<R>::T* __restrict__ out) {
    using T = typename C2<R>::T;
    const int64_t total = nn * F;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = t % nn, f = t / nn;
        out[t] = cvt<T>(A[src[k] * Bm + amat[f]]);
    }
}

// S_i -= (C_i S_{i-1}^-1) U_{i-1} for rows [a0, a0+nr) of slab i (grid: row blocks x 1 x F).
template <typename R>
__global__ void __launch_bounds__(kThreads) k_schur(int64_t wp, int64_t w, int64_t row0, int rb,
                                                    const int64_t* __restrict__ cptr, const int32_t* __restrict__ cidx,
                                                    const typename C2<R>::T* __restrict__ Cval, int64_t nC,
                                                    const int64_t* __restrict__ ucptr, const int32_t* __restrict__ ucrow,
                                                    const typename C2<R>::T* __restrict__ UCval, int64_t nU,
                                                    typename C2<R>::T* __restrict__ Sinv, int64_t totD, int64_t offPrev,
                                                    int64_t offCur) {
    using T = typename C2<R>::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* Rs = reinterpret_cast<T*>(smem_raw);
    const int64_t f = blockIdx.z;
    const int64_t a0 = (int64_t)blockIdx.x * rb;
    const int nr = (int)min((int64_t)rb, w - a0);
    const T* Sp = Sinv + f * totD + offPrev;
    T* Sc = Sinv + f * totD + offCur;
    const T* Cv = Cval + f * nC;
    const T* Uv = UCval + f * nU;
    for (int64_t idx = threadIdx.x; idx < (int64_t)nr * wp; idx += blockDim.x) {
        const int64_t a = idx / wp, col = idx % wp;
        const int64_t row = row0 + a0 + a;
        T acc = czero<T>();
        for (int64_t k = cptr[row]; k < cptr[row + 1]; ++k) cfma(acc, Cv[k], Sp[(int64_t)cidx[k] * wp + col]);
        Rs[idx] = acc;
    }
    __syncthreads();
    for (int64_t j = threadIdx.x; j < w; j += blockDim.x) {
        T acc[kMaxRows];
#pragma unroll
        for (int a = 0; a < kMaxRows; ++a) acc[a] = czero<T>();
        for (int64_t k = ucptr[row0 + j]; k < ucptr[row0 + j + 1]; ++k) {
            const int64_t r = ucrow[k];
            const T u = Uv[k];
#pragma unroll
            for (int a = 0; a < kMaxRows; ++a)
                if (a < nr) cfma(acc[a], Rs[a * wp + r], u);
        }
#pragma unroll
        for (int a = 0; a < kMaxRows; ++a)
            if (a < nr) {
                T& s = Sc[(a0 + a) * w + j];
                s.x -= acc[a].x;
                s.y -= acc[a].y;
            }
    }
}

// In-place inverse of pivot tile k (tb x tb, padded with the identity when tb < 64)
// with partial pivoting inside the tile; the inverse also goes to pinv (ld 64).
// Grid 1 x 1 x F.  Gauss-Jordan: pivot = largest |a_rc| on or below the diagonal, the
// lower row on ties (magnitudes compared in FP32); pivots with |a|^2 at or below
// rel_thr^2 max|a|^2 are replaced by that threshold and counted; the row swaps are
// applied as one column permutation at the end.
//
// 256 threads as a 16 x 16 grid: thread (ty, tx) holds rows ty + 16 i and columns
// tx + 16 j (i, j < 4) of the tile in registers.  The pivot loop runs over four
// column blocks of 16 with the block index a compile-time constant, so the pivot
// column and row sit at fixed register positions.  Step c:
//   (S) the owners of row p and row c leave them in shared memory, the owners of
//       column c leave it with rows c and p exchanged, the owner of a_pc forms the
//       reciprocal of the pivot;
//   (U) the owners of row p take the old row c; column c becomes the identity column
//       and row c of the multiplier row the reciprocal, so one rank-1 update forms
//       both the eliminated entries and the new column c; row c takes the scaled
//       pivot row; the owners of column c + 1 (two lanes per warp) reduce their rows
//       to one packed (|a|^2, row) key per warp.
// Two barriers per pivot, no tile in shared memory.
template <typename T> __device__ __forceinline__ T crecip(T v);
template <> __device__ __forceinline__ float2 crecip<float2>(float2 v) {
    const float s = __frcp_rn(v.x * v.x + v.y * v.y);
    return make_float2(v.x * s, -v.y * s);
}
template <> __device__ __forceinline__ double2 crecip<double2>(double2 v) {
    const double s = __drcp_rn(v.x * v.x + v.y * v.y);
    return make_double2(v.x * s, -v.y * s);
}

// (|a|^2 as FP32 bits, 63 - row): the unsigned maximum is the largest magnitude, then the lowest row
template <typename R> __device__ __forceinline__ unsigned long long pivot_key(R m2, int r) {
    return ((unsigned long long)__float_as_uint((float)m2) << 32) | (unsigned)(63 - r);
}

template <typename R> struct DiagShared {
    using T = typename C2<R>::T;
    T prow[kTile], orow[kTile], colc[kTile];
    unsigned long long cand[kDiagThreads / 32];
    int piv[kTile], perm[kTile], iperm[kTile];
    R red[kDiagThreads / 32];
    T inv;
};

// the key of the best row r > rmin (r < tb) of column 16 JN + tx among this thread's
// rows, combined over lanes tx and tx + 16; lane tx (== column % 16) stores it
template <int JN, typename R>
__device__ __forceinline__ void diag_candidates(const typename C2<R>::T (&a)[4][4], int cn, int rmin, int tb,
                                                DiagShared<R>& sh) {
    const int tid = threadIdx.x, lane = tid & 31, ty = tid >> 4, tx = tid & 15;
    unsigned long long key = 0;
    if (tx == (cn & 15)) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int r = ty + 16 * i;
            const R m2 = a[i][JN].x * a[i][JN].x + a[i][JN].y * a[i][JN].y;
            const unsigned long long kk = (r > rmin && r < tb) ? pivot_key<R>(m2, r) : 0ull;
            key = kk > key ? kk : key;
        }
    }
    const unsigned long long o = __shfl_xor_sync(0xffffffffu, key, 16);
    key = o > key ? o : key;
    if (lane == (cn & 15)) sh.cand[tid >> 5] = key;
}

template <int JC, typename R>
__device__ __forceinline__ void diag_block(typename C2<R>::T (&a)[4][4], int tb, R thr2, typename C2<R>::T thr_pivot,
                                           DiagShared<R>& sh, int32_t* __restrict__ pert) {
    using T = typename C2<R>::T;
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    for (int cl = 0; cl < 16; ++cl) {
        const int c = 16 * JC + cl;
        if (c >= tb) return;   // uniform
        unsigned long long best = 0;
#pragma unroll
        for (int q = 0; q < kDiagThreads / 32; ++q) best = sh.cand[q] > best ? sh.cand[q] : best;
        const int p = 63 - (int)(best & 0xffffffffu);
        // (S)
#pragma unroll
        for (int i = 0; i < 4; ++i)
            if (ty + 16 * i == p) {
#pragma unroll
                for (int j = 0; j < 4; ++j) sh.prow[tx + 16 * j] = a[i][j];
                if (tx == cl) {
                    const T v = a[i][JC];
                    const bool small = !(v.x * v.x + v.y * v.y > thr2);   // also catches a zero pivot
                    sh.inv = crecip(small ? thr_pivot : v);
                    if (small) atomicAdd(pert, 1);
                }
            }
        if (ty == cl && p != c) {
#pragma unroll
            for (int j = 0; j < 4; ++j) sh.orow[tx + 16 * j] = a[JC][j];
        }
        if (tx == cl) {
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int r = ty + 16 * i;
                sh.colc[(r == p || r == c) ? (r ^ p ^ c) : r] = a[i][JC];
            }
        }
        if (tid == 0) sh.piv[c] = p;
        __syncthreads();
        // (U)
        const T inv = sh.inv;
        T rj[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) rj[j] = cmul(sh.prow[tx + 16 * j], inv);
        if (p != c) {
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if (ty + 16 * i == p) {
#pragma unroll
                    for (int j = 0; j < 4; ++j) a[i][j] = sh.orow[tx + 16 * j];
                }
        }
        if (tx == cl) {   // after the swap: column c -> 0, its multiplier -> 1 / pivot
            rj[JC] = inv;
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i][JC] = mk((R)0, (R)0);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const T cr = sh.colc[ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const T t = cmul(cr, rj[j]);
                a[i][j].x -= t.x;
                a[i][j].y -= t.y;
            }
        }
        if (ty == cl) {
#pragma unroll
            for (int j = 0; j < 4; ++j) a[JC][j] = rj[j];
        }
        if (c + 1 < tb) {
            if (cl < 15) diag_candidates<JC, R>(a, c + 1, c, tb, sh);
            else if (JC < 3) diag_candidates<(JC < 3 ? JC + 1 : 3), R>(a, c + 1, c, tb, sh);
        }
        __syncthreads();
    }
}

template <typename R>
__global__ void __launch_bounds__(kDiagThreads, 1) k_gj_diag(int64_t w, int k, typename C2<R>::T* __restrict__ Sinv,
                                                         int64_t totD, int64_t offD, typename C2<R>::T* __restrict__ pinv,
                                                         R rel_thr, int32_t* __restrict__ perturbed) {
    using T = typename C2<R>::T;
    __shared__ DiagShared<R> sh;
    const int64_t f = blockIdx.z;
    T* M = Sinv + f * totD + offD;
    const int64_t k0 = (int64_t)k * kTile;
    const int tb = (int)min((int64_t)kTile, w - k0);
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int ty = tid >> 4, tx = tid & 15;
    T a[4][4];
    R mx = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int r = ty + 16 * i, cc = tx + 16 * j;
            T v;
            if (r < tb && cc < tb) {
                v = M[(k0 + r) * w + k0 + cc];
                mx = max(mx, v.x * v.x + v.y * v.y);
            } else {
                v = mk((R)(r == cc ? 1 : 0), (R)0);
            }
            a[i][j] = v;
        }
#pragma unroll
    for (int o = 16; o; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) sh.red[wid] = mx;
    diag_candidates<0, R>(a, 0, -1, tb, sh);
    __syncthreads();
    R thr2 = 0;
#pragma unroll
    for (int i = 0; i < kDiagThreads / 32; ++i) thr2 = max(thr2, sh.red[i]);
    thr2 *= rel_thr * rel_thr;   // |pivot|^2 at or below this is replaced
    const T thr_pivot = mk(thr2 > 0 ? (R)sqrt(thr2) : (R)1, (R)0);
    int32_t* pert = perturbed + f;
    diag_block<0, R>(a, tb, thr2, thr_pivot, sh, pert);
    diag_block<1, R>(a, tb, thr2, thr_pivot, sh, pert);
    diag_block<2, R>(a, tb, thr2, thr_pivot, sh, pert);
    diag_block<3, R>(a, tb, thr2, thr_pivot, sh, pert);
    if (tid == 0) {   // the swaps in reverse give the column permutation; iperm is its inverse
        for (int c = 0; c < kTile; ++c) sh.perm[c] = c;
        for (int c = tb - 1; c >= 0; --c) {
            const int q = sh.piv[c];
            if (q != c) { const int t = sh.perm[c]; sh.perm[c] = sh.perm[q]; sh.perm[q] = t; }
        }
        for (int c = 0; c < kTile; ++c) sh.iperm[sh.perm[c]] = c;
    }
    __syncthreads();
    // column cc of the unpermuted inverse is column iperm[cc] of the result
    T* P = pinv + f * kTile * kTile;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int r = ty + 16 * i, cc = tx + 16 * j;
            if (r < tb && cc < tb) {
                const int cd = sh.iperm[cc];
                M[(k0 + r) * w + k0 + cd] = a[i][j];
                P[r * kTile + cd] = a[i][j];
            }
        }
}

// mode 0: row panel  M[k, c] = Pinv M[k, c]       (grid: column tiles x 1 x F, c != k)
// mode 1: col panel  M[r, k] = -M[r, k] Pinv      (grid: row tiles x 1 x F, r != k)
// mode 2: update     M[r, c] -= M[r, k] M[k, c]   (grid: column tiles x row tiles x F, r, c != k),
//         skipping tile (la, la) when la >= 0
// mode 3: the update of tile (la, la) alone       (grid: 1 x 1 x F)
template <typename R>
__global__ void __launch_bounds__(kThreads) k_gj_panel(int mode, int64_t w, int k, typename C2<R>::T* __restrict__ Sinv,
                                                       int64_t totD, int64_t offD, const typename C2<R>::T* __restrict__ pinv,
                                                       int la) {
    using T = typename C2<R>::T;
    __shared__ Tile<R> sm;
    const int64_t f = blockIdx.z;
    T* M = Sinv + f * totD + offD;
    const T* P = pinv + f * kTile * kTile;
    const int64_t k0 = (int64_t)k * kTile;
    const int tb = (int)min((int64_t)kTile, w - k0);
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = czero<T>();
    int64_t r0, c0;
    int nr, nc;
    T* out;
    if (mode == 0) {
        if ((int)blockIdx.x == k) return;
        c0 = (int64_t)blockIdx.x * kTile;
        nc = (int)min((int64_t)kTile, w - c0);
        nr = tb;
        out = M + k0 * w + c0;
        tile_mac<R>(acc, P, kTile, out, w, nr, nc, tb, sm);
    } else if (mode == 1) {
        if ((int)blockIdx.x == k) return;
        r0 = (int64_t)blockIdx.x * kTile;
        nr = (int)min((int64_t)kTile, w - r0);
        nc = tb;
        out = M + r0 * w + k0;
        tile_mac<R>(acc, out, w, P, kTile, nr, nc, tb, sm);
    } else {
        const int bx = mode == 3 ? la : (int)blockIdx.x, by = mode == 3 ? la : (int)blockIdx.y;
        if (bx == k || by == k || (mode == 2 && bx == la && by == la)) return;
        r0 = (int64_t)by * kTile;
        c0 = (int64_t)bx * kTile;
        nr = (int)min((int64_t)kTile, w - r0);
        nc = (int)min((int64_t)kTile, w - c0);
        out = M + r0 * w + c0;
        tile_mac<R>(acc, M + r0 * w + k0, w, M + k0 * w + c0, w, nr, nc, tb, sm);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int r = ty + 16 * i, c = tx + 16 * j;
            if (r < nr && c < nc) {
                T& o = out[(int64_t)r * w + c];
                if (mode == 0) o = acc[i][j];
                else if (mode == 1) o = mk(-acc[i][j].x, -acc[i][j].y);
                else { o.x -= acc[i][j].x; o.y -= acc[i][j].y; }
            }
        }
}

// C = alpha A B + diag I for F batched w x w row-major blocks (batch stride
// ``stride``; C aliases neither A nor B).  Grid: column tiles x row tiles x F.
template <typename R>
__global__ void __launch_bounds__(kThreads) k_sq_gemm(int64_t w, const typename C2<R>::T* __restrict__ A,
                                                      int64_t sA, const typename C2<R>::T* __restrict__ B, int64_t sB,
                                                      typename C2<R>::T* __restrict__ C, int64_t sC, R alpha, R diag) {
    using T = typename C2<R>::T;
    __shared__ Tile<R> sm;
    const int64_t f = blockIdx.z;
    const int64_t c0 = (int64_t)blockIdx.x * kTile, r0 = (int64_t)blockIdx.y * kTile;
    const int nr = (int)min((int64_t)kTile, w - r0), nc = (int)min((int64_t)kTile, w - c0);
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = czero<T>();
    tile_mac<R>(acc, A + f * sA + r0 * w, w, B + f * sB + c0, w, nr, nc, w, sm);
    T* Cf = C + f * sC;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int r = ty + 16 * i, c = tx + 16 * j;
            if (r < nr && c < nc) {
                T v = mk(alpha * acc[i][j].x, alpha * acc[i][j].y);
                if (r0 + r == c0 + c) v.x += diag;
                Cf[(r0 + r) * w + c0 + c] = v;
            }
        }
}

// Per-block partial sums of |R_ij - delta_ij|^2 over a w x w block per factor, then
// their ordered total (deterministic): part[f][b], nrm2[f].
constexpr int kNormBlocks = 64;
template <typename R>
__global__ void k_dev_partial(int64_t w, const typename C2<R>::T* __restrict__ Rm, int64_t sq, double* __restrict__ part) {
    const int64_t f = blockIdx.y;
    const typename C2<R>::T* M = Rm + f * sq;
    double acc = 0.0;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < w * w; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t / w, c = t % w;
        const double x = (double)M[t].x - (r == c ? 1.0 : 0.0), y = (double)M[t].y;
        acc += x * x + y * y;
    }
    __shared__ double red[kThreads];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = kThreads / 2; o; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[f * kNormBlocks + blockIdx.x] = red[0];
}

// X <- Xn for the factors whose refinement residual ||I - S X||_F is below 1/2
// (Newton-Schulz only converges when the residual is below 1); counts the others.
template <typename R>
__global__ void k_copy_if(int64_t w, const typename C2<R>::T* __restrict__ Xn, int64_t sq, typename C2<R>::T* __restrict__ X,
                          int64_t totD, const double* __restrict__ part, int32_t* __restrict__ skipped) {
    const int64_t f = blockIdx.y;
    double n2 = 0.0;
    for (int b = 0; b < kNormBlocks; ++b) n2 += part[f * kNormBlocks + b];
    if (!(n2 < 0.25)) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(skipped + f, 1);
        return;
    }
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < w * w; t += (int64_t)gridDim.x * blockDim.x)
        X[f * totD + t] = Xn[f * sq + t];
}

// ------------------------------------------------------------------- solve ---
__device__ __forceinline__ float2 as_t(float2 v, float2) { return v; }
__device__ __forceinline__ float2 as_t(double2 v, float2) { return make_float2((float)v.x, (float)v.y); }
__device__ __forceinline__ double2 as_t(float2 v, double2) { return make_double2(v.x, v.y); }
__device__ __forceinline__ double2 as_t(double2 v, double2) { return v; }

// Y[pos] = X[perm[pos]] (restricted order -> slab order), converting the vector type
template <typename R, typename TI>
__global__ void k_gather(int64_t n, int64_t Bc, const int32_t* __restrict__ perm, const TI* __restrict__ X,
                         typename C2<R>::T* __restrict__ Y) {
    using T = typename C2<R>::T;
    const int64_t total = n * Bc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t pos = t / Bc, c = t % Bc;
        Y[t] = as_t(X[(int64_t)perm[pos] * Bc + c], T{});
    }
}

template <typename R, typename TI>
__global__ void k_scatter(int64_t n, int64_t Bc, const int32_t* __restrict__ perm, const typename C2<R>::T* __restrict__ Z,
                          TI* __restrict__ X) {
    const int64_t total = n * Bc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t pos = t / Bc, c = t % Bc;
        X[(int64_t)perm[pos] * Bc + c] = as_t(Z[t], TI{});
    }
}

// mode 0: Y[row] -= sum C[row,k] Z[prev0 + cidx[k]]    (forward coupling)
// mode 1: Y[row]  = sum U[row,k] Z[next0 + uidx[k]]    (backward coupling)
template <typename R>
__global__ void k_couple(int mode, int64_t w, int64_t row0, int64_t nb0, int64_t Bc, const int32_t* __restrict__ colfac,
                         const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                         const typename C2<R>::T* __restrict__ val, int64_t nval, const typename C2<R>::T* __restrict__ Z,
                         typename C2<R>::T* __restrict__ Y) {
    using T = typename C2<R>::T;
    const int64_t total = w * Bc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = row0 + t / Bc, c = t % Bc;
        const T* v = val + (int64_t)colfac[c] * nval;
        T s = czero<T>();
        for (int64_t k = ptr[row]; k < ptr[row + 1]; ++k) cfma(s, v[k], Z[(nb0 + idx[k]) * Bc + c]);
        T& y = Y[row * Bc + c];
        if (mode == 0) { y.x -= s.x; y.y -= s.y; }
        else y = s;
    }
}

struct Group {
    int32_t fac, col0, ncol, pad;
};

__global__ void k_narrow(int64_t nv, const double2* __restrict__ in, float2* __restrict__ out) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nv; t += (int64_t)gridDim.x * blockDim.x)
        out[t] = make_float2((float)in[t].x, (float)in[t].y);
}

// Out[r, cols of group g] = beta Out + alpha S_i^-1[r, :] Y[:, cols]: warp per row,
// lanes over the row of S_i^-1 (coalesced), 16 columns per pass.  Grid: row blocks x groups.
constexpr int kRowCols = 16;
template <typename R>
__global__ void __launch_bounds__(kThreads) k_rowmv(int64_t w, int64_t row0, int64_t Bc, const Group* __restrict__ groups,
                                                    const typename C2<R>::T* __restrict__ Sinv, int64_t totD, int64_t offD,
                                                    const typename C2<R>::T* __restrict__ Y, R alpha, int beta,
                                                    typename C2<R>::T* __restrict__ Out) {
    using T = typename C2<R>::T;
    const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= w) return;
    const Group g = groups[blockIdx.y];
    const T* S = Sinv + (int64_t)g.fac * totD + offD + r * w;
    const T* Yb = Y + row0 * Bc;
    for (int c0 = 0; c0 < g.ncol; c0 += kRowCols) {
        const int nc = min(kRowCols, g.ncol - c0);
        const int64_t cb = g.col0 + c0;
        T acc[kRowCols];
#pragma unroll
        for (int j = 0; j < kRowCols; ++j) acc[j] = czero<T>();
        for (int64_t k = lane; k < w; k += 32) {
            const T s = S[k];
            const T* yr = Yb + k * Bc + cb;
#pragma unroll
            for (int j = 0; j < kRowCols; ++j)
                if (j < nc) cfma(acc[j], s, yr[j]);
        }
#pragma unroll
        for (int j = 0; j < kRowCols; ++j) {
#pragma unroll
            for (int o = 16; o; o >>= 1) {
                acc[j].x += __shfl_xor_sync(0xffffffffu, acc[j].x, o);
                acc[j].y += __shfl_xor_sync(0xffffffffu, acc[j].y, o);
            }
        }
        if (lane < nc) {
            T v = acc[0];
#pragma unroll
            for (int j = 1; j < kRowCols; ++j)
                if (j == lane) v = acc[j];
            T& o = Out[(row0 + r) * Bc + cb + lane];
            const T res = mk(alpha * v.x, alpha * v.y);
            if (beta) { o.x += res.x; o.y += res.y; }
            else o = res;
        }
    }
}

// The same product for wide groups: 64 x 64 output tiles through tile_mac, with
// the K range split over ``splits`` CTAs when the tiles alone would not fill the
// GPU.  A split writes its partial tile to ``part``; the last split of a tile to
// arrive (per-tile counter) adds the partials in split order, so the result does
// not depend on arrival order, writes the output and resets the counter.
// Grid: column tiles x (row tiles * splits) x groups.
template <typename R>
__global__ void __launch_bounds__(kThreads) k_slab_gemm(int64_t w, int64_t row0, int64_t Bc,
                                                        const Group* __restrict__ groups,
                                                        const typename C2<R>::T* __restrict__ Sinv, int64_t totD,
                                                        int64_t offD, const typename C2<R>::T* __restrict__ Y, R alpha,
                                                        int beta, typename C2<R>::T* __restrict__ Out, int splits,
                                                        typename C2<R>::T* __restrict__ part, int32_t* __restrict__ cnt) {
    using T = typename C2<R>::T;
    __shared__ Tile<R> sm;
    __shared__ int s_last;
    const Group g = groups[blockIdx.z];
    const int rt = (int)blockIdx.y / splits, sp = (int)blockIdx.y % splits;
    const int64_t c0 = (int64_t)blockIdx.x * kTile, r0 = (int64_t)rt * kTile;
    if (c0 >= g.ncol) return;
    const int nr = (int)min((int64_t)kTile, w - r0), nc = (int)min((int64_t)kTile, (int64_t)g.ncol - c0);
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    const int64_t kper = (w + splits - 1) / splits;
    const int64_t ks0 = min(w, (int64_t)sp * kper), ks1 = min(w, ks0 + kper);
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = czero<T>();
    tile_mac<R>(acc, Sinv + (int64_t)g.fac * totD + offD + r0 * w + ks0, w, Y + (row0 + ks0) * Bc + g.col0 + c0, Bc, nr,
                nc, ks1 - ks0, sm);
    if (splits > 1) {
        const int64_t tile = ((int64_t)blockIdx.z * (gridDim.y / splits) + rt) * gridDim.x + blockIdx.x;
        T* mine = part + (tile * splits + sp) * (kTile * kTile);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) mine[(ty + 16 * i) * kTile + tx + 16 * j] = acc[i][j];
        __threadfence();
        __syncthreads();
        if (tid == 0) s_last = atomicAdd(cnt + tile, 1) == splits - 1;
        __syncthreads();
        if (!s_last) return;
        __threadfence();
        const T* all = part + tile * splits * (kTile * kTile);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int e = (ty + 16 * i) * kTile + tx + 16 * j;
                T v = czero<T>();
                for (int q = 0; q < splits; ++q) {
                    const T pq = __ldcg(all + (int64_t)q * kTile * kTile + e);
                    v.x += pq.x;
                    v.y += pq.y;
                }
                acc[i][j] = v;
            }
        if (tid == 0) cnt[tile] = 0;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int r = ty + 16 * i, c = tx + 16 * j;
            if (r < nr && c < nc) {
                T& o = Out[(row0 + r0 + r) * Bc + g.col0 + c0 + c];
                const T res = mk(alpha * acc[i][j].x, alpha * acc[i][j].y);
                if (beta) { o.x += res.x; o.y += res.y; }
                else o = res;
            }
        }
}

// The same product for groups of at most 16 columns (the training and per-point
// solves): 128 x 16 output tiles, so no work is spent on absent columns.  Thread t
// owns rows t / 4 and t / 4 + 64 and columns 4 (t % 4) .. + 3 (8 complex
// accumulators); S^-1 chunks are staged K-major ([k][row]) and Y chunks row-major in
// shared memory, double-buffered through registers.  K is split over CTAs as in
// k_slab_gemm (partials reduced by the last split in split order; part slots of
// kNarrowM x kNarrowN).  Grid: 1 x (row tiles * splits) x groups.
constexpr int kNarrowM = 128, kNarrowN = 16;
template <typename R> struct NarrowTile {
    using T = typename C2<R>::T;
    static constexpr int BK = sizeof(R) == 4 ? 32 : 16;
    T s[2][BK][kNarrowM + 1];
    T y[2][BK][kNarrowN];
};
template <typename R>
__global__ void __launch_bounds__(kThreads) k_slab_gemm16(int64_t w, int64_t row0, int64_t Bc,
                                                          const Group* __restrict__ groups,
                                                          const typename C2<R>::T* __restrict__ Sinv, int64_t totD,
                                                          int64_t offD, const typename C2<R>::T* __restrict__ Y, R alpha,
                                                          int beta, typename C2<R>::T* __restrict__ Out, int splits,
                                                          typename C2<R>::T* __restrict__ part, int32_t* __restrict__ cnt) {
    using T = typename C2<R>::T;
    constexpr int BK = NarrowTile<R>::BK;
    constexpr int LS = kNarrowM * BK / kThreads;   // S elements per thread and chunk
    constexpr int LY = BK * kNarrowN / kThreads;   // Y elements per thread and chunk
    extern __shared__ __align__(16) unsigned char smem_raw[];
    NarrowTile<R>& sm = *reinterpret_cast<NarrowTile<R>*>(smem_raw);
    __shared__ int s_last;
    const Group g = groups[blockIdx.z];
    const int rt = (int)blockIdx.y / splits, sp = (int)blockIdx.y % splits;
    const int64_t r0 = (int64_t)rt * kNarrowM;
    const int nr = (int)min((int64_t)kNarrowM, w - r0), nc = min(kNarrowN, g.ncol);
    const int tid = threadIdx.x, ty = tid >> 2, cx = (tid & 3) * 4;
    const int64_t kper = (w + splits - 1) / splits;
    const int64_t ks0 = min(w, (int64_t)sp * kper), ks1 = min(w, ks0 + kper);
    const T* S = Sinv + (int64_t)g.fac * totD + offD + r0 * w;
    const T* Yb = Y + row0 * Bc + g.col0;
    T rs[LS], ry[LY];
    auto load = [&](int64_t k0) {
#pragma unroll
        for (int q = 0; q < LS; ++q) {
            const int idx = tid + kThreads * q;
            const int r = idx / BK, kk = idx % BK;
            rs[q] = (r < nr && k0 + kk < ks1) ? S[(int64_t)r * w + k0 + kk] : czero<T>();
        }
#pragma unroll
        for (int q = 0; q < LY; ++q) {
            const int idx = tid + kThreads * q;
            const int kk = idx / kNarrowN, c = idx % kNarrowN;
            ry[q] = (c < nc && k0 + kk < ks1) ? Yb[(k0 + kk) * Bc + c] : czero<T>();
        }
    };
    auto store = [&](int buf) {
#pragma unroll
        for (int q = 0; q < LS; ++q) {
            const int idx = tid + kThreads * q;
            sm.s[buf][idx % BK][idx / BK] = rs[q];
        }
#pragma unroll
        for (int q = 0; q < LY; ++q) {
            const int idx = tid + kThreads * q;
            sm.y[buf][idx / kNarrowN][idx % kNarrowN] = ry[q];
        }
    };
    T acc[2][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = czero<T>();
    if (ks0 < ks1) {
        load(ks0);
        store(0);
        __syncthreads();
        int buf = 0;
        for (int64_t k0 = ks0; k0 < ks1; k0 += BK) {
            const bool more = k0 + BK < ks1;
            if (more) load(k0 + BK);
#pragma unroll 8
            for (int kk = 0; kk < BK; ++kk) {
                const T a0 = sm.s[buf][kk][ty], a1 = sm.s[buf][kk][ty + 64];
                T b[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) b[j] = sm.y[buf][kk][cx + j];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    cfma(acc[0][j], a0, b[j]);
                    cfma(acc[1][j], a1, b[j]);
                }
            }
            if (more) store(buf ^ 1);
            __syncthreads();
            buf ^= 1;
        }
    }
    if (splits > 1) {
        constexpr int kSlot = kNarrowM * kNarrowN;
        const int64_t tile = (int64_t)blockIdx.z * (gridDim.y / splits) + rt;
        T* mine = part + (tile * splits + sp) * kSlot;
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) mine[(ty + 64 * i) * kNarrowN + cx + j] = acc[i][j];
        __threadfence();
        __syncthreads();
        if (tid == 0) s_last = atomicAdd(cnt + tile, 1) == splits - 1;
        __syncthreads();
        if (!s_last) return;
        __threadfence();
        const T* all = part + tile * splits * kSlot;
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int e = (ty + 64 * i) * kNarrowN + cx + j;
                T v = czero<T>();
                for (int q = 0; q < splits; ++q) {
                    const T pq = __ldcg(all + (int64_t)q * kSlot + e);
                    v.x += pq.x;
                    v.y += pq.y;
                }
                acc[i][j] = v;
            }
        if (tid == 0) cnt[tile] = 0;
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int r = ty + 64 * i, c = cx + j;
            if (r < nr && c < nc) {
                T& o = Out[(row0 + r0 + r) * Bc + g.col0 + c];
                const T res = mk(alpha * acc[i][j].x, alpha * acc[i][j].y);
                if (beta) { o.x += res.x; o.y += res.y; }
                else o = res;
            }
        }
}

// K splits of a wide-group product: enough CTAs for two per SM, at least 256
// columns of K per split, at most max_splits (8 unless tuned).
inline int gemm_splits(int64_t tiles, int64_t w, int max_splits = 8) {
    int64_t sp = (2 * 152 + tiles - 1) / std::max<int64_t>(tiles, 1);
    sp = std::min<int64_t>(sp, std::max<int64_t>(1, w / 256));
    return (int)std::max<int64_t>(1, std::min<int64_t>(sp, std::max(1, max_splits)));
}

}  // namespace slab
}  // namespace emg

// ------------------------------------------------------------------- plan ---
struct emg_slab {
    emg_rplan* rp = nullptr;
    int64_t n = 0, nnz = 0;
    int m = 0;
    std::vector<int64_t> off, offD;   // slab boundaries (positions), dense block offsets
    int64_t totD = 0, maxw = 0, nC = 0, nU = 0;
    int32_t* perm = nullptr;          // slab position -> restricted index
    int64_t* dmap = nullptr;          // restricted entry -> dense index or -1
    int64_t *cptr = nullptr, *csrc = nullptr;
    int32_t* cidx = nullptr;
    int64_t *uptr = nullptr, *usrc = nullptr;
    int32_t* uidx = nullptr;
    int64_t *ucptr = nullptr, *ucsrc = nullptr;
    int32_t* ucrow = nullptr;
    // factors
    int prec = 0;                     // 1 complex FP32, 2 complex FP64
    int64_t F = 0;
    void *Sinv = nullptr, *Cval = nullptr, *Uval = nullptr, *UCval = nullptr, *pinv = nullptr;
    int32_t* perturbed = nullptr;     // [F] perturbed pivots, [F] skipped refinements
    int64_t n_perturbed = 0, n_refine_skipped = 0;
    // solve workspace
    int64_t ws_cols = 0;
    size_t ws_bytes = 0;
    void *Y = nullptr, *Z = nullptr;
    int32_t* colfac = nullptr;
    emg::slab::Group* groups = nullptr;
    int64_t ngroups_cap = 0;
    void* kpart = nullptr;            // split-K partial tiles of the wide-group products
    size_t kpart_bytes = 0;
    int32_t* kcnt = nullptr;          // per-tile arrival counters (zero between launches)
    int64_t kcnt_n = 0;
    int use_tc = 0;                   // wide-group products of FP32 factors on the tcgen05 tensor cores
    int tc_factor = 1;                // rank-64 updates of FP32 factorizations on the tcgen05 tensor cores
    int wide = 8;                     // column groups at least this wide use the tiled products
    int max_splits = 8;               // split-K cap of the tiled products
    int32_t* tc_status = nullptr;     // set by a tensor-core tile whose bounded wait ran out
};

namespace {
using namespace emg;

void slab_free_factors(emg_slab* s) {
    dfree(s->Sinv); dfree(s->Cval); dfree(s->Uval); dfree(s->UCval); dfree(s->pinv); dfree(s->perturbed);
    s->F = 0;
    s->prec = 0;
}

void slab_free(emg_slab* s) {
    if (!s) return;
    slab_free_factors(s);
    dfree(s->perm); dfree(s->dmap); dfree(s->cptr); dfree(s->csrc); dfree(s->cidx); dfree(s->uptr); dfree(s->usrc);
    dfree(s->uidx); dfree(s->ucptr); dfree(s->ucsrc); dfree(s->ucrow); dfree(s->Y); dfree(s->Z); dfree(s->colfac);
    dfree(s->groups); dfree(s->tc_status); dfree(s->kcnt);
    if (s->kpart) cudaFree(s->kpart);
    delete s;
}

template <typename V>
int upload(V** d, const std::vector<V>& h, const char* what) {
    int rc = dalloc(d, (int64_t)std::max<size_t>(h.size(), 1), what);
    if (rc) return rc;
    if (!h.empty()) EMG_CUDA(cudaMemcpy(*d, h.data(), sizeof(V) * h.size(), cudaMemcpyHostToDevice));
    return EMG_OK;
}

// Breadth-first levels over the nodes not yet placed, from one or more start
// nodes (all at level ``base``); returns the reached nodes in level order.
std::vector<int64_t> bfs(const std::vector<int64_t>& starts, const std::vector<int64_t>& ptr,
                         const std::vector<int32_t>& ind, std::vector<int32_t>& lev, int32_t base) {
    std::vector<int64_t> order;
    for (int64_t s : starts)
        if (lev[s] < 0) {
            lev[s] = base;
            order.push_back(s);
        }
    for (size_t h = 0; h < order.size(); ++h) {
        const int64_t v = order[h];
        for (int64_t k = ptr[v]; k < ptr[v + 1]; ++k) {
            const int64_t u = ind[k];
            if (lev[u] < 0) {
                lev[u] = lev[v] + 1;
                order.push_back(u);
            }
        }
    }
    return order;
}
}  // namespace

extern "C" int emg_slab_create(const emg_rplan* rp, int64_t n_seeds, const int64_t* seeds, const int64_t* order_key,
                               void* stream, emg_slab** out) {
    using namespace emg;
    EMG_CHECK_ARG(rp && out && n_seeds >= 0 && (n_seeds == 0 || seeds), "emg_slab_create: NULL argument");
    for (int64_t i = 0; i < n_seeds; ++i)
        EMG_CHECK_ARG(seeds[i] >= 0 && seeds[i] < rp->ns, "emg_slab_create: seed out of range");
    *out = nullptr;
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t n = rp->ns, nnz = rp->nnz;
    std::vector<int64_t> ptr(n + 1);
    std::vector<int32_t> ind(nnz);
    EMG_CUDA(cudaMemcpyAsync(ptr.data(), rp->rptr, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, st));
    if (nnz) EMG_CUDA(cudaMemcpyAsync(ind.data(), rp->rind, sizeof(int32_t) * nnz, cudaMemcpyDeviceToHost, st));
    EMG_CUDA(cudaStreamSynchronize(st));
    // levels: the seeds' components by one multi-source BFS from the seeds (e.g. the
    // DOFs next to one face: planar slabs); every other connected component by BFS
    // from a pseudo-peripheral node (three sweeps, each restarting from a
    // minimum-degree node of the last level)
    std::vector<int32_t> lev(n, -1), tmp(n, -1);
    int32_t base = 0;
    if (n_seeds > 0) {
        std::vector<int64_t> st0(seeds, seeds + n_seeds);
        std::vector<int64_t> ord = bfs(st0, ptr, ind, lev, base);
        for (int64_t v : ord) base = std::max(base, lev[v] + 1);
    }
    for (int64_t s0 = 0; s0 < n; ++s0) {
        if (lev[s0] >= 0) continue;
        int64_t start = s0;
        for (int sweep = 0; sweep < 3; ++sweep) {
            std::vector<int64_t> ord = bfs({start}, ptr, ind, tmp, 0);
            const int32_t last = tmp[ord.back()];
            int64_t best = ord.back();
            for (auto it = ord.rbegin(); it != ord.rend() && tmp[*it] == last; ++it)
                if (ptr[*it + 1] - ptr[*it] < ptr[best + 1] - ptr[best] ||
                    (ptr[*it + 1] - ptr[*it] == ptr[best + 1] - ptr[best] && *it < best))
                    best = *it;
            for (int64_t v : ord) tmp[v] = -1;
            start = best;
        }
        std::vector<int64_t> ord = bfs({start}, ptr, ind, lev, base);
        int32_t top = base;
        for (int64_t v : ord) top = std::max(top, lev[v]);
        base = top + 1;
    }
    const int m = base;
    auto* s = new emg_slab();
    s->rp = const_cast<emg_rplan*>(rp);
    s->n = n;
    s->nnz = nnz;
    s->m = m;
    s->off.assign(m + 1, 0);
    for (int64_t v = 0; v < n; ++v) s->off[lev[v] + 1]++;
    for (int i = 0; i < m; ++i) s->off[i + 1] += s->off[i];
    s->offD.assign(m + 1, 0);
    for (int i = 0; i < m; ++i) {
        const int64_t w = s->off[i + 1] - s->off[i];
        s->maxw = std::max(s->maxw, w);
        s->offD[i + 1] = s->offD[i] + w * w;
    }
    s->totD = s->offD[m];
    if (s->maxw > slab::kMaxWidth) {
        delete s;
        set_error("emg_slab_create: a slab is wider than 12288 DOFs (structure not slab-like)");
        return EMG_ERR_LIMIT;
    }
    // positions: slabs in order; inside a slab ascending order_key (then restricted
    // index), or restricted index without a key.  The order decides which DOFs share
    // a 64 x 64 pivot tile of the slab inverse, and with it the FP32 accuracy: a
    // spatially local order with the two DOFs of an entity adjacent keeps strongly
    // coupled DOFs in the same tile.
    std::vector<int32_t> perm(n);
    std::vector<int64_t> ipos(n), fill(s->off.begin(), s->off.end() - 1);
    std::vector<int64_t> vs(n);
    for (int64_t v = 0; v < n; ++v) vs[v] = v;
    std::stable_sort(vs.begin(), vs.end(), [&](int64_t a, int64_t b) {
        if (lev[a] != lev[b]) return lev[a] < lev[b];
        if (order_key && order_key[a] != order_key[b]) return order_key[a] < order_key[b];
        return a < b;
    });
    for (int64_t v : vs) {
        const int64_t p = fill[lev[v]]++;
        perm[p] = (int32_t)v;
        ipos[v] = p;
    }
    std::vector<int64_t> dmap(nnz, -1), cptr(n + 1, 0), uptr(n + 1, 0), ucptr(n + 1, 0);
    // count
    for (int64_t r = 0; r < n; ++r) {
        const int32_t lr = lev[r];
        for (int64_t k = ptr[r]; k < ptr[r + 1]; ++k) {
            const int64_t c = ind[k];
            const int32_t lc = lev[c];
            if (lc == lr - 1) cptr[ipos[r] + 1]++;
            else if (lc == lr + 1) { uptr[ipos[r] + 1]++; ucptr[ipos[c] + 1]++; }
            else if (lc != lr) {
                delete s;
                set_error("emg_slab_create: entry couples non-adjacent slabs");
                return EMG_ERR_MESH;
            }
        }
    }
    for (int64_t i = 0; i < n; ++i) { cptr[i + 1] += cptr[i]; uptr[i + 1] += uptr[i]; ucptr[i + 1] += ucptr[i]; }
    s->nC = cptr[n];
    s->nU = uptr[n];
    std::vector<int32_t> cidx(s->nC), uidx(s->nU), ucrow(s->nU);
    std::vector<int64_t> csrc(s->nC), usrc(s->nU), ucsrc(s->nU);
    std::vector<int64_t> cf(cptr.begin(), cptr.end() - 1), uf(uptr.begin(), uptr.end() - 1), ucf(ucptr.begin(), ucptr.end() - 1);
    // rows in slab-position order so each row's entries come out sorted by column position
    for (int64_t p = 0; p < n; ++p) {
        const int64_t r = perm[p];
        const int32_t lr = lev[r];
        std::vector<std::pair<int64_t, int64_t>> ents;   // (column position, entry)
        for (int64_t k = ptr[r]; k < ptr[r + 1]; ++k) ents.emplace_back(ipos[ind[k]], k);
        std::sort(ents.begin(), ents.end());
        for (auto& pe : ents) {
            const int64_t pc = pe.first, k = pe.second;
            const int32_t lc = lev[perm[pc]];
            if (lc == lr) {
                const int64_t w = s->off[lr + 1] - s->off[lr];
                dmap[k] = s->offD[lr] + (p - s->off[lr]) * w + (pc - s->off[lr]);
            } else if (lc == lr - 1) {
                cidx[cf[p]] = (int32_t)(pc - s->off[lc]);
                csrc[cf[p]++] = k;
            } else {
                uidx[uf[p]] = (int32_t)(pc - s->off[lc]);
                usrc[uf[p]++] = k;
                ucrow[ucf[pc]] = (int32_t)(p - s->off[lr]);
                ucsrc[ucf[pc]++] = k;
            }
        }
    }
    int rc = upload(&s->perm, perm, "slab perm");
    if (!rc) rc = upload(&s->dmap, dmap, "slab dmap");
    if (!rc) rc = upload(&s->cptr, cptr, "slab cptr");
    if (!rc) rc = upload(&s->cidx, cidx, "slab cidx");
    if (!rc) rc = upload(&s->csrc, csrc, "slab csrc");
    if (!rc) rc = upload(&s->uptr, uptr, "slab uptr");
    if (!rc) rc = upload(&s->uidx, uidx, "slab uidx");
    if (!rc) rc = upload(&s->usrc, usrc, "slab usrc");
    if (!rc) rc = upload(&s->ucptr, ucptr, "slab ucptr");
    if (!rc) rc = upload(&s->ucrow, ucrow, "slab ucrow");
    if (!rc) rc = upload(&s->ucsrc, ucsrc, "slab ucsrc");
    if (rc) {
        slab_free(s);
        return rc;
    }
    *out = s;
    return EMG_OK;
}

extern "C" void emg_slab_destroy(emg_slab* s) { slab_free(s); }

extern "C" int emg_slab_info(const emg_slab* s, int64_t* info) {
    EMG_CHECK_ARG(s && info, "emg_slab_info: NULL argument");
    info[0] = s->m;
    info[1] = s->maxw;
    info[2] = s->totD;
    info[3] = s->nC;
    info[4] = s->F;
    info[5] = s->prec;
    info[6] = s->n_perturbed;
    info[7] = s->n_refine_skipped;
    return EMG_OK;
}

extern "C" int emg_slab_levels(const emg_slab* s, int64_t* off_out, int32_t* perm_out) {
    EMG_CHECK_ARG(s && off_out, "emg_slab_levels: NULL argument");
    std::copy(s->off.begin(), s->off.end(), off_out);
    if (perm_out) EMG_CUDA(cudaMemcpy(perm_out, s->perm, sizeof(int32_t) * s->n, cudaMemcpyDeviceToHost));
    return EMG_OK;
}

namespace {
template <typename R>
int slab_factor_t(emg_slab* s, int64_t F, const int32_t* amat_h, int64_t Bm, const double2* A, int refine,
                  cudaStream_t st) {
    using namespace emg::slab;
    using T = typename C2<R>::T;
    slab_free_factors(s);
    int rc = dalloc(reinterpret_cast<T**>(&s->Sinv), F * s->totD, "slab inverse blocks");
    if (!rc) rc = dalloc(reinterpret_cast<T**>(&s->Cval), F * std::max<int64_t>(s->nC, 1), "slab C values");
    if (!rc) rc = dalloc(reinterpret_cast<T**>(&s->Uval), F * std::max<int64_t>(s->nU, 1), "slab U values");
    if (!rc) rc = dalloc(reinterpret_cast<T**>(&s->UCval), F * std::max<int64_t>(s->nU, 1), "slab U values (by column)");
    // two sets of pivot-tile inverses: step k's is read while step k + 1's is formed
    if (!rc) rc = dalloc(reinterpret_cast<T**>(&s->pinv), 2 * F * kTile * kTile, "slab pivot tiles");
    if (!rc) rc = dalloc(&s->perturbed, 2 * F, "slab pivot counters");
    if (rc) { slab_free_factors(s); return rc; }
    s->F = F;
    s->prec = sizeof(R) == 4 ? 1 : 2;
    int32_t* amat = nullptr;
    rc = dalloc(&amat, F, "slab amat");
    if (rc) { slab_free_factors(s); return rc; }
    struct Tmp { int32_t* p; ~Tmp() { if (p) cudaFree(p); } } tmp{amat};
    // Newton-Schulz scratch: a copy of S_i and the factor 2I - S_i X (F blocks of maxw^2)
    T *Scopy = nullptr, *Rbuf = nullptr;
    double* npart = nullptr;
    const int64_t sq = s->maxw * s->maxw;
    if (refine > 0) {
        rc = dalloc(&Scopy, F * sq, "slab refinement copy");
        if (!rc) rc = dalloc(&Rbuf, F * sq, "slab refinement factor");
        if (!rc) rc = dalloc(&npart, F * kNormBlocks, "slab refinement norms");
        if (rc) { dfree(Scopy); dfree(Rbuf); slab_free_factors(s); return rc; }
    }
    struct Tmp2 {
        T* a; T* b; double* c;
        ~Tmp2() { if (a) cudaFree(a); if (b) cudaFree(b); if (c) cudaFree(c); }
    } tmp2{Scopy, Rbuf, npart};
    EMG_CUDA(cudaMemcpyAsync(amat, amat_h, sizeof(int32_t) * F, cudaMemcpyHostToDevice, st));
    EMG_CUDA(cudaMemsetAsync(s->perturbed, 0, sizeof(int32_t) * 2 * F, st));
    T* Sinv = static_cast<T*>(s->Sinv);
    EMG_CUDA(cudaMemsetAsync(Sinv, 0, sizeof(T) * F * s->totD, st));
    k_values<R><<<grid_for(s->nnz * F, 256), 256, 0, st>>>(s->nnz, Bm, F, amat, A, s->dmap, s->totD, Sinv);
    if (s->nC)
        k_offvals<R><<<grid_for(s->nC * F, 256), 256, 0, st>>>(s->nC, Bm, F, amat, A, s->csrc, static_cast<T*>(s->Cval));
    if (s->nU) {
        k_offvals<R><<<grid_for(s->nU * F, 256), 256, 0, st>>>(s->nU, Bm, F, amat, A, s->usrc, static_cast<T*>(s->Uval));
        k_offvals<R><<<grid_for(s->nU * F, 256), 256, 0, st>>>(s->nU, Bm, F, amat, A, s->ucsrc, static_cast<T*>(s->UCval));
    }
    EMG_CUDA(cudaGetLastError());
    EMG_CUDA(cudaFuncSetAttribute(k_schur<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSchurSmem));
    const R rel_thr = sizeof(R) == 4 ? (R)1e-6 : (R)1e-13;
    // the side stream of the pivot-tile lookahead and its two events
    struct Side {
        cudaStream_t st = nullptr;
        cudaEvent_t tile_ready = nullptr, diag_done = nullptr;
        ~Side() {
            if (tile_ready) cudaEventDestroy(tile_ready);
            if (diag_done) cudaEventDestroy(diag_done);
            if (st) cudaStreamDestroy(st);
        }
    } side;
    // the pivot-tile inverses are on the critical path: the side stream gets the highest priority
    int prio_lo = 0, prio_hi = 0;
    EMG_CUDA(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
    EMG_CUDA(cudaStreamCreateWithPriority(&side.st, cudaStreamNonBlocking, prio_hi));
    const bool tc_update = sizeof(R) == 4 && s->tc_factor;
    if (tc_update && !s->tc_status) {
        rc = dalloc(&s->tc_status, 1, "slab tensor-core status");
        if (rc) return rc;
        EMG_CUDA(cudaMemsetAsync(s->tc_status, 0, sizeof(int32_t), st));
    }
    EMG_CUDA(cudaEventCreateWithFlags(&side.tile_ready, cudaEventDisableTiming));
    EMG_CUDA(cudaEventCreateWithFlags(&side.diag_done, cudaEventDisableTiming));
    for (int i = 0; i < s->m; ++i) {
        const int64_t w = s->off[i + 1] - s->off[i];
        if (i > 0) {
            const int64_t wp = s->off[i] - s->off[i - 1];
            // rows per CTA: enough CTAs for two per SM, at most kMaxRows, within shared memory
            const int64_t rb_grid = std::max<int64_t>(1, (w * F) / (2 * 152));
            const int rb = (int)std::max<int64_t>(
                1, std::min<int64_t>({(int64_t)kMaxRows, kSchurSmem / (wp * (int64_t)sizeof(T)), rb_grid}));
            const dim3 g((unsigned)((w + rb - 1) / rb), 1, (unsigned)F);
            k_schur<R><<<g, kThreads, (size_t)rb * wp * sizeof(T), st>>>(
                wp, w, s->off[i], rb, s->cptr, s->cidx, static_cast<const T*>(s->Cval), s->nC, s->ucptr, s->ucrow,
                static_cast<const T*>(s->UCval), s->nU, Sinv, s->totD, s->offD[i - 1], s->offD[i]);
        }
        const int nt = (int)((w + kTile - 1) / kTile);
        if (refine > 0)   // keep S_i for the refinement
            EMG_CUDA(cudaMemcpy2DAsync(Scopy, sizeof(T) * sq, Sinv + s->offD[i], sizeof(T) * s->totD, sizeof(T) * w * w,
                                       (size_t)F, cudaMemcpyDeviceToDevice, st));
        // Block Gauss-Jordan over the tile steps with a one-step lookahead: the pivot tile
        // of step k + 1 is updated first and inverted on the side stream while the rest
        // of step k's update and its column panel run on st.  Step k + 1 waits for it.
        T* const P0 = static_cast<T*>(s->pinv);
        auto pset = [&](int k) { return P0 + (int64_t)(k & 1) * F * kTile * kTile; };
        k_gj_diag<R><<<dim3(1, 1, (unsigned)F), kDiagThreads, 0, st>>>(w, 0, Sinv, s->totD, s->offD[i], pset(0),
                                                                  rel_thr, s->perturbed);
        for (int k = 0; k < nt; ++k) {
            if (k > 0) EMG_CUDA(cudaStreamWaitEvent(st, side.diag_done, 0));
            if (nt == 1) break;
            const T* P = pset(k);
            const int la = k + 1 < nt ? k + 1 : -1;
            k_gj_panel<R><<<dim3(nt, 1, (unsigned)F), kThreads, 0, st>>>(0, w, k, Sinv, s->totD, s->offD[i], P, -1);
            if (la >= 0) {
                k_gj_panel<R><<<dim3(1, 1, (unsigned)F), kThreads, 0, st>>>(3, w, k, Sinv, s->totD, s->offD[i], P, la);
                EMG_CUDA(cudaEventRecord(side.tile_ready, st));
                EMG_CUDA(cudaStreamWaitEvent(side.st, side.tile_ready, 0));
                k_gj_diag<R><<<dim3(1, 1, (unsigned)F), kDiagThreads, 0, side.st>>>(w, la, Sinv, s->totD, s->offD[i],
                                                                               pset(la), rel_thr, s->perturbed);
                EMG_CUDA(cudaEventRecord(side.diag_done, side.st));
            }
            if (tc_update)
                rc = emg::tc_gj_update(w, k, la, F, reinterpret_cast<float2*>(Sinv), s->totD, s->offD[i],
                                       s->tc_status, st);
            else
                k_gj_panel<R><<<dim3(nt, nt, (unsigned)F), kThreads, 0, st>>>(2, w, k, Sinv, s->totD, s->offD[i], P,
                                                                               la);
            if (rc) return rc;
            k_gj_panel<R><<<dim3(nt, 1, (unsigned)F), kThreads, 0, st>>>(1, w, k, Sinv, s->totD, s->offD[i], P, -1);
        }
        // X <- X (2I - S X): squares the residual I - S X of the inverse.  S_i's copy
        // is free once 2I - S X is formed and receives the new X.
        if (refine > 0) {
            T* X = Sinv + s->offD[i];
            const dim3 g((unsigned)nt, (unsigned)nt, (unsigned)F);
            k_sq_gemm<R><<<g, kThreads, 0, st>>>(w, Scopy, sq, X, s->totD, Rbuf, sq, (R)-1, (R)2);
            k_dev_partial<R><<<dim3(kNormBlocks, (unsigned)F), kThreads, 0, st>>>(w, Rbuf, sq, npart);
            k_sq_gemm<R><<<g, kThreads, 0, st>>>(w, X, s->totD, Rbuf, sq, Scopy, sq, (R)1, (R)0);
            k_copy_if<R><<<dim3(grid_for(w * w, kThreads, 1024), (unsigned)F), kThreads, 0, st>>>(
                w, Scopy, sq, X, s->totD, npart, s->perturbed + F);
        }
        EMG_CUDA(cudaGetLastError());
    }
    std::vector<int32_t> pc(2 * F);
    int32_t tcs = 0;
    EMG_CUDA(cudaMemcpyAsync(pc.data(), s->perturbed, sizeof(int32_t) * 2 * F, cudaMemcpyDeviceToHost, st));
    if (tc_update) EMG_CUDA(cudaMemcpyAsync(&tcs, s->tc_status, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    EMG_CUDA(cudaStreamSynchronize(st));
    if (tcs) {   // a tensor-core tile gave up waiting: the factors are not usable
        EMG_CUDA(cudaMemset(s->tc_status, 0, sizeof(int32_t)));
        slab_free_factors(s);
        set_error("slab factor: a tensor-core update tile timed out waiting for its MMAs");
        return EMG_ERR_CUDA;
    }
    s->n_perturbed = 0;
    s->n_refine_skipped = 0;
    for (int64_t f = 0; f < F; ++f) {
        s->n_perturbed += pc[f];
        s->n_refine_skipped += pc[F + f];
    }
    return EMG_OK;
}
}  // namespace

extern "C" int emg_slab_factor(emg_slab* s, int precision, int64_t F, const int32_t* amat, int64_t Bm, const double* A,
                               int refine, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(s && amat && A && F > 0 && Bm > 0 && (precision == 1 || precision == 2) && refine >= 0 && refine <= 1,
                  "emg_slab_factor: bad argument");
    for (int64_t f = 0; f < F; ++f) EMG_CHECK_ARG(amat[f] >= 0 && amat[f] < Bm, "emg_slab_factor: amat out of range");
    if (s->n == 0) return EMG_OK;
    const auto* Ad = reinterpret_cast<const double2*>(A);
    return precision == 1 ? slab_factor_t<float>(s, F, amat, Bm, Ad, refine, (cudaStream_t)stream)
                          : slab_factor_t<double>(s, F, amat, Bm, Ad, refine, (cudaStream_t)stream);
}

namespace {
// EMG_ERR_CUDA if a tensor-core tile of the last solve gave up waiting (and reset).
int tc_check(emg_slab* s, cudaStream_t st) {
    if (!s->tc_status || !s->use_tc) return EMG_OK;
    int32_t h = 0;
    EMG_CUDA(cudaMemcpyAsync(&h, s->tc_status, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    EMG_CUDA(cudaStreamSynchronize(st));
    if (h) {
        EMG_CUDA(cudaMemset(s->tc_status, 0, sizeof(int32_t)));
        set_error("slab solve: a tensor-core tile timed out waiting for its MMAs");
        return EMG_ERR_CUDA;
    }
    return EMG_OK;
}

// The slab solve as a GMRES preconditioner: column c uses factor cfac[c].
struct SlabPrecond : emg::Precond {
    emg_slab* s;
    std::vector<int32_t> cfac;
    std::vector<emg::slab::Group> groups;
    int64_t Bc = 0;
    SlabPrecond(emg_slab* s_, int64_t Bc_, const int32_t* cfac_) : s(s_), cfac(cfac_, cfac_ + Bc_), Bc(Bc_) {
        for (int64_t c = 0; c < Bc; ++c) {
            if (!groups.empty() && groups.back().fac == cfac[c] && groups.back().col0 + groups.back().ncol == c)
                groups.back().ncol++;
            else
                groups.push_back({cfac[c], (int32_t)c, 1, 0});
        }
    }
    int prepare(int64_t bc) override {
        using namespace emg;
        const size_t bytes = (s->prec == 1 ? sizeof(float2) : sizeof(double2)) * (size_t)s->n * (size_t)bc;
        if (bytes > s->ws_bytes || bc > s->ws_cols || !s->Y) {
            dfree(s->Y); dfree(s->Z); dfree(s->colfac);
            s->ws_cols = 0;
            s->ws_bytes = 0;
            EMG_CUDA(cudaMalloc(&s->Y, bytes));
            EMG_CUDA(cudaMalloc(&s->Z, bytes));
            int rc = dalloc(&s->colfac, bc, "slab colfac");
            if (rc) return rc;
            s->ws_cols = bc;
            s->ws_bytes = bytes;
        }
        // split-K scratch for the wide-group products (largest need over the slabs)
        int maxcol = 0;
        for (const auto& g : groups) maxcol = std::max(maxcol, (int)g.ncol);
        if (maxcol >= s->wide) {
            const int64_t ct = (maxcol + emg::slab::kTile - 1) / emg::slab::kTile, G = (int64_t)groups.size();
            size_t need = 0;
            int64_t tiles_max = 0;
            const bool narrow = maxcol <= emg::slab::kNarrowN;
            const int64_t tm = narrow ? emg::slab::kNarrowM : emg::slab::kTile;
            const int64_t slot = narrow ? (int64_t)emg::slab::kNarrowM * emg::slab::kNarrowN
                                        : (int64_t)emg::slab::kTile * emg::slab::kTile;
            for (int i = 0; i < s->m; ++i) {
                const int64_t w = s->off[i + 1] - s->off[i];
                const int64_t tiles = (narrow ? 1 : ct) * ((w + tm - 1) / tm) * G;
                const int sp = emg::slab::gemm_splits(tiles, w, s->max_splits);
                tiles_max = std::max(tiles_max, tiles);
                if (sp > 1)
                    need = std::max(need, (size_t)tiles * sp * (size_t)slot *
                                              (s->prec == 1 ? sizeof(float2) : sizeof(double2)));
            }
            if (need > s->kpart_bytes) {
                if (s->kpart) cudaFree(s->kpart);
                s->kpart = nullptr;
                s->kpart_bytes = 0;
                EMG_CUDA(cudaMalloc(&s->kpart, need));
                s->kpart_bytes = need;
            }
            if (tiles_max > s->kcnt_n) {
                dfree(s->kcnt);
                s->kcnt_n = 0;
                int rc = dalloc(&s->kcnt, tiles_max, "slab split-K counters");
                if (rc) return rc;
                EMG_CUDA(cudaMemset(s->kcnt, 0, sizeof(int32_t) * tiles_max));
                s->kcnt_n = tiles_max;
            }
        }
        if (!s->tc_status) {
            int rc = dalloc(&s->tc_status, 1, "slab tensor-core status");
            if (rc) return rc;
            EMG_CUDA(cudaMemset(s->tc_status, 0, sizeof(int32_t)));
        }
        if ((int64_t)groups.size() > s->ngroups_cap) {
            dfree(s->groups);
            int rc = dalloc(&s->groups, (int64_t)groups.size(), "slab groups");
            if (rc) return rc;
            s->ngroups_cap = (int64_t)groups.size();
        }
        EMG_CUDA(cudaMemcpy(s->colfac, cfac.data(), sizeof(int32_t) * bc, cudaMemcpyHostToDevice));
        EMG_CUDA(cudaMemcpy(s->groups, groups.data(), sizeof(emg::slab::Group) * groups.size(), cudaMemcpyHostToDevice));
        return EMG_OK;
    }
    template <typename R, typename TI>
    int run(const TI* in, TI* out, cudaStream_t st) {
        using namespace emg::slab;
        using T = typename C2<R>::T;
        T* Y = static_cast<T*>(s->Y);
        T* Z = static_cast<T*>(s->Z);
        const T* Sinv = static_cast<const T*>(s->Sinv);
        const T* Cv = static_cast<const T*>(s->Cval);
        const T* Uv = static_cast<const T*>(s->Uval);
        const unsigned G = (unsigned)groups.size();
        int maxcol = 0;
        for (const auto& g : groups) maxcol = std::max(maxcol, (int)g.ncol);
        static bool narrow_attr = false;   // per instantiation: the 128 x 16 tiles need 74 KB
        if (!narrow_attr) {
            EMG_CUDA(cudaFuncSetAttribute(k_slab_gemm16<R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)sizeof(NarrowTile<R>)));
            narrow_attr = true;
        }
        // dense slab product: warp-per-row for groups narrower than s->wide, 128 x 16
        // tiles up to 16 columns, 64 x 64 tiles for wider ones
        auto dense = [&](int64_t w, int64_t i, R alpha, int beta) {
            if constexpr (sizeof(R) == 4) {
                if (s->use_tc && maxcol >= s->wide) {
                    emg::tc_slab_product(w, s->off[i], Bc, s->groups, (int)G, maxcol,
                                         reinterpret_cast<const float2*>(Sinv), s->totD, s->offD[i],
                                         reinterpret_cast<const float2*>(Y), (float)alpha, beta,
                                         reinterpret_cast<float2*>(Z), s->tc_status, st);
                    return;
                }
            }
            if (maxcol >= s->wide && maxcol <= kNarrowN) {
                const int64_t rt = (w + kNarrowM - 1) / kNarrowM;
                const int sp = gemm_splits(rt * G, w, s->max_splits);
                k_slab_gemm16<R><<<dim3(1u, (unsigned)(rt * sp), G), kThreads, sizeof(NarrowTile<R>), st>>>(
                    w, s->off[i], Bc, s->groups, Sinv, s->totD, s->offD[i], Y, alpha, beta, Z, sp,
                    static_cast<T*>(s->kpart), s->kcnt);
            } else if (maxcol >= s->wide) {
                const int64_t ct = (maxcol + kTile - 1) / kTile, rt = (w + kTile - 1) / kTile;
                const int sp = gemm_splits(ct * rt * G, w, s->max_splits);
                k_slab_gemm<R><<<dim3((unsigned)ct, (unsigned)(rt * sp), G), kThreads, 0, st>>>(
                    w, s->off[i], Bc, s->groups, Sinv, s->totD, s->offD[i], Y, alpha, beta, Z, sp,
                    static_cast<T*>(s->kpart), s->kcnt);
            } else
                k_rowmv<R><<<dim3((unsigned)((w * 32 + kThreads - 1) / kThreads), G), kThreads, 0, st>>>(
                    w, s->off[i], Bc, s->groups, Sinv, s->totD, s->offD[i], Y, alpha, beta, Z);
        };
        k_gather<R, TI><<<grid_for(s->n * Bc, 256), 256, 0, st>>>(s->n, Bc, s->perm, in, Y);
        for (int i = 0; i < s->m; ++i) {
            const int64_t w = s->off[i + 1] - s->off[i];
            if (i > 0)
                k_couple<R><<<grid_for(w * Bc, 256), 256, 0, st>>>(0, w, s->off[i], s->off[i - 1], Bc, s->colfac, s->cptr,
                                                                   s->cidx, Cv, s->nC, Z, Y);
            dense(w, i, (R)1, 0);
        }
        for (int i = s->m - 2; i >= 0; --i) {
            const int64_t w = s->off[i + 1] - s->off[i];
            k_couple<R><<<grid_for(w * Bc, 256), 256, 0, st>>>(1, w, s->off[i], s->off[i + 1], Bc, s->colfac, s->uptr,
                                                               s->uidx, Uv, s->nU, Z, Y);
            dense(w, i, (R)-1, 1);
        }
        k_scatter<R, TI><<<grid_for(s->n * Bc, 256), 256, 0, st>>>(s->n, Bc, s->perm, Z, out);
        EMG_CUDA(cudaGetLastError());
        return EMG_OK;
    }
    int apply(const double2* in, double2* out, cudaStream_t st) override {
        return s->prec == 1 ? run<float, double2>(in, out, st) : run<double, double2>(in, out, st);
    }
};

// The same slab solve on FP32 vectors (FP32 factors only), for the inner FGMRES of
// the mixed-precision refinement.
struct SlabPrecond32 : emg::Precond32 {
    SlabPrecond base;
    SlabPrecond32(emg_slab* s_, int64_t Bc_, const int32_t* cfac_) : base(s_, Bc_, cfac_) {}
    int prepare(int64_t bc) override { return base.prepare(bc); }
    int apply(const float2* in, float2* out, cudaStream_t st) override { return base.run<float, float2>(in, out, st); }
};
}  // namespace

extern "C" int emg_slab_apply(emg_slab* s, int64_t Bc, const int32_t* cfac, const double* X_in, double* X_out,
                              void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(s && cfac && X_in && X_out && Bc > 0 && X_in != X_out, "emg_slab_apply: bad argument");
    EMG_CHECK_ARG(s->F > 0, "emg_slab_apply: no factorization");
    for (int64_t c = 0; c < Bc; ++c) EMG_CHECK_ARG(cfac[c] >= 0 && cfac[c] < s->F, "emg_slab_apply: cfac out of range");
    if (s->n == 0) return EMG_OK;
    SlabPrecond M(s, Bc, cfac);
    int rc = M.prepare(Bc);
    if (rc) return rc;
    rc = M.apply(reinterpret_cast<const double2*>(X_in), reinterpret_cast<double2*>(X_out), (cudaStream_t)stream);
    if (rc) return rc;
    return tc_check(s, (cudaStream_t)stream);
}

extern "C" int emg_gmres_slab(const emg_rplan* pc, emg_slab* s, int64_t Bc, const int32_t* cmat, int64_t Bm,
                              const double* A, const int32_t* cfac, const double* rhs, double* x, int restart,
                              int max_iter, double tol, int32_t* iters_out, double* resid_out, void* stream) {
    using namespace emg;
    emg_rplan* p = const_cast<emg_rplan*>(pc);
    EMG_CHECK_ARG(p && s && s->rp == p && cmat && A && cfac && rhs && x && iters_out && resid_out && Bc > 0 && Bm > 0,
                  "emg_gmres_slab: bad argument");
    EMG_CHECK_ARG(restart >= 1 && restart <= 256 && max_iter >= 1 && tol > 0, "emg_gmres_slab: restart must be in [1, 256]");
    EMG_CHECK_ARG(s->F > 0, "emg_gmres_slab: no factorization");
    for (int64_t c = 0; c < Bc; ++c) EMG_CHECK_ARG(cfac[c] >= 0 && cfac[c] < s->F, "emg_gmres_slab: cfac out of range");
    SlabPrecond M(s, Bc, cfac);
    MatArg Am;
    Am.A = reinterpret_cast<const double2*>(A);
    Am.Bm = Bm;
    Am.cmat = cmat;
    const int rc = gmres_run(p, Bc, Am, reinterpret_cast<const double2*>(rhs), reinterpret_cast<double2*>(x), restart,
                             max_iter, tol, iters_out, resid_out, (cudaStream_t)stream, M, true);
    return rc ? rc : tc_check(s, (cudaStream_t)stream);
}

extern "C" int emg_slab_set_factor_tensor_cores(emg_slab* s, int on) {
    EMG_CHECK_ARG(s, "emg_slab_set_factor_tensor_cores: NULL argument");
    s->tc_factor = on ? 1 : 0;
    return EMG_OK;
}

extern "C" int emg_slab_set_tensor_cores(emg_slab* s, int on) {
    EMG_CHECK_ARG(s, "emg_slab_set_tensor_cores: NULL argument");
    s->use_tc = on ? 1 : 0;
    return EMG_OK;
}

extern "C" int emg_slab_set_wide_group(emg_slab* s, int min_columns) {
    EMG_CHECK_ARG(s && min_columns >= 1, "emg_slab_set_wide_group: bad argument");
    s->wide = min_columns;
    return EMG_OK;
}

extern "C" int emg_slab_set_max_splits(emg_slab* s, int max_splits) {
    EMG_CHECK_ARG(s && max_splits >= 1 && max_splits <= 16, "emg_slab_set_max_splits: bad argument");
    s->max_splits = max_splits;
    return EMG_OK;
}

extern "C" int emg_gmres_slab_family(const emg_rplan* pc, emg_slab* s, int64_t Bc, int nfam, const double* fam,
                                     const double* coef, const int32_t* cfac, const double* rhs, double* x,
                                     int restart, int max_iter, double tol, int32_t* iters_out, double* resid_out,
                                     void* stream) {
    using namespace emg;
    emg_rplan* p = const_cast<emg_rplan*>(pc);
    EMG_CHECK_ARG(p && s && s->rp == p && fam && coef && cfac && rhs && x && iters_out && resid_out && Bc > 0 &&
                      nfam >= 1 && nfam <= kMaxFamily,
                  "emg_gmres_slab_family: bad argument");
    EMG_CHECK_ARG(restart >= 1 && restart <= 256 && max_iter >= 1 && tol > 0,
                  "emg_gmres_slab_family: restart must be in [1, 256]");
    EMG_CHECK_ARG(s->F > 0, "emg_gmres_slab_family: no factorization");
    for (int64_t c = 0; c < Bc; ++c)
        EMG_CHECK_ARG(cfac[c] >= 0 && cfac[c] < s->F, "emg_gmres_slab_family: cfac out of range");
    SlabPrecond M(s, Bc, cfac);
    MatArg Am;
    Am.nfam = nfam;
    Am.fam = reinterpret_cast<const double2*>(fam);
    Am.coef = reinterpret_cast<const double2*>(coef);
    return gmres_run(p, Bc, Am, reinterpret_cast<const double2*>(rhs), reinterpret_cast<double2*>(x), restart, max_iter,
                     tol, iters_out, resid_out, (cudaStream_t)stream, M, true);
}

extern "C" int emg_gmres_slab_mixed(const emg_rplan* pc, emg_slab* s, int64_t Bc, const int32_t* cmat, int64_t Bm,
                                    const double* A, const int32_t* cfac, const double* rhs, double* x, int restart,
                                    int max_iter, double tol, double inner_tol, int32_t* iters_out, double* resid_out,
                                    int32_t* steps_out, void* stream) {
    using namespace emg;
    emg_rplan* p = const_cast<emg_rplan*>(pc);
    EMG_CHECK_ARG(p && s && s->rp == p && cmat && A && cfac && rhs && x && iters_out && resid_out && Bc > 0 && Bm > 0,
                  "emg_gmres_slab_mixed: bad argument");
    EMG_CHECK_ARG(restart >= 1 && restart <= 256 && max_iter >= 1 && tol > 0 && inner_tol > 0 && inner_tol < 1,
                  "emg_gmres_slab_mixed: restart must be in [1, 256], tolerances in (0, 1)");
    EMG_CHECK_ARG(s->F > 0 && s->prec == 1, "emg_gmres_slab_mixed: needs FP32 slab factors");
    for (int64_t c = 0; c < Bc; ++c)
        EMG_CHECK_ARG(cfac[c] >= 0 && cfac[c] < s->F, "emg_gmres_slab_mixed: cfac out of range");
    if (p->ns == 0) return EMG_OK;
    // FP32 copy of the stored matrices for the inner products
    float2* A32 = nullptr;
    int rc = dalloc(&A32, p->nnz * Bm, "mixed FP32 matrices");
    if (rc) return rc;
    struct Free { float2* a; ~Free() { if (a) cudaFree(a); } } fr{A32};
    cudaStream_t st = (cudaStream_t)stream;
    slab::k_narrow<<<grid_for(p->nnz * Bm, 256), 256, 0, st>>>(p->nnz * Bm, reinterpret_cast<const double2*>(A), A32);
    EMG_CUDA(cudaGetLastError());
    SlabPrecond32 M(s, Bc, cfac);
    MatArg Am;
    Am.A = reinterpret_cast<const double2*>(A);
    Am.Bm = Bm;
    Am.cmat = cmat;
    rc = ir_run(p, Bc, Am, A32, reinterpret_cast<const double2*>(rhs), reinterpret_cast<double2*>(x), restart, max_iter,
                tol, inner_tol, iters_out, resid_out, steps_out, st, M);
    EMG_CUDA(cudaStreamSynchronize(st));   // A32 is freed on return
    return rc;
}
