// Surface (Robin, third-kind) boundary terms and frequency-matrix helpers.
//
//   ned2_tri_stiff_force  fem/mth/tri.py:575-695   waveport block + forcing vector
//   ned2_tri_stiff        fem/mth/tri.py:697-797   absorbing-boundary block
//   assemble_freq_matrix  fem/physics/edm/assembler.py:312-388  (K = E - k0^2 B + sum B_p)
//
// Port triangles are few (a port face, not the volume), so each triangle is one
// thread in FP64.  Their 8x8 blocks land on entries of the volume CSR pattern;
// the contributions are summed with a plan-time sorted segment list so every
// frequency sums in the same order (deterministic), then added to K.
#include "emg_common.cuh"

namespace emg {
namespace surf {

// simplex-area monomial integrals 2*prod(k!)/(sum k + 2)!, letters 0..3 (0 = absent),
// fem/mth/optimized.py:262-271
__constant__ double c_acoef[256];

struct cplx {
    double re, im;
};
__device__ __forceinline__ cplx cmul(cplx a, cplx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ cplx cscale(cplx a, double s) { return {a.re * s, a.im * s}; }
__device__ __forceinline__ cplx cadd(cplx a, cplx b) { return {a.re + b.re, a.im + b.im}; }

__device__ __forceinline__ double ac(int a, int b, int c, int d, double area) {
    return c_acoef[((a * 4 + b) * 4 + c) * 4 + d] * area;
}
__device__ __forceinline__ double dot2(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1]; }

// The 8x8 Robin block shared by both reference kernels (real geometric part);
// multiplied by ``coef`` (complex) either per term (tri_stiff) or at the end
// (tri_stiff_force) by the caller.
__device__ void robin_block(const double GL[3][2], const double Le[3], double Lt1, double Lt2, double Area,
                            double Bm[64]) {
    const int lem0[3] = {0, 1, 0}, lem1[3] = {1, 2, 2};
    for (int i = 0; i < 64; ++i) Bm[i] = 0.0;
    const int tA = 1, tB = 2, tC = 3;
    const double *GtA = GL[0], *GtB = GL[1], *GtC = GL[2];
    for (int ei = 0; ei < 3; ++ei) {
        const int i1 = lem0[ei], i2 = lem1[ei];
        const double Li = Le[ei];
        const int A = i1 + 1, B = i2 + 1;
        const double *GA = GL[i1], *GB = GL[i2];
        for (int ej = 0; ej < 3; ++ej) {
            const int j1 = lem0[ej], j2 = lem1[ej];
            const double Lj = Le[ej];
            const int C = j1 + 1, D = j2 + 1;
            const double *GC = GL[j1], *GD = GL[j2];
            const double aC = dot2(GA, GC), aD = dot2(GA, GD), bC = dot2(GB, GC), bD = dot2(GB, GD);
            const double L2 = Li * Lj;
            Bm[ei * 8 + ej] += L2 * (ac(A, B, C, D, Area) * aC - ac(A, B, C, C, Area) * aD - ac(A, A, C, D, Area) * bC + ac(A, A, C, C, Area) * bD);
            Bm[ei * 8 + ej + 4] += L2 * (ac(A, B, D, D, Area) * aC - ac(A, B, C, D, Area) * aD - ac(A, A, D, D, Area) * bC + ac(A, A, C, D, Area) * bD);
            Bm[(ei + 4) * 8 + ej] += L2 * (ac(B, B, C, D, Area) * aC - ac(B, B, C, C, Area) * aD - ac(A, B, C, D, Area) * bC + ac(A, B, C, C, Area) * bD);
            Bm[(ei + 4) * 8 + ej + 4] += L2 * (ac(B, B, D, D, Area) * aC - ac(B, B, C, D, Area) * aD - ac(A, B, D, D, Area) * bC + ac(A, B, C, D, Area) * bD);
        }
        const double aC = dot2(GA, GtC), aA = dot2(GA, GtA), bC = dot2(GB, GtC), bA = dot2(GB, GtA);
        const double aB = dot2(GA, GtB), bB = dot2(GB, GtB);
        Bm[ei * 8 + 3] += Li * Lt1 * (ac(A, B, tA, tB, Area) * aC - ac(A, B, tB, tC, Area) * aA - ac(A, A, tA, tB, Area) * bC + ac(A, A, tB, tC, Area) * bA);
        Bm[ei * 8 + 7] += Li * Lt2 * (ac(A, B, tB, tC, Area) * aA - ac(A, B, tC, tA, Area) * aB - ac(A, A, tB, tC, Area) * bA + ac(A, A, tC, tA, Area) * bB);
        Bm[3 * 8 + ei] += Lt1 * Li * (ac(tA, tB, A, B, Area) * aC - ac(tA, tB, A, A, Area) * bC - ac(tB, tC, A, B, Area) * aA + ac(tB, tC, A, A, Area) * bA);
        Bm[7 * 8 + ei] += Lt2 * Li * (ac(tB, tC, A, B, Area) * aA - ac(tB, tC, A, A, Area) * bA - ac(tC, tA, A, B, Area) * aB + ac(tC, tA, A, A, Area) * bB);
        Bm[(ei + 4) * 8 + 3] += Li * Lt1 * (ac(B, B, tA, tB, Area) * aC - ac(B, B, tB, tC, Area) * aA - ac(A, B, tA, tB, Area) * bC + ac(A, B, tB, tC, Area) * bA);
        Bm[(ei + 4) * 8 + 7] += Li * Lt2 * (ac(B, B, tB, tC, Area) * aA - ac(B, B, tC, tA, Area) * aB - ac(A, B, tB, tC, Area) * bA + ac(A, B, tC, tA, Area) * bB);
        Bm[3 * 8 + ei + 4] += Lt1 * Li * (ac(tA, tB, B, B, Area) * aC - ac(tA, tB, A, B, Area) * bC - ac(tB, tC, B, B, Area) * aA + ac(tB, tC, A, B, Area) * bA);
        Bm[7 * 8 + ei + 4] += Lt2 * Li * (ac(tB, tC, B, B, Area) * aA - ac(tB, tC, A, B, Area) * bA - ac(tC, tA, B, B, Area) * aB + ac(tC, tA, A, B, Area) * bB);
    }
    const double CC = dot2(GtC, GtC), AC = dot2(GtA, GtC), AA = dot2(GtA, GtA), BC = dot2(GtB, GtC);
    const double AB = dot2(GtA, GtB), BB = dot2(GtB, GtB);
    Bm[3 * 8 + 3] += Lt1 * Lt1 * (ac(tA, tB, tA, tB, Area) * CC - ac(tA, tB, tB, tC, Area) * AC - ac(tB, tC, tA, tB, Area) * AC + ac(tB, tC, tB, tC, Area) * AA);
    Bm[3 * 8 + 7] += Lt1 * Lt2 * (ac(tA, tB, tB, tC, Area) * AC - ac(tA, tB, tC, tA, Area) * BC - ac(tB, tC, tB, tC, Area) * AA + ac(tB, tC, tC, tA, Area) * AB);
    Bm[7 * 8 + 3] += Lt2 * Lt1 * (ac(tB, tC, tA, tB, Area) * AC - ac(tB, tC, tB, tC, Area) * AA - ac(tC, tA, tA, tB, Area) * BC + ac(tC, tA, tB, tC, Area) * AB);
    Bm[7 * 8 + 7] += Lt2 * Lt2 * (ac(tB, tC, tB, tC, Area) * AA - ac(tB, tC, tC, tA, Area) * AB - ac(tC, tA, tB, tC, Area) * AB + ac(tC, tA, tC, tA, Area) * BB);
}

// Thread per waveport triangle: 8x8 block (gamma applied) and forcing vector.
// lcs (2, 3, n): local x / y of the triangle's vertices; uinc (3, npts, n) complex;
// dpts (4, npts): weight, three barycentrics.
__global__ void k_tri_force(int64_t n, const double* __restrict__ lcs, const double2* __restrict__ uinc,
                            const double* __restrict__ dpts, int npts, double g_re, double g_im, double2* __restrict__ Bout,
                            double2* __restrict__ bout) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const double x1 = lcs[0 * 3 * n + 0 * n + t], x2 = lcs[0 * 3 * n + 1 * n + t], x3 = lcs[0 * 3 * n + 2 * n + t];
        const double y1 = lcs[1 * 3 * n + 0 * n + t], y2 = lcs[1 * 3 * n + 1 * n + t], y3 = lcs[1 * 3 * n + 2 * n + t];
        const double As[3] = {x2 * y3 - y2 * x3, x3 * y1 - y3 * x1, x1 * y2 - y1 * x2};
        const double Bs[3] = {y2 - y3, y3 - y1, y1 - y2};
        const double Cs[3] = {x3 - x2, x1 - x3, x2 - x1};
        const double xs[3] = {x1, x2, x3}, ys[3] = {y1, y2, y3};
        double Ds[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) Ds[i][j] = sqrt((xs[i] - xs[j]) * (xs[i] - xs[j]) + (ys[i] - ys[j]) * (ys[i] - ys[j]));
        const double GL[3][2] = {{Bs[0], Cs[0]}, {Bs[1], Cs[1]}, {Bs[2], Cs[2]}};
        const double det = (x1 - x3) * (y2 - y1) - (x1 - x2) * (y3 - y1);
        const double Area = 0.5 * fabs(det);
        const double signA = det > 0 ? -1.0 : (det < 0 ? 1.0 : 0.0);
        const double Lt1 = Ds[2][0], Lt2 = Ds[1][0];
        const double Le[3] = {Ds[0][1], Ds[1][2], Ds[0][2]};
        double Bm[64];
        robin_block(GL, Le, Lt1, Lt2, Area, Bm);
        const cplx coef = cscale(cplx{g_re, g_im}, 1.0 / ((2 * Area) * (2 * Area)));
        for (int i = 0; i < 64; ++i) {
            const cplx v = cscale(coef, Bm[i]);
            Bout[t * 64 + i] = make_double2(v.re, v.im);
        }
        const double A2 = Area * Area, A3 = Area * Area * Area;
        const int lem0[3] = {0, 1, 0}, lem1[3] = {1, 2, 2};
        cplx bv[8];
        for (int i = 0; i < 8; ++i) bv[i] = {0.0, 0.0};
        for (int ei = 0; ei < 3; ++ei) {
            const int i1 = lem0[ei], i2 = lem1[ei];
            const double Li = Ds[i1][i2];
            const double a1 = As[i1], a2 = As[i2], b1 = Bs[i1], b2 = Bs[i2], c1 = Cs[i1], c2 = Cs[i2];
            cplx s1 = {0, 0}, s2 = {0, 0};
            for (int k = 0; k < npts; ++k) {
                const double x = x1 * dpts[npts + k] + x2 * dpts[2 * npts + k] + x3 * dpts[3 * npts + k];
                const double y = y1 * dpts[npts + k] + y2 * dpts[2 * npts + k] + y3 * dpts[3 * npts + k];
                const double l1 = a1 + b1 * x + c1 * y, l2 = a2 + b2 * x + c2 * y;
                const double wx = b1 * l2 / (4 * A2) - b2 * l1 / (4 * A2);
                const double wy = c1 * l2 / (4 * A2) - c2 * l1 / (4 * A2);
                const double e1x = Li * wx * l1 / (2 * Area), e1y = Li * wy * l1 / (2 * Area);
                const double e2x = Li * wx * l2 / (2 * Area), e2y = Li * wy * l2 / (2 * Area);
                const double2 ux = uinc[(0 * npts + k) * n + t], uy = uinc[(1 * npts + k) * n + t];
                const double W = dpts[k];
                s1 = cadd(s1, cscale(cadd(cscale({ux.x, ux.y}, e1x), cscale({uy.x, uy.y}, e1y)), W));
                s2 = cadd(s2, cscale(cadd(cscale({ux.x, ux.y}, e2x), cscale({uy.x, uy.y}, e2y)), W));
            }
            bv[ei] = cadd(bv[ei], cscale(s1, signA * Area));
            bv[ei + 4] = cadd(bv[ei + 4], cscale(s2, signA * Area));
        }
        {
            cplx s3 = {0, 0}, s7 = {0, 0};
            for (int k = 0; k < npts; ++k) {
                const double x = x1 * dpts[npts + k] + x2 * dpts[2 * npts + k] + x3 * dpts[3 * npts + k];
                const double y = y1 * dpts[npts + k] + y2 * dpts[2 * npts + k] + y3 * dpts[3 * npts + k];
                const double l1 = As[0] + Bs[0] * x + Cs[0] * y, l2 = As[1] + Bs[1] * x + Cs[1] * y;
                const double l3 = As[2] + Bs[2] * x + Cs[2] * y;
                const double f1x = Lt1 * (-Bs[0] * l2 * l3 / (8 * A3) + Bs[2] * l1 * l2 / (8 * A3));
                const double f1y = Lt1 * (-Cs[0] * l2 * l3 / (8 * A3) + Cs[2] * l1 * l2 / (8 * A3));
                const double f2x = Lt2 * (Bs[0] * l2 * l3 / (8 * A3) - Bs[1] * l1 * l3 / (8 * A3));
                const double f2y = Lt2 * (Cs[0] * l2 * l3 / (8 * A3) - Cs[1] * l1 * l3 / (8 * A3));
                const double2 ux = uinc[(0 * npts + k) * n + t], uy = uinc[(1 * npts + k) * n + t];
                const double W = dpts[k];
                s3 = cadd(s3, cscale(cadd(cscale({ux.x, ux.y}, f1x), cscale({uy.x, uy.y}, f1y)), W));
                s7 = cadd(s7, cscale(cadd(cscale({ux.x, ux.y}, f2x), cscale({uy.x, uy.y}, f2y)), W));
            }
            bv[3] = cadd(bv[3], cscale(s3, signA * Area));
            bv[7] = cadd(bv[7], cscale(s7, signA * Area));
        }
        for (int i = 0; i < 8; ++i) bout[t * 8 + i] = make_double2(bv[i].re, bv[i].im);
    }
}

// Thread per absorbing-boundary triangle (ned2_tri_stiff): xyz (3, 3, n) coordinate
// rows by vertex; edge_len (3, n).
__global__ void k_tri_abc(int64_t n, const double* __restrict__ xyz, const double* __restrict__ edge_len, double g_re,
                          double g_im, double2* __restrict__ Bout) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        double v[3][3];   // v[coord][vertex]
        for (int c = 0; c < 3; ++c)
            for (int k = 0; k < 3; ++k) v[c][k] = xyz[(c * 3 + k) * n + t];
        double ax1[3] = {v[0][1] - v[0][0], v[1][1] - v[1][0], v[2][1] - v[2][0]};
        double ax2[3] = {v[0][2] - v[0][0], v[1][2] - v[1][0], v[2][2] - v[2][0]};
        const double n1 = sqrt(ax1[0] * ax1[0] + ax1[1] * ax1[1] + ax1[2] * ax1[2]);
        const double n2 = sqrt(ax2[0] * ax2[0] + ax2[1] * ax2[1] + ax2[2] * ax2[2]);
        for (int i = 0; i < 3; ++i) { ax1[i] /= n1; ax2[i] /= n2; }
        const double axn[3] = {ax1[1] * ax2[2] - ax1[2] * ax2[1], ax1[2] * ax2[0] - ax1[0] * ax2[2],
                               ax1[0] * ax2[1] - ax1[1] * ax2[0]};
        const double t2[3] = {axn[1] * ax1[2] - axn[2] * ax1[1], axn[2] * ax1[0] - axn[0] * ax1[2],
                              axn[0] * ax1[1] - axn[1] * ax1[0]};
        // local frame columns (ax1, -(axn x ax1), axn), inverted (the reference uses pinv)
        const double M[9] = {ax1[0], -t2[0], axn[0], ax1[1], -t2[1], axn[1], ax1[2], -t2[2], axn[2]};
        const double det = M[0] * (M[4] * M[8] - M[5] * M[7]) - M[1] * (M[3] * M[8] - M[5] * M[6]) + M[2] * (M[3] * M[7] - M[4] * M[6]);
        const double Mi[6] = {(M[4] * M[8] - M[5] * M[7]) / det, (M[2] * M[7] - M[1] * M[8]) / det,
                              (M[1] * M[5] - M[2] * M[4]) / det, (M[5] * M[6] - M[3] * M[8]) / det,
                              (M[0] * M[8] - M[2] * M[6]) / det, (M[2] * M[3] - M[0] * M[5]) / det};
        double xs[3], ys[3];
        for (int k = 0; k < 3; ++k) {
            xs[k] = Mi[0] * v[0][k] + Mi[1] * v[1][k] + Mi[2] * v[2][k];
            ys[k] = Mi[3] * v[0][k] + Mi[4] * v[1][k] + Mi[5] * v[2][k];
        }
        const double GL[3][2] = {{ys[1] - ys[2], xs[2] - xs[1]}, {ys[2] - ys[0], xs[0] - xs[2]}, {ys[0] - ys[1], xs[1] - xs[0]}};
        const double Area = 0.5 * fabs((xs[0] - xs[2]) * (ys[1] - ys[0]) - (xs[0] - xs[1]) * (ys[2] - ys[0]));
        const double Lt1 = sqrt((xs[2] - xs[0]) * (xs[2] - xs[0]) + (ys[2] - ys[0]) * (ys[2] - ys[0]));
        const double Lt2 = sqrt((xs[1] - xs[0]) * (xs[1] - xs[0]) + (ys[1] - ys[0]) * (ys[1] - ys[0]));
        const double Le[3] = {edge_len[t], edge_len[n + t], edge_len[2 * n + t]};
        double Bm[64];
        robin_block(GL, Le, Lt1, Lt2, Area, Bm);
        const cplx coef = cscale(cplx{g_re, g_im}, 1.0 / ((2 * Area) * (2 * Area)));
        for (int i = 0; i < 64; ++i) {
            const cplx vv = cscale(coef, Bm[i]);
            Bout[t * 64 + i] = make_double2(vv.re, vv.im);
        }
    }
}

// pos[i] = index of cols[i] in CSR row rows[i] (binary search), -1 if absent.
__global__ void k_positions(int64_t n, const int32_t* __restrict__ rows, const int32_t* __restrict__ cols,
                            const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices, int64_t* pos) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t lo = indptr[rows[i]], hi = indptr[rows[i] + 1] - 1;
        const int32_t c = cols[i];
        int64_t res = -1;
        while (lo <= hi) {
            const int64_t mid = (lo + hi) >> 1;
            const int32_t v = indices[mid];
            if (v == c) { res = mid; break; }
            if (v < c) lo = mid + 1; else hi = mid - 1;
        }
        pos[i] = res;
    }
}

// out[dst[s]] += alpha * sum_{k in [seg[s], seg[s+1])} src[perm[k]]   (fixed order)
__global__ void k_segment_add(int64_t n_seg, const int64_t* __restrict__ seg, const int64_t* __restrict__ perm,
                              const int64_t* __restrict__ dst, const double2* __restrict__ src, double a_re, double a_im,
                              double2* __restrict__ out) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n_seg; s += (int64_t)gridDim.x * blockDim.x) {
        double re = 0.0, im = 0.0;
        for (int64_t k = seg[s]; k < seg[s + 1]; ++k) {
            const double2 v = src[perm[k]];
            re += v.x;
            im += v.y;
        }
        double2 o = out[dst[s]];
        o.x += a_re * re - a_im * im;
        o.y += a_re * im + a_im * re;
        out[dst[s]] = o;
    }
}

// K = E - k0sq * B on the shared pattern.
__global__ void k_combine(int64_t nnz, const double2* __restrict__ E, const double2* __restrict__ B, double k0sq,
                          double2* __restrict__ K) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 e = E[i], b = B[i];
        K[i] = make_double2(e.x - b.x * k0sq, e.y - b.y * k0sq);
    }
}

}  // namespace surf

namespace {
bool g_acoef_ready[64] = {false};
int upload_acoef() {
    int dev = 0;
    EMG_CUDA(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64 && g_acoef_ready[dev]) return EMG_OK;
    static const double fact[10] = {1, 1, 2, 6, 24, 120, 720, 5040, 40320, 362880};
    double h[256];
    for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b)
            for (int c = 0; c < 4; ++c)
                for (int d = 0; d < 4; ++d) {
                    int k[4] = {0, 0, 0, 0};
                    k[a]++; k[b]++; k[c]++; k[d]++;
                    h[((a * 4 + b) * 4 + c) * 4 + d] = 2 * fact[k[1]] * fact[k[2]] * fact[k[3]] / fact[k[1] + k[2] + k[3] + 2];
                }
    EMG_CUDA(cudaMemcpyToSymbol(surf::c_acoef, h, sizeof(h)));
    if (dev >= 0 && dev < 64) g_acoef_ready[dev] = true;
    return EMG_OK;
}
}  // namespace
}  // namespace emg

extern "C" int emg_tri_robin_force(int64_t n_tris, const double* lcs_xy, const double* uinc, const double* dpts,
                                   int npts, double gamma_re, double gamma_im, double* B_out, double* b_out,
                                   void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(n_tris >= 0 && npts > 0, "emg_tri_robin_force: bad size");
    if (n_tris == 0) return EMG_OK;
    EMG_CHECK_ARG(lcs_xy && uinc && dpts && B_out && b_out, "emg_tri_robin_force: NULL array");
    int rc = upload_acoef();
    if (rc) return rc;
    surf::k_tri_force<<<grid_for(n_tris, 128), 128, 0, (cudaStream_t)stream>>>(
        n_tris, lcs_xy, reinterpret_cast<const double2*>(uinc), dpts, npts, gamma_re, gamma_im,
        reinterpret_cast<double2*>(B_out), reinterpret_cast<double2*>(b_out));
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}

extern "C" int emg_tri_robin_abc(int64_t n_tris, const double* xyz, const double* edge_lengths, double gamma_re,
                                 double gamma_im, double* B_out, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(n_tris >= 0, "emg_tri_robin_abc: bad size");
    if (n_tris == 0) return EMG_OK;
    EMG_CHECK_ARG(xyz && edge_lengths && B_out, "emg_tri_robin_abc: NULL array");
    int rc = upload_acoef();
    if (rc) return rc;
    surf::k_tri_abc<<<grid_for(n_tris, 128), 128, 0, (cudaStream_t)stream>>>(n_tris, xyz, edge_lengths, gamma_re,
                                                                               gamma_im, reinterpret_cast<double2*>(B_out));
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}

extern "C" int emg_csr_positions(int64_t n, const int32_t* rows, const int32_t* cols, const int64_t* indptr,
                                 const int32_t* indices, int64_t* pos, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(n >= 0, "emg_csr_positions: bad size");
    if (n == 0) return EMG_OK;
    EMG_CHECK_ARG(rows && cols && indptr && indices && pos, "emg_csr_positions: NULL array");
    surf::k_positions<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, rows, cols, indptr, indices, pos);
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}

extern "C" int emg_segment_add(int64_t n_seg, const int64_t* seg_ptr, const int64_t* perm, const int64_t* dst,
                               const double* src, double alpha_re, double alpha_im, double* out, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(n_seg >= 0, "emg_segment_add: bad size");
    if (n_seg == 0) return EMG_OK;
    EMG_CHECK_ARG(seg_ptr && perm && dst && src && out, "emg_segment_add: NULL array");
    surf::k_segment_add<<<grid_for(n_seg, 256), 256, 0, (cudaStream_t)stream>>>(
        n_seg, seg_ptr, perm, dst, reinterpret_cast<const double2*>(src), alpha_re, alpha_im,
        reinterpret_cast<double2*>(out));
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}

extern "C" int emg_combine(int64_t nnz, const double* E, const double* B, double k0sq, double* K, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(nnz >= 0, "emg_combine: bad size");
    if (nnz == 0) return EMG_OK;
    EMG_CHECK_ARG(E && B && K, "emg_combine: NULL array");
    surf::k_combine<<<grid_for(nnz, 256), 256, 0, (cudaStream_t)stream>>>(
        nnz, reinterpret_cast<const double2*>(E), reinterpret_cast<const double2*>(B), k0sq,
        reinterpret_cast<double2*>(K));
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}
