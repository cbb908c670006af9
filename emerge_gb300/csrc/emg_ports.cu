// Element matrices of the 2-D waveguide-port eigenproblem on the GPU: the
// counterpart of generalized_matrix_GQ (fem/physics/edm/nedeleclegrange2.py:224-382),
// which EMerge's modal port analysis evaluates per port-face triangle in a Numba
// loop (_matrix_builder, :385-417).
//
// One block per triangle.  Thread 0 forms the barycentric coefficients
// l_i = a_i + b_i x + c_i y (over 2 area, sign-corrected as tri_coefficients,
// :192-214), the DOF length scales and the materials; threads 0-5 then evaluate
// every basis function at one of the module's six quadrature points into shared
// memory; finally thread (i, j) sums entry (i, j) of A and B over the points.
//
// Basis (edge (p, q) from the local edge map, face = vertices 0, 1, 2):
//   N1 = (grad l_p l_q - grad l_q l_p) l_p,  N2 = (...) l_q,
//   curl N1 = 3 l_p (b_q c_p - b_p c_q),     curl N2 = 3 l_q (b_q c_p - b_p c_q),
//   F1 = -(grad l_0 l_2 - grad l_2 l_0) l_1, F2 = (grad l_0 l_1 - grad l_1 l_0) l_2,
//   vertex L_i = 2 l_i^2 - l_i, edge L = 4 l_p l_q.
// DOFs 0-2 N1 of the edges, 3 F1, 4-6 N2, 7 F2 (transverse); 8-10 vertex L,
// 11-13 edge L (longitudinal).
//   A[:8, :8] = curl.Ms_zz.curl - k0^2 N.Mm_t.N;  B = [[N.Ms_t.N, (grad L.Ms_t.N)^T],
//   [grad L.Ms_t.N, grad L.Ms_t.grad L - k0^2 L.Mm_zz.L]], times the DOF lengths
//   (edges: their length; F1: |v0 v2|; F2: |v0 v1|) and the area.
// As in the reference, the face-row / edge-column transverse entries are the
// mirror of the edge-row / face-column ones, and the face-face entries of the
// transverse B block are zero; with face_block = 1 those four entries are
// integrated like the others instead.  The zero block is an error of the
// reference's formulation: on a WR-90 port it moves the TE10 propagation constant
// 4.9 % above the analytic value at any mesh size (165.9 against 158.24 rad/m at
// 10 GHz), where the integrated block gives it to 2e-6 at h = 3 mm.
#include "emg_common.cuh"

namespace emg {
namespace ports {

// 6-point rule of nedeleclegrange2.py:218-221: weight, then barycentrics of vertices 0, 1, 2
__constant__ double c_rule[4][6] = {
    {0.22338159, 0.22338159, 0.22338159, 0.10995174, 0.10995174, 0.10995174},
    {0.10810302, 0.44594849, 0.44594849, 0.81684757, 0.09157621, 0.09157621},
    {0.44594849, 0.44594849, 0.10810302, 0.09157621, 0.09157621, 0.81684757},
    {0.44594849, 0.10810302, 0.44594849, 0.09157621, 0.81684757, 0.09157621}};

struct Tri {
    double a[3], b[3], c[3], area, L[14];
    int ep[3], eq[3];
    double2 Mst[4], Mmt[4], Msz, Mmz;
    double lam[3][6];
    double N[8][6][2], C[8][6], Lz[6][6], Gz[6][6][2];
};

__device__ __forceinline__ double2 cmul(double2 a, double r) { return make_double2(a.x * r, a.y * r); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }

// sum_q W_q u(q) . (M v(q)) for real 2-vector fields u, v and a complex 2x2 M
__device__ double2 wdot(const Tri& s, const double (*u)[2], const double2* M, const double (*v)[2]) {
    double2 r = make_double2(0.0, 0.0);
    for (int q = 0; q < 6; ++q) {
        const double2 m0 = cadd(cmul(M[0], v[q][0]), cmul(M[1], v[q][1]));
        const double2 m1 = cadd(cmul(M[2], v[q][0]), cmul(M[3], v[q][1]));
        r = cadd(r, cmul(cadd(cmul(m0, u[q][0]), cmul(m1, u[q][1])), c_rule[0][q]));
    }
    return r;
}

__global__ void __launch_bounds__(224) k_port_elem(int64_t n, const double* __restrict__ xy,
                                                   const int32_t* __restrict__ lem, const double2* __restrict__ Ms9,
                                                   const double2* __restrict__ Mm9, double k0, int face_block,
                                                   double2* __restrict__ Aout, double2* __restrict__ Bout) {
    __shared__ Tri s;
    const int64_t t = blockIdx.x;
    const int tid = threadIdx.x;
    if (t >= n) return;
    if (tid == 0) {
        double x[3], y[3];
        for (int k = 0; k < 3; ++k) {
            x[k] = xy[k * n + t];
            y[k] = xy[(3 + k) * n + t];
        }
        double a[3] = {x[1] * y[2] - y[1] * x[2], x[2] * y[0] - y[2] * x[0], x[0] * y[1] - y[0] * x[1]};
        double b[3] = {y[1] - y[2], y[2] - y[0], y[0] - y[1]};
        double c[3] = {x[2] - x[1], x[0] - x[2], x[1] - x[0]};
        const double sA = 0.5 * ((x[0] - x[2]) * (y[1] - y[0]) - (x[0] - x[1]) * (y[2] - y[0]));
        const double sg = sA > 0.0 ? 1.0 : (sA < 0.0 ? -1.0 : 0.0);
        const double ar = fabs(sA);
        for (int k = 0; k < 3; ++k) {
            s.a[k] = a[k] * sg / (2.0 * ar);
            s.b[k] = b[k] * sg / (2.0 * ar);
            s.c[k] = c[k] * sg / (2.0 * ar);
        }
        s.area = ar;
        auto dist = [&](int i, int j) { return sqrt((x[i] - x[j]) * (x[i] - x[j]) + (y[i] - y[j]) * (y[i] - y[j])); };
        for (int e = 0; e < 3; ++e) {
            s.ep[e] = lem[e * n + t];
            s.eq[e] = lem[(3 + e) * n + t];
            s.L[e] = s.L[4 + e] = dist(s.ep[e], s.eq[e]);
        }
        s.L[3] = dist(0, 2);
        s.L[7] = dist(0, 1);
        for (int k = 8; k < 14; ++k) s.L[k] = 1.0;
        s.Mst[0] = Ms9[0 * n + t]; s.Mst[1] = Ms9[1 * n + t]; s.Mst[2] = Ms9[3 * n + t]; s.Mst[3] = Ms9[4 * n + t];
        s.Mmt[0] = Mm9[0 * n + t]; s.Mmt[1] = Mm9[1 * n + t]; s.Mmt[2] = Mm9[3 * n + t]; s.Mmt[3] = Mm9[4 * n + t];
        s.Msz = Ms9[8 * n + t];
        s.Mmz = Mm9[8 * n + t];
    }
    __syncthreads();
    if (tid < 6) {
        const int q = tid;
        double px = 0.0, py = 0.0;
        {
            double x[3], y[3];
            for (int k = 0; k < 3; ++k) {
                x[k] = xy[k * n + t];
                y[k] = xy[(3 + k) * n + t];
            }
            px = x[0] * c_rule[1][q] + x[1] * c_rule[2][q] + x[2] * c_rule[3][q];
            py = y[0] * c_rule[1][q] + y[1] * c_rule[2][q] + y[2] * c_rule[3][q];
        }
        double l[3];
        for (int i = 0; i < 3; ++i) l[i] = s.lam[i][q] = s.a[i] + s.b[i] * px + s.c[i] * py;
        const double* b = s.b;
        const double* c = s.c;
        for (int e = 0; e < 3; ++e) {
            const int p = s.ep[e], r = s.eq[e];
            const double wx = b[p] * l[r] - b[r] * l[p], wy = c[p] * l[r] - c[r] * l[p];
            const double rot = b[r] * c[p] - b[p] * c[r];
            s.N[e][q][0] = wx * l[p];
            s.N[e][q][1] = wy * l[p];
            s.N[4 + e][q][0] = wx * l[r];
            s.N[4 + e][q][1] = wy * l[r];
            s.C[e][q] = 3.0 * l[p] * rot;
            s.C[4 + e][q] = 3.0 * l[r] * rot;
            s.Lz[3 + e][q] = 4.0 * l[p] * l[r];
            s.Gz[3 + e][q][0] = 4.0 * (b[p] * l[r] + b[r] * l[p]);
            s.Gz[3 + e][q][1] = 4.0 * (c[p] * l[r] + c[r] * l[p]);
        }
        s.N[3][q][0] = -(b[0] * l[2] - b[2] * l[0]) * l[1];
        s.N[3][q][1] = -(c[0] * l[2] - c[2] * l[0]) * l[1];
        s.N[7][q][0] = (b[0] * l[1] - b[1] * l[0]) * l[2];
        s.N[7][q][1] = (c[0] * l[1] - c[1] * l[0]) * l[2];
        s.C[3][q] = -b[1] * (c[0] * l[2] - c[2] * l[0]) + c[1] * (b[0] * l[2] - b[2] * l[0]) +
                    2.0 * (b[0] * c[2] - b[2] * c[0]) * l[1];
        s.C[7][q] = b[2] * (c[0] * l[1] - c[1] * l[0]) - c[2] * (b[0] * l[1] - b[1] * l[0]) -
                    2.0 * (b[0] * c[1] - b[1] * c[0]) * l[2];
        for (int i = 0; i < 3; ++i) {
            s.Lz[i][q] = 2.0 * l[i] * l[i] - l[i];
            s.Gz[i][q][0] = b[i] * (4.0 * l[i] - 1.0);
            s.Gz[i][q][1] = c[i] * (4.0 * l[i] - 1.0);
        }
    }
    __syncthreads();
    if (tid >= 196) return;
    int i = tid / 14, j = tid % 14;
    double2 A = make_double2(0.0, 0.0), B = make_double2(0.0, 0.0);
    const double k2 = k0 * k0;
    const bool face_i = (i == 3 || i == 7), face_j = (j == 3 || j == 7);
    if (i < 8 && j < 8) {
        // face rows x edge columns: the mirror of edge rows x face columns
        int ii = i, jj = j;
        if (face_i && !face_j) { ii = j; jj = i; }
        double cc = 0.0;
        for (int q = 0; q < 6; ++q) cc += c_rule[0][q] * s.C[ii][q] * s.C[jj][q];
        const double2 att = make_double2(s.Msz.x * cc, s.Msz.y * cc);
        const double2 btt = wdot(s, s.N[ii], s.Mmt, s.N[jj]);
        A = make_double2(att.x - k2 * btt.x, att.y - k2 * btt.y);
        if (!(face_i && face_j) || face_block) B = wdot(s, s.N[ii], s.Mst, s.N[jj]);
    } else if (i >= 8 && j < 8) {
        B = wdot(s, s.Gz[i - 8], s.Mst, s.N[j]);
    } else if (i < 8 && j >= 8) {
        B = wdot(s, s.Gz[j - 8], s.Mst, s.N[i]);
    } else {
        const double2 g = wdot(s, s.Gz[i - 8], s.Mst, s.Gz[j - 8]);
        double ll = 0.0;
        for (int q = 0; q < 6; ++q) ll += c_rule[0][q] * s.Lz[i - 8][q] * s.Lz[j - 8][q];
        B = make_double2(g.x - k2 * (s.Mmz.x * ll), g.y - k2 * (s.Mmz.y * ll));
    }
    const double sc = s.L[i] * s.L[j] * s.area;
    Aout[t * 196 + i * 14 + j] = make_double2(A.x * sc, A.y * sc);
    Bout[t * 196 + i * 14 + j] = make_double2(B.x * sc, B.y * sc);
}

}  // namespace ports
}  // namespace emg

extern "C" int emg_port_element_matrices(int64_t n_tris, const double* xy, const int32_t* local_edge_map,
                                         const double* Ms9, const double* Mm9, double k0, int face_block,
                                         double* A_out, double* B_out, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(n_tris >= 0, "emg_port_element_matrices: negative size");
    EMG_CHECK_ARG(n_tris == 0 || (xy && local_edge_map && Ms9 && Mm9 && A_out && B_out),
                  "emg_port_element_matrices: NULL array");
    EMG_CHECK_ARG(n_tris < (int64_t)INT32_MAX, "emg_port_element_matrices: too many triangles");
    if (n_tris == 0) return EMG_OK;
    ports::k_port_elem<<<(unsigned)n_tris, 224, 0, (cudaStream_t)stream>>>(
        n_tris, xy, local_edge_map, reinterpret_cast<const double2*>(Ms9), reinterpret_cast<const double2*>(Mm9), k0,
        face_block, reinterpret_cast<double2*>(A_out), reinterpret_cast<double2*>(B_out));
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}

// ------------------------------------------------------- port-mode fields ---
// The Nedelec-Lagrange-2 field of a port mode at points of the port plane, the
// counterpart of ned2_tri_interp_full (E) and ned2_tri_interp_curl (the H field up to
// the factor j / (omega mu0)) of fem/mth/tri.py:228-401.  Thread per point, FP64.
//
// Point location as the reference: every triangle is tested, in order, with the local
// coordinates from the inverse of [v2 - v1, v3 - v1] and the tolerances
// xi >= -1e-6, eta >= -1e-6, xi + eta <= 1.00000001; the last triangle that contains the
// point gives its value (the reference overwrites), a point in none gets zero.
//
// With the linear barycentric numerators l_i = a_i + b_i x + c_i y (tri_coefficients,
// fem/mth/optimized.py:404-426: a_1 = x2 y3 - y2 x3, b_1 = y2 - y3, c_1 = x3 - x2 and
// cyclic, all times the sign of the signed area; A = |area|) and the DOF values
// e_1..e_14 of the triangle (tri_to_field order, the first eight times the lengths
// L1 L2 L3 L3 L1 L2 L3 L1 of the edges (v0,v1), (v1,v2), (v0,v2)), write
//   W_pq(u) = u_p l_q - u_q l_p      (u = b for the x component, c for the y component)
// for the Whitney-type factor of the edge (p, q).  Then, with S = 8 A^3,
//   E_u = [ e1 W12 l1 + e2 W23 l2 + e3 W13 l1 - e4 W13 l2 + e5 W12 l2 + e6 W23 l3
//           + e7 W13 l3 + e8 W12 l3 ] / S,
//   E_z = l1 [ (e9 + e10 + e11)(l1 - A) + (e12 + e13 + e14) l2 ] / (2 A^2),
// and the curl terms are the reference's expressions for hx, hy, hz (the latter a
// polynomial in a_i, b_i, c_i, x, y restated term by term below), each times the
// corresponding diagonal entry of matinv(ur) of the triangle.
namespace emg {
namespace ports {

__device__ __forceinline__ double2 cz(double r) { return make_double2(r, 0.0); }
__device__ __forceinline__ double2 cm(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ double2 cs(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
__device__ __forceinline__ double2 ca(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csb(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }

__global__ void k_port_interp(int64_t npts, const double* __restrict__ xy, int64_t nT, const int32_t* __restrict__ tris,
                              int64_t nN, const double* __restrict__ nodes2, const int32_t* __restrict__ t2f,
                              const double2* __restrict__ field, const double2* __restrict__ urinv, double beta,
                              int which, double2* __restrict__ out) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npts; p += (int64_t)gridDim.x * blockDim.x) {
        const double x = xy[p], y = xy[npts + p];
        int64_t hit = -1;
        for (int64_t t = 0; t < nT; ++t) {
            const int32_t i1 = tris[t], i2 = tris[nT + t], i3 = tris[2 * nT + t];
            const double x1 = nodes2[i1], y1 = nodes2[nN + i1];
            const double m00 = nodes2[i2] - x1, m10 = nodes2[nN + i2] - y1;
            const double m01 = nodes2[i3] - x1, m11 = nodes2[nN + i3] - y1;
            const double det = m00 * m11 - m01 * m10;
            if (det == 0.0) continue;
            const double dx = x - x1, dy = y - y1;
            const double xi = (m11 * dx - m01 * dy) / det, eta = (-m10 * dx + m00 * dy) / det;
            if (xi + eta <= 1.00000001 && xi >= -1e-6 && eta >= -1e-6) hit = t;
        }
        double2 o0 = cz(0.0), o1 = cz(0.0), o2 = cz(0.0);
        if (hit >= 0) {
            const int64_t t = hit;
            const int32_t v[3] = {tris[t], tris[nT + t], tris[2 * nT + t]};
            double xs[3], ys[3];
            for (int k = 0; k < 3; ++k) { xs[k] = nodes2[v[k]]; ys[k] = nodes2[nN + v[k]]; }
            double a[3] = {xs[1] * ys[2] - ys[1] * xs[2], xs[2] * ys[0] - ys[2] * xs[0], xs[0] * ys[1] - ys[0] * xs[1]};
            double b[3] = {ys[1] - ys[2], ys[2] - ys[0], ys[0] - ys[1]};
            double c[3] = {xs[2] - xs[1], xs[0] - xs[2], xs[1] - xs[0]};
            const double sA = 0.5 * ((xs[0] - xs[2]) * (ys[1] - ys[0]) - (xs[0] - xs[1]) * (ys[2] - ys[0]));
            const double sg = sA > 0.0 ? 1.0 : (sA < 0.0 ? -1.0 : 0.0);
            const double A = fabs(sA);
            for (int k = 0; k < 3; ++k) { a[k] *= sg; b[k] *= sg; c[k] *= sg; }
            const double L1 = sqrt((xs[0] - xs[1]) * (xs[0] - xs[1]) + (ys[0] - ys[1]) * (ys[0] - ys[1]));
            const double L2 = sqrt((xs[1] - xs[2]) * (xs[1] - xs[2]) + (ys[1] - ys[2]) * (ys[1] - ys[2]));
            const double L3 = sqrt((xs[0] - xs[2]) * (xs[0] - xs[2]) + (ys[0] - ys[2]) * (ys[0] - ys[2]));
            const double mult[14] = {L1, L2, L3, L3, L1, L2, L3, L1, 1, 1, 1, 1, 1, 1};
            double2 e[15];
            for (int k = 0; k < 14; ++k) e[k + 1] = cs(mult[k], field[t2f[k * nT + t]]);
            const double l1 = a[0] + b[0] * x + c[0] * y, l2 = a[1] + b[1] * x + c[1] * y, l3 = a[2] + b[2] * x + c[2] * y;
            const double S = 8.0 * A * A * A;
            // transverse components for u = b (x) and u = c (y)
            auto trans = [&](const double* u) {
                const double W12 = u[0] * l2 - u[1] * l1, W23 = u[1] * l3 - u[2] * l2, W13 = u[0] * l3 - u[2] * l1;
                double2 s = cs(W12 * l1, e[1]);
                s = ca(s, cs(W23 * l2, e[2]));
                s = ca(s, cs(W13 * l1, e[3]));
                s = csb(s, cs(W13 * l2, e[4]));
                s = ca(s, cs(W12 * l2, e[5]));
                s = ca(s, cs(W23 * l3, e[6]));
                s = ca(s, cs(W13 * l3, e[7]));
                s = ca(s, cs(W12 * l3, e[8]));
                return s;
            };
            const double2 zs1 = ca(ca(e[9], e[10]), e[11]), zs2 = ca(ca(e[12], e[13]), e[14]);
            const double2 zpoly = ca(cs(l1 - A, zs1), cs(l2, zs2));
            if (which == 0) {
                o0 = cs(1.0 / S, trans(b));
                o1 = cs(1.0 / S, trans(c));
                o2 = cs(l1 / (2.0 * A * A), zpoly);
            } else {
                const double2 jB = make_double2(0.0, beta);
                const double2 gz_c = ca(cs(c[0], zs1), cs(c[1], zs2));
                const double2 gz_b = ca(cs(b[0], zs1), cs(b[1], zs2));
                const double2 hx = ca(cs(4.0 * A, ca(cs(c[0], zpoly), cs(l1, gz_c))), cm(jB, trans(c)));
                const double2 hy = csb(cs(4.0 * A, ca(cs(b[0], zpoly), cs(l1, gz_b))), cm(jB, trans(b)));
                // hz: the reference's polynomial (fem/mth/tri.py:392-393), grouped by DOF
                const double a1 = a[0], a2 = a[1], a3 = a[2], b1 = b[0], b2 = b[1], b3 = b[2];
                const double c1 = c[0], c2 = c[1], c3 = c[2];
                double k1 = -3 * a1 * b1 * c2 + 3 * a1 * b2 * c1 - 3 * b1 * b1 * c2 * x + 3 * b1 * b2 * c1 * x
                            - 3 * b1 * c1 * c2 * y + 3 * b2 * c1 * c1 * y;
                double k2 = -3 * a2 * b2 * c3 + 3 * a2 * b3 * c2 - 3 * b2 * b2 * c3 * x + 3 * b2 * b3 * c2 * x
                            - 3 * b2 * c2 * c3 * y + 3 * b3 * c2 * c2 * y;
                double k3 = -3 * a1 * b1 * c3 + 3 * a1 * b3 * c1 - 3 * b1 * b1 * c3 * x + 3 * b1 * b3 * c1 * x
                            - 3 * b1 * c1 * c3 * y + 3 * b3 * c1 * c1 * y;
                double k4 = a1 * b2 * c3 - a1 * b3 * c2 + 2 * a2 * b1 * c3 - 2 * a2 * b3 * c1 + a3 * b1 * c2
                            - a3 * b2 * c1 + 3 * b1 * b2 * c3 * x - 3 * b2 * b3 * c1 * x + 3 * b1 * c2 * c3 * y
                            - 3 * b3 * c1 * c2 * y;
                double k5 = -3 * a2 * b1 * c2 + 3 * a2 * b2 * c1 - 3 * b1 * b2 * c2 * x + 3 * b2 * b2 * c1 * x
                            - 3 * b1 * c2 * c2 * y + 3 * b2 * c1 * c2 * y;
                double k6 = -3 * a3 * b2 * c3 + 3 * a3 * b3 * c2 - 3 * b2 * b3 * c3 * x + 3 * b3 * b3 * c2 * x
                            - 3 * b2 * c3 * c3 * y + 3 * b3 * c2 * c3 * y;
                double k7 = -3 * a3 * b1 * c3 + 3 * a3 * b3 * c1 - 3 * b1 * b3 * c3 * x + 3 * b3 * b3 * c1 * x
                            - 3 * b1 * c3 * c3 * y + 3 * b3 * c1 * c3 * y;
                double k8 = a1 * b2 * c3 - a1 * b3 * c2 - a2 * b1 * c3 + a2 * b3 * c1 - 2 * a3 * b1 * c2
                            + 2 * a3 * b2 * c1 - 3 * b1 * b3 * c2 * x + 3 * b2 * b3 * c1 * x - 3 * b1 * c2 * c3 * y
                            + 3 * b2 * c1 * c3 * y;
                double2 hz = cs(k1, e[1]);
                hz = ca(hz, cs(k2, e[2]));
                hz = ca(hz, cs(k3, e[3]));
                hz = ca(hz, cs(k4, e[4]));
                hz = ca(hz, cs(k5, e[5]));
                hz = ca(hz, cs(k6, e[6]));
                hz = ca(hz, cs(k7, e[7]));
                hz = ca(hz, cs(k8, e[8]));
                const double2 d0 = urinv[t], d1 = urinv[nT + t], d2 = urinv[2 * nT + t];
                o0 = cm(cs(1.0 / S, hx), d0);
                o1 = cm(cs(1.0 / S, hy), d1);
                o2 = cm(cs(1.0 / S, hz), d2);
            }
        }
        out[p] = o0;
        out[npts + p] = o1;
        out[2 * npts + p] = o2;
    }
}

}  // namespace ports
}  // namespace emg

extern "C" int emg_port_interp(int64_t npts, const double* xy, int64_t n_tris, const int32_t* tris, int64_t n_nodes,
                               const double* nodes2, const int32_t* tri_to_field, const double* field,
                               const double* urinv_diag, double beta, int which, double* out, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(npts >= 0 && n_tris >= 0 && n_nodes >= 0, "emg_port_interp: negative size");
    EMG_CHECK_ARG(which == 0 || which == 1, "emg_port_interp: which must be 0 (E) or 1 (curl)");
    if (npts == 0) return EMG_OK;
    EMG_CHECK_ARG(xy && out && (n_tris == 0 || (tris && nodes2 && tri_to_field && field)),
                  "emg_port_interp: NULL array");
    EMG_CHECK_ARG(which == 0 || n_tris == 0 || urinv_diag, "emg_port_interp: the curl needs urinv_diag");
    ports::k_port_interp<<<grid_for(npts, 128), 128, 0, (cudaStream_t)stream>>>(
        npts, xy, n_tris, tris, n_nodes, nodes2, tri_to_field, reinterpret_cast<const double2*>(field),
        reinterpret_cast<const double2*>(urinv_diag), beta, which, reinterpret_cast<double2*>(out));
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}
