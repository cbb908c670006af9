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
