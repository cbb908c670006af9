// Second-order Nedelec field evaluation at arbitrary points: the GPU counterpart of
// ned2_tet_interp (fem/mth/tet.py:372-497), which EMerge uses for the S-parameter
// surface integrals (all_port_tets, fem/physics/edm/emfreq3d.py:648-653,703) and for
// field output.
//
// Thread per point.  Location follows the reference: a point belongs to a tet of
// ``tetids`` when its local coordinates xi = [v2-v1, v3-v1, v4-v1]^-1 (p - v1)
// satisfy xi >= -1e-6 and sum(xi) <= 1 + 1e-8, and the last such tet in list
// order wins (the reference overwrites in tet order), so the scan runs backwards
// and stops at the first hit.  Field: with the barycentric numerators
// A_i = a_i + b_i x + c_i y + d_i z = det(P) lambda_i (P rows (1, x_j, y_j, z_j))
// and 216 V^3 = |det P|^3,
//   edge (vertices 1, 2, length L):  L (e1 A1 + e2 A2)(g1 A2 - g2 A1) / 216 V^3
//   face (vertices 1, 2, 3):         (-e1 |v1v3| (g1 A3 - g3 A1) A2
//                                     + e2 |v1v2| (g1 A2 - g2 A1) A3) / 216 V^3
// for g = b, c, d (x, y, z components), vertices in the mesh's edges/tris order.
#include "emg_common.cuh"

namespace emg {
namespace interp {

__device__ __forceinline__ double det3(double a, double b, double c, double d, double e, double f, double g, double h,
                                       double i) {
    return a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
}

__device__ __forceinline__ int local_of(const int32_t* tv, int32_t gid) {
    return tv[0] == gid ? 0 : tv[1] == gid ? 1 : tv[2] == gid ? 2 : 3;
}

// The containing tet of point p (backwards over tetids) and its barycentric
// numerators, their gradients and 216 V^3; false when no tet contains p.
struct TetAt {
    int64_t t;
    int32_t tv[4];
    double vx[4], vy[4], vz[4];
    double A[4], gb[4], gc[4], gd[4];
    double den;
};

__device__ bool locate(double px, double py, double pz, const double* __restrict__ nodes, int64_t nN,
                       const int32_t* __restrict__ tets, int64_t nT, int64_t ntl, const int32_t* __restrict__ tetids,
                       TetAt& r) {
    for (int64_t it = ntl - 1; it >= 0; --it) {
        const int64_t t = tetids[it];
        if (t < 0 || t >= nT) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            r.tv[j] = tets[j * nT + t];
            r.vx[j] = nodes[r.tv[j]];
            r.vy[j] = nodes[nN + r.tv[j]];
            r.vz[j] = nodes[2 * nN + r.tv[j]];
        }
        const double* vx = r.vx;
        const double* vy = r.vy;
        const double* vz = r.vz;
        // local coordinates: solve [e1 e2 e3] xi = p - v1 by Cramer's rule
        const double e1x = vx[1] - vx[0], e1y = vy[1] - vy[0], e1z = vz[1] - vz[0];
        const double e2x = vx[2] - vx[0], e2y = vy[2] - vy[0], e2z = vz[2] - vz[0];
        const double e3x = vx[3] - vx[0], e3y = vy[3] - vy[0], e3z = vz[3] - vz[0];
        const double qx = px - vx[0], qy = py - vy[0], qz = pz - vz[0];
        const double dm = det3(e1x, e2x, e3x, e1y, e2y, e3y, e1z, e2z, e3z);
        if (dm == 0.0) continue;
        const double x0 = det3(qx, e2x, e3x, qy, e2y, e3y, qz, e2z, e3z) / dm;
        const double x1 = det3(e1x, qx, e3x, e1y, qy, e3y, e1z, qz, e3z) / dm;
        const double x2 = det3(e1x, e2x, qx, e1y, e2y, qy, e1z, e2z, qz) / dm;
        if (!(x0 + x1 + x2 <= 1.00000001 && x0 >= -1e-6 && x1 >= -1e-6 && x2 >= -1e-6)) continue;
        // barycentric numerators A_i(p) = det(P_i(p)), P_i = P with row i -> (1, p).
        // Moving row i to the top and subtracting it: det(P_i(p)) = (-1)^i det[v_j - p;
        // v_k - p; v_l - p] with (j, k, l) the other vertices in cyclic order (an even
        // permutation of ascending order), and grad det[a - p; b - p; c - p] =
        // -(b - a) x (c - a), so the coefficients (b_i, c_i, d_i) = -(-1)^i (v_k - v_j)
        // x (v_l - v_j).  det(P) = det[e1; e2; e3] = dm.
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int j = (i + 1) & 3, k = (i + 2) & 3, l = (i + 3) & 3;
            const double sg = (i & 1) ? -1.0 : 1.0;
            const double ax = vx[j] - px, ay = vy[j] - py, az = vz[j] - pz;
            const double bx = vx[k] - px, by = vy[k] - py, bz = vz[k] - pz;
            const double cx = vx[l] - px, cy = vy[l] - py, cz = vz[l] - pz;
            r.A[i] = sg * det3(ax, bx, cx, ay, by, cy, az, bz, cz);
            r.gb[i] = -sg * ((vy[k] - vy[j]) * (vz[l] - vz[j]) - (vz[k] - vz[j]) * (vy[l] - vy[j]));
            r.gc[i] = -sg * ((vz[k] - vz[j]) * (vx[l] - vx[j]) - (vx[k] - vx[j]) * (vz[l] - vz[j]));
            r.gd[i] = -sg * ((vx[k] - vx[j]) * (vy[l] - vy[j]) - (vy[k] - vy[j]) * (vx[l] - vx[j]));
        }
        r.den = fabs(dm) * fabs(dm) * fabs(dm);
        r.t = t;
        return true;
    }
    return false;
}

__device__ __forceinline__ double seg_len(const TetAt& r, int a, int b) {
    return sqrt((r.vx[a] - r.vx[b]) * (r.vx[a] - r.vx[b]) + (r.vy[a] - r.vy[b]) * (r.vy[a] - r.vy[b]) +
                (r.vz[a] - r.vz[b]) * (r.vz[a] - r.vz[b]));
}

__global__ void k_interp(int64_t np_, const double* __restrict__ pts, const double* __restrict__ nodes, int64_t nN,
                         const int32_t* __restrict__ tets, int64_t nT, const int32_t* __restrict__ edges, int64_t nE,
                         const int32_t* __restrict__ tris, int64_t nTri, const int32_t* __restrict__ t2f,
                         const double2* __restrict__ sol, int64_t ntl, const int32_t* __restrict__ tetids,
                         double2* __restrict__ E) {
    const int64_t ip = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (ip >= np_) return;
    const double px = pts[ip], py = pts[np_ + ip], pz = pts[2 * np_ + ip];
    double2 rx = make_double2(0, 0), ry = rx, rz = rx;
    TetAt r;
    if (locate(px, py, pz, nodes, nN, tets, nT, ntl, tetids, r)) {
        const double* A = r.A;
        const double* gb = r.gb;
        const double* gc = r.gc;
        const double* gd = r.gd;
        const double den = r.den;
        const int32_t* f = t2f + r.t;   // column t of (20, nT)
        for (int ie = 0; ie < 6; ++ie) {
            const int32_t eid = f[ie * nT];
            const int i1 = local_of(r.tv, edges[eid]), i2 = local_of(r.tv, edges[nE + eid]);
            const double L = seg_len(r, i1, i2);
            const double2 e1 = sol[f[ie * nT]], e2 = sol[f[(10 + ie) * nT]];
            const double2 sv = make_double2(e1.x * A[i1] + e2.x * A[i2], e1.y * A[i1] + e2.y * A[i2]);
            const double wx = L * (gb[i1] * A[i2] - gb[i2] * A[i1]) / den;
            const double wy = L * (gc[i1] * A[i2] - gc[i2] * A[i1]) / den;
            const double wz = L * (gd[i1] * A[i2] - gd[i2] * A[i1]) / den;
            rx.x += sv.x * wx; rx.y += sv.y * wx;
            ry.x += sv.x * wy; ry.y += sv.y * wy;
            rz.x += sv.x * wz; rz.y += sv.y * wz;
        }
        for (int jf = 0; jf < 4; ++jf) {
            const int64_t fid = f[(6 + jf) * nT] - nE;
            const int i1 = local_of(r.tv, tris[fid]), i2 = local_of(r.tv, tris[nTri + fid]),
                      i3 = local_of(r.tv, tris[2 * nTri + fid]);
            const double L1 = seg_len(r, i1, i3);
            const double L2 = seg_len(r, i1, i2);
            const double2 e1 = sol[f[(6 + jf) * nT]], e2 = sol[f[(16 + jf) * nT]];
            const double* g[3] = {gb, gc, gd};
            double w1[3], w2[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                w1[d] = -L1 * (g[d][i1] * A[i3] - g[d][i3] * A[i1]) * A[i2] / den;
                w2[d] = L2 * (g[d][i1] * A[i2] - g[d][i2] * A[i1]) * A[i3] / den;
            }
            rx.x += e1.x * w1[0] + e2.x * w2[0]; rx.y += e1.y * w1[0] + e2.y * w2[0];
            ry.x += e1.x * w1[1] + e2.x * w2[1]; ry.y += e1.y * w1[1] + e2.y * w2[1];
            rz.x += e1.x * w1[2] + e2.x * w2[2]; rz.y += e1.y * w1[2] + e2.y * w2[2];
        }
    }
    E[ip] = rx;
    E[np_ + ip] = ry;
    E[2 * np_ + ip] = rz;
}

// Line functional weights: for point p with step d (e.g. a voltage-line segment),
// the 20 DOFs of the containing tet and w_k = d . N_k(p), so that sum_k w_k x[dof_k]
// = d . E(p) for every solution x.  No containing tet: dofs -1, weights 0.
__global__ void k_weights(int64_t np_, const double* __restrict__ pts, const double* __restrict__ dirs,
                          const double* __restrict__ nodes, int64_t nN, const int32_t* __restrict__ tets, int64_t nT,
                          const int32_t* __restrict__ edges, int64_t nE, const int32_t* __restrict__ tris,
                          int64_t nTri, const int32_t* __restrict__ t2f, int64_t ntl,
                          const int32_t* __restrict__ tetids, int32_t* __restrict__ dof, double* __restrict__ w) {
    const int64_t ip = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (ip >= np_) return;
    const double px = pts[ip], py = pts[np_ + ip], pz = pts[2 * np_ + ip];
    const double dx = dirs[ip], dy = dirs[np_ + ip], dz = dirs[2 * np_ + ip];
    int32_t* od = dof + ip * 20;
    double* ow = w + ip * 20;
    TetAt r;
    if (!locate(px, py, pz, nodes, nN, tets, nT, ntl, tetids, r)) {
        for (int k = 0; k < 20; ++k) {
            od[k] = -1;
            ow[k] = 0.0;
        }
        return;
    }
    const double* A = r.A;
    const double den = r.den;
    const int32_t* f = t2f + r.t;
    for (int ie = 0; ie < 6; ++ie) {
        const int32_t eid = f[ie * nT];
        const int i1 = local_of(r.tv, edges[eid]), i2 = local_of(r.tv, edges[nE + eid]);
        const double L = seg_len(r, i1, i2);
        // d . L (g1 A2 - g2 A1) / den, times A1 (mode 1) or A2 (mode 2)
        const double q = L * (dx * (r.gb[i1] * A[i2] - r.gb[i2] * A[i1]) + dy * (r.gc[i1] * A[i2] - r.gc[i2] * A[i1]) +
                              dz * (r.gd[i1] * A[i2] - r.gd[i2] * A[i1])) / den;
        od[ie] = f[ie * nT];
        ow[ie] = q * A[i1];
        od[10 + ie] = f[(10 + ie) * nT];
        ow[10 + ie] = q * A[i2];
    }
    for (int jf = 0; jf < 4; ++jf) {
        const int64_t fid = f[(6 + jf) * nT] - nE;
        const int i1 = local_of(r.tv, tris[fid]), i2 = local_of(r.tv, tris[nTri + fid]),
                  i3 = local_of(r.tv, tris[2 * nTri + fid]);
        const double L1 = seg_len(r, i1, i3);
        const double L2 = seg_len(r, i1, i2);
        const double c1 = dx * (r.gb[i1] * A[i3] - r.gb[i3] * A[i1]) + dy * (r.gc[i1] * A[i3] - r.gc[i3] * A[i1]) +
                          dz * (r.gd[i1] * A[i3] - r.gd[i3] * A[i1]);
        const double c2 = dx * (r.gb[i1] * A[i2] - r.gb[i2] * A[i1]) + dy * (r.gc[i1] * A[i2] - r.gc[i2] * A[i1]) +
                          dz * (r.gd[i1] * A[i2] - r.gd[i2] * A[i1]);
        od[6 + jf] = f[(6 + jf) * nT];
        ow[6 + jf] = -L1 * c1 * A[i2] / den;
        od[16 + jf] = f[(16 + jf) * nT];
        ow[16 + jf] = L2 * c2 * A[i3] / den;
    }
}

}  // namespace interp
}  // namespace emg

extern "C" int emg_field_weights(int64_t n_points, const double* points, const double* dirs, int64_t n_nodes,
                                 const double* nodes, int64_t n_tets, const int32_t* tets, int64_t n_edges,
                                 const int32_t* edges, int64_t n_tris, const int32_t* tris,
                                 const int32_t* tet_to_field, int64_t n_tetids, const int32_t* tetids,
                                 int32_t* dofs_out, double* weights_out, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(points && dirs && nodes && tets && edges && tris && tet_to_field && dofs_out && weights_out &&
                      n_points >= 0 && n_tetids >= 0 && (n_tetids == 0 || tetids),
                  "emg_field_weights: bad argument");
    if (n_points == 0) return EMG_OK;
    interp::k_weights<<<(unsigned)((n_points + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
        n_points, points, dirs, nodes, n_nodes, tets, n_tets, edges, n_edges, tris, n_tris, tet_to_field, n_tetids,
        tetids, dofs_out, weights_out);
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}

extern "C" int emg_field_interp(int64_t n_points, const double* points, int64_t n_nodes, const double* nodes,
                                int64_t n_tets, const int32_t* tets, int64_t n_edges, const int32_t* edges,
                                int64_t n_tris, const int32_t* tris, const int32_t* tet_to_field, const double* solution,
                                int64_t n_tetids, const int32_t* tetids, double* E_out, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(points && nodes && tets && edges && tris && tet_to_field && solution && E_out && n_points >= 0 &&
                      n_tetids >= 0 && (n_tetids == 0 || tetids),
                  "emg_field_interp: bad argument");
    if (n_points == 0) return EMG_OK;
    interp::k_interp<<<(unsigned)((n_points + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
        n_points, points, nodes, n_nodes, tets, n_tets, edges, n_edges, tris, n_tris, tet_to_field,
        reinterpret_cast<const double2*>(solution), n_tetids, tetids, reinterpret_cast<double2*>(E_out));
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}
