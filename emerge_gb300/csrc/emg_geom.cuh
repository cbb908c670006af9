// Tetrahedron geometry with the reference's rounding (shared by the assembly kernels).
//
// tet_coefficients_bcd (fem/mth/optimized.py:343-369) evaluates 6V as an expanded
// 24-term determinant and the gradient cofactors as six-term 2x2 sums, in
// absolute coordinates.  The sums cancel heavily on fine meshes far from the
// origin, so the result is only reproducible term by term: every product and sum
// below uses the _rn intrinsics (no FMA contraction), in the reference's order.
#pragma once

#include <stdint.h>

namespace emg {
namespace geom {

// 6V terms: sign, vertex for x, vertex for y, vertex for z.
__constant__ int8_t c_vol_terms[24][4] = {
    {-1, 0, 1, 2}, {+1, 0, 1, 3}, {+1, 0, 2, 1}, {-1, 0, 2, 3}, {-1, 0, 3, 1}, {+1, 0, 3, 2},
    {+1, 1, 0, 2}, {-1, 1, 0, 3}, {-1, 1, 2, 0}, {+1, 1, 2, 3}, {+1, 1, 3, 0}, {-1, 1, 3, 2},
    {-1, 2, 0, 1}, {+1, 2, 0, 3}, {+1, 2, 1, 0}, {-1, 2, 1, 3}, {-1, 2, 3, 0}, {+1, 2, 3, 1},
    {+1, 3, 0, 1}, {-1, 3, 0, 2}, {-1, 3, 1, 0}, {+1, 3, 1, 2}, {+1, 3, 2, 0}, {-1, 3, 2, 1}};
// b_i terms (u,v) = (y,z): sign, u-vertex, v-vertex.  d_i: same terms with (x,y);
// c_i: negated terms with (x,z).
__constant__ int8_t c_cof_terms[4][6][3] = {
    {{-1, 1, 2}, {+1, 1, 3}, {+1, 2, 1}, {-1, 2, 3}, {-1, 3, 1}, {+1, 3, 2}},
    {{+1, 0, 2}, {-1, 0, 3}, {-1, 2, 0}, {+1, 2, 3}, {+1, 3, 0}, {-1, 3, 2}},
    {{-1, 0, 1}, {+1, 0, 3}, {+1, 1, 0}, {-1, 1, 3}, {-1, 3, 0}, {+1, 3, 1}},
    {{+1, 0, 1}, {-1, 0, 2}, {-1, 1, 0}, {+1, 1, 2}, {+1, 2, 0}, {-1, 2, 1}}};

// V and G[i] = (b_i, c_i, d_i) exactly as the reference rounds them.
__device__ inline void tet_bcd(const double x[4], const double y[4], const double z[4], double G[4][3],
                               double* V) {
    double s = 0.0;
    for (int k = 0; k < 24; ++k) {
        const double t = __ddiv_rn(__dmul_rn(__dmul_rn(x[c_vol_terms[k][1]], y[c_vol_terms[k][2]]),
                                             z[c_vol_terms[k][3]]), 6.0);
        s = c_vol_terms[k][0] > 0 ? __dadd_rn(s, t) : __dsub_rn(s, t);
    }
    *V = fabs(s);
    for (int i = 0; i < 4; ++i) {
        double sb = 0.0, sc = 0.0, sd = 0.0;
        for (int k = 0; k < 6; ++k) {
            const int sg = c_cof_terms[i][k][0], a = c_cof_terms[i][k][1], b = c_cof_terms[i][k][2];
            const double pb = __dmul_rn(y[a], z[b]), pc = __dmul_rn(x[a], z[b]), pd = __dmul_rn(x[a], y[b]);
            sb = sg > 0 ? __dadd_rn(sb, pb) : __dsub_rn(sb, pb);
            sc = sg > 0 ? __dsub_rn(sc, pc) : __dadd_rn(sc, pc);
            sd = sg > 0 ? __dadd_rn(sd, pd) : __dsub_rn(sd, pd);
        }
        G[i][0] = sb;
        G[i][1] = sc;
        G[i][2] = sd;
    }
}

}  // namespace geom
}  // namespace emg
