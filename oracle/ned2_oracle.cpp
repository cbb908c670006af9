// Oracle: CPU restatement of EMerge's second-order Nedelec assembly.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA path and the
// timed CPU baseline; only tests/, __graft_entry__.smoke() and bench.py's CPU
// legs may load it.  The product (emerge_gb300/) never calls it.
//
// It restates, function by function, the reference's arithmetic:
//   tet_coefficients_bcd   fem/mth/optimized.py:343-369   (same term order, no FMA)
//   compute_distances      fem/mth/optimized.py:428-436
//   volume_coeff           fem/mth/optimized.py:251-260
//   area_coeff             fem/mth/optimized.py:262-271
//   local_mapping          fem/mth/optimized.py:273-307
//   matinv                 fem/mth/optimized.py:440-461   (incl. its adj*det quirk)
//   ned2_tet_stiff_mass    fem/mth/tet.py:854-1088
//   _matrix_builder        fem/physics/edm/optimized_assembly.py:66-116
//   ned2_tri_stiff_force   fem/mth/tri.py:575-695
//   ned2_tri_stiff         fem/mth/tri.py:697-797
// Parity is pinned against fixtures produced by running the reference itself
// (tests/golden/make_golden.py).
//
// Compile with -ffp-contract=off: the volume and cofactor sums must round
// exactly like the reference's left-to-right IEEE evaluation.
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>

typedef std::complex<double> cd;

namespace {

// ---------------------------------------------------------------- geometry ---

// Terms of the 3x3 determinant expansion of 6V, in the reference's order:
// sign, and the vertex (0-based) taken for x, y, z.
const int kVolTerms[24][4] = {
    {-1, 0, 1, 2}, {+1, 0, 1, 3}, {+1, 0, 2, 1}, {-1, 0, 2, 3}, {-1, 0, 3, 1}, {+1, 0, 3, 2},
    {+1, 1, 0, 2}, {-1, 1, 0, 3}, {-1, 1, 2, 0}, {+1, 1, 2, 3}, {+1, 1, 3, 0}, {-1, 1, 3, 2},
    {-1, 2, 0, 1}, {+1, 2, 0, 3}, {+1, 2, 1, 0}, {-1, 2, 1, 3}, {-1, 2, 3, 0}, {+1, 2, 3, 1},
    {+1, 3, 0, 1}, {-1, 3, 0, 2}, {-1, 3, 1, 0}, {+1, 3, 1, 2}, {+1, 3, 2, 0}, {-1, 3, 2, 1}};

// 2x2 cofactor sums: for cofactor i, six terms (sign, u-vertex, v-vertex) of
// sum sign*u[a]*v[b].  b_i uses (u,v)=(y,z), c_i (x,z), d_i (x,y).
const int kCofB[4][6][3] = {
    {{-1, 1, 2}, {+1, 1, 3}, {+1, 2, 1}, {-1, 2, 3}, {-1, 3, 1}, {+1, 3, 2}},
    {{+1, 0, 2}, {-1, 0, 3}, {-1, 2, 0}, {+1, 2, 3}, {+1, 3, 0}, {-1, 3, 2}},
    {{-1, 0, 1}, {+1, 0, 3}, {+1, 1, 0}, {-1, 1, 3}, {-1, 3, 0}, {+1, 3, 1}},
    {{+1, 0, 1}, {-1, 0, 2}, {-1, 1, 0}, {+1, 1, 2}, {+1, 2, 0}, {-1, 2, 1}}};
// c_i and d_i have the opposite sign pattern of b_i (same vertex pairs).

double sum_terms2(const int t[6][3], int sgn, const double* u, const double* v) {
    double s = 0.0;
    for (int k = 0; k < 6; ++k) {
        double p = u[t[k][1]] * v[t[k][2]];
        s = (sgn * t[k][0] > 0) ? s + p : s - p;
    }
    return s;
}

}  // namespace

extern "C" {

void orc_tet_coefficients_bcd(const double* xs, const double* ys, const double* zs,
                              double* b, double* c, double* d, double* V) {
    double s = 0.0;
    for (int k = 0; k < 24; ++k) {
        double t = ((xs[kVolTerms[k][1]] * ys[kVolTerms[k][2]]) * zs[kVolTerms[k][3]]) / 6.0;
        s = (kVolTerms[k][0] > 0) ? s + t : s - t;
    }
    *V = std::fabs(s);
    for (int i = 0; i < 4; ++i) {
        b[i] = sum_terms2(kCofB[i], +1, ys, zs);
        c[i] = sum_terms2(kCofB[i], -1, xs, zs);
        d[i] = sum_terms2(kCofB[i], +1, xs, ys);
    }
}

void orc_compute_distances(const double* xs, const double* ys, const double* zs, int n, double* D) {
    for (int i = 0; i < n; ++i)
        for (int j = i; j < n; ++j) {
            double dx = xs[i] - xs[j], dy = ys[i] - ys[j], dz = zs[i] - zs[j];
            D[i * n + j] = std::sqrt(dx * dx + dy * dy + dz * dz);
            D[j * n + i] = D[i * n + j];
        }
}

// Closed-form monomial integral over the unit-measure simplex: prod(k_v!) / (sum k + 3)!
// where k_v counts how often vertex letter v (1..6; 0 = absent) occurs in (a,b,c,d).
double orc_volume_coeff(int a, int b, int c, int d) {
    static const double fact[10] = {1, 1, 2, 6, 24, 120, 720, 5040, 40320, 362880};
    int k[7] = {0, 0, 0, 0, 0, 0, 0};
    k[a]++; k[b]++; k[c]++; k[d]++;
    double num = fact[k[1]] * fact[k[2]] * fact[k[3]] * fact[k[4]] * fact[k[5]] * fact[k[6]];
    return num / fact[k[1] + k[2] + k[3] + k[4] + k[5] + k[6] + 3];
}

double orc_area_coeff(int a, int b, int c, int d) {
    static const double fact[10] = {1, 1, 2, 6, 24, 120, 720, 5040, 40320, 362880};
    int k[7] = {0, 0, 0, 0, 0, 0, 0};
    k[a]++; k[b]++; k[c]++; k[d]++;
    double num = fact[k[1]] * fact[k[2]] * fact[k[3]] * fact[k[4]] * fact[k[5]] * fact[k[6]];
    return 2 * num / fact[k[1] + k[2] + k[3] + k[4] + k[5] + k[6] + 2];
}

// out[j*ncol + t] = position of gids[j*ncol + t] among the 4 tet vertices (0 if absent).
void orc_local_mapping(const int64_t* vertex_ids, const int64_t* gids, int nrow, int ncol, int64_t* out) {
    for (int t = 0; t < ncol; ++t)
        for (int j = 0; j < nrow; ++j) {
            out[j * ncol + t] = 0;
            for (int k = 0; k < 4; ++k)
                if (vertex_ids[k] == gids[j * ncol + t]) { out[j * ncol + t] = k; break; }
        }
}

// 3x3 complex inverse as the reference computes it: diagonal fast path, and the
// adjugate multiplied (not divided) by the determinant otherwise.
void orc_matinv(const double* s_ri, double* out_ri) {
    const cd* s = reinterpret_cast<const cd*>(s_ri);
    cd* o = reinterpret_cast<cd*>(out_ri);
    for (int i = 0; i < 9; ++i) o[i] = 0.0;
    auto S = [&](int i, int j) { return s[3 * i + j]; };
    if (S(0, 1) == 0.0 && S(0, 2) == 0.0 && S(1, 0) == 0.0 && S(1, 2) == 0.0 && S(2, 0) == 0.0 && S(2, 1) == 0.0) {
        o[0] = 1.0 / S(0, 0);
        o[4] = 1.0 / S(1, 1);
        o[8] = 1.0 / S(2, 2);
        return;
    }
    cd det = S(0, 0) * S(1, 1) * S(2, 2) - S(0, 0) * S(1, 2) * S(2, 1) - S(0, 1) * S(1, 0) * S(2, 2) +
             S(0, 1) * S(1, 2) * S(2, 0) + S(0, 2) * S(1, 0) * S(2, 1) - S(0, 2) * S(1, 1) * S(2, 0);
    o[0] = S(1, 1) * S(2, 2) - S(1, 2) * S(2, 1);
    o[1] = -S(0, 1) * S(2, 2) + S(0, 2) * S(2, 1);
    o[2] = S(0, 1) * S(1, 2) - S(0, 2) * S(1, 1);
    o[3] = -S(1, 0) * S(2, 2) + S(1, 2) * S(2, 0);
    o[4] = S(0, 0) * S(2, 2) - S(0, 2) * S(2, 0);
    o[5] = -S(0, 0) * S(1, 2) + S(0, 2) * S(1, 0);
    o[6] = S(1, 0) * S(2, 1) - S(1, 1) * S(2, 0);
    o[7] = -S(0, 0) * S(2, 1) + S(0, 1) * S(2, 0);
    o[8] = S(0, 0) * S(1, 1) - S(0, 1) * S(1, 0);
    for (int i = 0; i < 9; ++i) o[i] *= det;
}

}  // extern "C"

namespace {

struct Vec3 { cd v[3]; };

inline Vec3 cross3(const Vec3& a, const Vec3& b) {
    return {{a.v[1] * b.v[2] - a.v[2] * b.v[1], a.v[2] * b.v[0] - a.v[0] * b.v[2], a.v[0] * b.v[1] - a.v[1] * b.v[0]}};
}
inline cd dot3(const Vec3& a, const Vec3& b) { return a.v[0] * b.v[0] + a.v[1] * b.v[1] + a.v[2] * b.v[2]; }
inline Vec3 mul3(const cd* M, const Vec3& a) {
    return {{M[0] * a.v[0] + M[1] * a.v[1] + M[2] * a.v[2], M[3] * a.v[0] + M[4] * a.v[1] + M[5] * a.v[2],
             M[6] * a.v[0] + M[7] * a.v[1] + M[8] * a.v[2]}};
}

// Volume-coefficient table indexed by vertex letters 0..4 (0 = absent).
struct VTable {
    double t[5][5][5][5];
    VTable() {
        for (int a = 0; a < 5; ++a) for (int b = 0; b < 5; ++b) for (int c = 0; c < 5; ++c) for (int d = 0; d < 5; ++d)
            t[a][b][c][d] = orc_volume_coeff(a, b, c, d);
    }
};
const VTable& vtable() { static VTable v; return v; }

}  // namespace

extern "C" {

// ned2_tet_stiff_mass (fem/mth/tet.py:854-1088).
//   verts (3,4) row-major x/y/z; edge_lengths (6); lem (2,6); ltm (3,4);
//   Ms, Mm (3,3) complex, row-major, interleaved re/im.
//   D, F: (20,20) complex row-major, interleaved.
void orc_tet_stiff_mass(const double* verts, const double* edge_lengths, const int64_t* lem, const int64_t* ltm,
                        const double* Ms_ri, const double* Mm_ri, double* D_ri, double* F_ri) {
    const cd* Ms = reinterpret_cast<const cd*>(Ms_ri);
    const cd* Mm = reinterpret_cast<const cd*>(Mm_ri);
    cd* D = reinterpret_cast<cd*>(D_ri);
    cd* F = reinterpret_cast<cd*>(F_ri);
    const double* xs = verts;
    const double* ys = verts + 4;
    const double* zs = verts + 8;
    double b[4], c[4], d[4], V;
    orc_tet_coefficients_bcd(xs, ys, zs, b, c, d, &V);
    double Ds[16];
    orc_compute_distances(xs, ys, zs, 4, Ds);
    Vec3 G[4];
    for (int i = 0; i < 4; ++i) G[i] = {{b[i], c[i], d[i]}};
    const double V6 = 6 * V;
    const double KA = 1.0 / std::pow(V6, 4);
    const double KB = 1.0 / std::pow(V6, 2);
    const auto& T = vtable().t;
    // vc(letters): volume coefficient scaled by 6V; letters are local vertex index + 1.
    auto vc = [&](int a, int bb, int cc, int dd) { return T[a][bb][cc][dd] * V6; };
    auto g = [&](int p, int q) { return dot3(G[p - 1], mul3(Mm, G[q - 1])); };       // G_p . Mm G_q
    auto cc = [&](int p, int q, int r, int s) {                                       // (G_p x G_q) . Ms (G_r x G_s)
        return dot3(cross3(G[p - 1], G[q - 1]), mul3(Ms, cross3(G[r - 1], G[s - 1])));
    };
    auto at = [&](cd* M, int r, int col) -> cd& { return M[r * 20 + col]; };

    for (int ei = 0; ei < 6; ++ei) {
        const int A = lem[ei] + 1, B = lem[6 + ei] + 1;
        const double L1 = edge_lengths[ei];
        for (int ej = 0; ej < 6; ++ej) {
            const int C = lem[ej] + 1, Dl = lem[6 + ej] + 1;
            const double L2 = edge_lengths[ej];
            const double Q2 = L1 * L2;
            const cd Q = Q2 * 9.0 * cc(A, B, C, Dl);
            at(D, ei, ej) = Q * vc(A, C, 0, 0);
            at(D, ei, ej + 10) = Q * vc(A, Dl, 0, 0);
            at(D, ei + 10, ej) = Q * vc(B, C, 0, 0);
            at(D, ei + 10, ej + 10) = Q * vc(B, Dl, 0, 0);
            const cd gAC = g(A, C), gAD = g(A, Dl), gBC = g(B, C), gBD = g(B, Dl);
            at(F, ei, ej) = Q2 * (vc(A, B, C, Dl) * gAC - vc(A, B, C, C) * gAD - vc(A, A, C, Dl) * gBC + vc(A, A, C, C) * gBD);
            at(F, ei, ej + 10) = Q2 * (vc(A, B, Dl, Dl) * gAC - vc(A, B, C, Dl) * gAD - vc(A, A, Dl, Dl) * gBC + vc(A, A, C, Dl) * gBD);
            at(F, ei + 10, ej) = Q2 * (vc(B, B, C, Dl) * gAC - vc(B, B, C, C) * gAD - vc(A, B, C, Dl) * gBC + vc(A, B, C, C) * gBD);
            at(F, ei + 10, ej + 10) = Q2 * (vc(B, B, Dl, Dl) * gAC - vc(B, B, C, Dl) * gAD - vc(A, B, Dl, Dl) * gBC + vc(A, B, C, Dl) * gBD);
        }
        for (int ej = 0; ej < 4; ++ej) {
            const int j1 = ltm[ej], j2 = ltm[4 + ej], jf = ltm[8 + ej];
            const int C = j1 + 1, Dl = j2 + 1, Fl = jf + 1;
            const double Lab2 = Ds[j1 * 4 + j2], Lac2 = Ds[j1 * 4 + jf];
            const cd AI = cc(A, B, C, Fl), AJ = cc(A, B, Dl, Fl), AK = cc(A, B, C, Dl);
            const cd gAF = g(A, Fl), gAC = g(A, C), gBF = g(B, Fl), gBC = g(B, C), gAD = g(A, Dl), gBD = g(B, Dl);
            at(D, ei, ej + 6) = L1 * Lac2 * (-6.0 * vc(A, Dl, 0, 0) * AI - 3.0 * vc(A, C, 0, 0) * AJ - 3.0 * vc(A, Fl, 0, 0) * AK);
            at(D, ei, ej + 16) = L1 * Lab2 * (6.0 * vc(A, Fl, 0, 0) * AK + 3.0 * vc(A, Dl, 0, 0) * AI - 3.0 * vc(A, C, 0, 0) * AJ);
            at(D, ei + 10, ej + 6) = L1 * Lac2 * (-6.0 * vc(B, Dl, 0, 0) * AI - 3.0 * vc(B, C, 0, 0) * AJ - 3.0 * vc(B, Fl, 0, 0) * AK);
            at(D, ei + 10, ej + 16) = L1 * Lab2 * (6.0 * vc(B, Fl, 0, 0) * AK + 3.0 * vc(B, Dl, 0, 0) * AI - 3.0 * vc(B, C, 0, 0) * AJ);
            at(F, ei, ej + 6) = L1 * Lac2 * (vc(A, B, C, Dl) * gAF - vc(A, B, Dl, Fl) * gAC - vc(A, A, C, Dl) * gBF + vc(A, A, Dl, Fl) * gBC);
            at(F, ei, ej + 16) = L1 * Lab2 * (vc(A, B, Dl, Fl) * gAC - vc(A, B, Fl, C) * gAD - vc(A, A, Dl, Fl) * gBC + vc(A, A, C, Fl) * gBD);
            at(F, ei + 10, ej + 6) = L1 * Lac2 * (vc(B, B, C, Dl) * gAF - vc(B, B, Dl, Fl) * gAC - vc(A, B, C, Dl) * gBF + vc(A, B, Dl, Fl) * gBC);
            at(F, ei + 10, ej + 16) = L1 * Lab2 * (vc(B, B, Dl, Fl) * gAC - vc(B, B, Fl, C) * gAD - vc(A, B, Dl, Fl) * gBC + vc(A, B, Fl, C) * gBD);
        }
    }
    // face rows x edge columns are the transposes of the edge x face blocks
    for (int M = 0; M < 2; ++M) {
        cd* X = M ? F : D;
        for (int f = 0; f < 4; ++f)
            for (int e = 0; e < 6; ++e) {
                at(X, 6 + f, e) = at(X, e, 6 + f);
                at(X, 16 + f, e) = at(X, e, 16 + f);
                at(X, 6 + f, 10 + e) = at(X, 10 + e, 6 + f);
                at(X, 16 + f, 10 + e) = at(X, 10 + e, 16 + f);
            }
    }
    for (int ei = 0; ei < 4; ++ei) {
        const int i1 = ltm[ei], i2 = ltm[4 + ei], fi = ltm[8 + ei];
        const int A = i1 + 1, B = i2 + 1, E = fi + 1;
        const double Lac1 = Ds[i1 * 4 + fi], Lab1 = Ds[i1 * 4 + i2];
        for (int ej = 0; ej < 4; ++ej) {
            const int j1 = ltm[ej], j2 = ltm[4 + ej], jf = ltm[8 + ej];
            const int C = j1 + 1, Dl = j2 + 1, Fl = jf + 1;
            const double Lac2 = Ds[j1 * 4 + jf], Lab2 = Ds[j1 * 4 + j2];
            const cd AK = cc(A, E, C, Fl), AL = cc(A, E, Dl, Fl), AM = cc(A, E, C, Dl);
            const cd AN = cc(B, E, C, Fl), AO = cc(B, E, Dl, Fl), AP = cc(B, E, C, Dl);
            const cd AQ = cc(A, B, C, Fl), AR = cc(A, B, Dl, Fl), AS = cc(A, B, C, Dl);
            const cd gEF = g(E, Fl), gEC = g(E, C), gAF = g(A, Fl), gAC = g(A, C), gED = g(E, Dl);
            const cd gAD = g(A, Dl), gBF = g(B, Fl), gBC = g(B, C), gBD = g(B, Dl);
            const double vAD = vc(A, Dl, 0, 0), vAC = vc(A, C, 0, 0), vAF = vc(A, Fl, 0, 0);
            const double vBF = vc(B, Fl, 0, 0), vBC = vc(B, C, 0, 0), vBD = vc(B, Dl, 0, 0);
            const double vDE = vc(E, Dl, 0, 0), vEF = vc(E, Fl, 0, 0), vCE = vc(E, C, 0, 0);
            // four-letter coefficients; the second one of the F[6+i][6+j] row pairs the
            // row face's B with (C, D, F) exactly as the reference does
            const double vABCD = vc(A, B, C, Dl), vABDF = vc(A, B, Dl, Fl), vACEF = vc(A, C, E, Fl);
            const double vABCF = vc(A, B, Fl, C), vBCDX = vc(B, C, Dl, Fl), vBDEF = vc(B, E, Dl, Fl);
            const double vACDE = vc(E, A, C, Dl), vBCEF = vc(B, E, Fl, C), vADEF = vc(E, A, Dl, Fl);
            const cd Q1 = 2.0 * vAD * AN + vAC * AO + vAF * AP;
            const cd Q2 = -2.0 * vAF * AP - vAD * AN + vAC * AO;
            at(D, 6 + ei, 6 + ej) = Lac1 * Lac2 * (4.0 * vBD * AK + 2.0 * vBC * AL + 2.0 * vBF * AM + Q1 + 2.0 * vDE * AQ + vCE * AR + vEF * AS);
            at(D, 6 + ei, 16 + ej) = Lac1 * Lab2 * (-4.0 * vBF * AM - 2.0 * vBD * AK + 2.0 * vBC * AL + Q2 - 2.0 * vEF * AS - vDE * AQ + vCE * AR);
            at(D, 16 + ei, 6 + ej) = Lab1 * Lac2 * (-4.0 * vDE * AQ - 2.0 * vCE * AR - 2.0 * vEF * AS - 2.0 * vBD * AK - vBC * AL - vBF * AM + Q1);
            at(D, 16 + ei, 16 + ej) = Lab1 * Lab2 * (4.0 * vEF * AS + 2.0 * vDE * AQ - 2.0 * vCE * AR + 2.0 * vBF * AM + vBD * AK - vBC * AL + Q2);
            at(F, 6 + ei, 6 + ej) = Lac1 * Lac2 * (vABCD * gEF - vABDF * gEC - vBCDX * gAF + vBDEF * gAC);
            at(F, 6 + ei, 16 + ej) = Lac1 * Lab2 * (vABDF * gEC - vABCF * gED - vBDEF * gAC + vBCEF * gAD);
            at(F, 16 + ei, 6 + ej) = Lab1 * Lac2 * (vBCDX * gAF - vBDEF * gAC - vACDE * gBF + vADEF * gBC);
            at(F, 16 + ei, 16 + ej) = Lab1 * Lab2 * (vBDEF * gAC - vBCEF * gAD - vADEF * gBC + vACEF * gBD);
        }
    }
    for (int i = 0; i < 400; ++i) { D[i] *= KA; F[i] *= KB; }
}

// _matrix_builder (fem/physics/edm/optimized_assembly.py:76-116) for tets [t0, t1):
// COO triplets for the curl-curl (E) and mass (B) matrices, 400 per tet, written at
// offset 400*(t - t0).  Array layouts are the reference's (numpy C order):
//   nodes (3,nN) f8; tets (4,nT); tris (3,nTri); edges (2,nE); tet_to_field (20,nT);
//   tet_to_edge (6,nT) all int64; ur, er (3,3,nT) complex interleaved.
void orc_matrix_builder(const double* nodes, int64_t nN, const int64_t* tets, int64_t nT, const int64_t* tris,
                        int64_t nTri, const int64_t* edges, int64_t nE, const double* edge_lengths,
                        const int64_t* tet_to_field, const int64_t* tet_to_edge, const double* ur, const double* er,
                        int64_t t0, int64_t t1, double* dataE, double* dataB, int64_t* rows, int64_t* cols) {
#pragma omp parallel for schedule(static)
    for (int64_t t = t0; t < t1; ++t) {
        const int64_t p = (t - t0) * 400;
        int64_t vid[4];
        double verts[12];
        for (int k = 0; k < 4; ++k) {
            vid[k] = tets[k * nT + t];
            for (int a = 0; a < 3; ++a) verts[a * 4 + k] = nodes[a * nN + vid[k]];
        }
        int64_t gtri[12], gedge[12], ltm[12], lem[12];
        for (int f = 0; f < 4; ++f) {
            const int64_t tri = tet_to_field[(6 + f) * nT + t] - nE;
            for (int j = 0; j < 3; ++j) gtri[j * 4 + f] = tris[j * nTri + tri];
        }
        for (int e = 0; e < 6; ++e) {
            const int64_t ed = tet_to_field[e * nT + t];
            for (int j = 0; j < 2; ++j) gedge[j * 6 + e] = edges[j * nE + ed];
        }
        orc_local_mapping(vid, gtri, 3, 4, ltm);
        orc_local_mapping(vid, gedge, 2, 6, lem);
        double el[6];
        for (int e = 0; e < 6; ++e) el[e] = edge_lengths[tet_to_edge[e * nT + t]];
        double urt[18], ert[18], Ms[18];
        for (int i = 0; i < 9; ++i) {
            urt[2 * i] = ur[2 * (i * nT + t)]; urt[2 * i + 1] = ur[2 * (i * nT + t) + 1];
            ert[2 * i] = er[2 * (i * nT + t)]; ert[2 * i + 1] = er[2 * (i * nT + t) + 1];
        }
        orc_matinv(urt, Ms);
        orc_tet_stiff_mass(verts, el, lem, ltm, Ms, ert, dataE + 2 * p, dataB + 2 * p);
        for (int ii = 0; ii < 20; ++ii) {
            const int64_t idx = tet_to_field[ii * nT + t];
            for (int jj = 0; jj < 20; ++jj) {
                rows[p + 20 * ii + jj] = idx;
                cols[p + ii + 20 * jj] = idx;
            }
        }
    }
}

}  // extern "C"

// ------------------------------------------------------------ surface terms ---

namespace {

struct ATable {
    double t[5][5][5][5];
    ATable() {
        for (int a = 0; a < 5; ++a) for (int b = 0; b < 5; ++b) for (int c = 0; c < 5; ++c) for (int d = 0; d < 5; ++d)
            t[a][b][c][d] = orc_area_coeff(a, b, c, d);
    }
};
const ATable& atable() { static ATable v; return v; }

inline double dot2(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1]; }

// The 8x8 Robin block shared by ned2_tri_stiff_force and ned2_tri_stiff.  ``Lij`` gives
// the edge length of local edge e (0..2); face lengths Lt1 = |v2 - v0|, Lt2 = |v1 - v0|.
// When ``coef_inside`` the per-entry factor multiplies each term (tri_stiff), otherwise
// the whole matrix is scaled afterwards (tri_stiff_force); both are restated.
void robin_block(const double (*GL)[2], const double* Le, double Lt1, double Lt2, double Area, cd coef,
                 bool coef_inside, cd* Bm) {
    static const int lem[2][3] = {{0, 1, 0}, {1, 2, 2}};
    const auto& T = atable().t;
    auto ac = [&](int a, int b, int c, int d) { return T[a][b][c][d] * Area; };
    const cd K = coef_inside ? coef : cd(1.0);
    auto at = [&](int r, int c) -> cd& { return Bm[r * 8 + c]; };
    const int tA = 1, tB = 2, tC = 3;
    const double *GtA = GL[0], *GtB = GL[1], *GtC = GL[2];
    for (int ei = 0; ei < 3; ++ei) {
        const int i1 = lem[0][ei], i2 = lem[1][ei];
        const double Li = Le[ei];
        const int A = i1 + 1, B = i2 + 1;
        const double *GA = GL[i1], *GB = GL[i2];
        for (int ej = 0; ej < 3; ++ej) {
            const int j1 = lem[0][ej], j2 = lem[1][ej];
            const double Lj = Le[ej];
            const int C = j1 + 1, D = j2 + 1;
            const double *GC = GL[j1], *GD = GL[j2];
            const double aC = dot2(GA, GC), aD = dot2(GA, GD), bC = dot2(GB, GC), bD = dot2(GB, GD);
            at(ei, ej) += Li * Lj * K * (ac(A, B, C, D) * aC - ac(A, B, C, C) * aD - ac(A, A, C, D) * bC + ac(A, A, C, C) * bD);
            at(ei, ej + 4) += Li * Lj * K * (ac(A, B, D, D) * aC - ac(A, B, C, D) * aD - ac(A, A, D, D) * bC + ac(A, A, C, D) * bD);
            at(ei + 4, ej) += Li * Lj * K * (ac(B, B, C, D) * aC - ac(B, B, C, C) * aD - ac(A, B, C, D) * bC + ac(A, B, C, C) * bD);
            at(ei + 4, ej + 4) += Li * Lj * K * (ac(B, B, D, D) * aC - ac(B, B, C, D) * aD - ac(A, B, D, D) * bC + ac(A, B, C, D) * bD);
        }
        const double aC = dot2(GA, GtC), aA = dot2(GA, GtA), bC = dot2(GB, GtC), bA = dot2(GB, GtA);
        const double aB = dot2(GA, GtB), bB = dot2(GB, GtB);
        at(ei, 3) += Li * Lt1 * K * (ac(A, B, tA, tB) * aC - ac(A, B, tB, tC) * aA - ac(A, A, tA, tB) * bC + ac(A, A, tB, tC) * bA);
        at(ei, 7) += Li * Lt2 * K * (ac(A, B, tB, tC) * aA - ac(A, B, tC, tA) * aB - ac(A, A, tB, tC) * bA + ac(A, A, tC, tA) * bB);
        at(3, ei) += Lt1 * Li * K * (ac(tA, tB, A, B) * aC - ac(tA, tB, A, A) * bC - ac(tB, tC, A, B) * aA + ac(tB, tC, A, A) * bA);
        at(7, ei) += Lt2 * Li * K * (ac(tB, tC, A, B) * aA - ac(tB, tC, A, A) * bA - ac(tC, tA, A, B) * aB + ac(tC, tA, A, A) * bB);
        at(ei + 4, 3) += Li * Lt1 * K * (ac(B, B, tA, tB) * aC - ac(B, B, tB, tC) * aA - ac(A, B, tA, tB) * bC + ac(A, B, tB, tC) * bA);
        at(ei + 4, 7) += Li * Lt2 * K * (ac(B, B, tB, tC) * aA - ac(B, B, tC, tA) * aB - ac(A, B, tB, tC) * bA + ac(A, B, tC, tA) * bB);
        at(3, ei + 4) += Lt1 * Li * K * (ac(tA, tB, B, B) * aC - ac(tA, tB, A, B) * bC - ac(tB, tC, B, B) * aA + ac(tB, tC, A, B) * bA);
        at(7, ei + 4) += Lt2 * Li * K * (ac(tB, tC, B, B) * aA - ac(tB, tC, A, B) * bA - ac(tC, tA, B, B) * aB + ac(tC, tA, A, B) * bB);
    }
    const double CC = dot2(GtC, GtC), AC = dot2(GtA, GtC), AA = dot2(GtA, GtA), BC = dot2(GtB, GtC);
    const double AB = dot2(GtA, GtB), BB = dot2(GtB, GtB);
    at(3, 3) += Lt1 * Lt1 * K * (ac(tA, tB, tA, tB) * CC - ac(tA, tB, tB, tC) * AC - ac(tB, tC, tA, tB) * AC + ac(tB, tC, tB, tC) * AA);
    at(3, 7) += Lt1 * Lt2 * K * (ac(tA, tB, tB, tC) * AC - ac(tA, tB, tC, tA) * BC - ac(tB, tC, tB, tC) * AA + ac(tB, tC, tC, tA) * AB);
    at(7, 3) += Lt2 * Lt1 * K * (ac(tB, tC, tA, tB) * AC - ac(tB, tC, tB, tC) * AA - ac(tC, tA, tA, tB) * BC + ac(tC, tA, tB, tC) * AB);
    at(7, 7) += Lt2 * Lt2 * K * (ac(tB, tC, tB, tC) * AA - ac(tB, tC, tC, tA) * AB - ac(tC, tA, tB, tC) * AB + ac(tC, tA, tC, tA) * BB);
}

}  // namespace

extern "C" {

// ned2_tri_stiff_force (fem/mth/tri.py:575-695).  lcs (>=2,3) row-major (x row, y row);
// Uinc (3,npts) complex; DPTs (4,npts) weights + barycentrics.  B (8,8), bvec (8) complex.
void orc_tri_stiff_force(const double* lcs, double gamma_re, double gamma_im, const double* Uinc_ri,
                         const double* DPTs, int npts, double* B_ri, double* b_ri) {
    const cd gamma(gamma_re, gamma_im);
    const cd* U = reinterpret_cast<const cd*>(Uinc_ri);
    cd* Bm = reinterpret_cast<cd*>(B_ri);
    cd* bv = reinterpret_cast<cd*>(b_ri);
    for (int i = 0; i < 64; ++i) Bm[i] = 0.0;
    for (int i = 0; i < 8; ++i) bv[i] = 0.0;
    const double x1 = lcs[0], x2 = lcs[1], x3 = lcs[2];
    const double y1 = lcs[3], y2 = lcs[4], y3 = lcs[5];
    const double As[3] = {x2 * y3 - y2 * x3, x3 * y1 - y3 * x1, x1 * y2 - y1 * x2};
    const double Bs[3] = {y2 - y3, y3 - y1, y1 - y2};
    const double Cs[3] = {x3 - x2, x1 - x3, x2 - x1};
    const double zz[3] = {0, 0, 0};
    double Ds[9];
    orc_compute_distances(lcs, lcs + 3, zz, 3, Ds);
    const double GL[3][2] = {{Bs[0], Cs[0]}, {Bs[1], Cs[1]}, {Bs[2], Cs[2]}};
    const double det = (x1 - x3) * (y2 - y1) - (x1 - x2) * (y3 - y1);
    const double Area = 0.5 * std::fabs(det);
    const double signA = det > 0 ? -1.0 : (det < 0 ? 1.0 : 0.0);
    const double Lt1 = Ds[2 * 3 + 0], Lt2 = Ds[1 * 3 + 0];
    static const int lem[2][3] = {{0, 1, 0}, {1, 2, 2}};
    const double Le[3] = {Ds[lem[0][0] * 3 + lem[1][0]], Ds[lem[0][1] * 3 + lem[1][1]], Ds[lem[0][2] * 3 + lem[1][2]]};
    robin_block(GL, Le, Lt1, Lt2, Area, gamma, false, Bm);
    // forcing vector: 6-point quadrature of N_i . U_inc (tri.py:668-693)
    const double A2 = Area * Area, A3 = Area * Area * Area;
    for (int ei = 0; ei < 3; ++ei) {
        const int i1 = lem[0][ei], i2 = lem[1][ei];
        const double Li = Ds[i1 * 3 + i2];
        const double a1 = As[i1], a2 = As[i2], b1 = Bs[i1], b2 = Bs[i2], c1 = Cs[i1], c2 = Cs[i2];
        cd s1 = 0.0, s2 = 0.0;
        for (int k = 0; k < npts; ++k) {
            const double x = x1 * DPTs[npts + k] + x2 * DPTs[2 * npts + k] + x3 * DPTs[3 * npts + k];
            const double y = y1 * DPTs[npts + k] + y2 * DPTs[2 * npts + k] + y3 * DPTs[3 * npts + k];
            const double l1 = a1 + b1 * x + c1 * y, l2 = a2 + b2 * x + c2 * y;
            const double wx = b1 * l2 / (4 * A2) - b2 * l1 / (4 * A2);
            const double wy = c1 * l2 / (4 * A2) - c2 * l1 / (4 * A2);
            const double e1x = Li * wx * l1 / (2 * Area), e1y = Li * wy * l1 / (2 * Area);
            const double e2x = Li * wx * l2 / (2 * Area), e2y = Li * wy * l2 / (2 * Area);
            const double W = DPTs[k];
            s1 += W * (e1x * U[k] + e1y * U[npts + k]);
            s2 += W * (e2x * U[k] + e2y * U[npts + k]);
        }
        bv[ei] += signA * Area * s1;
        bv[ei + 4] += signA * Area * s2;
    }
    {
        cd s3 = 0.0, s7 = 0.0;
        for (int k = 0; k < npts; ++k) {
            const double x = x1 * DPTs[npts + k] + x2 * DPTs[2 * npts + k] + x3 * DPTs[3 * npts + k];
            const double y = y1 * DPTs[npts + k] + y2 * DPTs[2 * npts + k] + y3 * DPTs[3 * npts + k];
            const double l1 = As[0] + Bs[0] * x + Cs[0] * y, l2 = As[1] + Bs[1] * x + Cs[1] * y;
            const double l3 = As[2] + Bs[2] * x + Cs[2] * y;
            const double f1x = Lt1 * (-Bs[0] * l2 * l3 / (8 * A3) + Bs[2] * l1 * l2 / (8 * A3));
            const double f1y = Lt1 * (-Cs[0] * l2 * l3 / (8 * A3) + Cs[2] * l1 * l2 / (8 * A3));
            const double f2x = Lt2 * (Bs[0] * l2 * l3 / (8 * A3) - Bs[1] * l1 * l3 / (8 * A3));
            const double f2y = Lt2 * (Cs[0] * l2 * l3 / (8 * A3) - Cs[1] * l1 * l3 / (8 * A3));
            const double W = DPTs[k];
            s3 += W * (f1x * U[k] + f1y * U[npts + k]);
            s7 += W * (f2x * U[k] + f2y * U[npts + k]);
        }
        bv[3] += signA * Area * s3;
        bv[7] += signA * Area * s7;
    }
    const cd COEFF = gamma / ((2 * Area) * (2 * Area));
    for (int i = 0; i < 64; ++i) Bm[i] *= COEFF;
}

// ned2_tri_stiff (fem/mth/tri.py:697-797): ABC Robin matrix of a 3-D triangle.
// vertices (3,3) row-major (x row, y row, z row); edge_lengths (3).
void orc_tri_stiff(const double* v, const double* edge_lengths, double gamma_re, double gamma_im, double* B_ri) {
    const cd gamma(gamma_re, gamma_im);
    cd* Bm = reinterpret_cast<cd*>(B_ri);
    for (int i = 0; i < 64; ++i) Bm[i] = 0.0;
    // local frame: ax1 along v1-v0, normal = ax1 x ax2n, ax2 = -(n x ax1)
    double ax1[3] = {v[1] - v[0], v[4] - v[3], v[7] - v[6]};
    double ax2[3] = {v[2] - v[0], v[5] - v[3], v[8] - v[6]};
    const double n1 = std::sqrt(ax1[0] * ax1[0] + ax1[1] * ax1[1] + ax1[2] * ax1[2]);
    const double n2 = std::sqrt(ax2[0] * ax2[0] + ax2[1] * ax2[1] + ax2[2] * ax2[2]);
    for (int i = 0; i < 3; ++i) { ax1[i] /= n1; ax2[i] /= n2; }
    const double axn[3] = {ax1[1] * ax2[2] - ax1[2] * ax2[1], ax1[2] * ax2[0] - ax1[0] * ax2[2], ax1[0] * ax2[1] - ax1[1] * ax2[0]};
    const double t2[3] = {axn[1] * ax1[2] - axn[2] * ax1[1], axn[2] * ax1[0] - axn[0] * ax1[2], axn[0] * ax1[1] - axn[1] * ax1[0]};
    // basis columns (ax1, -t2, axn); the reference inverts it with pinv, which for
    // this (orthogonal up to the non-unit normal) matrix is the exact inverse
    double M[9] = {ax1[0], -t2[0], axn[0], ax1[1], -t2[1], axn[1], ax1[2], -t2[2], axn[2]};
    // invert 3x3 (general)
    const double det = M[0] * (M[4] * M[8] - M[5] * M[7]) - M[1] * (M[3] * M[8] - M[5] * M[6]) + M[2] * (M[3] * M[7] - M[4] * M[6]);
    double Mi[9] = {(M[4] * M[8] - M[5] * M[7]) / det, (M[2] * M[7] - M[1] * M[8]) / det, (M[1] * M[5] - M[2] * M[4]) / det,
                    (M[5] * M[6] - M[3] * M[8]) / det, (M[0] * M[8] - M[2] * M[6]) / det, (M[2] * M[3] - M[0] * M[5]) / det,
                    (M[3] * M[7] - M[4] * M[6]) / det, (M[1] * M[6] - M[0] * M[7]) / det, (M[0] * M[4] - M[1] * M[3]) / det};
    double xs[3], ys[3];
    for (int k = 0; k < 3; ++k) {
        xs[k] = Mi[0] * v[k] + Mi[1] * v[3 + k] + Mi[2] * v[6 + k];
        ys[k] = Mi[3] * v[k] + Mi[4] * v[3 + k] + Mi[5] * v[6 + k];
    }
    const double x1 = xs[0], x2 = xs[1], x3 = xs[2], y1 = ys[0], y2 = ys[1], y3 = ys[2];
    const double GL[3][2] = {{y2 - y3, x3 - x2}, {y3 - y1, x1 - x3}, {y1 - y2, x2 - x1}};
    const double zz[3] = {0, 0, 0};
    double Ds[9];
    orc_compute_distances(xs, ys, zz, 3, Ds);
    const double Area = 0.5 * std::fabs((x1 - x3) * (y2 - y1) - (x1 - x2) * (y3 - y1));
    const double Lt1 = Ds[2 * 3 + 0], Lt2 = Ds[1 * 3 + 0];
    const cd COEFF = gamma / ((2 * Area) * (2 * Area));
    robin_block(GL, edge_lengths, Lt1, Lt2, Area, COEFF, true, Bm);
}

}  // extern "C"
