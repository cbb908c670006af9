// Float-float (pairs of FP32) assembly fill for GB300.
//
// GB300 executes FP64 at ~1/64 of its FP32 rate (1.2 vs 75 TFLOP/s measured),
// so a straight FP64 element integration is compute-bound an order of magnitude
// above the HBM floor of the write-once CSR fill.  This fill evaluates the
// closed-form Nedelec-2 element blocks (fem/mth/tet.py:854-1088) in float-float
// arithmetic (~48-bit significand, error-free products via FMA) on the FP32
// pipes, accumulates each CSR entry in float-float in a fixed order, and
// converts to FP64 with integer instructions when storing.  FP64 is used only
// once per tet: for the geometry (plan) and the material scales (per fill).
//
// Work decomposition (entity-owner, as in emg_assembly.cu):
//  * a warp owns one edge entity, or two face entities (rows r1/r2 each);
//  * phase A computes the 2x2 blocks (row entity x edge column) of every
//    incident tet, phase B the blocks with face columns; all lanes of a phase
//    run the same block formula (no divergence), results staged in shared memory;
//  * the owner phase: lane p sums, in ascending tet order, the staged entries
//    that land on column position p of the entity's rows, scales them by the
//    tet's complex material factors, and writes E and B once, coalesced.
#include "emg_common.cuh"
#include "emg_fill_df.cuh"
#include "emg_geom.cuh"

namespace emg {
namespace dfk {

struct df {
    float h, l;
};
__device__ __forceinline__ df mk(float h, float l) {
    df r;
    r.h = h;
    r.l = l;
    return r;
}
// fast two-sum (|a| >= |b| or a == 0)
__device__ __forceinline__ df fts(float a, float b) {
    const float s = __fadd_rn(a, b);
    return mk(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ df two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return mk(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}
__device__ __forceinline__ df operator+(df a, df b) {
    const df s = two_sum(a.h, b.h);
    return fts(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ df operator-(df a) { return mk(-a.h, -a.l); }
__device__ __forceinline__ df operator-(df a, df b) { return a + (-b); }
__device__ __forceinline__ df operator*(df a, df b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return fts(p, e);
}
__device__ __forceinline__ df operator*(df a, float c) {
    const float p = __fmul_rn(a.h, c);
    float e = __fmaf_rn(a.h, c, -p);
    e = __fmaf_rn(a.l, c, e);
    return fts(p, e);
}
__device__ __forceinline__ df operator*(float c, df a) { return a * c; }

// hi + lo rounded (toward zero in the last bit) to FP64 with integer instructions
// only (no FP64 pipe).  Requires |lo| <= ulp(hi)/2 (every df op renormalises).
// Subnormal hi (|x| < 2^-126) is returned as a signed zero.
__device__ __forceinline__ double to_double(df a) {
    const unsigned hb = __float_as_uint(a.h);
    const unsigned eh = (hb >> 23) & 0xffu;
    const unsigned long long sign = (unsigned long long)(hb & 0x80000000u) << 32;
    if (eh == 0u) return __longlong_as_double((long long)sign);
    const unsigned long long mant = (unsigned long long)(hb & 0x7fffffu) << 29;
    if (eh == 0xffu) return __longlong_as_double((long long)(sign | 0x7ff0000000000000ull | mant));
    const unsigned long long bits = sign | ((unsigned long long)(eh + 896u) << 52) | mant;
    const unsigned lb = __float_as_uint(a.l);
    const unsigned el = (lb >> 23) & 0xffu;
    if (el == 0u) return __longlong_as_double((long long)bits);
    const long long m = (long long)((lb & 0x7fffffu) | 0x800000u);
    const bool opp = ((lb ^ hb) & 0x80000000u) != 0u;
    // position of lo's last mantissa bit in units of hi's FP64 ulp; one more when
    // subtracting from an exact power of two (the result is in the lower binade)
    const int sh = (int)el - (int)eh + 29 + ((opp && (hb & 0x7fffffu) == 0u) ? 1 : 0);
    const long long add = sh >= 0 ? (m << sh) : (sh > -40 ? (m >> -sh) : 0ll);
    return __longlong_as_double((long long)(opp ? bits - (unsigned long long)add : bits + (unsigned long long)add));
}

// Compensated accumulator: running float sum plus running error, renormalised once.
struct acc {
    float s, e;
};
__device__ __forceinline__ void acc_fma(acc& a, df x, df y) {   // a += x * y
    const float p = __fmul_rn(x.h, y.h);
    float pe = __fmaf_rn(x.h, y.h, -p);
    pe = __fmaf_rn(x.h, y.l, pe);
    pe = __fmaf_rn(x.l, y.h, pe);
    const float t = __fadd_rn(a.s, p);
    const float bb = __fsub_rn(t, a.s);
    const float err = __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, bb)), __fsub_rn(p, bb));
    a.s = t;
    a.e = __fadd_rn(a.e, __fadd_rn(err, pe));
}

__device__ __forceinline__ df split(double x) {
    const float h = __double2float_rn(x);
    return mk(h, __double2float_rn(x - (double)h));
}

// ---------------------------------------------------------------- records ---
// Normalised tet invariants in float-float: G_p scaled by 2^-eG, lengths by 2^-eL.
struct __align__(16) Rec2 {
    float2 gram[10];    // G_p . G_q (p <= q)
    float2 cdot[21];    // (G_a x G_b) . (G_c x G_d) over vertex pairs P <= R
    float2 ds[6];       // vertex distances, pair order (0,1),(0,2),(0,3),(1,2),(1,3),(2,3)
    float2 len[6];      // mesh edge lengths of edge slots
    uint64_t lmap;      // packed local edge / face vertex maps (as TetRec::lmap)
    int32_t dof[20];
    int32_t pad[2];
};
static_assert(sizeof(Rec2) == 448, "Rec2 layout");

__constant__ int8_t c_pidx[4][4] = {{-1, 0, 1, 2}, {0, -1, 3, 4}, {1, 3, -1, 5}, {2, 4, 5, -1}};
__constant__ int8_t c_gidx[4][4] = {{0, 1, 2, 3}, {1, 4, 5, 6}, {2, 5, 7, 8}, {3, 6, 8, 9}};
// simplex monomial integrals x 7! (exact small integers), letters 0..4, 0 = absent
__constant__ float c_vint[625];

__device__ __forceinline__ int cidx(int P, int R) {
    if (P > R) { const int t = P; P = R; R = t; }
    return P * 6 - (P * (P - 1)) / 2 + (R - P);
}

// Thread per tet (plan time, FP64): invariants normalised by powers of two and
// the FP64 scales that undo the normalisation, the 1/(6V)^k factors and the 7!.
__global__ void k_prep2(const double* __restrict__ nodes, int64_t nN, const int32_t* __restrict__ tets, int64_t nT,
                        const int32_t* __restrict__ edges, int64_t nE, const int32_t* __restrict__ tris, int64_t nTri,
                        const int32_t* __restrict__ t2f, const int32_t* __restrict__ t2e,
                        const double* __restrict__ edge_len, Rec2* __restrict__ recs, double2* __restrict__ gscale,
                        int* err) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nT; t += (int64_t)gridDim.x * blockDim.x) {
        int32_t vid[4];
        double x[4], y[4], z[4];
        for (int k = 0; k < 4; ++k) {
            vid[k] = tets[k * nT + t];
            x[k] = nodes[vid[k]];
            y[k] = nodes[nN + vid[k]];
            z[k] = nodes[2 * nN + vid[k]];
        }
        double G[4][3], V;
        geom::tet_bcd(x, y, z, G, &V);
        double gmax = 0.0;
        for (int i = 0; i < 4; ++i)
            for (int c = 0; c < 3; ++c) gmax = fmax(gmax, fabs(G[i][c]));
        const int eG = gmax > 0.0 ? ilogb(gmax) : 0;
        for (int i = 0; i < 4; ++i)
            for (int c = 0; c < 3; ++c) G[i][c] = scalbn(G[i][c], -eG);
        Rec2 r;
        for (int p = 0; p < 4; ++p)
            for (int q = p; q < 4; ++q) {
                const df v = split(G[p][0] * G[q][0] + G[p][1] * G[q][1] + G[p][2] * G[q][2]);
                r.gram[c_gidx[p][q]] = make_float2(v.h, v.l);
            }
        const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {1, 2, 3, 2, 3, 3};
        double X[6][3], dsv[6], lenv[6];
        double lmax = 0.0;
        for (int P = 0; P < 6; ++P) {
            const double* u = G[pa[P]];
            const double* v = G[pb[P]];
            X[P][0] = u[1] * v[2] - u[2] * v[1];
            X[P][1] = u[2] * v[0] - u[0] * v[2];
            X[P][2] = u[0] * v[1] - u[1] * v[0];
            const double dx = x[pa[P]] - x[pb[P]], dy = y[pa[P]] - y[pb[P]], dz = z[pa[P]] - z[pb[P]];
            dsv[P] = sqrt(dx * dx + dy * dy + dz * dz);
            lmax = fmax(lmax, dsv[P]);
        }
        for (int P = 0; P < 6; ++P)
            for (int R = P; R < 6; ++R) {
                const df v = split(X[P][0] * X[R][0] + X[P][1] * X[R][1] + X[P][2] * X[R][2]);
                r.cdot[cidx(P, R)] = make_float2(v.h, v.l);
            }
        uint64_t lm = 0;
        bool ok = true;
        for (int e = 0; e < 6; ++e) {
            lenv[e] = edge_len[t2e[e * nT + t]];
            lmax = fmax(lmax, lenv[e]);
            const int32_t eid = t2f[e * nT + t];
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
        if (!ok) atomicOr(err, 1);
        const int eL = lmax > 0.0 ? ilogb(lmax) : 0;
        for (int P = 0; P < 6; ++P) {
            const df a = split(scalbn(dsv[P], -eL));
            const df b = split(scalbn(lenv[P], -eL));
            r.ds[P] = make_float2(a.h, a.l);
            r.len[P] = make_float2(b.h, b.l);
        }
        r.lmap = lm;
        for (int k = 0; k < 20; ++k) r.dof[k] = t2f[k * nT + t];
        r.pad[0] = r.pad[1] = 0;
        recs[t] = r;
        const double V6 = 6.0 * V;
        const double V6sq = V6 * V6;
        const double kd = V6 * (1.0 / (V6sq * V6sq));
        const double kf = V6 * (1.0 / V6sq);
        // D entries scale as len^2 G^4, F entries as len^2 G^2; the integers carry 7!
        gscale[t] = make_double2(scalbn(kd, 4 * eG + 2 * eL) / 5040.0, scalbn(kf, 2 * eG + 2 * eL) / 5040.0);
    }
}

// Per fill (FP64, thread per tet): complex scales sE = mu_inv * gscale.x and
// sB = eps * gscale.y, stored as float-float (re.h, re.l, im.h, im.l).
// *complex_mu (when given) becomes 1 if any tet's mu^-1 has a nonzero imaginary part.
__global__ void k_scales(const double2* __restrict__ gscale, const double2* __restrict__ eps,
                         const double2* __restrict__ mu_inv, int64_t nT, float4* __restrict__ tscale,
                         int* __restrict__ complex_mu) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nT; t += (int64_t)gridDim.x * blockDim.x) {
        const double2 g = gscale[t], m = mu_inv[t], e = eps[t];
        const df a = split(m.x * g.x), b = split(m.y * g.x), c = split(e.x * g.y), d = split(e.y * g.y);
        tscale[2 * t] = make_float4(a.h, a.l, b.h, b.l);
        tscale[2 * t + 1] = make_float4(c.h, c.l, d.h, d.l);
        if (complex_mu && (b.h != 0.f || b.l != 0.f)) atomicOr(complex_mu, 1);
    }
}

// ------------------------------------------------------------- the blocks ---
struct Tet {
    const Rec2* r;
    __device__ __forceinline__ df g(int p, int q) const {
        const float2 v = r->gram[c_gidx[p][q]];
        return mk(v.x, v.y);
    }
    __device__ __forceinline__ df cc(int p, int q, int s1, int s2) const {
        if (p == q || s1 == s2) return mk(0.f, 0.f);
        const float2 v = r->cdot[cidx(c_pidx[p][q], c_pidx[s1][s2])];
        return ((p < q) == (s1 < s2)) ? mk(v.x, v.y) : mk(-v.x, -v.y);
    }
    __device__ __forceinline__ df ds(int p, int q) const {
        const float2 v = r->ds[c_pidx[p][q]];
        return mk(v.x, v.y);
    }
    __device__ __forceinline__ df len(int e) const {
        const float2 v = r->len[e];
        return mk(v.x, v.y);
    }
};

__device__ __forceinline__ float v4(const float* vt, int a, int b, int c, int d) {
    return vt[(((a + 1) * 5 + (b + 1)) * 5 + (c + 1)) * 5 + (d + 1)];
}
__device__ __forceinline__ float v2(const float* vt, int a, int b) { return vt[((a + 1) * 5 + (b + 1)) * 25]; }
__device__ __forceinline__ void ev(uint64_t m, int e, int& a, int& b) {
    a = (int)((m >> (4 * e)) & 3);
    b = (int)((m >> (4 * e + 2)) & 3);
}
__device__ __forceinline__ void fv(uint64_t m, int f, int& a, int& b, int& c) {
    a = (int)((m >> (24 + 6 * f)) & 3);
    b = (int)((m >> (24 + 6 * f + 2)) & 3);
    c = (int)((m >> (24 + 6 * f + 4)) & 3);
}

// Block outputs: D[a][b], F[a][b] (row mode a, column mode b), as in emg_assembly.cu.
// The letters are local vertex labels (edge e = (A,B), face = (C,D,F) in the order the
// reference orients them); ``X`` reads the tet's invariants by those labels.
template <class X>
__device__ __forceinline__ void blk_ee(const X& T, const float* vt, int A, int B, int e, int C, int Dl, int j,
                                       df D[2][2], df F[2][2]) {
    const df Q2 = T.len(e) * T.len(j);
    const df Q = (Q2 * T.cc(A, B, C, Dl)) * 9.0f;
    D[0][0] = Q * v2(vt, A, C);
    D[0][1] = Q * v2(vt, A, Dl);
    D[1][0] = Q * v2(vt, B, C);
    D[1][1] = Q * v2(vt, B, Dl);
    const df gAC = T.g(A, C), gAD = T.g(A, Dl), gBC = T.g(B, C), gBD = T.g(B, Dl);
    F[0][0] = Q2 * (gAC * v4(vt, A, B, C, Dl) - gAD * v4(vt, A, B, C, C) - gBC * v4(vt, A, A, C, Dl) + gBD * v4(vt, A, A, C, C));
    F[0][1] = Q2 * (gAC * v4(vt, A, B, Dl, Dl) - gAD * v4(vt, A, B, C, Dl) - gBC * v4(vt, A, A, Dl, Dl) + gBD * v4(vt, A, A, C, Dl));
    F[1][0] = Q2 * (gAC * v4(vt, B, B, C, Dl) - gAD * v4(vt, B, B, C, C) - gBC * v4(vt, A, B, C, Dl) + gBD * v4(vt, A, B, C, C));
    F[1][1] = Q2 * (gAC * v4(vt, B, B, Dl, Dl) - gAD * v4(vt, B, B, C, Dl) - gBC * v4(vt, A, B, Dl, Dl) + gBD * v4(vt, A, B, C, Dl));
}

template <class X>
__device__ __forceinline__ void blk_ef(const X& T, const float* vt, int A, int B, int e, int C, int Dl, int Fl,
                                       df D[2][2], df F[2][2]) {
    const df L1 = T.len(e);
    const df c0 = L1 * T.ds(C, Fl), c1 = L1 * T.ds(C, Dl);
    const df AI = T.cc(A, B, C, Fl), AJ = T.cc(A, B, Dl, Fl), AK = T.cc(A, B, C, Dl);
    D[0][0] = c0 * (AI * (-6.0f * v2(vt, A, Dl)) - AJ * (3.0f * v2(vt, A, C)) - AK * (3.0f * v2(vt, A, Fl)));
    D[0][1] = c1 * (AK * (6.0f * v2(vt, A, Fl)) + AI * (3.0f * v2(vt, A, Dl)) - AJ * (3.0f * v2(vt, A, C)));
    D[1][0] = c0 * (AI * (-6.0f * v2(vt, B, Dl)) - AJ * (3.0f * v2(vt, B, C)) - AK * (3.0f * v2(vt, B, Fl)));
    D[1][1] = c1 * (AK * (6.0f * v2(vt, B, Fl)) + AI * (3.0f * v2(vt, B, Dl)) - AJ * (3.0f * v2(vt, B, C)));
    const df gAF = T.g(A, Fl), gAC = T.g(A, C), gBF = T.g(B, Fl), gBC = T.g(B, C), gAD = T.g(A, Dl), gBD = T.g(B, Dl);
    F[0][0] = c0 * (gAF * v4(vt, A, B, C, Dl) - gAC * v4(vt, A, B, Dl, Fl) - gBF * v4(vt, A, A, C, Dl) + gBC * v4(vt, A, A, Dl, Fl));
    F[0][1] = c1 * (gAC * v4(vt, A, B, Dl, Fl) - gAD * v4(vt, A, B, Fl, C) - gBC * v4(vt, A, A, Dl, Fl) + gBD * v4(vt, A, A, C, Fl));
    F[1][0] = c0 * (gAF * v4(vt, B, B, C, Dl) - gAC * v4(vt, B, B, Dl, Fl) - gBF * v4(vt, A, B, C, Dl) + gBC * v4(vt, A, B, Dl, Fl));
    F[1][1] = c1 * (gAC * v4(vt, B, B, Dl, Fl) - gAD * v4(vt, B, B, Fl, C) - gBC * v4(vt, A, B, Dl, Fl) + gBD * v4(vt, A, B, Fl, C));
}

// Face-face block; with ``want_d`` false only F is formed (the lower face-face blocks,
// where D follows from symmetry but F does not).
template <class X>
__device__ __forceinline__ void blk_ff(const X& T, const float* vt, int A, int B, int E, int C, int Dl, int Fl,
                                       df D[2][2], df F[2][2], bool want_d = true) {
    const df Lac1 = T.ds(A, E), Lab1 = T.ds(A, B), Lac2 = T.ds(C, Fl), Lab2 = T.ds(C, Dl);
    if (want_d) {
        const df AK = T.cc(A, E, C, Fl), AL = T.cc(A, E, Dl, Fl), AM = T.cc(A, E, C, Dl);
        const df AN = T.cc(B, E, C, Fl), AO = T.cc(B, E, Dl, Fl), AP = T.cc(B, E, C, Dl);
        const df AQ = T.cc(A, B, C, Fl), AR = T.cc(A, B, Dl, Fl), AS = T.cc(A, B, C, Dl);
        const float vAD = v2(vt, A, Dl), vAC = v2(vt, A, C), vAF = v2(vt, A, Fl);
        const float vBF = v2(vt, B, Fl), vBC = v2(vt, B, C), vBD = v2(vt, B, Dl);
        const float vDE = v2(vt, E, Dl), vEF = v2(vt, E, Fl), vCE = v2(vt, E, C);
        const df Q1 = AN * (2.0f * vAD) + AO * vAC + AP * vAF;
        const df Q2 = AO * vAC - AP * (2.0f * vAF) - AN * vAD;
        D[0][0] = (Lac1 * Lac2) * (AK * (4.0f * vBD) + AL * (2.0f * vBC) + AM * (2.0f * vBF) + Q1 + AQ * (2.0f * vDE) + AR * vCE + AS * vEF);
        D[0][1] = (Lac1 * Lab2) * (AL * (2.0f * vBC) - AM * (4.0f * vBF) - AK * (2.0f * vBD) + Q2 - AS * (2.0f * vEF) - AQ * vDE + AR * vCE);
        D[1][0] = (Lab1 * Lac2) * (Q1 - AQ * (4.0f * vDE) - AR * (2.0f * vCE) - AS * (2.0f * vEF) - AK * (2.0f * vBD) - AL * vBC - AM * vBF);
        D[1][1] = (Lab1 * Lab2) * (AS * (4.0f * vEF) + AQ * (2.0f * vDE) - AR * (2.0f * vCE) + AM * (2.0f * vBF) + AK * vBD - AL * vBC + Q2);
    }
    const df gEF = T.g(E, Fl), gEC = T.g(E, C), gAF = T.g(A, Fl), gAC = T.g(A, C), gED = T.g(E, Dl);
    const df gAD = T.g(A, Dl), gBF = T.g(B, Fl), gBC = T.g(B, C), gBD = T.g(B, Dl);
    const float vABCD = v4(vt, A, B, C, Dl), vABDF = v4(vt, A, B, Dl, Fl), vACEF = v4(vt, A, C, E, Fl);
    const float vABCF = v4(vt, A, B, Fl, C), vBCDX = v4(vt, B, C, Dl, Fl), vBDEF = v4(vt, B, E, Dl, Fl);
    const float vACDE = v4(vt, E, A, C, Dl), vBCEF = v4(vt, B, E, Fl, C), vADEF = v4(vt, E, A, Dl, Fl);
    F[0][0] = (Lac1 * Lac2) * (gEF * vABCD - gEC * vABDF - gAF * vBCDX + gAC * vBDEF);
    F[0][1] = (Lac1 * Lab2) * (gEC * vABDF - gED * vABCF - gAC * vBDEF + gAD * vBCEF);
    F[1][0] = (Lab1 * Lac2) * (gAF * vBCDX - gAC * vBDEF - gBF * vACDE + gBC * vADEF);
    F[1][1] = (Lab1 * Lab2) * (gAC * vBDEF - gAD * vBCEF - gBC * vADEF + gBD * vACEF);
}

// The reference's letters of a tet from its packed local maps (per-lane, general meshes).
__device__ __forceinline__ void blk_ee_lm(const Tet& T, const float* vt, uint64_t lm, int e, int j, df D[2][2],
                                          df F[2][2]) {
    int A, B, C, Dl;
    ev(lm, e, A, B);
    ev(lm, j, C, Dl);
    blk_ee(T, vt, A, B, e, C, Dl, j, D, F);
}
__device__ __forceinline__ void blk_ef_lm(const Tet& T, const float* vt, uint64_t lm, int e, int f, df D[2][2],
                                          df F[2][2]) {
    int A, B, C, Dl, Fl;
    ev(lm, e, A, B);
    fv(lm, f, C, Dl, Fl);
    blk_ef(T, vt, A, B, e, C, Dl, Fl, D, F);
}
__device__ __forceinline__ void blk_ff_lm(const Tet& T, const float* vt, uint64_t lm, int fi, int fj, df D[2][2],
                                          df F[2][2]) {
    int A, B, E, C, Dl, Fl;
    fv(lm, fi, A, B, E);
    fv(lm, fj, C, Dl, Fl);
    blk_ff(T, vt, A, B, E, C, Dl, Fl, D, F);
}

// ----------------------------------------------------------------- fill ---
constexpr int kWarps = 4;
constexpr int kKmax = kDfMaxInc;        // incidences per warp group
constexpr int kNmax = kDfMaxCols;       // columns per entity
constexpr int kGmax = 6;                // entities per warp group
constexpr int kColPool = 256;           // columns of all entities of a group (2 edges x kNmax; 6 faces x 32)

struct __align__(16) WarpSm {
    float4 stage[kKmax * 10][4];        // per item: D (4 df) then F (4 df)
    int64_t b1[kGmax], b2[kGmax];       // CSR offsets of each entity's two rows
    int32_t cols[kColPool];             // sorted columns of each entity (pooled)
    int32_t n[kGmax], k[kGmax], cofs[kGmax], kofs[kGmax];
    int32_t tet[kKmax];
    int8_t slot[kKmax];
    int8_t qent[kKmax];                 // entity (within the group) of each incidence
    uint8_t tab[kKmax][kNmax];          // (column slot j | column mode << 4) or 0xff
};
constexpr size_t kFillSmem = sizeof(WarpSm) * kWarps + 625 * sizeof(float);

__device__ __forceinline__ int find_col(const int32_t* cols, int n, int32_t c) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (cols[mid] < c) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ void store_df(float4* dst, const df X[2][2]) {
    dst[0] = make_float4(X[0][0].h, X[0][0].l, X[0][1].h, X[0][1].l);
    dst[1] = make_float4(X[1][0].h, X[1][0].l, X[1][1].h, X[1][1].l);
}

// groups[g] = (first index into gents, entity count); all entities of a group are
// the same kind (edges or faces) and together have at most kKmax incidences.
__global__ void __launch_bounds__(32 * kWarps) k_fill_df(const Rec2* __restrict__ recs, const int2* __restrict__ groups,
                                                         int64_t n_groups, const int32_t* __restrict__ gents,
                                                         const int32_t* __restrict__ partner,
                                                         const int64_t* __restrict__ inc_ptr, const int64_t* __restrict__ inc,
                                                         const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                                         const float4* __restrict__ tscale, double2* __restrict__ E,
                                                         double2* __restrict__ B) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    WarpSm* sm_all = reinterpret_cast<WarpSm*>(smem_raw);
    float* vt = reinterpret_cast<float*>(smem_raw + sizeof(WarpSm) * kWarps);
    for (int i = threadIdx.x; i < 625; i += blockDim.x) vt[i] = c_vint[i];
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    WarpSm& sm = sm_all[w];
    for (int64_t g = blockIdx.x * (int64_t)kWarps + w; g < n_groups; g += (int64_t)gridDim.x * kWarps) {
        const int2 gr = groups[g];
        const int nsub = gr.y;
        // per-entity metadata (lane u handles entity u), then prefix offsets by lane 0
        if (lane < nsub) {
            const int32_t r1 = gents[gr.x + lane];
            sm.b1[lane] = indptr[r1];
            sm.b2[lane] = indptr[partner[r1]];
            sm.n[lane] = (int)(indptr[r1 + 1] - indptr[r1]);
            sm.k[lane] = (int)(inc_ptr[r1 + 1] - inc_ptr[r1]);
        }
        __syncwarp();
        if (lane == 0) {
            int co = 0, ko = 0;
            for (int u = 0; u < nsub; ++u) {
                sm.cofs[u] = co;
                sm.kofs[u] = ko;
                co += sm.n[u];
                ko += sm.k[u];
            }
        }
        __syncwarp();
        const int ktot = sm.kofs[nsub - 1] + sm.k[nsub - 1];
        for (int u = 0; u < nsub; ++u) {
            const int64_t b1 = sm.b1[u];
            const int n = sm.n[u], co = sm.cofs[u];
            for (int c = lane; c < n; c += 32) sm.cols[co + c] = __ldg(indices + b1 + c);
            const int32_t r1 = gents[gr.x + u];
            const int64_t i0 = inc_ptr[r1];
            const int ko = sm.kofs[u];
            for (int q = lane; q < sm.k[u]; q += 32) {
                const int64_t code = inc[i0 + q];
                const int64_t t = code >> 4;
                sm.tet[ko + q] = (int32_t)t;
                sm.slot[ko + q] = (int8_t)(code & 15);
                sm.qent[ko + q] = (int8_t)u;
            }
            for (int q = 0; q < sm.k[u]; ++q)
                for (int c = lane; c < n; c += 32) sm.tab[ko + q][c] = 0xff;
        }
        __syncwarp();
        // phase A: edge columns (j = 0..5); phase B: face columns (j = 6..9)
        for (int ph = 0; ph < 2; ++ph) {
            const int per = ph == 0 ? 6 : 4;
            const int nitems = ktot * per;
            for (int a = lane; a < nitems; a += 32) {
                const int q = a / per;
                const int j = (ph == 0 ? 0 : 6) + a % per;
                const int s = sm.slot[q];
                const Rec2* rp = recs + sm.tet[q];
                const Tet T{rp};
                const uint64_t lm = rp->lmap;
                df D[2][2], F[2][2];
                if (s < 6) {
                    if (j < 6) blk_ee_lm(T, vt, lm, s, j, D, F);
                    else blk_ef_lm(T, vt, lm, s, j - 6, D, F);
                } else if (j < 6) {
                    df Dt[2][2], Ft[2][2];
                    blk_ef_lm(T, vt, lm, j, s - 6, Dt, Ft);
                    D[0][0] = Dt[0][0]; D[0][1] = Dt[1][0]; D[1][0] = Dt[0][1]; D[1][1] = Dt[1][1];
                    F[0][0] = Ft[0][0]; F[0][1] = Ft[1][0]; F[1][0] = Ft[0][1]; F[1][1] = Ft[1][1];
                } else {
                    blk_ff_lm(T, vt, lm, s - 6, j - 6, D, F);
                }
                float4* st = sm.stage[q * 10 + j];
                store_df(st, D);
                store_df(st + 2, F);
                const int u = sm.qent[q];
                const int32_t* cu = sm.cols + sm.cofs[u];
                const int p1 = find_col(cu, sm.n[u], __ldg(&rp->dof[j]));
                const int p2 = find_col(cu, sm.n[u], __ldg(&rp->dof[j + 10]));
                sm.tab[q][p1] = (uint8_t)j;
                sm.tab[q][p2] = (uint8_t)(j | 16);
            }
        }
        __syncwarp();
        // owner phase: position-parallel accumulation in ascending tet order
        for (int u = 0; u < nsub; ++u) {
            const int n = sm.n[u], ko = sm.kofs[u], ke = ko + sm.k[u];
            // material scales per incidence: sE, sB (re.h, re.l, im.h, im.l), read through L1
            bool e_real = true;
            for (int q = ko; q < ke; ++q) {
                const float4 se = __ldg(tscale + 2 * (int64_t)sm.tet[q]);
                e_real &= (se.z == 0.f && se.w == 0.f);
            }
            for (int p = lane; p < n; p += 32) {
#pragma unroll
                for (int a = 0; a < 2; ++a) {
                    acc er = {0.f, 0.f}, ei = {0.f, 0.f}, br = {0.f, 0.f}, bi = {0.f, 0.f};
                    for (int q = ko; q < ke; ++q) {
                        const uint8_t x = sm.tab[q][p];
                        if (x == 0xff) continue;
                        const int j = x & 15, b = x >> 4;
                        const float4* st = sm.stage[q * 10 + j];
                        const float4 dv = st[a];
                        const float4 fvv = st[2 + a];
                        const df Dv = b ? mk(dv.z, dv.w) : mk(dv.x, dv.y);
                        const df Fv = b ? mk(fvv.z, fvv.w) : mk(fvv.x, fvv.y);
                        const float4 se = __ldg(tscale + 2 * (int64_t)sm.tet[q]);
                        const float4 sb = __ldg(tscale + 2 * (int64_t)sm.tet[q] + 1);
                        acc_fma(er, mk(se.x, se.y), Dv);
                        if (!e_real) acc_fma(ei, mk(se.z, se.w), Dv);
                        acc_fma(br, mk(sb.x, sb.y), Fv);
                        acc_fma(bi, mk(sb.z, sb.w), Fv);
                    }
                    const int64_t o = (a == 0 ? sm.b1[u] : sm.b2[u]) + p;
                    E[o] = make_double2(to_double(fts(er.s, er.e)), e_real ? 0.0 : to_double(fts(ei.s, ei.e)));
                    B[o] = make_double2(to_double(fts(br.s, br.e)), to_double(fts(bi.s, bi.e)));
                }
            }
        }
        __syncwarp();
    }
}

// ------------------------------------------------ canonical-frame fill ---
// When every tet's edge and face orientations follow one order of its vertices (the
// reference orients edges and faces by ascending global vertex id, fem/mesh3d.py:252-271),
// relabelling the vertices by that order makes every edge (a,b) with a < b and every
// face (c,d,f) with c < d < f: the local maps become the same for all tets.  The block
// formulas then take warp-uniform letters, so one thread per tet evaluates the element
// blocks with all lanes on the same formula, each symmetric block once.
//   k_prep3    (plan, thread per tet): invariants in the canonical labels, float-float,
//              as 43 arrays of nT pairs (coalesced per invariant); the 20 DOF ids in the
//              canonical slot order; the canonical slot of every original slot.
//   k_inc_pos  (plan, warp per entity): the CSR position of each incident tet's 20
//              columns in the entity's row.
//   k_elem     (per fill, thread per tet): the element blocks of D and F into a staging
//              buffer laid out (tet, row pair, column)-major.
//   k_fill_st  (per fill, warp per entity group): the owner pass over the staging buffer.
constexpr int kInv = 43;                 // 10 Gram + 21 cross-product Gram + 6 distances + 6 edge lengths
constexpr int kInvDs = 31, kInvLen = 37;
constexpr int kElemThreads = 128;

__constant__ int8_t c_cedge[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
__constant__ int8_t c_cface[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};

// Invariants of one tet in shared memory, laid out [invariant][thread]; the invariant
// index is warp-uniform, so every read is a conflict-free row of the array.
struct SmTet {
    const float2* s;
    int tid;
    __device__ __forceinline__ df at(int k) const {
        const float2 v = s[k * kElemThreads + tid];
        return mk(v.x, v.y);
    }
    __device__ __forceinline__ df g(int p, int q) const { return at(c_gidx[p][q]); }
    __device__ __forceinline__ df cc(int p, int q, int s1, int s2) const {
        if (p == q || s1 == s2) return mk(0.f, 0.f);
        const df v = at(10 + cidx(c_pidx[p][q], c_pidx[s1][s2]));
        return ((p < q) == (s1 < s2)) ? v : -v;
    }
    __device__ __forceinline__ df ds(int p, int q) const { return at(kInvDs + c_pidx[p][q]); }
    __device__ __forceinline__ df len(int e) const { return at(kInvLen + e); }
};

// Plan time, thread per tet (FP64): the canonical invariants.  A tet whose orientations
// follow no single vertex order sets *noncanon (the plan then keeps the per-lane fill).
__global__ void k_prep3(const double* __restrict__ nodes, int64_t nN, const int32_t* __restrict__ tets, int64_t nT,
                        const int32_t* __restrict__ edges, int64_t nE, const int32_t* __restrict__ tris, int64_t nTri,
                        const int32_t* __restrict__ t2f, const int32_t* __restrict__ t2e,
                        const double* __restrict__ edge_len, float2* __restrict__ inv, int32_t* __restrict__ dofc,
                        uint64_t* __restrict__ cslot, double2* __restrict__ gscale, int* err, int* noncanon) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nT; t += (int64_t)gridDim.x * blockDim.x) {
        int32_t vid[4];
        double x[4], y[4], z[4];
        for (int k = 0; k < 4; ++k) {
            vid[k] = tets[k * nT + t];
            x[k] = nodes[vid[k]];
            y[k] = nodes[nN + vid[k]];
            z[k] = nodes[2 * nN + vid[k]];
        }
        // the reference's letters: edge slot e = (A_e, B_e), face slot f = (C_f, D_f, F_f)
        int ea[6], eb[6], fl[4][3];
        bool ok = true;
        for (int e = 0; e < 6; ++e) {
            const int32_t eid = t2f[e * nT + t];
            int loc[2] = {0, 0};
            if (eid < 0 || eid >= nE) ok = false;
            else
                for (int j = 0; j < 2; ++j) {
                    const int32_t g = edges[j * nE + eid];
                    loc[j] = -1;
                    for (int k = 0; k < 4; ++k) if (vid[k] == g) { loc[j] = k; break; }
                    if (loc[j] < 0) { ok = false; loc[j] = 0; }
                }
            ea[e] = loc[0];
            eb[e] = loc[1];
        }
        for (int f = 0; f < 4; ++f) {
            const int64_t tri = (int64_t)t2f[(6 + f) * nT + t] - nE;
            for (int j = 0; j < 3; ++j) {
                int loc = 0;
                if (tri < 0 || tri >= nTri) ok = false;
                else {
                    const int32_t g = tris[j * nTri + tri];
                    loc = -1;
                    for (int k = 0; k < 4; ++k) if (vid[k] == g) { loc = k; break; }
                    if (loc < 0) { ok = false; loc = 0; }
                }
                fl[f][j] = loc;
            }
        }
        if (!ok) { atomicOr(err, 1); continue; }
        // the vertex order the edges follow: rank = number of edges pointing into the vertex
        int rank[4] = {0, 0, 0, 0};
        for (int e = 0; e < 6; ++e) rank[eb[e]]++;
        int seen = 0;
        for (int k = 0; k < 4; ++k) seen |= 1 << rank[k];
        bool canon = (seen == 15);
        for (int f = 0; f < 4 && canon; ++f)
            canon = rank[fl[f][0]] < rank[fl[f][1]] && rank[fl[f][1]] < rank[fl[f][2]];
        if (!canon) { atomicOr(noncanon, 1); continue; }
        int sig[4];                     // vertex of each canonical label
        for (int k = 0; k < 4; ++k) sig[rank[k]] = k;
        double G0[4][3], V;
        geom::tet_bcd(x, y, z, G0, &V);
        double gmax = 0.0;
        for (int i = 0; i < 4; ++i)
            for (int c = 0; c < 3; ++c) gmax = fmax(gmax, fabs(G0[i][c]));
        const int eG = gmax > 0.0 ? ilogb(gmax) : 0;
        double G[4][3];
        for (int i = 0; i < 4; ++i)
            for (int c = 0; c < 3; ++c) G[i][c] = scalbn(G0[sig[i]][c], -eG);
        for (int p = 0; p < 4; ++p)
            for (int q = p; q < 4; ++q) {
                const df v = split(G[p][0] * G[q][0] + G[p][1] * G[q][1] + G[p][2] * G[q][2]);
                inv[(int64_t)c_gidx[p][q] * nT + t] = make_float2(v.h, v.l);
            }
        const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {1, 2, 3, 2, 3, 3};
        double X[6][3], dsv[6], lenv[6];
        double lmax = 0.0;
        for (int P = 0; P < 6; ++P) {
            const double* u = G[pa[P]];
            const double* v = G[pb[P]];
            X[P][0] = u[1] * v[2] - u[2] * v[1];
            X[P][1] = u[2] * v[0] - u[0] * v[2];
            X[P][2] = u[0] * v[1] - u[1] * v[0];
            const int a = sig[pa[P]], b = sig[pb[P]];
            const double dx = x[a] - x[b], dy = y[a] - y[b], dz = z[a] - z[b];
            dsv[P] = sqrt(dx * dx + dy * dy + dz * dz);
            lmax = fmax(lmax, dsv[P]);
        }
        for (int P = 0; P < 6; ++P)
            for (int R = P; R < 6; ++R) {
                const df v = split(X[P][0] * X[R][0] + X[P][1] * X[R][1] + X[P][2] * X[R][2]);
                inv[(int64_t)(10 + cidx(P, R)) * nT + t] = make_float2(v.h, v.l);
            }
        // canonical slot of every original slot, and the DOF ids in canonical slot order
        uint64_t cs = 0;
        for (int e = 0; e < 6; ++e) {
            const int a = rank[ea[e]], b = rank[eb[e]];             // a < b
            const int c = c_pidx[a][b];                             // canonical edge slot
            lenv[c] = edge_len[t2e[e * nT + t]];
            lmax = fmax(lmax, lenv[c]);
            cs |= (uint64_t)c << (4 * e);
            dofc[t * 20 + c] = t2f[e * nT + t];
            dofc[t * 20 + 10 + c] = t2f[(10 + e) * nT + t];
        }
        for (int f = 0; f < 4; ++f) {
            const int missing = 6 - rank[fl[f][0]] - rank[fl[f][1]] - rank[fl[f][2]];
            const int c = 3 - missing;                              // canonical face slot
            cs |= (uint64_t)(6 + c) << (4 * (6 + f));
            dofc[t * 20 + 6 + c] = t2f[(6 + f) * nT + t];
            dofc[t * 20 + 16 + c] = t2f[(16 + f) * nT + t];
        }
        cslot[t] = cs;
        const int eL = lmax > 0.0 ? ilogb(lmax) : 0;
        for (int P = 0; P < 6; ++P) {
            const df a = split(scalbn(dsv[P], -eL));
            const df b = split(scalbn(lenv[P], -eL));
            inv[(int64_t)(kInvDs + P) * nT + t] = make_float2(a.h, a.l);
            inv[(int64_t)(kInvLen + P) * nT + t] = make_float2(b.h, b.l);
        }
        const double V6 = 6.0 * V;
        const double V6sq = V6 * V6;
        const double kd = V6 * (1.0 / (V6sq * V6sq));
        const double kf = V6 * (1.0 / V6sq);
        gscale[t] = make_double2(scalbn(kd, 4 * eG + 2 * eL) / 5040.0, scalbn(kf, 2 * eG + 2 * eL) / 5040.0);
    }
}

// Incidences with canonical slots: (tet << 4) | canonical slot of the entity in the tet.
__global__ void k_inc_canon(const int64_t* __restrict__ inc, int64_t n, const uint64_t* __restrict__ cslot,
                            int64_t* __restrict__ inc_c) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t code = inc[i];
        const int64_t t = code >> 4;
        const int e = (int)(code & 15);
        inc_c[i] = (t << 4) | (int64_t)((cslot[t] >> (4 * e)) & 15);
    }
}

// Plan time, warp per entity: the CSR position (within the entity's row) of each of the
// 20 canonical column DOFs of each incident tet, one byte per column.  Entities whose
// rows are longer than 255 (outside every fast-fill class) are skipped.
__global__ void k_inc_pos(const int32_t* __restrict__ ent_list, int64_t n_ent, const int64_t* __restrict__ inc_ptr,
                          const int64_t* __restrict__ inc_c, const int32_t* __restrict__ dofc,
                          const int64_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                          uint8_t* __restrict__ ipos) {
    const int lane = threadIdx.x & 31;
    const int64_t wid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t e = wid; e < n_ent; e += nw) {
        const int32_t r = ent_list[e];
        const int64_t b0 = indptr[r];
        const int n = (int)(indptr[r + 1] - b0);
        if (n > 255) continue;
        const int64_t i0 = inc_ptr[r], k = inc_ptr[r + 1] - i0;
        for (int64_t x = lane; x < k * 20; x += 32) {
            const int64_t q = x / 20;
            const int jj = (int)(x % 20);
            const int64_t t = inc_c[i0 + q] >> 4;
            const int32_t c = dofc[t * 20 + jj];
            int lo = 0, hi = n - 1;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (indices[b0 + mid] < c) lo = mid + 1; else hi = mid;
            }
            ipos[(i0 + q) * 20 + jj] = (uint8_t)lo;
        }
    }
}

// Staging layout: for tet t, entity slot s (the row pair) and column c = j + 10 b
// (column slot j, mode b), one 32-byte unit of two float4: (D[0][c], D[1][c]) and
// (F[0][c], F[1][c]), float-float, rows 0 and 1 of the pair.  Units are interleaved over
// blocks of kStBlk consecutive tets, unit index ((t / kStBlk * 10 + s) * 20 + c) * kStBlk
// + t % kStBlk: the element kernel's warp (one tet per lane) stores whole lines, and the
// owner pass reads the 20 columns of a (tet, row pair) as 20 full sectors.
constexpr int kStBlk = 8;
__host__ __device__ __forceinline__ int64_t st_unit(int64_t t, int s, int c) {
    return ((t / kStBlk * 10 + s) * 20 + c) * kStBlk + (t % kStBlk);
}
__device__ __forceinline__ void st_col(float4* st, int64_t t, int s, int c, df d0, df d1, df f0, df f1) {
    float4* o = st + st_unit(t, s, c) * 2;
    o[0] = make_float4(d0.h, d0.l, d1.h, d1.l);
    o[1] = make_float4(f0.h, f0.l, f1.h, f1.l);
}

// block (s, j) into the rows of s, and (when s != j) its transpose into the rows of j;
// Ft (when given) is the F block of (j, s), which is not F^T for face-face pairs
__device__ __forceinline__ void st_pair(float4* st, int64_t t, int s, int j, const df D[2][2], const df F[2][2],
                                        const df (*Ft)[2]) {
#pragma unroll
    for (int b = 0; b < 2; ++b) st_col(st, t, s, j + 10 * b, D[0][b], D[1][b], F[0][b], F[1][b]);
    if (s == j) return;
#pragma unroll
    for (int b = 0; b < 2; ++b) {
        if (Ft) st_col(st, t, j, s + 10 * b, D[b][0], D[b][1], Ft[0][b], Ft[1][b]);
        else st_col(st, t, j, s + 10 * b, D[b][0], D[b][1], F[b][0], F[b][1]);
    }
}

// Per fill, thread per tet: the 20 x 20 element blocks of D and F, each symmetric block
// evaluated once and staged on both sides.
__global__ void __launch_bounds__(kElemThreads) k_elem(const float2* __restrict__ inv, int64_t nT,
                                                       float4* __restrict__ st) {
    __shared__ float2 sinv[kInv * kElemThreads];
    __shared__ float vt[625];
    const int tid = threadIdx.x;
    for (int i = tid; i < 625; i += kElemThreads) vt[i] = c_vint[i];
    for (int64_t t0 = (int64_t)blockIdx.x * kElemThreads; t0 < nT; t0 += (int64_t)gridDim.x * kElemThreads) {
        const int64_t t = t0 + tid;
        const bool on = t < nT;
        __syncthreads();
#pragma unroll 1
        for (int k = 0; k < kInv; ++k)
            sinv[k * kElemThreads + tid] = on ? __ldg(inv + (int64_t)k * nT + t) : make_float2(0.f, 0.f);
        __syncthreads();
        const SmTet T{sinv, tid};
        df D[2][2], F[2][2], Fl[2][2];
#pragma unroll 1
        for (int s = 0; s < 6; ++s) {
#pragma unroll 1
            for (int j = s; j < 6; ++j) {
                blk_ee(T, vt, c_cedge[s][0], c_cedge[s][1], s, c_cedge[j][0], c_cedge[j][1], j, D, F);
                if (on) st_pair(st, t, s, j, D, F, nullptr);
            }
#pragma unroll 1
            for (int f = 0; f < 4; ++f) {
                blk_ef(T, vt, c_cedge[s][0], c_cedge[s][1], s, c_cface[f][0], c_cface[f][1], c_cface[f][2], D, F);
                if (on) st_pair(st, t, s, 6 + f, D, F, nullptr);
            }
        }
#pragma unroll 1
        for (int fi = 0; fi < 4; ++fi) {
#pragma unroll 1
            for (int fj = fi; fj < 4; ++fj) {
                blk_ff(T, vt, c_cface[fi][0], c_cface[fi][1], c_cface[fi][2], c_cface[fj][0], c_cface[fj][1],
                       c_cface[fj][2], D, F, true);
                if (fj != fi)
                    blk_ff(T, vt, c_cface[fj][0], c_cface[fj][1], c_cface[fj][2], c_cface[fi][0], c_cface[fi][1],
                           c_cface[fi][2], Fl, Fl, false);
                if (on) st_pair(st, t, 6 + fi, 6 + fj, D, F, fj != fi ? Fl : nullptr);
            }
        }
    }
}

// One fast-fill entity in group order: its two CSR row offsets, first incidence, row
// length and incidence count (built at plan time, read with one load per entity).
struct __align__(16) EntDesc {
    int64_t b1, b2, i0;
    int32_t n, k;
};

__global__ void k_ent_desc(const int32_t* __restrict__ gents, int64_t n, const int32_t* __restrict__ partner,
                           const int64_t* __restrict__ inc_ptr, const int64_t* __restrict__ indptr,
                           EntDesc* __restrict__ d) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r = gents[i];
        EntDesc e;
        e.b1 = indptr[r];
        e.b2 = indptr[partner[r]];
        e.i0 = inc_ptr[r];
        e.n = (int32_t)(indptr[r + 1] - e.b1);
        e.k = (int32_t)(inc_ptr[r + 1] - e.i0);
        d[i] = e;
    }
}

// Owner pass, warp per entity group.  At the start of a group its entity descriptors and
// incidences go to shared memory; the group's incident tets then run as one sequence,
// entity after entity, each entity's tets in ascending order.  For each tet, lane c < 20
// takes column c (slot c % 10, mode c / 10) of the tet's staged row pair, i.e. one CSR
// position of the entity's rows, and adds the scaled D and F entries of both rows into
// the entity's accumulators in shared memory.  A tet's 20 columns are 20 different
// positions, so the lanes never collide, and every position sums its contributions in
// tet order (deterministic, bitwise repeatable).  The next tet's run is loaded while the
// current one is added, across entity boundaries too; an entity's rows are converted and
// stored after its last tet.  The kernel runs in two modes: IM = false accumulates Re E,
// Re B and Im B and writes E and B (Im E = 0); IM = true, launched after it, returns at
// once unless some tet's mu^-1 is complex, and then accumulates Im E and writes it.
constexpr int kAcc = 3;                 // accumulators per (row, position)
constexpr int kRing = 4;                // tets in flight per warp (prefetch distance kRing - 1)
struct __align__(16) RingSlot {
    float4 col[20][2];                  // the staged unit of each column: (D0, D1), (F0, F1)
    float4 sc[2];                       // the tet's material scales
    uint32_t pos[8];                    // the 20 CSR positions (bytes), padded
};
struct __align__(16) OwnSm {
    float2 acc[2 * kNmax * kAcc];       // [row][position][component] compensated (s, e)
    RingSlot ring[kRing];
    EntDesc ed[kGmax];
    int64_t iidx[kKmax];                // incidence index of each step
    int32_t tet[kKmax];
    int8_t slot[kKmax];
    int8_t ent[kKmax];                  // entity (within the group) of each step
    int32_t kofs[kGmax + 1];
};
constexpr int kOwnWarps = 4;
constexpr size_t kStSmem = sizeof(OwnSm) * kOwnWarps;

__device__ __forceinline__ void acc_sm(float2& c, df x, df y) {   // c += x * y
    const float p = __fmul_rn(x.h, y.h);
    float pe = __fmaf_rn(x.h, y.h, -p);
    pe = __fmaf_rn(x.h, y.l, pe);
    pe = __fmaf_rn(x.l, y.h, pe);
    const float t = __fadd_rn(c.x, p);
    const float bb = __fsub_rn(t, c.x);
    const float err = __fadd_rn(__fsub_rn(c.x, __fsub_rn(t, bb)), __fsub_rn(p, bb));
    c.y = __fadd_rn(c.y, __fadd_rn(err, pe));
    c.x = t;
}

__device__ __forceinline__ void cp16(void* smem, const void* gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
                 "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp4(void* smem, const void* gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
                 "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Asynchronous copies of step i's data into ring slot i % kRing: lane c < 20 its staged
// column unit, lanes 20-21 the tet's scales, lanes 22-26 the 20 position bytes.  Every
// lane commits one group per step (empty for idle lanes), so group counts stay aligned.
__device__ __forceinline__ void ring_issue(RingSlot& r, const float4* __restrict__ st, const float4* __restrict__ tscale,
                                           const uint8_t* __restrict__ ipos, int64_t t, int slot, int64_t iidx,
                                           int lane, bool im) {
    if (lane < 20) {
        const float4* u = st + st_unit(t, slot, lane) * 2;
        cp16(&r.col[lane][0], u);
        if (!im) cp16(&r.col[lane][1], u + 1);
    } else if (lane < 22) {
        cp16(&r.sc[lane - 20], tscale + 2 * t + (lane - 20));
    } else if (lane < 27) {
        cp4(&r.pos[lane - 22], ipos + iidx * 20 + 4 * (lane - 22));
    }
    cp_commit();
}

template <bool IM>
__global__ void __launch_bounds__(32 * kOwnWarps) k_fill_st(const float4* __restrict__ st, const uint8_t* __restrict__ ipos,
                                                            const int2* __restrict__ groups, int64_t n_groups,
                                                            const EntDesc* __restrict__ edesc,
                                                            const int64_t* __restrict__ inc_c,
                                                            const float4* __restrict__ tscale,
                                                            const int* __restrict__ complex_mu,
                                                            double2* __restrict__ E, double2* __restrict__ B) {
    if (IM && *complex_mu == 0) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    OwnSm* sm_all = reinterpret_cast<OwnSm*>(smem_raw);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    OwnSm& sm = sm_all[w];
    constexpr int nc = IM ? 1 : kAcc;
    for (int64_t g = blockIdx.x * (int64_t)kOwnWarps + w; g < n_groups; g += (int64_t)gridDim.x * kOwnWarps) {
        const int2 gr = groups[g];
        const int nsub = gr.y;
        if (lane < nsub) sm.ed[lane] = edesc[gr.x + lane];
        __syncwarp();
        if (lane == 0) {
            int ko = 0;
            for (int u = 0; u < nsub; ++u) {
                sm.kofs[u] = ko;
                ko += sm.ed[u].k;
            }
            sm.kofs[nsub] = ko;
        }
        __syncwarp();
        const int ktot = sm.kofs[nsub];
        int nmax = 0;
        for (int u = 0; u < nsub; ++u) nmax = max(nmax, sm.ed[u].n);
        if (lane < ktot) {
            int u = 0;
            while (lane >= sm.kofs[u + 1]) ++u;
            const int64_t ii = sm.ed[u].i0 + (lane - sm.kofs[u]);
            const int64_t code = inc_c[ii];
            sm.iidx[lane] = ii;
            sm.tet[lane] = (int32_t)(code >> 4);
            sm.slot[lane] = (int8_t)(code & 15);
            sm.ent[lane] = (int8_t)u;
        }
        for (int i = lane; i < 2 * nmax * nc; i += 32) sm.acc[i] = make_float2(0.f, 0.f);
        __syncwarp();
        for (int i = 0; i < kRing - 1; ++i) {
            if (i < ktot) ring_issue(sm.ring[i], st, tscale, ipos, sm.tet[i], sm.slot[i], sm.iidx[i], lane, IM);
            else cp_commit();
        }
        for (int i = 0; i < ktot; ++i) {
            const int u = sm.ent[i];
            const int n = sm.ed[u].n;
            const int ip = i + kRing - 1;
            if (ip < ktot) ring_issue(sm.ring[ip % kRing], st, tscale, ipos, sm.tet[ip], sm.slot[ip], sm.iidx[ip], lane, IM);
            else cp_commit();
            cp_wait<kRing - 1>();
            __syncwarp();
            const RingSlot& r = sm.ring[i % kRing];
            if (lane < 20) {
                const int cp = reinterpret_cast<const uint8_t*>(r.pos)[lane];
                const float4 cd = r.col[lane][0];
                const float4 cse = r.sc[0];
                float2* c0 = sm.acc + cp * nc;
                float2* c1 = sm.acc + (n + cp) * nc;
                const df D0 = mk(cd.x, cd.y), D1 = mk(cd.z, cd.w);
                if (IM) {
                    acc_sm(c0[0], mk(cse.z, cse.w), D0);
                    acc_sm(c1[0], mk(cse.z, cse.w), D1);
                } else {
                    const float4 cf = r.col[lane][1];
                    const float4 csb = r.sc[1];
                    const df F0 = mk(cf.x, cf.y), F1 = mk(cf.z, cf.w);
                    acc_sm(c0[0], mk(cse.x, cse.y), D0);
                    acc_sm(c1[0], mk(cse.x, cse.y), D1);
                    acc_sm(c0[1], mk(csb.x, csb.y), F0);
                    acc_sm(c1[1], mk(csb.x, csb.y), F1);
                    acc_sm(c0[2], mk(csb.z, csb.w), F0);
                    acc_sm(c1[2], mk(csb.z, csb.w), F1);
                }
            }
            __syncwarp();
            if (i + 1 == ktot || sm.ent[i + 1] != u) {
                const EntDesc& ed = sm.ed[u];
                for (int x = lane; x < 2 * n; x += 32) {
                    const int a = x >= n ? 1 : 0, p = x - a * n;
                    float2* c = sm.acc + (a * n + p) * nc;
                    const int64_t o = (a == 0 ? ed.b1 : ed.b2) + p;
                    if (IM) {
                        reinterpret_cast<double*>(E + o)[1] = to_double(fts(c[0].x, c[0].y));
                    } else {
                        E[o] = make_double2(to_double(fts(c[0].x, c[0].y)), 0.0);
                        B[o] = make_double2(to_double(fts(c[1].x, c[1].y)), to_double(fts(c[2].x, c[2].y)));
                    }
#pragma unroll
                    for (int cc = 0; cc < nc; ++cc) c[cc] = make_float2(0.f, 0.f);
                }
                __syncwarp();
            }
        }
    }
}

// ---------------------------------------------------- plan-time grouping ---
// Entity classes: 0 edge with k <= kKmax/2 (two per group), 1 edge with
// kKmax/2 < k <= kKmax (one per group), 2 face (kGmax per group), 3 FP64 fallback.
__global__ void k_classify(const int32_t* __restrict__ ent_list, int64_t n_ent, const int64_t* __restrict__ inc_ptr,
                           const int64_t* __restrict__ inc, const int64_t* __restrict__ indptr, int64_t* flags) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_ent; e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r = ent_list[e];
        const int64_t k = inc_ptr[r + 1] - inc_ptr[r];
        const int64_t n = indptr[r + 1] - indptr[r];
        int kind = -1;   // 0 edge, 1 face
        bool uniform = true;
        for (int64_t i = inc_ptr[r]; i < inc_ptr[r + 1]; ++i) {
            const int kk = ((inc[i] & 15) < 6) ? 0 : 1;
            if (kind < 0) kind = kk;
            uniform &= (kk == kind);
        }
        int cls = 3;
        if (uniform && kind == 0 && n <= kNmax && k <= kKmax / 2) cls = 0;
        else if (uniform && kind == 0 && n <= kNmax && k <= kKmax) cls = 1;
        else if (uniform && kind == 1 && n <= kColPool / kGmax && k <= kKmax / kGmax) cls = 2;
        for (int c = 0; c < 4; ++c) flags[c * (n_ent + 1) + e] = (c == cls) ? 1 : 0;
    }
}

// Scatter entities into the class-ordered list and write the groups.
__global__ void k_groups(const int32_t* __restrict__ ent_list, int64_t n_ent, const int64_t* flags,
                         const int64_t* scans, int64_t c0, int64_t c1, int64_t c2, int32_t* gents, int2* groups,
                         int32_t* slow) {
    const int64_t g0 = (c0 + 1) / 2, g1 = c1;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_ent; e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r = ent_list[e];
        if (flags[e]) {
            const int64_t i = scans[e];
            gents[i] = r;
            if ((i & 1) == 0) groups[i / 2] = make_int2((int)i, (int)(c0 - i < 2 ? c0 - i : 2));
        } else if (flags[(n_ent + 1) + e]) {
            const int64_t i = scans[(n_ent + 1) + e];
            gents[c0 + i] = r;
            groups[g0 + i] = make_int2((int)(c0 + i), 1);
        } else if (flags[2 * (n_ent + 1) + e]) {
            const int64_t i = scans[2 * (n_ent + 1) + e];
            gents[c0 + c1 + i] = r;
            if (i % kGmax == 0)
                groups[g0 + g1 + i / kGmax] = make_int2((int)(c0 + c1 + i), (int)(c2 - i < kGmax ? c2 - i : kGmax));
        } else {
            slow[scans[3 * (n_ent + 1) + e]] = r;
        }
    }
}

}  // namespace dfk

// ------------------------------------------------------------------ host ---
namespace {
bool g_vint_ready[64] = {false};

int upload_vint() {
    int dev = 0;
    EMG_CUDA(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64 && g_vint_ready[dev]) return EMG_OK;
    static const double fact[10] = {1, 1, 2, 6, 24, 120, 720, 5040, 40320, 362880};
    float h[625];
    for (int a = 0; a < 5; ++a)
        for (int b = 0; b < 5; ++b)
            for (int c = 0; c < 5; ++c)
                for (int d = 0; d < 5; ++d) {
                    int k[5] = {0, 0, 0, 0, 0};
                    k[a]++; k[b]++; k[c]++; k[d]++;
                    const double num = fact[k[1]] * fact[k[2]] * fact[k[3]] * fact[k[4]];
                    h[((a * 5 + b) * 5 + c) * 5 + d] = (float)(5040.0 * num / fact[k[1] + k[2] + k[3] + k[4] + 3]);
                }
    EMG_CUDA(cudaMemcpyToSymbol(dfk::c_vint, h, sizeof(h)));
    if (dev >= 0 && dev < 64) g_vint_ready[dev] = true;
    return EMG_OK;
}
}  // namespace

void df_plan_free(DfPlan* p) {
    dfree(p->recs);
    dfree(p->inv);
    dfree(p->dofc);
    dfree(p->inc_c);
    dfree(p->ipos);
    dfree(p->edesc);
    dfree(p->st);
    dfree(p->mu_flag);
    p->canon = false;
    dfree(p->gscale);
    dfree(p->tscale);
    dfree(p->groups);
    dfree(p->gents);
    dfree(p->slow);
    p->n_groups = p->n_slow = 0;
}

int df_plan_build(const double* nodes, int64_t nN, const int32_t* tets, int64_t nT, const int32_t* edges, int64_t nE,
                  const int32_t* tris, int64_t nTri, const int32_t* t2f, const int32_t* t2e, const double* edge_len,
                  const int32_t* ent_list, int64_t n_ent, const int32_t* partner, const int64_t* inc_ptr,
                  const int64_t* inc, int64_t n_inc, const int64_t* indptr, const int32_t* indices, DfPlan* p,
                  cudaStream_t s) {
    int rc = upload_vint();
    if (rc) return rc;
    *p = DfPlan();
    int* d_err = nullptr;
    int64_t *flags = nullptr, *scans = nullptr, *tmp = nullptr;
    uint64_t* cslot = nullptr;
    auto cleanup = [&]() { dfree(d_err); dfree(flags); dfree(scans); dfree(tmp); dfree(cslot); };
#define TRY(x) do { int _r = (x); if (_r) { cleanup(); df_plan_free(p); return _r; } } while (0)
#define TRYC(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) { cleanup(); df_plan_free(p); return cuda_status(_e, #x); } } while (0)
    TRY(dalloc(&d_err, 2, "df err"));
    TRY(dalloc(&p->gscale, nT, "df geometric scales"));
    TRY(dalloc(&p->tscale, 2 * nT, "df material scales"));
    TRYC(cudaMemsetAsync(d_err, 0, 2 * sizeof(int), s));
    const int T = 256;
    // canonical frame first; a mesh with a tet whose orientations follow no vertex order
    // keeps the per-lane records
    int h_flags[2] = {0, 0};
    if (nT > 0) {
        TRY(dalloc(&p->inv, (int64_t)dfk::kInv * nT, "df canonical invariants"));
        TRY(dalloc(&p->dofc, 20 * nT, "df canonical DOF ids"));
        TRY(dalloc(&cslot, nT, "df canonical slots"));
        dfk::k_prep3<<<grid_for(nT, T), T, 0, s>>>(nodes, nN, tets, nT, edges, nE, tris, nTri, t2f, t2e, edge_len,
                                                   p->inv, p->dofc, cslot, p->gscale, d_err, d_err + 1);
        TRYC(cudaGetLastError());
        TRYC(cudaMemcpyAsync(h_flags, d_err, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
        TRYC(cudaStreamSynchronize(s));
    }
    p->canon = nT > 0 && h_flags[0] == 0 && h_flags[1] == 0;
    if (p->canon) {
        TRY(dalloc(&p->inc_c, n_inc, "df canonical incidences"));
        if (n_inc > 0) {
            dfk::k_inc_canon<<<grid_for(n_inc, T), T, 0, s>>>(inc, n_inc, cslot, p->inc_c);
            TRYC(cudaGetLastError());
        }
        TRY(dalloc(&p->ipos, 20 * n_inc, "df CSR positions of the incidences"));
        if (n_ent > 0) {
            dfk::k_inc_pos<<<grid_for(n_ent * 32, T, 152u * 64u), T, 0, s>>>(ent_list, n_ent, inc_ptr, p->inc_c, p->dofc,
                                                                            indptr, indices, p->ipos);
            TRYC(cudaGetLastError());
        }
        TRY(dalloc(&p->st, (nT + dfk::kStBlk - 1) / dfk::kStBlk * dfk::kStBlk * 10 * 20 * 2,
                   "df staged element blocks"));
        TRY(dalloc(&p->mu_flag, 1, "df complex-mu flag"));
    } else {
        dfree(p->inv);
        dfree(p->dofc);
        TRY(dalloc(reinterpret_cast<dfk::Rec2**>(&p->recs), nT, "df records"));
        TRYC(cudaMemsetAsync(d_err, 0, 2 * sizeof(int), s));
        if (nT > 0) {
            dfk::k_prep2<<<grid_for(nT, T), T, 0, s>>>(nodes, nN, tets, nT, edges, nE, tris, nTri, t2f, t2e, edge_len,
                                                       reinterpret_cast<dfk::Rec2*>(p->recs), p->gscale, d_err);
            TRYC(cudaGetLastError());
        }
    }
    const int64_t L = n_ent + 1;
    TRY(dalloc(&flags, 4 * L, "df class flags"));
    TRY(dalloc(&scans, 4 * L, "df class scans"));
    TRY(dalloc(&tmp, scan_scratch_elems(L) + 1, "df scan scratch"));
    if (n_ent > 0) {
        dfk::k_classify<<<grid_for(n_ent, T), T, 0, s>>>(ent_list, n_ent, inc_ptr, inc, indptr, flags);
        TRYC(cudaGetLastError());
    }
    for (int c = 0; c < 4; ++c) TRY(scan_exclusive_i64(flags + c * L, scans + c * L, n_ent, tmp, s));
    int64_t cnt[4] = {0, 0, 0, 0};
    int h_err = 0;
    for (int c = 0; c < 4; ++c)
        TRYC(cudaMemcpyAsync(&cnt[c], scans + c * L + n_ent, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    TRYC(cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    TRYC(cudaStreamSynchronize(s));
    if (h_err) {
        set_error("mesh check failed: an edge/face vertex is not a vertex of its tet");
        TRY(EMG_ERR_MESH);
    }
    p->n_groups = (cnt[0] + 1) / 2 + cnt[1] + (cnt[2] + dfk::kGmax - 1) / dfk::kGmax;
    p->n_slow = cnt[3];
    TRY(dalloc(&p->groups, p->n_groups + 1, "df groups"));
    TRY(dalloc(&p->gents, cnt[0] + cnt[1] + cnt[2] + 1, "df group entities"));
    TRY(dalloc(&p->slow, p->n_slow + 1, "df slow list"));
    if (n_ent > 0) {
        dfk::k_groups<<<grid_for(n_ent, T), T, 0, s>>>(ent_list, n_ent, flags, scans, cnt[0], cnt[1], cnt[2], p->gents,
                                                        p->groups, p->slow);
        TRYC(cudaGetLastError());
    }
    if (p->canon) {
        const int64_t ng = cnt[0] + cnt[1] + cnt[2];
        TRY(dalloc(reinterpret_cast<dfk::EntDesc**>(&p->edesc), ng, "df entity descriptors"));
        if (ng > 0) {
            dfk::k_ent_desc<<<grid_for(ng, T), T, 0, s>>>(p->gents, ng, partner, inc_ptr, indptr,
                                                          reinterpret_cast<dfk::EntDesc*>(p->edesc));
            TRYC(cudaGetLastError());
        }
    }
    TRYC(cudaStreamSynchronize(s));
#undef TRY
#undef TRYC
    cleanup();
    return EMG_OK;
}

int df_fill(const DfPlan& p, int64_t nT, const int32_t* partner, const int64_t* inc_ptr, const int64_t* inc,
            const int64_t* indptr, const int32_t* indices, const double* eps, const double* mu_inv, double* E,
            double* B, cudaStream_t s) {
    static bool attr_set[64] = {false};
    int dev = 0;
    EMG_CUDA(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64 && !attr_set[dev]) {
        EMG_CUDA(cudaFuncSetAttribute(dfk::k_fill_df, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)dfk::kFillSmem));
        EMG_CUDA(cudaFuncSetAttribute(dfk::k_fill_st<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)dfk::kStSmem));
        EMG_CUDA(cudaFuncSetAttribute(dfk::k_fill_st<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)dfk::kStSmem));
        attr_set[dev] = true;
    }
    if (p.mu_flag) EMG_CUDA(cudaMemsetAsync(p.mu_flag, 0, sizeof(int), s));
    if (nT > 0) {
        dfk::k_scales<<<grid_for(nT, 256), 256, 0, s>>>(p.gscale, reinterpret_cast<const double2*>(eps),
                                                         reinterpret_cast<const double2*>(mu_inv), nT, p.tscale,
                                                         p.mu_flag);
        EMG_CUDA(cudaGetLastError());
    }
    if (p.n_groups > 0 && p.canon) {
        dfk::k_elem<<<grid_for(nT, dfk::kElemThreads, 152u * 64u), dfk::kElemThreads, 0, s>>>(p.inv, nT, p.st);
        EMG_CUDA(cudaGetLastError());
        const unsigned g = grid_for(p.n_groups, dfk::kOwnWarps, 152u * 16u);
        dfk::k_fill_st<false><<<g, 32 * dfk::kOwnWarps, dfk::kStSmem, s>>>(
            p.st, p.ipos, reinterpret_cast<const int2*>(p.groups), p.n_groups,
            reinterpret_cast<const dfk::EntDesc*>(p.edesc), p.inc_c, p.tscale, p.mu_flag,
            reinterpret_cast<double2*>(E), reinterpret_cast<double2*>(B));
        EMG_CUDA(cudaGetLastError());
        dfk::k_fill_st<true><<<g, 32 * dfk::kOwnWarps, dfk::kStSmem, s>>>(
            p.st, p.ipos, reinterpret_cast<const int2*>(p.groups), p.n_groups,
            reinterpret_cast<const dfk::EntDesc*>(p.edesc), p.inc_c, p.tscale, p.mu_flag,
            reinterpret_cast<double2*>(E), reinterpret_cast<double2*>(B));
        EMG_CUDA(cudaGetLastError());
    } else if (p.n_groups > 0) {
        const unsigned g = grid_for(p.n_groups, dfk::kWarps, 152u * 32u);
        dfk::k_fill_df<<<g, 32 * dfk::kWarps, dfk::kFillSmem, s>>>(
            reinterpret_cast<const dfk::Rec2*>(p.recs), reinterpret_cast<const int2*>(p.groups), p.n_groups, p.gents,
            partner, inc_ptr, inc, indptr, indices, p.tscale, reinterpret_cast<double2*>(E),
            reinterpret_cast<double2*>(B));
        EMG_CUDA(cudaGetLastError());
    }
    return EMG_OK;
}

}  // namespace emg
