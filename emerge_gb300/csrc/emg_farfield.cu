// Stratton-Chu far field on the GPU: the counterpart of stratton_chu_ff
// (fem/physics/edm/sc.py:26-140), which EMerge evaluates with a Numba prange loop
// over the surface sources.
//
// For every direction r = (cos th cos ph, cos th sin ph, sin th) and every kept
// source j (|E_j| > 1e-3 max|E|, sc.py:58-75), with G = exp(i k0 r.v_j):
//     ie = (n x E_j - Z0 r x (n x H_j)) G,   E_ff += Q r x ie,   Q = -i k0 / (4 pi)
// and H_ff = r x E_ff / Z0 (sc.py:104-140).  Inputs are FP32 / complex64 as the
// reference passes them.
//
//  k_ff_prep  thread per source: n x E, n x H (complex64), |E|^2, and the maximum
//             |E|^2 by an integer atomicMax on the float bits (non-negative floats
//             order like their bit patterns).
//  k_ff_sum   a block per (256 directions, chunk of kChunk sources): the chunk's
//             sources staged in shared memory, one direction per thread, FP32
//             accumulation of r x ie over the chunk, partial sums to global.
//  k_ff_out   thread per direction: the chunk partials summed in chunk order in
//             FP64 (deterministic), times Q; H = r x E / Z0.
#include "emg_common.cuh"

namespace emg {
namespace ff {

constexpr int kDirs = 256;      // directions per block (one per thread)
constexpr int kChunk = 512;     // sources per block
constexpr double kZ0 = 376.73031366857;

struct __align__(16) Src {
    float vx, vy, vz, keep;
    float2 ex, ey, ez;          // n x E
    float2 hx, hy, hz;          // n x H
};

__global__ void k_ff_prep(int64_t n, const float2* __restrict__ E, const float2* __restrict__ H,
                          const float* __restrict__ vis, const float* __restrict__ wns, Src* __restrict__ src,
                          float* __restrict__ emag2, unsigned* __restrict__ emax_bits) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const float2 Ex = E[j], Ey = E[n + j], Ez = E[2 * n + j];
        const float2 Hx = H[j], Hy = H[n + j], Hz = H[2 * n + j];
        const float nx = wns[j], ny = wns[n + j], nz = wns[2 * n + j];
        Src s;
        s.vx = vis[j];
        s.vy = vis[n + j];
        s.vz = vis[2 * n + j];
        s.keep = 0.f;
        s.ex = make_float2(ny * Ez.x - nz * Ey.x, ny * Ez.y - nz * Ey.y);
        s.ey = make_float2(nz * Ex.x - nx * Ez.x, nz * Ex.y - nx * Ez.y);
        s.ez = make_float2(nx * Ey.x - ny * Ex.x, nx * Ey.y - ny * Ex.y);
        s.hx = make_float2(ny * Hz.x - nz * Hy.x, ny * Hz.y - nz * Hy.y);
        s.hy = make_float2(nz * Hx.x - nx * Hz.x, nz * Hx.y - nx * Hz.y);
        s.hz = make_float2(nx * Hy.x - ny * Hx.x, nx * Hy.y - ny * Hx.y);
        src[j] = s;
        const float m2 = Ex.x * Ex.x + Ex.y * Ex.y + Ey.x * Ey.x + Ey.y * Ey.y + Ez.x * Ez.x + Ez.y * Ez.y;
        emag2[j] = m2;
        atomicMax(emax_bits, __float_as_uint(m2));
    }
}

// keep = |E|^2 > (max|E| * LR)^2, i.e. |E| > max|E| * LR
__global__ void k_ff_keep(int64_t n, const float* __restrict__ emag2, const unsigned* __restrict__ emax_bits,
                          float lr, Src* __restrict__ src) {
    const float emax = sqrtf(__uint_as_float(*emax_bits));
    const float thr = emax * lr;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
        src[j].keep = sqrtf(emag2[j]) > thr ? 1.f : 0.f;
}

__global__ void __launch_bounds__(kDirs) k_ff_sum(int64_t n_src, const Src* __restrict__ src, int64_t n_dir,
                                                  const float* __restrict__ theta, const float* __restrict__ phi,
                                                  float k0, float z0, float2* __restrict__ part) {
    __shared__ Src sm[kChunk];
    const int64_t j0 = (int64_t)blockIdx.y * kChunk;
    const int m = (int)min((int64_t)kChunk, n_src - j0);
    for (int i = threadIdx.x; i < m; i += blockDim.x) sm[i] = src[j0 + i];
    __syncthreads();
    const int64_t d = (int64_t)blockIdx.x * kDirs + threadIdx.x;
    if (d >= n_dir) return;
    float st, ct, sp, cp;
    sincosf(theta[d], &st, &ct);
    sincosf(phi[d], &sp, &cp);
    const float rx = ct * cp, ry = ct * sp, rz = st;
    const float kx = k0 * rx, ky = k0 * ry, kz = k0 * rz;
    float2 ax = make_float2(0.f, 0.f), ay = ax, az = ax;
    for (int i = 0; i < m; ++i) {
        const Src& s = sm[i];
        if (s.keep == 0.f) continue;
        float gs, gc;
        sincosf(kx * s.vx + ky * s.vy + kz * s.vz, &gs, &gc);
        // r x (n x H)
        const float2 bx = make_float2(ry * s.hz.x - rz * s.hy.x, ry * s.hz.y - rz * s.hy.y);
        const float2 by = make_float2(rz * s.hx.x - rx * s.hz.x, rz * s.hx.y - rx * s.hz.y);
        const float2 bz = make_float2(rx * s.hy.x - ry * s.hx.x, rx * s.hy.y - ry * s.hx.y);
        // ie = (n x E - Z0 r x (n x H)) G
        const float2 ux = make_float2(s.ex.x - z0 * bx.x, s.ex.y - z0 * bx.y);
        const float2 uy = make_float2(s.ey.x - z0 * by.x, s.ey.y - z0 * by.y);
        const float2 uz = make_float2(s.ez.x - z0 * bz.x, s.ez.y - z0 * bz.y);
        const float2 ix = make_float2(ux.x * gc - ux.y * gs, ux.x * gs + ux.y * gc);
        const float2 iy = make_float2(uy.x * gc - uy.y * gs, uy.x * gs + uy.y * gc);
        const float2 iz = make_float2(uz.x * gc - uz.y * gs, uz.x * gs + uz.y * gc);
        // r x ie
        ax.x += ry * iz.x - rz * iy.x; ax.y += ry * iz.y - rz * iy.y;
        ay.x += rz * ix.x - rx * iz.x; ay.y += rz * ix.y - rx * iz.y;
        az.x += rx * iy.x - ry * ix.x; az.y += rx * iy.y - ry * ix.y;
    }
    const int64_t base = (int64_t)blockIdx.y * 3 * n_dir;
    part[base + d] = ax;
    part[base + n_dir + d] = ay;
    part[base + 2 * n_dir + d] = az;
}

__global__ void k_ff_out(int64_t n_dir, int n_chunks, const float2* __restrict__ part,
                         const float* __restrict__ theta, const float* __restrict__ phi, double k0,
                         double2* __restrict__ Eout, double2* __restrict__ Hout) {
    for (int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; d < n_dir; d += (int64_t)gridDim.x * blockDim.x) {
        double2 s[3] = {make_double2(0, 0), make_double2(0, 0), make_double2(0, 0)};
        for (int c = 0; c < n_chunks; ++c)
            for (int k = 0; k < 3; ++k) {
                const float2 v = part[((int64_t)c * 3 + k) * n_dir + d];
                s[k].x += (double)v.x;
                s[k].y += (double)v.y;
            }
        // Q = -i k0 / (4 pi): Q (a + ib) = (k0/4pi) (b - ia)
        const double q = k0 / (4.0 * 3.14159265358979323846);
        double2 e[3];
        for (int k = 0; k < 3; ++k) e[k] = make_double2(q * s[k].y, -q * s[k].x);
        const double th = (double)theta[d], ph = (double)phi[d];
        const double rx = cos(th) * cos(ph), ry = cos(th) * sin(ph), rz = sin(th);
        const double2 h0 = make_double2((ry * e[2].x - rz * e[1].x) / kZ0, (ry * e[2].y - rz * e[1].y) / kZ0);
        const double2 h1 = make_double2((rz * e[0].x - rx * e[2].x) / kZ0, (rz * e[0].y - rx * e[2].y) / kZ0);
        const double2 h2 = make_double2((rx * e[1].x - ry * e[0].x) / kZ0, (rx * e[1].y - ry * e[0].y) / kZ0);
        Eout[d] = e[0];
        Eout[n_dir + d] = e[1];
        Eout[2 * n_dir + d] = e[2];
        Hout[d] = h0;
        Hout[n_dir + d] = h1;
        Hout[2 * n_dir + d] = h2;
    }
}

}  // namespace ff
}  // namespace emg

extern "C" int emg_stratton_chu(int64_t n_src, const float* E, const float* H, const float* vis, const float* wns,
                                int64_t n_dir, const float* theta, const float* phi, float k0, double* Eout,
                                double* Hout, void* stream) {
    using namespace emg;
    using namespace emg::ff;
    EMG_CHECK_ARG(n_src >= 0 && n_dir >= 0, "emg_stratton_chu: negative size");
    EMG_CHECK_ARG(n_dir == 0 || (theta && phi && Eout && Hout), "emg_stratton_chu: NULL output or direction array");
    EMG_CHECK_ARG(n_src == 0 || (E && H && vis && wns), "emg_stratton_chu: NULL source array");
    cudaStream_t s = (cudaStream_t)stream;
    if (n_dir == 0) return EMG_OK;
    const int64_t n_chunks = n_src > 0 ? (n_src + kChunk - 1) / kChunk : 0;
    EMG_CHECK_ARG(n_chunks < 65536 && (n_dir + kDirs - 1) / kDirs < (int64_t)INT32_MAX,
                  "emg_stratton_chu: more than 65535 * 512 sources");
    Src* src = nullptr;
    float* emag2 = nullptr;
    unsigned* emax = nullptr;
    float2* part = nullptr;
    int rc = EMG_OK;
    auto cleanup = [&]() { dfree(src); dfree(emag2); dfree(emax); dfree(part); };
    if ((rc = dalloc(&src, n_src, "far-field sources")) || (rc = dalloc(&emag2, n_src, "far-field |E|")) ||
        (rc = dalloc(&emax, 1, "far-field max")) || (rc = dalloc(&part, n_chunks * 3 * n_dir, "far-field partials"))) {
        cleanup();
        return rc;
    }
    cudaError_t e = cudaSuccess;
    if (n_src > 0) {
        e = cudaMemsetAsync(emax, 0, sizeof(unsigned), s);
        if (e == cudaSuccess) {
            k_ff_prep<<<grid_for(n_src, 256), 256, 0, s>>>(n_src, reinterpret_cast<const float2*>(E),
                                                          reinterpret_cast<const float2*>(H), vis, wns, src, emag2,
                                                          emax);
            k_ff_keep<<<grid_for(n_src, 256), 256, 0, s>>>(n_src, emag2, emax, 1e-3f, src);
            dim3 grid((unsigned)((n_dir + kDirs - 1) / kDirs), (unsigned)n_chunks);
            k_ff_sum<<<grid, kDirs, 0, s>>>(n_src, src, n_dir, theta, phi, k0, (float)kZ0, part);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess) {
        k_ff_out<<<grid_for(n_dir, 256), 256, 0, s>>>(n_dir, (int)n_chunks, part, theta, phi, (double)k0,
                                                      reinterpret_cast<double2*>(Eout),
                                                      reinterpret_cast<double2*>(Hout));
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cleanup();
    if (e != cudaSuccess) return cuda_status(e, "emg_stratton_chu");
    return EMG_OK;
}
