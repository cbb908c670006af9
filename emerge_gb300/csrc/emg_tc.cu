// 5th-generation tensor-core (tcgen05) kernels: a TF32 GEMM tile, the complex slab
// product of the slab solve (TF32), and the rank-64 Gauss-Jordan update of FP32 slab
// factorizations in split-TF32 (FP32-equivalent) precision (k_gj_update_tc, below).
//
// GEMM tile: D[M x N] = A[M x K] B[N x K]^T (row-major FP32 in and out, TF32 products, FP32
// accumulation in tensor memory).  One CTA of 128 threads owns a 128 x 64 tile of D:
//   - the operands of a 32-wide K chunk are staged by all threads into shared memory
//     in the canonical K-major, non-swizzled layout (8-row x 16-byte core matrices,
//     K-adjacent core matrices 128 B apart, M/N-adjacent 1024 / 1024 B apart);
//   - one elected thread issues four tcgen05.mma (K = 8 each) per chunk and commits
//     them to an mbarrier; every thread waits on it (bounded) before the next chunk
//     overwrites the staging buffers;
//   - the accumulator (128 lanes x 64 columns of TMEM) is read back with
//     tcgen05.ld.32x32b (warp w reads lanes 32w..32w+31) and stored.
// Every wait is bounded: on timeout the CTA records an error in *status, gives the
// MMAs it already committed one more bounded wait, skips the remaining work, and still
// frees its TMEM.  After a nonzero status the host discards the output tile and does
// not relaunch on the same data.
#include <cuda_bf16.h>

#include "emg_krylov.cuh"

namespace emg {
namespace tc {

constexpr int kM = 128, kN = 64, kK = 32, kThreads = 128;
constexpr uint32_t kTmemCols = 64;
// Waits on an mbarrier end after kWaitNs of wall time (the chunk's MMAs finish in well
// under a microsecond, so only a lost arrival gets there), polled with a short sleep so a
// busy SM does not time out early; kSpinLimit caps the polls as a second bound.
constexpr unsigned long long kWaitNs = 10ull * 1000ull * 1000ull;   // 10 ms
constexpr long long kSpinLimit = 1ll << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// UMMA shared-memory descriptor, K-major, no swizzle: start address, leading
// (K-direction) byte offset, stride (M/N-direction) byte offset, all >> 4; bits
// 46-47 = 0b01 (descriptor version).
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor, kind::tf32: D = F32 (bits 4-5 = 1), A = B = TF32 (format 2
// in bits 7-9 and 10-12), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_tf32(int m, int n) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase) {
    const unsigned long long t0 = global_ns();
    for (long long it = 0; it < kSpinLimit; ++it) {
        uint32_t done = 0;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(mbar), "r"(phase)
            : "memory");
        if (done) return true;
        if ((it & 63) == 63) {
            if (global_ns() - t0 > kWaitNs) return false;
            __nanosleep(256);
        }
    }
    return false;
}

// byte offset of element (r, k) of a [rows x 32] K-major tile in the canonical layout
__device__ __forceinline__ uint32_t tile_off(int r, int k) {
    return (uint32_t)(((r >> 3) * (kK / 4) + (k >> 2)) * 128 + (r & 7) * 16 + (k & 3) * 4);
}

__global__ void __launch_bounds__(kThreads) k_gemm_tf32(int64_t M, int64_t N, int64_t K, const float* __restrict__ A,
                                                        int64_t lda, const float* __restrict__ B, int64_t ldb,
                                                        float* __restrict__ D, int64_t ldd, int32_t* __restrict__ status) {
    __shared__ __align__(1024) float sa[kM * kK];
    __shared__ __align__(1024) float sb[kN * kK];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    __shared__ int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t m0 = (int64_t)blockIdx.y * kM, n0 = (int64_t)blockIdx.x * kN;
    if (tid == 0) {
        s_fail = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = tmem_base;
    const uint32_t mb = smem_u32(&mbar);
    uint32_t phase = 0;
    const int64_t nk = (K + kK - 1) / kK;
    for (int64_t kc = 0; kc < nk; ++kc) {
        const int64_t k0 = kc * kK;
        // stage A (128 x 32) and B (64 x 32), zero outside the matrices
        for (int idx = tid; idx < kM * kK; idx += kThreads) {
            const int r = idx / kK, k = idx % kK;
            const int64_t gr = m0 + r, gk = k0 + k;
            const float v = (gr < M && gk < K) ? A[gr * lda + gk] : 0.f;
            *reinterpret_cast<float*>(reinterpret_cast<char*>(sa) + tile_off(r, k)) = v;
        }
        for (int idx = tid; idx < kN * kK; idx += kThreads) {
            const int r = idx / kK, k = idx % kK;
            const int64_t gr = n0 + r, gk = k0 + k;
            const float v = (gr < N && gk < K) ? B[gr * ldb + gk] : 0.f;
            *reinterpret_cast<float*>(reinterpret_cast<char*>(sb) + tile_off(r, k)) = v;
        }
        // make the generic-proxy stores visible to the tensor core (async proxy)
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (tid == 0 && !s_fail) {
            const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
            const uint32_t idesc = idesc_tf32(kM, kN);
#pragma unroll
            for (int ks = 0; ks < kK / 8; ++ks) {
                // K = 8 TF32 = two core matrices along K: +256 B per step
                const uint64_t ad = make_desc(a0 + ks * 256, 128, 1024);
                const uint64_t bd = make_desc(b0 + ks * 256, 128, 1024);
                const uint32_t acc = (kc > 0 || ks > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(taddr),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb)
                         : "memory");
        }
        __syncthreads();
        if (!s_fail) {
            if (!mbar_wait(mb, phase)) s_fail = 1;
        }
        phase ^= 1;
        __syncthreads();
        if (s_fail) break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!s_fail) {
        // warp w reads TMEM lanes 32w..32w+31 (rows of the tile), 64 columns
        uint32_t v[kN];
        const uint32_t lane_addr = taddr + ((uint32_t)(warp * 32) << 16);
#pragma unroll
        for (int c0 = 0; c0 < kN; c0 += 16) {
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                "%14, %15}, [%16];"
                : "=r"(v[c0 + 0]), "=r"(v[c0 + 1]), "=r"(v[c0 + 2]), "=r"(v[c0 + 3]), "=r"(v[c0 + 4]), "=r"(v[c0 + 5]),
                  "=r"(v[c0 + 6]), "=r"(v[c0 + 7]), "=r"(v[c0 + 8]), "=r"(v[c0 + 9]), "=r"(v[c0 + 10]),
                  "=r"(v[c0 + 11]), "=r"(v[c0 + 12]), "=r"(v[c0 + 13]), "=r"(v[c0 + 14]), "=r"(v[c0 + 15])
                : "r"(lane_addr + (uint32_t)c0)
                : "memory");
        }
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        const int64_t row = m0 + warp * 32 + lane;
        if (row < M) {
#pragma unroll
            for (int c = 0; c < kN; ++c)
                if (n0 + c < N) D[row * ldd + n0 + c] = __uint_as_float(v[c]);
        }
    } else {
        // timed out: give the committed MMAs one more bounded wait before the TMEM goes
        if (tid == 0) {
            mbar_wait(mb, phase ^ 1);
            atomicExch(status, 1);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(kTmemCols) : "memory");
}

// Complex product of the slab solve on the tensor cores: Out[r0.., cols] =
// alpha * S[128 rows x K] Y[K x 64 cols] + beta * Out, complex64 interleaved in and
// out, TF32 products.  Real and imaginary parts of both operands are staged as four
// K-major tiles; per K step of 8 the real accumulator (TMEM columns 0-63) takes
// Sre Yre and -Sim Yim (negation in the instruction descriptor), the imaginary one
// (columns 64-127) Sre Yim and Sim Yre.  Grid: column tiles x row tiles x groups;
// each group g has its own S (factor) and column range (see emg_slab.cu).
struct TcGroup {
    int32_t fac, col0, ncol, pad;
};
constexpr int kCxSmem = 2 * kM * kK * 4 + 2 * kN * kK * 4;   // Sre, Sim, Yre, Yim tiles: 48 KB

__global__ void __launch_bounds__(kThreads) k_cgemm_tf32(int64_t w, int64_t row0, int64_t Bc,
                                                         const TcGroup* __restrict__ groups,
                                                         const float2* __restrict__ Sinv, int64_t totD, int64_t offD,
                                                         const float2* __restrict__ Y, float alpha, int beta,
                                                         float2* __restrict__ Out, int32_t* __restrict__ status) {
    extern __shared__ __align__(1024) unsigned char dsm[];
    char* sar = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(dsm) + 1023) & ~(uintptr_t)1023);
    char* sai = sar + kM * kK * 4;
    char* sbr = sai + kM * kK * 4;
    char* sbi = sbr + kN * kK * 4;
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    __shared__ int s_fail;
    const TcGroup g = groups[blockIdx.z];
    const int64_t c0 = (int64_t)blockIdx.x * kN, r0 = (int64_t)blockIdx.y * kM;
    if (c0 >= g.ncol) return;          // uniform per CTA, before any TMEM allocation
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const float2* S = Sinv + (int64_t)g.fac * totD + offD;
    const float2* Yb = Y + row0 * Bc + g.col0 + c0;
    const int ncl = (int)min((int64_t)kN, (int64_t)g.ncol - c0);
    if (tid == 0) {
        s_fail = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(2 * kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = tmem_base;
    const uint32_t mb = smem_u32(&mbar);
    uint32_t phase = 0;
    const int64_t nk = (w + kK - 1) / kK;
    for (int64_t kc = 0; kc < nk; ++kc) {
        const int64_t k0 = kc * kK;
        for (int idx = tid; idx < kM * kK; idx += kThreads) {
            const int r = idx / kK, k = idx % kK;
            const int64_t gr = r0 + r, gk = k0 + k;
            const float2 v = (gr < w && gk < w) ? S[gr * w + gk] : make_float2(0.f, 0.f);
            const uint32_t o = tile_off(r, k);
            *reinterpret_cast<float*>(sar + o) = v.x;
            *reinterpret_cast<float*>(sai + o) = v.y;
        }
        for (int idx = tid; idx < kN * kK; idx += kThreads) {
            const int k = idx / kN, c = idx % kN;
            const int64_t gk = k0 + k;
            const float2 v = (c < ncl && gk < w) ? Yb[gk * Bc + c] : make_float2(0.f, 0.f);
            const uint32_t o = tile_off(c, k);
            *reinterpret_cast<float*>(sbr + o) = v.x;
            *reinterpret_cast<float*>(sbi + o) = v.y;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (tid == 0 && !s_fail) {
            const uint32_t ar = smem_u32(sar), ai = smem_u32(sai), br = smem_u32(sbr), bi = smem_u32(sbi);
            const uint32_t id = idesc_tf32(kM, kN), idneg = id | (1u << 13);
            const uint32_t dre = taddr, dim = taddr + kTmemCols;
#pragma unroll
            for (int ks = 0; ks < kK / 8; ++ks) {
                const uint32_t off = ks * 256;
                const uint32_t first = (kc == 0 && ks == 0) ? 0u : 1u;
                const uint64_t dar = make_desc(ar + off, 128, 1024), dai = make_desc(ai + off, 128, 1024);
                const uint64_t dbr = make_desc(br + off, 128, 1024), dbi = make_desc(bi + off, 128, 1024);
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(dre),
                    "l"(dar), "l"(dbr), "r"(id), "r"(first)
                    : "memory");
                asm volatile("tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, 1;" ::"r"(dre), "l"(dai), "l"(dbi),
                             "r"(idneg)
                             : "memory");
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(dim),
                    "l"(dar), "l"(dbi), "r"(id), "r"(first)
                    : "memory");
                asm volatile("tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, 1;" ::"r"(dim), "l"(dai), "l"(dbr),
                             "r"(id)
                             : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb)
                         : "memory");
        }
        __syncthreads();
        if (!s_fail) {
            if (!mbar_wait(mb, phase)) s_fail = 1;
        }
        phase ^= 1;
        __syncthreads();
        if (s_fail) break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!s_fail) {
        const uint32_t lane_addr = taddr + ((uint32_t)(warp * 32) << 16);
        const int64_t r = r0 + warp * 32 + lane;
#pragma unroll
        for (int cb = 0; cb < kN; cb += 16) {
            uint32_t vr[16], vi[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                "%14, %15}, [%16];"
                : "=r"(vr[0]), "=r"(vr[1]), "=r"(vr[2]), "=r"(vr[3]), "=r"(vr[4]), "=r"(vr[5]), "=r"(vr[6]),
                  "=r"(vr[7]), "=r"(vr[8]), "=r"(vr[9]), "=r"(vr[10]), "=r"(vr[11]), "=r"(vr[12]), "=r"(vr[13]),
                  "=r"(vr[14]), "=r"(vr[15])
                : "r"(lane_addr + (uint32_t)cb)
                : "memory");
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                "%14, %15}, [%16];"
                : "=r"(vi[0]), "=r"(vi[1]), "=r"(vi[2]), "=r"(vi[3]), "=r"(vi[4]), "=r"(vi[5]), "=r"(vi[6]),
                  "=r"(vi[7]), "=r"(vi[8]), "=r"(vi[9]), "=r"(vi[10]), "=r"(vi[11]), "=r"(vi[12]), "=r"(vi[13]),
                  "=r"(vi[14]), "=r"(vi[15])
                : "r"(lane_addr + kTmemCols + (uint32_t)cb)
                : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (r < w) {
#pragma unroll
                for (int c = 0; c < 16; ++c) {
                    if (cb + c < ncl) {
                        float2& o = Out[(row0 + r) * Bc + g.col0 + c0 + cb + c];
                        const float2 res = make_float2(alpha * __uint_as_float(vr[c]), alpha * __uint_as_float(vi[c]));
                        if (beta) { o.x += res.x; o.y += res.y; }
                        else o = res;
                    }
                }
            }
        }
    } else if (tid == 0) {
        mbar_wait(mb, phase ^ 1);
        atomicExch(status, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(2 * kTmemCols)
                     : "memory");
}

// BF16 GEMM of the warm-start network (tcgen05 kind::f16, FP32 accumulation in TMEM):
// C[m][n] = sum_k A(m,k) B(k,n) (+ bias[n]) with A(m,k) = a[m sam + k sak] and
// B(k,n) = b[k sbk + n sbn], so one kernel serves the forward product and both
// backward products (transposes by strides).  One CTA of 128 threads owns a 128 x 64
// tile of C: 64-wide K chunks of A and B are staged by all threads into the canonical
// K-major layout (8-row x 16-byte core matrices, the same byte geometry as the TF32
// tiles above), one thread issues four MMAs (K = 16 each) per chunk, and every wait is
// bounded (a time-out sets *status, sticky, and skips the rest of the tile).
constexpr int kBfK = 64;   // K chunk (128 bytes of BF16 per row)
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}
__device__ __forceinline__ uint32_t bf_off(int r, int k) {   // byte offset of (r, k) in a [rows x 64] tile
    return (uint32_t)(((r >> 3) * (kBfK / 8) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

__global__ void __launch_bounds__(kThreads) k_gemm_bf16_tc(int M, int N, int K, const __nv_bfloat16* __restrict__ a,
                                                           int sam, int sak, const __nv_bfloat16* __restrict__ b,
                                                           int sbk, int sbn, const float* __restrict__ bias,
                                                           float* __restrict__ C, int ldc,
                                                           int32_t* __restrict__ status) {
    __shared__ __align__(1024) __nv_bfloat16 sa[kM * kBfK];
    __shared__ __align__(1024) __nv_bfloat16 sb[kN * kBfK];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    __shared__ int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * kM, n0 = blockIdx.x * kN;
    if (tid == 0) {
        s_fail = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = tmem_base;
    const uint32_t mb = smem_u32(&mbar);
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    // operands contiguous along K (16-byte aligned rows, K a multiple of 8) are staged
    // 8 elements (one core-matrix row) per load; others element by element
    const bool avec = sak == 1 && sam % 8 == 0 && K % 8 == 0 && (reinterpret_cast<uintptr_t>(a) & 15) == 0;
    const bool bvec = sbk == 1 && sbn % 8 == 0 && K % 8 == 0 && (reinterpret_cast<uintptr_t>(b) & 15) == 0;
    uint32_t phase = 0;
    const int nk = (K + kBfK - 1) / kBfK;
    for (int kc = 0; kc < nk; ++kc) {
        const int k0 = kc * kBfK;
        if (avec) {
            for (int idx = tid; idx < kM * (kBfK / 8); idx += kThreads) {
                const int r = idx / (kBfK / 8), k = (idx % (kBfK / 8)) * 8;
                const int gm = m0 + r, gk = k0 + k;
                *reinterpret_cast<uint4*>(reinterpret_cast<char*>(sa) + bf_off(r, k)) =
                    (gm < M && gk < K) ? *reinterpret_cast<const uint4*>(a + (size_t)gm * sam + gk)
                                       : make_uint4(0u, 0u, 0u, 0u);
            }
        } else {
            for (int idx = tid; idx < kM * kBfK; idx += kThreads) {
                const int r = idx / kBfK, k = idx % kBfK;
                const int gm = m0 + r, gk = k0 + k;
                *reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<char*>(sa) + bf_off(r, k)) =
                    (gm < M && gk < K) ? a[(size_t)gm * sam + (size_t)gk * sak] : zero;
            }
        }
        if (bvec) {
            for (int idx = tid; idx < kN * (kBfK / 8); idx += kThreads) {
                const int n = idx / (kBfK / 8), k = (idx % (kBfK / 8)) * 8;
                const int gn = n0 + n, gk = k0 + k;
                *reinterpret_cast<uint4*>(reinterpret_cast<char*>(sb) + bf_off(n, k)) =
                    (gn < N && gk < K) ? *reinterpret_cast<const uint4*>(b + (size_t)gn * sbn + gk)
                                       : make_uint4(0u, 0u, 0u, 0u);
            }
        } else {
            for (int idx = tid; idx < kN * kBfK; idx += kThreads) {
                const int n = idx / kBfK, k = idx % kBfK;
                const int gn = n0 + n, gk = k0 + k;
                *reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<char*>(sb) + bf_off(n, k)) =
                    (gn < N && gk < K) ? b[(size_t)gk * sbk + (size_t)gn * sbn] : zero;
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (tid == 0 && !s_fail) {
            const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
            const uint32_t idesc = idesc_bf16(kM, kN);
#pragma unroll
            for (int ks = 0; ks < kBfK / 16; ++ks) {
                // K = 16 BF16 = two core matrices along K: +256 B per step
                const uint64_t ad = make_desc(a0 + ks * 256, 128, 1024);
                const uint64_t bd = make_desc(b0 + ks * 256, 128, 1024);
                const uint32_t acc = (kc > 0 || ks > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(taddr),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb)
                         : "memory");
        }
        __syncthreads();
        if (!s_fail) {
            if (!mbar_wait(mb, phase)) s_fail = 1;
        }
        phase ^= 1;
        __syncthreads();
        if (s_fail) break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!s_fail) {
        const uint32_t lane_addr = taddr + ((uint32_t)(warp * 32) << 16);
        const int row = m0 + warp * 32 + lane;
#pragma unroll
        for (int c0 = 0; c0 < kN; c0 += 16) {
            uint32_t v[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                "%14, %15}, [%16];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15])
                : "r"(lane_addr + (uint32_t)c0)
                : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row < M) {
#pragma unroll
                for (int c = 0; c < 16; ++c) {
                    const int n = n0 + c0 + c;
                    if (n < N) C[(size_t)row * ldc + n] = __uint_as_float(v[c]) + (bias ? bias[n] : 0.f);
                }
            }
        }
    } else if (tid == 0) {
        mbar_wait(mb, phase ^ 1);   // one more bounded wait for the committed MMAs before the TMEM goes
        atomicExch(status, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(kTmemCols) : "memory");
}

// Rank-64 update of the block Gauss-Jordan inversion on the tensor cores, in
// FP32-equivalent precision: M[r, c] -= M[r, K] M[K, c] over a 128-row x 64-column
// block of the w x w complex64 matrix M (row-major, interleaved), K = the 64 columns /
// rows of pivot tile k.  Each operand x is split as hi = tf32(x) and lo = x - hi, and
// the product is accumulated from hi*hi + hi*lo + lo*hi (the lo*lo term is below FP32
// rounding), i.e. 12 MMAs (M = 128, N = 64, K = 8) per K step of 8 for the four real
// products of the complex one: the real accumulator (TMEM columns 0-63) takes
// Re*Re - Im*Im (negation in the instruction descriptor), the imaginary one (columns
// 64-127) Re*Im + Im*Re.
// One CTA of 256 threads per SM:
//   1. every thread loads its share of both operands (all 64 K) into registers, so
//      the whole block's loads are in flight at once;
//   2. they are split and stored as two 32-wide K chunks (192 KB of shared memory in
//      the canonical K-major layout; a half-warp stores one 8 x 4 core matrix);
//   3. one thread issues the 96 MMAs; meanwhile every thread loads its part of the
//      output block (coalesced rows);
//   4. the accumulators go TMEM -> shared memory, and the output block is written
//      back minus the product.
// Rows of tile k, and tile (la, la) when la >= 0, keep their values.  Grid: column
// tiles x row blocks of 128 x F (column tile k returns at once).
constexpr int kUpdM = 128, kUpdN = 64, kUpdTile = 64, kUpdThreads = 256;
constexpr int kUpdATile = kUpdM * kK * 4;                  // one 128 x 32 FP32 tile: 16 KB
constexpr int kUpdBTile = kUpdN * kK * 4;                  // one 64 x 32 FP32 tile: 8 KB
constexpr int kUpdChunk = 4 * kUpdATile + 4 * kUpdBTile;   // one K chunk: 96 KB
constexpr int kUpdSmem = 2 * kUpdChunk;                    // the epilogue reuses 66.5 KB of it
constexpr int kUpdLd = kUpdN + 1;                          // row stride of the staged product (float2)

__device__ __forceinline__ float tf32_hi(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__global__ void __launch_bounds__(kUpdThreads, 1) k_gj_update_tc(int64_t w, int k, int la, float2* __restrict__ Sinv,
                                                                  int64_t totD, int64_t offD,
                                                                  int32_t* __restrict__ status) {
    extern __shared__ __align__(1024) unsigned char dsm[];
    char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(dsm) + 1023) & ~(uintptr_t)1023);
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    __shared__ int s_fail;
    const int cx = (int)blockIdx.x;
    if (cx == k) return;               // uniform per CTA, before any TMEM allocation
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    float2* M = Sinv + (int64_t)blockIdx.z * totD + offD;
    const int64_t r0 = (int64_t)blockIdx.y * kUpdM, c0 = (int64_t)cx * kUpdN, k0 = (int64_t)k * kUpdTile;
    const int tb = (int)min((int64_t)kUpdTile, w - k0);
    const float2 z2 = make_float2(0.f, 0.f);
    if (tid == 0) {
        s_fail = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(2 * kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    // 1. operand loads.  A: warp item wi = warp + 8 it (it < 16) is row block wi / 8 and
    //    8-wide K block wi % 8; lane -> row (lane & 15) >> 1, K pair 2 (lane & 1) + 4 (lane >> 4).
    //    B: item wi = warp + 8 it (it < 8) is 16-wide column block wi / 16 and 4-deep K
    //    block wi % 16; lane -> column pair 2 (lane & 3) + 8 (lane >> 4), K (lane >> 2) & 3.
    const int ar = (lane & 15) >> 1, aq = ((lane & 1) << 1) + ((lane >> 4) << 2);
    const int bp = ((lane & 3) << 1) + ((lane >> 4) << 3), bk = (lane >> 2) & 3;
    float2 va[16][2], vb[8][2];
#pragma unroll
    for (int it = 0; it < 16; ++it) {
        const int wi = warp + 8 * it;
        const int64_t gr = r0 + (wi >> 3) * 8 + ar;
        const int kk = (wi & 7) * 8 + aq;
        const float2* src = M + gr * w + k0 + kk;
        va[it][0] = (gr < w && kk < tb) ? src[0] : z2;
        va[it][1] = (gr < w && kk + 1 < tb) ? src[1] : z2;
    }
#pragma unroll
    for (int it = 0; it < 8; ++it) {
        const int wi = warp + 8 * it;
        const int kk = (wi & 15) * 4 + bk;
        const int64_t gc = c0 + (wi >> 4) * 16 + bp;
        const float2* src = M + (k0 + kk) * w + gc;
        vb[it][0] = (kk < tb && gc < w) ? src[0] : z2;
        vb[it][1] = (kk < tb && gc + 1 < w) ? src[1] : z2;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = tmem_base;
    const uint32_t mb = smem_u32(&mbar);
    // 2. split and store: chunk kk / 32, tiles re hi, re lo, im hi, im lo (A then B)
#pragma unroll
    for (int it = 0; it < 16; ++it) {
        const int wi = warp + 8 * it;
        const int kk = (wi & 7) * 8 + aq, kc = kk & 31;
        char* cb = base + (kk >> 5) * kUpdChunk;
        const uint32_t o = (uint32_t)((((wi >> 3) * (kK / 4) + (kc >> 2)) * 128) + ar * 16 + (kc & 3) * 4);
        const float2 x0 = va[it][0], x1 = va[it][1];
        const float r0h = tf32_hi(x0.x), r1h = tf32_hi(x1.x), i0h = tf32_hi(x0.y), i1h = tf32_hi(x1.y);
        *reinterpret_cast<float2*>(cb + 0 * kUpdATile + o) = make_float2(r0h, r1h);
        *reinterpret_cast<float2*>(cb + 1 * kUpdATile + o) = make_float2(x0.x - r0h, x1.x - r1h);
        *reinterpret_cast<float2*>(cb + 2 * kUpdATile + o) = make_float2(i0h, i1h);
        *reinterpret_cast<float2*>(cb + 3 * kUpdATile + o) = make_float2(x0.y - i0h, x1.y - i1h);
    }
#pragma unroll
    for (int it = 0; it < 8; ++it) {
        const int wi = warp + 8 * it;
        const int kk = (wi & 15) * 4 + bk, kc = kk & 31;
        char* cb = base + (kk >> 5) * kUpdChunk + 4 * kUpdATile;
        const int n = (wi >> 4) * 16 + bp;
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int ne = n + e;
            const uint32_t o = (uint32_t)((((ne >> 3) * (kK / 4) + (kc >> 2)) * 128) + (ne & 7) * 16 + (kc & 3) * 4);
            const float2 x = vb[it][e];
            const float rh = tf32_hi(x.x), ih = tf32_hi(x.y);
            *reinterpret_cast<float*>(cb + 0 * kUpdBTile + o) = rh;
            *reinterpret_cast<float*>(cb + 1 * kUpdBTile + o) = x.x - rh;
            *reinterpret_cast<float*>(cb + 2 * kUpdBTile + o) = ih;
            *reinterpret_cast<float*>(cb + 3 * kUpdBTile + o) = x.y - ih;
        }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // 3. the MMAs (one thread), then every thread loads its part of the output block:
    //    element (idx / 64, idx % 64), idx = tid + 256 q
    if (tid == 0) {
        const uint32_t id = idesc_tf32(kUpdM, kUpdN), idneg = id | (1u << 13);
        const uint32_t dre = taddr, dim = taddr + kTmemCols;
#pragma unroll
        for (int ch = 0; ch < 2; ++ch) {
            const uint32_t a0 = smem_u32(base + ch * kUpdChunk), b0 = a0 + 4 * kUpdATile;
#pragma unroll
            for (int ks = 0; ks < kK / 8; ++ks) {
                const uint32_t off = ks * 256;
                const uint64_t arh = make_desc(a0 + 0 * kUpdATile + off, 128, 1024);
                const uint64_t arl = make_desc(a0 + 1 * kUpdATile + off, 128, 1024);
                const uint64_t aih = make_desc(a0 + 2 * kUpdATile + off, 128, 1024);
                const uint64_t ail = make_desc(a0 + 3 * kUpdATile + off, 128, 1024);
                const uint64_t brh = make_desc(b0 + 0 * kUpdBTile + off, 128, 1024);
                const uint64_t brl = make_desc(b0 + 1 * kUpdBTile + off, 128, 1024);
                const uint64_t bih = make_desc(b0 + 2 * kUpdBTile + off, 128, 1024);
                const uint64_t bil = make_desc(b0 + 3 * kUpdBTile + off, 128, 1024);
                const uint32_t first = (ch == 0 && ks == 0) ? 0u : 1u;
#define EMG_UMMA(D, A, B, ID, ACC)                                                              \
    asm volatile(                                                                               \
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"                                       \
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(D), "l"(A), "l"(B), \
        "r"(ID), "r"(ACC)                                                                       \
        : "memory")
                EMG_UMMA(dre, arh, brh, id, first);
                EMG_UMMA(dre, arh, brl, id, 1u);
                EMG_UMMA(dre, arl, brh, id, 1u);
                EMG_UMMA(dre, aih, bih, idneg, 1u);
                EMG_UMMA(dre, aih, bil, idneg, 1u);
                EMG_UMMA(dre, ail, bih, idneg, 1u);
                EMG_UMMA(dim, arh, bih, id, first);
                EMG_UMMA(dim, arh, bil, id, 1u);
                EMG_UMMA(dim, arl, bih, id, 1u);
                EMG_UMMA(dim, aih, brh, id, 1u);
                EMG_UMMA(dim, aih, brl, id, 1u);
                EMG_UMMA(dim, ail, brh, id, 1u);
#undef EMG_UMMA
            }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb)
                     : "memory");
    }
    constexpr int kQ = kUpdM * kUpdN / kUpdThreads;   // 32 output entries per thread
    float2 vc[kQ];
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
        const int idx = tid + kUpdThreads * q;
        const int64_t gr = r0 + idx / kUpdN, gc = c0 + idx % kUpdN;
        vc[q] = (gr < w && gc < w) ? M[gr * w + gc] : z2;
    }
    if (!mbar_wait(mb, 0u)) s_fail = 1;
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // 4. warp w reads TMEM lanes 32 (w % 4) .. + 31 (rows), columns 32 (w / 4) .. + 31
    if (!s_fail) {
        float2* P = reinterpret_cast<float2*>(base);
        const int row = (warp & 3) * 32 + lane, ch0 = (warp >> 2) * 32;
        const uint32_t lane_addr = taddr + ((uint32_t)((warp & 3) * 32) << 16);
#pragma unroll
        for (int cb = 0; cb < 32; cb += 16) {
            uint32_t vr[16], vi[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                "%14, %15}, [%16];"
                : "=r"(vr[0]), "=r"(vr[1]), "=r"(vr[2]), "=r"(vr[3]), "=r"(vr[4]), "=r"(vr[5]), "=r"(vr[6]),
                  "=r"(vr[7]), "=r"(vr[8]), "=r"(vr[9]), "=r"(vr[10]), "=r"(vr[11]), "=r"(vr[12]), "=r"(vr[13]),
                  "=r"(vr[14]), "=r"(vr[15])
                : "r"(lane_addr + (uint32_t)(ch0 + cb))
                : "memory");
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                "%14, %15}, [%16];"
                : "=r"(vi[0]), "=r"(vi[1]), "=r"(vi[2]), "=r"(vi[3]), "=r"(vi[4]), "=r"(vi[5]), "=r"(vi[6]),
                  "=r"(vi[7]), "=r"(vi[8]), "=r"(vi[9]), "=r"(vi[10]), "=r"(vi[11]), "=r"(vi[12]), "=r"(vi[13]),
                  "=r"(vi[14]), "=r"(vi[15])
                : "r"(lane_addr + kTmemCols + (uint32_t)(ch0 + cb))
                : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int c = 0; c < 16; ++c)
                P[row * kUpdLd + ch0 + cb + c] = make_float2(__uint_as_float(vr[c]), __uint_as_float(vi[c]));
        }
    }
    __syncthreads();
    if (!s_fail) {
        const float2* P = reinterpret_cast<const float2*>(base);
        const int64_t lr0 = (int64_t)la * kUpdTile;                   // rows of tile la
        const bool lacol = la >= 0 && cx == la;
#pragma unroll
        for (int q = 0; q < kQ; ++q) {
            const int idx = tid + kUpdThreads * q;
            const int r = idx / kUpdN, c = idx % kUpdN;
            const int64_t gr = r0 + r, gc = c0 + c;
            if (gr >= w || gc >= w || (gr >= k0 && gr < k0 + kUpdTile) || (lacol && gr >= lr0 && gr < lr0 + kUpdTile))
                continue;
            const float2 d = P[r * kUpdLd + c];
            M[gr * w + gc] = make_float2(vc[q].x - d.x, vc[q].y - d.y);
        }
    } else if (tid == 0) {
        mbar_wait(mb, 0u);   // one more bounded wait for the committed MMAs before the TMEM goes
        atomicExch(status, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(2 * kTmemCols)
                     : "memory");
}

}  // namespace tc
}  // namespace emg

// Launch hook for the slab solve (declared in emg_krylov.cuh).
namespace emg {
int tc_slab_product(int64_t w, int64_t row0, int64_t Bc, const void* groups, int G, int maxcol, const float2* Sinv,
                    int64_t totD, int64_t offD, const float2* Y, float alpha, int beta, float2* Out, int32_t* status,
                    cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        EMG_CUDA(cudaFuncSetAttribute(tc::k_cgemm_tf32, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::kCxSmem + 1024));
        attr = true;
    }
    const dim3 grid((unsigned)((maxcol + tc::kN - 1) / tc::kN), (unsigned)((w + tc::kM - 1) / tc::kM), (unsigned)G);
    tc::k_cgemm_tf32<<<grid, tc::kThreads, tc::kCxSmem + 1024, st>>>(
        w, row0, Bc, static_cast<const tc::TcGroup*>(groups), Sinv, totD, offD, Y, alpha, beta, Out, status);
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}
}  // namespace emg

// BF16 GEMM of the warm-start network on the tensor cores (declared in emg_mlp.cu).
namespace emg {
int tc_gemm_bf16(int M, int N, int K, const __nv_bfloat16* a, int sam, int sak, const __nv_bfloat16* b, int sbk,
                 int sbn, const float* bias, float* C, int ldc, int32_t* status, cudaStream_t st) {
    const dim3 grid((unsigned)((N + tc::kN - 1) / tc::kN), (unsigned)((M + tc::kM - 1) / tc::kM));
    tc::k_gemm_bf16_tc<<<grid, tc::kThreads, 0, st>>>(M, N, K, a, sam, sak, b, sbk, sbn, bias, C, ldc, status);
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}
}  // namespace emg

// Rank-64 Gauss-Jordan update of step k on the tensor cores (declared in emg_krylov.cuh).
namespace emg {
int tc_gj_update(int64_t w, int k, int la, int64_t F, float2* Sinv, int64_t totD, int64_t offD, int32_t* status,
                 cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        EMG_CUDA(cudaFuncSetAttribute(tc::k_gj_update_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      tc::kUpdSmem + 1024));
        attr = true;
    }
    const dim3 grid((unsigned)((w + tc::kUpdN - 1) / tc::kUpdN), (unsigned)((w + tc::kUpdM - 1) / tc::kUpdM),
                    (unsigned)F);
    tc::k_gj_update_tc<<<grid, tc::kUpdThreads, tc::kUpdSmem + 1024, st>>>(w, k, la, Sinv, totD, offD, status);
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}
}  // namespace emg

extern "C" int emg_tc_gemm_tf32(int64_t M, int64_t N, int64_t K, const float* A, int64_t lda, const float* B,
                                int64_t ldb, float* D, int64_t ldd, int32_t* status, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(A && B && D && status && M > 0 && N > 0 && K > 0 && lda >= K && ldb >= K && ldd >= N,
                  "emg_tc_gemm_tf32: bad argument");
    const dim3 grid((unsigned)((N + tc::kN - 1) / tc::kN), (unsigned)((M + tc::kM - 1) / tc::kM));
    tc::k_gemm_tf32<<<grid, tc::kThreads, 0, (cudaStream_t)stream>>>(M, N, K, A, lda, B, ldb, D, ldd, status);
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}
