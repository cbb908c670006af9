// Small MLP for the sweep warm start: BF16 weights and activations on the tcgen05
// tensor cores (kind::f16, FP32 accumulation in tensor memory; emg_tc.cu), FP32 master
// weights and Adam.
//
// The network maps features of (normalised frequency, port) to the coefficients
// of the sweep's converged-solution basis.  All GEMMs of the forward and the
// backward pass are one kernel (tc_gemm_bf16) with explicit strides:
//   forward   Z = H W^T + b         (batch x n) = (batch x k)(k x n)
//   weights   dW = dZ^T H           (n x k)     = (n x batch)(batch x k)
//   inputs    dH = dZ W             (batch x k) = (batch x n)(n x k)
// The problem sizes (<= a few hundred rows, 128 wide) make it launch-bound, so one
// 128 x 64 output tile per CTA with unpipelined staging is enough.  A tensor-core wait
// that runs out sets a sticky status, which the forward and the gradient requests
// report.
#include <cuda_bf16.h>

#include <cmath>
#include <vector>

#include "emg_common.cuh"

namespace emg {
// tcgen05 BF16 GEMM (emg_tc.cu): C[m][n] = sum_k A(m,k) B(k,n) (+ bias[n]),
// A(m,k) = a[m*sam + k*sak], B(k,n) = b[k*sbk + n*sbn]; *status (device) set to 1 if a
// bounded wait ran out.
int tc_gemm_bf16(int M, int N, int K, const __nv_bfloat16* a, int sam, int sak, const __nv_bfloat16* b, int sbk,
                 int sbn, const float* bias, float* C, int ldc, int32_t* status, cudaStream_t st);
namespace mlp {

// H = tanh(Z) in bf16 (act = 1) or H = Z in bf16 (act = 0)
__global__ void k_act(int n, const float* __restrict__ Z, int act, __nv_bfloat16* __restrict__ H) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        H[i] = __float2bfloat16_rn(act ? tanhf(Z[i]) : Z[i]);
}

// dZ = dH * (1 - tanh(Z)^2), as bf16 for the next GEMMs and fp32 for the bias gradient
__global__ void k_act_back(int n, const float* __restrict__ dH, const float* __restrict__ Z,
                           __nv_bfloat16* __restrict__ dZb, float* __restrict__ dZf) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float th = tanhf(Z[i]);
        const float v = dH[i] * (1.f - th * th);
        dZf[i] = v;
        dZb[i] = __float2bfloat16_rn(v);
    }
}

// Loss and its gradient: mean over the valid (rows < nb, cols < nout) entries of (Y - T)^2.
__global__ void k_loss(int nb, int nout, int ldy, const float* __restrict__ Y, const float* __restrict__ T,
                       float* __restrict__ dYf, __nv_bfloat16* __restrict__ dYb, float* __restrict__ loss, int rows_pad) {
    __shared__ float red[256];
    float s = 0.f;
    const float scale = 1.f / (float)(nb * nout);
    for (int i = threadIdx.x; i < rows_pad * ldy; i += blockDim.x) {
        const int r = i / ldy, c = i % ldy;
        float d = 0.f;
        if (r < nb && c < nout) {
            d = Y[i] - T[r * nout + c];
            s += d * d;
        }
        dYf[i] = 2.f * d * scale;
        dYb[i] = __float2bfloat16_rn(2.f * d * scale);
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *loss = red[0] * scale;
}

// db[n] = sum over rows of dZ[r][n] (rows < nb)
__global__ void k_bias_grad(int nb, int n, const float* __restrict__ dZ, float* __restrict__ db) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    float s = 0.f;
    for (int r = 0; r < nb; ++r) s += dZ[r * n + j];
    db[j] = s;
}

// Adam on the fp32 master parameters; refresh the bf16 weight copy.
__global__ void k_adam(int n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, float lr, float b1, float b2, float eps, float c1, float c2,
                       __nv_bfloat16* __restrict__ wb) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float a = b1 * m1[i] + (1.f - b1) * gi;
        const float v = b2 * m2[i] + (1.f - b2) * gi * gi;
        m1[i] = a;
        m2[i] = v;
        w[i] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
        wb[i] = __float2bfloat16_rn(w[i]);
    }
}

__global__ void k_to_bf16(int n, const float* __restrict__ x, __nv_bfloat16* __restrict__ y) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        y[i] = __float2bfloat16_rn(x[i]);
}

// pad rows/cols: dst (rows_pad x ld) from src (nb x ncols), zero elsewhere
__global__ void k_pad_in(int nb, int ncols, int rows_pad, int ld, const float* __restrict__ src,
                         __nv_bfloat16* __restrict__ dst) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rows_pad * ld; i += gridDim.x * blockDim.x) {
        const int r = i / ld, c = i % ld;
        dst[i] = __float2bfloat16_rn((r < nb && c < ncols) ? src[r * ncols + c] : 0.f);
    }
}

__global__ void k_unpad_out(int nb, int ncols, int ld, const float* __restrict__ src, float* __restrict__ dst) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nb * ncols; i += gridDim.x * blockDim.x)
        dst[i] = src[(i / ncols) * ld + i % ncols];
}

}  // namespace mlp
}  // namespace emg

// ------------------------------------------------------------------ C ABI ---
struct emg_mlp {
    int in = 0, hidden = 0, layers = 0, out = 0;        // layers = hidden layers
    int in_pad = 0, out_pad = 0, max_batch = 0;
    std::vector<int> K, N;                               // per linear layer
    std::vector<size_t> woff, boff;                      // offsets into the flat parameter array
    size_t nparam = 0;
    float* w = nullptr;                                  // fp32 master (weights and biases)
    float* g = nullptr;                                  // gradients
    float* m1 = nullptr;
    float* m2 = nullptr;
    __nv_bfloat16* wb = nullptr;                         // bf16 copy
    // activations: per layer l input H_l (bf16), pre-activation Z_l (fp32)
    std::vector<__nv_bfloat16*> H;
    std::vector<float*> Z;
    float* dYf = nullptr;
    __nv_bfloat16* dYb = nullptr;
    float* dH = nullptr;
    float* dZf = nullptr;
    __nv_bfloat16* dZb = nullptr;
    int32_t* tcstat = nullptr;                           // sticky tensor-core time-out flag
    int step = 0;
};

namespace {
using namespace emg;

void mlp_free(emg_mlp* p) {
    if (!p) return;
    dfree(p->w); dfree(p->g); dfree(p->m1); dfree(p->m2); dfree(p->wb);
    for (auto& h : p->H) dfree(h);
    for (auto& z : p->Z) dfree(z);
    dfree(p->dYf); dfree(p->dYb); dfree(p->dH); dfree(p->dZf); dfree(p->dZb); dfree(p->tcstat);
    delete p;
}

int pad_to(int x, int m) { return (x + m - 1) / m * m; }

int gemm(emg_mlp* p, int M, int N, int K, const __nv_bfloat16* a, int sam, int sak, const __nv_bfloat16* b, int sbk,
         int sbn, const float* bias, float* C, int ldc, cudaStream_t s) {
    return tc_gemm_bf16(M, N, K, a, sam, sak, b, sbk, sbn, bias, C, ldc, p->tcstat, s);
}

// EMG_ERR_CUDA if a tensor-core GEMM of this network has timed out (the flag stays set)
int tc_check(emg_mlp* p, cudaStream_t s) {
    int32_t h = 0;
    EMG_CUDA(cudaMemcpyAsync(&h, p->tcstat, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    EMG_CUDA(cudaStreamSynchronize(s));
    if (h) {
        set_error("mlp: a tensor-core GEMM timed out waiting for its MMAs; the network is not usable");
        return EMG_ERR_CUDA;
    }
    return EMG_OK;
}

// forward pass on padded input H[0] (rows_pad x in_pad); result in Z.back() (rows_pad x out_pad)
int forward(emg_mlp* p, int rows_pad, cudaStream_t s) {
    const int L = (int)p->K.size();
    for (int l = 0; l < L; ++l) {
        int rc = gemm(p, rows_pad, p->N[l], p->K[l], p->H[l], p->K[l], 1, p->wb + p->woff[l], 1, p->K[l],
                      p->w + p->boff[l], p->Z[l], p->N[l], s);
        if (rc) return rc;
        if (l + 1 < L) {
            const int n = rows_pad * p->N[l];
            mlp::k_act<<<(n + 255) / 256, 256, 0, s>>>(n, p->Z[l], 1, p->H[l + 1]);
        }
    }
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}

// backward from dY (already in dYf/dYb), fills p->g
int backward(emg_mlp* p, int nb, int rows_pad, cudaStream_t s) {
    const int L = (int)p->K.size();
    const __nv_bfloat16* dzb = p->dYb;
    const float* dzf = p->dYf;
    for (int l = L - 1; l >= 0; --l) {
        const int n = p->N[l], k = p->K[l];
        // dW = dZ^T H : (n x rows)(rows x k)
        int rc = gemm(p, n, k, rows_pad, dzb, 1, n, p->H[l], k, 1, nullptr, p->g + p->woff[l], k, s);
        if (rc) return rc;
        mlp::k_bias_grad<<<(n + 127) / 128, 128, 0, s>>>(nb, n, dzf, p->g + p->boff[l]);
        if (l > 0) {
            // dH = dZ W : (rows x n)(n x k)
            rc = gemm(p, rows_pad, k, n, dzb, n, 1, p->wb + p->woff[l], k, 1, nullptr, p->dH, k, s);
            if (rc) return rc;
            const int e = rows_pad * k;
            mlp::k_act_back<<<(e + 255) / 256, 256, 0, s>>>(e, p->dH, p->Z[l - 1], p->dZb, p->dZf);
            dzb = p->dZb;
            dzf = p->dZf;
            // the next iteration reads dZ of layer l-1 while writing dH: use separate buffers per step
            // (dH consumed above; dZ buffers hold layer l-1 now)
        }
    }
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}
}  // namespace

extern "C" int emg_mlp_create(int in_dim, int hidden, int hidden_layers, int out_dim, int max_batch, uint64_t seed,
                              emg_mlp** out) {
    using namespace emg;
    EMG_CHECK_ARG(out && in_dim > 0 && hidden > 0 && hidden % 16 == 0 && hidden_layers >= 1 && out_dim > 0 &&
                      max_batch > 0 && max_batch <= 4096 && hidden <= 1024,
                  "emg_mlp_create: bad dimensions (hidden must be a multiple of 16)");
    emg_mlp* p = new emg_mlp();
    p->in = in_dim; p->hidden = hidden; p->layers = hidden_layers; p->out = out_dim;
    p->in_pad = pad_to(in_dim, 16);
    p->out_pad = pad_to(out_dim, 16);
    p->max_batch = pad_to(max_batch, 16);
    p->K.push_back(p->in_pad);
    p->N.push_back(hidden);
    for (int l = 1; l < hidden_layers; ++l) { p->K.push_back(hidden); p->N.push_back(hidden); }
    p->K.push_back(hidden);
    p->N.push_back(p->out_pad);
    size_t off = 0;
    for (size_t l = 0; l < p->K.size(); ++l) {
        p->woff.push_back(off); off += (size_t)p->K[l] * p->N[l];
        p->boff.push_back(off); off += (size_t)p->N[l];
    }
    p->nparam = off;
    auto fail = [&](int rc) { mlp_free(p); return rc; };
    int rc;
    if ((rc = dalloc(&p->w, (int64_t)off, "mlp weights"))) return fail(rc);
    if ((rc = dalloc(&p->g, (int64_t)off, "mlp grads"))) return fail(rc);
    if ((rc = dalloc(&p->m1, (int64_t)off, "mlp adam m"))) return fail(rc);
    if ((rc = dalloc(&p->m2, (int64_t)off, "mlp adam v"))) return fail(rc);
    if ((rc = dalloc(&p->wb, (int64_t)off, "mlp bf16 weights"))) return fail(rc);
    const int R = p->max_batch;
    for (size_t l = 0; l < p->K.size(); ++l) {
        __nv_bfloat16* h = nullptr;
        float* z = nullptr;
        if ((rc = dalloc(&h, (int64_t)R * p->K[l], "mlp H"))) return fail(rc);
        p->H.push_back(h);
        if ((rc = dalloc(&z, (int64_t)R * p->N[l], "mlp Z"))) return fail(rc);
        p->Z.push_back(z);
    }
    const int wmax = std::max(hidden, std::max(p->in_pad, p->out_pad));
    if ((rc = dalloc(&p->dYf, (int64_t)R * p->out_pad, "mlp dY"))) return fail(rc);
    if ((rc = dalloc(&p->dYb, (int64_t)R * p->out_pad, "mlp dY bf16"))) return fail(rc);
    if ((rc = dalloc(&p->dH, (int64_t)R * wmax, "mlp dH"))) return fail(rc);
    if ((rc = dalloc(&p->dZf, (int64_t)R * wmax, "mlp dZ"))) return fail(rc);
    if ((rc = dalloc(&p->dZb, (int64_t)R * wmax, "mlp dZ bf16"))) return fail(rc);
    if ((rc = dalloc(&p->tcstat, 1, "mlp tensor-core status"))) return fail(rc);
    if (cudaMemset(p->tcstat, 0, sizeof(int32_t)) != cudaSuccess) return fail(cuda_status(cudaGetLastError(), "mlp"));
    // deterministic init: uniform(-1/sqrt(K), 1/sqrt(K)) weights from a splitmix64 stream, zero biases
    std::vector<float> h(off, 0.f);
    uint64_t st = seed;
    auto next = [&]() {
        st += 0x9E3779B97F4A7C15ull;
        uint64_t z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    for (size_t l = 0; l < p->K.size(); ++l) {
        const float lim = 1.f / std::sqrt((float)p->K[l]);
        const int kreal = (l == 0) ? in_dim : p->K[l];
        const int nreal = (l + 1 == p->K.size()) ? out_dim : p->N[l];
        for (int n = 0; n < p->N[l]; ++n)
            for (int k = 0; k < p->K[l]; ++k) {
                const double u = (double)(next() >> 11) / 9007199254740992.0;
                h[p->woff[l] + (size_t)n * p->K[l] + k] = (n < nreal && k < kreal) ? (float)((2 * u - 1) * lim) : 0.f;
            }
    }
    if (cudaMemcpy(p->w, h.data(), sizeof(float) * off, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(p->m1, 0, sizeof(float) * off) != cudaSuccess || cudaMemset(p->m2, 0, sizeof(float) * off) != cudaSuccess)
        return fail(cuda_status(cudaGetLastError(), "mlp init"));
    mlp::k_to_bf16<<<(unsigned)((off + 255) / 256), 256>>>((int)off, p->w, p->wb);
    if (cudaDeviceSynchronize() != cudaSuccess) return fail(cuda_status(cudaGetLastError(), "mlp init sync"));
    *out = p;
    return EMG_OK;
}

extern "C" int64_t emg_mlp_nparam(const emg_mlp* p) { return p ? (int64_t)p->nparam : -1; }

extern "C" int emg_mlp_get_params(const emg_mlp* p, float* host_out) {
    using namespace emg;
    EMG_CHECK_ARG(p && host_out, "emg_mlp_get_params: NULL");
    EMG_CUDA(cudaMemcpy(host_out, p->w, sizeof(float) * p->nparam, cudaMemcpyDeviceToHost));
    return EMG_OK;
}

extern "C" int emg_mlp_set_params(emg_mlp* p, const float* host_in) {
    using namespace emg;
    EMG_CHECK_ARG(p && host_in, "emg_mlp_set_params: NULL");
    EMG_CUDA(cudaMemcpy(p->w, host_in, sizeof(float) * p->nparam, cudaMemcpyHostToDevice));
    mlp::k_to_bf16<<<(unsigned)((p->nparam + 255) / 256), 256>>>((int)p->nparam, p->w, p->wb);
    EMG_CUDA(cudaDeviceSynchronize());
    return EMG_OK;
}

extern "C" int emg_mlp_forward(emg_mlp* p, int batch, const float* x, float* y, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(p && x && y && batch > 0 && pad_to(batch, 16) <= p->max_batch, "emg_mlp_forward: bad argument");
    cudaStream_t s = (cudaStream_t)stream;
    const int R = pad_to(batch, 16);
    mlp::k_pad_in<<<(R * p->in_pad + 255) / 256, 256, 0, s>>>(batch, p->in, R, p->in_pad, x, p->H[0]);
    int rc = forward(p, R, s);
    if (rc) return rc;
    mlp::k_unpad_out<<<(batch * p->out + 255) / 256, 256, 0, s>>>(batch, p->out, p->out_pad, p->Z.back(), y);
    EMG_CUDA(cudaGetLastError());
    return tc_check(p, s);
}

// One training step (forward, MSE loss, backward; Adam when lr > 0).  grads_out
// (optional, device, nparam floats) receives the gradient of the loss.
extern "C" int emg_mlp_train_step(emg_mlp* p, int batch, const float* x, const float* target, float lr,
                                  float* loss_out, float* grads_out, void* stream) {
    using namespace emg;
    EMG_CHECK_ARG(p && x && target && loss_out && batch > 0 && pad_to(batch, 16) <= p->max_batch,
                  "emg_mlp_train_step: bad argument");
    cudaStream_t s = (cudaStream_t)stream;
    const int R = pad_to(batch, 16);
    mlp::k_pad_in<<<(R * p->in_pad + 255) / 256, 256, 0, s>>>(batch, p->in, R, p->in_pad, x, p->H[0]);
    int rc = forward(p, R, s);
    if (rc) return rc;
    mlp::k_loss<<<1, 256, 0, s>>>(batch, p->out, p->out_pad, p->Z.back(), target, p->dYf, p->dYb, loss_out, R);
    rc = backward(p, batch, R, s);
    if (rc) return rc;
    if (grads_out) {
        EMG_CUDA(cudaMemcpyAsync(grads_out, p->g, sizeof(float) * p->nparam, cudaMemcpyDeviceToDevice, s));
        if ((rc = tc_check(p, s))) return rc;
    }
    if (lr > 0.f) {
        p->step++;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.f - std::pow(b1, (float)p->step), c2 = 1.f - std::pow(b2, (float)p->step);
        mlp::k_adam<<<(unsigned)((p->nparam + 255) / 256), 256, 0, s>>>((int)p->nparam, p->w, p->g, p->m1, p->m2, lr,
                                                                         b1, b2, 1e-8f, c1, c2, p->wb);
    }
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}

extern "C" void emg_mlp_destroy(emg_mlp* p) { mlp_free(p); }
