// Error reporting and a device-wide exclusive scan shared by the library.
#include "emg_common.cuh"

namespace emg {

namespace {
thread_local std::string g_last_error;

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int64_t kScanTile = (int64_t)kScanThreads * kScanItems;

// Block-wide exclusive scan of one tile; writes the tile total to tile_sums.
__global__ void k_scan_tiles(const int64_t* __restrict__ in, int64_t* __restrict__ out, int64_t n,
                             int64_t* __restrict__ tile_sums) {
    __shared__ int64_t warp_tot[kScanThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int64_t v[kScanItems];
    int64_t run = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = base + k;
        v[k] = (i < n) ? in[i] : 0;
        const int64_t t = v[k];
        v[k] = run;
        run += t;
    }
    // inclusive warp scan of per-thread totals
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t x = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int64_t w = (lane < kScanThreads / 32) ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kScanThreads / 32) warp_tot[lane] = w;
    }
    __syncthreads();
    const int64_t excl = x - run + (warp > 0 ? warp_tot[warp - 1] : 0);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = base + k;
        if (i < n) out[i] = v[k] + excl;
    }
    if (threadIdx.x == kScanThreads - 1) tile_sums[blockIdx.x] = excl + run;
}

// Sequential-by-chunks exclusive scan of the tile totals in one block.
__global__ void k_scan_sums(int64_t* sums, int64_t ntiles, int64_t* total) {
    __shared__ int64_t warp_tot[kScanThreads / 32];
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int64_t b0 = 0; b0 < ntiles; b0 += kScanThreads) {
        const int64_t i = b0 + threadIdx.x;
        const int64_t v = (i < ntiles) ? sums[i] : 0;
        int64_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int64_t w = (lane < kScanThreads / 32) ? warp_tot[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int64_t y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            if (lane < kScanThreads / 32) warp_tot[lane] = w;
        }
        __syncthreads();
        const int64_t incl = x + (warp > 0 ? warp_tot[warp - 1] : 0);
        const int64_t c = carry;
        if (i < ntiles) sums[i] = c + incl - v;
        __syncthreads();
        if (threadIdx.x == kScanThreads - 1) carry = c + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_add(int64_t* out, int64_t n, const int64_t* tile_sums) {
    const int64_t i = (int64_t)blockIdx.x * kScanTile;
    const int64_t add = tile_sums[blockIdx.x];
    for (int64_t k = threadIdx.x; k < kScanTile; k += blockDim.x)
        if (i + k < n) out[i + k] += add;
}

}  // namespace

void set_error(const std::string& msg) { g_last_error = msg; }
const std::string& last_error() { return g_last_error; }

int cuda_status(cudaError_t e, const char* what) {
    set_error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
    return EMG_ERR_CUDA;
}

int64_t scan_scratch_elems(int64_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

int scan_exclusive_i64(const int64_t* in, int64_t* out, int64_t n, int64_t* scratch, cudaStream_t s) {
    if (n <= 0) {
        EMG_CUDA(cudaMemsetAsync(out, 0, sizeof(int64_t), s));
        return EMG_OK;
    }
    const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    if (ntiles > (int64_t)INT32_MAX) {
        set_error("scan: too many elements");
        return EMG_ERR_LIMIT;
    }
    k_scan_tiles<<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, out, n, scratch);
    k_scan_sums<<<1, kScanThreads, 0, s>>>(scratch, ntiles, out + n);
    k_scan_add<<<(unsigned)ntiles, 256, 0, s>>>(out, n, scratch);
    EMG_CUDA(cudaGetLastError());
    return EMG_OK;
}

}  // namespace emg

extern "C" const char* emg_last_error(void) { return emg::last_error().c_str(); }
extern "C" const char* emg_version(void) { return "emerge_gb300 0.1 (sm_103a)"; }
