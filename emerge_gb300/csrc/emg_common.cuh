// Shared helpers of the emerge_gb300 CUDA library: error reporting, checked
// allocation, and a device-wide exclusive scan.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>

#include "../../include/emerge_gb300.h"

namespace emg {

// Thread-local message of the last failing C-ABI call.
void set_error(const std::string& msg);
const std::string& last_error();

// Returns EMG_ERR_CUDA (and records where) if ``e`` is an error.
int cuda_status(cudaError_t e, const char* what);

#define EMG_CUDA(call)                                                   \
    do {                                                                 \
        cudaError_t _e = (call);                                         \
        if (_e != cudaSuccess) return ::emg::cuda_status(_e, #call);     \
    } while (0)

#define EMG_CHECK_ARG(cond, msg)                 \
    do {                                         \
        if (!(cond)) {                           \
            ::emg::set_error(msg);               \
            return EMG_ERR_ARG;                  \
        }                                        \
    } while (0)

// Device allocation that records the failure instead of throwing.
template <typename T>
int dalloc(T** p, int64_t n, const char* what) {
    *p = nullptr;
    if (n <= 0) return EMG_OK;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * (size_t)n);
    if (e != cudaSuccess) {
        *p = nullptr;
        return cuda_status(e, what);
    }
    return EMG_OK;
}

template <typename T>
void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

// out[i] = sum(in[0..i)) for i in [0, n]; out has n+1 entries.  ``scratch``
// needs scan_scratch_elems(n) int64 entries.
int64_t scan_scratch_elems(int64_t n);
int scan_exclusive_i64(const int64_t* in, int64_t* out, int64_t n, int64_t* scratch, cudaStream_t s);

inline unsigned grid_for(int64_t n, int threads, unsigned cap = 152u * 64u) {
    int64_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    return (unsigned)(b > (int64_t)cap ? cap : b);
}

}  // namespace emg
