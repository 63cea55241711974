// Shared definitions for the tpr_gb300 CUDA sources (sm_103a only).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "tpr_gb.h"

#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ < 1000)
#error "tpr_gb300 kernels are written for sm_103a (Blackwell) only"
#endif

namespace tprgb {

// Status reporting (api.cu): records a thread-local message and returns code.
int fail(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);

#define TPRGB_CUDA(call)                                       \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return ::tprgb::cuda_fail(e_, #call); \
    } while (0)

// A launcher's one-time per-device value (a grid size from an occupancy
// query, "attributes set"), shared by every host thread that launches: 0
// until computed.  Publish it only after the work it stands for (e.g.
// cudaFuncSetAttribute) is done; two threads may both compute it, which is
// harmless (the calls are idempotent).
struct DeviceOnce {
    static constexpr int kDevices = 16;
    std::atomic<int> v[kDevices] = {};
    int get(int dev) const {
        return dev >= 0 && dev < kDevices ? v[dev].load(std::memory_order_acquire) : 0;
    }
    void set(int dev, int value) {
        if (dev >= 0 && dev < kDevices) v[dev].store(value, std::memory_order_release);
    }
};

__host__ __device__ constexpr inline bool is_pow2(long long v) {
    return v > 0 && (v & (v - 1)) == 0;
}

__host__ __device__ inline int ilog2(long long v) {
    int r = 0;
    while (v > 1) {
        v >>= 1;
        ++r;
    }
    return r;
}

template <typename T>
struct Eps;
template <>
struct Eps<float> {
    static constexpr float value = 1.1920928955078125e-07f;  // FLT_EPSILON
};
template <>
struct Eps<double> {
    static constexpr double value = 2.220446049250313080847e-16;  // DBL_EPSILON
};

// Device error word: kernels that wait on a barrier with an iteration limit
// record where they gave up here instead of trapping.
struct DeviceStatus {
    unsigned int code;    // 0 = ok, otherwise TPRGB_E*
    unsigned int where;   // kernel-specific site id
    unsigned int detail;  // e.g. the tile or system index
    unsigned int pad;
};

}  // namespace tprgb
