// Shared device helpers and the status convention of libngp_gb300.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <cstring>

#include "../../include/ngp_gb300.h"

namespace ngp {

constexpr float kSqrt3 = 1.732050807568877293527446341505872367f;
// Early-stop transmittance of the integrator (integrating.cu:12 of volume-rendering-jax).
constexpr float kTThreshold = 1e-4f;
constexpr int kWarp = 32;

// Number of SMs of the current device, cached per device.
int sm_count();

// Grid size for a grid-stride kernel: enough CTAs for `n` items, at most `per_sm` CTAs per SM.
inline unsigned grid_for(std::size_t n, unsigned block, unsigned per_sm) {
    std::size_t want = (n + block - 1) / block;
    std::size_t cap = (std::size_t)sm_count() * per_sm;
    if (want > cap) want = cap;
    return want == 0 ? 1u : (unsigned)want;
}

// Raises `kernel`'s dynamic shared-memory limit to `bytes` on the current device, once per
// (device, kernel, size); thread-safe.  Returns a status.
int set_smem_limit(const void *kernel, std::size_t bytes);

#define NGP_SMEM_LIMIT(kernel, bytes)                                                      \
    do {                                                                                   \
        const int s_ = ::ngp::set_smem_limit(reinterpret_cast<const void *>(kernel), (bytes)); \
        if (s_ != NGP_OK) return s_;                                                       \
    } while (0)

// Process-wide count of kernel launches made by this library (ngp_kernel_launches()).
void count_launches(unsigned n);

// Status of the last legacy-signature call on this host thread (the legacy signatures return
// void, as XLA custom calls do).
void set_last_status(int status, const char *msg);

#define NGP_CUDA_TRY(expr)                                                                 \
    do {                                                                                   \
        cudaError_t e_ = (expr);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            ::ngp::set_last_status(NGP_ERR_CUDA, cudaGetErrorString(e_));                  \
            return NGP_ERR_CUDA;                                                           \
        }                                                                                  \
    } while (0)

#define NGP_CHECK_ARG(cond, msg)                                                           \
    do {                                                                                   \
        if (!(cond)) {                                                                     \
            ::ngp::set_last_status(NGP_ERR_INVALID_ARGUMENT, msg);                         \
            return NGP_ERR_INVALID_ARGUMENT;                                               \
        }                                                                                  \
    } while (0)

// Read a POD descriptor from the opaque bytes; its length must match exactly (the contract of
// serde-helper/serde.h:31-41, reported as a status instead of an exception).
template <typename T>
inline int read_descriptor(const char *opaque, std::size_t len, T *out) {
    if (opaque == nullptr || len != sizeof(T)) {
        set_last_status(NGP_ERR_OPAQUE_SIZE, "opaque descriptor has the wrong length");
        return NGP_ERR_OPAQUE_SIZE;
    }
    std::memcpy(out, opaque, sizeof(T));
    return NGP_OK;
}

inline int launch_status() {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_status(NGP_ERR_CUDA, cudaGetErrorString(e));
        return NGP_ERR_CUDA;
    }
    set_last_status(NGP_OK, "ok");
    return NGP_OK;
}

// ------------------------------------------------------------------------------ device helpers

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Inclusive prefix sum across the full warp.
__device__ __forceinline__ std::uint32_t warp_inclusive_scan(std::uint32_t v) {
    const unsigned lane = lane_id();
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        std::uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= (unsigned)o) v += t;
    }
    return v;
}

}  // namespace ngp
