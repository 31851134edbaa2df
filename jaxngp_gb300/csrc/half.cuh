// 16-bit floating-point storage types of the mixed-precision entry points: conversions with
// round-to-nearest-even, packing of two values into one 32-bit word, the largest finite value (for
// overflow checks under loss scaling) and the operand format code of tcgen05.mma kind::f16.
#pragma once

#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_fp16.h>

namespace ngp {

struct Bf16Op {
    using T = __nv_bfloat16;
    static constexpr std::uint32_t kFmt = 1;      // kind::f16 operand format: BF16
    static constexpr float kMax = 3.38953139e38f;  // largest finite BF16
    static __device__ __forceinline__ T cvt(float x) { return __float2bfloat16(x); }
    static __device__ __forceinline__ std::uint32_t pack(float a, float b) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        return *reinterpret_cast<const std::uint32_t *>(&h);
    }
    static __device__ __forceinline__ float2 unpack(std::uint32_t w) {
        return __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&w));
    }
};

struct F16Op {
    using T = __half;
    static constexpr std::uint32_t kFmt = 0;  // kind::f16 operand format: FP16
    static constexpr float kMax = 65504.f;    // largest finite FP16
    static __device__ __forceinline__ T cvt(float x) { return __float2half_rn(x); }
    static __device__ __forceinline__ std::uint32_t pack(float a, float b) {
        const __half2 h = __floats2half2_rn(a, b);
        return *reinterpret_cast<const std::uint32_t *>(&h);
    }
    static __device__ __forceinline__ float2 unpack(std::uint32_t w) {
        return __half22float2(*reinterpret_cast<const __half2 *>(&w));
    }
};

// FP32 storage (the reference's type), for templates that take either.
struct F32Op {
    static constexpr float kMax = 3.40282347e38f;
};

}  // namespace ngp
