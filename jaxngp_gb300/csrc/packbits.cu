// Occupancy bitfield packing for sm_103a.
//
// Replaces volume-rendering-jax/lib/impl/packbits.cu:9-34 (pack_bits_kernel) behind the same
// ABI: cell 8*i+k is occupied when density > threshold, and is bit k of byte i.  Each thread
// packs one byte from two float4 loads of the density and of the threshold and writes the eight
// mask bytes as one 8-byte store.  A second entry takes the threshold as one device scalar, so
// the occupancy-grid refresh does not materialise a per-cell threshold array.
#include "common.cuh"

namespace ngp {
namespace {

template <bool kScalarThreshold>
__global__ void pack_bits_kernel(std::uint32_t n_bytes, const float *__restrict__ thr,
                                 const float *__restrict__ density, bool *__restrict__ mask,
                                 std::uint8_t *__restrict__ bits) {
    const std::size_t stride = (std::size_t)gridDim.x * blockDim.x;
    const float t_scalar = kScalarThreshold ? *thr : 0.f;
    for (std::size_t i = (std::size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_bytes; i += stride) {
        const float4 d0 = reinterpret_cast<const float4 *>(density)[2 * i];
        const float4 d1 = reinterpret_cast<const float4 *>(density)[2 * i + 1];
        float4 t0, t1;
        if (kScalarThreshold) {
            t0 = t1 = make_float4(t_scalar, t_scalar, t_scalar, t_scalar);
        } else {
            t0 = reinterpret_cast<const float4 *>(thr)[2 * i];
            t1 = reinterpret_cast<const float4 *>(thr)[2 * i + 1];
        }
        const unsigned p0 = d0.x > t0.x, p1 = d0.y > t0.y, p2 = d0.z > t0.z, p3 = d0.w > t0.w;
        const unsigned p4 = d1.x > t1.x, p5 = d1.y > t1.y, p6 = d1.z > t1.z, p7 = d1.w > t1.w;
        bits[i] = (std::uint8_t)(p0 | (p1 << 1) | (p2 << 2) | (p3 << 3) | (p4 << 4) | (p5 << 5) | (p6 << 6) | (p7 << 7));
        const unsigned lo = p0 | (p1 << 8) | (p2 << 16) | (p3 << 24);
        const unsigned hi = p4 | (p5 << 8) | (p6 << 16) | (p7 << 24);
        reinterpret_cast<uint2 *>(mask)[i] = make_uint2(lo, hi);
    }
}

}  // namespace

int launch_packbits(cudaStream_t stream, std::uint32_t n_bytes, const float *thr,
                    const float *density, bool *mask, std::uint8_t *bits, bool scalar_threshold) {
    NGP_CHECK_ARG(n_bytes > 0, "packbits: n_bytes must be a positive integer");
    NGP_CHECK_ARG(((std::uintptr_t)density & 15u) == 0 && ((std::uintptr_t)mask & 7u) == 0 &&
                      (scalar_threshold || ((std::uintptr_t)thr & 15u) == 0),
                  "packbits: density/threshold must be 16-byte aligned and the mask 8-byte aligned");
    const unsigned grid = grid_for(n_bytes, 256, 8);
    if (scalar_threshold) {
        pack_bits_kernel<true><<<grid, 256, 0, stream>>>(n_bytes, thr, density, mask, bits);
        count_launches(1);
    }
    else {
        pack_bits_kernel<false><<<grid, 256, 0, stream>>>(n_bytes, thr, density, mask, bits);
        count_launches(1);
    }
    return launch_status();
}

}  // namespace ngp
