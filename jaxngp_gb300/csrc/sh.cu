// Spherical-harmonics direction encoding: the drop-in for the reference's shjax op
// (deps/spherical-harmonics-encoding-jax/lib/impl/spherical_harmonics_encoding.cu, custom-call
// target spherical_harmonics_encoding_cuda_f32, descriptor {n, degree}).
//
// Real spherical harmonics of degrees 0..L-1 (L <= 8, L^2 values) of unit directions, by the
// published closed-form polynomials (those of tiny-cuda-nn that the reference adapts, and of its
// flax SphericalHarmonicsEncoder, models/encoders.py:361-406).  The coefficients are computed on
// the host from their closed forms (k sqrt(m) / (j sqrt(pi))) in double and rounded to float32 --
// the same float32 values as the reference's decimal literals -- and every polynomial keeps the
// reference's order of operations.  This translation unit is compiled with --fmad=false, so each
// operation rounds once, as the flax encoder's float32 ops do: the output is bit-identical to it.
//
// One thread per direction.  A CTA stages its rows in shared memory (row stride L^2 | 1, odd, so
// the per-thread writes do not collide in banks) and stores them as one contiguous block, so the
// global stores are coalesced whatever L is.
#include <cmath>

#include "common.cuh"

namespace ngp {
namespace {

constexpr int kShBlock = 128;

// Coefficient slots (names follow the first output that uses them).
enum : int {
    K0, K1, K4, K6a, K6b, K8, K9, K10, K11, K12, K14, K16, K17, K18, K19, K20a, K20b, K20c, K22, K24a, K24b, K25, K26,
    K27, K28, K29, K30, K32, K34, K36, K37, K38, K39, K40, K41, K42a, K42b, K42c, K42d, K44, K46, K48a, K48b, K49,
    K50, K51, K52, K53, K54, K55, K56, K58, K60, K62, KCount
};

struct ShCoef {
    float k[KCount];
};

ShCoef make_coef() {
    const double s = std::sqrt(3.14159265358979323846);
    auto c = [s](double num, double den) { return (float)(num / (den * s)); };
    ShCoef q{};
    float *k = q.k;
    k[K0] = c(1, 2);                          k[K1] = c(std::sqrt(3.0), 2);
    k[K4] = c(std::sqrt(15.0), 2);            k[K6a] = c(3 * std::sqrt(5.0), 4);
    k[K6b] = c(std::sqrt(5.0), 4);            k[K8] = c(std::sqrt(15.0), 4);
    k[K9] = c(std::sqrt(70.0), 8);            k[K10] = c(std::sqrt(105.0), 2);
    k[K11] = c(std::sqrt(42.0), 8);           k[K12] = c(std::sqrt(7.0), 4);
    k[K14] = c(std::sqrt(105.0), 4);          k[K16] = c(3 * std::sqrt(35.0), 4);
    k[K17] = c(3 * std::sqrt(70.0), 8);       k[K18] = c(3 * std::sqrt(5.0), 4);
    k[K19] = c(3 * std::sqrt(10.0), 8);       k[K20a] = c(-90, 16);
    k[K20b] = c(105, 16);                     k[K20c] = c(9, 16);
    k[K22] = c(3 * std::sqrt(5.0), 8);        k[K24a] = c(-18 * std::sqrt(35.0), 16);
    k[K24b] = c(3 * std::sqrt(35.0), 16);     k[K25] = c(3 * std::sqrt(154.0), 32);
    k[K26] = c(3 * std::sqrt(385.0), 4);      k[K27] = c(-std::sqrt(770.0), 32);
    k[K28] = c(std::sqrt(1155.0), 4);         k[K29] = c(std::sqrt(165.0), 16);
    k[K30] = c(std::sqrt(11.0), 16);          k[K32] = c(std::sqrt(1155.0), 8);
    k[K34] = c(3 * std::sqrt(385.0), 16);     k[K36] = c(std::sqrt(6006.0), 32);
    k[K37] = c(3 * std::sqrt(2002.0), 32);    k[K38] = c(3 * std::sqrt(91.0), 8);
    k[K39] = c(-std::sqrt(2730.0), 32);       k[K40] = c(std::sqrt(2730.0), 32);
    k[K41] = c(std::sqrt(273.0), 16);         k[K42a] = c(105 * std::sqrt(13.0), 32);
    k[K42b] = c(-315 * std::sqrt(13.0), 32);  k[K42c] = c(231 * std::sqrt(13.0), 32);
    k[K42d] = c(-5 * std::sqrt(13.0), 32);    k[K44] = c(std::sqrt(2730.0), 64);
    k[K46] = c(3 * std::sqrt(91.0), 32);      k[K48a] = c(15 * std::sqrt(6006.0), 64);
    k[K48b] = c(std::sqrt(6006.0), 64);       k[K49] = c(3 * std::sqrt(715.0), 64);
    k[K50] = c(3 * std::sqrt(10010.0), 32);   k[K51] = c(-3 * std::sqrt(385.0), 64);
    k[K52] = c(3 * std::sqrt(385.0), 8);      k[K53] = c(-3 * std::sqrt(35.0), 64);
    k[K54] = c(3 * std::sqrt(70.0), 32);      k[K55] = c(std::sqrt(105.0), 64);
    k[K56] = c(std::sqrt(15.0), 32);          k[K58] = c(std::sqrt(70.0), 64);
    k[K60] = c(3 * std::sqrt(385.0), 32);     k[K62] = c(3 * std::sqrt(10010.0), 64);
    return q;
}

// The L^2 values of one direction into o[0 .. L^2).
__device__ __forceinline__ void sh_eval(std::uint32_t L, float x, float y, float z, const float *__restrict__ k,
                                        float *o) {
    const float xy = x * y, xz = x * z, yz = y * z, x2 = x * x, y2 = y * y, z2 = z * z;
    const float x4 = x2 * x2, y4 = y2 * y2, z4 = z2 * z2;
    const float x6 = x4 * x2, y6 = y4 * y2, z6 = z4 * z2;
    o[0] = k[K0];
    if (L <= 1) return;
    o[1] = -k[K1] * y;
    o[2] = k[K1] * z;
    o[3] = -k[K1] * x;
    if (L <= 2) return;
    o[4] = k[K4] * xy;
    o[5] = -k[K4] * yz;
    o[6] = k[K6a] * z2 - k[K6b];
    o[7] = -k[K4] * xz;
    o[8] = k[K8] * x2 - k[K8] * y2;
    if (L <= 3) return;
    o[9] = k[K9] * y * (-3.0f * x2 + y2);
    o[10] = k[K10] * xy * z;
    o[11] = k[K11] * y * (1.0f - 5.0f * z2);
    o[12] = k[K12] * z * (5.0f * z2 - 3.0f);
    o[13] = k[K11] * x * (1.0f - 5.0f * z2);
    o[14] = k[K14] * z * (x2 - y2);
    o[15] = k[K9] * x * (-x2 + 3.0f * y2);
    if (L <= 4) return;
    o[16] = k[K16] * xy * (x2 - y2);
    o[17] = k[K17] * yz * (-3.0f * x2 + y2);
    o[18] = k[K18] * xy * (7.0f * z2 - 1.0f);
    o[19] = k[K19] * yz * (3.0f - 7.0f * z2);
    o[20] = k[K20a] * z2 + k[K20b] * z4 + k[K20c];
    o[21] = k[K19] * xz * (3.0f - 7.0f * z2);
    o[22] = k[K22] * (x2 - y2) * (7.0f * z2 - 1.0f);
    o[23] = k[K17] * xz * (-x2 + 3.0f * y2);
    o[24] = k[K24a] * x2 * y2 + k[K24b] * x4 + k[K24b] * y4;
    if (L <= 5) return;
    o[25] = k[K25] * y * (10.0f * x2 * y2 - 5.0f * x4 - y4);
    o[26] = k[K26] * xy * z * (x2 - y2);
    o[27] = k[K27] * y * (3.0f * x2 - y2) * (9.0f * z2 - 1.0f);
    o[28] = k[K28] * xy * z * (3.0f * z2 - 1.0f);
    o[29] = k[K29] * y * (14.0f * z2 - 21.0f * z4 - 1.0f);
    o[30] = k[K30] * z * (-70.0f * z2 + 63.0f * z4 + 15.0f);
    o[31] = k[K29] * x * (14.0f * z2 - 21.0f * z4 - 1.0f);
    o[32] = k[K32] * z * (x2 - y2) * (3.0f * z2 - 1.0f);
    o[33] = k[K27] * x * (x2 - 3.0f * y2) * (9.0f * z2 - 1.0f);
    o[34] = k[K34] * z * (-6.0f * x2 * y2 + x4 + y4);
    o[35] = k[K25] * x * (10.0f * x2 * y2 - x4 - 5.0f * y4);
    if (L <= 6) return;
    o[36] = k[K36] * xy * (-10.0f * x2 * y2 + 3.0f * x4 + 3.0f * y4);
    o[37] = k[K37] * yz * (10.0f * x2 * y2 - 5.0f * x4 - y4);
    o[38] = k[K38] * xy * (x2 - y2) * (11.0f * z2 - 1.0f);
    o[39] = k[K39] * yz * (3.0f * x2 - y2) * (11.0f * z2 - 3.0f);
    o[40] = k[K40] * xy * (-18.0f * z2 + 33.0f * z4 + 1.0f);
    o[41] = k[K41] * yz * (30.0f * z2 - 33.0f * z4 - 5.0f);
    o[42] = k[K42a] * z2 + k[K42b] * z4 + k[K42c] * z6 + k[K42d];
    o[43] = k[K41] * xz * (30.0f * z2 - 33.0f * z4 - 5.0f);
    o[44] = k[K44] * (x2 - y2) * (11.0f * z2 * (3.0f * z2 - 1.0f) - 7.0f * z2 + 1.0f);
    o[45] = k[K39] * xz * (x2 - 3.0f * y2) * (11.0f * z2 - 3.0f);
    o[46] = k[K46] * (11.0f * z2 - 1.0f) * (-6.0f * x2 * y2 + x4 + y4);
    o[47] = k[K37] * xz * (10.0f * x2 * y2 - x4 - 5.0f * y4);
    o[48] = k[K48a] * x2 * y4 - k[K48a] * x4 * y2 + k[K48b] * x6 - k[K48b] * y6;
    if (L <= 7) return;
    o[49] = k[K49] * y * (-21.0f * x2 * y4 + 35.0f * x4 * y2 - 7.0f * x6 + y6);
    o[50] = k[K50] * xy * z * (-10.0f * x2 * y2 + 3.0f * x4 + 3.0f * y4);
    o[51] = k[K51] * y * (13.0f * z2 - 1.0f) * (-10.0f * x2 * y2 + 5.0f * x4 + y4);
    o[52] = k[K52] * xy * z * (x2 - y2) * (13.0f * z2 - 3.0f);
    o[53] = k[K53] * y * (3.0f * x2 - y2) * (13.0f * z2 * (11.0f * z2 - 3.0f) - 27.0f * z2 + 3.0f);
    o[54] = k[K54] * xy * z * (-110.0f * z2 + 143.0f * z4 + 15.0f);
    o[55] = k[K55] * y * (-135.0f * z2 + 495.0f * z4 - 429.0f * z6 + 5.0f);
    o[56] = k[K56] * z * (315.0f * z2 - 693.0f * z4 + 429.0f * z6 - 35.0f);
    o[57] = k[K55] * x * (-135.0f * z2 + 495.0f * z4 - 429.0f * z6 + 5.0f);
    o[58] = k[K58] * z * (x2 - y2) * (143.0f * z2 * (3.0f * z2 - 1.0f) - 187.0f * z2 + 45.0f);
    o[59] = k[K53] * x * (x2 - 3.0f * y2) * (13.0f * z2 * (11.0f * z2 - 3.0f) - 27.0f * z2 + 3.0f);
    o[60] = k[K60] * z * (13.0f * z2 - 3.0f) * (-6.0f * x2 * y2 + x4 + y4);
    o[61] = k[K51] * x * (13.0f * z2 - 1.0f) * (-10.0f * x2 * y2 + x4 + 5.0f * y4);
    o[62] = k[K62] * z * (15.0f * x2 * y4 - 15.0f * x4 * y2 + x6 - y6);
    o[63] = k[K49] * x * (-35.0f * x2 * y4 + 21.0f * x4 * y2 - x6 + 7.0f * y6);
}

__global__ void __launch_bounds__(kShBlock) sh_encoding_kernel(std::uint32_t n, std::uint32_t L, ShCoef coef,
                                                               const float *__restrict__ xyz, float *__restrict__ out) {
    extern __shared__ float rows[];   // [kShBlock][L^2 | 1]
    const std::uint32_t d2 = L * L, ld = d2 | 1u;
    const std::size_t i0 = (std::size_t)blockIdx.x * kShBlock;
    const std::size_t i = i0 + threadIdx.x;
    if (i < n) {
        float o[64];
        sh_eval(L, xyz[i * 3 + 0], xyz[i * 3 + 1], xyz[i * 3 + 2], coef.k, o);
        for (std::uint32_t j = 0; j < d2; ++j) rows[threadIdx.x * ld + j] = o[j];
    }
    __syncthreads();
    const std::uint32_t n_here = (std::uint32_t)min((std::size_t)kShBlock, (std::size_t)n - i0);
    float *dst = out + i0 * d2;
    for (std::uint32_t e = threadIdx.x; e < n_here * d2; e += kShBlock) dst[e] = rows[(e / d2) * ld + e % d2];
}

}  // namespace

int launch_sh_encoding(cudaStream_t stream, std::uint32_t n, std::uint32_t degree, const float *xyz, float *out) {
    NGP_CHECK_ARG(degree >= 1 && degree <= 8, "spherical_harmonics_encoding: degree must be in 1..8");
    NGP_CHECK_ARG(n == 0 || (xyz != nullptr && out != nullptr), "spherical_harmonics_encoding: buffers missing");
    static const ShCoef coef = make_coef();
    if (n > 0) {
        const std::size_t smem = (std::size_t)kShBlock * ((degree * degree) | 1u) * sizeof(float);
        sh_encoding_kernel<<<(n + kShBlock - 1) / kShBlock, kShBlock, smem, stream>>>(n, degree, coef, xyz, out);
        count_launches(1);
    }
    return launch_status();
}

}  // namespace ngp
