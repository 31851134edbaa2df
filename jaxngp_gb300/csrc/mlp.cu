// SIMT parts of the MLPs for sm_103a: the learned proposal's FP32 MLP (forward and backward), the
// fixed-order sum of the field backward's per-CTA dL/dW partials, and the allocation-free entry
// point of the field backward.  The field MLP itself (NeRF.__call__, models/nerfs.py:39-86, with
// the NGP layout of make_nerf_ngp, nerfs.py:422-454) runs on the tensor cores in mlp_tc.cu, to
// FP32 accuracy for ngp_field_forward/_density/_backward and in BF16/FP16 for the mixed forms.
//
// Field weights are one packed array of 9408 floats, each kernel in flax's [in, out] row-major
// layout: W0 @0, W1 @2048, W2 @3072, W3 @5120, W4 @9216.
//
// The proposal MLP: a CTA of 256 threads loops over tiles of 64 points with the weights (and, for
// the backward, their transposes) in shared memory; every layer is a small register-blocked SIMT
// GEMM (each thread owns a 4-column strip, float4 weight loads, broadcast activation loads).  The
// backward recomputes the tile's activations, accumulates each thread's share of dL/dP in
// registers across all its tiles, and writes one partial per CTA; a second kernel sums the
// partials in a fixed order, so weight gradients are deterministic.
#include <mutex>

#include "common.cuh"

namespace ngp {
namespace {

constexpr int kTile = 64;
constexpr int kW0 = 0, kW1 = 2048, kW2 = 3072, kW3 = 5120, kW4 = 9216, kNW = 9408;
constexpr int kLd = 68;     // activation row stride (floats): 16-byte aligned rows

// Thread layout of a [ROWS x N] result over NT threads: each thread owns a 4-wide column strip
// and RPT rows spaced R apart; when there are more row groups than rows the extra threads idle.
template <int NT, int ROWS, int N>
struct Strip {
    static constexpr int G = N / 4;
    static constexpr int R = NT / G;
    static constexpr int RPT = ROWS >= R ? ROWS / R : 1;
    static constexpr bool kIdle = R > ROWS;
    static_assert(NT % G == 0 && (kIdle || ROWS % R == 0), "tile shape");
    static __device__ __forceinline__ int col0(int t) { return (t % G) * 4; }
    static __device__ __forceinline__ int row0(int t) { return t / G; }
};

// acc[q][j] += sum over k in [k0, k0 + 4) of A[row_q][k] * B[k][c0 + j], A read as one float4
// per row (rows 16-byte aligned), in k order.
template <int RPT>
__device__ __forceinline__ void fma4(float (&acc)[RPT][4], const float *A, int lda, const int *rows, const float *B,
                                     int ldb, int k0, int c0) {
    const float4 b0 = *reinterpret_cast<const float4 *>(B + (k0 + 0) * ldb + c0);
    const float4 b1 = *reinterpret_cast<const float4 *>(B + (k0 + 1) * ldb + c0);
    const float4 b2 = *reinterpret_cast<const float4 *>(B + (k0 + 2) * ldb + c0);
    const float4 b3 = *reinterpret_cast<const float4 *>(B + (k0 + 3) * ldb + c0);
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
        const float4 a = *reinterpret_cast<const float4 *>(A + rows[q] * lda + k0);
        acc[q][0] += a.x * b0.x;
        acc[q][1] += a.x * b0.y;
        acc[q][2] += a.x * b0.z;
        acc[q][3] += a.x * b0.w;
        acc[q][0] += a.y * b1.x;
        acc[q][1] += a.y * b1.y;
        acc[q][2] += a.y * b1.z;
        acc[q][3] += a.y * b1.w;
        acc[q][0] += a.z * b2.x;
        acc[q][1] += a.z * b2.y;
        acc[q][2] += a.z * b2.z;
        acc[q][3] += a.z * b2.w;
        acc[q][0] += a.w * b3.x;
        acc[q][1] += a.w * b3.y;
        acc[q][2] += a.w * b3.z;
        acc[q][3] += a.w * b3.w;
    }
}

// C[s][n] = act(sum_k A[s][k] * B[k][n]) for s < kTile, n < N (N % 4 == 0, K % 4 == 0).
template <int NT, int K, int N, bool kRelu>
__device__ __forceinline__ void mm(const float *A, int lda, const float *B, float *C, int ldc) {
    using S = Strip<NT, kTile, N>;
    static_assert(K % 4 == 0, "K must be a multiple of 4");
    const int t = threadIdx.x, c0 = S::col0(t), r0 = S::row0(t);
    if (S::kIdle && r0 >= kTile) return;
    int rows[S::RPT];
    float acc[S::RPT][4];
#pragma unroll
    for (int q = 0; q < S::RPT; ++q) {
        rows[q] = r0 + q * S::R;
        acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.f;
    }
#pragma unroll
    for (int k = 0; k < K; k += 4) fma4<S::RPT>(acc, A, lda, rows, B, N, k, c0);
#pragma unroll
    for (int q = 0; q < S::RPT; ++q) {
        float4 v = make_float4(acc[q][0], acc[q][1], acc[q][2], acc[q][3]);
        if (kRelu) v = make_float4(fmaxf(v.x, 0.f), fmaxf(v.y, 0.f), fmaxf(v.z, 0.f), fmaxf(v.w, 0.f));
        *reinterpret_cast<float4 *>(C + rows[q] * ldc + c0) = v;
    }
}

// Like mm, but the result is multiplied elementwise by (M[s][n] > 0) and written over M (the
// relu adjoint: M holds the layer's post-activation values).
template <int NT, int K, int N>
__device__ __forceinline__ void mm_mask_inplace(const float *A, int lda, const float *B, float *M, int ldm) {
    using S = Strip<NT, kTile, N>;
    static_assert(K % 4 == 0, "K must be a multiple of 4");
    const int t = threadIdx.x, c0 = S::col0(t), r0 = S::row0(t);
    if (S::kIdle && r0 >= kTile) return;
    int rows[S::RPT];
    float acc[S::RPT][4];
#pragma unroll
    for (int q = 0; q < S::RPT; ++q) {
        rows[q] = r0 + q * S::R;
        acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.f;
    }
#pragma unroll
    for (int k = 0; k < K; k += 4) fma4<S::RPT>(acc, A, lda, rows, B, N, k, c0);
#pragma unroll
    for (int q = 0; q < S::RPT; ++q) {
        float4 *p = reinterpret_cast<float4 *>(M + rows[q] * ldm + c0);
        const float4 m = *p;
        *p = make_float4(m.x > 0.f ? acc[q][0] : 0.f, m.y > 0.f ? acc[q][1] : 0.f,
                         m.z > 0.f ? acc[q][2] : 0.f, m.w > 0.f ? acc[q][3] : 0.f);
    }
}

// acc[m][n] += sum_s A[s][m] * D[s][n] over the tile's rows (the weight-gradient GEMM).  With four
// rows per thread the rows are consecutive, so A's four values of a sample are one float4.
template <int NT, int M, int N>
struct WGrad {
    using S = Strip<NT, M, N>;
    static constexpr bool kVec = S::RPT == 4;
    float acc[S::RPT][4];
    __device__ __forceinline__ bool owner() const { return !S::kIdle || S::row0((int)threadIdx.x) < M; }
    __device__ __forceinline__ int row(int m0, int q) const { return kVec ? m0 * 4 + q : m0 + q * S::R; }
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int q = 0; q < S::RPT; ++q) acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.f;
    }
    __device__ __forceinline__ void add(const float *A, int lda, const float *D, int ldd, int rows) {
        const int t = threadIdx.x, c0 = S::col0(t), m0 = S::row0(t);
        if (!owner()) return;
#pragma unroll 4
        for (int s = 0; s < rows; ++s) {
            const float4 d = *reinterpret_cast<const float4 *>(D + s * ldd + c0);
            if constexpr (kVec) {
                const float4 a4 = *reinterpret_cast<const float4 *>(A + s * lda + m0 * 4);
                const float a[4] = {a4.x, a4.y, a4.z, a4.w};
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    acc[q][0] += a[q] * d.x;
                    acc[q][1] += a[q] * d.y;
                    acc[q][2] += a[q] * d.z;
                    acc[q][3] += a[q] * d.w;
                }
            } else {
#pragma unroll
                for (int q = 0; q < S::RPT; ++q) {
                    const float a = A[s * lda + m0 + q * S::R];
                    acc[q][0] += a * d.x;
                    acc[q][1] += a * d.y;
                    acc[q][2] += a * d.z;
                    acc[q][3] += a * d.w;
                }
            }
        }
    }
    __device__ __forceinline__ void store(float *out) const {  // out: [M][N] row-major
        const int t = threadIdx.x, c0 = S::col0(t), m0 = S::row0(t);
        if (!owner()) return;
#pragma unroll
        for (int q = 0; q < S::RPT; ++q)
            *reinterpret_cast<float4 *>(out + row(m0, q) * N + c0) = make_float4(acc[q][0], acc[q][1], acc[q][2], acc[q][3]);
    }
};

__device__ __forceinline__ std::uint32_t active_count(std::uint32_t n, const std::uint32_t *count) {
    return count != nullptr ? min(n, *count) : n;
}

// dW[j] = sum over CTAs c (in order) of partials[c][j]; accumulate into dW when requested.
__global__ void reduce_partials_kernel(std::uint32_t n_parts, const float *__restrict__ partials,
                                       float *__restrict__ dW, int accumulate) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= kNW) return;
    float a = 0.f;
    for (std::uint32_t c = 0; c < n_parts; ++c) a += partials[(std::size_t)c * kNW + j];
    dW[j] = accumulate ? dW[j] + a : a;
}

// zero dL/denc rows in [active, n)
__global__ void zero_rows_kernel(std::uint32_t n, const std::uint32_t *__restrict__ count, float *__restrict__ x, int width) {
    const std::uint32_t a = active_count(n, count);
    const std::size_t stride = (std::size_t)gridDim.x * blockDim.x;
    for (std::size_t i = (std::size_t)a * width + (std::size_t)blockIdx.x * blockDim.x + threadIdx.x; i < (std::size_t)n * width; i += stride)
        x[i] = 0.f;
}

// ------------------------------------------------------------------- proposal-field MLP
//
// The learned proposal's density network: x = relu(relu(enc @ P0) @ P1) @ P2 with enc the
// 4-level hash encoding (8 features), P0 [8][64], P1 [64][64], P2 [64][1] packed in that order
// (4672 floats), x the log density.  Same tiling as the field MLP above (64 samples per tile,
// weights in shared memory); the backward recomputes the tile and keeps per-thread dL/dP shares
// across tiles, one partial per CTA.
constexpr int kP0 = 0, kP1 = 512, kP2 = 4608, kNP = 4672;

template <int NT>
__device__ __forceinline__ void load_prop_weights(const float *__restrict__ w, float *sP, float *sT) {
    // sP: P0 [8][64], P1 [64][64], P2 padded to [64][4] (columns 1..3 zero)
    for (int i = threadIdx.x; i < kP2; i += NT) sP[i] = w[i];
    for (int i = threadIdx.x; i < 256; i += NT) sP[kP2 + i] = (i % 4 == 0) ? w[kP2 + i / 4] : 0.f;
    if (sT != nullptr) {  // P1^T [64][64] @0, P0^T [64][8] @4096
        for (int i = threadIdx.x; i < 4096; i += NT) sT[(i % 64) * 64 + i / 64] = w[kP1 + i];
        for (int i = threadIdx.x; i < 512; i += NT) sT[4096 + (i % 64) * 8 + i / 64] = w[kP0 + i];
    }
    __syncthreads();
}

template <int NT>
__device__ __forceinline__ void load_enc8(const float *__restrict__ enc, std::size_t s0, int rows, float *X) {
    for (int i = threadIdx.x; i < kTile * 2; i += NT) {
        const int r = i / 2, c = (i % 2) * 4;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (r < rows) v = *reinterpret_cast<const float4 *>(enc + (s0 + r) * 8 + c);
        *reinterpret_cast<float4 *>(X + r * kLd + c) = v;
    }
}

template <int NT>
__global__ void __launch_bounds__(NT) prop_forward_kernel(std::uint32_t n, const std::uint32_t *__restrict__ count,
                                                          const float *__restrict__ enc, const float *__restrict__ w,
                                                          float *__restrict__ x) {
    extern __shared__ __align__(16) float smem[];
    float *sP = smem, *X0 = sP + kP2 + 256, *H1 = X0 + kTile * kLd, *H2 = H1 + kTile * kLd, *O = H2 + kTile * kLd;
    load_prop_weights<NT>(w, sP, nullptr);
    const std::uint32_t n_act = active_count(n, count);
    const std::uint32_t n_tiles = (n_act + kTile - 1) / kTile;
    for (std::uint32_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        const std::size_t s0 = (std::size_t)tile * kTile;
        const int rows = (int)min((std::uint32_t)kTile, n_act - (std::uint32_t)s0);
        load_enc8<NT>(enc, s0, rows, X0);
        __syncthreads();
        mm<NT, 8, 64, true>(X0, kLd, sP + kP0, H1, kLd);
        __syncthreads();
        mm<NT, 64, 64, true>(H1, kLd, sP + kP1, H2, kLd);
        __syncthreads();
        mm<NT, 64, 4, false>(H2, kLd, sP + kP2, O, 4);
        __syncthreads();
        for (int r = threadIdx.x; r < rows; r += NT) x[s0 + r] = O[r * 4];
        __syncthreads();
    }
}

// dL/dx rows past the active count are ignored; dL/denc rows past it are left unwritten.
template <int NT>
__global__ void __launch_bounds__(NT) prop_backward_kernel(std::uint32_t n, const std::uint32_t *__restrict__ count,
                                                           const float *__restrict__ enc, const float *__restrict__ w,
                                                           const float *__restrict__ dL_dx, float *__restrict__ dL_denc,
                                                           float *__restrict__ partials) {
    extern __shared__ __align__(16) float smem[];
    float *sP = smem, *sT = sP + kP2 + 256, *X0 = sT + 4608, *H1 = X0 + kTile * kLd, *H2 = H1 + kTile * kLd;
    float *G = H2 + kTile * kLd;   // dL/dx of the tile
    load_prop_weights<NT>(w, sP, sT);
    WGrad<NT, 8, 64> g0;
    WGrad<NT, 64, 64> g1;
    float g2 = 0.f;   // thread t < 64 owns dL/dP2[t]
    g0.zero();
    g1.zero();
    const std::uint32_t n_act = active_count(n, count);
    const std::uint32_t n_tiles = (n_act + kTile - 1) / kTile;
    for (std::uint32_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        const std::size_t s0 = (std::size_t)tile * kTile;
        const int rows = (int)min((std::uint32_t)kTile, n_act - (std::uint32_t)s0);
        load_enc8<NT>(enc, s0, rows, X0);
        for (int r = threadIdx.x; r < kTile; r += NT) G[r] = r < rows ? dL_dx[s0 + r] : 0.f;
        __syncthreads();
        mm<NT, 8, 64, true>(X0, kLd, sP + kP0, H1, kLd);
        __syncthreads();
        mm<NT, 64, 64, true>(H1, kLd, sP + kP1, H2, kLd);
        __syncthreads();
        if (threadIdx.x < 64) {  // dP2 += h2^T dx
            float a = 0.f;
            for (int s = 0; s < kTile; ++s) a += H2[s * kLd + threadIdx.x] * G[s];
            g2 += a;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < kTile * 64; i += NT) {  // dA2 = dx P2^T * (h2 > 0), over H2
            const int r = i / 64, c = i % 64;
            H2[r * kLd + c] = H2[r * kLd + c] > 0.f ? G[r] * sP[kP2 + c * 4] : 0.f;
        }
        __syncthreads();
        g1.add(H1, kLd, H2, kLd, kTile);
        __syncthreads();
        mm_mask_inplace<NT, 64, 64>(H2, kLd, sT, H1, kLd);  // dA1 over H1
        __syncthreads();
        g0.add(X0, kLd, H1, kLd, kTile);
        __syncthreads();
        mm<NT, 64, 8, false>(H1, kLd, sT + 4096, X0, kLd);  // dL/denc over X0
        __syncthreads();
        for (int i = threadIdx.x; i < rows * 2; i += NT) {
            const int r = i / 2, c = (i % 2) * 4;
            *reinterpret_cast<float4 *>(dL_denc + (s0 + r) * 8 + c) = *reinterpret_cast<const float4 *>(X0 + r * kLd + c);
        }
        __syncthreads();
    }
    float *p = partials + (std::size_t)blockIdx.x * kNP;
    g0.store(p + kP0);
    g1.store(p + kP1);
    if (threadIdx.x < 64) p[kP2 + threadIdx.x] = g2;
}

__global__ void reduce_partials_n_kernel(std::uint32_t n_parts, std::uint32_t n, const float *__restrict__ partials,
                                         float *__restrict__ dW, int accumulate) {
    const std::uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    float a = 0.f;
    for (std::uint32_t c = 0; c < n_parts; ++c) a += partials[(std::size_t)c * n + j];
    dW[j] = accumulate ? dW[j] + a : a;
}

constexpr std::size_t kPropFwdSmem = (std::size_t)(kP2 + 256 + 3 * kTile * kLd + kTile * 4) * sizeof(float);
constexpr std::size_t kPropBwdSmem = (std::size_t)(kP2 + 256 + 4608 + 3 * kTile * kLd + kTile) * sizeof(float);

}  // namespace

// ------------------------------------------------------------- allocation-free backward
//
// ngp_field_backward needs one dL/dW partial per CTA in a caller-provided scratch buffer.  Callers
// that cannot allocate device memory -- an XLA custom call bound through the legacy signature
// receives only its operand and result buffers, and embedders that run with a fixed,
// pre-reserved memory budget may not call cudaMalloc or any allocating library routine -- use
// ngp_field_backward_noalloc instead, whose partials live in the array below: room for
// kNoAllocMaxParts partials (256 x 9408 floats = 9.6 MB), held by every GPU that loads the library
// until the process exits.  The kernel (the tensor-core backward of ngp_field_backward) strides its
// CTAs over the batch's tiles, so a call launches min(SM count, kNoAllocMaxParts) CTAs, each of
// which writes its partial, and any batch would fit the array; the batch limit
// NGP_FIELD_BACKWARD_NOALLOC_MAX_SAMPLES is a deliberate, published bound of this entry point (a
// caller sizes its batches against it), not a property of the array.  Each call overwrites every
// partial it later reads, so nothing has to be cleared between calls; but all calls share the one
// array, so calls that overlap on the GPU (on different streams) race on it and must be ordered by
// the caller.
constexpr std::uint32_t kNoAllocMaxParts = 256;
constexpr std::uint32_t kNoAllocMaxSamples = NGP_FIELD_BACKWARD_NOALLOC_MAX_SAMPLES;
static_assert(kNoAllocMaxSamples == 524288u, "the published limit of ngp_field_backward_noalloc");
__device__ __align__(256) float g_noalloc_partials[kNoAllocMaxParts * kNW];

int mlp_partials_count() { return sm_count(); }
std::size_t mlp_partials_floats() { return (std::size_t)mlp_partials_count() * kNW; }

static bool aligned16(const void *p) { return ((std::uintptr_t)p & 15u) == 0; }

int launch_prop_forward(cudaStream_t stream, std::uint32_t n, const std::uint32_t *count, const float *enc,
                        const float *weights, float *x) {
    NGP_CHECK_ARG(aligned16(enc) && aligned16(weights), "proposal mlp: enc and weights must be 16-byte aligned");
    NGP_SMEM_LIMIT((prop_forward_kernel<256>), kPropFwdSmem);
    if (n == 0) return launch_status();
    const unsigned tiles = (n + kTile - 1) / kTile;
    const unsigned grid = tiles < (unsigned)sm_count() * 3 ? tiles : (unsigned)sm_count() * 3;
    prop_forward_kernel<256><<<grid, 256, kPropFwdSmem, stream>>>(n, count, enc, weights, x);
    count_launches(1);
    return launch_status();
}

std::size_t prop_partials_floats() { return (std::size_t)sm_count() * kNP; }

// `partials` holds prop_partials_floats() floats.
int launch_prop_backward(cudaStream_t stream, std::uint32_t n, const std::uint32_t *count, const float *enc,
                         const float *weights, const float *dL_dx, float *dL_denc, float *dL_dweights, float *partials,
                         bool accumulate) {
    NGP_CHECK_ARG(aligned16(enc) && aligned16(weights) && aligned16(dL_denc) && aligned16(partials),
                  "proposal mlp: buffers must be 16-byte aligned");
    NGP_SMEM_LIMIT((prop_backward_kernel<256>), kPropBwdSmem);
    const unsigned grid = (unsigned)sm_count();
    prop_backward_kernel<256><<<grid, 256, kPropBwdSmem, stream>>>(n, count, enc, weights, dL_dx, dL_denc, partials);
    count_launches(1);
    reduce_partials_n_kernel<<<(kNP + 255) / 256, 256, 0, stream>>>(grid, kNP, partials, dL_dweights, accumulate ? 1 : 0);
    count_launches(1);
    return launch_status();
}

// Sums `parts` dL/dW partials into dL_dweights (fixed order) and zeroes dL/denc rows past the
// active count: the tail shared by the FP32 and BF16 field backwards.
// Sums the per-CTA dL/dW partials in CTA order and zeroes the dL/denc rows past the active count
// (`row_floats` 32-bit words per row: 32 for FP32 encodings, 16 for 16-bit ones).
int launch_mlp_partials_reduce(cudaStream_t stream, unsigned parts, const float *partials, float *dL_dweights,
                               bool accumulate, std::uint32_t n, const std::uint32_t *count, float *dL_denc,
                               unsigned row_floats) {
    reduce_partials_kernel<<<(kNW + 255) / 256, 256, 0, stream>>>(parts, partials, dL_dweights, accumulate ? 1 : 0);
    count_launches(1);
    if (count != nullptr && n > 0) {
        zero_rows_kernel<<<grid_for((std::size_t)n * row_floats, 256, 4), 256, 0, stream>>>(n, count, dL_denc, row_floats);
        count_launches(1);
    }
    return launch_status();
}

// Device address of g_noalloc_partials on the current device, looked up once per device (the
// array's host-side name is only a stand-in and must never be handed to a kernel).
static int noalloc_scratch(float **out) {
    static std::mutex mu;
    static float *ptrs[64] = {nullptr};
    int dev = 0;
    NGP_CUDA_TRY(cudaGetDevice(&dev));
    NGP_CHECK_ARG(dev >= 0 && dev < 64, "field backward (no-alloc): device ordinal out of range");
    std::lock_guard<std::mutex> lock(mu);
    if (ptrs[dev] == nullptr) {
        void *p = nullptr;
        NGP_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_partials));
        ptrs[dev] = static_cast<float *>(p);
    }
    *out = ptrs[dev];
    return NGP_OK;
}

int launch_mlp_x6_backward(cudaStream_t, std::uint32_t, const std::uint32_t *, const float *, const float *,
                           const float *, const float *, const float *, float *, float *, unsigned, unsigned *);

int launch_mlp_backward_noalloc(cudaStream_t stream, std::uint32_t n, const std::uint32_t *count,
                                const float *enc, const float *dirs, const float *weights,
                                const float *dL_ddrgb, const float *grad_scale, float *dL_denc,
                                float *dL_dweights, bool accumulate) {
    if (n > kNoAllocMaxSamples) {
        set_last_status(NGP_ERR_CAPACITY,
                        "ngp_field_backward_noalloc: n_samples exceeds 524288, the published limit of this entry "
                        "point; use ngp_field_backward with a caller-provided scratch buffer");
        return NGP_ERR_CAPACITY;
    }
    float *scratch = nullptr;
    int st = noalloc_scratch(&scratch);
    if (st != NGP_OK) return st;
    unsigned parts = 0;
    st = launch_mlp_x6_backward(stream, n, count, enc, dirs, weights, dL_ddrgb, grad_scale, dL_denc, scratch,
                                kNoAllocMaxParts, &parts);
    if (st != NGP_OK) return st;
    return launch_mlp_partials_reduce(stream, parts, scratch, dL_dweights, accumulate, n, count, dL_denc, 32u);
}

}  // namespace ngp
