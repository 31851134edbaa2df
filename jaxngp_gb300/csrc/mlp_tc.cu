// Field MLP on the fifth-generation tensor cores (tcgen05), BF16 operands with FP32 accumulation:
// forward, density-only forward and backward with recomputation.  Same network, weights and
// buffers as the FP32 kernels in mlp.cu (models/nerfs.py:39-86, 89-128, 221-238, 422-454):
//
//   h1 = relu(enc @ W0)  [32->64]     x = h1 @ W1  [64->16]       sigma = exp(x[0])
//   h2 = relu([x, SH4(dir)] @ W2)  [32->64]   h3 = relu(h2 @ W3)  [64->64]
//   rgb = sigmoid(h3 @ W4)  [64->3]           drgb = [sigma, rgb]
//
// Layout.  A warpgroup (128 threads) owns a tile of 128 samples, one sample per thread, and runs
// the tile's layers as M=128 MMAs: the thread writes its sample's layer input as one BF16 row of a
// shared-memory operand (core-matrix layout, see tc.cuh), one elected thread issues the MMAs, the
// FP32 result lands in tensor memory (lane = sample), and every thread reads its row back with
// tcgen05.ld for the activation.  The weights are converted to BF16 once per CTA and stay in
// shared memory for its lifetime.  Several warpgroups per CTA work on independent tiles so that
// one warpgroup's MMA latency hides behind another's activation work.
//
// Backward.  The forward is recomputed for the tile and its layer inputs stay in shared memory;
// the adjoint of each layer is then one M=128 MMA for the data gradient (dX = dH @ W^T) and one
// M=64 MMA for the weight gradient (dW = X^T dH over the tile's 128 samples), the latter reading
// the same shared-memory rows as MN-major operands and accumulating in tensor memory across all
// of the warpgroup's tiles.  Relu adjoints overwrite the layer inputs in place once the MMAs that
// read them have completed.  At the end the warpgroups of a CTA add their dW into one partial;
// mlp.cu's reduction sums the partials in a fixed order.
//
// Every mbarrier wait gives up after kWaitLimit polls; the warpgroup then stops, records
// NGP_ERR_DEVICE for ngp_device_status(), and releases its tensor memory.
#include "common.cuh"
#include <cstring>
#include <type_traits>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "half.cuh"
#include "tc.cuh"

namespace ngp {

__device__ unsigned int g_device_error = 0;

namespace {

using tc::smem_addr;

constexpr int kW0 = 0, kW1 = 2048, kW2 = 3072, kW3 = 5120, kW4 = 9216, kNW = 9408;  // FP32 packed, flax [in][out]
constexpr int kRows = 128;                    // samples per tile (MMA M)
constexpr std::uint32_t kWaitLimit = 1u << 22;

// BF16 weight operands (element offsets).  Forward: B[n = out][k = in] (= W^T); backward data
// gradients: B[n = in][k = out] (= W).  Layer 4 has 3 outputs, padded to 16 with zeros.
constexpr int kF0 = 0, kF1 = 2048, kF2 = 3072, kF3 = 5120, kF4 = 9216, kFwdW = 10240;
constexpr int kG4 = 10240, kG3 = 11264, kG2 = 15360, kG1 = 16384, kG0 = 17408, kAllW = 19456;
static_assert(kFwdW % 8 == 0 && kAllW % 8 == 0, "weight pieces start on 16-byte boundaries");

// Per-warpgroup activation rows (element offsets): layer inputs of the tile, and the output-layer
// gradient for the backward.
constexpr int kX0 = 0, kH1 = 4096, kX2 = 12288, kH2 = 16384, kH3 = 24576, kDY = 32768, kX0b = 34816;
constexpr int kFwdAct = 32768, kBwdAct = 38912;
constexpr std::uint32_t kTileBytes = kRows * 32 * 2;   // one tile of 16-bit encodings

// Tensor-memory columns of a warpgroup.
constexpr std::uint32_t kDA = 0, kDB = 64;                                    // layer outputs
constexpr std::uint32_t kA0 = 80, kA1 = 112, kA2 = 128, kA3 = 160, kA4 = 224;  // dW accumulators

__device__ __forceinline__ std::uint32_t active_count(std::uint32_t n, const std::uint32_t *count) {
    return count != nullptr ? min(n, *count) : n;
}

bool aligned16(const void *p) { return ((std::uintptr_t)p & 15u) == 0; }

// Element offset of X[r][c] in a row-block buffer with `cols` 16-bit columns.
__device__ __forceinline__ int rb(int r, int c, int cols) {
    return (r >> 3) * (cols * 8) + (c >> 3) * 64 + (r & 7) * 8 + (c & 7);
}

// Stores v[0..n) as row r of a buffer with n columns (n % 8 == 0), 16 bytes at a time.
template <class E, int N>
__device__ __forceinline__ void store_row(typename E::T *buf, int r, const float *v) {
#pragma unroll
    for (int c = 0; c < N; c += 8) {
        uint4 q;
        q.x = E::pack(v[c + 0], v[c + 1]);
        q.y = E::pack(v[c + 2], v[c + 3]);
        q.z = E::pack(v[c + 4], v[c + 5]);
        q.w = E::pack(v[c + 6], v[c + 7]);
        *reinterpret_cast<uint4 *>(buf + rb(r, c, N)) = q;
    }
}

// Loads row r of a buffer with N columns.
template <class E, int N>
__device__ __forceinline__ void load_row(const typename E::T *buf, int r, float *v) {
#pragma unroll
    for (int c = 0; c < N; c += 8) {
        const uint4 q = *reinterpret_cast<const uint4 *>(buf + rb(r, c, N));
        const std::uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float2 f = E::unpack(w[j]);
            v[c + 2 * j] = f.x;
            v[c + 2 * j + 1] = f.y;
        }
    }
}

// False when a value is NaN or would not fit the 16-bit type (the overflow test of loss scaling).
template <class E, int N>
__device__ __forceinline__ bool row_fits(const float *v) {
    bool ok = true;
#pragma unroll
    for (int i = 0; i < N; ++i) ok &= fabsf(v[i]) <= E::kMax;
    return ok;
}

__device__ __forceinline__ void sh4(float x, float y, float z, float *o) {
    const float xy = x * y, xz = x * z, yz = y * z, x2 = x * x, y2 = y * y, z2 = z * z;
    o[0] = 0.28209479177387814f;
    o[1] = -0.48860251190291987f * y;
    o[2] = 0.48860251190291987f * z;
    o[3] = -0.48860251190291987f * x;
    o[4] = 1.0925484305920792f * xy;
    o[5] = -1.0925484305920792f * yz;
    o[6] = 0.94617469575755997f * z2 - 0.31539156525251999f;
    o[7] = -1.0925484305920792f * xz;
    o[8] = 0.54627421529603959f * x2 - 0.54627421529603959f * y2;
    o[9] = 0.59004358992664352f * y * (-3.0f * x2 + y2);
    o[10] = 2.8906114426405538f * xy * z;
    o[11] = 0.45704579946446572f * y * (1.0f - 5.0f * z2);
    o[12] = 0.3731763325901154f * z * (5.0f * z2 - 3.0f);
    o[13] = 0.45704579946446572f * x * (1.0f - 5.0f * z2);
    o[14] = 1.4453057213202769f * z * (x2 - y2);
    o[15] = 0.59004358992664352f * x * (-x2 + 3.0f * y2);
}

// Converts the FP32 weights into the 16-bit operand layouts (backward copies only when `bwd`).
template <class E>
__device__ void load_weights_tc(const float *__restrict__ w, typename E::T *sw, bool bwd) {
    using T = typename E::T;
    const int total = bwd ? kAllW : kFwdW;
    const T zero = E::cvt(0.f);
    for (int i = threadIdx.x; i < total; i += blockDim.x) sw[i] = zero;
    __syncthreads();
    for (int i = threadIdx.x; i < kNW; i += blockDim.x) {
        const T v = E::cvt(w[i]);
        if (i < kW1) {  // W0 [32][64]
            const int in = i / 64, out = i % 64;
            sw[kF0 + rb(out, in, 32)] = v;
            if (bwd) sw[kG0 + rb(in, out, 64)] = v;
        } else if (i < kW2) {  // W1 [64][16]
            const int j = i - kW1, in = j / 16, out = j % 16;
            sw[kF1 + rb(out, in, 64)] = v;
            if (bwd) sw[kG1 + rb(in, out, 16)] = v;
        } else if (i < kW3) {  // W2 [32][64]; the data gradient needs rows 0..15 (x) only
            const int j = i - kW2, in = j / 64, out = j % 64;
            sw[kF2 + rb(out, in, 32)] = v;
            if (bwd && in < 16) sw[kG2 + rb(in, out, 64)] = v;
        } else if (i < kW4) {  // W3 [64][64]
            const int j = i - kW3, in = j / 64, out = j % 64;
            sw[kF3 + rb(out, in, 64)] = v;
            if (bwd) sw[kG3 + rb(in, out, 64)] = v;
        } else {  // W4 [64][3]
            const int j = i - kW4, in = j / 3, out = j % 3;
            sw[kF4 + rb(out, in, 64)] = v;
            if (bwd) sw[kG4 + rb(in, out, 16)] = v;
        }
    }
}

// D (tmem) = A @ B^T with both operands K-major: A = rows of a buffer with K columns (M = 128
// samples), B = weight operand [N][K].
template <class E>
__device__ __forceinline__ void mma_kk(std::uint32_t d, const typename E::T *a, const typename E::T *b, int K, int N,
                                       bool acc) {
    const std::uint32_t id = tc::idesc_kf16(128, N, E::kFmt, false, false), sbo = (std::uint32_t)K * 16;
    const tc::SDesc da = tc::sdesc2(smem_addr(a), 128, sbo), db = tc::sdesc2(smem_addr(b), 128, sbo);
    for (int j = 0; j < K / 16; ++j) tc::mma_bf16(d, da, 16u * j, db, 16u * j, id, acc || j > 0);   // +256 bytes of K
}

// D (tmem, M = 64) += A^T @ B over the tile's 128 samples: A = buffer with 64 columns, B = buffer
// with N columns, both read MN-major (the sample index is the contraction).
template <class E>
__device__ __forceinline__ void mma_mn(std::uint32_t d, const typename E::T *a, const typename E::T *b, int N, bool acc) {
    const std::uint32_t id = tc::idesc_kf16(64, N, E::kFmt, true, true), la = 64 * 16, lb = (std::uint32_t)N * 16;
    const tc::SDesc da = tc::sdesc2(smem_addr(a), la, 128), db = tc::sdesc2(smem_addr(b), lb, 128);
    for (int j = 0; j < kRows / 16; ++j)   // 16 rows of K: +2 LBO
        tc::mma_bf16(d, da, j * 2 * la / 16, db, j * 2 * lb / 16, id, acc || j > 0);
}

// TMEM lane that holds row m of an M = 64 result: rows 16j..16j+15 sit in lanes 32j..32j+15
// (measured with known operands).
__device__ __forceinline__ int m64_lane(int m) { return (m >> 4) * 32 + (m & 15); }

struct WarpGroup {
    int g;             // warpgroup index in the CTA
    int r;             // this thread's row (sample) in the tile, = its TMEM lane
    std::uint32_t tm;  // tensor-memory address of the warpgroup's columns, lane base of this warp
    std::uint64_t *bar;
    std::uint32_t phase;
    int *fail;

    // Waits for the warpgroup's MMAs to complete; records a time-out.
    __device__ __forceinline__ void wait() {
        if (!tc::mbar_wait(bar, phase, kWaitLimit)) *fail = 1;
        phase ^= 1u;
        tc::fence_after();
    }
    // Makes this thread's shared-memory rows and tensor-memory reads ordered before the MMAs that
    // the elected thread issues next.
    __device__ __forceinline__ void sync() {
        tc::fence_async_smem();
        tc::fence_before();
        tc::bar_sync(1 + g, 128);
        tc::fence_after();
    }
};

// Forward through one tile; on return H1, X2, H2, H3 hold the layer inputs (16-bit), and x0 / rgb
// this thread's pre-activation density and colour.  With `fits` given, every layer input is also
// checked against the 16-bit range (loss scaling's overflow test).
template <class E, class After0>
__device__ __forceinline__ void tile_forward(WarpGroup &wg, const typename E::T *sw, typename E::T *act,
                                             const typename E::T *x0in, const float dir[3], float &x0, float rgb[3],
                                             bool *fits, After0 &&after0) {
    float v[64];
    const bool leader = wg.r == 0;
    // layer 0
    wg.sync();
    if (leader) { mma_kk<E>(wg.tm + kDA, x0in, sw + kF0, 32, 64, false); tc::commit(wg.bar); }
    wg.wait();
    after0();   // the layer-0 operand may be refilled from here on
    tc::ld64(wg.tm + kDA, v);
#pragma unroll
    for (int i = 0; i < 64; ++i) v[i] = fmaxf(v[i], 0.f);
    if (fits) *fits &= row_fits<E, 64>(v);
    store_row<E, 64>(act + kH1, wg.r, v);
    // layer 1
    wg.sync();
    if (leader) { mma_kk<E>(wg.tm + kDB, act + kH1, sw + kF1, 64, 16, false); tc::commit(wg.bar); }
    wg.wait();
    tc::ld16(wg.tm + kDB, v);
    x0 = v[0];
    sh4(dir[0], dir[1], dir[2], v + 16);
    if (fits) *fits &= row_fits<E, 16>(v);
    store_row<E, 32>(act + kX2, wg.r, v);
    // layer 2
    wg.sync();
    if (leader) { mma_kk<E>(wg.tm + kDA, act + kX2, sw + kF2, 32, 64, false); tc::commit(wg.bar); }
    wg.wait();
    tc::ld64(wg.tm + kDA, v);
#pragma unroll
    for (int i = 0; i < 64; ++i) v[i] = fmaxf(v[i], 0.f);
    if (fits) *fits &= row_fits<E, 64>(v);
    store_row<E, 64>(act + kH2, wg.r, v);
    // layer 3
    wg.sync();
    if (leader) { mma_kk<E>(wg.tm + kDA, act + kH2, sw + kF3, 64, 64, false); tc::commit(wg.bar); }
    wg.wait();
    tc::ld64(wg.tm + kDA, v);
#pragma unroll
    for (int i = 0; i < 64; ++i) v[i] = fmaxf(v[i], 0.f);
    if (fits) *fits &= row_fits<E, 64>(v);
    store_row<E, 64>(act + kH3, wg.r, v);
    // layer 4
    wg.sync();
    if (leader) { mma_kk<E>(wg.tm + kDB, act + kH3, sw + kF4, 64, 16, false); tc::commit(wg.bar); }
    wg.wait();
    tc::ld16(wg.tm + kDB, v);
#pragma unroll
    for (int c = 0; c < 3; ++c) rgb[c] = 1.f / (1.f + expf(-v[c]));
}

// One sample's encoding row, fetched ahead of its tile: FP32 values (rounded to the operand type
// when staged) or, with kHalf, the operand type's 32 values as they are stored.
template <class E, bool kHalf>
struct EncRow;

template <class E>
struct EncRow<E, false> {
    using In = float;
    float v[32];
    __device__ __forceinline__ void load(const float *__restrict__ enc, std::size_t s, bool valid) {
#pragma unroll
        for (int c = 0; c < 32; c += 4) {
            float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
            if (valid) q = *reinterpret_cast<const float4 *>(enc + s * 32 + c);
            v[c] = q.x;
            v[c + 1] = q.y;
            v[c + 2] = q.z;
            v[c + 3] = q.w;
        }
    }
    __device__ __forceinline__ void stage(typename E::T *buf, int r) const { store_row<E, 32>(buf, r, v); }
};

template <class E>
struct EncRow<E, true> {
    using In = typename E::T;
    uint4 q[4];
    __device__ __forceinline__ void load(const In *__restrict__ enc, std::size_t s, bool valid) {
        const uint4 *src = reinterpret_cast<const uint4 *>(enc + s * 32);
#pragma unroll
        for (int c = 0; c < 4; ++c) q[c] = valid ? src[c] : make_uint4(0u, 0u, 0u, 0u);
    }
    __device__ __forceinline__ void stage(typename E::T *buf, int r) const {
#pragma unroll
        for (int c = 0; c < 4; ++c) *reinterpret_cast<uint4 *>(buf + rb(r, c * 8, 32)) = q[c];
    }
};

// Zeroes row r of a 32-column 16-bit operand buffer (a tile row past the active count: a TMA copy
// brings whatever the buffer holds there, and a NaN in it would reach the weight gradients as
// NaN x 0).
template <class T>
__device__ __forceinline__ void zero_row32(T *buf, int r) {
#pragma unroll
    for (int c = 0; c < 4; ++c) *reinterpret_cast<uint4 *>(buf + rb(r, c * 8, 32)) = make_uint4(0u, 0u, 0u, 0u);
}

// dL/denc row of one sample: FP32, or the operand type when kHalf.
template <class E>
__device__ __forceinline__ void write_denc(float *__restrict__ out, std::size_t s, const float *v) {
#pragma unroll
    for (int c = 0; c < 32; c += 4)
        *reinterpret_cast<float4 *>(out + s * 32 + c) = make_float4(v[c], v[c + 1], v[c + 2], v[c + 3]);
}

template <class E>
__device__ __forceinline__ void write_denc(typename E::T *__restrict__ out, std::size_t s, const float *v) {
#pragma unroll
    for (int c = 0; c < 32; c += 8) {
        uint4 q;
        q.x = E::pack(v[c + 0], v[c + 1]);
        q.y = E::pack(v[c + 2], v[c + 3]);
        q.z = E::pack(v[c + 4], v[c + 5]);
        q.w = E::pack(v[c + 6], v[c + 7]);
        *reinterpret_cast<uint4 *>(out + s * 32 + c) = q;
    }
}

// Row r of tile `tile`: encoding (unless `enc` is null), direction (+z past the end) and, when `g`
// is given, dL/ddrgb.
template <class Row>
__device__ __forceinline__ void fetch_row(const typename Row::In *__restrict__ enc, const float *__restrict__ dirs,
                                          const float *__restrict__ dL_ddrgb, std::uint32_t tile, int r,
                                          std::uint32_t n_act, Row &row, float *dir, float4 *g) {
    const std::size_t s = (std::size_t)tile * kRows + r;
    const bool valid = s < n_act;
    if (enc != nullptr) row.load(enc, s, valid);   // null: the tile arrives by TMA
    dir[0] = valid ? dirs[s * 3 + 0] : 0.f;
    dir[1] = valid ? dirs[s * 3 + 1] : 0.f;
    dir[2] = valid ? dirs[s * 3 + 2] : 1.f;
    if (g != nullptr) *g = valid ? reinterpret_cast<const float4 *>(dL_ddrgb)[s] : make_float4(0.f, 0.f, 0.f, 0.f);
}

// TMA-fed tiles (kTma, 16-bit encodings only): a 4-D tensor map over enc [n][32] views it as
// [n/8 row groups][4 column chunks][8 rows][8 columns] (strides 512, 16 and 64 bytes), so one
// 128-row box lands in shared memory in exactly the operand's core-matrix layout; the leader
// issues the next tile's copy as soon as the layer-0 MMA has consumed the current one, and the copy
// overlaps layers 1-4.  Copy completion is an mbarrier transaction count; every wait is bounded.
template <class E, bool kHalf, bool kTma, int NWG>
__global__ void __launch_bounds__(NWG * 128, 1) mlp_tc_forward_kernel(
    std::uint32_t n, const std::uint32_t *__restrict__ count, const typename EncRow<E, kHalf>::In *__restrict__ enc,
    const float *__restrict__ dirs, const float *__restrict__ weights, float *__restrict__ drgb,
    const __grid_constant__ CUtensorMap enc_map) {
    static_assert(!kTma || kHalf, "TMA tiles carry 16-bit encodings");
    using T = typename E::T;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ std::uint64_t bars[NWG], tbars[NWG];
    __shared__ std::uint32_t tbase;
    __shared__ int fails[NWG];
    T *sw = reinterpret_cast<T *>(smem_raw);
    const int g = threadIdx.x / 128, r = threadIdx.x % 128, q = (threadIdx.x / 32) % 4;
    T *act = sw + kFwdW + g * kFwdAct;
    load_weights_tc<E>(weights, sw, false);
    if (threadIdx.x == 0) {
        for (int k = 0; k < NWG; ++k) {
            tc::mbar_init(&bars[k], 1);
            tc::mbar_init(&tbars[k], 1);
            fails[k] = 0;
        }
        tc::fence_mbar_init();
    }
    if (threadIdx.x < 32) tc::tmem_alloc(&tbase, 512);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    WarpGroup wg{g, r, tbase + (std::uint32_t)g * 128u + ((std::uint32_t)(q * 32) << 16), &bars[g], 0u, &fails[g]};
    const bool leader = r == 0;

    const std::uint32_t n_act = active_count(n, count);
    const std::uint32_t n_tiles = (n_act + kRows - 1) / kRows;
    const std::uint32_t step = gridDim.x * NWG;
    std::uint32_t tphase = 0;
    bool pending = false;   // a tile copy was issued and not yet waited for
    auto issue = [&](std::uint32_t t) {
        if (kTma && t < n_tiles) {
            if (leader) {
                tc::mbar_expect_tx(&tbars[g], kTileBytes);
                tc::tma_load_4d(act + kX0, &enc_map, 0, 0, 0, (int)(t * (kRows / 8)), &tbars[g]);
            }
            pending = true;
        }
    };
    EncRow<E, kHalf> next;  // the next tile's row, loaded while the current tile computes
    float nd[3];
    issue(blockIdx.x * NWG + g);
    fetch_row(kTma ? nullptr : enc, dirs, nullptr, blockIdx.x * NWG + g, r, n_act, next, nd, nullptr);
    for (std::uint32_t tile = blockIdx.x * NWG + g; tile < n_tiles; tile += step) {
        const std::size_t s = (std::size_t)tile * kRows + r;
        const bool valid = s < n_act;
        const EncRow<E, kHalf> cur = next;
        const float dir[3] = {nd[0], nd[1], nd[2]};
        fetch_row(kTma ? nullptr : enc, dirs, nullptr, tile + step, r, n_act, next, nd, nullptr);
        if (kTma) {
            if (!tc::mbar_wait(&tbars[g], tphase, kWaitLimit)) *wg.fail = 1;
            tphase ^= 1u;
            pending = false;
            if (!valid) zero_row32(act + kX0, r);
        } else {
            cur.stage(act + kX0, r);
        }
        float x0, rgb[3];
        tile_forward<E>(wg, sw, act, act + kX0, dir, x0, rgb, nullptr, [&] {
            if (!*wg.fail) issue(tile + step);
        });
        if (valid) reinterpret_cast<float4 *>(drgb)[s] = make_float4(expf(x0), rgb[0], rgb[1], rgb[2]);
        tc::bar_sync(1 + g, 128);
        if (*wg.fail) break;
    }
    if (kTma && pending && !tc::mbar_wait(&tbars[g], tphase, kWaitLimit)) *wg.fail = 1;   // leave no copy in flight
    if (*wg.fail && r == 0) atomicOr(&g_device_error, 1u);
    tc::fence_before();
    __syncthreads();
    if (threadIdx.x < 32) tc::tmem_free(tbase, 512);
}

// sigma only (NeRF.__call__ with dir=None, nerfs.py:71-72): layers 0 and 1.
template <class E, bool kHalf, int NWG>
__global__ void __launch_bounds__(NWG * 128, 1) mlp_tc_density_kernel(
    std::uint32_t n, const typename EncRow<E, kHalf>::In *__restrict__ enc, const float *__restrict__ weights,
    float *__restrict__ sigma) {
    using T = typename E::T;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ std::uint64_t bars[NWG];
    __shared__ std::uint32_t tbase;
    __shared__ int fails[NWG];
    T *sw = reinterpret_cast<T *>(smem_raw);
    const int g = threadIdx.x / 128, r = threadIdx.x % 128, q = (threadIdx.x / 32) % 4;
    T *act = sw + kFwdW + g * kFwdAct;
    load_weights_tc<E>(weights, sw, false);
    if (threadIdx.x == 0) {
        for (int k = 0; k < NWG; ++k) {
            tc::mbar_init(&bars[k], 1);
            fails[k] = 0;
        }
        tc::fence_mbar_init();
    }
    if (threadIdx.x < 32) tc::tmem_alloc(&tbase, 512);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    WarpGroup wg{g, r, tbase + (std::uint32_t)g * 128u + ((std::uint32_t)(q * 32) << 16), &bars[g], 0u, &fails[g]};
    const bool leader = r == 0;
    const std::uint32_t n_tiles = (n + kRows - 1) / kRows;
    for (std::uint32_t tile = blockIdx.x * NWG + g; tile < n_tiles; tile += gridDim.x * NWG) {
        const std::size_t s = (std::size_t)tile * kRows + r;
        const bool valid = s < n;
        float v[64];
        {
            EncRow<E, kHalf> row;
            row.load(enc, s, valid);
            row.stage(act + kX0, r);
        }
        wg.sync();
        if (leader) { mma_kk<E>(wg.tm + kDA, act + kX0, sw + kF0, 32, 64, false); tc::commit(wg.bar); }
        wg.wait();
        tc::ld64(wg.tm + kDA, v);
#pragma unroll
        for (int i = 0; i < 64; ++i) v[i] = fmaxf(v[i], 0.f);
        store_row<E, 64>(act + kH1, r, v);
        wg.sync();
        if (leader) { mma_kk<E>(wg.tm + kDB, act + kH1, sw + kF1, 64, 16, false); tc::commit(wg.bar); }
        wg.wait();
        tc::ld16(wg.tm + kDB, v);
        if (valid) sigma[s] = expf(v[0]);
        tc::bar_sync(1 + g, 128);
        if (*wg.fail) break;
    }
    if (*wg.fail && r == 0) atomicOr(&g_device_error, 1u);
    tc::fence_before();
    __syncthreads();
    if (threadIdx.x < 32) tc::tmem_free(tbase, 512);
}

// Backward.  `grad_scale` multiplies dL/ddrgb, and so does the loss scale when `ls` is given; with
// `ls`, a layer input or gradient that does not fit the 16-bit type (or dL/denc its storage type)
// sets ls->overflow.  `partials` receives one [9408] dL/dW partial per CTA.
template <class E, bool kHalf, bool kTma, int NWG>
__global__ void __launch_bounds__(NWG * 128, 1) mlp_tc_backward_kernel(
    std::uint32_t n, const std::uint32_t *__restrict__ count, const typename EncRow<E, kHalf>::In *__restrict__ enc,
    const float *__restrict__ dirs, const float *__restrict__ weights, const float *__restrict__ dL_ddrgb,
    const float *__restrict__ grad_scale, NgpLossScale *__restrict__ ls,
    typename EncRow<E, kHalf>::In *__restrict__ dL_denc, float *__restrict__ partials,
    const __grid_constant__ CUtensorMap enc_map) {
    static_assert(!kTma || kHalf, "TMA tiles carry 16-bit encodings");
    using T = typename E::T;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ std::uint64_t bars[NWG], wbars[NWG], tbars[NWG][2];
    __shared__ std::uint32_t tbase;
    __shared__ int fails[NWG];
    __shared__ int tiles_done[NWG];
    T *sw = reinterpret_cast<T *>(smem_raw);
    const int g = threadIdx.x / 128, r = threadIdx.x % 128, q = (threadIdx.x / 32) % 4;
    T *act = sw + kAllW + g * kBwdAct;
    load_weights_tc<E>(weights, sw, true);
    if (threadIdx.x == 0) {
        for (int k = 0; k < NWG; ++k) {
            tc::mbar_init(&bars[k], 1);
            tc::mbar_init(&wbars[k], 1);
            tc::mbar_init(&tbars[k][0], 1);
            tc::mbar_init(&tbars[k][1], 1);
            fails[k] = 0;
            tiles_done[k] = 0;
        }
        tc::fence_mbar_init();
    }
    if (threadIdx.x < 32) tc::tmem_alloc(&tbase, 512);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const std::uint32_t tm0 = tbase + (std::uint32_t)g * 256u;
    WarpGroup wg{g, r, tm0 + ((std::uint32_t)(q * 32) << 16), &bars[g], 0u, &fails[g]};
    // In the backward layers the warpgroup's thread 0 issues the data-gradient MMAs (completing on
    // bars[g]) and its thread 32, in another warp, the weight-gradient MMAs (completing on
    // wbars[g]), side by side; the epilogue reads the data gradient while the weight gradient still
    // runs and waits for it only before overwriting the rows it reads.
    const bool leader = r == 0, wleader = r == 32;
    std::uint32_t wphase = 0;
    auto wait_w = [&] {
        if (!tc::mbar_wait(&wbars[g], wphase, kWaitLimit)) *wg.fail = 1;
        wphase ^= 1u;
        tc::fence_after();
    };
    float gs = grad_scale != nullptr ? *grad_scale : 1.f;
    if (ls != nullptr) gs *= ls->scale;
    bool fits = true;
    bool *check = ls != nullptr ? &fits : nullptr;

    const std::uint32_t n_act = active_count(n, count);
    const std::uint32_t n_tiles = (n_act + kRows - 1) / kRows;
    bool first = true;
    const std::uint32_t step = gridDim.x * NWG;
    // TMA-fed tiles (kTma): two encoding buffers; tile i lands in buffer i % 2 while tile i - 1,
    // whose MMAs have all completed, frees the other for tile i + 1.
    std::uint32_t tphase[2] = {0u, 0u};
    bool pending[2] = {false, false};
    auto issue = [&](std::uint32_t t, int b) {
        if (kTma && t < n_tiles) {
            if (leader) {
                tc::mbar_expect_tx(&tbars[g][b], kTileBytes);
                tc::tma_load_4d(act + (b ? kX0b : kX0), &enc_map, 0, 0, 0, (int)(t * (kRows / 8)), &tbars[g][b]);
            }
            pending[b] = true;
        }
    };
    EncRow<E, kHalf> next;  // the next tile's row, loaded while the current tile computes
    float nd[3];
    float4 ng;
    issue(blockIdx.x * NWG + g, 0);
    fetch_row(kTma ? nullptr : enc, dirs, dL_ddrgb, blockIdx.x * NWG + g, r, n_act, next, nd, &ng);
    int buf = 0;
    for (std::uint32_t tile = blockIdx.x * NWG + g; tile < n_tiles; tile += step, buf ^= 1) {
        const std::size_t s = (std::size_t)tile * kRows + r;
        const bool valid = s < n_act;
        float v[64];
        const EncRow<E, kHalf> cur = next;
        const float dir[3] = {nd[0], nd[1], nd[2]};
        const float4 go = ng;
        fetch_row(kTma ? nullptr : enc, dirs, dL_ddrgb, tile + step, r, n_act, next, nd, &ng);
        T *X0 = act + ((kTma && buf) ? kX0b : kX0);
        if (kTma) {
            if (!tc::mbar_wait(&tbars[g][buf], tphase[buf], kWaitLimit)) *wg.fail = 1;
            tphase[buf] ^= 1u;
            pending[buf] = false;
            if (!valid) zero_row32(X0, r);
            if (!*wg.fail) issue(tile + step, buf ^ 1);
        } else {
            cur.stage(X0, r);
        }
        float x0, rgb[3];
        tile_forward<E>(wg, sw, act, X0, dir, x0, rgb, check, [] {});

        // output layer: dL/da4 (3, padded to 16) and dL/dx0 through the truncated exponential
        const float dx0 = gs * go.x * expf(fminf(fmaxf(x0, -15.f), 15.f));
        {
            float d[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) d[i] = 0.f;
            d[0] = gs * go.y * rgb[0] * (1.f - rgb[0]);
            d[1] = gs * go.z * rgb[1] * (1.f - rgb[1]);
            d[2] = gs * go.w * rgb[2] * (1.f - rgb[2]);
            if (check) fits &= row_fits<E, 3>(d);
            store_row<E, 16>(act + kDY, r, d);
        }
        // layer 4: dW4 += h3^T dA4;  dh3 = dA4 @ W4^T
        wg.sync();
        if (leader) {
            mma_kk<E>(tm0 + kDA, act + kDY, sw + kG4, 16, 64, false);
            tc::commit(wg.bar);
        } else if (wleader) {
            mma_mn<E>(tm0 + kA4, act + kH3, act + kDY, 16, !first);
            tc::commit(&wbars[g]);
        }
        wg.wait();
        tc::ld64(wg.tm + kDA, v);
        {
            float h[64];
            load_row<E, 64>(act + kH3, r, h);
#pragma unroll
            for (int i = 0; i < 64; ++i) v[i] = h[i] > 0.f ? v[i] : 0.f;
        }
        if (check) fits &= row_fits<E, 64>(v);
        wait_w();
        store_row<E, 64>(act + kH3, r, v);  // dA3 over h3
        // layer 3: dW3^T += dA3^T h2;  dh2 = dA3 @ W3^T
        wg.sync();
        if (leader) {
            mma_kk<E>(tm0 + kDA, act + kH3, sw + kG3, 64, 64, false);
            tc::commit(wg.bar);
        } else if (wleader) {
            mma_mn<E>(tm0 + kA3, act + kH3, act + kH2, 64, !first);
            tc::commit(&wbars[g]);
        }
        wg.wait();
        tc::ld64(wg.tm + kDA, v);
        {
            float h[64];
            load_row<E, 64>(act + kH2, r, h);
#pragma unroll
            for (int i = 0; i < 64; ++i) v[i] = h[i] > 0.f ? v[i] : 0.f;
        }
        if (check) fits &= row_fits<E, 64>(v);
        wait_w();
        store_row<E, 64>(act + kH2, r, v);  // dA2 over h2
        // layer 2: dW2^T += dA2^T [x, sh];  dx = dA2 @ W2[:16]^T
        wg.sync();
        if (leader) {
            mma_kk<E>(tm0 + kDB, act + kH2, sw + kG2, 64, 16, false);
            tc::commit(wg.bar);
        } else if (wleader) {
            mma_mn<E>(tm0 + kA2, act + kH2, act + kX2, 32, !first);
            tc::commit(&wbars[g]);
        }
        wg.wait();
        tc::ld16(wg.tm + kDB, v);
        v[0] += dx0;
        if (check) fits &= row_fits<E, 16>(v);
        wait_w();
        store_row<E, 16>(act + kX2, r, v);  // dx (16 columns) over [x, sh]
        // layer 1: dW1 += h1^T dx;  dh1 = dx @ W1^T
        wg.sync();
        if (leader) {
            mma_kk<E>(tm0 + kDA, act + kX2, sw + kG1, 16, 64, false);
            tc::commit(wg.bar);
        } else if (wleader) {
            mma_mn<E>(tm0 + kA1, act + kH1, act + kX2, 16, !first);
            tc::commit(&wbars[g]);
        }
        wg.wait();
        tc::ld64(wg.tm + kDA, v);
        {
            float h[64];
            load_row<E, 64>(act + kH1, r, h);
#pragma unroll
            for (int i = 0; i < 64; ++i) v[i] = h[i] > 0.f ? v[i] : 0.f;
        }
        if (check) fits &= row_fits<E, 64>(v);
        wait_w();
        store_row<E, 64>(act + kH1, r, v);  // dA1 over h1
        // layer 0: dW0^T += dA1^T enc;  denc = dA1 @ W0^T
        wg.sync();
        if (leader) {
            mma_kk<E>(tm0 + kDA, act + kH1, sw + kG0, 64, 32, false);
            tc::commit(wg.bar);
        } else if (wleader) {
            mma_mn<E>(tm0 + kA0, act + kH1, X0, 32, !first);
            tc::commit(&wbars[g]);
        }
        wg.wait();
        tc::ld32(wg.tm + kDA, v);
        if (valid) {
            if (check) fits &= kHalf ? row_fits<E, 32>(v) : row_fits<F32Op, 32>(v);
            write_denc<E>(dL_denc, s, v);
        }
        wait_w();   // the next tiles overwrite H1 and the encoding buffer
        first = false;
        tc::bar_sync(1 + g, 128);
        if (*wg.fail) break;
    }
#pragma unroll
    for (int b = 0; b < 2; ++b)   // leave no copy in flight
        if (kTma && pending[b] && !tc::mbar_wait(&tbars[g][b], tphase[b], kWaitLimit)) *wg.fail = 1;
    if (check != nullptr && !fits) atomicOr(&ls->overflow, 1u);
    if (r == 0) {
        tiles_done[g] = first ? 0 : 1;
        if (*wg.fail) atomicOr(&g_device_error, 1u);
    }

    // dW: every warpgroup writes its sums, in the packed [in][out] layout, over its own activation
    // rows (free now); the CTA then adds the warpgroups' copies in a fixed order into its partial.
    // Row m of an M = 64 accumulator sits in TMEM lane m64_lane(m); each element has one writer.
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    float *mine = reinterpret_cast<float *>(act);
    if (tiles_done[g]) {
        const int lane = q * 32 + (threadIdx.x & 31);
        const std::uint32_t base = tm0 + ((std::uint32_t)(q * 32) << 16);
        int m = -1;
        for (int k = 0; k < 64; ++k)
            if (m64_lane(k) == lane) m = k;
        float a[64];
        tc::ld32(base + kA0, a);  // dW0^T: row = out, 32 columns = in
        if (m >= 0)
            for (int i = 0; i < 32; ++i) mine[kW0 + i * 64 + m] = a[i];
        tc::ld16(base + kA1, a);  // dW1: row = in, 16 columns = out
        if (m >= 0)
            for (int o = 0; o < 16; ++o) mine[kW1 + m * 16 + o] = a[o];
        tc::ld32(base + kA2, a);  // dW2^T: row = out, 32 columns = in
        if (m >= 0)
            for (int i = 0; i < 32; ++i) mine[kW2 + i * 64 + m] = a[i];
        tc::ld64(base + kA3, a);  // dW3^T: row = out, 64 columns = in
        if (m >= 0)
            for (int i = 0; i < 64; ++i) mine[kW3 + i * 64 + m] = a[i];
        tc::ld16(base + kA4, a);  // dW4: row = in, columns 0..2 = out
        if (m >= 0)
            for (int o = 0; o < 3; ++o) mine[kW4 + m * 3 + o] = a[o];
    } else {
        for (int i = r; i < kNW; i += 128) mine[i] = 0.f;
    }
    __syncthreads();
    float *p = partials + (std::size_t)blockIdx.x * kNW;
    for (int i = threadIdx.x; i < kNW; i += NWG * 128) {
        float a = 0.f;
#pragma unroll
        for (int k = 0; k < NWG; ++k) a += reinterpret_cast<const float *>(sw + kAllW + k * kBwdAct)[i];
        p[i] = a;
    }
    tc::fence_before();
    __syncthreads();
    if (threadIdx.x < 32) tc::tmem_free(tbase, 512);
}

// ------------------------------------------------- FP32-accurate forward on the tensor cores
//
// The FP32 field forward (ngp_field_forward, ngp_field_density) with BF16 operands: every operand x
// is split into three BF16 pieces x1 + x2 + x3 (x1 = bf16(x), x2 = bf16(x - x1), x3 = bf16(x - x1 -
// x2); both differences exact in FP32), and each layer accumulates the six products of pieces whose
// orders add up to at most 4 -- a3 b1, a2 b2, a1 b3, a2 b1, a1 b2, a1 b1, smallest first -- in the
// FP32 accumulator.  The dropped products and the pieces' remainders are below 2^-24 relative:
// within FP32 rounding of the exact layer (1.3e-7 against FP64 in the CPU restatement of this scheme,
// about what a plain FP32 evaluation of the field gives).  Three warpgroups per CTA, each with one 128-row activation
// buffer of three pieces that every layer reads and the next layer's input then overwrites (the
// layer's MMAs have completed by then); the weights' three pieces stay in shared memory.
constexpr int kX6Piece = kRows * 64;                     // elements of one piece of an activation tile
constexpr int kX6WgAct = 3 * kX6Piece;                   // per warpgroup: three pieces
constexpr int kX6Wgs = 3;
constexpr std::size_t kX6Smem = (std::size_t)(3 * kFwdW + kX6Wgs * kX6WgAct) * 2;   // 204 KB

__device__ __forceinline__ void split3(float v, float &a, float &b, float &c) {
    a = __bfloat162float(__float2bfloat16_rn(v));
    const float r = v - a;   // exact
    b = __bfloat162float(__float2bfloat16_rn(r));
    c = r - b;               // exact; rounded to BF16 when stored
}

// The three pieces of (x, y) as packed BF16 pairs: the same values as split3, two at a time.
__device__ __forceinline__ void split3_pair(float x, float y, std::uint32_t &p1, std::uint32_t &p2, std::uint32_t &p3) {
    p1 = Bf16Op::pack(x, y);
    const float2 f1 = Bf16Op::unpack(p1);
    const float rx = x - f1.x, ry = y - f1.y;   // exact
    p2 = Bf16Op::pack(rx, ry);
    const float2 f2 = Bf16Op::unpack(p2);
    p3 = Bf16Op::pack(rx - f2.x, ry - f2.y);    // the differences exact, then rounded
}

// Columns [c0, c0 + C) of row r of a tile with N columns (c0, C multiples of 8) as three BF16
// pieces `piece` elements apart; v holds the C values.
template <int N, int C>
__device__ __forceinline__ void store_cols3(__nv_bfloat16 *buf, int piece, int r, int c0, const float *v) {
#pragma unroll
    for (int c = 0; c < C; c += 8) {
        uint4 q[3];
        split3_pair(v[c + 0], v[c + 1], q[0].x, q[1].x, q[2].x);
        split3_pair(v[c + 2], v[c + 3], q[0].y, q[1].y, q[2].y);
        split3_pair(v[c + 4], v[c + 5], q[0].z, q[1].z, q[2].z);
        split3_pair(v[c + 6], v[c + 7], q[0].w, q[1].w, q[2].w);
#pragma unroll
        for (int p = 0; p < 3; ++p) *reinterpret_cast<uint4 *>(buf + p * piece + rb(r, c0 + c, N)) = q[p];
    }
}

// Row r of a tile with N columns (N % 8 == 0) as three BF16 pieces `piece` elements apart.
template <int N>
__device__ __forceinline__ void store_row3(__nv_bfloat16 *buf, int piece, int r, const float *v) {
    store_cols3<N, N>(buf, piece, r, 0, v);
}

// The forward weight operands (W^T, layout of load_weights_tc) in three pieces, kFwdW elements apart.
__device__ void load_weights_x6(const float *__restrict__ w, __nv_bfloat16 *sw) {
    const __nv_bfloat16 zero = __float2bfloat16_rn(0.f);
    for (int i = threadIdx.x; i < 3 * kFwdW; i += blockDim.x) sw[i] = zero;
    __syncthreads();
    for (int i = threadIdx.x; i < kNW; i += blockDim.x) {
        int off;
        if (i < kW1) { const int in = i / 64, out = i % 64; off = kF0 + rb(out, in, 32); }
        else if (i < kW2) { const int j = i - kW1, in = j / 16, out = j % 16; off = kF1 + rb(out, in, 64); }
        else if (i < kW3) { const int j = i - kW2, in = j / 64, out = j % 64; off = kF2 + rb(out, in, 32); }
        else if (i < kW4) { const int j = i - kW3, in = j / 64, out = j % 64; off = kF3 + rb(out, in, 64); }
        else { const int j = i - kW4, in = j / 3, out = j % 3; off = kF4 + rb(out, in, 64); }
        float a, b, c;
        split3(w[i], a, b, c);
        sw[off] = __float2bfloat16_rn(a);
        sw[kFwdW + off] = __float2bfloat16_rn(b);
        sw[2 * kFwdW + off] = __float2bfloat16_rn(c);
    }
}

// D (tmem) = A @ B^T to FP32 accuracy: the six piece products, smallest first -- a3 b1, a2 b2,
// a1 b3, a2 b1, a1 b2, a1 b1 (A's pieces `a_piece`, B's `b_piece` elements apart).
__device__ __forceinline__ void mma_kk_x6(std::uint32_t d, const __nv_bfloat16 *a, int a_piece, const __nv_bfloat16 *b,
                                          int K, int N, int b_piece = kFwdW) {
    const int ap[6] = {2, 1, 0, 1, 0, 0}, bp[6] = {0, 1, 2, 0, 1, 0};
    const std::uint32_t id = tc::idesc_kf16(128, N, Bf16Op::kFmt, false, false), sbo = (std::uint32_t)K * 16;
    const tc::SDesc da = tc::sdesc2(smem_addr(a), 128, sbo), db = tc::sdesc2(smem_addr(b), 128, sbo);
    // pieces are a_piece / b_piece elements (2 bytes each) apart: a_piece / 8 in 16-byte units
#pragma unroll
    for (int k = 0; k < 6; ++k)
#pragma unroll
        for (int j = 0; j < K / 16; ++j)
            tc::mma_bf16(d, da, (std::uint32_t)(ap[k] * (a_piece / 8) + 16 * j), db,
                         (std::uint32_t)(bp[k] * (b_piece / 8) + 16 * j), id, k > 0 || j > 0);
}

// D (tmem, M = 64) (+)= A^T @ B over the tile's 128 samples to FP32 accuracy (mma_mn on the six
// piece products; A's pieces kX6Piece elements apart, B's b_piece).
__device__ __forceinline__ void mma_mn_x6(std::uint32_t d, const __nv_bfloat16 *a, const __nv_bfloat16 *b, int N,
                                          bool acc, int b_piece = kX6Piece) {
    const int ap[6] = {2, 1, 0, 1, 0, 0}, bp[6] = {0, 1, 2, 0, 1, 0};
    const std::uint32_t id = tc::idesc_kf16(64, N, Bf16Op::kFmt, true, true), la = 64 * 16, lb = (std::uint32_t)N * 16;
    const tc::SDesc da = tc::sdesc2(smem_addr(a), la, 128), db = tc::sdesc2(smem_addr(b), lb, 128);
    static_assert(kX6Piece % 8 == 0, "pieces start on 16-byte boundaries");
#pragma unroll
    for (int k = 0; k < 6; ++k)
#pragma unroll
        for (int j = 0; j < kRows / 16; ++j)
            tc::mma_bf16(d, da, (std::uint32_t)(ap[k] * (kX6Piece / 8)) + j * 2 * la / 16, db,
                         (std::uint32_t)(bp[k] * (b_piece / 8)) + j * 2 * lb / 16, id, acc || k > 0 || j > 0);
}

template <bool kDensity>
__global__ void __launch_bounds__(kX6Wgs * 128, 1) mlp_x6_forward_kernel(
    std::uint32_t n, const std::uint32_t *__restrict__ count, const float *__restrict__ enc,
    const float *__restrict__ dirs, const float *__restrict__ weights, float *__restrict__ out) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ std::uint64_t bars[kX6Wgs];
    __shared__ std::uint32_t tbase;
    __shared__ int fails[kX6Wgs];
    __nv_bfloat16 *sw = reinterpret_cast<__nv_bfloat16 *>(smem_raw);
    const int g = threadIdx.x / 128, r = threadIdx.x % 128, q = (threadIdx.x / 32) % 4;
    __nv_bfloat16 *act = sw + 3 * kFwdW + g * kX6WgAct;
    load_weights_x6(weights, sw);
    if (threadIdx.x == 0) {
        for (int k = 0; k < kX6Wgs; ++k) {
            tc::mbar_init(&bars[k], 1);
            fails[k] = 0;
        }
        tc::fence_mbar_init();
    }
    if (threadIdx.x < 32) tc::tmem_alloc(&tbase, 256);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    WarpGroup wg{g, r, tbase + (std::uint32_t)g * 64u + ((std::uint32_t)(q * 32) << 16), &bars[g], 0u, &fails[g]};
    const bool leader = r == 0;
    const std::uint32_t n_act = active_count(n, count);
    const std::uint32_t n_tiles = (n_act + kRows - 1) / kRows;
    for (std::uint32_t tile = blockIdx.x * kX6Wgs + g; tile < n_tiles; tile += gridDim.x * kX6Wgs) {
        const std::size_t s = (std::size_t)tile * kRows + r;
        const bool valid = s < n_act;
        float v[64];
        {
            EncRow<Bf16Op, false> row;
            row.load(enc, s, valid);
            store_row3<32>(act, kX6Piece, r, row.v);
        }
        // layer 0: h1 = relu(enc W0)
        wg.sync();
        if (leader) { mma_kk_x6(wg.tm, act, kX6Piece, sw + kF0, 32, 64); tc::commit(wg.bar); }
        wg.wait();
        tc::ld64(wg.tm, v);
#pragma unroll
        for (int i = 0; i < 64; ++i) v[i] = fmaxf(v[i], 0.f);
        store_row3<64>(act, kX6Piece, r, v);
        // layer 1: x = h1 W1
        wg.sync();
        if (leader) { mma_kk_x6(wg.tm, act, kX6Piece, sw + kF1, 64, 16); tc::commit(wg.bar); }
        wg.wait();
        tc::ld16(wg.tm, v);
        if (kDensity) {
            if (valid) out[s] = expf(v[0]);
        } else {
            const float x0 = v[0];
            float dir[3] = {0.f, 0.f, 1.f};
            if (valid) {
                dir[0] = dirs[s * 3 + 0];
                dir[1] = dirs[s * 3 + 1];
                dir[2] = dirs[s * 3 + 2];
            }
            sh4(dir[0], dir[1], dir[2], v + 16);
            store_row3<32>(act, kX6Piece, r, v);
            // layer 2: h2 = relu([x, sh] W2)
            wg.sync();
            if (leader) { mma_kk_x6(wg.tm, act, kX6Piece, sw + kF2, 32, 64); tc::commit(wg.bar); }
            wg.wait();
            tc::ld64(wg.tm, v);
#pragma unroll
            for (int i = 0; i < 64; ++i) v[i] = fmaxf(v[i], 0.f);
            store_row3<64>(act, kX6Piece, r, v);
            // layer 3: h3 = relu(h2 W3)
            wg.sync();
            if (leader) { mma_kk_x6(wg.tm, act, kX6Piece, sw + kF3, 64, 64); tc::commit(wg.bar); }
            wg.wait();
            tc::ld64(wg.tm, v);
#pragma unroll
            for (int i = 0; i < 64; ++i) v[i] = fmaxf(v[i], 0.f);
            store_row3<64>(act, kX6Piece, r, v);
            // layer 4: rgb = sigmoid(h3 W4)
            wg.sync();
            if (leader) { mma_kk_x6(wg.tm, act, kX6Piece, sw + kF4, 64, 16); tc::commit(wg.bar); }
            wg.wait();
            tc::ld16(wg.tm, v);
            if (valid) {
                reinterpret_cast<float4 *>(out)[s] =
                    make_float4(expf(x0), 1.f / (1.f + expf(-v[0])), 1.f / (1.f + expf(-v[1])), 1.f / (1.f + expf(-v[2])));
            }
        }
        tc::bar_sync(1 + g, 128);   // every thread has read the last layer before the next tile's rows
        if (*wg.fail) break;
    }
    if (*wg.fail && r == 0) atomicOr(&g_device_error, 1u);
    tc::fence_before();
    __syncthreads();
    if (threadIdx.x < 32) tc::tmem_free(tbase, 256);
}

// ------------------------------------------------ FP32-accurate backward on the tensor cores
//
// ngp_field_backward with the same three-piece BF16 products as the forward above.  A CTA (one per
// SM) works on one tile of 128 samples at a time with 256 threads, two per sample row: thread
// (r, h) owns columns [w h, w (h + 1)) of a layer of width 2w.  The recomputed forward leaves each
// thread's share of the layer inputs the backward needs again in registers (h1 values, x or the
// SH features, the encodings, and the relu decisions of h1, h2, h3 as bit masks; h2 stays in Q), so
// tensor memory holds only the current layer's result and the dW accumulators, and shared memory
// only the operands of the layer at hand: two three-piece buffers P and Q, 48 KB each, and dL/da4
// (D4, 12 KB), beside the weights' three pieces in both layouts (W^T for the forward, W for the
// data gradients).  Each adjoint step issues the data-gradient MMA (thread 0) and the
// weight-gradient MMA (thread 32; M = 64, the tile's samples as the contraction, accumulated in
// tensor memory across all tiles of the CTA) on the same operands; the next step's gradient and
// layer input then overwrite P and Q once both have completed.
constexpr int kB6Threads = 256;
constexpr int kB6Weights = 3 * kAllW;                                               // pieces kAllW apart
constexpr int kD4Piece = kRows * 16;                                                // one piece of dL/da4 [128][16]
constexpr std::size_t kB6Smem = (std::size_t)(kB6Weights + 2 * kX6WgAct + 3 * kD4Piece) * 2;   // 222 KB
static_assert(kB6Smem + 128 <= 232448, "the backward's shared memory fits one CTA per SM");
// Tensor-memory columns: every layer's result, then the dW accumulators.
constexpr std::uint32_t kTD = 0;
constexpr std::uint32_t kTA0 = 64, kTA1 = 96, kTA2 = 112, kTA3 = 144, kTA4 = 208, kTCols = 256;
static_assert(kTA4 + 16 <= kTCols, "tensor-memory columns");

// The weights' three pieces in the forward (W^T) and backward (W) operand layouts of load_weights_tc.
__device__ void load_weights_x6b(const float *__restrict__ w, __nv_bfloat16 *sw) {
    const __nv_bfloat16 zero = __float2bfloat16_rn(0.f);
    for (int i = threadIdx.x; i < kB6Weights; i += blockDim.x) sw[i] = zero;
    __syncthreads();
    for (int i = threadIdx.x; i < kNW; i += blockDim.x) {
        int f, b = -1;
        if (i < kW1) { const int in = i / 64, out = i % 64; f = kF0 + rb(out, in, 32); b = kG0 + rb(in, out, 64); }
        else if (i < kW2) { const int j = i - kW1, in = j / 16, out = j % 16; f = kF1 + rb(out, in, 64); b = kG1 + rb(in, out, 16); }
        else if (i < kW3) {
            const int j = i - kW2, in = j / 64, out = j % 64;
            f = kF2 + rb(out, in, 32);
            if (in < 16) b = kG2 + rb(in, out, 64);   // the data gradient needs the x rows only
        }
        else if (i < kW4) { const int j = i - kW3, in = j / 64, out = j % 64; f = kF3 + rb(out, in, 64); b = kG3 + rb(in, out, 64); }
        else { const int j = i - kW4, in = j / 3, out = j % 3; f = kF4 + rb(out, in, 64); b = kG4 + rb(in, out, 16); }
        float p[3];
        split3(w[i], p[0], p[1], p[2]);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const __nv_bfloat16 v = __float2bfloat16_rn(p[k]);
            sw[k * kAllW + f] = v;
            if (b >= 0) sw[k * kAllW + b] = v;
        }
    }
}

// relu over 32 values in place; bit i of the result is the decision v[i] > 0.
__device__ __forceinline__ std::uint32_t relu_bits32(float *v) {
    std::uint32_t m = 0;
#pragma unroll
    for (int i = 0; i < 32; ++i) {
        m |= (v[i] > 0.f ? 1u : 0u) << i;
        v[i] = fmaxf(v[i], 0.f);
    }
    return m;
}

// The relu adjoint: v[i] where bit i of m is set, else 0.
__device__ __forceinline__ void mask_bits32(float *v, std::uint32_t m) {
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = (m >> i) & 1u ? v[i] : 0.f;
}

// `grad_scale` multiplies dL/ddrgb; `partials` receives one [9408] dL/dW partial per CTA (grid =
// the SM count), zero for a CTA without tiles.  dL/denc rows past the active count are not written.
__global__ void __launch_bounds__(kB6Threads, 1) mlp_x6_backward_kernel(
    std::uint32_t n, const std::uint32_t *__restrict__ count, const float *__restrict__ enc,
    const float *__restrict__ dirs, const float *__restrict__ weights, const float *__restrict__ dL_ddrgb,
    const float *__restrict__ grad_scale, float *__restrict__ dL_denc, float *__restrict__ partials) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ std::uint64_t bar, wbar;   // data-path MMAs; weight-gradient MMAs
    __shared__ std::uint32_t tbase;
    __shared__ int fail;
    __nv_bfloat16 *sw = reinterpret_cast<__nv_bfloat16 *>(smem_raw);
    // P, Q: activation rows (three pieces); D4: dL/da4 (three pieces), apart from them so that Q
    // keeps h2 from the forward until layer 3's weight gradient reads it.
    __nv_bfloat16 *P = sw + kB6Weights, *Q = P + kX6WgAct, *D4 = Q + kX6WgAct;
    const int r = threadIdx.x % kRows, h = threadIdx.x / kRows;   // h is uniform over a warp
    load_weights_x6b(weights, sw);
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        tc::mbar_init(&wbar, 1);
        fail = 0;
        tc::fence_mbar_init();
    }
    if (threadIdx.x < 32) tc::tmem_alloc(&tbase, kTCols);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const std::uint32_t t0 = tbase;                                            // for the MMAs (lane 0)
    const std::uint32_t tm = tbase + ((std::uint32_t)((r / 32) * 32) << 16);   // this warp's lanes
    // Thread 0 issues the data path's MMAs and commits them to `bar`; thread 32 (another warp, so
    // the two issue streams run side by side) issues the weight gradients' MMAs and commits them to
    // `wbar`.  The two streams write different tensor-memory columns and only read shared memory.
    const bool leader = threadIdx.x == 0, wleader = threadIdx.x == 32;
    std::uint32_t phase = 0;
    auto sync = [&] {
        tc::fence_async_smem();
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
    };
    auto wait = [&] {
        if (!tc::mbar_wait(&bar, phase, kWaitLimit)) fail = 1;
        phase ^= 1u;
        tc::fence_after();
    };
    // A backward layer's data gradient (which the next layer waits for) completes on `bar`, its
    // weight gradient on `wbar`: the data gradient's epilogue reads tensor memory while the
    // weight-gradient MMAs still run, and waits for them only before it overwrites the P/Q rows
    // they read.
    std::uint32_t wphase = 0;
    auto wait_w = [&] {
        if (!tc::mbar_wait(&wbar, wphase, kWaitLimit)) fail = 1;
        wphase ^= 1u;
        tc::fence_after();
    };

    const float gs = grad_scale != nullptr ? *grad_scale : 1.f;
    const std::uint32_t n_act = active_count(n, count);
    const std::uint32_t n_tiles = (n_act + kRows - 1) / kRows;
    // This thread's inputs of a tile: encoding columns [16h, 16h + 16), and dL/ddrgb (h = 0) or the
    // direction (h = 1), fetched one tile ahead.
    float ne[16];
    float4 nx;
    auto fetch = [&](std::uint32_t tile) {
        const std::size_t s = (std::size_t)tile * kRows + r;
        const bool valid = s < n_act;
#pragma unroll
        for (int c = 0; c < 16; c += 4) {
            float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
            if (valid) q = *reinterpret_cast<const float4 *>(enc + s * 32 + 16 * h + c);
            ne[c] = q.x;
            ne[c + 1] = q.y;
            ne[c + 2] = q.z;
            ne[c + 3] = q.w;
        }
        if (h == 0) nx = valid ? reinterpret_cast<const float4 *>(dL_ddrgb)[s] : make_float4(0.f, 0.f, 0.f, 0.f);
        else nx = valid ? make_float4(dirs[s * 3 + 0], dirs[s * 3 + 1], dirs[s * 3 + 2], 0.f) : make_float4(0.f, 0.f, 1.f, 0.f);
    };
    bool first = true;
    fetch(blockIdx.x);
    for (std::uint32_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        const std::size_t s = (std::size_t)tile * kRows + r;
        const bool valid = s < n_act;
        float e[16], v[32], h1[32], h2[32], xs[16];   // h2 is dead once stored in Q
#pragma unroll
        for (int i = 0; i < 16; ++i) e[i] = ne[i];
        const float4 x4 = nx;
        fetch(tile + gridDim.x);

        // forward: h1 = relu(enc W0), x = h1 W1, h2 = relu([x, sh] W2), h3 = relu(h2 W3), a4 = h3 W4
        store_cols3<32, 16>(P, kX6Piece, r, 16 * h, e);
        sync();
        if (leader) { mma_kk_x6(t0 + kTD, P, kX6Piece, sw + kF0, 32, 64, kAllW); tc::commit(&bar); }
        wait();
        tc::ld32(tm + kTD + 32 * h, h1);
        const std::uint32_t m1 = relu_bits32(h1);
        store_cols3<64, 32>(Q, kX6Piece, r, 32 * h, h1);
        sync();
        if (leader) { mma_kk_x6(t0 + kTD, Q, kX6Piece, sw + kF1, 64, 16, kAllW); tc::commit(&bar); }
        wait();
        if (h == 0) tc::ld16(tm + kTD, xs);     // x
        else sh4(x4.x, x4.y, x4.z, xs);          // SH of the direction
        store_cols3<32, 16>(P, kX6Piece, r, 16 * h, xs);
        sync();
        if (leader) { mma_kk_x6(t0 + kTD, P, kX6Piece, sw + kF2, 32, 64, kAllW); tc::commit(&bar); }
        wait();
        tc::ld32(tm + kTD + 32 * h, h2);
        const std::uint32_t m2 = relu_bits32(h2);
        store_cols3<64, 32>(Q, kX6Piece, r, 32 * h, h2);
        sync();
        if (leader) { mma_kk_x6(t0 + kTD, Q, kX6Piece, sw + kF3, 64, 64, kAllW); tc::commit(&bar); }
        wait();
        tc::ld32(tm + kTD + 32 * h, v);
        const std::uint32_t m3 = relu_bits32(v);
        store_cols3<64, 32>(P, kX6Piece, r, 32 * h, v);   // P = h3
        sync();
        if (leader) { mma_kk_x6(t0 + kTD, P, kX6Piece, sw + kF4, 64, 16, kAllW); tc::commit(&bar); }
        wait();

        // output layer: dL/da4 (3 columns, padded to 16) and dL/dx0 through the truncated exponential
        float dx0 = 0.f;
        if (h == 0) {
            tc::ld16(tm + kTD, v);
            float d[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) d[i] = 0.f;
            const float g[3] = {x4.y, x4.z, x4.w};
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float rgb = 1.f / (1.f + expf(-v[c]));
                d[c] = gs * g[c] * rgb * (1.f - rgb);
            }
            dx0 = gs * x4.x * expf(fminf(fmaxf(xs[0], -15.f), 15.f));
            store_cols3<16, 16>(D4, kD4Piece, r, 0, d);   // D4 = dA4
        }
        // layer 4: dW4 += h3^T dA4;  dh3 = dA4 W4^T
        sync();
        if (leader) {
            mma_kk_x6(t0 + kTD, D4, kD4Piece, sw + kG4, 16, 64, kAllW);
            tc::commit(&bar);
        } else if (wleader) {
            mma_mn_x6(t0 + kTA4, P, D4, 16, !first, kD4Piece);
            tc::commit(&wbar);
        }
        wait();
        tc::ld32(tm + kTD + 32 * h, v);
        mask_bits32(v, m3);
        wait_w();
        store_cols3<64, 32>(P, kX6Piece, r, 32 * h, v);   // P = dA3; Q still holds h2
        // layer 3: dW3^T += dA3^T h2;  dh2 = dA3 W3^T
        sync();
        if (leader) {
            mma_kk_x6(t0 + kTD, P, kX6Piece, sw + kG3, 64, 64, kAllW);
            tc::commit(&bar);
        } else if (wleader) {
            mma_mn_x6(t0 + kTA3, P, Q, 64, !first);
            tc::commit(&wbar);
        }
        wait();
        tc::ld32(tm + kTD + 32 * h, v);
        mask_bits32(v, m2);
        wait_w();
        store_cols3<64, 32>(Q, kX6Piece, r, 32 * h, v);   // Q = dA2
        store_cols3<32, 16>(P, kX6Piece, r, 16 * h, xs);  // P = [x, sh]
        // layer 2: dW2^T += dA2^T [x, sh];  dx = dA2 W2[:16]^T
        sync();
        if (leader) {
            mma_kk_x6(t0 + kTD, Q, kX6Piece, sw + kG2, 64, 16, kAllW);
            tc::commit(&bar);
        } else if (wleader) {
            mma_mn_x6(t0 + kTA2, Q, P, 32, !first);
            tc::commit(&wbar);
        }
        wait();
        if (h == 0) {
            tc::ld16(tm + kTD, v);
            v[0] += dx0;
        }
        wait_w();
        if (h == 0) {
            store_cols3<16, 16>(P, kX6Piece, r, 0, v);    // P = dx
        }
        store_cols3<64, 32>(Q, kX6Piece, r, 32 * h, h1);  // Q = h1
        // layer 1: dW1 += h1^T dx;  dh1 = dx W1^T
        sync();
        if (leader) {
            mma_kk_x6(t0 + kTD, P, kX6Piece, sw + kG1, 16, 64, kAllW);
            tc::commit(&bar);
        } else if (wleader) {
            mma_mn_x6(t0 + kTA1, Q, P, 16, !first);
            tc::commit(&wbar);
        }
        wait();
        tc::ld32(tm + kTD + 32 * h, v);
        mask_bits32(v, m1);
        wait_w();
        store_cols3<64, 32>(Q, kX6Piece, r, 32 * h, v);   // Q = dA1
        store_cols3<32, 16>(P, kX6Piece, r, 16 * h, e);   // P = enc
        // layer 0: dW0^T += dA1^T enc;  denc = dA1 W0^T
        sync();
        if (leader) {
            mma_kk_x6(t0 + kTD, Q, kX6Piece, sw + kG0, 64, 32, kAllW);
            tc::commit(&bar);
        } else if (wleader) {
            mma_mn_x6(t0 + kTA0, Q, P, 32, !first);
            tc::commit(&wbar);
        }
        wait();
        tc::ld16(tm + kTD + 16 * h, v);
        if (valid) {
#pragma unroll
            for (int c = 0; c < 16; c += 4)
                *reinterpret_cast<float4 *>(dL_denc + s * 32 + 16 * h + c) = make_float4(v[c], v[c + 1], v[c + 2], v[c + 3]);
        }
        wait_w();   // the next tile overwrites P and Q
        first = false;
        tc::fence_before();
        __syncthreads();   // every thread has read the tile's results before the next tile's MMAs
        if (fail) break;
    }
    if (fail && threadIdx.x == 0) atomicOr(&g_device_error, 1u);

    // dW, in the packed [in][out] layout: row m of an M = 64 accumulator sits in TMEM lane
    // m64_lane(m); the two threads of a lane read different accumulators.
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    float *p = partials + (std::size_t)blockIdx.x * kNW;
    if (first) {
        for (int i = threadIdx.x; i < kNW; i += blockDim.x) p[i] = 0.f;
    } else {
        const int m = (r & 31) < 16 ? (r >> 5) * 16 + (r & 15) : -1;
        float a[64];
        if (h == 0) {
            tc::ld32(tm + kTA0, a);   // dW0^T: row = out, 32 columns = in
            if (m >= 0)
#pragma unroll
                for (int i = 0; i < 32; ++i) p[kW0 + i * 64 + m] = a[i];
            tc::ld16(tm + kTA1, a);   // dW1: row = in, 16 columns = out
            if (m >= 0)
#pragma unroll
                for (int o = 0; o < 16; ++o) p[kW1 + m * 16 + o] = a[o];
            tc::ld16(tm + kTA4, a);   // dW4: row = in, columns 0..2 = out
            if (m >= 0)
#pragma unroll
                for (int o = 0; o < 3; ++o) p[kW4 + m * 3 + o] = a[o];
        } else {
            tc::ld32(tm + kTA2, a);   // dW2^T: row = out, 32 columns = in
            if (m >= 0)
#pragma unroll
                for (int i = 0; i < 32; ++i) p[kW2 + i * 64 + m] = a[i];
            tc::ld64(tm + kTA3, a);   // dW3^T: row = out, 64 columns = in
            if (m >= 0)
#pragma unroll
                for (int i = 0; i < 64; ++i) p[kW3 + i * 64 + m] = a[i];
        }
    }
    tc::fence_before();
    __syncthreads();
    if (threadIdx.x < 32) tc::tmem_free(tbase, kTCols);
}

// ------------------------------------------------------------------ proposal network (FP16)
//
// The learned proposal's MLP x = relu(relu(enc @ P0) @ P1) @ P2 (enc 8 features; P0 [8][64],
// P1 [64][64], P2 [64][1] packed, 4672 floats) with FP16 operands and FP32 accumulation: layer 0
// has its K padded to 16 with zeros, layer 2 its N padded to 16.  Same structure as the field
// forward above (a warpgroup per tile of 128 points, one point per thread).
constexpr int kQ0 = 0, kQ1 = 1024, kQ2 = 5120, kQW = 6144;        // FP16 operands: P0^T [64][16], P1^T [64][64], P2^T [16][64]
constexpr int kQX = 0, kQH1 = 2048, kQH2 = 10240, kQAct = 18432;  // per warpgroup: X [128][16], H1, H2 [128][64]
constexpr int kPropWgs = 4;
constexpr std::size_t kPropSmem = (std::size_t)(kQW + kPropWgs * kQAct) * 2;

template <int NWG>
__global__ void __launch_bounds__(NWG * 128, 1) prop_f16_forward_kernel(
    std::uint32_t n, const std::uint32_t *__restrict__ count, const float *__restrict__ enc,
    const float *__restrict__ weights, float *__restrict__ x_out) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ std::uint64_t bars[NWG];
    __shared__ std::uint32_t tbase;
    __shared__ int fails[NWG];
    __half *sw = reinterpret_cast<__half *>(smem_raw);
    const int g = threadIdx.x / 128, r = threadIdx.x % 128, q = (threadIdx.x / 32) % 4;
    __half *act = sw + kQW + g * kQAct;
    for (int i = threadIdx.x; i < kQW; i += blockDim.x) sw[i] = __float2half_rn(0.f);
    __syncthreads();
    for (int i = threadIdx.x; i < 4672; i += blockDim.x) {
        const __half v = __float2half_rn(weights[i]);
        if (i < 512) {           // P0 [8][64] -> P0^T [64][16]
            const int in = i / 64, out = i % 64;
            sw[kQ0 + rb(out, in, 16)] = v;
        } else if (i < 4608) {   // P1 [64][64] -> P1^T
            const int j = i - 512, in = j / 64, out = j % 64;
            sw[kQ1 + rb(out, in, 64)] = v;
        } else {                 // P2 [64][1] -> P2^T row 0 of [16][64]
            sw[kQ2 + rb(0, i - 4608, 64)] = v;
        }
    }
    if (threadIdx.x == 0) {
        for (int k = 0; k < NWG; ++k) {
            tc::mbar_init(&bars[k], 1);
            fails[k] = 0;
        }
        tc::fence_mbar_init();
    }
    if (threadIdx.x < 32) tc::tmem_alloc(&tbase, 512);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    WarpGroup wg{g, r, tbase + (std::uint32_t)g * 128u + ((std::uint32_t)(q * 32) << 16), &bars[g], 0u, &fails[g]};
    const bool leader = r == 0;
    const std::uint32_t n_act = active_count(n, count);
    const std::uint32_t n_tiles = (n_act + kRows - 1) / kRows;
    for (std::uint32_t tile = blockIdx.x * NWG + g; tile < n_tiles; tile += gridDim.x * NWG) {
        const std::size_t s = (std::size_t)tile * kRows + r;
        const bool valid = s < n_act;
        float v[64];
#pragma unroll
        for (int c = 0; c < 16; ++c) v[c] = 0.f;
        if (valid) {
            const float4 a = reinterpret_cast<const float4 *>(enc + s * 8)[0];
            const float4 b = reinterpret_cast<const float4 *>(enc + s * 8)[1];
            v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
        }
        store_row<F16Op, 16>(act + kQX, r, v);
        wg.sync();
        if (leader) { mma_kk<F16Op>(wg.tm + kDA, act + kQX, sw + kQ0, 16, 64, false); tc::commit(wg.bar); }
        wg.wait();
        tc::ld64(wg.tm + kDA, v);
#pragma unroll
        for (int i = 0; i < 64; ++i) v[i] = fmaxf(v[i], 0.f);
        store_row<F16Op, 64>(act + kQH1, r, v);
        wg.sync();
        if (leader) { mma_kk<F16Op>(wg.tm + kDA, act + kQH1, sw + kQ1, 64, 64, false); tc::commit(wg.bar); }
        wg.wait();
        tc::ld64(wg.tm + kDA, v);
#pragma unroll
        for (int i = 0; i < 64; ++i) v[i] = fmaxf(v[i], 0.f);
        store_row<F16Op, 64>(act + kQH2, r, v);
        wg.sync();
        if (leader) { mma_kk<F16Op>(wg.tm + kDB, act + kQH2, sw + kQ2, 64, 16, false); tc::commit(wg.bar); }
        wg.wait();
        tc::ld16(wg.tm + kDB, v);
        if (valid) x_out[s] = v[0];
        tc::bar_sync(1 + g, 128);
        if (*wg.fail) break;
    }
    if (*wg.fail && r == 0) atomicOr(&g_device_error, 1u);
    tc::fence_before();
    __syncthreads();
    if (threadIdx.x < 32) tc::tmem_free(tbase, 512);
}

constexpr int kFwdWgs = 3, kBwdWgs = 2;
constexpr std::size_t kFwdSmem = (std::size_t)(kFwdW + kFwdWgs * kFwdAct) * 2;
constexpr std::size_t kBwdSmem = (std::size_t)(kAllW + kBwdWgs * kBwdAct) * 2;
static_assert(kBwdAct * 2 >= kNW * 4, "dW sums fit over a warpgroup's rows");

}  // namespace

// ------------------------------------------------------------------------------- launchers

namespace {

// Tensor map of 16-bit encodings enc [n][32] (n a multiple of 8) as the 4-D view [n/8][4][8][8]
// (row group, column chunk, row, column; byte strides 512, 16, 64) with a box of one 128-row tile:
// the box lands in shared memory in the MMA operand's core-matrix layout.  False when the CUDA
// driver entry point is unavailable or n does not qualify (the caller then loads the rows itself).
template <class E>
int encode_enc_map(CUtensorMap *map, const void *enc, std::uint32_t n, bool *ok) {
    *ok = false;
    std::memset(map, 0, sizeof(*map));
    if (n == 0 || n % 8 != 0) return NGP_OK;
    // looked up once per process (a function-local static is initialised exactly once, thread-safely)
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        (void)cudaGetLastError();
        return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
    }();
    if (fn == nullptr) return NGP_OK;
    const cuuint64_t dims[4] = {8, 8, 4, n / 8};
    const cuuint64_t strides[3] = {64, 16, 512};   // bytes: next row, next 8-column chunk, next 8-row group
    const cuuint32_t box[4] = {8, 8, 4, kRows / 8};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUtensorMapDataType dt = std::is_same<E, Bf16Op>::value ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
    const CUresult r = fn(map, dt, 4, const_cast<void *>(enc), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    NGP_CHECK_ARG(r == CUDA_SUCCESS, "mlp (tensor cores): cuTensorMapEncodeTiled rejected the encodings' tensor map");
    *ok = true;
    return NGP_OK;
}

template <class E, bool kHalf>
int launch_tc_forward(cudaStream_t stream, std::uint32_t n, const std::uint32_t *count, const void *enc,
                      const float *dirs, const float *weights, float *drgb) {
    using In = typename EncRow<E, kHalf>::In;
    NGP_CHECK_ARG(aligned16(enc) && aligned16(weights) && aligned16(drgb), "mlp (tensor cores): enc, weights and drgb must be 16-byte aligned");
    NGP_SMEM_LIMIT((mlp_tc_forward_kernel<E, kHalf, false, kFwdWgs>), kFwdSmem);
    if (kHalf) NGP_SMEM_LIMIT((mlp_tc_forward_kernel<E, kHalf, kHalf, kFwdWgs>), kFwdSmem);
    if (n == 0) return launch_status();
    CUtensorMap map;
    bool tma = false;
    if (kHalf) {
        const int st = encode_enc_map<E>(&map, enc, n, &tma);
        if (st != NGP_OK) return st;
    } else {
        std::memset(&map, 0, sizeof(map));
    }
    const unsigned tiles = (n + kRows - 1) / kRows;
    const unsigned want = (tiles + kFwdWgs - 1) / kFwdWgs;
    const unsigned grid = want < (unsigned)sm_count() ? want : (unsigned)sm_count();
    if (tma)
        mlp_tc_forward_kernel<E, kHalf, kHalf, kFwdWgs><<<grid, kFwdWgs * 128, kFwdSmem, stream>>>(
            n, count, static_cast<const In *>(enc), dirs, weights, drgb, map);
    else
        mlp_tc_forward_kernel<E, kHalf, false, kFwdWgs><<<grid, kFwdWgs * 128, kFwdSmem, stream>>>(
            n, count, static_cast<const In *>(enc), dirs, weights, drgb, map);
    count_launches(1);
    return launch_status();
}

template <class E, bool kHalf>
int launch_tc_density(cudaStream_t stream, std::uint32_t n, const void *enc, const float *weights, float *sigma) {
    using In = typename EncRow<E, kHalf>::In;
    NGP_CHECK_ARG(aligned16(enc) && aligned16(weights), "mlp (tensor cores): enc and weights must be 16-byte aligned");
    NGP_SMEM_LIMIT((mlp_tc_density_kernel<E, kHalf, kFwdWgs>), kFwdSmem);
    if (n == 0) return launch_status();
    const unsigned tiles = (n + kRows - 1) / kRows;
    const unsigned want = (tiles + kFwdWgs - 1) / kFwdWgs;
    const unsigned grid = want < (unsigned)sm_count() ? want : (unsigned)sm_count();
    mlp_tc_density_kernel<E, kHalf, kFwdWgs><<<grid, kFwdWgs * 128, kFwdSmem, stream>>>(n, static_cast<const In *>(enc),
                                                                                        weights, sigma);
    count_launches(1);
    return launch_status();
}

template <class E, bool kHalf>
int launch_tc_backward(cudaStream_t stream, std::uint32_t n, const std::uint32_t *count, const void *enc,
                       const float *dirs, const float *weights, const float *dL_ddrgb, const float *grad_scale,
                       NgpLossScale *ls, void *dL_denc, float *partials, unsigned *grid_out) {
    using In = typename EncRow<E, kHalf>::In;
    NGP_CHECK_ARG(aligned16(enc) && aligned16(weights) && aligned16(dL_ddrgb) && aligned16(dL_denc) && aligned16(partials),
                  "mlp (tensor cores): buffers must be 16-byte aligned");
    NGP_SMEM_LIMIT((mlp_tc_backward_kernel<E, kHalf, false, kBwdWgs>), kBwdSmem);
    if (kHalf) NGP_SMEM_LIMIT((mlp_tc_backward_kernel<E, kHalf, kHalf, kBwdWgs>), kBwdSmem);
    CUtensorMap map;
    bool tma = false;
    if (kHalf) {
        const int st = encode_enc_map<E>(&map, enc, n, &tma);
        if (st != NGP_OK) return st;
    } else {
        std::memset(&map, 0, sizeof(map));
    }
    const unsigned grid = (unsigned)sm_count();
    if (tma)
        mlp_tc_backward_kernel<E, kHalf, kHalf, kBwdWgs><<<grid, kBwdWgs * 128, kBwdSmem, stream>>>(
            n, count, static_cast<const In *>(enc), dirs, weights, dL_ddrgb, grad_scale, ls, static_cast<In *>(dL_denc),
            partials, map);
    else
        mlp_tc_backward_kernel<E, kHalf, false, kBwdWgs><<<grid, kBwdWgs * 128, kBwdSmem, stream>>>(
            n, count, static_cast<const In *>(enc), dirs, weights, dL_ddrgb, grad_scale, ls, static_cast<In *>(dL_denc),
            partials, map);
    count_launches(1);
    *grid_out = grid;
    return launch_status();
}

}  // namespace

int launch_mlp_bf16_forward(cudaStream_t stream, std::uint32_t n, const std::uint32_t *count, const float *enc,
                            const float *dirs, const float *weights, float *drgb) {
    return launch_tc_forward<Bf16Op, false>(stream, n, count, enc, dirs, weights, drgb);
}

int launch_mlp_bf16_density(cudaStream_t stream, std::uint32_t n, const float *enc, const float *weights, float *sigma) {
    return launch_tc_density<Bf16Op, false>(stream, n, enc, weights, sigma);
}

// `partials` holds at least sm_count() x 9408 floats; one partial per CTA, grid = sm_count().
int launch_mlp_bf16_backward(cudaStream_t stream, std::uint32_t n, const std::uint32_t *count, const float *enc,
                             const float *dirs, const float *weights, const float *dL_ddrgb, const float *grad_scale,
                             float *dL_denc, float *partials, unsigned *grid_out) {
    return launch_tc_backward<Bf16Op, false>(stream, n, count, enc, dirs, weights, dL_ddrgb, grad_scale, nullptr,
                                             dL_denc, partials, grid_out);
}

// The mixed-precision forms: `operand` NGP_DTYPE_BF16 or NGP_DTYPE_F16; `half_act` keeps the
// encodings and their gradient in the operand type instead of FP32.
#define NGP_TC_DISPATCH(call)                                                                          \
    do {                                                                                               \
        NGP_CHECK_ARG(operand == NGP_DTYPE_BF16 || operand == NGP_DTYPE_F16,                           \
                      "mlp (tensor cores): operand type must be NGP_DTYPE_BF16 or NGP_DTYPE_F16");     \
        if (operand == NGP_DTYPE_BF16) return half_act ? call(Bf16Op, true) : call(Bf16Op, false);    \
        return half_act ? call(F16Op, true) : call(F16Op, false);                                      \
    } while (0)

int launch_mlp_tc_forward(cudaStream_t stream, std::uint32_t operand, bool half_act, std::uint32_t n,
                          const std::uint32_t *count, const void *enc, const float *dirs, const float *weights,
                          float *drgb) {
#define NGP_CALL(E, H) launch_tc_forward<E, H>(stream, n, count, enc, dirs, weights, drgb)
    NGP_TC_DISPATCH(NGP_CALL);
#undef NGP_CALL
}

int launch_mlp_tc_density(cudaStream_t stream, std::uint32_t operand, bool half_act, std::uint32_t n, const void *enc,
                          const float *weights, float *sigma) {
#define NGP_CALL(E, H) launch_tc_density<E, H>(stream, n, enc, weights, sigma)
    NGP_TC_DISPATCH(NGP_CALL);
#undef NGP_CALL
}

int launch_mlp_tc_backward(cudaStream_t stream, std::uint32_t operand, bool half_act, std::uint32_t n,
                           const std::uint32_t *count, const void *enc, const float *dirs, const float *weights,
                           const float *dL_ddrgb, const float *grad_scale, NgpLossScale *ls, void *dL_denc,
                           float *partials, unsigned *grid_out) {
#define NGP_CALL(E, H) launch_tc_backward<E, H>(stream, n, count, enc, dirs, weights, dL_ddrgb, grad_scale, ls, dL_denc, partials, grid_out)
    NGP_TC_DISPATCH(NGP_CALL);
#undef NGP_CALL
}
#undef NGP_TC_DISPATCH

// The FP32 field forward and density on the tensor cores (mlp_x6_forward_kernel).
int launch_mlp_x6_forward(cudaStream_t stream, std::uint32_t n, const std::uint32_t *count, const float *enc,
                          const float *dirs, const float *weights, float *drgb) {
    NGP_CHECK_ARG(aligned16(enc) && aligned16(drgb), "mlp: enc and drgb must be 16-byte aligned");
    NGP_SMEM_LIMIT((mlp_x6_forward_kernel<false>), kX6Smem);
    if (n == 0) return launch_status();
    const unsigned tiles = (n + kRows - 1) / kRows;
    const unsigned want = (tiles + kX6Wgs - 1) / kX6Wgs;
    const unsigned grid = want < (unsigned)sm_count() ? want : (unsigned)sm_count();
    mlp_x6_forward_kernel<false><<<grid, kX6Wgs * 128, kX6Smem, stream>>>(n, count, enc, dirs, weights, drgb);
    count_launches(1);
    return launch_status();
}

int launch_mlp_x6_density(cudaStream_t stream, std::uint32_t n, const float *enc, const float *weights, float *sigma) {
    NGP_CHECK_ARG(aligned16(enc), "mlp: enc must be 16-byte aligned");
    NGP_SMEM_LIMIT((mlp_x6_forward_kernel<true>), kX6Smem);
    if (n == 0) return launch_status();
    const unsigned tiles = (n + kRows - 1) / kRows;
    const unsigned want = (tiles + kX6Wgs - 1) / kX6Wgs;
    const unsigned grid = want < (unsigned)sm_count() ? want : (unsigned)sm_count();
    mlp_x6_forward_kernel<true><<<grid, kX6Wgs * 128, kX6Smem, stream>>>(n, nullptr, enc, nullptr, weights, sigma);
    count_launches(1);
    return launch_status();
}

// The FP32 field backward on the tensor cores (mlp_x6_backward_kernel): one CTA per SM, at most
// `max_parts`, each writing one dL/dW partial to `partials` (that many x 9408 floats); their count
// in *grid_out.
int launch_mlp_x6_backward(cudaStream_t stream, std::uint32_t n, const std::uint32_t *count, const float *enc,
                           const float *dirs, const float *weights, const float *dL_ddrgb, const float *grad_scale,
                           float *dL_denc, float *partials, unsigned max_parts, unsigned *grid_out) {
    NGP_CHECK_ARG(aligned16(enc) && aligned16(dL_ddrgb) && aligned16(dL_denc) && aligned16(partials),
                  "mlp: buffers must be 16-byte aligned");
    NGP_CHECK_ARG(max_parts > 0, "mlp: no room for a dL/dW partial");
    NGP_SMEM_LIMIT(mlp_x6_backward_kernel, kB6Smem);
    const unsigned grid = (unsigned)sm_count() < max_parts ? (unsigned)sm_count() : max_parts;
    mlp_x6_backward_kernel<<<grid, kB6Threads, kB6Smem, stream>>>(n, count, enc, dirs, weights, dL_ddrgb, grad_scale,
                                                                   dL_denc, partials);
    count_launches(1);
    *grid_out = grid;
    return launch_status();
}

int launch_prop_f16_forward(cudaStream_t stream, std::uint32_t n, const std::uint32_t *count, const float *enc,
                            const float *weights, float *x) {
    NGP_CHECK_ARG(aligned16(enc), "proposal mlp (fp16): encodings must be 16-byte aligned");
    NGP_SMEM_LIMIT((prop_f16_forward_kernel<kPropWgs>), kPropSmem);
    if (n == 0) return launch_status();
    const unsigned tiles = (n + kRows - 1) / kRows;
    const unsigned want = (tiles + kPropWgs - 1) / kPropWgs;
    const unsigned grid = want < (unsigned)sm_count() ? want : (unsigned)sm_count();
    prop_f16_forward_kernel<kPropWgs><<<grid, kPropWgs * 128, kPropSmem, stream>>>(n, count, enc, weights, x);
    count_launches(1);
    return launch_status();
}

namespace {
// The bounded wait of the tensor-core kernels on an mbarrier that nothing completes: it gives up
// after `polls` polls and records the error word, as a kernel whose MMAs never finished would.
__global__ void bounded_wait_selftest_kernel(std::uint32_t polls) {
    __shared__ __align__(8) std::uint64_t bar;
    if (threadIdx.x != 0) return;
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
    if (!tc::mbar_wait(&bar, 0, polls)) atomicOr(&g_device_error, 1u);
}
}  // namespace

int launch_bounded_wait_selftest(cudaStream_t stream, std::uint32_t polls) {
    NGP_CHECK_ARG(polls > 0 && polls <= (1u << 20), "bounded-wait self-test: polls must be in [1, 2^20]");
    bounded_wait_selftest_kernel<<<1, 32, 0, stream>>>(polls);
    count_launches(1);
    return launch_status();
}

// Reads and clears the device error word (synchronises the device).
int device_status() {
    unsigned v = 0;
    NGP_CUDA_TRY(cudaDeviceSynchronize());
    NGP_CUDA_TRY(cudaMemcpyFromSymbol(&v, g_device_error, sizeof(v)));
    if (v != 0) {
        const unsigned zero = 0;
        NGP_CUDA_TRY(cudaMemcpyToSymbol(g_device_error, &zero, sizeof(zero)));
        set_last_status(NGP_ERR_DEVICE, "a tensor-core kernel gave up waiting for its MMAs");
        return NGP_ERR_DEVICE;
    }
    return launch_status();
}

}  // namespace ngp
