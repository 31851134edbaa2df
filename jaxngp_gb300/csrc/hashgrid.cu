// Multiresolution hash-grid encoder for sm_103a: forward gather and gradient scatter.
//
// Replaces HashGridEncoder.__call__ (models/encoders.py:83-256) and the scatter-add that JAX's
// autodiff makes of its gather (encoders.py:226).  In both directions a warp handles 32
// consecutive points at one level (lane = point): the level's scale, resolution and offset are
// uniform across the warp, and where neighbouring points share grid cells (samples along one
// ray, or rays of neighbouring pixels) the warp's gathers hit the same sectors.
//
// The index and weight arithmetic uses explicitly rounded intrinsics, one rounding per
// operation in the reference's order, so corner indices are bit-identical to the reference and
// encodings agree bit for bit with its float32 evaluation:
//   pos01  = (pos + bound) / (2*bound)                      encoders.py:87
//   ps     = pos01 * float32(scale_l) + 0.5                 encoders.py:216-218
//   corner = floor(ps) + {0,1}^3, converted to uint32       encoders.py:116-123
//            (saturating, as XLA converts on the GPU: a coordinate below the grid becomes 0)
//   index  = x + y*res + z*res^2           (dense levels)   encoders.py:134-155
//          = x ^ y*2654435761 ^ z*805459861 (hashed levels) encoders.py:157-177
//            then mod T, + offsets[l]; clamped to the table  encoders.py:179-189
//   weight = prod_d clip(o_d ? frac_d : 1 - frac_d, 0, 1)   encoders.py:191-213
//            (frac = modf's fractional part, signed like the coordinate)
//   enc    = sum over corners in corner order               encoders.py:231
#include "common.cuh"
#include "half.cuh"

namespace ngp {
namespace {

struct Corner8 {
    std::uint32_t idx[8];
    float w[8];
};

// Storage of a [rows][2] array (latent table, encodings, their gradients): FP32 pairs, or pairs of
// a 16-bit type packed in one 32-bit word.  get() widens to FP32; put() rounds to the type.
struct PairF32 {
    static constexpr std::uintptr_t kPairAlign = 16;
    static __device__ __forceinline__ float2 get(const void *a, std::size_t i) {
        return __ldg(reinterpret_cast<const float2 *>(a) + i);
    }
    // rows 2j and 2j + 1 in one 16-byte load
    static __device__ __forceinline__ void get_pair(const void *a, std::size_t j, float2 &lo, float2 &hi) {
        const float4 q = __ldg(reinterpret_cast<const float4 *>(a) + j);
        lo = make_float2(q.x, q.y);
        hi = make_float2(q.z, q.w);
    }
    static __device__ __forceinline__ void put(void *a, std::size_t i, float2 v) { reinterpret_cast<float2 *>(a)[i] = v; }
};

template <class E>
struct PairHalf {
    static constexpr std::uintptr_t kPairAlign = 8;
    static __device__ __forceinline__ float2 get(const void *a, std::size_t i) {
        return E::unpack(__ldg(reinterpret_cast<const std::uint32_t *>(a) + i));
    }
    static __device__ __forceinline__ void get_pair(const void *a, std::size_t j, float2 &lo, float2 &hi) {
        const uint2 q = __ldg(reinterpret_cast<const uint2 *>(a) + j);
        lo = E::unpack(q.x);
        hi = E::unpack(q.y);
    }
    static __device__ __forceinline__ void put(void *a, std::size_t i, float2 v) {
        reinterpret_cast<std::uint32_t *>(a)[i] = E::pack(v.x, v.y);
    }
};

// Float grid coordinate to uint32 as the reference's astype(jnp.uint32) runs on the GPU: negative
// and NaN give 0, values past the range 2^32 - 1; integral values in range convert exactly.
__device__ __forceinline__ std::uint32_t coord_u32(float v) {
    return v > 0.f ? (v < 4294967296.f ? (std::uint32_t)v : 0xFFFFFFFFu) : 0u;
}

// Table row of grid vertex (x, y, z) at level l, clamped to the table (encoders.py:134-189).
// `tmask` = T - 1 when T is a power of two (then h mod T = h & tmask), else 0.
__device__ __forceinline__ std::uint32_t level_row(const NgpHashGridDescriptor &d, std::uint32_t l, std::uint32_t tmask,
                                                   std::uint32_t x, std::uint32_t y, std::uint32_t z) {
    const std::uint32_t res = d.resolutions[l];
    const std::uint32_t h = l < d.first_hash_level ? (x + y * res + z * (res * res)) : (x ^ (y * 2654435761u) ^ (z * 805459861u));
    const std::uint32_t idx = (tmask != 0u ? (h & tmask) : h % d.T) + d.offsets[l];
    return idx < d.n_params - 1u ? idx : d.n_params - 1u;
}

__device__ __forceinline__ void level_corners(const NgpHashGridDescriptor &d, std::uint32_t l, std::uint32_t tmask,
                                              float px, float py, float pz, Corner8 &c) {
    const float b = d.bound;
    const float two_b = d.two_bound;
    // (pos + bound) / (2 * bound)
    const float ux = __fdiv_rn(__fadd_rn(px, b), two_b);
    const float uy = __fdiv_rn(__fadd_rn(py, b), two_b);
    const float uz = __fdiv_rn(__fadd_rn(pz, b), two_b);
    const float s = d.scales[l];
    const float sx = __fadd_rn(__fmul_rn(ux, s), 0.5f);
    const float sy = __fadd_rn(__fmul_rn(uy, s), 0.5f);
    const float sz = __fadd_rn(__fmul_rn(uz, s), 0.5f);
    const float fx = floorf(sx), fy = floorf(sy), fz = floorf(sz);
    // floor + {0, 1} in float, then converted (both corners of an axis below the grid become 0)
    const std::uint32_t xs[2] = {coord_u32(fx), coord_u32(__fadd_rn(fx, 1.f))};
    const std::uint32_t ys[2] = {coord_u32(fy), coord_u32(__fadd_rn(fy, 1.f))};
    const std::uint32_t zs[2] = {coord_u32(fz), coord_u32(__fadd_rn(fz, 1.f))};
    // modf's fractional part (the sign of the coordinate) and the clip to [0, 1] of
    // encoders.py:204-212: a point below the grid gives all its weight to the lower corner
    const float rx = __fsub_rn(sx, truncf(sx)), ry = __fsub_rn(sy, truncf(sy)), rz = __fsub_rn(sz, truncf(sz));
    const float wx[2] = {fminf(fmaxf(__fsub_rn(1.f, rx), 0.f), 1.f), fminf(fmaxf(rx, 0.f), 1.f)};
    const float wy[2] = {fminf(fmaxf(__fsub_rn(1.f, ry), 0.f), 1.f), fminf(fmaxf(ry, 0.f), 1.f)};
    const float wz[2] = {fminf(fmaxf(__fsub_rn(1.f, rz), 0.f), 1.f), fminf(fmaxf(rz, 0.f), 1.f)};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const std::uint32_t ox = (k >> 2) & 1, oy = (k >> 1) & 1, oz = k & 1;
        c.idx[k] = level_row(d, l, tmask, xs[ox], ys[oy], zs[oz]);
        c.w[k] = __fmul_rn(__fmul_rn(wx[ox], wy[oy]), wz[oz]);
    }
}

// enc[n, l*2 + f] for n < n_points (n_points read from `count` when given).  A CTA of 8 warps takes
// tiles of 32 S points, S = max(1, 8 / L) sub-tiles of 32: with S = 1 warp w computes levels
// w, w + 8, ... of the tile's 32 points (lane = point); with fewer levels than warps (the 4-level
// proposal table: S = 2), warp w computes level w % L of sub-tile w / L, so no warp idles.  The
// tile's rows [32 S][L] leave through shared memory as one contiguous block.
constexpr int kHgTile = 32, kHgWarps = 8, kHgRows = kHgTile * (NGP_MAX_LEVELS + 1);

template <class Tab, class Enc, bool kPaired>
__global__ void __launch_bounds__(kHgWarps * 32) hashgrid_forward_kernel(
    NgpHashGridDescriptor d, std::uint32_t n_points, const std::uint32_t *__restrict__ count,
    const float *__restrict__ pos, const void *__restrict__ latents, void *__restrict__ enc) {
    // rows[p * (L + 1) + l]: the padded row stride puts the lanes of a warp in different banks.
    // It needs 32 S (L + 1) entries: 32 (L + 1) <= kHgRows when S = 1, and 32 S L + 32 S <= 512
    // when S > 1 (then S L <= 8 and S <= 8).
    __shared__ float2 rows[kHgRows];
    std::uint32_t n_active = n_points;
    if (count != nullptr) n_active = min(n_active, *count);
    const std::uint32_t L = d.L, tmask = (d.T & (d.T - 1u)) == 0u ? d.T - 1u : 0u, last = d.n_params - 1u;
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    const std::uint32_t S = L < (std::uint32_t)kHgWarps ? (std::uint32_t)kHgWarps / L : 1u;
    const std::uint32_t sub = S > 1u ? warp / L : 0u;              // this warp's sub-tile
    const std::uint32_t l0 = S > 1u ? warp % L : warp;              // and its first level
    const std::uint32_t l_step = S > 1u ? L : (std::uint32_t)kHgWarps;
    const bool busy = sub < S;                                       // warps past S L idle
    const std::uint32_t tile_pts = kHgTile * S, Lp = L + 1u;
    const std::uint32_t n_tiles = (n_active + tile_pts - 1) / tile_pts;
    for (std::uint32_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        const std::uint32_t p = sub * kHgTile + lane;                // point within the tile
        const std::uint32_t n = tile * tile_pts + p;
        const bool in = busy && n < n_active;
        float px = 0.f, py = 0.f, pz = 0.f;
        if (in) {
            px = pos[(std::size_t)n * 3 + 0];
            py = pos[(std::size_t)n * 3 + 1];
            pz = pos[(std::size_t)n * 3 + 2];
        }
        for (std::uint32_t l = l0; busy && l < L; l += l_step) {
            float2 r = make_float2(0.f, 0.f);
            if (in) {
                Corner8 c;
                level_corners(d, l, tmask, px, py, pz, c);
                float2 v[8];
                if (kPaired) {
                    // Corners k and k + 4 differ only in x.  At a dense level their rows are
                    // consecutive, at a hashed level (x ^ ...) and (x + 1 ^ ...) differ only in bit
                    // 0 when x is even: in both cases, about half the time, they are the two rows
                    // of one aligned pair, fetched by one wide load.
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const std::uint32_t i0 = c.idx[k], i1 = c.idx[k + 4];
                        float2 lo, hi;
                        if ((i0 | 1u) <= last) {
                            Tab::get_pair(latents, i0 >> 1, lo, hi);
                            v[k] = (i0 & 1u) ? hi : lo;
                        } else {
                            v[k] = lo = hi = Tab::get(latents, i0);
                        }
                        v[k + 4] = (i0 ^ i1) == 1u ? ((i1 & 1u) ? hi : lo) : Tab::get(latents, i1);
                    }
                } else {
#pragma unroll
                    for (int k = 0; k < 8; ++k) v[k] = Tab::get(latents, c.idx[k]);
                }
                float a0 = __fmul_rn(v[0].x, c.w[0]), a1 = __fmul_rn(v[0].y, c.w[0]);
#pragma unroll
                for (int k = 1; k < 8; ++k) {
                    a0 = __fadd_rn(a0, __fmul_rn(v[k].x, c.w[k]));
                    a1 = __fadd_rn(a1, __fmul_rn(v[k].y, c.w[k]));
                }
                r = make_float2(a0, a1);
            }
            rows[p * Lp + l] = r;
        }
        __syncthreads();
        const std::uint32_t n_rows = min(tile_pts, n_active - tile * tile_pts);
        const std::size_t dst = (std::size_t)tile * tile_pts * L;
        for (std::uint32_t i = threadIdx.x; i < n_rows * L; i += blockDim.x) Enc::put(enc, dst + i, rows[(i / L) * Lp + i % L]);
        __syncthreads();
    }
}

// dL/dlatents[idx_k] += w_k * dL/denc[n, l]: the transpose of the gather.
//
// A warp takes 32 consecutive points at one level.  Consecutive points of a training batch walk
// along one ray, so at coarse levels runs of lanes share a corner; those runs are summed with a
// segmented warp reduction and their last lane issues the one float2 atomic for the run.  Levels
// where no two neighbouring lanes share a corner issue one atomic per lane.  Points whose incoming
// gradient is zero at that level (samples past a ray's termination) contribute nothing.
constexpr std::uint32_t kNone = 0xFFFFFFFFu;

// dL/dlatents[idx] += (vx, vy) for one corner of the warp's 32 points; `heads` marks the lanes that
// start a run of equal indices.  Runs are summed with a segmented warp scan and added by their last
// lane with one atomic; when every lane is a head each live lane adds its own value.
__device__ __forceinline__ void scatter_corner(float2 *__restrict__ dL_dlat, unsigned lane, std::uint32_t idx,
                                               unsigned heads, float vx, float vy) {
    if (heads == 0xffffffffu) {
        if (idx != kNone) atomicAdd(dL_dlat + idx, make_float2(vx, vy));
        return;
    }
    const int seg_start = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const float tx = __shfl_up_sync(0xffffffffu, vx, o);
        const float ty = __shfl_up_sync(0xffffffffu, vy, o);
        if ((int)lane - o >= seg_start) {
            vx += tx;
            vy += ty;
        }
    }
    const bool tail = lane == 31 || ((heads >> (lane + 1)) & 1u);
    if (tail && idx != kNone) atomicAdd(dL_dlat + idx, make_float2(vx, vy));
}

template <class Enc>
__global__ void __launch_bounds__(256) hashgrid_backward_kernel(
    NgpHashGridDescriptor d, std::uint32_t n_points, const std::uint32_t *__restrict__ count,
    const float *__restrict__ pos, const void *__restrict__ dL_denc, float2 *__restrict__ dL_dlat) {
    std::uint32_t n_active = n_points;
    if (count != nullptr) n_active = min(n_active, *count);
    const std::uint32_t tmask = (d.T & (d.T - 1u)) == 0u ? d.T - 1u : 0u;
    const unsigned lane = lane_id();
    const std::size_t n_groups = (std::size_t)((n_active + 31) / 32) * d.L;   // (32 points, level) per warp
    const std::size_t warp0 = ((std::size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const std::size_t n_warps = ((std::size_t)gridDim.x * blockDim.x) >> 5;
    for (std::size_t wg = warp0; wg < n_groups; wg += n_warps) {
        const std::uint32_t l = (std::uint32_t)(wg % d.L);
        const std::uint32_t n = (std::uint32_t)(wg / d.L) * 32u + lane;
        const bool in = n < n_active;
        float2 g = make_float2(0.f, 0.f);
        Corner8 c;
        if (in) {
            g = Enc::get(dL_denc, (std::size_t)n * d.L + l);
            level_corners(d, l, tmask, pos[(std::size_t)n * 3 + 0], pos[(std::size_t)n * 3 + 1], pos[(std::size_t)n * 3 + 2], c);
        } else {
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                c.idx[k] = kNone;
                c.w[k] = 0.f;
            }
        }
        const bool live = in && (g.x != 0.f || g.y != 0.f);
        if (__ballot_sync(0xffffffffu, live) == 0u) continue;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const std::uint32_t idx = live ? c.idx[k] : kNone;
            const float vx = live ? c.w[k] * g.x : 0.f, vy = live ? c.w[k] * g.y : 0.f;
            const std::uint32_t prev = __shfl_up_sync(0xffffffffu, idx, 1);   // every lane takes part
            const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || idx != prev);
            scatter_corner(dL_dlat, lane, idx, heads, vx, vy);
        }
    }
}

// Total variation of the table (encoders.py:236-254):
//   tv = tv_scale * mean over (level, point) of sum over the six axis neighbours a of the point's
//        corner 0 and the two features of (lat[a] - lat[corner 0])^2,
// the neighbours floor(pos_scaled) + (0,0,1), (0,1,0), (1,0,0), (0,0,-1), (0,-1,0), (-1,0,0)
// converted and indexed like the corners.  A warp takes 32 points at one level; each lane sums its
// squared differences in FP32, the warp sums its lanes and adds the total into a double
// accumulator.  With `dL_dlat`, 2 g (lat[a] - lat[c0]) is added to each neighbour's row and
// subtracted from corner 0's, g = tv_scale / (L n) times *grad_scale when given.
__global__ void __launch_bounds__(256) hashgrid_tv_kernel(NgpHashGridDescriptor d, std::uint32_t n_points,
                                                          const float *__restrict__ pos, const float2 *__restrict__ lat,
                                                          float tv_scale, const float *__restrict__ grad_scale,
                                                          float2 *__restrict__ dL_dlat, double *__restrict__ acc) {
    const std::uint32_t tmask = (d.T & (d.T - 1u)) == 0u ? d.T - 1u : 0u;
    const unsigned lane = lane_id();
    const std::size_t n_groups = (std::size_t)((n_points + 31) / 32) * d.L;
    const std::size_t warp0 = ((std::size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const std::size_t n_warps = ((std::size_t)gridDim.x * blockDim.x) >> 5;
    const float g2 = dL_dlat != nullptr
                         ? 2.f * (float)((double)tv_scale / ((double)d.L * (double)n_points)) *
                               (grad_scale != nullptr ? *grad_scale : 1.f)
                         : 0.f;
    float sum = 0.f;
    for (std::size_t wg = warp0; wg < n_groups; wg += n_warps) {
        const std::uint32_t l = (std::uint32_t)(wg % d.L);
        const std::uint32_t n = (std::uint32_t)(wg / d.L) * 32u + lane;
        if (n >= n_points) continue;
        const float s = d.scales[l];
        float f[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float u = __fdiv_rn(__fadd_rn(pos[(std::size_t)n * 3 + a], d.bound), d.two_bound);
            f[a] = floorf(__fadd_rn(__fmul_rn(u, s), 0.5f));
        }
        const std::uint32_t c0 = level_row(d, l, tmask, coord_u32(f[0]), coord_u32(f[1]), coord_u32(f[2]));
        const float2 v0 = __ldg(lat + c0);
        float sx = 0.f, sy = 0.f;
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            // neighbour j of encoders.py:41-48: axis z, y, x, then the same axes at -1
            const int axis = 2 - (j % 3);
            const float step = j < 3 ? 1.f : -1.f;
            const std::uint32_t x = coord_u32(axis == 0 ? __fadd_rn(f[0], step) : f[0]);
            const std::uint32_t y = coord_u32(axis == 1 ? __fadd_rn(f[1], step) : f[1]);
            const std::uint32_t z = coord_u32(axis == 2 ? __fadd_rn(f[2], step) : f[2]);
            const std::uint32_t r = level_row(d, l, tmask, x, y, z);
            const float2 v = __ldg(lat + r);
            const float dx = v.x - v0.x, dy = v.y - v0.y;
            sum += dx * dx + dy * dy;
            if (dL_dlat != nullptr) {
                atomicAdd(dL_dlat + r, make_float2(g2 * dx, g2 * dy));
                sx += dx;
                sy += dy;
            }
        }
        if (dL_dlat != nullptr) atomicAdd(dL_dlat + c0, make_float2(-g2 * sx, -g2 * sy));
    }
    const float w = warp_sum(sum);
    if (lane == 0 && w != 0.f) atomicAdd(acc, (double)w);
}

// tv = tv_scale * sum / (L n): 0 / 0 for n = 0, as the mean of an empty array.
__global__ void hashgrid_tv_finish_kernel(const double *__restrict__ acc, float tv_scale, std::uint32_t L,
                                          std::uint32_t n_points, float *__restrict__ tv) {
    tv[0] = (float)((double)tv_scale * (acc[0] / ((double)L * (double)n_points)));
}

}  // namespace

int check_hashgrid_descriptor(const NgpHashGridDescriptor &d) {
    NGP_CHECK_ARG(d.F == 2, "hashgrid: only F = 2 features per level is supported");
    NGP_CHECK_ARG(d.L >= 1 && d.L <= NGP_MAX_LEVELS, "hashgrid: L must be in [1, 32]");
    NGP_CHECK_ARG(d.T > 0 && d.n_params > 0 && d.first_hash_level <= d.L, "hashgrid: bad table sizes");
    NGP_CHECK_ARG(d.offsets[d.L] == d.n_params, "hashgrid: offsets[L] must equal n_params");
    NGP_CHECK_ARG(d.bound > 0.f && d.two_bound > 0.f, "hashgrid: bound must be positive");
    return NGP_OK;
}

namespace {

bool valid_dtype(std::uint32_t t) { return t == NGP_DTYPE_F32 || t == NGP_DTYPE_BF16 || t == NGP_DTYPE_F16; }

template <class Tab, bool kPaired>
void forward_for_table(cudaStream_t stream, std::uint32_t enc_type, unsigned grid, const NgpHashGridDescriptor &d,
                       const std::uint32_t *count, const float *pos, const void *latents, void *enc) {
    if (enc_type == NGP_DTYPE_BF16)
        hashgrid_forward_kernel<Tab, PairHalf<Bf16Op>, kPaired><<<grid, kHgWarps * 32, 0, stream>>>(d, d.n_coords, count, pos, latents, enc);
    else if (enc_type == NGP_DTYPE_F16)
        hashgrid_forward_kernel<Tab, PairHalf<F16Op>, kPaired><<<grid, kHgWarps * 32, 0, stream>>>(d, d.n_coords, count, pos, latents, enc);
    else
        hashgrid_forward_kernel<Tab, PairF32, kPaired><<<grid, kHgWarps * 32, 0, stream>>>(d, d.n_coords, count, pos, latents, enc);
}

// Paired loads are used for 16-bit tables (a pair of rows is 8 bytes; measured 12% faster on the
// training step's gather) and need the table's base aligned to a pair of rows.  An FP32 table
// keeps one 8-byte load per corner: its pair loads measured 6% slower (the second row of a pair
// sits in the sector the first load just brought into L1, so pairing saves no L2 traffic there).
template <class Tab>
void forward_for_table(cudaStream_t stream, std::uint32_t enc_type, unsigned grid, const NgpHashGridDescriptor &d,
                       const std::uint32_t *count, const float *pos, const void *latents, void *enc) {
    if (Tab::kPairAlign == 8 && ((std::uintptr_t)latents & (Tab::kPairAlign - 1)) == 0)
        forward_for_table<Tab, true>(stream, enc_type, grid, d, count, pos, latents, enc);
    else
        forward_for_table<Tab, false>(stream, enc_type, grid, d, count, pos, latents, enc);
}

}  // namespace

int launch_hashgrid_forward_mixed(cudaStream_t stream, const NgpHashGridDescriptor &d, std::uint32_t table_type,
                                  std::uint32_t enc_type, const std::uint32_t *count, const float *pos,
                                  const void *latents, void *enc) {
    int st = check_hashgrid_descriptor(d);
    if (st != NGP_OK) return st;
    NGP_CHECK_ARG(valid_dtype(table_type) && valid_dtype(enc_type), "hashgrid: unknown table or encoding type");
    const std::uintptr_t a = table_type == NGP_DTYPE_F32 ? 7u : 3u, b = enc_type == NGP_DTYPE_F32 ? 7u : 3u;
    NGP_CHECK_ARG(((std::uintptr_t)latents & a) == 0 && ((std::uintptr_t)enc & b) == 0,
                  "hashgrid: latents and encodings must be aligned to one row of two features");
    const std::size_t tile_pts = (std::size_t)kHgTile * (d.L < (std::uint32_t)kHgWarps ? kHgWarps / d.L : 1u);
    const std::size_t tiles = ((std::size_t)d.n_coords + tile_pts - 1) / tile_pts;
    if (tiles > 0) {
        const unsigned grid = grid_for(tiles, 1, 8);
        if (table_type == NGP_DTYPE_BF16)
            forward_for_table<PairHalf<Bf16Op>>(stream, enc_type, grid, d, count, pos, latents, enc);
        else if (table_type == NGP_DTYPE_F16)
            forward_for_table<PairHalf<F16Op>>(stream, enc_type, grid, d, count, pos, latents, enc);
        else
            forward_for_table<PairF32>(stream, enc_type, grid, d, count, pos, latents, enc);
        count_launches(1);
    }
    return launch_status();
}

int launch_hashgrid_forward(cudaStream_t stream, const NgpHashGridDescriptor &d,
                            const std::uint32_t *count, const float *pos, const float *latents,
                            float *enc) {
    return launch_hashgrid_forward_mixed(stream, d, NGP_DTYPE_F32, NGP_DTYPE_F32, count, pos, latents, enc);
}

int launch_hashgrid_backward_mixed(cudaStream_t stream, const NgpHashGridDescriptor &d, std::uint32_t enc_type,
                                   const std::uint32_t *count, const float *pos, const void *dL_denc,
                                   float *dL_dlatents, bool accumulate) {
    int st = check_hashgrid_descriptor(d);
    if (st != NGP_OK) return st;
    NGP_CHECK_ARG(valid_dtype(enc_type), "hashgrid: unknown encoding type");
    const std::uintptr_t b = enc_type == NGP_DTYPE_F32 ? 7u : 3u;
    NGP_CHECK_ARG(((std::uintptr_t)dL_denc & b) == 0 && ((std::uintptr_t)dL_dlatents & 7u) == 0,
                  "hashgrid: gradients must be aligned to one row of two features");
    if (!accumulate) NGP_CUDA_TRY(cudaMemsetAsync(dL_dlatents, 0, (std::size_t)d.n_params * 2 * sizeof(float), stream));
    const std::size_t items = (std::size_t)((d.n_coords + 31) / 32) * 32 * d.L;
    if (items > 0) {
        const unsigned grid = grid_for(items, 256, 8);
        float2 *out = reinterpret_cast<float2 *>(dL_dlatents);
        if (enc_type == NGP_DTYPE_BF16)
            hashgrid_backward_kernel<PairHalf<Bf16Op>><<<grid, 256, 0, stream>>>(d, d.n_coords, count, pos, dL_denc, out);
        else if (enc_type == NGP_DTYPE_F16)
            hashgrid_backward_kernel<PairHalf<F16Op>><<<grid, 256, 0, stream>>>(d, d.n_coords, count, pos, dL_denc, out);
        else
            hashgrid_backward_kernel<PairF32><<<grid, 256, 0, stream>>>(d, d.n_coords, count, pos, dL_denc, out);
        count_launches(1);
    }
    return launch_status();
}

// tv[0] <- the TV term of `latents` at d.n_coords points (0 when tv_scale <= 0); with dL_dlatents,
// its gradient (times *grad_scale when given) is added there.  `acc` is one double of scratch.
int launch_hashgrid_tv(cudaStream_t stream, const NgpHashGridDescriptor &d, float tv_scale, const float *pos,
                       const float *latents, const float *grad_scale, float *tv, float *dL_dlatents, double *acc) {
    int st = check_hashgrid_descriptor(d);
    if (st != NGP_OK) return st;
    NGP_CHECK_ARG(tv != nullptr && acc != nullptr, "hashgrid tv: tv and scratch buffers are required");
    NGP_CHECK_ARG(((std::uintptr_t)acc & 7u) == 0, "hashgrid tv: the scratch double must be 8-byte aligned");
    NGP_CHECK_ARG(((std::uintptr_t)latents & 7u) == 0 && ((std::uintptr_t)dL_dlatents & 7u) == 0,
                  "hashgrid tv: latents and gradients must be aligned to one row of two features");
    if (!(tv_scale > 0.f)) {   // encoders.py:253-254: no term, no gradient
        NGP_CUDA_TRY(cudaMemsetAsync(tv, 0, sizeof(float), stream));
        return launch_status();
    }
    NGP_CUDA_TRY(cudaMemsetAsync(acc, 0, sizeof(double), stream));
    const std::size_t items = (std::size_t)((d.n_coords + 31) / 32) * 32 * d.L;
    if (items > 0) {
        hashgrid_tv_kernel<<<grid_for(items, 256, 8), 256, 0, stream>>>(d, d.n_coords, pos,
                                                                      reinterpret_cast<const float2 *>(latents), tv_scale,
                                                                      grad_scale, reinterpret_cast<float2 *>(dL_dlatents), acc);
        count_launches(1);
    }
    hashgrid_tv_finish_kernel<<<1, 1, 0, stream>>>(acc, tv_scale, d.L, d.n_coords, tv);
    count_launches(1);
    return launch_status();
}

int launch_hashgrid_backward(cudaStream_t stream, const NgpHashGridDescriptor &d,
                             const std::uint32_t *count, const float *pos, const float *dL_denc,
                             float *dL_dlatents, bool accumulate) {
    return launch_hashgrid_backward_mixed(stream, d, NGP_DTYPE_F32, count, pos, dL_denc, dL_dlatents, accumulate);
}

}  // namespace ngp
