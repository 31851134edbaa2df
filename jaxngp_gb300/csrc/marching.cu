// Occupancy-grid ray marcher and Morton codes for sm_103a.
//
// Replaces volume-rendering-jax/lib/impl/marching.cu (march_rays :101-268, march_rays_inference
// :271-397, morton3d :399-414, morton3d_invert :416-433) behind the same custom-call ABI.
//
// This translation unit is compiled with --fmad=false: every float operation of the march is
// rounded on its own, in the reference's order, so per-ray sample counts and sample positions are
// bit-identical to the reference's arithmetic evaluated one rounding per operation (and to the
// CPU oracle).
//
// GB300 specifics: slot allocation is one atomic per warp (warp prefix sum of the per-ray sample
// counts) instead of one per ray; the sample-buffer tail that no ray wrote is zeroed by a second
// grid-stride kernel that reads the final counters, instead of ten full-buffer memsets up front;
// the refill of finished slots in the inference marcher is warp-aggregated too, and the inference
// launcher never blocks the host (the reference synchronises the stream at marching.cu:562).
#include <cstring>

#include <atomic>

#include "common.cuh"
#include "coarse.cuh"

namespace ngp {
namespace {

struct V3 {
    float x, y, z;
};

__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return min(max(v, lo), hi); }

// marching.cu:15-23.  The clamp bounds do not depend on t: MarchParams holds them, computed once
// with the same float operations (so every ds is bit-identical to evaluating them per call).
__device__ __forceinline__ float calc_ds_bounds(float t, float sp, float ds_lo, float ds_hi) {
    return clampf(t * sp, ds_lo, ds_hi);
}

// marching.cu:25-39
__device__ __forceinline__ std::uint32_t mip_from_xyz(V3 p, std::uint32_t K) {
    if (K == 1) return 0;
    int e;
    frexpf(fmaxf(fabsf(p.x), fmaxf(fabsf(p.y), fabsf(p.z))), &e);
    return (std::uint32_t)clampi(e, 0, (int)K - 1);
}
__device__ __forceinline__ std::uint32_t mip_from_ds(float ds, std::uint32_t G, std::uint32_t K) {
    if (K == 1) return 0;
    int e;
    frexpf(ds * (float)G, &e);
    return (std::uint32_t)clampi(e, 0, (int)K - 1);
}

// marching.cu:52-77
__device__ __forceinline__ std::uint32_t expand_bits(std::uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}
__device__ __forceinline__ std::uint32_t morton3(std::uint32_t x, std::uint32_t y, std::uint32_t z) {
    return expand_bits(x) | (expand_bits(y) << 1) | (expand_bits(z) << 2);
}
__device__ __forceinline__ std::uint32_t morton3_invert(std::uint32_t x) {
    x = x & 0x49249249u;
    x = (x | (x >> 2)) & 0xc30c30c3u;
    x = (x | (x >> 4)) & 0x0f00f00fu;
    x = (x | (x >> 8)) & 0xff0000ffu;
    x = (x | (x >> 16)) & 0x0000ffffu;
    return x;
}

struct MarchParams {
    std::uint32_t dns, K, G;
    float bound, sp, inv_G;
    float ds_lo, ds_hi;   // calc_ds clamp bounds: 2 sqrt3 min(bound,1) / dns and 2 sqrt3 bound / G
    // stepsize_portion == 0 (bound <= 1): clamp(t * 0, lo, hi) is min(lo, hi) for every t (a NaN
    // product is dropped by fmaxf), so the step is one constant
    bool const_ds;
    float ds_const;
    // K == 1: every sample is in cascade 0, whose half-width min(2^0, bound) and its reciprocal
    // are fixed per launch
    float mb0, inv_mb0;
    bool pow2_0;
};

__device__ __forceinline__ float calc_ds(float t, const MarchParams &m) {
    return m.const_ds ? m.ds_const : calc_ds_bounds(t, m.sp, m.ds_lo, m.ds_hi);
}

// x / mb where mb = min(2^cascade, bound).  When mb is a power of two the quotient is the product
// with its exact reciprocal, bit for bit (both are the exact value rounded once); otherwise divide.
__device__ __forceinline__ float div_mb(float x, float mb, float inv_mb, bool pow2) { return pow2 ? x * inv_mb : x / mb; }

// Loop caps.  A ray whose t_end is infinite (or so large that t + ds rounds back to t) would
// march forever; valid rays stay far below these caps (samples <= diagonal_n_steps * bound, empty
// voxels crossed <= 3 * G * K, steps inside one empty voxel <= bound * diag / (G * sqrt3)).
constexpr std::uint32_t kMaxMarchIters = 1u << 22;
constexpr std::uint32_t kMaxSkipIters = 1u << 20;

// marching.cu:79-98, :41-50, :174-176: is the cell under `pos` occupied?  Also returns the
// continuous grid position and the cascade's half-width for the empty-space skip.
// `expand` (optional) holds expand_bits(v) for v < G.
__device__ __forceinline__ bool occupied_at(const MarchParams &m, V3 pos, float ds,
                                            const std::uint8_t *__restrict__ bits, V3 &g, float &mb,
                                            const std::uint32_t *expand = nullptr) {
    std::uint32_t cascade = 0;
    bool pow2;
    float inv_mb;
    if (m.K == 1) {
        mb = m.mb0;
        pow2 = m.pow2_0;
        inv_mb = m.inv_mb0;
    } else {
        std::uint32_t c0 = mip_from_xyz(pos, m.K), c1 = mip_from_ds(ds, m.G, m.K);
        cascade = c0 > c1 ? c0 : c1;
        mb = fminf(scalbnf(1.0f, (int)cascade), m.bound);
        pow2 = (__float_as_uint(mb) & 0x007FFFFFu) == 0u && mb >= 1.17549435e-38f;
        inv_mb = pow2 ? __uint_as_float(0x7F000000u - __float_as_uint(mb)) : 0.f;  // 2^-e for mb = 2^e
    }
    float Gf = (float)m.G;
    g.x = ((div_mb(pos.x, mb, inv_mb, pow2) + 1.0f) * 0.5f) * Gf;
    g.y = ((div_mb(pos.y, mb, inv_mb, pow2) + 1.0f) * 0.5f) * Gf;
    g.z = ((div_mb(pos.z, mb, inv_mb, pow2) + 1.0f) * 0.5f) * Gf;
    int Gi = (int)m.G - 1;
    std::uint32_t gx = (std::uint32_t)clampi((int)floorf(g.x), 0, Gi);
    std::uint32_t gy = (std::uint32_t)clampi((int)floorf(g.y), 0, Gi);
    std::uint32_t gz = (std::uint32_t)clampi((int)floorf(g.z), 0, Gi);
    const std::uint32_t code = expand != nullptr ? (expand[gx] | (expand[gy] << 1) | (expand[gz] << 2)) : morton3(gx, gy, gz);
    std::uint32_t idx = cascade * (m.G * m.G * m.G) + code;
    return (__ldg(bits + (idx >> 3)) >> (idx & 7u)) & 1u;
}

// K == 1: the clamped integer cell of a position, packed (10 bits per axis), as occupied_at finds
// it -- the same operations in the same order -- so two positions with equal keys read the same
// occupancy bit.
__device__ __forceinline__ std::uint32_t cell_key(const MarchParams &m, V3 g) {
    const int Gi = (int)m.G - 1;
    return (std::uint32_t)clampi((int)floorf(g.x), 0, Gi) | ((std::uint32_t)clampi((int)floorf(g.y), 0, Gi) << 10) |
           ((std::uint32_t)clampi((int)floorf(g.z), 0, Gi) << 20);
}
__device__ __forceinline__ std::uint32_t cell_key_at(const MarchParams &m, V3 pos) {
    const float Gf = (float)m.G;
    const V3 g{((div_mb(pos.x, m.mb0, m.inv_mb0, m.pow2_0) + 1.0f) * 0.5f) * Gf,
               ((div_mb(pos.y, m.mb0, m.inv_mb0, m.pow2_0) + 1.0f) * 0.5f) * Gf,
               ((div_mb(pos.z, m.mb0, m.inv_mb0, m.pow2_0) + 1.0f) * 0.5f) * Gf};
    return cell_key(m, g);
}

// The march's constant step c from t > 0 in closed form: while every exact sum t + k c stays
// below t's next power of two `top` and c / ulp(t) is not an exact round-to-even tie, each rounded
// addition adds the same delta = fl(t + c) - t (a multiple of the ulp), so t after k additions is
// t + k delta, every operation exact.  Returns false where that cannot be shown for t and c
// (non-normal t; a tie); callers also keep their sums below `top` with a margin.
__device__ __forceinline__ bool chain_step(float t, float c, float &delta, float &top) {
    if (!(t > 0.f)) return false;
    const std::uint32_t e = __float_as_uint(t) & 0x7F800000u;
    if (e <= (24u << 23) || e >= (253u << 23)) return false;
    const float u = __uint_as_float(e - (23u << 23));    // ulp of t (a power of two)
    const float x = __fdiv_rn(c, u);                      // exact: u is a power of two
    if (x - floorf(x) == 0.5f) return false;
    top = __uint_as_float(e + (1u << 23));               // the next power of two
    delta = (t + c) - t;                                 // round(c / u) u, exact
    return true;
}

// marching.cu:182-189: advance past the empty voxel in whole steps.
__device__ __forceinline__ float skip_empty(const MarchParams &m, float t, V3 g, float mb, V3 pos,
                                            V3 d, V3 inv_d) {
    float nt = t + calc_ds(t, m);
    float nx = floorf((g.x + 0.5f) + 0.5f * copysignf(1.0f, d.x));
    float ny = floorf((g.y + 0.5f) + 0.5f * copysignf(1.0f, d.y));
    float nz = floorf((g.z + 0.5f) + 0.5f * copysignf(1.0f, d.z));
    float dx = (((nx * m.inv_G - 0.5f) * 2.0f) * mb - pos.x) * inv_d.x;
    float dy = (((ny * m.inv_G - 0.5f) * 2.0f) * mb - pos.y) * inv_d.y;
    float dz = (((nz * m.inv_G - 0.5f) * 2.0f) * mb - pos.z) * inv_d.z;
    float next_t = t + fmaxf(0.0f, fminf(dx, fminf(dy, dz)));
    if (m.const_ds) {
        // (a closed form of these additions, as chain_t has, measured 11% slower here: a skip
        // averages a few additions, fewer instructions than the form's guard and division)
        const float c = m.ds_const;
        for (std::uint32_t it = 0; nt < next_t && it < kMaxSkipIters; ++it) nt += c;
    } else {
        for (std::uint32_t it = 0; nt < next_t && it < kMaxSkipIters; ++it) nt += calc_ds(nt, m);
    }
    return nt;
}

__device__ __forceinline__ V3 at(V3 o, V3 d, float t) { return {o.x + t * d.x, o.y + t * d.y, o.z + t * d.z}; }

// Skipping an empty coarse block in one step (K = 1, constant step, G a multiple of 8, with the
// coarse grid of coarse.cuh: a block is marked when a cell of it, grown by one cell, is occupied).
//
// Inside an unmarked block every cell the march can look up is empty, even with its positions
// rounded (the one-cell growth), so the reference (marching.cu:174-190) goes from landing to
// landing -- each the first step of the chain t <- t + c at or past the exit of the landing's cell
// -- until it lands past the block.  Its last landing inside lies in the cell through which the
// ray leaves the block, whose exit plane is the block's face, so its next landing is the first
// chain point at or past `next_t` computed from that landing with the block's face plane.  Here
// the same formula is evaluated from the current point instead; the two values of next_t differ
// only by rounding, bounded by eps (the roundings of pos = o + t d, of plane - pos, 1/d, the
// product and the sum, for either point, with a factor of 4 to spare).  When no chain point lies
// within eps of the block's exit every landing the reference could make there is the same chain
// point, the one returned; otherwise (and when the chain would cross a power of two, where its
// step changes) this returns false and the march takes the cell-by-cell path.
__device__ __forceinline__ bool skip_block(const MarchParams &m, float t, V3 g, V3 pos, V3 o, V3 d, V3 inv_d,
                                           const std::uint8_t *__restrict__ coarse, float &t_land) {
    const int Gi = (int)m.G - 1, Gc = (int)(m.G >> 3);
    const int bx = clampi((int)floorf(g.x), 0, Gi) >> 3, by = clampi((int)floorf(g.y), 0, Gi) >> 3,
              bz = clampi((int)floorf(g.z), 0, Gi) >> 3;
    if (coarse[bx + by * Gc + bz * Gc * Gc] != 0) return false;
    if (d.x == 0.f || d.y == 0.f || d.z == 0.f) return false;
    const float u = 5.9604645e-8f;   // 2^-24
    const int b3[3] = {bx, by, bz};
    const float p3[3] = {pos.x, pos.y, pos.z}, o3[3] = {o.x, o.y, o.z}, d3[3] = {d.x, d.y, d.z},
                id3[3] = {inv_d.x, inv_d.y, inv_d.z};
    float dmin = __int_as_float(0x7f800000), err = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int nb = d3[a] > 0.f ? (b3[a] + 1) * 8 : b3[a] * 8;
        const float plane = (((float)nb * m.inv_G - 0.5f) * 2.0f) * m.mb0;
        const float dist = (plane - p3[a]) * id3[a];
        // rounding bound of t + dist from any point of the block's last cell on this ray (|t| <= t + dist)
        const float e = u * (fabsf(id3[a]) * (fabsf(o3[a]) + 2.0f * fabsf((t + fabsf(dist)) * d3[a]) + fabsf(plane)) +
                             4.0f * fabsf(dist) + 2.0f * (fabsf(t) + fabsf(dist)));
        dmin = fminf(dmin, dist);
        err = fmaxf(err, e);   // every axis: covers the axis that decides the minimum, ties included
    }
    if (!(err < 1e30f)) return false;
    const float eps = 4.0f * err;
    const float tx = t + fmaxf(0.0f, dmin);
    float delta, top;
    if (!chain_step(t, m.ds_const, delta, top)) return false;
    // the first chain point at or past tx + eps: j steps of delta from t (exact below `top`)
    float jf = ceilf((tx + eps - t) / delta);
    if (!(jf >= 2.0f && jf < 1.0e6f)) return false;
    for (int k = 0; k < 4 && t + (jf - 1.0f) * delta >= tx + eps; ++k) jf -= 1.0f;
    for (int k = 0; k < 4 && t + jf * delta < tx + eps; ++k) jf += 1.0f;
    const float tl = t + jf * delta, tp = t + (jf - 1.0f) * delta;
    if (!(tl >= tx + eps) || !(tp < tx - eps) || !(tl < top) || jf < 2.0f) return false;
    t_land = tl;
    return true;
}

// ------------------------------------------------------------------------------- march_rays

// True when the ray cannot take a sample: every cell the march could look up on [t0, t1) lies in
// a coarse block (8^3 cells grown by one cell) that holds no occupied cell.  The march looks up
// the cell under o + t d for t on [t0, t1) (rounded positions, clamped into the grid); the coarse
// DDA walks the blocks the same segment crosses, and the one-cell growth of every block covers
// both roundings.  Positions clamped from outside the grid are covered only within half a cell of
// its faces, so rays whose ends lie farther out are marched in full.  K = 1 only.
__device__ __forceinline__ bool no_sample_possible(const MarchParams &m, const V3 &o, const V3 &d, float t0, float t1,
                                                   const std::uint8_t *__restrict__ coarse) {
    if (m.K != 1 || (m.G & 7u) != 0u) return false;
    const float lim = m.mb0 + 0.5f * (2.0f * m.mb0 / (float)m.G);
    const V3 a = at(o, d, t0), b = at(o, d, t1);
    if (fabsf(a.x) > lim || fabsf(a.y) > lim || fabsf(a.z) > lim || fabsf(b.x) > lim || fabsf(b.y) > lim ||
        fabsf(b.z) > lim)
        return false;
    float ta, tb;
    return !coarse_ray_interval(o.x, o.y, o.z, d.x, d.y, d.z, t0, t1, coarse, (int)(m.G / 8u), m.mb0, ta, tb);
}

constexpr int kMarchBlock = 128;
constexpr int kMarchBlocksPerSm = 10;   // 40 warps per SM at <= 48 registers
std::atomic<int> g_march_blocks_per_sm{kMarchBlocksPerSm};

enum : int { kIdle = 0, kCount = 1, kWrite = 2 };

enum : int { kMarchAlloc = 0, kMarchCount = 1 };

// The march, one thread per ray (the reference's structure, marching.cu:101-268), with the
// arithmetic of occupied_at/skip_empty, same-cell loops (below) and, with a coarse grid, one-step
// skips of empty coarse blocks (skip_block).  Rays are visited in index order by a block-uniform
// grid-stride loop.  (A lane-refill design -- a lane that finishes its ray takes the next one
// from a queue -- measured 1.5x slower on the same work: the march is issue-bound at about 7 of
// 32 active threads per instruction either way, and the refill adds instructions without making
// the lanes more coherent; ordering the rays by camera and direction did not help either.)
//
// Per ray the arithmetic and the two passes (count, then write) are the reference's
// (marching.cu:162-192, :224-267).  A ray with no sample is valid (marching.cu:196-199); a ray
// that does not fit the budget is not (:206-209).  Two modes:
//
// kMarchAlloc (the drop-in march_rays): after counting, the rays of a warp take their slots with
// one atomic (a warp prefix sum of their counts), so which rays fit an overflowing budget follows
// the order in which warps finish counting, as in the reference, and the write pass resumes at
// the t of the ray's first occupied sample (the march state is t alone).  As in the reference
// (:135), a ray whose thread starts after the buffer filled is dropped (invalid) unmarched.
//
// kMarchCount: the count pass of the training march (launch_march_rays with `ordered`) for the
// rays after its leading ones; see below.
//
// The training march gives the reference kernel's result under one schedule: its threads run one
// at a time, in ray order.  Then ray r starts with the counter at P(r), the sum of the counts of
// the rays before it; it is dropped unmarched if P(r) >= budget (marching.cu:135), else it is
// valid with no samples, or fits (P(r) + n(r) <= budget), or is the one ray that does not fit
// (:206-209), after which every ray is dropped.  The rays that fit are a prefix of the batch's
// rays with samples, and the valid rays a prefix of the batch (its pixel indices are drawn at
// random, so an unbiased sample), and the result is deterministic.  The passes:
//
//  - the leading rays (march_lead_kernel, a warp per ray): counted in full, their counts summed
//    per chunk of kThreadBlock rays;
//  - the other rays (march_rays_kernel<kMarchCount>, a thread per ray), in chunks: each chunk
//    publishes the sum of its counts when done, and a frontier word holds (F, P): chunks [0, F)
//    are done and their counts sum to P.  A ray of chunk c >= F that reads P >= budget stops (or
//    never starts): it is dropped.  Its published count is then a lower bound of its count; see
//    ray_scan_fit_kernel for why the result stays exact;
//  - ray_scan_fit_kernel: the prefix sums P(r), the fit, the counters;
//  - march_write_kernel (a warp per ray): the samples of the rays that fit.
//
// Resident rays share the SMs round-robin, so the leading chunks of one launch over the whole
// batch finish only about when all of its first wave does, too late for the frontier to spare
// anything; hence the leading rays' launch of their own, where each ray runs at the speed of its
// chain of steps, shortened 32-fold by the warp's lookahead.  How many rays lead comes from the
// previous call: the index of its first dropped ray, which the call leaves in its `queue` word;
// this call leads with 1.25 times that many rays and 512 more (8192 on a first call, whose word
// is 0), at most kLeadMax.  A lead that falls short costs time, not exactness.  Once the leading
// rays fill the budget, a chunk of the others only records that its rays have no count.
constexpr int kThreadBlock = 256;
constexpr std::uint32_t kFrontierCheck = 32;   // a counting ray reads the frontier every this many steps
constexpr std::uint32_t kLeadMax = 16384;      // leading rays at most (a multiple of kThreadBlock)
static_assert(kLeadMax % kThreadBlock == 0, "the leading rays are whole chunks");

// The chunks of kThreadBlock rays the leading launch takes, given the previous call's word.
__device__ __forceinline__ std::uint32_t lead_chunks(std::uint32_t word, std::uint32_t n_rays) {
    std::uint64_t w = word == 0u ? 8192ull : (std::uint64_t)word + word / 4u + 512u;
    if (w > kLeadMax) w = kLeadMax;
    if (w > n_rays) w = n_rays;
    return (std::uint32_t)((w + kThreadBlock - 1) / kThreadBlock);
}

// The frontier word: F in the high half, P (saturated at 2^32 - 1, which no budget exceeds) in
// the low half.
__device__ __forceinline__ unsigned long long frontier_pack(std::uint32_t F, std::uint64_t P) {
    return ((unsigned long long)F << 32) | (P > 0xffffffffull ? 0xffffffffull : P);
}
__device__ __forceinline__ std::uint32_t frontier_sum(const unsigned long long *frontier) {
    return (std::uint32_t)*((const volatile unsigned long long *)frontier);
}

// The frontier's sum as a relaxed load that nothing waits for until its value is used (the march
// loop uses it one poll later, so the load's latency stays off the ray's chain of steps).
__device__ __forceinline__ std::uint32_t frontier_sum_async(const unsigned long long *frontier) {
    std::uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(frontier));   // P: the low half
    return v;
}

// Publishes chunk c's count sum and moves the frontier over the chunks done (one thread).  The
// attempts are bounded; a frontier left behind is moved on by the next chunk that finishes, and
// only ever lowers what the rays can skip.
__device__ __forceinline__ void publish_chunk(std::uint32_t c, std::uint32_t sum, std::uint32_t n_chunks,
                                              std::uint32_t total_samples,
                                              std::uint32_t *chunk_sums, std::uint32_t *chunk_done,
                                              unsigned long long *frontier) {
    *((volatile std::uint32_t *)(chunk_sums + c)) = sum;
    __threadfence();
    *((volatile std::uint32_t *)(chunk_done + c)) = 1u;
    __threadfence();
    if (frontier_sum(frontier) >= total_samples) return;   // full already: nothing more to skip
    for (int k = 0; k < 256; ++k) {
        const unsigned long long w = *((volatile unsigned long long *)frontier);
        const std::uint32_t F = (std::uint32_t)(w >> 32), P = (std::uint32_t)w;
        if (F >= n_chunks || *((volatile std::uint32_t *)(chunk_done + F)) == 0u) break;
        __threadfence();
        const std::uint32_t v = *((volatile std::uint32_t *)(chunk_sums + F));
        atomicCAS(frontier, w, frontier_pack(F + 1u, (std::uint64_t)P + v));   // on failure: look again
    }
}

// The write pass of one ray (marching.cu:224-267), one thread: its n samples from slot `start`,
// marching from t, the t of its first occupied sample (the march state is t alone).
__device__ __forceinline__ void write_ray_thread(const MarchParams &m, std::uint32_t r, std::uint32_t start,
                                                 std::uint32_t n, float t, float t1, V3 o, V3 d, V3 inv_d,
                                                 const std::uint8_t *__restrict__ bits, const std::uint32_t *expand,
                                                 const std::uint8_t *__restrict__ coarse, bool block_skip,
                                                 std::uint32_t *__restrict__ idcs, float *__restrict__ xyzs,
                                                 float *__restrict__ dirs, float *__restrict__ dss,
                                                 float *__restrict__ z_vals) {
    std::uint32_t k = 0, it = 0;
    auto put = [&](V3 p, float dsj, float tj) {
        const std::uint32_t s = start + k;
        idcs[s] = r;
        xyzs[(std::size_t)s * 3 + 0] = p.x;
        xyzs[(std::size_t)s * 3 + 1] = p.y;
        xyzs[(std::size_t)s * 3 + 2] = p.z;
        dirs[(std::size_t)s * 3 + 0] = d.x;
        dirs[(std::size_t)s * 3 + 1] = d.y;
        dirs[(std::size_t)s * 3 + 2] = d.z;
        dss[s] = dsj;
        z_vals[s] = tj;
        ++k;
    };
    while (k < n && t < t1 && it < kMaxMarchIters) {
        const V3 pos = at(o, d, t);
        const float ds = calc_ds(t, m);
        V3 g;
        float mb;
        if (occupied_at(m, pos, ds, bits, g, mb, expand)) {
            put(pos, ds, t);
            t = t + ds;
            if (m.K == 1) {
                const std::uint32_t key = cell_key(m, g);
                while (k < n && t < t1 && it < kMaxMarchIters) {
                    const V3 p2 = at(o, d, t);
                    if (cell_key_at(m, p2) != key) break;
                    const float ds2 = calc_ds(t, m);
                    put(p2, ds2, t);
                    t = t + ds2;
                    ++it;
                }
            }
        } else {
            float tb;
            if (block_skip && skip_block(m, t, g, pos, o, d, inv_d, coarse, tb))
                t = tb;
            else
                t = skip_empty(m, t, g, mb, pos, d, inv_d);
        }
        ++it;
    }
}

// One ray of march_rays_kernel (every lane of the warp calls it together; r >= n_rays idles).
// Returns the ray's count (as far as it was counted) in kMarchCount mode, else 0.
template <int kMode>
__device__ __forceinline__ std::uint32_t march_one(
    std::uint32_t r, std::uint32_t n_rays, std::uint32_t total_samples, const MarchParams &m, float n_cap, bool block_skip,
    const float *__restrict__ rays_o, const float *__restrict__ rays_d,
    const float *__restrict__ t_starts, const float *__restrict__ t_ends,
    const float *__restrict__ noises, const std::uint8_t *__restrict__ bits,
    std::uint32_t *__restrict__ next_loc, std::uint32_t *__restrict__ n_exceeded, bool *__restrict__ ray_is_valid,
    std::uint32_t *__restrict__ rays_n_samples, std::uint32_t *__restrict__ rays_startidx,
    std::uint32_t *__restrict__ idcs, float *__restrict__ xyzs, float *__restrict__ dirs,
    float *__restrict__ dss, float *__restrict__ z_vals, const std::uint8_t *__restrict__ coarse,
    const std::uint32_t *expand, const unsigned long long *frontier) {
    bool march = false;
    std::uint32_t n = 0, start = 0, it = 0;
    V3 o{0.f, 0.f, 0.f}, d{1.f, 1.f, 1.f}, inv_d{1.f, 1.f, 1.f};
    float t = 0.f, t1 = 0.f, t_hit = 0.f;
    if (r < n_rays) {
        if (kMode == kMarchAlloc && *((volatile std::uint32_t *)next_loc) >= total_samples) {
            ray_is_valid[r] = false;   // marching.cu:135
            rays_n_samples[r] = 0;
            rays_startidx[r] = 0;
        } else {
            o = {rays_o[r * 3 + 0], rays_o[r * 3 + 1], rays_o[r * 3 + 2]};
            d = {rays_d[r * 3 + 0], rays_d[r * 3 + 1], rays_d[r * 3 + 2]};
            const float t0 = t_starts[r];
            t1 = t_ends[r];
            if (t1 > t0 && !(coarse != nullptr && no_sample_possible(m, o, d, t0, t1, coarse))) {
                march = true;
                inv_d = {1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
                t = t0 + calc_ds(t0, m) * noises[r];
            } else {
                ray_is_valid[r] = t1 > t0;
                rays_n_samples[r] = 0;
                rays_startidx[r] = 0;
            }
        }
    }
    // ---- count pass (marching.cu:162-192)
    if (march) {
        std::uint32_t poll = 0, fsum = 0;
        while ((float)n < n_cap && t < t1 && it < kMaxMarchIters) {
            if (kMode == kMarchCount && it >= poll) {   // did the rays before this one fill the budget?
                if (fsum >= total_samples) break;       // (as of the previous poll)
                fsum = frontier_sum_async(frontier);
                poll = it + kFrontierCheck;
            }
            const V3 pos = at(o, d, t);
            const float ds = calc_ds(t, m);
            V3 g;
            float mb;
            if (occupied_at(m, pos, ds, bits, g, mb, expand)) {
                if (n == 0) t_hit = t;
                ++n;
                t = t + ds;
                if (m.K == 1) {
                    const std::uint32_t key = cell_key(m, g);
                    while ((float)n < n_cap && t < t1 && it < kMaxMarchIters) {
                        if (cell_key_at(m, at(o, d, t)) != key) break;
                        ++n;
                        t = t + calc_ds(t, m);
                        ++it;
                    }
                }
            } else {
                float tb;
                if (block_skip && skip_block(m, t, g, pos, o, d, inv_d, coarse, tb))
                    t = tb;
                else
                    t = skip_empty(m, t, g, mb, pos, d, inv_d);
            }
            ++it;
        }
    }
    if (kMode == kMarchCount) {
        if (march) {
            ray_is_valid[r] = true;   // ray_scan_fit_kernel decides
            rays_n_samples[r] = n;
            rays_startidx[r] = __float_as_uint(t_hit);   // for the write pass (ray_scan_fit_kernel)
        }
        return march ? n : 0u;   // no warp collective follows in this mode
    }
    // kMarchAlloc: one atomic per warp (warp prefix sum of the counts)
    const bool want = march && n > 0u;
    if (march && n == 0u) {
        ray_is_valid[r] = true;
        rays_n_samples[r] = 0;
        rays_startidx[r] = 0;
    }
    const unsigned wm = __ballot_sync(0xffffffffu, want);
    const std::uint32_t incl = warp_inclusive_scan(want ? n : 0u);
    const std::uint32_t total_w = __shfl_sync(0xffffffffu, incl, 31);
    std::uint32_t base = 0;
    if (wm != 0u) {
        const int leader = __ffs(wm) - 1;
        if ((int)lane_id() == leader) base = atomicAdd(next_loc, total_w);
        base = __shfl_sync(0xffffffffu, base, leader);
    }
    bool fits = false;
    if (want) {
        start = base + incl - n;
        fits = (std::uint64_t)start + n <= total_samples;
        ray_is_valid[r] = fits;
        rays_n_samples[r] = fits ? n : 0u;
        rays_startidx[r] = fits ? start : 0u;
    }
    const std::uint32_t over = warp_sum((want && !fits) ? n : 0u);
    if (lane_id() == 0 && over > 0u) atomicAdd(n_exceeded, over);
    // ---- write pass (marching.cu:224-267), from the first occupied sample
    if (want && fits)
        write_ray_thread(m, r, start, n, t_hit, t1, o, d, inv_d, bits, expand, coarse, block_skip, idcs, xyzs, dirs,
                         dss, z_vals);
    return 0u;
}

// kMarchAlloc: every ray.  kMarchCount: the chunks after the leading ones (their number from
// `split`, the previous call's word), whose count sums start the frontier.
template <int kMode>
__global__ void __launch_bounds__(kThreadBlock) march_rays_kernel(
    std::uint32_t n_rays, std::uint32_t total_samples, MarchParams m,
    const float *__restrict__ rays_o, const float *__restrict__ rays_d,
    const float *__restrict__ t_starts, const float *__restrict__ t_ends,
    const float *__restrict__ noises, const std::uint8_t *__restrict__ bits,
    std::uint32_t *__restrict__ next_loc, std::uint32_t *__restrict__ n_exceeded, bool *__restrict__ ray_is_valid,
    std::uint32_t *__restrict__ rays_n_samples, std::uint32_t *__restrict__ rays_startidx,
    std::uint32_t *__restrict__ idcs, float *__restrict__ xyzs, float *__restrict__ dirs,
    float *__restrict__ dss, float *__restrict__ z_vals, const std::uint8_t *__restrict__ coarse,
    std::uint32_t *__restrict__ chunk_sums, std::uint32_t *__restrict__ chunk_done,
    unsigned long long *__restrict__ frontier, const std::uint32_t *__restrict__ split) {
    __shared__ std::uint32_t expand[1024];
    __shared__ std::uint32_t red[kThreadBlock / 32];
    __shared__ int s_full;
    const std::uint32_t n_chunks = (n_rays + kThreadBlock - 1) / kThreadBlock;
    const std::uint32_t c_lo = kMode == kMarchCount ? lead_chunks(split != nullptr ? *split : 0u, n_rays) : 0u;
    if (c_lo + blockIdx.x >= n_chunks) return;
    for (std::uint32_t v = threadIdx.x; v < m.G; v += blockDim.x) expand[v] = expand_bits(v);
    if constexpr (kMode == kMarchCount) {
        // the leading chunks are done (an earlier launch): their sum starts the frontier
        std::uint32_t a = 0;
        for (std::uint32_t c = threadIdx.x; c < c_lo; c += kThreadBlock) a += chunk_sums[c];
        a = warp_sum(a);
        if (lane_id() == 0) red[threadIdx.x >> 5] = a;
        __syncthreads();
        if (threadIdx.x == 0) {
            std::uint64_t p = 0;
            for (int w = 0; w < kThreadBlock / 32; ++w) p += red[w];
            atomicCAS(frontier, 0ull, frontier_pack(c_lo, p));   // the first block sets it
        }
    }
    __syncthreads();
    const float n_cap = (float)m.dns * m.bound;
    const bool block_skip = coarse != nullptr && m.K == 1 && m.const_ds && (m.G & 7u) == 0u;
    // block-uniform trips: every lane of a block runs the same trips (the allocation's warp scan,
    // the count mode's block sum)
    for (std::uint32_t c = c_lo + blockIdx.x; c < n_chunks; c += gridDim.x) {
        const std::uint64_t base = (std::uint64_t)c * kThreadBlock;
        if (kMode == kMarchCount) {   // the rays before this chunk fill the budget: all are dropped
            if (threadIdx.x == 0) s_full = frontier_sum(frontier) >= total_samples;
            __syncthreads();
            const bool full = s_full;
            __syncthreads();
            if (full) {   // no count (ray_scan_fit_kernel drops them); the chunk's sum stays 0
                if (base + threadIdx.x < n_rays) rays_n_samples[base + threadIdx.x] = 0u;
                continue;
            }
        }
        const std::uint32_t n = march_one<kMode>(
            (std::uint32_t)(base + threadIdx.x), n_rays, total_samples, m, n_cap, block_skip, rays_o, rays_d, t_starts,
            t_ends, noises, bits, next_loc, n_exceeded, ray_is_valid, rays_n_samples, rays_startidx, idcs, xyzs, dirs,
            dss, z_vals, coarse, expand, frontier);
        if (kMode == kMarchCount) {   // the sum of the chunk's counts (rays [base, base + kThreadBlock))
            const std::uint32_t w = warp_sum(n);
            if (lane_id() == 0) red[threadIdx.x >> 5] = w;
            __syncthreads();
            if (threadIdx.x < 32) {
                const std::uint32_t x = warp_sum(threadIdx.x < kThreadBlock / 32 ? red[threadIdx.x] : 0u);
                if (threadIdx.x == 0) publish_chunk(c, x, n_chunks, total_samples, chunk_sums, chunk_done, frontier);
            }
            __syncthreads();
        }
    }
}


// The fit of the training march, in ray order (marching.cu:135, :196-209 under the one-at-a-time
// schedule).  A block takes kScanRays rays; the sums of the counts of the chunks before it give
// its prefix.  P(r) is the sum of the counts of the rays before r; ray r is dropped when
// P(r) >= budget (invalid, no samples), valid without samples when its count is 0, fits when
// P(r) + n(r) <= budget (it gets the t of its first occupied sample, which the count pass left in
// its start word, in its first sample slot of dss, where the write pass resumes from it), and
// otherwise is the ray that does not fit (invalid; its samples are the ones left out).  The
// counters: the samples of the rays not dropped, and those of the ray that did not fit.  `split`
// receives the first dropped or unfit ray (~0u when there is none).
//
// The counts are exact for every ray up to the first that is dropped or does not fit, q: a ray
// stops counting only on reading a frontier sum P >= budget, and no ray up to q can (the chunks
// before its own sum to at most P(ray) < budget).  From q on, counts may be lower bounds, but
// each computed P(r) for r > q is at least P(q) + n(q) > budget, or at least the frontier sum
// >= budget that stopped it: every ray after q is dropped, as in the exact result.
constexpr int kScanRays = 1024;
static_assert(kScanRays % kThreadBlock == 0, "a scan block takes whole count chunks");

__global__ void __launch_bounds__(kScanRays) ray_scan_fit_kernel(
    std::uint32_t n_rays, std::uint32_t total_samples, const std::uint32_t *__restrict__ chunk_sums,
    bool *__restrict__ valid, std::uint32_t *__restrict__ counts, std::uint32_t *__restrict__ startidx,
    float *__restrict__ dss, std::uint32_t *__restrict__ next_loc, std::uint32_t *__restrict__ n_exceeded,
    std::uint32_t *__restrict__ split) {
    __shared__ unsigned long long s_prefix;
    __shared__ std::uint32_t s_first;
    __shared__ std::uint32_t ws[kScanRays / 32], wt[kScanRays / 32], wo[kScanRays / 32];
    if (threadIdx.x == 0) s_first = 0xffffffffu;
    if (threadIdx.x < 32) {
        unsigned long long a = 0;
        const std::uint32_t chunks = blockIdx.x * (kScanRays / kThreadBlock);
        for (std::uint32_t b = threadIdx.x; b < chunks; b += 32) a += chunk_sums[b];
        a = warp_sum(a);
        if (threadIdx.x == 0) s_prefix = a;
    }
    const std::uint32_t r = blockIdx.x * kScanRays + threadIdx.x;
    const std::uint32_t n = r < n_rays ? counts[r] : 0u;
    const std::uint32_t incl = warp_inclusive_scan(n);
    if (lane_id() == 31) ws[threadIdx.x >> 5] = incl;
    __syncthreads();
    if (threadIdx.x < 32) {
        const std::uint32_t x = ws[threadIdx.x];
        ws[threadIdx.x] = warp_inclusive_scan(x) - x;
    }
    __syncthreads();
    const unsigned long long start = s_prefix + ws[threadIdx.x >> 5] + (incl - n);
    const bool counted = start < (unsigned long long)total_samples;   // not dropped (marching.cu:135)
    const bool fits = counted && n > 0u && start + n <= (unsigned long long)total_samples;
    const bool unfit = counted && n > 0u && !fits;
    if (r < n_rays) {
        if (!counted || n > 0u) valid[r] = fits;
        counts[r] = fits ? n : 0u;
        if (fits) dss[start] = __uint_as_float(startidx[r]);
        startidx[r] = fits ? (std::uint32_t)start : 0u;
        if (!counted || unfit) atomicMin(&s_first, r);   // shared memory: cheap
    }
    const std::uint32_t tot = warp_sum(counted ? n : 0u), over = warp_sum(unfit ? n : 0u);
    if (lane_id() == 0) {
        wt[threadIdx.x >> 5] = tot;
        wo[threadIdx.x >> 5] = over;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const std::uint32_t a = warp_sum(wt[threadIdx.x]), o = warp_sum(wo[threadIdx.x]);
        if (threadIdx.x == 0) {
            if (a > 0u) atomicAdd(next_loc, a);
            if (o > 0u) atomicAdd(n_exceeded, o);
            if (s_first != 0xffffffffu && split != nullptr) atomicMin(split, s_first);
        }
    }
}

// ------------------------------------------------------------- march_rays, a warp per ray

// Lane j's view of a 32-step lookahead from t: its candidate t after j occupied steps (the
// additions the sequential march makes, in its order), whether the march loop's condition still
// holds there (`live`, given the lane's part of it in `cond`), and whether the cell is occupied.
struct Lookahead {
    float t, ds, mb;
    V3 pos, g;
    bool live, occ;
};

// t after j occupied steps from t0 (j <= 31): the sequential additions t <- fl(t + calc_ds(t)).
// With the constant step c of a bound <= 1 march, and t0 > 0 normal with ulp u, every addition
// whose exact sum stays below the next power of two T adds the same multiple of u: the sum
// (t/u + c/u) u rounds to (t/u + round(c/u)) u for integral t/u, unless c/u lies exactly half
// way between integers (a round-to-even tie, whose result depends on t).  Then
// t_j = t0 + j delta with delta = fl(t0 + c) - t0, each operation exact.  The fast form is taken
// only when c/u is no tie and t0 + 32 (delta + c) < T (a margin over the largest sum,
// t0 + 30 delta + c); otherwise the additions are made one by one.
__device__ __forceinline__ float chain_t(const MarchParams &m, float t0, unsigned j) {
    float delta, top;
    if (m.const_ds && chain_step(t0, m.ds_const, delta, top) && t0 + 32.f * (delta + m.ds_const) < top)
        return t0 + (float)j * delta;
    float tj = t0;
    for (unsigned i = 0; i < j; ++i) tj = tj + calc_ds(tj, m);
    return tj;
}

__device__ __forceinline__ void look_ahead(const MarchParams &m, float t, unsigned lane, V3 o, V3 d, float t1,
                                           bool cond, const std::uint8_t *__restrict__ bits,
                                           const std::uint32_t *expand, Lookahead &a) {
    const float tj = chain_t(m, t, lane);
    a.t = tj;
    a.pos = at(o, d, tj);
    a.ds = calc_ds(tj, m);
    a.live = cond && tj < t1;
    a.occ = a.live && occupied_at(m, a.pos, a.ds, bits, a.g, a.mb, expand);
}

// After a lookahead that accepted k occupied steps: the t the sequential march reaches next, or
// false when its loop ends at lane k (k < 32 and the condition fails there).  Lane k, on an empty
// cell, crosses the empty coarse block it lies in at once when skip_block can (the thread march's
// step at the same t), else the cell (skip_empty, marching.cu:182-189); and it goes on crossing
// empty cells by itself -- the thread march's steps, its occupancy test and its step count -- up
// to kSkipRun of them, so that a run of empty cells costs one lookahead trip, not one each.
// `skips` receives the steps taken.
constexpr std::uint32_t kSkipRun = 32;

__device__ __forceinline__ bool advance_skip(const MarchParams &m, const Lookahead &a, unsigned lane, unsigned k,
                                             V3 o, V3 d, V3 inv_d, float t1, const std::uint8_t *__restrict__ bits,
                                             const std::uint32_t *expand, const std::uint8_t *__restrict__ coarse,
                                             bool block_skip, std::uint32_t it_k, float &t, std::uint32_t &skips) {
    if (k < 32u) {
        if (!__shfl_sync(0xffffffffu, a.live, k)) return false;
        float nt = 0.f;
        std::uint32_t ns = 0;
        if (lane == k) {
            float tt = a.t;
            V3 g = a.g, pos = a.pos;
            float mb = a.mb;
            for (;;) {   // it_k + ns: the step count before this skip
                float tb;
                tt = (block_skip && skip_block(m, tt, g, pos, o, d, inv_d, coarse, tb))
                         ? tb : skip_empty(m, tt, g, mb, pos, d, inv_d);
                ++ns;
                if (ns >= kSkipRun || !(tt < t1) || it_k + ns >= kMaxMarchIters) break;
                pos = at(o, d, tt);
                if (occupied_at(m, pos, calc_ds(tt, m), bits, g, mb, expand)) break;   // the next trip samples here
            }
            nt = tt;
        }
        t = __shfl_sync(0xffffffffu, nt, k);
        skips = __shfl_sync(0xffffffffu, ns, k);
    } else {
        const float nt = lane == 31u ? a.t + a.ds : 0.f;
        t = __shfl_sync(0xffffffffu, nt, 31);
        skips = 0;
    }
    return true;
}

constexpr int kWarpTrips = 256;   // trips with samples the count pass records per ray (per warp)

// The list form of the training march (the proposal sampler's per-ray fallback) marches a few
// thousand rays of a batch, each through occupied space.  With a lane per ray, each ray's chain of
// dependent steps would run alone while most of the GPU idled; here a warp takes one ray and looks
// 32 steps ahead.  All lanes test their candidate cells at once, and the warp accepts the samples
// up to the first lane whose cell is empty or whose step ends the ray.  Both passes (count, then
// write from the first occupied sample) follow march_rays_kernel's sequence, so each ray's count,
// validity and samples are bit-identical to it.  The budget probe checks the counter once per trip
// that reaches the ray's first occupied sample or every 16th after it, if the ray goes on.  The
// count pass records, per trip that took samples, the trip's starting t and how many it took
// (up to kWarpTrips trips); the write pass then replays those trips -- the same additions from
// the same t -- without looking at the grid again, and re-marches only a ray with more trips.
// Few warps are busy at once (one per listed ray), so no minimum residency is asked of the
// register allocator.
__global__ void __launch_bounds__(kMarchBlock) march_rays_warp_kernel(
    std::uint32_t n_rays, std::uint32_t total_samples, MarchParams m,
    const float *__restrict__ rays_o, const float *__restrict__ rays_d,
    const float *__restrict__ t_starts, const float *__restrict__ t_ends,
    const float *__restrict__ noises, const std::uint8_t *__restrict__ bits,
    std::uint32_t *__restrict__ next_loc, std::uint32_t *__restrict__ n_exceeded,
    std::uint32_t *__restrict__ queue, bool *__restrict__ ray_is_valid,
    std::uint32_t *__restrict__ rays_n_samples, std::uint32_t *__restrict__ rays_startidx,
    std::uint32_t *__restrict__ idcs, float *__restrict__ xyzs, float *__restrict__ dirs,
    float *__restrict__ dss, float *__restrict__ z_vals, const std::uint32_t *__restrict__ ray_list,
    const std::uint32_t *__restrict__ list_count) {
    __shared__ std::uint32_t expand[1024];  // expand_bits(v), v < G (G <= 1024)
    __shared__ float trip_t[kMarchBlock / 32][kWarpTrips];
    __shared__ std::uint8_t trip_k[kMarchBlock / 32][kWarpTrips];
    n_rays = min(n_rays, *list_count);
    for (std::uint32_t v = threadIdx.x; v < m.G; v += blockDim.x) expand[v] = expand_bits(v);
    __syncthreads();
    const unsigned lane = lane_id(), wib = threadIdx.x >> 5;
    const float n_cap = (float)m.dns * m.bound;
    for (;;) {
        std::uint32_t q = 0;
        if (lane == 0) q = atomicAdd(queue, 1u);
        q = __shfl_sync(0xffffffffu, q, 0);
        if (q >= n_rays) break;
        const std::uint32_t r = ray_list[q];
        const V3 o{rays_o[r * 3 + 0], rays_o[r * 3 + 1], rays_o[r * 3 + 2]};
        const V3 d{rays_d[r * 3 + 0], rays_d[r * 3 + 1], rays_d[r * 3 + 2]};
        const float t0 = t_starts[r], t1 = t_ends[r];
        if (!(t1 > t0)) {  // marching.cu:151
            if (lane == 0) {
                ray_is_valid[r] = false;
                rays_n_samples[r] = 0;
                rays_startidx[r] = 0;
            }
            continue;
        }
        const V3 inv_d{1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
        // ---- count pass (marching.cu:162-192)
        float t = t0 + calc_ds(t0, m) * noises[r], t_hit = 0.f;
        std::uint32_t n = 0, it = 0, trips = 0;
        bool dropped = false;
        for (;;) {
            Lookahead a;
            look_ahead(m, t, lane, o, d, t1, (float)(n + lane) < n_cap && it + lane < kMaxMarchIters, bits, expand, a);
            const unsigned stop = __ballot_sync(0xffffffffu, !a.occ);
            const unsigned k = stop != 0u ? (unsigned)__ffs(stop) - 1u : 32u;
            if (n == 0 && k > 0) t_hit = t;
            if (k > 0) {
                if (lane == 0 && trips < (std::uint32_t)kWarpTrips) {
                    trip_t[wib][trips] = t;
                    trip_k[wib][trips] = (std::uint8_t)k;
                }
                ++trips;
            }
            const std::uint32_t n0 = n;
            n += k;
            it += k;
            std::uint32_t skips = 0;
            const bool more = advance_skip(m, a, lane, k, o, d, inv_d, t1, bits, expand, nullptr, false, it, t, skips);
            if (!more) break;
            it += skips;   // each skip is a step of its own
            // a sample numbered 1, 17, 33, ... was taken in this trip: probe the budget (lane 0
            // reads the counter, so the whole warp takes the same decision)
            if (k > 0 && ((n0 + 15u) >> 4) != ((n + 15u) >> 4)) {
                int full = 0;
                if (lane == 0) full = *((volatile std::uint32_t *)next_loc) >= total_samples;
                if (__shfl_sync(0xffffffffu, full, 0)) {
                    dropped = true;
                    break;
                }
            }
        }
        if (dropped || n == 0) {  // over budget, or marching.cu:196-199: valid with no samples
            if (lane == 0) {
                ray_is_valid[r] = !dropped;
                rays_n_samples[r] = 0;
                rays_startidx[r] = 0;
            }
            continue;
        }
        std::uint32_t start = 0;
        if (lane == 0) start = atomicAdd(next_loc, n);
        start = __shfl_sync(0xffffffffu, start, 0);
        const bool fits = (std::uint64_t)start + n <= total_samples;
        if (lane == 0) {
            ray_is_valid[r] = fits;
            rays_n_samples[r] = fits ? n : 0u;
            rays_startidx[r] = fits ? start : 0u;
            if (!fits) atomicAdd(n_exceeded, n);
        }
        if (!fits) continue;
        // ---- write pass from the first occupied sample (marching.cu:224-267)
        __syncwarp();
        if (trips <= (std::uint32_t)kWarpTrips) {   // replay the recorded trips
            std::uint32_t w = 0;
            for (std::uint32_t e = 0; e < trips; ++e) {
                const unsigned k = trip_k[wib][e];
                if (lane < k) {
                    const float tj = chain_t(m, trip_t[wib][e], lane);
                    const V3 pos = at(o, d, tj);
                    const std::uint32_t s = start + w + lane;
                    idcs[s] = r;
                    xyzs[(std::size_t)s * 3 + 0] = pos.x;
                    xyzs[(std::size_t)s * 3 + 1] = pos.y;
                    xyzs[(std::size_t)s * 3 + 2] = pos.z;
                    dirs[(std::size_t)s * 3 + 0] = d.x;
                    dirs[(std::size_t)s * 3 + 1] = d.y;
                    dirs[(std::size_t)s * 3 + 2] = d.z;
                    dss[s] = calc_ds(tj, m);
                    z_vals[s] = tj;
                }
                w += k;
            }
            __syncwarp();   // the next ray's count pass overwrites the records
            continue;
        }
        t = t_hit;
        std::uint32_t w = 0;
        it = 0;
        for (;;) {
            Lookahead a;
            look_ahead(m, t, lane, o, d, t1, w + lane < n && it + lane < kMaxMarchIters, bits, expand, a);
            const unsigned stop = __ballot_sync(0xffffffffu, !a.occ);
            const unsigned k = stop != 0u ? (unsigned)__ffs(stop) - 1u : 32u;
            if (lane < k) {
                const std::uint32_t s = start + w + lane;
                idcs[s] = r;
                xyzs[(std::size_t)s * 3 + 0] = a.pos.x;
                xyzs[(std::size_t)s * 3 + 1] = a.pos.y;
                xyzs[(std::size_t)s * 3 + 2] = a.pos.z;
                dirs[(std::size_t)s * 3 + 0] = d.x;
                dirs[(std::size_t)s * 3 + 1] = d.y;
                dirs[(std::size_t)s * 3 + 2] = d.z;
                dss[s] = a.ds;
                z_vals[s] = a.t;
            }
            w += k;
            it += k;
            std::uint32_t skips = 0;
            if (!advance_skip(m, a, lane, k, o, d, inv_d, t1, bits, expand, nullptr, false, it, t, skips)) break;
            it += skips;
        }
    }
}

// ------------------------------------------------- the training march's warp-per-ray passes

// One ray by one warp, from t: the count (kWrite false: up to n_cap samples, and t_hit, the t of
// the first) or the writing of its n_write samples from slot `start` (kWrite true).  The steps
// are march_rays_kernel's, 32 at a time (look_ahead); every lane returns the same count.
template <bool kWrite>
__device__ __forceinline__ std::uint32_t warp_march(
    const MarchParams &m, V3 o, V3 d, V3 inv_d, float t, float t1, float n_cap, std::uint32_t n_write,
    const std::uint8_t *__restrict__ bits, const std::uint32_t *expand, const std::uint8_t *__restrict__ coarse,
    bool block_skip, unsigned lane, float &t_hit, std::uint32_t r, std::uint32_t start,
    std::uint32_t *__restrict__ idcs, float *__restrict__ xyzs, float *__restrict__ dirs,
    float *__restrict__ dss, float *__restrict__ z_vals) {
    std::uint32_t n = 0, it = 0;
    for (;;) {
        const bool cond = kWrite ? n + lane < n_write : (float)(n + lane) < n_cap;
        Lookahead a;
        look_ahead(m, t, lane, o, d, t1, cond && it + lane < kMaxMarchIters, bits, expand, a);
        const unsigned stop = __ballot_sync(0xffffffffu, !a.occ);
        const unsigned k = stop != 0u ? (unsigned)__ffs(stop) - 1u : 32u;
        if (kWrite) {
            if (lane < k) {
                const std::uint32_t s = start + n + lane;
                idcs[s] = r;
                xyzs[(std::size_t)s * 3 + 0] = a.pos.x;
                xyzs[(std::size_t)s * 3 + 1] = a.pos.y;
                xyzs[(std::size_t)s * 3 + 2] = a.pos.z;
                dirs[(std::size_t)s * 3 + 0] = d.x;
                dirs[(std::size_t)s * 3 + 1] = d.y;
                dirs[(std::size_t)s * 3 + 2] = d.z;
                dss[s] = a.ds;
                z_vals[s] = a.t;
            }
        } else if (n == 0u && k > 0u) {
            t_hit = t;   // lane 0's sample: the trip starts at it
        }
        n += k;
        it += k;
        std::uint32_t skips = 0;
        if (!advance_skip(m, a, lane, k, o, d, inv_d, t1, bits, expand, coarse, block_skip, it, t, skips)) break;
        it += skips;   // each skip is a step of its own
    }
    return n;
}

constexpr int kWarpBlock = 64;    // 2 rays at a time per block: a block frees its registers as soon as its rays are done
constexpr std::uint32_t kSmemCoarse = 4096;   // coarse grids up to 16^3 blocks (G <= 128) go to shared memory

// The coarse grid in shared memory when it fits (every block of a warp kernel reads it at each
// empty cell), else the global copy.
__device__ __forceinline__ const std::uint8_t *stage_coarse(const MarchParams &m, const std::uint8_t *coarse,
                                                            std::uint8_t *s_coarse) {
    if (coarse == nullptr) return nullptr;
    const std::uint32_t Gc = m.G >> 3, nc = Gc * Gc * Gc;
    if (nc > kSmemCoarse) return coarse;
    for (std::uint32_t i = threadIdx.x; i < nc; i += blockDim.x) s_coarse[i] = coarse[i];
    return s_coarse;
}

// The leading rays of the training march, counted in full, a warp per ray: validity, count and
// the t of the first sample (in the start word) per ray, and each chunk's count sum.
__global__ void __launch_bounds__(kWarpBlock) march_lead_kernel(
    std::uint32_t n_rays, MarchParams m, const float *__restrict__ rays_o, const float *__restrict__ rays_d,
    const float *__restrict__ t_starts, const float *__restrict__ t_ends, const float *__restrict__ noises,
    const std::uint8_t *__restrict__ bits, const std::uint8_t *__restrict__ coarse,
    const std::uint32_t *__restrict__ split, bool *__restrict__ ray_is_valid,
    std::uint32_t *__restrict__ rays_n_samples, std::uint32_t *__restrict__ rays_startidx,
    std::uint32_t *__restrict__ chunk_sums) {
    __shared__ std::uint32_t expand[1024];
    __shared__ std::uint8_t s_coarse[kSmemCoarse];
    const std::uint32_t lead =
        min(lead_chunks(split != nullptr ? *split : 0u, n_rays) * (std::uint32_t)kThreadBlock, n_rays);
    const std::uint32_t warp0 = blockIdx.x * (kWarpBlock / 32);
    if (warp0 >= lead) return;
    for (std::uint32_t v = threadIdx.x; v < m.G; v += blockDim.x) expand[v] = expand_bits(v);
    coarse = stage_coarse(m, coarse, s_coarse);
    __syncthreads();
    const unsigned lane = lane_id();
    const float n_cap = (float)m.dns * m.bound;
    const bool block_skip = coarse != nullptr && m.K == 1 && m.const_ds && (m.G & 7u) == 0u;
    for (std::uint32_t r = warp0 + (threadIdx.x >> 5); r < lead; r += gridDim.x * (kWarpBlock / 32)) {
        const V3 o{rays_o[r * 3 + 0], rays_o[r * 3 + 1], rays_o[r * 3 + 2]};
        const V3 d{rays_d[r * 3 + 0], rays_d[r * 3 + 1], rays_d[r * 3 + 2]};
        const float t0 = t_starts[r], t1 = t_ends[r];
        std::uint32_t n = 0;
        float t_hit = 0.f;
        if (t1 > t0 && !(coarse != nullptr && no_sample_possible(m, o, d, t0, t1, coarse))) {
            const V3 inv_d{1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
            n = warp_march<false>(m, o, d, inv_d, t0 + calc_ds(t0, m) * noises[r], t1, n_cap, 0u, bits, expand,
                                  coarse, block_skip, lane, t_hit, r, 0u, nullptr, nullptr, nullptr, nullptr, nullptr);
        }
        if (lane == 0) {
            ray_is_valid[r] = t1 > t0;   // marching.cu:151; ray_scan_fit_kernel decides the rest
            rays_n_samples[r] = n;
            rays_startidx[r] = __float_as_uint(t_hit);
            if (n > 0u) atomicAdd(chunk_sums + r / kThreadBlock, n);
        }
    }
}

// The samples of the rays that fit (marching.cu:224-267), a warp per ray, from the t of each
// ray's first sample (left in its first slot of dss); the rays that fit all come before the first
// dropped or unfit ray (`split`, all rays when null).  (A thread per ray where many rays of a
// chunk fit was measured slower on both a training budget and an unbounded one: the rays that fit
// are long, ~250 samples, in both.)
__global__ void __launch_bounds__(kWarpBlock) march_write_kernel(
    std::uint32_t n_rays, MarchParams m, const float *__restrict__ rays_o, const float *__restrict__ rays_d,
    const float *__restrict__ t_ends, const std::uint8_t *__restrict__ bits, const std::uint8_t *__restrict__ coarse,
    const std::uint32_t *__restrict__ split, const std::uint32_t *__restrict__ rays_n_samples,
    const std::uint32_t *__restrict__ rays_startidx, std::uint32_t *__restrict__ idcs, float *__restrict__ xyzs,
    float *__restrict__ dirs, float *__restrict__ dss, float *__restrict__ z_vals) {
    __shared__ std::uint32_t expand[1024];
    __shared__ std::uint8_t s_coarse[kSmemCoarse];
    const std::uint32_t end = split != nullptr ? min(*split, n_rays) : n_rays;
    const std::uint32_t warp0 = blockIdx.x * (kWarpBlock / 32);
    if (warp0 >= end) return;
    for (std::uint32_t v = threadIdx.x; v < m.G; v += blockDim.x) expand[v] = expand_bits(v);
    coarse = stage_coarse(m, coarse, s_coarse);
    __syncthreads();
    const unsigned lane = lane_id();
    const bool block_skip = coarse != nullptr && m.K == 1 && m.const_ds && (m.G & 7u) == 0u;
    for (std::uint32_t r = warp0 + (threadIdx.x >> 5); r < end; r += gridDim.x * (kWarpBlock / 32)) {
        const std::uint32_t n = rays_n_samples[r];
        if (n == 0u) continue;
        const std::uint32_t start = rays_startidx[r];
        const V3 o{rays_o[r * 3 + 0], rays_o[r * 3 + 1], rays_o[r * 3 + 2]};
        const V3 d{rays_d[r * 3 + 0], rays_d[r * 3 + 1], rays_d[r * 3 + 2]};
        const V3 inv_d{1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
        const float t = dss[start];
        __syncwarp();   // every lane has read the first slot before lane 0 overwrites it
        float unused = 0.f;
        warp_march<true>(m, o, d, inv_d, t, t_ends[r], 0.f, n, bits, expand, coarse, block_skip, lane, unused, r,
                         start, idcs, xyzs, dirs, dss, z_vals);
    }
}

// Zero the sample slots no ray wrote: [next_loc - n_exceeded, total_samples).  Every slot below
// that bound belongs to a ray that fit, because the counter only grows and the first ray that
// did not fit started exactly there.
__global__ void zero_sample_tail_kernel(std::uint32_t total_samples,
                                        const std::uint32_t *__restrict__ next_loc,
                                        const std::uint32_t *__restrict__ n_exceeded,
                                        std::uint32_t *__restrict__ idcs, float *__restrict__ xyzs,
                                        float *__restrict__ dirs, float *__restrict__ dss,
                                        float *__restrict__ z_vals) {
    std::uint32_t used = *next_loc - *n_exceeded;
    if (used > total_samples) used = total_samples;
    const std::size_t stride = (std::size_t)gridDim.x * blockDim.x;
    for (std::size_t s = used + (std::size_t)blockIdx.x * blockDim.x + threadIdx.x; s < total_samples; s += stride) {
        idcs[s] = 0;
        dss[s] = 0.f;
        z_vals[s] = 0.f;
        xyzs[s * 3 + 0] = 0.f;
        xyzs[s * 3 + 1] = 0.f;
        xyzs[s * 3 + 2] = 0.f;
        dirs[s * 3 + 0] = 0.f;
        dirs[s * 3 + 1] = 0.f;
        dirs[s * 3 + 2] = 0.f;
    }
}

// --------------------------------------------------------------------- march_rays_inference

__global__ void __launch_bounds__(256) march_rays_inference_kernel(
    std::uint32_t n_total_rays, std::uint32_t n_rays, std::uint32_t cap, MarchParams m,
    const float *__restrict__ rays_o, const float *__restrict__ rays_d,
    const float *__restrict__ t_starts, const float *__restrict__ t_ends,
    const std::uint8_t *__restrict__ bits, const bool *__restrict__ terminated,
    const std::uint32_t *__restrict__ indices_in, std::uint32_t *__restrict__ next_ray_index,
    std::uint32_t *__restrict__ indices_out, std::uint32_t *__restrict__ n_samples,
    float *__restrict__ t_starts_out, float *__restrict__ xyzs, float *__restrict__ dss,
    float *__restrict__ z_vals) {
    const std::uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in_range = i < n_rays;
    const bool refill = in_range && terminated[i];
    // marching.cu:300: finished slots take fresh rays, one atomic per warp, slot order in a warp
    const unsigned ballot = __ballot_sync(0xffffffffu, refill);
    const int leader = ballot != 0 ? __ffs(ballot) - 1 : 0;  // lowest refilling lane
    std::uint32_t base = 0;
    if (ballot != 0 && (int)lane_id() == leader) base = atomicAdd(next_ray_index, (unsigned)__popc(ballot));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (!in_range) return;
    const std::uint32_t r = refill ? base + __popc(ballot & ((1u << lane_id()) - 1u)) : indices_in[i];
    indices_out[i] = r;

    float *rx = xyzs + (std::size_t)i * cap * 3;
    float *rs = dss + (std::size_t)i * cap;
    float *rz = z_vals + (std::size_t)i * cap;
    std::uint32_t steps = 0;
    float t = 0.f;
    bool wrote_t = false;
    if (r < n_total_rays) {
        const V3 o = {rays_o[(std::size_t)r * 3 + 0], rays_o[(std::size_t)r * 3 + 1], rays_o[(std::size_t)r * 3 + 2]};
        const V3 d = {rays_d[(std::size_t)r * 3 + 0], rays_d[(std::size_t)r * 3 + 1], rays_d[(std::size_t)r * 3 + 2]};
        const float t0 = t_starts[r], t1 = t_ends[r];
        if (!(t1 < t0)) {  // marching.cu:317
            wrote_t = true;
            const V3 inv_d = {1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
            t = t0;
            for (std::uint32_t it = 0; steps < cap && t < t1 && it < kMaxMarchIters; ++it) {
                V3 pos = at(o, d, t);
                float ds = calc_ds(t, m);
                V3 g;
                float mb;
                if (occupied_at(m, pos, ds, bits, g, mb)) {
                    rx[steps * 3 + 0] = pos.x;
                    rx[steps * 3 + 1] = pos.y;
                    rx[steps * 3 + 2] = pos.z;
                    rs[steps] = ds;
                    rz[steps] = t;
                    ++steps;
                    t = t + ds;
                } else {
                    t = skip_empty(m, t, g, mb, pos, d, inv_d);
                }
            }
            if (t >= t1) {  // marching.cu:367-394: far-plane sample
                V3 pos = at(o, d, t1);
                float ds = calc_ds(t1, m);
                V3 g;
                float mb;
                if (occupied_at(m, pos, ds, bits, g, mb)) {
                    if (steps > 0 && rs[steps - 1] + rz[steps - 1] >= t1) rs[steps - 1] = t1 - rz[steps - 1];
                    if (steps < cap) {
                        rx[steps * 3 + 0] = pos.x;
                        rx[steps * 3 + 1] = pos.y;
                        rx[steps * 3 + 2] = pos.z;
                        rs[steps] = ds;
                        rz[steps] = t1;
                        ++steps;
                    } else {
                        t = t1;
                    }
                }
            }
        }
    }
    // zero the unused slots of this ray (the reference memsets the whole outputs up front)
    for (std::uint32_t k = steps; k < cap; ++k) {
        rx[k * 3 + 0] = 0.f;
        rx[k * 3 + 1] = 0.f;
        rx[k * 3 + 2] = 0.f;
        rs[k] = 0.f;
        rz[k] = 0.f;
    }
    n_samples[i] = steps;
    t_starts_out[i] = wrote_t ? t : 0.f;
}

// Marches one ray of the inference renderer from t0 for at most `cap` samples (marching.cu:315-396):
// sample k goes to sx[3k..3k+2], sd[k], sz[k].  Returns the number of samples; t_out receives the
// advanced t to scatter into t_starts (0 for a ray with t_end < t_start).
__device__ __forceinline__ std::uint32_t march_inference_ray(const MarchParams &m, std::uint32_t cap, const V3 &o,
                                                             const V3 &d, float t0, float t1,
                                                             const std::uint8_t *__restrict__ bits, float *sx,
                                                             float *sd, float *sz, float &t_out) {
    std::uint32_t steps = 0;
    float t = 0.f;
    if (!(t1 < t0)) {
        const V3 inv_d = {1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
        t = t0;
        for (std::uint32_t it = 0; steps < cap && t < t1 && it < kMaxMarchIters; ++it) {
            V3 pos = at(o, d, t);
            float ds = calc_ds(t, m);
            V3 g;
            float mb;
            if (occupied_at(m, pos, ds, bits, g, mb)) {
                sx[steps * 3 + 0] = pos.x;
                sx[steps * 3 + 1] = pos.y;
                sx[steps * 3 + 2] = pos.z;
                sd[steps] = ds;
                sz[steps] = t;
                ++steps;
                t = t + ds;
            } else {
                t = skip_empty(m, t, g, mb, pos, d, inv_d);
            }
        }
        if (t >= t1) {
            V3 pos = at(o, d, t1);
            float ds = calc_ds(t1, m);
            V3 g;
            float mb;
            if (occupied_at(m, pos, ds, bits, g, mb)) {
                if (steps > 0 && sd[steps - 1] + sz[steps - 1] >= t1) sd[steps - 1] = t1 - sz[steps - 1];
                if (steps < cap) {
                    sx[steps * 3 + 0] = pos.x;
                    sx[steps * 3 + 1] = pos.y;
                    sx[steps * 3 + 2] = pos.z;
                    sd[steps] = ds;
                    sz[steps] = t1;
                    ++steps;
                } else {
                    t = t1;
                }
            }
        }
    }
    t_out = t;
    return steps;
}

// In-place forms for the device-resident renderer: the slot indices and the next-ray counter are
// read and updated in place, the advanced t is scattered straight into t_starts (what
// marching/__init__.py:156 does with .at[].set on the host side), and each sample also gets its
// ray's direction (the field needs it; renderers/cuda.py:225 broadcasts rays_d[indices]).
//
// kCompact = false: samples stay in the slot's `cap` strided entries (unused ones zeroed).
// kCompact = true:  dss / z_vals stay strided, but positions and directions are packed densely:
// a warp reserves one range of *sample_count for its lanes' samples (one atomic per warp) and
// sample_start[i] records where slot i's samples begin, so the encoder and the MLP run on
// *sample_count samples instead of n * cap.
constexpr std::uint32_t kCompactMaxCap = 16;

template <bool kCompact>
__global__ void __launch_bounds__(256) march_rays_inference_inplace_kernel(
    std::uint32_t n_total_rays, std::uint32_t n_rays, std::uint32_t cap, MarchParams m,
    const float *__restrict__ rays_o, const float *__restrict__ rays_d, float *__restrict__ t_starts,
    const float *__restrict__ t_ends, const std::uint8_t *__restrict__ bits, const bool *__restrict__ terminated,
    std::uint32_t *__restrict__ indices, std::uint32_t *__restrict__ next_ray_index,
    std::uint32_t *__restrict__ n_samples, std::uint32_t *__restrict__ sample_start,
    std::uint32_t *__restrict__ sample_count, float *__restrict__ xyzs, float *__restrict__ dirs,
    float *__restrict__ dss, float *__restrict__ z_vals) {
    const std::uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in_range = i < n_rays;
    const bool refill = in_range && terminated[i];
    const unsigned ballot = __ballot_sync(0xffffffffu, refill);
    const int leader = ballot != 0 ? __ffs(ballot) - 1 : 0;
    std::uint32_t base = 0;
    if (ballot != 0 && (int)lane_id() == leader) base = atomicAdd(next_ray_index, (unsigned)__popc(ballot));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (!kCompact && !in_range) return;
    std::uint32_t r = n_total_rays;
    if (in_range) {
        r = refill ? base + __popc(ballot & ((1u << lane_id()) - 1u)) : indices[i];
        indices[i] = r;
    }
    float lx[kCompact ? kCompactMaxCap * 3 : 1];
    float *rx = kCompact ? lx : xyzs + (std::size_t)i * cap * 3;
    float *rs = dss + (std::size_t)i * cap, *rz = z_vals + (std::size_t)i * cap;
    std::uint32_t steps = 0;
    V3 d = {0.f, 0.f, 1.f};
    if (in_range && r < n_total_rays) {
        const V3 o = {rays_o[(std::size_t)r * 3 + 0], rays_o[(std::size_t)r * 3 + 1], rays_o[(std::size_t)r * 3 + 2]};
        d = {rays_d[(std::size_t)r * 3 + 0], rays_d[(std::size_t)r * 3 + 1], rays_d[(std::size_t)r * 3 + 2]};
        float t;
        steps = march_inference_ray(m, cap, o, d, t_starts[r], t_ends[r], bits, rx, rs, rz, t);
        t_starts[r] = t;  // marching.cu:396 + marching/__init__.py:156
    }
    if (in_range) {
        for (std::uint32_t k = steps; k < cap; ++k) {
            rs[k] = 0.f;
            rz[k] = 0.f;
        }
        n_samples[i] = steps;
    }
    if (!kCompact) {
        float *rdir = dirs + (std::size_t)i * cap * 3;
        for (std::uint32_t k = 0; k < cap; ++k) {
            const bool s = k < steps;
            if (!s) {
                rx[k * 3 + 0] = 0.f;
                rx[k * 3 + 1] = 0.f;
                rx[k * 3 + 2] = 0.f;
            }
            rdir[k * 3 + 0] = s ? d.x : 0.f;
            rdir[k * 3 + 1] = s ? d.y : 0.f;
            rdir[k * 3 + 2] = s ? d.z : 1.f;
        }
    } else {
        const std::uint32_t incl = warp_inclusive_scan(steps);
        const std::uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        std::uint32_t wbase = 0;
        if (lane_id() == 31 && total > 0) wbase = atomicAdd(sample_count, total);
        wbase = __shfl_sync(0xffffffffu, wbase, 31);
        const std::uint32_t start = wbase + incl - steps;
        if (in_range) sample_start[i] = start;
        for (std::uint32_t k = 0; k < steps; ++k) {
            float *px = xyzs + (std::size_t)(start + k) * 3, *pd = dirs + (std::size_t)(start + k) * 3;
            px[0] = rx[k * 3 + 0];
            px[1] = rx[k * 3 + 1];
            px[2] = rx[k * 3 + 2];
            pd[0] = d.x;
            pd[1] = d.y;
            pd[2] = d.z;
        }
    }
}

__global__ void copy_counter_kernel(const std::uint32_t *__restrict__ src, std::uint32_t *__restrict__ dst) {
    *dst = *src;
}

// --------------------------------------------------------------------------------- morton3d

__global__ void morton3d_kernel(std::uint32_t n, const std::uint32_t *__restrict__ xyz, std::uint32_t *__restrict__ idcs) {
    for (std::size_t i = (std::size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (std::size_t)gridDim.x * blockDim.x)
        idcs[i] = morton3(xyz[i * 3 + 0], xyz[i * 3 + 1], xyz[i * 3 + 2]);
}

__global__ void morton3d_invert_kernel(std::uint32_t n, const std::uint32_t *__restrict__ idcs, std::uint32_t *__restrict__ xyz) {
    for (std::size_t i = (std::size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (std::size_t)gridDim.x * blockDim.x) {
        std::uint32_t c = idcs[i];
        xyz[i * 3 + 0] = morton3_invert(c >> 0);
        xyz[i * 3 + 1] = morton3_invert(c >> 1);
        xyz[i * 3 + 2] = morton3_invert(c >> 2);
    }
}

MarchParams make_params(std::uint32_t dns, std::uint32_t K, std::uint32_t G, float bound, float sp) {
    MarchParams m;
    m.dns = dns;
    m.K = K;
    m.G = G;
    m.bound = bound;
    m.sp = sp;
    m.inv_G = 1.0f / (float)G;
    m.ds_lo = 2.0f * kSqrt3 * fminf(bound, 1.0f) / (float)dns;
    m.ds_hi = 2.0f * kSqrt3 * bound * m.inv_G;
    m.const_ds = sp == 0.0f;
    m.ds_const = fminf(m.ds_lo, m.ds_hi);
    m.mb0 = fminf(1.0f, bound);
    std::uint32_t u;
    std::memcpy(&u, &m.mb0, 4);
    m.pow2_0 = (u & 0x007FFFFFu) == 0u && m.mb0 >= 1.17549435e-38f;
    const std::uint32_t iu = 0x7F000000u - u;
    m.inv_mb0 = 0.f;
    if (m.pow2_0) std::memcpy(&m.inv_mb0, &iu, 4);
    return m;
}

}  // namespace

// ----------------------------------------------------------------------------- launchers


int set_march_blocks_per_sm(int n) {
    if (n < 0 || n > kMarchBlocksPerSm) return -1;
    return g_march_blocks_per_sm.exchange(n == 0 ? kMarchBlocksPerSm : n);
}

int launch_march_rays(cudaStream_t stream, const MarchingDescriptor &d, const float *rays_o,
                      const float *rays_d, const float *t_starts, const float *t_ends,
                      const float *noises, const std::uint8_t *bits, std::uint32_t *next_loc,
                      std::uint32_t *n_exceeded, bool *ray_is_valid, std::uint32_t *rays_n_samples,
                      std::uint32_t *rays_startidx, std::uint32_t *idcs, float *xyzs, float *dirs,
                      float *dss, float *z_vals, std::uint32_t *queue, bool ordered, const std::uint8_t *coarse) {
    NGP_CHECK_ARG(d.K > 0 && d.G > 0 && d.diagonal_n_steps > 0, "march_rays: K, G and diagonal_n_steps must be positive");
    NGP_CHECK_ARG(d.G <= 1024 && (d.G & (d.G - 1)) == 0, "march_rays: G must be a power of two <= 1024 (Morton codes of other sizes exceed G^3)");
    NGP_CHECK_ARG(d.K <= 16, "march_rays: at most 16 cascades");
    NGP_CHECK_ARG(d.bound > 0.f && d.stepsize_portion >= 0.f, "march_rays: bound must be positive, stepsize_portion non-negative");
    NGP_CUDA_TRY(cudaMemsetAsync(next_loc, 0, sizeof(std::uint32_t), stream));
    NGP_CUDA_TRY(cudaMemsetAsync(n_exceeded, 0, sizeof(std::uint32_t), stream));
    const MarchParams m = make_params(d.diagonal_n_steps, d.K, d.G, d.bound, d.stepsize_portion);
    if (d.n_rays > 0) {
        // a thread per ray, at most g_march_blocks_per_sm CTAs per SM (the kernel strides over the rest)
        const unsigned blocks_needed = (d.n_rays + kThreadBlock - 1) / kThreadBlock;
        const unsigned cap = (unsigned)sm_count() * (unsigned)g_march_blocks_per_sm.load(std::memory_order_relaxed);
        const unsigned grid = blocks_needed < cap ? blocks_needed : cap;
        const std::uint32_t n_chunks = (std::uint32_t)blocks_needed;   // count chunks of kThreadBlock rays
        if (ordered && 2ull * n_chunks + 3u <= d.total_samples &&
            (reinterpret_cast<std::uintptr_t>(idcs) & 3u) == 0u) {
            // the chunk sums, the chunks' done flags and the frontier borrow the sample-index
            // buffer's last 2 n_chunks + 3 words, which the write pass and the tail zeroing
            // overwrite after the fit has read them
            std::uint32_t *sums = idcs + (d.total_samples - n_chunks);
            std::uint32_t *done = sums - n_chunks;
            std::uint32_t *fw = done - 2;   // an 8-byte aligned pair in [done - 3, done)
            if (reinterpret_cast<std::uintptr_t>(fw) & 7u) --fw;
            unsigned long long *frontier = reinterpret_cast<unsigned long long *>(fw);
            NGP_CUDA_TRY(cudaMemsetAsync(done - 3, 0, sizeof(std::uint32_t) * (2 * n_chunks + 3), stream));
            // warp-per-ray grids: a warp per leading ray; for the writes, at most as many threads
            // as the thread-per-ray grid's cap
            const unsigned wpb = kWarpBlock / 32;
            const unsigned cap_w = cap * (unsigned)(kThreadBlock / kWarpBlock);
            const std::uint32_t lead_max = d.n_rays < kLeadMax ? d.n_rays : kLeadMax;
            const unsigned lead_grid = (lead_max + wpb - 1) / wpb;
            const unsigned write_need = (d.n_rays + wpb - 1) / wpb;
            const unsigned write_grid = write_need < cap_w ? write_need : cap_w;
            // the leading rays, then the rest (how many lead: `queue` as the previous call left it)
            march_lead_kernel<<<lead_grid < cap_w ? lead_grid : cap_w, kWarpBlock, 0, stream>>>(
                d.n_rays, m, rays_o, rays_d, t_starts, t_ends, noises, bits, coarse, queue, ray_is_valid,
                rays_n_samples, rays_startidx, sums);
            march_rays_kernel<kMarchCount><<<grid, kThreadBlock, 0, stream>>>(
                d.n_rays, d.total_samples, m, rays_o, rays_d, t_starts, t_ends, noises, bits, next_loc, n_exceeded,
                ray_is_valid, rays_n_samples, rays_startidx, idcs, xyzs, dirs, dss, z_vals, coarse, sums, done, frontier,
                queue);
            if (queue != nullptr) NGP_CUDA_TRY(cudaMemsetAsync(queue, 0xff, sizeof(std::uint32_t), stream));
            const std::uint32_t nb = (d.n_rays + kScanRays - 1) / kScanRays;
            ray_scan_fit_kernel<<<nb, kScanRays, 0, stream>>>(d.n_rays, d.total_samples, sums, ray_is_valid,
                                                               rays_n_samples, rays_startidx, dss, next_loc, n_exceeded,
                                                               queue);
            march_write_kernel<<<write_grid, kWarpBlock, 0, stream>>>(d.n_rays, m, rays_o, rays_d, t_ends, bits, coarse,
                                                                      queue, rays_n_samples, rays_startidx, idcs, xyzs,
                                                                      dirs, dss, z_vals);
            count_launches(4);
        } else {
            march_rays_kernel<kMarchAlloc><<<grid, kThreadBlock, 0, stream>>>(
                d.n_rays, d.total_samples, m, rays_o, rays_d, t_starts, t_ends, noises, bits, next_loc, n_exceeded,
                ray_is_valid, rays_n_samples, rays_startidx, idcs, xyzs, dirs, dss, z_vals, coarse, nullptr, nullptr,
                nullptr, nullptr);
            count_launches(1);
        }
    }
    if (d.total_samples > 0) {
        zero_sample_tail_kernel<<<grid_for(d.total_samples, 256, 8), 256, 0, stream>>>(
            d.total_samples, next_loc, n_exceeded, idcs, xyzs, dirs, dss, z_vals);
        count_launches(1);
    }
    return launch_status();
}

// The training march (probe form) over the rays ray_list[0 .. *list_count), allocating from the
// counters as they stand (they are not reset, and the unwritten tail is not zeroed: the caller
// allocates more samples after this and finishes the buffers itself).  d.n_rays bounds the list.
int launch_march_rays_list(cudaStream_t stream, const MarchingDescriptor &d, const float *rays_o, const float *rays_d,
                           const float *t_starts, const float *t_ends, const float *noises, const std::uint8_t *bits,
                           std::uint32_t *next_loc, std::uint32_t *n_exceeded, bool *ray_is_valid,
                           std::uint32_t *rays_n_samples, std::uint32_t *rays_startidx, std::uint32_t *idcs, float *xyzs,
                           float *dirs, float *dss, float *z_vals, std::uint32_t *queue, const std::uint32_t *ray_list,
                           const std::uint32_t *list_count) {
    NGP_CHECK_ARG(d.K > 0 && d.G > 0 && d.diagonal_n_steps > 0, "march_rays: K, G and diagonal_n_steps must be positive");
    NGP_CHECK_ARG(d.G <= 1024 && (d.G & (d.G - 1)) == 0, "march_rays: G must be a power of two <= 1024 (Morton codes of other sizes exceed G^3)");
    NGP_CHECK_ARG(d.K <= 16, "march_rays: at most 16 cascades");
    NGP_CHECK_ARG(d.bound > 0.f && d.stepsize_portion >= 0.f, "march_rays: bound must be positive, stepsize_portion non-negative");
    NGP_CHECK_ARG(queue != nullptr && ray_list != nullptr && list_count != nullptr, "march_rays (list): queue, ray list and its count are required");
    NGP_CUDA_TRY(cudaMemsetAsync(queue, 0, sizeof(std::uint32_t), stream));
    const MarchParams m = make_params(d.diagonal_n_steps, d.K, d.G, d.bound, d.stepsize_portion);
    if (d.n_rays > 0) {
        const unsigned warps_needed = d.n_rays;   // a warp per listed ray, at most n_rays of them
        const unsigned blocks_needed = (warps_needed + kMarchBlock / 32 - 1) / (kMarchBlock / 32);
        const unsigned cap = (unsigned)sm_count() * (unsigned)g_march_blocks_per_sm.load(std::memory_order_relaxed);
        const unsigned grid = blocks_needed < cap ? blocks_needed : cap;
        march_rays_warp_kernel<<<grid, kMarchBlock, 0, stream>>>(
            d.n_rays, d.total_samples, m, rays_o, rays_d, t_starts, t_ends, noises, bits, next_loc, n_exceeded, queue,
            ray_is_valid, rays_n_samples, rays_startidx, idcs, xyzs, dirs, dss, z_vals, ray_list, list_count);
        count_launches(1);
    }
    return launch_status();
}

int launch_march_rays_inference(cudaStream_t stream, const MarchingInferenceDescriptor &d,
                                const float *rays_o, const float *rays_d, const float *t_starts,
                                const float *t_ends, const std::uint8_t *bits,
                                const std::uint32_t *next_ray_index_in, const bool *terminated,
                                const std::uint32_t *indices_in, std::uint32_t *next_ray_index,
                                std::uint32_t *indices_out, std::uint32_t *n_samples,
                                float *t_starts_out, float *xyzs, float *dss, float *z_vals) {
    NGP_CHECK_ARG(d.K > 0 && d.G > 0 && d.diagonal_n_steps > 0, "march_rays_inference: K, G and diagonal_n_steps must be positive");
    NGP_CHECK_ARG(d.G <= 1024 && (d.G & (d.G - 1)) == 0, "march_rays_inference: G must be a power of two <= 1024");
    NGP_CHECK_ARG(d.K <= 16, "march_rays_inference: at most 16 cascades");
    NGP_CHECK_ARG(d.bound > 0.f && d.stepsize_portion >= 0.f, "march_rays_inference: bound must be positive");
    copy_counter_kernel<<<1, 1, 0, stream>>>(next_ray_index_in, next_ray_index);
    count_launches(1);
    const MarchParams m = make_params(d.diagonal_n_steps, d.K, d.G, d.bound, d.stepsize_portion);
    if (d.n_rays > 0) {
        march_rays_inference_kernel<<<(d.n_rays + 255) / 256, 256, 0, stream>>>(
            d.n_total_rays, d.n_rays, d.march_steps_cap, m, rays_o, rays_d, t_starts, t_ends, bits,
            terminated, indices_in, next_ray_index, indices_out, n_samples, t_starts_out, xyzs, dss,
            z_vals);
        count_launches(1);
    }
    return launch_status();
}

int launch_march_rays_inference_inplace(cudaStream_t stream, const MarchingInferenceDescriptor &d, const float *rays_o,
                                        const float *rays_d, float *t_starts, const float *t_ends,
                                        const std::uint8_t *bits, const bool *terminated, std::uint32_t *indices,
                                        std::uint32_t *next_ray_index, std::uint32_t *n_samples,
                                        std::uint32_t *sample_start, std::uint32_t *sample_count, float *xyzs,
                                        float *dirs, float *dss, float *z_vals) {
    NGP_CHECK_ARG(d.K > 0 && d.K <= 16 && d.G > 0 && d.G <= 1024 && (d.G & (d.G - 1)) == 0 && d.diagonal_n_steps > 0,
                  "march_rays_inference: bad K, G or diagonal_n_steps");
    const bool compact = sample_start != nullptr;
    NGP_CHECK_ARG(!compact || (sample_count != nullptr && d.march_steps_cap <= kCompactMaxCap),
                  "march_rays_inference (compact): needs sample_count and march_steps_cap <= 16");
    const MarchParams m = make_params(d.diagonal_n_steps, d.K, d.G, d.bound, d.stepsize_portion);
    if (d.n_rays > 0) {
        const unsigned grid = (d.n_rays + 255) / 256;
        if (compact)
            march_rays_inference_inplace_kernel<true><<<grid, 256, 0, stream>>>(
                d.n_total_rays, d.n_rays, d.march_steps_cap, m, rays_o, rays_d, t_starts, t_ends, bits, terminated,
                indices, next_ray_index, n_samples, sample_start, sample_count, xyzs, dirs, dss, z_vals);
        else
            march_rays_inference_inplace_kernel<false><<<grid, 256, 0, stream>>>(
                d.n_total_rays, d.n_rays, d.march_steps_cap, m, rays_o, rays_d, t_starts, t_ends, bits, terminated,
                indices, next_ray_index, n_samples, nullptr, nullptr, xyzs, dirs, dss, z_vals);
        count_launches(1);
    }
    return launch_status();
}

int launch_morton3d(cudaStream_t stream, std::uint32_t n, const std::uint32_t *xyz, std::uint32_t *idcs) {
    if (n > 0) {
        morton3d_kernel<<<grid_for(n, 256, 8), 256, 0, stream>>>(n, xyz, idcs);
        count_launches(1);
    }
    return launch_status();
}

int launch_morton3d_invert(cudaStream_t stream, std::uint32_t n, const std::uint32_t *idcs, std::uint32_t *xyz) {
    if (n > 0) {
        morton3d_invert_kernel<<<grid_for(n, 256, 8), 256, 0, stream>>>(n, idcs, xyz);
        count_launches(1);
    }
    return launch_status();
}

}  // namespace ngp
