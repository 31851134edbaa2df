// Learned proposal sampler for sm_103a: coarse occupancy blocks, per-ray occupied interval and
// sample-slot allocation, proposal bin points, inverse-CDF sampling and the proposal's
// log-density regression loss.  The reference has no proposal sampler; this is the project's own
// algorithm, restated for the tests in the CPU oracle (one rounding per float operation in the
// oracle's order: this file is built without FMA contraction).
//
// Training step with the proposal (per ray, R rays, a budget of S samples):
//   1. coarse DDA over blocks of 8^3 occupancy cells (grown by one cell): no occupied block ->
//      the ray is valid with no samples (it shows its background); else its interval [t_a, t_b]
//   2. a ray with an interval takes N_SAMPLES slots (one atomic per warp); rays past the budget
//      are invalid, as in march_rays (marching.cu:206-209 of the reference)
//   3. N_BINS points over the interval -> proposal field (hash grid + MLP, other files) -> log
//      densities -> N_SAMPLES stratified inverse-CDF samples written in march_rays' layout
//      (xyzs, dirs, dss, z_vals at rays_sample_startidx), so the field, the integrator and the
//      loss run unchanged
//   4. the proposal regresses the field's log density at the field's samples (loss kernel here)
#include "common.cuh"
#include "coarse.cuh"

namespace ngp {
namespace {

constexpr int kBins = 64;
constexpr float kEps = 1e-3f, kUnder = 2.0f;

__device__ __forceinline__ std::uint32_t expand_bits(std::uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

// coarse[cx + cy Gc + cz Gc^2] = any occupied fine cell in the block grown by one cell.
__global__ void coarse_grid_kernel(std::uint32_t G, const std::uint8_t *__restrict__ bits, std::uint8_t *__restrict__ coarse) {
    const std::uint32_t Gc = G / 8, n = Gc * Gc * Gc;
    const std::uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const int cx = (int)(c % Gc), cy = (int)((c / Gc) % Gc), cz = (int)(c / (Gc * Gc));
    const int lo[3] = {max(cx * 8 - 1, 0), max(cy * 8 - 1, 0), max(cz * 8 - 1, 0)};
    const int hi[3] = {min(cx * 8 + 8, (int)G - 1), min(cy * 8 + 8, (int)G - 1), min(cz * 8 + 8, (int)G - 1)};
    std::uint8_t any = 0;
    for (int z = lo[2]; z <= hi[2] && !any; ++z)
        for (int y = lo[1]; y <= hi[1] && !any; ++y)
            for (int x = lo[0]; x <= hi[0]; ++x) {
                const std::uint32_t m = expand_bits((std::uint32_t)x) | (expand_bits((std::uint32_t)y) << 1) |
                                        (expand_bits((std::uint32_t)z) << 2);
                if ((bits[m >> 3] >> (m & 7u)) & 1u) {
                    any = 1;
                    break;
                }
            }
    coarse[c] = any;
}

// Step 1-2: interval, slot allocation.  Slot j = startidx / spr of a fitting ray records the
// ray (ray_of_slot) and its interval (slot_ta, slot_tb).
__global__ void __launch_bounds__(256) proposal_rays_kernel(
    std::uint32_t n_rays, std::uint32_t total_samples, std::uint32_t spr, int Gc, float mb, const float *__restrict__ rays_o,
    const float *__restrict__ rays_d, const float *__restrict__ t_starts, const float *__restrict__ t_ends,
    const std::uint8_t *__restrict__ coarse, std::uint32_t *__restrict__ next_loc, std::uint32_t *__restrict__ n_exceeded,
    bool *__restrict__ ray_is_valid, std::uint32_t *__restrict__ rays_n_samples,
    std::uint32_t *__restrict__ rays_startidx, std::uint32_t *__restrict__ ray_of_slot, float *__restrict__ slot_ta,
    float *__restrict__ slot_tb) {
    const std::uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = r < n_rays;
    float ta = 0.f, tb = 0.f;
    bool hit = false;
    if (in)
        hit = coarse_ray_interval(rays_o[(std::size_t)r * 3 + 0], rays_o[(std::size_t)r * 3 + 1], rays_o[(std::size_t)r * 3 + 2],
                           rays_d[(std::size_t)r * 3 + 0], rays_d[(std::size_t)r * 3 + 1], rays_d[(std::size_t)r * 3 + 2],
                           t_starts[r], t_ends[r], coarse, Gc, mb, ta, tb);
    hit = hit && tb > ta;
    const std::uint32_t need = hit ? spr : 0u;
    const std::uint32_t incl = warp_inclusive_scan(need);
    const std::uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    std::uint32_t base = 0;
    if (lane_id() == 31)   // a warp without intervals reads the counter for its rays' validity
        base = total > 0 ? atomicAdd(next_loc, total) : *((volatile std::uint32_t *)next_loc);
    base = __shfl_sync(0xffffffffu, base, 31);
    const std::uint32_t start = base + incl - need;
    const bool fits = hit && (std::uint64_t)start + spr <= total_samples;
    const unsigned over = __ballot_sync(0xffffffffu, hit && !fits);
    if (lane_id() == 0 && over != 0u) atomicAdd(n_exceeded, (std::uint32_t)__popc(over) * spr);
    if (!in) return;
    if (!hit) {   // valid with no samples, unless taken up after the budget filled (marching.cu:135)
        ray_is_valid[r] = start < total_samples;
        rays_n_samples[r] = 0;
        rays_startidx[r] = 0;
        return;
    }
    ray_is_valid[r] = fits;
    rays_n_samples[r] = fits ? spr : 0u;
    rays_startidx[r] = fits ? start : 0u;
    if (fits) {
        const std::uint32_t j = start / spr;
        ray_of_slot[j] = r;
        slot_ta[j] = ta;
        slot_tb[j] = tb;
    }
}

// counts[0] = slots (fitting rays), counts[1] = bin points, counts[2] = samples.
__global__ void proposal_counts_kernel(std::uint32_t total_samples, std::uint32_t spr,
                                       const std::uint32_t *__restrict__ next_loc, std::uint32_t *__restrict__ counts) {
    const std::uint32_t slots = min(*next_loc / spr, total_samples / spr);
    counts[0] = slots;
    counts[1] = slots * kBins;
    counts[2] = slots * spr;
}

// Step 3a: bin centres of every slot's interval.
__global__ void __launch_bounds__(256) proposal_bin_points_kernel(
    const std::uint32_t *__restrict__ counts, const float *__restrict__ rays_o, const float *__restrict__ rays_d,
    const std::uint32_t *__restrict__ ray_of_slot, const float *__restrict__ slot_ta, const float *__restrict__ slot_tb,
    float *__restrict__ points) {
    const std::uint32_t n = counts[1];
    const std::size_t stride = (std::size_t)gridDim.x * blockDim.x;
    for (std::size_t p = (std::size_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += stride) {
        const std::uint32_t j = (std::uint32_t)(p / kBins), i = (std::uint32_t)(p % kBins);
        const std::uint32_t r = ray_of_slot[j];
        const float ta = slot_ta[j], delta = (slot_tb[j] - ta) / (float)kBins;
        const float c = ta + ((float)i + 0.5f) * delta;
        points[p * 3 + 0] = rays_o[(std::size_t)r * 3 + 0] + c * rays_d[(std::size_t)r * 3 + 0];
        points[p * 3 + 1] = rays_o[(std::size_t)r * 3 + 1] + c * rays_d[(std::size_t)r * 3 + 1];
        points[p * 3 + 2] = rays_o[(std::size_t)r * 3 + 2] + c * rays_d[(std::size_t)r * 3 + 2];
    }
}

__device__ __forceinline__ std::uint64_t splitmix(std::uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Step 3c: a warp per slot turns the bins' log densities into spr samples.  Lane l holds bins
// 2l and 2l+1; the exclusive prefix of the densities (transmittance) and the CDF are warp scans;
// every lane then inverts the CDF (binary search in shared memory) for the edges of its samples
// k = l, l + 32, ...: e_0 = t_a, e_k = F^-1(((k - 1/2) + xi_k) / spr) (0 < k < spr), e_spr = t_b,
// sample k at the middle of [e_k, e_k+1], standing for that interval.
constexpr int kSampleWarps = 4;

__device__ __forceinline__ float warp_inclusive_scan_f(float v) {
    const unsigned lane = lane_id();
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const float t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= (unsigned)o) v += t;
    }
    return v;
}

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float proposal_edge(int k, std::uint32_t spr, float ta, float tb, float delta, bool perturb,
                                               std::uint64_t seed, std::uint32_t r, const float *cdf, const float *pdf) {
    if (k <= 0) return ta;
    if (k >= (int)spr) return tb;
    float xi = 0.5f;
    if (perturb)
        xi = (float)(splitmix(seed ^ ((std::uint64_t)r * spr + (std::uint64_t)k) * 0x2545F4914F6CDD1Dull) >> 40) *
             (1.0f / 16777216.0f);
    const float u = (((float)k - 0.5f) + xi) / (float)spr;
    int lo = 0, hi = kBins - 1;   // first bin whose inclusive CDF exceeds u (the last bin if none)
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (u < cdf[mid]) hi = mid;
        else lo = mid + 1;
    }
    const float c_lo = lo > 0 ? cdf[lo - 1] : 0.f;
    const float frac = fminf(fmaxf((u - c_lo) / pdf[lo], 0.f), 1.f);
    return ta + ((float)lo + frac) * delta;
}

__global__ void __launch_bounds__(32 * kSampleWarps) proposal_sample_kernel(
    const std::uint32_t *__restrict__ counts, std::uint32_t spr, float mix, int perturb, std::uint64_t seed,
    const float *__restrict__ rays_o,
    const float *__restrict__ rays_d, const std::uint32_t *__restrict__ ray_of_slot, const float *__restrict__ slot_ta,
    const float *__restrict__ slot_tb, const float *__restrict__ x_bins, std::uint32_t *__restrict__ idcs,
    float *__restrict__ xyzs, float *__restrict__ dirs, float *__restrict__ dss, float *__restrict__ z_vals,
    const std::uint8_t *__restrict__ slot_flag, std::uint32_t total_samples, std::uint32_t *__restrict__ next_loc,
    std::uint32_t *__restrict__ n_exceeded, bool *__restrict__ ray_is_valid, std::uint32_t *__restrict__ rays_n_samples,
    std::uint32_t *__restrict__ rays_startidx) {
    __shared__ float cdf_s[kSampleWarps][kBins], pdf_s[kSampleWarps][kBins];
    float *cdf = cdf_s[threadIdx.x >> 5], *pdf = pdf_s[threadIdx.x >> 5];
    const unsigned lane = lane_id();
    const std::uint32_t n_slots = counts[0];
    const std::uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, n_warps = (gridDim.x * blockDim.x) >> 5;
    for (std::uint32_t j = warp0; j < n_slots; j += n_warps) {
        const std::uint32_t r = ray_of_slot[j];
        std::size_t s_base = (std::size_t)j * spr;
        if (next_loc != nullptr) {
            // allocating form: flagged slots were marched; the others take spr samples here
            if (slot_flag[j]) continue;
            std::uint32_t start = 0;
            if (lane == 0) {
                start = atomicAdd(next_loc, spr);
                const bool fits = (std::uint64_t)start + spr <= total_samples;
                if (!fits) atomicAdd(n_exceeded, spr);
                ray_is_valid[r] = fits;
                rays_n_samples[r] = fits ? spr : 0u;
                rays_startidx[r] = fits ? start : 0u;
            }
            start = __shfl_sync(0xffffffffu, start, 0);
            if ((std::uint64_t)start + spr > total_samples) continue;
            s_base = start;
        }
        const float ta = slot_ta[j], tb = slot_tb[j];
        const float delta = (tb - ta) / (float)kBins;
        const float2 xv = reinterpret_cast<const float2 *>(x_bins + (std::size_t)j * kBins)[lane];
        const float s0 = expf(fminf(fmaxf(xv.x, -15.f), 15.f)), s1 = expf(fminf(fmaxf(xv.y, -15.f), 15.f));
        const float pair = s0 + s1;
        const float acc0 = warp_inclusive_scan_f(pair) - pair, acc1 = acc0 + s0;
        const float w0 = expf(-(delta * acc0)) * -expm1f(-(s0 * delta));
        const float w1 = expf(-(delta * acc1)) * -expm1f(-(s1 * delta));
        const float W = warp_sum_f(w0 + w1);
        const float p0 = (1.0f - mix) * (W > 0.f ? w0 / W : 1.0f / (float)kBins) + mix / (float)kBins;
        const float p1 = (1.0f - mix) * (W > 0.f ? w1 / W : 1.0f / (float)kBins) + mix / (float)kBins;
        const float pp = p0 + p1;
        const float ci = warp_inclusive_scan_f(pp);
        cdf[2 * lane] = ci - pp + p0;
        cdf[2 * lane + 1] = ci;
        pdf[2 * lane] = p0;
        pdf[2 * lane + 1] = p1;
        __syncwarp();
        const float o[3] = {rays_o[(std::size_t)r * 3 + 0], rays_o[(std::size_t)r * 3 + 1], rays_o[(std::size_t)r * 3 + 2]};
        const float d[3] = {rays_d[(std::size_t)r * 3 + 0], rays_d[(std::size_t)r * 3 + 1], rays_d[(std::size_t)r * 3 + 2]};
        for (int k = (int)lane; k < (int)spr; k += 32) {
            const float e_lo = proposal_edge(k, spr, ta, tb, delta, perturb != 0, seed, r, cdf, pdf);
            const float e_hi = proposal_edge(k + 1, spr, ta, tb, delta, perturb != 0, seed, r, cdf, pdf);
            const float t = (e_lo + e_hi) * 0.5f;
            const std::size_t s = s_base + k;
            idcs[s] = r;
            xyzs[s * 3 + 0] = o[0] + t * d[0];
            xyzs[s * 3 + 1] = o[1] + t * d[1];
            xyzs[s * 3 + 2] = o[2] + t * d[2];
            dirs[s * 3 + 0] = d[0];
            dirs[s * 3 + 1] = d[1];
            dirs[s * 3 + 2] = d[2];
            z_vals[s] = t;
            dss[s] = e_hi - e_lo;
        }
        __syncwarp();
    }
}

// Fallback test (a warp per slot, lane l holding bins 2l and 2l + 1).  The occupancy grid says
// where the field's density is at least the grid's threshold; where the proposal's density is
// below that, the proposal misses mass the field has.  The transmittance it misses there is
// sum over occupied bins i of T_i (1 - exp(-max(0, threshold - sigma_i) delta)), T_i the
// proposal's transmittance before bin i.  A slot whose ray misses more than kMissLimit is flagged
// and its ray appended to the fallback list, for the occupancy-grid march.
constexpr float kMissLimit = 0.01f;

__global__ void __launch_bounds__(32 * kSampleWarps) proposal_judge_kernel(
    const std::uint32_t *__restrict__ counts, std::uint32_t G, float mb, const float *__restrict__ threshold,
    const float *__restrict__ rays_o, const float *__restrict__ rays_d, const std::uint32_t *__restrict__ ray_of_slot,
    const float *__restrict__ slot_ta, const float *__restrict__ slot_tb, const float *__restrict__ x_bins,
    const std::uint8_t *__restrict__ bits, std::uint8_t *__restrict__ slot_flag, std::uint32_t *__restrict__ fb_rays,
    std::uint32_t *__restrict__ fb_count, std::uint32_t *__restrict__ fb_total) {
    const unsigned lane = lane_id();
    const std::uint32_t n_slots = counts[0];
    const float thr = *threshold;
    const float Gf = (float)G;
    const int Gi = (int)G - 1;
    const std::uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, n_warps = (gridDim.x * blockDim.x) >> 5;
    for (std::uint32_t j = warp0; j < n_slots; j += n_warps) {
        const std::uint32_t r = ray_of_slot[j];
        const float ta = slot_ta[j], tb = slot_tb[j];
        const float delta = (tb - ta) / (float)kBins;
        const float2 xv = reinterpret_cast<const float2 *>(x_bins + (std::size_t)j * kBins)[lane];
        const float s[2] = {expf(fminf(fmaxf(xv.x, -15.f), 15.f)), expf(fminf(fmaxf(xv.y, -15.f), 15.f))};
        const float acc0 = warp_inclusive_scan_f(s[0] + s[1]) - (s[0] + s[1]);
        const float acc[2] = {acc0, acc0 + s[0]};
        const float o[3] = {rays_o[(std::size_t)r * 3 + 0], rays_o[(std::size_t)r * 3 + 1], rays_o[(std::size_t)r * 3 + 2]};
        const float d[3] = {rays_d[(std::size_t)r * 3 + 0], rays_d[(std::size_t)r * 3 + 1], rays_d[(std::size_t)r * 3 + 2]};
        float miss = 0.f;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const float t = ta + ((float)(2 * lane + h) + 0.5f) * delta;
            std::uint32_t c[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const float g = (((o[a] + t * d[a]) / mb + 1.0f) * 0.5f) * Gf;
                c[a] = (std::uint32_t)min(max((int)floorf(g), 0), Gi);
            }
            const std::uint32_t m = expand_bits(c[0]) | (expand_bits(c[1]) << 1) | (expand_bits(c[2]) << 2);
            const bool occ = (__ldg(bits + (m >> 3)) >> (m & 7u)) & 1u;
            if (occ && s[h] < thr) miss += expf(-(delta * acc[h])) * -expm1f(-((thr - s[h]) * delta));
        }
        miss = warp_sum_f(miss);
        if (lane == 0) {
            const bool fb = miss > kMissLimit;
            slot_flag[j] = fb ? 1 : 0;
            if (fb) {
                fb_rays[atomicAdd(fb_count, 1u)] = r;
                atomicAdd(fb_total, 1u);
            }
        }
    }
}

// counts[2] = the samples written ([0, next_loc - n_exceeded), capped at the budget); the slots
// past it are zeroed (as march_rays does).
__global__ void proposal_finish_kernel(std::uint32_t total_samples, const std::uint32_t *__restrict__ next_loc,
                                       const std::uint32_t *__restrict__ n_exceeded, std::uint32_t *__restrict__ counts,
                                       std::uint32_t *__restrict__ idcs, float *__restrict__ xyzs, float *__restrict__ dirs,
                                       float *__restrict__ dss, float *__restrict__ z_vals) {
    std::uint32_t used = *next_loc - *n_exceeded;
    if (used > total_samples) used = total_samples;
    if (blockIdx.x == 0 && threadIdx.x == 0) counts[2] = used;
    const std::size_t stride = (std::size_t)gridDim.x * blockDim.x;
    for (std::size_t q = used + (std::size_t)blockIdx.x * blockDim.x + threadIdx.x; q < total_samples; q += stride) {
        idcs[q] = 0;
        dss[q] = 0.f;
        z_vals[q] = 0.f;
        xyzs[q * 3 + 0] = 0.f;
        xyzs[q * 3 + 1] = 0.f;
        xyzs[q * 3 + 2] = 0.f;
        dirs[q * 3 + 0] = 0.f;
        dirs[q * 3 + 1] = 0.f;
        dirs[q * 3 + 2] = 0.f;
    }
}

// Step 4: dL/dx of the log-density regression over the first counts[count_index] points (or n
// when counts is NULL): L = sum w (x - log(sigma + eps))^2 / n with w = kUnder below the target.
// sigma is read with a stride (4 for drgbs rows).  loss[0] accumulates the sum.
__global__ void __launch_bounds__(256) proposal_loss_kernel(
    std::uint32_t n_max, const std::uint32_t *__restrict__ counts, int count_index, const float *__restrict__ x,
    const float *__restrict__ sigma, int sigma_stride, float *__restrict__ dL_dx, float *__restrict__ loss) {
    const std::uint32_t n = counts != nullptr ? min(n_max, counts[count_index]) : n_max;
    const float inv_n = n > 0 ? 1.0f / (float)n : 0.f;
    const std::uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (i < n) {
        const float y = logf(sigma[(std::size_t)i * sigma_stride] + kEps);
        const float res = x[i] - y;
        const float w = res < 0.f ? kUnder : 1.0f;
        dL_dx[i] = 2.0f * w * res * inv_n;
        l = w * res * res;
    } else if (i < n_max) {
        dL_dx[i] = 0.f;
    }
    l = warp_sum(l);
    if (lane_id() == 0 && l != 0.f) atomicAdd(loss, l);
}

}  // namespace

// ------------------------------------------------------------------------------- launchers

int launch_proposal_coarse(cudaStream_t stream, std::uint32_t G, const std::uint8_t *bits, std::uint8_t *coarse) {
    NGP_CHECK_ARG(G >= 8 && G % 8 == 0 && G <= 1024, "proposal: G must be a multiple of 8 in [8, 1024]");
    const std::uint32_t n = (G / 8) * (G / 8) * (G / 8);
    coarse_grid_kernel<<<(n + 127) / 128, 128, 0, stream>>>(G, bits, coarse);
    count_launches(1);
    return launch_status();
}

int launch_proposal_rays(cudaStream_t stream, std::uint32_t n_rays, std::uint32_t total_samples, std::uint32_t spr,
                         std::uint32_t G,
                         float bound, const float *rays_o, const float *rays_d, const float *t_starts,
                         const float *t_ends, const std::uint8_t *coarse, std::uint32_t *next_loc,
                         std::uint32_t *n_exceeded, bool *valid, std::uint32_t *n_samples, std::uint32_t *startidx,
                         std::uint32_t *ray_of_slot, float *slot_ta, float *slot_tb, std::uint32_t *counts) {
    NGP_CHECK_ARG(G >= 8 && G % 8 == 0 && G <= 1024, "proposal: G must be a multiple of 8 in [8, 1024]");
    NGP_CHECK_ARG(bound > 0.f, "proposal: bound must be positive");
    NGP_CHECK_ARG(spr >= 1 && spr <= 1024, "proposal: samples_per_ray must be in [1, 1024]");
    NGP_CUDA_TRY(cudaMemsetAsync(next_loc, 0, sizeof(std::uint32_t), stream));
    NGP_CUDA_TRY(cudaMemsetAsync(n_exceeded, 0, sizeof(std::uint32_t), stream));
    if (n_rays > 0) {
        proposal_rays_kernel<<<(n_rays + 255) / 256, 256, 0, stream>>>(
            n_rays, total_samples, spr, (int)(G / 8), fminf(1.0f, bound), rays_o, rays_d, t_starts, t_ends, coarse, next_loc,
            n_exceeded, valid, n_samples, startidx, ray_of_slot, slot_ta, slot_tb);
        count_launches(1);
    }
    proposal_counts_kernel<<<1, 1, 0, stream>>>(total_samples, spr, next_loc, counts);
    count_launches(1);
    return launch_status();
}

int launch_proposal_bin_points(cudaStream_t stream, std::uint32_t max_slots, const std::uint32_t *counts,
                               const float *rays_o, const float *rays_d, const std::uint32_t *ray_of_slot,
                               const float *slot_ta, const float *slot_tb, float *points) {
    if (max_slots > 0) {
        proposal_bin_points_kernel<<<grid_for((std::size_t)max_slots * kBins, 256, 8), 256, 0, stream>>>(
            counts, rays_o, rays_d, ray_of_slot, slot_ta, slot_tb, points);
        count_launches(1);
    }
    return launch_status();
}

int launch_proposal_sample(cudaStream_t stream, std::uint32_t max_slots, const std::uint32_t *counts, std::uint32_t spr,
                           float mix, bool perturb,
                           std::uint64_t seed, const float *rays_o, const float *rays_d,
                           const std::uint32_t *ray_of_slot, const float *slot_ta, const float *slot_tb,
                           const float *x_bins, std::uint32_t *idcs, float *xyzs, float *dirs, float *dss,
                           float *z_vals) {
    NGP_CHECK_ARG(mix >= 0.f && mix <= 1.f, "proposal: mix must be in [0, 1]");
    if (max_slots > 0) {
        const unsigned want = (max_slots + kSampleWarps - 1) / kSampleWarps;
        proposal_sample_kernel<<<grid_for(want, 1, 16), 32 * kSampleWarps, 0, stream>>>(
            counts, spr, mix, perturb ? 1 : 0, seed, rays_o, rays_d, ray_of_slot, slot_ta, slot_tb, x_bins, idcs, xyzs, dirs, dss,
            z_vals, nullptr, 0u, nullptr, nullptr, nullptr, nullptr, nullptr);
        count_launches(1);
    }
    return launch_status();
}

int launch_proposal_judge(cudaStream_t stream, std::uint32_t max_slots, const std::uint32_t *counts, std::uint32_t G,
                          float bound, const float *threshold, const float *rays_o, const float *rays_d,
                          const std::uint32_t *ray_of_slot, const float *slot_ta, const float *slot_tb,
                          const float *x_bins, const std::uint8_t *bits, std::uint8_t *slot_flag, std::uint32_t *fb_rays,
                          std::uint32_t *fb_count, std::uint32_t *fb_total) {
    NGP_CHECK_ARG(G >= 8 && G <= 1024 && (G & (G - 1)) == 0, "proposal judge: G must be a power of two in [8, 1024]");
    NGP_CHECK_ARG(bound > 0.f, "proposal judge: bound must be positive");
    NGP_CUDA_TRY(cudaMemsetAsync(fb_count, 0, sizeof(std::uint32_t), stream));
    if (max_slots > 0) {
        const unsigned want = (max_slots + kSampleWarps - 1) / kSampleWarps;
        proposal_judge_kernel<<<grid_for(want, 1, 16), 32 * kSampleWarps, 0, stream>>>(
            counts, G, fminf(1.0f, bound), threshold, rays_o, rays_d, ray_of_slot, slot_ta, slot_tb, x_bins, bits, slot_flag,
            fb_rays, fb_count, fb_total);
        count_launches(1);
    }
    return launch_status();
}

// The allocating form: after the fallback rays were marched (allocating from next_loc /
// n_exceeded), every unflagged slot takes spr samples from the same counters; counts[2] becomes
// the samples written and the rest of the buffers is zeroed.
int launch_proposal_sample_alloc(cudaStream_t stream, std::uint32_t max_slots, std::uint32_t total_samples,
                                 std::uint32_t *counts, std::uint32_t spr, float mix, bool perturb, std::uint64_t seed,
                                 const float *rays_o, const float *rays_d, const std::uint32_t *ray_of_slot,
                                 const float *slot_ta, const float *slot_tb, const float *x_bins,
                                 const std::uint8_t *slot_flag, std::uint32_t *next_loc, std::uint32_t *n_exceeded,
                                 std::uint32_t *idcs, float *xyzs, float *dirs, float *dss, float *z_vals, bool *valid,
                                 std::uint32_t *n_samples, std::uint32_t *startidx) {
    NGP_CHECK_ARG(mix >= 0.f && mix <= 1.f, "proposal: mix must be in [0, 1]");
    if (max_slots > 0) {
        const unsigned want = (max_slots + kSampleWarps - 1) / kSampleWarps;
        proposal_sample_kernel<<<grid_for(want, 1, 16), 32 * kSampleWarps, 0, stream>>>(
            counts, spr, mix, perturb ? 1 : 0, seed, rays_o, rays_d, ray_of_slot, slot_ta, slot_tb, x_bins, idcs, xyzs, dirs, dss,
            z_vals, slot_flag, total_samples, next_loc, n_exceeded, valid, n_samples, startidx);
        count_launches(1);
    }
    proposal_finish_kernel<<<grid_for(total_samples > 0 ? total_samples : 1, 256, 8), 256, 0, stream>>>(
        total_samples, next_loc, n_exceeded, counts, idcs, xyzs, dirs, dss, z_vals);
    count_launches(1);
    return launch_status();
}

int launch_proposal_loss(cudaStream_t stream, std::uint32_t n_max, const std::uint32_t *counts, int count_index,
                         const float *x, const float *sigma, int sigma_stride, float *dL_dx, float *loss) {
    NGP_CHECK_ARG(count_index >= 0 && count_index < 3 && sigma_stride >= 1, "proposal loss: bad count index or stride");
    if (n_max > 0) {
        proposal_loss_kernel<<<(n_max + 255) / 256, 256, 0, stream>>>(n_max, counts, count_index, x, sigma,
                                                                       sigma_stride, dL_dx, loss);
        count_launches(1);
    }
    return launch_status();
}

}  // namespace ngp
