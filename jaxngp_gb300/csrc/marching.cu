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
#include "common.cuh"

namespace ngp {
namespace {

struct V3 {
    float x, y, z;
};

__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return min(max(v, lo), hi); }

// marching.cu:15-23
__device__ __forceinline__ float calc_ds(float t, float sp, float bound, float inv_G, std::uint32_t dns) {
    return clampf(t * sp, 2.0f * kSqrt3 * fminf(bound, 1.0f) / (float)dns, 2.0f * kSqrt3 * bound * inv_G);
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
};

// Loop caps.  A ray whose t_end is infinite (or so large that t + ds rounds back to t) would
// march forever; valid rays stay far below these caps (samples <= diagonal_n_steps * bound, empty
// voxels crossed <= 3 * G * K, steps inside one empty voxel <= bound * diag / (G * sqrt3)).
constexpr std::uint32_t kMaxMarchIters = 1u << 22;
constexpr std::uint32_t kMaxSkipIters = 1u << 20;

// marching.cu:79-98, :41-50, :174-176: is the cell under `pos` occupied?  Also returns the
// continuous grid position and the cascade's half-width for the empty-space skip.
__device__ __forceinline__ bool occupied_at(const MarchParams &m, V3 pos, float ds,
                                            const std::uint8_t *__restrict__ bits, V3 &g, float &mb) {
    std::uint32_t c0 = mip_from_xyz(pos, m.K), c1 = mip_from_ds(ds, m.G, m.K);
    std::uint32_t cascade = c0 > c1 ? c0 : c1;
    mb = fminf(scalbnf(1.0f, (int)cascade), m.bound);
    float Gf = (float)m.G;
    g.x = ((pos.x / mb + 1.0f) * 0.5f) * Gf;
    g.y = ((pos.y / mb + 1.0f) * 0.5f) * Gf;
    g.z = ((pos.z / mb + 1.0f) * 0.5f) * Gf;
    int Gi = (int)m.G - 1;
    std::uint32_t gx = (std::uint32_t)clampi((int)floorf(g.x), 0, Gi);
    std::uint32_t gy = (std::uint32_t)clampi((int)floorf(g.y), 0, Gi);
    std::uint32_t gz = (std::uint32_t)clampi((int)floorf(g.z), 0, Gi);
    std::uint32_t idx = cascade * (m.G * m.G * m.G) + morton3(gx, gy, gz);
    return (__ldg(bits + (idx >> 3)) >> (idx & 7u)) & 1u;
}

// marching.cu:182-189: advance past the empty voxel in whole steps.
__device__ __forceinline__ float skip_empty(const MarchParams &m, float t, V3 g, float mb, V3 pos,
                                            V3 d, V3 inv_d) {
    float nt = t + calc_ds(t, m.sp, m.bound, m.inv_G, m.dns);
    float nx = floorf((g.x + 0.5f) + 0.5f * copysignf(1.0f, d.x));
    float ny = floorf((g.y + 0.5f) + 0.5f * copysignf(1.0f, d.y));
    float nz = floorf((g.z + 0.5f) + 0.5f * copysignf(1.0f, d.z));
    float dx = (((nx * m.inv_G - 0.5f) * 2.0f) * mb - pos.x) * inv_d.x;
    float dy = (((ny * m.inv_G - 0.5f) * 2.0f) * mb - pos.y) * inv_d.y;
    float dz = (((nz * m.inv_G - 0.5f) * 2.0f) * mb - pos.z) * inv_d.z;
    float next_t = t + fmaxf(0.0f, fminf(dx, fminf(dy, dz)));
    for (std::uint32_t it = 0; nt < next_t && it < kMaxSkipIters; ++it) nt += calc_ds(nt, m.sp, m.bound, m.inv_G, m.dns);
    return nt;
}

__device__ __forceinline__ V3 at(V3 o, V3 d, float t) { return {o.x + t * d.x, o.y + t * d.y, o.z + t * d.z}; }

// ------------------------------------------------------------------------------- march_rays

// One thread per ray.  Pass 1 counts the ray's samples; the warp then allocates one contiguous
// slot range with a single atomic; pass 2 re-marches the ray writing its samples.
__global__ void __launch_bounds__(256) march_rays_kernel(
    std::uint32_t n_rays, std::uint32_t total_samples, MarchParams m,
    const float *__restrict__ rays_o, const float *__restrict__ rays_d,
    const float *__restrict__ t_starts, const float *__restrict__ t_ends,
    const float *__restrict__ noises, const std::uint8_t *__restrict__ bits,
    std::uint32_t *__restrict__ next_loc, std::uint32_t *__restrict__ n_exceeded,
    bool *__restrict__ ray_is_valid, std::uint32_t *__restrict__ rays_n_samples,
    std::uint32_t *__restrict__ rays_startidx, std::uint32_t *__restrict__ idcs,
    float *__restrict__ xyzs, float *__restrict__ dirs, float *__restrict__ dss,
    float *__restrict__ z_vals) {
    const std::uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in_range = i < n_rays;
    // marching.cu:135: a ray that starts after the sample buffer filled up is dropped.
    bool live = in_range && *((volatile std::uint32_t *)next_loc) < total_samples;
    V3 o{0, 0, 0}, d{1, 1, 1};
    float t0 = 0.f, t1 = 0.f, noise = 0.f;
    if (live) {
        o = {rays_o[i * 3 + 0], rays_o[i * 3 + 1], rays_o[i * 3 + 2]};
        d = {rays_d[i * 3 + 0], rays_d[i * 3 + 1], rays_d[i * 3 + 2]};
        t0 = t_starts[i];
        t1 = t_ends[i];
        noise = noises[i];
        live = t1 > t0;  // marching.cu:151
    }
    const V3 inv_d = {1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
    const float t_first = t0 + calc_ds(t0, m.sp, m.bound, m.inv_G, m.dns) * noise;

    std::uint32_t n = 0;
    if (live) {
        const float n_cap = (float)m.dns * m.bound;
        float t = t_first;
        for (std::uint32_t it = 0; (float)n < n_cap && t < t1 && it < kMaxMarchIters; ++it) {
            V3 pos = at(o, d, t);
            float ds = calc_ds(t, m.sp, m.bound, m.inv_G, m.dns);
            V3 g;
            float mb;
            if (occupied_at(m, pos, ds, bits, g, mb)) {
                ++n;
                t = t + ds;
            } else {
                t = skip_empty(m, t, g, mb, pos, d, inv_d);
            }
        }
    }

    // warp-aggregated slot allocation (marching.cu:205 does one atomic per ray)
    const std::uint32_t incl = warp_inclusive_scan(n);
    const std::uint32_t warp_total = __shfl_sync(0xffffffffu, incl, 31);
    std::uint32_t base = 0;
    if (lane_id() == 31 && warp_total > 0) base = atomicAdd(next_loc, warp_total);
    base = __shfl_sync(0xffffffffu, base, 31);
    const std::uint32_t start = base + incl - n;
    const bool fits = n > 0 && (std::uint64_t)start + n <= total_samples;
    const std::uint32_t over = warp_sum((n > 0 && !fits) ? n : 0u);
    if (lane_id() == 0 && over > 0) atomicAdd(n_exceeded, over);

    if (in_range) {
        ray_is_valid[i] = live && (n == 0 || fits);
        rays_n_samples[i] = fits ? n : 0u;
        rays_startidx[i] = fits ? start : 0u;
    }
    if (!fits) return;

    std::uint32_t *ri = idcs + start;
    float *rx = xyzs + (std::size_t)start * 3, *rd = dirs + (std::size_t)start * 3;
    float *rs = dss + start, *rz = z_vals + start;
    std::uint32_t k = 0;
    float t = t_first;
    for (std::uint32_t it = 0; k < n && t < t1 && it < kMaxMarchIters; ++it) {
        V3 pos = at(o, d, t);
        float ds = calc_ds(t, m.sp, m.bound, m.inv_G, m.dns);
        V3 g;
        float mb;
        if (occupied_at(m, pos, ds, bits, g, mb)) {
            ri[k] = i;
            rx[k * 3 + 0] = pos.x;
            rx[k * 3 + 1] = pos.y;
            rx[k * 3 + 2] = pos.z;
            rd[k * 3 + 0] = d.x;
            rd[k * 3 + 1] = d.y;
            rd[k * 3 + 2] = d.z;
            rs[k] = ds;
            rz[k] = t;
            ++k;
            t = t + ds;
        } else {
            t = skip_empty(m, t, g, mb, pos, d, inv_d);
        }
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
                float ds = calc_ds(t, m.sp, m.bound, m.inv_G, m.dns);
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
                float ds = calc_ds(t1, m.sp, m.bound, m.inv_G, m.dns);
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
    return m;
}

}  // namespace

// ----------------------------------------------------------------------------- launchers

int launch_march_rays(cudaStream_t stream, const MarchingDescriptor &d, const float *rays_o,
                      const float *rays_d, const float *t_starts, const float *t_ends,
                      const float *noises, const std::uint8_t *bits, std::uint32_t *next_loc,
                      std::uint32_t *n_exceeded, bool *ray_is_valid, std::uint32_t *rays_n_samples,
                      std::uint32_t *rays_startidx, std::uint32_t *idcs, float *xyzs, float *dirs,
                      float *dss, float *z_vals) {
    NGP_CHECK_ARG(d.K > 0 && d.G > 0 && d.diagonal_n_steps > 0, "march_rays: K, G and diagonal_n_steps must be positive");
    NGP_CHECK_ARG(d.G <= 1024 && (d.G & (d.G - 1)) == 0, "march_rays: G must be a power of two <= 1024 (Morton codes of other sizes exceed G^3)");
    NGP_CHECK_ARG(d.K <= 16, "march_rays: at most 16 cascades");
    NGP_CHECK_ARG(d.bound > 0.f && d.stepsize_portion >= 0.f, "march_rays: bound must be positive, stepsize_portion non-negative");
    NGP_CUDA_TRY(cudaMemsetAsync(next_loc, 0, sizeof(std::uint32_t), stream));
    NGP_CUDA_TRY(cudaMemsetAsync(n_exceeded, 0, sizeof(std::uint32_t), stream));
    const MarchParams m = make_params(d.diagonal_n_steps, d.K, d.G, d.bound, d.stepsize_portion);
    if (d.n_rays > 0) {
        march_rays_kernel<<<(d.n_rays + 255) / 256, 256, 0, stream>>>(
            d.n_rays, d.total_samples, m, rays_o, rays_d, t_starts, t_ends, noises, bits, next_loc,
            n_exceeded, ray_is_valid, rays_n_samples, rays_startidx, idcs, xyzs, dirs, dss, z_vals);
        count_launches(1);
    }
    if (d.total_samples > 0) {
        zero_sample_tail_kernel<<<grid_for(d.total_samples, 256, 8), 256, 0, stream>>>(
            d.total_samples, next_loc, n_exceeded, idcs, xyzs, dirs, dss, z_vals);
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
