// Volume integrator for sm_103a: forward, backward and the inference continuation.
//
// Replaces volume-rendering-jax/lib/impl/integrating.cu (integrate_rays :24-104,
// integrate_rays_backward :106-240, integrate_rays_inference :242-322) behind the same ABI.
// Per ray the arithmetic is the reference's, in its order.  The opacity uses the accurate expf
// where the reference calls the __expf intrinsic: for small sigma*ds, 1 - __expf(-x) carries a
// relative error of up to ~1e-3 (the intrinsic's absolute error over x), which is enough to move
// a ray's early-termination step; expf keeps alpha within a few ulp of the exact value, the
// reading of the reference's source under an exact exponential (its CPU build in the tests).
//
// Differences in structure: no thread returns before the block-wide counter reduction (the
// reference returns early at :45/:263 and then reaches __syncthreads at :100/:318 with part of
// the block); counters are reduced per warp with shuffles and added with one atomic per warp;
// outputs beyond a ray's early-termination point are written as zeros by the ray itself, so the
// forward and inference launchers need no output memsets.
#include "common.cuh"

namespace ngp {
namespace {

// Per-ray sample ranges are clamped to the sample buffer, so malformed index arrays cannot make
// a thread read or write outside it.
__device__ __forceinline__ std::uint32_t clamp_range(std::uint32_t s, std::uint32_t n, std::uint32_t total) {
    return s >= total ? 0u : min(n, total - s);
}

// ---- integrate_rays (:24-104) and integrate_rays_backward (:106-240): a warp per ray with samples
//
// Warp w of W takes the rays w, w + W, w + 2W, ... 32 at a time: each lane finishes its own ray
// if it has no samples (the prediction is the background), and the warp then runs its rays with
// samples one after another, each as segments of 32 samples (lane = sample; loads and stores
// coalesced).  The interleaving spreads rays with samples over the warps however they cluster in
// the batch (a training batch's are a prefix of it).  The transmittance
// before each sample comes from a warp product scan of 1 - alpha, colour and depth sums from warp
// reductions (the backward's running sums from warp sum scans), carried from segment to segment;
// a sample counts while the transmittance before it is above 1e-4, which selects a prefix of the
// segment (the product never grows).  A thread per ray, as in the reference, walks a long ray's
// samples one dependent load after another.
//
// Products and sums formed in tree order differ from the reference's left-to-right order by a
// few ulps, which leaves colours within float rounding but could move the 1e-4 decision of a
// sample whose transmittance lies within those ulps of it.  So every decision is checked against
// a bound on the two products' difference (each is within (k + 1) roundings of the exact product
// after k factors); a ray with any decision inside the bound is run again by one lane in the
// reference's order.  Sample counts, `measured` and the terminated/background choice are then the
// reference's exactly.

// |T_tree - T_serial| <= thr * tol(k) when both are products of the same k factors.
__device__ __forceinline__ float decision_tol(std::uint32_t k) { return (float)(4u * (k + 2u)) * 5.9604645e-8f; }

__device__ __forceinline__ float warp_prod_incl(float v, unsigned lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const float t = __shfl_up_sync(0xffffffffu, v, o);
        if ((int)lane >= o) v *= t;
    }
    return v;
}

__device__ __forceinline__ float warp_sum_incl(float v, unsigned lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const float t = __shfl_up_sync(0xffffffffu, v, o);
        if ((int)lane >= o) v += t;
    }
    return v;
}

__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// One ray in the reference's order (one thread): colour/depth (rgbd), transmittance, samples used.
__device__ __forceinline__ std::uint32_t forward_serial(const float *rd, const float *rz, const float4 *rc, std::uint32_t n,
                                                        float4 &sums, float &T_out) {
    float depth = 0.f, T = 1.f, r = 0.f, g = 0.f, b = 0.f;
    std::uint32_t k = 0;
    for (; T > kTThreshold && k < n; ++k) {
        const float4 c = rc[k];
        const float alpha = 1.f - expf(-c.x * rd[k]);
        const float w = T * alpha;
        r += w * c.y;
        g += w * c.z;
        b += w * c.w;
        depth += w * rz[k];
        T *= 1.f - alpha;
    }
    sums = make_float4(r, g, b, depth);
    T_out = T;
    return k;
}

// The same ray by the whole warp (segments, scans).  Returns false when a decision fell within the
// tree/serial bound (every lane returns the same); the outputs are then unset.
__device__ __forceinline__ bool forward_warp(const float *rd, const float *rz, const float4 *rc, std::uint32_t n,
                                             unsigned lane, float4 &sums, float &T_out, std::uint32_t &used_out) {
    float T = 1.f, r = 0.f, g = 0.f, b = 0.f, dep = 0.f;
    std::uint32_t used = 0;
    for (std::uint32_t base = 0; base < n; base += 32) {
        const std::uint32_t cnt = min(32u, n - base);
        const bool in = lane < cnt;
        float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
        float dt = 0.f, z = 0.f;
        if (in) {
            c = rc[base + lane];
            dt = rd[base + lane];
            z = rz[base + lane];
        }
        const float a = in ? 1.f - expf(-c.x * dt) : 0.f;
        const float P = warp_prod_incl(1.f - a, lane);
        const float Pup = __shfl_up_sync(0xffffffffu, P, 1);
        const float Tq = T * (lane == 0 ? 1.f : Pup);
        const bool amb = in && fabsf(Tq - kTThreshold) <= kTThreshold * decision_tol(used + lane);
        if (__any_sync(0xffffffffu, amb)) return false;
        const bool use = in && Tq > kTThreshold;
        const std::uint32_t nu = __popc(__ballot_sync(0xffffffffu, use));
        const float w = use ? Tq * a : 0.f;
        r += warp_sumf(w * c.y);
        g += warp_sumf(w * c.z);
        b += warp_sumf(w * c.w);
        dep += warp_sumf(w * z);
        const float Pend = __shfl_sync(0xffffffffu, P, nu > 0 ? (int)nu - 1 : 0);
        if (nu > 0) T *= Pend;
        used += nu;
        if (nu < cnt || !(T > kTThreshold)) break;
    }
    if (fabsf(T - kTThreshold) <= kTThreshold * decision_tol(used)) return false;   // terminated or not
    sums = make_float4(r, g, b, dep);
    T_out = T;
    used_out = used;
    return true;
}

__device__ __forceinline__ float4 finish_rgbd(float4 sums, float T, float bg0, float bg1, float bg2) {
    if (T <= kTThreshold) {
        const float id = 1.f / (1.f - T);
        return make_float4(sums.x * id, sums.y * id, sums.z * id, sums.w * id);
    }
    return make_float4(sums.x + T * bg0, sums.y + T * bg1, sums.z + T * bg2, sums.w);
}

constexpr int kIntWarps = 8;   // warps per block of the warp-per-ray integrators

__global__ void __launch_bounds__(32 * kIntWarps) integrate_rays_kernel(
    std::uint32_t n_rays, std::uint32_t total_samples, const std::uint32_t *__restrict__ startidx,
    const std::uint32_t *__restrict__ n_samples, const float *__restrict__ bgs,
    const float *__restrict__ dss, const float *__restrict__ z_vals,
    const float *__restrict__ drgbs, std::uint32_t *__restrict__ measured,
    float *__restrict__ final_rgbds, float *__restrict__ final_opacities) {
    const unsigned lane = lane_id();
    const std::uint64_t W = (gridDim.x * blockDim.x) >> 5, w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    std::uint32_t used_total = 0;   // lane 0's tally for its warp
    for (std::uint64_t j0 = 0; w + j0 * W < n_rays; j0 += 32) {
        const std::uint64_t ii = w + (j0 + lane) * W;
        const std::uint32_t i = ii < n_rays ? (std::uint32_t)ii : 0xffffffffu;
        std::uint32_t s = 0, n = 0;
        if (ii < n_rays) {
            s = startidx[i];
            n = clamp_range(s, n_samples[i], total_samples);
            if (n == 0) {   // T = 1: the background
                final_opacities[i] = 0.f;
                reinterpret_cast<float4 *>(final_rgbds)[i] = make_float4(bgs[i * 3 + 0], bgs[i * 3 + 1], bgs[i * 3 + 2], 0.f);
            }
        }
        unsigned heavy = __ballot_sync(0xffffffffu, n > 0u);
        while (heavy != 0u) {
            const int src = __ffs(heavy) - 1;
            heavy &= heavy - 1u;
            const std::uint32_t ray = __shfl_sync(0xffffffffu, i, src);
            const std::uint32_t rs = __shfl_sync(0xffffffffu, s, src), rn = __shfl_sync(0xffffffffu, n, src);
            const float *rd = dss + rs, *rz = z_vals + rs;
            const float4 *rc = reinterpret_cast<const float4 *>(drgbs) + rs;
            float4 sums;
            float T;
            std::uint32_t used = 0;
            const bool fast = forward_warp(rd, rz, rc, rn, lane, sums, T, used);
            if (lane == 0) {
                if (!fast) used = forward_serial(rd, rz, rc, rn, sums, T);
                final_opacities[ray] = 1.f - T;
                reinterpret_cast<float4 *>(final_rgbds)[ray] =
                    finish_rgbd(sums, T, bgs[ray * 3 + 0], bgs[ray * 3 + 1], bgs[ray * 3 + 2]);
                used_total += used;
            }
        }
    }
    if (lane == 0 && used_total > 0) atomicAdd(measured, used_total);
}

// FP64 checker of integrate_rays (not used by any training or rendering path): the same loop --
// alpha = 1 - exp(-sigma ds), w = T alpha, colour and depth sums, T *= 1 - alpha, stop once
// T <= 1e-4, normalise a terminated ray by its opacity, else add T bg -- evaluated in double on the
// float inputs widened exactly.  It states the error of the float integrators (and of everything
// that feeds them) at full batch sizes.  Outputs per ray: colour and depth, the transmittance
// after the last composited sample, and the number of samples composited (a ray whose float and
// double transmittances cross 1e-4 at different samples composites different counts).
__global__ void __launch_bounds__(256) integrate_rays_fp64_kernel(
    std::uint32_t n_rays, std::uint32_t total_samples, const std::uint32_t *__restrict__ startidx,
    const std::uint32_t *__restrict__ n_samples, const float *__restrict__ bgs,
    const float *__restrict__ dss, const float *__restrict__ z_vals, const float *__restrict__ drgbs,
    double *__restrict__ rgbds, double *__restrict__ trans, std::uint32_t *__restrict__ used) {
    const std::uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_rays) return;
    const std::uint32_t s = startidx[i], n = clamp_range(s, n_samples[i], total_samples);
    const float *rd = dss + s, *rz = z_vals + s;
    const float4 *rc = reinterpret_cast<const float4 *>(drgbs) + s;
    double depth = 0.0, T = 1.0, r = 0.0, g = 0.0, b = 0.0;
    std::uint32_t k = 0;
    for (; T > (double)kTThreshold && k < n; ++k) {
        const float4 c = rc[k];
        const double alpha = 1.0 - exp(-(double)c.x * (double)rd[k]);
        const double w = T * alpha;
        r += w * (double)c.y;
        g += w * (double)c.z;
        b += w * (double)c.w;
        depth += w * (double)rz[k];
        T *= 1.0 - alpha;
    }
    double *o = rgbds + (std::size_t)i * 4;
    if (T <= (double)kTThreshold) {
        const double opacity = 1.0 - T;
        o[0] = r / opacity, o[1] = g / opacity, o[2] = b / opacity, o[3] = depth / opacity;
    } else {
        o[0] = r + T * (double)bgs[i * 3 + 0], o[1] = g + T * (double)bgs[i * 3 + 1];
        o[2] = b + T * (double)bgs[i * 3 + 2], o[3] = depth;
    }
    trans[i] = T;
    used[i] = k;
}

// kExact = false: the reference's gradient (integrating.cu:173-233): density gradients scaled by
// min(z^2, 1), the near-plane penalty added, the background counted in (final - cur) and again in
// bg * (1 - opacity), the opacity normalisation of terminated rays not differentiated.
// kExact = true: the adjoint of the forward as computed.  With out = colour (or depth) of the ray
// and cur_k the sum of the first k+1 weighted samples,
//   d out / d sigma_k = dt_k (T_{k+1} c_k - (out - cur_k)) / norm,   d out / d c_k = w_k / norm,
// where norm = 1 for a ray that reaches the background (out - cur_k already holds T_N bg) and
// norm = 1 - T_N = opacity for a terminated ray (out = cur_N / opacity).
struct RayGrad {
    float4 fr, go;      // final colour/depth of the ray, dL/dfinal (divided by the opacity: kExact, terminated)
    float bg[3], bgterm;
};

template <bool kExact>
__device__ __forceinline__ float4 sample_grad(const RayGrad &q, float near_distance, float4 c, float z, float dt, float w,
                                              float Tn, float cr, float cg, float cb, float cd) {
    const float dsig = dt * (q.go.x * (Tn * c.y - (q.fr.x - cr) - q.bg[0] * q.bgterm)
                           + q.go.y * (Tn * c.z - (q.fr.y - cg) - q.bg[1] * q.bgterm)
                           + q.go.z * (Tn * c.w - (q.fr.z - cb) - q.bg[2] * q.bgterm)
                           + q.go.w * (Tn * z - (q.fr.w - cd)));
    if (kExact) return make_float4(dsig, w * q.go.x, w * q.go.y, w * q.go.z);
    const float reg = ((double)c.x > 4e-5 && z < near_distance) ? 1e-4f : 0.0f;
    return make_float4(fminf(z * z, 1.f) * dsig + reg, w * q.go.x, w * q.go.y, w * q.go.z);
}

// One ray in the reference's order (one thread); returns the transmittance after the last sample.
template <bool kExact>
__device__ __forceinline__ float backward_serial(const RayGrad &q, float near_distance, const float *rd, const float *rz,
                                                 const float4 *rc, std::uint32_t n, float *gz, float4 *gc) {
    float T = 1.f, cr = 0.f, cg = 0.f, cb = 0.f, cd = 0.f;
    for (std::uint32_t k = 0; T > kTThreshold && k < n; ++k) {
        const float4 c = rc[k];
        const float z = rz[k], dt = rd[k];
        const float alpha = 1.f - expf(-c.x * dt);
        const float w = T * alpha;
        cr += w * c.y;
        cg += w * c.z;
        cb += w * c.w;
        cd += w * z;
        T *= 1.f - alpha;
        gz[k] = w * q.go.w;
        gc[k] = sample_grad<kExact>(q, near_distance, c, z, dt, w, T, cr, cg, cb, cd);
    }
    return T;
}

// The same ray by the whole warp; false (every lane) when a decision fell within the tree/serial
// bound -- the samples it wrote are then among those the serial pass writes again.
template <bool kExact>
__device__ __forceinline__ bool backward_warp(const RayGrad &q, float near_distance, const float *rd, const float *rz,
                                              const float4 *rc, std::uint32_t n, unsigned lane, float *gz, float4 *gc,
                                              float &T_out) {
    float T = 1.f, cr = 0.f, cg = 0.f, cb = 0.f, cd = 0.f;
    std::uint32_t used = 0;
    for (std::uint32_t base = 0; base < n; base += 32) {
        const std::uint32_t cnt = min(32u, n - base);
        const bool in = lane < cnt;
        float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
        float dt = 0.f, z = 0.f;
        if (in) {
            c = rc[base + lane];
            dt = rd[base + lane];
            z = rz[base + lane];
        }
        const float a = in ? 1.f - expf(-c.x * dt) : 0.f;
        const float P = warp_prod_incl(1.f - a, lane);
        const float Pup = __shfl_up_sync(0xffffffffu, P, 1);
        const float Tq = T * (lane == 0 ? 1.f : Pup);
        const bool amb = in && fabsf(Tq - kTThreshold) <= kTThreshold * decision_tol(used + lane);
        if (__any_sync(0xffffffffu, amb)) return false;
        const bool use = in && Tq > kTThreshold;
        const std::uint32_t nu = __popc(__ballot_sync(0xffffffffu, use));
        const float w = use ? Tq * a : 0.f;
        const float Tn = T * P;
        const float qr = cr + warp_sum_incl(w * c.y, lane);
        const float qg = cg + warp_sum_incl(w * c.z, lane);
        const float qb = cb + warp_sum_incl(w * c.w, lane);
        const float qd = cd + warp_sum_incl(w * z, lane);
        if (use) {
            gz[base + lane] = w * q.go.w;
            gc[base + lane] = sample_grad<kExact>(q, near_distance, c, z, dt, w, Tn, qr, qg, qb, qd);
        }
        if (nu > 0) {
            const int last = (int)nu - 1;
            T = __shfl_sync(0xffffffffu, Tn, last);
            cr = __shfl_sync(0xffffffffu, qr, last);
            cg = __shfl_sync(0xffffffffu, qg, last);
            cb = __shfl_sync(0xffffffffu, qb, last);
            cd = __shfl_sync(0xffffffffu, qd, last);
        }
        used += nu;
        if (nu < cnt || !(T > kTThreshold)) break;
    }
    if (fabsf(T - kTThreshold) <= kTThreshold * decision_tol(used)) return false;
    T_out = T;
    return true;
}

template <bool kExact>
__global__ void __launch_bounds__(32 * kIntWarps) integrate_rays_backward_kernel(
    std::uint32_t n_rays, std::uint32_t total_samples, float near_distance, const std::uint32_t *__restrict__ startidx,
    const std::uint32_t *__restrict__ n_samples, const float *__restrict__ bgs,
    const float *__restrict__ dss, const float *__restrict__ z_vals,
    const float *__restrict__ drgbs, const float *__restrict__ final_rgbds,
    const float *__restrict__ final_opacities, const float *__restrict__ dL_dfinal_rgbds,
    float *__restrict__ dL_dbgs, float *__restrict__ dL_dz_vals, float *__restrict__ dL_ddrgbs) {
    const unsigned lane = lane_id();
    const std::uint64_t W = (gridDim.x * blockDim.x) >> 5, w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    for (std::uint64_t j0 = 0; w + j0 * W < n_rays; j0 += 32) {
        const std::uint64_t ii = w + (j0 + lane) * W;
        const std::uint32_t i = ii < n_rays ? (std::uint32_t)ii : 0xffffffffu;
        std::uint32_t s = 0, n = 0;
        if (ii < n_rays) {
            s = startidx[i];
            n = clamp_range(s, n_samples[i], total_samples);
            if (n == 0) {   // T = 1 throughout: only the background has a gradient
                const float4 go = reinterpret_cast<const float4 *>(dL_dfinal_rgbds)[i];
                dL_dbgs[i * 3 + 0] = go.x;
                dL_dbgs[i * 3 + 1] = go.y;
                dL_dbgs[i * 3 + 2] = go.z;
            }
        }
        unsigned heavy = __ballot_sync(0xffffffffu, n > 0u);
        while (heavy != 0u) {
            const int src = __ffs(heavy) - 1;
            heavy &= heavy - 1u;
            const std::uint32_t ray = __shfl_sync(0xffffffffu, i, src);
            const std::uint32_t rs = __shfl_sync(0xffffffffu, s, src), rn = __shfl_sync(0xffffffffu, n, src);
            RayGrad q;
            q.fr = reinterpret_cast<const float4 *>(final_rgbds)[ray];
            const float fo = final_opacities[ray];
            const bool terminated = fo >= 1.f - kTThreshold;
            q.go = reinterpret_cast<const float4 *>(dL_dfinal_rgbds)[ray];
            q.bg[0] = bgs[ray * 3 + 0];
            q.bg[1] = bgs[ray * 3 + 1];
            q.bg[2] = bgs[ray * 3 + 2];
            q.bgterm = (kExact || terminated) ? 0.f : 1.f - fo;
            if (kExact && terminated) {
                const float inv = 1.f / fo;
                q.go = make_float4(q.go.x * inv, q.go.y * inv, q.go.z * inv, q.go.w * inv);
            }
            const float *rd = dss + rs, *rz = z_vals + rs;
            const float4 *rc = reinterpret_cast<const float4 *>(drgbs) + rs;
            float *gz = dL_dz_vals + rs;
            float4 *gc = reinterpret_cast<float4 *>(dL_ddrgbs) + rs;
            float T = 0.f;
            const bool fast = backward_warp<kExact>(q, near_distance, rd, rz, rc, rn, lane, gz, gc, T);
            __syncwarp();   // the fast pass's stores come before a serial rewrite of the same samples
            if (lane == 0) {
                if (!fast) T = backward_serial<kExact>(q, near_distance, rd, rz, rc, rn, gz, gc);
                if (T > kTThreshold) {
                    dL_dbgs[ray * 3 + 0] = T * q.go.x;
                    dL_dbgs[ray * 3 + 1] = T * q.go.y;
                    dL_dbgs[ray * 3 + 2] = T * q.go.z;
                }
            }
        }
    }
}

__global__ void __launch_bounds__(256) integrate_rays_inference_kernel(
    std::uint32_t n_total_rays, std::uint32_t n_rays, std::uint32_t cap,
    const float *__restrict__ rays_bg, const float *__restrict__ rays_rgbd,
    const float *__restrict__ rays_T, const std::uint32_t *__restrict__ n_samples,
    const std::uint32_t *__restrict__ indices, const float *__restrict__ dss,
    const float *__restrict__ z_vals, const float *__restrict__ drgbs,
    std::uint32_t *__restrict__ terminate_cnt, bool *__restrict__ terminated,
    float *__restrict__ rgbd_out, float *__restrict__ T_out) {
    const std::uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool term = false;
    if (i < n_rays) {
        const std::uint32_t n = min(n_samples[i], cap), r = indices[i];
        float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
        float Tw = 0.f;
        if (r < n_total_rays) {
            const float *rd = dss + (std::size_t)i * cap, *rz = z_vals + (std::size_t)i * cap;
            const float4 *rc = reinterpret_cast<const float4 *>(drgbs) + (std::size_t)i * cap;
            float T = rays_T[r];
            const float4 acc = reinterpret_cast<const float4 *>(rays_rgbd)[r];
            float cr = acc.x, cg = acc.y, cb = acc.z, cd = acc.w;
            for (std::uint32_t k = 0; T > kTThreshold && k < n; ++k) {
                const float4 c = rc[k];
                const float alpha = 1.f - expf(-c.x * rd[k]);
                const float w = T * alpha;
                cr += w * c.y;
                cg += w * c.z;
                cb += w * c.w;
                cd += w * rz[k];
                T *= (1.f - alpha);
            }
            if (T <= kTThreshold) {
                const float id = 1.f / (1.f - T);
                term = true;
                Tw = 0.f;
                out = make_float4(cr * id, cg * id, cb * id, cd * id);
            } else {
                term = n < cap;
                Tw = T;
                if (term) {
                    out = make_float4(cr + T * rays_bg[(std::size_t)r * 3 + 0], cg + T * rays_bg[(std::size_t)r * 3 + 1],
                                      cb + T * rays_bg[(std::size_t)r * 3 + 2], cd);
                } else {
                    out = make_float4(cr, cg, cb, cd);
                }
            }
        }
        terminated[i] = term;
        T_out[i] = Tw;
        reinterpret_cast<float4 *>(rgbd_out)[i] = out;
    }
    const std::uint32_t cnt = warp_sum(term ? 1u : 0u);
    if (lane_id() == 0 && cnt > 0) atomicAdd(terminate_cnt, cnt);
}

// In-place form for the device-resident renderer: each slot continues its ray straight in the
// full-frame arrays (what integrating/__init__.py:108-109 does with .at[].set), and the number of
// terminated rays is added to a running total instead of reset, so the host can poll it rarely.
__global__ void __launch_bounds__(256) integrate_rays_inference_inplace_kernel(
    std::uint32_t n_total_rays, std::uint32_t n_rays, std::uint32_t cap,
    const float *__restrict__ rays_bg, float *__restrict__ rays_rgbd, float *__restrict__ rays_T,
    const std::uint32_t *__restrict__ n_samples, const std::uint32_t *__restrict__ indices,
    const float *__restrict__ dss, const float *__restrict__ z_vals, const float *__restrict__ drgbs,
    const std::uint32_t *__restrict__ sample_start, std::uint32_t *__restrict__ terminate_total,
    bool *__restrict__ terminated) {
    const std::uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool term = false;
    if (i < n_rays) {
        const std::uint32_t n = min(n_samples[i], cap), r = indices[i];
        if (r < n_total_rays) {
            const float *rd = dss + (std::size_t)i * cap, *rz = z_vals + (std::size_t)i * cap;
            // the slot's colours: strided like dss, or packed from sample_start[i] (compact march)
            const float4 *rc = reinterpret_cast<const float4 *>(drgbs) +
                               (sample_start != nullptr ? (std::size_t)sample_start[i] : (std::size_t)i * cap);
            float T = rays_T[r];
            const float4 acc = reinterpret_cast<const float4 *>(rays_rgbd)[r];
            float cr = acc.x, cg = acc.y, cb = acc.z, cd = acc.w;
            for (std::uint32_t k = 0; T > kTThreshold && k < n; ++k) {
                const float4 c = rc[k];
                const float alpha = 1.f - expf(-c.x * rd[k]);
                const float w = T * alpha;
                cr += w * c.y;
                cg += w * c.z;
                cb += w * c.w;
                cd += w * rz[k];
                T *= (1.f - alpha);
            }
            float4 out;
            float Tw;
            if (T <= kTThreshold) {
                const float id = 1.f / (1.f - T);
                term = true;
                Tw = 0.f;
                out = make_float4(cr * id, cg * id, cb * id, cd * id);
            } else {
                term = n < cap;
                Tw = T;
                out = term ? make_float4(cr + T * rays_bg[(std::size_t)r * 3 + 0], cg + T * rays_bg[(std::size_t)r * 3 + 1],
                                         cb + T * rays_bg[(std::size_t)r * 3 + 2], cd)
                           : make_float4(cr, cg, cb, cd);
            }
            reinterpret_cast<float4 *>(rays_rgbd)[r] = out;
            rays_T[r] = Tw;
        }
        terminated[i] = term;
    }
    const std::uint32_t cnt = warp_sum(term ? 1u : 0u);
    if (lane_id() == 0 && cnt > 0) atomicAdd(terminate_total, cnt);
}

// Blocks of the warp-per-ray integrators: a warp per 32 rays, at most 16 blocks per SM (a warp
// then takes more than 32 rays).
unsigned warp_ray_grid(std::uint32_t n_rays) {
    const unsigned chunks = (n_rays + 31) / 32, blocks = (chunks + kIntWarps - 1) / kIntWarps;
    const unsigned cap = (unsigned)sm_count() * 16u;
    return blocks < cap ? blocks : cap;
}

}  // namespace

int launch_integrate_rays(cudaStream_t stream, const IntegratingDescriptor &d,
                          const std::uint32_t *startidx, const std::uint32_t *n_samples,
                          const float *bgs, const float *dss, const float *z_vals,
                          const float *drgbs, std::uint32_t *measured, float *final_rgbds,
                          float *final_opacities) {
    NGP_CUDA_TRY(cudaMemsetAsync(measured, 0, sizeof(std::uint32_t), stream));
    if (d.n_rays > 0) {
        integrate_rays_kernel<<<warp_ray_grid(d.n_rays), 32 * kIntWarps, 0, stream>>>(
            d.n_rays, d.total_samples, startidx, n_samples, bgs, dss, z_vals, drgbs, measured, final_rgbds, final_opacities);
        count_launches(1);
    }
    return launch_status();
}

int launch_integrate_rays_fp64(cudaStream_t stream, const IntegratingDescriptor &d, const std::uint32_t *startidx,
                               const std::uint32_t *n_samples, const float *bgs, const float *dss, const float *z_vals,
                               const float *drgbs, double *rgbds, double *trans, std::uint32_t *used) {
    NGP_CHECK_ARG(((std::uintptr_t)drgbs & 15u) == 0 && ((std::uintptr_t)rgbds & 7u) == 0 && ((std::uintptr_t)trans & 7u) == 0,
                  "integrate_rays_fp64: drgbs must be 16-byte and the double outputs 8-byte aligned");
    if (d.n_rays > 0) {
        integrate_rays_fp64_kernel<<<(d.n_rays + 255) / 256, 256, 0, stream>>>(d.n_rays, d.total_samples, startidx, n_samples,
                                                                             bgs, dss, z_vals, drgbs, rgbds, trans, used);
        count_launches(1);
    }
    return launch_status();
}

int launch_integrate_rays_backward(cudaStream_t stream, const IntegratingBackwardDescriptor &d,
                                   const std::uint32_t *startidx, const std::uint32_t *n_samples,
                                   const float *bgs, const float *dss, const float *z_vals,
                                   const float *drgbs, const float *final_rgbds,
                                   const float *final_opacities, const float *dL_dfinal_rgbds,
                                   float *dL_dbgs, float *dL_dz_vals, float *dL_ddrgbs, bool exact) {
    NGP_CHECK_ARG(d.near_distance >= 0.f, "integrate_rays_backward: near_distance must be non-negative");
    // samples past a ray's termination and slots that belong to no ray get zero gradients
    NGP_CUDA_TRY(cudaMemsetAsync(dL_dbgs, 0, (std::size_t)d.n_rays * 3 * sizeof(float), stream));
    NGP_CUDA_TRY(cudaMemsetAsync(dL_dz_vals, 0, (std::size_t)d.total_samples * sizeof(float), stream));
    NGP_CUDA_TRY(cudaMemsetAsync(dL_ddrgbs, 0, (std::size_t)d.total_samples * 4 * sizeof(float), stream));
    if (d.n_rays > 0) {
        if (exact)
            integrate_rays_backward_kernel<true><<<warp_ray_grid(d.n_rays), 32 * kIntWarps, 0, stream>>>(
                d.n_rays, d.total_samples, d.near_distance, startidx, n_samples, bgs, dss, z_vals, drgbs, final_rgbds,
                final_opacities, dL_dfinal_rgbds, dL_dbgs, dL_dz_vals, dL_ddrgbs);
        else
            integrate_rays_backward_kernel<false><<<warp_ray_grid(d.n_rays), 32 * kIntWarps, 0, stream>>>(
                d.n_rays, d.total_samples, d.near_distance, startidx, n_samples, bgs, dss, z_vals, drgbs, final_rgbds,
                final_opacities, dL_dfinal_rgbds, dL_dbgs, dL_dz_vals, dL_ddrgbs);
        count_launches(1);
    }
    return launch_status();
}

int launch_integrate_rays_inference(cudaStream_t stream, const IntegratingInferenceDescriptor &d,
                                    const float *rays_bg, const float *rays_rgbd,
                                    const float *rays_T, const std::uint32_t *n_samples,
                                    const std::uint32_t *indices, const float *dss,
                                    const float *z_vals, const float *drgbs,
                                    std::uint32_t *terminate_cnt, bool *terminated,
                                    float *rgbd_out, float *T_out) {
    NGP_CUDA_TRY(cudaMemsetAsync(terminate_cnt, 0, sizeof(std::uint32_t), stream));
    if (d.n_rays > 0) {
        integrate_rays_inference_kernel<<<(d.n_rays + 255) / 256, 256, 0, stream>>>(
            d.n_total_rays, d.n_rays, d.march_steps_cap, rays_bg, rays_rgbd, rays_T, n_samples,
            indices, dss, z_vals, drgbs, terminate_cnt, terminated, rgbd_out, T_out);
        count_launches(1);
    }
    return launch_status();
}

}  // namespace ngp

namespace ngp {
int launch_integrate_rays_inference_inplace(cudaStream_t stream, const IntegratingInferenceDescriptor &d,
                                            const float *rays_bg, float *rays_rgbd, float *rays_T,
                                            const std::uint32_t *n_samples, const std::uint32_t *indices,
                                            const float *dss, const float *z_vals, const float *drgbs,
                                            const std::uint32_t *sample_start, std::uint32_t *terminate_total,
                                            bool *terminated) {
    NGP_CHECK_ARG(((std::uintptr_t)rays_rgbd & 15u) == 0 && ((std::uintptr_t)drgbs & 15u) == 0,
                  "integrate_rays_inference: rays_rgbd and drgbs must be 16-byte aligned");
    if (d.n_rays > 0) {
        integrate_rays_inference_inplace_kernel<<<(d.n_rays + 255) / 256, 256, 0, stream>>>(
            d.n_total_rays, d.n_rays, d.march_steps_cap, rays_bg, rays_rgbd, rays_T, n_samples, indices, dss, z_vals,
            drgbs, sample_start, terminate_total, terminated);
        count_launches(1);
    }
    return launch_status();
}
}  // namespace ngp
