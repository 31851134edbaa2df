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

__global__ void __launch_bounds__(256) integrate_rays_kernel(
    std::uint32_t n_rays, std::uint32_t total_samples, const std::uint32_t *__restrict__ startidx,
    const std::uint32_t *__restrict__ n_samples, const float *__restrict__ bgs,
    const float *__restrict__ dss, const float *__restrict__ z_vals,
    const float *__restrict__ drgbs, std::uint32_t *__restrict__ measured,
    float *__restrict__ final_rgbds, float *__restrict__ final_opacities) {
    const std::uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    std::uint32_t used = 0;
    if (i < n_rays) {
        const std::uint32_t s = startidx[i], n = clamp_range(s, n_samples[i], total_samples);
        const float *rd = dss + s, *rz = z_vals + s;
        const float4 *rc = reinterpret_cast<const float4 *>(drgbs) + s;
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
        used = k;
        const float opacity = 1.f - T;
        final_opacities[i] = opacity;
        float4 out;
        if (T <= kTThreshold) {
            const float id = 1.f / opacity;
            out = make_float4(r * id, g * id, b * id, depth * id);
        } else {
            out = make_float4(r + T * bgs[i * 3 + 0], g + T * bgs[i * 3 + 1], b + T * bgs[i * 3 + 2], depth);
        }
        reinterpret_cast<float4 *>(final_rgbds)[i] = out;
    }
    used = warp_sum(used);
    if (lane_id() == 0 && used > 0) atomicAdd(measured, used);
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
template <bool kExact>
__global__ void __launch_bounds__(256) integrate_rays_backward_kernel(
    std::uint32_t n_rays, std::uint32_t total_samples, float near_distance, const std::uint32_t *__restrict__ startidx,
    const std::uint32_t *__restrict__ n_samples, const float *__restrict__ bgs,
    const float *__restrict__ dss, const float *__restrict__ z_vals,
    const float *__restrict__ drgbs, const float *__restrict__ final_rgbds,
    const float *__restrict__ final_opacities, const float *__restrict__ dL_dfinal_rgbds,
    float *__restrict__ dL_dbgs, float *__restrict__ dL_dz_vals, float *__restrict__ dL_ddrgbs) {
    const std::uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_rays) return;
    const std::uint32_t s = startidx[i], n = clamp_range(s, n_samples[i], total_samples);
    const float *rd = dss + s, *rz = z_vals + s;
    const float4 *rc = reinterpret_cast<const float4 *>(drgbs) + s;
    const float4 fr = reinterpret_cast<const float4 *>(final_rgbds)[i];
    const float fo = final_opacities[i];
    const bool terminated = fo >= 1.f - kTThreshold;
    float4 go = reinterpret_cast<const float4 *>(dL_dfinal_rgbds)[i];
    const float bg0 = bgs[i * 3 + 0], bg1 = bgs[i * 3 + 1], bg2 = bgs[i * 3 + 2];
    const float bgterm = (kExact || terminated) ? 0.f : 1.f - fo;
    if (kExact && terminated) {
        const float inv = 1.f / fo;
        go = make_float4(go.x * inv, go.y * inv, go.z * inv, go.w * inv);
    }
    float *gz = dL_dz_vals + s;
    float4 *gc = reinterpret_cast<float4 *>(dL_ddrgbs) + s;
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
        gz[k] = w * go.w;
        const float dsig = dt * (go.x * (T * c.y - (fr.x - cr) - bg0 * bgterm)
                               + go.y * (T * c.z - (fr.y - cg) - bg1 * bgterm)
                               + go.z * (T * c.w - (fr.z - cb) - bg2 * bgterm)
                               + go.w * (T * z - (fr.w - cd)));
        if (kExact) {
            gc[k] = make_float4(dsig, w * go.x, w * go.y, w * go.z);
        } else {
            const float reg = ((double)c.x > 4e-5 && z < near_distance) ? 1e-4f : 0.0f;
            const float scale = fminf(z * z, 1.f);
            gc[k] = make_float4(scale * dsig + reg, w * go.x, w * go.y, w * go.z);
        }
    }
    if (T > kTThreshold) {
        dL_dbgs[i * 3 + 0] = T * go.x;
        dL_dbgs[i * 3 + 1] = T * go.y;
        dL_dbgs[i * 3 + 2] = T * go.z;
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

}  // namespace

int launch_integrate_rays(cudaStream_t stream, const IntegratingDescriptor &d,
                          const std::uint32_t *startidx, const std::uint32_t *n_samples,
                          const float *bgs, const float *dss, const float *z_vals,
                          const float *drgbs, std::uint32_t *measured, float *final_rgbds,
                          float *final_opacities) {
    NGP_CUDA_TRY(cudaMemsetAsync(measured, 0, sizeof(std::uint32_t), stream));
    if (d.n_rays > 0) {
        integrate_rays_kernel<<<(d.n_rays + 255) / 256, 256, 0, stream>>>(
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
            integrate_rays_backward_kernel<true><<<(d.n_rays + 255) / 256, 256, 0, stream>>>(
                d.n_rays, d.total_samples, d.near_distance, startidx, n_samples, bgs, dss, z_vals, drgbs, final_rgbds,
                final_opacities, dL_dfinal_rgbds, dL_dbgs, dL_dz_vals, dL_ddrgbs);
        else
            integrate_rays_backward_kernel<false><<<(d.n_rays + 255) / 256, 256, 0, stream>>>(
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
