// Training-step kernels around the drop-in ops: batch construction, the fused
// integrate -> loss -> integrate-backward pass, Adam, and occupancy-grid maintenance.
//
// They restate, as single kernels, what the reference does with several XLA ops per step:
//   ray batch:       app/nerf/_utils.py:93-115 (rays from pixel indices), models/renderers/
//                    cuda.py:56-97 (AABB near/far), :118-121 (start jitter), _utils.py:134-137
//                    (random background), utils/data.py:443-465 (RGBA over background)
//   loss:            app/nerf/_utils.py:149-160 (Huber, delta 0.1, masked by ray_is_valid)
//   optimiser:       app/nerf/_utils.py:19-77 (optax adam + add_decayed_weights)
//   occupancy grid:  utils/types.py:1149-1225 (decay, sampling, density max), :1227-1239
//                    (threshold), :1241-1362 (marking cells no camera sees), :1385-1392
#include "common.cuh"
#include "half.cuh"

namespace ngp {
namespace {

// SplitMix64-based counter RNG: uniform floats in [0, 1) keyed by (seed, stream, index).
__device__ __forceinline__ std::uint64_t mix64(std::uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ std::uint64_t rng_u64(std::uint64_t seed, std::uint32_t stream, std::uint64_t i) {
    return mix64(seed ^ mix64(((std::uint64_t)stream << 48) ^ i));
}
__device__ __forceinline__ float rng_uniform(std::uint64_t seed, std::uint32_t stream, std::uint64_t i) {
    return (float)(rng_u64(seed, stream, i) >> 40) * (1.0f / 16777216.0f);
}

__global__ void __launch_bounds__(256) train_rays_kernel(
    NgpTrainRaysDescriptor d, const float *__restrict__ transforms, const std::uint8_t *__restrict__ rgbas,
    const std::uint32_t *__restrict__ perm, float *__restrict__ rays_o, float *__restrict__ rays_d,
    float *__restrict__ t_starts, float *__restrict__ t_ends, float *__restrict__ noises,
    float *__restrict__ bgs, float *__restrict__ gt) {
    const std::uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n_rays) return;
    const std::uint64_t n_pix = (std::uint64_t)d.width * d.height;
    std::uint64_t p;
    const std::uint64_t n_all = n_pix * d.n_views;
    if (perm != nullptr) {
        p = perm[i];
        if (p >= n_all) p = n_all - 1;  // out-of-range pixel indices are clamped
    } else {
        p = (std::uint64_t)(((unsigned __int128)rng_u64(d.seed, 0, i) * n_all) >> 64);
    }
    const std::uint32_t view = (std::uint32_t)(p / n_pix);
    const std::uint32_t pix = (std::uint32_t)(p % n_pix);
    const float px = (float)(pix % d.width), py = (float)(pix / d.width);
    // camera-space direction, CV -> CG axis flip (utils/types.py:417-439)
    float cx = ((px + 0.5f) - d.cx) / d.fx;
    float cy = -(((py + 0.5f) - d.cy) / d.fy);
    float cz = -1.0f;
    const float inv = rsqrtf(cx * cx + cy * cy + cz * cz);
    cx *= inv;
    cy *= inv;
    cz *= inv;
    const float *T = transforms + (std::size_t)view * 12;
    const float dx = cx * T[0] + cy * T[1] + cz * T[2];
    const float dy = cx * T[3] + cy * T[4] + cz * T[5];
    const float dz = cx * T[6] + cy * T[7] + cz * T[8];
    const float ox = T[9], oy = T[10], oz = T[11];
    rays_o[i * 3 + 0] = ox;
    rays_o[i * 3 + 1] = oy;
    rays_o[i * 3 + 2] = oz;
    rays_d[i * 3 + 0] = dx;
    rays_d[i * 3 + 1] = dy;
    rays_d[i * 3 + 2] = dz;
    // AABB intersection (renderers/cuda.py:56-97)
    const float eps = 1e-15f, b = d.bound;
    const float ex = signbit(dx) ? fminf(dx, -eps) : fmaxf(dx, eps);
    const float ey = signbit(dy) ? fminf(dy, -eps) : fmaxf(dy, eps);
    const float ez = signbit(dz) ? fminf(dz, -eps) : fmaxf(dz, eps);
    const float tx0 = (-b - ox) / ex, tx1 = (b - ox) / ex;
    const float ty0 = (-b - oy) / ey, ty1 = (b - oy) / ey;
    const float tz0 = (-b - oz) / ez, tz1 = (b - oz) / ez;
    const float ts = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fminf(tz0, tz1));
    const float te = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
    t_starts[i] = fmaxf(0.f, ts);
    t_ends[i] = te;
    noises[i] = d.perturb ? rng_uniform(d.seed, 1, i) : 0.f;
    float bg[3] = {d.bg[0], d.bg[1], d.bg[2]};
    if (d.random_bg) {
        bg[0] = rng_uniform(d.seed, 2, i);
        bg[1] = rng_uniform(d.seed, 3, i);
        bg[2] = rng_uniform(d.seed, 4, i);
    }
    const uchar4 px4 = reinterpret_cast<const uchar4 *>(rgbas)[p];
    const float a = px4.w / 255.f;
    const float rgb[3] = {px4.x / 255.f, px4.y / 255.f, px4.z / 255.f};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        bgs[i * 3 + c] = bg[c];
        gt[i * 3 + c] = rgb[c] * a + bg[c] * (1.f - a);
    }
}

// Per ray: integrate_rays forward (integrating.cu:24-104), Huber loss against the target, and
// integrate_rays_backward (integrating.cu:106-240) with dL/dfinal_rgbd from the loss; dL/ddepth
// is zero (the loss ignores depth).  Gradients are unnormalised; 1/n_valid is applied by the
// field backward through `grad_scale`.
//
// Two passes.  The light pass (a thread per ray) finishes every ray without samples -- its
// prediction is the background -- and appends the rays with samples to a list (one atomic per
// warp).  The heavy pass gives each listed ray a whole warp, warps taking rays from the list in
// turn, and runs the ray as segments of 32 samples (lane = sample, loads and stores coalesced):
// the transmittance before and after each sample comes from a warp product scan of 1 - alpha,
// the running colour sums of the backward from warp sum scans, the ray's totals from warp
// reductions, and the transmittance and sums carry from segment to segment.  Products and sums
// are formed in tree order rather than the reference's left-to-right order (a few ulps apart;
// the termination test is the reference's: a sample counts while the transmittance before it is
// above 1e-4).  Taking rays
// from a list keeps the warps evenly loaded however the rays with samples cluster in the batch
// (which rays fit the sample budget follows the order of the allocation atomics).  The loss sums
// are reduced per block before their one atomic each.
constexpr int kIlbWarps = 4;

// Inclusive warp scans (product and sum) and a warp sum that every lane receives.
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

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float huber_grad(float e, float delta, float *loss) {
    const float ae = fabsf(e);
    *loss += ae <= delta ? 0.5f * e * e : delta * (ae - 0.5f * delta);
    return ae <= delta ? e : copysignf(delta, e);
}

// Adds v[0..2] of every thread of the block into acc[0..2] (one atomic per quantity per block).
template <int NT>
__device__ __forceinline__ void block_accumulate(float l, float nv, float used, float *__restrict__ acc) {
    __shared__ float part[NT / 32][3];
    l = warp_sum(l);
    nv = warp_sum(nv);
    used = warp_sum(used);
    const unsigned w = threadIdx.x >> 5;
    if (lane_id() == 0) {
        part[w][0] = l;
        part[w][1] = nv;
        part[w][2] = used;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        float a = 0.f;
        for (int k = 0; k < NT / 32; ++k) a += part[k][threadIdx.x];
        if (a != 0.f) atomicAdd(acc + threadIdx.x, a);
    }
}

constexpr int kIlbLight = 256;

__global__ void __launch_bounds__(kIlbLight) integrate_loss_light_kernel(
    std::uint32_t n_rays, std::uint32_t total_samples, float delta, const bool *__restrict__ valid,
    const std::uint32_t *__restrict__ startidx, const std::uint32_t *__restrict__ n_samples,
    const float *__restrict__ bgs, const float *__restrict__ gt, float *__restrict__ acc,
    std::uint32_t *__restrict__ heavy_count, std::uint32_t *__restrict__ heavy) {
    const std::uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float loss = 0.f, nv = 0.f;
    bool is_heavy = false;
    if (i < n_rays) {
        const std::uint32_t s = startidx[i];
        const std::uint32_t n = s >= total_samples ? 0u : min(n_samples[i], total_samples - s);
        if (n == 0) {  // T = 1: the prediction is the background
            if (valid[i]) {
                nv = 1.f;
                float l = 0.f;
#pragma unroll
                for (int c = 0; c < 3; ++c) huber_grad(bgs[i * 3 + c] - gt[i * 3 + c], delta, &l);
                loss = l * (1.f / 3.f);
            }
        } else {
            is_heavy = true;
        }
    }
    const unsigned hb = __ballot_sync(0xffffffffu, is_heavy);
    if (hb != 0u) {
        std::uint32_t base = 0;
        if (lane_id() == 0) base = atomicAdd(heavy_count, (unsigned)__popc(hb));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (is_heavy) heavy[base + __popc(hb & ((1u << lane_id()) - 1u))] = i;
    }
    block_accumulate<kIlbLight>(loss, nv, 0.f, acc);
}

__global__ void __launch_bounds__(32 * kIlbWarps) integrate_loss_heavy_kernel(
    std::uint32_t total_samples, float near_distance, float delta, const bool *__restrict__ valid,
    const std::uint32_t *__restrict__ startidx, const std::uint32_t *__restrict__ n_samples,
    const float *__restrict__ bgs, const float *__restrict__ gt, const float *__restrict__ dss,
    const float *__restrict__ z_vals, const float *__restrict__ drgbs, const std::uint32_t *__restrict__ heavy_count,
    const std::uint32_t *__restrict__ heavy, float *__restrict__ dL_ddrgbs, float *__restrict__ acc) {
    const unsigned lane = lane_id();
    const std::uint32_t n_heavy = *heavy_count;
    const std::uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const std::uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
    float loss = 0.f, nv = 0.f, used_f = 0.f;   // lane 0's sums for its warp's rays

    for (std::uint32_t h = warp0; h < n_heavy; h += n_warps) {
        const std::uint32_t ray = heavy[h];
        const std::uint32_t s = startidx[ray];
        const std::uint32_t n = min(n_samples[ray], total_samples - s);
        const bool rv = valid[ray];
        float bg[3], tg[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            bg[c] = bgs[ray * 3 + c];
            tg[c] = gt[ray * 3 + c];
        }
        const float4 *rc = reinterpret_cast<const float4 *>(drgbs) + s;
        // ---- forward (integrating.cu:61-78) over 32-sample segments: lane q takes sample q of the
        // segment, a warp product scan of (1 - alpha) gives each sample's transmittance, sums are
        // warp reductions, and the transmittance is carried to the next segment.  A sample is
        // composited while the transmittance before it is above the threshold (a prefix of the
        // segment: the product never grows).
        float T = 1.f, r = 0.f, g = 0.f, b = 0.f, dep = 0.f;
        std::uint32_t used = 0;
        for (std::uint32_t base = 0; base < n; base += 32) {
            const std::uint32_t cnt = min(32u, n - base);
            const bool in = lane < cnt;
            float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
            float dt = 0.f, z = 0.f;
            if (in) {
                c = rc[base + lane];
                dt = dss[s + base + lane];
                z = z_vals[s + base + lane];
            }
            const float a = in ? 1.f - expf(-c.x * dt) : 0.f;
            const float P = warp_prod_incl(1.f - a, lane);
            const float Pup = __shfl_up_sync(0xffffffffu, P, 1);   // every lane takes part
            const float Pex = lane == 0 ? 1.f : Pup;
            const float Tq = T * Pex;
            const bool use = in && Tq > kTThreshold;
            const std::uint32_t nu = __popc(__ballot_sync(0xffffffffu, use));
            const float w = use ? Tq * a : 0.f;
            r += warp_sum(w * c.y);
            g += warp_sum(w * c.z);
            b += warp_sum(w * c.w);
            dep += warp_sum(w * z);
            const float Pend = __shfl_sync(0xffffffffu, P, nu > 0 ? (int)nu - 1 : 0);
            if (nu > 0) T *= Pend;
            used += nu;
            if (nu < cnt || !(T > kTThreshold)) break;
        }
        const float fo = 1.f - T;
        float fr[4];
        if (T <= kTThreshold) {
            const float id = 1.f / fo;
            fr[0] = r * id; fr[1] = g * id; fr[2] = b * id; fr[3] = dep * id;
        } else {
            fr[0] = r + T * bg[0]; fr[1] = g + T * bg[1]; fr[2] = b + T * bg[2]; fr[3] = dep;
        }
        // ---- loss and dL/dfinal_rgbd (mean over channels)
        float go[3] = {0.f, 0.f, 0.f}, l = 0.f;
        if (rv) {
#pragma unroll
            for (int c = 0; c < 3; ++c) go[c] = huber_grad(fr[c] - tg[c], delta, &l) * (1.f / 3.f);
        }
        if (lane == 0) {
            if (rv) {
                nv += 1.f;
                loss += l * (1.f / 3.f);
            }
            used_f += (float)used;
        }
        // ---- backward (integrating.cu:173-233), recomputing the forward with the same scans:
        // T_{k+1} from the product scan, the running colour/depth sums cur_k from inclusive sum
        // scans, both carried across segments
        const bool terminated = fo >= 1.f - kTThreshold;
        const float bgterm = terminated ? 0.f : 1.f - fo;
        float4 *gc = reinterpret_cast<float4 *>(dL_ddrgbs) + s;
        float Tb = 1.f, cr = 0.f, cg = 0.f, cb = 0.f, cd = 0.f;
        for (std::uint32_t base = 0; base < used; base += 32) {
            const std::uint32_t cnt = min(32u, used - base);
            const bool in = lane < cnt;
            float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
            float dt = 0.f, z = 0.f;
            if (in) {
                c = rc[base + lane];
                dt = dss[s + base + lane];
                z = z_vals[s + base + lane];
            }
            const float a = in ? 1.f - expf(-c.x * dt) : 0.f;
            const float P = warp_prod_incl(1.f - a, lane);
            const float Pup = __shfl_up_sync(0xffffffffu, P, 1);   // every lane takes part
            const float Pex = lane == 0 ? 1.f : Pup;
            const float w = Tb * Pex * a;
            const float Tn = Tb * P;
            const float qr = cr + warp_sum_incl(w * c.y, lane);
            const float qg = cg + warp_sum_incl(w * c.z, lane);
            const float qb = cb + warp_sum_incl(w * c.w, lane);
            const float qd = cd + warp_sum_incl(w * z, lane);
            if (in) {
                const float dsig = dt * (go[0] * (Tn * c.y - (fr[0] - qr) - bg[0] * bgterm)
                                       + go[1] * (Tn * c.z - (fr[1] - qg) - bg[1] * bgterm)
                                       + go[2] * (Tn * c.w - (fr[2] - qb) - bg[2] * bgterm)
                                       + 0.f * (Tn * z - (fr[3] - qd)));
                const float reg = ((double)c.x > 4e-5 && z < near_distance) ? 1e-4f : 0.0f;
                gc[base + lane] = make_float4(fminf(z * z, 1.f) * dsig + reg, w * go[0], w * go[1], w * go[2]);
            }
            const int lastl = (int)cnt - 1;
            Tb = __shfl_sync(0xffffffffu, Tn, lastl);
            cr = __shfl_sync(0xffffffffu, qr, lastl);
            cg = __shfl_sync(0xffffffffu, qg, lastl);
            cb = __shfl_sync(0xffffffffu, qb, lastl);
            cd = __shfl_sync(0xffffffffu, qd, lastl);
        }
        for (std::uint32_t k = used + lane; k < n; k += 32) gc[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    block_accumulate<32 * kIlbWarps>(loss, nv, used_f, acc);
}

// stats = [loss / n_valid, n_valid, measured_batch_size, samples before compaction];
// grad_scale = 1 / n_valid.  `count` holds the active-sample count from the marcher.
__global__ void finalize_loss_kernel(const float *__restrict__ acc, const std::uint32_t *__restrict__ count,
                                     float *__restrict__ stats, float *__restrict__ grad_scale) {
    const float nv = acc[1];
    const float inv = nv > 0.f ? 1.f / nv : 0.f;
    stats[0] = acc[0] * inv;
    stats[1] = nv;
    stats[2] = acc[2];
    stats[3] = (float)*count;
    *grad_scale = inv;
}

// zero dL_ddrgbs slots in [count, total) (slots no ray owns)
__global__ void zero_tail4_kernel(std::uint32_t total, const std::uint32_t *__restrict__ count, float4 *__restrict__ x) {
    const std::uint32_t a = min(total, *count);
    for (std::size_t s = a + (std::size_t)blockIdx.x * blockDim.x + threadIdx.x; s < total; s += (std::size_t)gridDim.x * blockDim.x)
        x[s] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// optax.adam (scale_by_adam, then scale by -lr) chained with add_decayed_weights, in that order
// (app/nerf/_utils.py:45-77), then optax.apply_updates:
//   m = b1 m + (1-b1) g;  v = b2 v + (1-b2) (g g);  mh = m / (1-b1^t);  vh = v / (1-b2^t)
//   update = -lr * mh / (sqrt(vh + eps_root) + eps) + wd * p;  p = p + update
// (the decay term is added after the learning-rate scaling, exactly as the reference chains it).
__global__ void __launch_bounds__(256) adam_kernel(NgpAdamDescriptor d, float bc1, float bc2,
                                                   float *__restrict__ p, float *__restrict__ g,
                                                   float *__restrict__ m, float *__restrict__ v) {
    const std::size_t stride = (std::size_t)gridDim.x * blockDim.x;
    const std::size_t n4 = d.n / 4;
    for (std::size_t i = (std::size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
        float4 pp = reinterpret_cast<float4 *>(p)[i];
        float4 gg = reinterpret_cast<float4 *>(g)[i];
        float4 mm = reinterpret_cast<float4 *>(m)[i];
        float4 vv = reinterpret_cast<float4 *>(v)[i];
        float *pa = &pp.x, *ga = &gg.x, *ma = &mm.x, *va = &vv.x;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            ma[c] = d.beta1 * ma[c] + (1.f - d.beta1) * ga[c];
            va[c] = d.beta2 * va[c] + (1.f - d.beta2) * (ga[c] * ga[c]);
            const float mh = ma[c] / bc1, vh = va[c] / bc2;
            const float upd = -d.lr * (mh / (sqrtf(vh + d.eps_root) + d.eps)) + d.weight_decay * pa[c];
            pa[c] = pa[c] + upd;
        }
        reinterpret_cast<float4 *>(p)[i] = pp;
        reinterpret_cast<float4 *>(m)[i] = mm;
        reinterpret_cast<float4 *>(v)[i] = vv;
        if (d.zero_grad) reinterpret_cast<float4 *>(g)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    for (std::size_t i = n4 * 4 + (std::size_t)blockIdx.x * blockDim.x + threadIdx.x; i < d.n; i += stride) {
        float mm = d.beta1 * m[i] + (1.f - d.beta1) * g[i];
        float vv = d.beta2 * v[i] + (1.f - d.beta2) * (g[i] * g[i]);
        const float upd = -d.lr * ((mm / bc1) / (sqrtf(vv / bc2 + d.eps_root) + d.eps)) + d.weight_decay * p[i];
        p[i] = p[i] + upd;
        m[i] = mm;
        v[i] = vv;
        if (d.zero_grad) g[i] = 0.f;
    }
}

// adam_kernel on FP32 master parameters with a dynamic loss scale and a 16-bit working copy
// (kHalf: 0 none, NGP_DTYPE_BF16 or NGP_DTYPE_F16).  With `ls`, a step whose overflow flag is set
// changes nothing but the zeroed gradient; otherwise the gradient is divided by the scale (a power
// of two: exact) and the bias corrections use the count of updates actually made.
template <int kHalf>
__device__ __forceinline__ void put_half(void *ph, std::size_t i, float x) {
    if constexpr (kHalf == (int)NGP_DTYPE_BF16) reinterpret_cast<__nv_bfloat16 *>(ph)[i] = Bf16Op::cvt(x);
    else if constexpr (kHalf == (int)NGP_DTYPE_F16) reinterpret_cast<__half *>(ph)[i] = F16Op::cvt(x);
}

template <int kHalf>
__global__ void __launch_bounds__(256) adam_mixed_kernel(NgpAdamDescriptor d, float bc1, float bc2,
                                                         float *__restrict__ p, float *__restrict__ g,
                                                         float *__restrict__ m, float *__restrict__ v,
                                                         const NgpLossScale *__restrict__ ls, void *__restrict__ ph) {
    const std::size_t stride = (std::size_t)gridDim.x * blockDim.x;
    const std::size_t n4 = d.n / 4;
    const std::size_t i0 = (std::size_t)blockIdx.x * blockDim.x + threadIdx.x;
    float inv = 1.f;
    if (ls != nullptr) {
        if (ls->overflow != 0u) {
            if (d.zero_grad) {
                for (std::size_t i = i0; i < n4; i += stride) reinterpret_cast<float4 *>(g)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
                for (std::size_t i = n4 * 4 + i0; i < d.n; i += stride) g[i] = 0.f;
            }
            return;
        }
        inv = 1.f / ls->scale;
        const float t = (float)(d.step - ls->skipped_steps);
        bc1 = 1.f - powf(d.beta1, t);
        bc2 = 1.f - powf(d.beta2, t);
    }
    for (std::size_t i = i0; i < n4; i += stride) {
        float4 pp = reinterpret_cast<float4 *>(p)[i];
        float4 gg = reinterpret_cast<float4 *>(g)[i];
        float4 mm = reinterpret_cast<float4 *>(m)[i];
        float4 vv = reinterpret_cast<float4 *>(v)[i];
        float *pa = &pp.x, *ga = &gg.x, *ma = &mm.x, *va = &vv.x;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const float gc = ls != nullptr ? ga[c] * inv : ga[c];
            ma[c] = d.beta1 * ma[c] + (1.f - d.beta1) * gc;
            va[c] = d.beta2 * va[c] + (1.f - d.beta2) * (gc * gc);
            const float mh = ma[c] / bc1, vh = va[c] / bc2;
            const float upd = -d.lr * (mh / (sqrtf(vh + d.eps_root) + d.eps)) + d.weight_decay * pa[c];
            pa[c] = pa[c] + upd;
        }
        reinterpret_cast<float4 *>(p)[i] = pp;
        reinterpret_cast<float4 *>(m)[i] = mm;
        reinterpret_cast<float4 *>(v)[i] = vv;
        if (d.zero_grad) reinterpret_cast<float4 *>(g)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        if constexpr (kHalf == (int)NGP_DTYPE_BF16) {
            reinterpret_cast<uint2 *>(ph)[i] = make_uint2(Bf16Op::pack(pp.x, pp.y), Bf16Op::pack(pp.z, pp.w));
        } else if constexpr (kHalf == (int)NGP_DTYPE_F16) {
            reinterpret_cast<uint2 *>(ph)[i] = make_uint2(F16Op::pack(pp.x, pp.y), F16Op::pack(pp.z, pp.w));
        }
    }
    for (std::size_t i = n4 * 4 + i0; i < d.n; i += stride) {
        const float gi = ls != nullptr ? g[i] * inv : g[i];
        float mm = d.beta1 * m[i] + (1.f - d.beta1) * gi;
        float vv = d.beta2 * v[i] + (1.f - d.beta2) * (gi * gi);
        const float upd = -d.lr * ((mm / bc1) / (sqrtf(vv / bc2 + d.eps_root) + d.eps)) + d.weight_decay * p[i];
        p[i] = p[i] + upd;
        m[i] = mm;
        v[i] = vv;
        if (d.zero_grad) g[i] = 0.f;
        put_half<kHalf>(ph, i, p[i]);
    }
}

__global__ void loss_scale_update_kernel(NgpLossScaleDescriptor d, NgpLossScale *__restrict__ ls) {
    NgpLossScale s = *ls;
    if (s.overflow != 0u) {
        s.scale = fmaxf(s.scale * d.backoff_factor, d.min_scale);
        s.good_steps = 0u;
        s.skipped_steps += 1u;
    } else if (++s.good_steps >= d.growth_interval) {
        s.scale = fminf(s.scale * d.growth_factor, d.max_scale);
        s.good_steps = 0u;
    }
    s.overflow = 0u;
    *ls = s;
}

__device__ __forceinline__ std::uint32_t morton_decode(std::uint32_t x) {
    x = x & 0x49249249u;
    x = (x | (x >> 2)) & 0xc30c30c3u;
    x = (x | (x >> 4)) & 0x0f00f00fu;
    x = (x | (x >> 8)) & 0xff0000ffu;
    x = (x | (x >> 16)) & 0x0000ffffu;
    return x;
}

// types.py:1161-1162: decay the cascade's live cells (cells marked untrainable hold -1).
__global__ void ogrid_decay_kernel(std::uint32_t n, float decay, float *__restrict__ density) {
    for (std::size_t i = (std::size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (std::size_t)gridDim.x * blockDim.x) {
        const float v = density[i];
        if (v >= 0.f) density[i] = v * decay;
    }
}

// types.py:1164-1204: choose cells and a random point inside each.  With update_all, point j is
// in cell j; otherwise the first half of the points go to cells drawn uniformly among live cells
// and the second half to cells drawn uniformly among occupied live cells (rejection sampling on
// the bitfield, as the paper describes; a draw that keeps failing falls back to a uniform cell).
// Dead cells get index 0xFFFFFFFF and are skipped downstream.
__global__ void ogrid_sample_kernel(std::uint32_t M, std::uint32_t update_all, std::uint32_t cas, std::uint32_t G,
                                    float bound, std::uint64_t seed, const float *__restrict__ density,
                                    const std::uint8_t *__restrict__ bits, std::uint32_t *__restrict__ cells,
                                    float *__restrict__ xyz) {
    const std::uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= M) return;
    const std::uint32_t G3 = G * G * G;
    const float *dcas = density + (std::size_t)cas * G3;
    std::uint32_t c;
    if (update_all) {
        c = j;
    } else {
        const bool want_occupied = j >= M / 2;
        c = (std::uint32_t)(rng_u64(seed, 5, j) % G3);
        for (int tries = 0; tries < 64; ++tries) {
            const std::uint32_t cand = (std::uint32_t)(rng_u64(seed, 6 + tries, j) % G3);
            const std::uint32_t gi = cas * G3 + cand;
            const bool live = dcas[cand] >= 0.f;
            const bool occ = (bits[gi >> 3] >> (gi & 7u)) & 1u;
            if (live && (!want_occupied || occ)) {
                c = cand;
                break;
            }
        }
    }
    if (dcas[c] < 0.f) {
        cells[j] = 0xFFFFFFFFu;
        xyz[j * 3 + 0] = xyz[j * 3 + 1] = xyz[j * 3 + 2] = 0.f;
        return;
    }
    cells[j] = c;
    const float mip_bound = fminf(bound, (float)(1u << cas));
    const float hcw = mip_bound / (float)G;
    const std::uint32_t g[3] = {morton_decode(c), morton_decode(c >> 1), morton_decode(c >> 2)};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float v = (float)g[a] / (float)(G - 1) * 2.f - 1.f;
        v *= mip_bound - hcw;
        v += (rng_uniform(seed, 100 + a, j) * 2.f - 1.f) * hcw;
        xyz[j * 3 + a] = v;
    }
}

// types.py:1218-1220: density = max(density, new) at the chosen cells.  Non-negative floats order
// like their bit patterns, so an integer atomicMax gives the float max.
__global__ void ogrid_max_kernel(std::uint32_t M, std::uint32_t cas, std::uint32_t G3,
                                 const std::uint32_t *__restrict__ cells, const float *__restrict__ sigma,
                                 float *__restrict__ density) {
    const std::uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= M) return;
    const std::uint32_t c = cells[j];
    if (c >= G3) return;  // dead cell marker (or an out-of-range index)
    const float s = fmaxf(sigma[j], 0.f);
    atomicMax(reinterpret_cast<int *>(density + (std::size_t)cas * G3 + c), __float_as_int(s));
}

// types.py:1227-1231 and :1385-1386: threshold = min(0.01 * diag / (2 min(bound,1) sqrt3),
// mean density over the live cells of cascade 0).
__global__ void ogrid_mean_kernel(std::uint32_t n, const float *__restrict__ density, float *__restrict__ acc) {
    float s = 0.f, c = 0.f;
    for (std::size_t i = (std::size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (std::size_t)gridDim.x * blockDim.x) {
        const float v = density[i];
        if (v >= 0.f) {
            s += v;
            c += 1.f;
        }
    }
    s = warp_sum(s);
    c = warp_sum(c);
    if (lane_id() == 0) {
        atomicAdd(acc, s);
        atomicAdd(acc + 1, c);
    }
}
__global__ void ogrid_threshold_kernel(float thr_step, const float *__restrict__ acc, float *__restrict__ thr) {
    const float mean = acc[1] > 0.f ? acc[0] / acc[1] : 0.f;
    *thr = fminf(thr_step, mean);
}

// types.py:1241-1362 for pinhole cameras: a cell stays trainable if any of its 8 corners lies in
// front of some training camera and projects inside its image; other cells get density -1.
__global__ void ogrid_mark_untrained_kernel(std::uint32_t K, std::uint32_t G, float bound, std::uint32_t n_views,
                                            const float *__restrict__ transforms, float fx, float fy, float cx,
                                            float cy, std::uint32_t width, std::uint32_t height,
                                            float *__restrict__ density) {
    const std::uint32_t G3 = G * G * G;
    const std::size_t n = (std::size_t)K * G3;
    for (std::size_t i = (std::size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (std::size_t)gridDim.x * blockDim.x) {
        const std::uint32_t level = (std::uint32_t)(i / G3), c = (std::uint32_t)(i % G3);
        const float mip_bound = fminf((float)(1u << level), bound);
        const float cw = 2.f * mip_bound / (float)G;
        const float gx = ((float)morton_decode(c) / (float)G - 0.5f) * 2.f * mip_bound;
        const float gy = ((float)morton_decode(c >> 1) / (float)G - 0.5f) * 2.f * mip_bound;
        const float gz = ((float)morton_decode(c >> 2) / (float)G - 0.5f) * 2.f * mip_bound;
        bool alive = false;
        for (std::uint32_t v = 0; v < n_views && !alive; ++v) {
            const float *T = transforms + (std::size_t)v * 12;
            for (int k = 0; k < 8 && !alive; ++k) {
                const float px = gx + cw * ((k >> 2) & 1) - T[9];
                const float py = gy + cw * ((k >> 1) & 1) - T[10];
                const float pz = gz + cw * (k & 1) - T[11];
                // p_cam = R^T p
                const float qx = px * T[0] + py * T[3] + pz * T[6];
                const float qy = px * T[1] + py * T[4] + pz * T[7];
                const float qz = px * T[2] + py * T[5] + pz * T[8];
                if (!(qz < 0.f)) continue;
                const float u = (qx / -qz * fx + cx) / (float)width;
                const float w = (qy / -qz * fy + cy) / (float)height;
                alive = u >= 0.f && u < 1.f && w >= 0.f && w < 1.f;
            }
        }
        if (!alive) density[i] = -1.f;
    }
}

}  // namespace

int launch_ogrid_decay(cudaStream_t stream, std::uint32_t n, float decay, float *density) {
    if (n > 0) {
        ogrid_decay_kernel<<<grid_for(n, 256, 8), 256, 0, stream>>>(n, decay, density);
        count_launches(1);
    }
    return launch_status();
}

int launch_ogrid_sample(cudaStream_t stream, std::uint32_t M, bool update_all, std::uint32_t cas, std::uint32_t G,
                        float bound, std::uint64_t seed, const float *density, const std::uint8_t *bits,
                        std::uint32_t *cells, float *xyz) {
    NGP_CHECK_ARG(G >= 2 && G <= 1024 && (G & (G - 1)) == 0, "ogrid: G must be a power of two in [2, 1024]");
    if (M > 0) {
        ogrid_sample_kernel<<<(M + 255) / 256, 256, 0, stream>>>(M, update_all ? 1u : 0u, cas, G, bound, seed, density,
                                                                bits, cells, xyz);
        count_launches(1);
    }
    return launch_status();
}

int launch_ogrid_max(cudaStream_t stream, std::uint32_t M, std::uint32_t cas, std::uint32_t G3,
                     const std::uint32_t *cells, const float *sigma, float *density) {
    if (M > 0) {
        ogrid_max_kernel<<<(M + 255) / 256, 256, 0, stream>>>(M, cas, G3, cells, sigma, density);
        count_launches(1);
    }
    return launch_status();
}

// `acc` is a 2-float scratch accumulator.
int launch_ogrid_threshold(cudaStream_t stream, std::uint32_t n_cas0, float thr_step, const float *density,
                           float *acc, float *thr) {
    NGP_CUDA_TRY(cudaMemsetAsync(acc, 0, 2 * sizeof(float), stream));
    ogrid_mean_kernel<<<grid_for(n_cas0, 256, 4), 256, 0, stream>>>(n_cas0, density, acc);
    count_launches(1);
    ogrid_threshold_kernel<<<1, 1, 0, stream>>>(thr_step, acc, thr);
    count_launches(1);
    return launch_status();
}

int launch_ogrid_mark_untrained(cudaStream_t stream, std::uint32_t K, std::uint32_t G, float bound,
                                std::uint32_t n_views, const float *transforms, float fx, float fy, float cx,
                                float cy, std::uint32_t width, std::uint32_t height, float *density) {
    NGP_CHECK_ARG(G >= 2 && G <= 1024 && (G & (G - 1)) == 0 && K >= 1 && K <= 16, "ogrid: bad K or G");
    ogrid_mark_untrained_kernel<<<grid_for((std::size_t)K * G * G * G, 256, 8), 256, 0, stream>>>(
        K, G, bound, n_views, transforms, fx, fy, cx, cy, width, height, density);
    count_launches(1);
    return launch_status();
}

int launch_train_rays(cudaStream_t stream, const NgpTrainRaysDescriptor &d, const float *transforms,
                      const std::uint8_t *rgbas, const std::uint32_t *perm, float *rays_o, float *rays_d,
                      float *t_starts, float *t_ends, float *noises, float *bgs, float *gt) {
    NGP_CHECK_ARG(d.width > 0 && d.height > 0 && d.n_views > 0 && d.bound > 0.f, "train_rays: bad camera");
    NGP_CHECK_ARG(((std::uintptr_t)rgbas & 3u) == 0, "train_rays: rgbas must be 4-byte aligned");
    if (d.n_rays > 0) {
        train_rays_kernel<<<(d.n_rays + 255) / 256, 256, 0, stream>>>(d, transforms, rgbas, perm, rays_o, rays_d,
                                                                     t_starts, t_ends, noises, bgs, gt);
        count_launches(1);
    }
    return launch_status();
}

// `scratch` holds 4 + n_rays words: the 3 loss sums (f32), the count of rays with samples (u32)
// and their list (u32).
int launch_integrate_loss_backward(cudaStream_t stream, const NgpIntegrateLossDescriptor &d, const bool *valid,
                                   const std::uint32_t *startidx, const std::uint32_t *n_samples,
                                   const float *bgs, const float *gt, const float *dss, const float *z_vals,
                                   const float *drgbs, const std::uint32_t *count, float *dL_ddrgbs,
                                   float *stats, float *grad_scale, float *scratch) {
    NGP_CHECK_ARG(((std::uintptr_t)drgbs & 15u) == 0 && ((std::uintptr_t)dL_ddrgbs & 15u) == 0,
                  "integrate_loss_backward: drgbs and dL_ddrgbs must be 16-byte aligned");
    float *acc = scratch;
    std::uint32_t *heavy_count = reinterpret_cast<std::uint32_t *>(scratch + 3);
    std::uint32_t *heavy = heavy_count + 1;
    NGP_CUDA_TRY(cudaMemsetAsync(scratch, 0, 4 * sizeof(float), stream));
    if (d.n_rays > 0) {
        integrate_loss_light_kernel<<<(d.n_rays + kIlbLight - 1) / kIlbLight, kIlbLight, 0, stream>>>(
            d.n_rays, d.total_samples, d.huber_delta, valid, startidx, n_samples, bgs, gt, acc, heavy_count, heavy);
        const unsigned warps = (d.n_rays + 31) / 32;
        const unsigned blocks_max = (warps + kIlbWarps - 1) / kIlbWarps;
        const unsigned cap = (unsigned)sm_count() * 16;
        integrate_loss_heavy_kernel<<<blocks_max < cap ? blocks_max : cap, 32 * kIlbWarps, 0, stream>>>(
            d.total_samples, d.near_distance, d.huber_delta, valid, startidx, n_samples, bgs, gt, dss, z_vals, drgbs,
            heavy_count, heavy, dL_ddrgbs, acc);
        count_launches(2);
    }
    if (d.total_samples > 0) {
        zero_tail4_kernel<<<grid_for(d.total_samples, 256, 4), 256, 0, stream>>>(
            d.total_samples, count, reinterpret_cast<float4 *>(dL_ddrgbs));
        count_launches(1);
    }
    finalize_loss_kernel<<<1, 1, 0, stream>>>(acc, count, stats, grad_scale);
    count_launches(1);
    return launch_status();
}

int launch_adam(cudaStream_t stream, const NgpAdamDescriptor &d, float *p, float *g, float *m, float *v) {
    NGP_CHECK_ARG(d.step >= 1, "adam: step is 1-based");
    NGP_CHECK_ARG((((std::uintptr_t)p | (std::uintptr_t)g | (std::uintptr_t)m | (std::uintptr_t)v) & 15u) == 0,
                  "adam: buffers must be 16-byte aligned");
    const float bc1 = 1.f - powf(d.beta1, (float)d.step);
    const float bc2 = 1.f - powf(d.beta2, (float)d.step);
    if (d.n > 0) {
        adam_kernel<<<grid_for(d.n / 4 + 1, 256, 8), 256, 0, stream>>>(d, bc1, bc2, p, g, m, v);
        count_launches(1);
    }
    return launch_status();
}

int launch_adam_mixed(cudaStream_t stream, const NgpAdamDescriptor &d, std::uint32_t half_copy, float *p, float *g,
                      float *m, float *v, const NgpLossScale *ls, void *ph) {
    NGP_CHECK_ARG(d.step >= 1, "adam: step is 1-based");
    NGP_CHECK_ARG((((std::uintptr_t)p | (std::uintptr_t)g | (std::uintptr_t)m | (std::uintptr_t)v) & 15u) == 0,
                  "adam: buffers must be 16-byte aligned");
    NGP_CHECK_ARG(half_copy == NGP_DTYPE_F32 || half_copy == NGP_DTYPE_BF16 || half_copy == NGP_DTYPE_F16,
                  "adam: unknown half-copy type");
    NGP_CHECK_ARG(half_copy == NGP_DTYPE_F32 || (ph != nullptr && ((std::uintptr_t)ph & 7u) == 0),
                  "adam: the 16-bit copy must be given and 8-byte aligned");
    const float bc1 = 1.f - powf(d.beta1, (float)d.step);
    const float bc2 = 1.f - powf(d.beta2, (float)d.step);
    if (d.n > 0) {
        const unsigned grid = grid_for(d.n / 4 + 1, 256, 8);
        if (half_copy == NGP_DTYPE_BF16)
            adam_mixed_kernel<(int)NGP_DTYPE_BF16><<<grid, 256, 0, stream>>>(d, bc1, bc2, p, g, m, v, ls, ph);
        else if (half_copy == NGP_DTYPE_F16)
            adam_mixed_kernel<(int)NGP_DTYPE_F16><<<grid, 256, 0, stream>>>(d, bc1, bc2, p, g, m, v, ls, ph);
        else
            adam_mixed_kernel<0><<<grid, 256, 0, stream>>>(d, bc1, bc2, p, g, m, v, ls, ph);
        count_launches(1);
    }
    return launch_status();
}

int launch_loss_scale_update(cudaStream_t stream, const NgpLossScaleDescriptor &d, NgpLossScale *ls) {
    NGP_CHECK_ARG(ls != nullptr && ((std::uintptr_t)ls & 3u) == 0, "loss scale: state buffer missing or misaligned");
    NGP_CHECK_ARG(d.growth_interval >= 1 && d.growth_factor >= 1.f && d.backoff_factor > 0.f && d.backoff_factor <= 1.f &&
                      d.min_scale > 0.f && d.max_scale >= d.min_scale,
                  "loss scale: bad descriptor");
    loss_scale_update_kernel<<<1, 1, 0, stream>>>(d, ls);
    count_launches(1);
    return launch_status();
}

}  // namespace ngp
