/*
 * CPU oracle for the volume-rendering ops of the NeRF hot path.  TEST INFRASTRUCTURE ONLY:
 * nothing in the product path links, loads or calls this file; only tests/, the smoke check and
 * the CPU baseline leg of bench.py do, and only as the checker.
 *
 * This is a plain-C restatement of the arithmetic of volume-rendering-jax:
 *   deps/volume-rendering-jax/lib/impl/packbits.cu:9-34       pack_bits_kernel
 *   deps/volume-rendering-jax/lib/impl/marching.cu:15-98      calc_ds, mip_from_xyz, mip_from_ds,
 *                                                             floor_grid_pos, expand_bits,
 *                                                             __morton3D(_invert),
 *                                                             get_grid_pos_and_intermediates
 *   deps/volume-rendering-jax/lib/impl/marching.cu:101-268    march_rays_kernel
 *   deps/volume-rendering-jax/lib/impl/marching.cu:271-397    march_rays_inference_kernel
 *   deps/volume-rendering-jax/lib/impl/marching.cu:399-433    morton3d(_invert)_kernel
 *   deps/volume-rendering-jax/lib/impl/integrating.cu:24-104  integrate_rays_kernel
 *   deps/volume-rendering-jax/lib/impl/integrating.cu:106-240 integrate_rays_backward_kernel
 *   deps/volume-rendering-jax/lib/impl/integrating.cu:242-322 integrate_rays_inference_kernel
 *
 * Floating point: one IEEE-754 binary32 rounding per operation, in the reference's operation
 * order.  The recipe compiles this file with -ffp-contract=off so no multiply-add is fused (the
 * CUDA marcher is compiled the same way, so per-ray sample counts agree bit for bit).  `expf`
 * stands in for the reference's `__expf`, so integrator outputs agree to a tolerance only.
 *
 * Atomic slot assignment (march_rays) and ray refill (march_rays_inference) are taken in ray /
 * slot index order, which is one legal schedule of the reference's atomics.  Parity tests compare
 * per ray, and only where no ray overflows the sample budget.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define SQRT3_F 1.732050807568877293527446341505872367f
#define T_THRESHOLD 1e-4f

/* ---------------------------------------------------------------- helpers (marching.cu:15-98) */

static inline float clampf_(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }
static inline int clampi_(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
static inline float signf_(float x) { return copysignf(1.0f, x); }

/* marching.cu:15-23 */
static inline float calc_ds(float ray_t, float stepsize_portion, float bound, float inv_grid_res,
                            uint32_t diagonal_n_steps) {
    return clampf_(ray_t * stepsize_portion,
                   2.0f * SQRT3_F * fminf(bound, 1.0f) / (float)diagonal_n_steps,
                   2.0f * SQRT3_F * bound * inv_grid_res);
}

/* marching.cu:25-31 */
static inline uint32_t mip_from_xyz(float x, float y, float z, uint32_t K) {
    if (K == 1) return 0;
    float const m = fmaxf(fabsf(x), fmaxf(fabsf(y), fabsf(z)));
    int e;
    frexpf(m, &e);
    return (uint32_t)clampi_(e, 0, (int)K - 1);
}

/* marching.cu:34-39 */
static inline uint32_t mip_from_ds(float ds, uint32_t G, uint32_t K) {
    if (K == 1) return 0;
    int e;
    frexpf(ds * (float)G, &e);
    return (uint32_t)clampi_(e, 0, (int)K - 1);
}

/* marching.cu:52-58 */
static inline uint32_t expand_bits(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

/* marching.cu:60-65 */
static inline uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
    return expand_bits(x) | (expand_bits(y) << 1) | (expand_bits(z) << 2);
}

/* marching.cu:70-77 */
static inline uint32_t morton3_invert(uint32_t x) {
    x = x & 0x49249249u;
    x = (x | (x >> 2)) & 0xc30c30c3u;
    x = (x | (x >> 4)) & 0x0f00f00fu;
    x = (x | (x >> 8)) & 0xff0000ffu;
    x = (x | (x >> 16)) & 0x0000ffffu;
    return x;
}

typedef struct { float x, y, z; } v3f;

/* marching.cu:79-98 followed by floor_grid_pos (:41-50) and the Morton lookup (:174-176).
 * Returns whether the cell is occupied; also returns the continuous grid position and mip bound
 * (needed by the empty-space skip). */
static inline int lookup(v3f pos, float ds, float bound, uint32_t K, uint32_t G,
                         const uint8_t *bitfield, v3f *grid_posf, float *mip_bound) {
    uint32_t const c0 = mip_from_xyz(pos.x, pos.y, pos.z, K);
    uint32_t const c1 = mip_from_ds(ds, G, K);
    uint32_t const cascade = c0 > c1 ? c0 : c1;
    float const mb = fminf(scalbnf(1.0f, (int)cascade), bound);
    float const Gf = (float)G;
    v3f g;
    g.x = ((pos.x / mb + 1.0f) * 0.5f) * Gf;
    g.y = ((pos.y / mb + 1.0f) * 0.5f) * Gf;
    g.z = ((pos.z / mb + 1.0f) * 0.5f) * Gf;
    uint32_t const gx = (uint32_t)clampi_((int)floorf(g.x), 0, (int)G - 1);
    uint32_t const gy = (uint32_t)clampi_((int)floorf(g.y), 0, (int)G - 1);
    uint32_t const gz = (uint32_t)clampi_((int)floorf(g.z), 0, (int)G - 1);
    uint32_t const idx = cascade * (G * G * G) + morton3(gx, gy, gz);
    *grid_posf = g;
    *mip_bound = mb;
    return (bitfield[idx >> 3] & (1u << (idx & 7u))) != 0;
}

/* marching.cu:182-189 (and :257-264, :352-359): skip to the next voxel boundary. */
static inline float skip_empty(float ray_t, v3f g, float mb, v3f pos, v3f d, v3f inv_d,
                               float inv_G, float sp, float bound, uint32_t dns) {
    float new_t = ray_t + calc_ds(ray_t, sp, bound, inv_G, dns);
    v3f ng, delta;
    ng.x = floorf((g.x + 0.5f) + 0.5f * signf_(d.x));
    ng.y = floorf((g.y + 0.5f) + 0.5f * signf_(d.y));
    ng.z = floorf((g.z + 0.5f) + 0.5f * signf_(d.z));
    delta.x = (((ng.x * inv_G - 0.5f) * 2.0f) * mb - pos.x) * inv_d.x;
    delta.y = (((ng.y * inv_G - 0.5f) * 2.0f) * mb - pos.y) * inv_d.y;
    delta.z = (((ng.z * inv_G - 0.5f) * 2.0f) * mb - pos.z) * inv_d.z;
    float const next_t = ray_t + fmaxf(0.0f, fminf(delta.x, fminf(delta.y, delta.z)));
    while (new_t < next_t) new_t += calc_ds(new_t, sp, bound, inv_G, dns);
    return new_t;
}

static inline v3f ray_at(v3f o, v3f d, float t) {
    v3f p = {o.x + t * d.x, o.y + t * d.y, o.z + t * d.z};
    return p;
}

/* ---------------------------------------------------------------------- packbits / morton */

/* packbits.cu:9-34 */
void oracle_packbits(uint32_t n_bytes, const float *thr, const float *density, uint8_t *occ_mask,
                     uint8_t *bitfield) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n_bytes; ++i) {
        uint8_t byte = 0;
        for (int k = 0; k < 8; ++k) {
            int const p = density[i * 8 + k] > thr[i * 8 + k];
            occ_mask[i * 8 + k] = (uint8_t)p;
            byte |= p ? (uint8_t)(1u << k) : 0u;
        }
        bitfield[i] = byte;
    }
}

/* marching.cu:399-414 */
void oracle_morton3d(uint32_t n, const uint32_t *xyz, uint32_t *idcs) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) idcs[i] = morton3(xyz[i * 3], xyz[i * 3 + 1], xyz[i * 3 + 2]);
}

/* marching.cu:416-433 */
void oracle_morton3d_invert(uint32_t n, const uint32_t *idcs, uint32_t *xyz) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        xyz[i * 3 + 0] = morton3_invert(idcs[i] >> 0);
        xyz[i * 3 + 1] = morton3_invert(idcs[i] >> 1);
        xyz[i * 3 + 2] = morton3_invert(idcs[i] >> 2);
    }
}

/* ------------------------------------------------------------------------------ march_rays */

typedef struct {
    uint32_t n_rays, total_samples, diagonal_n_steps, K, G;
    float bound, stepsize_portion;
} MarchDesc;

/* One ray of marching.cu:101-268.  When `write` is zero only the sample count is returned
 * (first pass, :162-192); otherwise up to `n_max` samples are written (second pass, :224-267). */
static uint32_t march_one(const MarchDesc *dsc, v3f o, v3f d, float t0, float t1, float noise,
                          const uint8_t *bitfield, int write, uint32_t n_max, uint32_t ray_index,
                          uint32_t *idcs, float *xyzs, float *dirs, float *dss, float *zs) {
    float const inv_G = 1.0f / (float)dsc->G;
    v3f const inv_d = {1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
    float const sp = dsc->stepsize_portion, bound = dsc->bound;
    uint32_t const dns = dsc->diagonal_n_steps;
    uint32_t n = 0;
    float ray_t = t0;
    ray_t += calc_ds(ray_t, sp, bound, inv_G, dns) * noise;
    for (;;) {
        if (write) {
            if (!(n < n_max && ray_t < t1)) break;
        } else {
            if (!((float)n < (float)dns * bound && ray_t < t1)) break;
        }
        v3f const pos = ray_at(o, d, ray_t);
        float const ds = calc_ds(ray_t, sp, bound, inv_G, dns);
        v3f g;
        float mb;
        int const occ = lookup(pos, ds, bound, dsc->K, dsc->G, bitfield, &g, &mb);
        if (occ) {
            if (write) {
                idcs[n] = ray_index;
                xyzs[n * 3 + 0] = pos.x; xyzs[n * 3 + 1] = pos.y; xyzs[n * 3 + 2] = pos.z;
                dirs[n * 3 + 0] = d.x;   dirs[n * 3 + 1] = d.y;   dirs[n * 3 + 2] = d.z;
                dss[n] = ds;
                zs[n] = ray_t;
            }
            ++n;
            ray_t = ray_t + ds;
        } else {
            ray_t = skip_empty(ray_t, g, mb, pos, d, inv_d, inv_G, sp, bound, dns);
        }
    }
    return n;
}

/* Outputs must be zero-filled by the caller, as the reference launcher does (marching.cu:474-483).
 * counters[0] = next_sample_write_location, counters[1] = number_of_exceeded_samples.
 * With early_exit, rays are taken one after another in ray order, and a ray that starts after the
 * buffer filled is dropped (marching.cu:135) -- the reference run one thread at a time.  Without
 * it, every ray is counted before any is placed, and only then are slots taken in ray order --
 * the reference when its whole grid is resident. */
void oracle_march_rays_ex(uint32_t n_rays, uint32_t total_samples, uint32_t diagonal_n_steps,
                       uint32_t K, uint32_t G, float bound, float stepsize_portion,
                       const float *rays_o, const float *rays_d, const float *t_starts,
                       const float *t_ends, const float *noises, const uint8_t *bitfield,
                       uint32_t *counters, uint8_t *ray_is_valid, uint32_t *rays_n_samples,
                       uint32_t *rays_sample_startidx, uint32_t *idcs, float *xyzs, float *dirs,
                       float *dss, float *z_vals, int early_exit) {
    MarchDesc const dsc = {n_rays, total_samples, diagonal_n_steps, K, G, bound, stepsize_portion};
    uint32_t *cnt = (uint32_t *)calloc(n_rays ? n_rays : 1, sizeof(uint32_t));
    uint8_t *live = (uint8_t *)calloc(n_rays ? n_rays : 1, 1);

#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)n_rays; ++i) {
        v3f const o = {rays_o[i * 3], rays_o[i * 3 + 1], rays_o[i * 3 + 2]};
        v3f const d = {rays_d[i * 3], rays_d[i * 3 + 1], rays_d[i * 3 + 2]};
        if (t_ends[i] <= t_starts[i]) { live[i] = 0; continue; }  /* :151 */
        live[i] = 1;
        cnt[i] = march_one(&dsc, o, d, t_starts[i], t_ends[i], noises[i], bitfield, 0, 0, 0,
                           NULL, NULL, NULL, NULL, NULL);
    }

    /* atomics of :135 and :205-209 taken in ray order */
    uint32_t loc = 0, exceeded = 0;
    for (uint32_t i = 0; i < n_rays; ++i) {
        if (early_exit && loc >= total_samples) { cnt[i] = 0; live[i] = 2; continue; }  /* :135 */
        if (!live[i]) continue;                                          /* :151 */
        if (cnt[i] == 0) { ray_is_valid[i] = 1; continue; }              /* :196-199 */
        uint32_t const start = loc;
        loc += cnt[i];
        if ((uint64_t)start + cnt[i] > total_samples) {
            exceeded += cnt[i];
            cnt[i] = 0;
            continue;
        }
        rays_n_samples[i] = cnt[i];
        ray_is_valid[i] = 1;
        rays_sample_startidx[i] = start;
    }
    counters[0] = loc;
    counters[1] = exceeded;

#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)n_rays; ++i) {
        uint32_t const n = rays_n_samples[i];
        if (n == 0) continue;
        uint32_t const s = rays_sample_startidx[i];
        v3f const o = {rays_o[i * 3], rays_o[i * 3 + 1], rays_o[i * 3 + 2]};
        v3f const d = {rays_d[i * 3], rays_d[i * 3 + 1], rays_d[i * 3 + 2]};
        march_one(&dsc, o, d, t_starts[i], t_ends[i], noises[i], bitfield, 1, n, (uint32_t)i,
                  idcs + s, xyzs + (size_t)s * 3, dirs + (size_t)s * 3, dss + s, z_vals + s);
    }
    free(cnt);
    free(live);
}

void oracle_march_rays(uint32_t n_rays, uint32_t total_samples, uint32_t diagonal_n_steps,
                       uint32_t K, uint32_t G, float bound, float stepsize_portion,
                       const float *rays_o, const float *rays_d, const float *t_starts,
                       const float *t_ends, const float *noises, const uint8_t *bitfield,
                       uint32_t *counters, uint8_t *ray_is_valid, uint32_t *rays_n_samples,
                       uint32_t *rays_sample_startidx, uint32_t *idcs, float *xyzs, float *dirs,
                       float *dss, float *z_vals) {
    oracle_march_rays_ex(n_rays, total_samples, diagonal_n_steps, K, G, bound, stepsize_portion, rays_o,
                         rays_d, t_starts, t_ends, noises, bitfield, counters, ray_is_valid,
                         rays_n_samples, rays_sample_startidx, idcs, xyzs, dirs, dss, z_vals, 1);
}

/* marching.cu:271-397.  Slots are processed in index order; terminated slots take the next ray
 * index in that order.  Outputs must be zero-filled by the caller (marching.cu:565-570);
 * next_ray_index must hold the input counter (marching.cu:561). */
void oracle_march_rays_inference(uint32_t n_total_rays, uint32_t n_rays, uint32_t diagonal_n_steps,
                                 uint32_t K, uint32_t G, uint32_t march_steps_cap, float bound,
                                 float stepsize_portion, const float *rays_o, const float *rays_d,
                                 const float *t_starts, const float *t_ends,
                                 const uint8_t *bitfield, const uint8_t *terminated,
                                 const uint32_t *indices_in, uint32_t *next_ray_index,
                                 uint32_t *indices_out, uint32_t *n_samples, float *t_starts_out,
                                 float *xyzs, float *dss, float *z_vals) {
    uint32_t *ridx = (uint32_t *)malloc((n_rays ? n_rays : 1) * sizeof(uint32_t));
    for (uint32_t i = 0; i < n_rays; ++i)
        ridx[i] = terminated[i] ? (*next_ray_index)++ : indices_in[i];
    float const inv_G = 1.0f / (float)G;
    uint32_t const G3 = G * G * G;
    (void)G3;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)n_rays; ++i) {
        uint32_t const r = ridx[i];
        indices_out[i] = r;
        if (r >= n_total_rays) continue;
        v3f const o = {rays_o[(size_t)r * 3], rays_o[(size_t)r * 3 + 1], rays_o[(size_t)r * 3 + 2]};
        v3f const d = {rays_d[(size_t)r * 3], rays_d[(size_t)r * 3 + 1], rays_d[(size_t)r * 3 + 2]};
        float const t0 = t_starts[r], t1 = t_ends[r];
        if (t1 < t0) continue;  /* :317 */
        float *rx = xyzs + (size_t)i * march_steps_cap * 3;
        float *rds = dss + (size_t)i * march_steps_cap;
        float *rz = z_vals + (size_t)i * march_steps_cap;
        v3f const inv_d = {1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
        uint32_t steps = 0;
        float ray_t = t0;
        while (steps < march_steps_cap && ray_t < t1) {
            v3f const pos = ray_at(o, d, ray_t);
            float const ds = calc_ds(ray_t, stepsize_portion, bound, inv_G, diagonal_n_steps);
            v3f g;
            float mb;
            if (lookup(pos, ds, bound, K, G, bitfield, &g, &mb)) {
                rx[steps * 3 + 0] = pos.x; rx[steps * 3 + 1] = pos.y; rx[steps * 3 + 2] = pos.z;
                rds[steps] = ds;
                rz[steps] = ray_t;
                ++steps;
                ray_t = ray_t + ds;
            } else {
                ray_t = skip_empty(ray_t, g, mb, pos, d, inv_d, inv_G, stepsize_portion, bound,
                                   diagonal_n_steps);
            }
        }
        if (ray_t >= t1) {  /* :367-394 far-plane sample */
            v3f const pos = ray_at(o, d, t1);
            float const ds = calc_ds(t1, stepsize_portion, bound, inv_G, diagonal_n_steps);
            v3f g;
            float mb;
            if (lookup(pos, ds, bound, K, G, bitfield, &g, &mb)) {
                if (steps > 0 && rds[steps - 1] + rz[steps - 1] >= t1) rds[steps - 1] = t1 - rz[steps - 1];
                if (steps < march_steps_cap) {
                    rx[steps * 3 + 0] = pos.x; rx[steps * 3 + 1] = pos.y; rx[steps * 3 + 2] = pos.z;
                    rds[steps] = ds;
                    rz[steps] = t1;
                    ++steps;
                } else {
                    ray_t = t1;
                }
            }
        }
        n_samples[i] = steps;
        t_starts_out[i] = ray_t;
    }
    free(ridx);
}

/* -------------------------------------------------------------------------- integrate_rays */

/* integrating.cu:24-104.  measured_batch_size is the sum over rays of the number of samples
 * composited before early termination (:98-103). */
void oracle_integrate_rays(uint32_t n_rays, const uint32_t *startidx, const uint32_t *n_samples,
                           const float *bgs, const float *dss, const float *z_vals,
                           const float *drgbs, uint32_t *measured_batch_size, float *final_rgbds,
                           float *final_opacities) {
    uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : total)
    for (int64_t i = 0; i < (int64_t)n_rays; ++i) {
        uint32_t const s = startidx[i], n = n_samples[i];
        const float *rd = dss + s, *rz = z_vals + s, *rc = drgbs + (size_t)s * 4;
        uint32_t k = 0;
        float depth = 0.f, T = 1.f, r = 0.f, g = 0.f, b = 0.f;
        for (; T > T_THRESHOLD && k < n; ++k) {
            float const alpha = 1.f - expf(-rc[k * 4] * rd[k]);
            float const w = T * alpha;
            r += w * rc[k * 4 + 1];
            g += w * rc[k * 4 + 2];
            b += w * rc[k * 4 + 3];
            depth += w * rz[k];
            T *= 1.f - alpha;
        }
        float const opacity = 1.f - T;
        final_opacities[i] = opacity;
        if (T <= T_THRESHOLD) {
            float const id = 1.f / opacity;
            final_rgbds[i * 4 + 0] = r * id;
            final_rgbds[i * 4 + 1] = g * id;
            final_rgbds[i * 4 + 2] = b * id;
            final_rgbds[i * 4 + 3] = depth * id;
        } else {
            final_rgbds[i * 4 + 0] = r + T * bgs[i * 3 + 0];
            final_rgbds[i * 4 + 1] = g + T * bgs[i * 3 + 1];
            final_rgbds[i * 4 + 2] = b + T * bgs[i * 3 + 2];
            final_rgbds[i * 4 + 3] = depth;
        }
        total += k;
    }
    *measured_batch_size = (uint32_t)total;
}

/* integrating.cu:106-240.  Outputs must be zero-filled by the caller (:412-414). */
void oracle_integrate_rays_backward(uint32_t n_rays, float near_distance, const uint32_t *startidx,
                                    const uint32_t *n_samples, const float *bgs, const float *dss,
                                    const float *z_vals, const float *drgbs,
                                    const float *final_rgbds, const float *final_opacities,
                                    const float *dL_dfinal_rgbds, float *dL_dbgs, float *dL_dz_vals,
                                    float *dL_ddrgbs) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n_rays; ++i) {
        uint32_t const s = startidx[i], n = n_samples[i];
        const float *bg = bgs + i * 3, *rd = dss + s, *rz = z_vals + s, *rc = drgbs + (size_t)s * 4;
        float const fr[4] = {final_rgbds[i * 4], final_rgbds[i * 4 + 1], final_rgbds[i * 4 + 2],
                             final_rgbds[i * 4 + 3]};
        float const fo = final_opacities[i];
        int const terminated = fo >= 1.f - T_THRESHOLD;
        float const go[4] = {dL_dfinal_rgbds[i * 4], dL_dfinal_rgbds[i * 4 + 1],
                             dL_dfinal_rgbds[i * 4 + 2], dL_dfinal_rgbds[i * 4 + 3]};
        float *gz = dL_dz_vals + s, *gc = dL_ddrgbs + (size_t)s * 4;
        float T = 1.f, cr = 0.f, cg = 0.f, cb = 0.f, cd = 0.f;
        float const bgterm = terminated ? 0.f : 1.f - fo;
        for (uint32_t k = 0; T > T_THRESHOLD && k < n; ++k) {
            float const z = rz[k], dt = rd[k], sigma = rc[k * 4];
            float const alpha = 1.f - expf(-sigma * dt);
            float const w = T * alpha;
            cr += w * rc[k * 4 + 1];
            cg += w * rc[k * 4 + 2];
            cb += w * rc[k * 4 + 3];
            cd += w * z;
            T *= 1.f - alpha;
            gz[k] = w * go[3];
            float const dsig = dt * (go[0] * (T * rc[k * 4 + 1] - (fr[0] - cr) - bg[0] * bgterm)
                                   + go[1] * (T * rc[k * 4 + 2] - (fr[1] - cg) - bg[1] * bgterm)
                                   + go[2] * (T * rc[k * 4 + 3] - (fr[2] - cb) - bg[2] * bgterm)
                                   + go[3] * (T * z - (fr[3] - cd)));
            float const reg = (sigma > 4e-5 && z < near_distance) ? 1e-4f : 0.0f;
            float const scale = fminf(z * z, 1.f);
            gc[k * 4 + 0] = scale * dsig + reg;
            gc[k * 4 + 1] = w * go[0];
            gc[k * 4 + 2] = w * go[1];
            gc[k * 4 + 3] = w * go[2];
        }
        if (T > T_THRESHOLD) {
            dL_dbgs[i * 3 + 0] = T * go[0];
            dL_dbgs[i * 3 + 1] = T * go[1];
            dL_dbgs[i * 3 + 2] = T * go[2];
        }
    }
}

/* integrating.cu:242-322.  Outputs must be zero-filled by the caller (:478-482). */
void oracle_integrate_rays_inference(uint32_t n_total_rays, uint32_t n_rays, uint32_t cap,
                                     const float *rays_bg, const float *rays_rgbd,
                                     const float *rays_T, const uint32_t *n_samples,
                                     const uint32_t *indices, const float *dss, const float *z_vals,
                                     const float *drgbs, uint32_t *terminate_cnt,
                                     uint8_t *terminated, float *rgbd_out, float *T_out) {
    uint32_t cnt = 0;
#pragma omp parallel for schedule(static) reduction(+ : cnt)
    for (int64_t i = 0; i < (int64_t)n_rays; ++i) {
        uint32_t const n = n_samples[i], r = indices[i];
        if (r < n_total_rays) {
            const float *rd = dss + (size_t)i * cap, *rz = z_vals + (size_t)i * cap;
            const float *rc = drgbs + (size_t)i * cap * 4;
            float T = rays_T[r];
            float cr = rays_rgbd[(size_t)r * 4 + 0], cg = rays_rgbd[(size_t)r * 4 + 1];
            float cb = rays_rgbd[(size_t)r * 4 + 2], cd = rays_rgbd[(size_t)r * 4 + 3];
            for (uint32_t k = 0; T > T_THRESHOLD && k < n; ++k) {
                float const alpha = 1.f - expf(-rc[k * 4] * rd[k]);
                float const w = T * alpha;
                cr += w * rc[k * 4 + 1];
                cg += w * rc[k * 4 + 2];
                cb += w * rc[k * 4 + 3];
                cd += w * rz[k];
                T *= (1.f - alpha);
            }
            if (T <= T_THRESHOLD) {
                float const id = 1.f / (1.f - T);
                terminated[i] = 1;
                T_out[i] = 0.f;
                rgbd_out[i * 4 + 0] = cr * id;
                rgbd_out[i * 4 + 1] = cg * id;
                rgbd_out[i * 4 + 2] = cb * id;
                rgbd_out[i * 4 + 3] = cd * id;
            } else {
                terminated[i] = n < cap;
                rgbd_out[i * 4 + 3] = cd;
                T_out[i] = T;
                if (terminated[i]) {
                    rgbd_out[i * 4 + 0] = cr + T * rays_bg[(size_t)r * 3 + 0];
                    rgbd_out[i * 4 + 1] = cg + T * rays_bg[(size_t)r * 3 + 1];
                    rgbd_out[i * 4 + 2] = cb + T * rays_bg[(size_t)r * 3 + 2];
                } else {
                    rgbd_out[i * 4 + 0] = cr;
                    rgbd_out[i * 4 + 1] = cg;
                    rgbd_out[i * 4 + 2] = cb;
                }
            }
        }
        cnt += terminated[i] ? 1u : 0u;
    }
    *terminate_cnt = cnt;
}
