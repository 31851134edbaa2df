// Driver appended (by oracle/build_ref.sh) after the reference's marching.cu in one translation
// unit, so that the reference's own march_rays_kernel, march_rays_inference_kernel,
// morton3d_kernel and morton3d_invert_kernel run on the CPU.  TEST INFRASTRUCTURE ONLY.
// Threads run in index order (one legal schedule of the reference's atomics); callers zero the
// outputs as the reference launchers do (marching.cu:474-483, :561-570).
extern "C" {
void ref_march_rays(std::uint32_t n_rays, std::uint32_t total_samples, std::uint32_t dns,
                    std::uint32_t K, std::uint32_t G, float bound, float sp, const float *o,
                    const float *d, const float *t0, const float *t1, const float *noise,
                    const std::uint8_t *bits, std::uint32_t *next_loc, std::uint32_t *n_exceeded,
                    bool *valid, std::uint32_t *n_samples, std::uint32_t *startidx,
                    std::uint32_t *idcs, float *xyzs, float *dirs, float *dss, float *zs) {
    run_grid((n_rays + 511) / 512, 512, false, [&]() {
        volrendjax::march_rays_kernel(n_rays, total_samples, dns, K, G, bound, sp, o, d, t0, t1,
                                      noise, bits, next_loc, n_exceeded, valid, n_samples,
                                      startidx, idcs, xyzs, dirs, dss, zs);
    });
}
void ref_march_rays_inference(std::uint32_t n_total, std::uint32_t n_rays, std::uint32_t dns,
                              std::uint32_t K, std::uint32_t G, std::uint32_t cap, float bound,
                              float sp, const float *o, const float *d, const float *t0,
                              const float *t1, const std::uint8_t *bits, const bool *terminated,
                              const std::uint32_t *indices_in, std::uint32_t *next_ray_index,
                              std::uint32_t *indices_out, std::uint32_t *n_samples,
                              float *t_out, float *xyzs, float *dss, float *zs) {
    run_grid((n_rays + 511) / 512, 512, false, [&]() {
        volrendjax::march_rays_inference_kernel(n_total, n_rays, dns, K, G, cap, bound, sp, o, d,
                                                t0, t1, bits, terminated, indices_in,
                                                next_ray_index, indices_out, n_samples, t_out,
                                                xyzs, dss, zs);
    });
}
void ref_morton3d(std::uint32_t n, const std::uint32_t *xyz, std::uint32_t *idcs) {
    run_grid((n + 511) / 512, 512, false, [&]() { volrendjax::morton3d_kernel(n, xyz, idcs); });
}
void ref_morton3d_invert(std::uint32_t n, const std::uint32_t *idcs, std::uint32_t *xyz) {
    run_grid((n + 511) / 512, 512, false,
             [&]() { volrendjax::morton3d_invert_kernel(n, idcs, xyz); });
}
}
