// Driver appended (by oracle/build_ref.sh) after the reference's integrating.cu in one
// translation unit, so that the reference's own integrate_rays_kernel,
// integrate_rays_backward_kernel and integrate_rays_inference_kernel run on the CPU.  TEST
// INFRASTRUCTURE ONLY.  Each block's threads run concurrently, so the block-shared counters and
// __syncthreads of integrating.cu:98-103 and :316-321 behave as on the GPU.  Callers zero the
// outputs as the reference launchers do (integrating.cu:351-353, :412-414, :478-482).
extern "C" {
void ref_integrate_rays(std::uint32_t n_rays, const std::uint32_t *startidx,
                        const std::uint32_t *n_samples, const float *bgs, const float *dss,
                        const float *zs, const float *drgbs, std::uint32_t *measured,
                        float *rgbds, float *opac) {
    run_grid((n_rays + 511) / 512, 512, true, [&]() {
        volrendjax::integrate_rays_kernel(n_rays, startidx, n_samples, bgs, dss, zs, drgbs,
                                          measured, rgbds, opac);
    });
}
void ref_integrate_rays_backward(std::uint32_t n_rays, float near, const std::uint32_t *startidx,
                                 const std::uint32_t *n_samples, const float *bgs,
                                 const float *dss, const float *zs, const float *drgbs,
                                 const float *rgbds, const float *opac, const float *g_rgbds,
                                 float *g_bgs, float *g_zs, float *g_drgbs) {
    run_grid((n_rays + 511) / 512, 512, false, [&]() {
        volrendjax::integrate_rays_backward_kernel(n_rays, near, startidx, n_samples, bgs, dss,
                                                   zs, drgbs, rgbds, opac, g_rgbds, g_bgs, g_zs,
                                                   g_drgbs);
    });
}
void ref_integrate_rays_inference(std::uint32_t n_total, std::uint32_t n_rays, std::uint32_t cap,
                                  const float *rays_bg, const float *rays_rgbd,
                                  const float *rays_T, const std::uint32_t *n_samples,
                                  const std::uint32_t *indices, const float *dss, const float *zs,
                                  const float *drgbs, std::uint32_t *terminate_cnt,
                                  bool *terminated, float *rgbd_out, float *T_out) {
    run_grid((n_rays + 511) / 512, 512, true, [&]() {
        volrendjax::integrate_rays_inference_kernel(n_total, n_rays, cap, rays_bg, rays_rgbd,
                                                    rays_T, n_samples, indices, dss, zs, drgbs,
                                                    terminate_cnt, terminated, rgbd_out, T_out);
    });
}
}
