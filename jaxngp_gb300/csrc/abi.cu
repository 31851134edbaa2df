// The C ABI of libngp_gb300: descriptor decoding, buffer unpacking and status handling for every
// entry point declared in include/ngp_gb300.h.  Buffer order follows volrendjax's lowering rules
// (deps/volume-rendering-jax/src/volrendjax/*/lowering.py): operands, then results.
#include <atomic>
#include <cstdio>
#include <mutex>
#include <set>
#include <tuple>

#include "common.cuh"

namespace ngp {

int launch_march_rays(cudaStream_t, const MarchingDescriptor &, const float *, const float *, const float *,
                      const float *, const float *, const std::uint8_t *, std::uint32_t *, std::uint32_t *,
                      bool *, std::uint32_t *, std::uint32_t *, std::uint32_t *, float *, float *, float *, float *,
                      std::uint32_t *, bool, const std::uint8_t *);
int launch_march_rays_inference(cudaStream_t, const MarchingInferenceDescriptor &, const float *, const float *,
                                const float *, const float *, const std::uint8_t *, const std::uint32_t *,
                                const bool *, const std::uint32_t *, std::uint32_t *, std::uint32_t *,
                                std::uint32_t *, float *, float *, float *, float *);
int launch_march_rays_inference_inplace(cudaStream_t, const MarchingInferenceDescriptor &, const float *, const float *,
                                        float *, const float *, const std::uint8_t *, const bool *, std::uint32_t *,
                                        std::uint32_t *, std::uint32_t *, std::uint32_t *, std::uint32_t *, float *,
                                        float *, float *, float *);
int launch_integrate_rays_inference_inplace(cudaStream_t, const IntegratingInferenceDescriptor &, const float *, float *,
                                            float *, const std::uint32_t *, const std::uint32_t *, const float *,
                                            const float *, const float *, const std::uint32_t *, std::uint32_t *,
                                            bool *);
int launch_morton3d(cudaStream_t, std::uint32_t, const std::uint32_t *, std::uint32_t *);
int launch_morton3d_invert(cudaStream_t, std::uint32_t, const std::uint32_t *, std::uint32_t *);
int launch_integrate_rays(cudaStream_t, const IntegratingDescriptor &, const std::uint32_t *, const std::uint32_t *,
                          const float *, const float *, const float *, const float *, std::uint32_t *, float *, float *);
int launch_integrate_rays_backward(cudaStream_t, const IntegratingBackwardDescriptor &, const std::uint32_t *,
                                   const std::uint32_t *, const float *, const float *, const float *, const float *,
                                   const float *, const float *, const float *, float *, float *, float *, bool);
int launch_integrate_rays_inference(cudaStream_t, const IntegratingInferenceDescriptor &, const float *, const float *,
                                    const float *, const std::uint32_t *, const std::uint32_t *, const float *,
                                    const float *, const float *, std::uint32_t *, bool *, float *, float *);
int launch_packbits(cudaStream_t, std::uint32_t, const float *, const float *, bool *, std::uint8_t *, bool);
int launch_sh_encoding(cudaStream_t, std::uint32_t, std::uint32_t, const float *, float *);
int launch_hashgrid_forward(cudaStream_t, const NgpHashGridDescriptor &, const std::uint32_t *, const float *,
                            const float *, float *);
int launch_hashgrid_backward(cudaStream_t, const NgpHashGridDescriptor &, const std::uint32_t *, const float *,
                             const float *, float *, bool);
int launch_integrate_rays_fp64(cudaStream_t, const IntegratingDescriptor &, const std::uint32_t *, const std::uint32_t *,
                               const float *, const float *, const float *, const float *, double *, double *,
                               std::uint32_t *);
int launch_hashgrid_tv(cudaStream_t, const NgpHashGridDescriptor &, float, const float *, const float *, const float *,
                       float *, float *, double *);
std::size_t mlp_partials_floats();
int launch_mlp_partials_reduce(cudaStream_t, unsigned, const float *, float *, bool, std::uint32_t, const std::uint32_t *,
                               float *, unsigned);
int launch_mlp_bf16_forward(cudaStream_t, std::uint32_t, const std::uint32_t *, const float *, const float *,
                            const float *, float *);
int launch_mlp_bf16_density(cudaStream_t, std::uint32_t, const float *, const float *, float *);
int launch_mlp_bf16_backward(cudaStream_t, std::uint32_t, const std::uint32_t *, const float *, const float *,
                             const float *, const float *, const float *, float *, float *, unsigned *);
int device_status();
int launch_mlp_x6_forward(cudaStream_t, std::uint32_t, const std::uint32_t *, const float *, const float *, const float *,
                          float *);
int launch_mlp_x6_density(cudaStream_t, std::uint32_t, const float *, const float *, float *);
int launch_mlp_x6_backward(cudaStream_t, std::uint32_t, const std::uint32_t *, const float *, const float *,
                           const float *, const float *, const float *, float *, float *, unsigned, unsigned *);
int launch_bounded_wait_selftest(cudaStream_t stream, std::uint32_t polls);
int set_march_blocks_per_sm(int);
int launch_proposal_judge(cudaStream_t, std::uint32_t, const std::uint32_t *, std::uint32_t, float, const float *,
                          const float *, const float *, const std::uint32_t *, const float *, const float *, const float *,
                          const std::uint8_t *, std::uint8_t *, std::uint32_t *, std::uint32_t *, std::uint32_t *);
int launch_proposal_sample_alloc(cudaStream_t, std::uint32_t, std::uint32_t, std::uint32_t *, std::uint32_t, float, bool,
                                 std::uint64_t, const float *, const float *, const std::uint32_t *, const float *,
                                 const float *, const float *, const std::uint8_t *, std::uint32_t *, std::uint32_t *,
                                 std::uint32_t *, float *, float *, float *, float *, bool *, std::uint32_t *,
                                 std::uint32_t *);
int launch_march_rays_list(cudaStream_t, const MarchingDescriptor &, const float *, const float *, const float *,
                           const float *, const float *, const std::uint8_t *, std::uint32_t *, std::uint32_t *, bool *,
                           std::uint32_t *, std::uint32_t *, std::uint32_t *, float *, float *, float *, float *,
                           std::uint32_t *, const std::uint32_t *, const std::uint32_t *);
int launch_mlp_tc_forward(cudaStream_t, std::uint32_t, bool, std::uint32_t, const std::uint32_t *, const void *,
                          const float *, const float *, float *);
int launch_mlp_tc_density(cudaStream_t, std::uint32_t, bool, std::uint32_t, const void *, const float *, float *);
int launch_mlp_tc_backward(cudaStream_t, std::uint32_t, bool, std::uint32_t, const std::uint32_t *, const void *,
                           const float *, const float *, const float *, const float *, NgpLossScale *, void *, float *,
                           unsigned *);
int launch_hashgrid_forward_mixed(cudaStream_t, const NgpHashGridDescriptor &, std::uint32_t, std::uint32_t,
                                  const std::uint32_t *, const float *, const void *, void *);
int launch_hashgrid_backward_mixed(cudaStream_t, const NgpHashGridDescriptor &, std::uint32_t, const std::uint32_t *,
                                   const float *, const void *, float *, bool);
int launch_adam_mixed(cudaStream_t, const NgpAdamDescriptor &, std::uint32_t, float *, float *, float *, float *,
                      const NgpLossScale *, void *);
int launch_loss_scale_update(cudaStream_t, const NgpLossScaleDescriptor &, NgpLossScale *);
int launch_proposal_coarse(cudaStream_t, std::uint32_t, const std::uint8_t *, std::uint8_t *);
int launch_proposal_rays(cudaStream_t, std::uint32_t, std::uint32_t, std::uint32_t, std::uint32_t, float, const float *,
                         const float *,
                         const float *, const float *, const std::uint8_t *, std::uint32_t *, std::uint32_t *, bool *,
                         std::uint32_t *, std::uint32_t *, std::uint32_t *, float *, float *, std::uint32_t *);
int launch_proposal_bin_points(cudaStream_t, std::uint32_t, const std::uint32_t *, const float *, const float *,
                               const std::uint32_t *, const float *, const float *, float *);
int launch_proposal_sample(cudaStream_t, std::uint32_t, const std::uint32_t *, std::uint32_t, float, bool, std::uint64_t,
                           const float *,
                           const float *, const std::uint32_t *, const float *, const float *, const float *,
                           std::uint32_t *, float *, float *, float *, float *);
int launch_proposal_loss(cudaStream_t, std::uint32_t, const std::uint32_t *, int, const float *, const float *, int,
                         float *, float *);
int launch_prop_forward(cudaStream_t, std::uint32_t, const std::uint32_t *, const float *, const float *, float *);
int launch_prop_backward(cudaStream_t, std::uint32_t, const std::uint32_t *, const float *, const float *, const float *,
                         float *, float *, float *, bool);
std::size_t prop_partials_floats();
int launch_prop_f16_forward(cudaStream_t, std::uint32_t, const std::uint32_t *, const float *, const float *, float *);
int launch_mlp_backward_noalloc(cudaStream_t, std::uint32_t, const std::uint32_t *, const float *, const float *,
                                const float *, const float *, const float *, float *, float *, bool);
int launch_render_blobs(cudaStream_t, const NgpRenderBlobsDescriptor &, const float *, const float *, const float *,
                        std::uint8_t *);
int launch_train_rays(cudaStream_t, const NgpTrainRaysDescriptor &, const float *, const std::uint8_t *,
                      const std::uint32_t *, float *, float *, float *, float *, float *, float *, float *);
int launch_integrate_loss_backward(cudaStream_t, const NgpIntegrateLossDescriptor &, const bool *,
                                   const std::uint32_t *, const std::uint32_t *, const float *, const float *,
                                   const float *, const float *, const float *, const std::uint32_t *, float *,
                                   float *, float *, float *);
int launch_adam(cudaStream_t, const NgpAdamDescriptor &, float *, float *, float *, float *);
int launch_ogrid_decay(cudaStream_t, std::uint32_t, float, float *);
int launch_ogrid_sample(cudaStream_t, std::uint32_t, bool, std::uint32_t, std::uint32_t, float, std::uint64_t,
                        const float *, const std::uint8_t *, std::uint32_t *, float *);
int launch_ogrid_max(cudaStream_t, std::uint32_t, std::uint32_t, std::uint32_t, const std::uint32_t *,
                     const float *, float *);
int launch_ogrid_threshold(cudaStream_t, std::uint32_t, float, const float *, float *, float *);
int launch_ogrid_mark_untrained(cudaStream_t, std::uint32_t, std::uint32_t, float, std::uint32_t, const float *,
                                float, float, float, float, std::uint32_t, std::uint32_t, float *);

namespace {
thread_local int t_status = NGP_OK;
thread_local char t_message[256] = "ok";

__global__ void march_count_kernel(const std::uint32_t *__restrict__ next_loc, const std::uint32_t *__restrict__ exceeded,
                                   std::uint32_t *__restrict__ count) {
    *count = *next_loc - *exceeded;
}
}  // namespace

static std::atomic<unsigned long long> g_launches{0};
void count_launches(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

void set_last_status(int status, const char *msg) {
    t_status = status;
    std::snprintf(t_message, sizeof(t_message), "%s", msg ? msg : "");
}

int sm_count() {
    static std::atomic<int> cached[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    int v = cached[dev].load(std::memory_order_relaxed);
    if (v == 0) {
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 152;
        cached[dev].store(v, std::memory_order_relaxed);
    }
    return v;
}

int set_smem_limit(const void *kernel, std::size_t bytes) {
    static std::mutex mu;
    static std::set<std::tuple<int, const void *, std::size_t>> done;
    int dev = 0;
    NGP_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_tuple(dev, kernel, bytes);
    if (done.count(key) != 0) return NGP_OK;
    NGP_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    done.insert(key);
    return NGP_OK;
}

}  // namespace ngp

using namespace ngp;

#define U32(i) static_cast<std::uint32_t *>(buffers[i])
#define CU32(i) static_cast<const std::uint32_t *>(buffers[i])
#define F32(i) static_cast<float *>(buffers[i])
#define CF32(i) static_cast<const float *>(buffers[i])
#define U8(i) static_cast<std::uint8_t *>(buffers[i])
#define CU8(i) static_cast<const std::uint8_t *>(buffers[i])
#define B8(i) static_cast<bool *>(buffers[i])
#define CB8(i) static_cast<const bool *>(buffers[i])

#define NGP_ENTRY(name)                                                                              \
    int name##_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);   \
    void name(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len) {          \
        name##_status(stream, buffers, opaque, opaque_len);                                          \
    }                                                                                                \
    int name##_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len)

#define NGP_DESC(T, var)                                                                             \
    T var;                                                                                           \
    do {                                                                                             \
        if (buffers == nullptr) {                                                                    \
            set_last_status(NGP_ERR_INVALID_ARGUMENT, "buffers is NULL");                            \
            return NGP_ERR_INVALID_ARGUMENT;                                                         \
        }                                                                                            \
        int st_ = read_descriptor(opaque, opaque_len, &var);                                         \
        if (st_ != NGP_OK) return st_;                                                               \
    } while (0)

extern "C" {

int ngp_last_status(void) { return t_status; }
const char *ngp_last_status_message(void) { return t_message; }
int ngp_abi_version(void) { return 1; }
unsigned long long ngp_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }
int ngp_device_status(void) { return device_status(); }
int ngp_selftest_bounded_wait(cudaStream_t stream, unsigned int polls) {
    return launch_bounded_wait_selftest(stream, polls);
}
int ngp_set_march_blocks_per_sm(int n) { return set_march_blocks_per_sm(n); }

NGP_ENTRY(pack_density_into_bits) {
    NGP_DESC(PackbitsDescriptor, d);
    return launch_packbits(stream, d.n_bytes, CF32(0), CF32(1), B8(2), U8(3), false);
}

NGP_ENTRY(ngp_packbits_scalar) {
    NGP_DESC(PackbitsDescriptor, d);
    return launch_packbits(stream, d.n_bytes, CF32(0), CF32(1), B8(2), U8(3), true);
}

NGP_ENTRY(march_rays) {
    NGP_DESC(MarchingDescriptor, d);
    return launch_march_rays(stream, d, CF32(0), CF32(1), CF32(2), CF32(3), CF32(4), CU8(5), U32(6), U32(7), B8(8),
                             U32(9), U32(10), U32(11), F32(12), F32(13), F32(14), F32(15), nullptr, true, nullptr);
}

NGP_ENTRY(ngp_march_rays_train) {
    NGP_DESC(MarchingDescriptor, d);
    NGP_CHECK_ARG(buffers[16] != nullptr, "ngp_march_rays_train: the queue counter (buffer 16) is required");
    return launch_march_rays(stream, d, CF32(0), CF32(1), CF32(2), CF32(3), CF32(4), CU8(5), U32(6), U32(7), B8(8),
                             U32(9), U32(10), U32(11), F32(12), F32(13), F32(14), F32(15), U32(16), true, CU8(17));
}

NGP_ENTRY(march_rays_inference) {
    NGP_DESC(MarchingInferenceDescriptor, d);
    return launch_march_rays_inference(stream, d, CF32(0), CF32(1), CF32(2), CF32(3), CU8(4), CU32(5), CB8(6),
                                       CU32(7), U32(8), U32(9), U32(10), F32(11), F32(12), F32(13), F32(14));
}

NGP_ENTRY(ngp_march_rays_inference_inplace) {
    NGP_DESC(MarchingInferenceDescriptor, d);
    return launch_march_rays_inference_inplace(stream, d, CF32(0), CF32(1), F32(2), CF32(3), CU8(4), CB8(5), U32(6),
                                               U32(7), U32(8), nullptr, nullptr, F32(9), F32(10), F32(11), F32(12));
}

NGP_ENTRY(ngp_march_rays_inference_compact) {
    NGP_DESC(MarchingInferenceDescriptor, d);
    NGP_CHECK_ARG(buffers[9] != nullptr && buffers[10] != nullptr, "march_rays_inference_compact: sample_start and sample_count are required");
    return launch_march_rays_inference_inplace(stream, d, CF32(0), CF32(1), F32(2), CF32(3), CU8(4), CB8(5), U32(6),
                                               U32(7), U32(8), U32(9), U32(10), F32(11), F32(12), F32(13), F32(14));
}

NGP_ENTRY(ngp_integrate_rays_inference_inplace) {
    NGP_DESC(IntegratingInferenceDescriptor, d);
    return launch_integrate_rays_inference_inplace(stream, d, CF32(0), F32(1), F32(2), CU32(3), CU32(4), CF32(5),
                                                   CF32(6), CF32(7), nullptr, U32(8), B8(9));
}

NGP_ENTRY(ngp_integrate_rays_inference_compact) {
    NGP_DESC(IntegratingInferenceDescriptor, d);
    NGP_CHECK_ARG(buffers[8] != nullptr, "integrate_rays_inference_compact: sample_start is required");
    return launch_integrate_rays_inference_inplace(stream, d, CF32(0), F32(1), F32(2), CU32(3), CU32(4), CF32(5),
                                                   CF32(6), CF32(7), CU32(8), U32(9), B8(10));
}

NGP_ENTRY(spherical_harmonics_encoding_cuda_f32) {
    NGP_DESC(SphericalHarmonicsEncodingDescriptor, d);
    return launch_sh_encoding(stream, d.n, d.degree, CF32(0), F32(1));
}

NGP_ENTRY(morton3d) {
    NGP_DESC(Morton3DDescriptor, d);
    return launch_morton3d(stream, d.length, CU32(0), U32(1));
}

NGP_ENTRY(morton3d_invert) {
    NGP_DESC(Morton3DDescriptor, d);
    return launch_morton3d_invert(stream, d.length, CU32(0), U32(1));
}

static bool misaligned16(const void *p) { return ((std::uintptr_t)p & 15u) != 0; }

NGP_ENTRY(integrate_rays) {
    NGP_DESC(IntegratingDescriptor, d);
    NGP_CHECK_ARG(!misaligned16(buffers[5]) && !misaligned16(buffers[7]), "integrate_rays: drgbs and final_rgbds must be 16-byte aligned");
    return launch_integrate_rays(stream, d, CU32(0), CU32(1), CF32(2), CF32(3), CF32(4), CF32(5), U32(6), F32(7), F32(8));
}

NGP_ENTRY(integrate_rays_backward) {
    NGP_DESC(IntegratingBackwardDescriptor, d);
    NGP_CHECK_ARG(!misaligned16(buffers[5]) && !misaligned16(buffers[6]) && !misaligned16(buffers[8]) && !misaligned16(buffers[11]),
                  "integrate_rays_backward: drgbs, final_rgbds, dL_dfinal_rgbds and dL_ddrgbs must be 16-byte aligned");
    return launch_integrate_rays_backward(stream, d, CU32(0), CU32(1), CF32(2), CF32(3), CF32(4), CF32(5), CF32(6),
                                          CF32(7), CF32(8), F32(9), F32(10), F32(11), false);
}

NGP_ENTRY(ngp_integrate_rays_backward_exact) {
    NGP_DESC(IntegratingBackwardDescriptor, d);
    NGP_CHECK_ARG(!misaligned16(buffers[5]) && !misaligned16(buffers[6]) && !misaligned16(buffers[8]) && !misaligned16(buffers[11]),
                  "integrate_rays_backward_exact: drgbs, final_rgbds, dL_dfinal_rgbds and dL_ddrgbs must be 16-byte aligned");
    return launch_integrate_rays_backward(stream, d, CU32(0), CU32(1), CF32(2), CF32(3), CF32(4), CF32(5), CF32(6),
                                          CF32(7), CF32(8), F32(9), F32(10), F32(11), true);
}

NGP_ENTRY(ngp_integrate_rays_fp64) {
    NGP_DESC(IntegratingDescriptor, d);
    return launch_integrate_rays_fp64(stream, d, CU32(0), CU32(1), CF32(2), CF32(3), CF32(4), CF32(5),
                                      static_cast<double *>(buffers[6]), static_cast<double *>(buffers[7]), U32(8));
}

NGP_ENTRY(integrate_rays_inference) {
    NGP_DESC(IntegratingInferenceDescriptor, d);
    NGP_CHECK_ARG(!misaligned16(buffers[1]) && !misaligned16(buffers[7]) && !misaligned16(buffers[10]),
                  "integrate_rays_inference: rays_rgbd, drgbs and rays_rgbd_out must be 16-byte aligned");
    return launch_integrate_rays_inference(stream, d, CF32(0), CF32(1), CF32(2), CU32(3), CU32(4), CF32(5), CF32(6),
                                           CF32(7), U32(8), B8(9), F32(10), F32(11));
}

NGP_ENTRY(ngp_march_count) {
    (void)opaque;
    (void)opaque_len;
    NGP_CHECK_ARG(buffers != nullptr, "buffers is NULL");
    NGP_CHECK_ARG(buffers[0] != nullptr && buffers[1] != nullptr && buffers[2] != nullptr,
                  "ngp_march_count: the two counters and the result are required");
    march_count_kernel<<<1, 1, 0, stream>>>(CU32(0), CU32(1), U32(2));
    count_launches(1);
    return launch_status();
}

NGP_ENTRY(ngp_hashgrid_forward) {
    NGP_DESC(NgpHashGridDescriptor, d);
    return launch_hashgrid_forward(stream, d, CU32(2), CF32(0), CF32(1), F32(3));
}

NGP_ENTRY(ngp_hashgrid_backward) {
    NGP_DESC(NgpHashGridDescriptor, d);
    return launch_hashgrid_backward(stream, d, CU32(2), CF32(0), CF32(1), F32(3), d.accumulate != 0);
}

NGP_ENTRY(ngp_hashgrid_tv) {
    NGP_DESC(NgpHashGridTVDescriptor, d);
    return launch_hashgrid_tv(stream, d.grid, d.tv_scale, CF32(0), CF32(1), CF32(2), F32(3),
                              d.with_grad != 0 ? F32(4) : nullptr, static_cast<double *>(buffers[5]));
}

NGP_ENTRY(ngp_render_blobs) {
    NGP_DESC(NgpRenderBlobsDescriptor, d);
    return launch_render_blobs(stream, d, CF32(0), CF32(1), CF32(2), U8(3));
}

NGP_ENTRY(ngp_field_forward) {
    NGP_DESC(NgpMlpDescriptor, d);
    return launch_mlp_x6_forward(stream, d.n_samples, CU32(3), CF32(0), CF32(1), CF32(2), F32(4));
}

NGP_ENTRY(ngp_field_density) {
    NGP_DESC(NgpMlpDescriptor, d);
    return launch_mlp_x6_density(stream, d.n_samples, CF32(0), CF32(1), F32(2));
}

NGP_ENTRY(ngp_field_backward) {
    NGP_DESC(NgpMlpDescriptor, d);
    unsigned parts = 0;
    const int st = launch_mlp_x6_backward(stream, d.n_samples, CU32(4), CF32(0), CF32(1), CF32(2), CF32(3), CF32(5),
                                          F32(7), F32(6), ~0u, &parts);
    if (st != NGP_OK) return st;
    return launch_mlp_partials_reduce(stream, parts, CF32(6), F32(8), d.accumulate != 0, d.n_samples, CU32(4), F32(7), 32u);
}

size_t ngp_field_backward_scratch_floats(void) { return mlp_partials_floats(); }

NGP_ENTRY(ngp_field_forward_bf16) {
    NGP_DESC(NgpMlpDescriptor, d);
    return launch_mlp_bf16_forward(stream, d.n_samples, CU32(3), CF32(0), CF32(1), CF32(2), F32(4));
}

NGP_ENTRY(ngp_field_density_bf16) {
    NGP_DESC(NgpMlpDescriptor, d);
    return launch_mlp_bf16_density(stream, d.n_samples, CF32(0), CF32(1), F32(2));
}

NGP_ENTRY(ngp_field_backward_bf16) {
    NGP_DESC(NgpMlpDescriptor, d);
    unsigned parts = 0;
    const int st = launch_mlp_bf16_backward(stream, d.n_samples, CU32(4), CF32(0), CF32(1), CF32(2), CF32(3), CF32(5),
                                            F32(7), F32(6), &parts);
    if (st != NGP_OK) return st;
    return launch_mlp_partials_reduce(stream, parts, CF32(6), F32(8), d.accumulate != 0, d.n_samples, CU32(4), F32(7), 32u);
}

NGP_ENTRY(ngp_field_forward_mixed) {
    NGP_DESC(NgpFieldMixedDescriptor, d);
    NGP_CHECK_ARG(d.activations == NGP_DTYPE_F32 || d.activations == d.operand,
                  "field (mixed): activations must be FP32 or the operand type");
    return launch_mlp_tc_forward(stream, d.operand, d.activations != NGP_DTYPE_F32, d.n_samples, CU32(3), buffers[0],
                                 CF32(1), CF32(2), F32(4));
}

NGP_ENTRY(ngp_field_density_mixed) {
    NGP_DESC(NgpFieldMixedDescriptor, d);
    NGP_CHECK_ARG(d.activations == NGP_DTYPE_F32 || d.activations == d.operand,
                  "field (mixed): activations must be FP32 or the operand type");
    return launch_mlp_tc_density(stream, d.operand, d.activations != NGP_DTYPE_F32, d.n_samples, buffers[0], CF32(1),
                                 F32(2));
}

NGP_ENTRY(ngp_field_backward_mixed) {
    NGP_DESC(NgpFieldMixedDescriptor, d);
    NGP_CHECK_ARG(d.activations == NGP_DTYPE_F32 || d.activations == d.operand,
                  "field (mixed): activations must be FP32 or the operand type");
    unsigned parts = 0;
    const int st = launch_mlp_tc_backward(stream, d.operand, d.activations != NGP_DTYPE_F32, d.n_samples, CU32(4),
                                          buffers[0], CF32(1), CF32(2), CF32(3), CF32(5),
                                          static_cast<NgpLossScale *>(buffers[6]), buffers[8], F32(7), &parts);
    if (st != NGP_OK) return st;
    return launch_mlp_partials_reduce(stream, parts, CF32(7), F32(9), d.accumulate != 0, d.n_samples, CU32(4), F32(8),
                                      d.activations != NGP_DTYPE_F32 ? 16u : 32u);
}

NGP_ENTRY(ngp_hashgrid_forward_mixed) {
    NGP_DESC(NgpHashGridMixedDescriptor, d);
    return launch_hashgrid_forward_mixed(stream, d.grid, d.table, d.encodings, CU32(2), CF32(0), buffers[1], buffers[3]);
}

NGP_ENTRY(ngp_hashgrid_backward_mixed) {
    NGP_DESC(NgpHashGridMixedDescriptor, d);
    return launch_hashgrid_backward_mixed(stream, d.grid, d.encodings, CU32(2), CF32(0), buffers[1], F32(3),
                                          d.grid.accumulate != 0);
}

NGP_ENTRY(ngp_adam_mixed) {
    NGP_DESC(NgpAdamMixedDescriptor, d);
    return launch_adam_mixed(stream, d.adam, d.half_copy, F32(0), F32(1), F32(2), F32(3),
                             static_cast<const NgpLossScale *>(buffers[4]), buffers[5]);
}

NGP_ENTRY(ngp_loss_scale_update) {
    NGP_DESC(NgpLossScaleDescriptor, d);
    return launch_loss_scale_update(stream, d, static_cast<NgpLossScale *>(buffers[0]));
}

NGP_ENTRY(ngp_field_backward_noalloc) {
    NGP_DESC(NgpMlpDescriptor, d);
    return launch_mlp_backward_noalloc(stream, d.n_samples, CU32(4), CF32(0), CF32(1), CF32(2), CF32(3), CF32(5),
                                       F32(6), F32(7), d.accumulate != 0);
}

NGP_ENTRY(ngp_train_rays) {
    NGP_DESC(NgpTrainRaysDescriptor, d);
    return launch_train_rays(stream, d, CF32(0), CU8(1), CU32(2), F32(3), F32(4), F32(5), F32(6), F32(7), F32(8),
                             F32(9));
}

NGP_ENTRY(ngp_integrate_loss_backward) {
    NGP_DESC(NgpIntegrateLossDescriptor, d);
    return launch_integrate_loss_backward(stream, d, CB8(0), CU32(1), CU32(2), CF32(3), CF32(4), CF32(5), CF32(6),
                                          CF32(7), CU32(8), F32(10), F32(11), F32(12), F32(9));
}

NGP_ENTRY(ngp_adam) {
    NGP_DESC(NgpAdamDescriptor, d);
    return launch_adam(stream, d, F32(0), F32(1), F32(2), F32(3));
}

NGP_ENTRY(ngp_ogrid_decay) {
    NGP_DESC(NgpOgridDescriptor, d);
    NGP_CHECK_ARG(d.cascade < d.K, "ogrid: cascade out of range");
    const std::uint32_t G3 = d.G * d.G * d.G;
    return launch_ogrid_decay(stream, G3, d.decay, F32(0) + (std::size_t)d.cascade * G3);
}

NGP_ENTRY(ngp_ogrid_sample) {
    NGP_DESC(NgpOgridDescriptor, d);
    NGP_CHECK_ARG(d.cascade < d.K && d.G > 1, "ogrid: cascade out of range");
    NGP_CHECK_ARG(!d.update_all || d.n_points == d.G * d.G * d.G, "ogrid: update_all needs one point per cell");
    return launch_ogrid_sample(stream, d.n_points, d.update_all != 0, d.cascade, d.G, d.bound, d.seed, CF32(0), CU8(1),
                               U32(2), F32(3));
}

NGP_ENTRY(ngp_ogrid_max) {
    NGP_DESC(NgpOgridDescriptor, d);
    return launch_ogrid_max(stream, d.n_points, d.cascade, d.G * d.G * d.G, CU32(0), CF32(1), F32(2));
}

NGP_ENTRY(ngp_ogrid_threshold) {
    NGP_DESC(NgpOgridDescriptor, d);
    return launch_ogrid_threshold(stream, d.G * d.G * d.G, d.threshold_step, CF32(0), F32(1), F32(2));
}

NGP_ENTRY(ngp_ogrid_mark_untrained) {
    NGP_DESC(NgpOgridDescriptor, d);
    return launch_ogrid_mark_untrained(stream, d.K, d.G, d.bound, d.n_views, CF32(0), d.fx, d.fy, d.cx, d.cy, d.width,
                                       d.height, F32(1));
}

NGP_ENTRY(ngp_proposal_coarse) {
    NGP_DESC(NgpProposalDescriptor, d);
    return launch_proposal_coarse(stream, d.G, CU8(0), U8(1));
}

static std::uint32_t proposal_spr(const NgpProposalDescriptor &d) {
    return d.samples_per_ray != 0 ? d.samples_per_ray : (std::uint32_t)NGP_PROPOSAL_SAMPLES;
}

NGP_ENTRY(ngp_proposal_rays) {
    NGP_DESC(NgpProposalDescriptor, d);
    return launch_proposal_rays(stream, d.n, d.total_samples, proposal_spr(d), d.G, d.bound, CF32(0), CF32(1), CF32(2), CF32(3), CU8(4),
                                U32(5), U32(6), B8(7), U32(8), U32(9), U32(10), F32(11), F32(12), U32(13));
}

NGP_ENTRY(ngp_proposal_bin_points) {
    NGP_DESC(NgpProposalDescriptor, d);
    return launch_proposal_bin_points(stream, d.total_samples / proposal_spr(d), CU32(0), CF32(1), CF32(2), CU32(3),
                                      CF32(4), CF32(5), F32(6));
}

NGP_ENTRY(ngp_proposal_sample) {
    NGP_DESC(NgpProposalDescriptor, d);
    const std::uint64_t seed = ((std::uint64_t)d.seed_hi << 32) | d.seed_lo;
    return launch_proposal_sample(stream, d.total_samples / proposal_spr(d), CU32(0), proposal_spr(d), d.mix, d.perturb != 0,
                                  seed,
                                  CF32(1),
                                  CF32(2), CU32(3), CF32(4), CF32(5), CF32(6), U32(7), F32(8), F32(9), F32(10), F32(11));
}

NGP_ENTRY(ngp_proposal_judge) {
    NGP_DESC(NgpProposalDescriptor, d);
    return launch_proposal_judge(stream, d.total_samples / proposal_spr(d), CU32(0), d.G, d.bound, CF32(8), CF32(1), CF32(2),
                                 CU32(3), CF32(4), CF32(5), CF32(6), CU8(7), U8(9), U32(10), U32(11), U32(12));
}

NGP_ENTRY(ngp_proposal_sample_alloc) {
    NGP_DESC(NgpProposalDescriptor, d);
    const std::uint64_t seed = ((std::uint64_t)d.seed_hi << 32) | d.seed_lo;
    return launch_proposal_sample_alloc(stream, d.total_samples / proposal_spr(d), d.total_samples, U32(0), proposal_spr(d),
                                        d.mix, d.perturb != 0, seed, CF32(1), CF32(2), CU32(3), CF32(4), CF32(5), CF32(6),
                                        CU8(7), U32(8), U32(9), U32(10), F32(11), F32(12), F32(13), F32(14), B8(15),
                                        U32(16), U32(17));
}

NGP_ENTRY(ngp_march_rays_fallback) {
    NGP_DESC(MarchingDescriptor, d);
    return launch_march_rays_list(stream, d, CF32(0), CF32(1), CF32(2), CF32(3), CF32(4), CU8(5), U32(6), U32(7), B8(8),
                                  U32(9), U32(10), U32(11), F32(12), F32(13), F32(14), F32(15), U32(16), CU32(17),
                                  CU32(18));
}

NGP_ENTRY(ngp_proposal_loss) {
    NGP_DESC(NgpProposalDescriptor, d);
    const bool all = d.count_index == 3 || buffers[0] == nullptr;
    return launch_proposal_loss(stream, d.n, all ? nullptr : CU32(0), all ? 0 : (int)d.count_index, CF32(1), CF32(2),
                                (int)d.sigma_stride, F32(3), F32(4));
}

NGP_ENTRY(ngp_proposal_mlp_forward) {
    NGP_DESC(NgpMlpDescriptor, d);
    return launch_prop_forward(stream, d.n_samples, CU32(2), CF32(0), CF32(1), F32(3));
}

NGP_ENTRY(ngp_proposal_mlp_forward_f16) {
    NGP_DESC(NgpMlpDescriptor, d);
    return launch_prop_f16_forward(stream, d.n_samples, CU32(2), CF32(0), CF32(1), F32(3));
}

NGP_ENTRY(ngp_proposal_mlp_backward) {
    NGP_DESC(NgpMlpDescriptor, d);
    return launch_prop_backward(stream, d.n_samples, CU32(3), CF32(0), CF32(1), CF32(2), F32(5), F32(6), F32(4),
                                d.accumulate != 0);
}

size_t ngp_proposal_backward_scratch_floats(void) { return prop_partials_floats(); }

}  // extern "C"
