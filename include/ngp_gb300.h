/*
 * libngp_gb300: GB300-native (sm_103a) kernels for the NeRF hot path of jaxngp, behind a C ABI.
 *
 * Every entry point takes the caller's CUDA stream, enqueues work on it and returns without
 * blocking the host.  Nothing allocates device memory except where noted (scratch is passed in).
 * Buffers are device pointers owned by the caller.
 *
 * Two signatures per op:
 *   void NAME(cudaStream_t, void **buffers, const char *opaque, size_t opaque_len)
 *       The XLA custom-call signature of the reference's volrendjax targets (registered there by
 *       deps/volume-rendering-jax/lib/ffi.cc:25-51).  `buffers` holds the operands in declaration
 *       order followed by the results, exactly as in volrendjax's per-op lowering.py; `opaque` holds
 *       the raw bytes of the op's descriptor struct.  Errors are recorded for ngp_last_status()
 *       instead of thrown (the reference throws std::runtime_error across the C boundary).
 *   int  NAME_status(same arguments)
 *       Same work; returns the status code directly.
 */
#ifndef NGP_GB300_H_
#define NGP_GB300_H_

#include <stddef.h>
#include <stdint.h>

#include <cuda_runtime_api.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------------ status codes */
#define NGP_OK 0
#define NGP_ERR_OPAQUE_SIZE 1      /* opaque length differs from sizeof(descriptor) */
#define NGP_ERR_INVALID_ARGUMENT 2 /* a descriptor field or pointer is out of contract */
#define NGP_ERR_CUDA 3             /* a CUDA runtime call or kernel launch failed */
#define NGP_ERR_DEVICE 4           /* a kernel reported an error through its status word */
#define NGP_ERR_CAPACITY 5         /* a size exceeds a fixed capacity of the entry point */

/* Status and message of the last call made on this host thread. */
int ngp_last_status(void);
const char *ngp_last_status_message(void);
/* ABI version of this library (bumped on any signature or descriptor change). */
int ngp_abi_version(void);
/* Number of kernels this library has launched in this process (all devices, all threads). */
unsigned long long ngp_kernel_launches(void);
/* Synchronises the current device, then returns NGP_ERR_DEVICE (and clears the flag) if a kernel
 * recorded a device-side error since the last call -- a tensor-core kernel whose bounded wait for
 * its MMAs ran out -- else NGP_OK, or NGP_ERR_CUDA if the synchronisation failed. */
int ngp_device_status(void);
/* Test hook of the failure path above: one thread waits, with the tensor-core kernels' bounded
 * wait, on an mbarrier that nothing completes; after `polls` polls (1..2^20) it gives up and
 * records the device error, which the next ngp_device_status() reports once.  Returns the launch
 * status. */
int ngp_selftest_bounded_wait(cudaStream_t stream, unsigned int polls);
/* At most this many CTAs per SM for the marches (march_rays, ngp_march_rays_train,
 * ngp_march_rays_fallback) on every later call on any thread -- they stride over the rest of the
 * rays; 0 restores the default (10: no limit below what fits).
 * A caller that runs the march on a second stream, beside other kernels, lowers it so those
 * kernels find room on every SM.  Returns the previous value, or -1 for n outside [0, 10]. */
int ngp_set_march_blocks_per_sm(int n);

/* ------------------------------------------------------- volrendjax descriptors (byte-exact) */
/* deps/volume-rendering-jax/lib/impl/volrend.h:23-29 */
typedef struct IntegratingDescriptor {
    uint32_t n_rays;
    uint32_t total_samples;
} IntegratingDescriptor;

/* volrend.h:32-42 */
typedef struct IntegratingBackwardDescriptor {
    uint32_t n_rays;
    uint32_t total_samples;
    float near_distance;
} IntegratingBackwardDescriptor;

/* volrend.h:45-54 */
typedef struct IntegratingInferenceDescriptor {
    uint32_t n_total_rays;
    uint32_t n_rays;
    uint32_t march_steps_cap;
} IntegratingInferenceDescriptor;

/* volrend.h:57-86 */
typedef struct MarchingDescriptor {
    uint32_t n_rays;
    uint32_t total_samples;
    uint32_t diagonal_n_steps;
    uint32_t K;
    uint32_t G;
    float bound;
    float stepsize_portion;
} MarchingDescriptor;

/* volrend.h:89-108 */
typedef struct MarchingInferenceDescriptor {
    uint32_t n_total_rays;
    uint32_t n_rays;
    uint32_t diagonal_n_steps, K, G;
    uint32_t march_steps_cap;
    float bound;
    float stepsize_portion;
} MarchingInferenceDescriptor;

/* volrend.h:110-113 */
typedef struct Morton3DDescriptor {
    uint32_t length;
} Morton3DDescriptor;

/* volrend.h:116-118 */
typedef struct PackbitsDescriptor {
    uint32_t n_bytes;
} PackbitsDescriptor;

/* ------------------------------------------------------------------ volrendjax entry points */
/* Replaces volrendjax::pack_density_into_bits (volrend.h:121-126; packbits.cu:76-83).
 * buffers: density_threshold f32[n], density_grid f32[n] -> occupied_mask bool[n],
 * occupancy_bitfield u8[n/8]; opaque: PackbitsDescriptor.  n_bytes == 0 is an error
 * (ffi.cc:57-59).  density and threshold 16-byte aligned, mask 8-byte aligned. */
void pack_density_into_bits(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int pack_density_into_bits_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* Replaces volrendjax::march_rays (volrend.h:128-133; marching.cu:669-676).
 * buffers: rays_o f32[R,3], rays_d f32[R,3], t_starts f32[R], t_ends f32[R], noises f32[R],
 * occupancy_bitfield u8[K*G^3/8] -> next_sample_write_location u32[1],
 * number_of_exceeded_samples u32[1], ray_is_valid bool[R], rays_n_samples u32[R],
 * rays_sample_startidx u32[R], idcs u32[S], xyzs f32[S,3], dirs f32[S,3], dss f32[S],
 * z_vals f32[S]; opaque: MarchingDescriptor.  The result is the reference kernel's under the
 * schedule in which its threads run one at a time in ray order (as ngp_march_rays_train below,
 * without a queue word or coarse blocks): deterministic, and the reference's own result whenever
 * the budget does not overflow; with overflow the reference's result depends on its schedule.
 * With fewer than 2 ceil(R / 256) + 3 sample slots the rays take slots in the order their warps
 * finish counting, as in the reference. */
void march_rays(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int march_rays_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* Replaces volrendjax::march_rays_inference (volrend.h:135-140; marching.cu:678-685), without
 * the host-blocking stream synchronisation of marching.cu:562.
 * buffers: rays_o f32[N,3], rays_d f32[N,3], t_starts f32[N], t_ends f32[N],
 * occupancy_bitfield u8[K*G^3/8], next_ray_index_in u32[1], terminated bool[n],
 * indices_in u32[n] -> next_ray_index u32[1], indices_out u32[n], n_samples u32[n],
 * t_starts_out f32[n], xyzs f32[n,cap,3], dss f32[n,cap], z_vals f32[n,cap];
 * opaque: MarchingInferenceDescriptor. */
void march_rays_inference(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int march_rays_inference_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* march_rays_inference for a device-resident render loop (the host loop of
 * models/renderers/cuda.py:326-361 without its per-iteration synchronisation): slot indices and the
 * next-ray counter are updated in place, the advanced t is written straight into t_starts (the
 * scatter of marching/__init__.py:156), and every sample also receives its ray's direction.
 * buffers: rays_o f32[N,3], rays_d f32[N,3], t_starts f32[N] (in/out), t_ends f32[N],
 * occupancy_bitfield u8[K*G^3/8], terminated bool[n], indices u32[n] (in/out),
 * next_ray_index u32[1] (in/out) -> n_samples u32[n], xyzs f32[n,cap,3], dirs f32[n,cap,3],
 * dss f32[n,cap], z_vals f32[n,cap].  opaque: MarchingInferenceDescriptor. */
void ngp_march_rays_inference_inplace(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_march_rays_inference_inplace_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* integrate_rays_inference for a device-resident render loop: each slot continues its ray directly
 * in rays_rgbd / rays_T (the scatter of integrating/__init__.py:108-109), and the number of rays
 * that terminated is added to terminate_total (not reset), so the host polls it only now and then.
 * buffers: rays_bg f32[N,3], rays_rgbd f32[N,4] (in/out), rays_T f32[N] (in/out), n_samples u32[n],
 * indices u32[n], dss f32[n,cap], z_vals f32[n,cap], drgbs f32[n,cap,4], terminate_total u32[1]
 * (in/out) -> terminated bool[n].  opaque: IntegratingInferenceDescriptor. */
void ngp_integrate_rays_inference_inplace(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_integrate_rays_inference_inplace_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* ngp_march_rays_inference_inplace with the samples' positions and directions packed densely, so
 * that the encoder and the MLP run on the samples that exist instead of n * cap entries (no
 * reference counterpart).  A warp reserves one range of sample_count for its slots' samples;
 * sample_start[i] is where slot i's samples begin.  dss and z_vals stay [n, cap].  The caller
 * zeroes sample_count before each call.  march_steps_cap <= 16.
 * buffers: rays_o f32[N,3], rays_d f32[N,3], t_starts f32[N] (in/out), t_ends f32[N],
 * occupancy_bitfield u8[K*G^3/8], terminated bool[n], indices u32[n] (in/out),
 * next_ray_index u32[1] (in/out) -> n_samples u32[n], sample_start u32[n], sample_count u32[1]
 * (in/out), xyzs f32[n*cap,3], dirs f32[n*cap,3], dss f32[n,cap], z_vals f32[n,cap].
 * opaque: MarchingInferenceDescriptor. */
void ngp_march_rays_inference_compact(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_march_rays_inference_compact_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* ngp_integrate_rays_inference_inplace reading slot i's colours from drgbs[sample_start[i] + k]
 * (the packed layout of ngp_march_rays_inference_compact).
 * buffers: rays_bg f32[N,3], rays_rgbd f32[N,4] (in/out), rays_T f32[N] (in/out), n_samples u32[n],
 * indices u32[n], dss f32[n,cap], z_vals f32[n,cap], drgbs f32[n*cap,4], sample_start u32[n],
 * terminate_total u32[1] (in/out) -> terminated bool[n].  opaque: IntegratingInferenceDescriptor. */
void ngp_integrate_rays_inference_compact(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_integrate_rays_inference_compact_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* Replaces volrendjax::morton3d (volrend.h:143-148; marching.cu:687-694).
 * buffers: xyzs u32[N,3] -> idcs u32[N]; opaque: Morton3DDescriptor. */
void morton3d(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int morton3d_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* Replaces volrendjax::morton3d_invert (volrend.h:149-154; marching.cu:696-703).
 * buffers: idcs u32[N] -> xyzs u32[N,3]; opaque: Morton3DDescriptor. */
void morton3d_invert(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int morton3d_invert_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* ------------------------------------------------ shjax (spherical-harmonics direction encoding) */
/* deps/spherical-harmonics-encoding-jax/lib/impl/spherical_harmonics_encoding.h:6-9 */
typedef struct SphericalHarmonicsEncodingDescriptor {
    uint32_t n;       /* directions */
    uint32_t degree;  /* L: outputs are the L^2 real harmonics of degrees 0..L-1, L in 1..8 */
} SphericalHarmonicsEncodingDescriptor;

/* Replaces shjax::spherical_harmonics_encoding_cuda_f32 (spherical_harmonics_encoding.h:11-16;
 * spherical_harmonics_encoding.cu:120-167), the custom-call target of
 * shjax.spherical_harmonics_encoding (src/shjax/__init__.py:120-134).
 * buffers: coord f32[n,3] (unit directions) -> encodings f32[n, L^2].
 * opaque: SphericalHarmonicsEncodingDescriptor.  The values equal the reference's flax
 * SphericalHarmonicsEncoder (models/encoders.py:361-406) bit for bit; L outside 1..8 returns
 * NGP_ERR_INVALID_ARGUMENT (the reference writes at most 64 values per direction). */
void spherical_harmonics_encoding_cuda_f32(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int spherical_harmonics_encoding_cuda_f32_status(cudaStream_t stream, void **buffers, const char *opaque,
                                                 size_t opaque_len);

/* Replaces volrendjax::integrate_rays (volrend.h:156-161; integrating.cu:512-519).
 * buffers: rays_sample_startidx u32[R], rays_n_samples u32[R], bgs f32[R,3], dss f32[S],
 * z_vals f32[S], drgbs f32[S,4] -> measured_batch_size u32[1], final_rgbds f32[R,4],
 * final_opacities f32[R]; opaque: IntegratingDescriptor.  drgbs/final_rgbds 16-byte aligned. */
void integrate_rays(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int integrate_rays_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* Replaces volrendjax::integrate_rays_backward (volrend.h:163-168; integrating.cu:521-528).
 * buffers: rays_sample_startidx, rays_n_samples, bgs, dss, z_vals, drgbs, final_rgbds,
 * final_opacities, dL_dfinal_rgbds f32[R,4] -> dL_dbgs f32[R,3], dL_dz_vals f32[S],
 * dL_ddrgbs f32[S,4]; opaque: IntegratingBackwardDescriptor. */
void integrate_rays_backward(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int integrate_rays_backward_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* The exact adjoint of integrate_rays as computed (no reference counterpart; the reference's
 * integrate_rays_backward scales density gradients by min(z^2, 1), adds a near-plane penalty,
 * counts the background twice in the density gradient of a ray that reaches it, and does not
 * differentiate the opacity normalisation of a terminated ray).  With out the ray's colour or
 * depth, cur_k the sum of its first k+1 weighted samples and norm = 1 (ray reaches the
 * background) or its opacity (terminated ray): d out/d sigma_k = dt_k (T_{k+1} c_k - (out -
 * cur_k)) / norm, d out/d c_k = w_k / norm, d out/d z_k = w_k / norm (depth), d out/d bg = T_N.
 * Same buffers and descriptor as integrate_rays_backward (near_distance unused). */
void ngp_integrate_rays_backward_exact(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_integrate_rays_backward_exact_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* FP64 checker of integrate_rays (no reference counterpart; used to state errors, not by any
 * training or rendering path): the same forward loop in double on the float inputs -- transmittance
 * product, colour and depth sums, termination once T <= 1e-4, opacity normalisation of terminated
 * rays, else + T bg.
 * buffers: rays_sample_startidx u32[R], rays_n_samples u32[R], bgs f32[R,3], dss f32[S], z_vals f32[S],
 * drgbs f32[S,4] -> rgbds f64[R,4], transmittance f64[R] (after the last composited sample),
 * n_used u32[R] (samples composited).  opaque: IntegratingDescriptor. */
void ngp_integrate_rays_fp64(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_integrate_rays_fp64_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* Replaces volrendjax::integrate_rays_inference (volrend.h:170-175; integrating.cu:530-537).
 * buffers: rays_bg f32[N,3], rays_rgbd f32[N,4], rays_T f32[N], n_samples u32[n],
 * indices u32[n], dss f32[n,cap], z_vals f32[n,cap], drgbs f32[n,cap,4] -> terminate_cnt u32[1],
 * terminated bool[n], rays_rgbd_out f32[n,4], rays_T_out f32[n];
 * opaque: IntegratingInferenceDescriptor. */
void integrate_rays_inference(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int integrate_rays_inference_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* march_rays for the training step: march_rays' result under one schedule of the reference
 * kernel (marching.cu:101-268) -- its threads run one at a time, in ray order -- so every buffer
 * and both counters are deterministic.  Ray r starts with the counter at the sum of the counts of
 * the rays before it; it is dropped (invalid, no samples) if that reaches the budget
 * (marching.cu:135), else it is valid without samples, or fits, or is the one ray that does not
 * fit (invalid; the counters' difference leaves its samples out); every later ray is dropped.
 * The valid rays are thus a prefix of the batch (march_rays, like the reference, fits rays in the
 * order in which they finish counting).  The rays past that prefix are not marched.  With coarse
 * occupancy blocks (ngp_proposal_coarse of the same bitfield; K = 1, G a multiple of 8) the march
 * crosses empty blocks in one step each and finishes a ray whose segment crosses no occupied block
 * at once -- valid, no samples -- with the same samples as the cell-by-cell march.  The pass's sums
 * per 256 rays, their done flags and its progress word borrow the last 2 ceil(n_rays / 256) + 3
 * words of idcs (overwritten by the samples and the zeroed tail); with fewer sample slots than
 * that the call allocates as march_rays does.
 * queue: in, the word the previous call on this batch size left (0 on a first call); out, the
 * index of the first ray dropped or unfit (0xFFFFFFFF when none is).  The leading rays -- 1.25
 * times that index plus 512 (8192 for 0), at most 16384 -- are counted alone, a warp per ray,
 * before the rest, which then find the budget full and are dropped unmarched: a caller that passes
 * the word back from call to call keeps the lead just above the rays the budget takes.
 * buffers: the 16 buffers of march_rays, then queue u32[1], then coarse u8[(G/8)^3] or NULL.
 * opaque: MarchingDescriptor. */
void ngp_march_rays_train(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_march_rays_train_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* march_rays' measured_batch_size_before_compaction on the device (marching/__init__.py:91):
 * buffers: next_sample_write_location u32[1], number_of_exceeded_samples u32[1] -> count u32[1].
 * opaque: none (length 0).  The result is the number of leading sample slots that hold samples. */
void ngp_march_count(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_march_count_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* -------------------------------------------------------------------- hash-grid encoder */
#define NGP_MAX_LEVELS 32

/* Static description of a HashGridEncoder (models/encoders.py:58-114): the per-level table the
 * flax module computes on the host in float64 (scale_l = N_min * b^l - 1, cast to float32;
 * res_l = ceil(scale_l) + 1; offsets = prefix sums of the level sizes). */
typedef struct NgpHashGridDescriptor {
    uint32_t n_coords;          /* number of query points */
    uint32_t L, F, T;           /* levels, features per level (2), max entries per level */
    uint32_t first_hash_level;  /* levels [0, first_hash_level) are dense */
    uint32_t n_params;          /* P = offsets[L], rows of the latent table */
    float bound;                /* positions are in [-bound, bound]^3 */
    float two_bound;            /* float32(2 * bound) */
    uint32_t accumulate;        /* backward: add into dL_dlatents instead of zero-filling it first */
    float scales[NGP_MAX_LEVELS];
    uint32_t resolutions[NGP_MAX_LEVELS];
    uint32_t offsets[NGP_MAX_LEVELS + 1];
} NgpHashGridDescriptor;

/* Replaces HashGridEncoder.__call__ without the TV term (models/encoders.py:83-233).
 * buffers: pos f32[N,3], latents f32[P,F], active_count u32[1] or NULL -> encodings f32[N,L*F]
 * (level-major columns).  With an active count, only the first min(N, *count) rows are
 * computed.  opaque: NgpHashGridDescriptor. */
void ngp_hashgrid_forward(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_hashgrid_forward_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* Replaces the gradient JAX derives for the gather of encoders.py:226 (a scatter-add).
 * buffers: pos f32[N,3], dL_denc f32[N,L*F], active_count u32[1] or NULL -> dL_dlatents f32[P,F].
 * The output is zero-filled first unless `accumulate` is set.  opaque: NgpHashGridDescriptor. */
void ngp_hashgrid_backward(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_hashgrid_backward_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* The total-variation term HashGridEncoder returns with tv_scale > 0 (models/encoders.py:236-254):
 * tv = tv_scale * mean over levels and points of the sum, over the six axis neighbours of the
 * point's corner 0 and the features, of (lat[neighbour] - lat[corner 0])^2.  Every point counts
 * (no active count: the reference averages over the whole sample buffer).  tv_scale <= 0 writes
 * tv = 0 and adds no gradient, as the reference returns 0.
 * buffers: pos f32[N,3], latents f32[P,2], grad_scale f32[1] or NULL -> tv f32[1], dL_dlatents
 * f32[P,2] (with_grad: d tv / d latents, times *grad_scale when given, ADDED to the buffer; NULL
 * otherwise), scratch f64[1] (overwritten).  opaque: NgpHashGridTVDescriptor (grid.n_coords = N;
 * grid.accumulate is ignored). */
typedef struct NgpHashGridTVDescriptor {
    NgpHashGridDescriptor grid;
    float tv_scale;
    uint32_t with_grad;
} NgpHashGridTVDescriptor;

void ngp_hashgrid_tv(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_hashgrid_tv_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* ------------------------------------------------------------------------- field MLP */
#define NGP_MLP_WEIGHTS 9408 /* W0[32,64] W1[64,16] W2[32,64] W3[64,64] W4[64,3], packed */

typedef struct NgpMlpDescriptor {
    uint32_t n_samples;
    uint32_t accumulate; /* backward only: add into dL_dweights instead of overwriting */
} NgpMlpDescriptor;

/* Replaces the XLA computation of NeRF.__call__ after the encoder (models/nerfs.py:64-86 with
 * make_nerf_ngp, nerfs.py:422-454): density MLP, truncated exp, SH degree 4, colour MLP, sigmoid.
 * FP32 accuracy on the tensor cores: every operand split into three BF16 pieces, six MMAs per
 * layer into FP32 accumulators (within FP32 rounding of the exact layer).
 * buffers: encodings f32[S,32], dirs f32[S,3], weights f32[9408], active_count u32[1] or NULL
 * -> drgbs f32[S,4].  opaque: NgpMlpDescriptor.  encodings and drgbs 16-byte aligned. */
void ngp_field_forward(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_field_forward_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* Density only (NeRF.__call__ with dir=None, nerfs.py:71-72).
 * buffers: encodings f32[S,32], weights f32[9408] -> sigma f32[S]. */
void ngp_field_density(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_field_density_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* Backward of ngp_field_forward (JAX autodiff of nerfs.py:39-128, with the truncated-exp
 * gradient of nerfs.py:230-234), recomputing the activations from the encodings.
 * buffers: encodings, dirs, weights, dL_ddrgbs f32[S,4], active_count u32[1] or NULL,
 * grad_scale f32[1] or NULL (multiplies dL_ddrgbs), scratch f32[ngp_field_backward_scratch_floats()]
 * -> dL_dencodings f32[S,32], dL_dweights f32[9408].  opaque: NgpMlpDescriptor. */
void ngp_field_backward(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_field_backward_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
size_t ngp_field_backward_scratch_floats(void);

/* No counterpart in the reference.  ngp_field_backward for callers that cannot allocate device
 * memory: an XLA custom call bound through the legacy signature receives only its operand and
 * result buffers, and an embedder running inside a fixed, pre-reserved memory budget may not call
 * cudaMalloc or any allocating library routine.  The per-CTA dL/dW partials live in a static
 * array inside the library (9.6 MB, room for the partials of 256 CTAs whatever the batch, held by
 * every GPU that loads the library until exit) instead of a caller-provided scratch buffer.  A call
 * takes at most NGP_FIELD_BACKWARD_NOALLOC_MAX_SAMPLES samples, a published bound of this entry
 * point; larger batches return NGP_ERR_CAPACITY.  The first call
 * on each device looks up the array's device address (cudaGetSymbolAddress); make that first call
 * before any stream capture.  All calls share the array: calls that overlap on the GPU (different
 * streams) race on it and must be ordered by the caller.  Nothing has to be cleared between calls.
 * buffers: encodings f32[S,32], dirs f32[S,3], weights f32[9408], dL_ddrgbs f32[S,4],
 * active_count u32[1] or NULL, grad_scale f32[1] or NULL -> dL_dencodings f32[S,32],
 * dL_dweights f32[9408].  opaque: NgpMlpDescriptor. */
#define NGP_FIELD_BACKWARD_NOALLOC_MAX_SAMPLES 524288
void ngp_field_backward_noalloc(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_field_backward_noalloc_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* The three field ops on the fifth-generation tensor cores: BF16 operands (weights, encodings and
 * activations rounded to BF16 on their way into each MMA), FP32 accumulation in tensor memory,
 * FP32 outputs and weight gradients.  Same buffers, descriptors and semantics as
 * ngp_field_forward / ngp_field_density / ngp_field_backward; the reference's MLP has no BF16
 * form (its flax Dense layers compute in the parameters' FP32).  The backward's scratch has the
 * size ngp_field_backward_scratch_floats() gives. */
void ngp_field_forward_bf16(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_field_forward_bf16_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
void ngp_field_density_bf16(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_field_density_bf16_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
void ngp_field_backward_bf16(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_field_backward_bf16_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* --------------------------------------------------------------- training-step kernels */
/* Camera of the training set: pinhole intrinsics plus one 3x4 camera-to-world matrix per view
 * (utils/types.py Camera; app/nerf/_utils.py:97-115 builds rays from them). */
typedef struct NgpTrainRaysDescriptor {
    uint32_t n_rays;       /* rays in the batch */
    uint32_t width, height, n_views;
    float fx, fy, cx, cy;
    float bound;           /* scene AABB half-width */
    uint32_t perturb;      /* jitter each ray's start by a uniform fraction of a step */
    uint32_t random_bg;    /* uniform random background colour per ray, else `bg` */
    float bg[3];
    uint64_t seed;         /* counter-based RNG seed for this step */
} NgpTrainRaysDescriptor;

/* Builds one training batch: for each ray, a pixel index (from `perm` when given, else drawn
 * uniformly), its world-space origin/direction (_utils.py:97-115), AABB near/far
 * (renderers/cuda.py:56-97), start jitter, background colour, and the ground-truth colour
 * blended over that background (utils/data.py:443-465).
 * buffers: transforms f32[V,12] (row-major 3x4 camera-to-world), rgbas u8[V*H*W,4],
 * perm u32[R] or NULL -> rays_o f32[R,3], rays_d f32[R,3], t_starts f32[R], t_ends f32[R],
 * noises f32[R], bgs f32[R,3], gt_rgbs f32[R,3].  opaque: NgpTrainRaysDescriptor. */
void ngp_train_rays(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_train_rays_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

typedef struct NgpIntegrateLossDescriptor {
    uint32_t n_rays;
    uint32_t total_samples;
    float near_distance;
    float huber_delta;     /* 0.1 (app/nerf/_utils.py:154) */
} NgpIntegrateLossDescriptor;

/* integrate_rays forward, the masked Huber loss of app/nerf/_utils.py:151-156 and
 * integrate_rays_backward in one pass per ray.  The loss is sum over valid rays of
 * mean_c huber(pred - gt) / n_valid; dL_ddrgbs are written unnormalised and `grad_scale`
 * receives 1/n_valid for the field backward.
 * buffers: ray_is_valid bool[R], rays_sample_startidx, rays_n_samples, bgs f32[R,3],
 * gt_rgbs f32[R,3], dss, z_vals, drgbs, active_count u32[1], scratch f32[4 + R] (loss sums and the
 * list of rays with samples) -> dL_ddrgbs f32[S,4],
 * stats f32[4] (loss, n_valid_rays, measured_batch_size, samples before compaction),
 * grad_scale f32[1].  opaque: NgpIntegrateLossDescriptor. */
void ngp_integrate_loss_backward(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_integrate_loss_backward_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

typedef struct NgpAdamDescriptor {
    uint32_t n;            /* parameters in this group */
    uint32_t step;         /* 1-based step count after this update */
    float lr, beta1, beta2, eps, eps_root;
    float weight_decay;    /* decoupled, added to the update (optax.add_decayed_weights) */
    uint32_t zero_grad;    /* write zeros into the gradient after reading it */
} NgpAdamDescriptor;

/* optax.adam(b1, b2, eps, eps_root) chained with add_decayed_weights (app/nerf/_utils.py:19-77)
 * for one parameter group, updating params and moments in place.
 * buffers: params f32[n], grads f32[n], m f32[n], v f32[n]; opaque: NgpAdamDescriptor. */
void ngp_adam(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_adam_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* ------------------------------------------------------------------ mixed precision */
/* No counterpart in the reference (its encoder table, activations and gradients are FP32).
 * 16-bit storage types: NGP_DTYPE_BF16 (8-bit exponent) and NGP_DTYPE_F16 (5-bit exponent, so
 * gradients need loss scaling); arithmetic accumulates in FP32 throughout and gradients reach the
 * FP32 parameters through FP32 atomics and sums. */
#define NGP_DTYPE_F32 0u
#define NGP_DTYPE_BF16 1u
#define NGP_DTYPE_F16 2u

/* Dynamic loss scale, kept on the device (16 bytes).  The field backward multiplies its incoming
 * gradient by `scale` and sets `overflow` when a value it stores does not fit its type; the Adam
 * update skips a step with `overflow` set (and divides the gradients by `scale` otherwise);
 * ngp_loss_scale_update then adjusts `scale` and clears `overflow`.  `skipped_steps` counts the
 * skipped updates (the Adam bias correction uses step - skipped_steps). */
typedef struct NgpLossScale {
    float scale;
    uint32_t overflow;
    uint32_t good_steps;     /* updates since the last change of scale */
    uint32_t skipped_steps;
} NgpLossScale;

typedef struct NgpLossScaleDescriptor {
    float growth_factor;     /* 2 */
    float backoff_factor;    /* 0.5 */
    uint32_t growth_interval;/* 2000 updates without overflow double the scale */
    float max_scale;         /* 2^24 */
    float min_scale;         /* 1 */
} NgpLossScaleDescriptor;

/* After both Adam updates of a step: on overflow, scale *= backoff (not below min_scale),
 * good_steps = 0, skipped_steps += 1; else good_steps += 1 and every growth_interval such steps
 * scale *= growth (not above max_scale).  Clears overflow.
 * buffers: loss_scale NgpLossScale[1] (updated in place, passed as the result). */
void ngp_loss_scale_update(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_loss_scale_update_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

typedef struct NgpFieldMixedDescriptor {
    uint32_t n_samples;
    uint32_t accumulate;     /* backward only: add into dL_dweights instead of overwriting */
    uint32_t operand;        /* MMA operand type: NGP_DTYPE_BF16 or NGP_DTYPE_F16 */
    uint32_t activations;    /* storage of encodings and dL_dencodings: NGP_DTYPE_F32 or `operand` */
} NgpFieldMixedDescriptor;

/* The field ops on the tensor cores with a chosen 16-bit operand type, FP32 accumulation and
 * FP32 outputs (drgbs, sigma, dL_dweights).  Encodings (and their gradient) are FP32 or stored in
 * the operand type; 16-bit encodings give the same result as their FP32 values, since those are
 * rounded to the operand type on the way into the first MMA.
 * forward:  encodings, dirs f32[S,3], weights f32[9408], active_count u32[1] or NULL -> drgbs f32[S,4]
 * density:  encodings, weights -> sigma f32[S]
 * backward: encodings, dirs, weights, dL_ddrgbs f32[S,4], active_count or NULL, grad_scale f32[1]
 *           or NULL, loss_scale NgpLossScale[1] or NULL, scratch f32[ngp_field_backward_scratch_floats()]
 *           -> dL_dencodings, dL_dweights f32[9408]
 * opaque: NgpFieldMixedDescriptor.  With a loss scale the gradients come out multiplied by its
 * scale, and a value that overflows its 16-bit type sets its overflow flag. */
void ngp_field_forward_mixed(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_field_forward_mixed_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
void ngp_field_density_mixed(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_field_density_mixed_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
void ngp_field_backward_mixed(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_field_backward_mixed_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

typedef struct NgpHashGridMixedDescriptor {
    NgpHashGridDescriptor grid;
    uint32_t table;          /* forward: latents' type (NGP_DTYPE_F32, _BF16 or _F16) */
    uint32_t encodings;      /* encodings / dL_dencodings type (NGP_DTYPE_F32, _BF16 or _F16) */
} NgpHashGridMixedDescriptor;

/* ngp_hashgrid_forward reading a 16-bit copy of the latent table and/or writing 16-bit encodings:
 * the corner values are widened to FP32 and interpolated in the FP32 order of the FP32 op, the
 * result rounded once to the encodings' type.
 * buffers: pos f32[N,3], latents [P,2] of `table`, active_count u32[1] or NULL -> encodings [N,L*2]
 * of `encodings`.  opaque: NgpHashGridMixedDescriptor. */
void ngp_hashgrid_forward_mixed(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_hashgrid_forward_mixed_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* ngp_hashgrid_backward with dL_dencodings of type `encodings` (`table` is ignored: the gradient
 * table is FP32, accumulated with FP32 atomics).
 * buffers: pos f32[N,3], dL_dencodings [N,L*2], active_count u32[1] or NULL -> dL_dlatents f32[P,2].
 * opaque: NgpHashGridMixedDescriptor. */
void ngp_hashgrid_backward_mixed(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_hashgrid_backward_mixed_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

typedef struct NgpAdamMixedDescriptor {
    NgpAdamDescriptor adam;
    uint32_t half_copy;      /* NGP_DTYPE_BF16 / _F16: also write the updated params in that type;
                              * NGP_DTYPE_F32: no copy */
} NgpAdamMixedDescriptor;

/* ngp_adam on FP32 master parameters with a dynamic loss scale and a 16-bit working copy.  With a
 * loss scale: a step whose overflow flag is set leaves params and moments unchanged (the gradient
 * is still zeroed when zero_grad is set); otherwise the gradient is divided by the scale first and
 * the bias correction uses step - skipped_steps.  Without one this is ngp_adam.
 * buffers: params f32[n], grads f32[n], m f32[n], v f32[n], loss_scale NgpLossScale[1] or NULL
 * -> params_half [n] of half_copy (or NULL).  opaque: NgpAdamMixedDescriptor. */
void ngp_adam_mixed(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_adam_mixed_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* ------------------------------------------------------------------ synthetic scene data */
typedef struct NgpRenderBlobsDescriptor {
    uint32_t n_rays;       /* pixels to render: view0 * H * W onwards, n_rays of them */
    uint32_t n_blobs;
    uint32_t n_steps;      /* quadrature steps across the scene box */
    uint32_t width, height, n_views;
    uint32_t view0;        /* first view rendered */
    uint32_t n_shells;
    float fx, fy, cx, cy;
    float bound;
} NgpRenderBlobsDescriptor;

/* Ground truth for the synthetic scenes: midpoint quadrature of the emission-absorption integral
 * through a sum of isotropic Gaussian density blobs (and thin spherical shells), colour the
 * density-weighted blend of the blob colours.  Output RGBA u8 with alpha = opacity and straight
 * (not premultiplied) colour, as an RGBA photograph of the object.
 * buffers: transforms f32[V,12], blobs f32[B,8] (cx, cy, cz, sigma, peak, r, g, b),
 * shells f32[S,8] (cx, cy, cz, radius, thickness, peak, c0, c1; colour (c0, c0, c1)) -> rgba u8[n_rays,4]. */
void ngp_render_blobs(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_render_blobs_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* ------------------------------------------------------------- occupancy-grid maintenance */
typedef struct NgpOgridDescriptor {
    uint32_t K, G;          /* cascades, grid resolution */
    uint32_t cascade;       /* cascade being updated */
    uint32_t n_points;      /* M: cells updated this round */
    uint32_t update_all;    /* point j is in cell j (the first 256 steps, types.py:1166-1169) */
    float bound;            /* scene AABB half-width */
    float decay;            /* 0.95 (types.py:1161) */
    float threshold_step;   /* 0.01 * diag / (2 min(bound,1) sqrt3) (types.py:1385-1386) */
    uint64_t seed;
    /* camera data for ngp_ogrid_mark_untrained */
    uint32_t n_views, width, height;
    float fx, fy, cx, cy;
} NgpOgridDescriptor;

/* types.py:1161-1162: density *= decay for the live cells (>= 0) of `cascade`.
 * buffers: density f32[K*G^3] (updated in place, passed as the result). */
void ngp_ogrid_decay(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_ogrid_decay_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* types.py:1164-1204: pick n_points cells of `cascade` and a uniform point in each (world space).
 * buffers: density f32[K*G^3], occupancy_bitfield u8[K*G^3/8] -> cells u32[M] (0xFFFFFFFF for a
 * dead cell), xyzs f32[M,3]. */
void ngp_ogrid_sample(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_ogrid_sample_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* types.py:1218-1220: density[cell] = max(density[cell], sigma).
 * buffers: cells u32[M], sigma f32[M] -> density f32[K*G^3] (in place). */
void ngp_ogrid_max(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_ogrid_max_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* types.py:1227-1231: threshold = min(threshold_step, mean live density of cascade 0).
 * buffers: density f32[K*G^3], scratch f32[2] -> threshold f32[1]. */
void ngp_ogrid_threshold(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_ogrid_threshold_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* types.py:1241-1362 (pinhole cameras): cells no training camera sees get density -1.
 * buffers: transforms f32[V,12] -> density f32[K*G^3] (in place). */
void ngp_ogrid_mark_untrained(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_ogrid_mark_untrained_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* packbits with one device-scalar threshold (no materialised per-cell threshold array).
 * buffers: threshold f32[1], density f32[n] -> occupied_mask bool[n], bitfield u8[n/8];
 * opaque: PackbitsDescriptor. */
void ngp_packbits_scalar(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_packbits_scalar_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* --------------------------------------------------------------------- learned proposal sampler
 * No reference counterpart (the reference samples by marching the occupancy grid only).  A ray's
 * samples come from a small density network instead of the march: a 3D DDA over coarse blocks of
 * 8^3 occupancy cells gives the ray's occupied interval (no interval: a valid ray with no
 * samples), the interval is cut into NGP_PROPOSAL_BINS bins, the proposal network's log density
 * at the bin centres defines a piecewise-constant pdf (mixed with a share `mix` of a uniform one), whose
 * inverse CDF at stratified levels cuts the interval into spr pieces (samples per ray), dense where
 * the pdf is high; a sample sits at the middle of each piece and stands for it (dss = its length),
 * written in march_rays' layout so that the field, the integrator and the loss run unchanged.  Slot j of a
 * fitting ray starts at sample j * spr, spr = the descriptor's samples_per_ray (default
 * NGP_PROPOSAL_SAMPLES); below, S/spr is the number of slots.  The network (4-level hash grid, MLP
 * 8 -> 64 -> 64 -> 1) regresses the field's log density at the field's samples. */
#define NGP_PROPOSAL_BINS 64
#define NGP_PROPOSAL_SAMPLES 48
#define NGP_PROPOSAL_WEIGHTS 4672 /* P0[8,64] P1[64,64] P2[64,1], packed */

typedef struct NgpProposalDescriptor {
    uint32_t n;             /* rays (proposal_rays) or points (proposal_loss) */
    uint32_t total_samples; /* sample budget S; slots = S / samples_per_ray */
    uint32_t G;             /* occupancy grid resolution (cascade 0; a multiple of 8) */
    float bound;
    uint32_t perturb;       /* proposal_sample: jitter the stratified draws */
    uint32_t seed_lo, seed_hi;
    uint32_t count_index;   /* proposal_loss: points bounded by counts[count_index] (0 slots, 1 bins,
                               2 samples); 3 = all n points */
    uint32_t sigma_stride;  /* proposal_loss: stride of the target densities (4 for drgbs rows) */
    uint32_t samples_per_ray; /* samples of a ray with an interval, 1..1024; 0 = NGP_PROPOSAL_SAMPLES */
    float mix;              /* proposal_sample: share of a uniform pdf mixed into the proposal's */
} NgpProposalDescriptor;

/* buffers: occupancy_bitfield u8[G^3/8] -> coarse u8[(G/8)^3]. */
void ngp_proposal_coarse(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_proposal_coarse_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* buffers: rays_o f32[R,3], rays_d f32[R,3], t_starts f32[R], t_ends f32[R], coarse u8[(G/8)^3]
 * -> next_sample_write_location u32[1], number_of_exceeded_samples u32[1], ray_is_valid bool[R],
 * rays_n_samples u32[R], rays_sample_startidx u32[R], ray_of_slot u32[S/spr], slot_t_start f32[S/spr],
 * slot_t_end f32[S/spr], counts u32[3] (slots, bin points, samples).  A ray without an interval
 * is valid with no samples unless it is taken up (a warp at a time) after the slots filled. */
void ngp_proposal_rays(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_proposal_rays_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* buffers: counts u32[3], rays_o, rays_d, ray_of_slot, slot_t_start, slot_t_end -> points f32[S/spr*64,3]. */
void ngp_proposal_bin_points(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_proposal_bin_points_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* buffers: counts u32[3], rays_o, rays_d, ray_of_slot, slot_t_start, slot_t_end, x_bins f32[S/spr*64]
 * -> idcs u32[S], xyzs f32[S,3], dirs f32[S,3], dss f32[S], z_vals f32[S]. */
void ngp_proposal_sample(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_proposal_sample_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* Per-ray fallback of the proposal sampler to the occupancy-grid march (no reference
 * counterpart).  Where the grid marks a bin's cell occupied, the field's density is at least the
 * grid's threshold; where the proposal's density is below it, the proposal misses mass the field
 * has.  A slot whose ray misses more than 1% of its transmittance -- the sum over occupied bins of
 * T_i (1 - exp(-max(0, threshold - sigma_i) delta)), T_i the proposal's transmittance before
 * bin i -- is flagged and its ray appended to the fallback list.
 * buffers: counts u32[3], rays_o, rays_d, ray_of_slot, slot_ta, slot_tb, x_bins f32[slots*64],
 * occupancy bitfield u8[G^3/8], threshold f32[1] -> slot_flag u8[slots], fallback_rays u32[R],
 * fallback_count u32[1] (zeroed by the call), fallback_total u32[1] (accumulated across calls).
 * opaque: NgpProposalDescriptor (n = R, total_samples, G, bound, samples_per_ray; K = 1). */
void ngp_proposal_judge(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_proposal_judge_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* The training march (ngp_march_rays_train's probe form) over the rays fallback_rays[0 ..
 * *fallback_count), allocating sample ranges from next_sample_write_location /
 * number_of_exceeded_samples as they stand: the counters are not reset and the unwritten tail is
 * not zeroed, because ngp_proposal_sample_alloc allocates after it.  A warp marches one listed ray
 * (32-step lookahead); each ray's count, validity and samples are those ngp_march_rays_train gives
 * it.
 * buffers: the 16 buffers of march_rays, then queue u32[1] (scratch, zeroed by the call),
 * fallback_rays u32[n], fallback_count u32[1].  opaque: MarchingDescriptor (n_rays bounds the list). */
void ngp_march_rays_fallback(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_march_rays_fallback_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* ngp_proposal_sample for the fallback flow: slots flagged by ngp_proposal_judge are skipped (their
 * rays were marched); every other slot takes samples_per_ray samples from the same counters (rays
 * past the budget are invalid, as in march_rays) and writes its ray's validity, count and start.
 * counts[2] becomes the number of samples written and the buffers past it are zeroed.
 * buffers: counts u32[3] (in/out), rays_o, rays_d, ray_of_slot, slot_ta, slot_tb, x_bins,
 * slot_flag u8[slots], next_sample_write_location u32[1], number_of_exceeded_samples u32[1] ->
 * idcs, xyzs, dirs, dss, z_vals, ray_is_valid, rays_n_samples, rays_sample_startidx.
 * opaque: NgpProposalDescriptor. */
void ngp_proposal_sample_alloc(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_proposal_sample_alloc_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* Log-density regression: dL/dx = 2 w (x - log(sigma + 1e-3)) / n, w = 2 below the target, else 1.
 * buffers: counts u32[3] or NULL, x f32[n], sigma f32[n*stride] -> dL_dx f32[n], loss f32[1]
 * (the loss sum is added; the caller zeroes it). */
void ngp_proposal_loss(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_proposal_loss_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);

/* The proposal network's MLP.  forward buffers: encodings f32[n,8], weights f32[4672],
 * active_count u32[1] or NULL -> x f32[n].  backward buffers: encodings, weights, dL_dx f32[n],
 * active_count or NULL, scratch f32[ngp_proposal_backward_scratch_floats()] -> dL_dencodings
 * f32[n,8], dL_dweights f32[4672].  opaque: NgpMlpDescriptor. */
void ngp_proposal_mlp_forward(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_proposal_mlp_forward_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
/* ngp_proposal_mlp_forward on the tensor cores (tcgen05, FP16 operands, FP32 accumulation); same
 * buffers.  The sampler evaluates its bins with it. */
void ngp_proposal_mlp_forward_f16(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_proposal_mlp_forward_f16_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
void ngp_proposal_mlp_backward(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
int ngp_proposal_mlp_backward_status(cudaStream_t stream, void **buffers, const char *opaque, size_t opaque_len);
size_t ngp_proposal_backward_scratch_floats(void);

#ifdef __cplusplus
}
#endif

#endif /* NGP_GB300_H_ */
