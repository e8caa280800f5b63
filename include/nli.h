/*
 * nli.h -- C ABI of the GB300 (sm_103a) multiscale non-local inpainting path.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, and
 * returns an int status (NLI_OK == 0).  Unless a function says "host
 * pointers", every array argument is a CUDA device pointer on the context's
 * device, and all work is enqueued on the context's stream.  Functions that
 * return a scalar result (an energy, a total difference) synchronise that
 * stream before returning.
 *
 * Data layout (identical to the reference containers):
 *   image  : float32, interleaved HWC, element (x, y, c) at C*(W*y + x) + c
 *            (image.hpp:481-485, FixedImage<T>::get_index)
 *   mask   : uint8 per pixel, 0 or 1 (FixedMask stores one bool per pixel)
 *   NNF    : int32 pairs, element (x, y) at 2*(W*y + x): the absolute centre
 *            (x, y) of the matched source patch, (-1, -1) for none
 *            (Image<Point>, patch_match.cpp:335)
 *   gradient: float32, 2C interleaved channels [gx_0, gy_0, gx_1, gy_1, ...]
 *            (gradient.cpp:36-70)
 *
 * Each declaration names the reference interface it replaces (file:line in
 * Tom-Zheng/non-local-inpainting).
 */
#ifndef NLI_H_
#define NLI_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
enum {
	NLI_OK = 0,
	NLI_E_INVALID = -1,          /* bad argument (null pointer, size <= 0, ...) */
	NLI_E_EMPTY_SOURCE = -2,     /* image_inpainting.cpp:382-384 "Empty source mask" */
	NLI_E_CHANNELS = -3,         /* l2_rgbd_patch_distance.cpp:112 "Channels do not match" */
	NLI_E_SHAPE = -4,            /* size mismatch; PatchMatch::calculate returns an empty
	                                image in this case (patch_match.cpp:317-322) */
	NLI_E_UNSUPPORTED = -5,      /* distance / updater / patch size with no GPU kernel */
	NLI_E_CUDA = -6,             /* a CUDA runtime call failed */
	NLI_E_TIMEOUT = -7,          /* a device-side wait ran out of its iteration budget */
	NLI_E_NOMEM = -8             /* device allocation failed */
};

/* APatchDistance subclasses (a_patch_distance.h:24) */
enum {
	NLI_DIST_L2_COMBINED = 0,    /* L2CombinedPatchDistance (l2_combined_patch_distance.cpp:39-148) */
	NLI_DIST_L2_RGBD = 1,        /* L2RGBDPatchDistance (l2_rgbd_patch_distance.cpp:41-117) */
	NLI_DIST_L2_NORM = 2,        /* L2NormPatchDistance (l2_norm_patch_distance.cpp:22-104) */
	NLI_DIST_L1_NORM = 3         /* L1NormPatchDistance (l1_norm_patch_distance.cpp:22-105) */
};

/* AImageUpdating subclasses (a_image_updating.h:27) */
enum {
	NLI_UPDATE_MEANS = 0,        /* PatchNonLocalMeans   (patch_non_local_means.cpp:23-100) */
	NLI_UPDATE_MEDIANS = 1,      /* PatchNonLocalMedians (patch_non_local_medians.cpp:23-127) */
	NLI_UPDATE_POISSON = 2,      /* PatchNonLocalPoisson (patch_non_local_poisson.cpp:36-477) */
	NLI_UPDATE_DEPTH = 3         /* PatchNonLocalDepth   (patch_non_local_depth.cpp:36-55) */
};

/* ImageInpainting::InitType, same order (image_inpainting.h:41) */
enum {
	NLI_INIT_BLACK = 0,
	NLI_INIT_AVG = 1,
	NLI_INIT_NONE = 2,
	NLI_INIT_POISSON = 3
};

#define NLI_MAX_PATCH 15      /* largest patch side with a GPU kernel */
#define NLI_MAX_SCALES 32

/* Parameters of an APatchDistance object (a_patch_distance.h:28,
 * l2_combined_patch_distance.h:31, l2_rgbd_patch_distance.h:31). */
typedef struct nli_distance_params {
	int32_t kind;        /* NLI_DIST_* */
	int32_t patch_x;     /* Shape::size_x of the patch */
	int32_t patch_y;     /* Shape::size_y of the patch */
	float   sigma;       /* Gaussian sigma of the intra-patch weights */
	float   lambda;      /* L2Combined: lambda.  L2RGBD: lambda_rgb */
	float   lambda_d;    /* L2RGBD: lambda of the depth channel */
} nli_distance_params;

/* Parameters of a PatchMatch object (patch_match.h:44-47). */
typedef struct nli_patchmatch_params {
	int32_t iterations;    /* sweeps per calculate() (reference default 10) */
	int32_t random_shots;  /* shots per random-search window (CLI: 30) */
	int32_t window;        /* largest random-search window; -1 = max(W, H) */
} nli_patchmatch_params;

/* Parameters of an AImageUpdating object (a_image_updating.h:28,
 * patch_non_local_poisson.h:29-33, patch_non_local_depth.h). */
typedef struct nli_update_params {
	int32_t method;      /* NLI_UPDATE_* */
	int32_t patch_x;
	int32_t patch_y;
	float   sigma;       /* Gaussian sigma of the patch weights */
	float   lambda;      /* NL-Poisson: lambda.  NL-depth: lambda_rgb */
	float   lambda_d;    /* NL-depth: lambda of the depth channel */
	float   cg_tol;      /* CG stops when |r|^2 < cg_tol * |r0|^2 */
	int32_t cg_iters;    /* CG iteration limit */
} nli_update_params;

/* Parameters of an ImageInpainting object (image_inpainting.h:44-50) plus
 * the objects it is wired to (main.cpp:236-270). */
typedef struct nli_process_params {
	nli_distance_params   distance;
	nli_patchmatch_params patchmatch;
	nli_update_params     update;
	int32_t iterations;         /* iterations_amount */
	float   tolerance;          /* stop a scale when sum (du)^2 <= tolerance */
	int32_t scales;             /* scales_amount */
	float   subsampling_rate;   /* see nli_subsampling_rate() */
	float   conf_decay_time;    /* confidence_decay_time */
	float   conf_asymptotic;    /* confidence_asymptotic_value */
	int32_t init;               /* NLI_INIT_* */
} nli_process_params;

/* What one process() call did (the reference prints these, image_inpainting.cpp:165-407). */
typedef struct nli_process_stats {
	int32_t scales;
	int32_t width[NLI_MAX_SCALES];       /* index 0 = finest */
	int32_t height[NLI_MAX_SCALES];
	int32_t iterations[NLI_MAX_SCALES];  /* inpaint_internal iterations per scale */
	double  last_difference[NLI_MAX_SCALES];
	int64_t patchmatch_calls;
	int64_t update_calls;
	int64_t cg_iterations;               /* summed over channels and solves */
	int64_t candidates;                  /* patch distances evaluated by PatchMatch */
	int64_t graph_iterations;            /* of the iterations, those run in captured loops
	                                        (NLI_TUNE_GRAPH_LOOP) */
	int32_t targets[NLI_MAX_SCALES];     /* PatchMatch target points per scale (the
	                                        extended domain minus the margin) */
	int32_t holes[NLI_MAX_SCALES];       /* hole pixels per scale (the CG's unknowns) */
	int64_t candidates_partial;          /* of the candidates, those stopped after the
	                                        early-termination test */
} nli_process_stats;

typedef struct nli_ctx nli_ctx;

/* ---- context ------------------------------------------------------------- */
const char *nli_version(void);
const char *nli_status_string(int status);
/* Creates a context on CUDA device `device` with its own non-blocking stream. */
int nli_ctx_create(int device, nli_ctx **out);
int nli_ctx_destroy(nli_ctx *ctx);
/* Enqueues all further work of this context on `stream` (a cudaStream_t;
 * NULL is the legacy default stream) instead of the context's own
 * non-blocking stream. */
int nli_ctx_set_stream(nli_ctx *ctx, void *stream);
/* Seed of the counter-based PatchMatch RNG.  The reference seeds rand() with
 * srand(time(NULL)) (main.cpp:273); a fixed seed makes runs repeatable. */
int nli_set_seed(nli_ctx *ctx, uint64_t seed);
int nli_ctx_synchronize(nli_ctx *ctx);
/* Message of the last failing call on this context (never NULL). */
const char *nli_last_error(nli_ctx *ctx);

/* ---- observability (the reference's METRICS / progress prints,
 * patch_match.cpp:383-507, image_inpainting.cpp:396-407) ------------------- */
/* Number of kernels this library has launched in this process. */
int64_t nli_launch_count(void);
/* Turns per-kernel GPU timing on or off (CUDA events around each launch on
 * the context stream) and clears the collected entries. */
int nli_ctx_set_profiling(nli_ctx *ctx, int enable);
/* Entry `index` (0-based, sorted by name) of the collected timings:
 * kernel name, launches and total milliseconds.  NLI_E_INVALID past the end. */
int nli_ctx_profile_entry(nli_ctx *ctx, int index, char *name, int name_len, int64_t *launches, double *ms);
/* Running totals of this context: PatchMatch distance evaluations counted
 * on the device, the part of them stopped early (after the first 32 taps
 * their partial sum already exceeded the current match), conjugate-gradient
 * iterations (summed over channels) and the same weighted by the number of
 * unknowns of each solve.  Any pointer may be NULL. */
int nli_ctx_counters(nli_ctx *ctx, int64_t *candidates, int64_t *candidates_partial, int64_t *cg_iterations,
                     int64_t *cg_unknown_iterations);

/* ---- numeric helpers (L1) ------------------------------------------------ */
/* GaussianWeights::calculate (gaussian_weights.cpp:19-79).  Host pointers:
 * writes size_x*size_y floats.  size_y == 1 gives the 1-D form used by the
 * pyramid filter (exp(-x^2/sigma^2), gaussian_weights.cpp:37). */
int nli_gaussian_weights(int size_x, int size_y, float sigma_x, float sigma_y, float *host_out);

/* ImageInpainting::calculate_subsampling_rate (image_inpainting.cpp:197-204). */
float nli_subsampling_rate(float size_ratio, unsigned int scales);

/* Sampling::_Details::get_sample_size (sampling.cpp:408-411). */
int nli_sample_size(int size, float factor);

/* Gradient::calculate, forward differences (gradient.cpp:20-75). */
int nli_gradient(nli_ctx *ctx, const float *image, int W, int H, int C, float *gradient);

/* Sampling::downsample_with_mask (sampling.cpp:114-202).  out_image must hold
 * oW*oH*C floats and out_mask oW*oH bytes, oW = nli_sample_size(W, factor). */
int nli_downsample_with_mask(nli_ctx *ctx, const float *image, const uint8_t *mask,
                             int W, int H, int C, float factor, float threshold, int mask_val,
                             float *out_image, uint8_t *out_mask);

/* Sampling::upsample, nearest neighbour (sampling.cpp:205-246, 387-406). */
int nli_upsample(nli_ctx *ctx, const float *image, int W, int H, int C,
                 int out_W, int out_H, float *out_image);

/* DistanceTransform::calculate (distance_transform.cpp:20-99): distance of
 * every pixel to the nearest pixel with mask == 0. */
int nli_distance_transform(nli_ctx *ctx, const uint8_t *mask, int W, int H, float *distances);

/* ImageInpainting::calculate_confidence_mask (image_inpainting.cpp:611-630). */
int nli_confidence_mask(nli_ctx *ctx, const uint8_t *mask, int W, int H,
                        float decay_time, float asymptotic_value, float *confidence);

/* ImageInpainting::get_extended_domain (image_inpainting.cpp:566-600). */
int nli_extended_domain(nli_ctx *ctx, const uint8_t *mask, int W, int H,
                        int patch_x, int patch_y, uint8_t *extended);

/* Source and target masks of one scale: target = extended domain, source =
 * its complement, eroded where the right or bottom neighbour is not source
 * when `erode` != 0 (image_inpainting.cpp:361-377), then a `margin` wide
 * border is cleared in both (add_margin, image_inpainting.cpp:641-657).
 * *source_empty is set as image_inpainting.cpp:368-384 computes it (before
 * the margin).  With erode == 0 this is the mask pair of propagate_weights
 * (image_inpainting.cpp:501-506, 545-549). */
int nli_scale_masks(nli_ctx *ctx, const uint8_t *extended, int W, int H, int margin, int erode,
                    uint8_t *source, uint8_t *target, int *source_empty);

/* Coarsest-scale hole filling, InitPoisson branch of ImageInpainting::process
 * (image_inpainting.cpp:125-153) -> poisson_solver_separable_simplest
 * (3rdparty/simpois/simpois.c:281-291).  Replaces image pixels where mask != 0. */
int nli_poisson_init(nli_ctx *ctx, float *image, const uint8_t *mask, int W, int H, int C);

/* ---- patch distances (L2a) ----------------------------------------------- */
/* APatchDistance::calculate over a list of pairs (a_patch_distance.h:34,
 * l2_combined_patch_distance.cpp:39-148, l2_rgbd_patch_distance.cpp:41-117,
 * l2_norm_patch_distance.cpp:22-104, l1_norm_patch_distance.cpp:22-105).
 * pairs: n x int32[4] = (source x, source y, target x, target y), patch
 * centres; every patch must lie inside its image.  Source and target are
 * initialize()d from `source` and `target` (gradients computed here).
 * Arithmetic follows the reference: per-tap float norms, double sums. */
int nli_distance_pairs(nli_ctx *ctx, const nli_distance_params *dist,
                       const float *source, int sW, int sH,
                       const float *target, int tW, int tH, int C,
                       const int32_t *pairs, int n, float *out);

/* Allocation-free nli_distance_pairs, for callers that cannot allocate
 * device memory while they run (a host framework that reserves the whole
 * device budget up front, or a latency-critical loop in which cudaMalloc /
 * cudaFree would synchronise the device).  No counterpart in the reference:
 * it computes exactly what nli_distance_pairs computes, but takes no context,
 * calls no cudaMalloc / cudaFree, and keeps its gradient images in a fixed
 * device array of NLI_NOALLOC_SCRATCH_BYTES that every process loading this
 * library holds on each device it uses until exit.  Work is enqueued on
 * `stream` (a cudaStream_t, NULL = legacy default stream) of the current
 * device.  The first call in a CUDA context (a device's primary context, or
 * a context the caller made current) looks up the array's device address in
 * that context; make that first call before any stream capture.  A context
 * re-created by cudaDeviceReset counts as a new one.  Returns NLI_E_INVALID
 * when the gradients needed (sW*sH*2C floats, plus tW*tH*2C when target is
 * a different image; none for the L2Norm/L1Norm kinds) exceed
 * NLI_NOALLOC_SCRATCH_BYTES.  All calls share the array: calls that overlap
 * on the GPU race and must be ordered by the caller. */
#define NLI_NOALLOC_SCRATCH_BYTES (8u << 20)
int nli_distance_pairs_noalloc(const nli_distance_params *dist,
                               const float *source, int sW, int sH,
                               const float *target, int tW, int tH, int C,
                               const int32_t *pairs, int n, float *out, void *stream);

/* Exhaustive nearest neighbour: for every target pixel with target_mask != 0,
 * the source pixel with source_mask != 0 of least distance (ties -> lowest
 * raster index y*sW + x).  Same arithmetic as nli_distance_pairs.  Points
 * whose patch would leave its image are skipped (NNF (-1,-1)). */
int nli_bruteforce_nnf(nli_ctx *ctx, const nli_distance_params *dist,
                       const float *source, const uint8_t *source_mask, int sW, int sH,
                       const float *target, const uint8_t *target_mask, int tW, int tH, int C,
                       int32_t *nnf, float *distance);

/* ---- correspondence (L3) ------------------------------------------------- */
/* PatchMatch::calculate (patch_match.cpp:311-512).  init_nnf may be NULL
 * (random initialisation, patch_match.cpp:361-381).  out_nnf gets tW*tH
 * pairs, (-1,-1) outside target_mask; out_distance (may be NULL) gets the
 * matched distance (FLT_MAX where none); *energy (may be NULL) gets the sum
 * of matched distances over the target points. */
int nli_patchmatch(nli_ctx *ctx, const nli_distance_params *dist, const nli_patchmatch_params *pm,
                   const float *source, const uint8_t *source_mask, int sW, int sH,
                   const float *target, const uint8_t *target_mask, int tW, int tH, int C,
                   const int32_t *init_nnf, int32_t *out_nnf, float *out_distance, double *energy);

/* PatchMatch::calculate as built with METRICS (patch_match.cpp:383-507,
 * 574-590): nli_patchmatch plus, per sweep (pm->iterations entries), the
 * sum of the matched distances after the sweep (total_distance) and the
 * number of target points the propagation step improved (propagations),
 * and the largest index of a first accepted random draw over the call
 * (*max_random_shots).  Each output may be NULL. */
int nli_patchmatch_metrics(nli_ctx *ctx, const nli_distance_params *dist, const nli_patchmatch_params *pm,
                           const float *source, const uint8_t *source_mask, int sW, int sH,
                           const float *target, const uint8_t *target_mask, int tW, int tH, int C,
                           const int32_t *init_nnf, int32_t *out_nnf, float *out_distance, double *energy,
                           double *total_distance, int64_t *propagations, int32_t *max_random_shots);

/* ---- image updating (L2b) ------------------------------------------------ */
/* AImageUpdating::update (a_image_updating.h:34-39): updates `image` in
 * place on `domain`, returns sum over domain of (old - new)^2.  `orig` may
 * alias `image`.  confidence may be NULL (all ones). */
int nli_update(nli_ctx *ctx, const nli_update_params *upd,
               float *image, const float *orig, const uint8_t *domain, const uint8_t *ext_domain,
               const int32_t *nnf, const float *confidence, int W, int H, int C,
               double *total_difference);

/* ---- adjoint of the image update ----------------------------------------- */
/* Backward of one update step with the NNF held fixed (no reference
 * counterpart: the reference is not differentiable).  The step is
 * out = U(image; lambda, sigma) as nli_update computes it with orig = image
 * (AImageUpdating::update, a_image_updating.h:34-39, as called by
 * image_inpainting.cpp:394).  Given out (the forward result) and grad_out =
 * dL/dout (W*H*C), writes grad_image = dL/dimage (W*H*C), *grad_lambda =
 * dL/dlambda (the channels using upd->lambda), *grad_lambda_d = dL/dlambda_d
 * (channel 3 of NLI_UPDATE_DEPTH, else 0) and *grad_sigma = dL/dsigma of the
 * Gaussian patch weights.  NL-means: backward of the weighted average.
 * NL-Poisson / NL-depth: a second CG solve A z = grad_out on the hole with
 * the forward's system (upd->cg_tol, upd->cg_iters), then the adjoints of
 * the coefficient gathers with the weights recomputed.  NL-medians returns
 * NLI_E_UNSUPPORTED (piecewise constant).  Device pointers; blocks until the
 * scalars are on the host. */
int nli_update_backward(nli_ctx *ctx, const nli_update_params *upd, const float *image, const float *out,
                        const uint8_t *domain, const uint8_t *ext_domain, const int32_t *nnf,
                        const float *confidence, int W, int H, int C, const float *grad_out,
                        float *grad_image, double *grad_lambda, double *grad_lambda_d, double *grad_sigma);

/* ---- multiscale driver (L4) ---------------------------------------------- */
/* ImageInpainting::process (image_inpainting.cpp:68-190).  Host pointers:
 * image (W*H*C floats), mask (W*H bytes), out (W*H*C floats).  The host
 * copies are part of the call.  stats may be NULL. */
int nli_process(nli_ctx *ctx, const nli_process_params *params,
                const float *image, const uint8_t *mask, int W, int H, int C,
                float *out, nli_process_stats *stats);

/* Same as nli_process with device pointers (no host copies). */
int nli_process_device(nli_ctx *ctx, const nli_process_params *params,
                       const float *image, const uint8_t *mask, int W, int H, int C,
                       float *out, nli_process_stats *stats);

/* ImageInpainting::keep_intermediate (image_inpainting.cpp:310-313): while
 * enabled, each nli_process / nli_process_device call on this context keeps
 * host copies of its pyramids, replaced by the next call:
 *   NLI_INTER_INPUT  per level (index 0 = finest) the image after
 *                    downsampling, before the coarsest initialisation
 *                    (get_input_image_pyramid, :103-108, 316-319);
 *   NLI_INTER_OUTPUT per level the inpainted image (get_output_image_pyramid);
 *   NLI_INTER_MASK   per level the hole mask, one byte per pixel (get_mask_pyramid);
 *   NLI_INTER_NNF    the final NNF of every level in the order the levels
 *                    are inpainted, coarsest first, W*H int32 pairs
 *                    (get_nnf_pyramid, :410-412).
 * Batches do not keep intermediates. */
#define NLI_INTER_INPUT 0
#define NLI_INTER_OUTPUT 1
#define NLI_INTER_MASK 2
#define NLI_INTER_NNF 3
int nli_ctx_keep_intermediate(nli_ctx *ctx, int enable);
/* Number of kept entries of `kind`. */
int nli_intermediate_count(nli_ctx *ctx, int kind);
/* Entry `index` of `kind`: sizes in *W, *H, *C (C is 1 for masks and 2 for
 * NNFs); when host_out is not NULL, its W*H*C elements (floats, bytes or
 * int32) are copied there. */
int nli_intermediate_get(nli_ctx *ctx, int kind, int index, int *W, int *H, int *C, void *host_out);

/* ---- colour and channel packing of the command-line caller ------------- */
/* IOUtility::rgb_to_lab (io_utility.cpp:268-289, 380-412): sRGB in 0..255,
 * 3 channels, to CIE L*a*b* (D65).  Device pointers, W*H pixels. */
int nli_rgb_to_lab(nli_ctx *ctx, const float *rgb, int W, int H, float *lab);
/* IOUtility::lab_to_rgb (io_utility.cpp:292-318, 415-449): the first three
 * channels of a C-channel (3 or 4) L*a*b* image to sRGB 0..255 (3 channels). */
int nli_lab_to_rgb(nli_ctx *ctx, const float *lab, int W, int H, int C, float *rgb);
/* IOUtility::cat (io_utility.cpp:452-470): RGB (3 channels) and depth (1)
 * into one 4-channel image. */
int nli_cat_depth(nli_ctx *ctx, const float *rgb, const float *depth, int W, int H, float *rgbd);
/* IOUtility::separate (io_utility.cpp:489-501): the reverse; rgb or depth
 * may be NULL. */
int nli_separate_depth(nli_ctx *ctx, const float *rgbd, int W, int H, float *rgb, float *depth);

/* ---- batched driver ------------------------------------------------------ */
/* Many independent image/mask pairs on one GPU.  The reference has no batch
 * entry point: it replaces a host loop of ImageInpainting::process calls
 * (image_inpainting.cpp:68-190; main.cpp:279 makes one).  Image i has its
 * own parameters params[i], sizes widths[i] x heights[i] x channels[i] and
 * buffers images[i], masks[i], outputs[i]; nli_process_batch takes host
 * pointers (copies inside the call), nli_process_batch_device device
 * pointers (ordered after the work already queued on the context's stream,
 * and the stream waits for the batch).  Up to the context's batch width of
 * images are in flight at once, each on its own stream.  Image i runs
 * exactly as nli_process after nli_set_seed(ctx, nli_batch_seed(seed, i)),
 * seed being the context's seed.  stats (n entries) and status (n entries,
 * the per-image result) may be NULL.  Returns NLI_OK when every image
 * succeeded, else the status of the first failed image (in index order). */
int nli_process_batch(nli_ctx *ctx, int n, const nli_process_params *params,
                      const float *const *images, const uint8_t *const *masks,
                      const int32_t *widths, const int32_t *heights, const int32_t *channels,
                      float *const *outputs, nli_process_stats *stats, int32_t *status);
int nli_process_batch_device(nli_ctx *ctx, int n, const nli_process_params *params,
                             const float *const *images, const uint8_t *const *masks,
                             const int32_t *widths, const int32_t *heights, const int32_t *channels,
                             float *const *outputs, nli_process_stats *stats, int32_t *status);
/* Images in flight in a batch (default 8, at least 1). */
int nli_ctx_set_batch_width(nli_ctx *ctx, int width);

/* Launch-shape knobs, set by the autotuner (non-local-inpainting_gb300/
 * autotune.py) or by hand; results do not depend on them beyond float
 * rounding of the CG sums:
 *   NLI_TUNE_CG_CLUSTER_CAP        CTAs per CG cluster at most (1..16, default 16)
 *   NLI_TUNE_CG_UNKNOWNS_PER_CTA   unknowns per CG CTA at least (default 1024)
 *   NLI_TUNE_BATCH_WIDTH           as nli_ctx_set_batch_width
 *   NLI_TUNE_PM_VARIANT            how 9x9 PatchMatch reads candidate windows:
 *                                  0 (default) target window in shared memory,
 *                                  source rows by plain loads; 1 source windows
 *                                  staged in shared memory by tensor copies;
 *                                  2 target window in registers.  The fields
 *                                  are identical for all three.
 *   NLI_TUNE_CG_PRECOND            NL-Poisson / NL-depth conjugate gradient:
 *                                  0 (default) plain CG as the reference
 *                                  (patch_non_local_poisson.cpp:387-477);
 *                                  1 Jacobi-preconditioned.  Both stop at
 *                                  |r|^2 < cg_tol |r0|^2 on the true
 *                                  residual; 1 needs fewer iterations and
 *                                  its solution differs within that
 *                                  tolerance.
 *   NLI_TUNE_GRAPH_LOOP            1 (default): after the first iteration of
 *                                  a scale, nli_process(_device) runs the
 *                                  remaining PatchMatch / update iterations
 *                                  as one CUDA graph whose while node tests
 *                                  the stopping rule on the device (no host
 *                                  round trip per iteration), and lockstep
 *                                  batches run each pyramid rank's loop as
 *                                  one graph; worker-context batches keep
 *                                  the host loop, where other images' work
 *                                  hides the round trips.  2: the graph in
 *                                  worker-context batches too.  0: the host
 *                                  loop everywhere.  Identical results; the
 *                                  graph is not used while profiling is on.
 *   NLI_TUNE_CG_SINGLE_MAX         CG systems (per channel) of at most this
 *                                  many unknowns are solved by one CTA with
 *                                  block barriers only, instead of a cluster
 *                                  (0..4096, default 1024).
 *   NLI_TUNE_BATCH_MODE            how nli_process_batch(_device) runs a
 *                                  batch: 1 (default) lockstep -- the images
 *                                  walk their pyramids together, one launch
 *                                  per kernel per pyramid rank covers every
 *                                  image, and each rank's iteration loop is
 *                                  one CUDA graph; 0 worker contexts -- up to
 *                                  the batch width of whole nli_process runs
 *                                  on their own streams.  Identical results.
 *   NLI_TUNE_PM_BOUND              PatchMatch skips a candidate whose patch
 *                                  statistics (of the image and its forward
 *                                  differences, weighted by the patch
 *                                  weights) differ from the target's by
 *                                  enough that its distance provably cannot
 *                                  beat the current match: 1 (default) by
 *                                  the weighted means (Jensen's
 *                                  inequality); 2 by the means and the
 *                                  weighted standard deviations (L2 kinds;
 *                                  L1 uses the means): fewer candidates
 *                                  evaluated, but slower on the 512x512
 *                                  benchmark; 0 every candidate is
 *                                  evaluated.  The bound keeps a rounding
 *                                  margin, so fields and distances are
 *                                  identical in all three.
 *   NLI_TUNE_BATCH_GROUPS          lockstep batches: the images of one
 *                                  launch-sharing group are dealt (largest
 *                                  first, to the least-loaded) into this many
 *                                  sub-groups that run concurrently on their
 *                                  own streams and workspaces, so one
 *                                  sub-group's per-rank tail (its slowest
 *                                  image) overlaps another's work (1..16,
 *                                  default 4).  Identical results.
 *   NLI_TUNE_PM_TILE               how the persistent PatchMatch kernels
 *                                  share out the target points: n > 0 a
 *                                  device work queue from which each warp
 *                                  takes n consecutive points per atomic
 *                                  grab (1..1024, default 1); 0 static
 *                                  ranges (block b takes the b-th contiguous
 *                                  range).  Identical fields.
 * nli_ctx_get_tuning reads them back. */
#define NLI_TUNE_CG_CLUSTER_CAP 0
#define NLI_TUNE_CG_UNKNOWNS_PER_CTA 1
#define NLI_TUNE_BATCH_WIDTH 2
#define NLI_TUNE_PM_VARIANT 3
#define NLI_TUNE_CG_PRECOND 4
#define NLI_TUNE_GRAPH_LOOP 5
#define NLI_TUNE_CG_SINGLE_MAX 6
#define NLI_TUNE_BATCH_MODE 7
#define NLI_TUNE_PM_BOUND 8
#define NLI_TUNE_BATCH_GROUPS 9
#define NLI_TUNE_PM_TILE 10
int nli_ctx_set_tuning(nli_ctx *ctx, int knob, int value);
int nli_ctx_get_tuning(nli_ctx *ctx, int knob, int *value);
/* The seed image `index` of a batch runs with. */
uint64_t nli_batch_seed(uint64_t seed, int index);
/* Host-side fault injection for tests: the `countdown`-th next growth of
 * the context's device workspace fails with NLI_E_NOMEM ("device
 * allocation failed (injected)") without calling cudaMalloc; 0 disarms.
 * The reference has no allocation failure path of its own (its containers
 * throw std::bad_alloc); this one checks that a failed call leaves the
 * context usable. */
int nli_debug_fail_allocation(nli_ctx *ctx, int countdown);
/* Test hook for the bounded device waits: the grid CG's grid barrier gives
 * up after `polls` polls (0 restores the default, 2^26).  A wait that runs
 * out sets the context's timeout word, every block of the kernel leaves,
 * and the call returns NLI_E_TIMEOUT ("a device-side wait timed out"); the
 * word is then cleared, so the context stays usable.  The reference has no
 * device waits; this checks the recovery path without hanging a GPU. */
int nli_debug_grid_wait_limit(nli_ctx *ctx, unsigned int polls);
/* Checked builds (libnli_gb300_checked.so, built with NLI_CHECKED): every
 * data-dependent gathered index -- source pixels of PatchMatch candidates,
 * NNF-shifted pixels of the updates, hole lists, CG neighbour codes -- is
 * tested against its buffer; the first out-of-range one is recorded as
 * (site << 32) | (index & 0xffffffff) and its access is skipped.  Reads and
 * clears that record into *word (0: none).  *checked is 1 in checked
 * builds, 0 otherwise (where *word is always 0). */
int nli_debug_check_status(nli_ctx *ctx, unsigned long long *word, int *checked);

#ifdef __cplusplus
}
#endif

#endif /* NLI_H_ */
