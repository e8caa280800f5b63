// The C ABI (include/nli.h): argument checking, context management and the
// translation of internal errors into status codes.  Every entry point that
// computes enqueues CUDA kernels; nothing here falls back to the CPU.
#include <atomic>
#include <cmath>
#include <cstring>
#include <iterator>
#include <new>

#include "nli_device.cuh"
#include "nli_internal.cuh"

namespace nli {

// GaussianWeights::calculate (gaussian_weights.cpp:19-79, SEGMENTS == 1):
// pixel-centre samples of exp(-(x^2/(2 sx^2) + y^2/(2 sy^2))) in double
// (1-D: exp(-x^2/sx^2)), mirrored from the top-left quarter, normalised by
// their float sum.  Computed once per object on the host, like the
// reference, and handed to the kernels as a table.
std::vector<float> gaussian_weights_host(unsigned sx, unsigned sy, float sigma_x, float sigma_y)
{
	std::vector<float> w((size_t)sx * sy, 0.0f);
	const double x_a = -(float)sx / 2, y_a = -(float)sy / 2;
	if (sy == 1) {
		for (unsigned i = 0; i <= sx / 2; i++) {
			double x = x_a + i + 0.5;
			double value = 0.0;
			value += exp(-(pow(x, 2) / pow(sigma_x, 2)));
			w[i] = value;
		}
	} else {
		for (unsigned i = 0; i <= sx / 2; i++)
			for (unsigned j = 0; j <= sy / 2; j++) {
				double x = x_a + i + 0.5, y = y_a + j + 0.5;
				double value = 0.0;
				value += exp(-(pow(x, 2) / (2 * pow(sigma_x, 2)) + pow(y, 2) / (2 * pow(sigma_y, 2))));
				w[(size_t)sx * j + i] = value;
			}
	}
	for (unsigned i = 0; i <= sx / 2; i++)
		for (unsigned j = 0; j <= sy / 2; j++) {
			float v = w[(size_t)sx * j + i];
			w[(size_t)sx * j + (sx - 1 - i)] = v;
			if (sy > 1) {
				w[(size_t)sx * (sy - 1 - j) + i] = v;
				w[(size_t)sx * (sy - 1 - j) + (sx - 1 - i)] = v;
			}
		}
	float sum = 0.0f;
	for (float v : w) sum += v;
	for (float &v : w) v /= sum;
	return w;
}

void fill_dist_args(DistArgs &a, const nli_distance_params &p, int C)
{
	NLI_REQUIRE(p.patch_x >= 1 && p.patch_y >= 1 && p.patch_x <= NLI_MAX_PATCH && p.patch_y <= NLI_MAX_PATCH,
	            NLI_E_UNSUPPORTED, "patch size outside 1.." + std::to_string(NLI_MAX_PATCH));
	NLI_REQUIRE(p.kind >= 0 && p.kind <= 3, NLI_E_UNSUPPORTED, "unknown distance kind");
	NLI_REQUIRE(C >= 1 && C <= 4, NLI_E_UNSUPPORTED, "images must have 1 to 4 channels");
	if (p.kind == NLI_DIST_L2_RGBD)
		NLI_REQUIRE(C == 4, NLI_E_CHANNELS, "L2 RGBD Distance: Channels do not match.");
	std::memset(&a, 0, sizeof(a));
	a.kind = p.kind;
	a.px = p.patch_x;
	a.py = p.patch_y;
	a.rx = p.patch_x / 2;
	a.ry = p.patch_y / 2;
	a.C = C;
	a.lambda = p.lambda;
	a.lambda_d = p.lambda_d;
	std::vector<float> w = gaussian_weights_host(p.patch_x, p.patch_y, p.sigma, p.sigma);
	std::memcpy(a.weights, w.data(), sizeof(float) * w.size());
}

void clear_timeout(nli_ctx *ctx)
{
	// after a synchronize: no kernel of the context is running
	NLI_CUDA(cudaMemset(&ctx->status->timeout, 0, sizeof(int)));
}

}  // namespace nli

using namespace nli;

static int fail(nli_ctx *ctx, const Error &e)
{
	if (ctx) ctx->last_error = e.message;
	return e.status;
}

#define API_BEGIN(ctx)                                                   \
	if (!(ctx)) return NLI_E_INVALID;                                    \
	try {                                                                \
		NLI_CUDA(cudaSetDevice((ctx)->device));

#define API_END(ctx)                                                     \
	}                                                                    \
	catch (const Error &e) {                                             \
		return fail(ctx, e);                                             \
	}                                                                    \
	catch (const std::bad_alloc &) {                                     \
		return fail(ctx, Error{NLI_E_NOMEM, "host allocation failed"}); \
	}                                                                    \
	catch (const std::exception &e) {                                    \
		return fail(ctx, Error{NLI_E_INVALID, e.what()});               \
	}                                                                    \
	return NLI_OK;

static void require_ptrs(std::initializer_list<const void *> ps)
{
	for (const void *p : ps) NLI_REQUIRE(p != nullptr, NLI_E_INVALID, "null pointer argument");
}

static void require_dims(int W, int H, int C)
{
	NLI_REQUIRE(W > 0 && H > 0, NLI_E_INVALID, "image sizes must be positive");
	NLI_REQUIRE(C >= 1 && C <= 4, NLI_E_UNSUPPORTED, "images must have 1 to 4 channels");
}

extern "C" {

const char *nli_version(void) { return "nli-gb300 1.0 (sm_103a)"; }

const char *nli_status_string(int s)
{
	switch (s) {
	case NLI_OK: return "ok";
	case NLI_E_INVALID: return "invalid argument";
	case NLI_E_EMPTY_SOURCE: return "empty source mask";
	case NLI_E_CHANNELS: return "channels do not match";
	case NLI_E_SHAPE: return "size mismatch";
	case NLI_E_UNSUPPORTED: return "unsupported configuration";
	case NLI_E_CUDA: return "CUDA error";
	case NLI_E_TIMEOUT: return "device wait timed out";
	case NLI_E_NOMEM: return "out of memory";
	}
	return "unknown status";
}

int nli_ctx_create(int device, nli_ctx **out)
{
	if (!out) return NLI_E_INVALID;
	*out = nullptr;
	nli_ctx *ctx = nullptr;
	try {
		ctx = new nli_ctx();
		ctx->device = device;
		NLI_CUDA(cudaSetDevice(device));
		NLI_CUDA(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking));
		ctx->stream = ctx->own_stream;
		NLI_CUDA(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device));
		NLI_CUDA(cudaDeviceGetAttribute(&ctx->max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
		NLI_CUDA(cudaMallocHost(&ctx->host_pinned, 4096));
		NLI_CUDA(cudaMalloc(&ctx->status, sizeof(DevStatus)));
		NLI_CUDA(cudaMemset(ctx->status, 0, sizeof(DevStatus)));
	} catch (const Error &e) {
		if (ctx) {
			if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
			if (ctx->host_pinned) cudaFreeHost(ctx->host_pinned);
			if (ctx->status) cudaFree(ctx->status);
			delete ctx;
		}
		return e.status;
	} catch (const std::bad_alloc &) {
		delete ctx;
		return NLI_E_NOMEM;
	}
	*out = ctx;
	return NLI_OK;
}

int nli_ctx_destroy(nli_ctx *ctx)
{
	if (!ctx) return NLI_E_INVALID;
	cudaSetDevice(ctx->device);
	cudaStreamSynchronize(ctx->stream);
	for (nli_ctx *w : ctx->workers) nli_ctx_destroy(w);
	ctx->workers.clear();
	for (auto &kv : ctx->bufs) kv.second.release();
	if (ctx->status) cudaFree(ctx->status);
	if (ctx->host_pinned) cudaFreeHost(ctx->host_pinned);
	if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
	delete ctx;
	return NLI_OK;
}

int nli_ctx_set_stream(nli_ctx *ctx, void *stream)
{
	if (!ctx) return NLI_E_INVALID;
	ctx->stream = (cudaStream_t)stream;
	return NLI_OK;
}

int nli_set_seed(nli_ctx *ctx, uint64_t seed)
{
	if (!ctx) return NLI_E_INVALID;
	ctx->seed = seed;
	try {
		NLI_CUDA(cudaMemsetAsync(&ctx->status->pm_calls, 0, sizeof(unsigned long long), ctx->stream));
	} catch (const Error &e) {
		return fail(ctx, e);
	}
	return NLI_OK;
}

int nli_ctx_synchronize(nli_ctx *ctx)
{
	API_BEGIN(ctx)
	NLI_CUDA(cudaStreamSynchronize(ctx->stream));
	API_END(ctx)
}

const char *nli_last_error(nli_ctx *ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

static std::atomic<long long> g_launches{0};
static thread_local long long t_launches = 0;

void nli_count_launch_internal(void)
{
	g_launches.fetch_add(1, std::memory_order_relaxed);
	t_launches++;
}

long long nli_thread_launch_count_internal(void) { return t_launches; }

void nli_add_launches_internal(long long n)
{
	g_launches.fetch_add(n, std::memory_order_relaxed);
	t_launches += n;
}

int64_t nli_launch_count(void) { return g_launches.load(); }

int nli_ctx_set_profiling(nli_ctx *ctx, int enable)
{
	API_BEGIN(ctx)
	ctx->settle_profile();
	ctx->prof.clear();
	ctx->profiling = enable != 0;
	API_END(ctx)
}

int nli_ctx_profile_entry(nli_ctx *ctx, int index, char *name, int name_len, int64_t *launches, double *ms)
{
	API_BEGIN(ctx)
	ctx->settle_profile();
	NLI_REQUIRE(index >= 0 && index < (int)ctx->prof.size(), NLI_E_INVALID, "profile index out of range");
	auto it = ctx->prof.begin();
	std::advance(it, index);
	if (name && name_len > 0) {
		std::strncpy(name, it->first.c_str(), name_len - 1);
		name[name_len - 1] = 0;
	}
	if (launches) *launches = it->second.launches;
	if (ms) *ms = it->second.ms;
	API_END(ctx)
}

int nli_ctx_counters(nli_ctx *ctx, int64_t *candidates, int64_t *candidates_partial, int64_t *cg_iterations,
                     int64_t *cg_unknown_iterations)
{
	if (!ctx) return NLI_E_INVALID;
	if (candidates) *candidates = ctx->candidates;
	if (candidates_partial) *candidates_partial = ctx->candidates_partial;
	if (cg_iterations) *cg_iterations = ctx->cg_iterations;
	if (cg_unknown_iterations) *cg_unknown_iterations = ctx->cg_unknown_iterations;
	return NLI_OK;
}

int nli_gaussian_weights(int size_x, int size_y, float sigma_x, float sigma_y, float *host_out)
{
	if (size_x <= 0 || size_y <= 0 || !host_out) return NLI_E_INVALID;
	std::vector<float> w = gaussian_weights_host(size_x, size_y, sigma_x, sigma_y);
	std::memcpy(host_out, w.data(), sizeof(float) * w.size());
	return NLI_OK;
}

float nli_subsampling_rate(float size_ratio, unsigned int scales)
{
	// float overloads of exp/log, as image_inpainting.cpp:203 resolves them
	if (size_ratio < 0.0 || size_ratio > 1.0) return 0.0f;
	return std::exp(std::log(size_ratio) / (float)(scales - 1));
}

int nli_sample_size(int size, float factor) { return sample_size_host(size, factor); }

int nli_gradient(nli_ctx *ctx, const float *image, int W, int H, int C, float *gradient)
{
	API_BEGIN(ctx)
	require_ptrs({image, gradient});
	require_dims(W, H, C);
	launch_gradient(ctx->stream, image, W, H, C, gradient);
	API_END(ctx)
}

int nli_downsample_with_mask(nli_ctx *ctx, const float *image, const uint8_t *mask, int W, int H, int C,
                             float factor, float threshold, int mask_val, float *out_image, uint8_t *out_mask)
{
	API_BEGIN(ctx)
	require_ptrs({image, mask, out_image, out_mask});
	require_dims(W, H, C);
	NLI_REQUIRE(factor > 0 && factor < 1.0f, NLI_E_INVALID, "downsampling factor must be in (0, 1)");
	downsample_with_mask_run(ctx, image, mask, W, H, C, factor, threshold, mask_val, out_image, out_mask);
	API_END(ctx)
}

int nli_upsample(nli_ctx *ctx, const float *image, int W, int H, int C, int out_W, int out_H, float *out_image)
{
	API_BEGIN(ctx)
	require_ptrs({image, out_image});
	require_dims(W, H, C);
	NLI_REQUIRE(out_W > 0 && out_H > 0, NLI_E_INVALID, "output sizes must be positive");
	upsample_run(ctx, image, W, H, C, out_W, out_H, out_image);
	API_END(ctx)
}

int nli_distance_transform(nli_ctx *ctx, const uint8_t *mask, int W, int H, float *distances)
{
	API_BEGIN(ctx)
	require_ptrs({mask, distances});
	require_dims(W, H, 1);
	distance_transform_run(ctx, mask, W, H, distances);
	API_END(ctx)
}

int nli_confidence_mask(nli_ctx *ctx, const uint8_t *mask, int W, int H, float decay_time, float asymptotic_value,
                        float *confidence)
{
	API_BEGIN(ctx)
	require_ptrs({mask, confidence});
	require_dims(W, H, 1);
	confidence_run(ctx, mask, W, H, decay_time, asymptotic_value, confidence);
	API_END(ctx)
}

int nli_extended_domain(nli_ctx *ctx, const uint8_t *mask, int W, int H, int patch_x, int patch_y, uint8_t *extended)
{
	API_BEGIN(ctx)
	require_ptrs({mask, extended});
	require_dims(W, H, 1);
	NLI_REQUIRE(patch_x >= 1 && patch_y >= 1, NLI_E_INVALID, "patch sizes must be positive");
	extended_domain_run(ctx, mask, W, H, patch_x, patch_y, extended);
	API_END(ctx)
}

int nli_scale_masks(nli_ctx *ctx, const uint8_t *extended, int W, int H, int margin, int erode, uint8_t *source,
                    uint8_t *target, int *source_empty)
{
	API_BEGIN(ctx)
	require_ptrs({extended, source, target});
	require_dims(W, H, 1);
	int *flag = ctx->buf<int>("scale_masks.flag", 1);
	scale_masks_run(ctx, extended, W, H, margin, erode, source, target, flag);
	if (source_empty) {
		NLI_CUDA(cudaMemcpyAsync(ctx->host_pinned, flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
		NLI_CUDA(cudaStreamSynchronize(ctx->stream));
		*source_empty = *(int *)ctx->host_pinned;
	}
	API_END(ctx)
}

int nli_poisson_init(nli_ctx *ctx, float *image, const uint8_t *mask, int W, int H, int C)
{
	API_BEGIN(ctx)
	require_ptrs({image, mask});
	require_dims(W, H, C);
	poisson_init_run(ctx, image, mask, W, H, C);
	API_END(ctx)
}

int nli_patchmatch(nli_ctx *ctx, const nli_distance_params *dist, const nli_patchmatch_params *pm,
                   const float *source, const uint8_t *source_mask, int sW, int sH, const float *target,
                   const uint8_t *target_mask, int tW, int tH, int C, const int32_t *init_nnf, int32_t *out_nnf,
                   float *out_distance, double *energy)
{
	API_BEGIN(ctx)
	require_ptrs({dist, pm, source, source_mask, target, target_mask, out_nnf});
	require_dims(sW, sH, C);
	require_dims(tW, tH, C);
	NLI_REQUIRE(pm->iterations >= 0 && pm->random_shots >= 0, NLI_E_INVALID, "negative PatchMatch parameter");
	patchmatch_run(ctx, *dist, *pm, source, source_mask, sW, sH, target, target_mask, tW, tH, C, init_nnf, out_nnf,
	               out_distance, energy);
	API_END(ctx)
}

int nli_patchmatch_metrics(nli_ctx *ctx, const nli_distance_params *dist, const nli_patchmatch_params *pm,
                           const float *source, const uint8_t *source_mask, int sW, int sH, const float *target,
                           const uint8_t *target_mask, int tW, int tH, int C, const int32_t *init_nnf,
                           int32_t *out_nnf, float *out_distance, double *energy, double *total_distance,
                           int64_t *propagations, int32_t *max_random_shots)
{
	API_BEGIN(ctx)
	require_ptrs({dist, pm, source, source_mask, target, target_mask, out_nnf});
	require_dims(sW, sH, C);
	require_dims(tW, tH, C);
	NLI_REQUIRE(pm->iterations >= 0 && pm->random_shots >= 0, NLI_E_INVALID, "negative PatchMatch parameter");
	PatchMatchMetricsHost m;
	double e = 0.0;
	patchmatch_run(ctx, *dist, *pm, source, source_mask, sW, sH, target, target_mask, tW, tH, C, init_nnf, out_nnf,
	               out_distance, &e, nullptr, -1, &m);
	if (energy) *energy = e;
	for (size_t i = 0; i < m.total_distance.size(); i++) {
		if (total_distance) total_distance[i] = m.total_distance[i];
		if (propagations) propagations[i] = m.propagations[i];
	}
	if (max_random_shots) *max_random_shots = m.max_random_shots;
	API_END(ctx)
}

int nli_ctx_keep_intermediate(nli_ctx *ctx, int enable)
{
	if (!ctx) return NLI_E_INVALID;
	ctx->keep_intermediate = enable != 0;
	return NLI_OK;
}

int nli_intermediate_count(nli_ctx *ctx, int kind)
{
	if (!ctx) return NLI_E_INVALID;
	switch (kind) {
	case NLI_INTER_INPUT: return (int)ctx->inter_input.size();
	case NLI_INTER_OUTPUT: return (int)ctx->inter_output.size();
	case NLI_INTER_MASK: return (int)ctx->inter_mask.size();
	case NLI_INTER_NNF: return (int)ctx->inter_nnf.size();
	default: return NLI_E_INVALID;
	}
}

int nli_intermediate_get(nli_ctx *ctx, int kind, int index, int *W, int *H, int *C, void *host_out)
{
	if (!ctx) return NLI_E_INVALID;
	const nli_ctx::Kept *k = nullptr;
	size_t elem = 0;
	switch (kind) {
	case NLI_INTER_INPUT:
		if (index >= 0 && index < (int)ctx->inter_input.size()) k = &ctx->inter_input[index];
		elem = sizeof(float);
		break;
	case NLI_INTER_OUTPUT:
		if (index >= 0 && index < (int)ctx->inter_output.size()) k = &ctx->inter_output[index];
		elem = sizeof(float);
		break;
	case NLI_INTER_MASK:
		if (index >= 0 && index < (int)ctx->inter_mask.size()) k = &ctx->inter_mask[index];
		elem = 1;
		break;
	case NLI_INTER_NNF:
		if (index >= 0 && index < (int)ctx->inter_nnf.size()) k = &ctx->inter_nnf[index];
		elem = sizeof(int32_t);
		break;
	default: break;
	}
	if (!k) return NLI_E_INVALID;
	if (W) *W = k->W;
	if (H) *H = k->H;
	if (C) *C = k->C;
	if (host_out) std::memcpy(host_out, k->data.data(), (size_t)k->W * k->H * k->C * elem);
	return NLI_OK;
}

int nli_update(nli_ctx *ctx, const nli_update_params *upd, float *image, const float *orig, const uint8_t *domain,
               const uint8_t *ext_domain, const int32_t *nnf, const float *confidence, int W, int H, int C,
               double *total_difference)
{
	API_BEGIN(ctx)
	require_ptrs({upd, image, orig, domain, ext_domain, nnf});
	require_dims(W, H, C);
	double t = update_run(ctx, *upd, image, orig, domain, ext_domain, nnf, confidence, W, H, C);
	if (total_difference) *total_difference = t;
	API_END(ctx)
}

int nli_process_device(nli_ctx *ctx, const nli_process_params *params, const float *image, const uint8_t *mask, int W,
                       int H, int C, float *out, nli_process_stats *stats)
{
	API_BEGIN(ctx)
	require_ptrs({params, image, mask, out});
	require_dims(W, H, C);
	process_run(ctx, *params, image, mask, W, H, C, out, stats);
	API_END(ctx)
}

int nli_process(nli_ctx *ctx, const nli_process_params *params, const float *image, const uint8_t *mask, int W, int H,
                int C, float *out, nli_process_stats *stats)
{
	API_BEGIN(ctx)
	require_ptrs({params, image, mask, out});
	require_dims(W, H, C);
	const size_t n = (size_t)W * H;
	float *d_img = ctx->buf<float>("process.h_in", n * C);
	uint8_t *d_mask = ctx->buf<uint8_t>("process.h_mask", n);
	float *d_out = ctx->buf<float>("process.h_out", n * C);
	NLI_CUDA(cudaMemcpyAsync(d_img, image, n * C * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
	NLI_CUDA(cudaMemcpyAsync(d_mask, mask, n, cudaMemcpyHostToDevice, ctx->stream));
	process_run(ctx, *params, d_img, d_mask, W, H, C, d_out, stats);
	NLI_CUDA(cudaMemcpyAsync(out, d_out, n * C * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
	NLI_CUDA(cudaStreamSynchronize(ctx->stream));
	API_END(ctx)
}

int nli_update_backward(nli_ctx *ctx, const nli_update_params *upd, const float *image, const float *out,
                        const uint8_t *domain, const uint8_t *ext_domain, const int32_t *nnf,
                        const float *confidence, int W, int H, int C, const float *grad_out, float *grad_image,
                        double *grad_lambda, double *grad_lambda_d, double *grad_sigma)
{
	API_BEGIN(ctx)
	require_ptrs({upd, image, out, domain, ext_domain, nnf, grad_out, grad_image, grad_lambda, grad_lambda_d,
	              grad_sigma});
	require_dims(W, H, C);
	update_backward_run(ctx, *upd, image, out, domain, ext_domain, nnf, confidence, W, H, C, grad_out, grad_image,
	                    grad_lambda, grad_lambda_d, grad_sigma);
	API_END(ctx)
}

int nli_rgb_to_lab(nli_ctx *ctx, const float *rgb, int W, int H, float *lab)
{
	API_BEGIN(ctx)
	require_ptrs({rgb, lab});
	require_dims(W, H, 3);
	rgb_to_lab_run(ctx, rgb, W * H, lab);
	API_END(ctx)
}

int nli_lab_to_rgb(nli_ctx *ctx, const float *lab, int W, int H, int C, float *rgb)
{
	API_BEGIN(ctx)
	require_ptrs({lab, rgb});
	require_dims(W, H, C);
	NLI_REQUIRE(C == 3 || C == 4, NLI_E_CHANNELS, "lab_to_rgb takes 3 or 4 channels");
	lab_to_rgb_run(ctx, lab, W * H, C, rgb);
	API_END(ctx)
}

int nli_cat_depth(nli_ctx *ctx, const float *rgb, const float *depth, int W, int H, float *rgbd)
{
	API_BEGIN(ctx)
	require_ptrs({rgb, depth, rgbd});
	require_dims(W, H, 4);
	cat_depth_run(ctx, rgb, depth, W * H, rgbd);
	API_END(ctx)
}

int nli_separate_depth(nli_ctx *ctx, const float *rgbd, int W, int H, float *rgb, float *depth)
{
	API_BEGIN(ctx)
	require_ptrs({rgbd});
	require_dims(W, H, 4);
	separate_depth_run(ctx, rgbd, W * H, rgb, depth);
	API_END(ctx)
}

static void require_batch(int n, const void *params, const void *images, const void *masks, const void *widths,
                          const void *heights, const void *channels, const void *outputs)
{
	NLI_REQUIRE(n >= 0, NLI_E_INVALID, "negative batch size");
	if (n > 0) require_ptrs({params, images, masks, widths, heights, channels, outputs});
}

int nli_process_batch(nli_ctx *ctx, int n, const nli_process_params *params, const float *const *images,
                      const uint8_t *const *masks, const int32_t *widths, const int32_t *heights,
                      const int32_t *channels, float *const *outputs, nli_process_stats *stats, int32_t *status)
{
	API_BEGIN(ctx)
	require_batch(n, params, images, masks, widths, heights, channels, outputs);
	process_batch_run(ctx, n, params, images, masks, widths, heights, channels, outputs, stats, status, true);
	API_END(ctx)
}

int nli_process_batch_device(nli_ctx *ctx, int n, const nli_process_params *params, const float *const *images,
                             const uint8_t *const *masks, const int32_t *widths, const int32_t *heights,
                             const int32_t *channels, float *const *outputs, nli_process_stats *stats,
                             int32_t *status)
{
	API_BEGIN(ctx)
	require_batch(n, params, images, masks, widths, heights, channels, outputs);
	process_batch_run(ctx, n, params, images, masks, widths, heights, channels, outputs, stats, status, false);
	API_END(ctx)
}

int nli_ctx_set_batch_width(nli_ctx *ctx, int width)
{
	if (!ctx || width < 1) return NLI_E_INVALID;
	ctx->batch_width = width;
	return NLI_OK;
}

uint64_t nli_batch_seed(uint64_t seed, int index) { return batch_seed(seed, index); }

int nli_debug_fail_allocation(nli_ctx *ctx, int countdown)
{
	if (!ctx || countdown < 0) return NLI_E_INVALID;
	ctx->fail_alloc_countdown = countdown;
	return NLI_OK;
}

int nli_debug_grid_wait_limit(nli_ctx *ctx, unsigned int polls)
{
	API_BEGIN(ctx)
	NLI_CUDA(cudaMemcpyAsync(&ctx->status->wait_limit, &polls, sizeof(polls), cudaMemcpyHostToDevice, ctx->stream));
	NLI_CUDA(cudaStreamSynchronize(ctx->stream));
	API_END(ctx)
}

int nli_debug_check_status(nli_ctx *ctx, unsigned long long *word, int *checked)
{
	API_BEGIN(ctx)
	require_ptrs({word, checked});
	NLI_CUDA(cudaStreamSynchronize(ctx->stream));
	*word = 0;
	for (unsigned long long w : {check_word_patchmatch(), check_word_update(), check_word_process()})
		if (!*word) *word = w;
#ifdef NLI_CHECKED
	*checked = 1;
#else
	*checked = 0;
#endif
	API_END(ctx)
}

int nli_ctx_set_tuning(nli_ctx *ctx, int knob, int value)
{
	if (!ctx) return NLI_E_INVALID;
	switch (knob) {
	case NLI_TUNE_CG_CLUSTER_CAP:
		if (value < 1 || value > 16) return NLI_E_INVALID;
		ctx->tune_cg_cluster_cap = value;
		return NLI_OK;
	case NLI_TUNE_CG_UNKNOWNS_PER_CTA:
		if (value < 1) return NLI_E_INVALID;
		ctx->tune_cg_unknowns_per_cta = value;
		return NLI_OK;
	case NLI_TUNE_BATCH_WIDTH:
		if (value < 1) return NLI_E_INVALID;
		ctx->batch_width = value;
		return NLI_OK;
	case NLI_TUNE_PM_VARIANT:
		if (value < 0 || value > 2) return NLI_E_INVALID;
		ctx->tune_pm_variant = value;
		return NLI_OK;
	case NLI_TUNE_CG_PRECOND:
		if (value != 0 && value != 1) return NLI_E_INVALID;
		ctx->tune_cg_precond = value;
		return NLI_OK;
	case NLI_TUNE_GRAPH_LOOP:
		if (value < 0 || value > 2) return NLI_E_INVALID;
		ctx->tune_graph_loop = value;
		return NLI_OK;
	case NLI_TUNE_CG_SINGLE_MAX:
		if (value < 0 || value > 4096) return NLI_E_INVALID;
		ctx->tune_cg_single_max = value;
		return NLI_OK;
	case NLI_TUNE_BATCH_MODE:
		if (value != 0 && value != 1) return NLI_E_INVALID;
		ctx->tune_batch_mode = value;
		return NLI_OK;
	case NLI_TUNE_PM_BOUND:
		if (value < 0 || value > 2) return NLI_E_INVALID;
		ctx->tune_pm_bound = value;
		return NLI_OK;
	case NLI_TUNE_BATCH_GROUPS:
		if (value < 1 || value > 16) return NLI_E_INVALID;
		ctx->tune_batch_groups = value;
		return NLI_OK;
	case NLI_TUNE_PM_TILE:
		if (value < 0 || value > 1024) return NLI_E_INVALID;
		ctx->tune_pm_tile = value;
		return NLI_OK;
	}
	return NLI_E_INVALID;
}

int nli_ctx_get_tuning(nli_ctx *ctx, int knob, int *value)
{
	if (!ctx || !value) return NLI_E_INVALID;
	switch (knob) {
	case NLI_TUNE_CG_CLUSTER_CAP: *value = ctx->tune_cg_cluster_cap; return NLI_OK;
	case NLI_TUNE_CG_UNKNOWNS_PER_CTA: *value = ctx->tune_cg_unknowns_per_cta; return NLI_OK;
	case NLI_TUNE_BATCH_WIDTH: *value = ctx->batch_width; return NLI_OK;
	case NLI_TUNE_PM_VARIANT: *value = ctx->tune_pm_variant; return NLI_OK;
	case NLI_TUNE_CG_PRECOND: *value = ctx->tune_cg_precond; return NLI_OK;
	case NLI_TUNE_GRAPH_LOOP: *value = ctx->tune_graph_loop; return NLI_OK;
	case NLI_TUNE_CG_SINGLE_MAX: *value = ctx->tune_cg_single_max; return NLI_OK;
	case NLI_TUNE_BATCH_MODE: *value = ctx->tune_batch_mode; return NLI_OK;
	case NLI_TUNE_PM_BOUND: *value = ctx->tune_pm_bound; return NLI_OK;
	case NLI_TUNE_BATCH_GROUPS: *value = ctx->tune_batch_groups; return NLI_OK;
	case NLI_TUNE_PM_TILE: *value = ctx->tune_pm_tile; return NLI_OK;
	}
	return NLI_E_INVALID;
}

}  // extern "C"
