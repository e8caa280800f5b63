// Internal declarations shared by the CUDA translation units of the
// GB300 (sm_103a) non-local inpainting library.  Not part of the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>  // header-only NVTX v3: ranges cost nothing without a tool attached
#include <stdint.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "nli.h"

namespace nli {

// ---------------------------------------------------------------- errors
struct Error {
	int status;
	std::string message;
};

#define NLI_CUDA(call)                                                                     \
	do {                                                                                   \
		cudaError_t e_ = (call);                                                           \
		if (e_ != cudaSuccess)                                                             \
			throw ::nli::Error{e_ == cudaErrorMemoryAllocation ? NLI_E_NOMEM : NLI_E_CUDA, \
			                   std::string(#call) + ": " + cudaGetErrorString(e_)};        \
	} while (0)

// Every kernel launch of the library is followed by this check, which also
// counts the launch (nli_launch_count).  The calling thread's own count
// tells a graph capture how many launches its body holds; replays of a
// captured body are added with nli_add_launches_internal.
extern "C" void nli_count_launch_internal(void);
extern "C" long long nli_thread_launch_count_internal(void);
extern "C" void nli_add_launches_internal(long long n);
#define NLI_CHECK_LAUNCH()                    \
	do {                                      \
		nli_count_launch_internal();          \
		NLI_CUDA(cudaGetLastError());         \
	} while (0)

#define NLI_REQUIRE(cond, status, msg)                  \
	do {                                                \
		if (!(cond)) throw ::nli::Error{(status), (msg)}; \
	} while (0)

// ------------------------------------------------------------- workspace
// Grow-only device buffer.  Reallocation happens only when a larger size is
// requested, so steady-state calls allocate nothing.
struct DevBuf {
	void *ptr = nullptr;
	size_t bytes = 0;
	void *ensure(size_t n)
	{
		if (n > bytes) {
			if (ptr) NLI_CUDA(cudaFree(ptr));
			ptr = nullptr;
			bytes = 0;
			size_t want = n + n / 8 + 256;
			NLI_CUDA(cudaMalloc(&ptr, want));
			bytes = want;
		}
		return ptr;
	}
	void release()
	{
		if (ptr) cudaFree(ptr);
		ptr = nullptr;
		bytes = 0;
	}
};

// Device-side status words written by kernels that wait (grid barriers),
// and the index of the context's PatchMatch calls since its seed was set
// (kept on the device so that a captured iteration loop draws the same
// random streams as launches from the host).
struct DevStatus {
	unsigned int barrier_count;
	unsigned int barrier_gen;
	int timeout;
	unsigned int wait_limit;  // grid barrier polls before giving up (0: the default)
	unsigned long long pm_calls;
};

}  // namespace nli

struct nli_ctx {
	int device = 0;
	cudaStream_t own_stream = nullptr;
	cudaStream_t stream = nullptr;
	uint64_t seed = 0x9e3779b97f4a7c15ULL;
	std::string last_error;
	int num_sms = 0;
	int cg_cluster_max = -1;  // largest thread-block cluster for the CG kernel (queried once)
	std::map<std::string, nli::DevBuf> bufs;
	// pinned host staging for small results
	void *host_pinned = nullptr;
	// device status block
	nli::DevStatus *status = nullptr;
	// running counters (for stats)
	int64_t candidates = 0;
	int64_t candidates_partial = 0;  // candidates rejected after the first 32 taps
	int64_t cg_iterations = 0;
	int64_t cg_unknown_iterations = 0;  // sum over solves of iterations x unknowns
	// optional per-region GPU timing with CUDA events (nli_ctx_set_profiling)
	struct ProfEntry {
		int64_t launches = 0;
		double ms = 0.0;
		std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
	};
	bool profiling = false;
	std::map<std::string, ProfEntry> prof;
	// ImageInpainting::keep_intermediate: host copies of the last process()'s
	// pyramids (image_inpainting.cpp:103-108, 316-337, 410-412)
	struct Kept {
		int W = 0, H = 0, C = 0;
		std::vector<unsigned char> data;
	};
	bool keep_intermediate = false;
	std::vector<Kept> inter_input, inter_output, inter_mask, inter_nnf;
	// batched processing (batch.cu): images in flight and their worker contexts
	int batch_width = 8;
	// tunable launch shapes (nli_ctx_set_tuning)
	int tune_cg_cluster_cap = 16;        // CTAs per CG cluster at most
	int tune_cg_unknowns_per_cta = 1024; // at least this many unknowns per CG CTA
	int tune_pm_variant = 0;             // 9x9 PatchMatch window reads (PmVariant)
	int tune_cg_precond = 0;             // NL-Poisson CG: 0 plain (the reference's), 1 Jacobi
	int tune_graph_loop = 1;             // iterations 1.. of a scale as one CUDA graph (while node):
	                                     // 1 in nli_process only, 2 also in batches, 0 never
	int tune_cg_single_max = 1024;       // CG systems of at most this many unknowns: one CTA
	int tune_batch_mode = 1;             // batches: 1 lockstep (process.cu), 0 worker contexts (batch.cu)
	int tune_pm_bound = 1;               // PatchMatch lower bound: 0 off, 1 patch means, 2 means and deviations
	int tune_batch_groups = 4;           // lockstep: concurrent sub-groups per launch-sharing group
	int tune_pm_tile = 1;                // PatchMatch: 0 static ranges, n > 0 work queue of n points per grab
	bool batch_worker = false;           // a worker context of nli_process_batch
	int max_smem_optin = 0;              // dynamic shared memory per block at most
	std::vector<nli_ctx *> workers;
	std::vector<cudaEvent_t> event_pool;

	cudaEvent_t take_event()
	{
		if (!event_pool.empty()) {
			cudaEvent_t e = event_pool.back();
			event_pool.pop_back();
			return e;
		}
		cudaEvent_t e;
		cudaEventCreate(&e);
		return e;
	}
	void settle_profile()
	{
		cudaStreamSynchronize(stream);
		for (auto &kv : prof) {
			for (auto &pr : kv.second.pending) {
				float ms = 0.f;
				cudaEventElapsedTime(&ms, pr.first, pr.second);
				kv.second.ms += ms;
				event_pool.push_back(pr.first);
				event_pool.push_back(pr.second);
			}
			kv.second.pending.clear();
		}
	}

	// Host-side fault injection (nli_debug_fail_allocation): when > 0, the
	// workspace growth that brings it to 0 fails as an out-of-memory error
	// without calling cudaMalloc.
	int fail_alloc_countdown = 0;

	// The launch-shape knobs (nli_ctx_set_tuning) a worker context takes
	// from its parent.
	void copy_tuning(const nli_ctx &o)
	{
		profiling = o.profiling;
		tune_cg_cluster_cap = o.tune_cg_cluster_cap;
		tune_cg_unknowns_per_cta = o.tune_cg_unknowns_per_cta;
		tune_pm_variant = o.tune_pm_variant;
		tune_cg_precond = o.tune_cg_precond;
		tune_graph_loop = o.tune_graph_loop;
		tune_cg_single_max = o.tune_cg_single_max;
		tune_pm_bound = o.tune_pm_bound;
		tune_pm_tile = o.tune_pm_tile;
	}

	template <class T>
	T *buf(const std::string &name, size_t count)
	{
		nli::DevBuf &b = bufs[name];
		const size_t n = count * sizeof(T);
		if (n > b.bytes && fail_alloc_countdown > 0 && --fail_alloc_countdown == 0)
			throw ::nli::Error{NLI_E_NOMEM, "device allocation failed (injected)"};
		return static_cast<T *>(b.ensure(n));
	}
};

namespace nli {

// NVTX range for profilers (scales, iterations, batch images).
struct NvtxRange {
	explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
	~NvtxRange() { nvtxRangePop(); }
	NvtxRange(const NvtxRange &) = delete;
	NvtxRange &operator=(const NvtxRange &) = delete;
};

// Times the kernels launched in its lifetime under `name` when the
// context's profiling is on (events on the context stream).
struct ProfScope {
	nli_ctx *ctx;
	const char *name;
	cudaEvent_t a = nullptr;
	ProfScope(nli_ctx *c, const char *n) : ctx(c), name(n)
	{
		if (ctx->profiling) {
			a = ctx->take_event();
			cudaEventRecord(a, ctx->stream);
		}
	}
	~ProfScope()
	{
		if (a) {
			cudaEvent_t b = ctx->take_event();
			cudaEventRecord(b, ctx->stream);
			auto &e = ctx->prof[name];
			e.launches++;
			e.pending.emplace_back(a, b);
		}
	}
};

// ------------------------------------------------------------ parameters
constexpr int kMaxTaps = NLI_MAX_PATCH * NLI_MAX_PATCH;

// Everything a distance evaluation needs, passed by value to kernels.
struct DistArgs {
	int kind;
	int px, py, rx, ry;  // patch size and radius (radius = size / 2)
	int C;               // image channels
	float lambda, lambda_d;
	float weights[kMaxTaps];  // Gaussian patch weights, row-major
};

// ---------------------------------------------------------- host helpers
std::vector<float> gaussian_weights_host(unsigned sx, unsigned sy, float sigma_x, float sigma_y);
void fill_dist_args(DistArgs &a, const nli_distance_params &p, int C);
// Resets the device timeout word once a timeout has been read and reported
// (the stream has been synchronised), so the context stays usable.
void clear_timeout(nli_ctx *ctx);

// ------------------------------------------------------------- launchers
// gradient.cu
void launch_gradient(cudaStream_t s, const float *img, int W, int H, int C, float *grad);
// Padded float4 pixel image read by the PatchMatch distance (gradient.cu).
void launch_pad4(cudaStream_t s, const float *img, int W, int H, int C, float4 *out);

// compact.cu: raster-order list of the pixels with mask != 0; returns count
int compact_mask(nli_ctx *ctx, const uint8_t *mask, int W, int H, int32_t *list, const char *tag);

// reductions
void launch_sum_partials(cudaStream_t s, const double *partials, int n, double *out);

// patchmatch.cu
struct PmStats {
	double energy;
};
// Per-sweep figures of the reference's METRICS build (patch_match.cpp:383-507).
struct PatchMatchMetricsHost {
	std::vector<double> total_distance;   // per sweep
	std::vector<int64_t> propagations;    // per sweep
	int max_random_shots = 0;
};
void patchmatch_run(nli_ctx *ctx, const nli_distance_params &dp, const nli_patchmatch_params &pm,
                    const float *src, const uint8_t *smask, int sW, int sH, const float *tgt,
                    const uint8_t *tmask, int tW, int tH, int C, const int32_t *init_nnf,
                    int32_t *out_nnf, float *out_dist, double *energy, const int32_t *tlist = nullptr,
                    int n_target = -1, PatchMatchMetricsHost *metrics = nullptr);

// Batched PatchMatch (lockstep batch driver): one image's call.  The image
// is both source and target; the driver supplies the scratch buffers.
constexpr int kBatchMax = 64;  // images per batched launch
struct PmBatchItem {
	const float *img;
	int W, H;
	const uint8_t *smask, *tmask;
	const int32_t *tlist;
	int nt;
	const int32_t *init;  // initial field or null
	int32_t *out;         // result field, W * H int2
	float4 *pad;          // (W + 1) * (H + 1) padded pixels
	int32_t *nnf_y;       // W * H int2
	float *dist_x, *dist_y;  // W * H
	uint64_t seed;
	unsigned long long *calls;    // the image's PatchMatch call index (device)
	unsigned long long *counter;  // the image's candidate counters (2, device) or null
	int flag;                     // index of the image's active flag
	float4 *mom;                  // (W + 1) * (H + 1) patch means of the lower bound, or null
	unsigned *vmax;               // the image's largest absolute value (float bits), with mom
};
// active: device flags (null: all), item i reads active[items[i].flag];
// inactive images are skipped.
void patchmatch_batch_run(nli_ctx *ctx, const nli_distance_params &dp, const nli_patchmatch_params &pm, int C, int n,
                          const PmBatchItem *items, const int *active);

// update.cu
// read_back false: nothing is read to the host; *total_dev (if given)
// receives the device address of the step's sum (du)^2 and *cg_iters_dev
// that of the per-channel CG iteration counts (null for NL-means/medians).
double update_run(nli_ctx *ctx, const nli_update_params &up, float *image, const float *orig,
                  const uint8_t *dom, const uint8_t *ext, const int32_t *nnf, const float *conf, int W,
                  int H, int C, const int32_t *hole_list = nullptr, int n_hole = -1,
                  bool read_back = true, const double **total_dev = nullptr, const int **cg_iters_dev = nullptr);

// Batched update (lockstep batch driver): one image's step.  The image is
// updated in place on its hole; orig as in update_run.
struct UpdBatchItem {
	int W, H;
	float *img;
	const float *orig;
	const uint8_t *dom, *ext;
	const int32_t *nnf;
	const float *conf;
	const int32_t *hole;
	int nh;
	double *total;  // device: the step's sum of (du)^2
	int *cg_iters;  // device: CG iterations per channel (4 ints; NL-Poisson / NL-depth)
	int flag;       // index of the image's active flag
};
// ups[i]: image i's update parameters (the patch and sigma are shared);
// active: device flags (null: all), item i reads active[items[i].flag].  Scratch lives in the
// context's workspace under per-image names; a first call sizes it.
void update_batch_run(nli_ctx *ctx, const nli_update_params *ups, int C, int n, const UpdBatchItem *items,
                      const int *active);

// Adjoint of one update with the NNF fixed (update.cu).
void update_backward_run(nli_ctx *ctx, const nli_update_params &up, const float *image, const float *out,
                         const uint8_t *dom, const uint8_t *ext, const int32_t *nnf, const float *conf, int W,
                         int H, int C, const float *grad_out, float *grad_image, double *grad_lambda,
                         double *grad_lambda_d, double *grad_sigma);

// pyramid.cu
void downsample_with_mask_run(nli_ctx *ctx, const float *img, const uint8_t *mask, int W, int H, int C,
                              float factor, float threshold, int mask_val, float *out_img,
                              uint8_t *out_mask);
void downsample_image_run(nli_ctx *ctx, const float *img, int W, int H, int C, float factor, float *out);
void downsample_mask_run(nli_ctx *ctx, const uint8_t *mask, int W, int H, float factor, float threshold,
                         uint8_t *out);
void upsample_run(nli_ctx *ctx, const float *img, int W, int H, int C, int oW, int oH, float *out);
void distance_transform_run(nli_ctx *ctx, const uint8_t *mask, int W, int H, float *out);
void confidence_run(nli_ctx *ctx, const uint8_t *mask, int W, int H, float decay, float asym, float *out);
void extended_domain_run(nli_ctx *ctx, const uint8_t *mask, int W, int H, int px, int py, uint8_t *out);
void scale_masks_run(nli_ctx *ctx, const uint8_t *ext, int W, int H, int margin, int erode, uint8_t *src,
                     uint8_t *tgt, int *empty_dev);
void poisson_init_run(nli_ctx *ctx, float *img, const uint8_t *mask, int W, int H, int C);
int sample_size_host(unsigned size, float factor);

// batch.cu
uint64_t batch_seed(uint64_t seed, int index);
void process_batch_run(nli_ctx *ctx, int n, const nli_process_params *params, const float *const *images,
                       const uint8_t *const *masks, const int32_t *widths, const int32_t *heights,
                       const int32_t *channels, float *const *outputs, nli_process_stats *stats, int32_t *status,
                       bool host_buffers);

// process.cu: the lockstep form of process_batch_run (NLI_TUNE_BATCH_MODE 1)
void lockstep_batch_run(nli_ctx *ctx, int n, const nli_process_params *params, const float *const *images,
                        const uint8_t *const *masks, const int32_t *widths, const int32_t *heights,
                        const int32_t *channels, float *const *outputs, nli_process_stats *stats, int32_t *status,
                        bool host_buffers);
// batch.cu: a worker context of a batch (its own stream and workspace), and
// the merge of its profile and counters into the parent
nli_ctx *new_worker(int device);
void merge_worker(nli_ctx *parent, nli_ctx *w);

// Records of the checked build's bounds tests, one per translation unit
// with instrumented kernels (0 elsewhere; read and cleared).
unsigned long long check_word_patchmatch();
unsigned long long check_word_update();
unsigned long long check_word_process();

// color.cu
void rgb_to_lab_run(nli_ctx *ctx, const float *rgb, int n, float *lab);
void lab_to_rgb_run(nli_ctx *ctx, const float *lab, int n, int C, float *rgb);
void cat_depth_run(nli_ctx *ctx, const float *rgb, const float *depth, int n, float *out);
void separate_depth_run(nli_ctx *ctx, const float *rgbd, int n, float *rgb, float *depth);

// process.cu
void process_run(nli_ctx *ctx, const nli_process_params &p, const float *img, const uint8_t *mask, int W,
                 int H, int C, float *out, nli_process_stats *stats);

}  // namespace nli
