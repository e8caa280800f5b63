// ImageInpainting::process (image_inpainting.cpp:68-190) on device buffers:
// the pyramid, the coarsest initialisation, and per scale the alternation of
// PatchMatch and the image update until sum (du)^2 <= tolerance or the
// iteration limit (inpaint_internal, :349-417), with propagate_weights
// (:492-557) between scales.  Host code only sequences kernels and reads one
// scalar per iteration for the stopping test.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <mutex>
#include <thread>

#include "nli_device.cuh"

namespace nli {

namespace {

struct Level {
	int W = 0, H = 0;
	float *img = nullptr;
	uint8_t *mask = nullptr;
	// built on first use
	bool prepared = false;
	uint8_t *ext = nullptr, *tgt = nullptr, *src_eroded = nullptr, *src_plain = nullptr;
	float *conf = nullptr;
	int32_t *tlist = nullptr, *hole = nullptr;
	int nt = 0, nh = 0;
	bool source_empty = false;
};

const char *kEmptySource =
    "ERROR: Empty source mask (no complete patches to copy from. This may happen due to a too big inpainting "
    "domain, too big patch, or too much downscaling)";

__global__ void k_avg_color(const float *__restrict__ img, const uint8_t *__restrict__ mask, int W, int H, int C,
                            int average, float *__restrict__ color)
{
	// get_initial_color (image_inpainting.cpp:446-480): raster-order float sums
	const int c = threadIdx.x;
	if (c >= C) return;
	float col = 0.0f;
	if (average) {
		float sum = 0.0f;
		int count = 0;
		for (int y = 0; y < H; y++)
			for (int x = 0; x < W; x++)
				if (!mask[y * W + x]) {
					sum = fa(sum, img[(size_t)C * (y * W + x) + c]);
					count++;
				}
		if (count > 0) col = __fdiv_rn(sum, (float)count);
	}
	color[c] = col;
}

__global__ void k_fill_color(float *__restrict__ img, const uint8_t *__restrict__ mask, int n, int C,
                             const float *__restrict__ color)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		if (mask[i])
			for (int c = 0; c < C; c++) img[(size_t)C * i + c] = color[c];
}

__device__ __forceinline__ int round_ref(float v)
{
	// ImageInpainting::round (image_inpainting.cpp:660-663)
	return (v > 0.0) ? (int)floor((double)v + 0.5) : (int)ceil((double)v - 0.5);
}

// NNF of the coarser level mapped onto the finer grid (image_inpainting.cpp:511-530).
__global__ void k_scale_nnf(const int32_t *__restrict__ hole, int nh, int lW, const int2 *__restrict__ nnf_l,
                            float sx, float sy, int uW, int uH, int2 *__restrict__ nnf_u)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= nh) return;
	const int p = hole[i];
	const int x = p % lW, y = p / lW;
	int2 n = nnf_l[p];
	if (n.x >= 0) {
		n.x = round_ref(fm((float)n.x, sx));
		n.y = round_ref(fm((float)n.y, sy));
		const int ux = round_ref(fm((float)x, sx)), uy = round_ref(fm((float)y, sy));
		if (nli_in_bounds((long long)uy * uW + ux, (long long)uW * uH, kSiteScaleNnf)) nnf_u[uy * uW + ux] = n;
	}
}

__global__ void k_copy_hole(const int32_t *__restrict__ hole, int nh, int C, const float *__restrict__ from,
                            float *__restrict__ to)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= nh * C) return;
	const int p = hole[i / C], c = i % C;
	to[(size_t)C * p + c] = from[(size_t)C * p + c];
}

__global__ void k_fill_int2(int2 *p, int n, int2 v)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = v;
}

// Device state of a captured iteration loop: iterations done on the level,
// the last sum (du)^2, and the CG iteration counts the host loop would have
// read after each update.
struct LoopState {
	int iter;
	int pad;
	double total;
	long long cg_iters, cg_unknown_iters;
};

// End of one captured iteration: the stopping test of inpaint_internal
// (image_inpainting.cpp:388-408: continue while iter < iterations and
// total > tolerance) decides whether the graph's while node runs again.
__global__ void k_loop_control(cudaGraphConditionalHandle h, LoopState *st, const double *total, const int *cg_iters,
                               int C, int nh, int iterations, double tolerance)
{
	const int i = st->iter + 1;
	st->iter = i;
	const double t = *total;
	st->total = t;
	if (cg_iters)
		for (int c = 0; c < C; c++) {
			st->cg_iters += cg_iters[c];
			st->cg_unknown_iters += (long long)cg_iters[c] * nh;
		}
	cudaGraphSetConditional(h, (i < iterations && t > tolerance) ? 1u : 0u);
}

struct Driver {
	nli_ctx *ctx;
	const nli_process_params &p;
	int C;
	std::vector<Level> lv;
	nli_process_stats *stats;
	int64_t pm_calls = 0, upd_calls = 0, graph_iters = 0;

	Driver(nli_ctx *c, const nli_process_params &pp, int CC, nli_process_stats *st) : ctx(c), p(pp), C(CC), stats(st) {}

	std::string tag(int l, const char *what) { return "proc." + std::to_string(l) + "." + what; }

	// host copy of a device buffer for keep_intermediate
	static nli_ctx::Kept keep(nli_ctx *ctx, const void *dev, int W, int H, int C, size_t elem)
	{
		nli_ctx::Kept k;
		k.W = W;
		k.H = H;
		k.C = C;
		k.data.resize((size_t)W * H * C * elem);
		NLI_CUDA(cudaMemcpyAsync(k.data.data(), dev, k.data.size(), cudaMemcpyDeviceToHost, ctx->stream));
		NLI_CUDA(cudaStreamSynchronize(ctx->stream));
		return k;
	}

	void prepare(int l)
	{
		Level &L = lv[l];
		if (L.prepared) return;
		const int n = L.W * L.H;
		const int px = p.update.patch_x, py = p.update.patch_y;
		L.ext = ctx->buf<uint8_t>(tag(l, "ext"), n);
		L.tgt = ctx->buf<uint8_t>(tag(l, "tgt"), n);
		L.src_eroded = ctx->buf<uint8_t>(tag(l, "srce"), n);
		L.src_plain = ctx->buf<uint8_t>(tag(l, "srcp"), n);
		L.conf = ctx->buf<float>(tag(l, "conf"), n);
		L.tlist = ctx->buf<int32_t>(tag(l, "tlist"), n);
		L.hole = ctx->buf<int32_t>(tag(l, "hole"), n);
		int *empty = ctx->buf<int>(tag(l, "empty"), 1);
		extended_domain_run(ctx, L.mask, L.W, L.H, px, py, L.ext);
		scale_masks_run(ctx, L.ext, L.W, L.H, px / 2, 0, L.src_plain, L.tgt, nullptr);
		scale_masks_run(ctx, L.ext, L.W, L.H, px / 2, 1, L.src_eroded, L.tgt, empty);
		confidence_run(ctx, L.mask, L.W, L.H, p.conf_decay_time, p.conf_asymptotic, L.conf);
		L.nt = compact_mask(ctx, L.tgt, L.W, L.H, L.tlist, "proc_t");
		L.nh = compact_mask(ctx, L.mask, L.W, L.H, L.hole, "proc_h");
		NLI_CUDA(cudaMemcpyAsync(ctx->host_pinned, empty, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
		NLI_CUDA(cudaStreamSynchronize(ctx->stream));
		L.source_empty = *(int *)ctx->host_pinned != 0;
		L.prepared = true;
		if (stats && l < NLI_MAX_SCALES) {
			stats->targets[l] = L.nt;
			stats->holes[l] = L.nh;
		}
	}

	void pm(const float *img, const uint8_t *src, const Level &L, const int32_t *init, int32_t *out)
	{
		patchmatch_run(ctx, p.distance, p.patchmatch, img, src, L.W, L.H, img, L.tgt, L.W, L.H, C, init, out, nullptr,
		               nullptr, L.tlist, L.nt);
		pm_calls++;
	}

	double update(Level &L, const float *orig, const int32_t *nnf, bool read_back)
	{
		upd_calls++;
		return update_run(ctx, p.update, L.img, orig, L.mask, L.ext, nnf, L.conf, L.W, L.H, C, L.hole, L.nh,
		                  read_back);
	}

	// inpaint_internal: returns the buffer holding the final NNF
	int32_t *inpaint(int l, const int32_t *initial)
	{
		Level &L = lv[l];
		prepare(l);
		const size_t n = (size_t)L.W * L.H;
		float *orig = ctx->buf<float>("proc.orig", n * C);
		NLI_CUDA(cudaMemcpyAsync(orig, L.img, n * C * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
		NLI_REQUIRE(!L.source_empty, NLI_E_EMPTY_SOURCE, kEmptySource);
		int32_t *bufs[2] = {ctx->buf<int32_t>("proc.nnfA", 2 * n), ctx->buf<int32_t>("proc.nnfB", 2 * n)};
		int cur = 0;
		const int32_t *nnf = initial;
		double total = DBL_MAX;
		int i;
		char label[64];
		std::snprintf(label, sizeof(label), "scale %d (%dx%d)", l, L.W, L.H);
		NvtxRange scale_range(label);
		// with the captured loop, iteration 0 runs from the host (it sizes
		// every buffer the graph then reuses) and the rest in one graph
		const bool graph =
		    (ctx->tune_graph_loop == 2 || (ctx->tune_graph_loop == 1 && !ctx->batch_worker)) && !ctx->profiling &&
		    L.nh > 0;
		for (i = 0; i < p.iterations && total > p.tolerance; i++) {
			if (graph && i == 1) {
				// iteration 0 left the field in one of the two buffers
				int32_t *field = const_cast<int32_t *>(nnf);
				int32_t *other = (field == bufs[0]) ? bufs[1] : bufs[0];
				if (graph_loop(L, orig, other, field, i, total)) break;
			}
			NvtxRange iteration_range("iteration");
			int32_t *out = (nnf == bufs[cur]) ? bufs[1 - cur] : bufs[cur];
			pm(L.img, L.src_eroded, L, nnf, out);
			nnf = out;
			cur = (out == bufs[0]) ? 1 : 0;
			total = update(L, orig, nnf, true);
		}
		if (stats && l < NLI_MAX_SCALES) {
			stats->iterations[l] = i;
			stats->last_difference[l] = total;
		}
		if (ctx->keep_intermediate) ctx->inter_nnf.push_back(keep(ctx, nnf, L.W, L.H, 2, sizeof(int32_t)));
		return const_cast<int32_t *>(nnf);
	}

	// Iterations i.. of a level as one CUDA graph: a while node whose body is
	// PatchMatch (A -> B), the update with B, B copied back to A and
	// k_loop_control, which evaluates the stopping test on the device.  The
	// field enters in B (after iteration i - 1) and leaves in B.  Returns
	// false, with nothing run, when the loop cannot be captured; the caller
	// then goes on from the host.  On return `i` and `total` are as the host
	// loop would leave them.
	bool graph_loop(Level &L, const float *orig, int32_t *A, int32_t *B, int &i, double &total)
	{
		// The body is captured on the context's own stream (capture is not
		// possible on the legacy default stream a caller may have set) and
		// the graph is launched on the context's current stream.
		cudaStream_t s = ctx->stream;
		cudaStream_t cap = ctx->own_stream ? ctx->own_stream : s;
		const size_t n = (size_t)L.W * L.H;
		LoopState *st = ctx->buf<LoopState>("proc.loop", 1);
		cudaGraph_t g = nullptr;
		cudaGraphExec_t ex = nullptr;
		const int64_t pm0 = pm_calls, up0 = upd_calls;
		const int64_t launches0 = nli_thread_launch_count_internal();
		bool capturing = false;
		try {
			NLI_CUDA(cudaGraphCreate(&g, 0));
			cudaGraphConditionalHandle h;
			NLI_CUDA(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
			cudaGraphNodeParams cp = {};
			cp.type = cudaGraphNodeTypeConditional;
			cp.conditional.handle = h;
			cp.conditional.type = cudaGraphCondTypeWhile;
			cp.conditional.size = 1;
			cudaGraphNode_t node;
			NLI_CUDA(cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp));
			cudaGraph_t body = cp.conditional.phGraph_out[0];
			NLI_CUDA(cudaStreamBeginCaptureToGraph(cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
			capturing = true;
			ctx->stream = cap;
			pm(L.img, L.src_eroded, L, A, B);
			const double *tdev = nullptr;
			const int *cgdev = nullptr;
			upd_calls++;
			update_run(ctx, p.update, L.img, orig, L.mask, L.ext, B, L.conf, L.W, L.H, C, L.hole, L.nh, false, &tdev,
			           &cgdev);
			NLI_REQUIRE(tdev != nullptr, NLI_E_UNSUPPORTED, "no device total to test");
			NLI_CUDA(cudaMemcpyAsync(A, B, 2 * n * sizeof(int32_t), cudaMemcpyDeviceToDevice, cap));
			k_loop_control<<<1, 1, 0, cap>>>(h, st, tdev, cgdev, C, L.nh, p.iterations, (double)p.tolerance);
			NLI_CHECK_LAUNCH();
			capturing = false;
			ctx->stream = s;
			NLI_CUDA(cudaStreamEndCapture(cap, &body));
			NLI_CUDA(cudaGraphInstantiate(&ex, g, 0));
		} catch (const Error &) {
			ctx->stream = s;
			if (capturing) {
				cudaGraph_t dummy = nullptr;
				cudaStreamEndCapture(cap, &dummy);
			}
			(void)cudaGetLastError();
			if (ex) cudaGraphExecDestroy(ex);
			if (g) cudaGraphDestroy(g);
			pm_calls = pm0;
			upd_calls = up0;
			nli_add_launches_internal(launches0 - nli_thread_launch_count_internal());  // nothing ran
			return false;
		}
		const int64_t body_launches = nli_thread_launch_count_internal() - launches0;
		// the field to A, the loop state, then the graph
		LoopState init = {i, 0, total, 0, 0};
		LoopState *hs = static_cast<LoopState *>(ctx->host_pinned);
		*hs = init;
		try {
			NLI_CUDA(cudaMemcpyAsync(A, B, 2 * n * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
			NLI_CUDA(cudaMemcpyAsync(st, hs, sizeof(LoopState), cudaMemcpyHostToDevice, s));
			NLI_CUDA(cudaGraphLaunch(ex, s));
			NLI_CUDA(cudaMemcpyAsync(hs, st, sizeof(LoopState), cudaMemcpyDeviceToHost, s));
			NLI_CUDA(cudaMemcpyAsync(reinterpret_cast<char *>(hs) + 64, &ctx->status->timeout, sizeof(int),
			                         cudaMemcpyDeviceToHost, s));
			NLI_CUDA(cudaStreamSynchronize(s));
		} catch (const Error &) {
			cudaGraphExecDestroy(ex);
			cudaGraphDestroy(g);
			throw;
		}
		cudaGraphExecDestroy(ex);
		cudaGraphDestroy(g);
		const int ran = hs->iter - i;
		// the host counters as the host loop would have left them
		pm_calls = pm0 + ran;
		upd_calls = up0 + ran;
		graph_iters += ran;
		nli_add_launches_internal(body_launches * (ran - 1));
		ctx->cg_iterations += hs->cg_iters;
		ctx->cg_unknown_iterations += hs->cg_unknown_iters;
		i = hs->iter;
		total = hs->total;
		if (*reinterpret_cast<const int *>(reinterpret_cast<char *>(hs) + 64) != 0) {
			clear_timeout(ctx);
			NLI_REQUIRE(false, NLI_E_TIMEOUT, "a device-side wait timed out");
		}
		return true;
	}

	// propagate_weights: returns the refined NNF of level l (the finer one)
	int32_t *propagate(int l)
	{
		Level &U = lv[l];
		Level &Lo = lv[l + 1];
		prepare(l);
		prepare(l + 1);
		const size_t nu = (size_t)U.W * U.H, nl = (size_t)Lo.W * Lo.H;
		int32_t *nnf_l = ctx->buf<int32_t>("proc.prop_nnf_l", 2 * nl);
		pm(Lo.img, Lo.src_plain, Lo, nullptr, nnf_l);
		int32_t *scaled = ctx->buf<int32_t>("proc.prop_scaled", 2 * nu);
		k_fill_int2<<<(int)std::min<size_t>((nu + 255) / 256, 4096), 256, 0, ctx->stream>>>(
		    reinterpret_cast<int2 *>(scaled), (int)nu, make_int2(-1, -1));
		NLI_CHECK_LAUNCH();
		const float sx = (float)U.W / Lo.W, sy = (float)U.H / Lo.H;
		if (Lo.nh > 0) {
			k_scale_nnf<<<(Lo.nh + 255) / 256, 256, 0, ctx->stream>>>(Lo.hole, Lo.nh, Lo.W,
			                                                          reinterpret_cast<const int2 *>(nnf_l), sx, sy,
			                                                          U.W, U.H, reinterpret_cast<int2 *>(scaled));
			NLI_CHECK_LAUNCH();
		}
		float *up = ctx->buf<float>("proc.upsampled", nu * C);
		upsample_run(ctx, Lo.img, Lo.W, Lo.H, C, U.W, U.H, up);
		if (U.nh > 0) {
			k_copy_hole<<<(U.nh * C + 255) / 256, 256, 0, ctx->stream>>>(U.hole, U.nh, C, up, U.img);
			NLI_CHECK_LAUNCH();
		}
		int32_t *refined = ctx->buf<int32_t>("proc.nnfA", 2 * nu);
		pm(up, U.src_plain, U, scaled, refined);
		update(U, U.img, refined, false);
		return refined;
	}

	void run(const float *img, const uint8_t *mask, int W, int H, float *out)
	{
		const int S = p.scales;
		NLI_REQUIRE(S >= 1 && S <= NLI_MAX_SCALES, NLI_E_INVALID, "scales must be in 1..32");
		NLI_REQUIRE(p.iterations >= 0, NLI_E_INVALID, "iterations cannot be negative");
		NLI_REQUIRE(p.update.patch_x >= 1 && p.update.patch_y >= 1, NLI_E_INVALID, "bad patch size");
		if (p.distance.kind == NLI_DIST_L2_RGBD || p.update.method == NLI_UPDATE_DEPTH)
			NLI_REQUIRE(C == 4, NLI_E_CHANNELS, "L2 RGBD Distance: Channels do not match.");
		lv.assign(S, Level());
		lv[0].W = W;
		lv[0].H = H;
		for (int i = 1; i < S; i++) {
			NLI_REQUIRE(p.subsampling_rate > 0 && p.subsampling_rate < 1.0f, NLI_E_INVALID,
			            "subsampling rate must be in (0, 1)");
			lv[i].W = sample_size_host(lv[i - 1].W, p.subsampling_rate);
			lv[i].H = sample_size_host(lv[i - 1].H, p.subsampling_rate);
			NLI_REQUIRE(lv[i].W > 0 && lv[i].H > 0, NLI_E_INVALID, "pyramid level would be empty");
		}
		for (int i = 0; i < S; i++) {
			const size_t n = (size_t)lv[i].W * lv[i].H;
			lv[i].img = ctx->buf<float>(tag(i, "img"), n * C);
			lv[i].mask = ctx->buf<uint8_t>(tag(i, "mask"), n);
		}
		if (stats) {
			std::memset(stats, 0, sizeof(*stats));
			stats->scales = S;
			for (int i = 0; i < S; i++) {
				stats->width[i] = lv[i].W;
				stats->height[i] = lv[i].H;
			}
		}
		const int64_t cand0 = ctx->candidates, cg0 = ctx->cg_iterations;
		unsigned long long *counter = ctx->buf<unsigned long long>("pm.counter", 2);
		NLI_CUDA(cudaMemsetAsync(counter, 0, 2 * sizeof(unsigned long long), ctx->stream));
		cudaStream_t s = ctx->stream;
		NLI_CUDA(cudaMemcpyAsync(lv[0].img, img, (size_t)W * H * C * sizeof(float), cudaMemcpyDeviceToDevice, s));
		NLI_CUDA(cudaMemcpyAsync(lv[0].mask, mask, (size_t)W * H, cudaMemcpyDeviceToDevice, s));
		// pyramid (image_inpainting.cpp:82-100)
		for (int i = 1; i < S; i++) {
			if (p.init != NLI_INIT_NONE) {
				downsample_with_mask_run(ctx, lv[i - 1].img, lv[i - 1].mask, lv[i - 1].W, lv[i - 1].H, C,
				                         p.subsampling_rate, 0.4f, 0, lv[i].img, lv[i].mask);
			} else {
				downsample_image_run(ctx, lv[i - 1].img, lv[i - 1].W, lv[i - 1].H, C, p.subsampling_rate, lv[i].img);
				downsample_mask_run(ctx, lv[i - 1].mask, lv[i - 1].W, lv[i - 1].H, p.subsampling_rate, 0.4f,
				                    lv[i].mask);
			}
		}
		if (ctx->keep_intermediate) {
			ctx->inter_input.clear();
			ctx->inter_output.clear();
			ctx->inter_mask.clear();
			ctx->inter_nnf.clear();
			for (int i = 0; i < S; i++) {
				ctx->inter_input.push_back(keep(ctx, lv[i].img, lv[i].W, lv[i].H, C, sizeof(float)));
				ctx->inter_mask.push_back(keep(ctx, lv[i].mask, lv[i].W, lv[i].H, 1, 1));
			}
		}
		// coarsest initialisation (:111-155)
		Level &top = lv[S - 1];
		if (p.init == NLI_INIT_AVG || p.init == NLI_INIT_BLACK) {
			float *color = ctx->buf<float>("proc.color", 4);
			k_avg_color<<<1, 32, 0, s>>>(top.img, top.mask, top.W, top.H, C, p.init == NLI_INIT_AVG, color);
			NLI_CHECK_LAUNCH();
			k_fill_color<<<(top.W * top.H + 255) / 256, 256, 0, s>>>(top.img, top.mask, top.W * top.H, C, color);
			NLI_CHECK_LAUNCH();
		} else if (p.init == NLI_INIT_POISSON) {
			poisson_init_run(ctx, top.img, top.mask, top.W, top.H, C);
		}
		int32_t *nnf = inpaint(S - 1, nullptr);
		for (int i = S - 2; i >= 0; i--) {
			nnf = propagate(i);
			nnf = inpaint(i, nnf);
		}
		NLI_CUDA(cudaMemcpyAsync(out, lv[0].img, (size_t)W * H * C * sizeof(float), cudaMemcpyDeviceToDevice, s));
		if (ctx->keep_intermediate)
			for (int i = 0; i < S; i++)
				ctx->inter_output.push_back(keep(ctx, lv[i].img, lv[i].W, lv[i].H, C, sizeof(float)));
		unsigned long long *hc = reinterpret_cast<unsigned long long *>(ctx->host_pinned);
		NLI_CUDA(cudaMemcpyAsync(hc, counter, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
		NLI_CUDA(cudaStreamSynchronize(s));
		ctx->candidates = cand0 + (int64_t)hc[0];
		ctx->candidates_partial += (int64_t)hc[1];
		if (stats) {
			stats->candidates_partial = (int64_t)hc[1];
			stats->patchmatch_calls = pm_calls;
			stats->update_calls = upd_calls;
			stats->cg_iterations = ctx->cg_iterations - cg0;
			stats->graph_iterations = graph_iters;
			stats->candidates = (int64_t)hc[0];
		}
	}
};

}  // namespace

NLI_CHECK_READER(check_word_process)

void process_run(nli_ctx *ctx, const nli_process_params &p, const float *img, const uint8_t *mask, int W, int H, int C,
                 float *out, nli_process_stats *stats)
{
	Driver d(ctx, p, C, stats);
	d.run(img, mask, W, H, out);
}

// ====================================================== lockstep batches
// Many images inpainted together, walking their pyramids in lockstep from
// the coarsest scale: at pyramid rank k every image with more than k
// scales works on its own scale S - 1 - k (small images finish their
// pyramids while large ones are still on their coarse scales, where a
// single image leaves most of the GPU idle).  Per rank:
//   - the scale transition of every image (propagate_weights,
//     image_inpainting.cpp:492-557): a batched PatchMatch call on the
//     coarser scales, the field scaled up and the image upsampled, a
//     batched PatchMatch call on the finer scales and a batched update;
//   - inpaint_internal (:349-417) for every image: iteration 0 from the
//     host, then one CUDA graph whose while node runs batched PatchMatch,
//     batched update, the field copy and k_lockstep_control -- the
//     reference's stopping test per image on the device -- while any image
//     of the rank still iterates.  Stopped images are skipped by every
//     kernel through their active flag.
// Each kernel launch covers every image of the rank (PatchMatch: one
// persistent launch per sweep over the concatenated target lists; updates:
// per-image block ranges; CG: one launch per CTA layout).  Image i runs with
// the seed nli_batch_seed(seed, i) and its own PatchMatch call index, and
// every per-image computation is the one-image path's (shared device
// functions, the same reduction partitions), so each output equals its
// plain nli_process run bit for bit.
namespace {

struct LkLoop {
	int iter;
	int pad;
	double total;
	long long cg_iters, cg_unknown_iters;
};

// Device state of a lockstep group.
struct LkDev {
	int active[kBatchMax];
	int any;
	int pad;
	unsigned long long calls[kBatchMax];
	unsigned long long cand[kBatchMax][2];
	double step_total[kBatchMax];
	int cg_step[kBatchMax][4];
	LkLoop loop[kBatchMax];
};

struct LkCtl {
	int n, C;
	int iterations[kBatchMax];
	double tol[kBatchMax];
	int nh[kBatchMax];
	int has_cg[kBatchMax];
};

// End of one lockstep iteration: inpaint_internal's stopping rule for
// every active image (continue while iter < iterations and total >
// tolerance), the CG iteration counts, and -- in a graph -- whether the
// while node runs again (any image still active).
__global__ void k_lockstep_control(cudaGraphConditionalHandle h, int use_cond, const __grid_constant__ LkCtl c,
                                   LkDev *d)
{
	if (threadIdx.x != 0) return;
	int any = 0;
	for (int i = 0; i < c.n; i++) {
		if (!d->active[i]) continue;
		LkLoop &L = d->loop[i];
		L.iter += 1;
		const double t = d->step_total[i];
		L.total = t;
		if (c.has_cg[i])
			for (int k = 0; k < c.C; k++) {
				L.cg_iters += d->cg_step[i][k];
				L.cg_unknown_iters += (long long)d->cg_step[i][k] * c.nh[i];
			}
		const int on = (L.iter < c.iterations[i] && t > c.tol[i]) ? 1 : 0;
		d->active[i] = on;
		any |= on;
	}
	d->any = any;
	if (use_cond) cudaGraphSetConditional(h, any ? 1u : 0u);
}

struct LkCopy {
	int n;
	int flag[kBatchMax];
	int count[kBatchMax];  // int2 elements
	const int2 *src[kBatchMax];
	int2 *dst[kBatchMax];
};

// The fields B -> A of the active images.
__global__ void k_copy_fields(const __grid_constant__ LkCopy c, const int *active)
{
	const int t = blockIdx.y;
	if (active && !active[c.flag[t]]) return;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < c.count[t]; i += gridDim.x * blockDim.x)
		c.dst[t][i] = c.src[t][i];
}

struct LkLevel {
	int W = 0, H = 0;
	float *img = nullptr;
	uint8_t *mask = nullptr, *ext = nullptr, *tgt = nullptr, *src_eroded = nullptr, *src_plain = nullptr;
	float *conf = nullptr;
	int32_t *tlist = nullptr, *hole = nullptr;
	int nt = 0, nh = 0;
	bool source_empty = false;
};

struct LkImage {
	int idx = 0;  // in the caller's arrays
	const nli_process_params *p = nullptr;
	int W = 0, H = 0, S = 0;
	const float *in = nullptr;
	const uint8_t *in_mask = nullptr;
	float *out = nullptr;
	nli_process_stats *stats = nullptr;
	int status = NLI_OK;
	std::string error;
	uint64_t seed = 0;
	std::vector<LkLevel> lv;
	float *orig = nullptr, *up = nullptr;
	int32_t *A = nullptr, *B = nullptr, *nnf_l = nullptr, *scaled = nullptr, *nnf_y = nullptr;
	float4 *pad = nullptr, *mom = nullptr;
	float *dist_x = nullptr, *dist_y = nullptr;
	unsigned *vmax = nullptr;
	int64_t pm_calls = 0, upd_calls = 0, graph_iters = 0;
	bool ok() const { return status == NLI_OK; }
};

// Bump allocator over one device buffer.
struct Arena {
	char *base = nullptr;
	size_t off = 0;
	template <class T>
	T *take(size_t count)
	{
		off = (off + 255) & ~(size_t)255;
		T *p = reinterpret_cast<T *>(base ? base + off : nullptr);
		off += count * sizeof(T);
		return p;
	}
};

class Lockstep {
  public:
	Lockstep(nli_ctx *c, int CC) : ctx(c), C(CC) {}

	nli_ctx *ctx;
	int C;
	std::vector<LkImage> im;
	LkDev *dev = nullptr;

	std::string tag(int g, const char *what) { return "lk." + std::to_string(g) + "." + what; }

	// Level sizes and the image's device arena (levels, fields, scratch).
	void layout(int g)
	{
		LkImage &m = im[g];
		const nli_process_params &p = *m.p;
		try {
			NLI_REQUIRE(m.W > 0 && m.H > 0, NLI_E_INVALID, "image sizes must be positive");
			NLI_REQUIRE(p.scales >= 1 && p.scales <= NLI_MAX_SCALES, NLI_E_INVALID, "scales must be in 1..32");
			NLI_REQUIRE(p.iterations >= 0, NLI_E_INVALID, "iterations cannot be negative");
			NLI_REQUIRE(p.update.patch_x >= 1 && p.update.patch_y >= 1, NLI_E_INVALID, "bad patch size");
			if (p.distance.kind == NLI_DIST_L2_RGBD || p.update.method == NLI_UPDATE_DEPTH)
				NLI_REQUIRE(C == 4, NLI_E_CHANNELS, "L2 RGBD Distance: Channels do not match.");
			m.S = p.scales;
			m.lv.assign(m.S, LkLevel());
			m.lv[0].W = m.W;
			m.lv[0].H = m.H;
			for (int i = 1; i < m.S; i++) {
				NLI_REQUIRE(p.subsampling_rate > 0 && p.subsampling_rate < 1.0f, NLI_E_INVALID,
				            "subsampling rate must be in (0, 1)");
				m.lv[i].W = sample_size_host(m.lv[i - 1].W, p.subsampling_rate);
				m.lv[i].H = sample_size_host(m.lv[i - 1].H, p.subsampling_rate);
				NLI_REQUIRE(m.lv[i].W > 0 && m.lv[i].H > 0, NLI_E_INVALID, "pyramid level would be empty");
			}
		} catch (const Error &e) {
			m.status = e.status;
			m.error = e.message;
			return;
		}
		// two passes: measure, then carve the buffer
		for (int pass = 0; pass < 2; pass++) {
			Arena a;
			if (pass == 1) a.base = static_cast<char *>(ctx->buf<char>(tag(g, "arena"), arena_bytes(g)));
			for (LkLevel &L : m.lv) {
				const size_t n = (size_t)L.W * L.H;
				L.img = a.take<float>(n * C);
				L.mask = a.take<uint8_t>(n);
				L.ext = a.take<uint8_t>(n);
				L.tgt = a.take<uint8_t>(n);
				L.src_eroded = a.take<uint8_t>(n);
				L.src_plain = a.take<uint8_t>(n);
				L.conf = a.take<float>(n);
				L.tlist = a.take<int32_t>(n);
				L.hole = a.take<int32_t>(n);
			}
			const size_t n0 = (size_t)m.W * m.H;
			m.orig = a.take<float>(n0 * C);
			m.up = a.take<float>(n0 * C);
			m.A = a.take<int32_t>(2 * n0);
			m.B = a.take<int32_t>(2 * n0);
			m.nnf_l = a.take<int32_t>(2 * n0);
			m.scaled = a.take<int32_t>(2 * n0);
			m.nnf_y = a.take<int32_t>(2 * n0);
			m.pad = a.take<float4>((size_t)(m.W + 1) * (m.H + 1));
			// patch means and deviations of the PatchMatch bound (4 tables)
			m.mom = a.take<float4>((size_t)(m.W + 1) * (m.H + 1) * 4);
			m.dist_x = a.take<float>(n0);
			m.dist_y = a.take<float>(n0);
			m.vmax = a.take<unsigned>(1);
			if (pass == 0) arena_size[g] = a.off + 256;
		}
	}
	std::vector<size_t> arena_size;
	size_t arena_bytes(int g) { return arena_size[g]; }

	// The pyramid and the coarsest initialisation (image_inpainting.cpp:82-155).
	void pyramid(int g)
	{
		LkImage &m = im[g];
		const nli_process_params &p = *m.p;
		cudaStream_t s = ctx->stream;
		NLI_CUDA(cudaMemcpyAsync(m.lv[0].img, m.in, (size_t)m.W * m.H * C * sizeof(float), cudaMemcpyDeviceToDevice,
		                         s));
		NLI_CUDA(cudaMemcpyAsync(m.lv[0].mask, m.in_mask, (size_t)m.W * m.H, cudaMemcpyDeviceToDevice, s));
		for (int i = 1; i < m.S; i++) {
			LkLevel &a = m.lv[i - 1], &b = m.lv[i];
			if (p.init != NLI_INIT_NONE) {
				downsample_with_mask_run(ctx, a.img, a.mask, a.W, a.H, C, p.subsampling_rate, 0.4f, 0, b.img, b.mask);
			} else {
				downsample_image_run(ctx, a.img, a.W, a.H, C, p.subsampling_rate, b.img);
				downsample_mask_run(ctx, a.mask, a.W, a.H, p.subsampling_rate, 0.4f, b.mask);
			}
		}
		LkLevel &top = m.lv[m.S - 1];
		if (p.init == NLI_INIT_AVG || p.init == NLI_INIT_BLACK) {
			float *color = ctx->buf<float>("proc.color", 4);
			k_avg_color<<<1, 32, 0, s>>>(top.img, top.mask, top.W, top.H, C, p.init == NLI_INIT_AVG, color);
			NLI_CHECK_LAUNCH();
			k_fill_color<<<(top.W * top.H + 255) / 256, 256, 0, s>>>(top.img, top.mask, top.W * top.H, C, color);
			NLI_CHECK_LAUNCH();
		} else if (p.init == NLI_INIT_POISSON) {
			poisson_init_run(ctx, top.img, top.mask, top.W, top.H, C);
		}
		// the masks, confidence and point lists of every scale
		int *empty = ctx->buf<int>("lk.empty", 1);
		for (int l = 0; l < m.S; l++) {
			LkLevel &L = m.lv[l];
			const int px = p.update.patch_x, py = p.update.patch_y;
			extended_domain_run(ctx, L.mask, L.W, L.H, px, py, L.ext);
			scale_masks_run(ctx, L.ext, L.W, L.H, px / 2, 0, L.src_plain, L.tgt, nullptr);
			scale_masks_run(ctx, L.ext, L.W, L.H, px / 2, 1, L.src_eroded, L.tgt, empty);
			confidence_run(ctx, L.mask, L.W, L.H, p.conf_decay_time, p.conf_asymptotic, L.conf);
			L.nt = compact_mask(ctx, L.tgt, L.W, L.H, L.tlist, "proc_t");
			L.nh = compact_mask(ctx, L.mask, L.W, L.H, L.hole, "proc_h");
			NLI_CUDA(cudaMemcpyAsync(ctx->host_pinned, empty, sizeof(int), cudaMemcpyDeviceToHost, s));
			NLI_CUDA(cudaStreamSynchronize(s));
			L.source_empty = *(int *)ctx->host_pinned != 0;
			if (m.stats && l < NLI_MAX_SCALES) {
				m.stats->targets[l] = L.nt;
				m.stats->holes[l] = L.nh;
			}
		}
	}

	// count: add the call to the image's statistics (the iterations of a
	// rank are counted from their loop states instead)
	PmBatchItem pm_item(int g, const float *img, const uint8_t *smask, const LkLevel &L, const int32_t *init,
	                    int32_t *out, bool count = true)
	{
		LkImage &m = im[g];
		PmBatchItem it;
		it.img = img;
		it.W = L.W;
		it.H = L.H;
		it.smask = smask;
		it.tmask = L.tgt;
		it.tlist = L.tlist;
		it.nt = L.nt;
		it.init = init;
		it.out = out;
		it.pad = m.pad;
		it.nnf_y = m.nnf_y;
		it.dist_x = m.dist_x;
		it.dist_y = m.dist_y;
		it.seed = m.seed;
		it.calls = &dev->calls[g];
		it.counter = dev->cand[g];
		it.flag = g;
		it.mom = ctx->tune_pm_bound ? m.mom : nullptr;
		it.vmax = m.vmax;
		if (count) m.pm_calls++;
		return it;
	}

	UpdBatchItem upd_item(int g, const LkLevel &L, const float *orig, const int32_t *nnf, bool count = true)
	{
		LkImage &m = im[g];
		UpdBatchItem it;
		it.W = L.W;
		it.H = L.H;
		it.img = L.img;
		it.orig = orig;
		it.dom = L.mask;
		it.ext = L.ext;
		it.nnf = nnf;
		it.conf = L.conf;
		it.hole = L.hole;
		it.nh = L.nh;
		it.total = &dev->step_total[g];
		it.cg_iters = dev->cg_step[g];
		it.flag = g;
		if (count) m.upd_calls++;
		return it;
	}

	void pm_batch(const std::vector<PmBatchItem> &items, const int *active)
	{
		if (items.empty()) return;
		const nli_process_params &p = *im[items[0].flag].p;
		patchmatch_batch_run(ctx, p.distance, p.patchmatch, C, (int)items.size(), items.data(), active);
	}

	void upd_batch(const std::vector<UpdBatchItem> &items, const int *active)
	{
		if (items.empty()) return;
		std::vector<nli_update_params> ups;
		for (const UpdBatchItem &it : items) ups.push_back(im[it.flag].p->update);
		update_batch_run(ctx, ups.data(), C, (int)items.size(), items.data(), active);
	}

	// propagate_weights into scale l(g) = S - 1 - k of every image of the rank
	void transition(const std::vector<int> &T, int k)
	{
		NvtxRange r("lockstep transition");
		std::vector<PmBatchItem> pm;
		for (int g : T) {
			LkImage &m = im[g];
			const LkLevel &Lo = m.lv[m.S - k];
			pm.push_back(pm_item(g, Lo.img, Lo.src_plain, Lo, nullptr, m.nnf_l));
		}
		pm_batch(pm, nullptr);
		cudaStream_t s = ctx->stream;
		for (int g : T) {
			LkImage &m = im[g];
			const LkLevel &Lo = m.lv[m.S - k];
			LkLevel &U = m.lv[m.S - 1 - k];
			const size_t nu = (size_t)U.W * U.H;
			k_fill_int2<<<(int)std::min<size_t>((nu + 255) / 256, 4096), 256, 0, s>>>(
			    reinterpret_cast<int2 *>(m.scaled), (int)nu, make_int2(-1, -1));
			NLI_CHECK_LAUNCH();
			const float sx = (float)U.W / Lo.W, sy = (float)U.H / Lo.H;
			if (Lo.nh > 0) {
				k_scale_nnf<<<(Lo.nh + 255) / 256, 256, 0, s>>>(Lo.hole, Lo.nh, Lo.W,
				                                                  reinterpret_cast<const int2 *>(m.nnf_l), sx, sy,
				                                                  U.W, U.H, reinterpret_cast<int2 *>(m.scaled));
				NLI_CHECK_LAUNCH();
			}
			upsample_run(ctx, Lo.img, Lo.W, Lo.H, C, U.W, U.H, m.up);
			if (U.nh > 0) {
				k_copy_hole<<<(U.nh * C + 255) / 256, 256, 0, s>>>(U.hole, U.nh, C, m.up, U.img);
				NLI_CHECK_LAUNCH();
			}
		}
		pm.clear();
		std::vector<UpdBatchItem> up;
		for (int g : T) {
			LkImage &m = im[g];
			const LkLevel &U = m.lv[m.S - 1 - k];
			pm.push_back(pm_item(g, m.up, U.src_plain, U, m.scaled, m.A));
			up.push_back(upd_item(g, U, U.img, m.A));
		}
		pm_batch(pm, nullptr);
		upd_batch(up, nullptr);
	}

	// One iteration's work for the images of T (skipping inactive ones):
	// PatchMatch A -> B (init: A, or none on the first iteration of the
	// coarsest scale), the update with B, B copied to A.
	void iteration(const std::vector<int> &T, int k, bool first, const int *active)
	{
		std::vector<PmBatchItem> pm;
		std::vector<UpdBatchItem> up;
		LkCopy cp;
		std::memset(&cp, 0, sizeof(cp));
		int maxn = 0;
		for (int g : T) {
			LkImage &m = im[g];
			const LkLevel &L = m.lv[m.S - 1 - k];
			const int32_t *init = (first && k == 0) ? nullptr : m.A;
			pm.push_back(pm_item(g, L.img, L.src_eroded, L, init, m.B, false));
			up.push_back(upd_item(g, L, m.orig, m.B, false));
			cp.flag[cp.n] = g;
			cp.count[cp.n] = L.W * L.H;
			cp.src[cp.n] = reinterpret_cast<const int2 *>(m.B);
			cp.dst[cp.n] = reinterpret_cast<int2 *>(m.A);
			maxn = std::max(maxn, L.W * L.H);
			cp.n++;
		}
		pm_batch(pm, active);
		upd_batch(up, active);
		k_copy_fields<<<dim3((unsigned)std::min((maxn + 255) / 256, 1024), (unsigned)cp.n), 256, 0, ctx->stream>>>(
		    cp, active);
		NLI_CHECK_LAUNCH();
	}

	LkCtl control_args(const std::vector<int> &T, int k)
	{
		LkCtl c;
		std::memset(&c, 0, sizeof(c));
		c.n = (int)im.size();
		c.C = C;
		for (int g : T) {
			const LkImage &m = im[g];
			const LkLevel &L = m.lv[m.S - 1 - k];
			c.iterations[g] = m.p->iterations;
			c.tol[g] = (double)m.p->tolerance;
			c.nh[g] = L.nh;
			c.has_cg[g] =
			    (m.p->update.method == NLI_UPDATE_POISSON || m.p->update.method == NLI_UPDATE_DEPTH) && L.nh > 0;
		}
		return c;
	}

	// Reads the loop states of the group (and the any-active flag).
	void read_state(LkDev *h)
	{
		NLI_CUDA(cudaMemcpyAsync(h, dev, sizeof(LkDev), cudaMemcpyDeviceToHost, ctx->stream));
		NLI_CUDA(cudaStreamSynchronize(ctx->stream));
	}

	// Iterations 1.. of the rank as one CUDA graph; false (nothing run) when
	// it cannot be captured.
	bool graph_loop(const std::vector<int> &T, int k, const LkCtl &ctl)
	{
		cudaStream_t s = ctx->stream;
		cudaStream_t cap = ctx->own_stream ? ctx->own_stream : s;
		cudaGraph_t g = nullptr;
		cudaGraphExec_t ex = nullptr;
		const int64_t launches0 = nli_thread_launch_count_internal();
		bool capturing = false;
		try {
			NLI_CUDA(cudaGraphCreate(&g, 0));
			cudaGraphConditionalHandle h;
			NLI_CUDA(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
			cudaGraphNodeParams cp = {};
			cp.type = cudaGraphNodeTypeConditional;
			cp.conditional.handle = h;
			cp.conditional.type = cudaGraphCondTypeWhile;
			cp.conditional.size = 1;
			cudaGraphNode_t node;
			NLI_CUDA(cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp));
			cudaGraph_t body = cp.conditional.phGraph_out[0];
			NLI_CUDA(cudaStreamBeginCaptureToGraph(cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
			capturing = true;
			ctx->stream = cap;
			iteration(T, k, false, dev->active);
			k_lockstep_control<<<1, 32, 0, cap>>>(h, 1, ctl, dev);
			NLI_CHECK_LAUNCH();
			capturing = false;
			ctx->stream = s;
			NLI_CUDA(cudaStreamEndCapture(cap, &body));
			NLI_CUDA(cudaGraphInstantiate(&ex, g, 0));
		} catch (const Error &) {
			ctx->stream = s;
			if (capturing) {
				cudaGraph_t dummy = nullptr;
				cudaStreamEndCapture(cap, &dummy);
			}
			(void)cudaGetLastError();
			if (ex) cudaGraphExecDestroy(ex);
			if (g) cudaGraphDestroy(g);
			nli_add_launches_internal(launches0 - nli_thread_launch_count_internal());  // nothing ran
			return false;
		}
		const int64_t body_launches = nli_thread_launch_count_internal() - launches0;
		try {
			NLI_CUDA(cudaGraphLaunch(ex, s));
			NLI_CUDA(cudaStreamSynchronize(s));
		} catch (const Error &) {
			cudaGraphExecDestroy(ex);
			cudaGraphDestroy(g);
			throw;
		}
		cudaGraphExecDestroy(ex);
		cudaGraphDestroy(g);
		last_body_launches = body_launches;
		return true;
	}
	int64_t last_body_launches = 0;

	void rank(int k)
	{
		std::vector<int> T;
		for (int g = 0; g < (int)im.size(); g++)
			if (im[g].ok() && im[g].S > k) T.push_back(g);
		if (T.empty()) return;
		char label[64];
		std::snprintf(label, sizeof(label), "lockstep rank %d (%zu images)", k, T.size());
		NvtxRange rr(label);
		if (k > 0) transition(T, k);
		// an empty source stops the image here (inpaint_internal, :382-384)
		std::vector<int> live;
		for (int g : T) {
			LkImage &m = im[g];
			if (m.lv[m.S - 1 - k].source_empty) {
				m.status = NLI_E_EMPTY_SOURCE;
				m.error = kEmptySource;
			} else {
				live.push_back(g);
			}
		}
		T.swap(live);
		if (T.empty()) return;
		cudaStream_t s = ctx->stream;
		// loop states: iteration 0 runs for every image with iterations > 0
		LkDev *h = static_cast<LkDev *>(host_state);
		std::memset(h->active, 0, sizeof(h->active));
		for (int g : T) {
			LkImage &m = im[g];
			const LkLevel &L = m.lv[m.S - 1 - k];
			NLI_CUDA(cudaMemcpyAsync(m.orig, L.img, (size_t)L.W * L.H * C * sizeof(float), cudaMemcpyDeviceToDevice,
			                         s));
			h->active[g] = (m.p->iterations > 0 && DBL_MAX > (double)m.p->tolerance) ? 1 : 0;
			h->loop[g] = LkLoop{0, 0, DBL_MAX, 0, 0};
		}
		NLI_CUDA(cudaMemcpyAsync(dev->active, h->active, sizeof(h->active), cudaMemcpyHostToDevice, s));
		NLI_CUDA(cudaMemcpyAsync(dev->loop, h->loop, sizeof(h->loop), cudaMemcpyHostToDevice, s));
		const LkCtl ctl = control_args(T, k);
		std::vector<int> first;
		for (int g : T)
			if (h->active[g]) first.push_back(g);
		bool graph_used = false;
		if (!first.empty()) {
			NvtxRange ir("lockstep iteration");
			iteration(first, k, true, dev->active);
			k_lockstep_control<<<1, 32, 0, s>>>(0, 0, ctl, dev);
			NLI_CHECK_LAUNCH();
			read_state(h);
			const bool graph = ctx->tune_graph_loop != 0 && !ctx->profiling;
			// the images that iterate at all: their scratch was sized by
			// iteration 0, so the graph's capture allocates nothing
			if (h->any && graph) {
				graph_used = graph_loop(first, k, ctl);
				if (graph_used) read_state(h);
			}
			while (h->any) {
				// host loop (profiling, or the graph could not be built)
				NvtxRange ir2("lockstep iteration");
				iteration(first, k, false, dev->active);
				k_lockstep_control<<<1, 32, 0, s>>>(0, 0, ctl, dev);
				NLI_CHECK_LAUNCH();
				read_state(h);
			}
		}
		if (graph_used) {
			int most = 0;
			for (int g : T) most = std::max(most, h->loop[g].iter);
			const int64_t replays = std::max(most - 1, 0);
			nli_add_launches_internal(last_body_launches * (replays - 1));
		}
		timeout_check();
		for (int g : T) {
			LkImage &m = im[g];
			const int l = m.S - 1 - k;
			const LkLoop &L = h->loop[g];
			m.pm_calls += L.iter;
			m.upd_calls += L.iter;
			if (graph_used && L.iter > 1) m.graph_iters += L.iter - 1;
			ctx->cg_iterations += L.cg_iters;
			ctx->cg_unknown_iterations += L.cg_unknown_iters;
			if (m.stats && l < NLI_MAX_SCALES) {
				m.stats->iterations[l] = L.iter;
				m.stats->last_difference[l] = L.total;
				m.stats->cg_iterations += L.cg_iters;
			}
		}
	}

	void timeout_check()
	{
		int *hf = reinterpret_cast<int *>(static_cast<char *>(host_state) + sizeof(LkDev));
		NLI_CUDA(cudaMemcpyAsync(hf, &ctx->status->timeout, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
		NLI_CUDA(cudaStreamSynchronize(ctx->stream));
		if (*hf != 0) {
			clear_timeout(ctx);
			NLI_REQUIRE(false, NLI_E_TIMEOUT, "a device-side wait timed out");
		}
	}

	void *host_state = nullptr;

	void run()
	{
		const int n = (int)im.size();
		arena_size.assign(n, 0);
		for (int g = 0; g < n; g++) layout(g);
		dev = ctx->buf<LkDev>("lk.dev", 1);
		NLI_CUDA(cudaMallocHost(&host_state, sizeof(LkDev) + 64));
		try {
			cudaStream_t s = ctx->stream;
			NLI_CUDA(cudaMemsetAsync(dev, 0, sizeof(LkDev), s));
			for (int g = 0; g < n; g++) {
				LkImage &m = im[g];
				if (!m.ok()) continue;
				if (m.stats) {
					std::memset(m.stats, 0, sizeof(*m.stats));
					m.stats->scales = m.S;
					for (int i = 0; i < m.S; i++) {
						m.stats->width[i] = m.lv[i].W;
						m.stats->height[i] = m.lv[i].H;
					}
				}
				pyramid(g);
			}
			int R = 0;
			for (const LkImage &m : im)
				if (m.ok()) R = std::max(R, m.S);
			for (int k = 0; k < R; k++) rank(k);
			LkDev *h = static_cast<LkDev *>(host_state);
			read_state(h);
			for (int g = 0; g < n; g++) {
				LkImage &m = im[g];
				if (!m.ok()) continue;
				NLI_CUDA(cudaMemcpyAsync(m.out, m.lv[0].img, (size_t)m.W * m.H * C * sizeof(float),
				                         cudaMemcpyDeviceToDevice, s));
				ctx->candidates += (int64_t)h->cand[g][0];
				ctx->candidates_partial += (int64_t)h->cand[g][1];
				if (m.stats) {
					m.stats->patchmatch_calls = m.pm_calls;
					m.stats->update_calls = m.upd_calls;
					m.stats->graph_iterations = m.graph_iters;
					m.stats->candidates = (int64_t)h->cand[g][0];
					m.stats->candidates_partial = (int64_t)h->cand[g][1];
				}
			}
		} catch (...) {
			cudaFreeHost(host_state);
			host_state = nullptr;
			throw;
		}
		cudaFreeHost(host_state);
		host_state = nullptr;
	}
};

}  // namespace

// Images whose scales can share launches: the same channel count,
// distance, PatchMatch parameters and update patch / sigma.
static bool same_group(const nli_process_params &a, int Ca, const nli_process_params &b, int Cb)
{
	return Ca == Cb && std::memcmp(&a.distance, &b.distance, sizeof(a.distance)) == 0 &&
	       std::memcmp(&a.patchmatch, &b.patchmatch, sizeof(a.patchmatch)) == 0 &&
	       a.update.patch_x == b.update.patch_x && a.update.patch_y == b.update.patch_y &&
	       a.update.sigma == b.update.sigma;
}

// Pixels over an image's whole pyramid: the load estimate by which a
// group's images are dealt into concurrent sub-groups.
static double pyramid_pixels(const nli_process_params &p, int W, int H)
{
	double total = 0.0;
	for (int i = 0; i < std::max(1, std::min(p.scales, NLI_MAX_SCALES)); i++) {
		total += (double)W * H;
		if (!(p.subsampling_rate > 0.f && p.subsampling_rate < 1.f)) break;
		W = sample_size_host(W, p.subsampling_rate);
		H = sample_size_host(H, p.subsampling_rate);
	}
	return total;
}

// Runs one lockstep group -- images `grp`, all of channel count C -- on
// context `c` (the caller's or a worker), writing each image's status.
static void lockstep_group_run(nli_ctx *c, const std::vector<int> &grp, int C, uint64_t seed,
                               const nli_process_params *params, const float *const *images,
                               const uint8_t *const *masks, const int32_t *widths, const int32_t *heights,
                               float *const *outputs, nli_process_stats *stats, bool host_buffers,
                               std::vector<int> &rcs, std::vector<std::string> &errors)
{
	cudaStream_t s = c->stream;
	Lockstep L(c, C);
	L.im.resize(grp.size());
	for (size_t g = 0; g < grp.size(); g++) {
		const int i = grp[g];
		LkImage &m = L.im[g];
		m.idx = i;
		m.p = &params[i];
		m.W = widths[i];
		m.H = heights[i];
		m.stats = stats ? stats + i : nullptr;
		m.seed = batch_seed(seed, i);
		if (host_buffers) {
			const size_t np = (size_t)m.W * m.H;
			float *d_img = c->buf<float>("lk." + std::to_string(g) + ".in", np * C);
			uint8_t *d_mask = c->buf<uint8_t>("lk." + std::to_string(g) + ".inmask", np);
			m.out = c->buf<float>("lk." + std::to_string(g) + ".out", np * C);
			NLI_CUDA(cudaMemcpyAsync(d_img, images[i], np * C * sizeof(float), cudaMemcpyHostToDevice, s));
			NLI_CUDA(cudaMemcpyAsync(d_mask, masks[i], np, cudaMemcpyHostToDevice, s));
			m.in = d_img;
			m.in_mask = d_mask;
		} else {
			m.in = images[i];
			m.in_mask = masks[i];
			m.out = outputs[i];
		}
	}
	L.run();
	for (size_t g = 0; g < grp.size(); g++) {
		const LkImage &m = L.im[g];
		rcs[m.idx] = m.status;
		errors[m.idx] = m.error;
		if (host_buffers && m.ok())
			NLI_CUDA(cudaMemcpyAsync(outputs[m.idx], m.out, (size_t)m.W * m.H * C * sizeof(float),
			                         cudaMemcpyDeviceToHost, s));
	}
	if (host_buffers) NLI_CUDA(cudaStreamSynchronize(s));
}

void lockstep_batch_run(nli_ctx *ctx, int n, const nli_process_params *params, const float *const *images,
                        const uint8_t *const *masks, const int32_t *widths, const int32_t *heights,
                        const int32_t *channels, float *const *outputs, nli_process_stats *stats, int32_t *status,
                        bool host_buffers)
{
	if (n <= 0) return;
	std::vector<std::string> errors(n);
	std::vector<int> rcs(n, NLI_OK);
	std::vector<bool> placed(n, false);
	for (int i = 0; i < n; i++) {
		if (!images[i] || !masks[i] || !outputs[i]) {
			rcs[i] = NLI_E_INVALID;
			errors[i] = "null pointer argument";
			placed[i] = true;
		} else if (channels[i] < 1 || channels[i] > 4) {
			rcs[i] = NLI_E_UNSUPPORTED;
			errors[i] = "images must have 1 to 4 channels";
			placed[i] = true;
		} else if (widths[i] <= 0 || heights[i] <= 0) {
			rcs[i] = NLI_E_INVALID;
			errors[i] = "image sizes must be positive";
			placed[i] = true;
		}
	}
	for (int first = 0; first < n; first++) {
		if (placed[first]) continue;
		// a group: the unplaced images like `first`, at most kBatchMax
		std::vector<int> grp;
		for (int i = first; i < n && (int)grp.size() < kBatchMax; i++)
			if (!placed[i] && same_group(params[first], channels[first], params[i], channels[i])) {
				grp.push_back(i);
				placed[i] = true;
			}
		const int C = channels[first];
		const int k = std::max(1, std::min(ctx->tune_batch_groups, (int)grp.size()));
		if (k == 1) {
			lockstep_group_run(ctx, grp, C, ctx->seed, params, images, masks, widths, heights, outputs, stats,
			                   host_buffers, rcs, errors);
			continue;
		}
		// deal the images, largest pyramid first, each to the least-loaded
		// sub-group; every sub-group runs on a worker context of its own
		std::vector<int> order = grp;
		std::vector<double> load(n, 0.0);
		for (int i : grp) load[i] = pyramid_pixels(params[i], widths[i], heights[i]);
		std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return load[a] > load[b]; });
		std::vector<std::vector<int>> sub(k);
		std::vector<double> sum(k, 0.0);
		for (int i : order) {
			const int t = (int)(std::min_element(sum.begin(), sum.end()) - sum.begin());
			sub[t].push_back(i);
			sum[t] += load[i];
		}
		for (auto &v : sub) std::sort(v.begin(), v.end());
		while ((int)ctx->workers.size() < k) ctx->workers.push_back(new_worker(ctx->device));
		// device inputs may come from work queued on the caller's stream
		cudaEvent_t ready = nullptr;
		NLI_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
		NLI_CUDA(cudaEventRecord(ready, ctx->stream));
		std::mutex fatal_lock;
		bool fatal = false;
		Error fatal_error{NLI_OK, ""};
		auto work = [&](int t) {
			nli_ctx *w = ctx->workers[t];
			try {
				NLI_CUDA(cudaSetDevice(w->device));
				w->copy_tuning(*ctx);
				NLI_CUDA(cudaStreamWaitEvent(w->stream, ready, 0));
				lockstep_group_run(w, sub[t], C, ctx->seed, params, images, masks, widths, heights, outputs,
				                   stats, host_buffers, rcs, errors);
			} catch (const Error &e) {
				std::lock_guard<std::mutex> g(fatal_lock);
				if (!fatal) fatal_error = e;
				fatal = true;
			} catch (const std::bad_alloc &) {
				std::lock_guard<std::mutex> g(fatal_lock);
				if (!fatal) fatal_error = Error{NLI_E_NOMEM, "host allocation failed"};
				fatal = true;
			}
		};
		std::vector<std::thread> threads;
		for (int t = 1; t < k; t++) threads.emplace_back(work, t);
		work(0);
		for (auto &th : threads) th.join();
		// the caller's stream continues after every sub-group's work
		for (int t = 0; t < k; t++) {
			nli_ctx *w = ctx->workers[t];
			NLI_CUDA(cudaEventRecord(ready, w->stream));
			NLI_CUDA(cudaStreamWaitEvent(ctx->stream, ready, 0));
			merge_worker(ctx, w);
		}
		NLI_CUDA(cudaEventDestroy(ready));
		if (fatal) throw fatal_error;
	}
	if (status)
		for (int i = 0; i < n; i++) status[i] = rcs[i];
	for (int i = 0; i < n; i++)
		if (!errors[i].empty()) throw Error{rcs[i], "image " + std::to_string(i) + ": " + errors[i]};
}

}  // namespace nli
