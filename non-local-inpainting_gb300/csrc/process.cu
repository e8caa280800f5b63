// ImageInpainting::process (image_inpainting.cpp:68-190) on device buffers:
// the pyramid, the coarsest initialisation, and per scale the alternation of
// PatchMatch and the image update until sum (du)^2 <= tolerance or the
// iteration limit (inpaint_internal, :349-417), with propagate_weights
// (:492-557) between scales.  Host code only sequences kernels and reads one
// scalar per iteration for the stopping test.
#include <cfloat>
#include <cmath>

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
                            float sx, float sy, int uW, int2 *__restrict__ nnf_u)
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
		nnf_u[uy * uW + ux] = n;
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
			                                                          U.W, reinterpret_cast<int2 *>(scaled));
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
			stats->patchmatch_calls = pm_calls;
			stats->update_calls = upd_calls;
			stats->cg_iterations = ctx->cg_iterations - cg0;
			stats->graph_iterations = graph_iters;
			stats->candidates = (int64_t)hc[0];
		}
	}
};

}  // namespace

void process_run(nli_ctx *ctx, const nli_process_params &p, const float *img, const uint8_t *mask, int W, int H, int C,
                 float *out, nli_process_stats *stats)
{
	Driver d(ctx, p, C, stats);
	d.run(img, mask, W, H, out);
}

}  // namespace nli
