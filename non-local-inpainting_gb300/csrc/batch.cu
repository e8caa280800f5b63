// Batched inpainting: many independent image/mask pairs in flight on one
// GPU.  The reference inpaints one image per ImageInpainting::process call
// (image_inpainting.cpp:68-190, called once by main.cpp:279); a host that
// has many images loops over that call.
//
// Here a batch is spread over `batch_width` worker contexts, each with its
// own CUDA stream and workspace, driven by one host thread each.  Workers
// pull images from a shared counter, largest first (the longest jobs start
// first, and a worker's workspace reaches its final size on its first image,
// so no later growth frees device memory while others run).  Kernels of
// different images overlap on the SMs: a coarse pyramid level or a CG
// cluster of one image fills only part of the GPU, and the host-side
// stopping test of one image's iteration overlaps the others' kernels.
//
// Image i runs exactly as nli_process would after
// nli_set_seed(ctx, nli_batch_seed(seed, i)), so a batch result equals the
// per-image plain runs bit for bit.
#include <atomic>
#include <thread>

#include "nli_internal.cuh"

namespace nli {

uint64_t batch_seed(uint64_t seed, int index)
{
	return seed ^ (0x9E3779B97F4A7C15ULL * (uint64_t)(index + 1));
}

nli_ctx *new_worker(int device)
{
	nli_ctx *w = nullptr;
	const int rc = nli_ctx_create(device, &w);
	NLI_REQUIRE(rc == NLI_OK, rc, "cannot create a batch worker context");
	w->batch_worker = true;
	return w;
}

// Adds a worker's profile and counters to the parent and clears them.
void merge_worker(nli_ctx *parent, nli_ctx *w)
{
	w->settle_profile();
	for (auto &kv : w->prof) {
		auto &e = parent->prof[kv.first];
		e.launches += kv.second.launches;
		e.ms += kv.second.ms;
	}
	w->prof.clear();
	parent->candidates += w->candidates;
	parent->candidates_partial += w->candidates_partial;
	parent->cg_iterations += w->cg_iterations;
	parent->cg_unknown_iterations += w->cg_unknown_iterations;
	w->candidates = w->candidates_partial = w->cg_iterations = w->cg_unknown_iterations = 0;
}

void process_batch_run(nli_ctx *ctx, int n, const nli_process_params *params, const float *const *images,
                       const uint8_t *const *masks, const int32_t *widths, const int32_t *heights,
                       const int32_t *channels, float *const *outputs, nli_process_stats *stats, int32_t *status,
                       bool host_buffers)
{
	if (n <= 0) return;
	if (ctx->tune_batch_mode == 1) {
		lockstep_batch_run(ctx, n, params, images, masks, widths, heights, channels, outputs, stats, status,
		                   host_buffers);
		return;
	}
	const int width = std::max(1, std::min(ctx->batch_width, n));
	while ((int)ctx->workers.size() < width) ctx->workers.push_back(new_worker(ctx->device));

	// largest images first
	std::vector<int> order(n);
	for (int i = 0; i < n; i++) order[i] = i;
	std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
		return (int64_t)widths[a] * heights[a] > (int64_t)widths[b] * heights[b];
	});

	// device inputs may come from work queued on the caller's stream
	cudaEvent_t ready = nullptr;
	if (!host_buffers) {
		NLI_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
		NLI_CUDA(cudaEventRecord(ready, ctx->stream));
	}
	std::atomic<int> next{0};
	std::vector<std::string> errors(n);
	std::vector<int> rcs(n, NLI_OK);
	auto work = [&](nli_ctx *w) {
		cudaSetDevice(w->device);
		w->copy_tuning(*ctx);
		if (ready) cudaStreamWaitEvent(w->stream, ready, 0);
		for (;;) {
			const int k = next.fetch_add(1);
			if (k >= n) break;
			const int i = order[k];
			int rc = NLI_OK;
			try {
				const int W = widths[i], H = heights[i], C = channels[i];
				NLI_REQUIRE(images[i] && masks[i] && outputs[i], NLI_E_INVALID, "null pointer argument");
				NLI_REQUIRE(W > 0 && H > 0, NLI_E_INVALID, "image sizes must be positive");
				NLI_REQUIRE(C >= 1 && C <= 4, NLI_E_UNSUPPORTED, "images must have 1 to 4 channels");
				char label[48];
				std::snprintf(label, sizeof(label), "batch image %d", i);
				NvtxRange image_range(label);
				w->seed = batch_seed(ctx->seed, i);
				NLI_CUDA(cudaMemsetAsync(&w->status->pm_calls, 0, sizeof(unsigned long long), w->stream));
				nli_process_stats *st = stats ? stats + i : nullptr;
				if (host_buffers) {
					const size_t np = (size_t)W * H;
					float *d_img = w->buf<float>("batch.in", np * C);
					uint8_t *d_mask = w->buf<uint8_t>("batch.mask", np);
					float *d_out = w->buf<float>("batch.out", np * C);
					NLI_CUDA(cudaMemcpyAsync(d_img, images[i], np * C * sizeof(float), cudaMemcpyHostToDevice,
					                         w->stream));
					NLI_CUDA(cudaMemcpyAsync(d_mask, masks[i], np, cudaMemcpyHostToDevice, w->stream));
					process_run(w, params[i], d_img, d_mask, W, H, C, d_out, st);
					NLI_CUDA(cudaMemcpyAsync(outputs[i], d_out, np * C * sizeof(float), cudaMemcpyDeviceToHost,
					                         w->stream));
					NLI_CUDA(cudaStreamSynchronize(w->stream));
				} else {
					process_run(w, params[i], images[i], masks[i], W, H, C, outputs[i], st);
				}
			} catch (const Error &e) {
				rc = e.status;
				errors[i] = e.message;
			} catch (const std::bad_alloc &) {
				rc = NLI_E_NOMEM;
				errors[i] = "host allocation failed";
			}
			rcs[i] = rc;
			if (status) status[i] = rc;
		}
	};
	std::vector<std::thread> threads;
	for (int t = 1; t < width; t++) threads.emplace_back(work, ctx->workers[t]);
	work(ctx->workers[0]);
	for (auto &t : threads) t.join();

	// the caller's stream continues after every worker's work
	for (int t = 0; t < width; t++) {
		nli_ctx *w = ctx->workers[t];
		cudaEvent_t done;
		NLI_CUDA(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
		NLI_CUDA(cudaEventRecord(done, w->stream));
		NLI_CUDA(cudaStreamWaitEvent(ctx->stream, done, 0));
		NLI_CUDA(cudaEventDestroy(done));
		merge_worker(ctx, w);
	}
	if (ready) NLI_CUDA(cudaEventDestroy(ready));
	for (int i = 0; i < n; i++)
		if (!errors[i].empty())
			throw Error{rcs[i], "image " + std::to_string(i) + ": " + errors[i]};
}

}  // namespace nli
