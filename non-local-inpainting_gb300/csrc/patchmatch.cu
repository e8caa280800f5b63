// PatchMatch::calculate (patch_match.cpp:311-512) as data-parallel sweeps.
//
// The reference visits target points in scanline order and lets each point
// see the matches its predecessors found in the same sweep.  Here every
// target point of a sweep is updated at once from the field of the previous
// sweep (a Jacobi sweep, so results do not depend on thread timing):
//   1. propagation: the matches of the 4 neighbours at distance 1 and of the
//      4 neighbours at a jump distance J (J = 16, 8, 4, 2, ... by sweep),
//      each shifted back by the neighbour's offset (the reference tries the
//      left/upper or right/lower neighbour at distance 1, :420-451);
//   2. random search around the best match after propagation, in windows
//      max(W,H), /2, ..., 1 with up to `random_shots` draws per window and
//      the first draw that lands in the source evaluated (:458-494).
// A candidate equal to the current match is not re-evaluated.  Random draws
// come from Philox4x32-10 keyed by the context seed and call counter.
#include "nli_device.cuh"

namespace nli {

struct PmArgs {
	const float4 *fs;
	const float4 *ft;
	const uint8_t *smask;
	const uint8_t *tmask;
	const int32_t *tlist;
	int sW, sH, tW, tH, nt;
	int shots, max_window;
	uint2 key;
	// patch extent around a centre: [x - rx, x + ex) x [y - ry, y + ey)
	int rx, ry, ex, ey;
};

// A source centre is usable when it is in the source mask and its whole
// patch lies in the image (the masks of the inpainting driver guarantee the
// latter through their margin; user masks may not).
__device__ __forceinline__ bool src_ok(const PmArgs &p, int x, int y)
{
	return x >= p.rx && y >= p.ry && x + p.ex <= p.sW && y + p.ey <= p.sH && p.smask[y * p.sW + x];
}

__device__ __forceinline__ bool tgt_patch_inside(const PmArgs &p, int x, int y)
{
	return x >= p.rx && y >= p.ry && x + p.ex <= p.tW && y + p.ey <= p.tH;
}

__device__ __forceinline__ bool tgt_ok(const PmArgs &p, int x, int y)
{
	return (unsigned)x < (unsigned)p.tW && (unsigned)y < (unsigned)p.tH && p.tmask[y * p.tW + x];
}

__device__ __forceinline__ void count_candidates(unsigned long long *counter, unsigned n)
{
	// warp-aggregated counter update
	unsigned v = n;
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
	if ((threadIdx.x & 31) == 0 && v) atomicAdd(counter, (unsigned long long)v);
}

template <int KIND, int C, int NF4>
__global__ void __launch_bounds__(128) k_pm_init(DistArgs a, PmArgs p, const int2 *__restrict__ init,
                                                 int2 *__restrict__ nnf, float *__restrict__ dist,
                                                 unsigned long long *counter)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	unsigned evals = 0;
	if (i < p.nt) {
		const int pix = p.tlist[i];
		const int x = pix % p.tW, y = pix / p.tW;
		Rng rng(p.key, (uint32_t)pix, 0xffffffffu);
		int2 n = init ? init[pix] : make_int2(-1, -1);
		int tries = 0;
		// patch_match.cpp:341-381: keep a seed match that lies in the source,
		// otherwise redraw it uniformly up to `shots` times
		if (init) {
			while (!src_ok(p, n.x, n.y) && tries < p.shots) {
				n.x = rng.below(p.sW);
				n.y = rng.below(p.sH);
				tries++;
			}
		} else {
			while ((n.x < 0 || !src_ok(p, n.x, n.y)) && tries < p.shots) {
				n.x = rng.below(p.sW);
				n.y = rng.below(p.sH);
				tries++;
			}
		}
		if (src_ok(p, n.x, n.y) && tgt_patch_inside(p, x, y)) {
			nnf[pix] = n;
			dist[pix] = dist_fast<KIND, C, NF4>(a, p.fs, p.sW, p.ft, p.tW, n.x, n.y, x, y);
			evals = 1;
		} else {
			nnf[pix] = make_int2(-1, -1);
			dist[pix] = FLT_MAX;
		}
	}
	count_candidates(counter, evals);
}

template <int KIND, int C, int NF4>
__global__ void __launch_bounds__(128) k_pm_sweep(DistArgs a, PmArgs p, int sweep, int jump,
                                                  const int2 *__restrict__ nnf_in, const float *__restrict__ dist_in,
                                                  int2 *__restrict__ nnf_out, float *__restrict__ dist_out,
                                                  unsigned long long *counter)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	unsigned evals = 0;
	if (i < p.nt) {
		const int pix = p.tlist[i];
		const int x = pix % p.tW, y = pix / p.tW;
		int2 best = nnf_in[pix];
		float bd = dist_in[pix];
		const bool inside = tgt_patch_inside(p, x, y);
		if (!inside) {
			best = make_int2(-1, -1);
			bd = FLT_MAX;
		}

		auto consider = [&](int cx, int cy) {
			if (inside && (cx != best.x || cy != best.y) && src_ok(p, cx, cy)) {
				const float d = dist_fast<KIND, C, NF4>(a, p.fs, p.sW, p.ft, p.tW, cx, cy, x, y);
				evals++;
				if (d < bd) {
					bd = d;
					best = make_int2(cx, cy);
				}
			}
		};

		// propagation
		const int steps[2] = {1, jump};
#pragma unroll 1
		for (int si = 0; si < (jump > 1 ? 2 : 1); si++) {
			const int s = steps[si];
			if (tgt_ok(p, x - s, y)) {
				int2 q = nnf_in[pix - s];
				if (q.x >= 0) consider(q.x + s, q.y);
			}
			if (tgt_ok(p, x + s, y)) {
				int2 q = nnf_in[pix + s];
				if (q.x >= 0) consider(q.x - s, q.y);
			}
			if (tgt_ok(p, x, y - s)) {
				int2 q = nnf_in[pix - s * p.tW];
				if (q.x >= 0) consider(q.x, q.y + s);
			}
			if (tgt_ok(p, x, y + s)) {
				int2 q = nnf_in[pix + s * p.tW];
				if (q.x >= 0) consider(q.x, q.y - s);
			}
		}

		// random search around the match after propagation
		Rng rng(p.key, (uint32_t)pix, (uint32_t)sweep);
		const int cx = best.x, cy = best.y;
#pragma unroll 1
		for (int w = p.max_window; w >= 1; w /= 2) {
			const int x_min = max(cx - w, 0), y_min = max(cy - w, 0);
			const int x_max = min(cx + w + 1, p.sW), y_max = min(cy + w + 1, p.sH);
#pragma unroll 1
			for (int k = 0; k < p.shots; k++) {
				const int rx = x_min + rng.below(x_max - x_min);
				const int ry = y_min + rng.below(y_max - y_min);
				if (src_ok(p, rx, ry)) {
					consider(rx, ry);
					break;
				}
			}
		}
		nnf_out[pix] = best;
		dist_out[pix] = bd;
	}
	count_candidates(counter, evals);
}

__global__ void k_fill_nnf(int2 *__restrict__ nnf, float *__restrict__ dist, int n)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		nnf[i] = make_int2(-1, -1);
		if (dist) dist[i] = FLT_MAX;
	}
}

__global__ void k_copy_targets(const int32_t *__restrict__ tlist, int nt, const int2 *__restrict__ nnf_src,
                               const float *__restrict__ dist_src, int2 *__restrict__ nnf_dst,
                               float *__restrict__ dist_dst)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= nt) return;
	const int pix = tlist[i];
	if (nnf_dst) nnf_dst[pix] = nnf_src[pix];
	if (dist_dst) dist_dst[pix] = dist_src[pix];
}

__global__ void k_energy(const int32_t *__restrict__ tlist, int nt, const float *__restrict__ dist,
                         double *__restrict__ partials)
{
	__shared__ double s[32];
	double v = 0.0;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nt; i += gridDim.x * blockDim.x) {
		const float d = dist[tlist[i]];
		if (d < FLT_MAX) v += (double)d;
	}
	v = block_sum<256>(v, s);
	if (threadIdx.x == 0) partials[blockIdx.x] = v;
}

// Jump distance of a sweep: 16, 8, 4, 2, 16, 8, ... (never above half the
// larger target side).
static int jump_for(int sweep, int tW, int tH)
{
	static const int seq[4] = {16, 8, 4, 2};
	int j = seq[sweep % 4];
	while (j > 1 && 2 * j > max(tW, tH)) j /= 2;
	return j;
}

template <int KIND, int C, int NF4>
static void run_sweeps(nli_ctx *ctx, const DistArgs &a, const PmArgs &p, int iterations, const int2 *init,
                       int2 *nnf_x, float *dist_x, int2 *nnf_y, float *dist_y, unsigned long long *counter)
{
	const int block = 128, grid = (p.nt + block - 1) / block;
	{
		ProfScope ps(ctx, "pm_init");
		k_pm_init<KIND, C, NF4><<<grid, block, 0, ctx->stream>>>(a, p, init, nnf_x, dist_x, counter);
		NLI_CHECK_LAUNCH();
	}
	for (int it = 0; it < iterations; it++) {
		const bool even = (it % 2) == 0;
		ProfScope ps(ctx, "pm_sweep");
		k_pm_sweep<KIND, C, NF4><<<grid, block, 0, ctx->stream>>>(
		    a, p, it, jump_for(it, p.tW, p.tH), even ? nnf_x : nnf_y, even ? dist_x : dist_y, even ? nnf_y : nnf_x,
		    even ? dist_y : dist_x, counter);
		NLI_CHECK_LAUNCH();
	}
}

void patchmatch_run(nli_ctx *ctx, const nli_distance_params &dp, const nli_patchmatch_params &pm, const float *src,
                    const uint8_t *smask, int sW, int sH, const float *tgt, const uint8_t *tmask, int tW, int tH,
                    int C, const int32_t *init_nnf, int32_t *out_nnf, float *out_dist, double *energy,
                    const int32_t *tlist, int n_target)
{
	DistArgs a;
	fill_dist_args(a, dp, C);
	NLI_REQUIRE(C == 1 || C == 3 || C == 4, NLI_E_UNSUPPORTED, "PatchMatch kernels cover 1, 3 or 4 channels");
	cudaStream_t s = ctx->stream;
	const int nS = sW * sH, nT = tW * tH;

	// packed features (gradients included) of source and target
	const int nf4 = a.nf4;
	float4 *fs = ctx->buf<float4>("pm.fs", (size_t)nS * nf4);
	launch_features(s, dp.kind, src, sW, sH, C, fs);
	float4 *ft = fs;
	if (!(tgt == src && tW == sW && tH == sH)) {
		ft = ctx->buf<float4>("pm.ft", (size_t)nT * nf4);
		launch_features(s, dp.kind, tgt, tW, tH, C, ft);
	}

	if (!tlist) {
		int32_t *l = ctx->buf<int32_t>("pm.tlist", nT);
		n_target = compact_mask(ctx, tmask, tW, tH, l, "pm");
		tlist = l;
	}

	const int2 *init = reinterpret_cast<const int2 *>(init_nnf);
	if (init_nnf && init_nnf == out_nnf) {
		int2 *copy = ctx->buf<int2>("pm.init_copy", nT);
		NLI_CUDA(cudaMemcpyAsync(copy, init_nnf, sizeof(int2) * nT, cudaMemcpyDeviceToDevice, s));
		init = copy;
	}
	int2 *nnf_x = reinterpret_cast<int2 *>(out_nnf);
	int2 *nnf_y = ctx->buf<int2>("pm.nnf_y", nT);
	float *dist_x = ctx->buf<float>("pm.dist_x", nT);
	float *dist_y = ctx->buf<float>("pm.dist_y", nT);
	unsigned long long *counter = ctx->buf<unsigned long long>("pm.counter", 1);
	k_fill_nnf<<<(nT + 255) / 256, 256, 0, s>>>(nnf_x, out_dist, nT);
	NLI_CHECK_LAUNCH();
	if (n_target > 0) {
		PmArgs p;
		p.fs = fs;
		p.ft = ft;
		p.smask = smask;
		p.tmask = tmask;
		p.tlist = tlist;
		p.sW = sW;
		p.sH = sH;
		p.tW = tW;
		p.tH = tH;
		p.nt = n_target;
		p.shots = pm.random_shots;
		p.max_window = (pm.window != -1) ? pm.window : max(sW, sH);
		p.rx = a.rx;
		p.ry = a.ry;
		p.ex = a.px - a.rx;
		p.ey = a.py - a.ry;
		const uint64_t call = ctx->call_counter++;
		const uint64_t k = ctx->seed ^ (call * 0x9E3779B97F4A7C15ULL);
		p.key = make_uint2((uint32_t)k, (uint32_t)(k >> 32) ^ (uint32_t)call);
		if (energy) NLI_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s));
#define NLI_PM_CASE(KIND, CC, NF)                                                                              \
	if (dp.kind == KIND && C == CC) {                                                                          \
		run_sweeps<KIND, CC, NF>(ctx, a, p, pm.iterations, init, nnf_x, dist_x, nnf_y, dist_y, counter);       \
		handled = true;                                                                                        \
	}
		bool handled = false;
		NLI_PM_CASE(NLI_DIST_L2_COMBINED, 3, 3)
		NLI_PM_CASE(NLI_DIST_L2_COMBINED, 1, 1)
		NLI_PM_CASE(NLI_DIST_L2_COMBINED, 4, 3)
		NLI_PM_CASE(NLI_DIST_L2_RGBD, 4, 3)
		NLI_PM_CASE(NLI_DIST_L2_NORM, 3, 1)
		NLI_PM_CASE(NLI_DIST_L2_NORM, 1, 1)
		NLI_PM_CASE(NLI_DIST_L2_NORM, 4, 1)
		NLI_PM_CASE(NLI_DIST_L1_NORM, 3, 1)
		NLI_PM_CASE(NLI_DIST_L1_NORM, 1, 1)
		NLI_PM_CASE(NLI_DIST_L1_NORM, 4, 1)
#undef NLI_PM_CASE
		NLI_REQUIRE(handled, NLI_E_UNSUPPORTED, "no PatchMatch kernel for this distance / channel count");
		const bool in_y = (pm.iterations % 2) == 1;
		const int grid = (n_target + 255) / 256;
		if (in_y || out_dist) {
			k_copy_targets<<<grid, 256, 0, s>>>(tlist, n_target, in_y ? nnf_y : nnf_x, in_y ? dist_y : dist_x,
			                                    in_y ? nnf_x : nullptr, out_dist);
			NLI_CHECK_LAUNCH();
		}
		if (energy) {
			const int eg = min(grid, 1024);
			double *partials = ctx->buf<double>("pm.energy", eg + 1);
			k_energy<<<eg, 256, 0, s>>>(tlist, n_target, in_y ? dist_y : dist_x, partials);
			NLI_CHECK_LAUNCH();
			launch_sum_partials(s, partials, eg, partials + eg);
			unsigned long long *hc = reinterpret_cast<unsigned long long *>(ctx->host_pinned);
			NLI_CUDA(cudaMemcpyAsync(hc, counter, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
			NLI_CUDA(cudaMemcpyAsync(hc + 1, partials + eg, sizeof(double), cudaMemcpyDeviceToHost, s));
			NLI_CUDA(cudaStreamSynchronize(s));
			ctx->candidates += (int64_t)hc[0];
			*energy = *reinterpret_cast<double *>(hc + 1);
		}
	} else if (energy) {
		*energy = 0.0;
	}
}

// Device counter of evaluated candidates of the last PatchMatch calls
// (read by the multiscale driver for its statistics).
unsigned long long *pm_counter(nli_ctx *ctx) { return ctx->buf<unsigned long long>("pm.counter", 1); }

}  // namespace nli
