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
//
// One warp works on one target point at a time (persistent warps).  Lane l
// holds taps l, l + 32, ... of the target patch in registers and reads the
// same taps of every candidate source patch from the plane-major feature
// image (36 bytes per pixel for 3 channels); the weighted distance is
// summed with a butterfly of shuffles.  All control flow is warp-uniform.
#include "nli_device.cuh"

namespace nli {

struct PmArgs {
	const float4 *fs4;  // source feature planes (P4 float4 planes of sW*sH)
	const float *fs1;   // source float plane (F1 == 1)
	const float4 *ft4;  // target feature planes
	const float *ft1;
	const uint8_t *smask;
	const uint8_t *tmask;
	const int32_t *tlist;
	int sW, sH, tW, tH, nt;
	int sN, tN;  // pixels per plane
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

// Feature planes of a (distance kind, channel count): P4 float4 planes and
// F1 float planes (same rule as feature_layout).
template <int KIND, int C>
struct Layout {
	static constexpr int comps = (KIND == NLI_DIST_L2_COMBINED || KIND == NLI_DIST_L2_RGBD) ? 3 * C : C;
	static constexpr int F1 = (comps % 4 == 1 && comps > 1) ? 1 : 0;
	static constexpr int P4 = (comps - F1 + 3) / 4;
	static constexpr int N = 4 * P4 + F1;
};

// Per-lane tap table: lane l owns taps l, l + 32, ... (NT slots); offsets
// and weights (already multiplied by the term coefficients and by
// 1 / patch area) are computed once per warp.
template <int NT>
struct TapTable {
	int soff[NT], toff[NT];
	float wa[NT], wb[NT], wc[NT], wd[NT];
	bool valid[NT];
};

template <int KIND, int NT>
__device__ __forceinline__ void make_taps(const DistArgs &a, const PmArgs &p, TapTable<NT> &T)
{
	const int lane = threadIdx.x & 31;
	const int taps = a.px * a.py;
	const float invP = 1.0f / (float)taps;
#pragma unroll
	for (int k = 0; k < NT; k++) {
		const int t = lane + 32 * k;
		T.valid[k] = t < taps;
		const int dy = t / a.px, dx = t - dy * a.px;
		T.soff[k] = (dy - a.ry) * p.sW + (dx - a.rx);
		T.toff[k] = (dy - a.ry) * p.tW + (dx - a.rx);
		const float w = T.valid[k] ? a.weights[t] * invP : 0.f;
		if (KIND == NLI_DIST_L2_NORM || KIND == NLI_DIST_L1_NORM) {
			T.wa[k] = w;
			T.wb[k] = T.wc[k] = T.wd[k] = 0.f;
		} else {
			T.wa[k] = w * a.lambda;
			T.wb[k] = w * (1.0f - a.lambda);
			T.wc[k] = w * a.lambda_d;
			T.wd[k] = w * (1.0f - a.lambda_d);
		}
	}
}

// Feature components of tap slot k of pixel `pix` (+ the slot's offset).
template <int KIND, int C, int NT>
__device__ __forceinline__ void load_comps(const float4 *__restrict__ f4, const float *__restrict__ f1, int npix,
                                           int pix, float (&f)[Layout<KIND, C>::N])
{
	using L = Layout<KIND, C>;
#pragma unroll
	for (int j = 0; j < L::P4; j++) {
		const float4 v = __ldg(f4 + (size_t)j * npix + pix);
		f[4 * j + 0] = v.x;
		f[4 * j + 1] = v.y;
		f[4 * j + 2] = v.z;
		f[4 * j + 3] = v.w;
	}
	if (L::F1) f[4 * L::P4] = __ldg(f1 + pix);
}

// The warp's target patch in shared memory: lane l keeps its slot k as
// float4 planes at v4[(k * P4 + j) * 32 + l] and the float plane at
// v1[k * 32 + l].  Each lane writes and reads only its own slots, so no
// synchronisation is needed.
template <int KIND, int C, int NT>
struct TargetPatch {
	float4 *v4;
	float *v1;
};

template <int KIND, int C, int NT>
__device__ __forceinline__ TargetPatch<KIND, C, NT> warp_target_slot()
{
	using L = Layout<KIND, C>;
	extern __shared__ float4 s_target[];
	constexpr int per_warp4 = NT * L::P4 * 32 + (NT * L::F1 * 32 + 3) / 4;
	TargetPatch<KIND, C, NT> P;
	P.v4 = s_target + (size_t)(threadIdx.x >> 5) * per_warp4;
	P.v1 = reinterpret_cast<float *>(P.v4 + NT * L::P4 * 32);
	return P;
}

template <int KIND, int C, int NT>
constexpr size_t target_smem_bytes(int warps)
{
	using L = Layout<KIND, C>;
	return (size_t)warps * (NT * L::P4 * 32 + (NT * L::F1 * 32 + 3) / 4) * sizeof(float4);
}

template <int KIND, int C, int NT>
__device__ __forceinline__ void load_target(const TapTable<NT> &T, const PmArgs &p, int tpix, TargetPatch<KIND, C, NT> &P)
{
	using L = Layout<KIND, C>;
	const int lane = threadIdx.x & 31;
#pragma unroll
	for (int k = 0; k < NT; k++) {
		const int q = tpix + T.toff[k];
#pragma unroll
		for (int j = 0; j < L::P4; j++)
			P.v4[(k * L::P4 + j) * 32 + lane] =
			    T.valid[k] ? __ldg(p.ft4 + (size_t)j * p.tN + q) : make_float4(0.f, 0.f, 0.f, 0.f);
		if (L::F1) P.v1[k * 32 + lane] = T.valid[k] ? __ldg(p.ft1 + q) : 0.f;
	}
}

// Distance of the target patch to the source patch centred at pixel spix;
// every lane returns the full sum.  All terms are non-negative, so once the
// sum over the first 32 taps reaches `bound` the candidate cannot beat the
// current match: that partial sum (>= bound) is returned without reading
// the rest of the patch (exact early termination).
template <int KIND, int C, int NT>
__device__ __forceinline__ float warp_distance(const TapTable<NT> &T, const TargetPatch<KIND, C, NT> &P,
                                               const PmArgs &p, int spix, float bound, unsigned &partial)
{
	float r = 0.f, head = 0.f;
#pragma unroll
	for (int k = 0; k < NT; k++) {
		if (k == 1) {
#pragma unroll
			for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
			head = r;
			if (head >= bound) {
				partial++;
				return head;
			}
			r = 0.f;
		}
		if (!T.valid[k]) continue;
		using L = Layout<KIND, C>;
		const int lane = threadIdx.x & 31;
		float f[L::N];
		load_comps<KIND, C, NT>(p.fs4, p.fs1, p.sN, spix + T.soff[k], f);
#pragma unroll
		for (int j = 0; j < L::P4; j++) {
			const float4 t4 = P.v4[(k * L::P4 + j) * 32 + lane];
			f[4 * j + 0] -= t4.x;
			f[4 * j + 1] -= t4.y;
			f[4 * j + 2] -= t4.z;
			f[4 * j + 3] -= t4.w;
		}
		if (L::F1) f[4 * L::P4] -= P.v1[k * 32 + lane];
		if (KIND == NLI_DIST_L1_NORM) {
			float n = 0.f;
#pragma unroll
			for (int c = 0; c < C; c++) n += fabsf(f[c]);
			r = fmaf(T.wa[k], n, r);
		} else if (KIND == NLI_DIST_L2_NORM) {
			float n = 0.f;
#pragma unroll
			for (int c = 0; c < C; c++) n = fmaf(f[c], f[c], n);
			r = fmaf(T.wa[k], n, r);
		} else if (KIND == NLI_DIST_L2_RGBD) {
			float n = 0.f, g = 0.f;
#pragma unroll
			for (int c = 0; c < 3; c++) n = fmaf(f[c], f[c], n);
#pragma unroll
			for (int c = 0; c < 6; c++) g = fmaf(f[4 + c], f[4 + c], g);
			r = fmaf(T.wa[k], n, r);
			r = fmaf(T.wb[k], g, r);
			r = fmaf(T.wc[k], f[3] * f[3], r);
			r = fmaf(T.wd[k], fmaf(f[10], f[10], f[11] * f[11]), r);
		} else {
			float n = 0.f, g = 0.f;
#pragma unroll
			for (int c = 0; c < C; c++) n = fmaf(f[c], f[c], n);
#pragma unroll
			for (int c = 0; c < 2 * C; c++) g = fmaf(f[C + c], f[C + c], g);
			r = fmaf(T.wa[k], n, r);
			r = fmaf(T.wb[k], g, r);
		}
	}
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
	return head + r;
}

// threads per block: one 32-warp block per SM for patches up to 96 taps;
// 8-warp blocks for larger patches (their target patches need more shared
// memory per warp)
template <int NT>
constexpr int pm_block() { return NT > 3 ? 256 : 1024; }

template <int KIND, int C, int NT>
__global__ void __launch_bounds__(pm_block<NT>(), NT > 3 ? 2 : 1) k_pm_init(DistArgs a, PmArgs p, const int2 *__restrict__ init,
                                                    int2 *__restrict__ nnf, float *__restrict__ dist,
                                                    unsigned long long *counter)
{
	const int lane = threadIdx.x & 31;
	TapTable<NT> T;
	make_taps<KIND, NT>(a, p, T);
	unsigned evals = 0, partial = 0;
	// block b takes the contiguous range [b * chunk, (b + 1) * chunk) of the
	// raster-ordered target list, its warps interleaved over the range, so
	// the warps of an SM work on neighbouring points and share source
	// neighbourhoods in L1
	const int chunk = (p.nt + gridDim.x - 1) / gridDim.x;
	const int end = min(p.nt, (int)(blockIdx.x + 1) * chunk);
	for (int wi = blockIdx.x * chunk + (threadIdx.x >> 5); wi < end; wi += blockDim.x >> 5) {
		const int pix = p.tlist[wi];
		const int x = pix % p.tW, y = pix / p.tW;
		Rng rng(p.key, (uint32_t)pix, 0xffffffffu);
		int2 n = init ? init[pix] : make_int2(-1, -1);
		int tries = 0;
		// patch_match.cpp:341-381: keep a seed match that lies in the
		// source, otherwise redraw it uniformly up to `shots` times
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
		float d = FLT_MAX;
		if (src_ok(p, n.x, n.y) && tgt_patch_inside(p, x, y)) {
			TargetPatch<KIND, C, NT> P = warp_target_slot<KIND, C, NT>();
			load_target<KIND, C, NT>(T, p, pix, P);
			d = warp_distance<KIND, C, NT>(T, P, p, n.y * p.sW + n.x, FLT_MAX, partial);
			evals++;
		} else {
			n = make_int2(-1, -1);
		}
		if (lane == 0) {
			nnf[pix] = n;
			dist[pix] = d;
		}
	}
	if (lane == 0 && evals) {
		atomicAdd(counter, (unsigned long long)evals);
		if (partial) atomicAdd(counter + 1, (unsigned long long)partial);
	}
}

template <int KIND, int C, int NT>
__global__ void __launch_bounds__(pm_block<NT>(), NT > 3 ? 2 : 1) k_pm_sweep(DistArgs a, PmArgs p, int sweep, int jump,
                                                     const int2 *__restrict__ nnf_in, const float *__restrict__ dist_in,
                                                     int2 *__restrict__ nnf_out, float *__restrict__ dist_out,
                                                     unsigned long long *counter)
{
	const int lane = threadIdx.x & 31;
	TapTable<NT> T;
	make_taps<KIND, NT>(a, p, T);
	unsigned evals = 0, partial = 0;
	// block b takes the contiguous range [b * chunk, (b + 1) * chunk) of the
	// raster-ordered target list, its warps interleaved over the range, so
	// the warps of an SM work on neighbouring points and share source
	// neighbourhoods in L1
	const int chunk = (p.nt + gridDim.x - 1) / gridDim.x;
	const int end = min(p.nt, (int)(blockIdx.x + 1) * chunk);
	for (int wi = blockIdx.x * chunk + (threadIdx.x >> 5); wi < end; wi += blockDim.x >> 5) {
		const int pix = p.tlist[wi];
		const int x = pix % p.tW, y = pix / p.tW;
		int2 best = nnf_in[pix];
		float bd = dist_in[pix];
		if (tgt_patch_inside(p, x, y)) {
			TargetPatch<KIND, C, NT> P = warp_target_slot<KIND, C, NT>();
			load_target<KIND, C, NT>(T, p, pix, P);
			auto consider = [&](int cx, int cy) {
				if ((cx != best.x || cy != best.y) && src_ok(p, cx, cy)) {
					const float d = warp_distance<KIND, C, NT>(T, P, p, cy * p.sW + cx, bd, partial);
					evals++;
					if (d < bd) {
						bd = d;
						best = make_int2(cx, cy);
					}
				}
			};
			// propagation from the neighbours at distance 1 and at the jump distance
#pragma unroll 1
			for (int si = 0; si < (jump > 1 ? 2 : 1); si++) {
				const int s = si ? jump : 1;
				if (tgt_ok(p, x - s, y)) {
					const int2 q = nnf_in[pix - s];
					if (q.x >= 0) consider(q.x + s, q.y);
				}
				if (tgt_ok(p, x + s, y)) {
					const int2 q = nnf_in[pix + s];
					if (q.x >= 0) consider(q.x - s, q.y);
				}
				if (tgt_ok(p, x, y - s)) {
					const int2 q = nnf_in[pix - s * p.tW];
					if (q.x >= 0) consider(q.x, q.y + s);
				}
				if (tgt_ok(p, x, y + s)) {
					const int2 q = nnf_in[pix + s * p.tW];
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
		} else {
			best = make_int2(-1, -1);
			bd = FLT_MAX;
		}
		if (lane == 0) {
			nnf_out[pix] = best;
			dist_out[pix] = bd;
		}
	}
	if (lane == 0 && evals) {
		atomicAdd(counter, (unsigned long long)evals);
		if (partial) atomicAdd(counter + 1, (unsigned long long)partial);
	}
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

template <int KIND, int C, int NT>
static void run_sweeps(nli_ctx *ctx, const DistArgs &a, const PmArgs &p, int iterations, const int2 *init,
                       int2 *nnf_x, float *dist_x, int2 *nnf_y, float *dist_y, unsigned long long *counter)
{
	// persistent: one block per SM (fewer when there are fewer points)
	const int block = pm_block<NT>();
	const int grid = (int)std::min<size_t>(((size_t)p.nt * 32 + block - 1) / block,
	                                       (size_t)ctx->num_sms * (NT > 3 ? 2 : 1));
	const size_t smem = target_smem_bytes<KIND, C, NT>(block / 32);
	static bool smem_attr = false;
	if (!smem_attr) {
		NLI_CUDA(cudaFuncSetAttribute(k_pm_init<KIND, C, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
		NLI_CUDA(cudaFuncSetAttribute(k_pm_sweep<KIND, C, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
		smem_attr = true;
	}
	{
		ProfScope ps(ctx, "pm_init");
		k_pm_init<KIND, C, NT><<<grid, block, smem, ctx->stream>>>(a, p, init, nnf_x, dist_x, counter);
		NLI_CHECK_LAUNCH();
	}
	for (int it = 0; it < iterations; it++) {
		const bool even = (it % 2) == 0;
		ProfScope ps(ctx, "pm_sweep");
		k_pm_sweep<KIND, C, NT><<<grid, block, smem, ctx->stream>>>(
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
	float4 *fs4 = ctx->buf<float4>("pm.fs4", (size_t)nS * a.p4);
	float *fs1 = a.f1 ? ctx->buf<float>("pm.fs1", (size_t)nS) : nullptr;
	launch_features(s, dp.kind, src, sW, sH, C, fs4, fs1);
	float4 *ft4 = fs4;
	float *ft1 = fs1;
	if (!(tgt == src && tW == sW && tH == sH)) {
		ft4 = ctx->buf<float4>("pm.ft4", (size_t)nT * a.p4);
		ft1 = a.f1 ? ctx->buf<float>("pm.ft1", (size_t)nT) : nullptr;
		launch_features(s, dp.kind, tgt, tW, tH, C, ft4, ft1);
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
	// [0]: candidates evaluated, [1]: of these, stopped after the first 32 taps
	unsigned long long *counter = ctx->buf<unsigned long long>("pm.counter", 2);
	k_fill_nnf<<<(nT + 255) / 256, 256, 0, s>>>(nnf_x, out_dist, nT);
	NLI_CHECK_LAUNCH();
	if (n_target > 0) {
		PmArgs p;
		p.fs4 = fs4;
		p.fs1 = fs1;
		p.ft4 = ft4;
		p.ft1 = ft1;
		p.sN = nS;
		p.tN = nT;
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
		if (energy) NLI_CUDA(cudaMemsetAsync(counter, 0, 2 * sizeof(unsigned long long), s));
#define NLI_PM_CASE(KIND, CC)                                                                              \
	if (dp.kind == KIND && C == CC) {                                                                          \
		if (a.px * a.py <= 96)                                                                                 \
			run_sweeps<KIND, CC, 3>(ctx, a, p, pm.iterations, init, nnf_x, dist_x, nnf_y, dist_y, counter);  \
		else                                                                                                   \
			run_sweeps<KIND, CC, 8>(ctx, a, p, pm.iterations, init, nnf_x, dist_x, nnf_y, dist_y, counter);  \
		handled = true;                                                                                        \
	}
		bool handled = false;
		NLI_PM_CASE(NLI_DIST_L2_COMBINED, 3)
		NLI_PM_CASE(NLI_DIST_L2_COMBINED, 1)
		NLI_PM_CASE(NLI_DIST_L2_COMBINED, 4)
		NLI_PM_CASE(NLI_DIST_L2_RGBD, 4)
		NLI_PM_CASE(NLI_DIST_L2_NORM, 3)
		NLI_PM_CASE(NLI_DIST_L2_NORM, 1)
		NLI_PM_CASE(NLI_DIST_L2_NORM, 4)
		NLI_PM_CASE(NLI_DIST_L1_NORM, 3)
		NLI_PM_CASE(NLI_DIST_L1_NORM, 1)
		NLI_PM_CASE(NLI_DIST_L1_NORM, 4)
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
			NLI_CUDA(cudaMemcpyAsync(hc, counter, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
			NLI_CUDA(cudaMemcpyAsync(hc + 2, partials + eg, sizeof(double), cudaMemcpyDeviceToHost, s));
			NLI_CUDA(cudaStreamSynchronize(s));
			ctx->candidates += (int64_t)hc[0];
			ctx->candidates_partial += (int64_t)hc[1];
			*energy = *reinterpret_cast<double *>(hc + 2);
		}
	} else if (energy) {
		*energy = 0.0;
	}
}

// Device counter of evaluated candidates of the last PatchMatch calls
// (read by the multiscale driver for its statistics).
unsigned long long *pm_counter(nli_ctx *ctx) { return ctx->buf<unsigned long long>("pm.counter", 1); }

}  // namespace nli
