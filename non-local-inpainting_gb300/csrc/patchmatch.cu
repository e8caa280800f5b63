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
// A candidate equal to the current match, or to an earlier candidate of the
// same step, is not re-evaluated (its distance would not be smaller).
// Random draws come from Philox4x32-10 keyed by the context seed and call
// counter.
//
// Layout and work split.  Images are read as one float4 per pixel (the C
// channels, zero-filled), with one extra column and row that repeat the
// last ones, so the forward differences u(x+1) - u(x) and u(y+1) - u(y) are
// exactly 0 on the last column / row, as Gradient::calculate sets them
// (gradient.cpp:37-63).  One warp works on one target point at a time
// (persistent warps); its target window (patch + 1 column + 1 row) sits in
// shared memory.  The warp's lanes are split into K = 32 / L sub-warps of
// L = patch width + 1 lanes (3 sub-warps of 10 lanes for 9x9 patches); each
// sub-warp evaluates one candidate, lane c walking down column c of the
// candidate's window.  Per row a lane loads one float4, forms the colour
// difference d = u_s - u_t, gets d of column c + 1 by a shuffle (x gradient
// difference) and keeps the previous row's d in registers (y gradient
// difference).  The gradient difference of the two patches is formed as a
// difference of colour differences, (u_s(x+1) - u_t(x+1)) - (u_s(x) - u_t(x)),
// which equals (gx_s - gx_t) up to float rounding.  The candidates of one
// step (propagation, then random search) are gathered first, one per lane,
// then evaluated K at a time and accepted in their sequential order with a
// strict "<", so the result equals evaluating them one after the other.
#include <cuda.h>  // CUtensorMap (the descriptor type; encoded through the runtime's driver entry point)

#include <atomic>

#include "nli_device.cuh"

namespace nli {

constexpr unsigned kFull = 0xffffffffu;

// ------------------------------------------------------- TMA staging
// With 9 x 9 patches each candidate's source window (rows x L float4) is
// copied into the warp's shared memory by one tensor copy
// (cp.async.bulk.tensor.2d) instead of being read row by row through L1.
// The copies of a step complete on the warp's mbarrier; waiting is bounded
// and a wait that runs out sets the context's timeout flag.
constexpr unsigned kTmaWaitLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity)
{
	uint32_t ok;
	asm volatile(
	    "{\n\t.reg .pred p;\n\t"
	    "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
	    "selp.u32 %0, 1, 0, p;\n\t}"
	    : "=r"(ok)
	    : "r"(smem_u32(bar)), "r"(parity)
	    : "memory");
	return ok != 0;
}

// Bounded wait for the phase `parity` of the barrier; false when it ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity)
{
	for (unsigned i = 0; i < kTmaWaitLimit; i++)
		if (mbar_try_wait(bar, parity)) return true;
	return false;
}

// Orders this thread's earlier generic-proxy accesses of shared memory
// before later async-proxy (tensor copy) writes to it.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Tile [x, x + box0) x [y, y + box1) of the 2-D tensor into dst; x counts
// floats and is a multiple of 4 (16 bytes) here.
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar)
{
	asm volatile(
	    "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
	        smem_u32(dst)),
	    "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
	    : "memory");
}

// How the fixed-size (9 x 9) kernels read a candidate's two windows
// (NLI_TUNE_PM_VARIANT): kPmShared keeps the target window in shared memory
// and loads source rows from global memory (32 warps per SM); kPmStaged also
// copies the source windows into shared memory by tensor copies; kPmRegs
// holds the lane's column of the target window in registers (16 warps per
// SM, twice the registers).  All three evaluate the same candidates with the
// same arithmetic.  Runtime-sized patches always use kPmShared.
enum PmVariant { kPmShared = 0, kPmStaged = 1, kPmRegs = 2 };

__host__ __device__ constexpr int pm_threads(int V) { return V == kPmRegs ? 512 : 1024; }

// Per-warp state of the staged path.
struct TmaState {
	const CUtensorMap *map;
	float4 *slots;    // K windows of rows x L float4, each slot_stride float4 apart
	int slot_stride;  // float4
	uint64_t *bar;
	unsigned phase;
	int *timeout;  // context status flag
};

struct PmArgs {
	const float4 *src;  // source pixels, (sW + 1) x (sH + 1), row stride sWp
	const float4 *tgt;  // target pixels, row stride tWp
	const uint8_t *smask;
	const uint8_t *tmask;
	const int32_t *tlist;
	int sW, sH, tW, tH, nt;
	int sWp, tWp;
	int shots, max_window;
	uint64_t seed;                     // the context's seed
	const unsigned long long *calls;   // PatchMatch calls so far, this one included
	// patch extent around a centre: [x - rx, x + ex) x [y - ry, y + ey)
	int rx, ry, ex, ey;
	// lanes per candidate, candidates per warp step, window rows
	int L, K, rows;
	float lambda, lambda_d;
	// patch-mean lower bound (null: off): the weighted patch means of the
	// padded source and target, one float4 per (W + 1) x (H + 1) position,
	// and the largest absolute pixel value of the images (as float bits)
	const float4 *smom, *tmom;
	const unsigned *vmax;
	// 1: the tables also hold the weighted standard deviations (of the
	// image and of its forward differences), and the bound uses them
	int dev;
	// device work queue (null: static ranges): the call's counters, one
	// per launch (init, then each sweep), zeroed before the init launch;
	// a warp takes `tile` consecutive target points per grab
	unsigned *queue;
	int tile;
};

// Philox key of this PatchMatch call: the seed mixed with the call's index
// (0 for the first call after the seed is set).
__device__ __forceinline__ uint2 pm_key(const PmArgs &p)
{
	const uint64_t call = *p.calls - 1ull;
	const uint64_t k = p.seed ^ (call * 0x9E3779B97F4A7C15ULL);
	return make_uint2((uint32_t)k, (uint32_t)(k >> 32) ^ (uint32_t)call);
}

template <int KIND>
struct Kind {
	static constexpr bool grad = KIND == NLI_DIST_L2_COMBINED || KIND == NLI_DIST_L2_RGBD;
};

// The work items [0, n) of a persistent PatchMatch launch, visited by the
// calling warp (f(i) for each of its items, in increasing order).  Without
// a queue, block b takes the contiguous range [b * chunk, (b + 1) * chunk)
// and its warps interleave over it, so the warps of an SM work on
// neighbouring points and share source neighbourhoods in L1.  With a queue
// (`queue` a counter zeroed before the launch), each warp takes `tile`
// consecutive items per atomic grab until the list is exhausted, so warps
// that drew cheap points take more and no SM idles while others finish.
// Every item's computation is independent of which warp does it and when
// (the sweeps read the previous field and the random streams are keyed by
// point), so both give the same field.
template <class F>
__device__ __forceinline__ void pm_for_each(int n, unsigned *queue, int tile, F &&f)
{
	if (queue) {
		const int lane = threadIdx.x & 31;
		for (;;) {
			unsigned base = 0u;
			if (lane == 0) base = atomicAdd(queue, (unsigned)tile);
			base = __shfl_sync(kFull, base, 0);
			if (base >= (unsigned)n) break;
			const int stop = min(n, (int)base + tile);
			for (int i = (int)base; i < stop; i++) f(i);
		}
	} else {
		const int chunk = (n + gridDim.x - 1) / gridDim.x;
		const int end = min(n, (int)(blockIdx.x + 1) * chunk);
		for (int i = blockIdx.x * chunk + (threadIdx.x >> 5); i < end; i += blockDim.x >> 5) f(i);
	}
}

// A source centre is usable when it is in the source mask and its whole
// patch lies in the image (the masks of the inpainting driver guarantee the
// latter through their margin; user masks may not).
__device__ __forceinline__ bool src_ok(const PmArgs &p, int x, int y)
{
	return x >= p.rx && y >= p.ry && x + p.ex <= p.sW && y + p.ey <= p.sH &&
	       nli_in_bounds((long long)y * p.sW + x, (long long)p.sW * p.sH, kSitePmMask) && p.smask[y * p.sW + x];
}

__device__ __forceinline__ bool tgt_patch_inside(const PmArgs &p, int x, int y)
{
	return x >= p.rx && y >= p.ry && x + p.ex <= p.tW && y + p.ey <= p.tH;
}

__device__ __forceinline__ bool tgt_ok(const PmArgs &p, int x, int y)
{
	return (unsigned)x < (unsigned)p.tW && (unsigned)y < (unsigned)p.tH && p.tmask[y * p.tW + x];
}

// Shared memory: per-tap weights (divided by the patch area) for all warps,
// padded to a float4 boundary, then one target window of rows x L float4
// per warp, then one 32-entry candidate list per warp.
__host__ __device__ inline int pm_weight_slots(int taps) { return (taps + 3) / 4; }

__host__ __device__ inline size_t pm_smem_bytes(int taps, int rows, int L, int warps)
{
	return sizeof(float4) * ((size_t)pm_weight_slots(taps) + (size_t)warps * rows * L) + sizeof(int) * 32 * warps;
}

__device__ __forceinline__ void load_weights(const DistArgs &a, float *s_w)
{
	const int taps = a.px * a.py;
	const float invP = 1.0f / (float)taps;
	for (int t = threadIdx.x; t < taps; t += blockDim.x) s_w[t] = a.weights[t] * invP;
	__syncthreads();
}

// The warp's target window: rows x L pixels starting at the patch corner.
// With up to 3 channels the unused fourth component carries the tap's
// weight (0 outside the patch), so the distance reads one float4 per row.
template <int KIND, int C, int P>
__device__ __forceinline__ void load_window(const PmArgs &p, const float *s_w, int x, int y, float4 *s_t)
{
	const int lane = threadIdx.x & 31;
	// compiled sizes for P x P patches (a division by a constant), else the call's
	constexpr int LP = P ? P + (Kind<KIND>::grad ? 1 : 0) : 1;
	const int L = P ? LP : p.L, rows = P ? LP : p.rows;
	const int px = P ? P : p.rx + p.ex, py = P ? P : p.ry + p.ey;
	const float4 *T = p.tgt + (size_t)(y - p.ry) * p.tWp + (x - p.rx);
	for (int e = lane; e < rows * L; e += 32) {
		const int r = P ? e / LP : e / L, c = e - r * L;
		float4 v = __ldg(T + (size_t)r * p.tWp + c);
		if (C <= 3) v.w = (r < py && c < px) ? s_w[r * px + c] : 0.f;
		s_t[e] = v;
	}
	__syncwarp();
}

// kPmRegs: the lane's column c of the same window, tw[r] = element r * L + c
// of load_window's, for a fixed P x P patch.
template <int KIND, int C, int P>
__device__ __forceinline__ void load_window_regs(const PmArgs &p, const float *s_w, int x, int y, float4 *tw)
{
	constexpr int L = P + (Kind<KIND>::grad ? 1 : 0);
	const int lane = threadIdx.x & 31;
	const int c = lane - (lane / L) * L;
	const float4 *T = p.tgt + (size_t)(y - p.ry) * p.tWp + (x - p.rx) + c;
#pragma unroll
	for (int r = 0; r < L; r++) {
		float4 v = __ldg(T + (size_t)r * p.tWp);
		if (C <= 3) v.w = (r < P && c < P) ? s_w[r * P + c] : 0.f;
		tw[r] = v;
	}
}

template <int C>
__device__ __forceinline__ float sq3(float4 d)
{
	float n = d.x * d.x;
	if (C > 1) n = fmaf(d.y, d.y, n);
	if (C > 2) n = fmaf(d.z, d.z, n);
	return n;
}

// sum of squares / absolute values over the first C components
template <int C>
__device__ __forceinline__ float sqc(float4 d)
{
	float n = sq3<C>(d);
	if (C > 3) n = fmaf(d.w, d.w, n);
	return n;
}

template <int C>
__device__ __forceinline__ float absc(float4 d)
{
	float n = fabsf(d.x);
	if (C > 1) n += fabsf(d.y);
	if (C > 2) n += fabsf(d.z);
	if (C > 3) n += fabsf(d.w);
	return n;
}

// a - b over the first C components (the others are left 0)
template <int C>
__device__ __forceinline__ float4 subc(float4 a, float4 b)
{
	return make_float4(a.x - b.x, (C > 1) ? a.y - b.y : 0.f, (C > 2) ? a.z - b.z : 0.f, (C > 3) ? a.w - b.w : 0.f);
}

template <int C>
__device__ __forceinline__ float4 shfl_down4(float4 v, int o)
{
	float4 r;
	r.x = __shfl_down_sync(kFull, v.x, o);
	r.y = (C > 1) ? __shfl_down_sync(kFull, v.y, o) : 0.f;
	r.z = (C > 2) ? __shfl_down_sync(kFull, v.z, o) : 0.f;
	r.w = (C > 3) ? __shfl_down_sync(kFull, v.w, o) : 0.f;
	return r;
}

// Sum over the L lanes of each sub-warp, left in its lane c == 0.
__device__ __forceinline__ float subwarp_sum(float v, int c, int L)
{
#pragma unroll
	for (int o = 1; o < 16; o <<= 1) {
		const float u = __shfl_down_sync(kFull, v, o);
		if (c + o < L) v += u;
	}
	return v;
}

// Per-lane sums of one candidate by term: colour and gradient differences
// of the colour channels (n, g) and of the depth channel (nd, gd, L2 RGBD).
struct Acc {
	float n, g, nd, gd;
};

// Contribution of one window row.  d: colour difference of this lane's
// pixel in row r, dp: of the row above; w, wp: their tap weights.
template <int KIND, int C>
__device__ __forceinline__ void row_terms(const float4 d, const float4 dp, float w, float wp, bool tap, bool tap_above,
                                          Acc &A)
{
	if (KIND == NLI_DIST_L1_NORM) {
		if (tap) A.n = fmaf(w, absc<C>(d), A.n);
		return;
	}
	if (KIND == NLI_DIST_L2_NORM) {
		if (tap) A.n = fmaf(w, sqc<C>(d), A.n);
		return;
	}
	// x gradient difference from the lane to the right (column c + 1)
	const float4 dr = shfl_down4<C>(d, 1);
	if (KIND == NLI_DIST_L2_RGBD) {
		if (tap) {
			const float4 gx = subc<4>(dr, d);
			A.n = fmaf(w, sq3<3>(d), A.n);
			A.g = fmaf(w, sq3<3>(gx), A.g);
			A.nd = fmaf(w, d.w * d.w, A.nd);
			A.gd = fmaf(w, gx.w * gx.w, A.gd);
		}
		if (tap_above) {
			const float4 gy = subc<4>(d, dp);
			A.g = fmaf(wp, sq3<3>(gy), A.g);
			A.gd = fmaf(wp, gy.w * gy.w, A.gd);
		}
	} else {
		if (tap) {
			const float4 gx = subc<C>(dr, d);
			A.n = fmaf(w, sqc<C>(d), A.n);
			A.g = fmaf(w, sqc<C>(gx), A.g);
		}
		if (tap_above) {
			const float4 gy = subc<C>(d, dp);
			A.g = fmaf(wp, sqc<C>(gy), A.g);
		}
	}
}

// The lane's share of the distance: the terms weighted by lambda, 1 - lambda
// (and lambda_d, 1 - lambda_d for the depth channel).
template <int KIND>
__device__ __forceinline__ float combine(const Acc &A, const PmArgs &p)
{
	if (KIND == NLI_DIST_L1_NORM || KIND == NLI_DIST_L2_NORM) return A.n;
	float v = fmaf(p.lambda, A.n, (1.0f - p.lambda) * A.g);
	if (KIND == NLI_DIST_L2_RGBD) v = fmaf(p.lambda_d, A.nd, fmaf(1.0f - p.lambda_d, A.gd, v));
	return v;
}

// float4 helpers of the patch statistics
__device__ __forceinline__ float4 f4_fma(float w, float4 v, float4 a)
{
	return make_float4(fmaf(w, v.x, a.x), fmaf(w, v.y, a.y), fmaf(w, v.z, a.z), fmaf(w, v.w, a.w));
}
__device__ __forceinline__ float4 f4_sub(float4 a, float4 b)
{
	return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w);
}
__device__ __forceinline__ float4 f4_wsq(float w, float4 d, float4 a)
{
	return make_float4(fmaf(w, d.x * d.x, a.x), fmaf(w, d.y * d.y, a.y), fmaf(w, d.z * d.z, a.z),
	                   fmaf(w, d.w * d.w, a.w));
}
__device__ __forceinline__ float4 f4_sqrt(float4 a)
{
	return make_float4(sqrtf(a.x), sqrtf(a.y), sqrtf(a.z), sqrtf(a.w));
}

// ------------------------------------------------ patch-mean lower bound
// Jensen's inequality gives, for weights v_k >= 0 summing to V,
//   sum_k v_k |d_k|^2 >= |sum_k v_k d_k|^2 / V,   sum_k v_k |d_k|_1 >= |sum_k v_k d_k|_1.
// With the kernel's tap weights v_k = w_k / P (sum 1 / P) and d_k the colour
// or gradient difference of tap k, sum_k w_k d_k is the difference of the
// two patches' weighted means of the image or of its forward differences;
// the mean of the differences is the difference of means one column (row)
// apart.  So a candidate whose patch means differ enough from the target's
// cannot beat the current match and is not evaluated.
//
// With the weighted standard deviations as well (PmArgs::dev, the L2
// kinds), the bound is tighter: for weights summing to 1,
//   sum_k w_k d_k^2 = (sum_k w_k d_k)^2 + sum_k w_k (d_k - mean d)^2,
// and with d = s - t the centred part is the squared weighted L2 distance of
// the centred patches, at least (sigma_s - sigma_t)^2 by the reverse
// triangle inequality.  So each channel's colour term is bounded by the
// squared mean difference plus the squared difference of standard
// deviations, and each gradient term likewise with the deviations of the
// forward differences.
//
// Exactness: every mean and deviation difference is shrunk by a slack (2e-4
// of the largest pixel value) that covers the float rounding of the tables
// (sums of 81 products: a few 1e-6 of the largest value) and of the
// kernel's per-tap differences, and the bound must exceed the current
// distance by a 1e-4 relative margin that covers the rounding of the
// kernel's sums; the field and distances are those of evaluating every
// candidate.
__device__ __forceinline__ float shrink(float v, float slack) { return fmaxf(fabsf(v) - slack, 0.f); }

// True when candidate (cx, cy) for target (x, y) provably cannot reach a
// distance below bd.  The target's means are read here too (the same
// address in every lane), so nothing stays live across the evaluations.
template <int KIND, int C>
__device__ __forceinline__ bool bound_rejects(const PmArgs &p, int x, int y, int cx, int cy, float bd)
{
	const float4 *M = p.smom + (size_t)cy * p.sWp + cx;
	const float4 *T = p.tmom + (size_t)y * p.tWp + x;
	const float slack = 2e-4f * __uint_as_float(__ldg(p.vmax));
	// per-channel terms, the depth channel of L2 RGBD kept apart; each
	// statistic is read, folded in and dropped in turn (few live registers)
	float col = 0.f, grad = 0.f, dcol = 0.f, dgrad = 0.f;
	auto add = [&](float4 d, bool g) {
		const float v[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
		for (int c = 0; c < C; c++) {
			const float e = shrink(v[c], slack);
			const bool depth = KIND == NLI_DIST_L2_RGBD && c == 3;
			if (KIND == NLI_DIST_L1_NORM)
				col += e;
			else if (depth)
				(g ? dgrad : dcol) += e * e;
			else
				(g ? grad : col) += e * e;
		}
	};
	const float4 m0 = __ldg(M), t0 = __ldg(T);
	add(f4_sub(m0, t0), false);
	if (Kind<KIND>::grad) {
		// the mean of the forward differences: means one column (row) apart
		add(f4_sub(f4_sub(__ldg(M + 1), m0), f4_sub(__ldg(T + 1), t0)), true);
		add(f4_sub(f4_sub(__ldg(M + p.sWp), m0), f4_sub(__ldg(T + p.tWp), t0)), true);
	}
	if (KIND != NLI_DIST_L1_NORM && p.dev) {
		// weighted standard deviations: of the image, of its x and y differences
		const size_t sn = (size_t)p.sWp * (p.sH + 1), tn = (size_t)p.tWp * (p.tH + 1);
		add(f4_sub(__ldg(M + sn), __ldg(T + tn)), false);
		if (Kind<KIND>::grad) {
			add(f4_sub(__ldg(M + 2 * sn), __ldg(T + 2 * tn)), true);
			add(f4_sub(__ldg(M + 3 * sn), __ldg(T + 3 * tn)), true);
		}
	}
	float lb = col;
	if (Kind<KIND>::grad) lb = fmaf(p.lambda, col, (1.0f - p.lambda) * grad);
	if (KIND == NLI_DIST_L2_RGBD) lb = fmaf(p.lambda_d, dcol, fmaf(1.0f - p.lambda_d, dgrad, lb));
	const float P = (float)((p.rx + p.ex) * (p.ry + p.ey));
	return lb * (1.0f - 1e-4f) >= bd * P;
}

// Weighted patch statistics of the padded image at every position of the
// (W + 1) x (H + 1) grid (window clamped to the grid): table 0 the weighted
// means; with `dev`, tables 1-3 (each n = (W + 1)(H + 1) float4 further) the
// weighted standard deviations of the image and of its forward differences
// in x and in y, sqrt(sum_k w_k (v_k - mean)^2), from a second, centred
// pass.  Also the largest absolute pixel value (atomicMax on the float bits
// of non-negative values).
__device__ __forceinline__ void moments_span(const DistArgs &a, const float4 *__restrict__ pad, int W, int H,
                                             float4 *__restrict__ mom, unsigned *vmax, int first, int stride,
                                             bool dev)
{
	const int Wp = W + 1, n = Wp * (H + 1);
	float vm = 0.f;
	const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
	for (int i = first; i < n; i += stride) {
		const int y = i / Wp, x = i - y * Wp;
		float4 acc = zero, ax = zero, ay = zero;
		for (int dy = 0; dy < a.py; dy++) {
			const int yy = min(max(y - a.ry + dy, 0), H);
			const float4 *row = pad + (size_t)yy * Wp, *below = pad + (size_t)min(yy + 1, H) * Wp;
			for (int dx = 0; dx < a.px; dx++) {
				const int xx = min(max(x - a.rx + dx, 0), W);
				const float4 v = __ldg(row + xx);
				const float w = a.weights[dy * a.px + dx];
				acc = f4_fma(w, v, acc);
				if (dev) {
					ax = f4_fma(w, f4_sub(__ldg(row + min(xx + 1, W)), v), ax);
					ay = f4_fma(w, f4_sub(__ldg(below + xx), v), ay);
				}
			}
		}
		mom[i] = acc;
		if (dev) {
			float4 s = zero, sx = zero, sy = zero;
			for (int dy = 0; dy < a.py; dy++) {
				const int yy = min(max(y - a.ry + dy, 0), H);
				const float4 *row = pad + (size_t)yy * Wp, *below = pad + (size_t)min(yy + 1, H) * Wp;
				for (int dx = 0; dx < a.px; dx++) {
					const int xx = min(max(x - a.rx + dx, 0), W);
					const float4 v = __ldg(row + xx);
					const float w = a.weights[dy * a.px + dx];
					s = f4_wsq(w, f4_sub(v, acc), s);
					sx = f4_wsq(w, f4_sub(f4_sub(__ldg(row + min(xx + 1, W)), v), ax), sx);
					sy = f4_wsq(w, f4_sub(f4_sub(__ldg(below + xx), v), ay), sy);
				}
			}
			mom[(size_t)n + i] = f4_sqrt(s);
			mom[2 * (size_t)n + i] = f4_sqrt(sx);
			mom[3 * (size_t)n + i] = f4_sqrt(sy);
		}
		const float4 v = __ldg(pad + i);
		vm = fmaxf(vm, fmaxf(fmaxf(fabsf(v.x), fabsf(v.y)), fmaxf(fabsf(v.z), fabsf(v.w))));
	}
	for (int o = 16; o > 0; o >>= 1) vm = fmaxf(vm, __shfl_xor_sync(0xffffffffu, vm, o));
	if ((threadIdx.x & 31) == 0 && vm > 0.f) atomicMax(vmax, __float_as_uint(vm));
}

__global__ void k_pm_moments(DistArgs a, const float4 *__restrict__ pad, int W, int H, float4 *__restrict__ mom,
                             unsigned *vmax, int dev)
{
	moments_span(a, pad, W, H, mom, vmax, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, dev != 0);
}

// Evaluates the n candidates held one per lane (packed x | y << 16, lane i
// holds candidate i) against the target window s_t, in steps of K, and
// accepts each in order when strictly better than the current match.  All
// lanes return the same best / bd.  Once the rows summed so far reach the
// current distance for every candidate of a step, the rest of the step is
// skipped (exact: all terms are non-negative).  P > 0: square P x P patch
// known at compile time (rows unrolled); P == 0: sizes from the arguments.
// kPmStaged: the step's source windows are copied into the warp's slots
// first (one tensor copy per candidate) and the rows are read from there.
// kPmRegs: the target rows come from tw (registers) instead of s_t.
template <int KIND, int C, int P, int V = kPmShared>
__device__ __forceinline__ void eval_candidates(const PmArgs &p, const float *s_w, const float4 *s_t, int mycand,
                                                int n, int2 &best, float &bd, unsigned &partial,
                                                TmaState *ts = nullptr, const float4 *tw = nullptr)
{
	constexpr bool TMA = V == kPmStaged;
	constexpr bool G = Kind<KIND>::grad;
	constexpr int PF = (C == 4) ? 1 : 2;  // rows of loads in flight (fewer for 4 channels: registers)
	if (TMA && ts->map == nullptr) return;  // this warp's staging gave up (timeout flagged)
	const int L = P ? P + G : p.L;
	const int K = P ? 32 / (P + G) : p.K;
	const int rows = P ? P + G : p.rows;
	const int px = P ? P : p.rx + p.ex;
	const int py = P ? P : p.ry + p.ey;
	const int lane = threadIdx.x & 31;
	const int sw = lane / L, c = lane - sw * L;
	const bool tapcol = c < px;
	const int check_row = rows / 2;
	const size_t sWp = (size_t)p.sWp;
	const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 1
	for (int b = 0; b < n; b += K) {
		const int idx = b + sw;
		const bool active = sw < K && idx < n;
		const bool act_col = active && tapcol;
		const int cand = __shfl_sync(kFull, mycand, active ? idx : 0);
		const int cx = cand & 0xffff, cy = cand >> 16;
		const float4 *S = p.src + (size_t)(cy - p.ry) * sWp + (cx - p.rx) + c;
		// row r of this lane's column of the candidate's window (a checked
		// build tests the index against the padded source)
		const long long s_base = (long long)(cy - p.ry) * (long long)sWp + (cx - p.rx) + c;
		const long long s_n = (long long)sWp * (p.sH + 1);
		auto ldrow = [&](int r) -> float4 {
			return nli_in_bounds(s_base + (long long)r * (long long)sWp, s_n, kSitePmSource) ? __ldg(S + (size_t)r * sWp)
			                                                                                 : zero;
		};
		const float4 *T = s_t + c;
		const float *Wt = s_w + c;
		const float4 *Sl = nullptr;  // this lane's column of its candidate's staged window
		if constexpr (TMA) {
			static_assert(P > 0, "the staged path is compiled for fixed patch sizes");
			constexpr int KC = 32 / (P + G);
			const int nact = min(K, n - b);
			int cs[KC];
#pragma unroll
			for (int s = 0; s < KC; s++) cs[s] = __shfl_sync(kFull, mycand, min(b + s, 31));
			__syncwarp();
			if (lane == 0) {
				fence_proxy_async();
				mbar_expect_tx(ts->bar, (unsigned)(nact * rows * L * sizeof(float4)));
#pragma unroll
				for (int s = 0; s < KC; s++)
					if (s < nact)
						tma_load_2d(ts->slots + s * ts->slot_stride, ts->map, 4 * ((cs[s] & 0xffff) - p.rx),
						            (cs[s] >> 16) - p.ry, ts->bar);
			}
			const bool landed = __all_sync(kFull, mbar_wait(ts->bar, ts->phase));
			if (!landed) {
				// the copies did not land in time: flag it, give them one more
				// bounded wait, and stop using this warp's slots
				if (lane == 0) atomicExch(ts->timeout, 1);
				mbar_wait(ts->bar, ts->phase);
				ts->map = nullptr;
				return;
			}
			ts->phase ^= 1u;
			Sl = ts->slots + (active ? sw : 0) * ts->slot_stride + c;
		}
		float4 v0 = (!TMA && active) ? ldrow(0) : zero;
		float4 v1 = (!TMA && PF == 2 && active && rows > 1) ? ldrow(1) : zero;
		float4 dp = zero;
		float wp = 0.f;
		Acc A = {0.f, 0.f, 0.f, 0.f};
		const float bound = bd;
		bool stop = false;
		auto row = [&](int r) {
			float4 v = v0;
			if (TMA) {
				v = active ? Sl[r * L] : zero;
			} else if (PF == 2) {
				v0 = v1;
				v1 = (active && r + 2 < rows) ? ldrow(r + 2) : zero;
			} else {
				v0 = (active && r + 1 < rows) ? ldrow(r + 1) : zero;
			}
			float4 t;
			if constexpr (V == kPmRegs)
				t = tw[r];
			else
				t = T[r * L];
			const float4 d = subc<C>(v, t);
			const bool tap = act_col && r < py;
			const float w = (C <= 3) ? t.w : (tap ? Wt[r * px] : 0.f);
			row_terms<KIND, C>(d, dp, w, wp, tap, G && act_col && r > 0, A);
			dp = d;
			wp = w;
		};
		auto check = [&]() {
			const float part = subwarp_sum(combine<KIND>(A, p), c, L);
			return __all_sync(kFull, !active || c != 0 || part >= bound);
		};
		if constexpr (P > 0) {
			// one test after the first (P + G) / 2 - 1 rows (4 of 10 for 9x9
			// L2 combined).  On the 512x512 benchmark without the lower bound
			// it stops 57.5 % of the candidates and is 1.6 % faster than a
			// test at half the window (65 % stopped); two tests (rows 5 and 7,
			// or 3 and 5 and 7) cost more than they save.  With the bound,
			// tests after rows 5, 6 or 7, or after 4 and 7, take the same
			// time within 0.3 %
			constexpr int kCheckRow = (P + G) / 2 - 2;
#pragma unroll
			for (int r = 0; r < P + G; r++) {
				row(r);
				if (r == kCheckRow && check()) {
					stop = true;
					break;
				}
			}
		} else {
#pragma unroll 1
			for (int r = 0; r < rows; r++) {
				row(r);
				if (r == check_row && check()) {
					stop = true;
					break;
				}
			}
		}
		const int in_step = min(K, n - b);
		if (stop) {
			partial += in_step;
			continue;
		}
		const float sum = subwarp_sum(combine<KIND>(A, p), c, L);
#pragma unroll 1
		for (int s = 0; s < in_step; s++) {
			const float ds = __shfl_sync(kFull, sum, s * L);
			if (ds < bd) {
				bd = ds;
				const int q = __shfl_sync(kFull, mycand, b + s);
				best = make_int2(q & 0xffff, q >> 16);
			}
		}
	}
}

// Candidates proposed one per lane, in lane order: keeps the valid ones that
// differ from the current match and from every lower lane's candidate and
// moves them to lanes 0..n-1 (mycand), in order.  Returns n.
__device__ __forceinline__ int compact_candidates(bool valid, int packed, const int2 &best, int *s_list, int &mycand)
{
	const int lane = threadIdx.x & 31;
	const unsigned below = (1u << lane) - 1u;
	valid = valid && packed != (best.x | (best.y << 16));
	const unsigned vmask = __ballot_sync(kFull, valid);
	const unsigned same = __match_any_sync(kFull, valid ? packed : -1);
	const bool keep = valid && (same & vmask & below) == 0;
	const unsigned kmask = __ballot_sync(kFull, keep);
	if (keep) s_list[__popc(kmask & below)] = packed;
	__syncwarp();
	const int n = __popc(kmask);
	mycand = (lane < n) ? s_list[lane] : 0;
	__syncwarp();
	return n;
}

// Shared memory of the PatchMatch kernels: per-tap weights, then per warp a
// target window (rows x L float4) and a candidate list (32 ints).
struct PmSmem {
	float *w;
	float4 *t;
	int *list;
	float4 *slots;  // staged path: K windows per warp
	int slot_stride;
	uint64_t *bar;
};

// Staged path layout (float4 units, from a 128-byte aligned base): the
// weights, then per warp a region of the target window, K window slots, the
// candidate list and the mbarrier, every part starting on 128 bytes.
__host__ __device__ inline int pm_round8(int v) { return (v + 7) & ~7; }

__host__ __device__ inline int pm_tma_region(int rows, int L, int K)
{
	return pm_round8(pm_round8(rows * L) * (1 + K) + 8 + 1);
}

__host__ __device__ inline size_t pm_smem_bytes_tma(int taps, int rows, int L, int K, int warps)
{
	return 128 + sizeof(float4) * ((size_t)pm_round8(pm_weight_slots(taps)) + (size_t)warps * pm_tma_region(rows, L, K));
}

template <int V>
__device__ __forceinline__ PmSmem pm_smem(const DistArgs &a, const PmArgs &p)
{
	extern __shared__ float4 s_pm[];
	const int warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
	PmSmem m;
	const int ws = pm_weight_slots(a.px * a.py);
	if (V != kPmStaged) {
		m.w = reinterpret_cast<float *>(s_pm);
		m.t = s_pm + ws + warp * p.rows * p.L;
		m.list = reinterpret_cast<int *>(s_pm + ws + warps * p.rows * p.L) + warp * 32;
		m.slots = nullptr;
		m.slot_stride = 0;
		m.bar = nullptr;
	} else {
		float4 *base = reinterpret_cast<float4 *>((reinterpret_cast<uintptr_t>(s_pm) + 127) & ~(uintptr_t)127);
		const int win = pm_round8(p.rows * p.L);
		float4 *r = base + pm_round8(ws) + (size_t)warp * pm_tma_region(p.rows, p.L, p.K);
		m.w = reinterpret_cast<float *>(base);
		m.t = r;
		m.slots = r + win;
		m.slot_stride = win;
		m.list = reinterpret_cast<int *>(r + win * (1 + p.K));
		m.bar = reinterpret_cast<uint64_t *>(r + win * (1 + p.K) + 8);
	}
	return m;
}

// One target point of the initial field (patch_match.cpp:329-381): its
// seed match (the init field's, else random draws), and that match's
// distance.  Called by one whole warp; lane 0 writes the results.
template <int KIND, int C, int P, int V>
__device__ __forceinline__ void pm_init_point(const PmArgs &p, const PmSmem &m, TmaState &ts, float4 *tw,
                                              const uint2 key, int pix, const int2 *__restrict__ init,
                                              int2 *__restrict__ nnf, float *__restrict__ dist, unsigned &evals,
                                              unsigned &partial)
{
	const int lane = threadIdx.x & 31;
	if (!nli_in_bounds(pix, (long long)p.tW * p.tH, kSitePmTarget)) return;
	const int x = pix % p.tW, y = pix / p.tW;
	Rng rng(key, (uint32_t)pix, 0xffffffffu);
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
	int2 best = make_int2(-1, -1);
	if (src_ok(p, n.x, n.y) && tgt_patch_inside(p, x, y)) {
		if constexpr (V == kPmRegs)
			load_window_regs<KIND, C, P>(p, m.w, x, y, tw);
		else
			load_window<KIND, C, P>(p, m.w, x, y, m.t);
		eval_candidates<KIND, C, P, V>(p, m.w, m.t, n.x | (n.y << 16), 1, best, d, partial, &ts, tw);
		evals++;
		__syncwarp();
	}
	if (lane == 0) {
		nnf[pix] = best;
		dist[pix] = d;
	}
}

template <int KIND, int C, int P, int V>
__global__ void __launch_bounds__(pm_threads(V), 1) k_pm_init(DistArgs a, PmArgs p, const int2 *__restrict__ init,
                                                      int2 *__restrict__ nnf, float *__restrict__ dist,
                                                      unsigned long long *counter,
                                                      const __grid_constant__ CUtensorMap tmap, int *timeout)
{
	const int lane = threadIdx.x & 31;
	const PmSmem m = pm_smem<V>(a, p);
	TmaState ts = {&tmap, m.slots, m.slot_stride, m.bar, 0u, timeout};
	if (V == kPmStaged && lane == 0) mbar_init(m.bar, 1);
	float4 tw[(V == kPmRegs) ? P + 1 : 1];
	load_weights(a, m.w);
	const uint2 key = pm_key(p);
	unsigned evals = 0, partial = 0;
	pm_for_each(p.nt, p.queue, p.tile, [&](int wi) {
		pm_init_point<KIND, C, P, V>(p, m, ts, tw, key, p.tlist[wi], init, nnf, dist, evals, partial);
	});
	if (lane == 0 && evals) {
		atomicAdd(counter, (unsigned long long)evals);
		if (partial) atomicAdd(counter + 1, (unsigned long long)partial);
	}
}

// metric_prop (may be NULL): this sweep's count of target points that the
// propagation step improved; metric_shots (may be NULL): the largest index
// of a first accepted random draw (patch_match.cpp:452-456, 481-485).
// One target point of a sweep: propagation from the previous sweep's
// field, then random search around the best match.  Called by one whole
// warp; lane 0 writes the results.
template <int KIND, int C, int P, int V>
__device__ __forceinline__ void pm_sweep_point(const PmArgs &p, const PmSmem &m, TmaState &ts, float4 *tw,
                                               const uint2 key, int windows, int pix, int sweep, int jump,
                                               const int2 *__restrict__ nnf_in, const float *__restrict__ dist_in,
                                               int2 *__restrict__ nnf_out, float *__restrict__ dist_out,
                                               unsigned &evals, unsigned &partial, unsigned &improved, int &max_shot)
{
	const int lane = threadIdx.x & 31;
	if (!nli_in_bounds(pix, (long long)p.tW * p.tH, kSitePmTarget)) return;
	const int x = pix % p.tW, y = pix / p.tW;
	int2 best = nnf_in[pix];
	float bd = dist_in[pix];
	if (tgt_patch_inside(p, x, y)) {
		if constexpr (V == kPmRegs)
			load_window_regs<KIND, C, P>(p, m.w, x, y, tw);
		else
			load_window<KIND, C, P>(p, m.w, x, y, m.t);
		const bool bounded = p.smom != nullptr;
		// propagation: lane 4s + k proposes the match of neighbour k
		// (left, right, up, down) at distance 1 (s = 0) or at the jump
		// distance (s = 1), shifted back by the neighbour's offset
		bool valid = false;
		int packed = 0;
		if (lane < (jump > 1 ? 8 : 4)) {
			const int s = (lane < 4) ? 1 : jump, k = lane & 3;
			const int nx = x + ((k == 0) ? -s : (k == 1) ? s : 0);
			const int ny = y + ((k == 2) ? -s : (k == 3) ? s : 0);
			if (tgt_ok(p, nx, ny) && nli_in_bounds((long long)ny * p.tW + nx, (long long)p.tW * p.tH, kSitePmField)) {
				const int2 q = nnf_in[ny * p.tW + nx];
				if (q.x >= 0) {
					const int cx = q.x + (x - nx), cy = q.y + (y - ny);
					valid = src_ok(p, cx, cy) && !(bounded && bound_rejects<KIND, C>(p, x, y, cx, cy, bd));
					packed = cx | (cy << 16);
				}
			}
		}
		int mycand;
		int n = compact_candidates(valid, packed, best, m.list, mycand);
		evals += n;
		const float bd_before = bd;
		eval_candidates<KIND, C, P, V>(p, m.w, m.t, mycand, n, best, bd, partial, &ts, tw);
		if (bd < bd_before) improved++;
		// random search around the match after propagation: lane k draws
		// in window max_window >> k from its own stream, up to `shots`
		// draws, and proposes the first that lands in the source
		valid = false;
		if (lane < windows) {
			const int w = p.max_window >> lane;
			const int x_min = max(best.x - w, 0), y_min = max(best.y - w, 0);
			const int x_max = min(best.x + w + 1, p.sW), y_max = min(best.y + w + 1, p.sH);
			Rng rng(key, (uint32_t)pix, (uint32_t)sweep, (uint32_t)lane);
#pragma unroll 1
			for (int t = 0; t < p.shots; t++) {
				const int rx = x_min + rng.below(x_max - x_min);
				const int ry = y_min + rng.below(y_max - y_min);
				if (src_ok(p, rx, ry)) {
					valid = !(bounded && bound_rejects<KIND, C>(p, x, y, rx, ry, bd));
					packed = rx | (ry << 16);
					max_shot = max(max_shot, t);
					break;
				}
			}
		}
		n = compact_candidates(valid, packed, best, m.list, mycand);
		evals += n;
		eval_candidates<KIND, C, P, V>(p, m.w, m.t, mycand, n, best, bd, partial, &ts, tw);
		__syncwarp();
	} else {
		best = make_int2(-1, -1);
		bd = FLT_MAX;
	}
	if (lane == 0) {
		nnf_out[pix] = best;
		dist_out[pix] = bd;
	}
}

// metric_prop (may be NULL): this sweep's count of target points that the
// propagation step improved; metric_shots (may be NULL): the largest index
// of a first accepted random draw (patch_match.cpp:452-456, 481-485).
template <int KIND, int C, int P, int V>
__global__ void __launch_bounds__(pm_threads(V), 1) k_pm_sweep(DistArgs a, PmArgs p, int sweep, int jump,
                                                       const int2 *__restrict__ nnf_in, const float *__restrict__ dist_in,
                                                       int2 *__restrict__ nnf_out, float *__restrict__ dist_out,
                                                       unsigned long long *counter, unsigned long long *metric_prop,
                                                       int *metric_shots, const __grid_constant__ CUtensorMap tmap,
                                                       int *timeout)
{
	const int lane = threadIdx.x & 31;
	const PmSmem m = pm_smem<V>(a, p);
	TmaState ts = {&tmap, m.slots, m.slot_stride, m.bar, 0u, timeout};
	if (V == kPmStaged && lane == 0) mbar_init(m.bar, 1);
	float4 tw[(V == kPmRegs) ? P + 1 : 1];
	load_weights(a, m.w);
	const uint2 key = pm_key(p);
	unsigned evals = 0, partial = 0, improved = 0;
	int max_shot = -1;
	// number of random-search windows: max_window, max_window / 2, ..., 1
	const int windows = 32 - __clz(p.max_window);
	pm_for_each(p.nt, p.queue ? p.queue + 1 + sweep : nullptr, p.tile, [&](int wi) {
		pm_sweep_point<KIND, C, P, V>(p, m, ts, tw, key, windows, p.tlist[wi], sweep, jump, nnf_in, dist_in, nnf_out,
		                              dist_out, evals, partial, improved, max_shot);
	});
	if (lane == 0 && evals) {
		atomicAdd(counter, (unsigned long long)evals);
		if (partial) atomicAdd(counter + 1, (unsigned long long)partial);
	}
	if (metric_prop && lane == 0 && improved) atomicAdd(metric_prop, (unsigned long long)improved);
	if (metric_shots) {
		max_shot = __reduce_max_sync(kFull, max_shot);
		if (lane == 0 && max_shot >= 0) atomicMax(metric_shots, max_shot);
	}
}

// Also advances the context's PatchMatch call index when `calls` is set.
__global__ void k_fill_nnf(int2 *__restrict__ nnf, float *__restrict__ dist, int n, unsigned long long *calls)
{
	if (calls && blockIdx.x == 0 && threadIdx.x == 0) *calls += 1ull;
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
__host__ __device__ inline int jump_for(int sweep, int tW, int tH)
{
	int j = 16 >> (sweep % 4);
	while (j > 1 && 2 * j > max(tW, tH)) j /= 2;
	return j;
}

// Device buffers of the METRICS build's per-sweep figures (NULL: not kept).
struct PmMetrics {
	double *energy = nullptr;              // per sweep: sum of matched distances
	unsigned long long *prop = nullptr;    // per sweep: points improved by propagation
	int *shots = nullptr;                  // largest accepted draw index
	double *partials = nullptr;            // scratch of the energy reduction
	int partial_blocks = 0;
};

static void sweep_energy(cudaStream_t s, const PmArgs &p, const float *dist, const PmMetrics &m, int sweep);

// cuTensorMapEncodeTiled through the runtime's driver entry point (no
// link against the driver library); null when the driver does not have it.
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled()
{
	static const EncodeTiledFn fn = [] {
		void *f = nullptr;
		cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
		if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
		        cudaSuccess ||
		    q != cudaDriverEntryPointSuccess) {
			(void)cudaGetLastError();
			return static_cast<EncodeTiledFn>(nullptr);
		}
		return reinterpret_cast<EncodeTiledFn>(f);
	}();
	return fn;
}

// The padded source as a 2-D float tensor (4 * sWp floats by sH + 1 rows)
// with a box of one candidate window (4 * L floats by rows).  False when it
// cannot be encoded; the caller then reads the windows with plain loads.
static bool encode_source_map(const PmArgs &p, CUtensorMap *map)
{
	const EncodeTiledFn enc = encode_tiled();
	if (!enc) return false;
	if ((reinterpret_cast<uintptr_t>(p.src) & 15) != 0 || 4 * p.L > 256 || p.rows > 256) return false;
	const cuuint64_t dim[2] = {(cuuint64_t)4 * p.sWp, (cuuint64_t)p.sH + 1};
	const cuuint64_t stride[1] = {(cuuint64_t)p.sWp * sizeof(float4)};
	const cuuint32_t box[2] = {(cuuint32_t)(4 * p.L), (cuuint32_t)p.rows};
	const cuuint32_t estride[2] = {1, 1};
	return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float4 *>(p.src), dim, stride, box, estride,
	           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
	           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int KIND, int C, int P, int V>
static void launch_sweeps(nli_ctx *ctx, const DistArgs &a, const PmArgs &p, int iterations, const int2 *init,
                          int2 *nnf_x, float *dist_x, int2 *nnf_y, float *dist_y, unsigned long long *counter,
                          const PmMetrics &mt, const CUtensorMap &map, size_t smem)
{
	// persistent: one block per SM (fewer when there are fewer points)
	const int block = pm_threads(V);
	const int grid = (int)std::min<size_t>(((size_t)p.nt * 32 + block - 1) / block, (size_t)ctx->num_sms);
	int *timeout = &ctx->status->timeout;
	// The kernels' dynamic shared-memory limit is raised once per device, to
	// the largest opt-in size (each launch passes the size it uses): a
	// function attribute set on every call costs a driver call per PatchMatch
	// call on every batch worker thread.
	static std::atomic<uint32_t> raised{0};  // one bit per device
	const uint32_t bit = 1u << (ctx->device & 31);
	if (!(raised.load(std::memory_order_acquire) & bit)) {
		NLI_REQUIRE(smem <= (size_t)ctx->max_smem_optin, NLI_E_UNSUPPORTED, "PatchMatch shared memory too large");
		NLI_CUDA(cudaFuncSetAttribute(k_pm_init<KIND, C, P, V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                              ctx->max_smem_optin));
		NLI_CUDA(cudaFuncSetAttribute(k_pm_sweep<KIND, C, P, V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
		                              ctx->max_smem_optin));
		raised.fetch_or(bit, std::memory_order_release);
	}
	NLI_REQUIRE(smem <= (size_t)ctx->max_smem_optin, NLI_E_UNSUPPORTED, "PatchMatch shared memory too large");
	{
		ProfScope ps(ctx, "pm_init");
		k_pm_init<KIND, C, P, V><<<grid, block, smem, ctx->stream>>>(a, p, init, nnf_x, dist_x, counter, map,
		                                                                timeout);
		NLI_CHECK_LAUNCH();
	}
	for (int it = 0; it < iterations; it++) {
		const bool even = (it % 2) == 0;
		ProfScope ps(ctx, "pm_sweep");
		k_pm_sweep<KIND, C, P, V><<<grid, block, smem, ctx->stream>>>(
		    a, p, it, jump_for(it, p.tW, p.tH), even ? nnf_x : nnf_y, even ? dist_x : dist_y, even ? nnf_y : nnf_x,
		    even ? dist_y : dist_x, counter, mt.prop ? mt.prop + it : nullptr, mt.shots, map, timeout);
		NLI_CHECK_LAUNCH();
		if (mt.energy) sweep_energy(ctx->stream, p, even ? dist_y : dist_x, mt, it);
	}
}

// Fixed-size patches take the context's variant; the staged one only when
// the tensor map encodes and its layout fits, else (and for runtime-sized
// patches) kPmShared.
template <int KIND, int C, int P>
static void run_sweeps(nli_ctx *ctx, const DistArgs &a, const PmArgs &p, int iterations, const int2 *init,
                       int2 *nnf_x, float *dist_x, int2 *nnf_y, float *dist_y, unsigned long long *counter,
                       const PmMetrics &mt)
{
	const int taps = a.px * a.py;
	CUtensorMap map;
	std::memset(&map, 0, sizeof(map));
	if constexpr (P > 0) {
		if (ctx->tune_pm_variant == kPmStaged) {
			const size_t smem = pm_smem_bytes_tma(taps, p.rows, p.L, p.K, pm_threads(kPmStaged) / 32);
			if (smem <= (size_t)ctx->max_smem_optin && encode_source_map(p, &map)) {
				launch_sweeps<KIND, C, P, kPmStaged>(ctx, a, p, iterations, init, nnf_x, dist_x, nnf_y, dist_y,
				                                     counter, mt, map, smem);
				return;
			}
		} else if (ctx->tune_pm_variant == kPmRegs) {
			launch_sweeps<KIND, C, P, kPmRegs>(ctx, a, p, iterations, init, nnf_x, dist_x, nnf_y, dist_y, counter,
			                                   mt, map, pm_smem_bytes(taps, p.rows, p.L, pm_threads(kPmRegs) / 32));
			return;
		}
	}
	launch_sweeps<KIND, C, P, kPmShared>(ctx, a, p, iterations, init, nnf_x, dist_x, nnf_y, dist_y, counter, mt, map,
	                                     pm_smem_bytes(taps, p.rows, p.L, pm_threads(kPmShared) / 32));
}

static void sweep_energy(cudaStream_t s, const PmArgs &p, const float *dist, const PmMetrics &m, int sweep)
{
	k_energy<<<m.partial_blocks, 256, 0, s>>>(p.tlist, p.nt, dist, m.partials);
	NLI_CHECK_LAUNCH();
	launch_sum_partials(s, m.partials, m.partial_blocks, m.energy + sweep);
}

// ====================================================== batched launches
// PatchMatch calls of up to kBatchMax images in one launch per kernel (the
// lockstep batch driver, lockstep.cu).  Every image is both source and
// target (as in the inpainting driver), with its own sizes, masks, target
// list, seed and call index; the distance, patch and PatchMatch parameters
// are shared.  Per target point the work is exactly that of the one-image
// kernels (the same device functions, Philox streams keyed by the image's
// own seed and call index), so each image's field equals its one-image
// call's bit for bit.
//
// The per-image arguments travel in the kernel's parameter space (a
// __grid_constant__ table read through the constant cache, not the L1 data
// pipe that bounds the sweep).  The persistent kernels see the concatenated
// target lists of the images still iterating (their `active` flag, written
// on the device between iterations) as one work list, distributed as the
// one-image kernels distribute theirs (pm_for_each: static block ranges or
// the device work queue).
struct PmBatchTask {
	PmArgs p;
	int flag;            // index of the image's active flag
	unsigned long long *counter;  // the image's candidate counters (2)
	const float *img;    // the image (source = target), HWC float
	const int2 *init;    // initial field or null
	int2 *nnf_x, *nnf_y;  // result (x) and the sweeps' second buffer
	float *dist_x, *dist_y;
};

struct PmBatchArgs {
	int n;
	const int *active;  // per image: still iterating (null: all)
	unsigned *queue;    // device work queue as PmArgs::queue (null: static ranges)
	int tile;
	PmBatchTask t[kBatchMax];
};

__device__ __forceinline__ bool batch_on(const int *active, int t) { return !active || active[t] != 0; }

// Exclusive prefix of the active images' target counts in s_pre[0..n]
// (s_pre[n] is the total); the whole block calls it.
__device__ __forceinline__ int pm_batch_prefix(const PmBatchArgs &B, int *s_pre)
{
	if (threadIdx.x < 32) {
		const int lane = threadIdx.x;
		const int t0 = 2 * lane, t1 = t0 + 1;
		const int v0 = (t0 < B.n && batch_on(B.active, B.t[t0].flag)) ? B.t[t0].p.nt : 0;
		const int v1 = (t1 < B.n && batch_on(B.active, B.t[t1].flag)) ? B.t[t1].p.nt : 0;
		int incl = v0 + v1;
#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			const int u = __shfl_up_sync(kFull, incl, o);
			if (lane >= o) incl += u;
		}
		const int excl = incl - v0 - v1;
		if (lane == 0) s_pre[0] = 0;
		s_pre[t0 + 1] = excl + v0;
		s_pre[t1 + 1] = excl + v0 + v1;
	}
	__syncthreads();
	return s_pre[B.n];
}

// Adds a warp's candidate counts to its image's counters and the launch's
// total, and clears them.
__device__ __forceinline__ void pm_batch_count(unsigned long long *image, unsigned long long *total, unsigned &evals,
                                               unsigned &partial)
{
	if ((threadIdx.x & 31) == 0 && evals) {
		atomicAdd(total, (unsigned long long)evals);
		if (partial) atomicAdd(total + 1, (unsigned long long)partial);
		if (image) {
			atomicAdd(image, (unsigned long long)evals);
			if (partial) atomicAdd(image + 1, (unsigned long long)partial);
		}
	}
	evals = partial = 0;
}

// The padded float4 pixels of every active image (k_pad4 per image); the
// largest-value word of its patch means is cleared.
__global__ void k_pad4_batch(const __grid_constant__ PmBatchArgs B, int C)
{
	const int t = blockIdx.y;
	const PmBatchTask &T = B.t[t];
	if (!batch_on(B.active, T.flag)) return;
	if (T.p.vmax && blockIdx.x == 0 && threadIdx.x == 0) *const_cast<unsigned *>(T.p.vmax) = 0u;
	pad4_span(T.img, T.p.sW, T.p.sH, C, const_cast<float4 *>(T.p.src), blockIdx.x * blockDim.x + threadIdx.x,
	          gridDim.x * blockDim.x);
}

// The patch means of every active image (k_pm_moments per image).
__global__ void k_pm_moments_batch(DistArgs a, const __grid_constant__ PmBatchArgs B)
{
	const int t = blockIdx.y;
	const PmBatchTask &T = B.t[t];
	if (!batch_on(B.active, T.flag) || !T.p.smom) return;
	moments_span(a, T.p.src, T.p.sW, T.p.sH, const_cast<float4 *>(T.p.smom), const_cast<unsigned *>(T.p.vmax),
	             blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, T.p.dev != 0);
}

// k_fill_nnf per active image: the result field to "none", and the image's
// call index advanced when it has target points.
__global__ void k_fill_nnf_batch(const __grid_constant__ PmBatchArgs B)
{
	const int t = blockIdx.y;
	const PmBatchTask &T = B.t[t];
	if (!batch_on(B.active, T.flag)) return;
	if (T.p.nt > 0 && blockIdx.x == 0 && threadIdx.x == 0) *const_cast<unsigned long long *>(T.p.calls) += 1ull;
	const int n = T.p.tW * T.p.tH;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		T.nnf_x[i] = make_int2(-1, -1);
}

template <int KIND, int C, int P>
__global__ void __launch_bounds__(pm_threads(kPmShared), 1)
    k_pm_init_batch(DistArgs a, const __grid_constant__ PmBatchArgs B, unsigned long long *counter)
{
	__shared__ int s_pre[kBatchMax + 1];
	const int lane = threadIdx.x & 31;
	const PmSmem m = pm_smem<kPmShared>(a, B.t[0].p);
	TmaState ts = {nullptr, nullptr, 0, nullptr, 0u, nullptr};
	float4 tw[1];
	load_weights(a, m.w);
	const int total = pm_batch_prefix(B, s_pre);
	unsigned evals = 0, partial = 0;
	int t = 0, tk = -1;
	uint2 key = make_uint2(0u, 0u);
	// a warp's items increase, so its image index only moves forward
	pm_for_each(total, B.queue, B.tile, [&](int wi) {
		while (wi >= s_pre[t + 1]) t++;
		const PmBatchTask &T = B.t[t];
		if (t != tk) {
			if (tk >= 0) pm_batch_count(B.t[tk].counter, counter, evals, partial);
			key = pm_key(T.p);
			tk = t;
		}
		pm_init_point<KIND, C, P, kPmShared>(T.p, m, ts, tw, key, T.p.tlist[wi - s_pre[t]], T.init, T.nnf_x,
		                                     T.dist_x, evals, partial);
	});
	if (tk >= 0) pm_batch_count(B.t[tk].counter, counter, evals, partial);
}

template <int KIND, int C, int P>
__global__ void __launch_bounds__(pm_threads(kPmShared), 1)
    k_pm_sweep_batch(DistArgs a, const __grid_constant__ PmBatchArgs B, int sweep, unsigned long long *counter)
{
	__shared__ int s_pre[kBatchMax + 1];
	const int lane = threadIdx.x & 31;
	const PmSmem m = pm_smem<kPmShared>(a, B.t[0].p);
	TmaState ts = {nullptr, nullptr, 0, nullptr, 0u, nullptr};
	float4 tw[1];
	load_weights(a, m.w);
	const int total = pm_batch_prefix(B, s_pre);
	unsigned evals = 0, partial = 0, improved = 0;
	int max_shot = -1;
	const bool even = (sweep % 2) == 0;
	int t = 0, tk = -1, windows = 0, jump = 1;
	uint2 key = make_uint2(0u, 0u);
	pm_for_each(total, B.queue ? B.queue + 1 + sweep : nullptr, B.tile, [&](int wi) {
		while (wi >= s_pre[t + 1]) t++;
		const PmBatchTask &T = B.t[t];
		if (t != tk) {
			if (tk >= 0) pm_batch_count(B.t[tk].counter, counter, evals, partial);
			key = pm_key(T.p);
			windows = 32 - __clz(T.p.max_window);
			jump = jump_for(sweep, T.p.tW, T.p.tH);
			tk = t;
		}
		pm_sweep_point<KIND, C, P, kPmShared>(T.p, m, ts, tw, key, windows, T.p.tlist[wi - s_pre[t]], sweep, jump,
		                                      even ? T.nnf_x : T.nnf_y, even ? T.dist_x : T.dist_y,
		                                      even ? T.nnf_y : T.nnf_x, even ? T.dist_y : T.dist_x, evals, partial,
		                                      improved, max_shot);
	});
	if (tk >= 0) pm_batch_count(B.t[tk].counter, counter, evals, partial);
}

// After an odd number of sweeps the field is in the second buffer: copy
// the target points back (k_copy_targets per active image).
__global__ void k_copy_targets_batch(const __grid_constant__ PmBatchArgs B)
{
	const int t = blockIdx.y;
	const PmBatchTask &T = B.t[t];
	if (!batch_on(B.active, T.flag)) return;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < T.p.nt; i += gridDim.x * blockDim.x) {
		const int pix = T.p.tlist[i];
		T.nnf_x[pix] = T.nnf_y[pix];
	}
}

template <int KIND, int C, int P>
static void run_batch_kernels(nli_ctx *ctx, const DistArgs &a, const PmBatchArgs &B, int iterations, size_t smem,
                              unsigned long long *counter)
{
	// dynamic shared memory up to the opt-in limit less the kernels' static
	// shared memory (the work-list prefix), raised once per device
	static std::atomic<uint32_t> raised{0};  // one bit per device
	// written by whichever thread raises the limit first (concurrent
	// sub-groups may race to it with the same value)
	static std::atomic<int> dyn_max[32];
	const uint32_t bit = 1u << (ctx->device & 31);
	if (!(raised.load(std::memory_order_acquire) & bit)) {
		cudaFuncAttributes fa_init, fa_sweep;
		NLI_CUDA(cudaFuncGetAttributes(&fa_init, k_pm_init_batch<KIND, C, P>));
		NLI_CUDA(cudaFuncGetAttributes(&fa_sweep, k_pm_sweep_batch<KIND, C, P>));
		const int dmax = ctx->max_smem_optin - (int)std::max(fa_init.sharedSizeBytes, fa_sweep.sharedSizeBytes);
		NLI_CUDA(cudaFuncSetAttribute(k_pm_init_batch<KIND, C, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, dmax));
		NLI_CUDA(cudaFuncSetAttribute(k_pm_sweep_batch<KIND, C, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, dmax));
		dyn_max[ctx->device & 31].store(dmax, std::memory_order_relaxed);
		raised.fetch_or(bit, std::memory_order_release);
	}
	NLI_REQUIRE(smem <= (size_t)dyn_max[ctx->device & 31].load(std::memory_order_relaxed), NLI_E_UNSUPPORTED,
	            "PatchMatch shared memory too large");
	const int block = pm_threads(kPmShared);
	const int grid = ctx->num_sms;
	{
		ProfScope ps(ctx, "pm_init");
		k_pm_init_batch<KIND, C, P><<<grid, block, smem, ctx->stream>>>(a, B, counter);
		NLI_CHECK_LAUNCH();
	}
	for (int it = 0; it < iterations; it++) {
		ProfScope ps(ctx, "pm_sweep");
		k_pm_sweep_batch<KIND, C, P><<<grid, block, smem, ctx->stream>>>(a, B, it, counter);
		NLI_CHECK_LAUNCH();
	}
}

void patchmatch_batch_run(nli_ctx *ctx, const nli_distance_params &dp, const nli_patchmatch_params &pm, int C, int n,
                          const PmBatchItem *items, const int *active)
{
	NLI_REQUIRE(n >= 1 && n <= kBatchMax, NLI_E_INVALID, "batched PatchMatch takes 1 to 64 images");
	DistArgs a;
	fill_dist_args(a, dp, C);
	const bool grad = dp.kind == NLI_DIST_L2_COMBINED || dp.kind == NLI_DIST_L2_RGBD;
	PmBatchArgs B;
	std::memset(&B, 0, sizeof(B));
	B.n = n;
	B.active = active;
	B.tile = ctx->tune_pm_tile;
	int maxpix = 0, maxpad = 0, maxnt = 0;
	for (int i = 0; i < n; i++) {
		const PmBatchItem &it = items[i];
		NLI_REQUIRE(it.W < 32768 && it.H < 32768, NLI_E_UNSUPPORTED, "PatchMatch source sides must be below 32768");
		PmBatchTask &T = B.t[i];
		PmArgs &p = T.p;
		p.src = p.tgt = it.pad;
		p.sWp = p.tWp = it.W + 1;
		p.smask = it.smask;
		p.tmask = it.tmask;
		p.tlist = it.tlist;
		p.sW = p.tW = it.W;
		p.sH = p.tH = it.H;
		p.nt = it.nt;
		p.shots = pm.random_shots;
		p.max_window = (pm.window != -1) ? pm.window : max(it.W, it.H);
		p.rx = a.rx;
		p.ry = a.ry;
		p.ex = a.px - a.rx;
		p.ey = a.py - a.ry;
		p.L = a.px + (grad ? 1 : 0);
		p.K = 32 / p.L;
		p.rows = a.py + (grad ? 1 : 0);
		p.lambda = a.lambda;
		p.lambda_d = a.lambda_d;
		p.seed = it.seed;
		p.calls = it.calls;
		p.smom = p.tmom = it.mom;
		p.vmax = it.mom ? it.vmax : nullptr;
		// the item's table holds room for the deviations (4 tables)
		p.dev = (it.mom && ctx->tune_pm_bound == 2 && dp.kind != NLI_DIST_L1_NORM) ? 1 : 0;
		p.queue = nullptr;  // the launch's queue is B.queue
		p.tile = 0;
		T.flag = it.flag;
		T.counter = it.counter;
		T.img = it.img;
		T.init = reinterpret_cast<const int2 *>(it.init);
		T.nnf_x = reinterpret_cast<int2 *>(it.out);
		T.nnf_y = reinterpret_cast<int2 *>(it.nnf_y);
		T.dist_x = it.dist_x;
		T.dist_y = it.dist_y;
		maxpix = max(maxpix, it.W * it.H);
		maxpad = max(maxpad, (it.W + 1) * (it.H + 1));
		maxnt = max(maxnt, it.nt);
	}
	cudaStream_t s = ctx->stream;
	const int per = 256;
	k_pad4_batch<<<dim3((unsigned)std::min((maxpad + per - 1) / per, 1024), (unsigned)n), per, 0, s>>>(B, C);
	NLI_CHECK_LAUNCH();
	k_fill_nnf_batch<<<dim3((unsigned)std::min((maxpix + per - 1) / per, 1024), (unsigned)n), per, 0, s>>>(B);
	NLI_CHECK_LAUNCH();
	if (B.t[0].p.smom) {
		k_pm_moments_batch<<<dim3((unsigned)std::min((maxpad + per - 1) / per, 1024), (unsigned)n), per, 0, s>>>(a,
		                                                                                                       B);
		NLI_CHECK_LAUNCH();
	}
	if (maxnt == 0) return;
	unsigned long long *counter = ctx->buf<unsigned long long>("pm.counter", 2);
	if (B.tile > 0) {
		const int slots = std::max(pm.iterations, 0) + 1;
		B.queue = ctx->buf<unsigned>("pm.queue", slots);
		NLI_CUDA(cudaMemsetAsync(B.queue, 0, sizeof(unsigned) * slots, s));
	}
	const int taps = a.px * a.py;
	const size_t smem = pm_smem_bytes(taps, B.t[0].p.rows, B.t[0].p.L, pm_threads(kPmShared) / 32);
	NLI_REQUIRE(smem <= (size_t)ctx->max_smem_optin, NLI_E_UNSUPPORTED, "PatchMatch shared memory too large");
	const bool p9 = a.px == 9 && a.py == 9;
	bool handled = false;
#define NLI_PMB_CASE(KIND, CC)                                                                  \
	if (dp.kind == KIND && C == CC) {                                                           \
		if (p9)                                                                                 \
			run_batch_kernels<KIND, CC, 9>(ctx, a, B, pm.iterations, smem, counter);          \
		else                                                                                    \
			run_batch_kernels<KIND, CC, 0>(ctx, a, B, pm.iterations, smem, counter);          \
		handled = true;                                                                         \
	}
	NLI_PMB_CASE(NLI_DIST_L2_COMBINED, 3)
	NLI_PMB_CASE(NLI_DIST_L2_COMBINED, 1)
	NLI_PMB_CASE(NLI_DIST_L2_COMBINED, 2)
	NLI_PMB_CASE(NLI_DIST_L2_COMBINED, 4)
	NLI_PMB_CASE(NLI_DIST_L2_RGBD, 4)
	NLI_PMB_CASE(NLI_DIST_L2_NORM, 3)
	NLI_PMB_CASE(NLI_DIST_L2_NORM, 1)
	NLI_PMB_CASE(NLI_DIST_L2_NORM, 2)
	NLI_PMB_CASE(NLI_DIST_L2_NORM, 4)
	NLI_PMB_CASE(NLI_DIST_L1_NORM, 3)
	NLI_PMB_CASE(NLI_DIST_L1_NORM, 1)
	NLI_PMB_CASE(NLI_DIST_L1_NORM, 2)
	NLI_PMB_CASE(NLI_DIST_L1_NORM, 4)
#undef NLI_PMB_CASE
	NLI_REQUIRE(handled, NLI_E_UNSUPPORTED, "no PatchMatch kernel for this distance / channel count");
	if (pm.iterations % 2 == 1) {
		k_copy_targets_batch<<<dim3((unsigned)std::min((maxnt + per - 1) / per, 1024), (unsigned)n), per, 0, s>>>(B);
		NLI_CHECK_LAUNCH();
	}
}

NLI_CHECK_READER(check_word_patchmatch)

void patchmatch_run(nli_ctx *ctx, const nli_distance_params &dp, const nli_patchmatch_params &pm, const float *src,
                    const uint8_t *smask, int sW, int sH, const float *tgt, const uint8_t *tmask, int tW, int tH,
                    int C, const int32_t *init_nnf, int32_t *out_nnf, float *out_dist, double *energy,
                    const int32_t *tlist, int n_target, PatchMatchMetricsHost *metrics)
{
	DistArgs a;
	fill_dist_args(a, dp, C);
	NLI_REQUIRE(sW < 32768 && sH < 32768, NLI_E_UNSUPPORTED, "PatchMatch source sides must be below 32768");
	cudaStream_t s = ctx->stream;
	const int nT = tW * tH;

	// padded float4 pixels of source and target
	float4 *s4 = ctx->buf<float4>("pm.src4", (size_t)(sW + 1) * (sH + 1));
	launch_pad4(s, src, sW, sH, C, s4);
	float4 *t4 = s4;
	if (!(tgt == src && tW == sW && tH == sH)) {
		t4 = ctx->buf<float4>("pm.tgt4", (size_t)(tW + 1) * (tH + 1));
		launch_pad4(s, tgt, tW, tH, C, t4);
	}

	// patch means for the lower bound (NLI_TUNE_PM_BOUND)
	float4 *smom = nullptr, *tmom = nullptr;
	unsigned *vmax = nullptr;
	// the deviation tables serve the L2 kinds (NLI_TUNE_PM_BOUND 2)
	const int dev = (ctx->tune_pm_bound == 2 && dp.kind != NLI_DIST_L1_NORM) ? 1 : 0;
	if (ctx->tune_pm_bound) {
		DistArgs da;
		fill_dist_args(da, dp, C);
		vmax = ctx->buf<unsigned>("pm.vmax", 1);
		NLI_CUDA(cudaMemsetAsync(vmax, 0, sizeof(unsigned), s));
		const int ns = (sW + 1) * (sH + 1);
		smom = ctx->buf<float4>("pm.smom", (size_t)ns * (dev ? 4 : 1));
		k_pm_moments<<<(ns + 255) / 256, 256, 0, s>>>(da, s4, sW, sH, smom, vmax, dev);
		NLI_CHECK_LAUNCH();
		tmom = smom;
		if (t4 != s4) {
			const int nt4 = (tW + 1) * (tH + 1);
			tmom = ctx->buf<float4>("pm.tmom", (size_t)nt4 * (dev ? 4 : 1));
			k_pm_moments<<<(nt4 + 255) / 256, 256, 0, s>>>(da, t4, tW, tH, tmom, vmax, dev);
			NLI_CHECK_LAUNCH();
		}
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
	// the call index advances only for calls with target points, as the
	// random streams are drawn only then
	k_fill_nnf<<<(nT + 255) / 256, 256, 0, s>>>(nnf_x, out_dist, nT, n_target > 0 ? &ctx->status->pm_calls : nullptr);
	NLI_CHECK_LAUNCH();
	if (n_target > 0) {
		PmArgs p;
		p.src = s4;
		p.tgt = t4;
		p.sWp = sW + 1;
		p.tWp = tW + 1;
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
		const bool grad = dp.kind == NLI_DIST_L2_COMBINED || dp.kind == NLI_DIST_L2_RGBD;
		p.L = a.px + (grad ? 1 : 0);
		p.K = 32 / p.L;
		p.rows = a.py + (grad ? 1 : 0);
		p.lambda = a.lambda;
		p.lambda_d = a.lambda_d;
		p.seed = ctx->seed;
		p.calls = &ctx->status->pm_calls;  // advanced by k_fill_nnf above
		p.smom = smom;
		p.tmom = tmom;
		p.vmax = vmax;
		p.dev = smom ? dev : 0;
		p.queue = nullptr;
		p.tile = ctx->tune_pm_tile;
		if (p.tile > 0) {
			const int slots = std::max(pm.iterations, 0) + 1;
			p.queue = ctx->buf<unsigned>("pm.queue", slots);
			NLI_CUDA(cudaMemsetAsync(p.queue, 0, sizeof(unsigned) * slots, s));
		}
		if (energy) NLI_CUDA(cudaMemsetAsync(counter, 0, 2 * sizeof(unsigned long long), s));
		PmMetrics mt;
		const int iters = std::max(pm.iterations, 0);
		if (metrics && iters > 0) {
			mt.energy = ctx->buf<double>("pm.m_energy", iters);
			mt.prop = ctx->buf<unsigned long long>("pm.m_prop", iters);
			mt.shots = ctx->buf<int>("pm.m_shots", 1);
			mt.partial_blocks = std::min((n_target + 255) / 256, 1024);
			mt.partials = ctx->buf<double>("pm.m_partials", mt.partial_blocks + 1);
			NLI_CUDA(cudaMemsetAsync(mt.prop, 0, sizeof(unsigned long long) * iters, s));
			NLI_CUDA(cudaMemsetAsync(mt.shots, 0, sizeof(int), s));
		}
		// 9 x 9 patches (the reference's default) have their rows unrolled
		const bool p9 = a.px == 9 && a.py == 9;
#define NLI_PM_CASE(KIND, CC)                                                                                \
	if (dp.kind == KIND && C == CC) {                                                                            \
		if (p9)                                                                                                  \
			run_sweeps<KIND, CC, 9>(ctx, a, p, pm.iterations, init, nnf_x, dist_x, nnf_y, dist_y, counter, mt); \
		else                                                                                                     \
			run_sweeps<KIND, CC, 0>(ctx, a, p, pm.iterations, init, nnf_x, dist_x, nnf_y, dist_y, counter, mt); \
		handled = true;                                                                                          \
	}
		bool handled = false;
		NLI_PM_CASE(NLI_DIST_L2_COMBINED, 3)
		NLI_PM_CASE(NLI_DIST_L2_COMBINED, 1)
		NLI_PM_CASE(NLI_DIST_L2_COMBINED, 2)
		NLI_PM_CASE(NLI_DIST_L2_COMBINED, 4)
		NLI_PM_CASE(NLI_DIST_L2_RGBD, 4)
		NLI_PM_CASE(NLI_DIST_L2_NORM, 3)
		NLI_PM_CASE(NLI_DIST_L2_NORM, 1)
		NLI_PM_CASE(NLI_DIST_L2_NORM, 2)
		NLI_PM_CASE(NLI_DIST_L2_NORM, 4)
		NLI_PM_CASE(NLI_DIST_L1_NORM, 3)
		NLI_PM_CASE(NLI_DIST_L1_NORM, 1)
		NLI_PM_CASE(NLI_DIST_L1_NORM, 2)
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
			NLI_CUDA(cudaMemcpyAsync(hc + 3, &ctx->status->timeout, sizeof(int), cudaMemcpyDeviceToHost, s));
			NLI_CUDA(cudaStreamSynchronize(s));
			if (*reinterpret_cast<const int *>(hc + 3) != 0) {
				clear_timeout(ctx);
				NLI_REQUIRE(false, NLI_E_TIMEOUT, "PatchMatch window copies timed out");
			}
			ctx->candidates += (int64_t)hc[0];
			ctx->candidates_partial += (int64_t)hc[1];
			*energy = *reinterpret_cast<double *>(hc + 2);
		}
		if (metrics && iters > 0) {
			metrics->total_distance.resize(iters);
			std::vector<unsigned long long> prop(iters);
			NLI_CUDA(cudaMemcpyAsync(metrics->total_distance.data(), mt.energy, sizeof(double) * iters,
			                         cudaMemcpyDeviceToHost, s));
			NLI_CUDA(cudaMemcpyAsync(prop.data(), mt.prop, sizeof(unsigned long long) * iters, cudaMemcpyDeviceToHost,
			                         s));
			NLI_CUDA(cudaMemcpyAsync(&metrics->max_random_shots, mt.shots, sizeof(int), cudaMemcpyDeviceToHost, s));
			NLI_CUDA(cudaStreamSynchronize(s));
			metrics->propagations.assign(prop.begin(), prop.end());
		}
	} else if (energy) {
		*energy = 0.0;
	}
}

// Device counter of evaluated candidates of the last PatchMatch calls
// (read by the multiscale driver for its statistics).
unsigned long long *pm_counter(nli_ctx *ctx) { return ctx->buf<unsigned long long>("pm.counter", 1); }

}  // namespace nli
