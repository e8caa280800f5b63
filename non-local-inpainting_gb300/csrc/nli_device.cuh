// Device-side helpers: reference-exact arithmetic, the counter-based RNG,
// the patch distances, reductions and a bounded grid barrier.
#pragma once

#include <cfloat>
#include <cstdint>

#include "nli_internal.cuh"

namespace nli {

// ------------------------------------------------------------------------
// Checked builds (NLI_CHECKED).  Data-dependent gathered indices (PatchMatch
// candidate windows, NNF-shifted pixels, hole lists, CG neighbour codes) go
// through nli_in_bounds: in a checked build an index outside [0, n) is
// recorded -- the first one per translation unit, as (site << 32) | index --
// and the access is skipped; otherwise the test compiles away.  The record
// is read and cleared by nli_debug_check_status.
enum CheckSite : unsigned {
	kSitePmSource = 1,    // PatchMatch: source window row of a candidate
	kSitePmMask = 2,      // PatchMatch: source mask at a candidate
	kSitePmField = 3,     // PatchMatch: a neighbour's match / the initial field
	kSitePmTarget = 4,    // PatchMatch: target list entry
	kSiteMeansSource = 10,  // NL-means / NL-medians: NNF-shifted source pixel
	kSiteHole = 11,         // hole list entry
	kSiteCoefSource = 12,   // NL-Poisson coefficient gather: NNF-shifted pixel
	kSiteCgNeighbour = 13,  // CG: neighbour code (owning CTA, index)
	kSiteScaleNnf = 20,     // scale transition: scaled field position
};

#ifdef NLI_CHECKED
static __device__ unsigned long long g_nli_check_word;

__device__ __forceinline__ bool nli_in_bounds(long long i, long long n, unsigned site)
{
	if (i >= 0 && i < n) return true;
	atomicCAS(&g_nli_check_word, 0ull, ((unsigned long long)site << 32) | (unsigned long long)(unsigned)i);
	return false;
}

// Host reader of this translation unit's record (read and cleared).
#define NLI_CHECK_READER(fn)                                                           \
	unsigned long long fn()                                                            \
	{                                                                                  \
		unsigned long long v = 0, z = 0;                                               \
		NLI_CUDA(cudaMemcpyFromSymbol(&v, g_nli_check_word, sizeof(v)));              \
		NLI_CUDA(cudaMemcpyToSymbol(g_nli_check_word, &z, sizeof(z)));                \
		return v;                                                                      \
	}
#else
__device__ __forceinline__ bool nli_in_bounds(long long, long long, unsigned) { return true; }

#define NLI_CHECK_READER(fn) \
	unsigned long long fn() { return 0; }
#endif

// ------------------------------------------------------------------------
// Reference-exact arithmetic.  The reference is compiled for the host with
// separate IEEE roundings for every product and sum (no fused multiply-add);
// these wrappers keep the CUDA compiler from contracting them.
__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }

// ------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC 2011): 10 rounds of two 32x32->64 multiplies with the
// published multipliers and Weyl key increments.
__device__ __forceinline__ uint4 philox(uint4 c, uint2 k)
{
#pragma unroll
	for (int i = 0; i < 10; i++) {
		uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
		uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
		c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
		k.x += 0x9E3779B9u;
		k.y += 0xBB67AE85u;
	}
	return c;
}

// A stream of 32-bit draws for one (pixel, sweep, stream) triple: four
// draws per Philox block, counter = (pixel, sweep, block index, tag ^
// stream << 16).
struct Rng {
	uint2 key;
	uint32_t pixel, sweep, block, tag;
	uint4 cur;
	int used;
	__device__ Rng(uint2 k, uint32_t p, uint32_t s, uint32_t stream = 0)
	    : key(k), pixel(p), sweep(s), block(0), tag(0x6e6c6900u ^ (stream << 16)), used(4)
	{
	}
	__device__ __forceinline__ uint32_t next()
	{
		if (used == 4) {
			cur = philox(make_uint4(pixel, sweep, block++, tag), key);
			used = 0;
		}
		uint32_t r = (used == 0) ? cur.x : (used == 1) ? cur.y : (used == 2) ? cur.z : cur.w;
		used++;
		return r;
	}
	// draw in [0, n), n >= 1, by the multiply-high range reduction of
	// D. Lemire, "Fast random integer generation in an interval" (2019)
	// (the reference draws rand() % n)
	__device__ __forceinline__ int below(int n) { return (int)__umulhi(next(), (uint32_t)n); }
};

// ------------------------------------------------------------------------
// Patch distances, reference-exact variant.  Reads the image and its
// gradient in the reference layouts (HWC and 2C-interleaved) and follows
// l2_combined_patch_distance.cpp:39-148, l2_rgbd_patch_distance.cpp:41-117,
// l2_norm_patch_distance.cpp:22-104 and l1_norm_patch_distance.cpp:22-105:
// float per-tap norms, float weight*norm products, double sums for the
// L2Combined/L2RGBD kinds, float sums for L2Norm/L1Norm.
__device__ inline float dist_exact(const DistArgs &a, const float *__restrict__ S,
                                   const float *__restrict__ GS, int sW, const float *__restrict__ T,
                                   const float *__restrict__ GT, int tW, int sx, int sy, int tx, int ty)
{
	const int C = a.C;
	const float *pw = a.weights;
	if (a.kind == NLI_DIST_L2_COMBINED || a.kind == NLI_DIST_L2_RGBD) {
		double D = 0.0, G = 0.0, Dd = 0.0, Gd = 0.0;
		for (int dy = -a.ry; dy < a.py - a.ry; dy++)
			for (int dx = -a.rx; dx < a.px - a.rx; dx++, ++pw) {
				const float w = *pw;
				const int si = C * (sW * (sy + dy) + (sx + dx));
				const int ti = C * (tW * (ty + dy) + (tx + dx));
				if (a.kind == NLI_DIST_L2_COMBINED && (C == 3 || C == 1)) {
					float norm, gnorm;
					if (C == 3) {
						float d0 = fs(S[si], T[ti]), d1 = fs(S[si + 1], T[ti + 1]), d2 = fs(S[si + 2], T[ti + 2]);
						norm = fa(fa(fm(d0, d0), fm(d1, d1)), fm(d2, d2));
						float e0 = fs(GS[2 * si], GT[2 * ti]), e1 = fs(GS[2 * si + 1], GT[2 * ti + 1]);
						float e2 = fs(GS[2 * si + 2], GT[2 * ti + 2]), e3 = fs(GS[2 * si + 3], GT[2 * ti + 3]);
						float e4 = fs(GS[2 * si + 4], GT[2 * ti + 4]), e5 = fs(GS[2 * si + 5], GT[2 * ti + 5]);
						gnorm = fa(fa(fa(fa(fa(fm(e0, e0), fm(e1, e1)), fm(e2, e2)), fm(e3, e3)), fm(e4, e4)),
						           fm(e5, e5));
					} else {
						float d0 = fs(S[si], T[ti]);
						norm = fm(d0, d0);
						float e0 = fs(GS[2 * si], GT[2 * ti]), e1 = fs(GS[2 * si + 1], GT[2 * ti + 1]);
						gnorm = fa(fm(e0, e0), fm(e1, e1));
					}
					D = da(D, (double)fm(w, norm));
					G = da(G, (double)fm(w, gnorm));
				} else {
					double n = 0.0, g = 0.0, nd = 0.0, gd = 0.0;
					for (int c = 0; c < C; c++) {
						float d = fs(S[si + c], T[ti + c]);
						float ex = fs(GS[2 * (si + c)], GT[2 * (ti + c)]);
						float ey = fs(GS[2 * (si + c) + 1], GT[2 * (ti + c) + 1]);
						float gg = fa(fm(ex, ex), fm(ey, ey));
						if (a.kind == NLI_DIST_L2_RGBD && c == 3) {
							nd = da(nd, (double)fm(d, d));
							gd = da(gd, (double)gg);
						} else {
							n = da(n, (double)fm(d, d));
							g = da(g, (double)gg);
						}
					}
					D = da(D, dm((double)w, n));
					G = da(G, dm((double)w, g));
					Dd = da(Dd, dm((double)w, nd));
					Gd = da(Gd, dm((double)w, gd));
				}
			}
		const double P = (double)((unsigned)a.px * (unsigned)a.py);
		double r = da(dm((double)a.lambda, D), dm((double)fs(1.0f, a.lambda), G));
		if (a.kind == NLI_DIST_L2_RGBD)
			r = da(da(r, dm((double)a.lambda_d, Dd)), dm((double)fs(1.0f, a.lambda_d), Gd));
		return __double2float_rn(__ddiv_rn(r, P));
	}
	// L2Norm / L1Norm: float accumulator
	float D = 0.0f;
	for (int dy = -a.ry; dy < a.py - a.ry; dy++)
		for (int dx = -a.rx; dx < a.px - a.rx; dx++, ++pw) {
			const float w = *pw;
			const int si = C * (sW * (sy + dy) + (sx + dx));
			const int ti = C * (tW * (ty + dy) + (tx + dx));
			float norm;
			if (a.kind == NLI_DIST_L2_NORM) {
				if (C == 3) {
					float d0 = fs(S[si], T[ti]), d1 = fs(S[si + 1], T[ti + 1]), d2 = fs(S[si + 2], T[ti + 2]);
					norm = fa(fa(fm(d0, d0), fm(d1, d1)), fm(d2, d2));
				} else if (C == 1) {
					float d0 = fs(S[si], T[ti]);
					norm = fm(d0, d0);
				} else {
					norm = 0.0f;
					for (int c = 0; c < C; c++) {
						float d = fs(S[si + c], T[ti + c]);
						norm = fa(norm, fm(d, d));
					}
				}
			} else {
				if (C == 3) {
					norm = fa(fa(fabsf(fs(S[si], T[ti])), fabsf(fs(S[si + 1], T[ti + 1]))),
					          fabsf(fs(S[si + 2], T[ti + 2])));
				} else {
					norm = 0.0f;
					for (int c = 0; c < C; c++) norm = fa(norm, fabsf(fs(S[si + c], T[ti + c])));
				}
			}
			D = fa(D, fm(w, norm));
		}
	return __fdiv_rn(D, (float)((unsigned)a.px * (unsigned)a.py));
}

// ------------------------------------------------------------------------
// Forward differences (k_gradient): elements first, first + stride, ... of
// the W * H * C values; output 2C interleaved channels per pixel.
__device__ __forceinline__ void gradient_span(const float *__restrict__ img, int W, int H, int C,
                                              float *__restrict__ grad, int first, int stride)
{
	const int n = W * H * C;
	for (int i = first; i < n; i += stride) {
		const int p = i / C;
		const int x = p % W, y = p / W;
		const float v = img[i];
		const float gx = (x == W - 1) ? 0.0f : __fsub_rn(img[i + C], v);
		const float gy = (y == H - 1) ? 0.0f : __fsub_rn(img[i + (size_t)C * W], v);
		reinterpret_cast<float2 *>(grad)[i] = make_float2(gx, gy);
	}
}

// ------------------------------------------------------------------------
// Padded float4 pixels (k_pad4): elements first, first + stride, ... of the
// (W + 1) x (H + 1) grid, the extra column and row repeating the last ones.
__device__ __forceinline__ void pad4_span(const float *__restrict__ img, int W, int H, int C, float4 *__restrict__ out,
                                          int first, int stride)
{
	const int Wp = W + 1, n = Wp * (H + 1);
	for (int i = first; i < n; i += stride) {
		const int y = i / Wp, x = i - y * Wp;
		const float *u = img + ((size_t)min(y, H - 1) * W + min(x, W - 1)) * C;
		float4 v = make_float4(u[0], 0.f, 0.f, 0.f);
		if (C > 1) v.y = u[1];
		if (C > 2) v.z = u[2];
		if (C > 3) v.w = u[3];
		out[i] = v;
	}
}

// ------------------------------------------------------------------------
// Reductions.
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
	return v;
}

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
	return v;
}

// Sum over the block (result valid in thread 0); fixed order, so repeatable.
template <int BLOCK>
__device__ __forceinline__ double block_sum(double v, double *smem /* BLOCK/32 */)
{
	v = warp_sum(v);
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	if (lane == 0) smem[wid] = v;
	__syncthreads();
	double t = 0.0;
	if (wid == 0) {
		t = (lane < BLOCK / 32) ? smem[lane] : 0.0;
		t = warp_sum(t);
	}
	__syncthreads();
	return t;
}

// ------------------------------------------------------------------------
// Grid-wide barrier for cooperatively launched kernels (all blocks are
// co-resident).  Spins at most st->wait_limit polls (2^26 when 0); on
// expiry it records a timeout in the status block and returns false so the
// kernel can leave.
__device__ __forceinline__ bool grid_barrier(DevStatus *st, unsigned nblocks)
{
	__syncthreads();
	bool ok = true;
	if (threadIdx.x == 0) {
		const unsigned set = *(volatile unsigned *)&st->wait_limit;
		const unsigned limit = set ? set : (1u << 26);
		volatile unsigned *gen = &st->barrier_gen;
		unsigned g = *gen;
		__threadfence();
		if (atomicAdd(&st->barrier_count, 1u) == nblocks - 1) {
			st->barrier_count = 0;
			__threadfence();
			atomicExch(&st->barrier_gen, g + 1);
		} else {
			unsigned polls = 0;
			while (*gen == g) {
				if (++polls > limit || *(volatile int *)&st->timeout) {
					atomicExch(&st->timeout, 1);
					ok = false;
					break;
				}
				__nanosleep(32);
			}
		}
		__threadfence();
	}
	__syncthreads();
	// every block learns about a timeout at its next barrier at the latest
	return ok && !*(volatile int *)&st->timeout;
}

}  // namespace nli
