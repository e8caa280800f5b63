// APatchDistance::calculate over explicit pair lists, and the exhaustive
// nearest-neighbour search used to pin PatchMatch on small crops.  Both use
// the reference-exact distance (nli_device.cuh, dist_exact).
#include <cuda.h>  // CUcontext, CUresult (driver entry points reached through the runtime)

#include <mutex>
#include <new>
#include <stdexcept>

#include "nli_device.cuh"

namespace nli {

__global__ void k_distance_pairs(DistArgs a, const float *__restrict__ S, const float *__restrict__ GS, int sW,
                                 int sH, const float *__restrict__ T, const float *__restrict__ GT, int tW, int tH,
                                 const int4 *__restrict__ pairs, int n, float *__restrict__ out)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const int4 q = pairs[i];
	const bool inside = q.x >= a.rx && q.y >= a.ry && q.x + (a.px - a.rx) <= sW && q.y + (a.py - a.ry) <= sH &&
	                    q.z >= a.rx && q.w >= a.ry && q.z + (a.px - a.rx) <= tW && q.w + (a.py - a.ry) <= tH;
	// a patch leaving its image has no defined distance: NaN
	out[i] = inside ? dist_exact(a, S, GS, sW, T, GT, tW, q.x, q.y, q.z, q.w) : __int_as_float(0x7fc00000);
}

// One block per target pixel; threads stride over the source pixels; the
// block keeps the least distance, ties going to the lowest raster index.
__global__ void k_bruteforce(DistArgs a, const float *__restrict__ S, const float *__restrict__ GS,
                             const uint8_t *__restrict__ smask, int sW, int sH, const float *__restrict__ T,
                             const float *__restrict__ GT, const uint8_t *__restrict__ tmask, int tW, int tH,
                             int2 *__restrict__ nnf, float *__restrict__ dist)
{
	const int t = blockIdx.x;
	const int tx = t % tW, ty = t / tW;
	const bool valid_t = tmask[t] && tx - a.rx >= 0 && ty - a.ry >= 0 && tx + (a.px - a.rx) <= tW &&
	                     ty + (a.py - a.ry) <= tH;
	if (!valid_t) {
		if (threadIdx.x == 0) {
			nnf[t] = make_int2(-1, -1);
			dist[t] = FLT_MAX;
		}
		return;
	}
	float best = FLT_MAX;
	int best_i = INT_MAX;
	const int ns = sW * sH;
	for (int s = threadIdx.x; s < ns; s += blockDim.x) {
		const int sx = s % sW, sy = s / sW;
		if (!smask[s]) continue;
		if (sx - a.rx < 0 || sy - a.ry < 0 || sx + (a.px - a.rx) > sW || sy + (a.py - a.ry) > sH) continue;
		const float d = dist_exact(a, S, GS, sW, T, GT, tW, sx, sy, tx, ty);
		if (d < best || (d == best && s < best_i)) {
			best = d;
			best_i = s;
		}
	}
	__shared__ float sd[1024];
	__shared__ int si[1024];
	sd[threadIdx.x] = best;
	si[threadIdx.x] = best_i;
	__syncthreads();
	for (int o = blockDim.x / 2; o > 0; o >>= 1) {
		if (threadIdx.x < o) {
			const float d2 = sd[threadIdx.x + o];
			const int i2 = si[threadIdx.x + o];
			if (d2 < sd[threadIdx.x] || (d2 == sd[threadIdx.x] && i2 < si[threadIdx.x])) {
				sd[threadIdx.x] = d2;
				si[threadIdx.x] = i2;
			}
		}
		__syncthreads();
	}
	if (threadIdx.x == 0) {
		const int b = si[0];
		nnf[t] = (b == INT_MAX) ? make_int2(-1, -1) : make_int2(b % sW, b / sW);
		dist[t] = sd[0];
	}
}

static void gradients_for(nli_ctx *ctx, const nli_distance_params &p, const float *src, int sW, int sH,
                          const float *tgt, int tW, int tH, int C, const float **gs, const float **gt)
{
	*gs = *gt = nullptr;
	if (p.kind != NLI_DIST_L2_COMBINED && p.kind != NLI_DIST_L2_RGBD) return;
	float *a = ctx->buf<float>("dist.gs", (size_t)sW * sH * 2 * C);
	launch_gradient(ctx->stream, src, sW, sH, C, a);
	*gs = a;
	if (tgt == src && tW == sW && tH == sH) {
		*gt = a;
		return;
	}
	float *b = ctx->buf<float>("dist.gt", (size_t)tW * tH * 2 * C);
	launch_gradient(ctx->stream, tgt, tW, tH, C, b);
	*gt = b;
}

}  // namespace nli

using namespace nli;

extern "C" int nli_distance_pairs(nli_ctx *ctx, const nli_distance_params *dist, const float *source, int sW, int sH,
                                  const float *target, int tW, int tH, int C, const int32_t *pairs, int n, float *out)
{
	if (!ctx) return NLI_E_INVALID;
	try {
		NLI_CUDA(cudaSetDevice(ctx->device));
		NLI_REQUIRE(dist && source && target && out && (pairs || n == 0), NLI_E_INVALID, "null pointer argument");
		NLI_REQUIRE(sW > 0 && sH > 0 && tW > 0 && tH > 0 && n >= 0, NLI_E_INVALID, "bad sizes");
		DistArgs a;
		fill_dist_args(a, *dist, C);
		if (n == 0) return NLI_OK;
		const float *gs, *gt;
		gradients_for(ctx, *dist, source, sW, sH, target, tW, tH, C, &gs, &gt);
		k_distance_pairs<<<(n + 127) / 128, 128, 0, ctx->stream>>>(a, source, gs, sW, sH, target, gt, tW, tH,
		                                                            reinterpret_cast<const int4 *>(pairs), n, out);
		NLI_CHECK_LAUNCH();
	} catch (const Error &e) {
		ctx->last_error = e.message;
		return e.status;
	} catch (const std::bad_alloc &) {
		ctx->last_error = "host allocation failed";
		return NLI_E_NOMEM;
	} catch (const std::exception &e) {
		ctx->last_error = e.what();
		return NLI_E_INVALID;
	}
	return NLI_OK;
}

extern "C" int nli_bruteforce_nnf(nli_ctx *ctx, const nli_distance_params *dist, const float *source,
                                  const uint8_t *source_mask, int sW, int sH, const float *target,
                                  const uint8_t *target_mask, int tW, int tH, int C, int32_t *nnf, float *distance)
{
	if (!ctx) return NLI_E_INVALID;
	try {
		NLI_CUDA(cudaSetDevice(ctx->device));
		NLI_REQUIRE(dist && source && source_mask && target && target_mask && nnf && distance, NLI_E_INVALID,
		            "null pointer argument");
		NLI_REQUIRE(sW > 0 && sH > 0 && tW > 0 && tH > 0, NLI_E_INVALID, "bad sizes");
		DistArgs a;
		fill_dist_args(a, *dist, C);
		const float *gs, *gt;
		gradients_for(ctx, *dist, source, sW, sH, target, tW, tH, C, &gs, &gt);
		k_bruteforce<<<tW * tH, 256, 0, ctx->stream>>>(a, source, gs, source_mask, sW, sH, target, gt, target_mask,
		                                                tW, tH, reinterpret_cast<int2 *>(nnf), distance);
		NLI_CHECK_LAUNCH();
	} catch (const Error &e) {
		ctx->last_error = e.message;
		return e.status;
	} catch (const std::bad_alloc &) {
		ctx->last_error = "host allocation failed";
		return NLI_E_NOMEM;
	} catch (const std::exception &e) {
		ctx->last_error = e.what();
		return NLI_E_INVALID;
	}
	return NLI_OK;
}

// ------------------------------------------------------------------------
// Allocation-free variant of nli_distance_pairs.
//
// Some callers cannot allocate device memory once they are running: host
// frameworks that reserve the whole device budget up front and forbid any
// further cudaMalloc, or latency-critical loops in which cudaMalloc /
// cudaFree would synchronise the device.  This entry point needs no context
// and no workspace: the gradient images it builds live in the fixed
// file-scope array below, which every process that loads this library
// holds on every device it uses until exit.  All calls share that array,
// so calls that overlap on the GPU (different streams, or different host
// threads without ordering) race on it; callers must order them.  Nothing
// in the array needs to start at zero: every element a call reads is
// written earlier in the same call.
namespace nli {

constexpr size_t kNoAllocScratchFloats = NLI_NOALLOC_SCRATCH_BYTES / sizeof(float);
static __device__ __align__(256) float g_noalloc_scratch[kNoAllocScratchFloats];

// The array's device address differs between CUDA contexts: each context
// (a device's primary context, a context a driver-API host made current,
// the primary context re-created after cudaDeviceReset) loads the module
// anew.  So the address is cached per context, keyed by the context's
// unique ID (cuCtxGetId: never reused within a process, unlike the handle),
// and looked up once per context with cudaGetSymbolAddress.
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

struct NoAllocEntry {
	unsigned long long ctx_id;
	float *ptr;
};
static std::vector<NoAllocEntry> g_noalloc_cache;
static std::mutex g_noalloc_mutex;

template <class Fn>
static Fn driver_fn(const char *name)
{
	void *f = nullptr;
	cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
	if (cudaGetDriverEntryPointByVersion(name, &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
	    q != cudaDriverEntryPointSuccess) {
		(void)cudaGetLastError();
		return nullptr;
	}
	return reinterpret_cast<Fn>(f);
}

// ID of the context current on this thread (0 when none is current yet).
static unsigned long long current_ctx_id()
{
	static const CtxGetCurrentFn get_current = driver_fn<CtxGetCurrentFn>("cuCtxGetCurrent");
	static const CtxGetIdFn get_id = driver_fn<CtxGetIdFn>("cuCtxGetId");
	NLI_REQUIRE(get_current && get_id, NLI_E_UNSUPPORTED, "the driver lacks cuCtxGetCurrent / cuCtxGetId");
	CUcontext c = nullptr;
	if (get_current(&c) != CUDA_SUCCESS || !c) return 0;
	unsigned long long id = 0;
	NLI_REQUIRE(get_id(c, &id) == CUDA_SUCCESS, NLI_E_CUDA, "cuCtxGetId failed");
	return id;
}

// Device address of the scratch array in the current context.  The first
// call in a context looks it up (that first call should come before any
// stream capture); later calls in the same context take it from the cache.
static float *noalloc_scratch()
{
	std::lock_guard<std::mutex> lock(g_noalloc_mutex);
	unsigned long long id = current_ctx_id();
	if (id != 0)
		for (const NoAllocEntry &e : g_noalloc_cache)
			if (e.ctx_id == id) return e.ptr;
	float *p = nullptr;
	// makes the device's primary context current when none is
	NLI_CUDA(cudaGetSymbolAddress((void **)&p, g_noalloc_scratch));
	if (id == 0) id = current_ctx_id();
	NLI_REQUIRE(id != 0, NLI_E_CUDA, "no CUDA context is current");
	g_noalloc_cache.push_back({id, p});
	return p;
}

}  // namespace nli

extern "C" int nli_distance_pairs_noalloc(const nli_distance_params *dist, const float *source, int sW, int sH,
                                          const float *target, int tW, int tH, int C, const int32_t *pairs, int n,
                                          float *out, void *stream)
{
	try {
		if (!dist || !source || !target || !out || (!pairs && n > 0)) return NLI_E_INVALID;
		if (sW <= 0 || sH <= 0 || tW <= 0 || tH <= 0 || n < 0) return NLI_E_INVALID;
		DistArgs a;
		fill_dist_args(a, *dist, C);
		const bool grad = dist->kind == NLI_DIST_L2_COMBINED || dist->kind == NLI_DIST_L2_RGBD;
		const bool same = target == source && tW == sW && tH == sH;
		const size_t gs = grad ? (size_t)sW * sH * 2 * C : 0;
		const size_t gt = (grad && !same) ? (size_t)tW * tH * 2 * C : 0;
		if (gs + gt > kNoAllocScratchFloats) return NLI_E_INVALID;  // beyond NLI_NOALLOC_SCRATCH_BYTES
		if (n == 0) return NLI_OK;
		float *scratch = noalloc_scratch();
		cudaStream_t s = (cudaStream_t)stream;
		const float *grad_s = nullptr, *grad_t = nullptr;
		if (grad) {
			launch_gradient(s, source, sW, sH, C, scratch);
			grad_s = scratch;
			grad_t = scratch;
			if (!same) {
				launch_gradient(s, target, tW, tH, C, scratch + gs);
				grad_t = scratch + gs;
			}
		}
		k_distance_pairs<<<(n + 127) / 128, 128, 0, s>>>(a, source, grad_s, sW, sH, target, grad_t, tW, tH,
		                                                  reinterpret_cast<const int4 *>(pairs), n, out);
		NLI_CHECK_LAUNCH();
	} catch (const Error &e) {
		return e.status;
	} catch (const std::bad_alloc &) {
		return NLI_E_NOMEM;
	} catch (const std::exception &) {
		return NLI_E_INVALID;
	}
	return NLI_OK;
}
