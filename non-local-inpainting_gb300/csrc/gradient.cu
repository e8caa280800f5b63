// Gradient::calculate (gradient.cpp:20-75), the packed feature image read
// by the PatchMatch distance, mask compaction and small reductions.
#include "nli_device.cuh"

namespace nli {

// Forward differences per channel, 0 on the last column / row; output has
// 2C interleaved channels [gx_0, gy_0, gx_1, gy_1, ...].  One thread per
// pixel and channel; consecutive threads touch consecutive addresses.
__global__ void k_gradient(const float *__restrict__ img, int W, int H, int C, float *__restrict__ grad)
{
	const int n = W * H * C;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const int p = i / C;
		const int x = p % W, y = p / W;
		const float v = img[i];
		const float gx = (x == W - 1) ? 0.0f : __fsub_rn(img[i + C], v);
		const float gy = (y == H - 1) ? 0.0f : __fsub_rn(img[i + (size_t)C * W], v);
		reinterpret_cast<float2 *>(grad)[i] = make_float2(gx, gy);
	}
}

void launch_gradient(cudaStream_t s, const float *img, int W, int H, int C, float *grad)
{
	const int n = W * H * C;
	const int block = 256, grid = (n + block - 1) / block;
	k_gradient<<<grid, block, 0, s>>>(img, W, H, C, grad);
	NLI_CHECK_LAUNCH();
}

// Features read by the PatchMatch distance, plane-major: per pixel the
// components [u_0..u_{C-1}, gx_0, gy_0, ..., gx_{C-1}, gy_{C-1}] (gradient
// kinds) or [u_0..u_{C-1}] (colour-only kinds); components 4j..4j+3 go to
// float4 plane j (p4 planes of W*H float4), a ninth component (C = 3
// gradient kinds: 9 components, 36 bytes per pixel) to one float plane.
// Missing components of the last float4 are zero.
void feature_layout(int kind, int C, int *p4, int *f1)
{
	const int comps = (kind == NLI_DIST_L2_COMBINED || kind == NLI_DIST_L2_RGBD) ? 3 * C : C;
	*f1 = (comps % 4 == 1 && comps > 1) ? 1 : 0;
	*p4 = (comps - *f1 + 3) / 4;
}

template <bool GRAD>
__global__ void k_features(const float *__restrict__ img, int W, int H, int C, int p4, int f1,
                           float4 *__restrict__ planes4, float *__restrict__ plane1)
{
	const int n = W * H;
	for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
		const int x = p % W, y = p / W;
		float f[16];
#pragma unroll
		for (int k = 0; k < 16; k++) f[k] = 0.f;
		const float *u = img + (size_t)p * C;
		for (int c = 0; c < C; c++) {
			const float v = u[c];
			f[c] = v;
			if (GRAD) {
				f[C + 2 * c] = (x == W - 1) ? 0.0f : __fsub_rn(u[C + c], v);
				f[C + 2 * c + 1] = (y == H - 1) ? 0.0f : __fsub_rn(u[(size_t)C * W + c], v);
			}
		}
		for (int k = 0; k < p4; k++)
			planes4[(size_t)k * n + p] = make_float4(f[4 * k], f[4 * k + 1], f[4 * k + 2], f[4 * k + 3]);
		if (f1) plane1[p] = f[4 * p4];
	}
}

void launch_features(cudaStream_t s, int kind, const float *img, int W, int H, int C, float4 *planes4, float *plane1)
{
	const int n = W * H;
	const int block = 256, grid = (n + block - 1) / block;
	int p4, f1;
	feature_layout(kind, C, &p4, &f1);
	if (kind == NLI_DIST_L2_COMBINED || kind == NLI_DIST_L2_RGBD)
		k_features<true><<<grid, block, 0, s>>>(img, W, H, C, p4, f1, planes4, plane1);
	else
		k_features<false><<<grid, block, 0, s>>>(img, W, H, C, p4, f1, planes4, plane1);
	NLI_CHECK_LAUNCH();
}

// ---------------------------------------------------------- compaction
// Raster-order list of the set pixels of a mask in three passes: per-tile
// counts, one exclusive scan, per-tile ordered writes.
constexpr int kTile = 1024;

__global__ void k_count(const uint8_t *__restrict__ mask, int n, int *__restrict__ counts)
{
	__shared__ int s[32];
	const int base = blockIdx.x * kTile;
	int c = 0;
	for (int i = threadIdx.x; i < kTile; i += blockDim.x) {
		const int p = base + i;
		c += (p < n && mask[p]) ? 1 : 0;
	}
	for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
	if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = c;
	__syncthreads();
	if (threadIdx.x == 0) {
		int t = 0;
		for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s[w];
		counts[blockIdx.x] = t;
	}
}

__global__ void k_scan(int *__restrict__ counts, int tiles, int *__restrict__ total)
{
	// single block: exclusive scan of the tile counts, sequential chunks per thread
	__shared__ int part[1024];
	const int T = blockDim.x;
	const int per = (tiles + T - 1) / T;
	const int b = threadIdx.x * per, e = min(b + per, tiles);
	int s = 0;
	for (int i = b; i < e; i++) s += counts[i];
	part[threadIdx.x] = s;
	__syncthreads();
	if (threadIdx.x == 0) {
		int run = 0;
		for (int i = 0; i < T; i++) {
			int v = part[i];
			part[i] = run;
			run += v;
		}
		*total = run;
	}
	__syncthreads();
	int run = part[threadIdx.x];
	for (int i = b; i < e; i++) {
		int v = counts[i];
		counts[i] = run;
		run += v;
	}
}

__global__ void k_write(const uint8_t *__restrict__ mask, int n, const int *__restrict__ offsets,
                        int32_t *__restrict__ list)
{
	// 1024 threads, one pixel each: block-wide ordered scan of the flags
	__shared__ int warp_tot[32];
	const int p = blockIdx.x * kTile + threadIdx.x;
	const int f = (p < n && mask[p]) ? 1 : 0;
	const unsigned bal = __ballot_sync(0xffffffffu, f);
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	const int in_warp = __popc(bal & ((1u << lane) - 1u));
	if (lane == 0) warp_tot[wid] = __popc(bal);
	__syncthreads();
	if (wid == 0) {
		int v = warp_tot[lane];
		int incl = v;
		for (int o = 1; o < 32; o <<= 1) {
			int t = __shfl_up_sync(0xffffffffu, incl, o);
			if (lane >= o) incl += t;
		}
		warp_tot[lane] = incl - v;
	}
	__syncthreads();
	if (f) list[offsets[blockIdx.x] + warp_tot[wid] + in_warp] = p;
}

int compact_mask(nli_ctx *ctx, const uint8_t *mask, int W, int H, int32_t *list, const char *tag)
{
	const int n = W * H;
	const int tiles = (n + kTile - 1) / kTile;
	int *counts = ctx->buf<int>(std::string("compact.counts.") + tag, tiles + 1);
	int *total = counts + tiles;
	k_count<<<tiles, 256, 0, ctx->stream>>>(mask, n, counts);
	NLI_CHECK_LAUNCH();
	k_scan<<<1, 1024, 0, ctx->stream>>>(counts, tiles, total);
	NLI_CHECK_LAUNCH();
	k_write<<<tiles, kTile, 0, ctx->stream>>>(mask, n, counts, list);
	NLI_CHECK_LAUNCH();
	NLI_CUDA(cudaMemcpyAsync(ctx->host_pinned, total, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
	NLI_CUDA(cudaStreamSynchronize(ctx->stream));
	return *(int *)ctx->host_pinned;
}

// Sum of n doubles in a fixed order (one block), for repeatable totals.
__global__ void k_sum_partials(const double *__restrict__ partials, int n, double *__restrict__ out)
{
	__shared__ double s[32];
	double v = 0.0;
	for (int i = threadIdx.x; i < n; i += blockDim.x) v += partials[i];
	v = block_sum<1024>(v, s);
	if (threadIdx.x == 0) *out = v;
}

void launch_sum_partials(cudaStream_t s, const double *partials, int n, double *out)
{
	k_sum_partials<<<1, 1024, 0, s>>>(partials, n, out);
	NLI_CHECK_LAUNCH();
}

}  // namespace nli
