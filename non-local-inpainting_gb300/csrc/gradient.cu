// Gradient::calculate (gradient.cpp:20-75), the padded pixel image read by
// the PatchMatch distance, mask compaction and small reductions.
#include "nli_device.cuh"

namespace nli {

// Forward differences per channel, 0 on the last column / row; output has
// 2C interleaved channels [gx_0, gy_0, gx_1, gy_1, ...].  One thread per
// pixel and channel; consecutive threads touch consecutive addresses.
__global__ void k_gradient(const float *__restrict__ img, int W, int H, int C, float *__restrict__ grad)
{
	gradient_span(img, W, H, C, grad, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

void launch_gradient(cudaStream_t s, const float *img, int W, int H, int C, float *grad)
{
	const int n = W * H * C;
	const int block = 256, grid = (n + block - 1) / block;
	k_gradient<<<grid, block, 0, s>>>(img, W, H, C, grad);
	NLI_CHECK_LAUNCH();
}

// Pixels read by the PatchMatch distance: one float4 per pixel (channels
// 0..C-1, the rest zero) over (W + 1) x (H + 1), the extra column and row
// repeating the last ones so that forward differences there are exactly 0.
__global__ void k_pad4(const float *__restrict__ img, int W, int H, int C, float4 *__restrict__ out)
{
	pad4_span(img, W, H, C, out, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

void launch_pad4(cudaStream_t s, const float *img, int W, int H, int C, float4 *out)
{
	const int n = (W + 1) * (H + 1);
	const int block = 256, grid = (n + block - 1) / block;
	k_pad4<<<grid, block, 0, s>>>(img, W, H, C, out);
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
