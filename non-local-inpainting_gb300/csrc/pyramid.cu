// Multiscale helpers, all with the reference's float arithmetic so that the
// pyramid, the masks and the coarsest fill are bit-identical to it:
//   Sampling::downsample_with_mask / downsample / upsample (sampling.cpp)
//   DistanceTransform::calculate (distance_transform.cpp:20-99)
//   ImageInpainting::calculate_confidence_mask, get_extended_domain,
//     add_margin and the source-mask erosion (image_inpainting.cpp)
//   poisson_solver_separable_simplest (3rdparty/simpois/simpois.c)
#include <cmath>

#include "nli_device.cuh"

namespace nli {

int sample_size_host(unsigned size, float factor) { return (int)((float)size * factor + 0.5); }

__device__ __forceinline__ int sym_a(int x, int size)
{
	// symmetric_boundary_condition_A (sampling.cpp:540-553)
	while ((x < 0) || (x >= size)) {
		if (x < 0) x = -x - 1;
		if (x >= size) x = 2 * size - x - 1;
	}
	return x;
}

__device__ __forceinline__ int neumann(int x, int size) { return max(0, min(size - 1, x)); }

// bilinear_interpolation (sampling.cpp:463-506), including its mixed
// float/double expressions on the axis-aligned branches.
__device__ float bilinear_exact(const float *__restrict__ in, int W, int H, float x, float y)
{
	const int id_x = (int)floorf(x), id_y = (int)floorf(y);
	const int x0 = neumann(id_x, W), y0 = neumann(id_y, H), x1 = neumann(id_x + 1, W), y1 = neumann(id_y + 1, H);
	const float p11 = in[x0 + W * y0];
	const float a = fs(x, (float)id_x), b = fs(y, (float)id_y);
	if (a == 0.0f || b == 0.0f) {
		if (a == 0.0f && b == 0.0f) return p11;
		if (a == 0.0f) {
			const float p12 = in[x0 + W * y1];
			return __double2float_rn(da(dm(ds(1.0, (double)b), (double)p11), (double)fm(b, p12)));
		}
		const float p21 = in[x1 + W * y0];
		return __double2float_rn(da(dm(ds(1.0, (double)a), (double)p11), (double)fm(a, p21)));
	}
	const float a_1 = __double2float_rn(ds(1.0, (double)a)), b_1 = __double2float_rn(ds(1.0, (double)b));
	const float p21 = in[x1 + W * y0], p12 = in[x0 + W * y1], p22 = in[x1 + W * y1];
	return fa(fm(b_1, fa(fm(a_1, p11), fm(a, p21))), fm(b, fa(fm(a_1, p12), fm(a, p22))));
}

struct Filter9 {
	float fx[9], fy[9];
};

// Planes: 0 = weight mask (with mask), 1..C = image channel (times mask).
// Horizontal pass of separate_convolution (sampling.cpp:415-437).
__global__ void k_conv_x(const float *__restrict__ img, const uint8_t *__restrict__ mask, int mask_val, int W, int H,
                         int C, int with_mask, Filter9 f, float *__restrict__ buf)
{
	const int P = with_mask ? C + 1 : C;
	const int n = W * H;
	for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n * P; idx += gridDim.x * blockDim.x) {
		const int k = idx / n, p = idx % n;
		const int x = p % W, y = p / W;
		float sum = 0.0f;
		for (int i = 8; i >= 0; i--) {
			const int id = sym_a(x + 4 - i, W);
			const int q = y * W + id;
			float v;
			if (with_mask) {
				const bool keep = (mask_val != 0) == (mask[q] != 0);
				v = (k == 0) ? (keep ? 1.0f : 0.0f) : (keep ? img[(size_t)C * q + (k - 1)] : 0.0f);
			} else {
				v = img[(size_t)C * q + k];
			}
			sum = fa(sum, fm(f.fx[i], v));
		}
		buf[(size_t)k * n + p] = sum;
	}
}

// Vertical pass (sampling.cpp:439-455).
__global__ void k_conv_y(const float *__restrict__ buf, int W, int H, int P, Filter9 f, float *__restrict__ out)
{
	const int n = W * H;
	for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n * P; idx += gridDim.x * blockDim.x) {
		const int k = idx / n, p = idx % n;
		const int x = p % W, y = p / W;
		float sum = 0.0f;
		for (int i = 8; i >= 0; i--) {
			const int id = sym_a(y + 4 - i, H);
			sum = fa(sum, fm(f.fy[i], buf[(size_t)k * n + (size_t)id * W + x]));
		}
		out[(size_t)k * n + p] = sum;
	}
}

// Centred-grid bilinear subsampling (sampling.cpp:330-371).
__global__ void k_sample(const float *__restrict__ filt, int W, int H, int C, int with_mask, int sW, int sH,
                         float factor_x, float factor_y, float min_x, float min_y, float threshold, int mask_val,
                         float *__restrict__ out_img, uint8_t *__restrict__ out_mask)
{
	const int n = W * H;
	const int m = sW * sH;
	for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < m; o += gridDim.x * blockDim.x) {
		const unsigned i = o / sW, j = o % sW;
		const float y = fa(min_y, fm((float)i, factor_y));
		const float x = fa(min_x, fm((float)j, factor_x));
		if (with_mask) {
			const float mv = bilinear_exact(filt, W, H, x, y);
			for (int c = 0; c < C; c++) {
				const float iv = bilinear_exact(filt + (size_t)(c + 1) * n, W, H, x, y);
				out_img[(size_t)C * o + c] = (mv > 1e-6) ? __fdiv_rn(iv, mv) : 0.f;
			}
			if (out_mask) out_mask[o] = mask_val ? (mv > threshold) : (mv < threshold);
		} else {
			for (int c = 0; c < C; c++) {
				const float v = bilinear_exact(filt + (size_t)c * n, W, H, x, y);
				if (out_img) out_img[(size_t)C * o + c] = v;
				if (out_mask) out_mask[o] = v > threshold;
			}
		}
	}
}

static Filter9 filters_for(float factor_x, float factor_y)
{
	Filter9 f;
	const float sx = (float)(0.62 * sqrt(pow(factor_x, 2) - 1));
	const float sy = (float)(0.62 * sqrt(pow(factor_y, 2) - 1));
	std::vector<float> gx = gaussian_weights_host(9, 1, sx, 0), gy = gaussian_weights_host(9, 1, sy, 0);
	for (int i = 0; i < 9; i++) {
		f.fx[i] = gx[i];
		f.fy[i] = gy[i];
	}
	return f;
}

static int grid_for(size_t n, int block = 256)
{
	size_t g = (n + block - 1) / block;
	return (int)std::min<size_t>(g, 65535u * 4);
}

static void downsample_generic(nli_ctx *ctx, const float *img, const uint8_t *mask, int mask_val, int W, int H, int C,
                               int with_mask, float factor, float threshold, float *out_img, uint8_t *out_mask)
{
	const int sW = sample_size_host(W, factor), sH = sample_size_host(H, factor);
	NLI_REQUIRE(sW > 0 && sH > 0, NLI_E_INVALID, "downsampled image would be empty");
	const float factor_x = (float)W / sW, factor_y = (float)H / sH;
	const Filter9 f = filters_for(factor_x, factor_y);
	const int P = with_mask ? C + 1 : C;
	const size_t n = (size_t)W * H;
	float *buf = ctx->buf<float>("pyr.buf", n * P);
	float *filt = ctx->buf<float>("pyr.filt", n * P);
	k_conv_x<<<grid_for(n * P), 256, 0, ctx->stream>>>(img, mask, mask_val, W, H, C, with_mask, f, buf);
	NLI_CHECK_LAUNCH();
	k_conv_y<<<grid_for(n * P), 256, 0, ctx->stream>>>(buf, W, H, P, f, filt);
	NLI_CHECK_LAUNCH();
	const float min_x = (float)(factor_x / 2.0 - 0.5), min_y = (float)(factor_y / 2.0 - 0.5);
	threshold = (float)fmax(0.0, fmin(1.0, threshold));
	k_sample<<<grid_for((size_t)sW * sH), 256, 0, ctx->stream>>>(filt, W, H, C, with_mask, sW, sH, factor_x, factor_y,
	                                                            min_x, min_y, threshold, mask_val, out_img, out_mask);
	NLI_CHECK_LAUNCH();
}

void downsample_with_mask_run(nli_ctx *ctx, const float *img, const uint8_t *mask, int W, int H, int C, float factor,
                              float threshold, int mask_val, float *out_img, uint8_t *out_mask)
{
	downsample_generic(ctx, img, mask, mask_val, W, H, C, 1, factor, threshold, out_img, out_mask);
}

void downsample_image_run(nli_ctx *ctx, const float *img, int W, int H, int C, float factor, float *out)
{
	downsample_generic(ctx, img, nullptr, 0, W, H, C, 0, factor, 0.0f, out, nullptr);
}

__global__ void k_mask_to_float(const uint8_t *__restrict__ m, int n, float *__restrict__ f)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) f[i] = m[i] ? 1.0f : 0.0f;
}

void downsample_mask_run(nli_ctx *ctx, const uint8_t *mask, int W, int H, float factor, float threshold, uint8_t *out)
{
	float *fm_ = ctx->buf<float>("pyr.maskf", (size_t)W * H);
	k_mask_to_float<<<grid_for((size_t)W * H), 256, 0, ctx->stream>>>(mask, W * H, fm_);
	NLI_CHECK_LAUNCH();
	downsample_generic(ctx, fm_, nullptr, 0, W, H, 1, 0, factor, threshold, nullptr, out);
}

// Nearest-neighbour upsampling (sampling.cpp:354-371, 387-406).
__global__ void k_upsample(const float *__restrict__ in, int W, int H, int C, int oW, int oH, float factor_x,
                           float factor_y, float min_x, float min_y, float *__restrict__ out)
{
	const int m = oW * oH;
	for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < m; o += gridDim.x * blockDim.x) {
		const unsigned i = o / oW, j = o % oW;
		const float y = __fdiv_rn(fs((float)i, min_y), factor_y);
		const float x = __fdiv_rn(fs((float)j, min_x), factor_x);
		const int ix = neumann((int)floor((double)x + 0.5), W), iy = neumann((int)floor((double)y + 0.5), H);
		for (int c = 0; c < C; c++) out[(size_t)C * o + c] = in[(size_t)C * (iy * W + ix) + c];
	}
}

void upsample_run(nli_ctx *ctx, const float *img, int W, int H, int C, int oW, int oH, float *out)
{
	const float factor_x = (float)oW / W, factor_y = (float)oH / H;
	const float min_x = (float)(factor_x / 2.0 - 0.5), min_y = (float)(factor_y / 2.0 - 0.5);
	k_upsample<<<grid_for((size_t)oW * oH), 256, 0, ctx->stream>>>(img, W, H, C, oW, oH, factor_x, factor_y, min_x,
	                                                               min_y, out);
	NLI_CHECK_LAUNCH();
}

// ---------------------------------------------------- distance transform
__global__ void k_dt_columns(const uint8_t *__restrict__ mask, int W, int H, float INF, float *__restrict__ g)
{
	const int x = blockIdx.x * blockDim.x + threadIdx.x;
	if (x >= W) return;
	float run = mask[x] ? INF : 0.0f;
	g[x] = run;
	for (int y = 1; y < H; y++) {
		run = mask[y * W + x] ? fa(run, 1.0f) : 0.0f;
		g[y * W + x] = run;
	}
	for (int y = H - 2; y >= 0; y--) {
		const float v = g[y * W + x];
		if (run < v) {
			run = fa(run, 1.0f);
			g[y * W + x] = run;
		} else {
			run = v;
		}
	}
}

__device__ __forceinline__ float dt_f(int x, int xi, float gi)
{
	const double dx = (double)(float)(x - xi), g = (double)gi;
	return __double2float_rn(__dsqrt_rn(da(dm(dx, dx), dm(g, g))));
}

// dt_f(x, i, gi) > dt_f(x, u, gu), decided without square roots where that
// is exact.  Both squares (x - i)^2 + gi^2 are integers (gi holds an integer
// column distance).  Below 2^21 the square roots of two different integers
// are more than 2 float ulps apart, so their float roundings (through
// double, each within half an ulp) keep the order of the integers; above
// it the rounded roots are
// compared as the reference compares them.
__device__ __forceinline__ bool dt_greater(int x, int i, float gi, int u, float gu)
{
	const double dxi = (double)(float)(x - i), dxu = (double)(float)(x - u);
	const double a = da(dm(dxi, dxi), dm((double)gi, (double)gi));
	const double b = da(dm(dxu, dxu), dm((double)gu, (double)gu));
	if (a < 2097152.0 && b < 2097152.0) return a > b;
	return dt_f(x, i, gi) > dt_f(x, u, gu);
}

__device__ __forceinline__ int dt_sep(int i, int u, float gi, float gu)
{
	const double fu = (double)(float)u, fi = (double)(float)i, du = (double)gu, di = (double)gi;
	const double num = ds(da(ds(dm(fu, fu), dm(fi, fi)), dm(du, du)), dm(di, di));
	return (int)__ddiv_rn(num, (double)(2 * (u - i)));
}

// Lower-envelope pass along each row (distance_transform.cpp:55-95).
__global__ void k_dt_rows(const float *__restrict__ g, int W, int H, int *__restrict__ s_buf, int *__restrict__ t_buf,
                          float *__restrict__ out)
{
	const int y = blockIdx.x * blockDim.x + threadIdx.x;
	if (y >= H) return;
	const float *gy = g + (size_t)y * W;
	int *s = s_buf + (size_t)y * W;
	int *t = t_buf + (size_t)y * W;
	int q = 0;
	s[0] = 0;
	t[0] = 0;
	for (int u = 1; u < W; u++) {
		while (q >= 0 && dt_greater(t[q], s[q], gy[s[q]], u, gy[u])) q--;
		if (q < 0) {
			q = 0;
			s[0] = u;
		} else {
			const unsigned w = 1 + dt_sep(s[q], u, gy[s[q]], gy[u]);
			if (w < (unsigned)W) {
				q++;
				s[q] = u;
				t[q] = (int)w;
			}
		}
	}
	for (int u = W - 1; u >= 0; u--) {
		out[(size_t)y * W + u] = dt_f(u, s[q], gy[s[q]]);
		if (u == t[q]) q--;
	}
}

// The row pass as a bounded search, one thread per pixel.  Both passes work
// on exact integers (column distances, squared offsets), so the row result
// is min over u of (x - u)^2 + g(u)^2 whatever the order of evaluation; the
// lower envelope above finds it for a whole row at once, this search looks
// outward from x while d^2 is below the best value found (any farther u
// cannot do better).  The final square root is rounded as dt_f rounds it,
// so both give the same floats; the search keeps every SM busy.
__global__ void k_dt_rows_search(const float *__restrict__ g, int W, int H, float *__restrict__ out)
{
	const size_t n = (size_t)W * H;
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
		const int x = (int)(i % W);
		const float *gy = g + (i - x);
		const unsigned long long gx = (unsigned long long)gy[x];
		unsigned long long best = gx * gx;
		for (unsigned long long d = 1; d * d < best; d++) {
			const bool lo = (long long)x - (long long)d >= 0, hi = x + d < (unsigned long long)W;
			if (!lo && !hi) break;
			if (lo) {
				const unsigned long long gu = (unsigned long long)gy[x - d];
				best = min(best, d * d + gu * gu);
			}
			if (hi) {
				const unsigned long long gu = (unsigned long long)gy[x + d];
				best = min(best, d * d + gu * gu);
			}
		}
		out[i] = best ? __double2float_rn(__dsqrt_rn((double)best)) : 0.0f;
	}
}

void distance_transform_run(nli_ctx *ctx, const uint8_t *mask, int W, int H, float *out)
{
	float *g = ctx->buf<float>("dt.g", (size_t)W * H);
	const float INF = (float)((unsigned)W + (unsigned)H);
	k_dt_columns<<<(W + 31) / 32, 32, 0, ctx->stream>>>(mask, W, H, INF, g);
	NLI_CHECK_LAUNCH();
	// bounded search per pixel up to 4096 columns (its work grows with the
	// hole's extent); the lower envelope, one thread per row, beyond
	if (W <= 4096) {
		const size_t n = (size_t)W * H;
		k_dt_rows_search<<<(int)std::min<size_t>((n + 255) / 256, 65535), 256, 0, ctx->stream>>>(g, W, H, out);
	} else {
		int *sb = ctx->buf<int>("dt.s", (size_t)W * H);
		int *tb = ctx->buf<int>("dt.t", (size_t)W * H);
		k_dt_rows<<<(H + 31) / 32, 32, 0, ctx->stream>>>(g, W, H, sb, tb, out);
	}
	NLI_CHECK_LAUNCH();
}

// c = (1 - asym) exp(-d / decay) + asym on the domain, 1 elsewhere
// (image_inpainting.cpp:611-630); exp is evaluated in double and rounded.
__global__ void k_confidence(const uint8_t *__restrict__ mask, const float *__restrict__ dist, int n, float decay,
                             float asym, int use_decay, float *__restrict__ out)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		float v = 1.0f;
		if (mask[i]) {
			if (use_decay) {
				const float e = __double2float_rn(exp((double)__fdiv_rn(-dist[i], decay)));
				v = fa(fm(fs(1.0f, asym), e), asym);
			} else {
				v = asym;
			}
		}
		out[i] = v;
	}
}

void confidence_run(nli_ctx *ctx, const uint8_t *mask, int W, int H, float decay, float asym, float *out)
{
	const int n = W * H;
	float *d = nullptr;
	if (decay > 0) {
		d = ctx->buf<float>("conf.dist", n);
		distance_transform_run(ctx, mask, W, H, d);
	}
	k_confidence<<<grid_for(n), 256, 0, ctx->stream>>>(mask, d, n, decay, asym, decay > 0 ? 1 : 0, out);
	NLI_CHECK_LAUNCH();
}

// ------------------------------------------------------ extended domain
// Boundary hole pixels (a 4-neighbour outside the hole or the image), then a
// separable box dilation of radius (px/2, py/2) (image_inpainting.cpp:566-600).
__global__ void k_boundary(const uint8_t *__restrict__ m, int W, int H, uint8_t *__restrict__ b)
{
	const int n = W * H;
	for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
		const int x = p % W, y = p / W;
		uint8_t v = 0;
		if (m[p]) {
			const bool sur = (x + 1 < W && m[p + 1]) && (x > 0 && m[p - 1]) && (y + 1 < H && m[p + W]) &&
			                 (y > 0 && m[p - W]);
			v = sur ? 0 : 1;
		}
		b[p] = v;
	}
}

__global__ void k_dilate_x(const uint8_t *__restrict__ b, int W, int H, int r, uint8_t *__restrict__ o)
{
	const int n = W * H;
	for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
		const int x = p % W;
		uint8_t v = 0;
		for (int i = max(x - r, 0); i <= min(x + r, W - 1) && !v; i++) v |= b[p - x + i];
		o[p] = v;
	}
}

__global__ void k_dilate_y_or(const uint8_t *__restrict__ b, const uint8_t *__restrict__ m, int W, int H, int r,
                              uint8_t *__restrict__ o)
{
	const int n = W * H;
	for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
		const int x = p % W, y = p / W;
		uint8_t v = m[p] ? 1 : 0;
		for (int j = max(y - r, 0); j <= min(y + r, H - 1) && !v; j++) v |= b[j * W + x];
		o[p] = v;
	}
}

void extended_domain_run(nli_ctx *ctx, const uint8_t *mask, int W, int H, int px, int py, uint8_t *out)
{
	const int n = W * H;
	uint8_t *b = ctx->buf<uint8_t>("ext.b", n);
	uint8_t *bx = ctx->buf<uint8_t>("ext.bx", n);
	k_boundary<<<grid_for(n), 256, 0, ctx->stream>>>(mask, W, H, b);
	NLI_CHECK_LAUNCH();
	k_dilate_x<<<grid_for(n), 256, 0, ctx->stream>>>(b, W, H, px / 2, bx);
	NLI_CHECK_LAUNCH();
	k_dilate_y_or<<<grid_for(n), 256, 0, ctx->stream>>>(bx, mask, W, H, py / 2, out);
	NLI_CHECK_LAUNCH();
}

// Source = complement of the extended domain, eroded where the right or
// lower neighbour is not source (checked against the un-eroded mask, which
// is what the reference's raster-order loop reads); `found` is set when an
// eroded source pixel exists (before the margin); then a `margin` border
// is cleared in both masks.
__global__ void k_scale_masks(const uint8_t *__restrict__ ext, int W, int H, int margin, int erode,
                              uint8_t *__restrict__ src, uint8_t *__restrict__ tgt, int *found)
{
	const int n = W * H;
	int any = 0;
	for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
		const int x = p % W, y = p / W;
		bool s = !ext[p];
		if (erode && s) {
			const bool right = (x + 1 < W) && !ext[p + 1];
			const bool down = (y + 1 < H) && !ext[p + W];
			s = right && down;
			any |= s ? 1 : 0;
		}
		const bool in_margin = x < margin || x >= W - margin || y < margin || y >= H - margin;
		src[p] = (s && !in_margin) ? 1 : 0;
		tgt[p] = (ext[p] && !in_margin) ? 1 : 0;
	}
	if (__syncthreads_or(any) && threadIdx.x == 0) atomicOr(found, 1);
}

__global__ void k_not_flag(const int *a, int *b) { *b = *a ? 0 : 1; }

void scale_masks_run(nli_ctx *ctx, const uint8_t *ext, int W, int H, int margin, int erode, uint8_t *src, uint8_t *tgt,
                     int *empty_dev)
{
	// empty_dev receives 1 when the eroded source is empty
	int *found = ctx->buf<int>("masks.found", 1);
	NLI_CUDA(cudaMemsetAsync(found, 0, sizeof(int), ctx->stream));
	const int n = W * H;
	k_scale_masks<<<grid_for(n), 256, 0, ctx->stream>>>(ext, W, H, margin, erode, src, tgt, found);
	NLI_CHECK_LAUNCH();
	if (empty_dev) {
		k_not_flag<<<1, 1, 0, ctx->stream>>>(found, empty_dev);
		NLI_CHECK_LAUNCH();
	}
}

// ---------------------------------------------------------------- simpois
// One block per channel.  Level 0 holds the image with NaN in the hole;
// level l+1 is the 2x2 NaN-aware block mean of level l (zoom_out_by_factor_two,
// simpois.c:153-175) until 1x1.  From the coarsest level up, the solution
// is initialised by bilinear zoom-in of the coarser solution
// (simpois.c:178-218) and refined by 10 in-place Gauss-Seidel sweeps with
// tstep 0.25 (simpois.c:82-100) over the NaN pixels in raster order.  The
// sweeps run as anti-diagonal wavefronts, sweep s on diagonal t - 2s at
// step t: each pixel then reads exactly the values the sequential raster
// order gives it (left/up already updated in this sweep, right/down not).
struct SpLevels {
	int n;
	int w[40], h[40];
	size_t off[40];  // offset of level l in the per-channel scratch (floats)
	size_t per_channel;
};

__device__ __forceinline__ float sp_get(const float *I, int w, int h, int i, int j)
{
	i = max(0, min(w - 1, i));
	j = max(0, min(h - 1, j));
	return I[i + j * w];
}

__global__ void __launch_bounds__(1024) k_simpois(float *__restrict__ img, const uint8_t *__restrict__ mask, int W,
                                                  int H, int C, SpLevels L, float *__restrict__ gscr,
                                                  float *__restrict__ uscr)
{
	const int c = blockIdx.x;
	float *G = gscr + (size_t)c * L.per_channel;
	float *U = uscr + (size_t)c * L.per_channel;
	// level 0 data
	for (int p = threadIdx.x; p < W * H; p += blockDim.x) G[p] = mask[p] ? __int_as_float(0x7fc00000) : img[(size_t)C * p + c];
	__syncthreads();
	for (int l = 0; l + 1 < L.n; l++) {
		const float *in = G + L.off[l];
		float *out = G + L.off[l + 1];
		const int iw = L.w[l], ih = L.h[l], ow = L.w[l + 1], oh = L.h[l + 1];
		for (int p = threadIdx.x; p < ow * oh; p += blockDim.x) {
			const int i = p % ow, j = p / ow;
			float a[4];
			a[0] = sp_get(in, iw, ih, 2 * i, 2 * j);
			a[1] = sp_get(in, iw, ih, 2 * i + 1, 2 * j);
			a[2] = sp_get(in, iw, ih, 2 * i, 2 * j + 1);
			a[3] = sp_get(in, iw, ih, 2 * i + 1, 2 * j + 1);
			float m = 0;
			int cx = 0;
			for (int k = 0; k < 4; k++)
				if (isfinite(a[k])) {
					m = fa(m, a[k]);
					cx += 1;
				}
			out[p] = cx ? __fdiv_rn(m, (float)cx) : __int_as_float(0x7fc00000);
		}
		__syncthreads();
	}
	for (int l = L.n - 1; l >= 0; l--) {
		const int w = L.w[l], h = L.h[l];
		const float *g = G + L.off[l];
		float *u = U + L.off[l];
		// initialisation: data outside the hole, zoom-in of the coarser solution inside
		for (int p = threadIdx.x; p < w * h; p += blockDim.x) {
			float init = 0.0f;
			if (l + 1 < L.n) {
				const float *us = U + L.off[l + 1];
				const int iw = L.w[l + 1], ih = L.h[l + 1];
				const int i = p % w, j = p / w;
				const float pp = __double2float_rn(((double)i - 0.5) / 2), qq = __double2float_rn(((double)j - 0.5) / 2);
				const int ip = (int)floorf(pp), iq = (int)floorf(qq);
				const float A = sp_get(us, iw, ih, ip, iq), B = sp_get(us, iw, ih, ip + 1, iq);
				const float Cc = sp_get(us, iw, ih, ip, iq + 1), D = sp_get(us, iw, ih, ip + 1, iq + 1);
				const float x = fs(pp, (float)ip), y = fs(qq, (float)iq);
				float r = 0;
				r = fa(r, fm(fm(A, fs(1.0f, x)), fs(1.0f, y)));
				r = fa(r, fm(fm(B, x), fs(1.0f, y)));
				r = fa(r, fm(fm(Cc, fs(1.0f, x)), y));
				r = fa(r, fm(fm(D, x), y));
				init = r;
			}
			u[p] = isfinite(g[p]) ? g[p] : init;
		}
		__syncthreads();
		const int niter = 10;
		const int ndiag = w + h - 1;
		const int steps = ndiag + 2 * (niter - 1);
		for (int t = 0; t < steps; t++) {
			// pairs (sweep s, pixel on diagonal k = t - 2s)
			const int s_lo = max(0, (t - (ndiag - 1) + 1) / 2), s_hi = min(niter - 1, t / 2);
			for (int s = s_lo; s <= s_hi; s++) {
				const int k = t - 2 * s;
				const int i_lo = max(0, k - (h - 1)), i_hi = min(w - 1, k);
				for (int i = i_lo + (int)threadIdx.x; i <= i_hi; i += blockDim.x) {
					const int j = k - i;
					const int ij = j * w + i;
					if (!isnan(g[ij])) continue;
					const float xv = sp_get(u, w, h, i, j);
					const float av = sp_get(u, w, h, i + 1, j), bv = sp_get(u, w, h, i, j + 1);
					const float cv = sp_get(u, w, h, i - 1, j), dv = sp_get(u, w, h, i, j - 1);
					float r = 0;
					if (isfinite(av)) r = fa(r, fs(av, xv));
					if (isfinite(bv)) r = fa(r, fs(bv, xv));
					if (isfinite(cv)) r = fa(r, fs(cv, xv));
					if (isfinite(dv)) r = fa(r, fs(dv, xv));
					u[ij] = fa(u[ij], fm(0.25f, fs(r, 0.0f)));
				}
			}
			__syncthreads();
		}
	}
	for (int p = threadIdx.x; p < W * H; p += blockDim.x)
		if (mask[p]) img[(size_t)C * p + c] = U[p];
}

void poisson_init_run(nli_ctx *ctx, float *img, const uint8_t *mask, int W, int H, int C)
{
	SpLevels L;
	L.n = 0;
	size_t off = 0;
	int w = W, h = H;
	for (int scale = 99;; scale--) {
		NLI_REQUIRE(L.n < 40, NLI_E_UNSUPPORTED, "image too large for the coarsest Poisson fill");
		L.w[L.n] = w;
		L.h[L.n] = h;
		L.off[L.n] = off;
		off += (size_t)w * h;
		L.n++;
		if (!(scale > 1 && (w > 1 || h > 1))) break;
		w = (int)ceil(w / 2.0);
		h = (int)ceil(h / 2.0);
	}
	L.per_channel = off;
	float *g = ctx->buf<float>("sp.g", off * C);
	float *u = ctx->buf<float>("sp.u", off * C);
	k_simpois<<<C, 1024, 0, ctx->stream>>>(img, mask, W, H, C, L, g, u);
	NLI_CHECK_LAUNCH();
}

}  // namespace nli
