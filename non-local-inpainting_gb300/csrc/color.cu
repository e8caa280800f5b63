// Colour conversions of the command-line caller (io_utility.cpp:268-318,
// 380-440) and the RGB-D channel packing (io_utility.cpp:442-500): sRGB
// (0..255) <-> CIE L*a*b* through XYZ (D65 white 95.047 / 100 / 108.883),
// one thread per pixel.  The reference's float / double evaluation order is
// kept; its float pow (powf) is evaluated as a double pow rounded to float.
#include "nli_device.cuh"

namespace nli {

__device__ __forceinline__ float powr(float x, float y) { return __double2float_rn(pow((double)x, (double)y)); }

__device__ __forceinline__ float srgb_expand(float v)
{
	// (v > 0.04045) ? pow((v + 0.055f) / 1.055f, 2.4f) : v / 12.92 (double)
	return ((double)v > 0.04045) ? powr(__fdiv_rn(fa(v, 0.055f), 1.055f), 2.4f)
	                             : __double2float_rn(__ddiv_rn((double)v, 12.92));
}

__device__ __forceinline__ float lab_f(float t)
{
	return (t > 0.008856f) ? powr(t, __fdiv_rn(1.0f, 3.0f)) : fa(fm(7.787f, t), __fdiv_rn(16.0f, 116.0f));
}

__global__ void k_rgb_to_lab(const float *__restrict__ rgb, int n, float *__restrict__ lab)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const float *c = rgb + (size_t)3 * i;
		// rgb_to_xyz (:380-396)
		float r = srgb_expand(__fdiv_rn(c[0], 255.0f)), g = srgb_expand(__fdiv_rn(c[1], 255.0f)),
		      b = srgb_expand(__fdiv_rn(c[2], 255.0f));
		r = fm(r, 100.0f);
		g = fm(g, 100.0f);
		b = fm(b, 100.0f);
		const float X = fa(fa(fm(r, 0.412453f), fm(g, 0.357580f)), fm(b, 0.180423f));
		const float Y = fa(fa(fm(r, 0.212671f), fm(g, 0.715160f)), fm(b, 0.072169f));
		const float Z = fa(fa(fm(r, 0.019334f), fm(g, 0.119193f)), fm(b, 0.950227f));
		// xyz_to_lab (:399-412)
		const float fx = lab_f(__fdiv_rn(X, 95.047f)), fy = lab_f(__fdiv_rn(Y, 100.000f)),
		            fz = lab_f(__fdiv_rn(Z, 108.883f));
		float *o = lab + (size_t)3 * i;
		o[0] = fs(fm(116.0f, fy), 16.0f);
		o[1] = fm(500.0f, fs(fx, fy));
		o[2] = fm(200.0f, fs(fy, fz));
	}
}

__device__ __forceinline__ float lab_finv(float t)
{
	const float t3 = powr(t, 3.0f);
	return (t3 > 0.008856f) ? t3 : __fdiv_rn(fs(t, __fdiv_rn(16.0f, 116.0f)), 7.787f);
}

__device__ __forceinline__ float srgb_compress(float v)
{
	return (v > 0.0031308f) ? fs(fm(1.055f, powr(v, __fdiv_rn(1.0f, 2.4f))), 0.055f) : fm(12.92f, v);
}

// lab_to_rgb: the first three channels of a C-channel image (C = 3 or 4;
// the depth channel of a 4-channel image is dropped, :297-318).
__global__ void k_lab_to_rgb(const float *__restrict__ lab, int n, int C, float *__restrict__ rgb)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const float *c = lab + (size_t)C * i;
		// lab_to_xyz (:415-429)
		const float fy = __fdiv_rn(fa(c[0], 16.0f), 116.0f);
		const float fx = __double2float_rn(__dadd_rn(__ddiv_rn((double)c[1], 500.0), (double)fy));
		const float fz = fs(fy, __fdiv_rn(c[2], 200.0f));
		const float X = fm(lab_finv(fx), 95.047f), Y = fm(lab_finv(fy), 100.000f), Z = fm(lab_finv(fz), 108.883f);
		// xyz_to_rgb (:432-449)
		const float x = __fdiv_rn(X, 100.0f), y = __fdiv_rn(Y, 100.0f), z = __fdiv_rn(Z, 100.0f);
		const float r = fa(fa(fm(x, 3.240479f), fm(y, -1.537150f)), fm(z, -0.498535f));
		const float g = fa(fa(fm(x, -0.969256f), fm(y, 1.875992f)), fm(z, 0.041556f));
		const float b = fa(fa(fm(x, 0.055648f), fm(y, -0.204043f)), fm(z, 1.057311f));
		float *o = rgb + (size_t)3 * i;
		o[0] = fm(srgb_compress(r), 255.0f);
		o[1] = fm(srgb_compress(g), 255.0f);
		o[2] = fm(srgb_compress(b), 255.0f);
	}
}

__global__ void k_cat_depth(const float *__restrict__ rgb, const float *__restrict__ depth, int n,
                            float *__restrict__ out)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		reinterpret_cast<float4 *>(out)[i] =
		    make_float4(rgb[(size_t)3 * i], rgb[(size_t)3 * i + 1], rgb[(size_t)3 * i + 2], depth[i]);
}

__global__ void k_separate_depth(const float *__restrict__ rgbd, int n, float *__restrict__ rgb,
                                 float *__restrict__ depth)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const float4 v = reinterpret_cast<const float4 *>(rgbd)[i];
		if (rgb) {
			rgb[(size_t)3 * i] = v.x;
			rgb[(size_t)3 * i + 1] = v.y;
			rgb[(size_t)3 * i + 2] = v.z;
		}
		if (depth) depth[i] = v.w;
	}
}

static int grid_of(int n) { return std::max(1, std::min((n + 255) / 256, 8192)); }

void rgb_to_lab_run(nli_ctx *ctx, const float *rgb, int n, float *lab)
{
	k_rgb_to_lab<<<grid_of(n), 256, 0, ctx->stream>>>(rgb, n, lab);
	NLI_CHECK_LAUNCH();
}

void lab_to_rgb_run(nli_ctx *ctx, const float *lab, int n, int C, float *rgb)
{
	k_lab_to_rgb<<<grid_of(n), 256, 0, ctx->stream>>>(lab, n, C, rgb);
	NLI_CHECK_LAUNCH();
}

void cat_depth_run(nli_ctx *ctx, const float *rgb, const float *depth, int n, float *out)
{
	k_cat_depth<<<grid_of(n), 256, 0, ctx->stream>>>(rgb, depth, n, out);
	NLI_CHECK_LAUNCH();
}

void separate_depth_run(nli_ctx *ctx, const float *rgbd, int n, float *rgb, float *depth)
{
	k_separate_depth<<<grid_of(n), 256, 0, ctx->stream>>>(rgbd, n, rgb, depth);
	NLI_CHECK_LAUNCH();
}

}  // namespace nli
