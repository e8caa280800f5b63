// AImageUpdating subclasses as gather kernels over the nearest-neighbour
// field:
//   NL-means   (patch_non_local_means.cpp:23-100)   - one thread per hole pixel
//   NL-medians (patch_non_local_medians.cpp:23-127) - one warp per hole pixel
//   NL-Poisson (patch_non_local_poisson.cpp:36-477) - coefficient gather,
//              right-hand side, and one cooperative kernel running the
//              conjugate gradient of every channel with fused stencil,
//              dot products and axpys
//   NL-depth   (patch_non_local_depth.cpp:36-55)    - NL-Poisson with a
//              per-channel lambda on the 4-channel image, orig = image
#include <cooperative_groups.h>

#include <atomic>

#include "nli_device.cuh"

namespace nli {

struct UpdArgs {
	int px, py, hx, hy;
	int W, H, C;
	float weights[kMaxTaps];
};

static void fill_upd_args(UpdArgs &u, const nli_update_params &p, int W, int H, int C)
{
	NLI_REQUIRE(p.patch_x >= 1 && p.patch_y >= 1 && p.patch_x <= NLI_MAX_PATCH && p.patch_y <= NLI_MAX_PATCH,
	            NLI_E_UNSUPPORTED, "patch size outside 1.." + std::to_string(NLI_MAX_PATCH));
	std::memset(&u, 0, sizeof(u));
	u.px = p.patch_x;
	u.py = p.patch_y;
	u.hx = p.patch_x / 2;
	u.hy = p.patch_y / 2;
	u.W = W;
	u.H = H;
	u.C = C;
	std::vector<float> w = gaussian_weights_host(p.patch_x, p.patch_y, p.sigma, p.sigma);
	std::memcpy(u.weights, w.data(), sizeof(float) * w.size());
}

// ------------------------------------------------------------- NL-means
// Reference arithmetic: float accumulators, separate roundings, the patch
// weight indexed from the clipped window corner (:71), confidence applied
// inside the domain only (:72-74).  New values go to a compact buffer and
// are scattered afterwards, so every pixel reads the pre-update image.
// One hole pixel: the new values into out[0..C) and (u_old - u_new)^2
// summed over the channels.  u supplies the patch and its weights; W, H,
// C are the image's.
__device__ __forceinline__ double nlmeans_pixel(const UpdArgs &u, int W, int H, int C, const float *__restrict__ img,
                                                int pix, const uint8_t *__restrict__ dom, const int2 *__restrict__ nnf,
                                                const float *__restrict__ conf, float *__restrict__ out)
{
	double acc = 0.0;
	if (!nli_in_bounds(pix, (long long)W * H, kSiteHole)) return 0.0;
	const int x = pix % W, y = pix / W;
	const int x_a = max(x - u.hx, 0), x_b = min(x + u.hx, W - 1);
	const int y_a = max(y - u.hy, 0), y_b = min(y + u.hy, H - 1);
	float tv[4] = {0.f, 0.f, 0.f, 0.f};
	float tw = 0.f;
	for (int ii = x_a; ii <= x_b; ii++)
		for (int jj = y_a; jj <= y_b; jj++) {
			int2 q = nnf[jj * W + ii];
			if (q.x != -1) {
				q.x += x - ii;
				q.y += y - jj;
				if (q.x >= 0 && q.y >= 0 && q.x < W && q.y < H &&
				    nli_in_bounds((long long)q.y * W + q.x, (long long)W * H, kSiteMeansSource)) {
					float w = u.weights[(jj - y_a) * u.px + (ii - x_a)];
					if (conf && dom[jj * W + ii]) w = fm(w, conf[jj * W + ii]);
					tw = fa(tw, w);
					const float *s = img + (size_t)C * (q.y * W + q.x);
					for (int c = 0; c < C; c++) tv[c] = fa(tv[c], fm(s[c], w));
				}
			}
		}
	for (int c = 0; c < C; c++) {
		const float prev = img[(size_t)C * pix + c];
		float v = prev;
		if (tw > 0.0f) {
			v = __fdiv_rn(tv[c], tw);
			const float d = fs(prev, v);
			acc += (double)fm(d, d);
		}
		out[c] = v;
	}
	return acc;
}

__global__ void __launch_bounds__(256) k_nlmeans(UpdArgs u, const float *__restrict__ img,
                                                 const int32_t *__restrict__ hole, int nh,
                                                 const uint8_t *__restrict__ dom, const int2 *__restrict__ nnf,
                                                 const float *__restrict__ conf, float *__restrict__ newval,
                                                 double *__restrict__ partials)
{
	__shared__ double red[8];
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	double acc = 0.0;
	if (i < nh) acc = nlmeans_pixel(u, u.W, u.H, u.C, img, hole[i], dom, nnf, conf, newval + (size_t)u.C * i);
	acc = block_sum<256>(acc, red);
	if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

__global__ void k_scatter_values(const int32_t *__restrict__ hole, int nh, int C, const float *__restrict__ newval,
                                 float *__restrict__ img)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= nh * C) return;
	const int k = i / C, c = i % C;
	img[(size_t)C * hole[k] + c] = newval[i];
}

// ------------------------------------------------------------ NL-medians
// One warp per hole pixel: the candidates of the 9x9 window are numbered
// in the reference's order (x outer, y inner, :61-62), ranked by value per
// channel with a warp-wide comparison (ties by candidate order), placed in
// shared memory in sorted order, and the weighted median is found by the
// reference's sequential subtraction (:110-127) in lane 0.
constexpr int kMedWarps = 4;

// Shared memory of one NL-medians warp.
struct MedSmem {
	float (*val)[kMaxTaps];  // [4][kMaxTaps] candidate values per channel
	float *w, *sv, *sw;       // weights, sorted values, their weights
};

// One hole pixel, computed by one whole warp: lane 0 writes the new values
// into out[0..C) and returns (u_old - u_new)^2 summed over the channels.
__device__ __forceinline__ double nlmedians_pixel(const UpdArgs &u, int W, int H, int C,
                                                  const float *__restrict__ img, int pix,
                                                  const uint8_t *__restrict__ dom, const int2 *__restrict__ nnf,
                                                  const float *__restrict__ conf, float *__restrict__ out, MedSmem sm)
{
	const int lane = threadIdx.x & 31;
	double acc = 0.0;
	if (!nli_in_bounds(pix, (long long)W * H, kSiteHole)) return 0.0;
	const int x = pix % W, y = pix / W;
	const int x_a = max(x - u.hx, 0), x_b = min(x + u.hx, W - 1);
	const int y_a = max(y - u.hy, 0), y_b = min(y + u.hy, H - 1);
	const int ny = y_b - y_a + 1;
	const int total = (x_b - x_a + 1) * ny;
	// collect valid candidates in reference order (compacted)
	int m = 0;
	for (int base = 0; base < total; base += 32) {
		const int k = base + lane;
		bool valid = false;
		float w = 0.f;
		int qx = 0, qy = 0;
		if (k < total) {
			const int ii = x_a + k / ny, jj = y_a + k % ny;
			int2 q = nnf[jj * W + ii];
			if (q.x != -1) {
				qx = q.x + x - ii;
				qy = q.y + y - jj;
				if (qx >= 0 && qy >= 0 && qx < W && qy < H &&
				    nli_in_bounds((long long)qy * W + qx, (long long)W * H, kSiteMeansSource)) {
					valid = true;
					w = u.weights[(jj - y_a) * u.px + (ii - x_a)];
					if (conf && dom[jj * W + ii]) w = fm(w, conf[jj * W + ii]);
				}
			}
		}
		const unsigned bal = __ballot_sync(0xffffffffu, valid);
		if (valid) {
			const int slot = m + __popc(bal & ((1u << lane) - 1u));
			sm.w[slot] = w;
			for (int c = 0; c < C; c++) sm.val[c][slot] = img[(size_t)C * (qy * W + qx) + c];
		}
		m += __popc(bal);
	}
	__syncwarp();
	if (m > 0) {
		// total weight, summed in candidate order (:80)
		float tw = 0.f;
		if (lane == 0)
			for (int k = 0; k < m; k++) tw = fa(tw, sm.w[k]);
		tw = __shfl_sync(0xffffffffu, tw, 0);
		for (int c = 0; c < C; c++) {
			for (int k = lane; k < m; k += 32) {
				const float v = sm.val[c][k];
				int rank = 0;
				for (int j = 0; j < m; j++) {
					const float o = sm.val[c][j];
					rank += (o < v || (o == v && j < k)) ? 1 : 0;
				}
				sm.sv[rank] = v;
				sm.sw[rank] = sm.w[k];
			}
			__syncwarp();
			if (lane == 0) {
				float median = 0.0f;
				float t = tw;
				const float half = tw / 2;
				for (int k = 0; k < m; k++) {
					t = fs(t, sm.sw[k]);
					if (t < half) {
						median = sm.sv[k];
						break;
					}
				}
				const float prev = img[(size_t)C * pix + c];
				const float d = fs(prev, median);
				acc += (double)fm(d, d);
				out[c] = median;
			}
			__syncwarp();
		}
	} else if (lane == 0) {
		for (int c = 0; c < C; c++) out[c] = img[(size_t)C * pix + c];
	}
	return acc;
}

// One warp per hole pixel: the candidates of the 9x9 window are numbered
// in the reference's order (x outer, y inner, :61-62), ranked by value per
// channel with a warp-wide comparison (ties by candidate order), placed in
// shared memory in sorted order, and the weighted median is found by the
// reference's sequential subtraction (:110-127) in lane 0.
__global__ void __launch_bounds__(32 * kMedWarps) k_nlmedians(UpdArgs u, const float *__restrict__ img,
                                                              const int32_t *__restrict__ hole, int nh,
                                                              const uint8_t *__restrict__ dom,
                                                              const int2 *__restrict__ nnf,
                                                              const float *__restrict__ conf,
                                                              float *__restrict__ newval, double *__restrict__ partials)
{
	__shared__ float s_val[kMedWarps][4][kMaxTaps];
	__shared__ float s_w[kMedWarps][kMaxTaps];
	__shared__ float s_sv[kMedWarps][kMaxTaps];
	__shared__ float s_sw[kMedWarps][kMaxTaps];
	__shared__ double red[kMedWarps];
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	const int i = blockIdx.x * kMedWarps + wid;
	double acc = 0.0;
	if (i < nh)
		acc = nlmedians_pixel(u, u.W, u.H, u.C, img, hole[i], dom, nnf, conf, newval + (size_t)u.C * i,
		                      MedSmem{s_val[wid], s_w[wid], s_sv[wid], s_sw[wid]});
	if (lane == 0) red[wid] = acc;
	__syncthreads();
	if (threadIdx.x == 0) {
		double t = 0.0;
		for (int w = 0; w < kMedWarps; w++) t += red[w];
		partials[blockIdx.x] = t;
	}
}

// ------------------------------------------------------------ NL-Poisson
// Coefficients of calculate_pde_coefficients (:139-232) as a gather: pixel
// q receives, from every extended-domain centre c whose window holds q
// (visited in raster order), w = conf(c) * g(q - c) and the image / gradient
// at n = nnf(c) + q - c when n lies in the image.  Stored unscaled:
//   S = sum w, U_c = sum w u_c(n), GX_c = sum w gx_c(n), GY_c = sum w gy_c(n);
// a1 = lambda S, a2 = (1-lambda) S, f1 = lambda U, F = (1-lambda) G.
// The pixels computed are the hole pixels and their left / upper
// neighbours (all that the right-hand side and the stencil read).
struct CoefOut {
	float *S;   // W*H
	float *U;   // W*H*C
	float *GX;  // W*H*C
	float *GY;  // W*H*C
};

__device__ __forceinline__ void gather_coef(const UpdArgs &u, int W, int H, int C, int qx, int qy,
                                            const uint8_t *__restrict__ ext, const int2 *__restrict__ nnf,
                                            const float *__restrict__ conf, const float *__restrict__ img,
                                            const float2 *__restrict__ grad, CoefOut out)
{
	float S = 0.f, U[4] = {0, 0, 0, 0}, GX[4] = {0, 0, 0, 0}, GY[4] = {0, 0, 0, 0};
	const int cy0 = max(qy - u.hy, 0), cy1 = min(qy + u.hy, H - 1);
	const int cx0 = max(qx - u.hx, 0), cx1 = min(qx + u.hx, W - 1);
	for (int cy = cy0; cy <= cy1; cy++)
		for (int cx = cx0; cx <= cx1; cx++) {
			const int c = cy * W + cx;
			if (!ext[c]) continue;
			const int2 nb = nnf[c];
			const int nx = nb.x + qx - cx, ny = nb.y + qy - cy;
			if (nx < 0 || ny < 0 || nx >= W || ny >= H) continue;
			float w = u.weights[(qy - cy + u.hy) * u.px + (qx - cx + u.hx)];
			if (conf) w = conf[c] * w;
			S += w;
			const float *iv = img + (size_t)C * (ny * W + nx);
			const float2 *gv = grad + (size_t)C * (ny * W + nx);
			for (int k = 0; k < C; k++) {
				U[k] = fmaf(w, iv[k], U[k]);
				const float2 g = gv[k];
				GX[k] = fmaf(w, g.x, GX[k]);
				GY[k] = fmaf(w, g.y, GY[k]);
			}
		}
	const int q = qy * W + qx;
	out.S[q] = S;
	for (int k = 0; k < C; k++) {
		out.U[(size_t)C * q + k] = U[k];
		out.GX[(size_t)C * q + k] = GX[k];
		out.GY[(size_t)C * q + k] = GY[k];
	}
}

// Hole pixel k and the neighbours it owns (see k_poisson_coef).
__device__ __forceinline__ void coef_hole_pixel(const UpdArgs &u, int W, int H, int C, int pix,
                                                const uint8_t *__restrict__ dom, const uint8_t *__restrict__ ext,
                                                const int2 *__restrict__ nnf, const float *__restrict__ conf,
                                                const float *__restrict__ img, const float2 *__restrict__ grad,
                                                CoefOut out)
{
	const int x = pix % W, y = pix / W;
	gather_coef(u, W, H, C, x, y, ext, nnf, conf, img, grad, out);
	// left neighbour: owned by this hole pixel when it is not a hole pixel
	if (x > 0 && !dom[pix - 1]) gather_coef(u, W, H, C, x - 1, y, ext, nnf, conf, img, grad, out);
	// upper neighbour: owned here when it is neither a hole pixel nor the left
	// neighbour of a hole pixel (then its right neighbour owns it)
	if (y > 0 && !dom[pix - W] && !(x + 1 < W && dom[pix - W + 1]))
		gather_coef(u, W, H, C, x, y - 1, ext, nnf, conf, img, grad, out);
}

__global__ void __launch_bounds__(128) k_poisson_coef(UpdArgs u, const int32_t *__restrict__ hole, int nh,
                                                      const uint8_t *__restrict__ dom,
                                                      const uint8_t *__restrict__ ext, const int2 *__restrict__ nnf,
                                                      const float *__restrict__ conf, const float *__restrict__ img,
                                                      const float2 *__restrict__ grad, CoefOut out)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= nh) return;
	coef_hole_pixel(u, u.W, u.H, u.C, hole[i], dom, ext, nnf, conf, img, grad, out);
}

// Item `item` (thread group of 8 lanes, `sub` = lane within the group).
__device__ __forceinline__ void coef8_item(const UpdArgs &u, int W, int H, int C, int item, int sub,
                                           const int32_t *__restrict__ hole, int nh, const uint8_t *__restrict__ dom,
                                           const uint8_t *__restrict__ ext, const int2 *__restrict__ nnf,
                                           const float *__restrict__ conf, const float *__restrict__ img,
                                           const float2 *__restrict__ grad, CoefOut out)
{
	bool owned = false;
	int qx = 0, qy = 0;
	if (item < 3 * nh) {
		const int k = item / 3, which = item - 3 * k;
		const int pix = hole[k];
		if (!nli_in_bounds(pix, (long long)W * H, kSiteHole)) return;  // the item's 8 lanes leave together
		const int x = pix % W, y = pix / W;
		if (which == 0) {
			owned = true;
			qx = x;
			qy = y;
		} else if (which == 1) {
			owned = x > 0 && !dom[pix - 1];
			qx = x - 1;
			qy = y;
		} else {
			owned = y > 0 && !dom[pix - W] && !(x + 1 < W && dom[pix - W + 1]);
			qx = x;
			qy = y - 1;
		}
	}
	// all 8 lanes of an item agree on `owned`; whole groups leave together
	if (!owned) return;
	const unsigned gmask = 0xffu << (threadIdx.x & 24);
	float S = 0.f, U[4] = {0, 0, 0, 0}, GX[4] = {0, 0, 0, 0}, GY[4] = {0, 0, 0, 0};
	const int taps = u.px * u.py;
	for (int t = sub; t < taps; t += 8) {
		const int ty = t / u.px, tx = t - ty * u.px;
		// centre c = q - (tap offset), tap offset = (tx - hx, ty - hy)
		const int cx = qx - (tx - u.hx), cy = qy - (ty - u.hy);
		if (cx < 0 || cy < 0 || cx >= W || cy >= H) continue;
		const int c = cy * W + cx;
		if (!ext[c]) continue;
		const int2 nb = nnf[c];
		const int nx = nb.x + qx - cx, ny = nb.y + qy - cy;
		if (nx < 0 || ny < 0 || nx >= W || ny >= H) continue;
		if (!nli_in_bounds((long long)ny * W + nx, (long long)W * H, kSiteCoefSource)) continue;
		float w = u.weights[t];
		if (conf) w = conf[c] * w;
		S += w;
		const float *iv = img + (size_t)C * (ny * W + nx);
		const float2 *gv = grad + (size_t)C * (ny * W + nx);
		for (int k = 0; k < C; k++) {
			U[k] = fmaf(w, iv[k], U[k]);
			const float2 g = gv[k];
			GX[k] = fmaf(w, g.x, GX[k]);
			GY[k] = fmaf(w, g.y, GY[k]);
		}
	}
#pragma unroll
	for (int o = 4; o > 0; o >>= 1) {
		S += __shfl_xor_sync(gmask, S, o);
#pragma unroll
		for (int k = 0; k < 4; k++) {
			if (k >= C) break;
			U[k] += __shfl_xor_sync(gmask, U[k], o);
			GX[k] += __shfl_xor_sync(gmask, GX[k], o);
			GY[k] += __shfl_xor_sync(gmask, GY[k], o);
		}
	}
	if (sub == 0) {
		const int q = qy * W + qx;
		out.S[q] = S;
		for (int k = 0; k < C; k++) {
			out.U[(size_t)C * q + k] = U[k];
			out.GX[(size_t)C * q + k] = GX[k];
			out.GY[(size_t)C * q + k] = GY[k];
		}
	}
}

// The same gather with 8 lanes per coefficient pixel: item (k, which) is
// hole pixel k itself (which 0), its left neighbour (1) or its upper
// neighbour (2) when that pixel is owned as in k_poisson_coef; lane j of
// the item's 8 takes window taps j, j + 8, ...; the 8 partial sums are
// added with shuffles.  Same terms as gather_coef, summed in a tree.
__global__ void __launch_bounds__(256) k_poisson_coef8(UpdArgs u, const int32_t *__restrict__ hole, int nh,
                                                       const uint8_t *__restrict__ dom,
                                                       const uint8_t *__restrict__ ext, const int2 *__restrict__ nnf,
                                                       const float *__restrict__ conf, const float *__restrict__ img,
                                                       const float2 *__restrict__ grad, CoefOut out)
{
	coef8_item(u, u.W, u.H, u.C, (blockIdx.x * blockDim.x + threadIdx.x) >> 3, threadIdx.x & 7, hole, nh, dom, ext,
	           nnf, conf, img, grad, out);
}

// Per unknown (hole pixel) data of the symmetric system
//   (a1 - div a2 grad) delta = b,  delta = 0 outside the hole,
// with the anisotropic Laplacian of calculate_anisotropic_laplacian
// (:291-356): links up/left take a2 of the neighbour, down/right take a2
// of the centre, links that leave the image are absent.
struct Unknown {
	float S;         // unscaled a1 / a2 at the centre
	float s_up, s_left, s_down, s_right;  // unscaled link coefficients (0 if no link)
	int n_up, n_left, n_down, n_right;    // unknown index of the neighbour, -1 if not a hole pixel
	// the same neighbours as (owning CTA << 20) | index within its range,
	// for the cluster kernel (-1 if not a hole pixel)
	int c_up, c_left, c_down, c_right;
	int links;  // bit 0: down link inside the image, bit 1: right link inside the image
};

struct PoissonArgs {
	int W, H, C, nh;
	float lambda[4];
	float tol;
	int limit;
};

// Right-hand side b and initial perturbation delta0 = image - orig
// (patch_non_local_poisson.cpp:62-82), and the per-unknown system data.
__device__ __forceinline__ void poisson_setup_unknown(const PoissonArgs &a, int chunk, int k,
                                                      const int32_t *__restrict__ hole,
                                                      const int32_t *__restrict__ hole_index, CoefOut co,
                                                      const float *__restrict__ img, const float *__restrict__ orig,
                                                      Unknown *__restrict__ unk, float *__restrict__ b,
                                                      float *__restrict__ x0)
{
	const int W = a.W, H = a.H, C = a.C;
	const int pix = hole[k];
	const int x = pix % W, y = pix / W;
	Unknown n;
	n.S = co.S[pix];
	n.s_up = (y != 0) ? co.S[pix - W] : 0.f;
	n.s_left = (x != 0) ? co.S[pix - 1] : 0.f;
	n.s_down = (y != H - 1) ? n.S : 0.f;
	n.s_right = (x != W - 1) ? n.S : 0.f;
	n.n_up = (y != 0) ? hole_index[pix - W] : -1;
	n.n_left = (x != 0) ? hole_index[pix - 1] : -1;
	n.n_down = (y != H - 1) ? hole_index[pix + W] : -1;
	n.n_right = (x != W - 1) ? hole_index[pix + 1] : -1;
	auto code = [chunk](int m) { return (m >= 0 && chunk > 0) ? ((m / chunk) << 20) | (m % chunk) : -1; };
	n.c_up = code(n.n_up);
	n.c_left = code(n.n_left);
	n.c_down = code(n.n_down);
	n.c_right = code(n.n_right);
	n.links = ((y != H - 1) ? 1 : 0) | ((x != W - 1) ? 2 : 0);
	unk[k] = n;
	for (int c = 0; c < C; c++) {
		const float lam = a.lambda[c], oml = 1.0f - lam;
		const float a1 = lam * n.S;
		const float f1 = lam * co.U[(size_t)C * pix + c];
		// backward divergence of F = (1-lambda) G on the domain (:235-285)
		float f2 = 0.f;
		if (lam != 1.0f) {
			const float fx = oml * co.GX[(size_t)C * pix + c];
			const float fy = oml * co.GY[(size_t)C * pix + c];
			const float fxl = (x > 0) ? oml * co.GX[(size_t)C * (pix - 1) + c] : 0.f;
			const float fyu = (y > 0) ? oml * co.GY[(size_t)C * (pix - W) + c] : 0.f;
			f2 = (x == 0) ? fx : (x == W - 1) ? -fxl : fx - fxl;
			f2 += (y == 0) ? fy : (y == H - 1) ? -fyu : fy - fyu;
		}
		// anisotropic Laplacian of the original image at the hole pixel
		const float o = orig[(size_t)C * pix + c];
		const float ou = (y != 0) ? orig[(size_t)C * (pix - W) + c] : 0.f;
		const float ol = (x != 0) ? orig[(size_t)C * (pix - 1) + c] : 0.f;
		const float od = (y != H - 1) ? orig[(size_t)C * (pix + W) + c] : 0.f;
		const float orr = (x != W - 1) ? orig[(size_t)C * (pix + 1) + c] : 0.f;
		const float lap = oml * (n.s_up * ou + n.s_left * ol + n.s_down * od + n.s_right * orr -
		                         o * (n.s_up + n.s_left + n.s_down + n.s_right));
		b[(size_t)c * a.nh + k] = f1 - f2 - a1 * o + lap;
		x0[(size_t)c * a.nh + k] = img[(size_t)C * pix + c] - o;
	}
}

__global__ void k_poisson_setup(PoissonArgs a, int chunk, const int32_t *__restrict__ hole,
                                const int32_t *__restrict__ hole_index, CoefOut co, const float *__restrict__ img,
                                const float *__restrict__ orig, Unknown *__restrict__ unk, float *__restrict__ b,
                                float *__restrict__ x0)
{
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= a.nh) return;
	poisson_setup_unknown(a, chunk, k, hole, hole_index, co, img, orig, unk, b, x0);
}

__device__ __forceinline__ float apply_A(const Unknown &n, float lam, const float *__restrict__ v, float vk)
{
	const float vu = (n.n_up >= 0) ? __ldcg(v + n.n_up) : 0.f;
	const float vl = (n.n_left >= 0) ? __ldcg(v + n.n_left) : 0.f;
	const float vd = (n.n_down >= 0) ? __ldcg(v + n.n_down) : 0.f;
	const float vr = (n.n_right >= 0) ? __ldcg(v + n.n_right) : 0.f;
	const float sum = n.s_up + n.s_left + n.s_down + n.s_right;
	const float lap = n.s_up * vu + n.s_left * vl + n.s_down * vd + n.s_right * vr - vk * sum;
	return lam * n.S * vk - (1.0f - lam) * lap;
}

constexpr int kCgBlock = 512;

// Deterministic grid reduction of the first nv of 8 values per block:
// every block sums the per-block partials in the same order, so all blocks
// see identical totals.
__device__ __forceinline__ void reduce_partials(const double *__restrict__ part, int nblocks, int nv, double *out,
                                                double *smem)
{
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	if (wid < nv) {
		double v = 0.0;
		for (int b = lane; b < nblocks; b += 32) v += __ldcg(part + (size_t)b * 8 + wid);
		v = warp_sum(v);
		if (lane == 0) smem[wid] = v;
	}
	__syncthreads();
	for (int c = 0; c < nv; c++) out[c] = smem[c];
	__syncthreads();
}

// Jacobi preconditioner of a row of the grid kernel's system (see
// jacobi_inv of the cluster kernel).
__device__ __forceinline__ float jacobi_inv_grid(const Unknown &n, float lam)
{
	const float dg = lam * n.S + (1.0f - lam) * (n.s_up + n.s_left + n.s_down + n.s_right);
	return (dg > 0.f) ? 1.0f / dg : 1.0f;
}

// Conjugate gradient of conjugte_gradient (:387-477) for all channels at
// once: r = b - A x0, d = r; per iteration q = A d, alpha = |r|^2 / <r,q>,
// x += alpha d, r -= alpha q, beta = |r_new|^2 / |r|^2, d = r + beta d; a
// channel stops when |r|^2 < tol |r0|^2 or after `limit` iterations.
// Vectors are float, inner products double.  The grid is co-resident
// (cooperative launch) and phases are separated by the bounded barrier.
// Ends by writing u = orig + x into the image and the partial sums of
// (u_old - u_new)^2.  PRE: Jacobi-preconditioned as the cluster kernel
// (z = M r kept in `z`, d = z + beta d, alpha = <r, z> / <z, q>), same
// stopping test.
template <bool PRE>
__global__ void __launch_bounds__(kCgBlock) k_poisson_cg(PoissonArgs a, const Unknown *__restrict__ unk,
                                                         const float *__restrict__ b, float *__restrict__ x,
                                                         float *__restrict__ r, float *__restrict__ d,
                                                         float *__restrict__ q, float *__restrict__ z,
                                                         double *__restrict__ part, DevStatus *st,
                                                         int *__restrict__ iters_out,
                                                         const int32_t *__restrict__ hole,
                                                         const float *orig, float *img,
                                                         double *__restrict__ diff_part,
                                                         const int *__restrict__ active_flag)
{
	// a batch image that has stopped iterating: every block leaves at once
	if (active_flag && *active_flag == 0) return;
	__shared__ double red[kCgBlock / 32][8];
	__shared__ double tot[8];
	const int nh = a.nh, C = a.C;
	const int NV = PRE ? 2 * C : C;  // sums of the residual phase: |r|^2 (and <r, z>)
	const unsigned nb = gridDim.x;
	const int stride = gridDim.x * blockDim.x;
	double *partA = part;                   // [nb][8]
	double *partB = part + (size_t)nb * 8;  // [nb][8]
	if (!PRE) z = r;

	auto block_partial = [&](double *v, double *dst, int nv) {
		// v[nv] per thread -> dst[blockIdx.x][c]
		const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
		for (int c = 0; c < nv; c++) {
			double s = warp_sum(v[c]);
			if (lane == 0) red[wid][c] = s;
		}
		__syncthreads();
		if (threadIdx.x < nv) {
			double s = 0.0;
			for (int w = 0; w < kCgBlock / 32; w++) s += red[w][threadIdx.x];
			__stcg(dst + (size_t)blockIdx.x * 8 + threadIdx.x, s);
		}
		__syncthreads();
	};

	// r = b - A x0 ; z = M r ; d = z ; |r0|^2 (and <r0, z0>)
	double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nh; k += stride) {
		const Unknown n = unk[k];
		for (int c = 0; c < C; c++) {
			const float *xc = x + (size_t)c * nh;
			const float rv = b[(size_t)c * nh + k] - apply_A(n, a.lambda[c], xc, __ldcg(xc + k));
			__stcg(r + (size_t)c * nh + k, rv);
			acc[c] += (double)rv * rv;
			float zv = rv;
			if (PRE) {
				zv = jacobi_inv_grid(n, a.lambda[c]) * rv;
				__stcg(z + (size_t)c * nh + k, zv);
				acc[C + c] += (double)rv * zv;
			}
			__stcg(d + (size_t)c * nh + k, zv);
		}
	}
	block_partial(acc, partB, NV);
	if (!grid_barrier(st, nb)) return;
	double nr0[4], nr[4], rho[4], t8[8];
	reduce_partials(partB, nb, NV, t8, &tot[0]);
	bool active[4];
	int it[4];
	for (int c = 0; c < 4; c++) {
		nr0[c] = (c < C) ? t8[c] : 0.0;
		nr[c] = nr0[c];
		rho[c] = (c < C) ? (PRE ? t8[C + c] : t8[c]) : 0.0;
		active[c] = (c < C) && (nr0[c] > 0);
		it[c] = 0;
	}
	for (;;) {
		bool any = false;
		for (int c = 0; c < C; c++) any |= active[c];
		if (!any) break;
		// q = A d ; <z, q>
		for (int c = 0; c < 8; c++) acc[c] = 0.0;
		for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nh; k += stride) {
			const Unknown n = unk[k];
			for (int c = 0; c < C; c++) {
				if (!active[c]) continue;
				const float *dc = d + (size_t)c * nh;
				const float qv = apply_A(n, a.lambda[c], dc, __ldcg(dc + k));
				__stcg(q + (size_t)c * nh + k, qv);
				acc[c] += (double)__ldcg(z + (size_t)c * nh + k) * qv;
			}
		}
		block_partial(acc, partA, C);
		if (!grid_barrier(st, nb)) return;
		double rq[8];
		reduce_partials(partA, nb, C, rq, &tot[0]);
		float alpha[4];
		for (int c = 0; c < C; c++) alpha[c] = active[c] ? (float)(rho[c] / rq[c]) : 0.f;
		// x += alpha d ; r -= alpha q ; z = M r ; |r|^2 (and <r, z>)
		for (int c = 0; c < 8; c++) acc[c] = 0.0;
		for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nh; k += stride) {
			Unknown n;
			if (PRE) n = unk[k];
			for (int c = 0; c < C; c++) {
				if (!active[c]) continue;
				const size_t o = (size_t)c * nh + k;
				const float dv = __ldcg(d + o);
				__stcg(x + o, __ldcg(x + o) + alpha[c] * dv);
				const float rv = __ldcg(r + o) - alpha[c] * __ldcg(q + o);
				__stcg(r + o, rv);
				acc[c] += (double)rv * rv;
				if (PRE) {
					const float zv = jacobi_inv_grid(n, a.lambda[c]) * rv;
					__stcg(z + o, zv);
					acc[C + c] += (double)rv * zv;
				}
			}
		}
		block_partial(acc, partB, NV);
		if (!grid_barrier(st, nb)) return;
		double nrn[8];
		reduce_partials(partB, nb, NV, nrn, &tot[0]);
		float beta[4];
		for (int c = 0; c < C; c++) {
			const double rhon = PRE ? nrn[C + c] : nrn[c];
			beta[c] = active[c] ? (float)(rhon / rho[c]) : 0.f;
			if (active[c]) {
				nr[c] = nrn[c];
				rho[c] = rhon;
			}
		}
		// d = z + beta d
		for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nh; k += stride) {
			for (int c = 0; c < C; c++) {
				if (!active[c]) continue;
				const size_t o = (size_t)c * nh + k;
				__stcg(d + o, __ldcg(z + o) + beta[c] * __ldcg(d + o));
			}
		}
		for (int c = 0; c < C; c++) {
			if (!active[c]) continue;
			const bool stop = (nr[c] < (double)a.tol * nr0[c]) || (it[c] >= a.limit);
			it[c]++;
			if (stop) active[c] = false;
		}
		if (!grid_barrier(st, nb)) return;
	}
	if (blockIdx.x == 0 && threadIdx.x < C) iters_out[threadIdx.x] = it[threadIdx.x];
	// u = orig + delta on the hole (:89-104)
	double dacc = 0.0;
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nh; k += stride) {
		const int pix = hole[k];
		for (int c = 0; c < C; c++) {
			const float o = orig[(size_t)C * pix + c];
			const float v = o + __ldcg(x + (size_t)c * nh + k);
			const float prev = img[(size_t)C * pix + c];
			const float dd = prev - v;
			dacc += (double)(dd * dd);
			img[(size_t)C * pix + c] = v;
		}
	}
	dacc = block_sum<kCgBlock>(dacc, &red[0][0]);
	if (threadIdx.x == 0) diff_part[blockIdx.x] = dacc;
}

// Conjugate gradient on thread-block clusters with every vector and the
// system itself in shared memory.  Cluster g of the grid solves channels
// [g * C, (g + 1) * C) of the Ctot-channel image; the channels are
// independent systems (the reference solves them one after the other), so
// one cluster per channel (C = 1) spreads the solve over more SMs and lets
// each channel stop at its own convergence.
//
// CTA `rank` of the cluster (up to 16 CTAs of 512 threads) owns the
// contiguous unknown range [rank * chunk, (rank + 1) * chunk), chunk <=
// 4096, and keeps in its shared memory the residual r, two alternating
// direction buffers, the solution x and a compact 24-byte record per
// unknown (its coefficients and 16-bit neighbour codes: owning CTA << 12 |
// index); q = A d stays in registers.  Neighbours owned by another CTA are
// read through distributed shared memory.  Iteration (as the reference's
// conjugte_gradient, patch_non_local_poisson.cpp:387-477, with the
// residual updated by recurrence): d = r + beta d_old (folded into the
// stencil phase, formed at the neighbours from r and d_old), q = A d,
// alpha = |r|^2 / <r, q>, x += alpha d, r -= alpha q, beta = |r'|^2 / |r|^2.
// Two cluster barriers per iteration; block partial sums are exchanged
// through distributed shared memory and added in rank order by one warp,
// so every CTA holds the same totals.  alpha and beta are formed once per
// CTA in double precision by that warp and published with one block
// barrier.  (Pushing the partials into every CTA before the barrier, so
// that the totals are read locally, measured no faster.)
constexpr int kClusterBlock = 512;
constexpr int kClusterMax = 16;
constexpr int kClusterMaxChunk = 4096;
constexpr int kClusterPerThread = kClusterMaxChunk / kClusterBlock;  // unknowns per thread
constexpr int kClusterVectors = 4;  // r, d (twice), x
constexpr int kNoNb = 0xFFFF;

struct UnkC {
	float S, s_up, s_left;
	uint32_t ud;     // up code << 16 | down code
	uint32_t lr;     // left code << 16 | right code
	uint32_t links;  // bit 0: down link inside the image, bit 1: right link inside the image
};

__device__ __forceinline__ void poisson_compact_unknown(const Unknown *__restrict__ unk, int k, int chunk,
                                                        UnkC *__restrict__ out)
{
	const Unknown n = unk[k];
	auto code = [chunk](int m) -> uint32_t {
		return (m >= 0) ? (uint32_t)(((m / chunk) << 12) | (m % chunk)) : (uint32_t)kNoNb;
	};
	UnkC c;
	c.S = n.S;
	c.s_up = n.s_up;
	c.s_left = n.s_left;
	c.ud = (code(n.n_up) << 16) | code(n.n_down);
	c.lr = (code(n.n_left) << 16) | code(n.n_right);
	c.links = (uint32_t)n.links;
	out[k] = c;
}

__global__ void k_poisson_compact(const Unknown *__restrict__ unk, int nh, int chunk, UnkC *__restrict__ out)
{
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= nh) return;
	poisson_compact_unknown(unk, k, chunk, out);
}

// 1 / the diagonal of an unknown's row, lam S + (1 - lam) (sum of its four
// link coefficients) (1 where that is not positive): the Jacobi
// preconditioner of the PRE kernels.
__device__ __forceinline__ float jacobi_inv(const UnkC &n, float lam)
{
	const float sum = n.s_up + n.s_left + ((n.links & 1) ? n.S : 0.f) + ((n.links & 2) ? n.S : 0.f);
	const float dg = lam * n.S + (1.0f - lam) * sum;
	return (dg > 0.f) ? 1.0f / dg : 1.0f;
}

// PRE: Jacobi-preconditioned CG (NLI_TUNE_CG_PRECOND): z = M r with M the
// inverse diagonal, d = z + beta d_old, alpha = <r, z> / <z, A d>, beta =
// <r', z'> / <r, z>.  The stopping test stays |r|^2 < tol |r0|^2 on the
// true residual, so the solve ends at the same residual as the plain CG,
// in fewer iterations.  Without PRE, z is r itself and the iteration is the
// reference's.
// The CTAs that solve one system: a thread-block cluster (barriers and
// distributed shared memory), or one CTA on its own (block barriers, its
// own shared memory) for systems of at most kClusterMaxChunk unknowns.  The
// one-CTA form performs the same arithmetic in the same order as a
// cluster of one CTA.
template <bool SINGLE>
struct CgTeam;

template <>
struct CgTeam<true> {
	__device__ int rank() const { return 0; }
	__device__ int size() const { return 1; }
	__device__ void sync() { __syncthreads(); }
	template <class T>
	__device__ T *map(T *p, int) const
	{
		return p;
	}
};

template <>
struct CgTeam<false> {
	cooperative_groups::cluster_group c;
	__device__ CgTeam() : c(cooperative_groups::this_cluster()) {}
	__device__ int rank() const { return (int)c.block_rank(); }
	__device__ int size() const { return (int)c.num_blocks(); }
	__device__ void sync() { c.sync(); }
	template <class T>
	__device__ T *map(T *p, int r)
	{
		return c.map_shared_rank(p, r);
	}
};

// The solve of channel group `group` (channels [group * C, (group + 1) * C)
// of the a.C-channel image) by the team's CTAs.
template <int C, bool PRE, bool SINGLE>
__device__ __forceinline__ void cg_team_solve(const PoissonArgs &a, int chunk, const UnkC *__restrict__ unk_g,
                                              const float *__restrict__ b, const float *__restrict__ x0,
                                              int *__restrict__ iters_out, const int32_t *__restrict__ hole,
                                              const float *orig, float *img, double *__restrict__ diff_part, int group)
{
	constexpr int NV = PRE ? 2 * C : C;  // sums of the residual phase: |r|^2 (and <r, z>)
	const int Ctot = a.C;
	CgTeam<SINGLE> cluster;
	extern __shared__ float smem[];
	__shared__ double red[kClusterBlock / 32][8];
	__shared__ double partA[8], partB[8], tot[8];
	__shared__ float s_coef[4];
	__shared__ int s_active[4];
	__shared__ double s_nr[4], s_rho[4];
	__shared__ float *base[3][kClusterMax];  // z (r without PRE), dA, dB of every CTA
	const int rank = cluster.rank(), ncta = cluster.size();
	const int cb = group * C;  // this cluster's first channel
	b += (size_t)cb * a.nh;
	x0 += (size_t)cb * a.nh;
	const int nh = a.nh;
	const int lo = rank * chunk, own = max(0, min(nh, lo + chunk) - lo);
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	const size_t vlen = (size_t)C * chunk;
	float *s_r = smem, *s_dA = smem + vlen, *s_dB = smem + 2 * vlen, *s_x = smem + 3 * vlen;
	float *s_z = PRE ? smem + 4 * vlen : s_r;
	UnkC *s_unk = reinterpret_cast<UnkC *>(smem + (kClusterVectors + (PRE ? 1 : 0)) * vlen);
	if (threadIdx.x < ncta) {
		base[0][threadIdx.x] = cluster.map(s_z, (int)threadIdx.x);
		base[1][threadIdx.x] = cluster.map(s_dA, (int)threadIdx.x);
		base[2][threadIdx.x] = cluster.map(s_dB, (int)threadIdx.x);
	}
	for (int l = threadIdx.x; l < own; l += blockDim.x) s_unk[l] = unk_g[lo + l];
	__syncthreads();

	// block partial sums of the first nv values into dst (written by warp 0;
	// read by the other CTAs after the next cluster barrier)
	auto block_reduce = [&](const float *v, double *dst, int nv) {
#pragma unroll
		for (int c = 0; c < NV; c++) {
			if (c >= nv) break;
			const float s = warp_sum(v[c]);
			if (lane == 0) red[wid][c] = (double)s;
		}
		__syncthreads();
		if (wid == 0) {
#pragma unroll
			for (int c = 0; c < NV; c++) {
				if (c >= nv) break;
				const double s = warp_sum((lane < kClusterBlock / 32) ? red[lane][c] : 0.0);
				if (lane == 0) dst[c] = s;
			}
		}
	};
	// cluster totals of the first nv block partials src, in rank order, left
	// in every lane of warp 0 (call from warp 0 only, after a cluster barrier)
	auto warp0_totals = [&](const double *src, double *out, int nv) {
#pragma unroll
		for (int c = 0; c < NV; c++) {
			if (c >= nv) break;
			const double v = warp_sum((lane < ncta) ? cluster.map(const_cast<double *>(src), lane)[c] : 0.0);
			out[c] = __shfl_sync(0xffffffffu, v, 0);
		}
	};
	// channel values of vector `v` (0: z, 1: dA, 2: dB) at a 16-bit code
	auto nb = [&](int v, uint32_t code) -> const float * {
		const int o = (int)(code >> 12), l = (int)(code & 0xFFF);
		const float *bp = (o == rank) ? (v == 0 ? s_z : v == 1 ? s_dA : s_dB) : base[v][o];
		return bp + (size_t)l * C;
	};

	// r0 = b - A x0 (x0 from global: neighbours may belong to other CTAs)
	float facc[8];
#pragma unroll
	for (int c = 0; c < 8; c++) facc[c] = 0.f;
	for (int l = threadIdx.x; l < own; l += blockDim.x) {
		const int k = lo + l;
		const UnkC n = s_unk[l];
		const uint32_t codes[4] = {n.ud >> 16, n.lr >> 16, n.ud & 0xFFFF, n.lr & 0xFFFF};
		const float coefs[4] = {n.s_up, n.s_left, (n.links & 1) ? n.S : 0.f, (n.links & 2) ? n.S : 0.f};
		const float sum = coefs[0] + coefs[1] + coefs[2] + coefs[3];
		int gk[4];
#pragma unroll
		for (int j = 0; j < 4; j++) {
			gk[j] = (codes[j] != kNoNb) ? (int)(codes[j] >> 12) * chunk + (int)(codes[j] & 0xFFF) : -1;
			if (gk[j] >= 0 && !nli_in_bounds(gk[j], nh, kSiteCgNeighbour)) gk[j] = -1;
		}
#pragma unroll
		for (int c = 0; c < C; c++) {
			const float *xc = x0 + (size_t)c * nh;
			const float xk = xc[k];
			float lap = -xk * sum;
#pragma unroll
			for (int j = 0; j < 4; j++)
				if (gk[j] >= 0) lap += coefs[j] * xc[gk[j]];
			const float rv = b[(size_t)c * nh + k] - (a.lambda[cb + c] * n.S * xk - (1.0f - a.lambda[cb + c]) * lap);
			s_r[(size_t)l * C + c] = rv;
			s_dA[(size_t)l * C + c] = 0.f;
			s_x[(size_t)l * C + c] = xk;
			facc[c] = fmaf(rv, rv, facc[c]);
			if (PRE) {
				const float zv = jacobi_inv(n, a.lambda[cb + c]) * rv;
				s_z[(size_t)l * C + c] = zv;
				facc[C + c] = fmaf(rv, zv, facc[C + c]);
			}
		}
	}
	block_reduce(facc, partB, NV);
	cluster.sync();
	double nr0[4], nr[4], rho[4];
	if (wid == 0) {
		double t[8];
		warp0_totals(partB, t, NV);
		if (lane == 0)
			for (int c = 0; c < NV; c++) tot[c] = t[c];
	}
	__syncthreads();
#pragma unroll
	for (int c = 0; c < C; c++) {
		nr0[c] = tot[c];
		rho[c] = PRE ? tot[C + c] : tot[c];
	}
	bool active[4];
	int it[4];
	float beta[4];
#pragma unroll
	for (int c = 0; c < 4; c++) {
		nr[c] = (c < C) ? nr0[c] : 0.0;
		if (c >= C) rho[c] = 0.0;
		active[c] = (c < C) && (nr0[c] > 0);
		it[c] = 0;
		beta[c] = 0.f;
	}
	int h = 0;  // direction buffer holding d_old: 0 -> dA, 1 -> dB
	float q[kClusterPerThread][C];
	for (;;) {
		bool any = false;
#pragma unroll
		for (int c = 0; c < C; c++) any |= active[c];
		if (!any) break;
		float *dold = h ? s_dB : s_dA, *dnew = h ? s_dA : s_dB;
		// d = z + beta d_old (own and neighbours) ; q = A d ; <z, q>
#pragma unroll
		for (int c = 0; c < 8; c++) facc[c] = 0.f;
#pragma unroll
		for (int u = 0; u < kClusterPerThread; u++) {
			const int l = threadIdx.x + u * kClusterBlock;
			if (l >= own) break;
			const UnkC n = s_unk[l];
			const uint32_t codes[4] = {n.ud >> 16, n.lr >> 16, n.ud & 0xFFFF, n.lr & 0xFFFF};
			const float coefs[4] = {n.s_up, n.s_left, (n.links & 1) ? n.S : 0.f, (n.links & 2) ? n.S : 0.f};
			const float sum = coefs[0] + coefs[1] + coefs[2] + coefs[3];
			const float *nr_[4], *nd_[4];
			bool has[4];
#pragma unroll
			for (int j = 0; j < 4; j++) {
				// a checked build tests the code's owning CTA and index
				has[j] = codes[j] != kNoNb &&
				         nli_in_bounds((long long)(codes[j] >> 12) * chunk + (codes[j] & 0xFFF),
				                       (long long)ncta * chunk, kSiteCgNeighbour) &&
				         nli_in_bounds(codes[j] & 0xFFF, chunk, kSiteCgNeighbour);
				nr_[j] = has[j] ? nb(0, codes[j]) : nullptr;
				nd_[j] = has[j] ? nb(1 + h, codes[j]) : nullptr;
			}
#pragma unroll
			for (int c = 0; c < C; c++) {
				if (!active[c]) continue;
				const size_t o = (size_t)l * C + c;
				const float rk = s_z[o];
				const float dk = rk + beta[c] * dold[o];
				float lap = -dk * sum;
#pragma unroll
				for (int j = 0; j < 4; j++)
					if (has[j]) lap += coefs[j] * (nr_[j][c] + beta[c] * nd_[j][c]);
				const float qv = a.lambda[cb + c] * n.S * dk - (1.0f - a.lambda[cb + c]) * lap;
				dnew[o] = dk;
				q[u][c] = qv;
				facc[c] = fmaf(rk, qv, facc[c]);
			}
		}
		block_reduce(facc, partA, C);
		cluster.sync();
		if (wid == 0) {
			double rq[4];
			warp0_totals(partA, rq, C);
#pragma unroll
			for (int c = 0; c < C; c++)
				if (lane == c) s_coef[c] = active[c] ? (float)(rho[c] / rq[c]) : 0.f;
		}
		__syncthreads();
		float alpha[4];
#pragma unroll
		for (int c = 0; c < C; c++) alpha[c] = s_coef[c];
		// x += alpha d ; r -= alpha q ; z = M r ; |r|^2 (and <r, z>)   (own unknowns only)
#pragma unroll
		for (int c = 0; c < 8; c++) facc[c] = 0.f;
#pragma unroll
		for (int u = 0; u < kClusterPerThread; u++) {
			const int l = threadIdx.x + u * kClusterBlock;
			if (l >= own) break;
			float minv[C];
			if (PRE) {
				const UnkC n = s_unk[l];
#pragma unroll
				for (int c = 0; c < C; c++) minv[c] = jacobi_inv(n, a.lambda[cb + c]);
			}
#pragma unroll
			for (int c = 0; c < C; c++) {
				if (!active[c]) continue;
				const size_t o = (size_t)l * C + c;
				s_x[o] += alpha[c] * dnew[o];
				const float rv = s_r[o] - alpha[c] * q[u][c];
				s_r[o] = rv;
				facc[c] = fmaf(rv, rv, facc[c]);
				if (PRE) {
					const float zv = minv[c] * rv;
					s_z[o] = zv;
					facc[C + c] = fmaf(rv, zv, facc[C + c]);
				}
			}
		}
		// partA / partB are rewritten only after the next cluster barrier,
		// by which time every CTA has read them
		block_reduce(facc, partB, NV);
		cluster.sync();
		if (wid == 0) {
			double nrn[8];
			warp0_totals(partB, nrn, NV);
#pragma unroll
			for (int c = 0; c < C; c++)
				if (lane == c && active[c]) {
					const double rhon = PRE ? nrn[C + c] : nrn[c];
					s_coef[c] = (float)(rhon / rho[c]);
					s_rho[c] = rhon;
					s_nr[c] = nrn[c];
					s_active[c] = ((nrn[c] < (double)a.tol * nr0[c]) || (it[c] >= a.limit)) ? 0 : 1;
				}
		}
		__syncthreads();
		// s_coef, s_nr and s_active are rewritten by warp 0 only after the
		// next block barrier, by which time every thread has read them
#pragma unroll
		for (int c = 0; c < C; c++) {
			if (!active[c]) continue;
			beta[c] = s_coef[c];
			nr[c] = s_nr[c];
			rho[c] = s_rho[c];
			it[c]++;
			active[c] = s_active[c] != 0;
		}
		h = 1 - h;
	}
	if (rank == 0 && threadIdx.x < C) iters_out[cb + threadIdx.x] = it[threadIdx.x];
	// u = orig + delta on the hole (:89-104)
	double dacc = 0.0;
	for (int l = threadIdx.x; l < own; l += blockDim.x) {
		const int pix = hole[lo + l];
#pragma unroll
		for (int c = 0; c < C; c++) {
			const float o = orig[(size_t)Ctot * pix + cb + c];
			const float v = o + s_x[(size_t)l * C + c];
			const float prev = img[(size_t)Ctot * pix + cb + c];
			const float dd = prev - v;
			dacc += (double)(dd * dd);
			img[(size_t)Ctot * pix + cb + c] = v;
		}
	}
	dacc = block_sum<kClusterBlock>(dacc, &red[0][0]);
	if (threadIdx.x == 0) diff_part[group * ncta + rank] = dacc;
	cluster.sync();  // no CTA leaves while others may still read its shared memory
}

template <int C, bool PRE>
__global__ void __launch_bounds__(kClusterBlock, 1)
    k_poisson_cg_cluster(PoissonArgs a, int chunk, const UnkC *__restrict__ unk_g, const float *__restrict__ b,
                         const float *__restrict__ x0, int *__restrict__ iters_out, const int32_t *__restrict__ hole,
                         const float *orig, float *img, double *__restrict__ diff_part)
{
	const int ncta = (int)cooperative_groups::this_cluster().num_blocks();
	cg_team_solve<C, PRE, false>(a, chunk, unk_g, b, x0, iters_out, hole, orig, img, diff_part,
	                             (int)blockIdx.x / ncta);
}

// One CTA per channel (systems of at most kClusterMaxChunk unknowns).
template <int C, bool PRE>
__global__ void __launch_bounds__(kClusterBlock, 1)
    k_poisson_cg_cta(PoissonArgs a, int chunk, const UnkC *__restrict__ unk_g, const float *__restrict__ b,
                     const float *__restrict__ x0, int *__restrict__ iters_out, const int32_t *__restrict__ hole,
                     const float *orig, float *img, double *__restrict__ diff_part)
{
	cg_team_solve<C, PRE, true>(a, chunk, unk_g, b, x0, iters_out, hole, orig, img, diff_part, (int)blockIdx.x);
}

__global__ void k_hole_index(const int32_t *__restrict__ hole, int nh, int32_t *__restrict__ index)
{
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k < nh) index[hole[k]] = k;
}

__global__ void k_fill_int(int32_t *p, int n, int v)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = v;
}

NLI_CHECK_READER(check_word_update)

static double read_total(nli_ctx *ctx, double *partials, int n, int *cg_iters_dev, int C, int nh = 0)
{
	launch_sum_partials(ctx->stream, partials, n, partials + n);
	char *h = static_cast<char *>(ctx->host_pinned);
	NLI_CUDA(cudaMemcpyAsync(h, partials + n, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
	if (cg_iters_dev)
		NLI_CUDA(cudaMemcpyAsync(h + 64, cg_iters_dev, sizeof(int) * 4, cudaMemcpyDeviceToHost, ctx->stream));
	// timeouts of the waits of this iteration's kernels (PatchMatch's tensor
	// copies, CG grid barriers)
	NLI_CUDA(cudaMemcpyAsync(h + 128, &ctx->status->timeout, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
	NLI_CUDA(cudaStreamSynchronize(ctx->stream));
	if (*reinterpret_cast<const int *>(h + 128) != 0) {
		clear_timeout(ctx);
		NLI_REQUIRE(false, NLI_E_TIMEOUT, "a device-side wait timed out");
	}
	if (cg_iters_dev) {
		const int *it = reinterpret_cast<const int *>(h + 64);
		for (int c = 0; c < C; c++) {
			ctx->cg_iterations += it[c];
			ctx->cg_unknown_iterations += (int64_t)it[c] * nh;
		}
	}
	return *reinterpret_cast<double *>(h);
}

static void (*cluster_kernel(int CC, bool pre))(PoissonArgs, int, const UnkC *, const float *, const float *, int *,
                                                const int32_t *, const float *, float *, double *)
{
	if (pre)
		return (CC == 1)   ? k_poisson_cg_cluster<1, true>
		       : (CC == 2) ? k_poisson_cg_cluster<2, true>
		       : (CC == 3) ? k_poisson_cg_cluster<3, true>
		                   : k_poisson_cg_cluster<4, true>;
	return (CC == 1)   ? k_poisson_cg_cluster<1, false>
	       : (CC == 2) ? k_poisson_cg_cluster<2, false>
	       : (CC == 3) ? k_poisson_cg_cluster<3, false>
	                   : k_poisson_cg_cluster<4, false>;
}

static void (*cta_kernel(int CC, bool pre))(PoissonArgs, int, const UnkC *, const float *, const float *, int *,
                                            const int32_t *, const float *, float *, double *)
{
	if (pre)
		return (CC == 1)   ? k_poisson_cg_cta<1, true>
		       : (CC == 2) ? k_poisson_cg_cta<2, true>
		       : (CC == 3) ? k_poisson_cg_cta<3, true>
		                   : k_poisson_cg_cta<4, true>;
	return (CC == 1)   ? k_poisson_cg_cta<1, false>
	       : (CC == 2) ? k_poisson_cg_cta<2, false>
	       : (CC == 3) ? k_poisson_cg_cta<3, false>
	                   : k_poisson_cg_cta<4, false>;
}

// Vectors of `chunk` floats per channel a cluster CTA keeps in shared
// memory: r, two direction buffers, x (and z when preconditioned).
static int cluster_vectors(bool pre) { return kClusterVectors + (pre ? 1 : 0); }

// shared-memory cluster kernel: kClusterVectors vectors x chunk floats per CTA, one cluster per channel
constexpr size_t kSmemBudget = 216 * 1024;

// Solver layout of a system of nh unknowns per channel: *ncta CTAs of
// *chunk unknowns each (one CTA with block barriers when *ncta is 1, a
// cluster when it is more), or *ncta = 0 for the cooperative grid CG.
static void cg_layout(nli_ctx *ctx, int nh, int *ncta, int *chunk)
{
	if (ctx->cg_cluster_max < 0) {
		// largest cluster the device runs with the biggest shared-memory footprint
		int maxc = 0;
		bool ok = true;
		for (int CC = 1; CC <= 4; CC++)
			for (int pre = 0; pre < 2; pre++) {
				ok &= cudaFuncSetAttribute(cluster_kernel(CC, pre), cudaFuncAttributeNonPortableClusterSizeAllowed,
				                           1) == 0;
				ok &= cudaFuncSetAttribute(cluster_kernel(CC, pre), cudaFuncAttributeMaxDynamicSharedMemorySize,
				                           (int)kSmemBudget) == 0;
				ok &= cudaFuncSetAttribute(cta_kernel(CC, pre), cudaFuncAttributeMaxDynamicSharedMemorySize,
				                           (int)kSmemBudget) == 0;
			}
		if (ok) {
			cudaLaunchConfig_t qc = {};
			qc.gridDim = dim3(kClusterMax);
			qc.blockDim = dim3(kClusterBlock);
			qc.dynamicSmemBytes = kSmemBudget;
			if (cudaOccupancyMaxPotentialClusterSize(&maxc, cluster_kernel(4, true), &qc) != cudaSuccess) maxc = 0;
		}
		cudaGetLastError();
		ctx->cg_cluster_max = std::min(maxc, kClusterMax);
	}
	*ncta = *chunk = 0;
	if (ctx->cg_cluster_max >= 1) {
		const int per = std::max(1, ctx->tune_cg_unknowns_per_cta);
		*ncta = std::max(1, std::min(std::min(ctx->cg_cluster_max, ctx->tune_cg_cluster_cap), (nh + per - 1) / per));
		*chunk = (nh + *ncta - 1) / *ncta;
		if ((size_t)cluster_vectors(ctx->tune_cg_precond) * *chunk * sizeof(float) + *chunk * sizeof(UnkC) >
		        kSmemBudget ||
		    *chunk > kClusterMaxChunk)
			*ncta = *chunk = 0;
		// small systems: one CTA, block barriers only (NLI_TUNE_CG_SINGLE_MAX)
		if (nh <= std::min(ctx->tune_cg_single_max, kClusterMaxChunk)) {
			*ncta = 1;
			*chunk = nh;
		}
	}
}

// Coefficients (gather), the compact system and its right-hand side b and
// start x0 = image - orig (patch_non_local_poisson.cpp:36-82).  Chooses the
// solver layout: `chunk` / `ncta` > 0 for the cluster CG.
struct PoissonSystem {
	PoissonArgs pa;
	CoefOut co;
	Unknown *unk;
	float *b, *x;
	int chunk = 0, ncta = 0;
};

static PoissonSystem poisson_system(nli_ctx *ctx, const UpdArgs &u, const nli_update_params &up, const float *image,
                                    const float *orig, const uint8_t *dom, const uint8_t *ext, const int2 *nnf,
                                    const float *conf, const int32_t *hole, const int32_t *hole_index, int nh)
{
	cudaStream_t s = ctx->stream;
	const int W = u.W, H = u.H, C = u.C;
	const size_t n = (size_t)W * H;
	PoissonSystem P;
	float *grad = ctx->buf<float>("poi.grad", n * 2 * C);
	launch_gradient(s, image, W, H, C, grad);
	P.co.S = ctx->buf<float>("poi.S", n);
	P.co.U = ctx->buf<float>("poi.U", n * C);
	P.co.GX = ctx->buf<float>("poi.GX", n * C);
	P.co.GY = ctx->buf<float>("poi.GY", n * C);
	{
		ProfScope ps(ctx, "poisson_coef");
		if (u.px % 2 == 1 && u.py % 2 == 1) {
			const long long threads = 3LL * nh * 8;
			k_poisson_coef8<<<(int)((threads + 255) / 256), 256, 0, s>>>(
			    u, hole, nh, dom, ext, nnf, conf, image, reinterpret_cast<const float2 *>(grad), P.co);
		} else {
			// even patch sides: the window of gather_coef is one wider than the patch
			k_poisson_coef<<<(nh + 127) / 128, 128, 0, s>>>(u, hole, nh, dom, ext, nnf, conf, image,
			                                                 reinterpret_cast<const float2 *>(grad), P.co);
		}
		NLI_CHECK_LAUNCH();
	}
	PoissonArgs &pa = P.pa;
	pa.W = W;
	pa.H = H;
	pa.C = C;
	pa.nh = nh;
	for (int c = 0; c < 4; c++) pa.lambda[c] = up.lambda;
	if (up.method == NLI_UPDATE_DEPTH) pa.lambda[3] = up.lambda_d;
	pa.tol = up.cg_tol;
	pa.limit = up.cg_iters;
	P.unk = ctx->buf<Unknown>("poi.unk", nh);
	P.b = ctx->buf<float>("poi.b", (size_t)nh * C);
	P.x = ctx->buf<float>("poi.x", (size_t)nh * C);

	cg_layout(ctx, nh, &P.ncta, &P.chunk);
	{
		ProfScope ps(ctx, "poisson_setup");
		k_poisson_setup<<<(nh + 255) / 256, 256, 0, s>>>(pa, P.chunk, hole, hole_index, P.co, image, orig, P.unk,
		                                                  P.b, P.x);
		NLI_CHECK_LAUNCH();
	}
	return P;
}

// Blocks of the cooperative grid CG for nh unknowns: co-resident, at most
// one per SM.
static int grid_cg_blocks(nli_ctx *ctx, int nh)
{
	int dev_blocks_per_sm = 0;
	const bool pre = ctx->tune_cg_precond != 0;
	const void *kern = pre ? (const void *)k_poisson_cg<true> : (const void *)k_poisson_cg<false>;
	NLI_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&dev_blocks_per_sm, kern, kCgBlock, 0));
	const int max_blocks = dev_blocks_per_sm * ctx->num_sms;
	NLI_REQUIRE(max_blocks > 0, NLI_E_CUDA, "conjugate gradient kernel cannot be made resident");
	int grid = (nh + kCgBlock - 1) / kCgBlock;
	return std::min(std::max(grid, 1), std::min(max_blocks, ctx->num_sms));
}

struct GridCgBufs {
	float *r, *d, *q, *z;  // nh * C each (z only when preconditioned)
	double *part;          // grid * 16
};

// The cooperative grid CG of system P on `grid` blocks.  active (may be
// null): a device flag; 0 makes every block leave at once.
static void launch_grid_cg(nli_ctx *ctx, const PoissonSystem &P, int grid, const GridCgBufs &g, int *iters,
                           const int32_t *hole, const float *orig, float *img, double *diff_part, const int *active)
{
	cudaStream_t s = ctx->stream;
	const bool pre = ctx->tune_cg_precond != 0;
	const void *kern = pre ? (const void *)k_poisson_cg<true> : (const void *)k_poisson_cg<false>;
	// the grid barrier's counters (the timeout word is left for the
	// iteration's readback)
	NLI_CUDA(cudaMemsetAsync(ctx->status, 0, offsetof(DevStatus, timeout), s));
	DevStatus *st = ctx->status;
	PoissonArgs pa = P.pa;
	const Unknown *unk = P.unk;
	const float *b = P.b;
	float *x = P.x;
	float *r = g.r, *d = g.d, *q = g.q, *z = g.z;
	double *part = g.part;
	void *args[] = {&pa,   &unk, &b,     &x,    (void *)&r, &d,         &q,         &z,
	                &part, &st,  &iters, (void *)&hole, &orig, &img, &diff_part, (void *)&active};
	// cooperative through the launch attribute, which stream capture takes
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(grid);
	cfg.blockDim = dim3(kCgBlock);
	cfg.dynamicSmemBytes = 0;
	cfg.stream = s;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeCooperative;
	attr[0].val.cooperative = 1;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	ProfScope ps(ctx, "poisson_cg");
	NLI_CUDA(cudaLaunchKernelExC(&cfg, kern, args));
	nli_count_launch_internal();
}

// Solves the system from x0 (the CG of :387-477) and writes u = orig + x on
// the hole into img, with per-block partial sums of (u_old - u_new)^2 in
// "poi.diff" (returns their count).
static int poisson_solve(nli_ctx *ctx, PoissonSystem &P, const int32_t *hole, const float *orig, float *img)
{
	cudaStream_t s = ctx->stream;
	const int nh = P.pa.nh, C = P.pa.C;
	int *iters = ctx->buf<int>("poi.iters", 4);
	if (P.ncta > 0) {
		const bool pre = ctx->tune_cg_precond != 0;
		const size_t smem = (size_t)cluster_vectors(pre) * P.chunk * sizeof(float) + P.chunk * sizeof(UnkC);
		UnkC *unkc = ctx->buf<UnkC>("poi.unkc", nh);
		k_poisson_compact<<<(nh + 255) / 256, 256, 0, s>>>(P.unk, nh, P.chunk, unkc);
		NLI_CHECK_LAUNCH();
		double *diff_part = ctx->buf<double>("poi.diff", (size_t)C * P.ncta + 1);
		if (P.ncta == 1) {
			// one CTA per channel: no cluster
			ProfScope ps(ctx, "poisson_cg");
			cta_kernel(1, pre)<<<C, kClusterBlock, smem, s>>>(P.pa, P.chunk, unkc, P.b, P.x, iters, hole, orig, img,
			                                                  diff_part);
			NLI_CHECK_LAUNCH();
			return C;
		}
		cudaLaunchConfig_t cfg = {};
		cfg.gridDim = dim3(C * P.ncta);
		cfg.blockDim = dim3(kClusterBlock);
		cfg.dynamicSmemBytes = smem;
		cfg.stream = s;
		cudaLaunchAttribute attr[1];
		attr[0].id = cudaLaunchAttributeClusterDimension;
		attr[0].val.clusterDim.x = P.ncta;
		attr[0].val.clusterDim.y = 1;
		attr[0].val.clusterDim.z = 1;
		cfg.attrs = attr;
		cfg.numAttrs = 1;
		ProfScope ps(ctx, "poisson_cg");
		NLI_CUDA(cudaLaunchKernelEx(&cfg, cluster_kernel(1, pre), P.pa, P.chunk, (const UnkC *)unkc, (const float *)P.b,
		                            (const float *)P.x, iters, hole, orig, img, diff_part));
		nli_count_launch_internal();
		return C * P.ncta;
	}
	const int grid = grid_cg_blocks(ctx, nh);
	double *part = ctx->buf<double>("poi.part", (size_t)grid * 16);
	double *diff_part = ctx->buf<double>("poi.diff", grid + 1);
	GridCgBufs g;
	g.r = ctx->buf<float>("poi.r", (size_t)nh * C);
	g.d = ctx->buf<float>("poi.d", (size_t)nh * C);
	g.q = ctx->buf<float>("poi.q", (size_t)nh * C);
	g.z = ctx->tune_cg_precond ? ctx->buf<float>("poi.z", (size_t)nh * C) : nullptr;
	g.part = part;
	launch_grid_cg(ctx, P, grid, g, iters, hole, orig, img, diff_part, nullptr);
	return grid;
}

static void poisson_run(nli_ctx *ctx, const UpdArgs &u, const nli_update_params &up, float *image, const float *orig,
                        const uint8_t *dom, const uint8_t *ext, const int2 *nnf, const float *conf,
                        const int32_t *hole, const int32_t *hole_index, int nh, int *n_partials)
{
	PoissonSystem P = poisson_system(ctx, u, up, image, orig, dom, ext, nnf, conf, hole, hole_index, nh);
	*n_partials = poisson_solve(ctx, P, hole, orig, image);
}

double update_run(nli_ctx *ctx, const nli_update_params &up, float *image, const float *orig, const uint8_t *dom,
                  const uint8_t *ext, const int32_t *nnf_i, const float *conf, int W, int H, int C,
                  const int32_t *hole, int nh, bool read_back, const double **total_dev, const int **cg_iters_dev)
{
	NLI_REQUIRE(up.method >= 0 && up.method <= 3, NLI_E_UNSUPPORTED, "unknown update method");
	if (up.method == NLI_UPDATE_DEPTH) NLI_REQUIRE(C == 4, NLI_E_CHANNELS, "Separate: Channels do not match.");
	UpdArgs u;
	fill_upd_args(u, up, W, H, C);
	cudaStream_t s = ctx->stream;
	const int2 *nnf = reinterpret_cast<const int2 *>(nnf_i);
	const int32_t *hole_index = nullptr;
	if (!hole) {
		int32_t *l = ctx->buf<int32_t>("upd.hole", (size_t)W * H);
		nh = compact_mask(ctx, dom, W, H, l, "upd");
		hole = l;
	}
	if (nh <= 0) return 0.0;
	if (up.method == NLI_UPDATE_POISSON || up.method == NLI_UPDATE_DEPTH) {
		int32_t *idx = ctx->buf<int32_t>("upd.hole_index", (size_t)W * H);
		k_fill_int<<<(W * H + 255) / 256, 256, 0, s>>>(idx, W * H, -1);
		NLI_CHECK_LAUNCH();
		k_hole_index<<<(nh + 255) / 256, 256, 0, s>>>(hole, nh, idx);
		NLI_CHECK_LAUNCH();
		hole_index = idx;
		int np = 0;
		poisson_run(ctx, u, up, image, orig, dom, ext, nnf, conf, hole, hole_index, nh, &np);
		double *diff_part = ctx->buf<double>("poi.diff", np + 1);
		if (!read_back) {
			launch_sum_partials(s, diff_part, np, diff_part + np);
			if (total_dev) *total_dev = diff_part + np;
			if (cg_iters_dev) *cg_iters_dev = ctx->buf<int>("poi.iters", 4);
			return 0.0;
		}
		return read_total(ctx, diff_part, np, ctx->buf<int>("poi.iters", 4), C, nh);
	}
	float *newval = ctx->buf<float>("upd.newval", (size_t)nh * C);
	int grid;
	double *partials;
	if (up.method == NLI_UPDATE_MEANS) {
		grid = (nh + 255) / 256;
		partials = ctx->buf<double>("upd.partials", grid + 1);
		ProfScope ps(ctx, "nlmeans");
		k_nlmeans<<<grid, 256, 0, s>>>(u, image, hole, nh, dom, nnf, conf, newval, partials);
	} else {
		grid = (nh + kMedWarps - 1) / kMedWarps;
		partials = ctx->buf<double>("upd.partials", grid + 1);
		ProfScope ps(ctx, "nlmedians");
		k_nlmedians<<<grid, 32 * kMedWarps, 0, s>>>(u, image, hole, nh, dom, nnf, conf, newval, partials);
	}
	NLI_CHECK_LAUNCH();
	k_scatter_values<<<(nh * C + 255) / 256, 256, 0, s>>>(hole, nh, C, newval, image);
	NLI_CHECK_LAUNCH();
	if (!read_back) {
		launch_sum_partials(s, partials, grid, partials + grid);
		if (total_dev) *total_dev = partials + grid;
		if (cg_iters_dev) *cg_iters_dev = nullptr;
		return 0.0;
	}
	return read_total(ctx, partials, grid, nullptr, C);
}

// ======================================================= batched updates
// The update step of up to kBatchMax images in one launch per kernel (the
// lockstep batch driver, lockstep.cu).  Each image keeps its own sizes,
// method, lambda and CG tolerance; the patch and its weights are shared.
// Every per-pixel / per-unknown value comes from the same device functions
// as the one-image kernels, and every reduction keeps the one-image
// partition (blocks of one image never straddle another image; each CG
// system has the same CTA layout), so each image's result and its sum of
// (u_old - u_new)^2 equal those of its one-image update bit for bit.
// Images whose active flag is 0 are skipped.  The per-image arguments
// travel in kernel parameter space (__grid_constant__ tables).
struct BTask {
	int img_index;  // index of the image's active flag
	int W, H, nh;
	float *img;
	const float *orig;
	const uint8_t *dom, *ext;
	const int2 *nnf;
	const float *conf;
	const int32_t *hole;
	float *newval;      // NL-means / NL-medians: new values of the hole
	double *partials;   // NL-means / NL-medians: per-block sums
	int32_t *hidx;      // NL-Poisson: unknown index per pixel
	float *grad;
	CoefOut co;
	Unknown *unk;
	UnkC *unkc;
	float *b, *x;
	PoissonArgs pa;
	int chunk, ncta;    // CG layout (ncta 0: grid CG)
	int *iters;
	double *diff;       // CG: partial sums of (du)^2
	int nparts;         // partial sums behind `total`
	double *total;      // this step's sum of (du)^2
};

struct BArgs {
	int n;
	const int *active;
	int blk[kBatchMax + 1];  // block prefix of the launch
	BTask t[kBatchMax];
};

__device__ __forceinline__ bool btask_on(const BArgs &B, int t) { return !B.active || B.active[B.t[t].img_index]; }

// The task whose block range [blk[t], blk[t + 1]) holds block b.
__device__ __forceinline__ int task_of_block(const BArgs &B, int b)
{
	int lo = 0, hi = B.n;
	while (hi - lo > 1) {
		const int mid = (lo + hi) >> 1;
		if (B.blk[mid] <= b)
			lo = mid;
		else
			hi = mid;
	}
	return lo;
}

__global__ void __launch_bounds__(256) k_nlmeans_batch(UpdArgs u, const __grid_constant__ BArgs B, int C)
{
	__shared__ double red[8];
	const int t = task_of_block(B, blockIdx.x);
	if (!btask_on(B, t)) return;
	const BTask &T = B.t[t];
	const int bl = blockIdx.x - B.blk[t];
	const int i = bl * 256 + threadIdx.x;
	double acc = 0.0;
	if (i < T.nh)
		acc = nlmeans_pixel(u, T.W, T.H, C, T.img, T.hole[i], T.dom, T.nnf, T.conf, T.newval + (size_t)C * i);
	acc = block_sum<256>(acc, red);
	if (threadIdx.x == 0) T.partials[bl] = acc;
}

__global__ void __launch_bounds__(32 * kMedWarps) k_nlmedians_batch(UpdArgs u, const __grid_constant__ BArgs B, int C)
{
	__shared__ float s_val[kMedWarps][4][kMaxTaps];
	__shared__ float s_w[kMedWarps][kMaxTaps];
	__shared__ float s_sv[kMedWarps][kMaxTaps];
	__shared__ float s_sw[kMedWarps][kMaxTaps];
	__shared__ double red[kMedWarps];
	const int t = task_of_block(B, blockIdx.x);
	if (!btask_on(B, t)) return;
	const BTask &T = B.t[t];
	const int bl = blockIdx.x - B.blk[t];
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	const int i = bl * kMedWarps + wid;
	double acc = 0.0;
	if (i < T.nh)
		acc = nlmedians_pixel(u, T.W, T.H, C, T.img, T.hole[i], T.dom, T.nnf, T.conf, T.newval + (size_t)C * i,
		                      MedSmem{s_val[wid], s_w[wid], s_sv[wid], s_sw[wid]});
	if (lane == 0) red[wid] = acc;
	__syncthreads();
	if (threadIdx.x == 0) {
		double tt = 0.0;
		for (int w = 0; w < kMedWarps; w++) tt += red[w];
		T.partials[bl] = tt;
	}
}

// New values into the image (k_scatter_values per image).
__global__ void k_scatter_batch(const __grid_constant__ BArgs B, int C)
{
	const int t = blockIdx.y;
	if (!btask_on(B, t)) return;
	const BTask &T = B.t[t];
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < T.nh * C; i += gridDim.x * blockDim.x) {
		const int k = i / C, c = i % C;
		T.img[(size_t)C * T.hole[k] + c] = T.newval[i];
	}
}

// The image's sum of (du)^2 from its partial sums (k_sum_partials per
// image: one 1024-thread block each, the same order).  which 0: the
// NL-means / NL-medians block sums, 1: the CG partial sums.
__global__ void __launch_bounds__(1024) k_total_batch(const __grid_constant__ BArgs B, int which)
{
	__shared__ double sm[32];
	const int t = blockIdx.x;
	if (!btask_on(B, t)) return;
	const BTask &T = B.t[t];
	const double *part = which ? T.diff : T.partials;
	double v = 0.0;
	for (int i = threadIdx.x; i < T.nparts; i += blockDim.x) v += part[i];
	v = block_sum<1024>(v, sm);
	if (threadIdx.x == 0) *T.total = v;
}

// Unknown index per pixel: -1, then k at hole pixel k.
__global__ void k_hidx_fill_batch(const __grid_constant__ BArgs B)
{
	const int t = blockIdx.y;
	if (!btask_on(B, t)) return;
	const BTask &T = B.t[t];
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < T.W * T.H; i += gridDim.x * blockDim.x) T.hidx[i] = -1;
}

__global__ void k_hidx_set_batch(const __grid_constant__ BArgs B)
{
	const int t = blockIdx.y;
	if (!btask_on(B, t)) return;
	const BTask &T = B.t[t];
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < T.nh; k += gridDim.x * blockDim.x) T.hidx[T.hole[k]] = k;
}

__global__ void k_gradient_batch(const __grid_constant__ BArgs B, int C)
{
	const int t = blockIdx.y;
	if (!btask_on(B, t)) return;
	const BTask &T = B.t[t];
	gradient_span(T.img, T.W, T.H, C, T.grad, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

__global__ void __launch_bounds__(256) k_coef8_batch(UpdArgs u, const __grid_constant__ BArgs B, int C)
{
	const int t = task_of_block(B, blockIdx.x);
	if (!btask_on(B, t)) return;
	const BTask &T = B.t[t];
	const int item = (((int)blockIdx.x - B.blk[t]) * 256 + (int)threadIdx.x) >> 3;
	coef8_item(u, T.W, T.H, C, item, threadIdx.x & 7, T.hole, T.nh, T.dom, T.ext, T.nnf, T.conf, T.img,
	           reinterpret_cast<const float2 *>(T.grad), T.co);
}

__global__ void __launch_bounds__(128) k_coef_batch(UpdArgs u, const __grid_constant__ BArgs B, int C)
{
	const int t = task_of_block(B, blockIdx.x);
	if (!btask_on(B, t)) return;
	const BTask &T = B.t[t];
	const int i = ((int)blockIdx.x - B.blk[t]) * 128 + (int)threadIdx.x;
	if (i >= T.nh) return;
	coef_hole_pixel(u, T.W, T.H, C, T.hole[i], T.dom, T.ext, T.nnf, T.conf, T.img,
	                reinterpret_cast<const float2 *>(T.grad), T.co);
}

__global__ void k_setup_batch(const __grid_constant__ BArgs B)
{
	const int t = task_of_block(B, blockIdx.x);
	if (!btask_on(B, t)) return;
	const BTask &T = B.t[t];
	const int k = ((int)blockIdx.x - B.blk[t]) * 256 + (int)threadIdx.x;
	if (k >= T.nh) return;
	poisson_setup_unknown(T.pa, T.chunk, k, T.hole, T.hidx, T.co, T.img, T.orig, T.unk, T.b, T.x);
}

__global__ void k_compact_batch(const __grid_constant__ BArgs B)
{
	const int t = blockIdx.y;
	if (!btask_on(B, t)) return;
	const BTask &T = B.t[t];
	if (T.ncta == 0) return;
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < T.nh; k += gridDim.x * blockDim.x)
		poisson_compact_unknown(T.unk, k, T.chunk, T.unkc);
}

// CG systems of one layout class (the same CTAs per system): system g of
// the launch is channel g % C of task g / C.
struct CgTask {
	int img_index;
	PoissonArgs a;
	int chunk;
	const UnkC *unk;
	const float *b, *x0;
	int *iters;
	const int32_t *hole;
	const float *orig;
	float *img;
	double *diff;
};

struct CgArgs {
	int n, C, ncta;
	const int *active;
	CgTask t[kBatchMax];
};

template <bool PRE, bool SINGLE>
__global__ void __launch_bounds__(kClusterBlock, 1) k_poisson_cg_batch(const __grid_constant__ CgArgs B)
{
	const int ncta = SINGLE ? 1 : B.ncta;
	const int g = (int)blockIdx.x / ncta;
	const int t = g / B.C, group = g - t * B.C;
	const CgTask &T = B.t[t];
	// a stopped image: every CTA of its clusters leaves before any barrier
	if (B.active && !B.active[T.img_index]) return;
	cg_team_solve<1, PRE, SINGLE>(T.a, T.chunk, T.unk, T.b, T.x0, T.iters, T.hole, T.orig, T.img, T.diff, group);
}

static void (*cg_batch_kernel(bool pre, bool single))(CgArgs)
{
	if (pre) return single ? k_poisson_cg_batch<true, true> : k_poisson_cg_batch<true, false>;
	return single ? k_poisson_cg_batch<false, true> : k_poisson_cg_batch<false, false>;
}

static std::string lk_name(int i, const char *what) { return "lk." + std::to_string(i) + "." + what; }

static int div_up(long long a, int b) { return (int)((a + b - 1) / b); }

// Elementwise launch over n images: blockIdx.y = image, grid-stride in x.
static dim3 per_image_grid(long long maxcount, int n, int block = 256)
{
	return dim3((unsigned)std::max(1, std::min(div_up(maxcount, block), 1024)), (unsigned)n);
}

void update_batch_run(nli_ctx *ctx, const nli_update_params *ups, int C, int n, const UpdBatchItem *items,
                      const int *active)
{
	NLI_REQUIRE(n >= 1 && n <= kBatchMax, NLI_E_INVALID, "batched updates take 1 to 64 images");
	cudaStream_t s = ctx->stream;
	UpdArgs u;
	fill_upd_args(u, ups[0], 0, 0, C);
	for (int i = 1; i < n; i++)
		NLI_REQUIRE(ups[i].patch_x == ups[0].patch_x && ups[i].patch_y == ups[0].patch_y &&
		                ups[i].sigma == ups[0].sigma,
		            NLI_E_INVALID, "batched updates share the patch and its sigma");
	BArgs M, D, P;  // NL-means, NL-medians, NL-Poisson / NL-depth images
	std::memset(&M, 0, sizeof(M));
	std::memset(&D, 0, sizeof(D));
	std::memset(&P, 0, sizeof(P));
	M.active = D.active = P.active = active;
	long long maxnh = 0, maxpix = 0;
	for (int i = 0; i < n; i++) {
		const UpdBatchItem &it = items[i];
		const nli_update_params &up = ups[i];
		NLI_REQUIRE(up.method >= 0 && up.method <= 3, NLI_E_UNSUPPORTED, "unknown update method");
		if (up.method == NLI_UPDATE_DEPTH) NLI_REQUIRE(C == 4, NLI_E_CHANNELS, "Separate: Channels do not match.");
		BArgs &B = (up.method == NLI_UPDATE_MEANS) ? M : (up.method == NLI_UPDATE_MEDIANS) ? D : P;
		BTask &T = B.t[B.n++];
		T.img_index = it.flag;
		T.W = it.W;
		T.H = it.H;
		T.nh = it.nh;
		T.img = it.img;
		T.orig = it.orig;
		T.dom = it.dom;
		T.ext = it.ext;
		T.nnf = reinterpret_cast<const int2 *>(it.nnf);
		T.conf = it.conf;
		T.hole = it.hole;
		T.total = it.total;
		T.iters = it.cg_iters;
		maxnh = std::max<long long>(maxnh, it.nh);
		maxpix = std::max<long long>(maxpix, (long long)it.W * it.H);
		const size_t np = (size_t)it.W * it.H;
		const size_t nh = (size_t)std::max(it.nh, 1);
		if (&B != &P) {
			const int per = (&B == &M) ? 256 : kMedWarps;
			T.nparts = div_up(it.nh, per);
			T.newval = ctx->buf<float>(lk_name(it.flag, "newval"), nh * C);
			T.partials = ctx->buf<double>(lk_name(it.flag, "partials"), (size_t)std::max(T.nparts, 1));
			continue;
		}
		PoissonArgs &pa = T.pa;
		pa.W = it.W;
		pa.H = it.H;
		pa.C = C;
		pa.nh = it.nh;
		for (int c = 0; c < 4; c++) pa.lambda[c] = up.lambda;
		if (up.method == NLI_UPDATE_DEPTH) pa.lambda[3] = up.lambda_d;
		pa.tol = up.cg_tol;
		pa.limit = up.cg_iters;
		T.hidx = ctx->buf<int32_t>(lk_name(it.flag, "hidx"), np);
		T.grad = ctx->buf<float>(lk_name(it.flag, "grad"), np * 2 * C);
		T.co.S = ctx->buf<float>(lk_name(it.flag, "S"), np);
		T.co.U = ctx->buf<float>(lk_name(it.flag, "U"), np * C);
		T.co.GX = ctx->buf<float>(lk_name(it.flag, "GX"), np * C);
		T.co.GY = ctx->buf<float>(lk_name(it.flag, "GY"), np * C);
		T.unk = ctx->buf<Unknown>(lk_name(it.flag, "unk"), nh);
		T.b = ctx->buf<float>(lk_name(it.flag, "b"), nh * C);
		T.x = ctx->buf<float>(lk_name(it.flag, "x"), nh * C);
		cg_layout(ctx, it.nh, &T.ncta, &T.chunk);
		if (it.nh == 0) {
			T.nparts = 0;  // nothing to solve: the step's sum is 0
		} else if (T.ncta > 0) {
			T.unkc = ctx->buf<UnkC>(lk_name(it.flag, "unkc"), nh);
			T.nparts = C * T.ncta;
		} else {
			T.nparts = grid_cg_blocks(ctx, it.nh);
		}
		T.diff = ctx->buf<double>(lk_name(it.flag, "diff"), (size_t)T.nparts + 1);
	}
	const int blk = 256;
	// ---- NL-means
	if (M.n > 0) {
		for (int t = 0; t < M.n; t++) M.blk[t + 1] = M.blk[t] + div_up(M.t[t].nh, 256);
		if (M.blk[M.n] > 0) {
			ProfScope ps(ctx, "nlmeans");
			k_nlmeans_batch<<<M.blk[M.n], 256, 0, s>>>(u, M, C);
			NLI_CHECK_LAUNCH();
		}
		k_scatter_batch<<<per_image_grid(maxnh * C, M.n), blk, 0, s>>>(M, C);
		NLI_CHECK_LAUNCH();
		k_total_batch<<<M.n, 1024, 0, s>>>(M, 0);
		NLI_CHECK_LAUNCH();
	}
	// ---- NL-medians
	if (D.n > 0) {
		for (int t = 0; t < D.n; t++) D.blk[t + 1] = D.blk[t] + div_up(D.t[t].nh, kMedWarps);
		if (D.blk[D.n] > 0) {
			ProfScope ps(ctx, "nlmedians");
			k_nlmedians_batch<<<D.blk[D.n], 32 * kMedWarps, 0, s>>>(u, D, C);
			NLI_CHECK_LAUNCH();
		}
		k_scatter_batch<<<per_image_grid(maxnh * C, D.n), blk, 0, s>>>(D, C);
		NLI_CHECK_LAUNCH();
		k_total_batch<<<D.n, 1024, 0, s>>>(D, 0);
		NLI_CHECK_LAUNCH();
	}
	if (P.n == 0) return;
	// ---- NL-Poisson / NL-depth: system set-up for every image
	k_hidx_fill_batch<<<per_image_grid(maxpix, P.n), blk, 0, s>>>(P);
	NLI_CHECK_LAUNCH();
	k_hidx_set_batch<<<per_image_grid(maxnh, P.n), blk, 0, s>>>(P);
	NLI_CHECK_LAUNCH();
	k_gradient_batch<<<per_image_grid(maxpix * C, P.n), blk, 0, s>>>(P, C);
	NLI_CHECK_LAUNCH();
	{
		ProfScope ps(ctx, "poisson_coef");
		if (u.px % 2 == 1 && u.py % 2 == 1) {
			for (int t = 0; t < P.n; t++) P.blk[t + 1] = P.blk[t] + div_up(3LL * P.t[t].nh * 8, 256);
			if (P.blk[P.n] > 0) k_coef8_batch<<<P.blk[P.n], 256, 0, s>>>(u, P, C);
		} else {
			for (int t = 0; t < P.n; t++) P.blk[t + 1] = P.blk[t] + div_up(P.t[t].nh, 128);
			if (P.blk[P.n] > 0) k_coef_batch<<<P.blk[P.n], 128, 0, s>>>(u, P, C);
		}
		if (P.blk[P.n] > 0) NLI_CHECK_LAUNCH();
	}
	{
		ProfScope ps(ctx, "poisson_setup");
		for (int t = 0; t < P.n; t++) P.blk[t + 1] = P.blk[t] + div_up(P.t[t].nh, 256);
		if (P.blk[P.n] > 0) {
			k_setup_batch<<<P.blk[P.n], 256, 0, s>>>(P);
			NLI_CHECK_LAUNCH();
		}
	}
	k_compact_batch<<<per_image_grid(maxnh, P.n), blk, 0, s>>>(P);
	NLI_CHECK_LAUNCH();
	// ---- the solves, one launch per CTA layout
	const bool pre = ctx->tune_cg_precond != 0;
	{
		static std::atomic<uint32_t> raised{0};  // one bit per device
		const uint32_t bit = 1u << (ctx->device & 31);
		if (!(raised.load(std::memory_order_acquire) & bit)) {
			for (int pr = 0; pr < 2; pr++)
				for (int sg = 0; sg < 2; sg++) {
					NLI_CUDA(cudaFuncSetAttribute(cg_batch_kernel(pr, sg), cudaFuncAttributeMaxDynamicSharedMemorySize,
					                              (int)kSmemBudget));
					if (!sg)
						NLI_CUDA(cudaFuncSetAttribute(cg_batch_kernel(pr, sg),
						                              cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
				}
			raised.fetch_or(bit, std::memory_order_release);
		}
	}
	for (int ncta = 1; ncta <= kClusterMax; ncta++) {
		CgArgs G;
		std::memset(&G, 0, sizeof(G));
		G.C = C;
		G.ncta = ncta;
		G.active = active;
		int maxchunk = 0;
		for (int t = 0; t < P.n; t++) {
			const BTask &T = P.t[t];
			if (T.ncta != ncta || T.nh == 0) continue;
			CgTask &g = G.t[G.n++];
			g.img_index = T.img_index;
			g.a = T.pa;
			g.chunk = T.chunk;
			g.unk = T.unkc;
			g.b = T.b;
			g.x0 = T.x;
			g.iters = T.iters;
			g.hole = T.hole;
			g.orig = T.orig;
			g.img = T.img;
			g.diff = T.diff;
			maxchunk = std::max(maxchunk, T.chunk);
		}
		if (G.n == 0) continue;
		const size_t smem = (size_t)cluster_vectors(pre) * maxchunk * sizeof(float) + maxchunk * sizeof(UnkC);
		ProfScope ps(ctx, "poisson_cg");
		if (ncta == 1) {
			cg_batch_kernel(pre, true)<<<G.n * C, kClusterBlock, smem, s>>>(G);
			NLI_CHECK_LAUNCH();
			continue;
		}
		cudaLaunchConfig_t cfg = {};
		cfg.gridDim = dim3(G.n * C * ncta);
		cfg.blockDim = dim3(kClusterBlock);
		cfg.dynamicSmemBytes = smem;
		cfg.stream = s;
		cudaLaunchAttribute attr[1];
		attr[0].id = cudaLaunchAttributeClusterDimension;
		attr[0].val.clusterDim.x = ncta;
		attr[0].val.clusterDim.y = 1;
		attr[0].val.clusterDim.z = 1;
		cfg.attrs = attr;
		cfg.numAttrs = 1;
		NLI_CUDA(cudaLaunchKernelEx(&cfg, cg_batch_kernel(pre, false), G));
		nli_count_launch_internal();
	}
	// systems too large for a cluster: the cooperative grid CG, one at a time
	for (int t = 0; t < P.n; t++) {
		const BTask &T = P.t[t];
		if (T.ncta != 0 || T.nh == 0) continue;
		const int i = T.img_index;  // names its scratch
		const size_t nh = (size_t)T.nh;
		PoissonSystem S;
		S.pa = T.pa;
		S.co = T.co;
		S.unk = T.unk;
		S.b = T.b;
		S.x = T.x;
		GridCgBufs g;
		g.r = ctx->buf<float>(lk_name(i, "r"), nh * C);
		g.d = ctx->buf<float>(lk_name(i, "d"), nh * C);
		g.q = ctx->buf<float>(lk_name(i, "q"), nh * C);
		g.z = pre ? ctx->buf<float>(lk_name(i, "z"), nh * C) : nullptr;
		g.part = ctx->buf<double>(lk_name(i, "part"), (size_t)T.nparts * 16);
		launch_grid_cg(ctx, S, T.nparts, g, T.iters, T.hole, T.orig, T.img, T.diff,
		               active ? active + T.img_index : nullptr);
	}
	k_total_batch<<<P.n, 1024, 0, s>>>(P, 1);
	NLI_CHECK_LAUNCH();
}

// ============================================================== adjoints
// Backward of one image update with the NNF held fixed: out = U(u; lambda,
// sigma) with orig = u (the update step of image_inpainting.cpp:394 on its
// own), given g = dL/dout.  The NNF is an integer argmin and is not
// differentiated.  Accumulation into dL/du is in double (atomics), then
// rounded to float.  sigma enters through the normalised Gaussian patch
// weights w_k = e_k / sum_j e_j, e_k = exp(-r_k^2 / (2 sigma^2))
// (gaussian_weights.cpp:19-79): dw_k/dsigma = w_k (rho_k - m), rho_k =
// r_k^2 / sigma^3, m = sum_j w_j rho_j.
struct AdjArgs {
	double sigma3;  // sigma^3
	double m;       // sum_j w_j rho_j of the weight table
};

__device__ __forceinline__ double tap_rho(const UpdArgs &u, const AdjArgs &a, int k)
{
	const int kx = k % u.px - u.hx, ky = k / u.px - u.hy;
	return (double)(kx * kx + ky * ky) / a.sigma3;
}

// Identity part: out = u outside the domain (and on domain pixels without
// any valid candidate, handled by the means kernel).
__global__ void k_adj_init(const float *__restrict__ g, const uint8_t *__restrict__ dom, int n, int C,
                           double *__restrict__ gacc)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n * C; i += gridDim.x * blockDim.x)
		gacc[i] = dom[i / C] ? 0.0 : (double)g[i];
}

// NL-means: out_c(p) = N_c / D, N_c = sum_i w_i u_c(s_i), D = sum_i w_i, with
// the forward's weights (clipped-corner table index, confidence inside the
// domain).  du(s_i) += g_c w_i / D; dsigma += sum_c g_c sum_i w_i rho_i
// (u_c(s_i) - out_c) / D (the normalisation term cancels in the ratio).
__global__ void __launch_bounds__(256) k_means_backward(UpdArgs u, AdjArgs a, const float *__restrict__ img,
                                                        const int32_t *__restrict__ hole, int nh,
                                                        const uint8_t *__restrict__ dom, const int2 *__restrict__ nnf,
                                                        const float *__restrict__ conf, const float *__restrict__ g,
                                                        double *__restrict__ gacc, double *__restrict__ partials)
{
	__shared__ double red[8];
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	double dsig = 0.0;
	if (i < nh) {
		const int W = u.W, H = u.H, C = u.C;
		const int pix = hole[i];
		const int x = pix % W, y = pix / W;
		const int x_a = max(x - u.hx, 0), x_b = min(x + u.hx, W - 1);
		const int y_a = max(y - u.hy, 0), y_b = min(y + u.hy, H - 1);
		float tv[4] = {0.f, 0.f, 0.f, 0.f};
		float tw = 0.f;
		for (int ii = x_a; ii <= x_b; ii++)
			for (int jj = y_a; jj <= y_b; jj++) {
				int2 q = nnf[jj * W + ii];
				if (q.x == -1) continue;
				q.x += x - ii;
				q.y += y - jj;
				if (q.x < 0 || q.y < 0 || q.x >= W || q.y >= H) continue;
				float w = u.weights[(jj - y_a) * u.px + (ii - x_a)];
				if (conf && dom[jj * W + ii]) w = fm(w, conf[jj * W + ii]);
				tw = fa(tw, w);
				const float *sv = img + (size_t)C * (q.y * W + q.x);
				for (int c = 0; c < C; c++) tv[c] = fa(tv[c], fm(sv[c], w));
			}
		const float *gp = g + (size_t)C * pix;
		if (tw > 0.0f) {
			float out[4];
			for (int c = 0; c < C; c++) out[c] = __fdiv_rn(tv[c], tw);
			const double inv = 1.0 / (double)tw;
			for (int ii = x_a; ii <= x_b; ii++)
				for (int jj = y_a; jj <= y_b; jj++) {
					int2 q = nnf[jj * W + ii];
					if (q.x == -1) continue;
					q.x += x - ii;
					q.y += y - jj;
					if (q.x < 0 || q.y < 0 || q.x >= W || q.y >= H) continue;
					const int k = (jj - y_a) * u.px + (ii - x_a);
					float w = u.weights[k];
					if (conf && dom[jj * W + ii]) w = fm(w, conf[jj * W + ii]);
					const double wd = (double)w * inv, rho = tap_rho(u, a, k);
					const size_t s = (size_t)C * (q.y * W + q.x);
					for (int c = 0; c < C; c++) {
						atomicAdd(gacc + s + c, (double)gp[c] * wd);
						dsig += (double)gp[c] * wd * rho * ((double)img[s + c] - (double)out[c]);
					}
				}
		} else {
			for (int c = 0; c < C; c++) atomicAdd(gacc + (size_t)C * pix + c, (double)gp[c]);
		}
	}
	dsig = block_sum<256>(dsig, red);
	if (threadIdx.x == 0) partials[blockIdx.x] = dsig;
}

// NL-Poisson, per pixel q: the adjoints of the coefficients S(q), U(q),
// GX(q), GY(q) for the residual F_k = lambda U_k - (1-lambda) D_k -
// lambda S_k out_k + (1-lambda) sum_nb s_nb(k) (out_nb - out_k) (D = the
// backward divergence of (GX, GY), s_up / s_left = S of that neighbour,
// s_down / s_right = S_k), weighted by the adjoint solution z = A^-1 g on
// the hole; the boundary-coupling part of dL/du for pixels outside the
// hole; and dL/dlambda per hole pixel.
struct AdjCoef {
	float *dS;   // W*H
	float *dU;   // W*H*C
	float *dGX;  // W*H*C
	float *dGY;  // W*H*C
	uint8_t *active;
};

__global__ void k_poisson_adj_coef(PoissonArgs pa, CoefOut co, AdjCoef ad, const uint8_t *__restrict__ dom,
                                   const float *__restrict__ out, const float *__restrict__ z,
                                   double *__restrict__ gacc,
                                   double *__restrict__ lam_part, int depth)
{
	__shared__ double red[2][8];
	const int W = pa.W, H = pa.H, C = pa.C;
	const int q = blockIdx.x * blockDim.x + threadIdx.x;
	double dl = 0.0, dld = 0.0;
	if (q < W * H) {
		const int x = q % W, y = q / W;
		const bool hq = dom[q] != 0;
		const bool hr = (x != W - 1) && dom[q + 1];
		const bool hd = (y != H - 1) && dom[q + W];
		const bool hl = (x != 0) && dom[q - 1];
		const bool hu = (y != 0) && dom[q - W];
		const bool act = hq || hr || hd;
		ad.active[q] = act ? 1 : 0;
		float dS = 0.f;
		for (int c = 0; c < C; c++) {
			const float lam = pa.lambda[c], oml = 1.0f - lam;
			const size_t o = (size_t)C * q + c;
			const float zq = hq ? z[o] : 0.f;
			const float zr = hr ? z[o + C] : 0.f;
			const float zd = hd ? z[o + (size_t)C * W] : 0.f;
			const float oq = out[o];
			if (act) {
				ad.dU[o] = lam * zq;
				ad.dGX[o] = (x != W - 1) ? oml * (zr - zq) : 0.f;
				ad.dGY[o] = (y != H - 1) ? oml * (zd - zq) : 0.f;
				float s = 0.f;
				if (hq) {
					s -= lam * oq;
					if (y != H - 1) s += oml * (out[o + (size_t)C * W] - oq);
					if (x != W - 1) s += oml * (out[o + C] - oq);
					s *= zq;
				}
				if (hd) s += zd * oml * (oq - out[o + (size_t)C * W]);
				if (hr) s += zr * oml * (oq - out[o + C]);
				dS += s;
			}
			if (hq) {
				// dF_k / dlambda
				const float Sk = co.S[q];
				float Dk = 0.f;
				if (x != W - 1) Dk += co.GX[o];
				if (x != 0) Dk -= co.GX[o - C];
				if (y != H - 1) Dk += co.GY[o];
				if (y != 0) Dk -= co.GY[o - (size_t)C * W];
				float lap = 0.f;
				if (y != 0) lap += co.S[q - W] * (out[o - (size_t)C * W] - oq);
				if (x != 0) lap += co.S[q - 1] * (out[o - C] - oq);
				if (y != H - 1) lap += Sk * (out[o + (size_t)C * W] - oq);
				if (x != W - 1) lap += Sk * (out[o + C] - oq);
				const double v = (double)zq * ((double)co.U[o] + Dk - (double)Sk * oq - lap);
				if (depth && c == 3)
					dld += v;
				else
					dl += v;
			} else {
				// the coupling into the hole's stencil, (1 - lambda) sum over
				// hole neighbours k of z_k s_q(k) (the identity part, g, is
				// already in gacc from k_adj_init)
				double v = 0.0;
				if (hd) v += (double)oml * z[o + (size_t)C * W] * co.S[q];       // q is the upper neighbour of k
				if (hu) v += (double)oml * z[o - (size_t)C * W] * co.S[q - W];   // q is the lower neighbour
				if (hr) v += (double)oml * z[o + C] * co.S[q];                   // q is the left neighbour
				if (hl) v += (double)oml * z[o - C] * co.S[q - 1];               // q is the right neighbour
				if (v != 0.0) atomicAdd(gacc + o, v);
			}
		}
		if (act) ad.dS[q] = dS;
	}
	dl = block_sum<256>(dl, red[0]);
	dld = block_sum<256>(dld, red[1]);
	if (threadIdx.x == 0) {
		lam_part[2 * blockIdx.x] = dl;
		lam_part[2 * blockIdx.x + 1] = dld;
	}
}

// Scatter of the coefficient adjoints through the gathers of
// k_poisson_coef: for every active q and every extended-domain centre c of
// its window with n = nnf(c) + q - c in the image,
//   du(n) += w dU(q), gx / gy of n (forward differences of u) take w dGX(q),
//   w dGY(q), and dsigma += dw/dsigma (dS(q) + sum_c dU u(n) + dGX gx(n) +
//   dGY gy(n)).
__global__ void __launch_bounds__(128) k_poisson_adj_scatter(UpdArgs u, AdjArgs a, AdjCoef ad,
                                                             const uint8_t *__restrict__ ext,
                                                             const int2 *__restrict__ nnf,
                                                             const float *__restrict__ conf,
                                                             const float *__restrict__ img,
                                                             const float2 *__restrict__ grad,
                                                             double *__restrict__ gacc, double *__restrict__ partials)
{
	__shared__ double red[4];
	const int W = u.W, H = u.H, C = u.C;
	const int q = blockIdx.x * blockDim.x + threadIdx.x;
	double dsig = 0.0;
	if (q < W * H && ad.active[q]) {
		const int qx = q % W, qy = q / W;
		float dU[4], dGX[4], dGY[4];
		for (int c = 0; c < C; c++) {
			dU[c] = ad.dU[(size_t)C * q + c];
			dGX[c] = ad.dGX[(size_t)C * q + c];
			dGY[c] = ad.dGY[(size_t)C * q + c];
		}
		const double dS = ad.dS[q];
		const int cy0 = max(qy - u.hy, 0), cy1 = min(qy + u.hy, H - 1);
		const int cx0 = max(qx - u.hx, 0), cx1 = min(qx + u.hx, W - 1);
		for (int cy = cy0; cy <= cy1; cy++)
			for (int cx = cx0; cx <= cx1; cx++) {
				const int c0 = cy * W + cx;
				if (!ext[c0]) continue;
				const int2 nb = nnf[c0];
				const int nx = nb.x + qx - cx, ny = nb.y + qy - cy;
				if (nx < 0 || ny < 0 || nx >= W || ny >= H) continue;
				const int k = (qy - cy + u.hy) * u.px + (qx - cx + u.hx);
				const double cf = conf ? (double)conf[c0] : 1.0;
				const double w = cf * (double)u.weights[k];
				const double dw = w * (tap_rho(u, a, k) - a.m);
				const int n = ny * W + nx;
				double t = dS;
				for (int c = 0; c < C; c++) {
					const size_t o = (size_t)C * n + c;
					const float2 gv = grad[o];
					t += (double)dU[c] * img[o] + (double)dGX[c] * gv.x + (double)dGY[c] * gv.y;
					double own = w * dU[c];
					if (nx != W - 1) {
						atomicAdd(gacc + o + C, w * dGX[c]);
						own -= w * dGX[c];
					}
					if (ny != H - 1) {
						atomicAdd(gacc + o + (size_t)C * W, w * dGY[c]);
						own -= w * dGY[c];
					}
					atomicAdd(gacc + o, own);
				}
				dsig += dw * t;
			}
	}
	dsig = block_sum<128>(dsig, red);
	if (threadIdx.x == 0) partials[blockIdx.x] = dsig;
}

__global__ void k_hole_to_planar(const float *__restrict__ g, const int32_t *__restrict__ hole, int nh, int C,
                                 float *__restrict__ b)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= nh * C) return;
	const int k = i % nh, c = i / nh;
	b[i] = g[(size_t)C * hole[k] + c];
}

__global__ void k_to_float(const double *__restrict__ a, size_t n, float *__restrict__ out)
{
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
		out[i] = (float)a[i];
}

static double sum_on_host(nli_ctx *ctx, const double *partials, int n, int stride, int offset)
{
	std::vector<double> h((size_t)n * stride);
	NLI_CUDA(cudaMemcpyAsync(h.data(), partials, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, ctx->stream));
	NLI_CUDA(cudaStreamSynchronize(ctx->stream));
	double s = 0.0;
	for (int i = 0; i < n; i++) s += h[(size_t)i * stride + offset];
	return s;
}

void update_backward_run(nli_ctx *ctx, const nli_update_params &up, const float *image, const float *out,
                         const uint8_t *dom, const uint8_t *ext, const int32_t *nnf_i, const float *conf, int W,
                         int H, int C, const float *grad_out, float *grad_image, double *grad_lambda,
                         double *grad_lambda_d, double *grad_sigma)
{
	NLI_REQUIRE(up.method == NLI_UPDATE_MEANS || up.method == NLI_UPDATE_POISSON || up.method == NLI_UPDATE_DEPTH,
	            NLI_E_UNSUPPORTED, "no adjoint for this update method (the weighted median is piecewise constant)");
	if (up.method == NLI_UPDATE_DEPTH) NLI_REQUIRE(C == 4, NLI_E_CHANNELS, "Separate: Channels do not match.");
	UpdArgs u;
	fill_upd_args(u, up, W, H, C);
	AdjArgs a;
	a.sigma3 = (double)up.sigma * up.sigma * up.sigma;
	a.m = 0.0;
	for (int k = 0; k < u.px * u.py; k++) {
		const int kx = k % u.px - u.hx, ky = k / u.px - u.hy;
		a.m += (double)u.weights[k] * (double)(kx * kx + ky * ky) / a.sigma3;
	}
	cudaStream_t s = ctx->stream;
	const size_t n = (size_t)W * H;
	const int2 *nnf = reinterpret_cast<const int2 *>(nnf_i);
	int32_t *hole = ctx->buf<int32_t>("adj.hole", n);
	const int nh = compact_mask(ctx, dom, W, H, hole, "adj");
	double *gacc = ctx->buf<double>("adj.gacc", n * C);
	k_adj_init<<<(int)std::min<size_t>((n * C + 255) / 256, 8192), 256, 0, s>>>(grad_out, dom, (int)n, C, gacc);
	NLI_CHECK_LAUNCH();
	*grad_lambda = 0.0;
	*grad_lambda_d = 0.0;
	*grad_sigma = 0.0;
	if (nh > 0 && up.method == NLI_UPDATE_MEANS) {
		const int grid = (nh + 255) / 256;
		double *part = ctx->buf<double>("adj.part", grid);
		k_means_backward<<<grid, 256, 0, s>>>(u, a, image, hole, nh, dom, nnf, conf, grad_out, gacc, part);
		NLI_CHECK_LAUNCH();
		*grad_sigma = sum_on_host(ctx, part, grid, 1, 0);
	} else if (nh > 0) {
		int32_t *idx = ctx->buf<int32_t>("upd.hole_index", n);
		k_fill_int<<<(int)((n + 255) / 256), 256, 0, s>>>(idx, (int)n, -1);
		NLI_CHECK_LAUNCH();
		k_hole_index<<<(nh + 255) / 256, 256, 0, s>>>(hole, nh, idx);
		NLI_CHECK_LAUNCH();
		// system of the forward step with orig = image; its right-hand side
		// is replaced by g on the hole, and z = A^-1 g is written as an image
		PoissonSystem P = poisson_system(ctx, u, up, image, image, dom, ext, nnf, conf, hole, idx, nh);
		k_hole_to_planar<<<(nh * C + 255) / 256, 256, 0, s>>>(grad_out, hole, nh, C, P.b);
		NLI_CHECK_LAUNCH();
		NLI_CUDA(cudaMemsetAsync(P.x, 0, sizeof(float) * nh * C, s));
		float *zimg = ctx->buf<float>("adj.z", n * C);
		float *zero = ctx->buf<float>("adj.zero", n * C);
		NLI_CUDA(cudaMemsetAsync(zimg, 0, sizeof(float) * n * C, s));
		NLI_CUDA(cudaMemsetAsync(zero, 0, sizeof(float) * n * C, s));
		const int np = poisson_solve(ctx, P, hole, zero, zimg);
		(void)read_total(ctx, ctx->buf<double>("poi.diff", np + 1), np, ctx->buf<int>("poi.iters", 4), C, nh);
		AdjCoef ad;
		ad.dS = ctx->buf<float>("adj.dS", n);
		ad.dU = ctx->buf<float>("adj.dU", n * C);
		ad.dGX = ctx->buf<float>("adj.dGX", n * C);
		ad.dGY = ctx->buf<float>("adj.dGY", n * C);
		ad.active = ctx->buf<uint8_t>("adj.active", n);
		const int grid = (int)((n + 255) / 256);
		double *lam_part = ctx->buf<double>("adj.lam", 2 * (size_t)grid);
		k_poisson_adj_coef<<<grid, 256, 0, s>>>(P.pa, P.co, ad, dom, out, zimg, gacc, lam_part,
		                                        up.method == NLI_UPDATE_DEPTH ? 1 : 0);
		NLI_CHECK_LAUNCH();
		const int grid2 = (int)((n + 127) / 128);
		double *sig_part = ctx->buf<double>("adj.sig", grid2);
		k_poisson_adj_scatter<<<grid2, 128, 0, s>>>(u, a, ad, ext, nnf, conf, image,
		                                            reinterpret_cast<const float2 *>(ctx->buf<float>("poi.grad", n * 2 * C)),
		                                            gacc, sig_part);
		NLI_CHECK_LAUNCH();
		*grad_lambda = sum_on_host(ctx, lam_part, grid, 2, 0);
		*grad_lambda_d = sum_on_host(ctx, lam_part, grid, 2, 1);
		*grad_sigma = sum_on_host(ctx, sig_part, grid2, 1, 0);
	}
	k_to_float<<<(int)std::min<size_t>((n * C + 255) / 256, 8192), 256, 0, s>>>(gacc, n * C, grad_image);
	NLI_CHECK_LAUNCH();
	NLI_CUDA(cudaStreamSynchronize(s));
}

}  // namespace nli
