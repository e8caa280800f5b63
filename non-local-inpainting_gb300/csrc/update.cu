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
__global__ void __launch_bounds__(256) k_nlmeans(UpdArgs u, const float *__restrict__ img,
                                                 const int32_t *__restrict__ hole, int nh,
                                                 const uint8_t *__restrict__ dom, const int2 *__restrict__ nnf,
                                                 const float *__restrict__ conf, float *__restrict__ newval,
                                                 double *__restrict__ partials)
{
	__shared__ double red[8];
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	double acc = 0.0;
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
				if (q.x != -1) {
					q.x += x - ii;
					q.y += y - jj;
					if (q.x >= 0 && q.y >= 0 && q.x < W && q.y < H) {
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
			newval[(size_t)C * i + c] = v;
		}
	}
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
	if (i < nh) {
		const int W = u.W, H = u.H, C = u.C;
		const int pix = hole[i];
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
					if (qx >= 0 && qy >= 0 && qx < W && qy < H) {
						valid = true;
						w = u.weights[(jj - y_a) * u.px + (ii - x_a)];
						if (conf && dom[jj * W + ii]) w = fm(w, conf[jj * W + ii]);
					}
				}
			}
			const unsigned bal = __ballot_sync(0xffffffffu, valid);
			if (valid) {
				const int slot = m + __popc(bal & ((1u << lane) - 1u));
				s_w[wid][slot] = w;
				for (int c = 0; c < C; c++) s_val[wid][c][slot] = img[(size_t)C * (qy * W + qx) + c];
			}
			m += __popc(bal);
		}
		__syncwarp();
		if (m > 0) {
			// total weight, summed in candidate order (:80)
			float tw = 0.f;
			if (lane == 0)
				for (int k = 0; k < m; k++) tw = fa(tw, s_w[wid][k]);
			tw = __shfl_sync(0xffffffffu, tw, 0);
			for (int c = 0; c < C; c++) {
				for (int k = lane; k < m; k += 32) {
					const float v = s_val[wid][c][k];
					int rank = 0;
					for (int j = 0; j < m; j++) {
						const float o = s_val[wid][c][j];
						rank += (o < v || (o == v && j < k)) ? 1 : 0;
					}
					s_sv[wid][rank] = v;
					s_sw[wid][rank] = s_w[wid][k];
				}
				__syncwarp();
				if (lane == 0) {
					float median = 0.0f;
					float t = tw;
					const float half = tw / 2;
					for (int k = 0; k < m; k++) {
						t = fs(t, s_sw[wid][k]);
						if (t < half) {
							median = s_sv[wid][k];
							break;
						}
					}
					const float prev = img[(size_t)C * pix + c];
					const float d = fs(prev, median);
					acc += (double)fm(d, d);
					newval[(size_t)C * i + c] = median;
				}
				__syncwarp();
			}
		} else if (lane == 0) {
			for (int c = 0; c < C; c++) newval[(size_t)C * i + c] = img[(size_t)C * pix + c];
		}
	}
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

__device__ __forceinline__ void gather_coef(const UpdArgs &u, int qx, int qy, const uint8_t *__restrict__ ext,
                                            const int2 *__restrict__ nnf, const float *__restrict__ conf,
                                            const float *__restrict__ img, const float2 *__restrict__ grad,
                                            CoefOut out)
{
	const int W = u.W, H = u.H, C = u.C;
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

__global__ void __launch_bounds__(128) k_poisson_coef(UpdArgs u, const int32_t *__restrict__ hole, int nh,
                                                      const uint8_t *__restrict__ dom,
                                                      const uint8_t *__restrict__ ext, const int2 *__restrict__ nnf,
                                                      const float *__restrict__ conf, const float *__restrict__ img,
                                                      const float2 *__restrict__ grad, CoefOut out)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= nh) return;
	const int W = u.W;
	const int pix = hole[i];
	const int x = pix % W, y = pix / W;
	gather_coef(u, x, y, ext, nnf, conf, img, grad, out);
	// left neighbour: owned by this hole pixel when it is not a hole pixel
	if (x > 0 && !dom[pix - 1]) gather_coef(u, x - 1, y, ext, nnf, conf, img, grad, out);
	// upper neighbour: owned here when it is neither a hole pixel nor the left
	// neighbour of a hole pixel (then its right neighbour owns it)
	if (y > 0 && !dom[pix - W] && !(x + 1 < W && dom[pix - W + 1]))
		gather_coef(u, x, y - 1, ext, nnf, conf, img, grad, out);
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
};

struct PoissonArgs {
	int W, H, C, nh;
	float lambda[4];
	float tol;
	int limit;
};

// Right-hand side b and initial perturbation delta0 = image - orig
// (patch_non_local_poisson.cpp:62-82), and the per-unknown system data.
__global__ void k_poisson_setup(PoissonArgs a, const int32_t *__restrict__ hole, const int32_t *__restrict__ hole_index,
                                CoefOut co, const float *__restrict__ img, const float *__restrict__ orig,
                                Unknown *__restrict__ unk, float *__restrict__ b, float *__restrict__ x0)
{
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= a.nh) return;
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

// Deterministic grid reduction: every block sums the per-block partials in
// the same order, so all blocks see identical totals.
__device__ __forceinline__ void reduce_partials(const double *__restrict__ part, int nblocks, int C, double *out,
                                                double *smem)
{
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	if (wid < C) {
		double v = 0.0;
		for (int b = lane; b < nblocks; b += 32) v += __ldcg(part + (size_t)b * 4 + wid);
		v = warp_sum(v);
		if (lane == 0) smem[wid] = v;
	}
	__syncthreads();
	for (int c = 0; c < C; c++) out[c] = smem[c];
	__syncthreads();
}

// Conjugate gradient of conjugte_gradient (:387-477) for all channels at
// once: r = b - A x0, d = r; per iteration q = A d, alpha = |r|^2 / <r,q>,
// x += alpha d, r -= alpha q, beta = |r_new|^2 / |r|^2, d = r + beta d; a
// channel stops when |r|^2 < tol |r0|^2 or after `limit` iterations.
// Vectors are float, inner products double.  The grid is co-resident
// (cooperative launch) and phases are separated by the bounded barrier.
// Ends by writing u = orig + x into the image and the partial sums of
// (u_old - u_new)^2.
__global__ void __launch_bounds__(kCgBlock) k_poisson_cg(PoissonArgs a, const Unknown *__restrict__ unk,
                                                         const float *__restrict__ b, float *__restrict__ x,
                                                         float *__restrict__ r, float *__restrict__ d,
                                                         float *__restrict__ q, double *__restrict__ part,
                                                         DevStatus *st, int *__restrict__ iters_out,
                                                         const int32_t *__restrict__ hole,
                                                         const float *orig, float *img,
                                                         double *__restrict__ diff_part)
{
	__shared__ double red[kCgBlock / 32][4];
	__shared__ double tot[4];
	const int nh = a.nh, C = a.C;
	const unsigned nb = gridDim.x;
	const int stride = gridDim.x * blockDim.x;
	double *partA = part;                 // [nb][4]
	double *partB = part + (size_t)nb * 4;  // [nb][4]

	auto block_partial = [&](double *v, double *dst) {
		// v[4] per thread -> dst[blockIdx.x][c]
		const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
		for (int c = 0; c < C; c++) {
			double s = warp_sum(v[c]);
			if (lane == 0) red[wid][c] = s;
		}
		__syncthreads();
		if (threadIdx.x < C) {
			double s = 0.0;
			for (int w = 0; w < kCgBlock / 32; w++) s += red[w][threadIdx.x];
			__stcg(dst + (size_t)blockIdx.x * 4 + threadIdx.x, s);
		}
		__syncthreads();
	};

	// r = b - A x0 ; d = r ; |r0|^2
	double acc[4] = {0, 0, 0, 0};
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nh; k += stride) {
		const Unknown n = unk[k];
		for (int c = 0; c < C; c++) {
			const float *xc = x + (size_t)c * nh;
			const float rv = b[(size_t)c * nh + k] - apply_A(n, a.lambda[c], xc, __ldcg(xc + k));
			__stcg(r + (size_t)c * nh + k, rv);
			__stcg(d + (size_t)c * nh + k, rv);
			acc[c] += (double)rv * rv;
		}
	}
	block_partial(acc, partB);
	if (!grid_barrier(st, nb)) return;
	double nr0[4], nr[4];
	reduce_partials(partB, nb, C, nr0, &tot[0]);
	bool active[4];
	int it[4];
	for (int c = 0; c < 4; c++) {
		nr[c] = (c < C) ? nr0[c] : 0.0;
		active[c] = (c < C) && (nr0[c] > 0);
		it[c] = 0;
	}
	for (;;) {
		bool any = false;
		for (int c = 0; c < C; c++) any |= active[c];
		if (!any) break;
		// q = A d ; <r, q>
		for (int c = 0; c < 4; c++) acc[c] = 0.0;
		for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nh; k += stride) {
			const Unknown n = unk[k];
			for (int c = 0; c < C; c++) {
				if (!active[c]) continue;
				const float *dc = d + (size_t)c * nh;
				const float qv = apply_A(n, a.lambda[c], dc, __ldcg(dc + k));
				__stcg(q + (size_t)c * nh + k, qv);
				acc[c] += (double)__ldcg(r + (size_t)c * nh + k) * qv;
			}
		}
		block_partial(acc, partA);
		if (!grid_barrier(st, nb)) return;
		double rq[4];
		reduce_partials(partA, nb, C, rq, &tot[0]);
		float alpha[4];
		for (int c = 0; c < C; c++) alpha[c] = active[c] ? (float)(nr[c] / rq[c]) : 0.f;
		// x += alpha d ; r -= alpha q ; |r|^2
		for (int c = 0; c < 4; c++) acc[c] = 0.0;
		for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nh; k += stride) {
			for (int c = 0; c < C; c++) {
				if (!active[c]) continue;
				const size_t o = (size_t)c * nh + k;
				const float dv = __ldcg(d + o);
				__stcg(x + o, __ldcg(x + o) + alpha[c] * dv);
				const float rv = __ldcg(r + o) - alpha[c] * __ldcg(q + o);
				__stcg(r + o, rv);
				acc[c] += (double)rv * rv;
			}
		}
		block_partial(acc, partB);
		if (!grid_barrier(st, nb)) return;
		double nrn[4];
		reduce_partials(partB, nb, C, nrn, &tot[0]);
		float beta[4];
		for (int c = 0; c < C; c++) {
			beta[c] = active[c] ? (float)(nrn[c] / nr[c]) : 0.f;
			if (active[c]) nr[c] = nrn[c];
		}
		// d = r + beta d
		for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nh; k += stride) {
			for (int c = 0; c < C; c++) {
				if (!active[c]) continue;
				const size_t o = (size_t)c * nh + k;
				__stcg(d + o, __ldcg(r + o) + beta[c] * __ldcg(d + o));
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

__global__ void k_hole_index(const int32_t *__restrict__ hole, int nh, int32_t *__restrict__ index)
{
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k < nh) index[hole[k]] = k;
}

__global__ void k_fill_int(int32_t *p, int n, int v)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = v;
}

static double read_total(nli_ctx *ctx, double *partials, int n, int *cg_iters_dev, int C, int nh = 0)
{
	launch_sum_partials(ctx->stream, partials, n, partials + n);
	char *h = static_cast<char *>(ctx->host_pinned);
	NLI_CUDA(cudaMemcpyAsync(h, partials + n, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
	if (cg_iters_dev)
		NLI_CUDA(cudaMemcpyAsync(h + 64, cg_iters_dev, sizeof(int) * 4, cudaMemcpyDeviceToHost, ctx->stream));
	NLI_CUDA(cudaStreamSynchronize(ctx->stream));
	if (cg_iters_dev) {
		const int *it = reinterpret_cast<const int *>(h + 64);
		for (int c = 0; c < C; c++) {
			ctx->cg_iterations += it[c];
			ctx->cg_unknown_iterations += (int64_t)it[c] * nh;
		}
	}
	return *reinterpret_cast<double *>(h);
}

static void poisson_run(nli_ctx *ctx, const UpdArgs &u, const nli_update_params &up, float *image, const float *orig,
                        const uint8_t *dom, const uint8_t *ext, const int2 *nnf, const float *conf,
                        const int32_t *hole, const int32_t *hole_index, int nh, double *partials_out,
                        int *n_partials)
{
	cudaStream_t s = ctx->stream;
	const int W = u.W, H = u.H, C = u.C;
	const size_t n = (size_t)W * H;
	float *grad = ctx->buf<float>("poi.grad", n * 2 * C);
	launch_gradient(s, image, W, H, C, grad);
	CoefOut co;
	co.S = ctx->buf<float>("poi.S", n);
	co.U = ctx->buf<float>("poi.U", n * C);
	co.GX = ctx->buf<float>("poi.GX", n * C);
	co.GY = ctx->buf<float>("poi.GY", n * C);
	{
	ProfScope ps(ctx, "poisson_coef");
	k_poisson_coef<<<(nh + 127) / 128, 128, 0, s>>>(u, hole, nh, dom, ext, nnf, conf, image,
	                                                 reinterpret_cast<const float2 *>(grad), co);
	NLI_CHECK_LAUNCH();
	}
	PoissonArgs pa;
	pa.W = W;
	pa.H = H;
	pa.C = C;
	pa.nh = nh;
	for (int c = 0; c < 4; c++) pa.lambda[c] = up.lambda;
	if (up.method == NLI_UPDATE_DEPTH) pa.lambda[3] = up.lambda_d;
	pa.tol = up.cg_tol;
	pa.limit = up.cg_iters;
	Unknown *unk = ctx->buf<Unknown>("poi.unk", nh);
	float *b = ctx->buf<float>("poi.b", (size_t)nh * C);
	float *x = ctx->buf<float>("poi.x", (size_t)nh * C);
	float *r = ctx->buf<float>("poi.r", (size_t)nh * C);
	float *d = ctx->buf<float>("poi.d", (size_t)nh * C);
	float *q = ctx->buf<float>("poi.q", (size_t)nh * C);
	{
		ProfScope ps(ctx, "poisson_setup");
		k_poisson_setup<<<(nh + 255) / 256, 256, 0, s>>>(pa, hole, hole_index, co, image, orig, unk, b, x);
		NLI_CHECK_LAUNCH();
	}

	int dev_blocks_per_sm = 0;
	NLI_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&dev_blocks_per_sm, k_poisson_cg, kCgBlock, 0));
	const int max_blocks = dev_blocks_per_sm * ctx->num_sms;
	NLI_REQUIRE(max_blocks > 0, NLI_E_CUDA, "conjugate gradient kernel cannot be made resident");
	int grid = (nh + kCgBlock - 1) / kCgBlock;
	grid = std::min(std::max(grid, 1), std::min(max_blocks, ctx->num_sms));
	double *part = ctx->buf<double>("poi.part", (size_t)grid * 8);
	double *diff_part = ctx->buf<double>("poi.diff", grid + 1);
	int *iters = ctx->buf<int>("poi.iters", 4);
	NLI_CUDA(cudaMemsetAsync(ctx->status, 0, sizeof(DevStatus), s));
	DevStatus *st = ctx->status;
	const float *orig_c = orig;
	void *args[] = {&pa, &unk, &b, &x, &r, &d, &q, &part, &st, &iters, (void *)&hole, &orig_c, &image, &diff_part};
	{
		ProfScope ps(ctx, "poisson_cg");
		NLI_CUDA(cudaLaunchCooperativeKernel((const void *)k_poisson_cg, dim3(grid), dim3(kCgBlock), args, 0, s));
		nli_count_launch_internal();
	}
	*n_partials = grid;
	(void)partials_out;
}

double update_run(nli_ctx *ctx, const nli_update_params &up, float *image, const float *orig, const uint8_t *dom,
                  const uint8_t *ext, const int32_t *nnf_i, const float *conf, int W, int H, int C,
                  const int32_t *hole, int nh, bool read_back)
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
		poisson_run(ctx, u, up, image, orig, dom, ext, nnf, conf, hole, hole_index, nh, nullptr, &np);
		double *diff_part = ctx->buf<double>("poi.diff", np + 1);
		if (!read_back) {
			launch_sum_partials(s, diff_part, np, diff_part + np);
			return 0.0;
		}
		const double t = read_total(ctx, diff_part, np, ctx->buf<int>("poi.iters", 4), C, nh);
		int *hs = static_cast<int *>(ctx->host_pinned) + 128;
		NLI_CUDA(cudaMemcpy(hs, &ctx->status->timeout, sizeof(int), cudaMemcpyDeviceToHost));
		NLI_REQUIRE(*hs == 0, NLI_E_TIMEOUT, "conjugate gradient grid barrier timed out");
		return t;
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
		return 0.0;
	}
	return read_total(ctx, partials, grid, nullptr, C);
}

}  // namespace nli
