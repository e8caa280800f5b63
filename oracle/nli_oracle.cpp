/*
 * TEST INFRASTRUCTURE ONLY -- the oracle.
 *
 * A CPU restatement, in this repository's own code, of the multiscale
 * non-local inpainting path of Tom-Zheng/non-local-inpainting.  Each
 * function cites the reference lines it follows.  It keeps the reference's
 * arithmetic types and evaluation order (float per-tap norms, double sums,
 * no FMA contraction -- built with -ffp-contract=off) and draws random
 * numbers from the C library rand() in the same order as the reference's
 * serial PatchMatch, so after srand(seed) it reproduces the reference bit for
 * bit.  That is checked against golden vectors produced by the reference
 * itself (tests/golden/, made by tests/golden/make_golden.py).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
 * this library, and only as the checker / the timed CPU implementation.  The
 * GPU product never links or calls it.
 *
 * Exported symbols are prefixed orc_ and take the structs of include/nli.h.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <ctime>

#include "nli.h"

using std::max;
using std::min;
using std::vector;

namespace {

std::string g_error;

struct Pt {
	int x, y;
};

/* ---------------------------------------------------------------- images */
struct Img {
	int W = 0, H = 0, C = 0;
	vector<float> v;
	Img() {}
	Img(int w, int h, int c, float fill = 0.f) : W(w), H(h), C(c), v((size_t)w * h * c, fill) {}
	float &at(int x, int y, int c = 0) { return v[(size_t)C * ((size_t)W * y + x) + c]; }
	float at(int x, int y, int c = 0) const { return v[(size_t)C * ((size_t)W * y + x) + c]; }
	bool empty() const { return v.empty(); }
};

struct Msk {
	int W = 0, H = 0;
	vector<uint8_t> v;
	Msk() {}
	Msk(int w, int h, uint8_t fill = 0) : W(w), H(h), v((size_t)w * h, fill) {}
	/* FixedMask::test: range checked, false outside (mask.cpp:223-272). */
	bool test(int x, int y) const
	{
		if ((unsigned)x >= (unsigned)W || (unsigned)y >= (unsigned)H) return false;
		return v[(size_t)y * W + x] != 0;
	}
	bool get(int x, int y) const { return v[(size_t)y * W + x] != 0; }
	void set(int x, int y, bool b)
	{
		if ((unsigned)x >= (unsigned)W || (unsigned)y >= (unsigned)H) return;
		v[(size_t)y * W + x] = b ? 1 : 0;
	}
	/* Raster order (MaskIterator / FixedMask::next, mask.cpp:378-390). */
	vector<Pt> points() const
	{
		vector<Pt> p;
		for (int y = 0; y < H; y++)
			for (int x = 0; x < W; x++)
				if (v[(size_t)y * W + x]) p.push_back(Pt{x, y});
		return p;
	}
	bool any() const
	{
		for (uint8_t b : v)
			if (b) return true;
		return false;
	}
};

struct Nnf {
	int W = 0, H = 0;
	vector<Pt> v;
	Nnf() {}
	Nnf(int w, int h) : W(w), H(h), v((size_t)w * h, Pt{-1, -1}) {}
	Pt &at(int x, int y) { return v[(size_t)y * W + x]; }
	const Pt &at(int x, int y) const { return v[(size_t)y * W + x]; }
	bool empty() const { return v.empty(); }
};

Img make_img(const float *p, int W, int H, int C)
{
	Img im(W, H, C);
	std::memcpy(im.v.data(), p, sizeof(float) * im.v.size());
	return im;
}

Msk make_msk(const uint8_t *p, int W, int H)
{
	Msk m(W, H);
	for (size_t i = 0; i < m.v.size(); i++) m.v[i] = p[i] ? 1 : 0;
	return m;
}

Nnf make_nnf(const int32_t *p, int W, int H)
{
	Nnf n(W, H);
	for (size_t i = 0; i < n.v.size(); i++) n.v[i] = Pt{p[2 * i], p[2 * i + 1]};
	return n;
}

void put_nnf(const Nnf &n, int32_t *p)
{
	for (size_t i = 0; i < n.v.size(); i++) {
		p[2 * i] = n.v[i].x;
		p[2 * i + 1] = n.v[i].y;
	}
}

/* ------------------------------------------------------ GaussianWeights */
/* GaussianWeights::calculate, gaussian_weights.cpp:19-79 (SEGMENTS == 1,
 * gaussian_weights.h:23). */
vector<float> gaussian_weights(unsigned sx, unsigned sy, float sigma_x, float sigma_y)
{
	vector<float> w((size_t)sx * sy, 0.0f);
	const unsigned SEG = 1;
	double x_a = -(float)sx / 2;
	double y_a = -(float)sy / 2;
	double step = 1.0 / SEG;
	double half_step = 0.5 / SEG;
	if (sy == 1) {
		for (unsigned i = 0; i <= sx / 2; i++) {
			double value = 0.0;
			for (unsigned s = 0; s < SEG; s++) {
				double x = x_a + i + step * s + half_step;
				value += exp(-(pow(x, 2) / pow(sigma_x, 2)));
			}
			w[i] = value;
		}
	} else {
		for (unsigned i = 0; i <= sx / 2; i++)
			for (unsigned j = 0; j <= sy / 2; j++) {
				double value = 0.0;
				for (unsigned s = 0; s < SEG; s++) {
					double x = x_a + i + step * s + half_step;
					double y = y_a + j + step * s + half_step;
					value += exp(-(pow(x, 2) / (2 * pow(sigma_x, 2)) + pow(y, 2) / (2 * pow(sigma_y, 2))));
				}
				w[sx * j + i] = value;
			}
	}
	for (unsigned i = 0; i <= sx / 2; i++)
		for (unsigned j = 0; j <= sy / 2; j++) {
			float value = w[sx * j + i];
			w[sx * j + (sx - 1 - i)] = value;
			if (sy > 1) {
				w[sx * (sy - 1 - j) + i] = value;
				w[sx * (sy - 1 - j) + (sx - 1 - i)] = value;
			}
		}
	float sum = 0.0;
	for (size_t i = 0; i < w.size(); i++) sum += w[i];
	for (size_t i = 0; i < w.size(); i++) w[i] /= sum;
	return w;
}

/* ------------------------------------------------------------- Gradient */
/* Gradient::calculate, forward in x and y (gradient.cpp:20-75). */
Img gradient(const Img &im)
{
	Img g(im.W, im.H, 2 * im.C);
	for (int x = 0; x < im.W; x++)
		for (int y = 0; y < im.H; y++)
			for (int c = 0; c < im.C; c++) {
				g.at(x, y, 2 * c) = (x == im.W - 1) ? 0.0f : im.at(x + 1, y, c) - im.at(x, y, c);
				g.at(x, y, 2 * c + 1) = (y == im.H - 1) ? 0.0f : im.at(x, y + 1, c) - im.at(x, y, c);
			}
	return g;
}

/* ------------------------------------------------------------ distances */
struct Distance {
	nli_distance_params p;
	vector<float> w;   /* patch weights, lazily built as in the reference */
	Img src, tgt, gs, gt;

	explicit Distance(const nli_distance_params &prm) : p(prm) {}

	/* initialize(): L2Combined / L2RGBD compute both gradients
	 * (l2_combined_patch_distance.cpp:29-36, l2_rgbd_patch_distance.cpp:31-38). */
	void initialize(const Img &s, const Img &t)
	{
		src = s;
		tgt = t;
		if (p.kind == NLI_DIST_L2_COMBINED || p.kind == NLI_DIST_L2_RGBD) {
			gs = gradient(s);
			gt = gradient(t);
		}
	}

	float calculate(Pt sp, Pt tp)
	{
		if (w.empty()) w = gaussian_weights(p.patch_x, p.patch_y, p.sigma, p.sigma);
		switch (p.kind) {
		case NLI_DIST_L2_COMBINED: return l2_combined(sp, tp);
		case NLI_DIST_L2_RGBD: return l2_rgbd(sp, tp);
		case NLI_DIST_L2_NORM: return l2_norm(sp, tp);
		default: return l1_norm(sp, tp);
		}
	}

	/* l2_combined_patch_distance.cpp:39-148 */
	float l2_combined(Pt sp, Pt tp)
	{
		const int rx = p.patch_x / 2, ry = p.patch_y / 2, C = src.C;
		const float *S = src.v.data(), *T = tgt.v.data(), *GS = gs.v.data(), *GT = gt.v.data();
		const float *pw = w.data();
		double distance = 0.0, gdistance = 0.0;
		for (int dy = -ry; dy < p.patch_y - ry; dy++)
			for (int dx = -rx; dx < p.patch_x - rx; dx++, ++pw) {
				float weight = *pw;
				int si = C * (src.W * (sp.y + dy) + (sp.x + dx));
				int ti = C * (tgt.W * (tp.y + dy) + (tp.x + dx));
				if (C == 3 || C == 1) {
					float norm = 0, gnorm = 0;
					if (C == 3) {
						float d0 = S[si] - T[ti], d1 = S[si + 1] - T[ti + 1], d2 = S[si + 2] - T[ti + 2];
						norm = d0 * d0 + d1 * d1 + d2 * d2;
						float e[6];
						for (int k = 0; k < 6; k++) e[k] = GS[si * 2 + k] - GT[ti * 2 + k];
						gnorm = e[0] * e[0] + e[1] * e[1] + e[2] * e[2] + e[3] * e[3] + e[4] * e[4] + e[5] * e[5];
					} else {
						float d0 = S[si] - T[ti];
						norm = d0 * d0;
						float e0 = GS[si * 2] - GT[ti * 2], e1 = GS[si * 2 + 1] - GT[ti * 2 + 1];
						gnorm = e0 * e0 + e1 * e1;
					}
					distance += weight * norm;
					gdistance += weight * gnorm;
				} else {
					double norm = 0.0, gnorm = 0.0;
					for (int c = 0; c < C; c++) {
						float a = S[si + c], b = T[ti + c];
						norm += (a - b) * (a - b);
						float gxa = GS[(si + c) * 2], gxb = GT[(ti + c) * 2];
						float gya = GS[(si + c) * 2 + 1], gyb = GT[(ti + c) * 2 + 1];
						gnorm += (gxa - gxb) * (gxa - gxb) + (gya - gyb) * (gya - gyb);
					}
					distance += weight * norm;
					gdistance += weight * gnorm;
				}
			}
		return (p.lambda * distance + (1 - p.lambda) * gdistance) / ((unsigned)p.patch_x * (unsigned)p.patch_y);
	}

	/* l2_rgbd_patch_distance.cpp:41-117 */
	float l2_rgbd(Pt sp, Pt tp)
	{
		const int rx = p.patch_x / 2, ry = p.patch_y / 2, C = src.C;
		if (C != 4) throw std::runtime_error("L2 RGBD Distance: Channels do not match.");
		const float *S = src.v.data(), *T = tgt.v.data(), *GS = gs.v.data(), *GT = gt.v.data();
		const float *pw = w.data();
		double distance = 0.0, distance_depth = 0.0, gdistance = 0.0, gdistance_depth = 0.0;
		for (int dy = -ry; dy < p.patch_y - ry; dy++)
			for (int dx = -rx; dx < p.patch_x - rx; dx++, ++pw) {
				float weight = *pw;
				double norm = 0.0, norm_depth = 0.0, gnorm = 0.0, gnorm_depth = 0.0;
				int si = C * (src.W * (sp.y + dy) + (sp.x + dx));
				int ti = C * (tgt.W * (tp.y + dy) + (tp.x + dx));
				for (int c = 0; c < C; c++) {
					float a = S[si + c], b = T[ti + c];
					float gxa = GS[(si + c) * 2], gxb = GT[(ti + c) * 2];
					float gya = GS[(si + c) * 2 + 1], gyb = GT[(ti + c) * 2 + 1];
					if (c == 3) {
						norm_depth += (a - b) * (a - b);
						gnorm_depth += (gxa - gxb) * (gxa - gxb) + (gya - gyb) * (gya - gyb);
					} else {
						norm += (a - b) * (a - b);
						gnorm += (gxa - gxb) * (gxa - gxb) + (gya - gyb) * (gya - gyb);
					}
				}
				distance += weight * norm;
				distance_depth += weight * norm_depth;
				gdistance += weight * gnorm;
				gdistance_depth += weight * gnorm_depth;
			}
		return (p.lambda * distance + (1 - p.lambda) * gdistance + p.lambda_d * distance_depth +
		        (1 - p.lambda_d) * gdistance_depth) /
		       ((unsigned)p.patch_x * (unsigned)p.patch_y);
	}

	/* l2_norm_patch_distance.cpp:22-104 (float accumulator) */
	float l2_norm(Pt sp, Pt tp)
	{
		const int rx = p.patch_x / 2, ry = p.patch_y / 2, C = src.C;
		const float *S = src.v.data(), *T = tgt.v.data();
		const float *pw = w.data();
		float distance = 0.0;
		for (int dy = -ry; dy < p.patch_y - ry; dy++)
			for (int dx = -rx; dx < p.patch_x - rx; dx++, ++pw) {
				float weight = *pw;
				int si = C * (src.W * (sp.y + dy) + (sp.x + dx));
				int ti = C * (tgt.W * (tp.y + dy) + (tp.x + dx));
				float norm;
				if (C == 3) {
					float d0 = S[si] - T[ti], d1 = S[si + 1] - T[ti + 1], d2 = S[si + 2] - T[ti + 2];
					norm = d0 * d0 + d1 * d1 + d2 * d2;
				} else if (C == 1) {
					float d0 = S[si] - T[ti];
					norm = d0 * d0;
				} else {
					norm = 0.0;
					for (int c = 0; c < C; c++) {
						float a = S[si + c], b = T[ti + c];
						norm += (a - b) * (a - b);
					}
				}
				distance += weight * norm;
			}
		return distance / ((unsigned)p.patch_x * (unsigned)p.patch_y);
	}

	/* l1_norm_patch_distance.cpp:22-105 (float accumulator) */
	float l1_norm(Pt sp, Pt tp)
	{
		const int rx = p.patch_x / 2, ry = p.patch_y / 2, C = src.C;
		const float *S = src.v.data(), *T = tgt.v.data();
		const float *pw = w.data();
		float distance = 0.0;
		for (int dy = -ry; dy < p.patch_y - ry; dy++)
			for (int dx = -rx; dx < p.patch_x - rx; dx++, ++pw) {
				float weight = *pw;
				int si = C * (src.W * (sp.y + dy) + (sp.x + dx));
				int ti = C * (tgt.W * (tp.y + dy) + (tp.x + dx));
				float norm;
				if (C == 3) {
					norm = std::fabs(S[si] - T[ti]) + std::fabs(S[si + 1] - T[ti + 1]) +
					       std::fabs(S[si + 2] - T[ti + 2]);
				} else if (C == 1) {
					norm = std::fabs(S[si] - T[ti]);
				} else {
					norm = 0.0;
					for (int c = 0; c < C; c++) norm += std::fabs(S[si + c] - T[ti + c]);
				}
				distance += weight * norm;
			}
		return distance / ((unsigned)p.patch_x * (unsigned)p.patch_y);
	}
};

/* ----------------------------------------------------------- PatchMatch */
struct PmMetrics {
	vector<double> energy;
	vector<int> propagations;
};

/* PatchMatch::calculate, serial build (patch_match.cpp:311-512), with the
 * METRICS bookkeeping (:383-397, :452-455, :501-507). */
Nnf patchmatch_serial(Distance &dist, const nli_patchmatch_params &pm, const Img &source,
                      const Msk &smask, const Img &target, const Msk &tmask, const Nnf &init,
                      PmMetrics *metrics, vector<float> *out_dist)
{
	dist.initialize(source, target);
	const int tW = target.W, tH = target.H, sW = source.W, sH = source.H;
	vector<float> distances((size_t)tW * tH, std::numeric_limits<float>::max());
	Nnf nb(tW, tH);
	vector<Pt> tp = tmask.points();
	const int shots = pm.random_shots;

	if (!init.empty() && init.W == tW && init.H == tH) {
		for (size_t i = 0; i < tp.size(); i++) {
			Pt p = tp[i];
			Pt n = init.at(p.x, p.y);
			int tries = 0;
			while (!smask.test(n.x, n.y) && tries < shots) {
				n.x = rand() % sW;
				n.y = rand() % sH;
				tries++;
			}
			if (smask.test(n.x, n.y)) {
				nb.at(p.x, p.y) = n;
				distances[(size_t)p.y * tW + p.x] = dist.calculate(n, p);
			}
		}
	} else {
		for (size_t i = 0; i < tp.size(); i++) {
			Pt p = tp[i];
			Pt n = Pt{-1, -1};
			int tries = 0;
			while ((n.x < 0 || !smask.get(n.x, n.y)) && tries < shots) {
				n.x = rand() % sW;
				n.y = rand() % sH;
				tries++;
			}
			if (smask.test(n.x, n.y)) {
				nb.at(p.x, p.y) = n;
				distances[(size_t)p.y * tW + p.x] = dist.calculate(n, p);
			}
		}
	}

	for (int iter = 0; iter < pm.iterations; iter++) {
		int props = 0;
		double total = 0.0;
		int index, index_end, shift;
		if (iter % 2 == 0) {
			index = 0;
			index_end = (int)tp.size();
			shift = -1;
		} else {
			index = (int)tp.size() - 1;
			index_end = -1;
			shift = 1;
		}
		for (; index != index_end; index -= shift) {
			int x = tp[index].x, y = tp[index].y;
			float d = distances[(size_t)y * tW + x];
			float original = d;
			Pt n{-1, -1};
			if (tmask.test(x + shift, y)) {
				Pt c = nb.at(x + shift, y);
				c.x -= shift;
				if (smask.test(c.x, c.y)) {
					float cd = dist.calculate(c, Pt{x, y});
					if (cd < d) {
						d = cd;
						n = c;
					}
				}
			}
			if (tmask.test(x, y + shift)) {
				Pt c = nb.at(x, y + shift);
				c.y -= shift;
				if (smask.test(c.x, c.y)) {
					float cd = dist.calculate(c, Pt{x, y});
					if (cd < d) {
						d = cd;
						n = c;
					}
				}
			}
			if (n.x < 0) n = nb.at(x, y);
			else props++;

			int max_window = (pm.window != -1) ? pm.window : max(sW, sH);
			Pt center = n;
			for (int ws = max_window; ws >= 1; ws /= 2) {
				int x_min = max(center.x - ws, 0);
				int y_min = max(center.y - ws, 0);
				int x_max = min(center.x + ws + 1, sW);
				int y_max = min(center.y + ws + 1, sH);
				for (int k = 0; k < shots; k++) {
					Pt c;
					c.x = x_min + rand() % (x_max - x_min);
					c.y = y_min + rand() % (y_max - y_min);
					if (smask.test(c.x, c.y)) {
						float cd = dist.calculate(c, Pt{x, y});
						if (cd < d) {
							d = cd;
							n = c;
						}
						break;
					}
				}
			}
			if (original > d) {
				distances[(size_t)y * tW + x] = d;
				nb.at(x, y) = n;
			}
			total += min(original, d);
		}
		if (metrics) {
			metrics->energy.push_back(total);
			metrics->propagations.push_back(props);
		}
	}
	if (out_dist) *out_dist = distances;
	return nb;
}

/* Base of the OpenMP PatchMatch's per-thread seeds when set by
 * orc_set_parallel_seed (the reference takes time(NULL), :145). */
bool g_par_seed_set = false;
unsigned g_par_seed = 0;

/* PatchMatch::calculate, OpenMP build (patch_match.cpp:65-302).  Thread t
 * draws from rand_r with seed base + t; the reference's base is time(NULL)
 * (:145), so its runs do not repeat.  With orc_set_parallel_seed and a fixed
 * thread count the base is fixed and the run repeats (used to make reference
 * outputs of large images, where the serial variant is too slow). */
Nnf patchmatch_omp(Distance &dist, const nli_patchmatch_params &pm, const Img &source,
                   const Msk &smask, const Img &target, const Msk &tmask, const Nnf &init)
{
	dist.initialize(source, target);
	const int tW = target.W, tH = target.H, sW = source.W, sH = source.H;
	vector<float> d_odd((size_t)tW * tH, std::numeric_limits<float>::max()), d_even = d_odd;
	Nnf n_odd(tW, tH), n_even(tW, tH);
	vector<Pt> tp = tmask.points();
	const int shots = pm.random_shots;
	const bool use_init = !init.empty() && init.W == tW && init.H == tH;
	for (size_t i = 0; i < tp.size(); i++) {
		Pt p = tp[i];
		Pt n = use_init ? init.at(p.x, p.y) : Pt{-1, -1};
		int tries = 0;
		if (use_init) {
			while (!smask.test(n.x, n.y) && tries < shots) {
				n.x = rand() % sW;
				n.y = rand() % sH;
				tries++;
			}
		} else {
			while ((n.x < 0 || !smask.get(n.x, n.y)) && tries < shots) {
				n.x = rand() % sW;
				n.y = rand() % sH;
				tries++;
			}
		}
		if (smask.test(n.x, n.y)) {
			n_odd.at(p.x, p.y) = n;
			n_even.at(p.x, p.y) = n;
			float dd = dist.calculate(n, p);
			d_odd[(size_t)p.y * tW + p.x] = dd;
			d_even[(size_t)p.y * tW + p.x] = dd;
		}
	}
	int xmin = tW, xmax = -1;
	for (Pt p : tp) {
		xmin = min(xmin, p.x);
		xmax = max(xmax, p.x);
	}
	int bbox_w = tp.empty() ? 0 : xmax - xmin + 1;
	unsigned seed0 = g_par_seed_set ? g_par_seed : (unsigned)time(NULL);
	int nthreads = 1;
#ifdef _OPENMP
	nthreads = omp_get_max_threads();
#endif
	if (bbox_w > 0) nthreads = min(nthreads, (int)tp.size() / (2 * bbox_w));
	if (nthreads < 1) nthreads = 1;
#pragma omp parallel num_threads(nthreads)
	{
		int tid = 0, nt = 1;
#ifdef _OPENMP
		tid = omp_get_thread_num();
		nt = omp_get_num_threads();
#endif
		unsigned seed = seed0 + tid;
		int chunk = (int)tp.size() / nt;
		Nnf *mine_n = (tid % 2) ? &n_odd : &n_even;
		Nnf *other_n = (tid % 2) ? &n_even : &n_odd;
		vector<float> *mine_d = (tid % 2) ? &d_odd : &d_even;
		vector<float> *other_d = (tid % 2) ? &d_even : &d_odd;
		for (int iter = 0; iter < pm.iterations; iter++) {
			int ib, ie, shift;
			if (iter % 2 == 0) {
				ib = chunk * tid;
				ie = (tid < nt - 1) ? chunk * (tid + 1) : (int)tp.size();
				shift = -1;
			} else {
				ib = (tid < nt - 1) ? chunk * (tid + 1) - 1 : (int)tp.size() - 1;
				ie = chunk * tid - 1;
				shift = 1;
			}
			for (int index = ib; index != ie; index -= shift) {
				int x = tp[index].x, y = tp[index].y;
				float d = (*mine_d)[(size_t)y * tW + x];
				float original = d;
				Pt n{-1, -1};
				if (tmask.test(x + shift, y)) {
					Pt c = mine_n->at(x + shift, y);
					c.x -= shift;
					if (smask.test(c.x, c.y)) {
						float cd = dist.calculate(c, Pt{x, y});
						if (cd < d) {
							d = cd;
							n = c;
						}
					}
				}
				if (tmask.test(x, y + shift)) {
					Pt c = mine_n->at(x, y + shift);
					c.y -= shift;
					if (smask.test(c.x, c.y)) {
						float cd = dist.calculate(c, Pt{x, y});
						if (cd < d) {
							d = cd;
							n = c;
						}
					}
				}
				if (n.x < 0) n = mine_n->at(x, y);
				int max_window = (pm.window != -1) ? pm.window : max(sW, sH);
				Pt center = n;
				for (int ws = max_window; ws >= 1; ws /= 2) {
					int x_min = max(center.x - ws, 0), y_min = max(center.y - ws, 0);
					int x_max = min(center.x + ws + 1, sW), y_max = min(center.y + ws + 1, sH);
					for (int k = 0; k < shots; k++) {
						Pt c;
						c.x = x_min + rand_r(&seed) % (x_max - x_min);
						c.y = y_min + rand_r(&seed) % (y_max - y_min);
						if (smask.test(c.x, c.y)) {
							float cd = dist.calculate(c, Pt{x, y});
							if (cd < d) {
								d = cd;
								n = c;
							}
							break;
						}
					}
				}
				if (original > d) {
					(*mine_d)[(size_t)y * tW + x] = d;
					mine_n->at(x, y) = n;
				}
			}
#pragma omp barrier
			if (iter < pm.iterations - 1) {
				int count = 0;
				for (int index = ie + shift; index != ib + shift && count < bbox_w; index += shift, count++) {
					Pt p = tp[index];
					(*other_d)[(size_t)p.y * tW + p.x] = (*mine_d)[(size_t)p.y * tW + p.x];
					other_n->at(p.x, p.y) = mine_n->at(p.x, p.y);
				}
			} else {
				for (int index = ie + shift; index != ib + shift; index += shift) {
					Pt p = tp[index];
					other_n->at(p.x, p.y) = mine_n->at(p.x, p.y);
				}
			}
#pragma omp barrier
		}
	}
	return n_odd;
}

/* --------------------------------------------------------- image updates */
/* PatchNonLocalMeans::update, patch_non_local_means.cpp:23-100. */
double update_means(Img &image, const Msk &dom, const Nnf &nnf, const Img &conf, const vector<float> &w,
                    int px, int py)
{
	const int hx = px / 2, hy = py / 2, C = image.C;
	double total = 0.0;
	vector<Pt> pts = dom.points();
	vector<float> tv(C);
	for (Pt p : pts) {
		int x = p.x, y = p.y;
		int x_a = max(x - hx, 0), x_b = min(x + hx, image.W - 1);
		int y_a = max(y - hy, 0), y_b = min(y + hy, image.H - 1);
		for (int c = 0; c < C; c++) tv[c] = 0.0;
		float tw = 0.0;
		for (int i = x_a; i <= x_b; i++)
			for (int j = y_a; j <= y_b; j++) {
				Pt q = nnf.at(i, j);
				if (q.x != -1) {
					q.x += x - i;
					q.y += y - j;
					if (q.x >= 0 && q.y >= 0 && q.x < image.W && q.y < image.H) {
						float weight = w[(size_t)px * (j - y_a) + (i - x_a)];
						if (!conf.empty() && dom.test(i, j)) weight *= conf.at(i, j);
						tw += weight;
						for (int c = 0; c < C; c++) tv[c] += image.at(q.x, q.y, c) * weight;
					}
				}
			}
		if (tw > 0.0) {
			for (int c = 0; c < C; c++) {
				float color = tv[c] / tw;
				float prev = image.at(x, y, c);
				total += (prev - color) * (prev - color);
				image.at(x, y, c) = color;
			}
		}
	}
	return total;
}

/* PatchNonLocalMedians::update and compute_weighted_median,
 * patch_non_local_medians.cpp:23-127 (std::sort by colour, weights
 * subtracted in sorted order until below half). */
double update_medians(Img &image, const Msk &dom, const Nnf &nnf, const Img &conf, const vector<float> &w,
                      int px, int py)
{
	const int hx = px / 2, hy = py / 2, C = image.C;
	double total = 0.0;
	vector<Pt> pts = dom.points();
	for (Pt p : pts) {
		int x = p.x, y = p.y;
		int x_a = max(x - hx, 0), x_b = min(x + hx, image.W - 1);
		int y_a = max(y - hy, 0), y_b = min(y + hy, image.H - 1);
		float tw = 0.0;
		vector<vector<std::pair<float, float>>> cw(C);
		for (int c = 0; c < C; c++) cw[c].reserve((size_t)px * py);
		for (int i = x_a; i <= x_b; i++)
			for (int j = y_a; j <= y_b; j++) {
				Pt q = nnf.at(i, j);
				if (q.x == -1) continue;
				q.x += x - i;
				q.y += y - j;
				if (q.x >= 0 && q.y >= 0 && q.x < image.W && q.y < image.H) {
					float weight = w[(size_t)px * (j - y_a) + (i - x_a)];
					if (!conf.empty() && dom.test(i, j)) weight *= conf.at(i, j);
					tw += weight;
					for (int c = 0; c < C; c++) cw[c].push_back(std::pair<float, float>(image.at(q.x, q.y, c), weight));
				}
			}
		if (cw[0].size() == 0) continue;
		for (int c = 0; c < C; c++) {
			std::sort(cw[c].begin(), cw[c].end(),
			          [](const std::pair<float, float> &a, const std::pair<float, float> &b) {
				          return a.first < b.first;
			          });
			float median = 0.0;
			float total_weight = tw;
			float half = total_weight / 2;
			for (auto &e : cw[c]) {
				total_weight -= e.second;
				if (total_weight < half) {
					median = e.first;
					break;
				}
			}
			float prev = image.at(x, y, c);
			total += (prev - median) * (prev - median);
			image.at(x, y, c) = median;
		}
	}
	return total;
}

/* calculate_anisotropic_laplacian, patch_non_local_poisson.cpp:291-356. */
void anisotropic_laplacian(double *u, const double *a, const Msk &m)
{
	const int W = m.W, H = m.H;
	vector<Pt> pts = m.points();
	vector<double> buf(pts.size());
	for (size_t i = 0; i < pts.size(); i++) {
		Pt p = pts[i];
		int idx = W * p.y + p.x;
		double at_, ab, ar, al, ut, ub, ur, ul;
		if (p.y != 0) {
			at_ = a[idx - W];
			ut = u[idx - W];
		} else at_ = ut = 0;
		if (p.x != 0) {
			al = a[idx - 1];
			ul = u[idx - 1];
		} else al = ul = 0;
		if (p.y != H - 1) {
			ab = a[idx];
			ub = u[idx + W];
		} else ab = ub = 0;
		if (p.x != W - 1) {
			ar = a[idx];
			ur = u[idx + 1];
		} else ar = ur = 0;
		buf[i] = ut * at_ + ul * al + ub * ab + ur * ar - u[idx] * (at_ + al + ab + ar);
	}
	for (size_t i = 0; i < pts.size(); i++) u[W * pts[i].y + pts[i].x] = buf[i];
}

/* conjugte_gradient, patch_non_local_poisson.cpp:387-477. */
int conjugate_gradient(double *x, const double *a1, const double *a2, const double *b, const Msk &m,
                       float tol, int limit)
{
	const int W = m.W, n = m.W * m.H;
	vector<Pt> pts = m.points();
	vector<double> al(n), d(n, 0.0), r(pts.size(), 0.0);
	std::memcpy(al.data(), x, sizeof(double) * n);
	anisotropic_laplacian(al.data(), a2, m);
	double nr0 = 0.0;
	for (size_t i = 0; i < pts.size(); i++) {
		int idx = W * pts[i].y + pts[i].x;
		r[i] = b[idx] - a1[idx] * x[idx] + al[idx];
		d[idx] = r[i];
		nr0 += r[i] * r[i];
	}
	int iteration = 0;
	double nr = nr0;
	bool stop = !(nr0 > 0);
	while (!stop) {
		std::memcpy(al.data(), d.data(), sizeof(double) * n);
		anisotropic_laplacian(al.data(), a2, m);
		double rdotq = 0.0;
		for (size_t i = 0; i < pts.size(); i++) {
			int idx = W * pts[i].y + pts[i].x;
			rdotq += r[i] * (a1[idx] * d[idx] - al[idx]);
		}
		double alpha = nr / rdotq;
		for (size_t i = 0; i < pts.size(); i++) {
			int idx = W * pts[i].y + pts[i].x;
			x[idx] += alpha * d[idx];
		}
		double nr_old = nr;
		std::memcpy(al.data(), x, sizeof(double) * n);
		anisotropic_laplacian(al.data(), a2, m);
		nr = 0.0;
		for (size_t i = 0; i < pts.size(); i++) {
			int idx = W * pts[i].y + pts[i].x;
			r[i] = b[idx] - a1[idx] * x[idx] + al[idx];
			nr += r[i] * r[i];
		}
		double beta = nr / nr_old;
		for (size_t i = 0; i < pts.size(); i++) {
			int idx = W * pts[i].y + pts[i].x;
			d[idx] = r[i] + beta * d[idx];
		}
		stop = ((nr < tol * nr0) || (iteration >= limit));
		iteration++;
	}
	return iteration;
}

/* PatchNonLocalPoisson::update with calculate_pde_coefficients and
 * calculate_divergence (patch_non_local_poisson.cpp:36-285). */
double update_poisson(Img &image, const Img &orig, const Msk &dom, const Msk &ext, const Nnf &nnf,
                      const Img &conf, const vector<float> &w, int px, int py, float lambda, float cg_tol,
                      int cg_iters, int64_t *cg_count)
{
	const int W = image.W, H = image.H, C = image.C, n = W * H;
	Img grad = gradient(image);
	vector<double> a1(n, 0.0), a2(n, 0.0);
	vector<vector<double>> f1(C, vector<double>(n, 0.0)), f2(C, vector<double>(n, 0.0));
	vector<vector<double>> F1(C, vector<double>(n, 0.0)), F2(C, vector<double>(n, 0.0));
	vector<vector<double>> pert(C, vector<double>(n, 0.0));
	const int hx = px / 2, hy = py / 2;
	/* calculate_pde_coefficients over the extended domain (:139-232) */
	for (Pt it : ext.points()) {
		int x_first = max(it.x - hx, 0), x_last = min(it.x + hx, W - 1);
		int y_first = max(it.y - hy, 0), y_last = min(it.y + hy, H - 1);
		Pt nb = nnf.at(it.x, it.y);
		float confidence = (!conf.empty() && ext.test(it.x, it.y)) ? conf.at(it.x, it.y) : 1.0;
		for (int x = x_first; x <= x_last; x++)
			for (int y = y_first; y <= y_last; y++) {
				int nx = nb.x + x - it.x, ny = nb.y + y - it.y;
				if (nx >= 0 && ny >= 0 && nx < W && ny < H) {
					int idx = W * y + x;
					double weight = confidence * w[(size_t)px * (y - it.y + hy) + (x - it.x + hx)];
					a1[idx] += weight * lambda;
					a2[idx] += weight * (1 - lambda);
					for (int c = 0; c < C; c++) {
						f1[c][idx] += weight * image.at(nx, ny, c) * lambda;
						F1[c][idx] += weight * grad.at(nx, ny, c * 2) * (1 - lambda);
						F2[c][idx] += weight * grad.at(nx, ny, c * 2 + 1) * (1 - lambda);
					}
				}
			}
	}
	if (lambda != 1) {
		/* backward divergence on the extended domain (:235-285) */
		vector<Pt> ep = ext.points();
		for (int c = 0; c < C; c++)
			for (Pt it : ep) {
				int idx = W * it.y + it.x;
				double &dv = f2[c][idx];
				if (it.x == 0) dv = F1[c][idx];
				else if (it.x == W - 1) dv = -F1[c][idx - 1];
				else dv = F1[c][idx] - F1[c][idx - 1];
				if (it.y == 0) dv += F2[c][idx];
				else if (it.y == H - 1) dv += -F2[c][idx - W];
				else dv += F2[c][idx] - F2[c][idx - W];
			}
	}
	vector<vector<double>> oc(C, vector<double>(n));
	for (int i = 0; i < n; i++)
		for (int c = 0; c < C; c++) oc[c][i] = orig.v[(size_t)i * C + c];
	vector<Pt> pts = dom.points();
	for (int c = 0; c < C; c++) {
		vector<double> ch = oc[c];
		anisotropic_laplacian(ch.data(), a2.data(), dom);
		for (Pt it : pts) {
			int idx = W * it.y + it.x;
			f1[c][idx] += -f2[c][idx] - a1[idx] * oc[c][idx] + ch[idx];
			pert[c][idx] = image.at(it.x, it.y, c) - oc[c][idx];
		}
		int it_count = conjugate_gradient(pert[c].data(), a1.data(), a2.data(), f1[c].data(), dom, cg_tol, cg_iters);
		if (cg_count) *cg_count += it_count;
	}
	double total = 0.0;
	for (Pt it : pts) {
		int idx = W * it.y + it.x;
		for (int c = 0; c < C; c++) {
			float color = oc[c][idx] + pert[c][idx];
			float prev = image.at(it.x, it.y, c);
			total += (prev - color) * (prev - color);
			image.at(it.x, it.y, c) = color;
		}
	}
	return total;
}

struct Updater {
	nli_update_params p;
	vector<float> w;
	int64_t cg_iterations = 0;
	explicit Updater(const nli_update_params &prm) : p(prm) {}

	double update(Img &image, const Img &orig, const Msk &dom, const Msk &ext, const Nnf &nnf, const Img &conf)
	{
		if (w.empty()) w = gaussian_weights(p.patch_x, p.patch_y, p.sigma, p.sigma);
		switch (p.method) {
		case NLI_UPDATE_MEANS: return update_means(image, dom, nnf, conf, w, p.patch_x, p.patch_y);
		case NLI_UPDATE_MEDIANS: return update_medians(image, dom, nnf, conf, w, p.patch_x, p.patch_y);
		case NLI_UPDATE_POISSON:
			return update_poisson(image, orig, dom, ext, nnf, conf, w, p.patch_x, p.patch_y, p.lambda, p.cg_tol,
			                      p.cg_iters, &cg_iterations);
		default: {
			/* PatchNonLocalDepth::update (patch_non_local_depth.cpp:36-55): the
			 * inner solvers use tolerance 1e-6 and 1000 iterations whatever
			 * the constructor got (:31-33), and `orig` is the current image (:49). */
			if (image.C != 4) throw std::runtime_error("Separate: Channels do not match.");
			Img rgb(image.W, image.H, 3), depth(image.W, image.H, 1);
			for (int y = 0; y < image.H; y++)
				for (int x = 0; x < image.W; x++) {
					for (int c = 0; c < 3; c++) rgb.at(x, y, c) = image.at(x, y, c);
					depth.at(x, y) = image.at(x, y, 3);
				}
			Img rgb_orig = rgb, depth_orig = depth;
			double total = 0;
			total += update_poisson(rgb, rgb_orig, dom, ext, nnf, conf, w, p.patch_x, p.patch_y, p.lambda,
			                        0.000001f, 1000, &cg_iterations);
			total += update_poisson(depth, depth_orig, dom, ext, nnf, conf, w, p.patch_x, p.patch_y, p.lambda_d,
			                        0.000001f, 1000, &cg_iterations);
			for (int y = 0; y < image.H; y++)
				for (int x = 0; x < image.W; x++) {
					for (int c = 0; c < 3; c++) image.at(x, y, c) = rgb.at(x, y, c);
					image.at(x, y, 3) = depth.at(x, y);
				}
			return total;
		}
		}
	}
};

/* -------------------------------------------------------------- Sampling */
int sample_size(unsigned size, float factor) { return (int)((float)size * factor + 0.5); }

/* symmetric_boundary_condition_A, sampling.cpp:540-553 */
int symmetric_a(int x, int size)
{
	while ((x < 0) || (x >= size)) {
		if (x < 0) x = -x - 1;
		if (x >= size) x = 2 * size - x - 1;
	}
	return x;
}

int neumann(int x, int size) { return max(0, min(size - 1, x)); }

/* separate_convolution, sampling.cpp:415-460 */
void separate_convolution(const float *in, float *out, int W, int H, const float *fx, const float *fy, int nx, int ny)
{
	vector<float> buf((size_t)W * H);
	int radius = (nx - 1) / 2;
	for (int y = 0; y < H; y++)
		for (int x = 0; x < W; x++) {
			float sum = 0.0;
			for (int i = nx - 1; i >= 0; i--) {
				int id = symmetric_a(x + radius - i, W);
				sum += fx[i] * in[y * W + id];
			}
			buf[(size_t)y * W + x] = sum;
		}
	radius = (ny - 1) / 2;
	for (int y = 0; y < H; y++)
		for (int x = 0; x < W; x++) {
			float sum = 0.0;
			for (int i = ny - 1; i >= 0; i--) {
				int id = symmetric_a(y + radius - i, H);
				sum += fy[i] * buf[(size_t)id * W + x];
			}
			out[(size_t)y * W + x] = sum;
		}
}

/* bilinear_interpolation, sampling.cpp:463-506 */
float bilinear(const float *in, int W, int H, float x, float y)
{
	int id_x = std::floor(x), id_y = std::floor(y);
	int x0 = neumann(id_x, W), y0 = neumann(id_y, H), x1 = neumann(id_x + 1, W), y1 = neumann(id_y + 1, H);
	const float p11 = in[x0 + W * y0];
	float a = x - id_x, b = y - id_y;
	float result = 0.0;
	if ((!a) || (!b)) {
		if ((!a) && (!b)) result = p11;
		else if (!a) {
			const float p12 = in[x0 + W * y1];
			result = (1.0 - b) * p11 + b * p12;
		} else {
			const float p21 = in[x1 + W * y0];
			result = (1.0 - a) * p11 + a * p21;
		}
	} else {
		float a_1 = 1.0 - a, b_1 = 1.0 - b;
		const float p21 = in[x1 + W * y0], p12 = in[x0 + W * y1], p22 = in[x1 + W * y1];
		result = b_1 * (a_1 * p11 + a * p21) + b * (a_1 * p12 + a * p22);
	}
	return result;
}

/* downsample_internal(_with_mask), sampling.cpp:250-385 */
void downsample_channel(const float *in, const float *msk_in, float *out, float *msk_out, int W, int H, int sW, int sH)
{
	float factor_x = (float)W / sW, factor_y = (float)H / sH;
	vector<float> fx = gaussian_weights(9, 1, (float)(0.62 * sqrt(pow(factor_x, 2) - 1)), 0);
	vector<float> fy = gaussian_weights(9, 1, (float)(0.62 * sqrt(pow(factor_y, 2) - 1)), 0);
	vector<float> img_f((size_t)W * H), msk_f;
	if (msk_in) {
		vector<float> imx((size_t)W * H);
		for (size_t i = 0; i < imx.size(); i++) imx[i] = msk_in[i] ? in[i] : 0.;
		msk_f.resize((size_t)W * H);
		separate_convolution(msk_in, msk_f.data(), W, H, fx.data(), fy.data(), 9, 9);
		separate_convolution(imx.data(), img_f.data(), W, H, fx.data(), fy.data(), 9, 9);
	} else {
		separate_convolution(in, img_f.data(), W, H, fx.data(), fy.data(), 9, 9);
	}
	float min_x = factor_x / 2.0 - 0.5, min_y = factor_y / 2.0 - 0.5;
	for (unsigned i = 0; i < (unsigned)sH; i++) {
		float y = min_y + i * factor_y;
		for (unsigned j = 0; j < (unsigned)sW; j++) {
			float x = min_x + j * factor_x;
			if (msk_in) {
				float mv = bilinear(msk_f.data(), W, H, x, y);
				float iv = bilinear(img_f.data(), W, H, x, y);
				out[i * sW + j] = (mv > 1e-6) ? iv / mv : 0.f;
				msk_out[i * sW + j] = mv;
			} else {
				out[i * sW + j] = bilinear(img_f.data(), W, H, x, y);
			}
		}
	}
}

/* Sampling::downsample_with_mask, sampling.cpp:114-202 */
void downsample_with_mask(const Img &im, const Msk &m, float factor, float threshold, bool mask_val, Img &out_im,
                          Msk &out_m)
{
	int sW = sample_size(im.W, factor), sH = sample_size(im.H, factor);
	vector<float> fm((size_t)im.W * im.H);
	for (size_t i = 0; i < fm.size(); i++) fm[i] = (mask_val == (m.v[i] != 0)) ? 1.0 : 0.0;
	out_im = Img(sW, sH, im.C);
	out_m = Msk(sW, sH);
	vector<float> cin((size_t)im.W * im.H), cout((size_t)sW * sH), mout((size_t)sW * sH);
	for (int c = 0; c < im.C; c++) {
		for (size_t i = 0; i < cin.size(); i++) cin[i] = im.v[i * im.C + c];
		downsample_channel(cin.data(), fm.data(), cout.data(), mout.data(), im.W, im.H, sW, sH);
		for (size_t i = 0; i < cout.size(); i++) out_im.v[i * im.C + c] = cout[i];
	}
	threshold = fmax(0.0, fmin(1.0, threshold));
	for (size_t i = 0; i < mout.size(); i++) out_m.v[i] = mask_val ? (mout[i] > threshold) : (mout[i] < threshold);
}

/* Sampling::downsample of an image and of a mask (sampling.cpp:19-111),
 * the InitNone branch of ImageInpainting::process (image_inpainting.cpp:91-94). */
Img downsample_image(const Img &im, float factor)
{
	int sW = sample_size(im.W, factor), sH = sample_size(im.H, factor);
	Img out(sW, sH, im.C);
	vector<float> cin((size_t)im.W * im.H), cout((size_t)sW * sH);
	for (int c = 0; c < im.C; c++) {
		for (size_t i = 0; i < cin.size(); i++) cin[i] = im.v[i * im.C + c];
		downsample_channel(cin.data(), nullptr, cout.data(), nullptr, im.W, im.H, sW, sH);
		for (size_t i = 0; i < cout.size(); i++) out.v[i * im.C + c] = cout[i];
	}
	return out;
}

Msk downsample_mask(const Msk &m, float factor, float threshold)
{
	int sW = sample_size(m.W, factor), sH = sample_size(m.H, factor);
	vector<float> fm((size_t)m.W * m.H, 0.0f), sm((size_t)sW * sH, 0.0f);
	for (size_t i = 0; i < fm.size(); i++)
		if (m.v[i]) fm[i] = 1.0;
	downsample_channel(fm.data(), nullptr, sm.data(), nullptr, m.W, m.H, sW, sH);
	threshold = fmax(0.0, fmin(1.0, threshold));
	Msk out(sW, sH);
	for (size_t i = 0; i < sm.size(); i++)
		if (sm[i] > threshold) out.v[i] = 1;
	return out;
}

/* Sampling::upsample with nearest_interpolation, sampling.cpp:205-246, 354-406 */
Img upsample(const Img &im, int sW, int sH)
{
	Img out(sW, sH, im.C);
	float factor_x = (float)sW / im.W, factor_y = (float)sH / im.H;
	float min_x = factor_x / 2.0 - 0.5, min_y = factor_y / 2.0 - 0.5;
	for (unsigned i = 0; i < (unsigned)sH; i++) {
		float y = (i - min_y) / factor_y;
		for (unsigned j = 0; j < (unsigned)sW; j++) {
			float x = (j - min_x) / factor_x;
			int ix = neumann((int)std::floor(x + 0.5), im.W), iy = neumann((int)std::floor(y + 0.5), im.H);
			for (int c = 0; c < im.C; c++) out.at(j, i, c) = im.at(ix, iy, c);
		}
	}
	return out;
}

/* ----------------------------------------------------- DistanceTransform */
float dt_f(int x, int xi, float gi) { return sqrt(pow((float)(x - xi), 2) + pow(gi, 2)); }
int dt_sep(int i, int u, float gi, float gu)
{
	return (pow((float)u, 2) - pow((float)i, 2) + pow(gu, 2) - pow(gi, 2)) / (2 * (u - i));
}

/* DistanceTransform::calculate, distance_transform.cpp:20-99 */
vector<float> distance_transform(const Msk &m)
{
	const int W = m.W, H = m.H;
	vector<float> g((size_t)W * H), out((size_t)W * H);
	const float INF = (unsigned)W + (unsigned)H;
	for (int x = 0; x < W; x++) {
		g[x] = m.get(x, 0) ? INF : 0.0f;
		for (int y = 1; y < H; y++) g[(size_t)y * W + x] = m.get(x, y) ? g[(size_t)(y - 1) * W + x] + 1.0f : 0.0f;
		for (int y = H - 2; y >= 0; y--)
			if (g[(size_t)(y + 1) * W + x] < g[(size_t)y * W + x]) g[(size_t)y * W + x] = g[(size_t)(y + 1) * W + x] + 1.0f;
	}
	vector<int> s(W), t(W);
	for (int y = 0; y < H; y++) {
		const float *gy = &g[(size_t)y * W];
		int q = 0;
		s[0] = 0;
		t[0] = 0;
		for (int u = 1; u < W; u++) {
			while (q >= 0 && dt_f(t[q], s[q], gy[s[q]]) > dt_f(t[q], u, gy[u])) q--;
			if (q < 0) {
				q = 0;
				s[0] = u;
			} else {
				unsigned w = 1 + dt_sep(s[q], u, gy[s[q]], gy[u]);
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
	return out;
}

/* ImageInpainting::calculate_confidence_mask, image_inpainting.cpp:611-630 */
Img confidence_mask(const Msk &dom, float decay, float asym)
{
	Img c(dom.W, dom.H, 1, 1.0f);
	if (decay > 0) {
		vector<float> d = distance_transform(dom);
		for (Pt p : dom.points()) {
			float dist = d[(size_t)p.y * dom.W + p.x];
			c.at(p.x, p.y) = (1 - asym) * std::exp(-dist / decay) + asym;
		}
	} else {
		for (Pt p : dom.points()) c.at(p.x, p.y) = asym;
	}
	return c;
}

/* ImageInpainting::get_extended_domain, image_inpainting.cpp:566-600 */
Msk extended_domain(const Msk &dom, int px, int py)
{
	const int rx = px / 2, ry = py / 2;
	Msk e = dom;
	for (Pt p : dom.points()) {
		int x = p.x, y = p.y;
		bool surrounded = dom.test(x + 1, y) && dom.test(x - 1, y) && dom.test(x, y + 1) && dom.test(x, y - 1);
		if (!surrounded) {
			int xa = max(x - rx, 0), xb = min(x + rx, dom.W - 1);
			int ya = max(y - ry, 0), yb = min(y + ry, dom.H - 1);
			for (int i = xa; i <= xb; i++)
				for (int j = ya; j <= yb; j++)
					if (!dom.get(i, j)) e.set(i, j, true);
		}
	}
	return e;
}

/* ImageInpainting::add_margin, image_inpainting.cpp:641-657 */
void add_margin(Msk &a, Msk &b, int margin)
{
	for (int i = 0; i < margin; i++) {
		for (int x = 0; x < a.W; x++) {
			a.set(x, i, false);
			a.set(x, a.H - i - 1, false);
			b.set(x, i, false);
			b.set(x, b.H - i - 1, false);
		}
		for (int y = 0; y < a.H; y++) {
			a.set(i, y, false);
			a.set(a.W - i - 1, y, false);
			b.set(i, y, false);
			b.set(b.W - i - 1, y, false);
		}
	}
}

/* Source/target masks of inpaint_internal (image_inpainting.cpp:359-384) and
 * of propagate_weights (:501-506, :545-549). */
bool scale_masks(const Msk &ext, int margin, bool erode, Msk &source, Msk &target)
{
	target = ext;
	source = ext;
	for (auto &b : source.v) b = !b;
	bool empty = true;
	if (erode) {
		for (int j = 0; j < source.H; j++)
			for (int i = 0; i < source.W; i++)
				if (source.test(i, j)) {
					if (!source.test(i + 1, j)) source.set(i, j, false);
					else if (!source.test(i, j + 1)) source.set(i, j, false);
					else empty = false;
				}
	}
	add_margin(source, target, margin);
	return empty;
}

/* ------------------------------------------------------------- simpois */
/* 3rdparty/simpois/simpois.c: multiscale Gauss-Seidel Laplace extension,
 * called as poisson_rec(out, in, NULL, w, h, .25, 10, 99, 0) per channel
 * (simpois.c:281-291). */
float sp_get(const float *I, int w, int h, int i, int j)
{
	if (i < 0) i = 0;
	if (j < 0) j = 0;
	if (i >= w) i = w - 1;
	if (j >= h) j = h - 1;
	return I[i + j * w];
}

/* laplacian_neum, simpois.c:61-79 */
float sp_laplacian_neum(const float *I, int w, int h, int i, int j)
{
	float x = sp_get(I, w, h, i, j);
	float a = sp_get(I, w, h, i + 1, j), b = sp_get(I, w, h, i, j + 1);
	float c = sp_get(I, w, h, i - 1, j), d = sp_get(I, w, h, i, j - 1);
	float r = 0;
	if (std::isfinite(a)) r += a - x;
	if (std::isfinite(b)) r += b - x;
	if (std::isfinite(c)) r += c - x;
	if (std::isfinite(d)) r += d - x;
	return r;
}

/* zoom_out_by_factor_two, simpois.c:153-175 */
void sp_zoom_out(float *out, int ow, int oh, const float *in, int iw, int ih)
{
	for (int j = 0; j < oh; j++)
		for (int i = 0; i < ow; i++) {
			float a[4], m = 0;
			a[0] = sp_get(in, iw, ih, 2 * i, 2 * j);
			a[1] = sp_get(in, iw, ih, 2 * i + 1, 2 * j);
			a[2] = sp_get(in, iw, ih, 2 * i, 2 * j + 1);
			a[3] = sp_get(in, iw, ih, 2 * i + 1, 2 * j + 1);
			int cx = 0;
			for (int k = 0; k < 4; k++)
				if (std::isfinite(a[k])) {
					m += a[k];
					cx += 1;
				}
			out[ow * j + i] = cx ? m / cx : NAN;
		}
}

/* zoom_in_by_factor_two with bilinear_interpolation, simpois.c:178-218 */
void sp_zoom_in(float *out, int ow, int oh, const float *in, int iw, int ih)
{
	for (int j = 0; j < oh; j++)
		for (int i = 0; i < ow; i++) {
			float p = (i - 0.5) / 2, q = (j - 0.5) / 2;
			int ip = std::floor(p), iq = std::floor(q);
			float a = sp_get(in, iw, ih, ip, iq), b = sp_get(in, iw, ih, ip + 1, iq);
			float c = sp_get(in, iw, ih, ip, iq + 1), d = sp_get(in, iw, ih, ip + 1, iq + 1);
			float x = p - ip, y = q - iq;
			float r = 0;
			r += a * (1 - x) * (1 - y);
			r += b * (x) * (1 - y);
			r += c * (1 - x) * (y);
			r += d * (x) * (y);
			out[ow * j + i] = r;
		}
}

/* poisson_rec + poisson_extension_with_init + gauss_seidel_iteration,
 * simpois.c:82-100, 126-150, 228-263 (tstep 0.25, niter 10, no data term,
 * no CG refinement). */
void sp_rec(float *u, const float *g, int w, int h, float tstep, int niter, int scale)
{
	vector<float> init((size_t)w * h, 0.0f);
	if (scale > 1 && (w > 1 || h > 1)) {
		int ws = ceil(w / 2.0), hs = ceil(h / 2.0);
		vector<float> gs((size_t)ws * hs), us((size_t)ws * hs);
		sp_zoom_out(gs.data(), ws, hs, g, w, h);
		sp_rec(us.data(), gs.data(), ws, hs, tstep, niter, scale - 1);
		sp_zoom_in(init.data(), w, h, us.data(), ws, hs);
	}
	vector<std::pair<int, int>> omega;
	for (int j = 0; j < h; j++)
		for (int i = 0; i < w; i++)
			if (std::isnan(g[j * w + i])) omega.push_back(std::make_pair(i, j));
	for (int i = 0; i < w * h; i++) u[i] = std::isfinite(g[i]) ? g[i] : init[i];
	for (int it = 0; it < niter; it++)
		for (auto &o : omega) {
			int ij = o.second * w + o.first;
			float l = sp_laplacian_neum(u, w, h, o.first, o.second);
			float d = 0;
			u[ij] = u[ij] + tstep * (l - d);
		}
}

void poisson_init(Img &im, const Msk &m)
{
	const int W = im.W, H = im.H, C = im.C;
	vector<float> in((size_t)W * H), out((size_t)W * H);
	for (int c = 0; c < C; c++) {
		for (int j = 0; j < H; j++)
			for (int i = 0; i < W; i++) in[i + j * W] = m.test(i, j) ? NAN : im.at(i, j, c);
		sp_rec(out.data(), in.data(), W, H, .25, 10, 99);
		for (int j = 0; j < H; j++)
			for (int i = 0; i < W; i++) im.at(i, j, c) = out[i + j * W];
	}
}

/* ------------------------------------------------------- ImageInpainting */
struct Inpainter {
	nli_process_params p;
	Distance dist;
	Updater upd;
	bool parallel;
	nli_process_stats *stats;
	vector<Img> pyr;
	vector<Msk> mpyr;

	Inpainter(const nli_process_params &prm, bool par, nli_process_stats *st)
	    : p(prm), dist(prm.distance), upd(prm.update), parallel(par), stats(st)
	{
	}

	Nnf pm(const Img &s, const Msk &sm, const Img &t, const Msk &tm, const Nnf &init)
	{
		if (stats) stats->patchmatch_calls++;
		if (parallel) return patchmatch_omp(dist, p.patchmatch, s, sm, t, tm, init);
		return patchmatch_serial(dist, p.patchmatch, s, sm, t, tm, init, nullptr, nullptr);
	}

	double update(Img &image, const Img &orig, const Msk &dom, const Msk &ext, const Nnf &nnf, const Img &conf)
	{
		if (stats) stats->update_calls++;
		return upd.update(image, orig, dom, ext, nnf, conf);
	}

	static int iround(float v) { return (v > 0.0) ? floor(v + 0.5) : ceil(v - 0.5); }

	/* inpaint_internal, image_inpainting.cpp:349-417 */
	Nnf inpaint_internal(Img &image, const Msk &dom, const Img &conf, const Nnf &initial, int level)
	{
		int px = p.update.patch_x, py = p.update.patch_y;
		Img original = image;
		Msk ext = extended_domain(dom, px, py);
		Msk source, target;
		bool empty = scale_masks(ext, px / 2, true, source, target);
		if (empty)
			throw std::runtime_error(
			    "ERROR: Empty source mask (no complete patches to copy from. This may happen due to a too big "
			    "inpainting domain, too big patch, or too much downscaling)");
		Nnf nnf = initial;
		double total = std::numeric_limits<double>::max();
		int i;
		for (i = 0; i < p.iterations && total > p.tolerance; i++) {
			nnf = pm(image, source, image, target, nnf);
			total = update(image, original, dom, ext, nnf, conf);
		}
		if (stats && level < NLI_MAX_SCALES) {
			stats->iterations[level] = i;
			stats->last_difference[level] = total;
		}
		return nnf;
	}

	/* propagate_weights, image_inpainting.cpp:492-557 */
	Nnf propagate(Img &upper, const Msk &udom, const Img &uconf, const Img &lower, const Msk &ldom)
	{
		int px = p.update.patch_x, py = p.update.patch_y, half = px / 2;
		Msk lext = extended_domain(ldom, px, py), lsrc, ltgt;
		scale_masks(lext, half, false, lsrc, ltgt);
		Nnf nnf = pm(lower, lsrc, lower, ltgt, Nnf());
		float sx = (float)upper.W / lower.W, sy = (float)upper.H / lower.H;
		Nnf scaled(upper.W, upper.H);
		for (Pt it : ldom.points()) {
			Pt n = nnf.at(it.x, it.y);
			if (n.x >= 0) {
				n.x = iround((float)n.x * sx);
				n.y = iround((float)n.y * sy);
				int x = iround((float)it.x * sx), y = iround((float)it.y * sy);
				scaled.at(x, y) = n;
			}
		}
		Img up = upsample(lower, upper.W, upper.H);
		for (Pt it : udom.points())
			for (int c = 0; c < up.C; c++) upper.at(it.x, it.y, c) = up.at(it.x, it.y, c);
		Msk uext = extended_domain(udom, px, py), usrc, utgt;
		scale_masks(uext, half, false, usrc, utgt);
		Nnf refined = pm(up, usrc, up, utgt, scaled);
		update(upper, upper, udom, uext, refined, uconf);
		return refined;
	}

	/* ImageInpainting::process, image_inpainting.cpp:68-190 */
	Img process(const Img &in, const Msk &mask)
	{
		const int S = p.scales;
		pyr.assign(S, Img());
		mpyr.assign(S, Msk());
		pyr[0] = in;
		mpyr[0] = mask;
		for (int i = 1; i < S; i++) {
			if (p.init != NLI_INIT_NONE) {
				downsample_with_mask(pyr[i - 1], mpyr[i - 1], p.subsampling_rate, 0.4f, false, pyr[i], mpyr[i]);
			} else {
				pyr[i] = downsample_image(pyr[i - 1], p.subsampling_rate);
				mpyr[i] = downsample_mask(mpyr[i - 1], p.subsampling_rate, 0.4f);
			}
		}
		if (stats) {
			stats->scales = S;
			for (int i = 0; i < S && i < NLI_MAX_SCALES; i++) {
				stats->width[i] = pyr[i].W;
				stats->height[i] = pyr[i].H;
			}
		}
		Img &top = pyr.back();
		const Msk &tm = mpyr.back();
		if (p.init == NLI_INIT_AVG || p.init == NLI_INIT_BLACK) {
			vector<float> color(top.C, 0.0f);
			if (p.init == NLI_INIT_AVG)
				for (int c = 0; c < top.C; c++) {
					float sum = 0.0f;
					int count = 0;
					for (int y = 0; y < top.H; y++)
						for (int x = 0; x < top.W; x++)
							if (!tm.get(x, y)) {
								sum += top.at(x, y, c);
								count++;
							}
					if (count > 0) color[c] = sum / (float)count;
				}
			for (Pt q : tm.points())
				for (int c = 0; c < top.C; c++) top.at(q.x, q.y, c) = color[c];
		} else if (p.init == NLI_INIT_POISSON) {
			poisson_init(top, tm);
		}
		Img conf = confidence_mask(tm, p.conf_decay_time, p.conf_asymptotic);
		Nnf nnf = inpaint_internal(top, tm, conf, Nnf(), S - 1);
		for (int i = S - 2; i >= 0; i--) {
			Img c = confidence_mask(mpyr[i], p.conf_decay_time, p.conf_asymptotic);
			nnf = propagate(pyr[i], mpyr[i], c, pyr[i + 1], mpyr[i + 1]);
			nnf = inpaint_internal(pyr[i], mpyr[i], c, nnf, i);
		}
		if (stats) stats->cg_iterations = upd.cg_iterations;
		return pyr[0];
	}
};

}  // namespace

#define ORC_TRY(...)                        \
	try {                                   \
		__VA_ARGS__;                        \
	} catch (const std::exception &e) {     \
		g_error = e.what();                 \
		return NLI_E_EMPTY_SOURCE;          \
	}                                       \
	return NLI_OK;

extern "C" {

const char *orc_last_error(void) { return g_error.c_str(); }
void orc_srand(unsigned seed) { srand(seed); }
/* enable != 0: the OpenMP PatchMatch's thread seeds start at `seed` instead
 * of time(NULL). */
void orc_set_parallel_seed(int enable, unsigned seed)
{
	g_par_seed_set = enable != 0;
	g_par_seed = seed;
}
void orc_set_threads(int n)
{
#ifdef _OPENMP
	if (n > 0) omp_set_num_threads(n);
#else
	(void)n;
#endif
}
int orc_max_threads(void)
{
#ifdef _OPENMP
	return omp_get_max_threads();
#else
	return 1;
#endif
}

int orc_gradient(const float *img, int W, int H, int C, float *out)
{
	Img g = gradient(make_img(img, W, H, C));
	std::memcpy(out, g.v.data(), sizeof(float) * g.v.size());
	return NLI_OK;
}

int orc_gaussian_weights(int sx, int sy, float sigma_x, float sigma_y, float *out)
{
	vector<float> w = gaussian_weights(sx, sy, sigma_x, sigma_y);
	std::memcpy(out, w.data(), sizeof(float) * w.size());
	return NLI_OK;
}

int orc_distance_pairs(const nli_distance_params *p, const float *src, int sW, int sH, const float *tgt, int tW,
                       int tH, int C, const int32_t *pairs, int n, float *out)
{
	ORC_TRY({
		Distance d(*p);
		d.initialize(make_img(src, sW, sH, C), make_img(tgt, tW, tH, C));
		for (int i = 0; i < n; i++)
			out[i] = d.calculate(Pt{pairs[4 * i], pairs[4 * i + 1]}, Pt{pairs[4 * i + 2], pairs[4 * i + 3]});
	});
}

/* Exhaustive argmin with the reference distance; ties keep the lowest
 * raster index of the source.  Patches leaving either image are skipped. */
int orc_bruteforce_nnf(const nli_distance_params *p, const float *src, const uint8_t *smask, int sW, int sH,
                       const float *tgt, const uint8_t *tmask, int tW, int tH, int C, int32_t *nnf, float *dist)
{
	if (p->kind == NLI_DIST_L2_RGBD && C != 4) {
		g_error = "L2 RGBD Distance: Channels do not match.";
		return NLI_E_CHANNELS;
	}
	Distance d(*p);
	d.initialize(make_img(src, sW, sH, C), make_img(tgt, tW, tH, C));
	d.w = gaussian_weights(p->patch_x, p->patch_y, p->sigma, p->sigma);
	const int rx = p->patch_x / 2, ry = p->patch_y / 2;
#pragma omp parallel for schedule(dynamic, 4)
	for (int t = 0; t < tW * tH; t++) {
		int tx = t % tW, ty = t / tW;
		nnf[2 * t] = -1;
		nnf[2 * t + 1] = -1;
		dist[t] = std::numeric_limits<float>::max();
		if (!tmask[t]) continue;
		if (tx - rx < 0 || ty - ry < 0 || tx + (p->patch_x - rx) > tW || ty + (p->patch_y - ry) > tH) continue;
		float best = std::numeric_limits<float>::max();
		int bx = -1, by = -1;
		for (int sy = ry; sy + (p->patch_y - ry) <= sH; sy++)
			for (int sx = rx; sx + (p->patch_x - rx) <= sW; sx++) {
				if (!smask[sy * sW + sx]) continue;
				float v = d.calculate(Pt{sx, sy}, Pt{tx, ty});
				if (v < best) {
					best = v;
					bx = sx;
					by = sy;
				}
			}
		nnf[2 * t] = bx;
		nnf[2 * t + 1] = by;
		dist[t] = best;
	}
	return NLI_OK;
}

/* PatchMatch::calculate after srand(seed) (serial, parallel == 0), or the
 * OpenMP variant (parallel != 0, no metrics). */
int orc_patchmatch(unsigned seed, int parallel, const nli_distance_params *p, const nli_patchmatch_params *pm,
                   const float *src, const uint8_t *smask, int sW, int sH, const float *tgt, const uint8_t *tmask,
                   int tW, int tH, int C, const int32_t *init_nnf, int32_t *out_nnf, float *out_dist, double *energy,
                   int32_t *propagations)
{
	ORC_TRY({
		Distance d(*p);
		srand(seed);
		Nnf init;
		if (init_nnf) init = make_nnf(init_nnf, tW, tH);
		PmMetrics m;
		vector<float> dd;
		Nnf out = parallel ? patchmatch_omp(d, *pm, make_img(src, sW, sH, C), make_msk(smask, sW, sH),
		                                    make_img(tgt, tW, tH, C), make_msk(tmask, tW, tH), init)
		                   : patchmatch_serial(d, *pm, make_img(src, sW, sH, C), make_msk(smask, sW, sH),
		                                       make_img(tgt, tW, tH, C), make_msk(tmask, tW, tH), init, &m, &dd);
		put_nnf(out, out_nnf);
		if (out_dist && !dd.empty()) std::memcpy(out_dist, dd.data(), sizeof(float) * dd.size());
		for (size_t i = 0; i < m.energy.size(); i++) {
			if (energy) energy[i] = m.energy[i];
			if (propagations) propagations[i] = m.propagations[i];
		}
	});
}

/* Reference distance of a whole NNF: sum over target points with a valid
 * match of calculate(nnf(p), p). */
int orc_nnf_energy(const nli_distance_params *p, const float *src, int sW, int sH, const float *tgt, int tW, int tH,
                   int C, const uint8_t *tmask, const int32_t *nnf, double *energy)
{
	ORC_TRY({
		Distance d(*p);
		d.initialize(make_img(src, sW, sH, C), make_img(tgt, tW, tH, C));
		double e = 0.0;
		for (int t = 0; t < tW * tH; t++) {
			if (!tmask[t] || nnf[2 * t] < 0) continue;
			e += d.calculate(Pt{nnf[2 * t], nnf[2 * t + 1]}, Pt{t % tW, t / tW});
		}
		*energy = e;
	});
}

int orc_update(const nli_update_params *p, float *image, const float *orig, const uint8_t *dom, const uint8_t *ext,
               const int32_t *nnf, const float *conf, int W, int H, int C, double *total)
{
	ORC_TRY({
		Updater u(*p);
		Img im = make_img(image, W, H, C);
		Img org = make_img(orig, W, H, C);
		Img cm;
		if (conf) cm = make_img(conf, W, H, 1);
		*total = u.update(im, org, make_msk(dom, W, H), make_msk(ext, W, H), make_nnf(nnf, W, H), cm);
		std::memcpy(image, im.v.data(), sizeof(float) * im.v.size());
	});
}

int orc_sample_size(int size, float factor) { return sample_size(size, factor); }

int orc_downsample_with_mask(const float *img, const uint8_t *mask, int W, int H, int C, float factor, float threshold,
                             int mask_val, float *out_img, uint8_t *out_mask)
{
	Img oi;
	Msk om;
	downsample_with_mask(make_img(img, W, H, C), make_msk(mask, W, H), factor, threshold, mask_val != 0, oi, om);
	std::memcpy(out_img, oi.v.data(), sizeof(float) * oi.v.size());
	std::memcpy(out_mask, om.v.data(), om.v.size());
	return NLI_OK;
}

int orc_upsample(const float *img, int W, int H, int C, int oW, int oH, float *out)
{
	Img o = upsample(make_img(img, W, H, C), oW, oH);
	std::memcpy(out, o.v.data(), sizeof(float) * o.v.size());
	return NLI_OK;
}

int orc_distance_transform(const uint8_t *mask, int W, int H, float *out)
{
	vector<float> d = distance_transform(make_msk(mask, W, H));
	std::memcpy(out, d.data(), sizeof(float) * d.size());
	return NLI_OK;
}

int orc_confidence_mask(const uint8_t *mask, int W, int H, float decay, float asym, float *out)
{
	Img c = confidence_mask(make_msk(mask, W, H), decay, asym);
	std::memcpy(out, c.v.data(), sizeof(float) * c.v.size());
	return NLI_OK;
}

int orc_extended_domain(const uint8_t *mask, int W, int H, int px, int py, uint8_t *out)
{
	Msk e = extended_domain(make_msk(mask, W, H), px, py);
	std::memcpy(out, e.v.data(), e.v.size());
	return NLI_OK;
}

int orc_scale_masks(const uint8_t *ext, int W, int H, int margin, int erode, uint8_t *source, uint8_t *target,
                    int *source_empty)
{
	Msk s, t;
	*source_empty = scale_masks(make_msk(ext, W, H), margin, erode != 0, s, t) ? 1 : 0;
	std::memcpy(source, s.v.data(), s.v.size());
	std::memcpy(target, t.v.data(), t.v.size());
	return NLI_OK;
}

int orc_poisson_init(float *img, const uint8_t *mask, int W, int H, int C)
{
	Img im = make_img(img, W, H, C);
	poisson_init(im, make_msk(mask, W, H));
	std::memcpy(img, im.v.data(), sizeof(float) * im.v.size());
	return NLI_OK;
}

/* Colour conversions of the command-line caller, restated from
 * io_utility.cpp:380-449 (sRGB <-> XYZ <-> L*a*b*, D65 white), keeping its
 * float / double evaluation order and its float pow. */
static float orc_srgb_expand(float v)
{
	return (v > 0.04045) ? std::pow((v + 0.055f) / 1.055f, 2.4f) : v / 12.92;
}

static float orc_lab_f(float t) { return (t > 0.008856f) ? std::pow(t, 1.0f / 3.0f) : (7.787f * t) + (16.0f / 116.0f); }

int orc_rgb_to_lab(const float *rgb, int W, int H, float *lab)
{
	for (long i = 0; i < (long)W * H; i++) {
		const float *c = rgb + 3 * i;
		float r = orc_srgb_expand(c[0] / 255.0f), g = orc_srgb_expand(c[1] / 255.0f), b = orc_srgb_expand(c[2] / 255.0f);
		r *= 100.0f;
		g *= 100.0f;
		b *= 100.0f;
		const float X = r * 0.412453f + g * 0.357580f + b * 0.180423f;
		const float Y = r * 0.212671f + g * 0.715160f + b * 0.072169f;
		const float Z = r * 0.019334f + g * 0.119193f + b * 0.950227f;
		const float fx = orc_lab_f(X / 95.047f), fy = orc_lab_f(Y / 100.000f), fz = orc_lab_f(Z / 108.883f);
		lab[3 * i] = (116.0f * fy) - 16.0f;
		lab[3 * i + 1] = 500.0f * (fx - fy);
		lab[3 * i + 2] = 200.0f * (fy - fz);
	}
	return NLI_OK;
}

static float orc_lab_finv(float t)
{
	const float t3 = std::pow(t, 3.0f);
	return (t3 > 0.008856f) ? t3 : (t - 16.0f / 116.0f) / 7.787f;
}

static float orc_srgb_compress(float v)
{
	return (v > 0.0031308f) ? 1.055f * std::pow(v, 1.0f / 2.4f) - 0.055f : 12.92f * v;
}

int orc_lab_to_rgb(const float *lab, int W, int H, int C, float *rgb)
{
	for (long i = 0; i < (long)W * H; i++) {
		const float *c = lab + (long)C * i;
		const float fy = (c[0] + 16.0f) / 116.0f;
		const float fx = c[1] / 500.0 + fy;
		const float fz = fy - c[2] / 200.0f;
		const float X = orc_lab_finv(fx) * 95.047f, Y = orc_lab_finv(fy) * 100.000f, Z = orc_lab_finv(fz) * 108.883f;
		const float x = X / 100.0f, y = Y / 100.0f, z = Z / 100.0f;
		const float r = x * 3.240479f + y * -1.537150f + z * -0.498535f;
		const float g = x * -0.969256f + y * 1.875992f + z * 0.041556f;
		const float b = x * 0.055648f + y * -0.204043f + z * 1.057311f;
		rgb[3 * i] = orc_srgb_compress(r) * 255.0f;
		rgb[3 * i + 1] = orc_srgb_compress(g) * 255.0f;
		rgb[3 * i + 2] = orc_srgb_compress(b) * 255.0f;
	}
	return NLI_OK;
}

float orc_subsampling_rate(float ratio, unsigned scales)
{
	/* float overloads of exp/log, as the reference resolves them */
	if (ratio < 0.0 || ratio > 1.0) return 0.0;
	return std::exp(std::log(ratio) / (float)(scales - 1));
}

/* ImageInpainting::process after srand(seed); parallel != 0 uses the OpenMP
 * PatchMatch (repeatable only under orc_set_parallel_seed with a fixed
 * thread count).  stats may be NULL. */
int orc_process(unsigned seed, int parallel, const nli_process_params *p, const float *img, const uint8_t *mask, int W,
                int H, int C, float *out, nli_process_stats *stats)
{
	ORC_TRY({
		if (stats) std::memset(stats, 0, sizeof(*stats));
		Inpainter ii(*p, parallel != 0, stats);
		srand(seed);
		Img r = ii.process(make_img(img, W, H, C), make_msk(mask, W, H));
		std::memcpy(out, r.v.data(), sizeof(float) * r.v.size());
	});
}

} /* extern "C" */
