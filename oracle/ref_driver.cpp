/*
 * Test infrastructure only (oracle).  A thin extern "C" driver around the
 * UNMODIFIED reference sources of Tom-Zheng/non-local-inpainting, compiled
 * from their own files by oracle/build.py into oracle/_ref/libnliref.so.  It
 * is used to generate the golden vectors under tests/golden/ and to pin the
 * C++ restatement in oracle/nli_oracle.cpp.  Nothing in the product links it.
 *
 * Every function mirrors one reference entry point; private members are
 * reached by re-declaring `private` as `public` while the reference headers
 * are parsed (access control does not change symbol names).
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <string>
#include <vector>
#include <stdexcept>
#include <utility>
#include <limits>
#include <algorithm>
#include <iostream>
#include <sstream>
#include <iomanip>

#define private public
#define protected public
#include "image.h"
#include "mask.h"
#include "point.h"
#include "shape.h"
#include "gradient.h"
#include "gaussian_weights.h"
#include "sampling.h"
#include "distance_transform.h"
#include "a_patch_distance.h"
#include "l2_combined_patch_distance.h"
#include "l2_rgbd_patch_distance.h"
#include "l2_norm_patch_distance.h"
#include "l1_norm_patch_distance.h"
#include "patch_match.h"
#include "a_image_updating.h"
#include "patch_non_local_means.h"
#include "patch_non_local_medians.h"
#include "patch_non_local_poisson.h"
#include "patch_non_local_depth.h"
#include "image_inpainting.h"
#include "io_utility.h"
#undef private
#undef protected

#include "../include/nli.h"

extern "C" void poisson_solver_separable_simplest(float *out, float *in, float *dat,
                                                  int w, int h, int pd, int niter);

static std::string g_last_error;

#define REF_TRY(...)                                            \
	try {                                                       \
		__VA_ARGS__;                                            \
	} catch (const std::exception &e) {                         \
		g_last_error = e.what();                                \
		return -2;                                              \
	}                                                           \
	return 0;

static Image<float> to_image(const float *data, int W, int H, int C)
{
	Image<float> img((uint)W, (uint)H, (uint)C);
	std::memcpy(img.raw(), data, sizeof(float) * (size_t)W * H * C);
	return img;
}

static void from_image(const FixedImage<float> &img, float *out)
{
	std::memcpy(out, img.raw(), sizeof(float) * (size_t)img.get_size_x() * img.get_size_y() *
	                                img.get_number_of_channels());
}

static Mask to_mask(const uint8_t *data, int W, int H)
{
	Mask m((uint)W, (uint)H);
	for (int y = 0; y < H; y++)
		for (int x = 0; x < W; x++)
			if (data[y * W + x]) m.mask(x, y);
	return m;
}

static void from_mask(const FixedMask &m, uint8_t *out)
{
	int W = m.get_size_x(), H = m.get_size_y();
	for (int y = 0; y < H; y++)
		for (int x = 0; x < W; x++) out[y * W + x] = m.get(x, y) ? 1 : 0;
}

static Image<Point> to_nnf(const int32_t *data, int W, int H)
{
	Image<Point> nnf((uint)W, (uint)H, Point(-1, -1));
	for (int i = 0; i < W * H; i++) nnf.raw()[i] = Point(data[2 * i], data[2 * i + 1]);
	return nnf;
}

static void from_nnf(const FixedImage<Point> &nnf, int32_t *out)
{
	int n = nnf.get_size_x() * nnf.get_size_y();
	for (int i = 0; i < n; i++) {
		out[2 * i] = nnf.raw()[i].x;
		out[2 * i + 1] = nnf.raw()[i].y;
	}
}

static APatchDistance *make_distance(const nli_distance_params *p, Shape &shape)
{
	shape = Shape(p->patch_x, p->patch_y);
	switch (p->kind) {
	case NLI_DIST_L2_COMBINED: return new L2CombinedPatchDistance(p->lambda, shape, p->sigma);
	case NLI_DIST_L2_RGBD: return new L2RGBDPatchDistance(p->lambda, p->lambda_d, shape, p->sigma);
	case NLI_DIST_L2_NORM: return new L2NormPatchDistance(shape, p->sigma);
	case NLI_DIST_L1_NORM: return new L1NormPatchDistance(shape, p->sigma);
	}
	throw std::runtime_error("unknown distance kind");
}

static AImageUpdating *make_updating(const nli_update_params *p)
{
	Shape shape(p->patch_x, p->patch_y);
	switch (p->method) {
	case NLI_UPDATE_MEANS: return new PatchNonLocalMeans(shape, p->sigma);
	case NLI_UPDATE_MEDIANS: return new PatchNonLocalMedians(shape, p->sigma);
	case NLI_UPDATE_POISSON:
		return new PatchNonLocalPoisson(shape, p->sigma, p->lambda, p->cg_tol, p->cg_iters);
	case NLI_UPDATE_DEPTH:
		return new PatchNonLocalDepth(shape, p->sigma, p->lambda, p->lambda_d, p->cg_tol, p->cg_iters);
	}
	throw std::runtime_error("unknown update method");
}

extern "C" {

const char *ref_last_error(void) { return g_last_error.c_str(); }

void ref_srand(unsigned seed) { srand(seed); }

int ref_gradient(const float *img, int W, int H, int C, float *out)
{
	REF_TRY(from_image(Gradient::calculate(to_image(img, W, H, C)), out));
}

int ref_gaussian_weights(int sx, int sy, float sigma_x, float sigma_y, float *out)
{
	REF_TRY(from_image(GaussianWeights::calculate(sx, sy, sigma_x, sigma_y), out));
}

int ref_distance_pairs(const nli_distance_params *p, const float *src, int sW, int sH,
                       const float *tgt, int tW, int tH, int C, const int32_t *pairs, int n,
                       float *out)
{
	REF_TRY({
		Shape shape;
		APatchDistance *d = make_distance(p, shape);
		d->initialize(to_image(src, sW, sH, C), to_image(tgt, tW, tH, C));
		for (int i = 0; i < n; i++)
			out[i] = d->calculate(Point(pairs[4 * i], pairs[4 * i + 1]),
			                      Point(pairs[4 * i + 2], pairs[4 * i + 3]));
		delete d;
	});
}

/* Exhaustive argmin with reference distances; ties keep the lowest raster
 * index of the source (strict < while scanning in raster order). */
int ref_bruteforce_nnf(const nli_distance_params *p, const float *src, const uint8_t *smask,
                       int sW, int sH, const float *tgt, const uint8_t *tmask, int tW, int tH,
                       int C, int32_t *nnf, float *dist)
{
	REF_TRY({
		Shape shape;
		APatchDistance *d = make_distance(p, shape);
		d->initialize(to_image(src, sW, sH, C), to_image(tgt, tW, tH, C));
		int rx = p->patch_x / 2, ry = p->patch_y / 2;
		for (int ty = 0; ty < tH; ty++)
			for (int tx = 0; tx < tW; tx++) {
				int t = ty * tW + tx;
				nnf[2 * t] = -1;
				nnf[2 * t + 1] = -1;
				dist[t] = std::numeric_limits<float>::max();
				if (!tmask[t]) continue;
				if (tx - rx < 0 || ty - ry < 0 || tx + (p->patch_x - rx) > tW ||
				    ty + (p->patch_y - ry) > tH)
					continue;
				float best = std::numeric_limits<float>::max();
				int bx = -1, by = -1;
				for (int sy = ry; sy + (p->patch_y - ry) <= sH; sy++)
					for (int sx = rx; sx + (p->patch_x - rx) <= sW; sx++) {
						if (!smask[sy * sW + sx]) continue;
						float v = d->calculate(Point(sx, sy), Point(tx, ty));
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
		delete d;
	});
}

/* One PatchMatch::calculate call after srand(seed).  energy (iterations
 * doubles) and propagations (iterations ints) are the METRICS vectors
 * (patch_match.cpp:501-507); either may be NULL. */
int ref_patchmatch(unsigned seed, const nli_distance_params *p, const nli_patchmatch_params *pm,
                   const float *src, const uint8_t *smask, int sW, int sH, const float *tgt,
                   const uint8_t *tmask, int tW, int tH, int C, const int32_t *init_nnf,
                   int32_t *out_nnf, double *energy, int32_t *propagations)
{
	REF_TRY({
		Shape shape;
		APatchDistance *d = make_distance(p, shape);
		PatchMatch match(d, pm->iterations, pm->random_shots, pm->window);
		srand(seed);
		Image<Point> init;
		if (init_nnf) init = to_nnf(init_nnf, tW, tH);
		Image<Point> out = match.calculate(to_image(src, sW, sH, C), to_mask(smask, sW, sH),
		                                   to_image(tgt, tW, tH, C), to_mask(tmask, tW, tH), init);
		if (out.is_empty()) {
			delete d;
			throw std::runtime_error("PatchMatch returned an empty field");
		}
		from_nnf(out, out_nnf);
		std::vector<double> e = match.get_total_distance_per_iteration();
		std::vector<int> pr = match.get_propagations_per_iteration_metric();
		for (size_t i = 0; i < e.size(); i++) {
			if (energy) energy[i] = e[i];
			if (propagations) propagations[i] = pr[i];
		}
		delete d;
	});
}

int ref_update(const nli_update_params *p, float *image, const float *orig, const uint8_t *dom,
               const uint8_t *ext, const int32_t *nnf, const float *conf, int W, int H, int C,
               double *total)
{
	REF_TRY({
		AImageUpdating *u = make_updating(p);
		Image<float> img = to_image(image, W, H, C);
		Image<float> org = (orig == image) ? img : to_image(orig, W, H, C);
		Image<float> cm;
		if (conf) cm = to_image(conf, W, H, 1);
		*total = u->update(img, org, to_mask(dom, W, H), to_mask(ext, W, H), to_nnf(nnf, W, H), cm);
		from_image(img, image);
		delete u;
	});
}

int ref_sample_size(int size, float factor) { return Sampling::_Details::get_sample_size(size, factor); }

int ref_downsample_with_mask(const float *img, const uint8_t *mask, int W, int H, int C,
                             float factor, float threshold, int mask_val, float *out_img,
                             uint8_t *out_mask)
{
	REF_TRY({
		std::pair<Image<float>, Mask> r = Sampling::downsample_with_mask(
		    to_image(img, W, H, C), to_mask(mask, W, H), factor, threshold, mask_val != 0);
		from_image(r.first, out_img);
		from_mask(r.second, out_mask);
	});
}

int ref_upsample(const float *img, int W, int H, int C, int oW, int oH, float *out)
{
	REF_TRY(from_image(Sampling::upsample(to_image(img, W, H, C), Shape(oW, oH)), out));
}

int ref_distance_transform(const uint8_t *mask, int W, int H, float *out)
{
	REF_TRY(from_image(DistanceTransform::calculate(to_mask(mask, W, H)), out));
}

int ref_confidence_mask(const uint8_t *mask, int W, int H, float decay, float asym, float *out)
{
	REF_TRY({
		ImageInpainting ii;
		from_image(ii.calculate_confidence_mask(to_mask(mask, W, H), decay, asym), out);
	});
}

int ref_extended_domain(const uint8_t *mask, int W, int H, int px, int py, uint8_t *out)
{
	REF_TRY({
		ImageInpainting ii;
		from_mask(ii.get_extended_domain(to_mask(mask, W, H), Shape(px, py)), out);
	});
}

/* Mask pair of one scale as inpaint_internal builds it (image_inpainting.cpp:
 * 359-384, erode = 1) or as propagate_weights builds it (:501-506, erode = 0).
 * The erosion loop is inline in inpaint_internal and is restated here. */
int ref_scale_masks(const uint8_t *ext, int W, int H, int margin, int erode, uint8_t *source,
                    uint8_t *target, int *source_empty)
{
	REF_TRY({
		Mask e = to_mask(ext, W, H);
		Mask target_mask = e.clone();
		Mask source_mask = e.clone_invert();
		bool empty = true;
		if (erode) {
			for (uint j = 0; j < source_mask.get_size_y(); j++)
				for (uint i = 0; i < source_mask.get_size_x(); i++)
					if (source_mask.test(i, j) == true) {
						if (source_mask.test(i + 1, j) == false) source_mask.unmask(i, j);
						else if (source_mask.test(i, j + 1) == false) source_mask.unmask(i, j);
						else empty = false;
					}
		}
		ImageInpainting ii;
		ii.add_margin(source_mask, target_mask, margin);
		from_mask(source_mask, source);
		from_mask(target_mask, target);
		*source_empty = empty ? 1 : 0;
	});
}

/* InitPoisson branch of ImageInpainting::process (image_inpainting.cpp:
 * 125-153) on an HWC image, in place. */
int ref_poisson_init(float *img, const uint8_t *mask, int W, int H, int C)
{
	std::vector<float> in((size_t)W * H * C), out((size_t)W * H * C);
	for (int c = 0; c < C; c++)
		for (int j = 0; j < H; j++)
			for (int i = 0; i < W; i++)
				in[i + j * W + c * W * H] = mask[j * W + i] ? NAN : img[C * (W * j + i) + c];
	poisson_solver_separable_simplest(out.data(), in.data(), NULL, W, H, C, 10);
	for (int c = 0; c < C; c++)
		for (int j = 0; j < H; j++)
			for (int i = 0; i < W; i++) img[C * (W * j + i) + c] = out[i + j * W + c * W * H];
	return 0;
}

/* IOUtility::rgb_to_lab / lab_to_rgb (io_utility.cpp:268-318) on W*H pixels. */
int ref_rgb_to_lab(const float *rgb, int W, int H, float *lab)
{
	Image<float> in((unsigned)W, (unsigned)H, 3u);
	std::memcpy(in.raw(), rgb, sizeof(float) * 3 * W * H);
	Image<float> out = IOUtility::rgb_to_lab(in);
	std::memcpy(lab, out.raw(), sizeof(float) * 3 * W * H);
	return 0;
}

int ref_lab_to_rgb(const float *lab, int W, int H, int C, float *rgb)
{
	Image<float> in((unsigned)W, (unsigned)H, (unsigned)C);
	std::memcpy(in.raw(), lab, sizeof(float) * C * W * H);
	Image<float> out = IOUtility::lab_to_rgb(in);
	std::memcpy(rgb, out.raw(), sizeof(float) * 3 * W * H);
	return 0;
}

float ref_subsampling_rate(float ratio, unsigned scales)
{
	return ImageInpainting::calculate_subsampling_rate(ratio, scales);
}

/* ImageInpainting::process wired as main.cpp:236-279 does, after srand(seed). */
int ref_process(unsigned seed, const nli_process_params *p, const float *img, const uint8_t *mask,
                int W, int H, int C, float *out)
{
	REF_TRY({
		ImageInpainting ii(p->iterations, p->tolerance, p->scales, p->subsampling_rate,
		                   p->conf_decay_time, p->conf_asymptotic,
		                   (ImageInpainting::InitType)p->init);
		Shape shape;
		APatchDistance *d = make_distance(&p->distance, shape);
		AImageUpdating *u = make_updating(&p->update);
		PatchMatch *pmatch = new PatchMatch(d, p->patchmatch.iterations, p->patchmatch.random_shots,
		                                    p->patchmatch.window);
		ii.set_weights_updating(pmatch);
		ii.set_image_updating(u);
		srand(seed);
		Image<float> result = ii.process(to_image(img, W, H, C), to_mask(mask, W, H));
		from_image(result, out);
		delete pmatch;
		delete d;
		delete u;
	});
}

} /* extern "C" */
