// Host program written against the reference's class interface (wired as
// main.cpp:236-284 wires it), built against the drop-in headers and
// libnli_dropin.so by tests/test_gpu_dropin.py.
//
//   dropin_demo METHOD W H C image.f32 mask.u8 out.f32 SEED
//
// METHOD is nlmeans | nlpoisson | nldepth.  Also exercises the PatchMatch,
// AImageUpdating and APatchDistance objects directly and prints a summary.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "image_inpainting.h"
#include "l2_combined_patch_distance.h"
#include "l2_rgbd_patch_distance.h"
#include "patch_match.h"
#include "patch_non_local_depth.h"
#include "patch_non_local_means.h"
#include "patch_non_local_poisson.h"

static std::vector<char> read_file(const char *name)
{
	FILE *f = fopen(name, "rb");
	if (!f) throw std::runtime_error(std::string("cannot open ") + name);
	std::vector<char> v;
	char buf[1 << 16];
	size_t n;
	while ((n = fread(buf, 1, sizeof(buf), f)) > 0) v.insert(v.end(), buf, buf + n);
	fclose(f);
	return v;
}

int main(int argc, char **argv)
{
	if (argc < 9) {
		fprintf(stderr, "usage: %s METHOD W H C image.f32 mask.u8 out.f32 SEED\n", argv[0]);
		return 1;
	}
	try {
		const std::string method = argv[1];
		const uint W = atoi(argv[2]), H = atoi(argv[3]), C = atoi(argv[4]);
		std::vector<char> ib = read_file(argv[5]), mb = read_file(argv[6]);
		Image<float> input(W, H, C);
		memcpy(input.raw(), ib.data(), sizeof(float) * W * H * C);
		Mask mask(W, H);
		for (uint y = 0; y < H; y++)
			for (uint x = 0; x < W; x++)
				if (mb[y * W + x]) mask.mask(x, y);
		nli_dropin::set_seed(strtoull(argv[8], nullptr, 10));

		// parameters as the CLI sets them (main.cpp:68-82, 217-229)
		const int patch_side = 9, scales = 3;
		Shape patch(patch_side, patch_side);
		const float sigma = 10000.0f, lambda = 0.05f;
		const float rate = ImageInpainting::calculate_subsampling_rate(0.45f, scales);
		ImageInpainting inpainting(20, 0.1f, scales, rate, 5.0f, 0.1f, ImageInpainting::InitPoisson);
		APatchDistance *distance;
		AImageUpdating *updating;
		if (method == "nlmeans") {
			updating = new PatchNonLocalMeans(patch, sigma);
			distance = new L2CombinedPatchDistance(lambda, patch, sigma);
		} else if (method == "nlpoisson") {
			updating = new PatchNonLocalPoisson(patch, sigma, lambda, 0.0001f, 1000);
			distance = new L2CombinedPatchDistance(lambda, patch, sigma);
		} else {
			updating = new PatchNonLocalDepth(patch, sigma, 1.0f, 0.0f, 0.000001f, 1000);
			distance = new L2RGBDPatchDistance(1.0f, 0.0f, patch, sigma);
		}
		PatchMatch *patch_match = new PatchMatch(distance, 10, 30, -1);
		inpainting.set_weights_updating(patch_match);
		inpainting.set_image_updating(updating);
		inpainting.keep_intermediate(true);
		Image<float> output = inpainting.process(input, mask);
		printf("pyramid levels %zu masks %zu nnfs %zu finest nnf %ux%u\n", inpainting.get_output_image_pyramid().size(),
		       inpainting.get_mask_pyramid().size(), inpainting.get_nnf_pyramid().size(),
		       inpainting.get_nnf_pyramid().back().get_size_x(), inpainting.get_nnf_pyramid().back().get_size_y());

		FILE *f = fopen(argv[7], "wb");
		fwrite(output.raw(), sizeof(float), (size_t)W * H * C, f);
		fclose(f);
		const nli_process_stats &st = inpainting.get_statistics();
		printf("scales %d iterations", st.scales);
		for (int i = 0; i < st.scales; i++) printf(" %d", st.iterations[i]);
		printf("\n");

		// the objects on their own: one PatchMatch call and one update on the
		// finest scale with the reference's mask construction
		Mask target(W, H), source(W, H, true);
		for (int y = 0; y < (int)H; y++)
			for (int x = 0; x < (int)W; x++)
				if (mask.test((uint)x, (uint)y))
					for (int j = -4; j <= 4; j++)
						for (int i = -4; i <= 4; i++) {
							target.mask(x + i, y + j);
							source.unmask(x + i, y + j);
						}
		for (uint y = 0; y < H; y++)
			for (uint x = 0; x < W; x++)
				if (x < 4 || y < 4 || x >= W - 4 || y >= H - 4) {
					target.unmask(x, y);
					source.unmask(x, y);
				}
		Image<Point> nnf = patch_match->calculate(output, source, output, target);
		printf("patchmatch energy per sweep %.6g .. %.6g, propagations in sweep 1: %d\n",
		       patch_match->get_total_distance_per_iteration().front(),
		       patch_match->get_total_distance_per_iteration().back(),
		       patch_match->get_propagations_per_iteration_metric().front());
		Point t0 = target.get_masked_points()[0];
		printf("distance %.6g\n", distance->calculate(nnf(t0), t0));
		Image<float> copy = output.clone();
		double total = updating->update(copy, output, mask, target, nnf, Image<float>());
		printf("update total %.6g\n", total);
		Image<Point> bad = patch_match->calculate(output, Mask(W + 1, H), output, target);
		printf("size mismatch gives empty field: %d\n", bad.is_empty() ? 1 : 0);
		delete patch_match;
		delete distance;
		delete updating;
	} catch (const std::exception &e) {
		fprintf(stderr, "exception: %s\n", e.what());
		return 2;
	}
	return 0;
}
