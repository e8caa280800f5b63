// nli_inpaint: the reference's command-line program (main.cpp) on the GPU
// library, built on the drop-in classes of include/nli_inpainting.hpp.
//
//   nli_inpaint input mask output [OPTIONS]
//
// Same options, defaults, checks, messages and object wiring as main.cpp:65-284
// (-method nlmeans|nlmedians|nlpoisson|nldepth, -patch, -iters, -scales,
// -coarse (0: the automatic rule of :166-177), -conft, -confa, -lambda,
// -init, -psigma, -shownnf, -showpyr, -depth, -lambdar, -lambdad), plus
// -seed N (the reference seeds its generator with time(NULL)).  The image is
// inpainted in CIE L*a*b* (:117, :307) with the conversions on the GPU.
//
// Image files: the reference reads and writes through iio on libpng; here
// PNG (csrc/png_codec.cpp, the samples iio's reader returns), binary /
// ASCII PNM (P6, P5, P3, P2) and PFM (PF, Pf) are read with iio's channel
// rules (io_utility.cpp:120-170 over iio.c iio_read_image_float(_vec)), and
// results are written as 8-bit PNG for names ending in ".png" (rounded and
// clamped to 0..255 as iio converts floats), PFM for ".pfm" and binary
// P6 / P5 otherwise.  The composed output name of :287-303 ends in ".png"
// as the reference's.  The inpainted depth goes to inpainted_depth.pfm
// (exact) and to inpainted_depth.png as 8-bit grey in all three channels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <sstream>
#include <string>
#include <vector>

#include "nli_inpainting.hpp"
#include "png_codec.h"

namespace {

// main.cpp:43-58: removes "-name value" (or "-name" when default_value is
// NULL) from argv and returns the value.
const char *pick_option(int *c, char ***v, const char *name, const char *default_value)
{
	int argc = *c;
	char **argv = *v;
	int id = default_value ? 1 : 0;
	for (int i = 0; i < argc - id; i++) {
		if (argv[i][0] == '-' && 0 == strcmp(argv[i] + 1, name)) {
			char *r = argv[i + id] + 1 - id;
			*c -= (id + 1);
			for (int j = i; j < argc - id; j++) (*v)[j] = (*v)[j + id + 1];
			return r;
		}
	}
	return default_value;
}

// ----------------------------------------------------------- image files
// Samples as iio holds them: PNM and PFM are read into floats, PNG into
// 8- or 16-bit integers; the kind matters for the grey conversion.
enum SampleKind { kFloat, kU8, kU16 };

struct Raster {
	int W = 0, H = 0, C = 0;
	SampleKind kind = kFloat;
	std::vector<float> v;
};

Raster read_png(const std::string &name)
{
	FILE *f = fopen(name.c_str(), "rb");
	if (!f) throw std::runtime_error("cannot open " + name);
	std::vector<uint8_t> bytes;
	unsigned char buf[65536];
	size_t n;
	while ((n = fread(buf, 1, sizeof(buf), f)) > 0) bytes.insert(bytes.end(), buf, buf + n);
	fclose(f);
	nli_png::Image im;
	std::string err;
	if (!nli_png::decode(bytes.data(), bytes.size(), im, err)) throw std::runtime_error(name + ": " + err);
	Raster r;
	r.W = im.width;
	r.H = im.height;
	r.C = im.channels;
	r.kind = (im.depth == 16) ? kU16 : kU8;
	r.v.assign(im.samples.begin(), im.samples.end());
	return r;
}

int read_token(FILE *f)
{
	int c = fgetc(f);
	while (c == '#' || isspace(c)) {
		if (c == '#')
			while (c != '\n' && c != EOF) c = fgetc(f);
		c = fgetc(f);
	}
	int v = 0;
	bool any = false;
	while (c >= '0' && c <= '9') {
		v = v * 10 + (c - '0');
		any = true;
		c = fgetc(f);
	}
	if (!any) throw std::runtime_error("malformed image header");
	return v;
}

Raster read_image(const std::string &name)
{
	FILE *f = fopen(name.c_str(), "rb");
	if (!f) throw std::runtime_error("cannot open " + name);
	unsigned char sig[8] = {0};
	const size_t got = fread(sig, 1, 8, f);
	if (nli_png::is_png(sig, got)) {
		fclose(f);
		return read_png(name);
	}
	rewind(f);
	char m[3] = {0, 0, 0};
	if (fread(m, 1, 2, f) != 2 || m[0] != 'P') {
		fclose(f);
		throw std::runtime_error(name + ": not a PNG, PNM or PFM file");
	}
	Raster r;
	if (m[1] == 'F' || m[1] == 'f') {
		r.C = (m[1] == 'F') ? 3 : 1;
		char line[256];
		if (!fgets(line, sizeof(line), f) || !fgets(line, sizeof(line), f) || sscanf(line, "%d %d", &r.W, &r.H) != 2) {
			fclose(f);
			throw std::runtime_error(name + ": malformed PFM header");
		}
		if (!fgets(line, sizeof(line), f)) {
			fclose(f);
			throw std::runtime_error(name + ": malformed PFM header");
		}
		const double scale = atof(line);
		r.v.resize((size_t)r.W * r.H * r.C);
		std::vector<float> row((size_t)r.W * r.C);
		for (int y = r.H - 1; y >= 0; y--) {  // PFM rows run bottom to top
			if (fread(row.data(), sizeof(float), row.size(), f) != row.size()) {
				fclose(f);
				throw std::runtime_error(name + ": truncated PFM data");
			}
			if (scale > 0)  // big-endian data
				for (float &x : row) {
					uint32_t u;
					std::memcpy(&u, &x, 4);
					u = (u >> 24) | ((u >> 8) & 0xff00u) | ((u << 8) & 0xff0000u) | (u << 24);
					std::memcpy(&x, &u, 4);
				}
			std::memcpy(&r.v[(size_t)y * r.W * r.C], row.data(), row.size() * sizeof(float));
		}
	} else {
		const bool ascii = (m[1] == '2' || m[1] == '3');
		r.C = (m[1] == '3' || m[1] == '6') ? 3 : 1;
		if (!(m[1] == '2' || m[1] == '3' || m[1] == '5' || m[1] == '6')) {
			fclose(f);
			throw std::runtime_error(name + ": unsupported PNM type");
		}
		r.W = read_token(f);
		r.H = read_token(f);
		const int maxval = read_token(f);
		r.v.resize((size_t)r.W * r.H * r.C);
		if (ascii) {
			for (float &x : r.v) x = (float)read_token(f);
		} else if (maxval < 256) {
			std::vector<unsigned char> b(r.v.size());
			if (fread(b.data(), 1, b.size(), f) != b.size()) {
				fclose(f);
				throw std::runtime_error(name + ": truncated PNM data");
			}
			for (size_t i = 0; i < b.size(); i++) r.v[i] = b[i];
		} else {
			std::vector<unsigned char> b(2 * r.v.size());
			if (fread(b.data(), 1, b.size(), f) != b.size()) {
				fclose(f);
				throw std::runtime_error(name + ": truncated PNM data");
			}
			for (size_t i = 0; i < r.v.size(); i++) r.v[i] = (float)(b[2 * i] << 8 | b[2 * i + 1]);
		}
	}
	fclose(f);
	return r;
}

// IOUtility::read_rgb_image (io_utility.cpp:150-171): channels 0, 1, 2,
// the second and third taken from the first when the file has fewer (so a
// grey + alpha file gives grey, alpha, grey).
Image<float> rgb_image(const Raster &r)
{
	Image<float> im((uint)r.W, (uint)r.H, 3u);
	float *d = im.raw();
	for (size_t p = 0; p < (size_t)r.W * r.H; p++) {
		const float *s = &r.v[p * r.C];
		d[3 * p] = s[0];
		d[3 * p + 1] = r.C > 1 ? s[1] : s[0];
		d[3 * p + 2] = r.C > 2 ? s[2] : s[0];
	}
	return im;
}

// IOUtility::read_mono_image (io_utility.cpp:120-145) over iio's
// iio_read_image_float: one channel as it is; three or four channels to
// 0.299 R + 0.587 G + 0.114 B in double (iio_hacky_uncolorize(a)), stored
// back into the file's sample type (truncated for 8-bit PNG, a float for
// PNM and PFM); 16-bit colour and grey + alpha files are refused.
Image<float> mono_image(const Raster &r, const std::string &name)
{
	const bool colour = r.C == 3 || r.C == 4;
	if (!(r.C == 1 || colour) || (colour && r.kind == kU16))
		throw std::runtime_error("read_mono_image: cannot read " + name);
	Image<float> im((uint)r.W, (uint)r.H, 1u);
	float *d = im.raw();
	for (size_t p = 0; p < (size_t)r.W * r.H; p++) {
		const float *s = &r.v[p * r.C];
		if (!colour) {
			d[p] = s[0];
		} else {
			const double g = .299 * s[0] + .587 * s[1] + .114 * s[2];
			d[p] = (r.kind == kU8) ? (float)(uint8_t)g : (float)g;
		}
	}
	return im;
}

bool ends_with(const std::string &s, const char *suffix)
{
	const size_t n = strlen(suffix);
	return s.size() >= n && s.compare(s.size() - n, n, suffix) == 0;
}

// iio's float to byte conversion: T8(0.5 + v), 0..255 (iio.c convert_datum)
unsigned char to_byte(float v) { return (unsigned char)std::min(255.0f, std::max(0.0f, std::round(v))); }

void write_image(const std::string &name, const float *v, int W, int H, int C)
{
	if (ends_with(name, ".png") || ends_with(name, ".PNG")) {
		std::vector<uint8_t> b((size_t)W * H * C);
		for (size_t i = 0; i < b.size(); i++) b[i] = to_byte(v[i]);
		const std::vector<uint8_t> png = nli_png::encode8(b.data(), W, H, C);
		FILE *f = fopen(name.c_str(), "wb");
		if (!f) throw std::runtime_error("cannot write " + name);
		const size_t put = fwrite(png.data(), 1, png.size(), f);
		fclose(f);
		if (put != png.size()) throw std::runtime_error("cannot write " + name);
		return;
	}
	FILE *f = fopen(name.c_str(), "wb");
	if (!f) throw std::runtime_error("cannot write " + name);
	const bool pfm = ends_with(name, ".pfm");
	if (pfm) {
		fprintf(f, "%s\n%d %d\n-1.0\n", C == 3 ? "PF" : "Pf", W, H);
		for (int y = H - 1; y >= 0; y--) fwrite(v + (size_t)y * W * C, sizeof(float), (size_t)W * C, f);
	} else {
		fprintf(f, "%s\n%d %d\n255\n", C == 3 ? "P6" : "P5", W, H);
		std::vector<unsigned char> b((size_t)W * H * C);
		for (size_t i = 0; i < b.size(); i++) b[i] = to_byte(v[i]);
		fwrite(b.data(), 1, b.size(), f);
	}
	fclose(f);
}

// ------------------------------------------------ GPU helpers (C ABI)
struct Dev {
	void *p = nullptr;
	explicit Dev(size_t n)
	{
		if (cudaMalloc(&p, n) != cudaSuccess) throw std::runtime_error("cudaMalloc failed");
	}
	~Dev() { cudaFree(p); }
};

Image<float> convert(const Image<float> &in, bool to_lab)
{
	const int W = in.get_size_x(), H = in.get_size_y(), C = in.get_number_of_channels();
	const size_t n = (size_t)W * H;
	Dev a(n * C * sizeof(float)), b(n * 3 * sizeof(float));
	if (cudaMemcpy(a.p, in.raw(), n * C * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
		throw std::runtime_error("cudaMemcpy failed");
	nli_ctx *ctx = nli_dropin::default_context();
	if (to_lab)
		nli_dropin::check(nli_rgb_to_lab(ctx, (const float *)a.p, W, H, (float *)b.p));
	else
		nli_dropin::check(nli_lab_to_rgb(ctx, (const float *)a.p, W, H, C, (float *)b.p));
	nli_dropin::check(nli_ctx_synchronize(ctx));
	Image<float> out((uint)W, (uint)H, 3u);
	if (cudaMemcpy(out.raw(), b.p, n * 3 * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
		throw std::runtime_error("cudaMemcpy failed");
	return out;
}

// largest distance from a hole pixel to the nearest known pixel (the
// DistanceTransform of main.cpp:168-174, on the GPU)
float max_hole_distance(const Mask &mask)
{
	const int W = mask.get_size_x(), H = mask.get_size_y();
	const size_t n = (size_t)W * H;
	Dev m(n), d(n * sizeof(float));
	if (cudaMemcpy(m.p, mask.bytes(), n, cudaMemcpyHostToDevice) != cudaSuccess)
		throw std::runtime_error("cudaMemcpy failed");
	nli_ctx *ctx = nli_dropin::default_context();
	nli_dropin::check(nli_distance_transform(ctx, (const uint8_t *)m.p, W, H, (float *)d.p));
	nli_dropin::check(nli_ctx_synchronize(ctx));
	std::vector<float> h(n);
	if (cudaMemcpy(h.data(), d.p, n * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
		throw std::runtime_error("cudaMemcpy failed");
	float mx = 0;
	for (float v : h) mx = (v > mx) ? v : mx;
	return mx;
}

int run(int argc, char *argv[])
{
	int patch_side = atoi(pick_option(&argc, &argv, "patch", "7"));
	int inpainting_iterations = atoi(pick_option(&argc, &argv, "iters", "200"));
	std::string method_name = pick_option(&argc, &argv, "method", "nlmeans");
	int scales_amount = atoi(pick_option(&argc, &argv, "scales", "11"));
	float coarsest_rate = atof(pick_option(&argc, &argv, "coarse", "0.1"));
	float confidence_decay_time = atof(pick_option(&argc, &argv, "conft", "5.0"));
	float confidence_asymptotic_value = atof(pick_option(&argc, &argv, "confa", "0.1"));
	float lambda = atof(pick_option(&argc, &argv, "lambda", "0.05"));
	std::string initialization_type_name = pick_option(&argc, &argv, "init", "poisson");
	float patch_sigma = atof(pick_option(&argc, &argv, "psigma", "10000.0"));
	std::string show_nnf_file = pick_option(&argc, &argv, "shownnf", "");
	std::string show_pyramid_file = pick_option(&argc, &argv, "showpyr", "");
	std::string depth_name = pick_option(&argc, &argv, "depth", "");
	float lambda_rgb = atof(pick_option(&argc, &argv, "lambdar", "0.05"));
	float lambda_d = atof(pick_option(&argc, &argv, "lambdad", "0.05"));
	const char *seed_opt = pick_option(&argc, &argv, "seed", "");
	if (argc < 4) {
		fprintf(stderr, "USAGE:\n%s input mask output [OPTIONS]\n\n", argv[0]);
		fprintf(stderr, "Available options are:\n");
		fprintf(stderr, " -method \tmethod name [nlmeans/nlmedians/nlpoisson/nldepth] (%s)\n", method_name.c_str());
		fprintf(stderr, " -patch  \tpatch side (%d)\n", patch_side);
		fprintf(stderr, " -iters  \tinpainting iterations (%d)\n", inpainting_iterations);
		fprintf(stderr, " -scales \tscales amount (%d)\n", scales_amount);
		fprintf(stderr, " -coarse \tcoarsest rate (%g)\n", coarsest_rate);
		fprintf(stderr, " -conft  \tconfidence decay time (%g)\n", confidence_decay_time);
		fprintf(stderr, " -confa  \tconfidence asymptotic value (%g)\n", confidence_asymptotic_value);
		fprintf(stderr, " -lambda \tlambda (%g)\n", lambda);
		fprintf(stderr, " -init   \tinitialization type [poisson/black/avg/none] (%s)\n",
		        initialization_type_name.c_str());
		fprintf(stderr, " -psigma \tGaussian patch weights (%g)\n", patch_sigma);
		fprintf(stderr, " -showpyr\tPREFIX write intermediate pyramid results\n");
		fprintf(stderr, " -shownnf\tFILENAME write illustration of the final NNF\n");
		fprintf(stderr, " -depth  \tFILENAME depth map (nldepth); -lambdar, -lambdad its lambdas\n");
		fprintf(stderr, " -seed   \tN random seed (default: time)\n");
		return 1;
	}
	const std::string input_name = argv[1], mask_name = argv[2], output_name = argv[3];

	Image<float> input = convert(rgb_image(read_image(input_name)), true);
	Image<float> mask_image = mono_image(read_image(mask_name), mask_name);
	if (input.get_size_x() != mask_image.get_size_x() || input.get_size_y() != mask_image.get_size_y())
		throw std::runtime_error("ERROR: Input image and mask should be of the same size");
	bool is_mask_empty = true;
	Mask mask(mask_image.get_size_x(), mask_image.get_size_y());
	for (uint y = 0; y < mask_image.get_size_y(); y++)
		for (uint x = 0; x < mask_image.get_size_x(); x++)
			if (mask_image.raw()[(size_t)y * mask_image.get_size_x() + x] > 0) {
				mask.mask(x, y);
				is_mask_empty = false;
			}
	if (is_mask_empty) throw std::runtime_error("ERROR: Mask should not be empty (all black)");

	bool depth_exists = false;
	if (!depth_name.empty()) {
		depth_exists = true;
		Image<float> depth = mono_image(read_image(depth_name), depth_name);
		if (depth.get_size_x() != input.get_size_x() || depth.get_size_y() != input.get_size_y())
			throw std::runtime_error("cat: Size does not match.");
		Image<float> rgbd(input.get_size_x(), input.get_size_y(), 4u);
		for (size_t p = 0; p < (size_t)input.get_size_x() * input.get_size_y(); p++) {
			for (int c = 0; c < 3; c++) rgbd.raw()[4 * p + c] = input.raw()[3 * p + c];
			rgbd.raw()[4 * p + 3] = depth.raw()[p];
		}
		input = rgbd;
	}

	// automatic coarsest rate (Newson's rule, :160-177)
	if (coarsest_rate == 0) coarsest_rate = std::min(1.5f * patch_side / max_hole_distance(mask), 1.f);
	if (patch_side <= 0) throw std::runtime_error("ERROR: patch_side needs to be a positive integer.");
	if ((coarsest_rate > 1) || (coarsest_rate < 0))
		throw std::runtime_error("ERROR: coarsest rate should be between 0 and 1.");
	if (inpainting_iterations < 0) throw std::runtime_error("ERROR: inpainting_iterations cannot be negative.");
	if (confidence_decay_time <= 0.f) throw std::runtime_error("ERROR: confidence_decay_time needs to be positive.");
	if ((lambda > 1.f) || (lambda < 0.f)) throw std::runtime_error("ERROR: lambda should be between 0 and 1.");
	if (scales_amount < 1) throw std::runtime_error("ERROR: number of scales must be at least 1.");
	if (std::abs(coarsest_rate - 1.0f) < 0.00001f) {
		scales_amount = 1;
		printf("\tnote: since the coarsest scale size ratio is 1.0, the number of scales is set to 1\n");
	}
	ImageInpainting::InitType init_type;
	if (initialization_type_name == "poisson")
		init_type = ImageInpainting::InitPoisson;
	else if (initialization_type_name == "black")
		init_type = ImageInpainting::InitBlack;
	else if (initialization_type_name == "avg")
		init_type = ImageInpainting::InitAvg;
	else if (initialization_type_name == "none")
		init_type = ImageInpainting::InitNone;
	else
		throw std::runtime_error("ERROR: Unknown initialization type");

	const float tolerance = 0.1f;
	const float subsampling_rate = ImageInpainting::calculate_subsampling_rate(coarsest_rate, scales_amount);
	Shape patch(patch_side, patch_side);
	const float weights_update_sigma = patch_sigma;
	const int patch_match_iterations = 10, random_shots_limit = 30;
	ImageInpainting image_inpainting(inpainting_iterations, tolerance, scales_amount, subsampling_rate,
	                                 confidence_decay_time, confidence_asymptotic_value, init_type);
	APatchDistance *patch_distance;
	AImageUpdating *image_updating;
	if (method_name == "nlmeans") {
		image_updating = new PatchNonLocalMeans(patch, weights_update_sigma);
		patch_distance = new L2NormPatchDistance(patch, weights_update_sigma);
	} else if (method_name == "nlmedians") {
		image_updating = new PatchNonLocalMedians(patch, weights_update_sigma);
		patch_distance = new L1NormPatchDistance(patch, weights_update_sigma);
	} else if (method_name == "nlpoisson") {
		image_updating = new PatchNonLocalPoisson(patch, weights_update_sigma, lambda, 0.000001f, 1000);
		patch_distance = new L2CombinedPatchDistance(lambda, patch, weights_update_sigma);
	} else if (method_name == "nldepth") {
		if (!depth_exists) throw std::runtime_error("Specify depth input using -depth [filename]");
		image_updating = new PatchNonLocalDepth(patch, weights_update_sigma, lambda_rgb, lambda_d, 0.000001f, 1000);
		patch_distance = new L2RGBDPatchDistance(lambda_rgb, lambda_d, patch, weights_update_sigma);
	} else {
		throw std::runtime_error("ERROR: Unknown method name");
	}
	PatchMatch *patch_match = new PatchMatch(patch_distance, patch_match_iterations, random_shots_limit, -1);
	image_inpainting.set_weights_updating(patch_match);
	image_inpainting.set_image_updating(image_updating);
	nli_dropin::set_seed(seed_opt[0] ? strtoull(seed_opt, nullptr, 10) : (uint64_t)time(NULL));
	image_inpainting.keep_intermediate(!show_nnf_file.empty() || !show_pyramid_file.empty());
	Image<float> output = image_inpainting.process(input, mask);
	const nli_process_stats &st = image_inpainting.get_statistics();
	for (int i = st.scales - 1; i >= 0; i--)
		printf("\tinpainting scale %d: %d iterations\n", st.scales - i, st.iterations[i]);
	delete patch_match;
	delete patch_distance;
	delete image_updating;

	std::stringstream output_str;
	output_str << output_name << "_" << method_name;
	if (method_name == "nlpoisson") output_str << "_l" << lambda;
	output_str << "_sc" << scales_amount << "_" << coarsest_rate;
	if (init_type == ImageInpainting::InitAvg)
		output_str << "_initavg";
	else if (init_type == ImageInpainting::InitBlack)
		output_str << "_init000";
	else
		output_str << "_initnone";
	output_str << "_ps" << patch_side << "_" << weights_update_sigma;
	output_str << "_conf" << confidence_decay_time << "_" << confidence_asymptotic_value << ".png";
	const int W = output.get_size_x(), H = output.get_size_y(), C = output.get_number_of_channels();
	Image<float> rgb = convert(output, false);
	write_image(output_str.str(), rgb.raw(), W, H, 3);
	printf("%s\n", output_str.str().c_str());
	if (depth_exists) {
		std::vector<float> d((size_t)W * H), d3((size_t)W * H * 3);
		for (size_t p = 0; p < d.size(); p++) d[p] = d3[3 * p] = d3[3 * p + 1] = d3[3 * p + 2] = output.raw()[(size_t)C * p + 3];
		write_image("inpainted_depth.pfm", d.data(), W, H, 1);
		write_image("inpainted_depth.png", d3.data(), W, H, 3);
	}
	if (!show_pyramid_file.empty()) {
		std::vector<Image<float> > pyr = image_inpainting.get_output_image_pyramid();
		for (size_t n = 0; n < pyr.size(); n++) {
			std::stringstream s;
			s << show_pyramid_file << n << ".png";
			Image<float> lv = convert(pyr[n], false);
			write_image(s.str(), lv.raw(), lv.get_size_x(), lv.get_size_y(), 3);
		}
	}
	// NNF illustration: hole boundary and NNF discontinuities in black (:320-372)
	if (!show_nnf_file.empty()) {
		std::vector<Image<Point> > nnf_pyramid = image_inpainting.get_nnf_pyramid();
		Image<Point> last = nnf_pyramid[nnf_pyramid.size() - 1];
		Image<float> show = rgb;
		float *sv = show.raw();
		for (int c = 0; c < 3; c++)
			for (int y = 1; y < H; y++)
				for (int x = 1; x < W; x++) {
					const bool m = mask.test((uint)x, (uint)y);
					if (m != mask.test((uint)x - 1, (uint)y) || m != mask.test((uint)x, (uint)y - 1))
						sv[((size_t)y * W + x) * 3 + c] = 0;
					if (m) {
						const Point a = last((uint)x - 1, (uint)y), b = last((uint)x, (uint)y);
						if (a.x - (x - 1) != b.x - x || a.y - y != b.y - y) sv[((size_t)y * W + x) * 3 + c] = 0;
						const Point u = last((uint)x, (uint)y - 1);
						if (u.x - x != b.x - x || u.y - (y - 1) != b.y - y) sv[((size_t)y * W + x) * 3 + c] = 0;
					}
				}
		write_image(show_nnf_file, sv, W, H, 3);
	}
	return 0;
}

}  // namespace

int main(int argc, char *argv[])
{
	try {
		return run(argc, argv);
	} catch (const std::exception &e) {
		fprintf(stderr, "%s\n", e.what());
		return 1;
	}
}
