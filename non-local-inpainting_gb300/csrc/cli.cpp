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
#include <map>
#include <memory>
#include <stdexcept>
#include <utility>
#include <sstream>
#include <string>
#include <vector>

#include "nli_inpainting.hpp"
#include "png_codec.h"

namespace {

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

// ---------------------------------------------------------- command line
// The program's options: the reference's names and defaults (main.cpp:68-82)
// and -seed.  The accepted syntax is the reference's: "-name value" pairs
// anywhere on the line, every other word a positional argument, in order.
struct OptionSpec {
	const char *name;
	const char *default_value;
	const char *help;  // printf format of the usage line; %s is the default
};

const OptionSpec kOptions[] = {
    {"method", "nlmeans", " -method \tmethod name [nlmeans/nlmedians/nlpoisson/nldepth] (%s)"},
    {"patch", "7", " -patch  \tpatch side (%s)"},
    {"iters", "200", " -iters  \tinpainting iterations (%s)"},
    {"scales", "11", " -scales \tscales amount (%s)"},
    {"coarse", "0.1", " -coarse \tcoarsest rate (%s)"},
    {"conft", "5.0", " -conft  \tconfidence decay time (%s)"},
    {"confa", "0.1", " -confa  \tconfidence asymptotic value (%s)"},
    {"lambda", "0.05", " -lambda \tlambda (%s)"},
    {"init", "poisson", " -init   \tinitialization type [poisson/black/avg/none] (%s)"},
    {"psigma", "10000.0", " -psigma \tGaussian patch weights (%s)"},
    {"showpyr", "", " -showpyr\tPREFIX write intermediate pyramid results%s"},
    {"shownnf", "", " -shownnf\tFILENAME write illustration of the final NNF%s"},
    {"depth", "", " -depth  \tFILENAME depth map (nldepth)%s"},
    {"lambdar", "0.05", " -lambdar\tlambda of the colour channels, nldepth (%s)"},
    {"lambdad", "0.05", " -lambdad\tlambda of the depth channel, nldepth (%s)"},
    {"seed", "", " -seed   \tN random seed (default: time)%s"},
};

const OptionSpec *find_option(const char *word)
{
	if (word[0] != '-') return nullptr;
	for (const OptionSpec &o : kOptions)
		if (strcmp(word + 1, o.name) == 0) return &o;
	return nullptr;
}

class CommandLine {
  public:
	CommandLine(int argc, char **argv) : program_(argc > 0 ? argv[0] : "nli_inpaint")
	{
		for (int i = 1; i < argc; i++) {
			const OptionSpec *o = find_option(argv[i]);
			if (!o) {
				positional_.push_back(argv[i]);
				continue;
			}
			if (i + 1 >= argc) throw std::runtime_error(std::string("ERROR: option -") + o->name + " needs a value");
			if (!values_.emplace(o->name, argv[i + 1]).second)
				throw std::runtime_error(std::string("ERROR: option -") + o->name + " given twice");
			i++;
		}
	}
	std::string text(const char *name) const
	{
		auto it = values_.find(name);
		if (it != values_.end()) return it->second;
		for (const OptionSpec &o : kOptions)
			if (strcmp(o.name, name) == 0) return o.default_value;
		throw std::logic_error(std::string("no option ") + name);
	}
	int integer(const char *name) const { return atoi(text(name).c_str()); }
	float real(const char *name) const { return (float)atof(text(name).c_str()); }
	bool given(const char *name) const { return !text(name).empty(); }
	const std::vector<std::string> &positional() const { return positional_; }
	void usage(FILE *out) const
	{
		fprintf(out, "USAGE:\n%s input mask output [OPTIONS]\n\nAvailable options are:\n", program_.c_str());
		for (const OptionSpec &o : kOptions) {
			fprintf(out, o.help, text(o.name).c_str());
			fputc('\n', out);
		}
	}

  private:
	std::string program_;
	std::map<std::string, std::string> values_;
	std::vector<std::string> positional_;
};

// ------------------------------------------------------------- settings
// What a run needs, read from the command line and checked with the
// reference's messages (main.cpp:160-215).
struct Settings {
	std::string input, mask, output;
	std::string method, init_name;
	std::string nnf_file, pyramid_prefix, depth_file;
	int patch = 0, iterations = 0, scales = 0;
	float coarse = 0, conf_decay = 0, conf_asym = 0, lambda = 0, psigma = 0, lambda_rgb = 0, lambda_d = 0;
	ImageInpainting::InitType init = ImageInpainting::InitPoisson;
	uint64_t seed = 0;
};

ImageInpainting::InitType init_type_named(const std::string &name)
{
	static const std::pair<const char *, ImageInpainting::InitType> kInits[] = {
	    {"poisson", ImageInpainting::InitPoisson},
	    {"black", ImageInpainting::InitBlack},
	    {"avg", ImageInpainting::InitAvg},
	    {"none", ImageInpainting::InitNone},
	};
	for (const auto &e : kInits)
		if (name == e.first) return e.second;
	throw std::runtime_error("ERROR: Unknown initialization type");
}

Settings read_settings(const CommandLine &cl)
{
	Settings s;
	s.input = cl.positional()[0];
	s.mask = cl.positional()[1];
	s.output = cl.positional()[2];
	s.method = cl.text("method");
	s.init_name = cl.text("init");
	s.nnf_file = cl.text("shownnf");
	s.pyramid_prefix = cl.text("showpyr");
	s.depth_file = cl.text("depth");
	s.patch = cl.integer("patch");
	s.iterations = cl.integer("iters");
	s.scales = cl.integer("scales");
	s.coarse = cl.real("coarse");
	s.conf_decay = cl.real("conft");
	s.conf_asym = cl.real("confa");
	s.lambda = cl.real("lambda");
	s.psigma = cl.real("psigma");
	s.lambda_rgb = cl.real("lambdar");
	s.lambda_d = cl.real("lambdad");
	s.seed = cl.given("seed") ? strtoull(cl.text("seed").c_str(), nullptr, 10) : (uint64_t)time(NULL);
	return s;
}

// The checks of main.cpp:178-215, after the automatic coarsest rate is known.
void check_settings(Settings &s)
{
	if (s.patch <= 0) throw std::runtime_error("ERROR: patch_side needs to be a positive integer.");
	if (s.coarse > 1 || s.coarse < 0) throw std::runtime_error("ERROR: coarsest rate should be between 0 and 1.");
	if (s.iterations < 0) throw std::runtime_error("ERROR: inpainting_iterations cannot be negative.");
	if (s.conf_decay <= 0.f) throw std::runtime_error("ERROR: confidence_decay_time needs to be positive.");
	if (s.lambda > 1.f || s.lambda < 0.f) throw std::runtime_error("ERROR: lambda should be between 0 and 1.");
	if (s.scales < 1) throw std::runtime_error("ERROR: number of scales must be at least 1.");
	if (std::abs(s.coarse - 1.0f) < 0.00001f) {
		s.scales = 1;
		printf("\tnote: since the coarsest scale size ratio is 1.0, the number of scales is set to 1\n");
	}
	s.init = init_type_named(s.init_name);
}

// ---------------------------------------------------------------- inputs
struct Inputs {
	Image<float> image;  // L*a*b* (and depth as a fourth channel)
	Mask mask;
	bool has_depth = false;
};

Mask hole_mask(const Image<float> &m)
{
	Mask hole(m.get_size_x(), m.get_size_y());
	bool any = false;
	for (uint y = 0; y < m.get_size_y(); y++)
		for (uint x = 0; x < m.get_size_x(); x++)
			if (m.raw()[(size_t)y * m.get_size_x() + x] > 0) {
				hole.mask(x, y);
				any = true;
			}
	if (!any) throw std::runtime_error("ERROR: Mask should not be empty (all black)");
	return hole;
}

Image<float> with_depth(const Image<float> &lab, const Image<float> &depth)
{
	if (depth.get_size_x() != lab.get_size_x() || depth.get_size_y() != lab.get_size_y())
		throw std::runtime_error("cat: Size does not match.");
	Image<float> rgbd(lab.get_size_x(), lab.get_size_y(), 4u);
	const size_t n = (size_t)lab.get_size_x() * lab.get_size_y();
	for (size_t p = 0; p < n; p++) {
		std::copy(lab.raw() + 3 * p, lab.raw() + 3 * p + 3, rgbd.raw() + 4 * p);
		rgbd.raw()[4 * p + 3] = depth.raw()[p];
	}
	return rgbd;
}

Inputs load_inputs(const Settings &s)
{
	Inputs in;
	in.image = convert(rgb_image(read_image(s.input)), true);
	const Image<float> m = mono_image(read_image(s.mask), s.mask);
	if (in.image.get_size_x() != m.get_size_x() || in.image.get_size_y() != m.get_size_y())
		throw std::runtime_error("ERROR: Input image and mask should be of the same size");
	in.mask = hole_mask(m);
	if (!s.depth_file.empty()) {
		in.image = with_depth(in.image, mono_image(read_image(s.depth_file), s.depth_file));
		in.has_depth = true;
	}
	return in;
}

// --------------------------------------------------------------- methods
// A method: its image update and the patch distance the reference pairs it
// with on the command line (main.cpp:245-263).  The inner CG solves run to
// 1e-6 relative residual or 1000 iterations, as there.
struct Method {
	std::unique_ptr<APatchDistance> distance;
	std::unique_ptr<AImageUpdating> updating;
};

Method make_method(const Settings &s, bool has_depth)
{
	Shape patch(s.patch, s.patch);  // the classes take it by non-const reference, as the reference's
	Method m;
	if (s.method == "nlmeans") {
		m.updating.reset(new PatchNonLocalMeans(patch, s.psigma));
		m.distance.reset(new L2NormPatchDistance(patch, s.psigma));
	} else if (s.method == "nlmedians") {
		m.updating.reset(new PatchNonLocalMedians(patch, s.psigma));
		m.distance.reset(new L1NormPatchDistance(patch, s.psigma));
	} else if (s.method == "nlpoisson") {
		m.updating.reset(new PatchNonLocalPoisson(patch, s.psigma, s.lambda, 0.000001f, 1000));
		m.distance.reset(new L2CombinedPatchDistance(s.lambda, patch, s.psigma));
	} else if (s.method == "nldepth") {
		if (!has_depth) throw std::runtime_error("Specify depth input using -depth [filename]");
		m.updating.reset(new PatchNonLocalDepth(patch, s.psigma, s.lambda_rgb, s.lambda_d, 0.000001f, 1000));
		m.distance.reset(new L2RGBDPatchDistance(s.lambda_rgb, s.lambda_d, patch, s.psigma));
	} else {
		throw std::runtime_error("ERROR: Unknown method name");
	}
	return m;
}

// --------------------------------------------------------------- outputs
// The result's file name, composed from the parameters as the reference
// composes it (main.cpp:287-303), except that Poisson initialisation is
// named "_initpoisson": the reference names it "_initnone" like -init none.
std::string composed_name(const Settings &s)
{
	const char *init_tag = s.init == ImageInpainting::InitAvg     ? "_initavg"
	                       : s.init == ImageInpainting::InitBlack ? "_init000"
	                       : s.init == ImageInpainting::InitNone  ? "_initnone"
	                                                               : "_initpoisson";
	std::ostringstream o;
	o << s.output << "_" << s.method;
	if (s.method == "nlpoisson") o << "_l" << s.lambda;
	o << "_sc" << s.scales << "_" << s.coarse << init_tag << "_ps" << s.patch << "_" << s.psigma << "_conf"
	  << s.conf_decay << "_" << s.conf_asym << ".png";
	return o.str();
}

void write_depth(const Image<float> &out)
{
	const int W = out.get_size_x(), H = out.get_size_y(), C = out.get_number_of_channels();
	std::vector<float> d((size_t)W * H), grey3((size_t)W * H * 3);
	for (size_t p = 0; p < d.size(); p++) {
		d[p] = out.raw()[(size_t)C * p + 3];
		std::fill(grey3.begin() + 3 * p, grey3.begin() + 3 * p + 3, d[p]);
	}
	write_image("inpainted_depth.pfm", d.data(), W, H, 1);
	write_image("inpainted_depth.png", grey3.data(), W, H, 3);
}

void write_pyramid(const std::string &prefix, const std::vector<Image<float> > &levels)
{
	for (size_t n = 0; n < levels.size(); n++) {
		const Image<float> rgb = convert(levels[n], false);
		write_image(prefix + std::to_string(n) + ".png", rgb.raw(), rgb.get_size_x(), rgb.get_size_y(), 3);
	}
}

// The illustration of the finest NNF (main.cpp:315-374): the result with the
// hole boundary and every break of the field's offset between horizontal or
// vertical neighbours in black.
void write_nnf_illustration(const std::string &file, const Image<float> &rgb, const Mask &mask,
                            const Image<Point> &nnf)
{
	const int W = rgb.get_size_x(), H = rgb.get_size_y();
	std::vector<float> v(rgb.raw(), rgb.raw() + (size_t)W * H * 3);
	auto offset = [&](int x, int y) {
		const Point q = nnf((uint)x, (uint)y);
		return std::make_pair(q.x - x, q.y - y);
	};
	for (int y = 1; y < H; y++)
		for (int x = 1; x < W; x++) {
			const bool inside = mask.test((uint)x, (uint)y);
			bool dark = inside != mask.test((uint)x - 1, (uint)y) || inside != mask.test((uint)x, (uint)y - 1);
			if (inside) dark = dark || offset(x - 1, y) != offset(x, y) || offset(x, y - 1) != offset(x, y);
			if (dark) std::fill(v.begin() + 3 * ((size_t)y * W + x), v.begin() + 3 * ((size_t)y * W + x) + 3, 0.f);
		}
	write_image(file, v.data(), W, H, 3);
}

int run(int argc, char *argv[])
{
	const CommandLine cl(argc, argv);
	if (cl.positional().size() < 3) {
		cl.usage(stderr);
		return 1;
	}
	Settings s = read_settings(cl);
	const Inputs in = load_inputs(s);
	// -coarse 0: the automatic coarsest rate (Newson's rule, main.cpp:160-177)
	if (s.coarse == 0) s.coarse = std::min(1.5f * s.patch / max_hole_distance(in.mask), 1.f);
	check_settings(s);

	ImageInpainting inpainting(s.iterations, 0.1f, s.scales,
	                           ImageInpainting::calculate_subsampling_rate(s.coarse, s.scales), s.conf_decay,
	                           s.conf_asym, s.init);
	Method method = make_method(s, in.has_depth);
	PatchMatch weights(method.distance.get(), 10, 30, -1);
	inpainting.set_weights_updating(&weights);
	inpainting.set_image_updating(method.updating.get());
	nli_dropin::set_seed(s.seed);
	inpainting.keep_intermediate(!s.nnf_file.empty() || !s.pyramid_prefix.empty());
	const Image<float> output = inpainting.process(in.image, in.mask);
	const nli_process_stats &st = inpainting.get_statistics();
	for (int i = st.scales - 1; i >= 0; i--)
		printf("\tinpainting scale %d: %d iterations\n", st.scales - i, st.iterations[i]);

	const std::string name = composed_name(s);
	const Image<float> rgb = convert(output, false);
	write_image(name, rgb.raw(), rgb.get_size_x(), rgb.get_size_y(), 3);
	printf("%s\n", name.c_str());
	if (in.has_depth) write_depth(output);
	if (!s.pyramid_prefix.empty()) write_pyramid(s.pyramid_prefix, inpainting.get_output_image_pyramid());
	if (!s.nnf_file.empty()) write_nnf_illustration(s.nnf_file, rgb, in.mask, inpainting.get_nnf_pyramid().back());
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
