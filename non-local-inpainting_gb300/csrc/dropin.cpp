// C++ drop-in classes of include/nli_inpainting.hpp over the C ABI: they
// copy the host containers to the device, call nli.h and copy results back
// into the caller's (shared) buffers.  Built into libnli_dropin.so.
#include <cuda_runtime.h>

#include <cstdlib>
#include <mutex>

#include "nli_inpainting.hpp"

Point Point::empty(-1, -1);
Shape Shape::empty(0, 0);

namespace nli_dropin {

static nli_ctx *g_ctx = nullptr;
static std::mutex g_mutex;

nli_ctx *default_context()
{
	std::lock_guard<std::mutex> lock(g_mutex);
	if (!g_ctx) {
		int rc = nli_ctx_create(0, &g_ctx);
		if (rc != NLI_OK) throw std::runtime_error(std::string("nli_ctx_create failed: ") + nli_status_string(rc));
		nli_set_seed(g_ctx, (uint64_t)rand() * 2654435761ull + 1);
	}
	return g_ctx;
}

void set_seed(uint64_t seed) { nli_set_seed(default_context(), seed); }

void check(int status)
{
	if (status != NLI_OK) throw std::runtime_error(nli_last_error(default_context()));
}

// Device buffer owned by the drop-in objects.
struct DevMem {
	void *p = nullptr;
	size_t n = 0;
	explicit DevMem(size_t bytes) : n(bytes)
	{
		if (bytes && cudaMalloc(&p, bytes) != cudaSuccess) throw std::runtime_error("cudaMalloc failed");
	}
	~DevMem()
	{
		if (p) cudaFree(p);
	}
	DevMem(const DevMem &) = delete;
	DevMem &operator=(const DevMem &) = delete;
	template <class T>
	T *as() const
	{
		return static_cast<T *>(p);
	}
};

static std::unique_ptr<DevMem> upload(const void *host, size_t bytes)
{
	std::unique_ptr<DevMem> d(new DevMem(bytes));
	if (bytes && cudaMemcpy(d->p, host, bytes, cudaMemcpyHostToDevice) != cudaSuccess)
		throw std::runtime_error("cudaMemcpy to the device failed");
	return d;
}

static void download(void *host, const DevMem &d, size_t bytes)
{
	if (bytes && cudaMemcpy(host, d.p, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
		throw std::runtime_error("cudaMemcpy from the device failed");
}

static size_t bytes_of(const FixedImage<float> &im)
{
	return sizeof(float) * (size_t)im.get_size_x() * im.get_size_y() * im.get_number_of_channels();
}

static size_t bytes_of(const FixedMask &m) { return (size_t)m.get_size_x() * m.get_size_y(); }

struct DevicePair {
	std::unique_ptr<DevMem> src, tgt;
};

}  // namespace nli_dropin

using namespace nli_dropin;

// ---------------------------------------------------------------- distances
void APatchDistance::initialize(FixedImage<float> source, FixedImage<float> target)
{
	_source = source;
	_target = target;
	std::shared_ptr<DevicePair> d = std::make_shared<DevicePair>();
	d->src = upload(source.raw(), bytes_of(source));
	if (target.raw() != source.raw()) d->tgt = upload(target.raw(), bytes_of(target));
	_device = d;
}

float APatchDistance::gpu_distance(const Point &s, const Point &t)
{
	nli_distance_params p = gpu_params();
	if (p.kind < 0) throw std::runtime_error("no GPU kernel for this patch distance");
	if (!_device) initialize(_source, _target);
	DevicePair *d = static_cast<DevicePair *>(_device.get());
	const float *src = d->src->as<float>();
	const float *tgt = d->tgt ? d->tgt->as<float>() : src;
	const int32_t pair[4] = {s.x, s.y, t.x, t.y};
	std::unique_ptr<DevMem> dp = upload(pair, sizeof(pair));
	DevMem out(sizeof(float));
	check(nli_distance_pairs(default_context(), &p, src, _source.get_size_x(), _source.get_size_y(), tgt,
	                         _target.get_size_x(), _target.get_size_y(), _source.get_number_of_channels(),
	                         dp->as<int32_t>(), 1, out.as<float>()));
	float r;
	check(nli_ctx_synchronize(default_context()));
	download(&r, out, sizeof(float));
	return r;
}

static nli_distance_params dparams(int kind, Shape s, float sigma, float lambda, float lambda_d)
{
	nli_distance_params p;
	p.kind = kind;
	p.patch_x = s.size_x;
	p.patch_y = s.size_y;
	p.sigma = sigma;
	p.lambda = lambda;
	p.lambda_d = lambda_d;
	return p;
}

nli_distance_params L2CombinedPatchDistance::gpu_params() const
{
	return dparams(NLI_DIST_L2_COMBINED, _patch_size, _gaussian_sigma, _lambda, 0.f);
}

nli_distance_params L2RGBDPatchDistance::gpu_params() const
{
	return dparams(NLI_DIST_L2_RGBD, _patch_size, _gaussian_sigma, _lambda_rgb, _lambda_d);
}

nli_distance_params L2NormPatchDistance::gpu_params() const
{
	return dparams(NLI_DIST_L2_NORM, _patch_size, _gaussian_sigma, 1.f, 0.f);
}

nli_distance_params L1NormPatchDistance::gpu_params() const
{
	return dparams(NLI_DIST_L1_NORM, _patch_size, _gaussian_sigma, 1.f, 0.f);
}

// --------------------------------------------------------------- PatchMatch
Image<Point> PatchMatch::calculate(FixedImage<float> source, FixedMask source_mask, FixedImage<float> target,
                                   FixedMask target_mask, Image<Point> initial_field)
{
	if ((!initial_field.is_empty() && initial_field.get_size() != target.get_size()) ||
	    source.get_size() != source_mask.get_size() || target.get_size() != target_mask.get_size() || !_d)
		return Image<Point>();
	nli_distance_params dp = _d->gpu_params();
	if (dp.kind < 0) throw std::runtime_error("no GPU kernel for this patch distance");
	_d->initialize(source, target);
	const int sW = source.get_size_x(), sH = source.get_size_y(), tW = target.get_size_x(), tH = target.get_size_y();
	const int C = source.get_number_of_channels();
	std::unique_ptr<DevMem> s = upload(source.raw(), bytes_of(source));
	std::unique_ptr<DevMem> t = (target.raw() == source.raw()) ? nullptr : upload(target.raw(), bytes_of(target));
	std::unique_ptr<DevMem> sm = upload(source_mask.bytes(), bytes_of(source_mask));
	std::unique_ptr<DevMem> tm = upload(target_mask.bytes(), bytes_of(target_mask));
	std::unique_ptr<DevMem> init;
	if (!initial_field.is_empty()) init = upload(initial_field.raw(), sizeof(Point) * (size_t)tW * tH);
	DevMem out(sizeof(Point) * (size_t)tW * tH);
	nli_patchmatch_params pm = gpu_params();
	double energy = 0.0;
	const float *sp = s->as<float>();
	std::vector<double> total((size_t)std::max(_iters, 1));
	std::vector<int64_t> prop((size_t)std::max(_iters, 1));
	int32_t shots = 0;
	check(nli_patchmatch_metrics(default_context(), &dp, &pm, sp, sm->as<uint8_t>(), sW, sH,
	                             t ? t->as<float>() : sp, tm->as<uint8_t>(), tW, tH, C,
	                             init ? init->as<int32_t>() : nullptr, out.as<int32_t>(), nullptr, &energy,
	                             total.data(), prop.data(), &shots));
	Image<Point> nnf(tW, tH, Point(-1, -1));
	download(nnf.raw(), out, sizeof(Point) * (size_t)tW * tH);
	const size_t sweeps = (size_t)std::max(_iters, 0);
	_energy.assign(total.begin(), total.begin() + sweeps);
	_propagations.assign(prop.begin(), prop.begin() + sweeps);
	_max_shots = shots;
	return nnf;
}

// ------------------------------------------------------------ image updates
double AImageUpdating::update(Image<float> image, Image<float> original_image, FixedMask inpainting_domain,
                              FixedMask extended_inpainting_domain, FixedImage<Point> nnf,
                              FixedImage<float> confidence_mask)
{
	const int W = image.get_size_x(), H = image.get_size_y(), C = image.get_number_of_channels();
	nli_update_params up = gpu_params();
	std::unique_ptr<DevMem> im = upload(image.raw(), bytes_of(image));
	const bool same = original_image.raw() == image.raw();
	std::unique_ptr<DevMem> org = same ? nullptr : upload(original_image.raw(), bytes_of(original_image));
	std::unique_ptr<DevMem> dom = upload(inpainting_domain.bytes(), bytes_of(inpainting_domain));
	std::unique_ptr<DevMem> ext = upload(extended_inpainting_domain.bytes(), bytes_of(extended_inpainting_domain));
	std::unique_ptr<DevMem> nn = upload(nnf.raw(), sizeof(Point) * (size_t)W * H);
	std::unique_ptr<DevMem> cf = confidence_mask.is_empty() ? nullptr : upload(confidence_mask.raw(), bytes_of(confidence_mask));
	double total = 0.0;
	float *ip = im->as<float>();
	check(nli_update(default_context(), &up, ip, same ? ip : org->as<float>(), dom->as<uint8_t>(), ext->as<uint8_t>(),
	                 nn->as<int32_t>(), cf ? cf->as<float>() : nullptr, W, H, C, &total));
	download(image.raw(), *im, bytes_of(image));  // the caller's buffer (shared), as in the reference
	return total;
}

static nli_update_params uparams(int method, Shape s, float sigma, float lambda, float lambda_d, float tol, int iters)
{
	nli_update_params p;
	p.method = method;
	p.patch_x = s.size_x;
	p.patch_y = s.size_y;
	p.sigma = sigma;
	p.lambda = lambda;
	p.lambda_d = lambda_d;
	p.cg_tol = tol;
	p.cg_iters = iters;
	return p;
}

nli_update_params PatchNonLocalMeans::gpu_params() const
{
	return uparams(NLI_UPDATE_MEANS, _patch_size, _gaussian_sigma, 0.f, 0.f, 0.f, 0);
}

nli_update_params PatchNonLocalMedians::gpu_params() const
{
	return uparams(NLI_UPDATE_MEDIANS, _patch_size, _gaussian_sigma, 0.f, 0.f, 0.f, 0);
}

nli_update_params PatchNonLocalPoisson::gpu_params() const
{
	return uparams(NLI_UPDATE_POISSON, _patch_size, _gaussian_sigma, _lambda, 0.f, _tol, _iters);
}

nli_update_params PatchNonLocalDepth::gpu_params() const
{
	return uparams(NLI_UPDATE_DEPTH, _patch_size, _gaussian_sigma, _lambda_rgb, _lambda_d, 0.000001f, 1000);
}

// ----------------------------------------------------------- ImageInpainting
Image<float> ImageInpainting::process(FixedImage<float> in, FixedMask mask)
{
	if (!_pm || !_upd || !_pm->get_distance_calculation())
		throw std::runtime_error("ImageInpainting: PatchMatch, its distance and the image updating must be set");
	nli_process_params p;
	p.distance = _pm->get_distance_calculation()->gpu_params();
	if (p.distance.kind < 0) throw std::runtime_error("no GPU kernel for this patch distance");
	p.patchmatch = _pm->gpu_params();
	p.update = _upd->gpu_params();
	p.iterations = _iters;
	p.tolerance = _tol;
	p.scales = _scales;
	p.subsampling_rate = _rate;
	p.conf_decay_time = _conft;
	p.conf_asymptotic = _confa;
	p.init = (int32_t)_init;
	Image<float> out(in.get_size_x(), in.get_size_y(), in.get_number_of_channels());
	nli_ctx *ctx = default_context();
	check(nli_ctx_keep_intermediate(ctx, _keep ? 1 : 0));
	check(nli_process(ctx, &p, in.raw(), mask.bytes(), in.get_size_x(), in.get_size_y(), in.get_number_of_channels(),
	                  out.raw(), &_stats));
	_input_pyr.clear();
	_output_pyr.clear();
	_mask_pyr.clear();
	_nnf_pyr.clear();
	if (_keep) {
		int W, H, C;
		for (int kind : {NLI_INTER_INPUT, NLI_INTER_OUTPUT}) {
			for (int i = 0; i < nli_intermediate_count(ctx, kind); i++) {
				check(nli_intermediate_get(ctx, kind, i, &W, &H, &C, nullptr));
				Image<float> im((uint)W, (uint)H, (uint)C);
				check(nli_intermediate_get(ctx, kind, i, nullptr, nullptr, nullptr, im.raw()));
				(kind == NLI_INTER_INPUT ? _input_pyr : _output_pyr).push_back(im);
			}
		}
		for (int i = 0; i < nli_intermediate_count(ctx, NLI_INTER_MASK); i++) {
			check(nli_intermediate_get(ctx, NLI_INTER_MASK, i, &W, &H, &C, nullptr));
			std::vector<uint8_t> b((size_t)W * H);
			check(nli_intermediate_get(ctx, NLI_INTER_MASK, i, nullptr, nullptr, nullptr, b.data()));
			Mask m((uint)W, (uint)H);
			for (int y = 0; y < H; y++)
				for (int x = 0; x < W; x++)
					if (b[(size_t)y * W + x]) m.mask((uint)x, (uint)y);
			_mask_pyr.push_back(m);
		}
		for (int i = 0; i < nli_intermediate_count(ctx, NLI_INTER_NNF); i++) {
			check(nli_intermediate_get(ctx, NLI_INTER_NNF, i, &W, &H, &C, nullptr));
			Image<Point> nnf((uint)W, (uint)H, Point(-1, -1));
			check(nli_intermediate_get(ctx, NLI_INTER_NNF, i, nullptr, nullptr, nullptr, nnf.raw()));
			_nnf_pyr.push_back(nnf);
		}
	}
	return out;
}
