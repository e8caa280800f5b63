/*
 * nli_inpainting.hpp -- C++ drop-in for the host code of
 * Tom-Zheng/non-local-inpainting, implemented over the C ABI of nli.h.
 *
 * The classes keep the reference's names, constructors and virtual
 * interfaces (a_patch_distance.h, l2_combined_patch_distance.h,
 * l2_rgbd_patch_distance.h, l2_norm_patch_distance.h,
 * l1_norm_patch_distance.h, patch_match.h, a_image_updating.h,
 * patch_non_local_{means,medians,poisson,depth}.h, image_inpainting.h) so
 * that host code written against the reference (main.cpp:236-284) links
 * against libnli_dropin.so unchanged; the forwarding headers in
 * include/nli_dropin/ carry the reference's header names.  Every
 * computation runs on the GPU through nli.h; there is no CPU path.
 *
 * The containers carry the reference's Image / Mask / Point / Shape API
 * that this interface and host code like its callers use (Mask and
 * FixedMask in full: iterators, channel overloads, at(), first / last /
 * next / prev, bounding box, clone / clone_invert), with the same
 * semantics: copying an Image or Mask shares its buffer (image.hpp:93-112,
 * 555-558), constructing an Image from a FixedImage or a Mask from a
 * FixedMask copies it (image.hpp:561-577, mask.cpp:559-563), pixels are
 * interleaved HWC, and FixedMask::test is range-checked.
 */
#ifndef NLI_INPAINTING_HPP_
#define NLI_INPAINTING_HPP_

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "nli.h"

typedef unsigned int uint;

/* ---------------------------------------------------------------- point.h */
struct Point {
	int x, y;
	Point() : x(0), y(0) {}
	Point(int x_, int y_) : x(x_), y(y_) {}
	bool operator==(const Point &o) const { return x == o.x && y == o.y; }
	bool operator!=(const Point &o) const { return !(*this == o); }
	Point operator+(const Point &o) const { return Point(x + o.x, y + o.y); }
	Point operator-(const Point &o) const { return Point(x - o.x, y - o.y); }
	static Point empty;
};

/* ---------------------------------------------------------------- shape.h */
struct Shape {
	unsigned int size_x, size_y;
	Shape() : size_x(0), size_y(0) {}
	Shape(unsigned int sx, unsigned int sy) : size_x(sx), size_y(sy) {}
	bool operator==(const Shape &o) const { return size_x == o.size_x && size_y == o.size_y; }
	bool operator!=(const Shape &o) const { return !(*this == o); }
	bool is_empty() const { return size_x == 0 || size_y == 0; }
	bool contains(const Point &p) const { return contains(p.x, p.y); }
	bool contains(int x, int y) const { return x >= 0 && y >= 0 && (unsigned)x < size_x && (unsigned)y < size_y; }
	static Shape empty;
};

/* ---------------------------------------------------------------- image.h */
template <class T>
class FixedImage {
public:
	FixedImage() : _sx(0), _sy(0), _c(0) {}
	FixedImage(uint sx, uint sy, uint c = 1) { init(sx, sy, c, T()); }
	FixedImage(uint sx, uint sy, T v) { init(sx, sy, 1, v); }
	FixedImage(uint sx, uint sy, uint c, T v) { init(sx, sy, c, v); }
	FixedImage(Shape s, uint c = 1) { init(s.size_x, s.size_y, c, T()); }
	FixedImage(Shape s, T v) { init(s.size_x, s.size_y, 1, v); }
	FixedImage(Shape s, uint c, T v) { init(s.size_x, s.size_y, c, v); }
	virtual ~FixedImage() {}

	uint get_size_x() const { return _sx; }
	uint get_size_y() const { return _sy; }
	uint get_number_of_channels() const { return _c; }
	Shape get_size() const { return Shape(_sx, _sy); }
	bool is_empty() const { return !_d || _d->empty(); }
	bool is_not_empty() const { return !is_empty(); }
	const T *raw() const { return _d ? _d->data() : nullptr; }
	const T &operator()(uint x, uint y) const { return (*_d)[idx(x, y, 0)]; }
	const T &operator()(uint x, uint y, uint c) const { return (*_d)[idx(x, y, c)]; }
	const T &operator()(Point p) const { return (*_d)[idx(p.x, p.y, 0)]; }
	const T &operator()(Point p, uint c) const { return (*_d)[idx(p.x, p.y, c)]; }

protected:
	uint _sx, _sy, _c;
	std::shared_ptr<std::vector<T>> _d;
	void init(uint sx, uint sy, uint c, T v)
	{
		_sx = sx;
		_sy = sy;
		_c = c;
		_d = std::make_shared<std::vector<T>>((size_t)sx * sy * c, v);
	}
	size_t idx(uint x, uint y, uint c) const { return (size_t)_c * ((size_t)_sx * y + x) + c; }
	template <class U>
	friend class Image;
};

template <class T>
class Image : public FixedImage<T> {
public:
	Image() {}
	Image(uint sx, uint sy, uint c = 1) : FixedImage<T>(sx, sy, c) {}
	Image(uint sx, uint sy, T v) : FixedImage<T>(sx, sy, v) {}
	Image(uint sx, uint sy, uint c, T v) : FixedImage<T>(sx, sy, c, v) {}
	Image(Shape s, uint c = 1) : FixedImage<T>(s, c) {}
	Image(Shape s, T v) : FixedImage<T>(s, v) {}
	Image(Shape s, uint c, T v) : FixedImage<T>(s, c, v) {}
	Image(const Image &o) : FixedImage<T>(o) {}  // shares the buffer
	Image(const FixedImage<T> &o) : FixedImage<T>(o)  // deep copy
	{
		if (o._d) this->_d = std::make_shared<std::vector<T>>(*o._d);
	}
	Image &operator=(const Image &o)
	{
		FixedImage<T>::operator=(o);
		return *this;
	}

	using FixedImage<T>::operator();
	using FixedImage<T>::raw;
	T *raw() { return this->_d ? this->_d->data() : nullptr; }
	T &operator()(uint x, uint y) { return (*this->_d)[this->idx(x, y, 0)]; }
	T &operator()(uint x, uint y, uint c) { return (*this->_d)[this->idx(x, y, c)]; }
	T &operator()(Point p) { return (*this->_d)[this->idx(p.x, p.y, 0)]; }
	T &operator()(Point p, uint c) { return (*this->_d)[this->idx(p.x, p.y, c)]; }
	void fill(T v)
	{
		if (this->_d) std::fill(this->_d->begin(), this->_d->end(), v);
	}
	Image clone() const { return Image(static_cast<const FixedImage<T> &>(*this)); }
};

/* ----------------------------------------------------------------- mask.h */
/* A flag per pixel (bool, as the reference stores them, mask.h), shared
 * between copies like an Image's buffer.  Iteration visits the set pixels
 * in raster order (mask.cpp:158-179, 332-381; mask_iterator.cpp). */
class FixedMask;

class MaskIterator {
public:
	typedef const Point &const_reference;
	typedef const Point *const_pointer;
	MaskIterator() : _mask(nullptr), _current(-1, -1), _reverse(false) {}
	MaskIterator(const FixedMask *mask, Point current, bool reverse = false)
	    : _mask(mask), _current(current), _reverse(reverse)
	{
	}
	bool operator==(const MaskIterator &o) const
	{
		return _mask == o._mask && _current == o._current && _reverse == o._reverse;
	}
	bool operator!=(const MaskIterator &o) const { return !(*this == o); }
	inline MaskIterator &operator++();
	inline MaskIterator &operator--();
	MaskIterator operator++(int)
	{
		MaskIterator before(*this);
		++*this;
		return before;
	}
	MaskIterator operator--(int)
	{
		MaskIterator before(*this);
		--*this;
		return before;
	}
	const_reference operator*() const { return _current; }
	const_pointer operator->() const { return &_current; }

private:
	const FixedMask *_mask;
	Point _current;
	bool _reverse;
};

class FixedMask {
public:
	typedef MaskIterator iterator;

	FixedMask() : _sx(0), _sy(0) {}
	FixedMask(uint sx, uint sy) { init(sx, sy, false); }
	FixedMask(uint sx, uint sy, bool v) { init(sx, sy, v); }
	FixedMask(Shape s) { init(s.size_x, s.size_y, false); }
	FixedMask(Shape s, bool v) { init(s.size_x, s.size_y, v); }
	virtual ~FixedMask() {}

	uint get_size_x() const { return _sx; }
	uint get_size_y() const { return _sy; }
	uint get_number_of_channels() const { return 1; }
	Shape get_size() const { return Shape(_sx, _sy); }
	bool is_empty() const { return !_d || count() == 0; }
	bool is_not_empty() const { return !is_empty(); }

	/* raster order; end() is Point(size_x, size_y), rend() Point(-1, -1) */
	iterator begin() const { return iterator(this, first()); }
	iterator end() const { return iterator(this, Point((int)_sx, (int)_sy)); }
	iterator rbegin() const { return iterator(this, last(), true); }
	iterator rend() const { return iterator(this, Point(-1, -1), true); }

	/* without range checking */
	bool operator()(uint x, uint y) const { return _d.get()[index(x, y, 0)]; }
	bool operator()(Point p) const { return (*this)((uint)p.x, (uint)p.y); }
	bool get(uint x, uint y) const { return _d.get()[index(x, y, 0)]; }
	bool get(uint x, uint y, uint channel) const { return _d.get()[index(x, y, channel)]; }
	bool get(Point p) const { return get((uint)p.x, (uint)p.y); }
	bool get(Point p, uint channel) const { return get((uint)p.x, (uint)p.y, channel); }
	/* false outside the image or beyond the one channel (mask.cpp:223-272) */
	bool test(uint x, uint y) const { return x < _sx && y < _sy && get(x, y); }
	bool test(uint x, uint y, uint channel) const { return channel == 0 && test(x, y); }
	bool test(Point p) const { return p.x >= 0 && p.y >= 0 && test((uint)p.x, (uint)p.y); }
	bool test(Point p, uint channel) const { return channel == 0 && test(p); }

	/* deep copies; clone_invert flips every flag */
	FixedMask clone() const
	{
		FixedMask c;
		c.copy_from(*this, false);
		return c;
	}
	FixedMask clone_invert() const
	{
		FixedMask c;
		c.copy_from(*this, true);
		return c;
	}

	/* raster order (mask.cpp:378-390) */
	std::vector<Point> get_masked_points() const
	{
		std::vector<Point> v;
		for (iterator it = begin(); it != end(); ++it) v.push_back(*it);
		return v;
	}

	/* the first / last set pixel in raster order: Point(size_x, size_y) /
	 * Point(-1, -1) when none is set (mask.cpp:332-349, 425-454) */
	Point first() const
	{
		for (uint y = 0; y < _sy; y++)
			for (uint x = 0; x < _sx; x++)
				if (get(x, y)) return Point((int)x, (int)y);
		return Point((int)_sx, (int)_sy);
	}
	Point last() const
	{
		for (int y = (int)_sy - 1; y >= 0; y--)
			for (int x = (int)_sx - 1; x >= 0; x--)
				if (get((uint)x, (uint)y)) return Point(x, y);
		return Point(-1, -1);
	}
	/* the next / previous set pixel after / before `current` in raster
	 * order, else Point(size_x, size_y) / Point(-1, -1) (mask.cpp:352-381);
	 * from rend() / end() they start at the first / last pixel */
	Point next(const Point &current) const
	{
		int y = current.y, x0 = current.x + 1;
		if (y < 0) y = x0 = 0;
		for (; y < (int)_sy; y++, x0 = 0)
			for (int x = std::max(x0, 0); x < (int)_sx; x++)
				if (get((uint)x, (uint)y)) return Point(x, y);
		return Point((int)_sx, (int)_sy);
	}
	Point prev(const Point &current) const
	{
		int y = current.y, x0 = current.x - 1;
		if (y >= (int)_sy) {
			y = (int)_sy - 1;
			x0 = (int)_sx - 1;
		}
		for (; y >= 0; y--, x0 = (int)_sx - 1)
			for (int x = std::min(x0, (int)_sx - 1); x >= 0; x--)
				if (get((uint)x, (uint)y)) return Point(x, y);
		return Point(-1, -1);
	}
	/* corners of the smallest rectangle holding every set pixel, both
	 * Point(-1, -1) when none is set (mask.cpp:384-401, 460-486) */
	Point bounding_box_top_left() const { return bounding_box(true); }
	Point bounding_box_bottom_right() const { return bounding_box(false); }

	/* flags as bytes 0/1, row-major, as the C ABI takes them */
	const uint8_t *bytes() const { return reinterpret_cast<const uint8_t *>(_d.get()); }

protected:
	uint _sx, _sy;
	std::shared_ptr<bool> _d;
	size_t count() const { return (size_t)_sx * _sy; }
	size_t index(uint x, uint y, uint channel) const { return (size_t)_sx * y + x + channel; }
	void init(uint sx, uint sy, bool v)
	{
		_sx = sx;
		_sy = sy;
		_d = std::shared_ptr<bool>(new bool[std::max<size_t>(count(), 1)], std::default_delete<bool[]>());
		std::fill(_d.get(), _d.get() + count(), v);
	}
	void copy_from(const FixedMask &o, bool invert)
	{
		_sx = o._sx;
		_sy = o._sy;
		_d.reset();
		if (!o._d) return;
		init(o._sx, o._sy, false);
		for (size_t i = 0; i < count(); i++) _d.get()[i] = invert ? !o._d.get()[i] : o._d.get()[i];
	}
	Point bounding_box(bool top_left) const
	{
		int x0 = (int)_sx, y0 = (int)_sy, x1 = -1, y1 = -1;
		for (uint y = 0; y < _sy; y++)
			for (uint x = 0; x < _sx; x++)
				if (get(x, y)) {
					x0 = std::min(x0, (int)x);
					y0 = std::min(y0, (int)y);
					x1 = std::max(x1, (int)x);
					y1 = std::max(y1, (int)y);
				}
		if (x1 < 0) return Point(-1, -1);
		return top_left ? Point(x0, y0) : Point(x1, y1);
	}
	friend class Mask;
};

MaskIterator &MaskIterator::operator++()
{
	if (_mask) _current = _reverse ? _mask->prev(_current) : _mask->next(_current);
	return *this;
}

MaskIterator &MaskIterator::operator--()
{
	if (_mask) _current = _reverse ? _mask->next(_current) : _mask->prev(_current);
	return *this;
}

class Mask : public FixedMask {
public:
	typedef MaskIterator iterator;

	Mask() {}
	Mask(uint sx, uint sy) : FixedMask(sx, sy) {}
	Mask(uint sx, uint sy, bool v) : FixedMask(sx, sy, v) {}
	Mask(Shape s) : FixedMask(s) {}
	Mask(Shape s, bool v) : FixedMask(s, v) {}
	Mask(const Mask &o) : FixedMask(o) {}  // shares the flags
	Mask(const FixedMask &o) { copy_from(o, false); }  // deep copy
	Mask &operator=(const Mask &o)
	{
		FixedMask::operator=(o);
		return *this;
	}
	Mask &operator=(const FixedMask &o)  // deep copy
	{
		if (&o != this) copy_from(o, false);
		return *this;
	}

	/* without range checking */
	using FixedMask::operator();
	bool &operator()(uint x, uint y) { return _d.get()[index(x, y, 0)]; }
	bool &operator()(uint x, uint y, uint channel) { return _d.get()[index(x, y, channel)]; }
	bool &operator()(Point p) { return (*this)((uint)p.x, (uint)p.y); }
	bool &operator()(Point p, uint channel) { return (*this)((uint)p.x, (uint)p.y, channel); }
	/* with range checking: std::out_of_range outside the image or beyond
	 * the one channel */
	bool &at(uint x, uint y) { return at(x, y, 0u); }
	bool &at(uint x, uint y, uint channel)
	{
		if (x >= _sx || y >= _sy || channel != 0) throw std::out_of_range("Mask::at: position out of range");
		return _d.get()[index(x, y, channel)];
	}
	bool &at(Point p) { return at(p, 0u); }
	bool &at(Point p, uint channel)
	{
		if (p.x < 0 || p.y < 0) throw std::out_of_range("Mask::at: position out of range");
		return at((uint)p.x, (uint)p.y, channel);
	}

	/* set / clear with range checking (nothing happens out of range).
	 * Every unmask overload clears: the reference's unmask(x, y, channel),
	 * unmask(Point) and unmask(Point, channel) set the flag instead
	 * (mask.cpp:844-878), which no caller on the inpainting path reaches. */
	void mask(uint x, uint y) { set(x, y, 0, true); }
	void mask(uint x, uint y, uint channel) { set(x, y, channel, true); }
	void mask(Point p) { set(p, 0, true); }
	void mask(Point p, uint channel) { set(p, channel, true); }
	void unmask(uint x, uint y) { set(x, y, 0, false); }
	void unmask(uint x, uint y, uint channel) { set(x, y, channel, false); }
	void unmask(Point p) { set(p, 0, false); }
	void unmask(Point p, uint channel) { set(p, channel, false); }

	void invert()
	{
		for (size_t i = 0; i < count(); i++) _d.get()[i] = !_d.get()[i];
	}
	Mask clone() const { return Mask(static_cast<const FixedMask &>(*this)); }
	Mask clone_invert() const
	{
		Mask m = clone();
		m.invert();
		return m;
	}

private:
	void set(uint x, uint y, uint channel, bool v)
	{
		if (x < _sx && y < _sy && channel == 0) _d.get()[index(x, y, 0)] = v;
	}
	void set(Point p, uint channel, bool v)
	{
		if (p.x >= 0 && p.y >= 0) set((uint)p.x, (uint)p.y, channel, v);
	}
};

/* -------------------------------------------------------- GPU context use */
namespace nli_dropin {
/* The context all drop-in objects use (device 0, created on first use).  Its
 * PatchMatch seed is drawn from rand() when it is created, so host code that
 * calls srand() first (main.cpp:273) controls the GPU random draws too. */
nli_ctx *default_context();
void set_seed(uint64_t seed);
/* Throws std::runtime_error with the context's message unless status == NLI_OK. */
void check(int status);
}  // namespace nli_dropin

/* ------------------------------------------------------ a_patch_distance.h */
class APatchDistance {
public:
	APatchDistance() : _patch_size(7, 7), _gaussian_sigma(1.0f) {}
	APatchDistance(Shape &patch_size, float gaussian_sigma) : _patch_size(patch_size), _gaussian_sigma(gaussian_sigma) {}
	virtual ~APatchDistance() {}
	/* Keeps the images and uploads them for calculate(). */
	virtual void initialize(FixedImage<float> source, FixedImage<float> target);
	/* One distance evaluated on the GPU (nli_distance_pairs). */
	virtual float calculate(const Point &source_point, const Point &target_point) = 0;

	float get_gaussian_sigma() { return _gaussian_sigma; }
	void set_gaussian_sigma(float s) { _gaussian_sigma = s; }
	Shape get_patch_size() { return _patch_size; }
	void set_patch_size(Shape s) { _patch_size = s; }
	/* Parameters of the GPU kernel for this distance (kind < 0: none). */
	virtual nli_distance_params gpu_params() const
	{
		nli_distance_params p;
		p.kind = -1;
		return p;
	}

protected:
	FixedImage<float> _source, _target;
	Shape _patch_size;
	float _gaussian_sigma;
	std::shared_ptr<void> _device;  // device copies of source and target
	float gpu_distance(const Point &s, const Point &t);
};

class L2CombinedPatchDistance : public APatchDistance {
public:
	L2CombinedPatchDistance() : APatchDistance(), _lambda(0.5f) {}
	L2CombinedPatchDistance(float lambda, Shape &patch_size, float gaussian_sigma)
	    : APatchDistance(patch_size, gaussian_sigma), _lambda(lambda) {}
	virtual float calculate(const Point &s, const Point &t) { return gpu_distance(s, t); }
	virtual nli_distance_params gpu_params() const;

private:
	float _lambda;
};

class L2RGBDPatchDistance : public APatchDistance {
public:
	L2RGBDPatchDistance() : APatchDistance(), _lambda_rgb(0.5f), _lambda_d(0.5f) {}
	L2RGBDPatchDistance(float lambda_rgb, float lambda_d, Shape &patch_size, float gaussian_sigma)
	    : APatchDistance(patch_size, gaussian_sigma), _lambda_rgb(lambda_rgb), _lambda_d(lambda_d) {}
	virtual float calculate(const Point &s, const Point &t) { return gpu_distance(s, t); }
	virtual nli_distance_params gpu_params() const;

private:
	float _lambda_rgb, _lambda_d;
};

class L2NormPatchDistance : public APatchDistance {
public:
	L2NormPatchDistance() : APatchDistance() {}
	L2NormPatchDistance(Shape &patch_size, float gaussian_sigma) : APatchDistance(patch_size, gaussian_sigma) {}
	virtual float calculate(const Point &s, const Point &t) { return gpu_distance(s, t); }
	virtual nli_distance_params gpu_params() const;
};

class L1NormPatchDistance : public APatchDistance {
public:
	L1NormPatchDistance() : APatchDistance() {}
	L1NormPatchDistance(Shape &patch_size, float gaussian_sigma) : APatchDistance(patch_size, gaussian_sigma) {}
	virtual float calculate(const Point &s, const Point &t) { return gpu_distance(s, t); }
	virtual nli_distance_params gpu_params() const;
};

/* ----------------------------------------------------------- patch_match.h */
class PatchMatch {
public:
	PatchMatch() : _d(0), _iters(10), _window(-1), _shots(20) {}
	PatchMatch(APatchDistance *d) : _d(d), _iters(10), _window(-1), _shots(20) {}
	PatchMatch(int iteration_count, int random_shots_limit = 20, int search_window_size = -1)
	    : _d(0), _iters(iteration_count), _window(search_window_size), _shots(random_shots_limit) {}
	PatchMatch(APatchDistance *d, int iteration_count, int random_shots_limit = 20, int search_window_size = -1)
	    : _d(d), _iters(iteration_count), _window(search_window_size), _shots(random_shots_limit) {}

	/* Empty image on a size mismatch or without a distance (patch_match.cpp:317-322). */
	Image<Point> calculate(FixedImage<float> source, FixedMask source_mask, FixedImage<float> target,
	                       FixedMask target_mask, Image<Point> initial_field = Image<Point>());

	int get_iteration_count() { return _iters; }
	void set_iteration_count(int n) { _iters = n; }
	int get_search_window_size() { return _window; }
	void set_search_window_size(int w) { _window = w; }
	int get_random_shots_limit() { return _shots; }
	void set_random_shots_limit(int n) { _shots = n; }
	void set_distance_calculation(APatchDistance *d) { _d = d; }
	APatchDistance *get_distance_calculation() { return _d; }
	nli_patchmatch_params gpu_params() const
	{
		nli_patchmatch_params p;
		p.iterations = _iters;
		p.random_shots = _shots;
		p.window = _window;
		return p;
	}
	/* The figures of the reference's METRICS build for the last calculate()
	 * (patch_match.cpp:383-507): per sweep the sum of the matched distances
	 * and the number of points the propagation improved, and the largest
	 * index of a first accepted random draw. */
	std::vector<double> get_total_distance_per_iteration() { return _energy; }
	std::vector<int> get_propagations_per_iteration_metric() { return _propagations; }
	int get_max_random_shots_count() { return _max_shots; }

private:
	APatchDistance *_d;
	int _iters, _window, _shots;
	std::vector<double> _energy;
	std::vector<int> _propagations;
	int _max_shots = 0;
};

/* ------------------------------------------------------ a_image_updating.h */
class AImageUpdating {
public:
	AImageUpdating() : _patch_size(7, 7), _gaussian_sigma(1.0f) {}
	AImageUpdating(Shape patch_size, float gaussian_sigma) : _patch_size(patch_size), _gaussian_sigma(gaussian_sigma) {}
	virtual ~AImageUpdating() {}
	/* Updates `image` in place on `inpainting_domain`; returns sum (old - new)^2. */
	virtual double update(Image<float> image, Image<float> original_image, FixedMask inpainting_domain,
	                      FixedMask extended_inpainting_domain, FixedImage<Point> nnf,
	                      FixedImage<float> confidence_mask);
	float get_gaussian_sigma() { return _gaussian_sigma; }
	void set_gaussian_sigma(float s) { _gaussian_sigma = s; }
	Shape get_patch_size() { return _patch_size; }
	void set_patch_size(Shape s) { _patch_size = s; }
	virtual nli_update_params gpu_params() const = 0;

protected:
	Shape _patch_size;
	float _gaussian_sigma;
};

class PatchNonLocalMeans : public AImageUpdating {
public:
	PatchNonLocalMeans() {}
	PatchNonLocalMeans(Shape patch_size, float gaussian_sigma) : AImageUpdating(patch_size, gaussian_sigma) {}
	virtual nli_update_params gpu_params() const;
};

class PatchNonLocalMedians : public AImageUpdating {
public:
	PatchNonLocalMedians() {}
	PatchNonLocalMedians(Shape patch_size, float gaussian_sigma) : AImageUpdating(patch_size, gaussian_sigma) {}
	virtual nli_update_params gpu_params() const;
};

class PatchNonLocalPoisson : public AImageUpdating {
public:
	PatchNonLocalPoisson() : _lambda(0.5f), _tol(0.0000001f), _iters(1000) {}
	PatchNonLocalPoisson(Shape patch_size, float gaussian_sigma, float lambda,
	                     float conjugate_gradient_tolerance = 1e-10, int conjugate_gradient_iterations_limit = 1000)
	    : AImageUpdating(patch_size, gaussian_sigma), _lambda(lambda), _tol(conjugate_gradient_tolerance),
	      _iters(conjugate_gradient_iterations_limit) {}
	virtual nli_update_params gpu_params() const;

private:
	float _lambda, _tol;
	int _iters;
};

/* The inner solvers use tolerance 1e-6 and 1000 iterations whatever the
 * constructor gets, as in the reference (patch_non_local_depth.cpp:23-34). */
class PatchNonLocalDepth : public AImageUpdating {
public:
	PatchNonLocalDepth() : _lambda_rgb(0.5f), _lambda_d(0.5f) {}
	PatchNonLocalDepth(Shape patch_size, float gaussian_sigma, float lambda_rgb, float lambda_d, float, int)
	    : AImageUpdating(patch_size, gaussian_sigma), _lambda_rgb(lambda_rgb), _lambda_d(lambda_d) {}
	virtual nli_update_params gpu_params() const;

private:
	float _lambda_rgb, _lambda_d;
};

/* ------------------------------------------------------ image_inpainting.h */
class ImageInpainting {
public:
	enum InitType { InitBlack, InitAvg, InitNone, InitPoisson };

	ImageInpainting()
	    : _pm(0), _upd(0), _iters(5), _tol(0), _scales(3), _rate(0.5f), _conft(5.0f), _confa(0.1f), _init(InitPoisson) {}
	ImageInpainting(int iterations_amount, float tolerance, int scales_amount, float subsampling_rate,
	                float confidence_decay_time, float confidence_asymptotic_value, InitType initialization_type)
	    : _pm(0), _upd(0), _iters(iterations_amount), _tol(tolerance), _scales(scales_amount), _rate(subsampling_rate),
	      _conft(confidence_decay_time), _confa(confidence_asymptotic_value), _init(initialization_type) {}

	static float calculate_subsampling_rate(float size_ratio, unsigned int scales_amount)
	{
		return nli_subsampling_rate(size_ratio, scales_amount);
	}
	/* Throws std::runtime_error("ERROR: Empty source mask ...") as the
	 * reference does (image_inpainting.cpp:382-384). */
	Image<float> process(FixedImage<float> in, FixedMask mask);

	int get_iterations_amount() { return _iters; }
	void set_iterations_amount(int n) { _iters = n; }
	float get_tolerance() { return _tol; }
	void set_tolerance(float v) { _tol = v; }
	int get_scales_amount() { return _scales; }
	void set_scales_amount(int n) { _scales = n; }
	float get_subsampling_rate() { return _rate; }
	void set_subsampling_rate(float r) { _rate = r; }
	float get_confidence_decay_time() { return _conft; }
	void set_confidence_decay_time(float v) { _conft = v; }
	float get_confidence_asymptotic_value() { return _confa; }
	void set_confidence_asymptotic_value(float v) { _confa = v; }
	PatchMatch *get_weights_updating() { return _pm; }
	void set_weights_updating(PatchMatch *pm) { _pm = pm; }
	AImageUpdating *get_image_updating() { return _upd; }
	void set_image_updating(AImageUpdating *u) { _upd = u; }
	/* Per-scale iteration counts etc. of the last process() call. */
	const nli_process_stats &get_statistics() const { return _stats; }
	/* Keep the pyramids of the next process() calls
	 * (image_inpainting.cpp:103-108, 310-337, 410-412). */
	void keep_intermediate(bool value = true) { _keep = value; }
	std::vector<Image<float> > get_input_image_pyramid() { return _input_pyr; }
	std::vector<Image<float> > get_output_image_pyramid() { return _output_pyr; }
	std::vector<Mask> get_mask_pyramid() { return _mask_pyr; }
	std::vector<Image<Point> > get_nnf_pyramid() { return _nnf_pyr; }

private:
	PatchMatch *_pm;
	AImageUpdating *_upd;
	int _iters;
	float _tol;
	int _scales;
	float _rate, _conft, _confa;
	InitType _init;
	nli_process_stats _stats;
	bool _keep = false;
	std::vector<Image<float> > _input_pyr, _output_pyr;
	std::vector<Mask> _mask_pyr;
	std::vector<Image<Point> > _nnf_pyr;
};

#endif /* NLI_INPAINTING_HPP_ */
