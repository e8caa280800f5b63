// Host code written against the reference's container interface (mask.h,
// mask_iterator.h, image.h), compiled against the drop-in header alone and
// run on the CPU by tests/test_dropin_containers.py.  It walks an
// inpainting domain the way the reference's updates do
// (patch_non_local_means.cpp:45: an iterator over the FixedMask, reading
// the image at each point) and checks the rest of the Mask API: reverse
// iteration, first / last / next / prev, the bounding box, channel
// overloads, range-checked at(), mask / unmask with Points, deep copies and
// clone_invert.  Prints "mask api ok" and exits 0 when every check holds.
#include <cstdio>
#include <stdexcept>
#include <vector>

#include "nli_inpainting.hpp"

#define EXPECT(c)                                                   \
	do {                                                            \
		if (!(c)) {                                                 \
			fprintf(stderr, "check failed line %d: %s\n", __LINE__, #c); \
			return 1;                                               \
		}                                                           \
	} while (0)

// sum of the image over the domain, visiting it as the updates do
static double domain_sum(const FixedImage<float> &image, const FixedMask &domain)
{
	double s = 0.0;
	for (FixedMask::iterator it = domain.begin(); it != domain.end(); ++it) {
		const Point p = *it;
		s += image(p.x, p.y);
		s += 0.0 * it->x;
	}
	return s;
}

int main()
{
	const uint W = 7, H = 5;
	Image<float> image(W, H, 1u);
	for (uint y = 0; y < H; y++)
		for (uint x = 0; x < W; x++) image(x, y) = (float)(10 * y + x);

	Mask m(W, H);
	EXPECT(m.begin() == m.end() && m.rbegin() == m.rend());
	EXPECT(m.first() == Point((int)W, (int)H) && m.last() == Point(-1, -1));
	EXPECT(m.bounding_box_top_left() == Point(-1, -1) && m.bounding_box_bottom_right() == Point(-1, -1));
	const Point set[] = {Point(2, 1), Point(5, 1), Point(0, 3), Point(4, 3), Point(6, 4)};
	for (const Point &p : set) m.mask(p);
	m.mask(Point(-1, 2));   // out of range: nothing happens
	m.mask(9u, 9u);
	m.mask(1u, 1u, 1u);     // channel 1 of a one-channel mask: nothing happens

	// forward iteration in raster order, the same as get_masked_points
	std::vector<Point> seen;
	for (Mask::iterator it = m.begin(); it != m.end(); it++) seen.push_back(*it);
	const std::vector<Point> pts = m.get_masked_points();
	EXPECT(seen.size() == 5 && pts.size() == 5);
	for (int i = 0; i < 5; i++) EXPECT(seen[i] == set[i] && pts[i] == set[i]);
	EXPECT(domain_sum(image, m) == 12.0 + 15.0 + 30.0 + 34.0 + 46.0);
	// reverse iteration, and stepping back from end()
	std::vector<Point> back;
	for (FixedMask::iterator it = m.rbegin(); it != m.rend(); ++it) back.push_back(*it);
	EXPECT(back.size() == 5);
	for (int i = 0; i < 5; i++) EXPECT(back[i] == set[4 - i]);
	FixedMask::iterator e = m.end();
	--e;
	EXPECT(*e == set[4]);
	EXPECT(m.first() == set[0] && m.last() == set[4]);
	EXPECT(m.next(set[1]) == set[2] && m.prev(set[2]) == set[1] && m.next(set[4]) == Point((int)W, (int)H) &&
	       m.prev(set[0]) == Point(-1, -1));
	EXPECT(m.bounding_box_top_left() == Point(0, 1) && m.bounding_box_bottom_right() == Point(6, 4));

	// channel overloads and range checks
	EXPECT(m.get(2, 1) && m.get(Point(2, 1)) && m.get(2u, 1u, 0u) && m.get(Point(2, 1), 0u));
	EXPECT(m.test(Point(5, 1)) && m.test(5u, 1u, 0u) && !m.test(5u, 1u, 1u) && !m.test(Point(5, 1), 1u));
	EXPECT(!m.test(Point(-1, 0)) && !m.test(W, 0u));
	bool thrown = false;
	try {
		m.at(W, 0u) = true;
	} catch (const std::out_of_range &) {
		thrown = true;
	}
	EXPECT(thrown);
	m.at(Point(1, 4)) = true;
	EXPECT(m(1u, 4u) && m.at(1u, 4u));
	m(Point(1, 4)) = false;
	EXPECT(!m.test(1u, 4u));

	// copies share the flags; clones do not; FixedMask -> Mask copies
	Mask shared = m;
	shared.unmask(Point(0, 3));   // clears (the reference's overload sets)
	EXPECT(!m.test(0u, 3u));
	m.mask(Point(0, 3));
	EXPECT(shared.test(0u, 3u));
	FixedMask fixed = m;                 // a FixedMask view sharing the flags
	Mask copy(fixed);                    // deep copy
	copy.unmask(2u, 1u);
	EXPECT(m.test(2u, 1u) && !copy.test(2u, 1u));
	Mask assigned;
	assigned = fixed;                    // deep copy
	assigned.unmask(5u, 1u, 0u);
	EXPECT(m.test(5u, 1u) && !assigned.test(5u, 1u));
	FixedMask fc = fixed.clone(), fi = fixed.clone_invert();
	EXPECT(fc.get_masked_points().size() == 5 && fi.get_masked_points().size() == W * H - 5);
	for (uint y = 0; y < H; y++)
		for (uint x = 0; x < W; x++) EXPECT(fi.get(x, y) != m.get(x, y) && fc.get(x, y) == m.get(x, y));
	Mask mi = m.clone_invert();
	EXPECT(mi.first() == Point(0, 0) && mi.get_masked_points().size() == W * H - 5);
	// the C ABI view of the flags
	EXPECT(m.bytes()[1 * W + 2] == 1 && m.bytes()[0] == 0);
	printf("mask api ok\n");
	return 0;
}
