// PNG codec of the command-line program (see png_codec.h).  DEFLATE
// decoding uses canonical Huffman codes as RFC 1951 section 3.2 defines
// them: codes of equal length are consecutive integers in symbol order, so a
// code is decoded bit by bit by comparing it with the first code of each
// length.
#include "png_codec.h"

#include <algorithm>
#include <cstring>

namespace nli_png {

// ------------------------------------------------------------ checksums
namespace {
struct CrcTable {
	uint32_t v[256];
	CrcTable()
	{
		for (uint32_t n = 0; n < 256; n++) {
			uint32_t c = n;
			for (int k = 0; k < 8; k++) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : (c >> 1);
			v[n] = c;
		}
	}
};
}  // namespace

uint32_t crc32(const uint8_t *data, size_t size, uint32_t crc)
{
	static const CrcTable table;  // initialised once, thread-safe
	crc = ~crc;
	for (size_t i = 0; i < size; i++) crc = table.v[(crc ^ data[i]) & 0xff] ^ (crc >> 8);
	return ~crc;
}

uint32_t adler32(const uint8_t *data, size_t size, uint32_t adler)
{
	uint32_t a = adler & 0xffff, b = adler >> 16;
	for (size_t i = 0; i < size; i++) {
		a = (a + data[i]) % 65521u;
		b = (b + a) % 65521u;
	}
	return (b << 16) | a;
}

namespace {

// ------------------------------------------------------------- inflate
struct Bits {
	const uint8_t *p;
	size_t n, pos = 0;
	uint32_t buf = 0;
	int count = 0;
	bool overrun = false;
	Bits(const uint8_t *d, size_t s) : p(d), n(s) {}
	// the next k (<= 16) bits, least significant first
	uint32_t take(int k)
	{
		while (count < k) {
			if (pos >= n) {
				overrun = true;
				return 0;
			}
			buf |= (uint32_t)p[pos++] << count;
			count += 8;
		}
		const uint32_t v = buf & ((1u << k) - 1u);
		buf >>= k;
		count -= k;
		return v;
	}
	void align()
	{
		buf = 0;
		count = 0;
	}
};

constexpr int kMaxBits = 15;

struct Huffman {
	uint16_t count[kMaxBits + 1];  // codes of each length
	uint16_t symbol[320];          // symbols ordered by code
};

// Builds the decoding tables from code lengths; false when the lengths
// over-subscribe the code space.  An incomplete code is accepted (a
// distance code with one symbol is legal).
bool build(Huffman &h, const uint8_t *lengths, int n)
{
	std::memset(h.count, 0, sizeof(h.count));
	for (int s = 0; s < n; s++) h.count[lengths[s]]++;
	if (h.count[0] == n) return true;  // no codes
	int left = 1;
	for (int len = 1; len <= kMaxBits; len++) {
		left <<= 1;
		left -= h.count[len];
		if (left < 0) return false;
	}
	uint16_t offs[kMaxBits + 1];
	offs[1] = 0;
	for (int len = 1; len < kMaxBits; len++) offs[len + 1] = offs[len] + h.count[len];
	for (int s = 0; s < n; s++)
		if (lengths[s] != 0) h.symbol[offs[lengths[s]]++] = (uint16_t)s;
	return true;
}

// One symbol; -1 on a code that is not in the table or on running out of input.
int decode_symbol(Bits &in, const Huffman &h)
{
	int code = 0, first = 0, index = 0;
	for (int len = 1; len <= kMaxBits; len++) {
		code |= (int)in.take(1);
		if (in.overrun) return -1;
		const int cnt = h.count[len];
		if (code - cnt < first) return h.symbol[index + (code - first)];
		index += cnt;
		first += cnt;
		first <<= 1;
		code <<= 1;
	}
	return -1;
}

const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool codes(Bits &in, std::vector<uint8_t> &out, const Huffman &lit, const Huffman &dist, size_t limit,
           std::string &error)
{
	for (;;) {
		if (out.size() > limit) {
			error = "more data than the image holds";
			return false;
		}
		const int sym = decode_symbol(in, lit);
		if (sym < 0) {
			error = "invalid literal/length code";
			return false;
		}
		if (sym < 256) {
			out.push_back((uint8_t)sym);
		} else if (sym == 256) {
			return true;
		} else {
			const int li = sym - 257;
			if (li >= 29) {
				error = "invalid length symbol";
				return false;
			}
			const size_t len = kLenBase[li] + in.take(kLenExtra[li]);
			const int ds = decode_symbol(in, dist);
			if (ds < 0 || ds >= 30) {
				error = "invalid distance code";
				return false;
			}
			const size_t d = kDistBase[ds] + in.take(kDistExtra[ds]);
			if (in.overrun) {
				error = "truncated compressed data";
				return false;
			}
			if (d > out.size()) {
				error = "distance beyond the start of the output";
				return false;
			}
			const size_t from = out.size() - d;
			for (size_t k = 0; k < len; k++) out.push_back(out[from + k]);
		}
	}
}

bool inflate_raw(Bits &in, std::vector<uint8_t> &out, size_t limit, std::string &error)
{
	static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
	bool last = false;
	while (!last) {
		last = in.take(1) != 0;
		const uint32_t type = in.take(2);
		if (in.overrun) {
			error = "truncated compressed data";
			return false;
		}
		if (type == 0) {  // stored
			in.align();
			if (in.pos + 4 > in.n) {
				error = "truncated stored block";
				return false;
			}
			const uint32_t len = in.p[in.pos] | (in.p[in.pos + 1] << 8);
			const uint32_t nlen = in.p[in.pos + 2] | (in.p[in.pos + 3] << 8);
			in.pos += 4;
			if ((len ^ 0xffffu) != nlen) {
				error = "stored block length check failed";
				return false;
			}
			if (in.pos + len > in.n) {
				error = "truncated stored block";
				return false;
			}
			if (out.size() + len > limit + 258) {
				error = "more data than the image holds";
				return false;
			}
			out.insert(out.end(), in.p + in.pos, in.p + in.pos + len);
			in.pos += len;
		} else if (type == 1) {  // fixed Huffman codes
			struct Fixed {
				Huffman lit, dist;
				Fixed()
				{
					uint8_t l[288];
					for (int s = 0; s < 144; s++) l[s] = 8;
					for (int s = 144; s < 256; s++) l[s] = 9;
					for (int s = 256; s < 280; s++) l[s] = 7;
					for (int s = 280; s < 288; s++) l[s] = 8;
					build(lit, l, 288);
					uint8_t dl[30];
					for (int s = 0; s < 30; s++) dl[s] = 5;
					build(dist, dl, 30);
				}
			};
			static const Fixed fixed;  // initialised once, thread-safe
			if (!codes(in, out, fixed.lit, fixed.dist, limit, error)) return false;
		} else if (type == 2) {  // dynamic Huffman codes
			const int nlen = (int)in.take(5) + 257, ndist = (int)in.take(5) + 1, ncode = (int)in.take(4) + 4;
			if (nlen > 286 || ndist > 30) {
				error = "too many length or distance codes";
				return false;
			}
			uint8_t lengths[320];
			std::memset(lengths, 0, sizeof(lengths));
			for (int k = 0; k < ncode; k++) lengths[order[k]] = (uint8_t)in.take(3);
			Huffman lencode, lit, dist;
			if (in.overrun || !build(lencode, lengths, 19)) {
				error = "invalid code-length code";
				return false;
			}
			int k = 0;
			while (k < nlen + ndist) {
				int sym = decode_symbol(in, lencode);
				if (sym < 0) {
					error = "invalid code-length symbol";
					return false;
				}
				if (sym < 16) {
					lengths[k++] = (uint8_t)sym;
					continue;
				}
				uint8_t value = 0;
				int repeat;
				if (sym == 16) {
					if (k == 0) {
						error = "repeat with no previous length";
						return false;
					}
					value = lengths[k - 1];
					repeat = 3 + (int)in.take(2);
				} else if (sym == 17) {
					repeat = 3 + (int)in.take(3);
				} else {
					repeat = 11 + (int)in.take(7);
				}
				if (k + repeat > nlen + ndist) {
					error = "too many code lengths";
					return false;
				}
				while (repeat--) lengths[k++] = value;
			}
			if (lengths[256] == 0) {
				error = "no end-of-block code";
				return false;
			}
			if (!build(lit, lengths, nlen) || !build(dist, lengths + nlen, ndist)) {
				error = "invalid literal/length or distance code lengths";
				return false;
			}
			if (!codes(in, out, lit, dist, limit, error)) return false;
		} else {
			error = "invalid block type";
			return false;
		}
	}
	return true;
}

bool inflate_zlib(const uint8_t *data, size_t size, std::vector<uint8_t> &out, size_t limit, std::string &error);

}  // namespace

bool zlib_inflate(const uint8_t *data, size_t size, std::vector<uint8_t> &out, std::string &error)
{
	return inflate_zlib(data, size, out, SIZE_MAX - 65536, error);
}

namespace {

bool inflate_zlib(const uint8_t *data, size_t size, std::vector<uint8_t> &out, size_t limit, std::string &error)
{
	if (size < 6) {
		error = "zlib stream too short";
		return false;
	}
	const int cmf = data[0], flg = data[1];
	if ((cmf & 0x0f) != 8 || (cmf >> 4) > 7 || ((cmf << 8) | flg) % 31 != 0) {
		error = "not a zlib deflate stream";
		return false;
	}
	if (flg & 0x20) {
		error = "zlib preset dictionaries are not supported";
		return false;
	}
	Bits in(data + 2, size - 2);
	out.clear();
	if (!inflate_raw(in, out, limit, error)) return false;
	in.align();
	if (in.pos + 4 > in.n) {
		error = "missing Adler-32 check";
		return false;
	}
	const uint8_t *a = in.p + in.pos;
	const uint32_t want = ((uint32_t)a[0] << 24) | ((uint32_t)a[1] << 16) | ((uint32_t)a[2] << 8) | a[3];
	if (adler32(out.data(), out.size()) != want) {
		error = "Adler-32 mismatch";
		return false;
	}
	return true;
}

}  // namespace

// ------------------------------------------------------------------ PNG
namespace {

const uint8_t kSignature[8] = {137, 80, 78, 71, 13, 10, 26, 10};

uint32_t be32(const uint8_t *p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

void put32(std::vector<uint8_t> &v, uint32_t x)
{
	v.push_back((uint8_t)(x >> 24));
	v.push_back((uint8_t)(x >> 16));
	v.push_back((uint8_t)(x >> 8));
	v.push_back((uint8_t)x);
}

int paeth(int a, int b, int c)
{
	const int p = a + b - c;
	const int pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
	if (pa <= pb && pa <= pc) return a;
	return (pb <= pc) ? b : c;
}

// Reverses the row filters of one (sub-)image in place: rows of `rowbytes`
// bytes each preceded by their filter type byte.
bool unfilter(uint8_t *d, int rows, size_t rowbytes, int bpp, std::string &error)
{
	const uint8_t *prev = nullptr;
	for (int y = 0; y < rows; y++) {
		uint8_t *row = d + (size_t)y * (rowbytes + 1);
		const int type = row[0];
		uint8_t *r = row + 1;
		for (size_t i = 0; i < rowbytes; i++) {
			const int a = (i >= (size_t)bpp) ? r[i - bpp] : 0;
			const int b = prev ? prev[i] : 0;
			const int c = (prev && i >= (size_t)bpp) ? prev[i - bpp] : 0;
			int pred;
			switch (type) {
			case 0: pred = 0; break;
			case 1: pred = a; break;
			case 2: pred = b; break;
			case 3: pred = (a + b) >> 1; break;
			case 4: pred = paeth(a, b, c); break;
			default: error = "invalid row filter type"; return false;
			}
			r[i] = (uint8_t)(r[i] + pred);
		}
		prev = r;
	}
	return true;
}

struct Header {
	uint32_t width = 0, height = 0;
	int depth = 0, color = 0, interlace = 0;
	int raw_channels() const { return color == 0 ? 1 : color == 2 ? 3 : color == 3 ? 1 : color == 4 ? 2 : 4; }
};

// value of sample `k` (in units of `depth` bits) of a defiltered row
inline uint32_t sample(const uint8_t *row, size_t k, int depth)
{
	if (depth == 8) return row[k];
	if (depth == 16) return ((uint32_t)row[2 * k] << 8) | row[2 * k + 1];
	const size_t bit = k * depth;
	const int shift = 8 - depth - (int)(bit & 7);
	return (row[bit >> 3] >> shift) & ((1u << depth) - 1u);
}

}  // namespace

bool is_png(const uint8_t *data, size_t size) { return size >= 8 && std::memcmp(data, kSignature, 8) == 0; }

bool decode(const uint8_t *data, size_t size, Image &out, std::string &error)
{
	if (!is_png(data, size)) {
		error = "not a PNG file";
		return false;
	}
	Header h;
	std::vector<uint8_t> idat, palette, trns;
	bool have_header = false, ended = false;
	size_t pos = 8;
	while (pos + 12 <= size && !ended) {
		const uint32_t len = be32(data + pos);
		if (len > size - pos - 12) {
			error = "truncated chunk";
			return false;
		}
		const uint8_t *type = data + pos + 4, *body = data + pos + 8;
		const bool critical = (type[0] & 0x20) == 0;
		if (crc32(type, len + 4) != be32(body + len)) {
			if (critical) {
				error = "CRC error in a critical chunk";
				return false;
			}
			pos += 12 + len;  // an ancillary chunk with a bad CRC is dropped
			continue;
		}
		if (!std::memcmp(type, "IHDR", 4)) {
			if (len != 13) {
				error = "bad IHDR";
				return false;
			}
			h.width = be32(body);
			h.height = be32(body + 4);
			h.depth = body[8];
			h.color = body[9];
			h.interlace = body[12];
			if (body[10] != 0 || body[11] != 0 || h.interlace > 1) {
				error = "unsupported compression, filter or interlace method";
				return false;
			}
			have_header = true;
		} else if (!std::memcmp(type, "PLTE", 4)) {
			palette.assign(body, body + len);
		} else if (!std::memcmp(type, "tRNS", 4)) {
			trns.assign(body, body + len);
		} else if (!std::memcmp(type, "IDAT", 4)) {
			idat.insert(idat.end(), body, body + len);
		} else if (!std::memcmp(type, "IEND", 4)) {
			ended = true;
		} else if (critical) {
			error = "unknown critical chunk";
			return false;
		}
		pos += 12 + len;
	}
	if (!have_header || idat.empty()) {
		error = "missing IHDR or IDAT";
		return false;
	}
	const int d = h.depth, ct = h.color;
	const bool ok_depth = (ct == 0 && (d == 1 || d == 2 || d == 4 || d == 8 || d == 16)) ||
	                      (ct == 3 && (d == 1 || d == 2 || d == 4 || d == 8)) ||
	                      ((ct == 2 || ct == 4 || ct == 6) && (d == 8 || d == 16));
	if (!ok_depth) {
		error = "invalid colour type / bit depth";
		return false;
	}
	if (h.width == 0 || h.height == 0 || h.width > (1u << 24) || h.height > (1u << 24) ||
	    (uint64_t)h.width * h.height > (1ull << 28)) {
		error = "image size out of range";
		return false;
	}
	if (ct == 3 && (palette.empty() || palette.size() % 3 != 0 || palette.size() / 3 > (1u << d))) {
		error = "missing or invalid palette";
		return false;
	}
	const int W = (int)h.width, H = (int)h.height, rc = h.raw_channels();
	const int bpp = std::max(1, rc * d / 8);
	// defiltered raw pixels of the whole image, rows of rowbytes(W) bytes
	auto rowbytes = [&](int w) { return ((size_t)w * rc * d + 7) / 8; };
	// the inflated size is bounded (extra data after the image, which libpng
	// tolerates, is accepted up to 1 MiB and ignored)
	const size_t expected = h.interlace ? (size_t)H * (rowbytes(W) + 1) * 2 + 64 : (size_t)H * (rowbytes(W) + 1);
	std::vector<uint8_t> raw;
	if (!inflate_zlib(idat.data(), idat.size(), raw, expected + (1u << 20), error)) return false;
	std::vector<uint8_t> full((size_t)H * rowbytes(W));
	static const int ax0[7] = {0, 4, 0, 2, 0, 1, 0}, ay0[7] = {0, 0, 4, 0, 2, 0, 1};
	static const int adx[7] = {8, 8, 4, 4, 2, 2, 1}, ady[7] = {8, 8, 8, 4, 4, 2, 2};
	const int passes = h.interlace ? 7 : 1;
	size_t at = 0;
	for (int ps = 0; ps < passes; ps++) {
		const int x0 = h.interlace ? ax0[ps] : 0, y0 = h.interlace ? ay0[ps] : 0;
		const int dx = h.interlace ? adx[ps] : 1, dy = h.interlace ? ady[ps] : 1;
		const int pw = (W - x0 + dx - 1) / dx, ph = (H - y0 + dy - 1) / dy;
		if (pw <= 0 || ph <= 0) continue;
		const size_t rb = rowbytes(pw), need = (size_t)ph * (rb + 1);
		if (at + need > raw.size()) {
			error = "not enough image data";
			return false;
		}
		if (!unfilter(raw.data() + at, ph, rb, bpp, error)) return false;
		for (int y = 0; y < ph; y++) {
			const uint8_t *src = raw.data() + at + (size_t)y * (rb + 1) + 1;
			uint8_t *dst = full.data() + (size_t)(y0 + y * dy) * rowbytes(W);
			if (!h.interlace) {
				std::memcpy(dst, src, rb);
				continue;
			}
			for (int x = 0; x < pw; x++) {  // scatter the pass's pixels
				const int X = x0 + x * dx;
				if (d >= 8) {
					const size_t bytes = (size_t)rc * d / 8;
					std::memcpy(dst + (size_t)X * bytes, src + (size_t)x * bytes, bytes);
				} else {
					const uint32_t v = sample(src, (size_t)x, d);
					const size_t bit = (size_t)X * d;
					const int shift = 8 - d - (int)(bit & 7);
					dst[bit >> 3] = (uint8_t)((dst[bit >> 3] & ~(((1u << d) - 1u) << shift)) | (v << shift));
				}
			}
		}
		at += need;
	}

	// expansion (libpng's PNG_TRANSFORM_EXPAND as iio requests it)
	const bool key = !trns.empty() && (ct == 0 || ct == 2);
	const bool pal_alpha = !trns.empty() && ct == 3;
	out.width = W;
	out.height = H;
	out.depth = (d == 16) ? 16 : 8;
	out.channels = (ct == 3) ? (pal_alpha ? 4 : 3) : rc + (key ? 1 : 0);
	const uint32_t maxv = (d == 16) ? 65535u : 255u;
	out.samples.assign((size_t)W * H * out.channels, 0);
	uint32_t kg = 0, kr = 0, kgreen = 0, kb = 0;
	if (key && ct == 0 && trns.size() >= 2) kg = ((uint32_t)trns[0] << 8 | trns[1]) & ((d == 16) ? 0xffffu : ((1u << d) - 1u));
	if (key && ct == 2 && trns.size() >= 6) {
		kr = (uint32_t)trns[0] << 8 | trns[1];
		kgreen = (uint32_t)trns[2] << 8 | trns[3];
		kb = (uint32_t)trns[4] << 8 | trns[5];
	}
	for (int y = 0; y < H; y++) {
		const uint8_t *row = full.data() + (size_t)y * rowbytes(W);
		uint16_t *o = out.samples.data() + (size_t)y * W * out.channels;
		for (int x = 0; x < W; x++, o += out.channels) {
			if (ct == 3) {
				const uint32_t idx = sample(row, (size_t)x, d);
				if (idx >= palette.size() / 3) {
					error = "palette index out of range";
					return false;
				}
				o[0] = palette[3 * idx];
				o[1] = palette[3 * idx + 1];
				o[2] = palette[3 * idx + 2];
				if (pal_alpha) o[3] = (idx < trns.size()) ? trns[idx] : 255;
			} else if (ct == 0) {
				const uint32_t v = sample(row, (size_t)x, d);
				o[0] = (uint16_t)((d < 8) ? v * (255u / ((1u << d) - 1u)) : v);
				if (key) o[1] = (uint16_t)((trns.size() >= 2 && v == kg) ? 0 : maxv);
			} else if (ct == 2) {
				const uint32_t r = sample(row, (size_t)3 * x, d), g = sample(row, (size_t)3 * x + 1, d),
				               b = sample(row, (size_t)3 * x + 2, d);
				o[0] = (uint16_t)r;
				o[1] = (uint16_t)g;
				o[2] = (uint16_t)b;
				if (key) o[3] = (uint16_t)((trns.size() >= 6 && r == kr && g == kgreen && b == kb) ? 0 : maxv);
			} else {
				for (int c = 0; c < rc; c++) o[c] = (uint16_t)sample(row, (size_t)rc * x + c, d);
			}
		}
	}
	return true;
}

namespace {

// LSB-first bit packing of a DEFLATE stream
struct BitWriter {
	std::vector<uint8_t> &out;
	uint32_t buf = 0;
	int count = 0;
	explicit BitWriter(std::vector<uint8_t> &o) : out(o) {}
	void put(uint32_t v, int n)
	{
		buf |= v << count;
		count += n;
		while (count >= 8) {
			out.push_back((uint8_t)buf);
			buf >>= 8;
			count -= 8;
		}
	}
	// a Huffman code: its bits go out most significant first
	void code(uint32_t c, int n)
	{
		uint32_t r = 0;
		for (int k = 0; k < n; k++) r |= ((c >> k) & 1u) << (n - 1 - k);
		put(r, n);
	}
	void flush()
	{
		if (count > 0) out.push_back((uint8_t)buf);
		buf = 0;
		count = 0;
	}
};

// literal / length symbol in the fixed code of RFC 1951 section 3.2.6
void fixed_symbol(BitWriter &w, int s)
{
	if (s < 144)
		w.code(0x30 + s, 8);
	else if (s < 256)
		w.code(0x190 + (s - 144), 9);
	else if (s < 280)
		w.code(s - 256, 7);
	else
		w.code(0xC0 + (s - 280), 8);
}

// One fixed-Huffman DEFLATE block over the whole input, with greedy LZ77
// matches found through 3-byte hash chains (window 32 KiB, matches 3..258).
std::vector<uint8_t> deflate_fixed(const uint8_t *in, size_t n)
{
	std::vector<uint8_t> out;
	BitWriter w(out);
	w.put(1, 1);  // last block
	w.put(1, 2);  // fixed codes
	constexpr int kHashBits = 15, kChain = 48;
	constexpr size_t kWindow = 32768, kMaxMatch = 258;
	std::vector<int32_t> head((size_t)1 << kHashBits, -1), prev(n, -1);
	auto hash = [&](size_t i) {
		const uint32_t v = (uint32_t)in[i] << 16 | (uint32_t)in[i + 1] << 8 | in[i + 2];
		return (v * 2654435761u) >> (32 - kHashBits);
	};
	auto insert = [&](size_t i) {
		if (i + 2 >= n) return;
		const uint32_t h = hash(i);
		prev[i] = head[h];
		head[h] = (int32_t)i;
	};
	size_t i = 0;
	while (i < n) {
		size_t best = 0, best_dist = 0;
		if (i + 2 < n) {
			const size_t limit = std::min(kMaxMatch, n - i);
			int32_t cand = head[hash(i)];
			for (int k = 0; k < kChain && cand >= 0 && i - (size_t)cand <= kWindow; k++, cand = prev[cand]) {
				size_t len = 0;
				while (len < limit && in[cand + len] == in[i + len]) len++;
				if (len > best) {
					best = len;
					best_dist = i - (size_t)cand;
					if (len == limit) break;
				}
			}
		}
		if (best >= 3) {
			int li = 28;
			while (kLenBase[li] > best) li--;
			fixed_symbol(w, 257 + li);
			w.put((uint32_t)(best - kLenBase[li]), kLenExtra[li]);
			int di = 29;
			while (kDistBase[di] > best_dist) di--;
			w.code((uint32_t)di, 5);
			w.put((uint32_t)(best_dist - kDistBase[di]), kDistExtra[di]);
			for (size_t k = 0; k < best; k++) insert(i + k);
			i += best;
		} else {
			fixed_symbol(w, in[i]);
			insert(i);
			i++;
		}
	}
	fixed_symbol(w, 256);
	w.flush();
	return out;
}

}  // namespace

std::vector<uint8_t> encode8(const uint8_t *samples, int width, int height, int channels)
{
	static const uint8_t colour[5] = {0, 0, 4, 2, 6};
	std::vector<uint8_t> png(kSignature, kSignature + 8);
	auto chunk = [&](const char *type, const std::vector<uint8_t> &body) {
		put32(png, (uint32_t)body.size());
		const size_t start = png.size();
		png.insert(png.end(), type, type + 4);
		png.insert(png.end(), body.begin(), body.end());
		put32(png, crc32(png.data() + start, body.size() + 4));
	};
	std::vector<uint8_t> ihdr;
	put32(ihdr, (uint32_t)width);
	put32(ihdr, (uint32_t)height);
	ihdr.push_back(8);
	ihdr.push_back(colour[channels]);
	ihdr.push_back(0);  // deflate
	ihdr.push_back(0);  // adaptive filtering
	ihdr.push_back(0);  // not interlaced
	chunk("IHDR", ihdr);
	// each row with the filter of smallest sum of |signed residual| (the
	// usual adaptive heuristic)
	const size_t rb = (size_t)width * channels;
	const int bpp = channels;
	std::vector<uint8_t> filtered;
	filtered.reserve((size_t)height * (rb + 1));
	std::vector<uint8_t> trial[5];
	for (auto &t : trial) t.resize(rb);
	for (int y = 0; y < height; y++) {
		const uint8_t *r = samples + (size_t)y * rb;
		const uint8_t *up = y > 0 ? r - rb : nullptr;
		uint64_t best_cost = UINT64_MAX;
		int best = 0;
		for (int f = 0; f < 5; f++) {
			uint64_t cost = 0;
			for (size_t i = 0; i < rb; i++) {
				const int a = (i >= (size_t)bpp) ? r[i - bpp] : 0;
				const int b = up ? up[i] : 0;
				const int c = (up && i >= (size_t)bpp) ? up[i - bpp] : 0;
				const int pred = f == 0 ? 0 : f == 1 ? a : f == 2 ? b : f == 3 ? ((a + b) >> 1) : paeth(a, b, c);
				const uint8_t v = (uint8_t)(r[i] - pred);
				trial[f][i] = v;
				cost += (uint64_t)(v < 128 ? v : 256 - v);
			}
			if (cost < best_cost) {
				best_cost = cost;
				best = f;
			}
		}
		filtered.push_back((uint8_t)best);
		filtered.insert(filtered.end(), trial[best].begin(), trial[best].end());
	}
	std::vector<uint8_t> z = {0x78, 0x01};
	const std::vector<uint8_t> d = deflate_fixed(filtered.data(), filtered.size());
	z.insert(z.end(), d.begin(), d.end());
	put32(z, adler32(filtered.data(), filtered.size()));
	chunk("IDAT", z);
	chunk("IEND", {});
	return png;
}

}  // namespace nli_png
