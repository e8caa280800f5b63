// Test driver for the command-line program's PNG codec
// (non-local-inpainting_gb300/csrc/png_codec.cpp), built by tests/test_png.py:
//   png_tool decode IN.png OUT     -> int32 width, height, channels, depth; uint16 samples
//   png_tool encode W H C IN OUT.png  (IN: W*H*C bytes)
//   png_tool inflate IN OUT        (zlib stream)
// Exit status 2 with the decoder's message on stderr for a rejected input.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "png_codec.h"

static std::vector<uint8_t> slurp(const char *name)
{
	std::vector<uint8_t> v;
	FILE *f = fopen(name, "rb");
	if (!f) return v;
	unsigned char buf[65536];
	size_t n;
	while ((n = fread(buf, 1, sizeof(buf), f)) > 0) v.insert(v.end(), buf, buf + n);
	fclose(f);
	return v;
}

static void spill(const char *name, const void *p, size_t n)
{
	FILE *f = fopen(name, "wb");
	fwrite(p, 1, n, f);
	fclose(f);
}

int main(int argc, char **argv)
{
	if (argc < 2) return 1;
	const std::string cmd = argv[1];
	if (cmd == "decode" && argc == 4) {
		std::vector<uint8_t> in = slurp(argv[2]);
		nli_png::Image im;
		std::string err;
		if (!nli_png::decode(in.data(), in.size(), im, err)) {
			fprintf(stderr, "%s\n", err.c_str());
			return 2;
		}
		std::vector<uint8_t> out(16 + 2 * im.samples.size());
		const int32_t hdr[4] = {im.width, im.height, im.channels, im.depth};
		std::memcpy(out.data(), hdr, 16);
		std::memcpy(out.data() + 16, im.samples.data(), 2 * im.samples.size());
		spill(argv[3], out.data(), out.size());
		return 0;
	}
	if (cmd == "encode" && argc == 7) {
		const int W = atoi(argv[2]), H = atoi(argv[3]), C = atoi(argv[4]);
		std::vector<uint8_t> in = slurp(argv[5]);
		if (in.size() != (size_t)W * H * C) return 1;
		std::vector<uint8_t> png = nli_png::encode8(in.data(), W, H, C);
		spill(argv[6], png.data(), png.size());
		return 0;
	}
	if (cmd == "inflate" && argc == 4) {
		std::vector<uint8_t> in = slurp(argv[2]), out;
		std::string err;
		if (!nli_png::zlib_inflate(in.data(), in.size(), out, err)) {
			fprintf(stderr, "%s\n", err.c_str());
			return 2;
		}
		spill(argv[3], out.data(), out.size());
		return 0;
	}
	return 1;
}
