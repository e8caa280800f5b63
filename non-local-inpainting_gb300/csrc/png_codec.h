// PNG reading and writing for the command-line program, without libpng:
// the reference reads and writes its images through iio on libpng
// (3rdparty/iio/iio.c read_beheaded_png, iio_save_image_as_png), which is
// not available here.  Host code only.
//
// Decoding follows the PNG specification (ISO/IEC 15948) and zlib / DEFLATE
// (RFC 1950 / RFC 1951) and returns the samples the way iio's reader sees
// them after libpng's PNG_TRANSFORM_EXPAND: palette images become RGB (RGBA
// when a tRNS chunk is present), grey images of 1, 2 or 4 bits are scaled
// to 8 bits, a tRNS colour key becomes an alpha channel, and 16-bit samples
// stay 16-bit.  Interlaced (Adam7) images are supported.
//
// Encoding writes 8-bit grey, grey + alpha, RGB or RGBA images, each row
// with the adaptive filter of smallest residual, compressed with the fixed
// Huffman code of DEFLATE over greedy LZ77 matches.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace nli_png {

struct Image {
	int width = 0, height = 0;
	int channels = 0;   // 1 grey, 2 grey + alpha, 3 RGB, 4 RGBA (after expansion)
	int depth = 0;      // 8 or 16 bits per sample (after expansion)
	std::vector<uint16_t> samples;  // width * height * channels, row-major, interleaved
};

// True when the bytes start with the PNG signature.
bool is_png(const uint8_t *data, size_t size);

// Decodes a whole PNG file held in memory.  Returns false with a message in
// `error` on a malformed or unsupported file.
bool decode(const uint8_t *data, size_t size, Image &out, std::string &error);

// Encodes 8-bit samples (width * height * channels, channels 1..4).
std::vector<uint8_t> encode8(const uint8_t *samples, int width, int height, int channels);

// zlib stream (RFC 1950) inflation, exposed for tests: false on a malformed
// stream or an Adler-32 mismatch.
bool zlib_inflate(const uint8_t *data, size_t size, std::vector<uint8_t> &out, std::string &error);

uint32_t crc32(const uint8_t *data, size_t size, uint32_t crc = 0);
uint32_t adler32(const uint8_t *data, size_t size, uint32_t adler = 1);

}  // namespace nli_png
