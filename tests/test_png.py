"""The command-line program's PNG codec (csrc/png_codec.cpp, which stands in
for iio on libpng) against an independent Python encoder built on the
standard library's zlib: every colour type and bit depth, colour-key and
palette transparency, Adam7 interlacing, all five row filters, stored /
fixed / dynamic DEFLATE blocks, split IDAT chunks and corrupt files.  The
expected samples follow libpng's PNG_TRANSFORM_EXPAND, which iio's reader
asks for (3rdparty/iio/iio.c read_beheaded_png): palette to RGB(A), grey of
1/2/4 bits scaled to 8 bits, tRNS to an alpha channel, 16 bits kept.  The
encoder's files are decoded with zlib and checked the same way.  No GPU."""
import os
import struct
import subprocess
import zlib

import numpy as np
import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "non-local-inpainting_gb300", "csrc")


@pytest.fixture(scope="module")
def tool(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("png") / "png_tool")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", CSRC, os.path.join(ROOT, "tests", "cpp", "png_tool.cpp"),
                    os.path.join(CSRC, "png_codec.cpp"), "-o", out], check=True)
    return out


# ------------------------------------------------------- reference encoder
def chunk(kind, body):
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xffffffff)


def pack_row(samples, depth):
    """One row of raw samples (1-D uint) to bytes."""
    if depth == 16:
        return samples.astype(">u2").tobytes()
    if depth == 8:
        return samples.astype(np.uint8).tobytes()
    per = 8 // depth
    n = (len(samples) + per - 1) // per
    out = bytearray(n)
    for i, v in enumerate(samples):
        out[i // per] |= int(v) << (8 - depth * (i % per + 1))
    return bytes(out)


def paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)


def filter_rows(rows, bpp, types):
    out, prev = bytearray(), bytes(len(rows[0])) if rows else b""
    for y, row in enumerate(rows):
        t = types[y % len(types)]
        f = bytearray(len(row))
        for i in range(len(row)):
            a = row[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            pred = [0, a, b, (a + b) >> 1, paeth(a, b, c)][t]
            f[i] = (row[i] - pred) & 0xff
        out += bytes([t]) + bytes(f)
        prev = row
    return bytes(out)


ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


def make_png(raw, color, depth, palette=None, trns=None, interlace=False, filters=(0,), level=6, split=1,
             extra=b""):
    """raw: (H, W, rc) array of raw sample values (palette indices for colour
    type 3)."""
    H, W, rc = raw.shape
    bpp = max(1, rc * depth // 8)

    def image_bytes(sub):
        rows = [pack_row(sub[y].reshape(-1), depth) for y in range(sub.shape[0])]
        return filter_rows(rows, bpp, filters) if rows and sub.shape[1] else b""
    if interlace:
        data = b"".join(image_bytes(raw[y0::dy, x0::dx]) for x0, y0, dx, dy in ADAM7)
    else:
        data = image_bytes(raw)
    z = zlib.compress(data, level)
    parts = [z[i * len(z) // split:(i + 1) * len(z) // split] for i in range(split)]
    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", W, H, depth, color, 0, 0, int(interlace)))
    png += extra
    if palette is not None:
        png += chunk(b"PLTE", bytes(np.asarray(palette, np.uint8).reshape(-1)))
    if trns is not None:
        png += chunk(b"tRNS", trns)
    for p in parts:
        png += chunk(b"IDAT", p)
    return png + chunk(b"IEND", b"")


def expand(raw, color, depth, palette=None, trns=None):
    """The samples libpng's EXPAND transform yields."""
    mx = 65535 if depth == 16 else 255
    if color == 3:
        pal = np.asarray(palette, np.uint16)
        rgb = pal[raw[..., 0]]
        if trns is None:
            return rgb
        alpha = np.full(len(pal), 255, np.uint16)
        alpha[:len(trns)] = np.frombuffer(trns, np.uint8)
        return np.concatenate([rgb, alpha[raw[..., 0]][..., None]], -1)
    v = raw.astype(np.uint16)
    if color == 0 and depth < 8:
        v = v * (255 // ((1 << depth) - 1))
    if trns is not None and color in (0, 2):
        key = np.frombuffer(trns, ">u2").astype(np.int64)
        if color == 0:
            key = key & (0xffff if depth == 16 else (1 << depth) - 1)
        hit = np.all(raw.astype(np.int64) == key.reshape(1, 1, -1), -1)
        v = np.concatenate([v, np.where(hit, 0, mx).astype(np.uint16)[..., None]], -1)
    return v


def decode(tool, tmp, png):
    src, dst = str(tmp / "in.png"), str(tmp / "out.bin")
    with open(src, "wb") as f:
        f.write(png)
    r = subprocess.run([tool, "decode", src, dst], capture_output=True, text=True)
    if r.returncode != 0:
        return None, r.stderr.strip()
    b = open(dst, "rb").read()
    W, H, C, D = struct.unpack("<4i", b[:16])
    return (np.frombuffer(b[16:], "<u2").reshape(H, W, C), D), ""


CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}
CASES = [(0, 1), (0, 2), (0, 4), (0, 8), (0, 16), (2, 8), (2, 16), (3, 1), (3, 2), (3, 4), (3, 8), (4, 8), (4, 16),
         (6, 8), (6, 16)]


def random_raw(rng, color, depth, H, W, npal=None):
    top = (npal if color == 3 else 1 << depth) - 1
    return rng.integers(0, top + 1, (H, W, CHANNELS[color])).astype(np.uint32)


@pytest.mark.parametrize("interlace", [False, True])
@pytest.mark.parametrize("color,depth", CASES)
def test_decode_every_format(tool, tmp_path, color, depth, interlace):
    rng = np.random.default_rng(color * 100 + depth + 7 * interlace)
    H, W = 13, 11  # odd sizes exercise partial Adam7 passes and row padding
    npal = min(1 << depth, 200) if color == 3 else None
    raw = random_raw(rng, color, depth, H, W, npal)
    palette = rng.integers(0, 256, (npal, 3)) if color == 3 else None
    for trns in (None, "set"):
        t = None
        if trns and color == 0:
            t = struct.pack(">H", int(raw[3, 4, 0]))
        elif trns and color == 2:
            t = struct.pack(">HHH", *[int(x) for x in raw[5, 2]])
        elif trns and color == 3:
            t = bytes(rng.integers(0, 256, max(1, npal // 2)).astype(np.uint8))
        elif trns:
            continue  # colour types with alpha take no tRNS
        png = make_png(raw, color, depth, palette, t, interlace, filters=(0, 1, 2, 3, 4), level=9)
        got, err = decode(tool, tmp_path, png)
        assert got is not None, err
        samples, d = got
        assert d == (16 if depth == 16 else 8)
        assert np.array_equal(samples, expand(raw, color, depth, palette, t))


@pytest.mark.parametrize("level", [0, 1, 6, 9])
def test_deflate_blocks_and_split_idat(tool, tmp_path, level):
    """Stored (level 0), fixed and dynamic Huffman blocks, the stream split
    over several IDAT chunks; a larger smooth image gives long matches."""
    y, x = np.mgrid[0:96, 0:150]
    raw = np.stack([(x * 3 + y) % 256, (y * 5) % 256, (x ^ y) % 256], -1).astype(np.uint32)
    png = make_png(raw, 2, 8, filters=(4, 0, 1, 2, 3), level=level, split=5)
    (samples, d), err = decode(tool, tmp_path, png)
    assert np.array_equal(samples, raw)


def test_zlib_streams(tool, tmp_path):
    rng = np.random.default_rng(3)
    blobs = [b"", bytes(rng.integers(0, 256, 70000).astype(np.uint8)), b"abc" * 40000,
             bytes(rng.integers(0, 4, 5000).astype(np.uint8))]
    for i, blob in enumerate(blobs):
        for level in (0, 1, 9):
            src, dst = str(tmp_path / "z"), str(tmp_path / "u")
            with open(src, "wb") as f:
                f.write(zlib.compress(blob, level))
            r = subprocess.run([tool, "inflate", src, dst], capture_output=True, text=True)
            assert r.returncode == 0, (i, level, r.stderr)
            assert open(dst, "rb").read() == blob


def test_rejects_corrupt_files(tool, tmp_path):
    raw = np.arange(48, dtype=np.uint32).reshape(4, 4, 3) * 5
    good = make_png(raw, 2, 8)
    assert decode(tool, tmp_path, good)[0] is not None
    # an ancillary chunk with a bad CRC is skipped, as libpng does by default
    bad_anc = chunk(b"tEXt", b"k\x00v")[:-1] + b"\x00"
    assert decode(tool, tmp_path, make_png(raw, 2, 8, extra=bad_anc))[0] is not None
    idat = good.index(b"IDAT")
    flipped = bytearray(good)
    flipped[idat + 6] ^= 0x40  # a byte of the compressed data: IDAT CRC no longer matches
    cases = {"truncated": good[:len(good) // 2], "bad crc": bytes(flipped), "not png": b"P6\n1 1\n255\n\x00\x00\x00",
             "bad depth": make_png(raw, 2, 8)[:16] + struct.pack(">IIBBBBB", 4, 4, 4, 2, 0, 0, 0)}
    cases["bad depth"] = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", 4, 4, 4, 2, 0, 0, 0)) + \
        good[good.index(b"IDAT") - 4:]
    for name, png in cases.items():
        got, err = decode(tool, tmp_path, png)
        assert got is None and err, name


def unfilter8(raw, H, W, C):
    """Reverses the row filters of an 8-bit image (bytes per pixel C)."""
    stride = W * C
    rows = np.frombuffer(raw, np.uint8).reshape(H, stride + 1)
    out = np.zeros((H, stride), np.int64)
    for y in range(H):
        t, r = rows[y, 0], rows[y, 1:].astype(np.int64)
        up = out[y - 1] if y > 0 else np.zeros(stride, np.int64)
        cur = np.zeros(stride, np.int64)
        for i in range(stride):
            a = cur[i - C] if i >= C else 0
            b = up[i]
            c = up[i - C] if i >= C else 0
            pred = [0, a, b, (a + b) >> 1, paeth(a, b, c)][t]
            cur[i] = (r[i] + pred) & 0xff
        out[y] = cur
    return out.astype(np.uint8).reshape(H, W, C)


def read_png_python(data):
    """Reader for the encoder's output (8-bit, any row filters)."""
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, hdr = 8, b"", None
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        assert struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0] == zlib.crc32(kind + body) & 0xffffffff
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat += body
        pos += 12 + n
    W, H, depth, color = hdr[:4]
    C = {0: 1, 4: 2, 2: 3, 6: 4}[color]
    assert depth == 8
    return unfilter8(zlib.decompress(idat), H, W, C)


@pytest.mark.parametrize("C", [1, 2, 3, 4])
def test_encoder(tool, tmp_path, C):
    """Random (incompressible) and smooth images: zlib inflates the stream,
    the filters undo to the input, and the smooth image compresses."""
    rng = np.random.default_rng(C)
    y, x = np.mgrid[0:120, 0:160]
    smooth = np.stack([(x + y) % 256, (2 * x) % 256, (y * 3) % 256, np.full_like(x, 200)], -1)[..., :C]
    for img in (rng.integers(0, 256, (1, 1, C)), rng.integers(0, 256, (23, 37, C)), smooth):
        img = np.ascontiguousarray(img).astype(np.uint8)
        H, W = img.shape[:2]
        src, dst = str(tmp_path / "raw"), str(tmp_path / "o.png")
        img.tofile(src)
        subprocess.run([tool, "encode", str(W), str(H), str(C), src, dst], check=True)
        data = open(dst, "rb").read()
        assert np.array_equal(read_png_python(data), img)
        (samples, d), err = decode(tool, tmp_path, data)  # and our own decoder reads it back
        assert np.array_equal(samples, img)
        if img is smooth or H == 120:
            assert len(data) < img.size // 4, (len(data), img.size)


@pytest.fixture(scope="module")
def checked_tool(tmp_path_factory):
    """The test driver built with AddressSanitizer and UBSan (skipped where
    the compiler lacks them)."""
    out = str(tmp_path_factory.mktemp("png_asan") / "png_tool")
    r = subprocess.run(["g++", "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
                        "-std=c++17", "-I", CSRC, os.path.join(ROOT, "tests", "cpp", "png_tool.cpp"),
                        os.path.join(CSRC, "png_codec.cpp"), "-o", out], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("no sanitizer runtime: " + r.stderr[-200:])
    good = str(tmp_path_factory.mktemp("png_asan_probe") / "g.png")
    with open(good, "wb") as f:
        f.write(make_png(np.zeros((2, 2, 3), np.uint32), 2, 8))
    r = subprocess.run([out, "decode", good, good + ".bin"], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("sanitized binaries do not run here: " + r.stderr[-200:])
    return out


def test_decoder_survives_corruption(checked_tool, tmp_path):
    """Structure-aware corruption (chunk CRCs recomputed, so the inflater,
    the filters and the expansion see the damage): every file is either
    decoded or rejected with a message, with no sanitizer report."""
    import random
    rng, rnd = np.random.default_rng(11), random.Random(11)
    seeds = []
    for color, depth in CASES:
        npal = min(1 << depth, 200) if color == 3 else None
        raw = random_raw(rng, color, depth, 9, 7, npal)
        pal = rng.integers(0, 256, (npal, 3)) if color == 3 else None
        png = make_png(raw, color, depth, pal, None, interlace=bool(rng.integers(2)), filters=(0, 1, 2, 3, 4),
                       level=int(rng.integers(0, 10)))
        pos, chunks = 8, []
        while pos < len(png):
            n = struct.unpack(">I", png[pos:pos + 4])[0]
            chunks.append((png[pos + 4:pos + 8], png[pos + 8:pos + 8 + n]))
            pos += 12 + n
        seeds.append(chunks)
    outcomes = {0: 0, 2: 0}
    for it in range(300):
        chunks = []
        mode = rnd.random()
        for kind, body in rnd.choice(seeds):
            b = bytearray(body)
            if kind == b"IDAT" and mode < 0.4 and b:
                for _ in range(rnd.randint(1, 4)):
                    b[rnd.randrange(len(b))] = rnd.randrange(256)
            elif kind == b"IDAT" and mode < 0.8:
                data = bytearray(zlib.decompress(bytes(b)))
                for _ in range(rnd.randint(1, 4)):
                    data[rnd.randrange(len(data))] = rnd.randrange(256)
                data = data[:rnd.randrange(len(data) + 1)] if rnd.random() < 0.3 else data + bytes(rnd.randrange(40))
                b = bytearray(zlib.compress(bytes(data), rnd.randrange(10)))
            elif kind in (b"IHDR", b"PLTE") and mode >= 0.8 and b:
                b[rnd.randrange(len(b))] = rnd.randrange(256)
            chunks.append(chunk(kind, bytes(b)))
        src = str(tmp_path / "f.png")
        with open(src, "wb") as f:
            f.write(b"\x89PNG\r\n\x1a\n" + b"".join(chunks))
        r = subprocess.run([checked_tool, "decode", src, str(tmp_path / "f.bin")], capture_output=True, text=True)
        assert r.returncode in (0, 2), (it, r.returncode, r.stderr[-800:])
        assert r.returncode == 0 or r.stderr.strip()
        outcomes[r.returncode] += 1
    assert outcomes[0] > 10 and outcomes[2] > 10, outcomes
