"""The command-line caller of the path: colour conversions on the GPU
against the reference's (golden vectors), RGB-D packing, and nli_inpaint
(main.cpp's program on the drop-in classes) against the same steps driven
through the C ABI."""
import os
import struct
import subprocess
import zlib

import numpy as np
import pytest

import __graft_entry__ as ge
from conftest import ROOT

pytestmark = pytest.mark.gpu
CLI = os.path.join(ROOT, "non-local-inpainting_gb300", "nli_inpaint")


def test_lab_conversions(gpu_ctx, units):
    # the GPU evaluates the reference's float pow as a double pow rounded to float
    lab = gpu_ctx.rgb_to_lab(units["lab_rgb_in"]).cpu().numpy()
    assert np.abs(lab - units["lab_out"]).max() <= 1e-4
    back = gpu_ctx.lab_to_rgb(units["lab_out"]).cpu().numpy()
    assert np.abs(back - units["lab_rgb_back"]).max() <= 1e-3
    assert np.abs(back - units["lab_rgb_in"]).max() <= 0.02  # the round trip
    # a depth channel is dropped (the reference's own 4-channel path reads
    # freed memory, io_utility.cpp:303-307)
    back4 = gpu_ctx.lab_to_rgb(units["lab4_in"]).cpu().numpy()
    assert np.array_equal(back4, back)


def test_depth_packing(gpu_ctx):
    rng = np.random.default_rng(1)
    rgb = rng.uniform(0, 255, (13, 17, 3)).astype(np.float32)
    depth = rng.uniform(0.5, 5, (13, 17)).astype(np.float32)
    rgbd = gpu_ctx.cat_depth(rgb, depth).cpu().numpy()
    assert np.array_equal(rgbd, np.concatenate([rgb, depth[..., None]], -1))
    r, d = gpu_ctx.separate_depth(rgbd)
    assert np.array_equal(r.cpu().numpy(), rgb) and np.array_equal(d.cpu().numpy(), depth)


def write_pnm(path, a):
    a = np.clip(np.round(a), 0, 255).astype(np.uint8)
    H, W = a.shape[:2]
    with open(path, "wb") as f:
        f.write(b"P6\n" if a.ndim == 3 else b"P5\n")
        f.write(b"%d %d\n255\n" % (W, H))
        f.write(a.tobytes())


def write_png(path, a):
    """8-bit PNG of an (H, W) or (H, W, C) array with the standard library."""
    a = np.asarray(a, np.uint8)
    if a.ndim == 2:
        a = a[..., None]
    H, W, C = a.shape
    raw = b"".join(b"\x00" + a[y].tobytes() for y in range(H))

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xffffffff)
    color = {1: 0, 2: 4, 3: 2, 4: 6}[C]
    data = (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", W, H, 8, color, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))
    with open(path, "wb") as f:
        f.write(data)


def paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)


def read_png(path):
    """The program's PNG output: 8-bit, adaptive row filters."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat = 8, b""
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        if kind == b"IHDR":
            W, H, depth, color = struct.unpack(">IIBB", body[:10])
        elif kind == b"IDAT":
            idat += body
        pos += 12 + n
    C = {0: 1, 4: 2, 2: 3, 6: 4}[color]
    assert depth == 8
    rows = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(H, W * C + 1)
    out = np.zeros((H, W * C), np.int64)
    for y in range(H):
        t, r = int(rows[y, 0]), rows[y, 1:].astype(np.int64)
        up = out[y - 1] if y > 0 else np.zeros(W * C, np.int64)
        for i in range(W * C):
            a = out[y, i - C] if i >= C else 0
            c = up[i - C] if i >= C else 0
            out[y, i] = (r[i] + [0, a, up[i], (a + up[i]) >> 1, paeth(a, up[i], c)][t]) & 0xff
    return out.astype(np.uint8).reshape(H, W, C)


@pytest.fixture(scope="module")
def cli():
    ge.build()
    assert os.path.exists(CLI)
    return CLI


def test_cli_matches_c_abi(cli, gpu_ctx, tmp_path):
    from nli_gb300 import workloads as wl
    img, mask, _ = wl.config2(seed=8, size=72, scales=3)
    img8 = np.clip(np.round(img), 0, 255)
    write_pnm(tmp_path / "in.ppm", img8)
    write_pnm(tmp_path / "mask.pgm", mask * 255)
    r = subprocess.run([cli, "in.ppm", "mask.pgm", "out", "-method", "nlmeans", "-patch", "9", "-scales", "3",
                        "-coarse", "0.5", "-iters", "10", "-seed", "5", "-shownnf", "nnf.png", "-showpyr", "pyr_"],
                       cwd=tmp_path, capture_output=True, text=True)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stderr
    name = "out_nlmeans_sc3_0.5_initpoisson_ps9_10000_conf5_0.1.png"  # main.cpp's composed name, with Poisson initialisation named as such
    assert name in r.stdout
    got = read_png(tmp_path / name)
    # the same steps through the C ABI: Lab, process with the CLI's pairing
    # (nlmeans with L2Norm distances), back to RGB, rounded
    p = wl.params("nlmeans", distance="l2", patch=9, scales=3, coarse=0.5, iters=10)
    p.patchmatch.random_shots = 30
    lab = gpu_ctx.rgb_to_lab(img8.astype(np.float32)).cpu().numpy()
    gpu_ctx.set_seed(5)
    out, _ = gpu_ctx.process(lab, mask, p)
    v = gpu_ctx.lab_to_rgb(out).cpu().numpy().astype(np.float64)
    v = np.where(v >= 0, np.floor(v + 0.5), np.ceil(v - 0.5))  # std::round: halves away from zero
    want = np.clip(v, 0, 255).astype(np.uint8)
    assert np.array_equal(got, want)
    known = mask == 0
    assert np.abs(got[known].astype(int) - img8[known].astype(int)).max() <= 1  # Lab round trip
    for n in range(3):
        assert read_png(tmp_path / ("pyr_%d.png" % n)).shape[2] == 3
    nnf_img = read_png(tmp_path / "nnf.png")
    assert nnf_img.shape == got.shape and (nnf_img == 0).any()


def test_cli_png_inputs_and_channel_rules(cli, gpu_ctx, tmp_path):
    """PNG input and mask files, read with iio's rules: a grey + alpha image
    gives (grey, alpha, grey); a colour mask is reduced to
    0.299 R + 0.587 G + 0.114 B truncated to a byte, so (1, 0, 0) is not a
    hole pixel and (0, 2, 0) is."""
    from nli_gb300 import workloads as wl
    img, mask, _ = wl.config2(seed=9, size=64, scales=3)
    grey = np.clip(np.round(img[..., 0]), 0, 255).astype(np.uint8)
    alpha = np.clip(np.round(img[..., 1]), 0, 255).astype(np.uint8)
    write_png(tmp_path / "in.png", np.stack([grey, alpha], -1))
    cmask = np.zeros(mask.shape + (3,), np.uint8)
    cmask[mask != 0] = (0, 2, 0)
    decoy = (mask == 0) & (np.arange(mask.size).reshape(mask.shape) % 7 == 0)
    cmask[decoy] = (1, 0, 0)
    write_png(tmp_path / "mask.png", cmask)
    r = subprocess.run([cli, "in.png", "mask.png", "out", "-method", "nlmeans", "-patch", "9", "-scales", "3",
                        "-coarse", "0.5", "-iters", "8", "-seed", "3"], cwd=tmp_path, capture_output=True, text=True)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stderr
    got = read_png(tmp_path / "out_nlmeans_sc3_0.5_initpoisson_ps9_10000_conf5_0.1.png")
    rgb = np.stack([grey, alpha, grey], -1).astype(np.float32)
    p = wl.params("nlmeans", distance="l2", patch=9, scales=3, coarse=0.5, iters=8)
    p.patchmatch.random_shots = 30
    lab = gpu_ctx.rgb_to_lab(rgb).cpu().numpy()
    gpu_ctx.set_seed(3)
    out, _ = gpu_ctx.process(lab, (mask != 0).astype(np.uint8), p)
    v = gpu_ctx.lab_to_rgb(out).cpu().numpy().astype(np.float64)
    v = np.where(v >= 0, np.floor(v + 0.5), np.ceil(v - 0.5))
    assert np.array_equal(got, np.clip(v, 0, 255).astype(np.uint8))


def test_cli_errors(cli, tmp_path):
    img = np.full((40, 40, 3), 100.0)
    write_pnm(tmp_path / "in.ppm", img)
    write_pnm(tmp_path / "mask.pgm", np.zeros((40, 40)))
    r = subprocess.run([cli, "in.ppm", "mask.pgm", "out"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode != 0 and "ERROR: Mask should not be empty (all black)" in r.stderr
    write_pnm(tmp_path / "mask2.pgm", np.ones((30, 40)) * 255)
    r = subprocess.run([cli, "in.ppm", "mask2.pgm", "out"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode != 0 and "ERROR: Input image and mask should be of the same size" in r.stderr
    r = subprocess.run([cli, "in.ppm"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 1 and "USAGE" in r.stderr


def test_cli_depth(cli, tmp_path):
    from nli_gb300 import workloads as wl
    img, mask, _ = wl.config3(seed=2, w=80, h=64, scales=3)
    write_pnm(tmp_path / "in.ppm", img[..., :3])
    write_pnm(tmp_path / "mask.pgm", mask * 255)
    d = img[..., 3]
    with open(tmp_path / "depth.pfm", "wb") as f:
        f.write(b"Pf\n%d %d\n-1.0\n" % (d.shape[1], d.shape[0]))
        f.write(np.ascontiguousarray(d[::-1]).astype("<f4").tobytes())
    r = subprocess.run([cli, "in.ppm", "mask.pgm", "out", "-method", "nldepth", "-depth", "depth.pfm", "-lambdar", "1.0",
                        "-lambdad", "0.0", "-patch", "9", "-scales", "3", "-coarse", "0.5", "-iters", "5", "-seed", "1"],
                       cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    with open(tmp_path / "inpainted_depth.pfm", "rb") as f:
        raw = f.read()
    hdr = raw.split(b"\n", 3)
    out_d = np.frombuffer(hdr[3], "<f4").reshape(d.shape)[::-1]
    known = mask == 0
    assert np.array_equal(out_d[known], d[known])  # known depth untouched
    assert np.isfinite(out_d).all() and (out_d[~known] > 0.3).all()
    dpng = read_png(tmp_path / "inpainted_depth.png")
    want = np.clip(np.floor(out_d.astype(np.float64) + 0.5), 0, 255).astype(np.uint8)
    assert np.array_equal(dpng, np.repeat(want[..., None], 3, -1))
