"""Seeded synthetic inputs with the shapes and value ranges of the benchmark
configurations (the reference ships no dataset; its README example images
cannot be decoded here).  All generators use ``numpy.random.default_rng``.

Images are float32 HWC in [0, 255] (depth channel in metres), masks uint8
(1 = hole, the inpainting domain).
"""
from __future__ import annotations

import math

import numpy as np

from . import _abi


def _grid(w, h):
    y, x = np.mgrid[0:h, 0:w].astype(np.float32)
    return x, y


def smooth_stripes(w, h, rng, period=12.0, noise=3.0):
    """Smooth colour gradient + sinusoidal stripes of the given period with a
    random orientation + Gaussian noise."""
    x, y = _grid(w, h)
    img = np.empty((h, w, 3), np.float32)
    theta = rng.uniform(0, math.pi)
    phase = x * math.cos(theta) + y * math.sin(theta)
    stripes = np.sin(2 * math.pi * phase / period)
    for c in range(3):
        a, b, c0 = rng.uniform(-0.4, 0.4, size=3)
        base = 128 + 60 * (a * x / w + b * y / h) * 2 + 20 * c0
        img[..., c] = base + rng.uniform(25, 45) * stripes
    img += rng.normal(0, noise, size=img.shape).astype(np.float32)
    return np.clip(img, 0, 255).astype(np.float32)


def voronoi_texture(w, h, seeds, rng):
    """Piecewise-smooth image: Voronoi cells with a uniform random colour in
    [0,255] and a per-cell oriented sinusoid."""
    sx = rng.uniform(0, w, seeds)
    sy = rng.uniform(0, h, seeds)
    x, y = _grid(w, h)
    d = (x[..., None] - sx) ** 2 + (y[..., None] - sy) ** 2
    label = np.argmin(d, axis=-1)
    colour = rng.uniform(0, 255, size=(seeds, 3)).astype(np.float32)
    theta = rng.uniform(0, math.pi, seeds)
    period = rng.uniform(6, 20, seeds)
    amp = rng.uniform(8, 30, seeds)
    ph = x * np.cos(theta)[label] + y * np.sin(theta)[label]
    tex = amp[label] * np.sin(2 * math.pi * ph / period[label])
    img = colour[label] + tex[..., None]
    return np.clip(img, 0, 255).astype(np.float32), label


def disc_mask(w, h, r):
    x, y = _grid(w, h)
    return (((x - (w - 1) / 2) ** 2 + (y - (h - 1) / 2) ** 2) <= r * r).astype(np.uint8)


def ellipse_mask(w, h, count, coverage, rng, margin=0.08):
    """Union of `count` random ellipses scaled to cover about `coverage` of the
    pixels, kept `margin` (fraction of the side) away from the border."""
    x, y = _grid(w, h)
    cx = rng.uniform(margin * w, (1 - margin) * w, count)
    cy = rng.uniform(margin * h, (1 - margin) * h, count)
    ax = rng.uniform(0.5, 1.5, count)
    ay = rng.uniform(0.5, 1.5, count)
    th = rng.uniform(0, math.pi, count)

    def mask_for(s):
        m = np.zeros((h, w), bool)
        for i in range(count):
            dx, dy = x - cx[i], y - cy[i]
            u = dx * math.cos(th[i]) + dy * math.sin(th[i])
            v = -dx * math.sin(th[i]) + dy * math.cos(th[i])
            m |= (u / (s * ax[i])) ** 2 + (v / (s * ay[i])) ** 2 <= 1
        return m

    lo, hi = 1.0, 0.5 * max(w, h)
    for _ in range(30):
        mid = 0.5 * (lo + hi)
        if mask_for(mid).mean() < coverage:
            lo = mid
        else:
            hi = mid
    return mask_for(0.5 * (lo + hi)).astype(np.uint8)


def stroke_mask(w, h, strokes, width_range, rng, coverage=None, margin=0.05):
    """Random brush strokes (polylines of discs) with widths in width_range;
    if `coverage` is given, strokes are lengthened until it is reached."""
    x, y = _grid(w, h)
    m = np.zeros((h, w), bool)
    segs = []
    for _ in range(strokes):
        px = rng.uniform(margin * w, (1 - margin) * w)
        py = rng.uniform(margin * h, (1 - margin) * h)
        ang = rng.uniform(0, 2 * math.pi)
        r = rng.uniform(*width_range) / 2
        segs.append([px, py, ang, r])
    step = 4.0
    for _ in range(400):
        for s in segs:
            s[2] += rng.normal(0, 0.25)
            nx = min(max(s[0] + step * math.cos(s[2]), margin * w), (1 - margin) * w)
            ny = min(max(s[1] + step * math.sin(s[1] * 0 + s[2]), margin * h), (1 - margin) * h)
            s[0], s[1] = nx, ny
            x0, x1 = int(max(nx - s[3] - 1, 0)), int(min(nx + s[3] + 2, w))
            y0, y1 = int(max(ny - s[3] - 1, 0)), int(min(ny + s[3] + 2, h))
            m[y0:y1, x0:x1] |= (x[y0:y1, x0:x1] - nx) ** 2 + (y[y0:y1, x0:x1] - ny) ** 2 <= s[3] ** 2
        if coverage is not None and m.mean() >= coverage:
            break
    return m.astype(np.uint8)


def depth_planes(w, h, label_count, rng, noise=0.01):
    """Depth map of 3-8 seeded random planes, values in [0.5, 5.0] m, plus
    Gaussian noise."""
    n = int(rng.integers(3, 9))
    x, y = _grid(w, h)
    sx = rng.uniform(0, w, n)
    sy = rng.uniform(0, h, n)
    lab = np.argmin((x[..., None] - sx) ** 2 + (y[..., None] - sy) ** 2, axis=-1)
    d0 = rng.uniform(0.8, 4.5, n)
    gx = rng.uniform(-1.5, 1.5, n) / w
    gy = rng.uniform(-1.5, 1.5, n) / h
    d = d0[lab] + gx[lab] * (x - w / 2) + gy[lab] * (y - h / 2)
    d = np.clip(d, 0.5, 5.0) + rng.normal(0, noise, size=d.shape)
    return d.astype(np.float32)


def params(method="nlmeans", distance=None, patch=9, psigma=10000.0, lam=0.05, lam_r=0.05, lam_d=0.05,
           cg_tol=1e-6, cg_iters=1000, iters=200, tol=0.1, scales=5, coarse=0.1, conft=5.0, confa=0.1,
           init="poisson", pm_iters=10, shots=30, window=-1):
    """nli_process_params wired as the reference CLI wires them
    (main.cpp:217-270); `distance` defaults to the CLI pairing except that
    nlmeans pairs with L2Combined (the configuration of the benchmarks)."""
    m = {"nlmeans": _abi.NLI_UPDATE_MEANS, "nlmedians": _abi.NLI_UPDATE_MEDIANS,
         "nlpoisson": _abi.NLI_UPDATE_POISSON, "nldepth": _abi.NLI_UPDATE_DEPTH}[method]
    if distance is None:
        distance = {"nlmeans": "l2combined", "nlmedians": "l1", "nlpoisson": "l2combined",
                    "nldepth": "l2rgbd"}[method]
    k = {"l2combined": _abi.NLI_DIST_L2_COMBINED, "l2rgbd": _abi.NLI_DIST_L2_RGBD,
         "l2": _abi.NLI_DIST_L2_NORM, "l1": _abi.NLI_DIST_L1_NORM}[distance]
    ini = {"black": 0, "avg": 1, "none": 2, "poisson": 3}[init]
    p = _abi.ProcessParams()
    p.distance.kind = k
    p.distance.patch_x = p.distance.patch_y = patch
    p.distance.sigma = psigma
    p.distance.lambda_ = lam_r if method == "nldepth" else lam
    p.distance.lambda_d = lam_d
    p.patchmatch.iterations = pm_iters
    p.patchmatch.random_shots = shots
    p.patchmatch.window = window
    p.update.method = m
    p.update.patch_x = p.update.patch_y = patch
    p.update.sigma = psigma
    p.update.lambda_ = lam_r if method == "nldepth" else lam
    p.update.lambda_d = lam_d
    p.update.cg_tol = cg_tol
    p.update.cg_iters = cg_iters
    p.iterations = iters
    p.tolerance = tol
    p.scales = scales
    p.subsampling_rate = _abi.subsampling_rate(coarse, scales) if scales > 1 else 0.5
    p.conf_decay_time = conft
    p.conf_asymptotic = confa
    p.init = ini
    return p


def config1(seed=0, size=256):
    """256x256 RGB smooth gradient + stripes (period 12) + noise sigma 3,
    centred disc of radius 32 (scaled with `size`); nlmeans + L2Combined,
    lambda 0.05, psigma 10000, patch 9, scales 5, coarse 0.1, iters 200,
    conft 5, confa 0.1, init poisson."""
    rng = np.random.default_rng(seed)
    img = smooth_stripes(size, size, rng)
    mask = disc_mask(size, size, 32 * size / 256)
    return img, mask, params("nlmeans", scales=5, coarse=0.1, iters=200)


def config2(seed=0, size=512, scales=8, iters=200):
    """512x512 Voronoi (40 seeds) + oriented sinusoids, union of 6 ellipses
    (~15%); nlpoisson + L2Combined, lambda 0.05, patch 9, scales 8,
    CG tolerance 1e-4; other parameters at the CLI defaults."""
    rng = np.random.default_rng(seed)
    img, _ = voronoi_texture(size, size, 40, rng)
    mask = ellipse_mask(size, size, 6, 0.15, rng)
    return img, mask, params("nlpoisson", scales=scales, coarse=0.1, cg_tol=1e-4, iters=iters)


def config3(seed=0, w=640, h=480, scales=9, iters=200):
    """640x480 Voronoi (60 seeds) RGB + depth of 3-8 planes in [0.5,5] m with
    noise 0.01; 10 brush strokes of width 8-24 px (~12%); nldepth + L2RGBD,
    lambda_rgb 1.0, lambda_d 0.0, patch 9, scales 9."""
    rng = np.random.default_rng(seed)
    rgb, _ = voronoi_texture(w, h, 60, rng)
    depth = depth_planes(w, h, 60, rng)
    img = np.concatenate([rgb, depth[..., None]], axis=-1).astype(np.float32)
    mask = stroke_mask(w, h, 10, (8, 24), rng, coverage=0.12)
    return img, mask, params("nldepth", scales=scales, coarse=0.1, lam_r=1.0, lam_d=0.0, iters=iters)


def config5(seed=0, count=64, min_side=128, max_side=1024):
    """Uneven batch: `count` pairs, side log-uniform in [min_side, max_side],
    aspect 0.5-2, holes 5-30% (ellipses + strokes), mixed nlmeans/nlpoisson,
    patch 9, scales = |round(log(size*0.1)/log(0.75))|, coarse 0 (the
    automatic rule of main.cpp:166-177 is applied by the caller)."""
    rng = np.random.default_rng(seed)
    items = []
    for i in range(count):
        side = math.exp(rng.uniform(math.log(min_side), math.log(max_side)))
        aspect = math.exp(rng.uniform(math.log(0.5), math.log(2.0)))
        w = max(32, int(round(side * math.sqrt(aspect))))
        h = max(32, int(round(side / math.sqrt(aspect))))
        w, h = min(w, max_side), min(h, max_side)
        img, _ = voronoi_texture(w, h, int(rng.integers(20, 60)), rng)
        cov = rng.uniform(0.05, 0.30)
        if rng.uniform() < 0.5:
            mask = ellipse_mask(w, h, int(rng.integers(2, 7)), cov, rng)
        else:
            mask = stroke_mask(w, h, int(rng.integers(4, 12)), (8, 24), rng, coverage=cov)
        method = "nlmeans" if i % 2 == 0 else "nlpoisson"
        scales = abs(int(round(math.log(min(w, h) * 0.1) / math.log(0.75))))
        items.append((img, mask, method, max(scales, 1)))
    return items


def coarsest_rate_auto(mask, patch=9):
    """The CLI's rule for -coarse 0 (main.cpp:166-177): coarsest rate =
    min(1.5 * patch / max distance to the hole boundary, 1), in float."""
    from scipy.ndimage import distance_transform_edt
    d = distance_transform_edt(np.asarray(mask) != 0)
    max_dist = np.float32(d.max()) if d.size else np.float32(0)
    if max_dist <= 0:
        return 1.0
    r = np.float32(1.5) * np.float32(patch) / max_dist
    return float(min(r, np.float32(1.0)))


def config5_params(mask, method, scales, iters=200):
    """Parameters of one batch item: the CLI defaults for `method`, the
    automatic coarsest rate, and one scale when that rate is 1 (main.cpp:199-202)."""
    coarse = coarsest_rate_auto(mask)
    if abs(coarse - 1.0) < 1e-5:
        scales = 1
    return params(method, scales=scales, coarse=coarse, iters=iters)

