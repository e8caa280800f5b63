"""The vectorised FP64 evaluation of tests/update64.py (Plan, means_fast,
poisson_fast), used for the full-size finite differences, against its
reference form (the autograd-capable expressions) on small seeded cases:
NL-means, NL-Poisson and NL-depth (per-channel lambda), at two sigmas.
CPU only."""
import numpy as np
import pytest
import torch

import update64


def case(seed, H=40, W=44, C=3):
    from nli_gb300 import workloads as wl
    from scipy.ndimage import binary_dilation
    rng = np.random.default_rng(seed)
    img, _ = wl.voronoi_texture(W, H, 6, rng)
    if C == 4:
        img = np.concatenate([img, rng.uniform(0.5, 5, (H, W, 1)).astype(np.float32)], -1)
    dom = wl.ellipse_mask(W, H, 2, 0.15, rng) != 0
    ext = binary_dilation(dom, iterations=4)
    nnf = np.stack([rng.integers(4, W - 5, (H, W)), rng.integers(4, H - 5, (H, W))], -1).astype(np.int64)
    nnf[rng.uniform(size=(H, W)) < 0.1] = -1
    conf = rng.uniform(0.1, 1.0, (H, W))
    u = img.astype(np.float64) + rng.normal(0, 2, img.shape)
    return u, nnf, dom, ext, conf


@pytest.mark.parametrize("sigma", [10000.0, 2.5])
def test_means_fast(sigma):
    u, nnf, dom, ext, conf = case(1)
    plan = update64.Plan(nnf, dom, ext, conf)
    ref = update64.means(torch.from_numpy(u), sigma, nnf, dom, conf).numpy()
    got = update64.means_fast(u, sigma, plan)
    assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()


@pytest.mark.parametrize("sigma", [10000.0, 2.5])
def test_poisson_fast(sigma):
    u, nnf, dom, ext, conf = case(2)
    plan = update64.Plan(nnf, dom, ext, conf)
    ref = update64.poisson(torch.from_numpy(u), 0.05, sigma, nnf, dom, ext, conf).numpy()
    got = update64.poisson_fast(u, 0.05, sigma, plan)
    assert np.abs(got - ref).max() <= 1e-8 * np.abs(ref).max()


def test_depth_fast():
    u, nnf, dom, ext, conf = case(3, C=4)
    plan = update64.Plan(nnf, dom, ext, conf)
    lams = [0.3, 0.3, 0.3, 0.6]
    ref = update64.poisson(torch.from_numpy(u), None, 3.0, nnf, dom, ext, conf, lam_channels=lams).numpy()
    got = update64.poisson_fast(u, None, 3.0, plan, lam_channels=lams)
    assert np.abs(got - ref).max() <= 1e-8 * np.abs(ref).max()
