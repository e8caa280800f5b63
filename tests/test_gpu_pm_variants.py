"""The three ways the 9x9 PatchMatch kernels read a candidate's windows --
target window in shared memory with plain source loads (the default),
source windows staged into shared memory by tensor copies
(cp.async.bulk.tensor), target window in registers -- give bit-identical
fields: the same candidates in the same order, the same float arithmetic.  Every distance kind and
channel count with a 9x9 kernel, the init kernel alone (0 sweeps), sources
smaller and larger than the target, and whole multiscale runs."""
import numpy as np
import pytest

from nli_gb300 import _abi

pytestmark = pytest.mark.gpu

CASES = [(_abi.NLI_DIST_L2_COMBINED, 3), (_abi.NLI_DIST_L2_COMBINED, 1), (_abi.NLI_DIST_L2_COMBINED, 2),
         (_abi.NLI_DIST_L2_COMBINED, 4), (_abi.NLI_DIST_L2_RGBD, 4), (_abi.NLI_DIST_L2_NORM, 3),
         (_abi.NLI_DIST_L2_NORM, 2), (_abi.NLI_DIST_L1_NORM, 1), (_abi.NLI_DIST_L1_NORM, 4)]


def npy(t):
    return t.cpu().numpy() if hasattr(t, "cpu") else np.asarray(t)


def scene(C, seed, w, h, r):
    from nli_gb300 import workloads as wl
    rng = np.random.default_rng(seed)
    img, _ = wl.voronoi_texture(w, h, 9, rng)
    if C == 4:
        img = np.concatenate([img, rng.uniform(0.5, 5, (h, w, 1)).astype(np.float32)], -1)
    elif C < 3:
        img = np.ascontiguousarray(img[..., :C])
    return img, wl.disc_mask(w, h, r)


VARIANTS = (0, 1, 2)


def run_all(ctx, fn):
    out = []
    for v in VARIANTS:
        ctx.set_tuning(ctx.TUNE_PM_VARIANT, v)
        try:
            out.append(fn())
        finally:
            ctx.set_tuning(ctx.TUNE_PM_VARIANT, 0)
    return out


@pytest.mark.parametrize("iters", [0, 1, 6])
@pytest.mark.parametrize("kind,C", CASES)
def test_staged_equals_plain(gpu_ctx, kind, C, iters):
    img, mask = scene(C, 10 * kind + C, 120, 96, 14)
    d = _abi.DistanceParams()
    d.kind, d.patch_x, d.patch_y, d.sigma, d.lambda_, d.lambda_d = kind, 9, 9, 3.0, 0.4, 0.3
    pm = _abi.PatchMatchParams(iters, 30, -1)
    ext = npy(gpu_ctx.extended_domain(mask, 9, 9))
    s, t, _ = gpu_ctx.scale_masks(ext, 4, True)
    s, t = npy(s), npy(t)

    def one():
        gpu_ctx.set_seed(77)
        nnf, dist, e = gpu_ctx.patchmatch(d, pm, img, s, img, t)
        return npy(nnf), npy(dist), e
    (n0, d0, e0), *rest = run_all(gpu_ctx, one)
    for v, (n1, d1, e1) in zip(VARIANTS[1:], rest):
        assert np.array_equal(n1, n0), v
        assert np.array_equal(d1, d0), v
        assert e1 == e0, v


@pytest.mark.parametrize("sw,sh", [(64, 48), (200, 150)])
def test_staged_other_source_sizes(gpu_ctx, sw, sh):
    """Source and target of different sizes (the tensor map spans the padded
    source, the windows are read from the source only)."""
    from nli_gb300 import workloads as wl
    rng = np.random.default_rng(sw)
    src, _ = wl.voronoi_texture(sw, sh, 9, rng)
    tgt, _ = wl.voronoi_texture(100, 90, 9, rng)
    smask = np.zeros((sh, sw), np.uint8)
    smask[4:sh - 5, 4:sw - 5] = 1
    tmask = np.zeros((90, 100), np.uint8)
    tmask[20:70, 15:85] = 1
    d = _abi.DistanceParams()
    d.kind, d.patch_x, d.patch_y, d.sigma, d.lambda_, d.lambda_d = _abi.NLI_DIST_L2_COMBINED, 9, 9, 3.0, 0.4, 0.3
    pm = _abi.PatchMatchParams(5, 20, -1)

    def one():
        gpu_ctx.set_seed(5)
        nnf, dist, _ = gpu_ctx.patchmatch(d, pm, src, smask, tgt, tmask)
        return npy(nnf), npy(dist)
    (n0, d0), *rest = run_all(gpu_ctx, one)
    for v, (n1, d1) in zip(VARIANTS[1:], rest):
        assert np.array_equal(n1, n0) and np.array_equal(d1, d0), v
    m = tmask.astype(bool)
    assert (smask[n0[m][:, 1], n0[m][:, 0]] == 1).all()


@pytest.mark.parametrize("method", ["nlpoisson", "nlmeans"])
def test_staged_process(gpu_ctx, method):
    from nli_gb300 import workloads as wl
    img, mask, _ = wl.config2(seed=3, size=256, scales=3)
    p = wl.params(method, scales=3, iters=8, cg_tol=1e-4)

    def one():
        gpu_ctx.set_seed(11)
        return gpu_ctx.process(img, mask, p)[0]
    a, *rest = run_all(gpu_ctx, one)
    for v, b in zip(VARIANTS[1:], rest):
        assert np.array_equal(a, b), v


def test_variant_knob(gpu_ctx):
    assert gpu_ctx.get_tuning(gpu_ctx.TUNE_PM_VARIANT) == 0
    with pytest.raises(Exception):
        gpu_ctx.set_tuning(gpu_ctx.TUNE_PM_VARIANT, 3)
    assert gpu_ctx.get_tuning(gpu_ctx.TUNE_PM_VARIANT) == 0
