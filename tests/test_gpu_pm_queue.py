"""The device work queue of the persistent PatchMatch kernels
(NLI_TUNE_PM_TILE): warps take n consecutive target points per atomic grab
instead of static block ranges.  Every point's computation is independent
of which warp does it and when, so the fields, distances, energies and
candidate counts must be bit for bit those of the static ranges -- for
every tile, every window variant of the 9x9 kernels, runtime-sized
patches, tiles larger than the target list, and whole plain and lockstep
runs."""
import numpy as np
import pytest

from nli_gb300 import _abi

pytestmark = pytest.mark.gpu

TILES = (1, 3, 8, 64, 1024)  # 0 (static ranges) is the comparison


def npy(t):
    return t.cpu().numpy() if hasattr(t, "cpu") else np.asarray(t)


def scene(seed, w, h, r, C=3):
    from nli_gb300 import workloads as wl
    rng = np.random.default_rng(seed)
    img, _ = wl.voronoi_texture(w, h, 12, rng)
    if C == 4:
        img = np.concatenate([img, rng.uniform(0.5, 5, (h, w, 1)).astype(np.float32)], -1)
    return img, wl.disc_mask(w, h, r)


def per_tile(ctx, fn, tiles=(0,) + TILES):
    out = {}
    for t in tiles:
        ctx.set_tuning(ctx.TUNE_PM_TILE, t)
        try:
            c0 = ctx.counters()
            r = fn()
            c1 = ctx.counters()
            out[t] = (r, c1["candidates"] - c0["candidates"], c1["candidates_partial"] - c0["candidates_partial"])
        finally:
            ctx.set_tuning(ctx.TUNE_PM_TILE, 1)
    return out


@pytest.mark.parametrize("kind,C,P,variant", [(_abi.NLI_DIST_L2_COMBINED, 3, 9, 0), (_abi.NLI_DIST_L2_COMBINED, 3, 9, 1),
                                              (_abi.NLI_DIST_L2_COMBINED, 3, 9, 2), (_abi.NLI_DIST_L2_RGBD, 4, 9, 0),
                                              (_abi.NLI_DIST_L2_NORM, 3, 7, 0), (_abi.NLI_DIST_L1_NORM, 3, 5, 0)])
def test_queue_keeps_fields(gpu_ctx, kind, C, P, variant):
    img, mask = scene(3 * kind + P, 150, 120, 18, C)
    d = _abi.DistanceParams(kind, P, P, 10000.0, 0.05, 0.4)
    pm = _abi.PatchMatchParams(7, 30, -1)
    ext = npy(gpu_ctx.extended_domain(mask, P, P))
    s, t, _ = gpu_ctx.scale_masks(ext, P // 2, True)

    def one():
        gpu_ctx.set_seed(23)
        nnf, dist, e = gpu_ctx.patchmatch(d, pm, img, s, img, t)
        gpu_ctx.set_seed(24)
        nnf2, dist2, e2 = gpu_ctx.patchmatch(d, pm, img, s, img, t, init=nnf)
        return npy(nnf), npy(dist), e, npy(nnf2), npy(dist2), e2

    gpu_ctx.set_tuning(gpu_ctx.TUNE_PM_VARIANT, variant)
    try:
        res = per_tile(gpu_ctx, one)
    finally:
        gpu_ctx.set_tuning(gpu_ctx.TUNE_PM_VARIANT, 0)
    ref, n_ref, p_ref = res[0]
    assert n_ref > 0
    for tile, (r, n, p) in res.items():
        for a, b in zip(r, ref):
            assert np.array_equal(np.asarray(a), np.asarray(b)), tile
        assert (n, p) == (n_ref, p_ref), tile


def test_queue_whole_runs_plain_and_lockstep(gpu_ctx):
    from nli_gb300 import workloads as wl
    rng = np.random.default_rng(9)
    items, params = [], []
    for i in range(5):
        w, h = int(rng.integers(60, 130)), int(rng.integers(60, 130))
        img, _ = wl.voronoi_texture(w, h, 10, rng)
        items.append((img, wl.ellipse_mask(w, h, 2, 0.12, rng)))
        params.append(wl.params("nlmeans" if i % 2 else "nlpoisson", scales=3, coarse=0.5, iters=6, cg_tol=1e-4))

    def runs():
        plain = []
        for i, ((img, mask), p) in enumerate(zip(items, params)):
            gpu_ctx.set_seed(gpu_ctx.batch_seed(77, i))
            plain.append(gpu_ctx.process(img, mask, p)[0])
        gpu_ctx.set_seed(77)
        batch, _ = gpu_ctx.process_batch(items, params)
        return plain, batch

    res = per_tile(gpu_ctx, runs, tiles=(0, 1, 4, 32))
    (plain0, batch0), _, _ = res[0]
    for i in range(len(items)):
        assert np.array_equal(batch0[i], plain0[i]), i
    for tile, ((plain, batch), _, _) in res.items():
        for i in range(len(items)):
            assert np.array_equal(plain[i], plain0[i]), (tile, i)
            assert np.array_equal(batch[i], plain0[i]), (tile, i)


def test_tile_knob_validates(gpu_ctx):
    from nli_gb300 import NliError
    for bad in (-1, 1025):
        with pytest.raises(NliError):
            gpu_ctx.set_tuning(gpu_ctx.TUNE_PM_TILE, bad)
    gpu_ctx.set_tuning(gpu_ctx.TUNE_PM_TILE, 1024)
    assert gpu_ctx.get_tuning(gpu_ctx.TUNE_PM_TILE) == 1024
    gpu_ctx.set_tuning(gpu_ctx.TUNE_PM_TILE, 1)
