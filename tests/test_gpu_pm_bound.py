"""The lower bounds of PatchMatch (NLI_TUNE_PM_BOUND): a candidate whose
weighted patch means (1, the default), or means and standard deviations
(2), differ enough from the target's is not evaluated, because it
provably cannot beat the current match.  The bounds keep a rounding
margin, so the fields and distances must be bit for bit those of
evaluating every candidate -- for every distance kind and channel count,
patch sizes with and without compiled rows, separate source and target
images, other patch weights, and whole runs (plain and batched) -- while
fewer candidates are evaluated, and fewer with the deviations than with
the means alone."""
import numpy as np
import pytest

from nli_gb300 import _abi

pytestmark = pytest.mark.gpu

CASES = [(_abi.NLI_DIST_L2_COMBINED, 3, 9), (_abi.NLI_DIST_L2_COMBINED, 1, 9), (_abi.NLI_DIST_L2_COMBINED, 4, 7),
         (_abi.NLI_DIST_L2_RGBD, 4, 9), (_abi.NLI_DIST_L2_NORM, 3, 9), (_abi.NLI_DIST_L2_NORM, 2, 5),
         (_abi.NLI_DIST_L1_NORM, 3, 9), (_abi.NLI_DIST_L1_NORM, 1, 7)]


def npy(t):
    return t.cpu().numpy() if hasattr(t, "cpu") else np.asarray(t)


def scene(C, seed, w, h, r):
    from nli_gb300 import workloads as wl
    rng = np.random.default_rng(seed)
    img, _ = wl.voronoi_texture(w, h, 12, rng)
    if C == 4:
        img = np.concatenate([img, rng.uniform(0.5, 5, (h, w, 1)).astype(np.float32)], -1)
    elif C < 3:
        img = np.ascontiguousarray(img[..., :C])
    return img, wl.disc_mask(w, h, r)


def both(ctx, fn):
    """(result, candidates evaluated) with the bound off, by means, by
    means and deviations."""
    out = []
    for b in (0, 1, 2):
        ctx.set_tuning(ctx.TUNE_PM_BOUND, b)
        try:
            c0 = ctx.counters()["candidates"]
            r = fn()
            out.append((r, ctx.counters()["candidates"] - c0))
        finally:
            ctx.set_tuning(ctx.TUNE_PM_BOUND, 1)
    return out


@pytest.mark.parametrize("sigma", [10000.0, 2.5])
@pytest.mark.parametrize("kind,C,P", CASES)
def test_bound_keeps_fields(gpu_ctx, kind, C, P, sigma):
    img, mask = scene(C, 7 * kind + C + P, 140, 110, 16)
    d = _abi.DistanceParams(kind, P, P, sigma, 0.3, 0.6)
    pm = _abi.PatchMatchParams(6, 30, -1)
    ext = npy(gpu_ctx.extended_domain(mask, P, P))
    s, t, _ = gpu_ctx.scale_masks(ext, P // 2, True)

    def one():
        gpu_ctx.set_seed(17)
        nnf, dist, e = gpu_ctx.patchmatch(d, pm, img, s, img, t)
        gpu_ctx.set_seed(18)
        nnf2, dist2, _ = gpu_ctx.patchmatch(d, pm, img, s, img, t, init=nnf)  # a warm start, as the driver's
        return npy(nnf), npy(dist), e, npy(nnf2), npy(dist2)

    (off, n_off), (on, n_on), (dv, n_dv) = both(gpu_ctx, one)
    for a, b, c in zip(off, on, dv):
        assert np.array_equal(np.asarray(a), np.asarray(b))
        assert np.array_equal(np.asarray(a), np.asarray(c))
    assert n_dv <= n_on <= n_off


def test_bound_separate_source_and_target(gpu_ctx):
    from nli_gb300 import workloads as wl
    rng = np.random.default_rng(4)
    src, _ = wl.voronoi_texture(130, 100, 10, rng)
    tgt, _ = wl.voronoi_texture(90, 120, 10, rng)
    tgt *= 0.5  # different value ranges: the slack follows the larger
    d = _abi.DistanceParams(_abi.NLI_DIST_L2_COMBINED, 9, 9, 10000.0, 0.05, 0.0)
    pm = _abi.PatchMatchParams(5, 30, -1)
    smask = np.zeros((100, 130), np.uint8)
    smask[4:-4, 4:-4] = 1
    tmask = np.zeros((120, 90), np.uint8)
    tmask[4:-4, 4:-4] = 1

    def one():
        gpu_ctx.set_seed(3)
        nnf, dist, e = gpu_ctx.patchmatch(d, pm, src, smask, tgt, tmask)
        return npy(nnf), npy(dist), e

    (off, n_off), (on, n_on), (dv, n_dv) = both(gpu_ctx, one)
    for a, b, c in zip(off, on, dv):
        assert np.array_equal(np.asarray(a), np.asarray(b))
        assert np.array_equal(np.asarray(a), np.asarray(c))
    assert n_dv <= n_on < n_off


def test_bound_whole_runs(gpu_ctx):
    """Whole multiscale runs, plain and lockstep-batched: identical outputs
    and statistics other than the candidate counts, which drop."""
    from test_gpu_lockstep import mixed_batch
    items, params = mixed_batch(seed=51, count=4)

    def runs():
        outs = []
        for i, ((img, mask), p) in enumerate(zip(items, params)):
            gpu_ctx.set_seed(gpu_ctx.batch_seed(8, i))
            outs.append(gpu_ctx.process(img, mask, p))
        gpu_ctx.set_seed(8)
        outs.append(gpu_ctx.process_batch(items, params))
        return outs

    (off, n_off), (on, n_on), (dv, n_dv) = both(gpu_ctx, runs)
    for other in (on, dv):
        for (o1, s1), (o2, s2) in zip(off[:-1], other[:-1]):
            assert np.array_equal(o1, o2)
            assert s1["iterations"] == s2["iterations"] and s1["last_difference"] == s2["last_difference"]
        for o1, o2 in zip(off[-1][0], other[-1][0]):
            assert np.array_equal(o1, o2)
    assert n_dv < n_on < n_off
    print("candidates evaluated: %d without a bound, %d with the means (%.1f %%), %d with means and deviations "
          "(%.1f %%)" % (n_off, n_on, 100.0 * n_on / n_off, n_dv, 100.0 * n_dv / n_off))
