"""Lockstep batches (NLI_TUNE_BATCH_MODE 1, the default): the images of a
batch walk their pyramids together, one launch per kernel per pyramid rank
covering every image, each rank's iteration loop one CUDA graph, and the
sub-groups of a group running concurrently on worker contexts.  Every
image must equal its plain nli_process run with the per-image seed bit for
bit -- output and statistics -- whatever the mix of sizes, methods, channel
counts and parameters (images that cannot share launches form separate
groups), with the graph or the host loop, and beyond 64 images."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STAT_KEYS = ("scales", "width", "height", "iterations", "last_difference", "patchmatch_calls", "update_calls",
             "cg_iterations", "candidates", "candidates_partial", "targets", "holes")


def mixed_batch(seed=21, count=8):
    """Uneven sizes (40-110 px), RGB NL-means / NL-Poisson with 2-4 scales,
    plus NL-medians (L1 distance) and RGB-D NL-depth images."""
    from nli_gb300 import workloads as wl
    rng = np.random.default_rng(seed)
    items, params = [], []
    for i in range(count):
        side = float(np.exp(rng.uniform(np.log(40), np.log(110))))
        aspect = float(np.exp(rng.uniform(np.log(0.6), np.log(1.7))))
        w, h = max(36, int(round(side * aspect ** 0.5))), max(36, int(round(side / aspect ** 0.5)))
        img, _ = wl.voronoi_texture(w, h, int(rng.integers(6, 16)), rng)
        mask = wl.ellipse_mask(w, h, 2, float(rng.uniform(0.06, 0.15)), rng)
        method = "nlmeans" if i % 2 == 0 else "nlpoisson"
        scales = 2 + i % 3
        items.append((img, mask))
        params.append(wl.params(method, scales=scales, coarse=0.5, iters=12, cg_tol=1e-4))
    for j in range(2):
        img, _ = wl.voronoi_texture(56 + 8 * j, 48, 8, rng)
        mask = wl.ellipse_mask(56 + 8 * j, 48, 2, 0.1, rng)
        items.append((img, mask))
        params.append(wl.params("nlmedians", scales=2, coarse=0.5, iters=8))
    for j in range(2):
        rgb, _ = wl.voronoi_texture(64, 52 + 6 * j, 8, rng)
        depth = wl.depth_planes(64, 52 + 6 * j, 4, rng)
        img = np.concatenate([rgb, depth[..., None]], -1).astype(np.float32)
        mask = wl.stroke_mask(64, 52 + 6 * j, 3, (4, 8), rng, coverage=0.1)
        items.append((img, mask))
        params.append(wl.params("nldepth", scales=2, coarse=0.5, lam_r=1.0, lam_d=0.0, iters=8))
    return items, params


def plain(ctx, items, params, seed):
    outs, stats = [], []
    for i, ((img, mask), p) in enumerate(zip(items, params)):
        ctx.set_seed(ctx.batch_seed(seed, i))
        o, st = ctx.process(img, mask, p)
        outs.append(o)
        stats.append(st)
    return outs, stats


def lockstep(ctx, items, params, seed):
    ctx.set_seed(seed)
    ctx.set_tuning(ctx.TUNE_BATCH_MODE, 1)
    return ctx.process_batch(items, params)


def same_stats(a, b):
    for k in STAT_KEYS:
        assert a[k] == b[k], (k, a[k], b[k])


def test_lockstep_equals_plain_mixed(gpu_ctx):
    items, params = mixed_batch()
    want, wst = plain(gpu_ctx, items, params, 99)
    got, gst = lockstep(gpu_ctx, items, params, 99)
    for i in range(len(items)):
        assert np.array_equal(got[i], want[i]), i
        same_stats(gst[i], wst[i])
        # rank loops ran in graphs past the first iteration
        assert gst[i]["graph_iterations"] == sum(max(it - 1, 0) for it in gst[i]["iterations"][:gst[i]["scales"]])


def test_lockstep_host_loop_and_profiling(gpu_ctx):
    """The host loop (graph off, or per-kernel profiling on) gives the
    graph's results."""
    items, params = mixed_batch(seed=22, count=4)
    ref, rst = lockstep(gpu_ctx, items, params, 5)
    gpu_ctx.set_tuning(gpu_ctx.TUNE_GRAPH_LOOP, 0)
    try:
        got, gst = lockstep(gpu_ctx, items, params, 5)
    finally:
        gpu_ctx.set_tuning(gpu_ctx.TUNE_GRAPH_LOOP, 1)
    gpu_ctx.set_profiling(True)
    try:
        got2, _ = lockstep(gpu_ctx, items, params, 5)
        prof = gpu_ctx.profile()
    finally:
        gpu_ctx.set_profiling(False)
    for i in range(len(items)):
        assert np.array_equal(got[i], ref[i]) and np.array_equal(got2[i], ref[i]), i
        assert gst[i]["graph_iterations"] == 0
        for k in ("iterations", "last_difference", "cg_iterations", "candidates"):
            assert gst[i][k] == rst[i][k]
    assert "pm_sweep" in prof and "poisson_cg" in prof and "nlmeans" in prof


def test_lockstep_more_than_64_images(gpu_ctx):
    """Groups hold at most 64 images; a larger batch runs as several."""
    from nli_gb300 import workloads as wl
    rng = np.random.default_rng(3)
    items, params = [], []
    for i in range(70):
        w, h = int(rng.integers(36, 48)), int(rng.integers(36, 48))
        img, _ = wl.voronoi_texture(w, h, 5, rng)
        items.append((img, wl.disc_mask(w, h, 5 + i % 3)))
        params.append(wl.params("nlmeans" if i % 2 else "nlpoisson", scales=2, coarse=0.6, iters=3, cg_tol=1e-4))
    want, wst = plain(gpu_ctx, items, params, 12)
    got, gst = lockstep(gpu_ctx, items, params, 12)
    for i in range(len(items)):
        assert np.array_equal(got[i], want[i]), i
        same_stats(gst[i], wst[i])


def test_lockstep_iteration_edge_cases(gpu_ctx):
    """No iterations at all, and a tolerance that stops every scale after
    its first iteration, next to ordinary images."""
    items, params = mixed_batch(seed=23, count=4)
    params[0].iterations = 0
    params[1].tolerance = 1e30
    want, wst = plain(gpu_ctx, items, params, 8)
    got, gst = lockstep(gpu_ctx, items, params, 8)
    for i in range(len(items)):
        assert np.array_equal(got[i], want[i]), i
        same_stats(gst[i], wst[i])
    assert all(it == 0 for it in gst[0]["iterations"][:gst[0]["scales"]])
    assert all(it == 1 for it in gst[1]["iterations"][:gst[1]["scales"]])


def test_lockstep_device_buffers(gpu_ctx):
    items, params = mixed_batch(seed=24, count=4)
    want, _ = plain(gpu_ctx, items, params, 31)
    gpu_ctx.set_seed(31)
    got, _ = gpu_ctx.process_batch_device(items, params)
    for i in range(len(items)):
        assert np.array_equal(got[i].cpu().numpy(), want[i]), i


def test_lockstep_worker_mode_agrees(gpu_ctx):
    """The worker-context form (NLI_TUNE_BATCH_MODE 0) gives the same
    images."""
    items, params = mixed_batch(seed=25, count=4)
    ref, _ = lockstep(gpu_ctx, items, params, 17)
    gpu_ctx.set_tuning(gpu_ctx.TUNE_BATCH_MODE, 0)
    try:
        gpu_ctx.set_seed(17)
        got, _ = gpu_ctx.process_batch(items, params)
    finally:
        gpu_ctx.set_tuning(gpu_ctx.TUNE_BATCH_MODE, 1)
    for i in range(len(items)):
        assert np.array_equal(got[i], ref[i]), i


@pytest.mark.parametrize("single_max", [0, 4096])
def test_single_cta_cg_threshold(gpu_ctx, single_max):
    """Moving the one-CTA / cluster boundary of the CG changes only the
    rounding of its sums; plain and lockstep still agree bit for bit."""
    items, params = mixed_batch(seed=26, count=4)
    gpu_ctx.set_tuning(gpu_ctx.TUNE_CG_SINGLE_MAX, single_max)
    try:
        want, _ = plain(gpu_ctx, items, params, 44)
        got, _ = lockstep(gpu_ctx, items, params, 44)
    finally:
        gpu_ctx.set_tuning(gpu_ctx.TUNE_CG_SINGLE_MAX, 1024)
    for i in range(len(items)):
        assert np.array_equal(got[i], want[i]), i


@pytest.mark.parametrize("groups", [1, 3, 16])
def test_lockstep_concurrent_groups(gpu_ctx, groups):
    """Sub-groups of one launch-sharing group run concurrently on worker
    contexts (NLI_TUNE_BATCH_GROUPS); every image still equals its plain
    run, with host and with device buffers, and the per-image statistics
    and the context's counters are those of the plain runs."""
    items, params = mixed_batch(seed=27, count=8)
    want, wst = plain(gpu_ctx, items, params, 61)
    gpu_ctx.set_tuning(gpu_ctx.TUNE_BATCH_GROUPS, groups)
    try:
        got, gst = lockstep(gpu_ctx, items, params, 61)
        gpu_ctx.set_seed(61)
        dev, _ = gpu_ctx.process_batch_device(items, params)
    finally:
        gpu_ctx.set_tuning(gpu_ctx.TUNE_BATCH_GROUPS, 4)
    for i in range(len(items)):
        assert np.array_equal(got[i], want[i]), i
        assert np.array_equal(dev[i].cpu().numpy(), want[i]), i
        same_stats(gst[i], wst[i])
