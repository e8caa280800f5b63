"""The captured iteration loop (NLI_TUNE_GRAPH_LOOP = 1, the default):
after the first iteration of a scale, the PatchMatch / update iterations
run as one CUDA graph whose while node evaluates inpaint_internal's
stopping test on the device.  Outputs, per-scale iteration counts, final
differences and counters must equal the host loop's exactly, on every
update method, on both CG layouts (cluster, and the cooperative grid kernel
forced by a cluster cap of 1), with the preconditioned CG, and in batches."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STAT_KEYS = ("scales", "iterations", "last_difference", "patchmatch_calls", "update_calls", "cg_iterations",
             "candidates")


def run(ctx, img, mask, p, graph, seed=5):
    ctx.set_tuning(ctx.TUNE_GRAPH_LOOP, graph)
    try:
        ctx.set_seed(seed)
        l0 = ctx.launch_count()
        out, st = ctx.process(img, mask, p)
        return out, st, ctx.launch_count() - l0
    finally:
        ctx.set_tuning(ctx.TUNE_GRAPH_LOOP, 1)


def same(a, b):
    """a: the graph run, b: the host loop's."""
    out_a, st_a, n_a = a
    out_b, st_b, n_b = b
    assert st_b["graph_iterations"] == 0
    if any(i > 1 for i in st_b["iterations"]):
        # every iteration after a scale's first ran inside the graph
        assert st_a["graph_iterations"] == sum(max(i - 1, 0) for i in st_a["iterations"]), st_a
    assert np.array_equal(out_a, out_b)
    for k in STAT_KEYS:
        assert st_a[k] == st_b[k], (k, st_a[k], st_b[k])
    # the graph adds one launch per iteration it runs: the loop control kernel
    assert n_a == n_b + st_a["graph_iterations"], (n_a, n_b, st_a["graph_iterations"])


@pytest.mark.parametrize("method", ["nlpoisson", "nlmeans", "nlmedians"])
def test_graph_equals_host_loop(gpu_ctx, method):
    from nli_gb300 import workloads as wl
    img, mask, _ = wl.config2(seed=2, size=160, scales=4)
    p = wl.params(method, scales=4, coarse=0.3, iters=12, cg_tol=1e-4)
    same(run(gpu_ctx, img, mask, p, 1), run(gpu_ctx, img, mask, p, 0))


def test_graph_nldepth(gpu_ctx):
    from nli_gb300 import workloads as wl
    img, mask, _ = wl.config3(seed=4, w=80, h=64, scales=3)
    p = wl.params("nldepth", scales=3, coarse=0.5, lam_r=0.5, lam_d=0.2, iters=10)
    same(run(gpu_ctx, img, mask, p, 1), run(gpu_ctx, img, mask, p, 0))


@pytest.mark.parametrize("precond", [0, 1])
def test_graph_grid_cg_layout(gpu_ctx, precond):
    """Cluster cap 1: every level with more than 4096 unknowns per channel
    solves on the cooperative grid kernel, captured in the graph."""
    from nli_gb300 import workloads as wl
    img, mask, _ = wl.config2(seed=4, size=256, scales=3)
    p = wl.params("nlpoisson", scales=3, coarse=0.4, iters=8, cg_tol=1e-4)
    gpu_ctx.set_tuning(gpu_ctx.TUNE_CG_CLUSTER_CAP, 1)
    gpu_ctx.set_tuning(gpu_ctx.TUNE_CG_PRECOND, precond)
    try:
        same(run(gpu_ctx, img, mask, p, 1), run(gpu_ctx, img, mask, p, 0))
    finally:
        gpu_ctx.set_tuning(gpu_ctx.TUNE_CG_CLUSTER_CAP, 16)
        gpu_ctx.set_tuning(gpu_ctx.TUNE_CG_PRECOND, 0)


def test_graph_stops_on_tolerance_and_limit(gpu_ctx):
    """A large tolerance stops after the first iteration (no graph); an
    iteration limit of 2 runs exactly one graph iteration."""
    from nli_gb300 import workloads as wl
    img, mask, _ = wl.config2(seed=3, size=128, scales=2)
    for tol, iters in ((1e30, 50), (0.0, 2), (0.0, 1)):
        p = wl.params("nlmeans", scales=2, coarse=0.5, iters=iters, tol=tol)
        a, b = run(gpu_ctx, img, mask, p, 1), run(gpu_ctx, img, mask, p, 0)
        same(a, b)
        assert a[1]["graph_iterations"] == (2 if iters == 2 else 0)
        if tol > 1:
            assert all(i == 1 for i in a[1]["iterations"][:2])
        else:
            assert all(i == iters for i in a[1]["iterations"][:2])


@pytest.mark.parametrize("mode", [0, 1])
def test_graph_batch_equals_host_loop(gpu_ctx, mode):
    """Lockstep batches (NLI_TUNE_BATCH_MODE 1) run each rank's iterations in
    a graph whenever the graph loop is on; the worker-context form (0) only
    with NLI_TUNE_GRAPH_LOOP = 2 (1 keeps its host loop).  Outputs are
    identical either way."""
    from test_gpu_batch import small_batch
    items, params = small_batch(count=5, seed=21)
    gpu_ctx.set_tuning(gpu_ctx.TUNE_BATCH_MODE, mode)
    try:
        gpu_ctx.set_seed(9)
        gpu_ctx.set_tuning(gpu_ctx.TUNE_GRAPH_LOOP, 1)
        outs_1, st_1 = gpu_ctx.process_batch(items, params)
        if mode == 0:
            assert all(s["graph_iterations"] == 0 for s in st_1)
        else:
            assert all(s["graph_iterations"] > 0 for s in st_1)
        gpu_ctx.set_seed(9)
        gpu_ctx.set_tuning(gpu_ctx.TUNE_GRAPH_LOOP, 2)
        outs_g, st_g = gpu_ctx.process_batch(items, params)
        assert all(s["graph_iterations"] > 0 for s in st_g)
        for a, b in zip(outs_g, outs_1):
            assert np.array_equal(a, b)
        gpu_ctx.set_tuning(gpu_ctx.TUNE_GRAPH_LOOP, 0)
        gpu_ctx.set_seed(9)
        outs_h, st_h = gpu_ctx.process_batch(items, params)
        assert all(s["graph_iterations"] == 0 for s in st_h)
    finally:
        gpu_ctx.set_tuning(gpu_ctx.TUNE_GRAPH_LOOP, 1)
        gpu_ctx.set_tuning(gpu_ctx.TUNE_BATCH_MODE, 1)
    for a, b in zip(outs_g, outs_h):
        assert np.array_equal(a, b)


def test_graph_knob(gpu_ctx):
    from nli_gb300 import NliError
    assert gpu_ctx.get_tuning(gpu_ctx.TUNE_GRAPH_LOOP) == 1
    with pytest.raises(NliError):
        gpu_ctx.set_tuning(gpu_ctx.TUNE_GRAPH_LOOP, 3)
