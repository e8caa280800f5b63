"""Batched driver (nli_process_batch / nli_process_batch_device): uneven
image/mask pairs with mixed methods in flight together; every image must
equal its plain nli_process run with the per-image seed, bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small_batch(count=6, seed=11):
    """A config-5-shaped batch at small sizes: sides 40-96, aspect 0.5-2,
    ellipse or stroke holes, alternating nlmeans / nlpoisson, 3 scales."""
    from nli_gb300 import workloads as wl
    rng = np.random.default_rng(seed)
    items, params = [], []
    for i in range(count):
        side = float(np.exp(rng.uniform(np.log(40), np.log(96))))
        aspect = float(np.exp(rng.uniform(np.log(0.5), np.log(2.0))))
        w, h = max(32, int(round(side * aspect ** 0.5))), max(32, int(round(side / aspect ** 0.5)))
        img, _ = wl.voronoi_texture(w, h, int(rng.integers(6, 16)), rng)
        if i % 3 == 2:
            mask = wl.stroke_mask(w, h, 3, (4, 8), rng, coverage=0.12)
        else:
            mask = wl.ellipse_mask(w, h, 2, 0.12, rng)
        method = "nlmeans" if i % 2 == 0 else "nlpoisson"
        items.append((img, mask))
        params.append(wl.params(method, scales=3, coarse=0.5, iters=15, cg_tol=1e-4))
    return items, params


def plain(ctx, items, params, seed):
    outs = []
    for i, ((img, mask), p) in enumerate(zip(items, params)):
        ctx.set_seed(ctx.batch_seed(seed, i))
        outs.append(ctx.process(img, mask, p)[0])
    return outs


@pytest.mark.parametrize("width", [1, 4, 8])
def test_batch_equals_plain_runs(gpu_ctx, width):
    items, params = small_batch()
    seed = 777
    want = plain(gpu_ctx, items, params, seed)
    gpu_ctx.set_seed(seed)
    gpu_ctx.set_batch_width(width)
    got, stats = gpu_ctx.process_batch(items, params)
    for i, (g, w) in enumerate(zip(got, want)):
        assert np.array_equal(g, w), i
        assert stats[i]["scales"] == params[i].scales


def test_batch_device_equals_plain_runs(gpu_ctx):
    items, params = small_batch(count=5, seed=12)
    seed = 4242
    want = plain(gpu_ctx, items, params, seed)
    gpu_ctx.set_seed(seed)
    gpu_ctx.set_batch_width(3)
    got, _ = gpu_ctx.process_batch_device(items, params)
    for i, (g, w) in enumerate(zip(got, want)):
        assert np.array_equal(g.cpu().numpy(), w), i


def test_batch_reports_failed_image(gpu_ctx):
    """An image whose source mask is empty fails alone; the others finish."""
    from nli_gb300 import NliError
    items, params = small_batch(count=4, seed=13)
    img, mask = items[1]
    items[1] = (img, np.ones_like(mask))  # everything masked: no source
    gpu_ctx.set_seed(5)
    gpu_ctx.set_batch_width(4)
    with pytest.raises(NliError) as e:
        gpu_ctx.process_batch(items, params)
    assert e.value.status == -2  # NLI_E_EMPTY_SOURCE
    assert list(gpu_ctx.last_batch_status) == [0, -2, 0, 0]


def test_empty_batch(gpu_ctx):
    assert gpu_ctx.process_batch([], []) == ([], [])


def test_injected_allocation_failure_leaves_context_usable():
    """Host-side fault injection: a workspace growth fails as out of memory
    in the middle of process(); the call returns NLI_E_NOMEM with its
    message, and the same context then runs the image to the same output as
    a fresh context."""
    import nli_gb300 as pkg
    from nli_gb300 import NliError
    from nli_gb300 import workloads as wl
    img, mask, _ = wl.config2(seed=6, size=96, scales=3)
    p = wl.params("nlpoisson", scales=3, coarse=0.5, iters=4, cg_tol=1e-4)
    ctx = pkg.Context(0)
    try:
        ctx.fail_allocation(5)
        with pytest.raises(NliError) as e:
            ctx.process(img, mask, p)
        assert e.value.status == -8 and "injected" in str(e.value)  # NLI_E_NOMEM
        ctx.fail_allocation(0)
        ctx.set_seed(3)
        out, _ = ctx.process(img, mask, p)
    finally:
        ctx.close()
    fresh = pkg.Context(0)
    try:
        fresh.set_seed(3)
        ref, _ = fresh.process(img, mask, p)
    finally:
        fresh.close()
    assert np.array_equal(out, ref)
