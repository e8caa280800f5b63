"""Bounded device waits and the checked build, tested the way a shared GPU
allows: nothing here faults, traps or hangs.

* The grid CG's grid barrier is a bounded software spin.  With its poll
  limit forced down (nli_debug_grid_wait_limit) on a system that takes the
  grid layout, the wait runs out: the kernel's blocks leave, the call
  returns NLI_E_TIMEOUT with its message, the timeout word is cleared, and
  the same context then computes the clean run's result.
* The checked build (NLI_CHECKED) bounds-tests every data-dependent
  gathered index.  On valid inputs of every method it must record nothing
  and compute exactly what the ordinary build computes.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def grid_case(ctx):
    """A 192x192 NL-Poisson update whose ~5.5k unknowns exceed one CTA's
    shared memory; with an unknowns-per-CTA floor of 2^30 no cluster is
    formed, so it takes the grid CG."""
    from nli_gb300 import workloads as wl
    img, mask, p = wl.config2(seed=31, size=192, scales=1)
    ext = ctx.extended_domain(mask, 9, 9)
    src, tgt, _ = ctx.scale_masks(ext, 4, True)
    d_img = ctx._f32(img)
    ctx.set_seed(9)
    nnf, _, _ = ctx.patchmatch(p.distance, p.patchmatch, d_img, src, d_img, tgt)
    conf = ctx.confidence_mask(mask, p.conf_decay_time, p.conf_asymptotic)
    return img, mask, ext, nnf, conf, p


def test_grid_barrier_timeout_and_recovery(gpu_ctx):
    from nli_gb300 import NliError
    ctx = gpu_ctx
    img, mask, ext, nnf, conf, p = grid_case(ctx)
    assert int(mask.sum()) > 4096
    ctx.set_tuning(ctx.TUNE_CG_UNKNOWNS_PER_CTA, 1 << 30)
    try:
        clean, t_clean = ctx.update(p.update, img, img, mask, ext, nnf, conf)
        ctx.grid_wait_limit(1)
        with pytest.raises(NliError) as e:
            ctx.update(p.update, img, img, mask, ext, nnf, conf)
        assert e.value.status == -7 and "timed out" in str(e.value)  # NLI_E_TIMEOUT
        ctx.grid_wait_limit(0)
        again, t_again = ctx.update(p.update, img, img, mask, ext, nnf, conf)
    finally:
        ctx.grid_wait_limit(0)
        ctx.set_tuning(ctx.TUNE_CG_UNKNOWNS_PER_CTA, 1024)
    assert np.array_equal(again.cpu().numpy(), clean.cpu().numpy())
    assert t_again == t_clean


@pytest.fixture(scope="module")
def checked_ctx():
    import __graft_entry__ as ge
    pkg = ge.package()
    from nli_gb300 import build as nb
    path = nb.build(checked=True)
    ctx = pkg.Context(0, lib_path=path)
    yield ctx
    ctx.close()


def small_cases():
    from nli_gb300 import workloads as wl
    out = []
    img, mask, p = wl.config1(seed=41, size=72)
    p.scales, p.subsampling_rate, p.iterations = 2, wl._abi.subsampling_rate(0.6, 2), 10
    out.append(("means", img, mask, p))
    img, mask, _ = wl.config2(seed=42, size=72, scales=2)
    out.append(("poisson", img, mask, wl.params("nlpoisson", scales=2, coarse=0.6, iters=8, cg_tol=1e-4)))
    img, mask, _ = wl.config1(seed=43, size=64)
    out.append(("medians", img, mask, wl.params("nlmedians", scales=2, coarse=0.6, iters=6)))
    img, mask, _ = wl.config3(seed=44, w=80, h=64, scales=2)
    out.append(("depth", img, mask, wl.params("nldepth", scales=2, coarse=0.6, lam_r=1.0, lam_d=0.0, iters=6)))
    return out


def test_checked_build_records_nothing_and_matches(gpu_ctx, checked_ctx):
    word, checked = checked_ctx.check_status()
    assert checked and word == 0
    assert gpu_ctx.check_status() == (0, False)
    for name, img, mask, p in small_cases():
        gpu_ctx.set_seed(5)
        checked_ctx.set_seed(5)
        want, _ = gpu_ctx.process(img, mask, p)
        got, _ = checked_ctx.process(img, mask, p)
        assert checked_ctx.check_status() == (0, True), name
        assert np.array_equal(got, want), name
    # a batch (lockstep kernels) as well
    items = [(img, mask) for _, img, mask, _ in small_cases()[:2]]
    params = [p for _, _, _, p in small_cases()[:2]]
    gpu_ctx.set_seed(6)
    checked_ctx.set_seed(6)
    want, _ = gpu_ctx.process_batch(items, params)
    got, _ = checked_ctx.process_batch(items, params)
    assert checked_ctx.check_status() == (0, True)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)
