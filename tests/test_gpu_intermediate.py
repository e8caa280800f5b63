"""Observability of the reference: PatchMatch's METRICS figures
(patch_match.cpp:383-507) and ImageInpainting::keep_intermediate pyramids
(image_inpainting.cpp:103-108, 310-337, 410-412)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def pm_case(ctx, size=96, seed=3):
    from nli_gb300 import workloads as wl
    img, mask, p = wl.config2(seed=seed, size=size, scales=3)
    ext = ctx.extended_domain(mask, 9, 9)
    src, tgt, _ = ctx.scale_masks(ext, 4, True)
    u = ctx.poisson_init(img, mask)
    return u, src, tgt, p


def test_patchmatch_metrics(gpu_ctx):
    u, src, tgt, p = pm_case(gpu_ctx)
    gpu_ctx.set_seed(9)
    nnf, d, e, total, prop, shots = gpu_ctx.patchmatch_metrics(p.distance, p.patchmatch, u, src, u, tgt)
    gpu_ctx.set_seed(9)
    nnf2, _, e2 = gpu_ctx.patchmatch(p.distance, p.patchmatch, u, src, u, tgt)
    assert np.array_equal(nnf.cpu().numpy(), nnf2.cpu().numpy())  # the figures do not change the result
    assert e == e2
    assert len(total) == len(prop) == p.patchmatch.iterations
    assert total[-1] == e  # total after the last sweep is the field's energy
    assert all(b <= a for a, b in zip(total, total[1:]))  # a sweep never worsens a match
    n_targets = int(tgt.sum().item())
    assert all(0 <= v <= n_targets for v in prop) and prop[0] > 0
    assert 0 <= shots < p.patchmatch.random_shots


def test_keep_intermediate(gpu_ctx):
    from nli_gb300 import workloads as wl
    img, mask, _ = wl.config2(seed=5, size=96, scales=3)
    p = wl.params("nlpoisson", scales=3, coarse=0.5, iters=10, cg_tol=1e-4)
    gpu_ctx.set_seed(21)
    plain, st = gpu_ctx.process(img, mask, p)
    gpu_ctx.keep_intermediate(True)
    try:
        gpu_ctx.set_seed(21)
        out, st2 = gpu_ctx.process(img, mask, p)
        inputs = gpu_ctx.intermediate(gpu_ctx.INTER_INPUT)
        outputs = gpu_ctx.intermediate(gpu_ctx.INTER_OUTPUT)
        masks = gpu_ctx.intermediate(gpu_ctx.INTER_MASK)
        nnfs = gpu_ctx.intermediate(gpu_ctx.INTER_NNF)
    finally:
        gpu_ctx.keep_intermediate(False)
    assert np.array_equal(out, plain)  # keeping copies does not change the result
    assert len(inputs) == len(outputs) == len(masks) == len(nnfs) == p.scales
    for i in range(p.scales):
        assert inputs[i].shape == (st2["height"][i], st2["width"][i], 3)
        assert outputs[i].shape == inputs[i].shape and masks[i].shape == inputs[i].shape[:2]
    assert np.array_equal(inputs[0], img) and np.array_equal(masks[0], mask.astype(np.uint8))
    assert np.array_equal(outputs[0], out)
    # NNFs in inpainting order: coarsest first, finest last
    for k, i in enumerate(reversed(range(p.scales))):
        assert nnfs[k].shape == (st2["height"][i], st2["width"][i], 2)
    # the pyramid levels are the masked downsampling of the level above
    for i in range(1, p.scales):
        di, dm = gpu_ctx.downsample_with_mask(inputs[i - 1], masks[i - 1], p.subsampling_rate, 0.4, 0)
        assert np.array_equal(di.cpu().numpy(), inputs[i]) and np.array_equal(dm.cpu().numpy(), masks[i])
    # every hole pixel of the finest level away from the image border has a match
    inner = np.zeros_like(mask, dtype=bool)
    inner[4:-4, 4:-4] = True
    assert (nnfs[-1][(mask != 0) & inner][:, 0] >= 0).all()
