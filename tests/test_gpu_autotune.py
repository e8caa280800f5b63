"""The autotuner: every CG launch shape gives the same update up to the
rounding of the CG sums, the PatchMatch variants and bound and the batch
forms give identical results, and each tuner applies its choice."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tune_cg(gpu_ctx):
    from nli_gb300 import autotune
    case = autotune.poisson_case(gpu_ctx, size=192, seed=3)
    upd, u, mask, ext, nnf, conf = case
    outs = {}
    for cap, per in ((4, 512), (16, 1024), (16, 2048)):
        autotune.apply(gpu_ctx, cg=(cap, per))
        outs[(cap, per)] = gpu_ctx.update(upd, u, u, mask, ext, nnf, conf)[0].cpu().numpy()
    ref = outs[(16, 1024)]
    hole = mask != 0
    for k, o in outs.items():
        rel = np.abs(o[hole] - ref[hole]).max() / np.abs(ref[hole]).max()
        assert rel < 1e-3, (k, rel)  # CG stopped at tolerance 1e-4 from different sum orders
    res = autotune.tune_cg(gpu_ctx, case, caps=(4, 16), per_cta=(512, 1024), repeats=1)
    assert res["best"] in res["ms"] and len(res["ms"]) == 4
    assert gpu_ctx.get_tuning(gpu_ctx.TUNE_CG_CLUSTER_CAP) == res["best"][0]
    assert gpu_ctx.get_tuning(gpu_ctx.TUNE_CG_UNKNOWNS_PER_CTA) == res["best"][1]
    autotune.apply(gpu_ctx, cg=(16, 1024))  # back to the defaults for later tests


def test_tune_pm_variant(gpu_ctx):
    from nli_gb300 import autotune
    case = autotune.patchmatch_case(gpu_ctx, size=160, seed=2)
    res = autotune.tune_pm_variant(gpu_ctx, case, repeats=1)
    assert sorted(res["ms"]) == [0, 1, 2] and res["best"] in res["ms"]
    assert gpu_ctx.get_tuning(gpu_ctx.TUNE_PM_VARIANT) == res["best"]
    autotune.apply(gpu_ctx, pm_variant=0)
    assert gpu_ctx.get_tuning(gpu_ctx.TUNE_PM_VARIANT) == 0


def test_tuning_knobs_validate(gpu_ctx):
    from nli_gb300 import NliError
    with pytest.raises(NliError):
        gpu_ctx.set_tuning(gpu_ctx.TUNE_CG_CLUSTER_CAP, 17)
    with pytest.raises(NliError):
        gpu_ctx.set_tuning(99, 1)
    gpu_ctx.set_tuning(gpu_ctx.TUNE_BATCH_WIDTH, 5)
    assert gpu_ctx.get_tuning(gpu_ctx.TUNE_BATCH_WIDTH) == 5
    gpu_ctx.set_tuning(gpu_ctx.TUNE_BATCH_WIDTH, 8)


def test_cache_file_round_trip(gpu_ctx, tmp_path):
    from nli_gb300 import autotune
    path = str(tmp_path / "tuning.json")
    key = autotune.device_key(0)
    assert autotune.load(gpu_ctx, path, key) is None
    autotune.save(path, "other device", cg=(8, 512))
    autotune.save(path, key, cg=(12, 2048), batch_width=6, pm_variant=0)
    try:
        got = autotune.load(gpu_ctx, path, key)
        assert got == {"cg": [12, 2048], "batch_width": 6, "pm_variant": 0}
        assert gpu_ctx.get_tuning(gpu_ctx.TUNE_CG_CLUSTER_CAP) == 12
        assert gpu_ctx.get_tuning(gpu_ctx.TUNE_CG_UNKNOWNS_PER_CTA) == 2048
        assert gpu_ctx.get_tuning(gpu_ctx.TUNE_BATCH_WIDTH) == 6
        assert autotune.load(gpu_ctx, path, "missing") is None
    finally:
        autotune.apply(gpu_ctx, cg=(16, 1024), batch_width=8, pm_variant=0)


def test_tune_cg_single_and_pm_bound(gpu_ctx):
    from nli_gb300 import autotune
    cases = [autotune.poisson_case(gpu_ctx, size=s, seed=1) for s in (48, 96)]
    res = autotune.tune_cg_single(gpu_ctx, cases, limits=(0, 1024, 4096), repeats=1)
    assert sorted(res["ms"]) == [0, 1024, 4096]
    assert gpu_ctx.get_tuning(gpu_ctx.TUNE_CG_SINGLE_MAX) == res["best"]
    case = autotune.patchmatch_case(gpu_ctx, size=160, seed=2)
    res = autotune.tune_pm_bound(gpu_ctx, case, repeats=1)
    assert sorted(res["ms"]) == [0, 1, 2]
    assert gpu_ctx.get_tuning(gpu_ctx.TUNE_PM_BOUND) == res["best"]
    autotune.apply(gpu_ctx, cg_single=1024, pm_bound=1)


def test_tune_batch_mode_and_groups(gpu_ctx):
    import torch
    from nli_gb300 import autotune
    from nli_gb300 import workloads as wl
    rng = np.random.default_rng(4)
    items, params = [], []
    for i in range(6):
        w, h = int(rng.integers(48, 96)), int(rng.integers(48, 96))
        img, _ = wl.voronoi_texture(w, h, 8, rng)
        mask = wl.ellipse_mask(w, h, 2, 0.1, rng)
        items.append((torch.from_numpy(img).cuda(), torch.from_numpy(mask).cuda()))
        params.append(wl.params("nlmeans" if i % 2 else "nlpoisson", scales=2, coarse=0.5, iters=4, cg_tol=1e-4))
    try:
        res = autotune.tune_batch_mode(gpu_ctx, items, params)
        assert sorted(res["ms"]) == [0, 1] and gpu_ctx.get_tuning(gpu_ctx.TUNE_BATCH_MODE) == res["best"]
        res = autotune.tune_batch_groups(gpu_ctx, items, params, groups=(1, 3))
        assert sorted(res["ms"]) == [1, 3] and gpu_ctx.get_tuning(gpu_ctx.TUNE_BATCH_GROUPS) == res["best"]
    finally:
        autotune.apply(gpu_ctx, batch_mode=1, batch_groups=4)


def test_tune_pm_tile(gpu_ctx):
    from nli_gb300 import autotune
    case = autotune.patchmatch_case(gpu_ctx, size=160, seed=2)
    res = autotune.tune_pm_tile(gpu_ctx, case, tiles=(0, 8), repeats=1)
    assert sorted(res["ms"]) == [0, 8]
    assert gpu_ctx.get_tuning(gpu_ctx.TUNE_PM_TILE) == res["best"]
    autotune.apply(gpu_ctx, pm_tile=1)
