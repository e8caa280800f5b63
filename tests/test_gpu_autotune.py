"""The autotuner's CG launch shapes: every candidate gives the same update
up to the rounding of the CG sums, and the chosen shape is applied."""
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
