"""Host-side logic that needs no GPU: the autotuner's cache file and
re-application (against a recording stand-in for the context), the
benchmark's workload table and throughput arithmetic, and the ABI's tuning
constants as the Python binding and the C header declare them."""
import json
import os
import re

import pytest

import bench
from nli_gb300 import autotune


class FakeCtx:
    """Records what autotune.apply sets; the knob numbers are the binding's."""

    def __init__(self):
        import nli_gb300 as pkg
        for k in ("TUNE_CG_CLUSTER_CAP", "TUNE_CG_UNKNOWNS_PER_CTA", "TUNE_BATCH_WIDTH", "TUNE_PM_VARIANT",
                  "TUNE_CG_PRECOND", "TUNE_GRAPH_LOOP", "TUNE_CG_SINGLE_MAX", "TUNE_BATCH_MODE", "TUNE_PM_BOUND",
                  "TUNE_BATCH_GROUPS", "TUNE_PM_TILE"):
            setattr(self, k, getattr(pkg.Context, k))
        self.tuning = {}
        self.batch_width = None

    def set_tuning(self, knob, value):
        self.tuning[knob] = value

    def set_batch_width(self, width):
        self.batch_width = width


def test_cache_round_trip_on_host(tmp_path):
    path = str(tmp_path / "tuning.json")
    ctx = FakeCtx()
    assert autotune.load(ctx, path, "dev") is None
    autotune.save(path, "dev", cg=(12, 2048), batch_width=6, pm_variant=2)
    autotune.save(path, "other", cg=(4, 512))
    assert autotune.load(ctx, path, "missing") is None
    got = autotune.load(ctx, path, "dev")
    assert got == {"cg": [12, 2048], "batch_width": 6, "pm_variant": 2}
    assert ctx.tuning == {ctx.TUNE_CG_CLUSTER_CAP: 12, ctx.TUNE_CG_UNKNOWNS_PER_CTA: 2048, ctx.TUNE_PM_VARIANT: 2}
    assert ctx.batch_width == 6
    with open(path) as f:
        table = json.load(f)
    assert set(table) == {"dev", "other"} and table["other"] == {"cg": [4, 512]}
    assert not os.path.exists(path + ".tmp")


def test_cache_round_trip_every_knob(tmp_path):
    path = str(tmp_path / "tuning.json")
    ctx = FakeCtx()
    autotune.save(path, "dev", cg=(8, 1024), batch_width=4, pm_variant=1, cg_single=2048, pm_bound=0,
                  batch_mode=1, batch_groups=4, pm_tile=16)
    got = autotune.load(ctx, path, "dev")
    assert got == {"cg": [8, 1024], "batch_width": 4, "pm_variant": 1, "cg_single": 2048, "pm_bound": 0,
                   "batch_mode": 1, "batch_groups": 4, "pm_tile": 16}
    assert ctx.tuning == {ctx.TUNE_CG_CLUSTER_CAP: 8, ctx.TUNE_CG_UNKNOWNS_PER_CTA: 1024, ctx.TUNE_PM_VARIANT: 1,
                          ctx.TUNE_CG_SINGLE_MAX: 2048, ctx.TUNE_PM_BOUND: 0, ctx.TUNE_BATCH_MODE: 1,
                          ctx.TUNE_BATCH_GROUPS: 4, ctx.TUNE_PM_TILE: 16}
    assert ctx.batch_width == 4


def test_tuning_constants_match_the_header():
    """The binding's TUNE_* numbers are the header's NLI_TUNE_* defines."""
    import nli_gb300 as pkg
    here = os.path.dirname(os.path.abspath(__file__))
    header = open(os.path.join(here, "..", "include", "nli.h")).read()
    defines = dict((m.group(1), int(m.group(2))) for m in re.finditer(r"#define NLI_(TUNE_\w+) (\d+)", header))
    assert len(defines) == 11
    for name, value in defines.items():
        assert getattr(pkg.Context, name) == value, name


def test_bench_workloads_and_throughput():
    assert set(bench.WORKLOADS) == {"nlpoisson512", "nlmeans256", "nldepth640"}
    for name in bench.WORKLOADS:
        bench.WORKLOAD = name
        try:
            assert bench.workload_desc() == bench.WORKLOADS[name]
            assert bench.flop_per_candidate() == (44 * 81 + 8 if name == "nldepth640" else 31 * 81 + 8)
        finally:
            bench.WORKLOAD = "nlpoisson512"
    # whole-job throughput: N ranks x steps x Mpix per rank and step / seconds
    assert bench.job_throughput(2, 5, 0.262144, 1000.0) == pytest.approx(2 * 5 * 0.262144)


def test_formula_candidates():
    """The reference's candidate count per process(): per scale, calls
    (iterations plus one per transition the scale takes part in) x N_t x
    (1 + I (2 + floor(log2 max(W, H)) + 1))."""
    st = {"scales": 3, "width": [512, 256, 128], "height": [400, 200, 100], "targets": [1000, 300, 50],
          "iterations": [5, 7, 9]}
    want = (5 + 1) * 1000 * (1 + 10 * (2 + 10)) + (7 + 2) * 300 * (1 + 10 * (2 + 9)) + \
        (9 + 1) * 50 * (1 + 10 * (2 + 8))
    assert bench.formula_candidates(st, 10) == want
    st1 = {"scales": 1, "width": [64], "height": [64], "targets": [20], "iterations": [3]}
    assert bench.formula_candidates(st1, 4) == 3 * 20 * (1 + 4 * (2 + 7))


def test_batch_reference_gaps_only_compare_the_same_batch(tmp_path, monkeypatch):
    """References are compared only with the batch they were made from
    (seed, count, largest side): another batch's item i is another image."""
    import numpy as np
    rng = np.random.default_rng(0)
    img = rng.uniform(0, 255, (20, 30, 3)).astype(np.float32)
    mask = np.zeros((20, 30), np.uint8)
    mask[5:10, 5:12] = 1
    ref_hole = img[mask > 0] + 2.0
    np.savez(tmp_path / "batch_reference_01.npz", hole=ref_hole, index=1, batch=np.array([5, 64, 1024]))
    monkeypatch.setattr(bench, "GOLDEN", str(tmp_path))
    out = img.copy()
    out[mask > 0] += 1.0  # closer to the truth than the reference
    items = [(img, mask, "nlmeans", 2)] * 2
    rows = bench.batch_reference_gaps(items, [img, out], (5, 64, 1024))
    assert len(rows) == 1 and rows[0]["index"] == 1
    assert rows[0]["gap_db"] == pytest.approx(20 * np.log10(2.0), rel=1e-6)
    assert bench.batch_reference_gaps(items, [img, out], (5, 32, 768)) == []
