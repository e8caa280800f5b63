"""End-to-end on the full-size benchmark configurations (1: 256x256 nlmeans,
2: 512x512 nlpoisson, 3: 640x480 nldepth), against the reference's own
output for the same inputs: three input seeds per configuration
(tests/golden/config*_reference*.npz, produced by the serial reference build
with srand(101) by tests/golden/make_golden.py --full --seeds).

The GPU PatchMatch draws different random numbers and sweeps in parallel,
so the inpainting reaches a different (similar) solution; like the
reference's own runs with different seeds, runs with different PatchMatch
seeds differ in hole PSNR by a few tenths of a dB.  The contract is the
metric's: the hole-region PSNR of the GPU output against the ground truth
(the synthetic image before masking) may not fall more than 0.1 dB below
the reference's.  It is tested on means: per input seed, the mean over
eight GPU PatchMatch seeds (the reference has one run per input); then the
mean over the three input seeds of (reference - GPU), per channel group.
The per-run figures are printed."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

SEEDS = (0, 1, 2)
PM_SEEDS = tuple(range(101, 109))  # GPU PatchMatch seeds per input
MAX_GAP_DB = 0.1  # reference PSNR minus ours, mean over the input seeds


def psnr(a, b, peak):
    mse = float(np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2))
    return float("inf") if mse == 0 else 10 * np.log10(peak * peak / mse)


def reference_path(name, seed):
    return os.path.join(GOLDEN, "%s_reference.npz" % name if seed == 0 else "%s_reference_seed%d.npz" % (name, seed))


def run_seed(gpu_ctx, name, seed):
    from nli_gb300 import workloads as wl
    g = np.load(reference_path(name, seed))
    img, mask, p = getattr(wl, name)(seed=seed)
    hole = mask > 0
    ref_hole = g["hole"]
    # colour channels on a 0-255 peak; the depth channel of configuration 3
    # (metres) on its own range
    chans = [(slice(0, 3), 255.0)]
    if img.shape[2] == 4:
        chans.append((slice(3, 4), float(img[..., 3].max() - img[..., 3].min())))
    rows = []
    for pm_seed in PM_SEEDS:
        gpu_ctx.set_seed(pm_seed)
        out, st = gpu_ctx.process(img, mask, p)
        assert np.isfinite(out).all()
        assert np.array_equal(out[~hole], img[~hole])
        for sl, peak in chans:
            o, r, t = out[hole][:, sl], ref_hole[:, sl], img[hole][:, sl]
            rows.append({"seed": seed, "pm_seed": pm_seed, "channels": "%d:%d" % (sl.start, sl.stop),
                         "psnr_gpu_vs_ref": psnr(o, r, peak), "psnr_gpu_vs_truth": psnr(o, t, peak),
                         "psnr_ref_vs_truth": psnr(r, t, peak)})
    return rows, st


@pytest.mark.parametrize("name", ["config1", "config2", "config3"])
def test_full_size_vs_reference(gpu_ctx, name):
    rows = []
    for seed in SEEDS:
        r, st = run_seed(gpu_ctx, name, seed)
        rows += r
    groups = sorted({r["channels"] for r in rows})
    summary = []
    for ch in groups:
        per_input = []
        for seed in SEEDS:
            sel = [r for r in rows if r["channels"] == ch and r["seed"] == seed]
            per_input.append((float(np.mean([r["psnr_gpu_vs_truth"] for r in sel])), sel[0]["psnr_ref_vs_truth"],
                              float(np.std([r["psnr_gpu_vs_truth"] for r in sel]))))
        gpu = float(np.mean([a for a, _, _ in per_input]))
        ref = float(np.mean([b for _, b, _ in per_input]))
        summary.append({"channels": ch, "per_input": [{"seed": s, "gpu_mean": a, "gpu_std": c, "reference": b}
                                                      for s, (a, b, c) in zip(SEEDS, per_input)],
                        "mean_psnr_gpu_vs_truth": gpu, "mean_psnr_ref_vs_truth": ref, "mean_gap_db": ref - gpu})
    print(json.dumps({"workload": name, "seeds": list(SEEDS), "rows": rows, "summary": summary}))
    for r in rows:
        # a sanity bound per seed: the two outputs are the same kind of fill
        assert r["psnr_gpu_vs_ref"] > 15.0, r
    for s in summary:
        assert s["mean_gap_db"] <= MAX_GAP_DB, s
