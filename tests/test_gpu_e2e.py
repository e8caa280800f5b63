"""End-to-end on the full-size benchmark configurations (1: 256x256 nlmeans,
2: 512x512 nlpoisson, 3: 640x480 nldepth), against the reference's own
output for the same input (tests/golden/config*_reference.npz, produced by
the serial reference build with srand(101)).

The GPU PatchMatch draws different random numbers and sweeps in parallel,
so the inpainting reaches a different (similar) solution: the comparison
is the hole-region PSNR of the GPU output against the reference output, and
the gap between the reference's and the GPU's hole PSNR against the ground
truth (the synthetic image before masking)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def psnr(a, b, peak):
    mse = float(np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2))
    return float("inf") if mse == 0 else 10 * np.log10(peak * peak / mse)


@pytest.mark.parametrize("name", ["config1", "config2", "config3"])
def test_full_size_vs_reference(gpu_ctx, name):
    from nli_gb300 import workloads as wl
    g = np.load(os.path.join(GOLDEN, "%s_reference.npz" % name))
    img, mask, p = getattr(wl, name)(seed=0)
    gpu_ctx.set_seed(101)
    out, st = gpu_ctx.process(img, mask, p)
    hole = mask > 0
    ref_hole = g["hole"]
    rows = []
    # colour channels on a 0-255 peak; the depth channel of configuration 3
    # (metres) on its own range
    chans = [(slice(0, 3), 255.0)]
    if img.shape[2] == 4:
        chans.append((slice(3, 4), float(img[..., 3].max() - img[..., 3].min())))
    for sl, peak in chans:
        o, r, t = out[hole][:, sl], ref_hole[:, sl], img[hole][:, sl]
        vs_ref = psnr(o, r, peak)
        gpu_gt, ref_gt = psnr(o, t, peak), psnr(r, t, peak)
        rows.append({"channels": "%d:%d" % (sl.start, sl.stop), "psnr_gpu_vs_ref": vs_ref,
                     "psnr_gpu_vs_truth": gpu_gt, "psnr_ref_vs_truth": ref_gt, "gap_db": ref_gt - gpu_gt})
    report = {"workload": name, "iterations_gpu": st["iterations"], "rows": rows}
    print(json.dumps(report))
    assert np.isfinite(out).all()
    assert np.array_equal(out[~hole], img[~hole])
    for r in rows:
        assert r["psnr_gpu_vs_ref"] > 15.0, r
        assert r["gap_db"] < 3.0, r
