"""The Jacobi-preconditioned conjugate gradient (NLI_TUNE_CG_PRECOND = 1)
against the FP64 oracle at full size (the 512x512 NL-Poisson workload), on
both solver layouts (thread-block clusters, and the cooperative grid kernel
forced by a cluster cap of 1), and whole runs of the NL-Poisson and NL-depth
workloads against the reference's own output.  Its stopping test is the
plain CG's (|r|^2 < tol |r0|^2 on the true residual), so its distance to the
exact solution must be of the same size as the reference arithmetic's, in
fewer iterations."""
import json
import os

import numpy as np
import pytest
import torch

import update64
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case(gpu_ctx):
    from nli_gb300 import workloads as wl
    img, mask, p = wl.config2(seed=0, size=512)
    ext = gpu_ctx.extended_domain(mask, 9, 9)
    src, tgt, _ = gpu_ctx.scale_masks(ext, 4, True)
    u = gpu_ctx.poisson_init(img, mask)
    gpu_ctx.set_seed(1)
    nnf, _, _ = gpu_ctx.patchmatch(p.distance, p.patchmatch, u, src, u, tgt)
    conf = gpu_ctx.confidence_mask(mask, 5.0, 0.1)
    return dict(u=u.cpu().numpy(), mask=mask, ext=ext.cpu().numpy(), nnf=nnf.cpu().numpy(), conf=conf.cpu().numpy())


def hole_rel(a, b, mask):
    m = mask != 0
    return float(np.abs(a[m].astype(np.float64) - b[m]).max() / np.abs(b[m]).max())


def run_update(ctx, upd, c, precond, cap):
    ctx.set_tuning(ctx.TUNE_CG_PRECOND, precond)
    ctx.set_tuning(ctx.TUNE_CG_CLUSTER_CAP, cap)
    try:
        before = ctx.counters()["cg_iterations"]
        out = ctx.update(upd, c["u"], c["u"], c["mask"], c["ext"], c["nnf"], c["conf"])[0].cpu().numpy()
        return out, ctx.counters()["cg_iterations"] - before
    finally:
        ctx.set_tuning(ctx.TUNE_CG_PRECOND, 0)
        ctx.set_tuning(ctx.TUNE_CG_CLUSTER_CAP, 16)


@pytest.mark.parametrize("cap", [16, 1], ids=["cluster", "grid"])
@pytest.mark.parametrize("tol", [1e-4, 1e-6])
def test_precond_vs_fp64(gpu_ctx, oracle, case, tol, cap):
    from nli_gb300 import workloads as wl
    upd = wl.params("nlpoisson", cg_tol=tol).update
    c = case
    exact = update64.poisson(torch.from_numpy(c["u"]).double(), upd.lambda_, upd.sigma, c["nnf"], c["mask"] != 0,
                             c["ext"], c["conf"].astype(np.float64), solver="sparse").numpy()
    ref = oracle.update(upd, c["u"], c["u"], c["mask"], c["ext"], c["nnf"], c["conf"])[0]
    plain, it_plain = run_update(gpu_ctx, upd, c, 0, cap)
    pre, it_pre = run_update(gpu_ctx, upd, c, 1, cap)
    m = c["mask"] != 0
    e_ref, e_plain, e_pre = hole_rel(ref, exact, m), hole_rel(plain, exact, m), hole_rel(pre, exact, m)
    print(json.dumps({"tol": tol, "layout": "cluster" if cap > 1 else "grid", "err_reference": e_ref,
                      "err_plain": e_plain, "err_jacobi": e_pre, "cg_iterations_plain": it_plain,
                      "cg_iterations_jacobi": it_pre}))
    assert np.array_equal(pre[~m], c["u"][~m])
    assert e_pre <= 3.0 * e_ref + 1e-5, (e_pre, e_ref)
    assert it_pre < it_plain, (it_pre, it_plain)


@pytest.mark.parametrize("name", ["config2", "config3"])
def test_precond_full_size_vs_reference(gpu_ctx, name):
    """Whole runs with the preconditioned solver: the gates of the plain
    end-to-end test (hole PSNR against the reference's output and the gap to
    the reference's PSNR against the ground truth); the figures are printed."""
    from nli_gb300 import workloads as wl
    g = np.load(os.path.join(GOLDEN, "%s_reference.npz" % name))
    img, mask, p = getattr(wl, name)(seed=0)
    gpu_ctx.set_tuning(gpu_ctx.TUNE_CG_PRECOND, 1)
    try:
        gpu_ctx.set_seed(101)
        out, st = gpu_ctx.process(img, mask, p)
    finally:
        gpu_ctx.set_tuning(gpu_ctx.TUNE_CG_PRECOND, 0)
    hole = mask > 0
    o, r, t = out[hole][:, :3], g["hole"][:, :3], img[hole][:, :3]

    def psnr(a, b):
        mse = float(np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2))
        return 10 * np.log10(255.0 ** 2 / mse)
    row = {"workload": name, "psnr_gpu_vs_ref": psnr(o, r), "psnr_gpu_vs_truth": psnr(o, t),
           "psnr_ref_vs_truth": psnr(r, t), "cg_iterations": st["cg_iterations"]}
    row["gap_db"] = row["psnr_ref_vs_truth"] - row["psnr_gpu_vs_truth"]
    print(json.dumps(row))
    assert np.isfinite(out).all() and np.array_equal(out[~hole], img[~hole])
    assert row["psnr_gpu_vs_ref"] > 15.0 and row["gap_db"] < 3.0, row


def test_precond_knob(gpu_ctx):
    from nli_gb300 import NliError
    assert gpu_ctx.get_tuning(gpu_ctx.TUNE_CG_PRECOND) == 0
    with pytest.raises(NliError):
        gpu_ctx.set_tuning(gpu_ctx.TUNE_CG_PRECOND, 2)
