"""Errors against an FP64 oracle at full size (the 512x512 workload of the
NL-Poisson benchmark): the update step computed by the GPU and by the
reference's own arithmetic (the oracle restatement), both measured against
the FP64 re-expression of tests/update64.py (exact sparse solve for
NL-Poisson).  The GPU's error must not exceed the reference's by more than
the stated margins; the figures are printed."""
import numpy as np
import pytest
import torch

import update64

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
    return dict(p=p, u=u.cpu().numpy(), mask=mask, ext=ext.cpu().numpy(), nnf=nnf.cpu().numpy(),
                conf=conf.cpu().numpy())


def hole_rel(a, b, mask):
    m = mask != 0
    return float(np.abs(a[m].astype(np.float64) - b[m]).max() / np.abs(b[m]).max())


def test_nlmeans_vs_fp64(gpu_ctx, oracle, case):
    from nli_gb300 import workloads as wl
    upd = wl.params("nlmeans").update
    u, mask, ext, nnf, conf = case["u"], case["mask"], case["ext"], case["nnf"], case["conf"]
    ours = gpu_ctx.update(upd, u, u, mask, ext, nnf, conf)[0].cpu().numpy()
    ref = oracle.update(upd, u, u, mask, ext, nnf, conf)[0]
    exact = update64.means(torch.from_numpy(u).double(), upd.sigma, nnf, mask != 0, conf.astype(np.float64)).numpy()
    e_ours, e_ref = hole_rel(ours, exact, mask), hole_rel(ref, exact, mask)
    print("NL-means 512x512 vs FP64: GPU %.3g, reference arithmetic %.3g (max relative, hole)" % (e_ours, e_ref))
    assert np.array_equal(ours, ref)  # the reference's float arithmetic, reproduced
    assert e_ours < 1e-5


@pytest.mark.parametrize("tol", [1e-4, 1e-6])
def test_nlpoisson_vs_fp64(gpu_ctx, oracle, case, tol):
    """CG tolerance 1e-4 (the benchmark's) and 1e-6 (the command line's):
    both solvers stop at the same relative residual, so their distance to
    the exact FP64 solution is of the same size."""
    from nli_gb300 import workloads as wl
    upd = wl.params("nlpoisson", cg_tol=tol).update
    u, mask, ext, nnf, conf = case["u"], case["mask"], case["ext"], case["nnf"], case["conf"]
    ours = gpu_ctx.update(upd, u, u, mask, ext, nnf, conf)[0].cpu().numpy()
    ref = oracle.update(upd, u, u, mask, ext, nnf, conf)[0]
    exact = update64.poisson(torch.from_numpy(u).double(), upd.lambda_, upd.sigma, nnf, mask != 0, ext,
                             conf.astype(np.float64), solver="sparse").numpy()
    e_ours, e_ref = hole_rel(ours, exact, mask), hole_rel(ref, exact, mask)
    print("NL-Poisson 512x512, CG tol %g, vs FP64 exact solve: GPU %.3g, reference %.3g (max relative, hole)"
          % (tol, e_ours, e_ref))
    assert e_ours <= 3.0 * e_ref + 1e-5, (e_ours, e_ref)
