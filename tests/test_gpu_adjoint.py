"""Adjoint kernels of the image update (NNF held fixed): gradients with
respect to the image, lambda and the patch-weight sigma, from the CUDA
backward (through the torch.autograd.Function), against an FP64 PyTorch
re-expression of the same step (tests/update64.py): its autograd gradients
at small sizes and FP64 central finite differences (step 1e-3) along random
directions.  Tolerance: 1e-4 relative."""
import numpy as np
import pytest
import torch

import update64

pytestmark = pytest.mark.gpu


def make_case(ctx, size, seed, method, sigma=10000.0, lam=0.05):
    from nli_gb300 import workloads as wl
    img, mask, _ = wl.config2(seed=seed, size=size, scales=3)
    p = wl.params(method, scales=3, coarse=0.5, iters=10, cg_tol=1e-12, cg_iters=1000, psigma=sigma, lam=lam)
    ext = ctx.extended_domain(mask, 9, 9)
    src, tgt, _ = ctx.scale_masks(ext, 4, True)
    u = ctx.poisson_init(img, mask)  # hole filled smoothly, as the coarsest level starts
    ctx.set_seed(seed)
    nnf, _, _ = ctx.patchmatch(p.distance, p.patchmatch, u, src, u, tgt)
    conf = ctx.confidence_mask(mask, 5.0, 0.1)
    rng = np.random.default_rng(seed + 1)
    target = torch.from_numpy(rng.uniform(0, 255, img.shape).astype(np.float32)).cuda()
    return dict(p=p, u=u, mask=mask, ext=ext, nnf=nnf, conf=conf, target=target, hole=torch.from_numpy(mask != 0).cuda())


def ours(ctx, case, lam, sigma):
    from nli_gb300.autograd import image_update
    u = case["u"].detach().clone().requires_grad_(True)
    lt = torch.tensor(lam, dtype=torch.float64, requires_grad=True)
    st = torch.tensor(sigma, dtype=torch.float64, requires_grad=True)
    out = image_update(ctx, case["p"].update, u, lt, st, case["mask"], case["ext"], case["nnf"], case["conf"])
    loss = (((out - case["target"]) ** 2) * case["hole"][..., None]).sum()
    loss.backward()
    return out.detach(), u.grad.double().cpu(), float(lt.grad), float(st.grad)


def ref64(case, method, lam, sigma, u=None, solver="dense"):
    """(loss, out) of the FP64 re-expression; u defaults to the case image."""
    u = case["u"].double().cpu() if u is None else u
    nnf = case["nnf"].cpu().numpy().reshape(u.shape[0], u.shape[1], 2)
    dom = case["mask"] != 0
    ext = case["ext"].cpu().numpy() if torch.is_tensor(case["ext"]) else case["ext"]
    conf = case["conf"].double().cpu().numpy()
    if method == "nlmeans":
        out = update64.means(u, sigma, nnf, dom, conf)
    else:
        out = update64.poisson(u, lam, sigma, nnf, dom, ext, conf, solver=solver)
    t = case["target"].double().cpu()
    loss = (((out - t) ** 2) * torch.from_numpy(dom)[..., None]).sum()
    return loss, out


def rel(a, b):
    return float(torch.linalg.norm(a - b) / max(float(torch.linalg.norm(b)), 1e-300))


@pytest.mark.parametrize("method,sigma", [("nlmeans", 10000.0), ("nlmeans", 3.0), ("nlpoisson", 10000.0),
                                          ("nlpoisson", 3.0)])
def test_gradients_match_fp64_autograd(gpu_ctx, method, sigma):
    case = make_case(gpu_ctx, 64, 21, method, sigma=sigma)
    lam = 0.05
    out, gu, gl, gs = ours(gpu_ctx, case, lam, sigma)
    u64 = case["u"].double().cpu().requires_grad_(True)
    l64 = torch.tensor(lam, dtype=torch.float64, requires_grad=True)
    s64 = torch.tensor(sigma, dtype=torch.float64, requires_grad=True)
    loss, out64 = ref64(case, method, l64, s64, u=u64)
    loss.backward()
    print("64x64 %s sigma %g: out %.3g, d/du %.3g, d/dlambda %.3g, d/dsigma %.3g (relative to FP64)" % (
        method, sigma, rel(out.double().cpu(), out64.detach()), rel(gu, u64.grad),
        abs(gl - float(l64.grad)) / abs(float(l64.grad)) if l64.grad is not None else 0.0,
        abs(gs - float(s64.grad)) / abs(float(s64.grad))))
    assert rel(out.double().cpu(), out64.detach()) < 1e-5
    assert rel(gu, u64.grad) < 1e-4, rel(gu, u64.grad)
    if method == "nlmeans":
        assert gl == 0.0  # NL-means does not depend on lambda
    else:
        assert abs(gl - float(l64.grad)) <= 1e-4 * abs(float(l64.grad)), (gl, float(l64.grad))
    assert abs(gs - float(s64.grad)) <= 1e-4 * abs(float(s64.grad)) + 1e-12, (gs, float(s64.grad))


@pytest.mark.parametrize("method", ["nlmeans", "nlpoisson"])
def test_directional_finite_differences(gpu_ctx, method):
    """64 random directions over (known pixels, lambda, sigma); central
    differences of the FP64 loss with step 1e-3."""
    sigma, lam = 3.0, 0.05
    case = make_case(gpu_ctx, 48, 22, method, sigma=sigma)
    _, gu, gl, gs = ours(gpu_ctx, case, lam, sigma)
    known = torch.from_numpy(case["mask"] == 0)[..., None].double()
    u0 = case["u"].double().cpu()
    rng = np.random.default_rng(5)
    eps = 1e-3
    worst = 0.0
    for _ in range(64):
        vu = torch.from_numpy(rng.standard_normal(u0.shape)) * known
        vl = float(rng.standard_normal()) * (0.01 if method == "nlpoisson" else 0.0)
        vs = float(rng.standard_normal())
        with torch.no_grad():
            lp, _ = ref64(case, method, lam + eps * vl, sigma + eps * vs, u=u0 + eps * vu)
            lm, _ = ref64(case, method, lam - eps * vl, sigma - eps * vs, u=u0 - eps * vu)
        fd = float(lp - lm) / (2 * eps)
        terms = (float((gu * vu).sum()), gl * vl, gs * vs)
        an = sum(terms)
        # relative to the size of the directional terms: a random direction
        # can make the image and sigma parts cancel almost exactly
        scale = max(abs(fd), sum(abs(t) for t in terms), 1e-9)
        worst = max(worst, abs(an - fd) / scale)
    print("48x48 %s: worst relative error over 64 directions %.3g" % (method, worst))
    assert worst < 1e-4, worst


@pytest.mark.parametrize("method", ["nlmeans", "nlpoisson"])
def test_full_size_512_finite_differences(gpu_ctx, method):
    """The differentiation workload at full size: 512x512 Voronoi image,
    ~15% ellipse hole, NNF from a seeded PatchMatch run, lambda 0.05,
    sigma 10000; gradients against FP64 central differences (step 1e-3,
    the vectorised FP64 evaluation with a sparse direct solve) along 64
    random directions over (known pixels, lambda, sigma)."""
    sigma, lam = 10000.0, 0.05
    case = make_case(gpu_ctx, 512, 4, method, sigma=sigma)
    _, gu, gl, gs = ours(gpu_ctx, case, lam, sigma)
    dom = case["mask"] != 0
    u0 = case["u"].double().cpu().numpy()
    H, W = dom.shape
    nnf = case["nnf"].cpu().numpy().reshape(H, W, 2)
    plan = update64.Plan(nnf, dom, case["ext"].cpu().numpy(), case["conf"].double().cpu().numpy())
    t = case["target"].double().cpu().numpy()
    gun = gu.numpy()

    def loss(u, l, s):
        out = update64.means_fast(u, s, plan) if method == "nlmeans" else update64.poisson_fast(u, l, s, plan)
        return float((((out - t) ** 2) * dom[..., None]).sum())

    rng = np.random.default_rng(6)
    eps = 1e-3
    worst = 0.0
    for _ in range(64):
        vu = rng.standard_normal(u0.shape) * (~dom)[..., None]
        vl = float(rng.standard_normal()) * (0.01 if method == "nlpoisson" else 0.0)
        vs = float(rng.standard_normal()) * 1e3
        fd = (loss(u0 + eps * vu, lam + eps * vl, sigma + eps * vs) -
              loss(u0 - eps * vu, lam - eps * vl, sigma - eps * vs)) / (2 * eps)
        terms = (float((gun * vu).sum()), gl * vl, gs * vs)
        scale = max(abs(fd), sum(abs(x) for x in terms), 1e-9)
        worst = max(worst, abs(sum(terms) - fd) / scale)
    print("512x512 %s: worst relative error over 64 directions %.3g" % (method, worst))
    assert worst < 1e-4, worst


@pytest.mark.parametrize("method", ["nlmeans", "nlpoisson"])
def test_replayed_steps(gpu_ctx, method):
    """Three update steps replayed with one checkpointed NNF: gradients
    through the chain against the chained FP64 re-expression (autograd) and
    FP64 central differences along 8 random directions."""
    from nli_gb300.autograd import replay_updates
    sigma, lam, steps = 3.0, 0.05, 3
    case = make_case(gpu_ctx, 48, 23, method, sigma=sigma)
    u = case["u"].detach().clone().requires_grad_(True)
    lt = torch.tensor(lam, dtype=torch.float64, requires_grad=True)
    st = torch.tensor(sigma, dtype=torch.float64, requires_grad=True)
    out = replay_updates(gpu_ctx, case["p"].update, u, lt, st, case["mask"], case["ext"], case["nnf"], case["conf"],
                         steps=steps)
    loss = (((out - case["target"]) ** 2) * case["hole"][..., None]).sum()
    loss.backward()
    gu, gl, gs = u.grad.double().cpu(), float(lt.grad), float(st.grad)

    nnf = case["nnf"].cpu().numpy().reshape(48, 48, 2)
    dom = case["mask"] != 0
    ext = case["ext"].cpu().numpy()
    conf = case["conf"].double().cpu().numpy()
    t = case["target"].double().cpu()

    def f64(u0, l, s):
        x = u0
        for _ in range(steps):
            x = update64.means(x, s, nnf, dom, conf) if method == "nlmeans" else \
                update64.poisson(x, l, s, nnf, dom, ext, conf)
        return (((x - t) ** 2) * torch.from_numpy(dom)[..., None]).sum()

    u64 = case["u"].double().cpu().requires_grad_(True)
    l64 = torch.tensor(lam, dtype=torch.float64, requires_grad=True)
    s64 = torch.tensor(sigma, dtype=torch.float64, requires_grad=True)
    f64(u64, l64, s64).backward()
    assert rel(gu, u64.grad) < 1e-4, rel(gu, u64.grad)
    if method == "nlpoisson":
        assert abs(gl - float(l64.grad)) <= 1e-4 * abs(float(l64.grad))
    assert abs(gs - float(s64.grad)) <= 1e-4 * abs(float(s64.grad))
    rng = np.random.default_rng(8)
    u0 = case["u"].double().cpu()
    known = torch.from_numpy(~dom)[..., None].double()
    eps, worst = 1e-3, 0.0
    for _ in range(8):
        vu = torch.from_numpy(rng.standard_normal(u0.shape)) * known
        vl = float(rng.standard_normal()) * (0.01 if method == "nlpoisson" else 0.0)
        vs = float(rng.standard_normal())
        with torch.no_grad():
            fd = float(f64(u0 + eps * vu, lam + eps * vl, sigma + eps * vs) -
                       f64(u0 - eps * vu, lam - eps * vl, sigma - eps * vs)) / (2 * eps)
        terms = (float((gu * vu).sum()), gl * vl, gs * vs)
        worst = max(worst, abs(sum(terms) - fd) / max(abs(fd), sum(abs(x) for x in terms)))
    print("%d replayed %s steps: worst relative error %.3g" % (steps, method, worst))
    assert worst < 1e-4, worst


def make_depth_case(ctx, size, seed, sigma, lam_rgb, lam_d):
    """An RGB-D image (Voronoi colours, depth planes in metres), its hole, and
    the NNF of a seeded L2 RGBD PatchMatch run; NL-depth update parameters
    with lambda_rgb / lambda_d (patch_non_local_depth.cpp:36-55)."""
    from nli_gb300 import workloads as wl
    rng = np.random.default_rng(seed)
    rgb, _ = wl.voronoi_texture(size, size, 10, rng)
    depth = wl.depth_planes(size, size, 4, rng)
    img = np.concatenate([rgb, depth[..., None]], -1).astype(np.float32)
    mask = wl.ellipse_mask(size, size, 2, 0.12, rng)
    p = wl.params("nldepth", scales=3, coarse=0.5, iters=10, cg_tol=1e-12, cg_iters=1000, psigma=sigma,
                  lam_r=lam_rgb, lam_d=lam_d)
    ext = ctx.extended_domain(mask, 9, 9)
    src, tgt, _ = ctx.scale_masks(ext, 4, True)
    u = ctx.poisson_init(img, mask)
    ctx.set_seed(seed)
    nnf, _, _ = ctx.patchmatch(p.distance, p.patchmatch, u, src, u, tgt)
    conf = ctx.confidence_mask(mask, 5.0, 0.1)
    scale = np.array([255.0, 255.0, 255.0, 5.0], np.float32)
    target = torch.from_numpy((rng.uniform(0, 1, img.shape) * scale).astype(np.float32)).cuda()
    return dict(p=p, u=u, mask=mask, ext=ext, nnf=nnf, conf=conf, target=target,
                hole=torch.from_numpy(mask != 0).cuda())


def ours_depth(ctx, case, lam, lam_d, sigma):
    from nli_gb300.autograd import image_update
    u = case["u"].detach().clone().requires_grad_(True)
    lt = torch.tensor(lam, dtype=torch.float64, requires_grad=True)
    ldt = torch.tensor(lam_d, dtype=torch.float64, requires_grad=True)
    st = torch.tensor(sigma, dtype=torch.float64, requires_grad=True)
    out = image_update(ctx, case["p"].update, u, lt, st, case["mask"], case["ext"], case["nnf"], case["conf"],
                       lam_d=ldt)
    loss = (((out - case["target"]) ** 2) * case["hole"][..., None]).sum()
    loss.backward()
    return out.detach(), u.grad.double().cpu(), float(lt.grad), float(ldt.grad), float(st.grad)


def ref64_depth(case, lam, lam_d, sigma, u=None):
    u = case["u"].double().cpu() if u is None else u
    H, W = case["mask"].shape
    nnf = case["nnf"].cpu().numpy().reshape(H, W, 2)
    dom = case["mask"] != 0
    out = update64.poisson(u, None, sigma, nnf, dom, case["ext"].cpu().numpy(), case["conf"].double().cpu().numpy(),
                           lam_channels=[lam, lam, lam, lam_d])
    t = case["target"].double().cpu()
    return (((out - t) ** 2) * torch.from_numpy(dom)[..., None]).sum(), out


@pytest.mark.parametrize("sigma", [10000.0, 3.0])
def test_depth_gradients_match_fp64_autograd(gpu_ctx, sigma):
    """NL-depth (one solve, lambda_rgb on the colour channels, lambda_d on
    depth): dL/du, dL/dlambda_rgb, dL/dlambda_d and dL/dsigma against FP64
    autograd."""
    lam, lam_d = 0.3, 0.6
    case = make_depth_case(gpu_ctx, 56, 31, sigma, lam, lam_d)
    out, gu, gl, gld, gs = ours_depth(gpu_ctx, case, lam, lam_d, sigma)
    u64 = case["u"].double().cpu().requires_grad_(True)
    l64 = torch.tensor(lam, dtype=torch.float64, requires_grad=True)
    ld64 = torch.tensor(lam_d, dtype=torch.float64, requires_grad=True)
    s64 = torch.tensor(sigma, dtype=torch.float64, requires_grad=True)
    loss, out64 = ref64_depth(case, l64, ld64, s64, u=u64)
    loss.backward()
    errs = (rel(out.double().cpu(), out64.detach()), rel(gu, u64.grad),
            abs(gl - float(l64.grad)) / abs(float(l64.grad)), abs(gld - float(ld64.grad)) / abs(float(ld64.grad)),
            abs(gs - float(s64.grad)) / max(abs(float(s64.grad)), 1e-300))
    print("56x56 NL-depth sigma %g: out %.3g, d/du %.3g, d/dlambda_rgb %.3g, d/dlambda_d %.3g, d/dsigma %.3g" % (
        (sigma,) + errs))
    assert errs[0] < 1e-5
    assert errs[1] < 1e-4 and errs[2] < 1e-4 and errs[3] < 1e-4
    assert abs(gs - float(s64.grad)) <= 1e-4 * abs(float(s64.grad)) + 1e-12


def test_depth_directional_finite_differences(gpu_ctx):
    """32 random directions over (known pixels, lambda_rgb, lambda_d, sigma);
    central differences of the FP64 loss, step 1e-3."""
    sigma, lam, lam_d = 3.0, 0.3, 0.6
    case = make_depth_case(gpu_ctx, 40, 32, sigma, lam, lam_d)
    _, gu, gl, gld, gs = ours_depth(gpu_ctx, case, lam, lam_d, sigma)
    known = torch.from_numpy(case["mask"] == 0)[..., None].double()
    u0 = case["u"].double().cpu()
    rng = np.random.default_rng(9)
    eps, worst = 1e-3, 0.0
    for _ in range(32):
        vu = torch.from_numpy(rng.standard_normal(u0.shape)) * known
        vl, vld, vs = (float(x) for x in rng.standard_normal(3) * np.array([0.01, 0.01, 1.0]))
        with torch.no_grad():
            lp, _ = ref64_depth(case, lam + eps * vl, lam_d + eps * vld, sigma + eps * vs, u=u0 + eps * vu)
            lm, _ = ref64_depth(case, lam - eps * vl, lam_d - eps * vld, sigma - eps * vs, u=u0 - eps * vu)
        fd = float(lp - lm) / (2 * eps)
        terms = (float((gu * vu).sum()), gl * vl, gld * vld, gs * vs)
        scale = max(abs(fd), sum(abs(t) for t in terms), 1e-9)
        worst = max(worst, abs(sum(terms) - fd) / scale)
    print("40x40 NL-depth: worst relative error over 32 directions %.3g" % worst)
    assert worst < 1e-4, worst


@pytest.mark.parametrize("method", ["nlmeans", "nlpoisson"])
def test_replay_across_two_scales(gpu_ctx, method):
    """A two-scale replay with the NNF pyramid a process() run checkpoints
    (keep_intermediate): two update steps on the coarse scale with its final
    NNF, the result upsampled into the fine scale's hole as
    propagate_weights does, two update steps on the fine scale with its NNF.
    Gradients through the whole chain against the chained FP64
    re-expression (autograd) and FP64 central differences.  The fine steps
    read the fine image only at known pixels (the sources of an NNF are
    complete patches outside the hole), so no gradient reaches the coarse
    scale: it must be exactly zero there, as in FP64."""
    from nli_gb300 import workloads as wl
    from nli_gb300.autograd import replay_updates
    sigma, lam, steps = 3.0, 0.05, 2
    img, mask, _ = wl.config2(seed=33, size=56, scales=2)
    p = wl.params(method, scales=2, coarse=0.6, iters=6, cg_tol=1e-12, cg_iters=1000, psigma=sigma, lam=lam)
    gpu_ctx.keep_intermediate(True)
    try:
        gpu_ctx.set_seed(34)
        gpu_ctx.process(img, mask, p)
        inputs = gpu_ctx.intermediate(gpu_ctx.INTER_INPUT)
        masks = gpu_ctx.intermediate(gpu_ctx.INTER_MASK)
        nnfs = gpu_ctx.intermediate(gpu_ctx.INTER_NNF)  # coarsest first
    finally:
        gpu_ctx.keep_intermediate(False)
    (Hc, Wc), (Hf, Wf) = masks[1].shape, masks[0].shape
    # the nearest-neighbour upsampling of the library as a gather index
    idx_img = np.arange(Hc * Wc, dtype=np.float32).reshape(Hc, Wc, 1)
    up_idx = torch.from_numpy(gpu_ctx.upsample(idx_img, Wf, Hf).cpu().numpy()[..., 0].round().astype(np.int64))
    mc, mf = masks[1], masks[0]
    lev = []
    for m, nnf in ((mc, nnfs[0]), (mf, nnfs[1])):
        ext = gpu_ctx.extended_domain(m, 9, 9)
        conf = gpu_ctx.confidence_mask(m, 5.0, 0.1)
        lev.append((m, ext, torch.from_numpy(nnf).cuda(), conf))
    uc0 = gpu_ctx.poisson_init(inputs[1], mc)
    rng = np.random.default_rng(35)
    target = torch.from_numpy(rng.uniform(0, 255, inputs[0].shape).astype(np.float32)).cuda()
    hole_f = torch.from_numpy(mf != 0).cuda()
    fine_in = torch.from_numpy(inputs[0]).cuda()
    # ours
    uc = uc0.detach().clone().requires_grad_(True)
    uf_known = fine_in.clone().requires_grad_(True)
    lt = torch.tensor(lam, dtype=torch.float64, requires_grad=True)
    st = torch.tensor(sigma, dtype=torch.float64, requires_grad=True)
    m_c, e_c, n_c, c_c = lev[0]
    m_f, e_f, n_f, c_f = lev[1]
    oc = replay_updates(gpu_ctx, p.update, uc, lt, st, m_c, e_c, n_c, c_c, steps=steps)
    up = oc.reshape(-1, 3)[up_idx.cuda().reshape(-1)].reshape(Hf, Wf, 3)
    uf = torch.where(hole_f[..., None], up, uf_known)
    of = replay_updates(gpu_ctx, p.update, uf, lt, st, m_f, e_f, n_f, c_f, steps=steps)
    loss = (((of - target) ** 2) * hole_f[..., None]).sum()
    loss.backward()
    g_c, g_f = uc.grad.double().cpu(), uf_known.grad.double().cpu()
    gl, gs = float(lt.grad), float(st.grad)
    assert float(g_c.abs().max()) == 0.0  # nothing reaches the coarse scale

    # FP64 chain
    np_c = [a if not torch.is_tensor(a) else a.cpu().numpy() for a in lev[0]]
    np_f = [a if not torch.is_tensor(a) else a.cpu().numpy() for a in lev[1]]
    t64, hole64 = target.double().cpu(), torch.from_numpy(mf != 0)

    def step64(x, lv, l, s):
        m, ext, nnf, conf = lv
        H, W = m.shape
        nnf = nnf.reshape(H, W, 2)
        conf = conf.astype(np.float64)
        if method == "nlmeans":
            return update64.means(x, s, nnf, m != 0, conf)
        return update64.poisson(x, l, s, nnf, m != 0, ext, conf)

    def chain64(uc_, uf_, l, s):
        x = uc_
        for _ in range(steps):
            x = step64(x, np_c, l, s)
        u2 = torch.where(hole64[..., None], x.reshape(-1, 3)[up_idx.reshape(-1)].reshape(Hf, Wf, 3), uf_)
        for _ in range(steps):
            u2 = step64(u2, np_f, l, s)
        return (((u2 - t64) ** 2) * hole64[..., None]).sum()

    uc64 = uc0.double().cpu().requires_grad_(True)
    uf64 = fine_in.double().cpu().requires_grad_(True)
    l64 = torch.tensor(lam, dtype=torch.float64, requires_grad=True)
    s64 = torch.tensor(sigma, dtype=torch.float64, requires_grad=True)
    chain64(uc64, uf64, l64, s64).backward()
    assert float(uc64.grad.abs().max()) < 1e-9 * float(uf64.grad.abs().max())
    assert rel(g_f, uf64.grad) < 1e-4, rel(g_f, uf64.grad)
    if method == "nlpoisson":
        assert abs(gl - float(l64.grad)) <= 1e-4 * abs(float(l64.grad))
    assert abs(gs - float(s64.grad)) <= 1e-4 * abs(float(s64.grad))
    known = torch.from_numpy(mf == 0)[..., None].double()
    u0c, u0f = uc0.double().cpu(), fine_in.double().cpu()
    eps, worst = 1e-3, 0.0
    for _ in range(6):
        vf = torch.from_numpy(rng.standard_normal(u0f.shape)) * known
        vl = float(rng.standard_normal()) * (0.01 if method == "nlpoisson" else 0.0)
        vs = float(rng.standard_normal())
        with torch.no_grad():
            fd = float(chain64(u0c, u0f + eps * vf, lam + eps * vl, sigma + eps * vs) -
                       chain64(u0c, u0f - eps * vf, lam - eps * vl, sigma - eps * vs)) / (2 * eps)
        terms = (float((g_f * vf).sum()), gl * vl, gs * vs)
        worst = max(worst, abs(sum(terms) - fd) / max(abs(fd), sum(abs(x) for x in terms)))
    print("two-scale %s replay: worst relative error %.3g" % (method, worst))
    assert worst < 1e-4, worst
