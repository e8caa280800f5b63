"""Parity of the CUDA path (through the C ABI) with the reference, via the
golden vectors it produced and the oracle restatement.

Bars (from the project's contract):
  * pyramid, masks, distance transform, coarsest fill, gradient: bit-exact;
  * patch distances: reference-exact kernel, within 1e-5 relative (expected
    bit-exact);
  * exhaustive NNF on a crop: bit-exact integer offsets;
  * PatchMatch: final NNF energy within 1% of the reference's;
  * updates given the reference's NNF: NL-means / NL-Poisson / NL-depth within
    1e-4 relative, NL-medians selects the same candidate value;
  * end-to-end: hole PSNR against the reference output reported, and the gap
    of hole PSNR against the ground truth bounded.
"""
import numpy as np
import pytest

from conftest import hole_psnr, params_from_array
from nli_gb300 import _abi
from nli_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def dparams(kind, sigma=10000.0, lam=0.05, lam_d=0.3, patch=9):
    return _abi.DistanceParams(kind, patch, patch, sigma, lam, lam_d)


def uparams(method, lam=0.05, lam_d=0.0, tol=1e-4, iters=1000, sigma=10000.0, patch=9):
    return _abi.UpdateParams(method, patch, patch, sigma, lam, lam_d, tol, iters)


def npy(t):
    return t.cpu().numpy()


def test_gradient(gpu_ctx, units):
    assert np.array_equal(npy(gpu_ctx.gradient(units["grad_in3"])), units["grad_out3"])
    assert np.array_equal(npy(gpu_ctx.gradient(units["grad_in4"])), units["grad_out4"])


def test_gaussian_weights(gpu_ctx, units):
    for i, (sx, sy, a, b) in enumerate(units["gw_args"]):
        assert np.array_equal(gpu_ctx.gaussian_weights(int(sx), int(sy), a, b), units["gw_%d" % i])


def test_distance_pairs(gpu_ctx, units):
    for i, (kind, C, sigma) in enumerate(units["dist_cases"]):
        d = dparams(int(kind), sigma=sigma, lam=0.05 if kind == 0 else 0.7, lam_d=0.2)
        got = npy(gpu_ctx.distance_pairs(d, units["dist_src_%d" % i], units["dist_tgt_%d" % i],
                                         units["dist_pairs_%d" % i]))
        ref = units["dist_out_%d" % i]
        rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-30)
        assert rel.max() <= 1e-5, (kind, C, rel.max())
        assert np.array_equal(got, ref), (kind, C, "not bit-exact", int((got != ref).sum()))


def test_bruteforce_nnf(gpu_ctx, units):
    nnf, d = gpu_ctx.bruteforce_nnf(dparams(0), units["bf_img"], units["bf_src"], units["bf_img"], units["bf_tgt"])
    assert np.array_equal(npy(nnf), units["bf_nnf"])
    assert np.array_equal(npy(d), units["bf_dist"])


def test_bruteforce_matches_oracle_rgbd(gpu_ctx, oracle):
    rng = np.random.default_rng(5)
    rgb, _ = wl.voronoi_texture(34, 28, 5, rng)
    img = np.concatenate([rgb, wl.depth_planes(34, 28, 3, rng)[..., None]], -1)
    mask = wl.disc_mask(34, 28, 4)
    s, t, _ = oracle.scale_masks(oracle.extended_domain(mask), 4, True)
    d = dparams(1, lam=1.0, lam_d=0.0)
    nnf, dd = gpu_ctx.bruteforce_nnf(d, img, s, img, t)
    rn, rd = oracle.bruteforce_nnf(d, img, s, img, t)
    assert np.array_equal(npy(nnf), rn) and np.array_equal(npy(dd), rd)


def test_masks_and_transforms(gpu_ctx, units):
    m = units["mask"]
    assert np.array_equal(npy(gpu_ctx.extended_domain(m, 9, 9)), units["ext"])
    assert np.array_equal(npy(gpu_ctx.extended_domain(m, 7, 5)), units["ext75"])
    for erode in (0, 1):
        s, t, e = gpu_ctx.scale_masks(units["ext"], 4, erode)
        assert np.array_equal(npy(s), units["src_%d" % erode]) and np.array_equal(npy(t), units["tgt_%d" % erode])
        if erode:
            assert e == bool(units["empty_%d" % erode])
    assert np.array_equal(npy(gpu_ctx.distance_transform(m)), units["dt"])
    for key, (dec, asy) in (("conf", (5.0, 0.1)), ("conf2", (2.5, 0.3))):
        got = npy(gpu_ctx.confidence_mask(m, dec, asy))
        ulp = np.abs(got.view(np.int32).astype(np.int64) - units[key].view(np.int32).astype(np.int64))
        assert ulp.max() <= 1, key  # exp rounded from double on the GPU, expf on the host


def test_pyramid(gpu_ctx, units):
    for i, f in enumerate((0.5623413, 0.7196857, 0.75, 0.5)):
        oi, om = gpu_ctx.downsample_with_mask(units["pyr_img"], units["pyr_mask"], f, 0.4, False)
        assert np.array_equal(npy(oi), units["down_img_%d" % i]), f
        assert np.array_equal(npy(om), units["down_mask_%d" % i]), f
        assert np.array_equal(npy(gpu_ctx.upsample(oi, 57, 45)), units["up_%d" % i]), f


def test_poisson_init(gpu_ctx, units):
    got = npy(gpu_ctx.poisson_init(units["pinit_in"], units["pinit_mask"]))
    assert np.array_equal(got, units["pinit_out"])


def test_poisson_init_sizes(gpu_ctx, oracle):
    rng = np.random.default_rng(3)
    for (w, h) in ((26, 26), (51, 51), (64, 48), (7, 5), (1, 1), (130, 77)):
        img = rng.uniform(0, 255, (h, w, 3)).astype(np.float32)
        mask = (rng.uniform(size=(h, w)) < 0.3).astype(np.uint8)
        if w * h == 1:
            mask[:] = 0
        assert np.array_equal(npy(gpu_ctx.poisson_init(img, mask)), oracle.poisson_init(img, mask)), (w, h)


def test_patchmatch_energy(gpu_ctx, units, oracle):
    """Final NNF energy within 1% of the reference's (random init and seeded init)."""
    p = wl.params("nlmeans")
    img, src, tgt = units["pm_img"], units["pm_src"], units["pm_tgt"]
    for init, ref_energy in ((None, units["pm_energy0"][-1]), (units["pm_nnf0"], units["pm_energy1"][-1])):
        nnf, d, e = gpu_ctx.patchmatch(p.distance, p.patchmatch, img, src, img, tgt, init=init)
        nnf = npy(nnf)
        # every target point matched inside the source, nothing else
        t = tgt.astype(bool)
        assert (nnf[~t] == -1).all()
        sx, sy = nnf[t][:, 0], nnf[t][:, 1]
        assert (src[sy, sx] == 1).all()
        # energy recomputed with the reference-exact distance
        e_exact = oracle.nnf_energy(p.distance, img, img, tgt, nnf)
        assert abs(e_exact - e) <= 1e-4 * e_exact
        assert e_exact <= 1.01 * ref_energy, (e_exact, ref_energy)


def test_patchmatch_deterministic(gpu_ctx, units):
    p = wl.params("nlmeans")
    img, src, tgt = units["pm_img"], units["pm_src"], units["pm_tgt"]
    gpu_ctx.set_seed(77)
    a = npy(gpu_ctx.patchmatch(p.distance, p.patchmatch, img, src, img, tgt)[0])
    gpu_ctx.set_seed(77)
    b = npy(gpu_ctx.patchmatch(p.distance, p.patchmatch, img, src, img, tgt)[0])
    assert np.array_equal(a, b)


def test_patchmatch_converges_to_bruteforce(gpu_ctx, units):
    """With enough sweeps on a small crop PatchMatch reaches the exhaustive
    minimum energy (within 1%)."""
    img, s, t = units["bf_img"], units["bf_src"], units["bf_tgt"]
    pm = _abi.PatchMatchParams(40, 30, -1)
    nnf, d, e = gpu_ctx.patchmatch(dparams(0), pm, img, s, img, t)
    e_bf = float(units["bf_dist"][t.astype(bool)].astype(np.float64).sum())
    assert e <= 1.01 * e_bf


def test_updates_given_reference_nnf(gpu_ctx, units):
    cur, img, mask, conf = units["upd_cur"], units["pm_img"], units["pm_mask"], units["upd_conf"]
    ext = npy(gpu_ctx.extended_domain(mask, 9, 9))
    nnf = units["pm_nnf1"]
    m = mask.astype(bool)
    for meth, lam in ((0, 0.05), (1, 0.05), (2, 0.05), (2, 1.0)):
        out, tot = gpu_ctx.update(uparams(meth, lam=lam), cur, img, mask, ext, nnf, conf)
        out = npy(out)
        key = "upd_%d_%g" % (meth, lam)
        ref = units[key]
        assert np.array_equal(out[~m], ref[~m]), key
        if meth == 0:
            assert np.array_equal(out, ref), key  # reference arithmetic reproduced
        elif meth == 1:
            assert np.array_equal(out, ref), key  # same selected candidate values
        else:
            rel = np.abs(out[m] - ref[m]) / np.maximum(np.abs(ref[m]), 1.0)
            assert rel.max() <= 1e-4, (key, rel.max())
        rt = float(units[key + "_total"])
        assert abs(tot - rt) <= 1e-4 * max(rt, 1.0), (key, tot, rt)
    out, tot = gpu_ctx.update(uparams(3, lam=1.0, lam_d=0.0, tol=1e-6), units["upd_cur4"], None, mask, ext, nnf,
                              conf, same_orig=True)
    out, ref = npy(out), units["upd_3"]
    rel = np.abs(out[m] - ref[m]) / np.maximum(np.abs(ref[m]), 1.0)
    assert rel.max() <= 1e-4, rel.max()


@pytest.mark.parametrize("name", ["means", "medians", "poisson", "depth", "avg_l2norm", "initnone"])
def test_process_small_vs_reference(gpu_ctx, small_cases, name):
    """End-to-end on small seeded cases: hole PSNR of the GPU output against
    the reference output, and against the ground truth compared with the
    reference's own."""
    p = params_from_array(small_cases[name + "_params"])
    img, mask, ref = small_cases[name + "_img"], small_cases[name + "_mask"], small_cases[name + "_out"]
    out, st = gpu_ctx.process(img, mask, p)
    m = mask.astype(bool)
    assert np.array_equal(out[~m], img[~m])
    assert np.isfinite(out).all()
    peak = 255.0
    vs_ref = hole_psnr(out, ref, mask, peak)
    gap = hole_psnr(ref, img, mask, peak) - hole_psnr(out, img, mask, peak)
    print("%s: PSNR(gpu, ref) = %.2f dB, PSNR gap vs ground truth = %.2f dB, iterations %s" % (
        name, vs_ref, gap, st["iterations"]))
    assert vs_ref > 20.0, vs_ref
    assert gap < 3.0, gap


def test_process_deterministic(gpu_ctx, small_cases):
    p = params_from_array(small_cases["poisson_params"])
    img, mask = small_cases["poisson_img"], small_cases["poisson_mask"]
    gpu_ctx.set_seed(5)
    a, _ = gpu_ctx.process(img, mask, p)
    gpu_ctx.set_seed(5)
    b, _ = gpu_ctx.process(img, mask, p)
    assert np.array_equal(a, b)


def test_empty_source_error(gpu_ctx):
    img, mask, p = wl.config1(seed=0, size=96)
    with pytest.raises(RuntimeError, match="Empty source mask"):
        gpu_ctx.process(img, mask, p)


def test_rgbd_requires_four_channels(gpu_ctx):
    img = np.zeros((40, 40, 3), np.float32)
    pairs = np.array([[10, 10, 20, 20]], np.int32)
    with pytest.raises(RuntimeError, match="Channels do not match"):
        gpu_ctx.distance_pairs(dparams(1), img, img, pairs)
