"""Generates the golden vectors in tests/golden/ by running the REFERENCE
implementation (its unmodified sources, compiled by oracle/build.py into
oracle/_ref/libnliref.so) on small seeded inputs.

    python tests/golden/make_golden.py            # unit + small process cases
    python tests/golden/make_golden.py --full     # full-size configs 1-3 (slow)
    python tests/golden/make_golden.py --full --seeds 1,2 --skip-units config2
                                                  # the same configurations for other
                                                  # input seeds (one file per seed)
    python tests/golden/make_golden.py --batch 8,15 --skip-units
                                                  # items of the seeded 64-image uneven
                                                  # batch (see batch_items)

Full-size configurations run the serial reference build (srand(101)).  The
uneven-batch items are too large for the serial build (their pyramids have up
to 16 nearly full-size scales), so they run the pinned restatement with the
reference's OpenMP PatchMatch (the variant the reference's own Release build
compiles), its thread seeds fixed by orc_set_parallel_seed and 4 threads, so
that a rerun reproduces them.

Only runs where the reference sources are present.  The fixtures are
committed; the tests read them and never need the reference.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build as oracle_build  # noqa: E402
import __graft_entry__ as ge  # noqa: E402

pkg = ge.package()
from nli_gb300 import workloads as wl  # noqa: E402
from nli_gb300 import _abi  # noqa: E402
from oracle import oracle as O  # noqa: E402


def quiet(fn, *a, **k):
    """Runs fn with the process's stdout (fd 1) sent to /dev/null: the
    reference prints progress lines."""
    sys.stdout.flush()
    saved = os.dup(1)
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)
    try:
        return fn(*a, **k)
    finally:
        import ctypes
        ctypes.CDLL(None).fflush(None)
        os.dup2(saved, 1)
        os.close(devnull)
        os.close(saved)


def dparams(kind, sigma=10000.0, lam=0.05, lam_d=0.3, patch=9):
    return _abi.DistanceParams(kind, patch, patch, sigma, lam, lam_d)


def uparams(method, lam=0.05, lam_d=0.0, tol=1e-4, iters=1000, sigma=10000.0, patch=9):
    return _abi.UpdateParams(method, patch, patch, sigma, lam, lam_d, tol, iters)


def small_configs():
    """(name, image, mask, params) of the small end-to-end cases."""
    out = []
    img, mask, p = wl.config1(seed=11, size=80)
    p.scales, p.subsampling_rate = 3, _abi.subsampling_rate(0.4, 3)
    out.append(("means", img, mask, p))
    img, mask, p = wl.config1(seed=12, size=64)
    p.scales, p.subsampling_rate = 2, _abi.subsampling_rate(0.6, 2)
    p.update.method, p.distance.kind = _abi.NLI_UPDATE_MEDIANS, _abi.NLI_DIST_L1_NORM
    out.append(("medians", img, mask, p))
    img, mask, p = wl.config2(seed=13, size=72, scales=3)
    p.subsampling_rate, p.iterations = _abi.subsampling_rate(0.45, 3), 25
    out.append(("poisson", img, mask, p))
    img, mask, p = wl.config3(seed=14, w=80, h=64, scales=3)
    p.subsampling_rate, p.iterations = _abi.subsampling_rate(0.45, 3), 15
    out.append(("depth", img, mask, p))
    img, mask, p = wl.config1(seed=15, size=64)
    p.scales, p.subsampling_rate, p.init = 2, _abi.subsampling_rate(0.6, 2), _abi.NLI_INIT_AVG
    p.distance.kind = _abi.NLI_DIST_L2_NORM
    out.append(("avg_l2norm", img, mask, p))
    img, mask, p = wl.config1(seed=16, size=64)
    p.scales, p.subsampling_rate, p.init = 2, _abi.subsampling_rate(0.6, 2), _abi.NLI_INIT_NONE
    out.append(("initnone", img, mask, p))
    return out


def params_to_array(p):
    """Flat float64 record of a ProcessParams (tests rebuild it)."""
    return np.array([p.distance.kind, p.distance.patch_x, p.distance.patch_y, p.distance.sigma, p.distance.lambda_,
                     p.distance.lambda_d, p.patchmatch.iterations, p.patchmatch.random_shots, p.patchmatch.window,
                     p.update.method, p.update.patch_x, p.update.patch_y, p.update.sigma, p.update.lambda_,
                     p.update.lambda_d, p.update.cg_tol, p.update.cg_iters, p.iterations, p.tolerance, p.scales,
                     p.subsampling_rate, p.conf_decay_time, p.conf_asymptotic, p.init], np.float64)


def unit_cases(ref):
    rng = np.random.default_rng(2024)
    g = {}
    # gradient
    im3 = rng.uniform(0, 255, (23, 31, 3)).astype(np.float32)
    im4 = rng.uniform(0, 5, (17, 19, 4)).astype(np.float32)
    g["grad_in3"], g["grad_out3"] = im3, ref.gradient(im3)
    g["grad_in4"], g["grad_out4"] = im4, ref.gradient(im4)
    # Gaussian weights
    gw = [(9, 9, 10000.0, 10000.0), (9, 9, 1.7, 1.7), (7, 5, 2.0, 3.0), (9, 1, 0.62 * 1.03, 0.0),
          (9, 1, 0.8, 0.0), (5, 5, 0.5, 0.5)]
    g["gw_args"] = np.array(gw, np.float64)
    for i, (sx, sy, a, b) in enumerate(gw):
        g["gw_%d" % i] = ref.gaussian_weights(int(sx), int(sy), a, b)
    # distances: (kind, C, sigma)
    dcases = [(0, 3, 10000.0), (0, 3, 2.0), (0, 1, 10000.0), (0, 4, 3.0), (1, 4, 10000.0), (2, 3, 10000.0),
              (3, 3, 4.0)]
    g["dist_cases"] = np.array(dcases, np.float64)
    for i, (kind, C, sigma) in enumerate(dcases):
        src = rng.uniform(0, 255, (36, 44, C)).astype(np.float32)
        tgt = rng.uniform(0, 255, (30, 40, C)).astype(np.float32)
        pairs = np.stack([rng.integers(4, 40, 300), rng.integers(4, 32, 300), rng.integers(4, 36, 300),
                          rng.integers(4, 26, 300)], 1).astype(np.int32)
        d = dparams(int(kind), sigma=sigma, lam=0.05 if kind == 0 else 0.7, lam_d=0.2)
        g["dist_src_%d" % i], g["dist_tgt_%d" % i], g["dist_pairs_%d" % i] = src, tgt, pairs
        g["dist_out_%d" % i] = ref.distance_pairs(d, src, tgt, pairs)
    # scale masks / ext domain / DT / confidence on a ragged mask touching the border
    m = wl.ellipse_mask(53, 41, 4, 0.2, rng, margin=0.0)
    m[0, 10:14] = 1
    m[-1, :3] = 1
    g["mask"] = m
    g["ext"] = ref.extended_domain(m, 9, 9)
    g["ext75"] = ref.extended_domain(m, 7, 5)
    for erode in (0, 1):
        s, t, e = ref.scale_masks(g["ext"], 4, erode)
        g["src_%d" % erode], g["tgt_%d" % erode], g["empty_%d" % erode] = s, t, np.array(e)
    g["dt"] = ref.distance_transform(m)
    g["conf"] = ref.confidence_mask(m, 5.0, 0.1)
    g["conf2"] = ref.confidence_mask(m, 2.5, 0.3)
    # pyramid
    img = wl.voronoi_texture(57, 45, 12, rng)[0]
    g["pyr_img"], g["pyr_mask"] = img, m[:45, :53].copy() if False else wl.ellipse_mask(57, 45, 3, 0.15, rng)
    for i, f in enumerate((0.5623413, 0.7196857, 0.75, 0.5)):
        oi, om = ref.downsample_with_mask(g["pyr_img"], g["pyr_mask"], f, 0.4, False)
        g["down_img_%d" % i], g["down_mask_%d" % i] = oi, om
        g["up_%d" % i] = ref.upsample(oi, 57, 45)
    # coarsest Poisson fill
    g["pinit_in"], g["pinit_mask"] = g["down_img_0"], g["down_mask_0"]
    g["pinit_out"] = ref.poisson_init(g["down_img_0"], g["down_mask_0"])
    # colour conversions of the command-line caller: every 8-bit grey level
    # and seeded random colours (0..255) through rgb_to_lab and back
    lrng = np.random.default_rng(77)
    lv = np.arange(256, dtype=np.float32)
    rgb = np.concatenate([np.stack([lv, lv, lv], -1)[None], lrng.uniform(0, 255, (1, 256, 3)).astype(np.float32),
                          np.round(lrng.uniform(0, 255, (1, 256, 3))).astype(np.float32)], axis=1)
    g["lab_rgb_in"] = rgb
    g["lab_out"] = ref.rgb_to_lab(rgb)
    g["lab_rgb_back"] = ref.lab_to_rgb(g["lab_out"])
    # a 4-channel (L*a*b* + depth) input: the reference's lab_to_rgb reads its
    # separated copy after that copy is destroyed (io_utility.cpp:303-307),
    # so its output is not stored; the intended result drops the depth
    g["lab4_in"] = np.concatenate([g["lab_out"], lrng.uniform(0.5, 5, rgb.shape[:2] + (1,)).astype(np.float32)], -1)
    # PatchMatch + updates on one 64x64 scale
    img, mask, p = wl.config1(seed=21, size=64)
    ext = ref.extended_domain(mask, 9, 9)
    src, tgt, _ = ref.scale_masks(ext, 4, 1)
    d = p.distance
    nnf0, e0, pr0, _ = ref.patchmatch(d, p.patchmatch, img, src, img, tgt, seed=7)
    nnf1, e1, pr1, _ = ref.patchmatch(d, p.patchmatch, img, src, img, tgt, init=nnf0, seed=8)
    g.update(pm_img=img, pm_mask=mask, pm_src=src, pm_tgt=tgt, pm_nnf0=nnf0, pm_energy0=e0, pm_props0=pr0,
             pm_nnf1=nnf1, pm_energy1=e1, pm_props1=pr1)
    conf = ref.confidence_mask(mask, 5.0, 0.1)
    cur = img.copy()
    cur[mask > 0] = rng.uniform(0, 255, (int(mask.sum()), 3)).astype(np.float32)
    g["upd_cur"], g["upd_conf"] = cur, conf
    for meth, lam in ((0, 0.05), (1, 0.05), (2, 0.05), (2, 1.0)):
        out, tot = ref.update(uparams(meth, lam=lam), cur, img, mask, ext, nnf1, conf)
        key = "upd_%d_%g" % (meth, lam)
        g[key], g[key + "_total"] = out, np.array(tot)
    depth = wl.depth_planes(64, 64, 4, rng)[..., None]
    cur4 = np.concatenate([cur, depth], -1).astype(np.float32)
    g["upd_cur4"] = cur4
    out, tot = ref.update(uparams(3, lam=1.0, lam_d=0.0), cur4, cur4, mask, ext, nnf1, conf, same_orig=True)
    g["upd_3"], g["upd_3_total"] = out, np.array(tot)
    # brute force on a crop
    bimg = wl.voronoi_texture(36, 30, 6, rng)[0]
    bmask = wl.disc_mask(36, 30, 5)
    bext = ref.extended_domain(bmask, 9, 9)
    bs, bt, _ = ref.scale_masks(bext, 4, 1)
    nnf, dd = ref.bruteforce_nnf(dparams(0), bimg, bs, bimg, bt)
    g.update(bf_img=bimg, bf_src=bs, bf_tgt=bt, bf_nnf=nnf, bf_dist=dd)
    return g


# the seeded uneven batch whose items have reference outputs: its seed, size
# and the parameters of the batch comparison
BATCH_SEED, BATCH_COUNT, BATCH_MAX_SIDE = 5, 64, 1024
BATCH_PAR_SEED, BATCH_THREADS = 4242, 4


def batch_items(indices):
    """(index, image, mask, params) of the chosen items of the seeded batch."""
    items = wl.config5(seed=BATCH_SEED, count=BATCH_COUNT, max_side=BATCH_MAX_SIDE)
    out = []
    for i in indices:
        img, mask, method, scales = items[i]
        out.append((i, img, mask, wl.config5_params(mask, method, scales)))
    return out


def full_reference_path(name, seed):
    return os.path.join(HERE, "%s_reference.npz" % name if seed == 0 else "%s_reference_seed%d.npz" % (name, seed))


def batch_reference_path(index):
    return os.path.join(HERE, "batch_reference_%02d.npz" % index)


def _arg(flag):
    return sys.argv[sys.argv.index(flag) + 1] if flag in sys.argv else None


def main():
    import time
    names = [a for a in sys.argv[1:] if a.startswith("config")]
    if "--skip-units" not in sys.argv:
        oracle_build.build_reference()
        ref = O.Reference()
        g = quiet(unit_cases, ref)
        np.savez_compressed(os.path.join(HERE, "units.npz"), **g)
        cases = {}
        for name, img, mask, p in small_configs():
            out = quiet(ref.process, img, mask, p, seed=101)
            cases[name + "_img"], cases[name + "_mask"] = img, mask
            cases[name + "_params"], cases[name + "_out"] = params_to_array(p), out
        np.savez_compressed(os.path.join(HERE, "process_small.npz"), **cases)
    if "--full" in sys.argv:
        oracle_build.build_reference()
        ref = O.Reference()
        seeds = [int(x) for x in (_arg("--seeds") or "0").split(",")]
        for seed in seeds:
            for name, fn in (("config1", lambda: wl.config1(seed=seed)), ("config2", lambda: wl.config2(seed=seed)),
                             ("config3", lambda: wl.config3(seed=seed))):
                if names and name not in names:
                    continue
                img, mask, p = fn()
                t0 = time.time()
                out = quiet(ref.process, img, mask, p, seed=101)
                np.savez_compressed(full_reference_path(name, seed), hole=out[mask > 0],
                                    params=params_to_array(p), seed=np.array(101), input_seed=np.array(seed))
                print(name, "seed", seed, "done in %.0f s" % (time.time() - t0), flush=True)
    if _arg("--batch"):
        orc = O.Oracle()
        orc.set_threads(BATCH_THREADS)
        orc.set_parallel_seed(BATCH_PAR_SEED)
        for i, img, mask, p in batch_items([int(x) for x in _arg("--batch").split(",")]):
            t0 = time.time()
            out = quiet(orc.process, img, mask, p, seed=101, parallel=True)
            np.savez_compressed(batch_reference_path(i), hole=out[mask > 0], params=params_to_array(p),
                                seed=np.array(101), parallel_seed=np.array(BATCH_PAR_SEED),
                                threads=np.array(BATCH_THREADS), index=np.array(i),
                                batch=np.array([BATCH_SEED, BATCH_COUNT, BATCH_MAX_SIDE]))
            print("batch item", i, img.shape, "done in %.0f s" % (time.time() - t0), flush=True)


if __name__ == "__main__":
    main()
