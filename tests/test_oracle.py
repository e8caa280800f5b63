"""The oracle restatement (oracle/nli_oracle.cpp) against golden vectors
produced by the reference implementation itself (tests/golden/make_golden.py).
Everything here is expected to be bit-exact: the restatement keeps the
reference's float/double evaluation order and its rand() call sequence."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, params_from_array
from nli_gb300 import _abi


def dparams(kind, sigma=10000.0, lam=0.05, lam_d=0.3, patch=9):
    return _abi.DistanceParams(kind, patch, patch, sigma, lam, lam_d)


def uparams(method, lam=0.05, lam_d=0.0, tol=1e-4, iters=1000, sigma=10000.0, patch=9):
    return _abi.UpdateParams(method, patch, patch, sigma, lam, lam_d, tol, iters)


def test_gradient(oracle, units):
    assert np.array_equal(oracle.gradient(units["grad_in3"]), units["grad_out3"])
    assert np.array_equal(oracle.gradient(units["grad_in4"]), units["grad_out4"])


def test_gaussian_weights(oracle, units):
    for i, (sx, sy, a, b) in enumerate(units["gw_args"]):
        assert np.array_equal(oracle.gaussian_weights(int(sx), int(sy), a, b), units["gw_%d" % i])


def test_distances(oracle, units):
    for i, (kind, C, sigma) in enumerate(units["dist_cases"]):
        d = dparams(int(kind), sigma=sigma, lam=0.05 if kind == 0 else 0.7, lam_d=0.2)
        got = oracle.distance_pairs(d, units["dist_src_%d" % i], units["dist_tgt_%d" % i], units["dist_pairs_%d" % i])
        assert np.array_equal(got, units["dist_out_%d" % i]), (kind, C)


def test_masks_and_transforms(oracle, units):
    m = units["mask"]
    assert np.array_equal(oracle.extended_domain(m, 9, 9), units["ext"])
    assert np.array_equal(oracle.extended_domain(m, 7, 5), units["ext75"])
    for erode in (0, 1):
        s, t, e = oracle.scale_masks(units["ext"], 4, erode)
        assert np.array_equal(s, units["src_%d" % erode]) and np.array_equal(t, units["tgt_%d" % erode])
        assert e == bool(units["empty_%d" % erode])
    assert np.array_equal(oracle.distance_transform(m), units["dt"])
    assert np.array_equal(oracle.confidence_mask(m, 5.0, 0.1), units["conf"])
    assert np.array_equal(oracle.confidence_mask(m, 2.5, 0.3), units["conf2"])


def test_pyramid(oracle, units):
    for i, f in enumerate((0.5623413, 0.7196857, 0.75, 0.5)):
        oi, om = oracle.downsample_with_mask(units["pyr_img"], units["pyr_mask"], f, 0.4, False)
        assert np.array_equal(oi, units["down_img_%d" % i]) and np.array_equal(om, units["down_mask_%d" % i])
        assert np.array_equal(oracle.upsample(oi, 57, 45), units["up_%d" % i])


def test_poisson_init(oracle, units):
    assert np.array_equal(oracle.poisson_init(units["pinit_in"], units["pinit_mask"]), units["pinit_out"])


def test_patchmatch(oracle, units):
    p = _abi.ProcessParams()
    from nli_gb300 import workloads as wl
    p = wl.params("nlmeans")
    img, src, tgt = units["pm_img"], units["pm_src"], units["pm_tgt"]
    nnf0, e0, pr0, _ = oracle.patchmatch(p.distance, p.patchmatch, img, src, img, tgt, seed=7)
    assert np.array_equal(nnf0, units["pm_nnf0"])
    assert np.array_equal(e0, units["pm_energy0"]) and np.array_equal(pr0, units["pm_props0"])
    nnf1, e1, pr1, _ = oracle.patchmatch(p.distance, p.patchmatch, img, src, img, tgt, init=nnf0, seed=8)
    assert np.array_equal(nnf1, units["pm_nnf1"]) and np.array_equal(e1, units["pm_energy1"])


def test_updates(oracle, units):
    cur, img, mask, conf = units["upd_cur"], units["pm_img"], units["pm_mask"], units["upd_conf"]
    ext = oracle.extended_domain(mask, 9, 9)
    nnf = units["pm_nnf1"]
    for meth, lam in ((0, 0.05), (1, 0.05), (2, 0.05), (2, 1.0)):
        out, tot = oracle.update(uparams(meth, lam=lam), cur, img, mask, ext, nnf, conf)
        key = "upd_%d_%g" % (meth, lam)
        assert np.array_equal(out, units[key]), key
        assert tot == float(units[key + "_total"]), key
    out, tot = oracle.update(uparams(3, lam=1.0, lam_d=0.0), units["upd_cur4"], None, mask, ext, nnf, conf,
                             same_orig=True)
    assert np.array_equal(out, units["upd_3"]) and tot == float(units["upd_3_total"])


def test_lab_conversions(oracle, units):
    """io_utility.cpp:268-318 restated: bit-exact with the reference on every
    grey level and seeded colours, both directions.  With a depth channel the
    reference reads freed memory (io_utility.cpp:303-307); the restatement
    drops the depth channel, as that code intends."""
    assert np.array_equal(oracle.rgb_to_lab(units["lab_rgb_in"]), units["lab_out"])
    assert np.array_equal(oracle.lab_to_rgb(units["lab_out"]), units["lab_rgb_back"])
    assert np.array_equal(oracle.lab_to_rgb(units["lab4_in"]), units["lab_rgb_back"])


def test_bruteforce(oracle, units):
    nnf, d = oracle.bruteforce_nnf(dparams(0), units["bf_img"], units["bf_src"], units["bf_img"], units["bf_tgt"])
    assert np.array_equal(nnf, units["bf_nnf"]) and np.array_equal(d, units["bf_dist"])


@pytest.mark.parametrize("name", ["means", "medians", "poisson", "depth", "avg_l2norm", "initnone"])
def test_process_small(oracle, small_cases, name):
    p = params_from_array(small_cases[name + "_params"])
    out = oracle.process(small_cases[name + "_img"], small_cases[name + "_mask"], p, seed=101)
    assert np.array_equal(out, small_cases[name + "_out"])


def test_process_config1_full(oracle):
    path = os.path.join(GOLDEN, "config1_reference.npz")
    if not os.path.exists(path):
        pytest.skip("full-size golden not generated")
    from nli_gb300 import workloads as wl
    g = np.load(path)
    img, mask, _ = wl.config1(seed=0)
    p = params_from_array(g["params"])
    out = oracle.process(img, mask, p, seed=int(g["seed"]))
    assert np.array_equal(out[mask > 0], g["hole"])


def test_empty_source_error(oracle):
    from nli_gb300 import workloads as wl
    img, mask, p = wl.config1(seed=0, size=96)  # coarse 0.1 at 96 px leaves no complete source patch
    with pytest.raises(RuntimeError, match="Empty source mask"):
        oracle.process(img, mask, p, seed=1)
