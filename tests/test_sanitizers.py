"""Host code under AddressSanitizer and UBSan (compute-sanitizer is not
available for the device code): the oracle restatement runs whole
process() calls for every update method, the distances, brute force,
PatchMatch, the pyramid helpers and the colour conversions from a
sanitized build, in a child process with the sanitizer runtime preloaded.
Any report fails the test.  Skipped where the compiler has no sanitizer
runtime.  No GPU."""
import os
import subprocess
import sys
import textwrap

import pytest

from conftest import ROOT

SCRIPT = textwrap.dedent("""
    import sys
    sys.path[:0] = [{root!r}, {oracle!r}]
    import __graft_entry__ as ge
    ge.package()
    import oracle as O
    from nli_gb300 import workloads as wl, _abi
    orc = O.Oracle(path={lib!r})
    img, mask, _ = wl.config2(seed=1, size=40, scales=2)
    for method in ("nlmeans", "nlmedians", "nlpoisson"):
        orc.process(img, mask, wl.params(method, scales=2, coarse=0.6, iters=2, cg_tol=1e-4), seed=3)
    rgbd, dmask, _ = wl.config3(seed=3, w=48, h=40, scales=2)
    orc.process(rgbd, dmask, wl.params("nldepth", scales=2, coarse=0.6, iters=2, lam_r=0.5, lam_d=0.3), seed=3)
    for kind in (0, 1, 2, 3):
        im = rgbd if kind == _abi.NLI_DIST_L2_RGBD else img
        m = dmask if kind == _abi.NLI_DIST_L2_RGBD else mask
        d = _abi.DistanceParams()
        d.kind, d.patch_x, d.patch_y, d.sigma, d.lambda_, d.lambda_d = kind, 7, 5, 3.0, 0.3, 0.4
        ext = orc.extended_domain(m, 7, 5)
        s, t, _ = orc.scale_masks(ext, 3, True)
        orc.bruteforce_nnf(d, im, s, im, t)
        orc.patchmatch(d, _abi.PatchMatchParams(3, 10, -1), im, s, im, t, seed=1)
    orc.lab_to_rgb(orc.rgb_to_lab(img))
    orc.distance_transform(mask)
    print("clean")
""")


def test_oracle_under_asan_ubsan(tmp_path):
    libasan = subprocess.run(["gcc", "-print-file-name=libasan.so"], capture_output=True, text=True).stdout.strip()
    if not os.path.isabs(libasan) or not os.path.exists(libasan):
        pytest.skip("no AddressSanitizer runtime")
    lib = str(tmp_path / "libnlioracle_asan.so")
    r = subprocess.run(["g++", "-O1", "-g", "-fsanitize=address,undefined", "-fno-omit-frame-pointer", "-std=c++17",
                        "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "oracle", "nli_oracle.cpp"), "-o", lib, "-lm"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("sanitized build failed: " + r.stderr[-200:])
    script = tmp_path / "run.py"
    script.write_text(SCRIPT.format(root=ROOT, oracle=os.path.join(ROOT, "oracle"), lib=lib))
    # the C++ runtime right after the sanitizer's, so that its exception
    # entry points resolve for the interceptors
    libstdcxx = subprocess.run(["g++", "-print-file-name=libstdc++.so.6"], capture_output=True,
                               text=True).stdout.strip()
    env = dict(os.environ, LD_PRELOAD=libasan + ((":" + libstdcxx) if os.path.isabs(libstdcxx) else ""),
               ASAN_OPTIONS="detect_leaks=0", UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([sys.executable, str(script)], capture_output=True, text=True, env=env, timeout=900)
    report = r.stdout + r.stderr
    if r.returncode != 0 and "AddressSanitizer" not in report and "runtime error" not in report:
        pytest.skip("the sanitizer runtime cannot be preloaded here: " + report[-300:])
    assert "AddressSanitizer" not in report and "runtime error" not in report, report[-3000:]
    assert r.returncode == 0 and "clean" in r.stdout, report[-2000:]
