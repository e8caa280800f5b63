"""The C++ drop-in (include/nli_inpainting.hpp, libnli_dropin.so): a host
program written against the reference's class interface and wired like the
reference's main.cpp is compiled here and run; its output must equal the
C ABI's nli_process output for the same parameters and seed."""
import os
import subprocess

import numpy as np
import pytest

import __graft_entry__ as ge
from conftest import ROOT

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def demo(tmp_path_factory):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ge.build()
    pkg_dir = os.path.join(ROOT, "non-local-inpainting_gb300")
    exe = str(tmp_path_factory.mktemp("dropin") / "dropin_demo")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include", "nli_dropin"), "-I",
                    os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "dropin_demo.cpp"), "-o", exe,
                    "-L", pkg_dir, "-lnli_dropin", "-lnli_gb300", "-Wl,-rpath," + pkg_dir], check=True)
    return exe


def params_for(method):
    from nli_gb300 import _abi
    from nli_gb300 import workloads as wl
    if method == "nlmeans":
        p = wl.params("nlmeans", scales=3, coarse=0.45, iters=20)
    elif method == "nlpoisson":
        p = wl.params("nlpoisson", scales=3, coarse=0.45, iters=20, cg_tol=1e-4)
    else:
        p = wl.params("nldepth", scales=3, coarse=0.45, iters=20, lam_r=1.0, lam_d=0.0, cg_tol=1e-6)
    p.subsampling_rate = _abi.subsampling_rate(0.45, 3)
    return p


@pytest.mark.parametrize("method", ["nlmeans", "nlpoisson", "nldepth"])
def test_dropin_program_matches_c_abi(demo, gpu_ctx, tmp_path, method):
    from nli_gb300 import workloads as wl
    if method == "nldepth":
        img, mask, _ = wl.config3(seed=4, w=80, h=64, scales=3)
    else:
        img, mask, _ = wl.config2(seed=3, size=72, scales=3)
    H, W, C = img.shape
    (tmp_path / "img.f32").write_bytes(np.ascontiguousarray(img, np.float32).tobytes())
    (tmp_path / "mask.u8").write_bytes(np.ascontiguousarray(mask, np.uint8).tobytes())
    seed = 4242
    r = subprocess.run([demo, method, str(W), str(H), str(C), str(tmp_path / "img.f32"), str(tmp_path / "mask.u8"),
                        str(tmp_path / "out.f32"), str(seed)], capture_output=True, text=True)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stderr
    out = np.frombuffer((tmp_path / "out.f32").read_bytes(), np.float32).reshape(H, W, C)
    gpu_ctx.set_seed(seed)
    ref, _ = gpu_ctx.process(img, mask, params_for(method))
    assert np.array_equal(out, ref)
    assert "size mismatch gives empty field: 1" in r.stdout
    assert "pyramid levels 3 masks 3 nnfs 3 finest nnf %dx%d" % (W, H) in r.stdout
