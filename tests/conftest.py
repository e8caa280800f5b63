import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__ as ge  # noqa: E402

pkg = ge.package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests of the CUDA path")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    return O.Oracle()


@pytest.fixture(scope="session")
def units():
    return dict(np.load(os.path.join(GOLDEN, "units.npz")))


@pytest.fixture(scope="session")
def small_cases():
    return dict(np.load(os.path.join(GOLDEN, "process_small.npz")))


def params_from_array(a):
    """Inverse of tests/golden/make_golden.py:params_to_array."""
    from nli_gb300 import _abi
    p = _abi.ProcessParams()
    v = [float(x) for x in a]
    p.distance.kind, p.distance.patch_x, p.distance.patch_y = int(v[0]), int(v[1]), int(v[2])
    p.distance.sigma, p.distance.lambda_, p.distance.lambda_d = v[3], v[4], v[5]
    p.patchmatch.iterations, p.patchmatch.random_shots, p.patchmatch.window = int(v[6]), int(v[7]), int(v[8])
    p.update.method, p.update.patch_x, p.update.patch_y = int(v[9]), int(v[10]), int(v[11])
    p.update.sigma, p.update.lambda_, p.update.lambda_d = v[12], v[13], v[14]
    p.update.cg_tol, p.update.cg_iters = v[15], int(v[16])
    p.iterations, p.tolerance, p.scales = int(v[17]), v[18], int(v[19])
    p.subsampling_rate, p.conf_decay_time, p.conf_asymptotic, p.init = v[20], v[21], v[22], int(v[23])
    return p


def hole_psnr(a, b, mask, peak=255.0):
    m = mask.astype(bool)
    d = (a[m].astype(np.float64) - b[m].astype(np.float64)) ** 2
    mse = d.mean()
    return float("inf") if mse == 0 else 10 * np.log10(peak * peak / mse)


@pytest.fixture(scope="session")
def gpu_ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ge.build()
    ctx = pkg.Context(0)
    ctx.set_seed(1234)
    yield ctx
    ctx.close()
