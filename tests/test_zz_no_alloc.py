"""The allocation-free distance entry point (nli_distance_pairs_noalloc).

It exists for callers that cannot allocate device memory while they run,
so it keeps its scratch in a fixed device array instead of a context
workspace.  Checked here against the ordinary nli_distance_pairs on the same
device buffers, for two calls in a row (the shared array keeps the previous
call's contents), and for the size limit.  The file is named to be collected
last, so a run that stops at the first failure has run everything else.
"""
import ctypes as ct

import numpy as np
import pytest

import __graft_entry__ as ge
from nli_gb300 import _abi

pytestmark = pytest.mark.gpu

NOALLOC_BYTES = 8 << 20  # NLI_NOALLOC_SCRATCH_BYTES in include/nli.h


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ge.build()
    pkg = ge.package()
    ctx = pkg.Context(0)
    lib = ctx.lib
    f = lib.nli_distance_pairs_noalloc
    P = ct.c_void_p
    f.restype = ct.c_int
    f.argtypes = [ct.POINTER(_abi.DistanceParams), P, ct.c_int, ct.c_int, P, ct.c_int, ct.c_int, ct.c_int, P,
                  ct.c_int, P, P]
    yield torch, ctx, f
    ctx.close()


def _noalloc(torch, f, d, src, tgt, pairs):
    out = torch.empty(pairs.shape[0], dtype=torch.float32, device=src.device)
    stream = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = f(ct.byref(d), ct.c_void_p(src.data_ptr()), src.shape[1], src.shape[0], ct.c_void_p(tgt.data_ptr()),
           tgt.shape[1], tgt.shape[0], src.shape[2], ct.c_void_p(pairs.data_ptr()), pairs.shape[0],
           ct.c_void_p(out.data_ptr()), stream)
    return rc, out


@pytest.mark.parametrize("kind,C,separate", [(0, 3, False), (0, 3, True), (1, 4, False), (2, 3, True)])
def test_noalloc_matches_distance_pairs_twice(env, kind, C, separate):
    torch, ctx, f = env
    rng = np.random.default_rng(31 + kind)
    for call in range(2):  # two calls in a row share the scratch array
        H, W = (60 + 7 * call, 80 - 5 * call)
        src = torch.from_numpy(rng.uniform(0, 255, (H, W, C)).astype(np.float32)).cuda()
        tgt = torch.from_numpy(rng.uniform(0, 255, (H - 4, W + 3, C)).astype(np.float32)).cuda() if separate else src
        n = 500
        pairs = np.stack([rng.integers(4, W - 5, n), rng.integers(4, H - 5, n),
                          rng.integers(4, tgt.shape[1] - 5, n), rng.integers(4, tgt.shape[0] - 5, n)], 1)
        pairs = torch.from_numpy(pairs.astype(np.int32)).cuda()
        d = _abi.DistanceParams(kind, 9, 9, 10000.0 if kind != 2 else 3.0, 0.05 if kind == 0 else 0.7, 0.2)
        ref = ctx.distance_pairs(d, src, tgt, pairs).cpu().numpy()
        rc, out = _noalloc(torch, f, d, src, tgt, pairs)
        assert rc == 0
        got = out.cpu().numpy()
        rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-30)
        assert rel.max() <= 1e-5, rel.max()


def test_noalloc_rejects_sizes_beyond_its_array(env):
    torch, ctx, f = env
    # gradients of a 640x480x4 image need 640*480*8 floats = 9.8 MB > 8 MiB
    src = torch.zeros((480, 640, 4), dtype=torch.float32, device="cuda")
    pairs = torch.tensor([[10, 10, 20, 20]], dtype=torch.int32, device="cuda")
    d = _abi.DistanceParams(1, 9, 9, 10000.0, 1.0, 0.0)
    assert 480 * 640 * 8 * 4 > NOALLOC_BYTES
    rc, _ = _noalloc(torch, f, d, src, src, pairs)
    assert rc == _abi.NLI_E_INVALID
