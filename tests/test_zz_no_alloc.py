"""The allocation-free distance entry point (nli_distance_pairs_noalloc).

It exists for callers that cannot allocate device memory while they run,
so it keeps its scratch in a fixed device array instead of a context
workspace.  It runs the same gradient and distance kernels as
nli_distance_pairs, so its output must be bit-identical to that entry
point's and to the reference's own distances (the golden vectors), for two
calls in a row (the shared array keeps the previous call's contents).  The
size limit is checked at its boundary.  The file is named to be collected
last, so a run that stops at the first failure has run everything else.
"""
import ctypes as ct
import os

import numpy as np
import pytest

import __graft_entry__ as ge
from nli_gb300 import _abi

pytestmark = pytest.mark.gpu

NOALLOC_BYTES = 8 << 20  # NLI_NOALLOC_SCRATCH_BYTES in include/nli.h
NOALLOC_FLOATS = NOALLOC_BYTES // 4
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "units.npz")


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
    out = torch.full((pairs.shape[0],), -1.0, dtype=torch.float32, device=src.device)
    stream = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
    C = src.shape[2] if src.dim() == 3 else 1
    rc = f(ct.byref(d), ct.c_void_p(src.data_ptr()), src.shape[1], src.shape[0], ct.c_void_p(tgt.data_ptr()),
           tgt.shape[1], tgt.shape[0], C, ct.c_void_p(pairs.data_ptr()), pairs.shape[0],
           ct.c_void_p(out.data_ptr()), stream)
    torch.cuda.synchronize()
    return rc, out


def _same(got, ref):
    """Bit-identical, NaN (pairs whose patch leaves its image) included."""
    return np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def _pairs(rng, n, sW, sH, tW, tH, r=4):
    return np.stack([rng.integers(r, sW - r, n), rng.integers(r, sH - r, n), rng.integers(r, tW - r, n),
                     rng.integers(r, tH - r, n)], 1).astype(np.int32)


@pytest.mark.parametrize("kind,C,separate", [(0, 3, False), (0, 3, True), (1, 4, False), (2, 3, True)])
def test_noalloc_bit_identical_to_distance_pairs_twice(env, kind, C, separate):
    torch, ctx, f = env
    rng = np.random.default_rng(31 + kind)
    for call in range(2):  # two calls in a row share the scratch array
        H, W = (60 + 7 * call, 80 - 5 * call)
        src = torch.from_numpy(rng.uniform(0, 255, (H, W, C)).astype(np.float32)).cuda()
        tgt = torch.from_numpy(rng.uniform(0, 255, (H - 4, W + 3, C)).astype(np.float32)).cuda() if separate else src
        n = 500
        # some pairs leave their image on purpose (their distance is NaN)
        pairs = _pairs(rng, n, W, H, tgt.shape[1], tgt.shape[0], r=2)
        pairs = torch.from_numpy(pairs).cuda()
        d = _abi.DistanceParams(kind, 9, 9, 10000.0 if kind != 2 else 3.0, 0.05 if kind == 0 else 0.7, 0.2)
        ref = ctx.distance_pairs(d, src, tgt, pairs).cpu().numpy()
        rc, out = _noalloc(torch, f, d, src, tgt, pairs)
        assert rc == 0
        got = out.cpu().numpy()
        assert np.isnan(ref).any()
        assert _same(got, ref), int((got != ref).sum())


def test_noalloc_matches_reference_golden_distances(env):
    """The reference's own distances (units.npz, made from the reference
    sources): every distance kind and channel count, bit-exact, twice."""
    torch, ctx, f = env
    units = np.load(GOLDEN)
    for _ in range(2):
        for i, (kind, C, sigma) in enumerate(units["dist_cases"]):
            d = _abi.DistanceParams(int(kind), 9, 9, float(sigma), 0.05 if kind == 0 else 0.7, 0.2)
            src = torch.from_numpy(units["dist_src_%d" % i]).cuda()
            tgt = torch.from_numpy(units["dist_tgt_%d" % i]).cuda()
            pairs = torch.from_numpy(units["dist_pairs_%d" % i]).cuda()
            rc, out = _noalloc(torch, f, d, src, tgt, pairs)
            assert rc == 0
            assert _same(out.cpu().numpy(), units["dist_out_%d" % i]), (kind, C)


def _split(total):
    """Two image shapes (W, H) whose pixel counts add up to `total`, both
    sides at least 16."""
    for sH in range(300, 700):
        for tH in range(300, 700):
            rest = total - 1000 * sH
            if rest > 0 and rest % tH == 0 and rest // tH >= 16:
                return (1000, sH), (rest // tH, tH)
    raise AssertionError("no split of %d" % total)


@pytest.mark.parametrize("extra", [0, 1])
def test_noalloc_size_limit_with_separate_target(env, extra):
    """Source and target gradients together: exactly the array is accepted
    (and bit-identical), one pixel more is rejected, though each image's
    gradients alone fit."""
    torch, ctx, f = env
    C = 1
    (sW, sH), (tW, tH) = _split(NOALLOC_FLOATS // (2 * C) + extra)
    assert (sW * sH + tW * tH) * 2 * C == NOALLOC_FLOATS + 2 * C * extra
    assert sW * sH * 2 * C <= NOALLOC_FLOATS and tW * tH * 2 * C <= NOALLOC_FLOATS
    rng = np.random.default_rng(7 + extra)
    src = torch.from_numpy(rng.uniform(0, 255, (sH, sW, C)).astype(np.float32)).cuda()
    tgt = torch.from_numpy(rng.uniform(0, 255, (tH, tW, C)).astype(np.float32)).cuda()
    # pairs near the far corners, so the last gradient floats are read
    pairs = np.concatenate([_pairs(rng, 300, sW, sH, tW, tH),
                            np.array([[sW - 5, sH - 5, tW - 5, tH - 5], [4, 4, tW - 5, tH - 5]], np.int32)])
    pairs = torch.from_numpy(pairs).cuda()
    d = _abi.DistanceParams(0, 9, 9, 10000.0, 0.05, 0.2)
    rc, out = _noalloc(torch, f, d, src, tgt, pairs)
    if extra:
        assert rc == _abi.NLI_E_INVALID
        return
    assert rc == 0
    ref = ctx.distance_pairs(d, src, tgt, pairs).cpu().numpy()
    assert _same(out.cpu().numpy(), ref)


def test_noalloc_rejects_sizes_beyond_its_array(env):
    torch, ctx, f = env
    # gradients of a 640x480x4 image need 640*480*8 floats = 9.8 MB > 8 MiB
    src = torch.zeros((480, 640, 4), dtype=torch.float32, device="cuda")
    pairs = torch.tensor([[10, 10, 20, 20]], dtype=torch.int32, device="cuda")
    d = _abi.DistanceParams(1, 9, 9, 10000.0, 1.0, 0.0)
    assert 480 * 640 * 8 * 4 > NOALLOC_BYTES
    rc, _ = _noalloc(torch, f, d, src, src, pairs)
    assert rc == _abi.NLI_E_INVALID


def test_noalloc_norm_kinds_need_no_scratch(env):
    """The L1 / L2 norm kinds use no gradients, so an image larger than the
    array is accepted and matches nli_distance_pairs bit for bit."""
    torch, ctx, f = env
    rng = np.random.default_rng(3)
    src = torch.from_numpy(rng.uniform(0, 255, (1000, 1200, 4)).astype(np.float32)).cuda()
    assert 1200 * 1000 * 4 * 4 > NOALLOC_BYTES
    pairs = torch.from_numpy(_pairs(rng, 400, 1200, 1000, 1200, 1000)).cuda()
    for kind in (2, 3):
        d = _abi.DistanceParams(kind, 9, 9, 10000.0, 0.05, 0.2)
        rc, out = _noalloc(torch, f, d, src, src, pairs)
        assert rc == 0
        ref = ctx.distance_pairs(d, src, src, pairs).cpu().numpy()
        assert _same(out.cpu().numpy(), ref)
