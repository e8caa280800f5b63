"""CPU-side checks of the C ABI library: it builds, loads, exports every
function include/nli.h declares, and its host-only helpers agree with the
oracle.  No kernel is launched here."""
import ctypes as ct
import os

import numpy as np
import pytest

import __graft_entry__ as ge
from conftest import ROOT

pkg = ge.package()


@pytest.fixture(scope="module")
def lib():
    from nli_gb300 import build
    build.build()
    return pkg.load()


def test_exports_every_declared_symbol(lib):
    names = pkg.exported_symbols()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_library_is_sm103a():
    from nli_gb300 import build
    assert "arch=compute_103a,code=sm_103a" in build.ARCH


def test_host_helpers_match_oracle(lib, oracle):
    for (sx, sy, a, b) in [(9, 9, 10000.0, 10000.0), (9, 9, 1.3, 1.3), (9, 1, 0.7, 0.0), (7, 5, 2.0, 3.0)]:
        out = np.empty((sy, sx), np.float32)
        assert lib.nli_gaussian_weights(sx, sy, a, b, out.ctypes.data_as(ct.c_void_p)) == 0
        assert np.array_equal(out, oracle.gaussian_weights(sx, sy, a, b))
    for size in (26, 51, 256, 511, 640, 1023):
        for f in (0.5623413, 0.7196857, 0.7499, 0.75):
            assert lib.nli_sample_size(size, f) == oracle.sample_size(size, f)
    for r in (0.05, 0.1, 0.25, 0.5):
        for s in (2, 5, 8, 9, 11):
            assert lib.nli_subsampling_rate(r, s) == oracle.subsampling_rate(r, s)
            from nli_gb300 import _abi
            assert np.float32(_abi.subsampling_rate(r, s)) == np.float32(lib.nli_subsampling_rate(r, s))


def test_status_strings(lib):
    for s in (0, -1, -2, -3, -4, -5, -6, -7, -8):
        assert lib.nli_status_string(s)


def test_null_arguments_rejected(lib):
    assert lib.nli_ctx_create(0, None) == -1
    assert lib.nli_ctx_destroy(None) == -1
    assert lib.nli_gradient(None, None, 1, 1, 3, None) == -1
    assert lib.nli_gaussian_weights(0, 9, 1.0, 1.0, None) == -1


def test_header_documents_reference_interfaces():
    txt = open(os.path.join(ROOT, "include", "nli.h")).read()
    for ref in ("patch_match.cpp", "image_inpainting.cpp", "patch_non_local_poisson.cpp",
                "l2_combined_patch_distance.cpp", "l2_rgbd_patch_distance.cpp", "sampling.cpp"):
        assert ref in txt
