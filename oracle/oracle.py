"""TEST INFRASTRUCTURE ONLY -- ctypes front end of the oracle libraries.

``Oracle()`` wraps oracle/_build/libnlioracle.so (the restatement in
nli_oracle.cpp, available on every machine).  ``Reference()`` wraps
oracle/_ref/libnliref.so (the reference sources themselves, only where they
were compiled).  Both expose the same methods on numpy arrays.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg use this module.
"""
from __future__ import annotations

import ctypes as ct
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
import __graft_entry__ as _ge  # noqa: E402

_abi = _ge.package()._abi

P = ct.c_void_p
F = ct.c_float
I = ct.c_int
D = ct.POINTER(ct.c_double)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _u8(a):
    return np.ascontiguousarray(a, dtype=np.uint8)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(P)


class _Lib:
    prefix = ""
    parallel_arg = False

    def __init__(self, path):
        self.lib = ct.CDLL(path)
        pre = self.prefix
        L = self.lib

        def proto(name, res, args):
            f = getattr(L, pre + name)
            f.restype = res
            f.argtypes = args
            return f

        dp, pp, up, prp = (ct.POINTER(_abi.DistanceParams), ct.POINTER(_abi.PatchMatchParams),
                           ct.POINTER(_abi.UpdateParams), ct.POINTER(_abi.ProcessParams))
        self._err = proto("last_error", ct.c_char_p, [])
        self._gradient = proto("gradient", I, [P, I, I, I, P])
        self._gw = proto("gaussian_weights", I, [I, I, F, F, P])
        self._pairs = proto("distance_pairs", I, [dp, P, I, I, P, I, I, I, P, I, P])
        self._bf = proto("bruteforce_nnf", I, [dp, P, P, I, I, P, P, I, I, I, P, P])
        pm_args = [ct.c_uint] + ([I] if self.parallel_arg else []) + [
            dp, pp, P, P, I, I, P, P, I, I, I, P, P] + ([P] if self.parallel_arg else []) + [D, P]
        self._pm = proto("patchmatch", I, pm_args)
        self._upd = proto("update", I, [up, P, P, P, P, P, P, I, I, I, D])
        self._ss = proto("sample_size", I, [I, F])
        self._down = proto("downsample_with_mask", I, [P, P, I, I, I, F, F, I, P, P])
        self._up = proto("upsample", I, [P, I, I, I, I, I, P])
        self._dt = proto("distance_transform", I, [P, I, I, P])
        self._conf = proto("confidence_mask", I, [P, I, I, F, F, P])
        self._ext = proto("extended_domain", I, [P, I, I, I, I, P])
        self._sm = proto("scale_masks", I, [P, I, I, I, I, P, P, ct.POINTER(I)])
        self._pinit = proto("poisson_init", I, [P, P, I, I, I])
        self._rate = proto("subsampling_rate", F, [F, ct.c_uint])
        self._rgb2lab = proto("rgb_to_lab", I, [P, I, I, P])
        self._lab2rgb = proto("lab_to_rgb", I, [P, I, I, I, P])
        proc_args = [ct.c_uint] + ([I] if self.parallel_arg else []) + [prp, P, P, I, I, I, P] + (
            [ct.POINTER(_abi.ProcessStats)] if self.parallel_arg else [])
        self._proc = proto("process", I, proc_args)

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError("%s failed (%d): %s" % (what, rc, self._err().decode()))

    @staticmethod
    def _dims(img):
        if img.ndim == 2:
            return img.shape[1], img.shape[0], 1
        return img.shape[1], img.shape[0], img.shape[2]

    def gradient(self, img):
        img = _f32(img)
        W, H, C = self._dims(img)
        out = np.empty((H, W, 2 * C), np.float32)
        self._check(self._gradient(_ptr(img), W, H, C, _ptr(out)), "gradient")
        return out

    def gaussian_weights(self, sx, sy, sigma_x, sigma_y):
        out = np.empty((sy, sx), np.float32)
        self._check(self._gw(sx, sy, sigma_x, sigma_y, _ptr(out)), "gaussian_weights")
        return out

    def distance_pairs(self, dist, src, tgt, pairs):
        src, tgt, pairs = _f32(src), _f32(tgt), _i32(pairs)
        sW, sH, C = self._dims(src)
        tW, tH, _ = self._dims(tgt)
        out = np.empty(len(pairs), np.float32)
        self._check(self._pairs(ct.byref(dist), _ptr(src), sW, sH, _ptr(tgt), tW, tH, C, _ptr(pairs),
                                len(pairs), _ptr(out)), "distance_pairs")
        return out

    def bruteforce_nnf(self, dist, src, smask, tgt, tmask):
        src, tgt, smask, tmask = _f32(src), _f32(tgt), _u8(smask), _u8(tmask)
        sW, sH, C = self._dims(src)
        tW, tH, _ = self._dims(tgt)
        nnf = np.empty((tH, tW, 2), np.int32)
        d = np.empty((tH, tW), np.float32)
        self._check(self._bf(ct.byref(dist), _ptr(src), _ptr(smask), sW, sH, _ptr(tgt), _ptr(tmask), tW, tH, C,
                             _ptr(nnf), _ptr(d)), "bruteforce_nnf")
        return nnf, d

    def patchmatch(self, dist, pm, src, smask, tgt, tmask, init=None, seed=0, parallel=False):
        src, tgt, smask, tmask = _f32(src), _f32(tgt), _u8(smask), _u8(tmask)
        init = None if init is None else _i32(init)
        sW, sH, C = self._dims(src)
        tW, tH, _ = self._dims(tgt)
        nnf = np.empty((tH, tW, 2), np.int32)
        energy = np.zeros(max(pm.iterations, 1), np.float64)
        props = np.zeros(max(pm.iterations, 1), np.int32)
        d = np.full((tH, tW), np.finfo(np.float32).max, np.float32)
        args = [seed] + ([1 if parallel else 0] if self.parallel_arg else []) + [
            ct.byref(dist), ct.byref(pm), _ptr(src), _ptr(smask), sW, sH, _ptr(tgt), _ptr(tmask), tW, tH, C,
            _ptr(init), _ptr(nnf)] + ([_ptr(d)] if self.parallel_arg else []) + [
            energy.ctypes.data_as(D), _ptr(props)]
        self._check(self._pm(*args), "patchmatch")
        return nnf, energy, props, d

    def update(self, upd, image, orig, dom, ext, nnf, conf, same_orig=False):
        image = _f32(image).copy()
        W, H, C = self._dims(image)
        orig_arr = image if same_orig else _f32(orig)
        dom, ext, nnf = _u8(dom), _u8(ext), _i32(nnf)
        conf = None if conf is None else _f32(conf)
        tot = ct.c_double()
        self._check(self._upd(ct.byref(upd), _ptr(image), _ptr(orig_arr), _ptr(dom), _ptr(ext), _ptr(nnf),
                              _ptr(conf), W, H, C, ct.byref(tot)), "update")
        return image, tot.value

    def sample_size(self, size, factor):
        return self._ss(size, factor)

    def downsample_with_mask(self, img, mask, factor, threshold=0.4, mask_val=False):
        img, mask = _f32(img), _u8(mask)
        W, H, C = self._dims(img)
        sW, sH = self.sample_size(W, factor), self.sample_size(H, factor)
        out = np.empty((sH, sW, C), np.float32)
        om = np.empty((sH, sW), np.uint8)
        self._check(self._down(_ptr(img), _ptr(mask), W, H, C, factor, threshold, 1 if mask_val else 0, _ptr(out),
                               _ptr(om)), "downsample_with_mask")
        return out, om

    def upsample(self, img, oW, oH):
        img = _f32(img)
        W, H, C = self._dims(img)
        out = np.empty((oH, oW, C), np.float32)
        self._check(self._up(_ptr(img), W, H, C, oW, oH, _ptr(out)), "upsample")
        return out

    def distance_transform(self, mask):
        mask = _u8(mask)
        out = np.empty(mask.shape, np.float32)
        self._check(self._dt(_ptr(mask), mask.shape[1], mask.shape[0], _ptr(out)), "distance_transform")
        return out

    def confidence_mask(self, mask, decay=5.0, asym=0.1):
        mask = _u8(mask)
        out = np.empty(mask.shape, np.float32)
        self._check(self._conf(_ptr(mask), mask.shape[1], mask.shape[0], decay, asym, _ptr(out)), "confidence")
        return out

    def extended_domain(self, mask, px=9, py=9):
        mask = _u8(mask)
        out = np.empty(mask.shape, np.uint8)
        self._check(self._ext(_ptr(mask), mask.shape[1], mask.shape[0], px, py, _ptr(out)), "extended_domain")
        return out

    def scale_masks(self, ext, margin, erode):
        ext = _u8(ext)
        s = np.empty(ext.shape, np.uint8)
        t = np.empty(ext.shape, np.uint8)
        empty = I()
        self._check(self._sm(_ptr(ext), ext.shape[1], ext.shape[0], margin, 1 if erode else 0, _ptr(s), _ptr(t),
                             ct.byref(empty)), "scale_masks")
        return s, t, bool(empty.value)

    def poisson_init(self, img, mask):
        img = _f32(img).copy()
        mask = _u8(mask)
        W, H, C = self._dims(img)
        self._check(self._pinit(_ptr(img), _ptr(mask), W, H, C), "poisson_init")
        return img

    def subsampling_rate(self, ratio, scales):
        return self._rate(ratio, scales)

    def rgb_to_lab(self, rgb):
        rgb = _f32(rgb)
        out = np.empty(rgb.shape[:2] + (3,), np.float32)
        self._check(self._rgb2lab(_ptr(rgb), rgb.shape[1], rgb.shape[0], _ptr(out)), "rgb_to_lab")
        return out

    def lab_to_rgb(self, lab):
        lab = _f32(lab)
        out = np.empty(lab.shape[:2] + (3,), np.float32)
        self._check(self._lab2rgb(_ptr(lab), lab.shape[1], lab.shape[0], lab.shape[2], _ptr(out)), "lab_to_rgb")
        return out


class Oracle(_Lib):
    """The restatement (oracle/nli_oracle.cpp)."""
    prefix = "orc_"
    parallel_arg = True

    def __init__(self, path=None, timing=False):
        """timing: the build with the reference's Release flags (for timing
        only; the default build is the bit-exact checker)."""
        if path is None:
            sys.path.insert(0, HERE)
            try:
                import build as ob
            finally:
                sys.path.pop(0)
            path = ob.build_timing() if timing else ob.build_oracle()
        super().__init__(path)
        self._energy = self.lib.orc_nnf_energy
        self._energy.restype = I
        self._energy.argtypes = [ct.POINTER(_abi.DistanceParams), P, I, I, P, I, I, I, P, P, D]
        self.max_threads = self.lib.orc_max_threads()
        self.lib.orc_set_parallel_seed.restype = None
        self.lib.orc_set_parallel_seed.argtypes = [I, ct.c_uint]
        self.lib.orc_set_threads.restype = None
        self.lib.orc_set_threads.argtypes = [I]

    def set_parallel_seed(self, seed):
        """Fixes the base of the OpenMP PatchMatch's thread seeds (None: time(NULL),
        as the reference)."""
        self.lib.orc_set_parallel_seed(0 if seed is None else 1, 0 if seed is None else int(seed))

    def set_threads(self, n):
        self.lib.orc_set_threads(int(n))
        self.max_threads = self.lib.orc_max_threads()

    def nnf_energy(self, dist, src, tgt, tmask, nnf):
        src, tgt, tmask, nnf = _f32(src), _f32(tgt), _u8(tmask), _i32(nnf)
        sW, sH, C = self._dims(src)
        tW, tH, _ = self._dims(tgt)
        e = ct.c_double()
        self._check(self._energy(ct.byref(dist), _ptr(src), sW, sH, _ptr(tgt), tW, tH, C, _ptr(tmask), _ptr(nnf),
                                 ct.byref(e)), "nnf_energy")
        return e.value

    def process(self, img, mask, params, seed=0, parallel=False, return_stats=False):
        img, mask = _f32(img), _u8(mask)
        W, H, C = self._dims(img)
        out = np.empty_like(img)
        st = _abi.ProcessStats()
        self._check(self._proc(seed, 1 if parallel else 0, ct.byref(params), _ptr(img), _ptr(mask), W, H, C,
                               _ptr(out), ct.byref(st)), "process")
        return (out, st.as_dict()) if return_stats else out


class Reference(_Lib):
    """The reference sources compiled by oracle/build.py (serial, METRICS)."""
    prefix = "ref_"
    parallel_arg = False
    PATH = os.path.join(HERE, "_ref", "libnliref.so")

    def __init__(self, path=None):
        super().__init__(path or self.PATH)

    @classmethod
    def available(cls):
        return os.path.exists(cls.PATH)

    def process(self, img, mask, params, seed=0):
        img, mask = _f32(img), _u8(mask)
        W, H, C = self._dims(img)
        out = np.empty_like(img)
        self._check(self._proc(seed, ct.byref(params), _ptr(img), _ptr(mask), W, H, C, _ptr(out)), "process")
        return out
