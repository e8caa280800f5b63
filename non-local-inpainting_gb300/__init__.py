"""GB300-native (sm_103a) multiscale non-local inpainting.

Python front end of the C ABI in include/nli.h (libnli_gb300.so, built
in-tree by build.py).  Device arrays are torch CUDA tensors; the multiscale
`process` also accepts host numpy arrays (the host copies are then part of
the call, as in nli_process).  There is no CPU implementation here: every
call runs CUDA kernels, and loading fails loudly when the library is
missing.
"""
from __future__ import annotations

import ctypes as ct
import os

import numpy as np

from . import _abi
from ._abi import (DistanceParams, PatchMatchParams, ProcessParams, ProcessStats,  # noqa: F401
                   UpdateParams)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnli_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "nli.h")

_lib = None
_libs = {}
# the checked build (NLI_CHECKED: bounds tests on gathered indices), built on
# demand by build.build(checked=True)
CHECKED_LIB_PATH = os.path.join(HERE, "libnli_gb300_checked.so")

P = ct.c_void_p
I = ct.c_int
F = ct.c_float


class NliError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s (%d): %s" % (_abi_status(status), status, message))
        self.status = status


def _abi_status(s):
    names = {0: "ok", -1: "invalid argument", -2: "empty source mask", -3: "channels do not match",
             -4: "size mismatch", -5: "unsupported", -6: "CUDA error", -7: "timeout", -8: "out of memory"}
    return names.get(s, "status")


def exported_symbols():
    """Names of the functions declared in include/nli.h."""
    import re
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(nli_[a-z_0-9]+)\s*\(", txt, re.M)))


def load(path=LIB_PATH):
    """Loads libnli_gb300.so, or another build of it at `path` (raises if
    it was not built)."""
    global _lib
    if path in _libs:
        return _libs[path]
    if not os.path.exists(path):
        raise ImportError("%s not found: run __graft_entry__.build()" % path)
    L = ct.CDLL(path)

    def proto(name, res, args):
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args

    dp, pp, up, prp, st = (ct.POINTER(DistanceParams), ct.POINTER(PatchMatchParams), ct.POINTER(UpdateParams),
                           ct.POINTER(ProcessParams), ct.POINTER(ProcessStats))
    proto("nli_version", ct.c_char_p, [])
    proto("nli_status_string", ct.c_char_p, [I])
    proto("nli_ctx_create", I, [I, ct.POINTER(P)])
    proto("nli_ctx_destroy", I, [P])
    proto("nli_ctx_set_stream", I, [P, P])
    proto("nli_set_seed", I, [P, ct.c_uint64])
    proto("nli_ctx_synchronize", I, [P])
    proto("nli_last_error", ct.c_char_p, [P])
    proto("nli_gaussian_weights", I, [I, I, F, F, P])
    proto("nli_subsampling_rate", F, [F, ct.c_uint])
    proto("nli_sample_size", I, [I, F])
    proto("nli_gradient", I, [P, P, I, I, I, P])
    proto("nli_downsample_with_mask", I, [P, P, P, I, I, I, F, F, I, P, P])
    proto("nli_upsample", I, [P, P, I, I, I, I, I, P])
    proto("nli_distance_transform", I, [P, P, I, I, P])
    proto("nli_confidence_mask", I, [P, P, I, I, F, F, P])
    proto("nli_extended_domain", I, [P, P, I, I, I, I, P])
    proto("nli_scale_masks", I, [P, P, I, I, I, I, P, P, ct.POINTER(I)])
    proto("nli_poisson_init", I, [P, P, P, I, I, I])
    proto("nli_distance_pairs", I, [P, dp, P, I, I, P, I, I, I, P, I, P])
    proto("nli_bruteforce_nnf", I, [P, dp, P, P, I, I, P, P, I, I, I, P, P])
    proto("nli_patchmatch", I, [P, dp, pp, P, P, I, I, P, P, I, I, I, P, P, P, ct.POINTER(ct.c_double)])
    proto("nli_update", I, [P, up, P, P, P, P, P, P, I, I, I, ct.POINTER(ct.c_double)])
    proto("nli_patchmatch_metrics", I, [P, dp, pp, P, P, I, I, P, P, I, I, I, P, P, P, ct.POINTER(ct.c_double),
                                        P, P, ct.POINTER(ct.c_int32)])
    proto("nli_rgb_to_lab", I, [P, P, I, I, P])
    proto("nli_lab_to_rgb", I, [P, P, I, I, I, P])
    proto("nli_cat_depth", I, [P, P, P, I, I, P])
    proto("nli_separate_depth", I, [P, P, I, I, P, P])
    proto("nli_ctx_keep_intermediate", I, [P, I])
    proto("nli_intermediate_count", I, [P, I])
    proto("nli_intermediate_get", I, [P, I, I, ct.POINTER(I), ct.POINTER(I), ct.POINTER(I), P])
    proto("nli_update_backward", I, [P, up, P, P, P, P, P, P, I, I, I, P, P, ct.POINTER(ct.c_double),
                                     ct.POINTER(ct.c_double), ct.POINTER(ct.c_double)])
    proto("nli_process", I, [P, prp, P, P, I, I, I, P, st])
    proto("nli_process_device", I, [P, prp, P, P, I, I, I, P, st])
    proto("nli_process_batch", I, [P, I, prp, P, P, P, P, P, P, st, P])
    proto("nli_process_batch_device", I, [P, I, prp, P, P, P, P, P, P, st, P])
    proto("nli_ctx_set_batch_width", I, [P, I])
    proto("nli_batch_seed", ct.c_uint64, [ct.c_uint64, I])
    proto("nli_debug_fail_allocation", I, [P, I])
    proto("nli_debug_grid_wait_limit", I, [P, ct.c_uint])
    proto("nli_debug_check_status", I, [P, ct.POINTER(ct.c_ulonglong), ct.POINTER(I)])
    proto("nli_ctx_set_tuning", I, [P, I, I])
    proto("nli_ctx_get_tuning", I, [P, I, ct.POINTER(I)])
    proto("nli_launch_count", ct.c_int64, [])
    proto("nli_ctx_set_profiling", I, [P, I])
    proto("nli_ctx_profile_entry", I, [P, I, ct.c_char_p, I, ct.POINTER(ct.c_int64), ct.POINTER(ct.c_double)])
    proto("nli_ctx_counters", I, [P, ct.POINTER(ct.c_int64), ct.POINTER(ct.c_int64), ct.POINTER(ct.c_int64),
                                  ct.POINTER(ct.c_int64)])
    _libs[path] = L
    if path == LIB_PATH:
        _lib = L
    return L


def _ptr(t):
    """Device pointer of a torch tensor (None passes NULL)."""
    if t is None:
        return None
    return ct.c_void_p(t.data_ptr())


def _dims(t):
    if t.dim() == 2:
        return t.shape[1], t.shape[0], 1
    return t.shape[1], t.shape[0], t.shape[2]


class Context:
    """One nli_ctx: a CUDA device, a stream, the PatchMatch seed and the
    device workspace.  Not thread-safe (one per host thread)."""

    def __init__(self, device=0, lib_path=LIB_PATH):
        import torch
        self.torch = torch
        self.lib = load(lib_path)
        self.device = device
        torch.cuda.init()
        h = ct.c_void_p()
        self.h = None
        self._check(self.lib.nli_ctx_create(device, ct.byref(h)), ctx=None)
        self.h = h
        # order the library's kernels with torch's own work on this device
        self.set_stream(torch.cuda.current_stream(device))

    def close(self):
        if getattr(self, "h", None):
            self.lib.nli_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, ctx="self"):
        if rc != 0:
            msg = self.lib.nli_last_error(self.h).decode() if ctx is not None and self.h else ""
            raise NliError(rc, msg)

    def set_seed(self, seed):
        self._check(self.lib.nli_set_seed(self.h, seed))

    def set_stream(self, stream):
        """Runs subsequent calls on a torch.cuda.Stream."""
        self._check(self.lib.nli_ctx_set_stream(self.h, ct.c_void_p(stream.cuda_stream)))

    def synchronize(self):
        self._check(self.lib.nli_ctx_synchronize(self.h))

    # -- observability
    def launch_count(self):
        return int(self.lib.nli_launch_count())

    def set_profiling(self, enable):
        self._check(self.lib.nli_ctx_set_profiling(self.h, 1 if enable else 0))

    def profile(self):
        """{kernel: (launches, total ms)} collected since set_profiling(True)."""
        out, i = {}, 0
        name = ct.create_string_buffer(64)
        n, ms = ct.c_int64(), ct.c_double()
        while self.lib.nli_ctx_profile_entry(self.h, i, name, 64, ct.byref(n), ct.byref(ms)) == 0:
            out[name.value.decode()] = (n.value, ms.value)
            i += 1
        return out

    def counters(self):
        a, p, b, c = ct.c_int64(), ct.c_int64(), ct.c_int64(), ct.c_int64()
        self._check(self.lib.nli_ctx_counters(self.h, ct.byref(a), ct.byref(p), ct.byref(b), ct.byref(c)))
        return {"candidates": a.value, "candidates_partial": p.value, "cg_iterations": b.value,
                "cg_unknown_iterations": c.value}

    # -- device tensors helpers
    def _f32(self, a):
        t = self.torch
        if isinstance(a, np.ndarray):
            a = t.from_numpy(np.ascontiguousarray(a, np.float32))
        return a.to(device="cuda:%d" % self.device, dtype=t.float32).contiguous()

    def _u8(self, a):
        t = self.torch
        if isinstance(a, np.ndarray):
            a = t.from_numpy(np.ascontiguousarray(a).astype(np.uint8))
        return a.to(device="cuda:%d" % self.device, dtype=t.uint8).contiguous()

    def _i32(self, a):
        t = self.torch
        if isinstance(a, np.ndarray):
            a = t.from_numpy(np.ascontiguousarray(a, np.int32))
        return a.to(device="cuda:%d" % self.device, dtype=t.int32).contiguous()

    def _empty(self, shape, dtype):
        return self.torch.empty(shape, dtype=dtype, device="cuda:%d" % self.device)

    # -- L1 helpers
    def gradient(self, img):
        img = self._f32(img)
        W, H, C = _dims(img)
        out = self._empty((H, W, 2 * C), self.torch.float32)
        self._check(self.lib.nli_gradient(self.h, _ptr(img), W, H, C, _ptr(out)))
        return out

    def gaussian_weights(self, sx, sy, sigma_x, sigma_y):
        out = np.empty((sy, sx), np.float32)
        rc = self.lib.nli_gaussian_weights(sx, sy, sigma_x, sigma_y, out.ctypes.data_as(P))
        if rc:
            raise NliError(rc, "gaussian_weights")
        return out

    def sample_size(self, size, factor):
        return self.lib.nli_sample_size(size, factor)

    def downsample_with_mask(self, img, mask, factor, threshold=0.4, mask_val=False):
        img, mask = self._f32(img), self._u8(mask)
        W, H, C = _dims(img)
        sW, sH = self.sample_size(W, factor), self.sample_size(H, factor)
        oi = self._empty((sH, sW, C), self.torch.float32)
        om = self._empty((sH, sW), self.torch.uint8)
        self._check(self.lib.nli_downsample_with_mask(self.h, _ptr(img), _ptr(mask), W, H, C, factor, threshold,
                                                      1 if mask_val else 0, _ptr(oi), _ptr(om)))
        return oi, om

    def upsample(self, img, oW, oH):
        img = self._f32(img)
        W, H, C = _dims(img)
        out = self._empty((oH, oW, C), self.torch.float32)
        self._check(self.lib.nli_upsample(self.h, _ptr(img), W, H, C, oW, oH, _ptr(out)))
        return out

    def distance_transform(self, mask):
        mask = self._u8(mask)
        out = self._empty(tuple(mask.shape), self.torch.float32)
        self._check(self.lib.nli_distance_transform(self.h, _ptr(mask), mask.shape[1], mask.shape[0], _ptr(out)))
        return out

    def confidence_mask(self, mask, decay=5.0, asym=0.1):
        mask = self._u8(mask)
        out = self._empty(tuple(mask.shape), self.torch.float32)
        self._check(self.lib.nli_confidence_mask(self.h, _ptr(mask), mask.shape[1], mask.shape[0], decay, asym,
                                                 _ptr(out)))
        return out

    def extended_domain(self, mask, px=9, py=9):
        mask = self._u8(mask)
        out = self._empty(tuple(mask.shape), self.torch.uint8)
        self._check(self.lib.nli_extended_domain(self.h, _ptr(mask), mask.shape[1], mask.shape[0], px, py, _ptr(out)))
        return out

    def scale_masks(self, ext, margin, erode):
        ext = self._u8(ext)
        s = self._empty(tuple(ext.shape), self.torch.uint8)
        t = self._empty(tuple(ext.shape), self.torch.uint8)
        e = I()
        self._check(self.lib.nli_scale_masks(self.h, _ptr(ext), ext.shape[1], ext.shape[0], margin, 1 if erode else 0,
                                             _ptr(s), _ptr(t), ct.byref(e)))
        return s, t, bool(e.value)

    def poisson_init(self, img, mask):
        img = self._f32(img).clone()
        mask = self._u8(mask)
        W, H, C = _dims(img)
        self._check(self.lib.nli_poisson_init(self.h, _ptr(img), _ptr(mask), W, H, C))
        return img

    # -- L2a / L3
    def distance_pairs(self, dist, src, tgt, pairs):
        src, tgt, pairs = self._f32(src), self._f32(tgt), self._i32(pairs)
        sW, sH, C = _dims(src)
        tW, tH, _ = _dims(tgt)
        out = self._empty((pairs.shape[0],), self.torch.float32)
        self._check(self.lib.nli_distance_pairs(self.h, ct.byref(dist), _ptr(src), sW, sH, _ptr(tgt), tW, tH, C,
                                                _ptr(pairs), pairs.shape[0], _ptr(out)))
        return out

    def bruteforce_nnf(self, dist, src, smask, tgt, tmask):
        src, tgt, smask, tmask = self._f32(src), self._f32(tgt), self._u8(smask), self._u8(tmask)
        sW, sH, C = _dims(src)
        tW, tH, _ = _dims(tgt)
        nnf = self._empty((tH, tW, 2), self.torch.int32)
        d = self._empty((tH, tW), self.torch.float32)
        self._check(self.lib.nli_bruteforce_nnf(self.h, ct.byref(dist), _ptr(src), _ptr(smask), sW, sH, _ptr(tgt),
                                                _ptr(tmask), tW, tH, C, _ptr(nnf), _ptr(d)))
        return nnf, d

    def patchmatch(self, dist, pm, src, smask, tgt, tmask, init=None, want_energy=True):
        src, tgt, smask, tmask = self._f32(src), self._f32(tgt), self._u8(smask), self._u8(tmask)
        init = None if init is None else self._i32(init)
        sW, sH, C = _dims(src)
        tW, tH, _ = _dims(tgt)
        nnf = self._empty((tH, tW, 2), self.torch.int32)
        d = self._empty((tH, tW), self.torch.float32)
        e = ct.c_double()
        self._check(self.lib.nli_patchmatch(self.h, ct.byref(dist), ct.byref(pm), _ptr(src), _ptr(smask), sW, sH,
                                            _ptr(tgt), _ptr(tmask), tW, tH, C, _ptr(init), _ptr(nnf), _ptr(d),
                                            ct.byref(e) if want_energy else None))
        return nnf, d, e.value

    # -- L2b
    def update(self, upd, image, orig, dom, ext, nnf, conf=None, same_orig=False):
        """Returns (updated image, total difference); `image` is not modified."""
        img = self._f32(image).clone()
        W, H, C = _dims(img)
        org = img if same_orig else self._f32(orig)
        dom, ext, nnf = self._u8(dom), self._u8(ext), self._i32(nnf)
        conf = None if conf is None else self._f32(conf)
        tot = ct.c_double()
        self._check(self.lib.nli_update(self.h, ct.byref(upd), _ptr(img), _ptr(org), _ptr(dom), _ptr(ext), _ptr(nnf),
                                        _ptr(conf), W, H, C, ct.byref(tot)))
        return img, tot.value

    def patchmatch_metrics(self, dist, pm, src, smask, tgt, tmask, init=None):
        """PatchMatch with the reference's METRICS figures: returns (nnf,
        distance, energy, total distance per sweep, propagations per sweep,
        max random-shot index)."""
        src, tgt, smask, tmask = self._f32(src), self._f32(tgt), self._u8(smask), self._u8(tmask)
        init = None if init is None else self._i32(init)
        sW, sH, C = _dims(src)
        tW, tH, _ = _dims(tgt)
        nnf = self._empty((tH, tW, 2), self.torch.int32)
        d = self._empty((tH, tW), self.torch.float32)
        n = max(pm.iterations, 1)
        tot = (ct.c_double * n)()
        prop = (ct.c_int64 * n)()
        e, shots = ct.c_double(), ct.c_int32()
        self._check(self.lib.nli_patchmatch_metrics(self.h, ct.byref(dist), ct.byref(pm), _ptr(src), _ptr(smask), sW,
                                                    sH, _ptr(tgt), _ptr(tmask), tW, tH, C, _ptr(init), _ptr(nnf),
                                                    _ptr(d), ct.byref(e), tot, prop, ct.byref(shots)))
        k = pm.iterations
        return nnf, d, e.value, list(tot)[:k], list(prop)[:k], shots.value

    def rgb_to_lab(self, rgb):
        """IOUtility::rgb_to_lab on the GPU (sRGB 0..255, 3 channels)."""
        rgb = self._f32(rgb)
        W, H, _ = _dims(rgb)
        out = self._empty((H, W, 3), self.torch.float32)
        self._check(self.lib.nli_rgb_to_lab(self.h, _ptr(rgb), W, H, _ptr(out)))
        return out

    def lab_to_rgb(self, lab):
        """IOUtility::lab_to_rgb on the GPU (3 or 4 channels in, 3 out)."""
        lab = self._f32(lab)
        W, H, C = _dims(lab)
        out = self._empty((H, W, 3), self.torch.float32)
        self._check(self.lib.nli_lab_to_rgb(self.h, _ptr(lab), W, H, C, _ptr(out)))
        return out

    def cat_depth(self, rgb, depth):
        rgb, depth = self._f32(rgb), self._f32(depth)
        W, H, _ = _dims(rgb)
        out = self._empty((H, W, 4), self.torch.float32)
        self._check(self.lib.nli_cat_depth(self.h, _ptr(rgb), _ptr(depth), W, H, _ptr(out)))
        return out

    def separate_depth(self, rgbd):
        rgbd = self._f32(rgbd)
        W, H, _ = _dims(rgbd)
        rgb = self._empty((H, W, 3), self.torch.float32)
        depth = self._empty((H, W), self.torch.float32)
        self._check(self.lib.nli_separate_depth(self.h, _ptr(rgbd), W, H, _ptr(rgb), _ptr(depth)))
        return rgb, depth

    INTER_INPUT, INTER_OUTPUT, INTER_MASK, INTER_NNF = 0, 1, 2, 3

    def keep_intermediate(self, enable=True):
        """ImageInpainting::keep_intermediate for the next process() calls."""
        self._check(self.lib.nli_ctx_keep_intermediate(self.h, 1 if enable else 0))

    def intermediate(self, kind):
        """Kept pyramid of `kind` (INTER_INPUT / OUTPUT / MASK: per level,
        finest first; INTER_NNF: per inpainted level, coarsest first) as
        numpy arrays."""
        count = self.lib.nli_intermediate_count(self.h, kind)
        if count < 0:
            raise NliError(count, "bad intermediate kind")
        dtype = {0: np.float32, 1: np.float32, 2: np.uint8, 3: np.int32}[kind]
        out = []
        for i in range(count):
            W, H, C = I(), I(), I()
            self._check(self.lib.nli_intermediate_get(self.h, kind, i, ct.byref(W), ct.byref(H), ct.byref(C), None))
            a = np.empty((H.value, W.value, C.value), dtype)
            self._check(self.lib.nli_intermediate_get(self.h, kind, i, None, None, None, a.ctypes.data_as(P)))
            out.append(a[..., 0] if kind == 2 else a)
        return out

    def update_backward(self, upd, image, out, dom, ext, nnf, conf, grad_out):
        """Adjoint of update(upd, image, image, ...) with the NNF fixed:
        returns (dL/dimage, dL/dlambda, dL/dlambda_d, dL/dsigma)."""
        img, out, g = self._f32(image), self._f32(out), self._f32(grad_out)
        W, H, C = _dims(img)
        dom, ext, nnf = self._u8(dom), self._u8(ext), self._i32(nnf)
        conf = None if conf is None else self._f32(conf)
        gi = self.torch.empty_like(img)
        dl, dld, ds = ct.c_double(), ct.c_double(), ct.c_double()
        self._check(self.lib.nli_update_backward(self.h, ct.byref(upd), _ptr(img), _ptr(out), _ptr(dom), _ptr(ext),
                                                 _ptr(nnf), _ptr(conf), W, H, C, _ptr(g), _ptr(gi), ct.byref(dl),
                                                 ct.byref(dld), ct.byref(ds)))
        return gi, dl.value, dld.value, ds.value

    # -- L4
    def process(self, img, mask, params, stats=True):
        """ImageInpainting::process on host arrays (numpy in, numpy out)."""
        img = np.ascontiguousarray(img, np.float32)
        mask = np.ascontiguousarray(mask).astype(np.uint8)
        H, W = img.shape[:2]
        C = 1 if img.ndim == 2 else img.shape[2]
        out = np.empty_like(img)
        st = ProcessStats()
        self._check(self.lib.nli_process(self.h, ct.byref(params), img.ctypes.data_as(P), mask.ctypes.data_as(P),
                                         W, H, C, out.ctypes.data_as(P), ct.byref(st)))
        return out, st.as_dict()

    def set_batch_width(self, width):
        """Images in flight at once in process_batch."""
        self._check(self.lib.nli_ctx_set_batch_width(self.h, width))

    def _batch_arrays(self, items, params, device):
        n = len(items)
        pa = (ProcessParams * n)(*params)
        arr = lambda T, vals: (T * n)(*vals)  # noqa: E731
        if device:
            dims = [_dims(img) for img, _ in items]
            ptr = lambda t: t.data_ptr()  # noqa: E731
        else:
            dims = [(img.shape[1], img.shape[0], 1 if img.ndim == 2 else img.shape[2]) for img, _ in items]
            ptr = lambda a: a.ctypes.data  # noqa: E731
        return (n, pa, arr(ct.c_void_p, [ptr(i) for i, _ in items]), arr(ct.c_void_p, [ptr(m) for _, m in items]),
                arr(ct.c_int32, [d[0] for d in dims]), arr(ct.c_int32, [d[1] for d in dims]),
                arr(ct.c_int32, [d[2] for d in dims]))

    def process_batch(self, items, params):
        """Many (image, mask) host pairs with one params entry each; returns
        ([outputs], [stats]).  Image i is computed as process() after
        set_seed(batch_seed(seed, i))."""
        items = [(np.ascontiguousarray(i, np.float32), np.ascontiguousarray(m).astype(np.uint8)) for i, m in items]
        outs = [np.empty_like(i) for i, _ in items]
        n, pa, ims, ms, ws, hs, cs = self._batch_arrays(items, params, False)
        op = (ct.c_void_p * n)(*[o.ctypes.data for o in outs])
        st = (ProcessStats * n)()
        status = (ct.c_int32 * n)()
        rc = self.lib.nli_process_batch(self.h, n, pa, ims, ms, ws, hs, cs, op, st, status)
        self.last_batch_status = list(status)
        self._check(rc)
        return outs, [s.as_dict() for s in st]

    def process_batch_device(self, items, params, outs=None):
        """process_batch on device tensors; returns ([outputs], [stats])."""
        items = [(self._f32(i), self._u8(m)) for i, m in items]
        if outs is None:
            outs = [self.torch.empty_like(i) for i, _ in items]
        n, pa, ims, ms, ws, hs, cs = self._batch_arrays(items, params, True)
        op = (ct.c_void_p * n)(*[o.data_ptr() for o in outs])
        st = (ProcessStats * n)()
        status = (ct.c_int32 * n)()
        rc = self.lib.nli_process_batch_device(self.h, n, pa, ims, ms, ws, hs, cs, op, st, status)
        self.last_batch_status = list(status)
        self._check(rc)
        return outs, [s.as_dict() for s in st]

    TUNE_CG_CLUSTER_CAP, TUNE_CG_UNKNOWNS_PER_CTA, TUNE_BATCH_WIDTH, TUNE_PM_VARIANT, TUNE_CG_PRECOND, TUNE_GRAPH_LOOP = 0, 1, 2, 3, 4, 5
    TUNE_CG_SINGLE_MAX, TUNE_BATCH_MODE, TUNE_PM_BOUND, TUNE_BATCH_GROUPS, TUNE_PM_TILE = 6, 7, 8, 9, 10

    def set_tuning(self, knob, value):
        self._check(self.lib.nli_ctx_set_tuning(self.h, knob, value))

    def get_tuning(self, knob):
        v = I()
        self._check(self.lib.nli_ctx_get_tuning(self.h, knob, ct.byref(v)))
        return v.value

    def batch_seed(self, seed, index):
        return int(self.lib.nli_batch_seed(seed, index))

    def fail_allocation(self, countdown):
        """Test hook: the countdown-th next workspace growth fails with
        NLI_E_NOMEM (nli_debug_fail_allocation); 0 disarms."""
        self._check(self.lib.nli_debug_fail_allocation(self.h, countdown))

    def grid_wait_limit(self, polls):
        """Test hook: the grid CG's barrier gives up after `polls` polls
        (nli_debug_grid_wait_limit); 0 restores the default."""
        self._check(self.lib.nli_debug_grid_wait_limit(self.h, polls))

    def check_status(self):
        """(word, checked) of nli_debug_check_status: the first out-of-range
        gathered index of a checked build ((site << 32) | index), cleared."""
        w, c = ct.c_ulonglong(), I()
        self._check(self.lib.nli_debug_check_status(self.h, ct.byref(w), ct.byref(c)))
        return int(w.value), bool(c.value)

    def process_device(self, img, mask, params, out=None):
        """ImageInpainting::process on device tensors; returns (out, stats)."""
        img, mask = self._f32(img), self._u8(mask)
        W, H, C = _dims(img)
        if out is None:
            out = self.torch.empty_like(img)
        st = ProcessStats()
        self._check(self.lib.nli_process_device(self.h, ct.byref(params), _ptr(img), _ptr(mask), W, H, C, _ptr(out),
                                                ct.byref(st)))
        return out, st.as_dict()
