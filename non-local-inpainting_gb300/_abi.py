"""ctypes mirror of include/nli.h (structs, enums, status codes)."""
from __future__ import annotations

import ctypes as ct

NLI_OK = 0
NLI_E_INVALID = -1
NLI_E_EMPTY_SOURCE = -2
NLI_E_CHANNELS = -3
NLI_E_SHAPE = -4
NLI_E_UNSUPPORTED = -5
NLI_E_CUDA = -6
NLI_E_TIMEOUT = -7
NLI_E_NOMEM = -8

NLI_DIST_L2_COMBINED = 0
NLI_DIST_L2_RGBD = 1
NLI_DIST_L2_NORM = 2
NLI_DIST_L1_NORM = 3

NLI_UPDATE_MEANS = 0
NLI_UPDATE_MEDIANS = 1
NLI_UPDATE_POISSON = 2
NLI_UPDATE_DEPTH = 3

NLI_INIT_BLACK = 0
NLI_INIT_AVG = 1
NLI_INIT_NONE = 2
NLI_INIT_POISSON = 3

NLI_MAX_SCALES = 32


class DistanceParams(ct.Structure):
    _fields_ = [("kind", ct.c_int32), ("patch_x", ct.c_int32), ("patch_y", ct.c_int32),
                ("sigma", ct.c_float), ("lambda_", ct.c_float), ("lambda_d", ct.c_float)]


class PatchMatchParams(ct.Structure):
    _fields_ = [("iterations", ct.c_int32), ("random_shots", ct.c_int32), ("window", ct.c_int32)]


class UpdateParams(ct.Structure):
    _fields_ = [("method", ct.c_int32), ("patch_x", ct.c_int32), ("patch_y", ct.c_int32),
                ("sigma", ct.c_float), ("lambda_", ct.c_float), ("lambda_d", ct.c_float),
                ("cg_tol", ct.c_float), ("cg_iters", ct.c_int32)]


class ProcessParams(ct.Structure):
    _fields_ = [("distance", DistanceParams), ("patchmatch", PatchMatchParams),
                ("update", UpdateParams), ("iterations", ct.c_int32), ("tolerance", ct.c_float),
                ("scales", ct.c_int32), ("subsampling_rate", ct.c_float),
                ("conf_decay_time", ct.c_float), ("conf_asymptotic", ct.c_float),
                ("init", ct.c_int32)]


class ProcessStats(ct.Structure):
    _fields_ = [("scales", ct.c_int32),
                ("width", ct.c_int32 * NLI_MAX_SCALES), ("height", ct.c_int32 * NLI_MAX_SCALES),
                ("iterations", ct.c_int32 * NLI_MAX_SCALES),
                ("last_difference", ct.c_double * NLI_MAX_SCALES),
                ("patchmatch_calls", ct.c_int64), ("update_calls", ct.c_int64),
                ("cg_iterations", ct.c_int64), ("candidates", ct.c_int64),
                ("graph_iterations", ct.c_int64),
                ("targets", ct.c_int32 * NLI_MAX_SCALES), ("holes", ct.c_int32 * NLI_MAX_SCALES),
                ("candidates_partial", ct.c_int64)]

    def as_dict(self):
        n = self.scales
        return {"scales": n, "width": list(self.width[:n]), "height": list(self.height[:n]),
                "iterations": list(self.iterations[:n]),
                "last_difference": list(self.last_difference[:n]),
                "patchmatch_calls": self.patchmatch_calls, "update_calls": self.update_calls,
                "cg_iterations": self.cg_iterations, "candidates": self.candidates,
                "graph_iterations": self.graph_iterations, "targets": list(self.targets[:n]),
                "holes": list(self.holes[:n]), "candidates_partial": self.candidates_partial}


_libm = None


def subsampling_rate(size_ratio, scales):
    """ImageInpainting::calculate_subsampling_rate (image_inpainting.cpp:197-204).
    The reference evaluates exp(log(r)/(S-1)) with the float overloads of
    exp and log (expf/logf of the C library), reproduced here through libm."""
    global _libm
    import numpy as np
    if _libm is None:
        _libm = ct.CDLL("libm.so.6")
        _libm.expf.restype = ct.c_float
        _libm.expf.argtypes = [ct.c_float]
        _libm.logf.restype = ct.c_float
        _libm.logf.argtypes = [ct.c_float]
    r = np.float32(size_ratio)
    if r < 0 or r > 1:
        return 0.0
    q = np.float32(_libm.logf(float(r))) / np.float32(scales - 1)
    return float(_libm.expf(float(np.float32(q))))


def copy_params(p):
    q = ProcessParams()
    ct.pointer(q)[0] = p
    return q
