"""Build recipe for the oracle (test infrastructure only).

Two libraries:

* ``oracle/_build/libnlioracle.so`` -- the C++ restatement of the reference
  algorithm in ``oracle/nli_oracle.cpp`` (this repository's own code).  Built
  on every machine, including the GPU machine.
* ``oracle/_build/libnlioracle_timing.so`` -- the same restatement built with
  the reference's Release flags, only to time the reference algorithm on the
  host cores (the CPU baseline).
* ``oracle/_ref/libnliref.so`` (serial, ``-DMETRICS``) and
  ``oracle/_ref/libnliref_omp.so`` (OpenMP) -- the UNMODIFIED reference
  sources compiled where they lie (``NLI_REFERENCE_DIR``, by default
  ``/root/reference``) together with ``oracle/ref_driver.cpp``.  Built only
  when that directory holds them.  The
  reference's own CMake build cannot run here (CMake 4 rejects its minimum
  version and its iio.h forces libpng/libjpeg/libtiff, which are absent), so
  this recipe compiles the sources directly with the flags of the reference's
  Release build (-O3, -std=c99 for simpois) and replaces the image-file
  library by ``oracle/iio_stub`` (file I/O is not on the inpainting path).
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
# Where the reference sources lie: NLI_REFERENCE_DIR, else the development
# container's mount; the reference build is skipped where neither holds them.
REFERENCE = os.environ.get("NLI_REFERENCE_DIR", "/root/reference")
REF_OUT = os.path.join(HERE, "_ref")
BUILD_OUT = os.path.join(HERE, "_build")

# Reference translation units of the inpainting path (main.cpp is the CLI).
REF_SOURCES = [
    "a_image_updating.cpp", "image_inpainting.cpp", "l1_norm_patch_distance.cpp",
    "l2_norm_patch_distance.cpp", "l2_combined_patch_distance.cpp", "a_patch_distance.cpp",
    "point.cpp", "distance_transform.cpp", "patch_match.cpp", "gaussian_weights.cpp",
    "patch_non_local_means.cpp", "patch_non_local_poisson.cpp", "sampling.cpp",
    "io_utility.cpp", "mask_iterator.cpp", "patch_non_local_medians.cpp", "shape.cpp",
    "gradient.cpp", "mask.cpp", "patch_non_local_depth.cpp", "l2_rgbd_patch_distance.cpp",
]

# Plain IEEE single/double arithmetic on every host: no FMA contraction, so
# x86_64 and aarch64 builds round identically.
FP_FLAGS = ["-ffp-contract=off"]


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d))


def build_oracle(force=False):
    """Compile the restatement; returns the path of libnlioracle.so."""
    os.makedirs(BUILD_OUT, exist_ok=True)
    out = os.path.join(BUILD_OUT, "libnlioracle.so")
    src = os.path.join(HERE, "nli_oracle.cpp")
    deps = [src, os.path.join(REPO, "include", "nli.h"), __file__]
    if not force and _newer(out, deps):
        return out
    _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", *FP_FLAGS,
          "-I", os.path.join(REPO, "include"), src, "-o", out + ".tmp", "-lm"])
    os.replace(out + ".tmp", out)
    return out


# The flags of the reference's own Release build (CMakeLists.txt: Release
# -O3 -DNDEBUG, OpenMP compile flags on the target, the compiler's default
# floating-point contraction), for timing the reference algorithm on the
# host cores.  Not bit-exact with the reference's float/double rounding on
# hosts whose compiler contracts multiply-adds (aarch64), so never used as
# the parity checker.
TIMING_FLAGS = ["-O3", "-DNDEBUG", "-std=gnu++17", "-fopenmp"]


def build_timing(force=False):
    """Compile the restatement with the reference's Release flags; returns
    the path of libnlioracle_timing.so."""
    os.makedirs(BUILD_OUT, exist_ok=True)
    out = os.path.join(BUILD_OUT, "libnlioracle_timing.so")
    src = os.path.join(HERE, "nli_oracle.cpp")
    deps = [src, os.path.join(REPO, "include", "nli.h"), __file__]
    if not force and _newer(out, deps):
        return out
    _run(["g++", *TIMING_FLAGS, "-fPIC", "-shared", "-I", os.path.join(REPO, "include"), src,
          "-o", out + ".tmp", "-lm"])
    os.replace(out + ".tmp", out)
    return out


def reference_available():
    return os.path.isfile(os.path.join(REFERENCE, "patch_match.cpp"))


def _build_ref_variant(name, extra, force):
    objdir = os.path.join(REF_OUT, "obj_" + name)
    os.makedirs(objdir, exist_ok=True)
    out = os.path.join(REF_OUT, "libnliref%s.so" % ("" if name == "serial" else "_" + name))
    driver = os.path.join(HERE, "ref_driver.cpp")
    stub = os.path.join(HERE, "iio_stub", "iio_stub.c")
    deps = [os.path.join(REFERENCE, s) for s in REF_SOURCES] + [driver, stub, __file__]
    if not force and _newer(out, deps):
        return out
    inc = ["-I", os.path.join(HERE, "iio_stub"), "-I", REFERENCE]
    jobs = []
    for s in REF_SOURCES:
        jobs.append(["g++", "-O3", "-DNDEBUG", "-fPIC", "-w", *FP_FLAGS, *extra, *inc, "-c",
                     os.path.join(REFERENCE, s), "-o", os.path.join(objdir, s + ".o")])
    jobs.append(["gcc", "-O3", "-DNDEBUG", "-std=c99", "-fPIC", "-w", *FP_FLAGS, "-c",
                 os.path.join(REFERENCE, "3rdparty", "simpois", "simpois.c"),
                 "-o", os.path.join(objdir, "simpois.o")])
    jobs.append(["gcc", "-O2", "-fPIC", *inc, "-c", stub, "-o", os.path.join(objdir, "iio_stub.o")])
    jobs.append(["g++", "-O2", "-fPIC", "-w", *FP_FLAGS, *extra, *inc, "-I",
                 os.path.join(REPO, "include"), "-c", driver,
                 "-o", os.path.join(objdir, "ref_driver.o")])
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs))
    objs = [os.path.join(objdir, f) for f in sorted(os.listdir(objdir)) if f.endswith(".o")]
    _run(["g++", "-shared", *extra, *objs, "-o", out + ".tmp", "-lm"])
    os.replace(out + ".tmp", out)
    return out


def build_reference(force=False):
    """Compile the reference sources (only where /root/reference exists)."""
    if not reference_available():
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    serial = _build_ref_variant("serial", ["-DMETRICS"], force)
    _build_ref_variant("omp", ["-fopenmp"], force)
    return serial


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_oracle(force))
    print(build_timing(force))
    print(build_reference(force))
