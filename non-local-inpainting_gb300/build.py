"""Compiles the CUDA library in-tree: non-local-inpainting_gb300/libnli_gb300.so
for sm_103a (GB300), one nvcc process per translation unit, in parallel."""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnli_gb300.so")
DROPIN = os.path.join(HERE, "libnli_dropin.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")

SOURCES = ["api.cu", "gradient.cu", "distance.cu", "patchmatch.cu", "update.cu", "pyramid.cu", "process.cu",
           "batch.cu", "color.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra=(), checked=False):
    """Compiles libnli_gb300.so (and the drop-in library and the command-line
    program); checked=True instead compiles libnli_gb300_checked.so with
    NLI_CHECKED, the build whose kernels bounds-test every gathered index."""
    if checked:
        return _build_lib(os.path.join(OBJ, "checked"), LIB_CHECKED, force, verbose, list(extra) + ["-DNLI_CHECKED"])
    _build_lib(OBJ, LIB, force, verbose, extra)
    build_dropin(force)
    build_cli(force)
    return LIB


LIB_CHECKED = os.path.join(HERE, "libnli_gb300_checked.so")


def _build_lib(objdir, lib, force, verbose, extra):
    OBJ = objdir
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "nli.h"))
    nvcc = _nvcc()
    jobs, objs = [], []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, __file__] + headers):
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            print(o)
    if force or jobs or _stale(lib, objs):
        _run([nvcc, *ARCH, "-shared", *objs, "-o", lib + ".tmp", "-lcudart"])
        os.replace(lib + ".tmp", lib)
    return lib


def build_dropin(force=False):
    """libnli_dropin.so: the C++ classes of include/nli_inpainting.hpp over the C ABI."""
    src = os.path.join(CSRC, "dropin.cpp")
    deps = [src, LIB, os.path.join(ROOT, "include", "nli_inpainting.hpp"), os.path.join(ROOT, "include", "nli.h")]
    if not force and not _stale(DROPIN, deps):
        return DROPIN
    _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", os.path.join(ROOT, "include"),
          "-I", os.path.join(CUDA_HOME, "include"), src, "-o", DROPIN + ".tmp", "-L", HERE, "-lnli_gb300",
          "-L", os.path.join(CUDA_HOME, "lib64"), "-lcudart", "-Wl,-rpath,$ORIGIN"])
    os.replace(DROPIN + ".tmp", DROPIN)
    return DROPIN


CLI = os.path.join(HERE, "nli_inpaint")


def build_cli(force=False):
    """nli_inpaint: the reference's command-line program over the drop-in classes."""
    src = os.path.join(CSRC, "cli.cpp")
    png = [os.path.join(CSRC, "png_codec.cpp"), os.path.join(CSRC, "png_codec.h")]
    deps = [src, LIB, DROPIN, os.path.join(ROOT, "include", "nli_inpainting.hpp"),
            os.path.join(ROOT, "include", "nli.h")] + png
    if not force and not _stale(CLI, deps):
        return CLI
    _run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA_HOME, "include"),
          "-I", CSRC, src, png[0], "-o", CLI + ".tmp", "-L", HERE, "-lnli_dropin", "-lnli_gb300",
          "-L", os.path.join(CUDA_HOME, "lib64"), "-lcudart", "-Wl,-rpath,$ORIGIN"])
    os.replace(CLI + ".tmp", CLI)
    return CLI


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
