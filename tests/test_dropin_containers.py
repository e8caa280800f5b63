"""The drop-in's container API (include/nli_inpainting.hpp) compiled into a
host program written like the reference's own callers
(tests/cpp/mask_api.cpp) and run on the CPU: mask iteration in raster order
and in reverse, first / last / next / prev, the bounding box, channel
overloads, range-checked at(), mask / unmask by Point, sharing copies and
deep copies (mask.h, mask_iterator.h, mask.cpp:158-486, 844-878)."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT


def test_mask_api_program(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "mask_api")
    src = os.path.join(ROOT, "tests", "cpp", "mask_api.cpp")
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), src, "-o",
                    exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "mask api ok" in r.stdout
