"""Host logic of the tensor-core launch: the grouped tile list and its stable
partition into input-chunk stages (cpptraj_gb300/csrc/gbr_tiles.h), compiled
with g++ and checked against a direct restatement over 20,000 random output
regions, tile shapes and chunk counts (no GPU needed)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def cuda_include():
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "vector_types.h")):
            return os.path.join(d, "include")
    return None


def test_staged_tile_list_matches_direct(tmp_path):
    gxx = shutil.which("g++")
    inc = cuda_include()
    if gxx is None or inc is None:
        pytest.skip("g++ or the CUDA headers not available")
    exe = str(tmp_path / "tiles_check")
    subprocess.run([gxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I", inc,
                    "-I", os.path.join(ROOT, "cpptraj_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "tiles_check.cpp"), "-o", exe],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout
