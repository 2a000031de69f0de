"""The drop-in inside cpptraj itself: cpptraj_gb300/integration/gb_rmsd.patch
applied to a copy of the reference's src/ tree, and the patched translation
units compiled with -DGB_RMSD against the reference's own headers and
include/gbrmsd.h.

Patched: Analysis_Rms2d::Calculate_2D (src/Analysis_Rms2d.cpp:196-295; fit,
nofit, dme and qrmsd through gbr_allpairs), MetricArray::calcFrameDistances
(src/Cluster/MetricArray.cpp:766-801; one RMS metric into an in-memory
pairwise cache) and two read accessors in src/Cluster/Metric_RMS.h.  The
patch only inserts lines.  Skipped where the reference tree is absent
(GBR_REFERENCE_SRC, default the survey location)."""
import os
import shutil
import subprocess

import pytest

from cpptraj_gb300 import gbrmsd

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PATCH = os.path.join(ROOT, "cpptraj_gb300", "integration", "gb_rmsd.patch")
REF_SRC = os.environ.get("GBR_REFERENCE_SRC", "/root/reference/src")
UNITS = ["Analysis_Rms2d.cpp", "Cluster/MetricArray.cpp"]


def test_patch_only_inserts_lines():
    body = open(PATCH).read().splitlines()
    files = [ln.split()[1] for ln in body if ln.startswith("--- ")]
    assert files == ["a/src/Analysis_Rms2d.cpp", "a/src/Cluster/MetricArray.cpp", "a/src/Cluster/Metric_RMS.h"]
    removed = [ln for ln in body if ln.startswith("-") and not ln.startswith("--- ")]
    assert removed == []
    added = [ln for ln in body if ln.startswith("+") and not ln.startswith("+++ ")]
    assert any("gbr_allpairs(" in ln for ln in added)


@pytest.fixture(scope="module")
def patched_tree(tmp_path_factory):
    if not os.path.isdir(REF_SRC):
        pytest.skip("reference source tree not present")
    if shutil.which("patch") is None or shutil.which("g++") is None:
        pytest.skip("patch / g++ not available")
    top = tmp_path_factory.mktemp("cpptraj")
    shutil.copytree(REF_SRC, top / "src")
    r = subprocess.run(["patch", "-p1", "-i", PATCH], cwd=top, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return top


@pytest.mark.parametrize("unit", UNITS)
def test_patched_unit_compiles(patched_tree, unit):
    obj = patched_tree / (os.path.basename(unit) + ".o")
    cmd = ["g++", "-std=c++11", "-fopenmp", "-Wall", "-Werror=return-type", "-DGB_RMSD",
           "-I" + os.path.join(ROOT, "include"), "-I" + str(patched_tree / "src"),
           "-c", str(patched_tree / "src" / unit), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    assert "warning" not in r.stderr, r.stderr[-4000:]
    # every library symbol the unit needs is one include/gbrmsd.h declares
    nm = subprocess.run(["nm", "-u", str(obj)], capture_output=True, text=True).stdout
    used = {ln.split()[-1] for ln in nm.splitlines() if ln.split() and ln.split()[-1].startswith("gbr_")}
    assert used and used <= set(gbrmsd.EXPORTED), used
