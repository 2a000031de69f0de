"""The C ABI from C++: tests/cpp/rms2d_caller.cpp, written like the cpptraj-side
call sites of the drop-in (a patched Analysis_Rms2d::Calculate_2D), is compiled with g++ against include/gbrmsd.h and
libgbrmsd.so, run on the GPU, and its TRI / FULL / dme outputs are compared
with the FP64 oracle (1e-4 Angstrom, the bar of this path)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from cpptraj_gb300 import gbrmsd, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def compile_caller(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    libdir = os.path.dirname(gbrmsd.LIB_PATH)
    exe = str(tmp_path / "rms2d_caller")
    cmd = [gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "rms2d_caller.cpp"), "-o", exe,
           "-L", libdir, "-lgbrmsd", "-Wl,-rpath," + libdir]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_header_compiles_as_c_and_cpp(tmp_path):
    """The header is plain C: it must compile as C99 and as C++ (no GPU needed)."""
    for cc, std, src in (("gcc", "-std=c99", "c.c"), ("g++", "-std=c++11", "c.cpp")):
        comp = shutil.which(cc)
        if comp is None:
            pytest.skip(f"{cc} not available")
        p = tmp_path / src
        p.write_text('#include "gbrmsd.h"\nint main(void) { return (int)GBR_OK; }\n')
        subprocess.run([comp, std, "-Wall", "-Werror", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), str(p)],
                       check=True, capture_output=True, text=True)


@pytest.mark.gpu
def test_cpp_caller_matches_oracle(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if not os.path.exists(gbrmsd.LIB_PATH):
        from cpptraj_gb300 import build
        build.build()
    exe = compile_caller(tmp_path)
    X, m = synth.trajectory(91, 130, 211, 0.2, 2.5, np.float64, True)
    F, N = X.shape[0], X.shape[1]
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as fh:
        fh.write(np.int64(F).tobytes() + np.int32(N).tobytes() + np.int32(1).tobytes())
        fh.write(X.tobytes() + m.tobytes())
    r = subprocess.run([exe, str(inp), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    vals = np.fromfile(out, dtype=np.float32)
    ntri, nr = F * (F - 1) // 2, F // 2
    tri, full, dme = vals[:ntri], vals[ntri:ntri + nr * (F - nr)], vals[ntri + nr * (F - nr):]
    assert dme.size == ntri
    np.testing.assert_allclose(tri, oracle.allpairs_f64(X, tgt_mass=m), rtol=0, atol=1e-4)
    np.testing.assert_allclose(full, oracle.allpairs_f64(X[:nr], X[nr:], tgt_mass=m), rtol=0, atol=1e-4)
    np.testing.assert_allclose(dme, oracle.allpairs_f64(X, mode=oracle.DME), rtol=0, atol=1e-5)
