"""C-ABI checks that need no GPU: the library loads, exports every function
include/gbrmsd.h declares, and its host-only index arithmetic matches the
oracle's."""
import os
import re

import numpy as np
import pytest

import oracle
from cpptraj_gb300 import gbrmsd

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names.update(re.findall(r"\b(gbr_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(gbrmsd.LIB_PATH):
        from cpptraj_gb300 import build
        build.build()
    return gbrmsd.load()


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert set(names) == set(gbrmsd.EXPORTED)
    for n in names:
        assert hasattr(lib, n), n


@pytest.mark.parametrize("n_ref,n_tgt,kind,rb,re_", [
    (10, 10, 0, 0, -1), (10, 10, 0, 3, 7), (1, 1, 0, 0, -1), (2, 2, 0, 0, -1),
    (10, 14, 1, 0, -1), (10, 14, 1, 3, 14), (500, 500, 0, 499, 500), (7, 3, 1, 0, 0)])
def test_output_count_matches_oracle(lib, n_ref, n_tgt, kind, rb, re_):
    got = gbrmsd.output_count(n_ref, n_tgt, kind, rb, re_)
    want = oracle.n_out(n_ref, n_tgt, kind, rb, None if re_ < 0 else re_)
    assert got == want


def test_header_enums_match_binding():
    text = open(os.path.join(ROOT, "include", "gbrmsd.h")).read()
    for name, val in (("GBR_F32", 0), ("GBR_F64", 1), ("GBR_FIT", 0), ("GBR_NOFIT", 1), ("GBR_TRI", 0),
                      ("GBR_FULL", 1), ("GBR_PREC_FP32", 0), ("GBR_PREC_TC", 1), ("GBR_PREC_FP64", 2)):
        assert re.search(rf"\b{name}\s*=\s*{val}\b", text), name


class _NoCallLib:
    """Stands in for the library inside a Handle: argument checks must reject a
    bad call before any pointer reaches it."""

    def __getattr__(self, name):
        def fail(*a, **k):
            raise AssertionError(f"{name} was called with arguments the wrapper should have rejected")
        return fail


@pytest.fixture()
def stub_handle(lib):
    h = gbrmsd.Handle.__new__(gbrmsd.Handle)
    h.lib = _NoCallLib()
    h.h = None
    h.device = 0
    return h


def test_wrapper_rejects_bad_buffers(stub_handle):
    h = stub_handle
    X = np.zeros((4, 5, 3), np.float32)
    cases = [
        (ValueError, lambda: h.allpairs(np.zeros((4, 5), np.float32))),
        (TypeError, lambda: h.allpairs(X.astype(np.float16))),
        (TypeError, lambda: h.allpairs(X, out=np.zeros(6, np.float64))),
        (ValueError, lambda: h.allpairs(X, out=np.zeros(5, np.float32))),
        (ValueError, lambda: h.allpairs(X, tgt_mass=np.ones(4))),
        (ValueError, lambda: h.allpairs(X, np.zeros((3, 6, 3), np.float32))),
        (ValueError, lambda: h.allpairs(X, np.zeros((3, 5, 3), np.float64))),
        (ValueError, lambda: h.allpairs(X, np.zeros((3, 5, 3), np.float32), out=np.zeros(11, np.float32))),
        (ValueError, lambda: h.superpose(X[0, :4], X)),
        (ValueError, lambda: h.superpose(X[0], X, mass=np.ones(6))),
        (ValueError, lambda: h.superpose(X[0], X, move=np.zeros((3, 2, 3), np.float32))),
        (TypeError, lambda: h.backward(X.astype(np.float64))),
        (ValueError, lambda: h.backward(X, g=np.ones(5, np.float32))),
        (TypeError, lambda: h.backward(X, g=np.ones(6, np.float64))),
        (ValueError, lambda: h.backward(X, rmsd_out=np.zeros(5, np.float32))),
        (ValueError, lambda: h.backward(X, grad=np.zeros((4, 5, 2), np.float32))),
        (ValueError, lambda: h.cluster_centroids(X, np.array([0, 1], np.int32), np.array([[0, 2]], np.int64))),
        (ValueError, lambda: h.cluster_centroids(X, np.array([0, 1], np.int32), np.array([0, 2]), mass=np.ones(3))),
        (TypeError, lambda: h.allpairs_batched([X, X.astype(np.float64)])),
        (ValueError, lambda: h.allpairs_batched([X], masses=[np.ones(4)])),
        (ValueError, lambda: h.allpairs_batched([X], masses=[None, None])),
        (ValueError, lambda: h.allpairs_stream(X, lambda *a: None, mass=np.ones(2))),
        (ValueError, lambda: h.write_cmatrix("unused.cmatrix", X[:, :, :2])),
    ]
    for exc, call in cases:
        with pytest.raises(exc):
            call()
