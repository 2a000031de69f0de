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
