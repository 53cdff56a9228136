"""The C-ABI library loads and exports every symbol include/iemic_gb300.h declares."""
import os
import re

from iemic import ocean as O
from iemic import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "iemic_gb300.h")).read()
    return sorted(set(re.findall(r"\b(iemic_[a-z_0-9]+)\s*\(", src)))


def test_header_symbols_have_signatures():
    assert set(header_symbols()) == set(O.SIGNATURES)


def test_library_builds_and_exports_all_symbols():
    lib = O.load_library(B.build())
    for s in header_symbols():
        assert hasattr(lib, s), s
