"""The C-ABI library loads and exports every symbol that include/esmcuda.h declares (no GPU
needed: no compute call is made)."""
import ctypes
import os
import re

import pytest

from esmgb import build as B
from esmgb import device as DV
from esmgb import surrogate as SG

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "esmcuda.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|const char \*|void \*)\s*(esm_\w+)\s*\(", src, re.M)))


def test_header_and_binding_agree():
    assert sorted(DV.EXPORTS + SG.EXPORTS) == declared_symbols()


def test_library_exports_all_symbols():
    path = B.build()
    lib = ctypes.CDLL(path)
    for name in declared_symbols():
        assert hasattr(lib, name), name
