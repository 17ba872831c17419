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


def test_header_constants_match_the_binding():
    """The family enum (order and count), the probe seed and the stat layout of the header agree
    with the Python side."""
    from esmgb import cabi
    from esmgb.model import FAMILIES, FAMILY_RATES
    src = open(os.path.join(ROOT, "include", "esmcuda.h")).read()
    enum = re.search(r"enum \{ (ESM_FAM_UNIT = 0,[^}]*)\}", src).group(1)
    names = [x.strip().split("=")[0].strip() for x in enum.split(",") if x.strip()]
    assert names[-1] == "ESM_NFAM"
    assert [n[len("ESM_FAM_"):].lower() for n in names[:-1]] == list(FAMILIES)
    assert cabi.NFAM == len(FAMILIES) == len(FAMILY_RATES)
    from oracle import oracle as O
    assert DV.NSTAT == O.NSTAT == 2 * (cabi.NFAM + 1) + 1
    xor = int(re.search(r"esm_probe_seed\(uint64_t seed\) \{ return seed \^ (0x[0-9A-Fa-f]+)ull; \}", src).group(1), 16)
    assert cabi.probe_seed(12345) == 12345 ^ xor


def _device_count():
    try:
        rt = ctypes.CDLL("libcudart.so")
    except OSError:
        for name in ("libcudart.so.13", "libcudart.so.12"):
            try:
                rt = ctypes.CDLL(name)
                break
            except OSError:
                rt = None
        if rt is None:
            return 0
    n = ctypes.c_int(0)
    return n.value if rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 else 0


def test_no_gpu_fails_loudly():
    """Without a usable GPU every entry point that needs one returns an error with the CUDA
    message (no CPU fallback): creating a chain and a batch raises EsmError."""
    if _device_count() > 0:
        pytest.skip("a GPU is present")
    from esmgb.model import make_model
    m = make_model(10, 15, 24, seed=1)
    with pytest.raises(DV.EsmError, match="esm_create: status -2: .*CUDA|cuda"):
        DV.DeviceChain(m, 4, precision=32, seed=1)
    L = DV.load()
    h = ctypes.c_void_p()
    assert L.esm_batch_create(None, 0, ctypes.byref(h)) != 0     # no contexts: refused, not a crash
