"""CPU-side checks of the C-ABI library (no GPU): it builds, loads, exports
every entry point include/nqes.h declares, and fails loudly without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

import __graft_entry__ as ge

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def pkg():
    ge._load_build_module().build_library()
    return ge.load_package()


def declared_symbols():
    with open(os.path.join(ROOT, "include", "nqes.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nqes_[a-zA-Z_]+)\s*\(", text)))


def test_header_declares_the_abi():
    syms = declared_symbols()
    for must in ["nqes_create", "nqes_destroy", "nqes_sr_step", "nqes_correlations", "nqes_set_weights",
                 "nqes_get_weights", "nqes_last_error"]:
        assert must in syms


def test_library_exports_every_declared_symbol(pkg):
    lib = ctypes.CDLL(pkg.LIB_PATH)
    for s in declared_symbols():
        assert hasattr(lib, s), s
    assert set(pkg.EXPORTS) == set(declared_symbols())


def test_no_gpu_fails_loudly(pkg):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(pkg.NqesError) as e:
        pkg.Context(4, 8, 2, np.zeros((4, 4)), 1.0)
    assert e.value.status == pkg.ERR_CUDA


def test_invalid_shape_rejected(pkg):
    lib = pkg.load_library()
    h = ctypes.c_void_p()
    J = np.zeros((4, 4))
    st = lib.nqes_create(4, 8, 5, J.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 1.0, 0, ctypes.byref(h))
    assert st == pkg.ERR_INVALID
    assert b"shape" in lib.nqes_last_error(None)
