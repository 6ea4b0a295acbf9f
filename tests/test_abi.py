"""The C-ABI library loads and exports every entry point include/*.h declares.

No compute calls here (no GPU in the CPU suite): only symbol lookup, the
version / default-parameter calls, and pd_create's error path without a
device.
"""
import ctypes
import glob
import os
import re

import pytest

from conftest import ROOT


def declared(header):
    src = open(header).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    return sorted(set(re.findall(r"\b(pd_[a-z0-9_]+)\s*\(", src)))


def test_c_abi_exports_every_declared_symbol(pdg):
    lib = ctypes.CDLL(pdg.native.LIB_PATH)
    names = declared(os.path.join(ROOT, "include", "pd_gb300.h"))
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the Python mirror binds the same set
    assert set(names) <= set(pdg.native.EXPORTED)


def test_every_header_is_covered(pdg):
    """Each include/*.h declares only symbols some built library exports."""
    libs = [ctypes.CDLL(p) for p in glob.glob(os.path.join(os.path.dirname(pdg.native.LIB_PATH), "lib*.so"))]
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        if h.endswith("pd_dropin.h"):
            continue  # C++ names, checked in test_dropin.py
        for n in declared(h):
            assert any(hasattr(l, n) for l in libs), (h, n)


def test_version_and_defaults_without_gpu(pdg):
    L = pdg.native.lib()
    assert L.pd_abi_version() == 1
    p = pdg.default_params()
    assert p.precision == 0 and p.det_guard == 1e-10 and p.rho == 2440.0


def test_create_fails_loudly_without_device(pdg):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(pdg.PdError) as e:
        pdg.native.Context(pdg.default_params())
    assert e.value.code == -2  # PD_ERR_CUDA: there is no silent CPU path


def test_params_validation_is_host_side(pdg):
    L = pdg.native.lib()
    p = pdg.default_params(rho=-1.0)
    h = ctypes.c_void_p()
    assert L.pd_create(ctypes.byref(p), ctypes.byref(h)) == -1
    assert b"invalid" in L.pd_last_error(None)
