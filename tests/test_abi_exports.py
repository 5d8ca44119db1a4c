"""The C-ABI library loads and exports every function include/rk_gpu.h
declares (CPU only: no compute call is made)."""
import ctypes
import os
import re

from conftest import ROOT


def declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rk_[a-z0-9_]+)\s*\(", text)))


def test_header_symbols_exported(gpu_lib):
    names = declared("rk_gpu.h")
    assert len(names) >= 20
    lib = ctypes.CDLL(gpu_lib.LIBPATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) <= set(gpu_lib.SIGNATURES), set(names) - set(gpu_lib.SIGNATURES)


def test_abi_version(gpu_lib):
    lib = gpu_lib.load()
    assert lib.rk_abi_version() == 1
