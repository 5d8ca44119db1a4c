"""CPU checks of the C++ host library: it loads and exports its C API, and a
missing CUDA device is reported as an error rather than a CPU fallback."""
import ctypes
import os

from conftest import CONF, ROOT

LIB = os.path.join(ROOT, "rockable_gb300", "_lib", "librk_host.so")


def test_host_exports(gpu_lib):
    lib = ctypes.CDLL(LIB)
    for name in ["rkh_open", "rkh_error", "rkh_close", "rkh_read_driving", "rkh_console_run", "rkh_run",
                 "rkh_save_conf"]:
        assert hasattr(lib, name), name


def test_no_cpu_fallback_without_gpu(gpu_lib, golden_dir):
    import torch
    if torch.cuda.is_available():
        import pytest
        pytest.skip("a GPU is present")
    lib = ctypes.CDLL(LIB)
    lib.rkh_open.restype = ctypes.c_void_p
    lib.rkh_error.restype = ctypes.c_char_p
    h = lib.rkh_open(str(golden_dir / "512_particles" / CONF["512_particles"]).encode())
    assert not h
    assert b"CUDA device" in lib.rkh_error()
