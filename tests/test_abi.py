"""The C-ABI library builds, loads and exports every function include/tlq.h
declares (no GPU calls)."""
import ctypes
import os
import re

from tests.conftest import ROOT


def header_functions():
    src = open(os.path.join(ROOT, "include", "tlq.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(tlq_[a-z0-9_]+)\s*\(", src)))


def test_library_builds_and_exports_header(gpu_lib):
    names = header_functions()
    assert len(names) >= 29
    missing = [n for n in names if not hasattr(gpu_lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    from tlaloque_gb300.tlq import EXPORTS
    assert sorted(EXPORTS) == header_functions()


def test_status_strings_without_gpu(gpu_lib):
    gpu_lib.tlq_status_string.restype = ctypes.c_char_p
    assert gpu_lib.tlq_status_string(0) == b"ok"
    assert b"time step" in gpu_lib.tlq_status_string(3)


def test_invalid_config_is_rejected_before_any_device_work(gpu_lib):
    """tlq_create validates the configuration first: bad input is an error
    code, not a crash (no GPU is touched for these)."""
    from tlaloque_gb300.tlq import CConfig, ERR_CONFIG
    c = CConfig()
    gpu_lib.tlq_config_default(ctypes.byref(c))
    h = ctypes.c_void_p()
    c.nx = 1
    assert gpu_lib.tlq_create(ctypes.byref(c), ctypes.byref(h)) == ERR_CONFIG
    gpu_lib.tlq_config_default(ctypes.byref(c))
    c.limiter = 9
    assert gpu_lib.tlq_create(ctypes.byref(c), ctypes.byref(h)) == ERR_CONFIG
    gpu_lib.tlq_config_default(ctypes.byref(c))
    c.bc[2] = 7
    assert gpu_lib.tlq_create(ctypes.byref(c), ctypes.byref(h)) == ERR_CONFIG
    assert not h.value
