"""The C-ABI library builds, loads and exports every entry point that
include/imsrg_gpu.h declares (no device calls: this runs without a GPU)."""
import ctypes
import os
import re

from conftest import ROOT


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "imsrg_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(imsrg_gpu_\w+)\s*\(", src)))


def test_library_exports_all_declared_symbols():
    import build as pkg_build
    lib_path = pkg_build.build()
    lib = ctypes.CDLL(lib_path)
    syms = declared_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_python_mirror_binds_every_symbol():
    from imsrg_gpu import api
    assert set(api.SYMBOLS) == set(declared_symbols())


def test_strerror_needs_no_device():
    import build as pkg_build
    lib = ctypes.CDLL(pkg_build.build())
    lib.imsrg_gpu_strerror.restype = ctypes.c_char_p
    assert lib.imsrg_gpu_strerror(0) == b"ok"
    assert b"clipping" in lib.imsrg_gpu_strerror(4)
    assert lib.imsrg_gpu_strerror(999) == b"unknown status"
