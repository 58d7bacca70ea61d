"""CPU checks of the C ABI: the library loads and exports every symbol the header declares."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "graphyt_gpu.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gy_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "gy_step" in syms and "gy_create" in syms and "gy_initialize" in syms
    assert len(syms) >= 25


def test_library_exports_every_declared_symbol(gpu_lib):
    for name in declared_symbols():
        assert hasattr(gpu_lib, name), name


def test_python_binding_covers_header(gpu_lib):
    from graphyt_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_abi_version(gpu_lib):
    assert gpu_lib.gy_abi_version() == 4


def test_create_rejects_inconsistent_grid(gpu_lib):
    """Nx*Ny*Nz != numNodes (Nodes.cpp:12 vs :71-73) is refused before any CUDA work."""
    from graphyt_gb300 import _lib
    g = _lib.GridDesc()
    g.L[0], g.L[1], g.L[2] = 1.2, 1.2, 1.2
    g.cellsize = 0.1
    g.psep = 0.05
    h = ctypes.c_void_p()
    assert gpu_lib.gy_create(ctypes.byref(g), -1, ctypes.byref(h)) == _lib.GY_ERR_ARG
    g.L[0] = g.L[1] = g.L[2] = 1.0
    g.psep = 0.2  # psep > cellsize
    assert gpu_lib.gy_create(ctypes.byref(g), -1, ctypes.byref(h)) == _lib.GY_ERR_UNSUPPORTED


def test_null_handles_are_errors(gpu_lib):
    from graphyt_gb300 import _lib
    assert gpu_lib.gy_step(None, 0.0, 0) == _lib.GY_ERR_ARG
    assert gpu_lib.gy_destroy(None) == _lib.GY_ERR_ARG
    assert gpu_lib.gy_last_error(None) == b"null handle"


def test_resort_rejects_bad_input_before_cuda(gpu_lib):
    """gy_resort_keys checks its host arrays before any CUDA work: previous keys that are not
    non-decreasing, negative keys and negative counts are argument errors; nothing to sort
    is success."""
    import numpy as np
    from graphyt_gb300 import _lib

    def call(keys, prev, n=None):
        keys = np.ascontiguousarray(keys, np.int32)
        prev = np.ascontiguousarray(prev, np.int32)
        out = np.zeros(max(len(keys), 1), np.int32)
        srt = np.zeros(max(len(keys), 1), np.int32)
        ip = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        return gpu_lib.gy_resort_keys(ip(keys), ip(prev), len(keys) if n is None else n, ip(out), ip(srt), -1)

    assert call([0, 1, 2, 3], [0, 2, 1, 3]) == _lib.GY_ERR_ARG     # previous order not sorted
    assert call([0, -1, 2, 3], [0, 1, 2, 3]) == _lib.GY_ERR_ARG    # negative key
    assert call([0, 1], [0, 1], n=-1) == _lib.GY_ERR_ARG
    assert call([], [], n=0) == _lib.GY_OK
