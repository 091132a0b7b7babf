"""ctypes loaders for the in-tree native libraries.

The CUDA path has no fallback: if ``libtmcore_gpu.so`` is missing or cannot
be loaded, :func:`gpu` raises.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(_HERE, "_lib")

_meshgen = None
_gpu = None

c_i32p = ctypes.POINTER(ctypes.c_int32)
c_f64p = ctypes.POINTER(ctypes.c_double)
c_f32p = ctypes.POINTER(ctypes.c_float)


def _load(name: str, autobuild: bool) -> ctypes.CDLL:
    path = os.path.join(LIBDIR, name)
    if not os.path.exists(path):
        if not autobuild:
            raise RuntimeError(f"{path} is missing: run tmcore_gb300._build.build() first")
        from . import _build
        _build.build()
    return ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)


def meshgen(autobuild: bool = True) -> ctypes.CDLL:
    global _meshgen
    if _meshgen is None:
        lib = _load("libtmc_meshgen.so", autobuild)
        lib.tmc_meshgen_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
        lib.tmc_meshgen_create.restype = ctypes.c_int
        lib.tmc_meshgen_destroy.argtypes = [ctypes.c_void_p]
        lib.tmc_meshgen_destroy.restype = None
        lib.tmc_meshgen_dims.argtypes = [ctypes.c_void_p, c_i32p]
        lib.tmc_meshgen_dims.restype = ctypes.c_int
        lib.tmc_meshgen_error.argtypes = [ctypes.c_void_p]
        lib.tmc_meshgen_error.restype = ctypes.c_char_p
        lib.tmc_meshgen_get_i32.argtypes = [ctypes.c_void_p, ctypes.c_char_p, c_i32p]
        lib.tmc_meshgen_get_i32.restype = ctypes.c_int64
        lib.tmc_meshgen_get_f64.argtypes = [ctypes.c_void_p, ctypes.c_char_p, c_f64p]
        lib.tmc_meshgen_get_f64.restype = ctypes.c_int64
        _meshgen = lib
    return _meshgen


def gpu(autobuild: bool = True) -> ctypes.CDLL:
    """The CUDA library with argtypes declared (see include/tmcore_gpu.h)."""
    global _gpu
    if _gpu is None:
        from . import abi
        _gpu = abi.declare(_load("libtmcore_gpu.so", autobuild))
    return _gpu
