"""The C ABI library builds, loads and exports every symbol include/*.h declares (no GPU calls)."""
import ctypes
import glob
import os

from conftest import ROOT


def test_library_exports_header_symbols():
    from tmcore_gb300 import _lib, abi

    lib = _lib.gpu()
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        names += abi.header_symbols(open(h).read())
    assert "tmc_create" in names and "tmc_step" in names
    for n in names:
        assert hasattr(lib, n), n
    # every header symbol has ctypes types declared
    assert set(names) <= set(abi.SYMBOLS), set(names) - set(abi.SYMBOLS)


def test_struct_layout_matches_header():
    from tmcore_gb300 import abi

    # 6 int32 dims + 29 pointers; params: fixed layout checked by size
    assert ctypes.sizeof(abi.MeshDesc) == 6 * 4 + 29 * ctypes.sizeof(ctypes.c_void_p)
    # dt, 4 int32, apvm_weight, 3 int32 + 4 bytes padding, radius/g/omega, 16 int32
    assert ctypes.sizeof(abi.Params) == 8 + 16 + 8 + 12 + 4 + 24 + 64


def test_create_fails_cleanly_without_gpu_or_with_bad_args():
    """Bad arguments return an error code and a message; nothing aborts."""
    from tmcore_gb300 import _lib, abi

    lib = _lib.gpu()
    h = ctypes.c_void_p()
    assert lib.tmc_create(None, None, ctypes.byref(h)) == abi.TMC_E_ARG
    assert lib.tmc_step(None, 1) == abi.TMC_E_ARG
    p = abi.Params()
    lib.tmc_default_params(ctypes.byref(p))
    assert p.time_scheme == 2 and p.pv_scheme == 3 and p.radius == 6371220.0
