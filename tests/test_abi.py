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


def test_member_layout_arguments_checked_before_device_set_up():
    """member_layout 1 refuses member counts that are not a multiple of 16
    (TMC_E_ARG) and options its kernels do not implement (TMC_E_UNSUP) before
    any CUDA call, so these checks hold without a GPU."""
    from conftest import icos
    from tmcore_gb300 import _lib, abi
    from tmcore_gb300.gpu import default_params, mesh_desc

    lib = _lib.gpu()
    d, keep = mesh_desc(icos(2))
    cases = [
        (dict(members=40, member_layout=1, precision=1, pv_scheme=1, apvm_weight=0.0, adv_order=2), abi.TMC_E_ARG),
        (dict(members=32, member_layout=2, precision=1, pv_scheme=1, apvm_weight=0.0, adv_order=2), abi.TMC_E_ARG),
        (dict(members=32, member_layout=1, precision=1, pv_scheme=3, interp_pv_order=5), abi.TMC_E_UNSUP),
        (dict(members=32, member_layout=1, precision=1, pv_scheme=2), abi.TMC_E_UNSUP),
        (dict(members=32, member_layout=1, precision=1, pv_scheme=1, apvm_weight=0.0, adv_order=2, n_tracers=1),
         abi.TMC_E_UNSUP),
        (dict(members=32, member_layout=1, precision=0, pv_scheme=1, apvm_weight=0.0, adv_order=2), abi.TMC_E_UNSUP),
    ]
    for kw, code in cases:
        p = default_params(dt=600.0, **kw)
        h = ctypes.c_void_p()
        assert lib.tmc_create(ctypes.byref(d), ctypes.byref(p), ctypes.byref(h)) == code, kw
        assert h.value and lib.tmc_last_error(h)
        lib.tmc_destroy(h)
    # accepted combinations pass these checks (here they then fail at the device)
    for kw in (dict(pv_scheme=1, apvm_weight=0.0), dict(pv_scheme=3, interp_pv_order=3, apvm_weight=0.5),
               dict(pv_scheme=3, interp_pv_order=4)):
        p = default_params(dt=600.0, members=32, member_layout=1, precision=1, adv_order=2, **kw)
        h = ctypes.c_void_p()
        rc = lib.tmc_create(ctypes.byref(d), ctypes.byref(p), ctypes.byref(h))
        assert rc not in (abi.TMC_E_ARG, abi.TMC_E_UNSUP), (kw, rc)
        lib.tmc_destroy(h)
