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


def test_every_entry_point_refuses_null_arguments():
    """Every exported function, called with null pointers and zero scalars,
    returns an error code (the destroy and close functions return TMC_OK for
    a null handle, and the error-message functions a message) and does not
    crash: it runs in a child process, which must exit normally."""
    import json
    import subprocess
    import sys

    code = (
        "import ctypes, json\n"
        "from tmcore_gb300 import _lib, abi\n"
        "lib = _lib.gpu()\n"
        "ints = (ctypes.c_int32, ctypes.c_int, ctypes.c_int64, ctypes.c_uint64)\n"
        "out = {}\n"
        "for name, (res, args) in abi.SYMBOLS.items():\n"
        "    vals = [0 if a in ints else 0.0 if a in (ctypes.c_double, ctypes.c_float) else None for a in args]\n"
        "    r = getattr(lib, name)(*vals)\n"
        "    out[name] = r.decode() if isinstance(r, bytes) else r\n"
        "print(json.dumps(out))\n"
    )
    p = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    out = json.loads(p.stdout.strip().splitlines()[-1])
    from tmcore_gb300 import abi

    assert set(out) == set(abi.SYMBOLS)
    for name, r in out.items():
        if name.endswith(("_destroy", "_close")):
            assert r == abi.TMC_OK, name
        elif name.endswith(("last_error", "_error")):
            assert isinstance(r, str) and r, name
        else:
            assert isinstance(r, int) and r < 0, (name, r)
