"""History diagnostics on the device (history_mod.F90:124-174 with
mpas_reconstruct_1d) against the FP64 oracle."""
import numpy as np
import pytest

from conftest import rel_max

pytestmark = pytest.mark.gpu


def test_reconstruct_bit_exact(mesh4):
    from oracle.oracle import Oracle
    from tmcore_gb300.gpu import TMCoreGPU

    g = TMCoreGPU(mesh4, dt=600.0, pv_scheme=1, apvm_weight=0.0)
    o = Oracle(mesh4, dt=600.0)
    u = np.random.default_rng(3).standard_normal(mesh4.nEdges) * 20.0
    a, b = g.reconstruct(u), o.reconstruct(u)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    g.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_history_fields(mesh4, precision):
    from oracle.oracle import Oracle
    from tmcore_gb300 import cases
    from tmcore_gb300.gpu import TMCoreGPU

    g = TMCoreGPU(mesh4, dt=600.0, pv_scheme=1, apvm_weight=0.0, precision=precision)
    o = Oracle(mesh4, dt=600.0, pv_scheme=1, apvm_weight=0.0)
    gd, u, ghs = cases.jet_bumps(mesh4, seed=31)
    g.set_initial(gd, u, ghs)
    o.set_initial(gd, u, ghs)
    g.step(3)
    o.step(3)
    f = g.history_fields()
    go, _, uo = o.state()
    pvo, voro = o.vertex()
    zo, mo = o.reconstruct(uo)[3:]
    tol = 1e-12 if precision == 0 else 1e-4
    assert rel_max(f["u"], uo) < tol
    assert rel_max(f["h"], (go + ghs) / 9.80616) < (1e-14 if precision == 0 else 1e-6)
    assert rel_max(f["zonal"], zo) < tol and rel_max(f["meridional"], mo) < max(tol, 1e-12) * 10
    assert rel_max(f["div"], o.op("div", uo, out_size=mesh4.nCells)) < (1e-10 if precision == 0 else 1e-2)
    assert rel_max(f["pv"], pvo) < (1e-12 if precision == 0 else 1e-4)
    assert rel_max(f["vor"], voro) < (1e-10 if precision == 0 else 1e-2)
    g.close()


def test_history_file(mesh4, tmp_path):
    """Two records of the history file (history_mod.F90 fields), read back with scipy."""
    import os

    from scipy.io import netcdf_file

    from tmcore_gb300 import cases
    from tmcore_gb300.gpu import HistoryWriter, TMCoreGPU

    g = TMCoreGPU(mesh4, dt=600.0, pv_scheme=1, apvm_weight=0.0)
    gd, u, ghs = cases.jet_bumps(mesh4, seed=33)
    g.set_initial(gd, u, ghs)
    p = os.path.join(tmp_path, "h0.nc")
    hw = HistoryWriter(p, mesh4)
    hw.write(g, 0.0)
    f0 = g.history_fields()
    g.step(6)
    hw.write(g, 3600.0)
    f1 = g.history_fields()
    d1 = g.diag()
    hw.close()
    with netcdf_file(p, "r", mmap=False) as nc:
        assert nc.variables["time"][:].tolist() == [0.0, 3600.0]
        assert np.array_equal(nc.variables["u"][0], f0["u"]) and np.array_equal(nc.variables["u"][1], f1["u"])
        assert np.array_equal(nc.variables["h"][1], f1["h"]) and np.array_equal(nc.variables["vor"][1], f1["vor"])
        assert np.array_equal(nc.variables["zonalWind"][1], f1["zonal"])
        assert nc.variables["tm"][1] == d1[0] and nc.variables["te"][1] == d1[1]
        assert np.array_equal(nc.variables["xCell"][:], mesh4.xCell)
    g.close()
