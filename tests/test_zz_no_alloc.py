"""tmc_mass_energy_noalloc: the entry point for callers that cannot allocate
device memory (a host sharing the GPU with a framework whose allocator owns
all device memory, or one whose policy forbids allocations while it runs).

It is called through the C ABI on device arrays and must agree with
tmc_get_diag's mass and energy on the same state, on two calls in a row
(the second call reuses the library's fixed scratch array).  This file is
collected last so that a failure here does not stop the rest of the suite.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_mass_energy_noalloc_matches_get_diag():
    torch = pytest.importorskip("torch")
    from conftest import icos
    from tmcore_gb300 import _lib, abi, cases
    from tmcore_gb300.gpu import REF_RADIUS, TMCoreGPU

    m = icos(5)
    gd, u, ghs = cases.jet_bumps(m, seed=9)
    model = TMCoreGPU(m, dt=600.0, pv_scheme=1, apvm_weight=0.0)
    model.set_initial(gd, u, ghs)
    model.step(3)
    ref = model.diag()
    gd1, iap1, _ = model.get_state(with_u=True)[:3]
    model.close()

    r2 = REF_RADIUS * REF_RADIUS
    area_c = m.areaCell * r2                 # mesh_mod.F90:219
    area_e = (m.dvEdge * m.dcEdge) * r2      # mesh_mod.F90:178, :221
    dev = torch.device("cuda:0")

    def on_gpu(a):
        return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)

    d_gd, d_ghs, d_ac = on_gpu(gd1), on_gpu(ghs), on_gpu(area_c)
    d_iap, d_ae = on_gpu(iap1), on_gpu(area_e)
    out = torch.zeros(2, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()

    lib = _lib.gpu()
    for call in range(2):
        out.fill_(-1.0)
        torch.cuda.synchronize()
        rc = lib.tmc_mass_energy_noalloc(d_gd.data_ptr(), d_ghs.data_ptr(), d_ac.data_ptr(), m.nCells,
                                         d_iap.data_ptr(), d_ae.data_ptr(), m.nEdges, out.data_ptr(), None)
        assert rc == abi.TMC_OK, (call, rc)
        torch.cuda.synchronize()
        mass, energy = out.cpu().numpy()
        assert abs(mass - ref[0]) <= 1e-13 * abs(ref[0]), (call, mass, ref[0])
        assert abs(energy - ref[1]) <= 1e-13 * abs(ref[1]), (call, energy, ref[1])

    # sizes beyond the fixed scratch array are refused before any launch
    too_many = abi.TMC_NOALLOC_MAX_ELEMENTS + 1
    rc = lib.tmc_mass_energy_noalloc(d_gd.data_ptr(), d_ghs.data_ptr(), d_ac.data_ptr(), too_many,
                                     d_iap.data_ptr(), d_ae.data_ptr(), m.nEdges, out.data_ptr(), None)
    assert rc == abi.TMC_E_ARG
    assert lib.tmc_mass_energy_noalloc(None, None, None, 1, None, None, 1, None, None) == abi.TMC_E_ARG
