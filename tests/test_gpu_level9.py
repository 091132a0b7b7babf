"""The level-9 configuration (2,621,442 cells, 7,864,320 edges, 5,242,880
vertices; seeded jet + mountains, 4 coupled tracers, CRK4 with dt = 45 s,
centred pv) on the GPU against the CPU FP64 oracle, through the C ABI.

This is the mesh the throughput figures are quoted on.  Index and layout
errors that only appear past 2^21 or 2^22 elements (renumbering tables,
slot-major connectivity, the partial-sum grids of the reductions) would
show here and not on the level-3 to level-5 meshes of the other tests.

* one spatial_operators call (tmcore_swm_mod.F90:92-125) is bit-identical;
* three CRK4 steps (time_scheme_mod.F90:109-154) agree to 1e-13 relative
  max-norm in h, u and each tracer (only beta's global sums are reduced in
  another order);
* the FP32-state path stays within 1e-5 relative h error of the FP64 oracle.
"""
import numpy as np
import pytest

from conftest import icos, rel_max

pytestmark = pytest.mark.gpu

LEVEL, DT, NTR = 9, 45.0, 4


@pytest.fixture(scope="module")
def level9():
    from tmcore_gb300 import cases

    m = icos(LEVEL)
    gd, u, ghs = cases.jet_bumps(m, seed=0)
    q = cases.smooth_tracers(m, NTR, seed=0)
    return m, gd, u, ghs, q * gd[None, :]


@pytest.fixture(scope="module")
def oracle9(level9):
    from oracle.oracle import Oracle

    m, gd, u, ghs, qgd = level9
    o = Oracle(m, dt=DT, pv_scheme=1, apvm_weight=0.0, adv_order=2, n_tracers=NTR)
    o.set_initial(gd, u, ghs)
    o.set_tracers(qgd)
    yield o
    o.close()


def _gpu(level9, precision):
    from tmcore_gb300.gpu import TMCoreGPU

    m, gd, u, ghs, qgd = level9
    g = TMCoreGPU(m, dt=DT, pv_scheme=1, apvm_weight=0.0, adv_order=2, n_tracers=NTR, precision=precision)
    g.set_initial(gd, u, ghs)
    g.set_tracers(qgd)
    return g


def test_level9_spatial_operators_bit_exact(level9, oracle9):
    g = _gpu(level9, 0)
    gd0, iap0, _ = oracle9.state()
    tg_o, tu_o = oracle9.spatial_operators(gd0, iap0)
    tg_g, tu_g = g.spatial_operators(gd0, iap0)
    g.close()
    assert np.array_equal(tg_g, tg_o), rel_max(tg_g, tg_o)
    assert np.array_equal(tu_g, tu_o), rel_max(tu_g, tu_o)


def test_level9_steps_match_oracle(level9, oracle9):
    g = _gpu(level9, 0)
    gg0, ig0, _ = g.get_state()
    go0, io0, _ = oracle9.state()
    assert np.array_equal(gg0, go0) and np.array_equal(ig0, io0)
    d0 = g.diag()
    oracle9.step(3)
    g.step(3)
    go, io, uo = oracle9.state()
    gg, ig, ug = g.get_state()
    qo, qg = oracle9.tracers(), g.get_tracers()
    d1 = g.diag()
    g.close()
    assert rel_max(gg, go) < 1e-13, rel_max(gg, go)
    assert rel_max(ig, io) < 1e-13, rel_max(ig, io)
    assert rel_max(ug, uo) < 1e-13, rel_max(ug, uo)
    for k in range(NTR):
        assert rel_max(qg[k], qo[k]) < 1e-13, (k, rel_max(qg[k], qo[k]))
    assert abs(d1[0] - d0[0]) / d0[0] < 1e-14                  # mass to round-off
    assert abs(d1[4] - oracle9.diag()[4]) < 1e-13              # beta


def test_level9_fp32_path_against_oracle(level9):
    """Three steps of the FP32-state path (FP64 metrics, gd accumulation and
    sums) against a fresh oracle run of the same three steps."""
    from oracle.oracle import Oracle

    m, gd, u, ghs, qgd = level9
    o = Oracle(m, dt=DT, pv_scheme=1, apvm_weight=0.0, adv_order=2, n_tracers=NTR)
    o.set_initial(gd, u, ghs)
    o.set_tracers(qgd)
    o.step(3)
    go, _, uo = o.state()
    qo = o.tracers()
    o.close()
    g = _gpu(level9, 1)
    d0 = g.diag()
    g.step(3)
    gg, _, ug = g.get_state()
    qg = g.get_tracers()
    d1 = g.diag()
    g.close()
    assert rel_max(gg, go) < 1e-5, rel_max(gg, go)
    assert rel_max(ug, uo) < 1e-4, rel_max(ug, uo)
    for k in range(NTR):
        assert rel_max(qg[k] / gg, qo[k] / go) < 1e-4, k
    assert abs(d1[0] - d0[0]) / d0[0] < 1e-13                  # FP64 gd accumulation keeps mass
