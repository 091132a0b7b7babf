"""Namelist surface beyond the CRK4 / APVM / upwind defaults, on the GPU
against the CPU FP64 oracle through the C ABI: the conservative APVM
(pv_scheme 2, operators_mod.F90:318-357), the CRK3 and PC2 integrators
(time_scheme_mod.F90:65-107, :156-184) and the prescribed-wind adv model
(tmcore_adv_mod.F90:62-97 with adv_scheme_sg11_mod.F90:33-48).

Per element the FP64 device arithmetic follows the reference's order; the
global sums (beta, the conservative-APVM epsilon) are reduced in a different
order, and the adv model's wind uses CUDA's sin/cos, so the bars here are
tolerances rather than bit identity.
"""
import numpy as np
import pytest

from conftest import rel_max

pytestmark = pytest.mark.gpu

_DEVICE_ONLY = ("precision", "renumber", "use_graph", "diag_every", "block_size", "stencils", "adv_wind")


def _models(mesh, **kw):
    from oracle.oracle import Oracle
    from tmcore_gb300.gpu import TMCoreGPU

    okw = {k: v for k, v in kw.items() if k not in _DEVICE_ONLY}
    return TMCoreGPU(mesh, **kw), Oracle(mesh, **okw)


def _ic(mesh, seed=0):
    from tmcore_gb300 import cases

    return cases.jet_bumps(mesh, seed=seed)


def test_conservative_apvm_spatial_operators(mesh4):
    g, o = _models(mesh4, dt=600.0, pv_scheme=2)
    gd, u, ghs = _ic(mesh4, seed=6)
    o.set_initial(gd, u, ghs)
    g.set_initial(gd, u, ghs)
    gd0, iap0, _ = o.state()
    tg_o, tu_o = o.spatial_operators(gd0, iap0)
    tg_g, tu_g = g.spatial_operators(gd0, iap0)
    # the gd tendency does not depend on pv; iap_u's only through epsilon's sums
    assert np.array_equal(tg_g, tg_o)
    assert rel_max(tu_g, tu_o) < 1e-12
    g.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_conservative_apvm_steps(mesh4, precision):
    g, o = _models(mesh4, dt=600.0, pv_scheme=2, precision=precision)
    gd, u, ghs = _ic(mesh4, seed=7)
    o.set_initial(gd, u, ghs)
    g.set_initial(gd, u, ghs)
    o.step(12)
    g.step(12)
    go, _, uo = o.state()
    gg, _, ug = g.get_state()
    tol_h, tol_u = (1e-12, 1e-11) if precision == 0 else (1e-5, 1e-3)
    assert rel_max(gg, go) < tol_h and rel_max(ug, uo) < tol_u
    do, dg = o.diag(), g.diag()
    assert abs(dg[0] - do[0]) / do[0] < 1e-12
    g.close()


@pytest.mark.parametrize("time_scheme", [1, 3])
@pytest.mark.parametrize("cfg", [
    dict(pv_scheme=1, apvm_weight=0.0),
    dict(pv_scheme=3, interp_pv_order=3, n_tracers=2, tracer_adv_order=3, tracer_adv_mono=1),
    dict(pv_scheme=2, conserve_energy=0),
])
def test_time_schemes_match_oracle(mesh4, time_scheme, cfg):
    from tmcore_gb300 import cases

    g, o = _models(mesh4, dt=600.0, time_scheme=time_scheme, **cfg)
    gd, u, ghs = _ic(mesh4, seed=8)
    o.set_initial(gd, u, ghs)
    g.set_initial(gd, u, ghs)
    ntr = cfg.get("n_tracers", 0)
    if ntr:
        qgd = cases.smooth_tracers(mesh4, ntr, seed=8) * gd[None, :]
        o.set_tracers(qgd)
        g.set_tracers(qgd)
    o.step(1)
    g.step(1)
    go, io, _ = o.state()
    gg, ig, _ = g.get_state()
    assert rel_max(gg, go) < 1e-14 and rel_max(ig, io) < 1e-13
    assert abs(g.diag()[4] - o.diag()[4]) < 1e-13
    o.step(9)
    g.step(9)
    go, _, uo = o.state()
    gg, _, ug = g.get_state()
    assert rel_max(gg, go) < 1e-12 and rel_max(ug, uo) < 1e-11
    if ntr:
        assert rel_max(g.get_tracers(), o.tracers()) < 1e-12
    g.close()


@pytest.mark.parametrize("time_scheme", [1, 3])
def test_time_schemes_fp32(mesh5, time_scheme):
    from tmcore_gb300.gpu import TMCoreGPU

    gd, u, ghs = _ic(mesh5, seed=0)
    a = TMCoreGPU(mesh5, dt=300.0, time_scheme=time_scheme, pv_scheme=1, apvm_weight=0.0, precision=0)
    b = TMCoreGPU(mesh5, dt=300.0, time_scheme=time_scheme, pv_scheme=1, apvm_weight=0.0, precision=1)
    for m in (a, b):
        m.set_initial(gd, u, ghs)
        m.step(48)
    ga, _, ua = a.get_state()
    gb, _, ub = b.get_state()
    assert rel_max(gb, ga) < 1e-5 and rel_max(ub, ua) < 1e-3
    da, db = a.diag(), b.diag()
    assert abs(db[0] - da[0]) / da[0] < 1e-12
    a.close()
    b.close()


@pytest.mark.parametrize("wind,order,time_scheme", [(1, 3, 2), (2, 5, 2), (2, 5, 3), (1, 4, 1)])
def test_adv_model_matches_oracle(mesh4, wind, order, time_scheme):
    from tmcore_gb300 import cases

    m = mesh4
    q0 = cases.cosine_bell(m) if wind == 1 else cases.deformation_flow(m, "gaussian_hills")
    dt = 3600.0
    kw = dict(dt=dt, adv_order=order, adv_mono=1, conserve_energy=0, time_scheme=time_scheme)
    g, o = _models(m, adv_wind=wind, **kw)
    o.adv_set_initial(q0, wind)
    g.adv_set_initial(q0)
    qg, ug = g.adv_state()
    qo, uo = o.adv_state()
    assert np.array_equal(qg, qo)
    assert rel_max(ug, uo) < 1e-14
    n = 24
    o.adv_step(n)
    g.step(n)
    qo, uo = o.adv_state()
    qg, ug = g.adv_state()
    assert rel_max(qg, qo) < 1e-12
    assert rel_max(ug, uo) < 1e-13
    assert g.adv_elapsed() == pytest.approx(n * dt, rel=0, abs=1e-9)
    d = g.diag()
    m0 = np.sum(q0 * m.areaCell) * 6371220.0 ** 2  # device areas are radius-scaled
    assert abs(d[0] - m0) / m0 < 1e-12
    g.close()


def test_adv_model_rejects_swm_entry_points(mesh3):
    from tmcore_gb300 import cases
    from tmcore_gb300.gpu import TMCError, TMCoreGPU

    g = TMCoreGPU(mesh3, dt=3600.0, adv_wind=1, adv_order=3, conserve_energy=0)
    gd, u, ghs = _ic(mesh3)
    with pytest.raises(TMCError):
        g.set_initial(gd, u, ghs)
    g.adv_set_initial(cases.cosine_bell(mesh3))
    g.step(2)
    assert np.all(np.isfinite(g.adv_state()[0]))
    g.close()


@pytest.mark.parametrize("cfg", [dict(pv_scheme=1, apvm_weight=0.0), dict(pv_scheme=3, adv_order=3, adv_mono=1)])
def test_flux_4th_order_correct(mesh4, cfg):
    """E-gradient correction with the reference's deriv3OnCell (tmcore_swm_mod.F90:183-195)."""
    g, o = _models(mesh4, dt=600.0, flux_4th_order_correct=1, **cfg)
    gd, u, ghs = _ic(mesh4, seed=9)
    o.set_initial(gd, u, ghs)
    g.set_initial(gd, u, ghs)
    gd0, iap0, _ = o.state()
    tg_o, tu_o = o.spatial_operators(gd0, iap0)
    tg_g, tu_g = g.spatial_operators(gd0, iap0)
    assert np.array_equal(tg_g, tg_o)
    assert np.array_equal(tu_g, tu_o)
    o.step(5)
    g.step(5)
    go, _, uo = o.state()
    gg, _, ug = g.get_state()
    assert rel_max(gg, go) < 1e-12 and rel_max(ug, uo) < 1e-11
    g.close()
