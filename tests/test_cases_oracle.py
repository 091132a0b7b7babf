"""The reference's shallow-water test cases that carry a physics answer, set up
by tmcore_gb300.cases and run by the CPU FP64 oracle:

* the Rossby-Haurwitz wave of wavenumber 4
  (rossby_haurwitz_wave_test_mod.F90:21-63) keeps its shape and moves at the
  Haurwitz angular speed;
* the linear Rossby wave (linearized_rossby_wave_test_mod.F90:81-287)
  converges to its analytic solution at later times;
* the Galewsky jet (jet_zonal_flow_test_mod.F90:27-84) without its bump is
  balanced up to a truncation error that converges with resolution, and its
  balance integral agrees with QUADPACK."""
import numpy as np
import pytest

from conftest import icos

ORACLE = pytest.importorskip("oracle.oracle")


def _run(mesh, case, dt, seconds):
    o = ORACLE.Oracle(mesh, dt=dt, pv_scheme=1, apvm_weight=0.0)
    o.set_initial(*case)
    d0 = o.diag()
    o.step(int(round(seconds / dt)))
    return o.state(), d0, o.diag()


def _corr(w, x, y):
    return np.sum(w * x * y) / np.sqrt(np.sum(w * x * x) * np.sum(w * y * y))


def test_rossby_haurwitz_wave_moves_at_its_angular_speed():
    from tmcore_gb300 import cases
    from tmcore_gb300.gpu import REF_G, REF_OMEGA, REF_RADIUS

    m = icos(4)
    (g1, _, _), d0, d1 = _run(m, cases.rossby_haurwitz_wave(m), 600.0, 86400.0)
    assert abs(d1[0] - d0[0]) < 1e-13 * d0[0]
    # the wave part of the depth: what is left after the zonally symmetric term
    a, R, w, K, om = REF_RADIUS, cases.RH_R, cases.RH_W, cases.RH_K, REF_OMEGA
    c = np.cos(m.latCell)
    aa = 0.5 * w * (2 * om + w) * c ** 2 + 0.25 * K ** 2 * c ** (2 * R) * (
        (R + 1) * c ** 2 + 2 * R ** 2 - R - 2 - 2 * R ** 2 * c ** -2.0)
    bb = (2 * (om + w) * K / ((R + 1) * (R + 2))) * c ** R * ((R ** 2 + 2 * R + 2) - ((R + 1) * c) ** 2)
    cc = 0.25 * K ** 2 * c ** (2 * R) * ((R + 1) * c ** 2 - R - 2)
    sim = g1 - REF_G * cases.RH_H0 - a * a * aa

    def wave(shift):
        lon = m.lonCell - shift
        return a * a * (bb * np.cos(R * lon) + cc * np.cos(2 * R * lon))

    moved = _corr(m.areaCell, sim, wave(cases.rossby_haurwitz_angular_speed() * 86400.0))
    still = _corr(m.areaCell, sim, wave(0.0))
    assert moved > 0.99 and moved > still + 0.2, (moved, still)  # measured 0.996 and 0.71
    # the reference's w and K are single-precision literals
    assert cases.RH_W == float(np.float32(7.848e-6)) and cases.RH_W != 7.848e-6


def test_linearized_rossby_wave_converges_to_its_analytic_solution():
    from tmcore_gb300 import cases
    from tmcore_gb300.gpu import REF_G

    T = 2 * 86400.0
    errs = []
    for level, dt in ((4, 600.0), (5, 300.0)):
        m = icos(level)
        ic = cases.linearized_rossby_wave(m)
        (g1, _, _), _, _ = _run(m, ic, dt, T)
        exact = cases.linearized_rossby_wave(m, t=T)[0] - REF_G * cases.LRW_H0
        sim = g1 - REF_G * cases.LRW_H0
        start = ic[0] - REF_G * cases.LRW_H0
        norm = np.sqrt(np.sum(m.areaCell * exact ** 2))
        errs.append(np.sqrt(np.sum(m.areaCell * (sim - exact) ** 2)) / norm)
        # the wave has moved: the initial pattern is far from the state at T
        assert np.sqrt(np.sum(m.areaCell * (sim - start) ** 2)) / norm > 0.5
    assert errs[1] < 0.5 * errs[0] and errs[1] < 0.1, errs  # measured 0.20 and 0.069
    assert cases.lrw_phase_speed() < 0.0  # westward


def test_galewsky_jet_balance_converges():
    from tmcore_gb300 import cases
    from tmcore_gb300.gpu import REF_G

    du = []
    for level, dt in ((3, 600.0), (4, 300.0), (5, 150.0)):
        m = icos(level)
        gd, u, ghs = cases.jet_zonal_flow(m)
        lon = np.where(m.lonCell > np.pi, m.lonCell - 2 * np.pi, m.lonCell)
        bump = REF_G * 120.0 * np.cos(m.latCell) * np.exp(-(lon * 3.0) ** 2) * np.exp(
            -((np.pi / 4 - m.latCell) * 15.0) ** 2)
        if level == 5:
            # 120 m cos(lat) near 45 degrees north: about 84.9 m at its peak
            assert 84.0 < np.max(bump) / REF_G < 86.0
        (_, _, u1), _, _ = _run(m, (gd - bump, u, ghs), dt, 6 * 3600.0)
        du.append(np.max(np.abs(u1 - u)) / np.max(np.abs(u)))
    assert du[2] < du[1] < du[0] and du[2] < 0.03, du  # measured 0.135, 0.056, 0.014
    assert np.max(np.abs(u)) > 79.0  # the 80 m/s jet on the edges


def test_galewsky_balance_integral_matches_quadpack():
    integrate = pytest.importorskip("scipy.integrate")
    from tmcore_gb300 import cases
    from tmcore_gb300.gpu import REF_OMEGA, REF_RADIUS

    a = REF_RADIUS

    def f(p):
        u = cases._jet_u(np.array([p]))[0]
        return a * u * (2 * REF_OMEGA * np.sin(p) + np.tan(p) / a * u)

    lats = np.linspace(-1.5, 1.5, 13)
    ours = cases._jet_balance_integral(lats, a, REF_OMEGA)
    scale = np.max(np.abs(ours))
    for lat, v in zip(lats, ours):
        tight = integrate.quad(f, -0.5 * np.pi, lat, epsabs=1e-12, epsrel=1e-13, limit=200)[0]
        # QUADPACK qags with the reference's tolerances (epsabs 1e-10, epsrel 1e-3)
        loose = integrate.quad(f, -0.5 * np.pi, lat, epsabs=1e-10, epsrel=1e-3, limit=50)[0]
        assert abs(v - tight) < 1e-12 * scale and abs(v - loose) < 1e-6 * scale, (lat, v, tight, loose)


def test_cases_by_name():
    from tmcore_gb300 import cases

    m = icos(3)
    for name in cases.SWM_CASES:
        gd, u, ghs = cases.by_name(name, m, seed=1)
        assert gd.shape == (m.nCells,) and u.shape == (m.nEdges,) and ghs.shape == (m.nCells,), name
        assert np.all(np.isfinite(gd)) and np.all(np.isfinite(u)) and np.all(gd > 0), name
    with pytest.raises(ValueError):
        cases.by_name("no_such_case", m)
