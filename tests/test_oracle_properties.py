"""Property tests of the CPU FP64 oracle on random fields (hypothesis).

The reference's design guarantees these for any input, not only for the
seeded fields of test_oracle.py; hypothesis draws the fields:

* the operators are linear (div_operator, curl_operator, the c2e / c2v
  interpolations: operators_mod.F90:40-55, 76-123);
* the curl of a discrete gradient vanishes and the area-weighted divergence
  of any edge flux sums to zero over the sphere;
* q.F_perp does no work for any flux and any edge pv
  (calc_tangent_vor_flux, operators_mod.F90:239-260);
* interpolation keeps constants;
* CRK4 with beta (time_scheme_mod.F90:109-154) conserves mass and energy to
  round-off from any positive-depth state.
"""
import numpy as np
import pytest

from conftest import icos

hyp = pytest.importorskip("hypothesis")
st = pytest.importorskip("hypothesis.strategies")
ORACLE = pytest.importorskip("oracle.oracle")

from hypothesis import given, settings  # noqa: E402

RADIUS = 6371220.0
SETTINGS = dict(max_examples=25, deadline=None, derandomize=True)


@pytest.fixture(scope="module")
def mesh():
    return icos(2)


@pytest.fixture(scope="module")
def oracle(mesh):
    o = ORACLE.Oracle(mesh)
    yield o
    o.close()


def fields(seed, n, scale):
    return scale * np.random.default_rng(seed).standard_normal(n)


seeds = st.integers(min_value=0, max_value=2**31 - 1)
scales = st.floats(min_value=1e-3, max_value=1e3)
coefs = st.floats(min_value=-10.0, max_value=10.0)


@settings(**SETTINGS)
@given(seed=seeds, a=coefs, b=coefs, scale=scales)
def test_operators_are_linear(mesh, oracle, seed, a, b, scale):
    nc, ne, nv = mesh.nCells, mesh.nEdges, mesh.nVertices
    cases = [("div", ne, nc), ("curl", ne, nv), ("c2e", nc, ne), ("c2v", nc, nv)]
    for k, (name, nin, nout) in enumerate(cases):
        x = fields(seed + 2 * k, nin, scale)
        y = fields(seed + 2 * k + 1, nin, scale)
        lhs = oracle.op(name, a * x + b * y, out_size=nout)
        rhs = a * oracle.op(name, x, out_size=nout) + b * oracle.op(name, y, out_size=nout)
        ref = np.max(np.abs(a * oracle.op(name, x, out_size=nout))) + np.max(
            np.abs(b * oracle.op(name, y, out_size=nout))) + 1e-300
        assert np.max(np.abs(lhs - rhs)) <= 1e-13 * ref, name


@settings(**SETTINGS)
@given(seed=seeds, scale=scales, offset=coefs)
def test_curl_of_gradient_vanishes(mesh, oracle, seed, scale, offset):
    f = fields(seed, mesh.nCells, scale) + offset * scale
    dc = mesh.dcEdge * RADIUS
    c1, c2 = mesh.cellsOnEdge[:, 0] - 1, mesh.cellsOnEdge[:, 1] - 1
    grad = (f[c2] - f[c1]) / dc
    curl = oracle.op("curl", grad, out_size=mesh.nVertices)
    assert np.max(np.abs(curl)) <= 1e-12 * np.max(np.abs(grad)) / np.min(dc)


@settings(**SETTINGS)
@given(seed=seeds, scale=scales)
def test_divergence_sums_to_zero(mesh, oracle, seed, scale):
    fe = fields(seed, mesh.nEdges, scale)
    div = oracle.op("div", fe, out_size=mesh.nCells)
    area = mesh.areaCell * RADIUS ** 2
    assert abs(np.sum(div * area)) <= 1e-12 * np.sum(np.abs(div * area))


@settings(**SETTINGS)
@given(seed=seeds, scale=scales, depth=st.floats(min_value=0.5, max_value=5e4))
def test_tangent_vor_flux_does_no_work(mesh, oracle, seed, scale, depth):
    rng = np.random.default_rng(seed)
    u = scale * rng.standard_normal(mesh.nEdges)
    ge = depth * rng.uniform(0.5, 2.0, mesh.nEdges)
    pe = rng.standard_normal(mesh.nEdges)
    flx = oracle.op("tangent_vor_flux", u, ge, pe, out_size=mesh.nEdges)
    terms = oracle.area_edge() * u * ge * flx
    assert abs(np.sum(terms)) <= 1e-13 * np.sum(np.abs(terms))


@settings(**SETTINGS)
@given(c=st.floats(min_value=-1e6, max_value=1e6, allow_subnormal=False))
def test_interpolation_keeps_constants(mesh, oracle, c):
    one = np.full(mesh.nCells, c)
    tol = 1e-14 * max(abs(c), 1e-300)
    assert np.max(np.abs(oracle.op("c2e", one, out_size=mesh.nEdges) - c)) <= tol
    assert np.max(np.abs(oracle.op("c2v", one, out_size=mesh.nVertices) - c)) <= 10 * tol


@settings(max_examples=20, deadline=None, derandomize=True)
@given(seed=seeds, amp=st.floats(min_value=0.0, max_value=0.05), umax=st.floats(min_value=0.0, max_value=20.0),
       hs=st.floats(min_value=0.0, max_value=2000.0), time_scheme=st.sampled_from([1, 2, 3]),
       pv=st.sampled_from([(1, 3, 0.0), (1, 3, 0.5), (2, 3, 0.0), (3, 3, 0.0), (3, 4, 0.0), (3, 5, 0.0),
                           (3, 6, 0.0)]))
def test_time_schemes_conserve_mass_and_energy(mesh, seed, amp, umax, hs, time_scheme, pv):
    """From a random positive-depth state, random (divergent) wind and random
    topography: CRK3, CRK4 and PC2 with their energy-conserving beta
    (time_scheme_mod.F90:94-100, :139-146, :174-180) keep total mass and total
    energy (tmcore_swm_mod.F90:215-231) to round-off, for centred pv with and
    without APVM, the conservative APVM and upwind pv of orders 3-6 (each a pv
    on edges inside the energy-neutral q.F_perp)."""
    pv_scheme, order, apvm = pv
    rng = np.random.default_rng(seed)
    g, h0 = 9.80616, 5000.0
    ghs = g * hs * rng.uniform(0.0, 1.0, mesh.nCells)
    gd = g * h0 * (1.0 + amp * rng.uniform(-1.0, 1.0, mesh.nCells)) - ghs
    u = umax * rng.uniform(-1.0, 1.0, mesh.nEdges)
    o = ORACLE.Oracle(mesh, dt=600.0, pv_scheme=pv_scheme, interp_pv_order=order, apvm_weight=apvm, adv_order=2,
                      time_scheme=time_scheme, conserve_energy=1)
    try:
        o.set_initial(gd, u, ghs)
        d0 = o.diag()
        o.step(3)
        d1 = o.diag()
        vor = o.vertex()[1]
    finally:
        o.close()
    assert abs(d1[0] - d0[0]) <= 1e-13 * abs(d0[0])  # mass
    assert abs(d1[1] - d0[1]) <= 1e-12 * abs(d0[1])  # energy
    # absolute vorticity (tmcore_swm_mod.F90:249-255): the curl sums to zero
    assert abs(d1[3] - d0[3]) <= 1e-12 * max(np.max(np.abs(vor)), 1e-300) + 1e-18


@pytest.mark.parametrize("kw", [dict(pv_scheme=1), dict(pv_scheme=2), dict(pv_scheme=3, interp_pv_order=3),
                                dict(pv_scheme=1, time_scheme=1), dict(pv_scheme=1, time_scheme=3),
                                dict(pv_scheme=1, apvm_weight=0.5), dict(pv_scheme=1, adv_order=3)])
def test_state_at_rest_stays_at_rest(mesh, kw):
    """A flat depth and no wind make every tendency zero.  The reference's
    CRK4 and CRK3 beta (time_scheme_mod.F90:145, :99) and its conservative
    APVM epsilon (operators_mod.F90:349-351) are then 0 / 0; the oracle takes
    beta = 1 (as the reference's PC2 does, :178) and epsilon = 0, so the state
    stays exactly at rest."""
    gd = np.full(mesh.nCells, 9.80616 * 5000.0)
    o = ORACLE.Oracle(mesh, dt=600.0, conserve_energy=1, **kw)
    try:
        o.set_initial(gd, np.zeros(mesh.nEdges), np.zeros(mesh.nCells))
        o.step(2)
        g1, i1 = o.state()[:2]
        d = o.diag()
    finally:
        o.close()
    assert np.array_equal(g1, gd) and not np.any(i1)
    assert np.all(np.isfinite(d)) and d[4] == 1.0


@pytest.fixture(scope="module")
def mesh3():
    return icos(3)


@settings(max_examples=12, deadline=None, derandomize=True)
@given(seed=seeds, order=st.sampled_from([2, 3, 4, 5, 6]), mono=st.sampled_from([0, 1]),
       c=st.floats(min_value=1e-3, max_value=1e3), umax=st.floats(min_value=0.0, max_value=30.0))
def test_tracers_keep_constants_and_mass(mesh3, seed, order, mono, c, umax):
    """Coupled tracers from a random state, random wind: a constant mixing
    ratio stays that constant (the sg11 edge value of a constant is the
    constant, adv_scheme_sg11_mod.F90:42-45 with the upwind correction of
    operators_mod.F90:423-472), and a random tracer's mass is conserved."""
    m = mesh3
    rng = np.random.default_rng(seed)
    gd = 9.80616 * 5000.0 * (1.0 + 0.05 * rng.uniform(-1.0, 1.0, m.nCells))
    u = umax * rng.uniform(-1.0, 1.0, m.nEdges)
    q = np.stack([np.full(m.nCells, c), rng.uniform(0.0, 1.0, m.nCells)])
    o = ORACLE.Oracle(m, dt=600.0, pv_scheme=1, apvm_weight=0.0, n_tracers=2, tracer_adv_order=order,
                      tracer_adv_mono=mono)
    try:
        o.set_initial(gd, u, np.zeros(m.nCells))
        o.set_tracers(q * gd[None, :])
        g0 = o.state()[0]
        m0 = np.sum(o.tracers()[1] * m.areaCell)
        o.step(3)
        g1 = o.state()[0]
        qt = o.tracers()
    finally:
        o.close()
    assert np.all(np.isfinite(qt)) and np.all(np.isfinite(g1))
    assert np.max(np.abs(qt[0] / g1 - c)) <= 1e-12 * c
    assert abs(np.sum(qt[1] * m.areaCell) - m0) <= 1e-12 * abs(m0)
    assert np.all(g0 > 0)


@settings(max_examples=15, deadline=None, derandomize=True)
@given(seed=seeds, wind=st.sampled_from([1, 2]), order=st.sampled_from([2, 3, 4, 5, 6]),
       mono=st.sampled_from([0, 1]), time_scheme=st.sampled_from([1, 2, 3]),
       c=st.floats(min_value=-1e3, max_value=1e3))
def test_prescribed_wind_advection_conserves_and_keeps_constants(mesh3, seed, wind, order, mono, time_scheme, c):
    """The adv model (tmcore_adv_mod.F90:78-97, adv_scheme_sg11_mod.F90:33-48)
    under the cosine-bell and deformation winds: a random scalar's total is
    conserved to round-off (flux form), and a constant stays that constant
    (the winds are non-divergent and the sg11 edge value of a constant is the
    constant)."""
    m = mesh3
    q = np.random.default_rng(seed).uniform(0.0, 1.0, m.nCells)
    out = []
    for q0 in (q, np.full(m.nCells, c)):
        o = ORACLE.Oracle(m, dt=3600.0, adv_order=order, adv_mono=mono, time_scheme=time_scheme, conserve_energy=0)
        try:
            o.adv_set_initial(q0, wind)
            o.adv_step(4)
            out.append(o.adv_state()[0])
        finally:
            o.close()
    m0 = np.sum(q * m.areaCell)
    assert np.all(np.isfinite(out[0]))
    assert abs(np.sum(out[0] * m.areaCell) - m0) <= 1e-12 * abs(m0)
    assert np.max(np.abs(out[1] - c)) <= 1e-11 * max(abs(c), 1e-300)
