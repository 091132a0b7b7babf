"""GPU (sm_103a) against the CPU FP64 oracle, through the C ABI.

The FP64 device path is compiled without FMA contraction and follows the
reference's per-element expression order, so single operators and one
spatial_operators call must be BIT-IDENTICAL to the oracle.  Multi-step runs
differ only through the order of the global sums (beta, invariants), which
the device reduces with compensated double-double arithmetic: the bar there
is a 1e-11 relative max-norm on h and u after one simulated day (checked on
level 5 with dt = 600 s, 144 steps).
"""
import numpy as np
import pytest

from conftest import icos, rel_max

pytestmark = pytest.mark.gpu


def _models(mesh, **kw):
    from oracle.oracle import Oracle
    from tmcore_gb300.gpu import TMCoreGPU

    okw = {k: v for k, v in kw.items() if k not in ("precision", "renumber", "use_graph", "diag_every",
                                                    "block_size", "stencils")}
    return TMCoreGPU(mesh, **kw), Oracle(mesh, **okw)


def _ic(mesh, seed=0):
    from tmcore_gb300 import cases

    return cases.jet_bumps(mesh, seed=seed)


@pytest.mark.parametrize("renumber", [0, 1])
def test_operators_bit_exact(mesh4, renumber):
    g, o = _models(mesh4, dt=600.0, pv_scheme=1, apvm_weight=0.0, renumber=renumber, stencils=1)
    rng = np.random.default_rng(1)
    fe = rng.standard_normal(mesh4.nEdges)
    fc = rng.standard_normal(mesh4.nCells) + 3.0
    fv = rng.standard_normal(mesh4.nVertices)
    nc, ne, nv = mesh4.nCells, mesh4.nEdges, mesh4.nVertices
    assert np.array_equal(g.op("div", fe), o.op("div", fe, out_size=nc))
    assert np.array_equal(g.op("curl", fe), o.op("curl", fe, out_size=nv))
    assert np.array_equal(g.op("c2e", fc), o.op("c2e", fc, out_size=ne))
    assert np.array_equal(g.op("c2v", fc), o.op("c2v", fc, out_size=nv))
    assert np.array_equal(g.op("v2c", fv), o.op("v2c", fv, out_size=nc))
    assert np.array_equal(g.op("v2e", fv), o.op("v2e", fv, out_size=ne))
    assert np.array_equal(g.op("kinetic_energy", fe), o.op("kinetic_energy", fe, out_size=nc))
    assert np.array_equal(g.op("tangent_wind", fe), o.op("tangent_wind", fe, out_size=ne))
    ge = rng.uniform(1e4, 5e4, ne)
    pe = rng.standard_normal(ne) * 1e-8
    assert np.array_equal(g.tangent_vor_flux(fe, ge, pe), o.op("tangent_vor_flux", fe, ge, pe, out_size=ne))
    for order in (3, 4, 5):
        for mono in (0, 1):
            a = g.upwind_correction(fc, fe, np.zeros(ne), order, mono)
            b = o.upwind_correction(fc, fe, np.zeros(ne), order, mono)
            assert np.array_equal(a, b), (order, mono)
    g.close()


@pytest.mark.parametrize("cfg", [
    dict(pv_scheme=1, apvm_weight=0.0),
    dict(pv_scheme=1, apvm_weight=0.5),
    dict(pv_scheme=3, interp_pv_order=3),
    dict(pv_scheme=3, interp_pv_order=4),
    dict(pv_scheme=3, interp_pv_order=5),
    dict(pv_scheme=1, apvm_weight=0.0, adv_order=3, adv_mono=1),
    dict(pv_scheme=3, interp_pv_order=3, adv_order=4),
])
def test_spatial_operators_bit_exact(mesh4, cfg):
    g, o = _models(mesh4, dt=600.0, **cfg)
    gd, u, ghs = _ic(mesh4)
    o.set_initial(gd, u, ghs)
    g.set_initial(gd, u, ghs)
    gd0, iap0, _ = o.state()
    tg_o, tu_o = o.spatial_operators(gd0, iap0)
    tg_g, tu_g = g.spatial_operators(gd0, iap0)
    assert np.array_equal(tg_g, tg_o)
    assert np.array_equal(tu_g, tu_o)
    g.close()


def test_initial_state_and_diag(mesh4):
    g, o = _models(mesh4, dt=600.0, pv_scheme=1, apvm_weight=0.0)
    gd, u, ghs = _ic(mesh4, seed=3)
    o.set_initial(gd, u, ghs)
    g.set_initial(gd, u, ghs)
    go, io, uo = o.state()
    gg, ig, ug = g.get_state()
    assert np.array_equal(gg, go) and np.array_equal(ig, io)
    # the oracle keeps the initial-condition u; the device reports iap_u / sqrt(gd_edge)
    assert rel_max(ug, uo) < 4e-16
    pvo, voro = o.vertex()
    pvg, vorg = g.get_vertex()
    # vorticity and pv of the device follow from that u (1-ulp differences in u)
    assert rel_max(pvg, pvo) < 1e-14 and rel_max(vorg, voro) < 1e-12
    do, dg = o.diag(), g.diag()
    assert abs(dg[0] - do[0]) <= 1e-14 * abs(do[0])
    assert abs(dg[1] - do[1]) <= 1e-14 * abs(do[1])
    assert abs(dg[2] - do[2]) <= 1e-13 * abs(do[2])
    assert abs(dg[3] - do[3]) <= 1e-10 * np.max(np.abs(voro))
    g.close()


@pytest.mark.parametrize("cfg", [
    dict(pv_scheme=1, apvm_weight=0.0),
    dict(pv_scheme=3, interp_pv_order=3, apvm_weight=0.5),
])
def test_steps_match_oracle(mesh4, cfg):
    g, o = _models(mesh4, dt=600.0, **cfg)
    gd, u, ghs = _ic(mesh4, seed=1)
    o.set_initial(gd, u, ghs)
    g.set_initial(gd, u, ghs)
    o.step(1)
    g.step(1)
    go, io, _ = o.state()
    gg, ig, _ = g.get_state()
    # one step: only beta's summation order differs
    assert rel_max(gg, go) < 1e-14 and rel_max(ig, io) < 1e-14
    assert abs(g.diag()[4] - o.diag()[4]) < 1e-14
    o.step(20)
    g.step(20)
    go, io, uo = o.state()
    gg, ig, ug = g.get_state()
    assert rel_max(gg, go) < 1e-12 and rel_max(ug, uo) < 1e-12
    g.close()


def test_one_day_level5_parity_and_invariants(mesh5):
    """Spec bar: h and u within 1e-11 relative max-norm after one day;
    mass conserved to round-off; energy and enstrophy drift as the oracle's."""
    g, o = _models(mesh5, dt=600.0, pv_scheme=1, apvm_weight=0.0)
    gd, u, ghs = _ic(mesh5, seed=0)
    o.set_initial(gd, u, ghs)
    g.set_initial(gd, u, ghs)
    d0o, d0g = o.diag(), g.diag()
    o.step(144)
    g.step(144)
    go, io, uo = o.state()
    gg, ig, ug = g.get_state()
    assert rel_max(gg, go) < 1e-11
    assert rel_max(ug, uo) < 1e-11
    d1o, d1g = o.diag(), g.diag()
    assert abs(d1g[0] - d0g[0]) / d0g[0] < 1e-13            # mass to round-off
    assert abs(d1g[1] - d0g[1]) / d0g[1] < 1e-12            # energy conserved by beta
    dz_o = (d1o[2] - d0o[2]) / d0o[2]
    dz_g = (d1g[2] - d0g[2]) / d0g[2]
    assert abs(dz_g - dz_o) <= 1e-3 * abs(dz_o)             # enstrophy drift to 3 digits
    g.close()


@pytest.mark.parametrize("seed,cfg", [(0, dict(pv_scheme=1, apvm_weight=0.0)),
                                      (1, dict(pv_scheme=3, interp_pv_order=3))])
def test_five_day_level5_config(mesh5, seed, cfg):
    """The level-5 parity configuration in full: 5 simulated days (720 CRK4
    steps of 600 s) of centred pv (no diffusion) and of the shipped
    pv_scheme 3.  Measured on a GB300: h and u within 2.3e-15 and 1.3e-14
    relative max-norm of the oracle, mass and energy drift below 2e-16, and
    the enstrophy drift equal to the oracle's to 9 digits; the bounds leave
    margin for another GPU of the same architecture."""
    g, o = _models(mesh5, dt=600.0, **cfg)
    gd, u, ghs = _ic(mesh5, seed=seed)
    o.set_initial(gd, u, ghs)
    g.set_initial(gd, u, ghs)
    d0o, d0g = o.diag(), g.diag()
    o.step(720)
    g.step(720)
    go, io, uo = o.state()
    gg, ig, ug = g.get_state()
    assert rel_max(gg, go) < 1e-12 and rel_max(ug, uo) < 1e-12, (rel_max(gg, go), rel_max(ug, uo))
    d1o, d1g = o.diag(), g.diag()
    assert abs(d1g[0] - d0g[0]) / d0g[0] < 1e-13
    assert abs(d1g[1] - d0g[1]) / d0g[1] < 1e-12
    dz_o = (d1o[2] - d0o[2]) / d0o[2]
    dz_g = (d1g[2] - d0g[2]) / d0g[2]
    assert abs(dz_g - dz_o) <= 1e-6 * abs(dz_o)
    g.close()


@pytest.mark.parametrize("tracer_order", [0, 3, 5])
def test_tracers_match_oracle(mesh4, tracer_order):
    from tmcore_gb300 import cases

    kw = dict(dt=600.0, pv_scheme=1, apvm_weight=0.0, n_tracers=3, tracer_adv_order=tracer_order,
              tracer_adv_mono=1)
    g, o = _models(mesh4, **kw)
    gd, u, ghs = _ic(mesh4, seed=2)
    q = cases.smooth_tracers(mesh4, 3, seed=2)
    q[2] = 1.0  # a constant mixing ratio must stay constant
    qgd = q * gd[None, :]
    o.set_initial(gd, u, ghs)
    g.set_initial(gd, u, ghs)
    o.set_tracers(qgd)
    g.set_tracers(qgd)
    o.step(10)
    g.step(10)
    qo, qg = o.tracers(), g.get_tracers()
    assert rel_max(qg, qo) < 1e-13
    gg, _, _ = g.get_state()
    assert np.max(np.abs(qg[2] / gg - 1.0)) < 1e-12
    g.close()


def test_time_integrate_host_arrays(mesh4):
    from tmcore_gb300.gpu import TMCoreGPU

    gd, u, ghs = _ic(mesh4, seed=4)
    a = TMCoreGPU(mesh4, dt=600.0, pv_scheme=1, apvm_weight=0.0)
    b = TMCoreGPU(mesh4, dt=600.0, pv_scheme=1, apvm_weight=0.0, use_graph=0)
    a.set_initial(gd, u, ghs)
    b.set_initial(gd, u, ghs)
    g0, i0, _ = a.get_state()
    g1, i1, _ = a.time_integrate(g0, i0)
    b.step(1)
    gb, ib, _ = b.get_state()
    assert np.array_equal(g1, gb) and np.array_equal(i1, ib)
    a.close()
    b.close()


@pytest.mark.parametrize("tracer_order,n_tracers,use_graph,diag_every",
                         [(2, 2, 1, 1), (3, 2, 1, 1), (2, 4, 1, 1), (2, 1, 1, 2), (2, 4, 0, 1), (2, 3, 1, 1)])
def test_time_integrate_host_arrays_with_tracers(mesh4, tracer_order, n_tracers, use_graph, diag_every):
    """FP32 with coupled tracers: tmc_time_integrate on host arrays equals the
    same steps of the device-resident state, bit for bit.  With second-order
    tracers the edge preparation runs before the tracer copy has arrived; with
    1, 2 or 4 of them all of stage 1 but its tracer terms does (a tracer-free
    cell pass, then k_tracers_fast), in the step graph's tail or launched one
    by one, on diagnostic steps and others.  Three tracers keep the fused
    program."""
    from tmcore_gb300 import cases
    from tmcore_gb300.gpu import TMCoreGPU

    gd, u, ghs = _ic(mesh4, seed=5)
    qgd = cases.smooth_tracers(mesh4, n_tracers, seed=1) * gd[None, :]
    kw = dict(dt=600.0, precision=1, pv_scheme=1, apvm_weight=0.0, n_tracers=n_tracers,
              tracer_adv_order=tracer_order, use_graph=use_graph, diag_every=diag_every)
    a, b = TMCoreGPU(mesh4, **kw), TMCoreGPU(mesh4, **kw)
    for g in (a, b):
        g.set_initial(gd, u, ghs)
        g.set_tracers(qgd)
    g0, i0, _ = a.get_state()
    q0 = a.get_tracers()
    for _ in range(3):
        g0, i0, q0 = a.time_integrate(g0, i0, q0)
        b.step(1)
    gb, ib, _ = b.get_state()
    assert np.array_equal(g0, gb) and np.array_equal(i0, ib)
    assert np.array_equal(q0, b.get_tracers())
    a.close()
    b.close()


def test_renumbering_is_invisible(mesh4):
    from tmcore_gb300.gpu import TMCoreGPU

    gd, u, ghs = _ic(mesh4, seed=5)
    out = []
    for r in (0, 1, 2):  # as given, Hilbert, Morton
        g = TMCoreGPU(mesh4, dt=600.0, pv_scheme=3, renumber=r)
        g.set_initial(gd, u, ghs)
        tg, tu = g.spatial_operators(*g.get_state()[:2])
        out.append((tg, tu))
        g.close()
    for k in (1, 2):
        assert np.array_equal(out[0][0], out[k][0]) and np.array_equal(out[0][1], out[k][1])


def test_fp32_path_error_small(mesh5):
    from tmcore_gb300.gpu import TMCoreGPU

    gd, u, ghs = _ic(mesh5, seed=0)
    a = TMCoreGPU(mesh5, dt=600.0, pv_scheme=1, apvm_weight=0.0, precision=0)
    b = TMCoreGPU(mesh5, dt=600.0, pv_scheme=1, apvm_weight=0.0, precision=1)
    for m in (a, b):
        m.set_initial(gd, u, ghs)
        m.step(144)
    ga, _, ua = a.get_state()
    gb, _, ub = b.get_state()
    h_err = rel_max(gb, ga)
    assert h_err < 1e-5, h_err
    assert rel_max(ub, ua) < 1e-3
    da, db = a.diag(), b.diag()
    assert abs(db[0] - da[0]) / da[0] < 1e-12  # FP64 gd accumulation keeps mass
    a.close()
    b.close()


@pytest.mark.parametrize("order", [3, 4])
def test_fp32_upwind_pv_error_small(mesh5, order):
    """The FP32 path with upwind pv (pv_scheme 3, the shipped namelist's
    scheme; packed FP32 stencils, one edge per thread) against the FP64 path,
    which is the oracle's arithmetic: one simulated day at level 5."""
    from tmcore_gb300.gpu import TMCoreGPU

    gd, u, ghs = _ic(mesh5, seed=6)
    kw = dict(dt=600.0, pv_scheme=3, interp_pv_order=order)
    a = TMCoreGPU(mesh5, **kw, precision=0)
    b = TMCoreGPU(mesh5, **kw, precision=1)
    for m in (a, b):
        m.set_initial(gd, u, ghs)
    ta = a.spatial_operators(*a.get_state()[:2])
    tb = b.spatial_operators(*a.get_state()[:2])
    # FP32 pv differences in the fit stencils: measured 2.4e-4 (order 3)
    assert rel_max(tb[1], ta[1]) < 1e-3, rel_max(tb[1], ta[1])
    for m in (a, b):
        m.step(144)
    ga, _, ua = a.get_state()
    gb, _, ub = b.get_state()
    assert rel_max(gb, ga) < 1e-5, rel_max(gb, ga)
    assert rel_max(ub, ua) < 1e-3
    a.close()
    b.close()


@pytest.mark.parametrize("cfg", [
    dict(pv_scheme=1, apvm_weight=0.0, adv_order=3, adv_mono=1),
    dict(pv_scheme=3, interp_pv_order=3, adv_order=4, adv_mono=1),
    dict(pv_scheme=3, interp_pv_order=5, adv_order=5, adv_mono=1, n_tracers=2, tracer_adv_order=5,
         tracer_adv_mono=1),
])
def test_steps_match_oracle_upwind_orders(mesh4, cfg):
    """The fused stages keep the next stage's iap_u in registers: upwind
    corrections (adv_order >= 3) must take their side from quantities that
    are stored."""
    from tmcore_gb300 import cases

    g, o = _models(mesh4, dt=600.0, **cfg)
    gd, u, ghs = _ic(mesh4, seed=10)
    o.set_initial(gd, u, ghs)
    g.set_initial(gd, u, ghs)
    ntr = cfg.get("n_tracers", 0)
    if ntr:
        qgd = cases.smooth_tracers(mesh4, ntr, seed=10) * gd[None, :]
        o.set_tracers(qgd)
        g.set_tracers(qgd)
    o.step(1)
    g.step(1)
    go, io, _ = o.state()
    gg, ig, _ = g.get_state()
    assert rel_max(gg, go) < 1e-14 and rel_max(ig, io) < 1e-14
    o.step(9)
    g.step(9)
    go, _, uo = o.state()
    gg, _, ug = g.get_state()
    assert rel_max(gg, go) < 1e-12 and rel_max(ug, uo) < 1e-11
    if ntr:
        assert rel_max(g.get_tracers(), o.tracers()) < 1e-12
    g.close()


def test_health_error_on_blown_up_state(mesh4):
    """A state outside the physical range (a negative depth) turns the step's
    fields non-finite; tmc_get_diag reports it as TMC_E_HEALTH and the handle
    stays usable: a valid state set afterwards steps normally."""
    from tmcore_gb300 import abi
    from tmcore_gb300.gpu import TMCError, TMCoreGPU

    for prec in (0, 1):
        g = TMCoreGPU(mesh4, dt=600.0, pv_scheme=1, apvm_weight=0.0, precision=prec)
        gd, u, ghs = _ic(mesh4, seed=3)
        bad = gd.copy()
        bad[::7] = -bad[::7]
        g.set_initial(bad, u, ghs)
        g.step(2)
        with pytest.raises(TMCError) as e:
            g.diag()
        assert e.value.code == abi.TMC_E_HEALTH
        g.set_initial(gd, u, ghs)
        g.step(2)
        assert np.all(np.isfinite(g.diag()))
        g.close()


def test_device_pointers_match_host_arrays(mesh4):
    """The state and field calls accept device arrays as well as host arrays
    (the copy direction comes from unified addressing): the same calls with
    CUDA tensors give bit-identical results."""
    import ctypes

    torch = pytest.importorskip("torch")
    from tmcore_gb300.gpu import TMCoreGPU

    f64p = ctypes.POINTER(ctypes.c_double)
    dev = torch.device("cuda:0")

    def dptr(t):
        return ctypes.cast(t.data_ptr(), f64p)

    g = TMCoreGPU(mesh4, dt=600.0, pv_scheme=3, interp_pv_order=3)
    gd, u, ghs = _ic(mesh4, seed=11)
    g.set_initial(gd, u, ghs)
    g.step(2)
    gd1, iap1, _ = g.get_state()
    tg_h, tu_h = g.spatial_operators(gd1, iap1)
    d_gd = torch.from_numpy(gd1).to(dev)
    d_iap = torch.from_numpy(iap1).to(dev)
    d_tg = torch.zeros_like(d_gd)
    d_tu = torch.zeros_like(d_iap)
    torch.cuda.synchronize()
    assert g.lib.tmc_spatial_operators(g.h, dptr(d_gd), dptr(d_iap), dptr(d_tg), dptr(d_tu)) == 0
    assert np.array_equal(d_tg.cpu().numpy(), tg_h) and np.array_equal(d_tu.cpu().numpy(), tu_h)
    # set_state / get_state through device arrays
    assert g.lib.tmc_set_state(g.h, dptr(d_gd), dptr(d_iap)) == 0
    o_gd, o_iap = torch.zeros_like(d_gd), torch.zeros_like(d_iap)
    assert g.lib.tmc_get_state(g.h, dptr(o_gd), dptr(o_iap), None) == 0
    assert np.array_equal(o_gd.cpu().numpy(), gd1) and np.array_equal(o_iap.cpu().numpy(), iap1)
    # time_integrate: device arrays in and out equal host arrays in and out
    n_gd, n_iap = torch.zeros_like(d_gd), torch.zeros_like(d_iap)
    assert g.lib.tmc_time_integrate(g.h, dptr(d_gd), dptr(d_iap), None, dptr(n_gd), dptr(n_iap), None) == 0
    h_gd, h_iap = np.empty_like(gd1), np.empty_like(iap1)
    assert g.lib.tmc_time_integrate(g.h, gd1.ctypes.data_as(f64p), iap1.ctypes.data_as(f64p), None,
                                    h_gd.ctypes.data_as(f64p), h_iap.ctypes.data_as(f64p), None) == 0
    assert np.array_equal(n_gd.cpu().numpy(), h_gd) and np.array_equal(n_iap.cpu().numpy(), h_iap)
    g.close()


def test_handles_on_concurrent_host_threads(mesh4):
    """One handle per host thread: two threads create, step and read their own
    handles at the same time (ctypes releases the GIL during the calls); each
    result equals the same run made alone."""
    import threading

    from tmcore_gb300.gpu import TMCoreGPU

    def run(seed, prec, out, key):
        g = TMCoreGPU(mesh4, dt=600.0, pv_scheme=1, apvm_weight=0.0, precision=prec)
        g.set_initial(*_ic(mesh4, seed=seed))
        for _ in range(5):
            g.step(4)
            g.diag()
        out[key] = g.get_state()
        g.close()

    jobs = [(21, 0), (22, 1), (23, 1)]
    together, alone = {}, {}
    threads = [threading.Thread(target=run, args=(s, p, together, k)) for k, (s, p) in enumerate(jobs)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for k, (s, p) in enumerate(jobs):
        run(s, p, alone, k)
        assert all(np.array_equal(a, b) for a, b in zip(together[k], alone[k])), k


@pytest.mark.parametrize("prec,layout,members,scheme", [
    (0, 0, 1, dict(pv_scheme=1, apvm_weight=0.5)),
    (1, 0, 1, dict(pv_scheme=3, interp_pv_order=3, n_tracers=2)),
    (1, 0, 3, dict(pv_scheme=1, apvm_weight=0.0)),
    (1, 1, 32, dict(pv_scheme=3, interp_pv_order=4)),
])
def test_concurrent_branches_match_the_serial_program(mesh4, prec, layout, members, scheme):
    """The step runs a stage's vertex and pv-on-edge passes on a second stream
    beside the cell pass (a fork and a join in the captured graph).  The same
    steps launched one pass after another (the per-pass timing path of
    tmc_time_steps) give bit-identical states and invariants, for the FP64
    and FP32 single models, member-outermost and member-innermost ensembles."""
    from tmcore_gb300 import cases
    from tmcore_gb300.gpu import TMCoreGPU

    kw = dict(dt=600.0, precision=prec, diag_every=1, **scheme)
    if members > 1:
        kw.update(members=members, member_layout=layout)
    a, b = TMCoreGPU(mesh4, **kw), TMCoreGPU(mesh4, **kw)
    for g in (a, b):
        for m in range(members):
            if members > 1:
                g.select_member(m)
            gd, u, ghs = _ic(mesh4, seed=40 + m)
            g.set_initial(gd, u, ghs)
            if scheme.get("n_tracers"):
                g.set_tracers(cases.smooth_tracers(mesh4, 2, seed=m) * gd[None, :])
    a.step(6)                                 # graph steps: concurrent branches
    b.time_steps(6, total=False, flux=True)   # eager steps with per-pass events: serial
    for m in range(members):
        if members > 1:
            a.select_member(m)
            b.select_member(m)
        assert all(np.array_equal(x, y) for x, y in zip(a.get_state(), b.get_state())), m
    assert np.array_equal(a.diag_all() if members > 1 else a.diag(), b.diag_all() if members > 1 else b.diag())
    a.close()
    b.close()


@pytest.mark.parametrize("kw", [
    dict(precision=0),
    dict(precision=1, n_tracers=2),
    dict(precision=1, time_scheme=1),
    dict(precision=1, members=2),
    dict(precision=1, members=16, member_layout=1),
    dict(precision=0, pv_scheme=2),
    dict(precision=1, pv_scheme=2),
])
def test_state_at_rest_stays_at_rest(mesh4, kw):
    """A flat depth and no wind: every tendency is zero, so CRK4's (and
    CRK3's) beta would be 0 / 0 (time_scheme_mod.F90:145, :99), and so would
    the conservative APVM's epsilon (operators_mod.F90:349-351).  The device
    takes beta = 1 there, as the reference's PC2 does (:178), and epsilon = 0,
    as the oracle does: the state stays exactly as it was, with finite
    invariants."""
    from tmcore_gb300 import cases
    from tmcore_gb300.gpu import TMCoreGPU

    gd = np.full(mesh4.nCells, 9.80616 * 5000.0)
    u = np.zeros(mesh4.nEdges)
    ghs = np.zeros(mesh4.nCells)
    kw = {"pv_scheme": 1, **kw}
    g = TMCoreGPU(mesh4, dt=600.0, apvm_weight=0.0, conserve_energy=1, **kw)
    members = kw.get("members", 1)
    for m in range(members):
        if members > 1:
            g.select_member(m)
        g.set_initial(gd, u, ghs)
        if kw.get("n_tracers"):
            g.set_tracers(cases.smooth_tracers(mesh4, kw["n_tracers"], seed=3) * gd[None, :])
    before = []
    for m in range(members):
        if members > 1:
            g.select_member(m)
        before.append(g.get_state()[0])
    g.step(3)
    d = g.diag_all() if members > 1 else g.diag()[None, :]
    assert np.all(np.isfinite(d))
    assert np.all(d[:, 4] == 1.0)
    for m in range(members):
        if members > 1:
            g.select_member(m)
        g1, i1, _ = g.get_state()
        assert np.array_equal(g1, before[m]) and not np.any(i1)
    g.close()
