"""Member-innermost ensembles (tmc_params.member_layout = 1): arrays
[element][member], 32 (or 16) lanes per element, one or two members per lane.

The kernels repeat the FP32 single-model expressions, but the compiler
contracts multiplies and adds into FMAs differently in the two kernels, so
FP32 fields differ in the last bit here and there; the gd tendency is a
cancellation of large flux terms, which turns those bits into relative
differences of about 1e-8 in gd after a few steps.  A member that read a
wrong neighbour or another member's data would be off by 1e-3 or more.  The
invariants come from compensated sums over another partition (FP32 terms for
energy, enstrophy and absolute vorticity; FP64 gd for mass)."""
import numpy as np
import pytest

from conftest import rel_max

pytestmark = pytest.mark.gpu

M = 32
KW = dict(precision=1, pv_scheme=1, apvm_weight=0.0, adv_order=2)


def _ics(mesh, n, seed0):
    from tmcore_gb300 import cases

    return [cases.jet_bumps(mesh, seed=seed0 + m) for m in range(n)]


def _ensemble(mesh, ics, layout, **kw):
    from tmcore_gb300.gpu import TMCoreGPU

    ens = TMCoreGPU(mesh, members=len(ics), member_layout=layout, **{**KW, **kw})
    for m, (gd, u, ghs) in enumerate(ics):
        ens.select_member(m)
        ens.set_initial(gd, u, ghs)
    return ens


def _single(mesh, ic, **kw):
    from tmcore_gb300.gpu import TMCoreGPU

    one = TMCoreGPU(mesh, **KW, **kw)
    one.set_initial(*ic)
    return one


# 16 and 48: a warp covers two elements of 16 members; 64: two members per lane
@pytest.mark.parametrize("members", [16, M, 48, 2 * M])
def test_members_match_single_runs_without_beta(mesh4, members):
    kw = dict(dt=600.0, conserve_energy=0, diag_every=1)
    ics = _ics(mesh4, members, 100)
    ens = _ensemble(mesh4, ics, 1, **kw)
    outer = _ensemble(mesh4, ics, 0, **kw)
    ens.step(7)
    outer.step(7)
    for m in (0, 13, members - 1):
        one = _single(mesh4, ics[m], **kw)
        one.step(7)
        ens.select_member(m)
        outer.select_member(m)
        ge, ie, ue = ens.get_state()
        g1, i1, u1 = one.get_state()
        go, io, _ = outer.get_state()
        errs = (rel_max(ge, g1), rel_max(ie, i1), rel_max(ue, u1), rel_max(ge, go), rel_max(ie, io))
        assert max(errs[0], errs[3]) < 1e-6 and max(errs[1], errs[2], errs[4]) < 1e-5, (m, errs)
        pe, ve = ens.get_vertex()
        p1, v1 = one.get_vertex()
        assert rel_max(pe, p1) < 1e-5 and rel_max(ve, v1) < 1e-5, m
        de, d1 = ens.diag(), one.diag()
        assert abs(de[0] - d1[0]) <= 1e-13 * abs(d1[0]), (de[0], d1[0])  # mass: FP64 gd, conserved by both
        assert abs(de[1] - d1[1]) <= 1e-8 * abs(d1[1]), (de[1], d1[1])   # energy
        assert abs(de[2] - d1[2]) <= 1e-6 * abs(d1[2]), (de[2], d1[2])   # potential enstrophy
        assert abs(de[3] - d1[3]) <= 1e-9 * 2 * 7.292e-5, (de[3], d1[3])  # absolute vorticity (mean of f + vor)
        assert de[4] == 1.0
        one.close()
    ens.close()
    outer.close()


@pytest.mark.parametrize("members", [M, 2 * M])
def test_members_match_single_runs_with_beta(mesh4, members):
    kw = dict(dt=600.0, conserve_energy=1, diag_every=1)
    ics = _ics(mesh4, members, 200)
    ens = _ensemble(mesh4, ics, 1, **kw)
    ens.step(10)
    all_diag = ens.diag_all()
    for m in (0, 7, members - 1):
        one = _single(mesh4, ics[m], **kw)
        one.step(10)
        ens.select_member(m)
        ge, ie, _ = ens.get_state()
        g1, i1, _ = one.get_state()
        assert rel_max(ge, g1) < 1e-6, (m, rel_max(ge, g1))
        assert rel_max(ie, i1) < 1e-5, (m, rel_max(ie, i1))
        d1 = one.diag()
        assert abs(all_diag[m, 4] - d1[4]) < 1e-6, (m, all_diag[m, 4], d1[4])  # beta
        assert abs(all_diag[m, 0] - d1[0]) <= 1e-12 * abs(d1[0])
        one.close()
    ens.close()


# the reference namelist's pv scheme (upwind, interp_pv_order 3; its
# apvm_weight 0.5 applies to pv_scheme 1 only), and order 4; 128 members:
# four members per lane
@pytest.mark.parametrize("members,order", [(M, 3), (2 * M, 3), (48, 4), (4 * M, 3)])
def test_upwind_pv_members_match_single_runs(mesh4, members, order):
    from tmcore_gb300.gpu import TMCoreGPU

    kw = dict(dt=600.0, conserve_energy=1, diag_every=1, precision=1, pv_scheme=3, interp_pv_order=order,
              apvm_weight=0.5, adv_order=2)
    ics = _ics(mesh4, members, 1100)
    ens = TMCoreGPU(mesh4, members=members, member_layout=1, **kw)
    for m, (gd, u, ghs) in enumerate(ics):
        ens.select_member(m)
        ens.set_initial(gd, u, ghs)
    ens.step(8)
    all_diag = ens.diag_all()
    for m in (0, 21, members - 1):
        one = TMCoreGPU(mesh4, **kw)
        one.set_initial(*ics[m])
        one.step(8)
        ens.select_member(m)
        ge, ie, ue = ens.get_state()
        g1, i1, u1 = one.get_state()
        errs = (rel_max(ge, g1), rel_max(ie, i1), rel_max(ue, u1))
        assert errs[0] < 1e-6 and max(errs[1:]) < 1e-5, (m, errs)
        d1 = one.diag()
        assert abs(all_diag[m, 4] - d1[4]) < 1e-6, (m, all_diag[m, 4], d1[4])  # beta
        assert abs(all_diag[m, 0] - d1[0]) <= 1e-12 * abs(d1[0])
        one.close()
    ens.close()


def test_mass_conserved_and_energy_steady(mesh4):
    kw = dict(dt=600.0, conserve_energy=1, diag_every=1)
    ens = _ensemble(mesh4, _ics(mesh4, 2 * M, 300), 1, **kw)
    d0 = ens.diag_all()
    ens.step(24)
    d1 = ens.diag_all()
    assert np.all(np.isfinite(d1))
    assert np.max(np.abs(d1[:, 0] - d0[:, 0]) / d0[:, 0]) < 1e-13
    assert np.max(np.abs(d1[:, 1] - d0[:, 1]) / d0[:, 1]) < 1e-6
    ens.close()


def test_history_fields_of_a_member(mesh4):
    kw = dict(dt=600.0, conserve_energy=0)
    ics = _ics(mesh4, M, 400)
    ens = _ensemble(mesh4, ics, 1, **kw)
    one = _single(mesh4, ics[5], **kw)
    ens.step(3)
    one.step(3)
    ens.select_member(5)
    he, h1 = ens.history_fields(), one.history_fields()
    for k in h1:
        assert rel_max(he[k], h1[k]) < (1e-4 if k == "div" else 1e-5), (k, rel_max(he[k], h1[k]))
    ens.close()
    one.close()


def test_autotune_and_group(mesh3, mesh4):
    from tmcore_gb300.gpu import TMCoreGroup

    kw = dict(conserve_energy=1, diag_every=0)
    a = _ensemble(mesh4, _ics(mesh4, 64, 500), 1, dt=300.0, **kw)
    before = a.get_state()
    sizes = a.autotune(steps=2)
    assert max(sizes.values()) <= 256
    assert all(np.array_equal(x, y) for x, y in zip(before, a.get_state()))
    # a group of two member-innermost ensembles (levels 3 and 4) equals separate stepping
    g3 = _ensemble(mesh3, _ics(mesh3, M, 600), 1, dt=600.0, **kw)
    s3 = _ensemble(mesh3, _ics(mesh3, M, 600), 1, dt=600.0, **kw)
    s4 = _ensemble(mesh4, _ics(mesh4, 64, 500), 1, dt=300.0, **kw)
    grp = TMCoreGroup([g3, a], cycle_seconds=600.0)
    grp.run(2)
    s3.step(2)
    s4.step(4)
    for x, y in ((g3, s3), (a, s4)):
        for m in (0, 31):
            x.select_member(m)
            y.select_member(m)
            assert all(np.array_equal(p, q) for p, q in zip(x.get_state(), y.get_state()))
    grp.close()
    for x in (a, g3, s3, s4):
        x.close()


@pytest.mark.parametrize("members,scheme", [(16, {}), (32, dict(pv_scheme=3, interp_pv_order=3)),
                                            (64, dict(pv_scheme=3, interp_pv_order=4))])
def test_batched_group_matches_separate_runs(mesh3, mesh4, members, scheme):
    """tmc_group_create_ex mode 1: three ensembles (level 4 at dt 150 s and
    300 s, level 3 at dt 600 s) advanced by one launch per pass over all of
    them, two 600-s cycles (4, 2 and 1 steps per cycle: sub-steps with one,
    two and three meshes), against each ensemble stepped alone.  The batch
    kernels run the single-mesh kernels' per-block code, but the compiler
    contracts multiplies and adds into FMAs differently in the two, so FP32
    values differ in the last bit here and there (about 1e-9 relative in the
    double-float gd after 8 steps); a block given the wrong mesh, member
    group or block offset would be off by 1e-3 or more."""
    from tmcore_gb300.gpu import TMCoreGroup

    kw = dict(conserve_energy=1, diag_every=0, **scheme)
    setups = [(mesh4, 150.0, 700), (mesh3, 600.0, 600), (mesh4, 300.0, 500)]
    grouped = [_ensemble(m, _ics(m, members, s), 1, dt=dt, **kw) for m, dt, s in setups]
    alone = [_ensemble(m, _ics(m, members, s), 1, dt=dt, **kw) for m, dt, s in setups]
    grp = TMCoreGroup(grouped, cycle_seconds=600.0, mode=1)
    grp.run(2)
    for (m, dt, _), y in zip(setups, alone):
        y.step(int(round(2 * 600.0 / dt)))
    for x, y in zip(grouped, alone):
        for m in (0, members - 1):
            x.select_member(m)
            y.select_member(m)
            gx, ix, ux = x.get_state()
            gy, iy, uy = y.get_state()
            assert rel_max(gx, gy) < 1e-8, rel_max(gx, gy)
            assert rel_max(ix, iy) < 1e-5 and rel_max(ux, uy) < 1e-5, (rel_max(ix, iy), rel_max(ux, uy))
        # beta of the last step, per member
        bx, by = x.diag_all()[:, 4], y.diag_all()[:, 4]
        assert np.max(np.abs(bx - by)) < 1e-6, np.max(np.abs(bx - by))
    grp.close()
    for x in grouped + alone:
        x.close()


def test_batched_group_refusals(mesh3):
    from tmcore_gb300 import abi
    from tmcore_gb300.gpu import TMCError, TMCoreGroup

    kw = dict(conserve_energy=1, diag_every=0, dt=600.0)
    a = _ensemble(mesh3, _ics(mesh3, 16, 0), 1, **kw)
    b = _ensemble(mesh3, _ics(mesh3, 32, 0), 1, **kw)
    c = _ensemble(mesh3, _ics(mesh3, 16, 0), 0, **kw)
    for pair in ((a, b), (a, c)):
        with pytest.raises(TMCError) as e:
            TMCoreGroup(list(pair), cycle_seconds=600.0, mode=1)
        assert e.value.code == abi.TMC_E_UNSUP
    for x in (a, b, c):
        x.close()


def test_member_layout_refusals(mesh3):
    from tmcore_gb300 import abi
    from tmcore_gb300.gpu import ClosureMLP, TMCError, TMCoreGPU

    with pytest.raises(TMCError) as e:
        TMCoreGPU(mesh3, dt=600.0, members=40, member_layout=1, **KW)
    assert e.value.code == abi.TMC_E_ARG
    for kw in (dict(pv_scheme=3, interp_pv_order=5), dict(pv_scheme=2, apvm_weight=0.5)):
        with pytest.raises(TMCError) as e:
            TMCoreGPU(mesh3, dt=600.0, members=32, member_layout=1, precision=1, **kw)
        assert e.value.code == abi.TMC_E_UNSUP


def test_closure_features_match_member_outermost(mesh4):
    """tmc_closure_features of a member of a member-innermost ensemble equals
    the member-outermost export of the same state (to FP32 rounding)."""
    ics = _ics(mesh4, M, 900)
    inner, outer = _ensemble(mesh4, ics, 1, dt=600.0), _ensemble(mesh4, ics, 0, dt=600.0)
    for m in (0, 17):
        inner.select_member(m)
        outer.select_member(m)
        fi, pi = inner.closure_features()
        fo, po = outer.closure_features()
        for k in range(fi.shape[1]):
            assert rel_max(fi[:, k], fo[:, k]) < 1e-5, (m, k, rel_max(fi[:, k], fo[:, k]))
        assert rel_max(pi, po) < 1e-5
    inner.close()
    outer.close()


@pytest.mark.parametrize("every_stage", [True, False])
def test_closure_matches_member_outermost(mesh4, every_stage):
    """The learned closure in the member-innermost step (network on rows
    [edge][member]) agrees with the member-outermost step to FP32 rounding;
    a member whose switch is off evolves as the plain model."""
    from tmcore_gb300.gpu import ClosureMLP, TMCoreGPU

    net = ClosureMLP(seed=2)
    p = net.params
    p *= 0.5
    net.params = p
    net.set_scaling(np.zeros(24), np.ones(24), 1e-9)  # corrections of order 1e-9 (pv ~ 1e-8)
    ics = _ics(mesh4, M, 800)
    kw = dict(dt=600.0, conserve_energy=1)
    inner, outer, plain = _ensemble(mesh4, ics, 1, **kw), _ensemble(mesh4, ics, 0, **kw), _ensemble(mesh4, ics, 1, **kw)
    for x in (inner, outer):
        x.set_closure(net)
        x.set_closure_stages(every_stage)
        x.set_member_closure(5, False)
    for x in (inner, outer, plain):
        x.step(6)
    assert not inner.closure_status()
    for m in (0, 5, M - 1):
        for x in (inner, outer, plain):
            x.select_member(m)
        gi, ii, _ = inner.get_state()
        go, io, _ = outer.get_state()
        gp, ip, _ = plain.get_state()
        assert rel_max(gi, go) < 1e-6 and rel_max(ii, io) < 1e-5, (m, rel_max(gi, go), rel_max(ii, io))
        if m == 5:
            assert rel_max(gi, gp) < 1e-6 and rel_max(ii, ip) < 1e-5, m
        else:
            assert rel_max(ii, ip) > 1e-4, (m, rel_max(ii, ip))  # the closure acts
    for x in (inner, outer, plain):
        x.close()
    net.close()


def test_ordering_autotuner(mesh4):
    """The ordering autotuner times element orders x member layouts (and the
    lane layouts of member_layout 1), skips layouts the options do not allow,
    and its choice runs."""
    from tmcore_gb300 import tune
    from tmcore_gb300.gpu import TMCoreGPU

    ics = _ics(mesh4, M, 700)
    best, timings = tune.autotune_ordering(mesh4, ics, steps=2, dt=600.0, **KW)
    nl = len(tune.lane_candidates(M))
    assert len(timings) == 3 * nl + 3 and all("ms_per_step" in t for t in timings), timings
    assert best["renumber"] in (0, 1, 2) and best["member_layout"] in (0, 1)
    ens = TMCoreGPU(mesh4, **best)
    for m, (gd, u, ghs) in enumerate(ics):
        ens.select_member(m)
        ens.set_initial(gd, u, ghs)
    ens.step(3)
    assert np.all(np.isfinite(ens.diag_all()))
    ens.close()
    # pv_scheme 2 has no member-innermost kernels: only member_layout 0 is timed
    kw = dict(KW, pv_scheme=2)
    best, timings = tune.autotune_ordering(mesh4, ics, steps=1, orders=(1,), dt=600.0, **kw)
    assert best["member_layout"] == 0
    assert [t["member_layout"] for t in timings if "error" in t] == [1] * nl
