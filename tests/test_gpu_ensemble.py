"""Ensembles: tmc_params.members > 1 runs independent FP32 models of one mesh
with one launch per pass (member = blockIdx.y).  Every member must evolve
exactly as the same model run alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ic(mesh, seed):
    from tmcore_gb300 import cases

    return cases.jet_bumps(mesh, seed=seed)


@pytest.mark.parametrize("cfg", [
    dict(pv_scheme=1, apvm_weight=0.0),
    dict(pv_scheme=3, interp_pv_order=3, n_tracers=2),
    dict(pv_scheme=2, adv_order=3, adv_mono=1),
])
def test_members_evolve_as_single_models(mesh4, cfg):
    from tmcore_gb300 import cases
    from tmcore_gb300.gpu import TMCoreGPU

    M = 5
    kw = dict(dt=600.0, precision=1, **cfg)
    ens = TMCoreGPU(mesh4, members=M, **kw)
    ntr = cfg.get("n_tracers", 0)
    ics = []
    for m in range(M):
        gd, u, ghs = _ic(mesh4, seed=20 + m)
        q = cases.smooth_tracers(mesh4, ntr, seed=20 + m) * gd[None, :] if ntr else None
        ics.append((gd, u, ghs, q))
        ens.select_member(m)
        ens.set_initial(gd, u, ghs)
        if ntr:
            ens.set_tracers(q)
    ens.step(7)
    for m in (0, 2, M - 1):
        one = TMCoreGPU(mesh4, **kw)
        gd, u, ghs, q = ics[m]
        one.set_initial(gd, u, ghs)
        if ntr:
            one.set_tracers(q)
        one.step(7)
        ens.select_member(m)
        ge, ie, ue = ens.get_state()
        g1, i1, u1 = one.get_state()
        assert np.array_equal(ge, g1) and np.array_equal(ie, i1), m
        assert np.array_equal(ens.diag(), one.diag()), m
        if ntr:
            assert np.array_equal(ens.get_tracers(), one.get_tracers())
        one.close()
    ens.close()


def test_member_selection_bounds(mesh3):
    from tmcore_gb300.gpu import TMCError, TMCoreGPU

    ens = TMCoreGPU(mesh3, dt=600.0, precision=1, members=3)
    with pytest.raises(TMCError):
        ens.select_member(3)
    with pytest.raises(TMCError):
        ens.spatial_operators(np.ones(mesh3.nCells), np.ones(mesh3.nEdges))
    ens.close()
    with pytest.raises(TMCError):  # FP64 ensembles are not built
        TMCoreGPU(mesh3, dt=600.0, precision=0, members=3)


@pytest.mark.parametrize("members", [1, 6])
def test_autotune_keeps_state_and_results(mesh5, members):
    from tmcore_gb300.gpu import TMCoreGPU

    kw = dict(dt=300.0, precision=1, pv_scheme=1, apvm_weight=0.0, members=members)
    a, b = TMCoreGPU(mesh5, **kw), TMCoreGPU(mesh5, **kw)
    for m in range(members):
        gd, u, ghs = _ic(mesh5, seed=40 + m)
        for x in (a, b):
            x.select_member(m)
            x.set_initial(gd, u, ghs)
    before = a.get_state()
    sizes = a.autotune(steps=2)
    assert all(s in (64, 128, 192, 256, 384, 512) for s in sizes.values())
    if members > 1:
        assert max(sizes.values()) <= 256
    after = a.get_state()
    assert all(np.array_equal(x, y) for x, y in zip(before, after))
    a.step(10)
    b.step(10)
    for m in range(members):
        a.select_member(m)
        b.select_member(m)
        ga, _, ua = a.get_state()
        gb, _, ub = b.get_state()
        # only beta's block partition changes with the block sizes
        assert np.max(np.abs(ga - gb)) / np.max(np.abs(gb)) < 1e-6
        assert np.all(np.isfinite(ua))
    a.close()
    b.close()


def test_group_of_levels_matches_separate_runs(mesh3, mesh4):
    """A mixed batch (two mesh levels, dt = 600 / 300 s, ensembles of 2):
    one graph per 600-s cycle equals stepping each model on its own."""
    from tmcore_gb300.gpu import TMCoreGPU, TMCoreGroup

    spec = [(mesh3, 600.0), (mesh4, 300.0)]
    grouped, alone = [], []
    for mesh, dt in spec:
        kw = dict(dt=dt, precision=1, pv_scheme=1, apvm_weight=0.0, members=2)
        g, a = TMCoreGPU(mesh, **kw), TMCoreGPU(mesh, **kw)
        for m in range(2):
            gd, u, ghs = _ic(mesh, seed=60 + m)
            for x in (g, a):
                x.select_member(m)
                x.set_initial(gd, u, ghs)
        grouped.append(g)
        alone.append(a)
    grp = TMCoreGroup(grouped, cycle_seconds=600.0)
    grp.run(3)
    for (mesh, dt), g, a in zip(spec, grouped, alone):
        a.step(int(3 * 600.0 / dt))
        for m in range(2):
            g.select_member(m)
            a.select_member(m)
            sg, sa = g.get_state(), a.get_state()
            assert all(np.array_equal(x, y) for x, y in zip(sg, sa))
    grp.close()
    for x in grouped + alone:
        x.close()
