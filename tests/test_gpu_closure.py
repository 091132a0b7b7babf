"""The learned closure inside the FP32 step: features, a zero network that
changes nothing, the per-member switch of an ensemble, the training pipeline
and what the trained network gains over the plain method on held-out seeds."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ic(mesh, seed):
    from tmcore_gb300 import cases

    return cases.jet_bumps(mesh, seed=seed)


KW = dict(dt=600.0, precision=1, pv_scheme=1, apvm_weight=0.0)


def test_features_match_state(mesh4):
    from tmcore_gb300.gpu import TMCoreGPU

    m = mesh4
    g = TMCoreGPU(m, **KW)
    gd, u, ghs = _ic(m, 80)
    g.set_initial(gd, u, ghs)
    g.step(2)
    f, pv = g.closure_features()
    gd1, _, u1 = g.get_state()
    pvv, _ = g.get_vertex()
    c1, c2 = m.cellsOnEdge[:, 0] - 1, m.cellsOnEdge[:, 1] - 1
    v1, v2 = m.verticesOnEdge[:, 0] - 1, m.verticesOnEdge[:, 1] - 1
    r = 6371220.0
    assert np.allclose(f[:, 0], u1, rtol=1e-5, atol=1e-5 * np.max(np.abs(u1)))
    assert np.allclose(f[:, 2], 0.5 * (gd1[c1] + gd1[c2]), rtol=1e-5)
    assert np.allclose(f[:, 8], gd1[c1], rtol=1e-6) and np.allclose(f[:, 9], gd1[c2], rtol=1e-6)
    assert np.allclose(f[:, 4], pvv[v1], rtol=1e-4, atol=1e-6 * np.max(np.abs(pvv)))
    assert np.allclose(f[:, 16], m.dvEdge * r, rtol=1e-6) and np.allclose(f[:, 17], m.dcEdge * r, rtol=1e-6)
    assert np.allclose(f[:, 14], 2 * 7.292e-5 * np.sin(m.latVertex[v1]), rtol=1e-6, atol=1e-12)
    # centred pv on edges (pv_scheme 1 without APVM)
    assert np.allclose(pv, 0.5 * (pvv[v1] + pvv[v2]), rtol=1e-4, atol=1e-6 * np.max(np.abs(pvv)))
    g.close()


def test_zero_network_changes_nothing(mesh4):
    from tmcore_gb300.gpu import ClosureMLP, TMCoreGPU

    net = ClosureMLP(seed=1)
    net.params = np.zeros(9985, np.float32)
    a, b = TMCoreGPU(mesh4, **KW), TMCoreGPU(mesh4, **KW)
    gd, u, ghs = _ic(mesh4, 81)
    for x in (a, b):
        x.set_initial(gd, u, ghs)
    a.set_closure(net)
    a.step(6)
    b.step(6)
    assert not a.closure_status()
    sa, sb = a.get_state(), b.get_state()
    assert all(np.array_equal(x, y) for x, y in zip(sa, sb))
    a.close()
    b.close()
    net.close()


@pytest.mark.parametrize("every_stage", [True, False])
def test_member_switch(mesh4, every_stage):
    """Member 1 with the closure switched off evolves exactly as the plain
    model; member 0 with it on does not (network in every stage, or in stage
    1 with its output held for stages 2-4)."""
    from tmcore_gb300.gpu import ClosureMLP, TMCoreGPU

    net = ClosureMLP(seed=2)
    p = net.params
    p *= 0.5
    net.params = p
    net.set_scaling(np.zeros(24), np.ones(24), 1e-9)  # corrections of order 1e-9 (pv ~ 1e-8)
    ens = TMCoreGPU(mesh4, members=2, **KW)
    plain = TMCoreGPU(mesh4, **KW)
    gd, u, ghs = _ic(mesh4, 82)
    for k in range(2):
        ens.select_member(k)
        ens.set_initial(gd, u, ghs)
    plain.set_initial(gd, u, ghs)
    ens.set_closure(net)
    ens.set_closure_stages(every_stage)
    ens.set_member_closure(1, False)
    ens.step(6)
    plain.step(6)
    ens.select_member(1)
    s1, sp = ens.get_state(), plain.get_state()
    assert all(np.array_equal(x, y) for x, y in zip(s1, sp))
    ens.select_member(0)
    s0 = ens.get_state()
    assert not np.array_equal(s0[0], sp[0])
    assert np.all(np.isfinite(s0[0])) and np.all(np.isfinite(s0[2]))
    with pytest.raises(Exception):
        TMCoreGPU(mesh4, dt=600.0, precision=0).set_closure(net)
    ens.close()
    plain.close()
    net.close()


def test_training_data_and_training_small():
    """Level-4 FP64 runs coarse-grained to level 3: finite features, a
    non-zero PV-on-edge residual, and a loss that falls."""
    from tmcore_gb300 import closure

    X, Y = closure.training_data(fine_level=4, coarse_level=3, runs=1, days=0.25, samples_per_run=2)
    assert X.shape == (2 * 1920, 24) and Y.shape == (2 * 1920,)
    assert np.all(np.isfinite(X)) and np.all(np.isfinite(Y)) and np.std(Y) > 0
    net, losses, sc = closure.train(X, Y, steps=150, batch=1920, lr=3e-3)
    assert losses[-10:].mean() < 0.7 * losses[:3].mean()
    net.close()


def test_fallback_switches_off_a_drifting_member(mesh4):
    from tmcore_gb300.closure import FallbackMonitor
    from tmcore_gb300.gpu import ClosureMLP, TMCoreGPU

    good = ClosureMLP(seed=3)
    good.params = np.zeros(9985, np.float32)
    bad = ClosureMLP(seed=4)
    bad.set_scaling(np.zeros(24), np.ones(24), 1e-6)  # pv corrections 100x the pv itself
    for net, expect in ((good, 0), (bad, 3)):
        ens = TMCoreGPU(mesh4, members=3, diag_every=0, **KW)
        for k in range(3):
            gd, u, ghs = _ic(mesh4, 90 + k)
            ens.select_member(k)
            ens.set_initial(gd, u, ghs)
        ens.set_closure(net)
        mon = FallbackMonitor(ens, 3, tol=1e-4, every=4)
        mon.step(12)
        assert len({m for m, _ in mon.fallbacks}) == expect
        for k in range(3):
            ens.select_member(k)
            assert np.all(np.isfinite(ens.get_state()[0]))
        ens.close()
    good.close()
    bad.close()


def test_trained_closure_gains_on_held_out_seeds():
    """Level-6 FP64 runs coarse-grained to level 4 train the network; on 8
    held-out seeds, one day on level 4 with the closure (in every stage, and
    in stage 1 held for the others) has a lower u error against the
    coarse-grained level-6 truth than level 4 without it, and no higher h
    error; the plain level-5 run, scored the same way, is more accurate than
    plain level 4 (the comparison itself is sound)."""
    from tmcore_gb300 import closure

    X, Y = closure.training_data(fine_level=6, coarse_level=4, runs=8, days=2.0, samples_per_run=16)
    net, losses, _ = closure.train(X, Y, steps=1500)
    assert np.mean(losses[-20:]) < 0.5 * losses[0]
    r = closure.evaluate(net, fine_level=6, coarse_level=4, members=8, days=1.0, samples=1)
    e = {k: (v["h"][0], v["u"][0]) for k, v in r["error"].items()}
    assert not r["closure_timed_out"]
    for k in ("closure", "closure_stage1"):
        assert e[k][1] < 0.99 * e["plain"][1], e
        assert e[k][0] < 1.002 * e["plain"][0], e
    assert e["plain_finer"][0] < e["plain"][0] and e["plain_finer"][1] < e["plain"][1]
    net.close()
