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
    net, losses, sc = closure.train(X, Y, steps=150, batch=1920, lr=3e-3, head=0)
    assert losses[-10:].mean() < 0.7 * losses[:3].mean()
    net.close()


def test_training_data_from_an_fp32_ensemble():
    """The training runs as one member-innermost FP32 ensemble (16 runs): the
    run-0 samples agree with the FP64 run of the same seed to far below the
    residual's size (FP32 edge state, double-float gd), and a kept fraction of
    edges gives that many rows per sample."""
    from tmcore_gb300 import closure

    kw = dict(fine_level=4, coarse_level=3, days=0.25, samples_per_run=2)
    X64, Y64 = closure.training_data(runs=1, **kw)
    X32, Y32 = closure.training_data(runs=16, truth="fp32", **kw)
    ne = 1920
    assert X32.shape == (2 * 16 * ne, 24) and np.all(np.isfinite(X32)) and np.all(np.isfinite(Y32))
    for s in range(2):  # FP64 rows: run-major; FP32 rows: sample-major
        y64, y32 = Y64[s * ne:(s + 1) * ne], Y32[s * 16 * ne:s * 16 * ne + ne]
        assert np.linalg.norm(y32 - y64) < 1e-2 * np.linalg.norm(y64), np.linalg.norm(y32 - y64) / np.linalg.norm(y64)
        x64, x32 = X64[s * ne:(s + 1) * ne], X32[s * 16 * ne:s * 16 * ne + ne]
        assert np.max(np.abs(x32 - x64) / (np.std(x64, 0) + 1e-30)) < 1e-2
    Xh, Yh = closure.training_data(runs=16, truth="fp32", edge_frac=0.25, **kw)
    assert Xh.shape == (2 * 16 * (ne // 4), 24) and np.all(np.isfinite(Yh))


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


def test_trained_closure_on_held_out_seeds():
    """Level-6 FP64 runs coarse-grained to level 4 train the network with
    both output heads; one day on 8 held-out seeds, scored against the
    coarse-grained level-6 truth.  The unconstrained head (0) and the sign
    head (2, the default: the correction kept only where it removes potential
    enstrophy) lower the u error of level 4 without them and keep h; the APVM
    head (1, a learned non-negative APVM weight) is no worse than level 4
    without it.  The plain level-5 run, scored the same way, is more
    accurate than plain level 4 (the comparison itself is sound)."""
    from tmcore_gb300 import closure

    X, Y = closure.training_data(fine_level=6, coarse_level=4, runs=8, days=2.0, samples_per_run=16)
    for head in (0, 1, 2):
        net, losses, _ = closure.train(X, Y, steps=1500, head=head, dt=closure.level_dt(4))
        assert np.mean(losses[-20:]) < 0.9 * losses[0]
        r = closure.evaluate(net, fine_level=6, coarse_level=4, members=8, days=1.0, samples=1, apvm_weight=0.0)
        e = {k: (v["h"][0], v["u"][0]) for k, v in r["error"].items()}
        assert not r["closure_timed_out"]
        for k in ("closure", "closure_stage1"):
            if head in (0, 2):
                assert e[k][1] < 0.99 * e["plain"][1], e
                assert e[k][0] < 1.002 * e["plain"][0], e
            else:
                assert e[k][1] <= 1.001 * e["plain"][1], e
                assert e[k][0] <= 1.001 * e["plain"][0], e
        assert e["plain_finer"][0] < e["plain"][0] and e["plain_finer"][1] < e["plain"][1]
        net.close()


# ---------------------------------------------------------------------------
# The APVM head (tmc_mlp_set_head(n, 1, dt)): the network predicts a
# non-negative per-edge APVM weight, and the correction added to pv_edge is
# -softplus(y) dt (v dq/dt + u dq/dn) (operators_mod.F90:296-316 with a
# learned weight).  Mass and energy hold by construction; potential enstrophy
# can only be removed.
# ---------------------------------------------------------------------------
def _apvm_net(dt, feats, seed=11, head=1, frac=0.01):
    from tmcore_gb300.gpu import ClosureMLP

    net = ClosureMLP(seed=seed)
    xs = feats.std(0).astype(np.float64)
    xs[xs == 0] = 1.0
    # head 2's correction is y * y_scale: a fraction of pv's spread
    ys = frac * float(np.std(feats[:, 3])) if head == 2 else 1.0
    net.set_scaling(feats.mean(0), 1.0 / xs, ys)
    net.set_head(head, dt)
    return net


def _numpy_apvm_correction(net, feats, dt, head=1, ys=1.0):
    """The network on the features, in numpy with its BF16 roundings, then the head."""
    from mlp_model import forward_np

    xs = feats.std(0).astype(np.float64)
    xs[xs == 0] = 1.0
    xn = ((feats - feats.mean(0).astype(np.float32)) * (1.0 / xs).astype(np.float32)).astype(np.float32)
    y, _, _ = forward_np(net.params, xn, round_act=True)
    f = feats.astype(np.float64)
    if head == 2:
        return np.where(y * f[:, 1] * f[:, 22] <= 0.0, y * ys, 0.0)
    return -np.logaddexp(0.0, y) * dt * (f[:, 1] * f[:, 22] + f[:, 0] * f[:, 23])


@pytest.mark.parametrize("layout,members,head", [(0, 1, 1), (1, 16, 1), (0, 1, 2), (1, 16, 2)])
def test_apvm_head_correction_matches_numpy(mesh4, layout, members, head):
    """The correction k_closure adds to pv_edge in the step equals the network
    evaluated in numpy on the exported features (BF16 tolerance), in both
    member layouts, for the APVM head (1) and the sign head (2)."""
    from tmcore_gb300.gpu import TMCoreGPU

    g = TMCoreGPU(mesh4, members=members, member_layout=layout, **KW)
    for k in range(members):
        gd, u, ghs = _ic(mesh4, 100 + k)
        g.select_member(k)
        g.set_initial(gd, u, ghs)
    g.step(3)
    m = members - 1
    g.select_member(m)
    feats, _ = g.closure_features()
    net = _apvm_net(KW["dt"], feats, head=head)
    g.set_closure(net)
    g.set_closure_stages(False)
    g.step(1)
    g.select_member(m)
    dq = g.closure_correction()
    ys = 0.01 * float(np.std(feats[:, 3])) if head == 2 else 1.0
    ref = _numpy_apvm_correction(net, feats, KW["dt"], head, ys)
    scale = np.max(np.abs(ref))
    assert scale > 0 and np.all(np.isfinite(dq))
    if head == 2:
        # BF16 roundings may flip y's sign where y is near 0 (both sides near 0 there)
        assert np.max(np.abs(dq - ref)) < 5e-2 * scale, np.max(np.abs(dq - ref)) / scale
        assert np.mean(dq == 0.0) > 0.05 and np.mean(dq != 0.0) > 0.05  # both branches taken
    else:
        assert np.max(np.abs(dq - ref)) < 3e-2 * scale, np.max(np.abs(dq - ref)) / scale
    assert np.sqrt(np.mean((dq - ref) ** 2)) < 1e-2 * np.sqrt(np.mean(ref ** 2))
    # the head's sign: never against APVM's direction
    d = (feats[:, 1] * feats[:, 22]) if head == 2 else (feats[:, 1] * feats[:, 22] + feats[:, 0] * feats[:, 23])
    assert np.all(dq * d <= 0.0)
    g.close()
    net.close()


@pytest.mark.parametrize("head", [1, 2])
def test_apvm_head_conserves_mass_energy_and_dissipates_enstrophy(mesh4, head):
    """50 FP32 steps with a nonzero correction of the APVM head (1) or the
    sign head (2) in every stage: mass stays within 1e-13, energy drifts no
    more than the plain run's (beta and the energy-conserving q.F_perp form),
    and potential enstrophy is never above the plain run's after any step."""
    from tmcore_gb300.gpu import TMCoreGPU

    gd, u, ghs = _ic(mesh4, 120)
    kw = dict(KW, diag_every=1)
    a, b = TMCoreGPU(mesh4, **kw), TMCoreGPU(mesh4, **kw)
    for m in (a, b):
        m.set_initial(gd, u, ghs)
    feats, _ = a.closure_features()
    # head 2: corrections of 0.2% of pv's spread, about the size of trained ones
    net = _apvm_net(KW["dt"], feats, seed=12, head=head, frac=0.002)
    a.set_closure(net)
    d0a, d0b = a.diag(), b.diag()
    moved = 0.0
    for _ in range(50):
        a.step(1)
        b.step(1)
        da, db = a.diag(), b.diag()
        assert da[2] <= db[2] * (1.0 + 1e-12), (da[2], db[2])
        moved = max(moved, abs(da[2] - db[2]) / db[2])
    assert moved > 1e-7  # the correction did act
    assert abs(da[0] - d0a[0]) / d0a[0] < 1e-13
    drift_a = abs(da[1] - d0a[1]) / d0a[1]
    drift_b = abs(db[1] - d0b[1]) / d0b[1]
    assert drift_a <= max(10.0 * drift_b, 1e-11), (drift_a, drift_b)
    assert not a.closure_status()
    a.close()
    b.close()
    net.close()
