"""The bounded completion waits of the tensor-core kernels, made to run out.

tmc_mlp_set_wait_limit(n, 0) gives every first wait of an MMA step a limit of
zero polls, so it gives up at once although the MMAs it waits for do
complete.  The kernel then flags the timeout, waits with the normal limit
for the MMAs it issued, frees its tensor memory and returns: no completion
is withheld and no wait is unbounded.  The host must see TMC_E_HEALTH, and
the same network and model handles must work normally once the limit is
restored (the tensor memory was released and the context is intact).

The reference has no counterpart; its errors abort the run
(time_scheme_mod.F90:60).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KW = dict(dt=600.0, precision=1, pv_scheme=1, apvm_weight=0.0)


def _net(seed=2, y_scale=1.0):
    from tmcore_gb300.gpu import ClosureMLP

    net = ClosureMLP(seed=seed)
    net.set_scaling(np.zeros(24), np.ones(24), y_scale)
    return net


def _rows(n, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, 24)).astype(np.float32)
    y = (0.3 * np.tanh(x[:, 0] * x[:, 1]) + 0.1 * x[:, 2]).astype(np.float32)
    return x, y


def test_forward_wait_timeout_then_recovery():
    from tmcore_gb300 import abi
    from tmcore_gb300.gpu import TMCError

    net = _net()
    x, _ = _rows(128 * 300)
    y0 = net.forward(x)
    net.set_wait_limit(0)
    with pytest.raises(TMCError) as e:
        net.forward(x)
    assert e.value.code == abi.TMC_E_HEALTH
    net.set_wait_limit(-1)
    y1 = net.forward(x)
    assert np.array_equal(y0, y1)
    net.close()


def test_trainer_wait_timeout_then_recovery():
    from tmcore_gb300 import abi
    from tmcore_gb300.gpu import TMCError

    net = _net(3)
    x, y = _rows(128 * 320, seed=1)
    g0, l0 = net.gradient(x, y)
    p0 = net.params.copy()
    net.set_dataset(x, y)
    net.set_wait_limit(0)
    with pytest.raises(TMCError) as e:
        net.gradient(x, y)
    assert e.value.code == abi.TMC_E_HEALTH
    with pytest.raises(TMCError) as e:
        net.train(2, batch=128 * 160)
    assert e.value.code == abi.TMC_E_HEALTH
    # a batch with an incomplete gradient is not applied
    assert np.array_equal(net.params, p0)
    net.set_wait_limit(-1)
    g1, l1 = net.gradient(x, y)  # blocks summed in a fixed order: bit-reproducible
    assert np.array_equal(g0, g1) and l0 == l1
    losses = net.train(2, batch=128 * 160)
    assert np.all(np.isfinite(losses)) and not np.array_equal(net.params, p0)
    net.close()


def test_closure_wait_timeout_in_the_step(mesh4):
    """The closure in the FP32 step: a timed-out network leaves the edges
    uncorrected and the step goes on; tmc_get_diag reports TMC_E_HEALTH once
    (reading clears the flag), and the handle steps normally afterwards."""
    from tmcore_gb300 import abi, cases
    from tmcore_gb300.gpu import TMCError, TMCoreGPU

    gd, u, ghs = cases.jet_bumps(mesh4, seed=82)
    net = _net(4, y_scale=1e-12)  # corrections far below pv (~1e-8): the run stays physical
    a, b = TMCoreGPU(mesh4, **KW), TMCoreGPU(mesh4, **KW)
    for m in (a, b):
        m.set_initial(gd, u, ghs)
    net.set_wait_limit(0)
    a.set_closure(net)
    a.step(2)
    b.step(2)
    with pytest.raises(TMCError) as e:
        a.diag()
    assert e.value.code == abi.TMC_E_HEALTH
    assert not a.closure_status()  # reported once
    # no network output reached pv_edge: the plain run's state
    assert all(np.array_equal(x, y) for x, y in zip(a.get_state(), b.get_state()))
    # tmc_time_integrate reports it too
    g0, i0, _ = a.get_state()
    with pytest.raises(TMCError) as e:
        a.time_integrate(g0, i0)
    assert e.value.code == abi.TMC_E_HEALTH
    # the limit restored: the network corrects pv_edge again, no error
    net.set_wait_limit(-1)
    a.set_closure(net)
    a.set_state(g0, i0)
    a.step(2)
    d = a.diag()
    assert np.all(np.isfinite(d)) and not a.closure_status()
    a.close()
    b.close()
    net.close()
