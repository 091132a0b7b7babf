"""The per-member invariant-drift fallback (tmcore_gb300.closure.FallbackMonitor)
as host logic, on a fake ensemble (no GPU): the failure is made on the host,
as a member whose energy drifts or whose invariants stop being finite."""
import numpy as np

from conftest import ROOT  # noqa: F401  (puts the repository root on sys.path)


class FakeEnsemble:
    """The calls FallbackMonitor makes on a TMCoreGPU ensemble.  Member m's
    state is a number that counts its steps; its energy drifts from 1 by
    rate[m] per step (or turns NaN from step nan_at[m] on)."""

    def __init__(self, members, rate, nan_at=None):
        self.members = members
        self.rate = np.asarray(rate, float)
        self.nan_at = nan_at or {}
        self.steps = np.zeros(members)  # the "state" of each member
        self.closure_on = np.ones(members, bool)
        self.cur = 0
        self.calls = []

    def diag_all(self):
        d = np.zeros((self.members, 5))
        d[:, 0] = 1e3  # mass, conserved
        d[:, 1] = 1.0 + self.rate * self.steps
        for m, s in self.nan_at.items():
            if self.steps[m] >= s:
                d[m, 1] = np.nan
        d[:, 4] = 1.0
        return d

    def step(self, n):
        self.steps += n
        self.calls.append(("step", n))

    def select_member(self, m):
        self.cur = m

    def get_state(self, with_u=False):
        return (np.array([self.steps[self.cur]]), np.array([0.0]))

    def set_state(self, gd, iap):
        self.steps[self.cur] = gd[0]
        self.calls.append(("set_state", self.cur, float(gd[0])))

    def set_member_closure(self, m, on):
        self.closure_on[m] = bool(on)


def test_drifting_member_switched_off_and_rolled_back():
    from tmcore_gb300.closure import FallbackMonitor

    # member 1 drifts 1e-5 per step: past 1e-3 after step 100, first seen at the check of step 104
    ens = FakeEnsemble(4, [0.0, 1e-5, 0.0, 1e-9])
    mon = FallbackMonitor(ens, 4, tol=1e-3, every=8)
    mon.step(200)
    assert mon.fallbacks == [(1, 104)]
    assert list(ens.closure_on) == [True, False, True, True]
    # rolled back to its checkpoint of the previous check (step 96), then stepped on without the closure
    assert ("set_state", 1, 96.0) in ens.calls
    assert ens.steps[1] == 96 + (200 - 104)
    assert ens.steps[0] == 200
    # the steps are taken in blocks that end at the checks
    assert all(c[1] <= 8 for c in ens.calls if c[0] == "step")
    # largest drift seen per member
    assert mon.max_drift[0] == 0.0
    assert abs(mon.max_drift[3] - 200e-9) < 1e-15
    assert mon.max_drift[1] > 1e-3


def test_non_finite_member_switched_off_once():
    from tmcore_gb300.closure import FallbackMonitor

    ens = FakeEnsemble(3, [0.0, 0.0, 0.0], nan_at={2: 30})
    mon = FallbackMonitor(ens, 3, tol=1e-3, every=10)
    mon.step(35)
    assert mon.fallbacks == [(2, 30)]
    assert ("set_state", 2, 20.0) in ens.calls
    assert not ens.closure_on[2] and ens.closure_on[:2].all()
    assert np.isinf(mon.max_drift[2])
    # a member already switched off is not switched again
    ens.nan_at = {2: 0}
    mon.step(20)
    assert mon.fallbacks == [(2, 30)]
    # its checkpoint is no longer refreshed; the others' are, at the last check (step 50)
    assert mon.ckpt[2][0][0] == 20.0 and mon.ckpt[0][0][0] == 50.0
