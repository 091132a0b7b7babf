"""The ordering autotuner (tmcore_gb300.tune.autotune_ordering) as host logic,
on a fake handle (no GPU): every (member layout, element order) candidate is
built with the same parameters, a refused candidate is recorded with its
error, and the fastest one is returned."""
import pytest

from conftest import ROOT  # noqa: F401  (puts the repository root on sys.path)


def test_autotune_ordering_picks_the_fastest(monkeypatch):
    from tmcore_gb300 import tune
    from tmcore_gb300.gpu import TMCError

    # ms per step of each candidate; layout 1 with Morton order is refused
    cost = {(1, 1): 5.0, (1, 2): None, (1, 0): 5.5, (0, 1): 9.0, (0, 2): 4.0, (0, 0): 9.5}
    made, closed = [], []

    class FakeHandle:
        def __init__(self, mesh, **kw):
            key = (kw["member_layout"], kw["renumber"])
            if cost[key] is None:
                raise TMCError(-4, "member_layout 1 refuses this")
            self.key, self.kw, self.states = key, kw, []
            made.append(kw)

        def select_member(self, m):
            self.m = m

        def set_initial(self, gd, u, ghs):
            self.states.append((self.m, gd))

        def autotune(self, steps):
            return {"cell": 128}

        def step(self, n):
            pass

        def synchronize(self):
            pass

        def time_steps(self, n, total=True, flux=False):
            assert len(self.states) == 2  # every member set before timing
            return cost[self.key] * n, None, None, 40 * n

        def close(self):
            closed.append(self.key)

    monkeypatch.setattr(tune, "TMCoreGPU", FakeHandle)
    ics = [("gd0", "u0", "ghs0"), ("gd1", "u1", "ghs1")]
    best, timings = tune.autotune_ordering("mesh", ics, steps=3, dt=300.0, precision=1)
    assert best == {"dt": 300.0, "precision": 1, "members": 2, "renumber": 2, "member_layout": 0, "member_lanes": 0}
    assert len(timings) == 6
    refused = [(t["member_layout"], t["renumber"]) for t in timings if "error" in t]
    assert refused == [(1, 2)]
    assert {t["renumber"]: t["ms_per_step"] for t in timings if t.get("member_layout") == 0} == {1: 9.0, 2: 4.0, 0: 9.5}
    # every candidate built with the caller's parameters, and closed
    assert all(k["dt"] == 300.0 and k["members"] == 2 for k in made)
    assert sorted(closed) == sorted(k for k, v in cost.items() if v is not None)


def test_autotune_ordering_single_model_and_nothing_buildable(monkeypatch):
    from tmcore_gb300 import tune
    from tmcore_gb300.gpu import TMCError

    layouts = []

    class Refuses:
        def __init__(self, mesh, **kw):
            layouts.append(kw["member_layout"])
            raise TMCError(-4, "no")

    monkeypatch.setattr(tune, "TMCoreGPU", Refuses)
    with pytest.raises(TMCError):
        tune.autotune_ordering("mesh", [("gd", "u", "ghs")], dt=300.0)
    # one member: only member_layout 0 is tried, in every element order
    assert layouts == [0, 0, 0]


def test_lane_layouts():
    """member_layout 1's lane layouts (the library's lanes_for rule) and the
    distinct ones the autotuner times."""
    from tmcore_gb300 import tune

    assert tune.lane_layout(16, 0) == (1, 16) and tune.lane_layout(16, 8) == (2, 8)
    assert tune.lane_layout(16, 32) is None and tune.lane_layout(48, 32) is None
    assert tune.lane_layout(512, 0) == (2, 32) and tune.lane_layout(96, 16) == (2, 16)
    assert tune.lane_layout(32, 0) == (1, 32) and tune.lane_layout(32, 12) is None
    assert tune.lane_candidates(16) == [0, 8]
    assert tune.lane_candidates(48) == [0, 8]
    assert tune.lane_candidates(32) == [0, 8, 16]
    assert tune.lane_candidates(512) == [0, 8, 16]
