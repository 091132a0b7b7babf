"""The byte models bench.py divides by to report roofline fractions (no GPU):
the scope model against the figures derived from it for the level-9 and
level-6 ensemble configurations, and the internal consistency of the
pass-by-pass models."""
import pytest

from conftest import ROOT  # noqa: F401  (puts the repository root on sys.path)

L9 = (2621442, 7864320, 5242880)
L6 = (40962, 122880, 81920)
L5 = (10242, 30720, 20480)


def test_scope_model_figures():
    import bench

    def scope(nc, ne, nv, S):
        return bench.step_model_bytes(nc, ne, nv, S, 0)

    # the scope model evaluated for the roofline and parity configurations
    assert scope(*L9, 8) / 1e9 == pytest.approx(9.311, abs=1e-3)
    assert scope(*L9, 4) / 1e9 == pytest.approx(7.969, abs=1e-3)
    assert scope(*L5, 8) / 1e9 == pytest.approx(0.0364, abs=1e-4)
    assert bench.ensemble_model_bytes(*L6, 4, 512) / 1e9 == pytest.approx(10.84, abs=1e-2)
    # one member sharing the mesh is the single model
    assert bench.ensemble_model_bytes(*L6, 4, 1) == pytest.approx(scope(*L6, 4))


def test_pass_models_are_consistent():
    import bench

    for S, ntr in ((4, 4), (8, 0), (4, 0)):
        b = bench.pass_bytes(*L9, S, ntr)
        assert set(b) == {"cell", "vertex", "edge_pv", "edge_flux", "final"}
        assert all(v > 0 for v in b.values())
        assert bench.step_bytes(*L9, S, ntr) == pytest.approx(
            4 * (b["cell"] + b["vertex"] + b["edge_pv"] + b["edge_flux"]) + b["final"])
    # tracers and FP64 state add bytes
    assert bench.step_bytes(*L9, 4, 4) > bench.step_bytes(*L9, 4, 0)
    assert bench.step_bytes(*L9, 8, 0) > bench.step_bytes(*L9, 4, 0)
    # member-innermost ensembles: the mesh once per pass, state per member
    p1 = bench.inner_ensemble_pass_bytes(*L6, 1)
    p2 = bench.inner_ensemble_pass_bytes(*L6, 2)
    p512 = bench.inner_ensemble_pass_bytes(*L6, 512)
    for k in p1:
        per_member = p2[k] - p1[k]
        assert per_member > 0
        assert p512[k] == pytest.approx(p1[k] + 511 * per_member)
    assert bench.inner_ensemble_step_bytes(*L6, 512) / 1e9 == pytest.approx(23.35, abs=0.01)
