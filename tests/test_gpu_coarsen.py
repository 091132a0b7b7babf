"""Coarse-graining of a fine-mesh state onto a coarser mesh (closure training
data): the device maps against a numpy restatement with a k-d tree."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cell_map(fine, coarse):
    """Nearest coarse generator of each fine cell, and whether the second
    nearest is as near to round-off (refined icosahedral meshes put fine
    generators on coarse Voronoi boundaries, where either choice is right)."""
    from scipy.spatial import cKDTree

    pc = np.stack([coarse.xCell, coarse.yCell, coarse.zCell], 1)
    pf = np.stack([fine.xCell, fine.yCell, fine.zCell], 1)
    d, i = cKDTree(pc).query(pf, k=2)
    return i[:, 0], (d[:, 1] - d[:, 0]) < 1e-9 * d[:, 1]


@pytest.mark.parametrize("levels", [(4, 2), (5, 3)])
def test_cells_match_numpy_and_conserve_mass(levels):
    from conftest import icos
    from tmcore_gb300.gpu import Coarsener

    fine, coarse = icos(levels[0]), icos(levels[1])
    cg = Coarsener(fine, coarse)
    assert cg.unmatched() == 0
    rng = np.random.default_rng(0)
    gd = 5e4 + 1e3 * rng.standard_normal(fine.nCells)
    gc, _, _ = cg(gd=gd)
    mp = cg.cell_map()
    # every fine cell goes to a nearest coarse generator (ties: either one)
    pc = np.stack([coarse.xCell, coarse.yCell, coarse.zCell], 1)
    pf = np.stack([fine.xCell, fine.yCell, fine.zCell], 1)
    near, _ = _cell_map(fine, coarse)
    d_dev = np.sum((pf - pc[mp]) ** 2, 1)
    d_min = np.sum((pf - pc[near]) ** 2, 1)
    assert np.all(d_dev <= d_min * (1 + 1e-9) + 1e-18)
    A = fine.areaCell
    asum = np.bincount(mp, A, coarse.nCells)
    ref = np.bincount(mp, A * gd, coarse.nCells) / asum
    assert np.max(np.abs(gc - ref)) < 1e-12 * np.max(np.abs(ref))
    assert abs(np.sum(asum * gc) - np.sum(A * gd)) < 1e-12 * np.sum(A * gd)
    c1, _, _ = cg(gd=np.full(fine.nCells, 7.0))
    assert np.allclose(c1, 7.0, rtol=1e-14)
    cg.close()


def test_edge_flux_averaging_of_a_rotation():
    """u = -dpsi/dv telescopes along the aggregate boundary: the coarse-grained
    normal velocity of a solid-body rotation approximates the coarse one."""
    from conftest import icos
    from tmcore_gb300 import cases
    from tmcore_gb300.gpu import Coarsener

    fine, coarse = icos(5), icos(3)
    r, u0 = 6371220.0, 20.0
    uf = cases._uv_from_psi(fine, -r * u0 * np.sin(fine.latVertex), r)
    uc = cases._uv_from_psi(coarse, -r * u0 * np.sin(coarse.latVertex), r)
    cg = Coarsener(fine, coarse)
    _, ug, pe = cg(u=uf, pv_edge=np.full(fine.nEdges, 3.0))
    assert np.sqrt(np.mean((ug - uc) ** 2)) < 0.1 * np.sqrt(np.mean(uc ** 2))
    assert np.allclose(pe, 3.0, rtol=1e-14)
    cg.close()
