"""Coarse-graining of a fine-mesh state onto a coarser mesh (closure training
data and held-out truth).  CPU: the maps (built without CUDA) reproduce
smooth fields within bounds set by the coarse resolution.  GPU: the device
gathers apply exactly those maps, and the cell map is a nearest-generator
map (checked with a k-d tree)."""
import numpy as np
import pytest


def _unit(a):
    return a / np.linalg.norm(a, axis=-1, keepdims=True)


def _pts(m, kind):
    return _unit(np.stack([m.vars["x" + kind], m.vars["y" + kind], m.vars["z" + kind]], 1))


def _normals(m):
    xc, xe = _pts(m, "Cell"), _pts(m, "Edge")
    c = m.vars["cellsOnEdge"] - 1
    d = xc[c[:, 1]] - xc[c[:, 0]]
    d -= np.sum(d * xe, 1, keepdims=True) * xe
    return _unit(d)


def _wind(x):
    """A solid-body rotation about a tilted axis plus a non-divergent wave."""
    axis = _unit(np.array([0.3, -0.2, 1.0]))
    g = np.stack([2 * x[:, 0] * x[:, 2], np.zeros(len(x)), x[:, 0] ** 2], 1)
    g -= np.sum(g * x, 1, keepdims=True) * x
    return np.cross(axis, x) + 0.5 * np.cross(x, g)


def _scalar(x):
    return x[:, 0] ** 2 + 0.5 * x[:, 1] * x[:, 2] + x[:, 2]


def _apply(rows, x):
    start, idx, w = rows
    out = np.zeros(len(start) - 1)
    for i in range(len(out)):
        s = 0.0
        for k in range(start[i], start[i + 1]):
            s += w[k] * x[idx[k]]
        out[i] = s
    return out


# (fine, coarse, bound on the cell error relative to the field's spread, bound on the u error)
CASES = [(4, 3, 6e-3, 1e-2), (5, 4, 3e-3, 6e-3), (5, 3, 6e-3, 8e-3), (6, 4, 2e-3, 5e-3)]


@pytest.mark.parametrize("fl,cl,cell_tol,u_tol", CASES)
def test_maps_reproduce_smooth_fields(fl, cl, cell_tol, u_tol):
    from conftest import icos
    from tmcore_gb300.gpu import Coarsener

    f, c = icos(fl), icos(cl)
    cg = Coarsener(f, c, device=-1)  # maps only: no CUDA
    assert cg.unmatched() == 0
    cells, u, pe = cg.rows(0), cg.rows(1), cg.rows(2)
    assert np.all(np.diff(cells[0]) > 0) and np.all(np.diff(pe[0]) > 0)
    # cell rows are weighted means; edge-scalar rows are means
    assert np.allclose(np.add.reduceat(cells[2], cells[0][:-1]), 1.0, rtol=0, atol=1e-13)
    assert np.allclose(np.add.reduceat(pe[2], pe[0][:-1]), 1.0, rtol=0, atol=1e-13)
    assert np.all(cells[2] > 0)
    hc = np.add.reduceat(cells[2] * _scalar(_pts(f, "Cell"))[cells[1]], cells[0][:-1])
    ref = _scalar(_pts(c, "Cell"))
    assert np.linalg.norm(hc - ref) < cell_tol * np.linalg.norm(ref - ref.mean())
    uf = np.sum(_wind(_pts(f, "Edge")) * _normals(f), 1)
    uc = np.add.reduceat(u[2] * uf[u[1]], u[0][:-1])
    ref = np.sum(_wind(_pts(c, "Edge")) * _normals(c), 1)
    assert np.linalg.norm(uc - ref) < u_tol * np.linalg.norm(ref)
    cg.close()


def test_edge_rows_are_local():
    """A coarse edge's velocity row draws on fine edges near it only (the
    strip and the TRiSK stencils of its edges)."""
    from conftest import icos
    from tmcore_gb300.gpu import Coarsener

    f, c = icos(5), icos(3)
    cg = Coarsener(f, c, device=-1)
    start, idx, _ = cg.rows(1)
    xe_f, xe_c = _pts(f, "Edge"), _pts(c, "Edge")
    dv = np.max(c.vars["dvEdge"]) / np.linalg.norm([c.xCell[0], c.yCell[0], c.zCell[0]])
    rows = np.repeat(np.arange(c.nEdges), np.diff(start))
    ang = np.arccos(np.clip(np.sum(xe_f[idx] * xe_c[rows], 1), -1, 1))
    assert np.max(ang) < 1.5 * dv
    cg.close()


@pytest.mark.gpu
@pytest.mark.parametrize("levels", [(4, 2), (5, 3)])
def test_device_applies_the_maps(levels):
    from conftest import icos
    from tmcore_gb300.gpu import Coarsener

    fine, coarse = icos(levels[0]), icos(levels[1])
    cg = Coarsener(fine, coarse)
    rng = np.random.default_rng(0)
    gd = 5e4 + 1e3 * rng.standard_normal(fine.nCells)
    u = 20 * rng.standard_normal(fine.nEdges)
    pe = 1e-8 * rng.standard_normal(fine.nEdges)
    gc, uc, pc = cg(gd=gd, u=u, pv_edge=pe)
    for which, x, y in ((0, gd, gc), (1, u, uc), (2, pe, pc)):
        ref = _apply(cg.rows(which), x)
        assert np.max(np.abs(y - ref)) <= 1e-14 * np.max(np.abs(ref))
    c1, _, _ = cg(gd=np.full(fine.nCells, 7.0))
    assert np.allclose(c1, 7.0, rtol=1e-14)
    cg.close()


@pytest.mark.gpu
def test_cell_map_is_nearest_generator():
    from scipy.spatial import cKDTree

    from conftest import icos
    from tmcore_gb300.gpu import Coarsener

    fine, coarse = icos(5), icos(3)
    cg = Coarsener(fine, coarse)
    mp = cg.cell_map()
    pc = np.stack([coarse.xCell, coarse.yCell, coarse.zCell], 1)
    pf = np.stack([fine.xCell, fine.yCell, fine.zCell], 1)
    d, near = cKDTree(pc).query(pf)
    d_dev = np.sum((pf - pc[mp]) ** 2, 1)
    # ties (fine generators on coarse Voronoi boundaries): either one
    assert np.all(d_dev <= d ** 2 * (1 + 1e-9) + 1e-18)
    cg.close()
