"""Generated MPAS meshes: topology, geometry and TRiSK weight identities."""
import numpy as np
import pytest

from conftest import icos


@pytest.mark.parametrize("level", [0, 1, 2, 3, 4])
def test_counts_and_euler(level):
    m = icos(level)
    nc, ne, nv = m.nCells, m.nEdges, m.nVertices
    assert nc == 10 * 4 ** level + 2
    assert ne == 3 * (nc - 2) and nv == 2 * (nc - 2)
    # Euler characteristic (sphere_geometry_mod.F90:45-59): V - E + F = 2
    assert nc - ne + nv == 2
    assert np.sum(m.nEdgesOnCell == 5) == 12
    assert np.all(m.nEdgesOnEdge == m.nEdgesOnCell[m.cellsOnEdge[:, 0] - 1] + m.nEdgesOnCell[m.cellsOnEdge[:, 1] - 1] - 2)


@pytest.mark.parametrize("level", [2, 4])
def test_areas(level):
    m = icos(level)
    assert abs(m.areaCell.sum() / (4 * np.pi) - 1) < 1e-13
    assert abs(m.areaTriangle.sum() / (4 * np.pi) - 1) < 1e-13
    assert np.all(m.kiteAreasOnVertex > 0)
    assert np.allclose(m.kiteAreasOnVertex.sum(1), m.areaTriangle, rtol=1e-14)
    assert np.all(m.dvEdge > 0) and np.all(m.dcEdge > 0)


def test_connectivity_consistency():
    m = icos(3)
    # edgesOnCell(i,c) is the edge shared with cellsOnCell(i,c) (poly_fit_mod.F90:156-160, :233-245)
    for c in range(m.nCells):
        for i in range(m.nEdgesOnCell[c]):
            e = m.edgesOnCell[c, i] - 1
            assert set(m.cellsOnEdge[e]) == {c + 1, m.cellsOnCell[c, i]}
    # each edge joins verticesOnCell(i) and verticesOnCell(i+1)
    for c in range(m.nCells):
        n = m.nEdgesOnCell[c]
        for i in range(n):
            e = m.edgesOnCell[c, i] - 1
            assert set(m.verticesOnEdge[e]) == {m.verticesOnCell[c, i], m.verticesOnCell[c, (i + 1) % n]}


def test_orientation():
    """normal from cellsOnEdge(1) to (2); tangent k x n from verticesOnEdge(1) to (2)."""
    m = icos(3)
    xc = np.stack([m.xCell, m.yCell, m.zCell], 1)
    xv = np.stack([m.xVertex, m.yVertex, m.zVertex], 1)
    xe = np.stack([m.xEdge, m.yEdge, m.zEdge], 1)
    n = xc[m.cellsOnEdge[:, 1] - 1] - xc[m.cellsOnEdge[:, 0] - 1]
    t = np.cross(xe, n)
    d = xv[m.verticesOnEdge[:, 1] - 1] - xv[m.verticesOnEdge[:, 0] - 1]
    assert np.all(np.sum(t * d, 1) > 0)


def test_trisk_antisymmetry():
    """areaEdge(e) w(e,e') = -areaEdge(e') w(e',e): the zero-work property of q.F_perp."""
    m = icos(3)
    ae = m.dvEdge * m.dcEdge
    eoe, w, n = m.edgesOnEdge - 1, m.weightsOnEdge, m.nEdgesOnEdge
    wmax = np.abs(w).max()
    for e in range(m.nEdges):
        for j in range(n[e]):
            ep = eoe[e, j]
            k = list(eoe[ep, :n[ep]]).index(e)
            assert abs(ae[e] * w[e, j] + ae[ep] * w[ep, k]) <= 1e-14 * ae[e] * wmax


def test_trisk_tangent_reconstruction_converges():
    errs = []
    for level in (2, 3, 4):
        m = icos(level)
        xe = np.stack([m.xEdge, m.yEdge, m.zEdge], 1)
        xc = np.stack([m.xCell, m.yCell, m.zCell], 1)
        n = xc[m.cellsOnEdge[:, 1] - 1] - xc[m.cellsOnEdge[:, 0] - 1]
        n -= np.sum(n * xe, 1)[:, None] * xe
        n /= np.linalg.norm(n, axis=1)[:, None]
        t = np.cross(xe, n)
        vel = np.stack([-xe[:, 1], xe[:, 0], 0 * xe[:, 0]], 1) + 0.3 * np.stack([0 * xe[:, 0], -xe[:, 2], xe[:, 1]], 1)
        un, ut = np.sum(vel * n, 1), np.sum(vel * t, 1)
        eoe = m.edgesOnEdge - 1
        rec = np.sum(m.weightsOnEdge * np.where(eoe >= 0, un[np.clip(eoe, 0, None)], 0.0), 1)
        errs.append(np.abs(rec - ut).max() / np.abs(ut).max())
    assert errs[0] > errs[1] > errs[2]
    assert errs[2] < 0.02


def test_netcdf_roundtrip(tmp_path):
    from tmcore_gb300 import mesh

    m = icos(2)
    p = tmp_path / "x1.162.grid.nc"
    m.write(str(p))
    r = mesh.read_mpas(str(p))
    assert r.dims == m.dims
    for k in ("edgesOnEdge", "weightsOnEdge", "kiteAreasOnVertex", "cellsOnEdge", "dvEdge", "latVertex"):
        assert np.array_equal(r.vars[k], m.vars[k]), k
