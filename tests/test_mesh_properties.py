"""Property tests of the mesh generator (hypothesis): for any refinement
level and any number of Lloyd iterations the generated MPAS mesh keeps its
topology (Euler characteristic, 12 pentagons), its geometry (cell and
triangle areas tiling the sphere, positive kites and lengths), the MPAS
orientation conventions, and the TRiSK weights' antisymmetry
areaEdge(e) w(e,e') = -areaEdge(e') w(e',e) (the zero-work property of
q.F_perp)."""
import numpy as np
import pytest

pytest.importorskip("hypothesis")

from hypothesis import given, settings, strategies as st  # noqa: E402


@settings(max_examples=15, deadline=None, derandomize=True)
@given(level=st.integers(min_value=0, max_value=3), iters=st.integers(min_value=0, max_value=40))
def test_mesh_identities_for_any_lloyd_iterations(level, iters):
    from tmcore_gb300 import mesh

    m = mesh.generate_icos(level, iters)
    nc, ne, nv = m.nCells, m.nEdges, m.nVertices
    assert nc == 10 * 4 ** level + 2 and nc - ne + nv == 2
    assert np.sum(m.nEdgesOnCell == 5) == 12
    assert abs(m.areaCell.sum() / (4 * np.pi) - 1) < 1e-13
    assert abs(m.areaTriangle.sum() / (4 * np.pi) - 1) < 1e-13
    assert np.all(m.kiteAreasOnVertex > 0) and np.all(m.dvEdge > 0) and np.all(m.dcEdge > 0)
    xc = np.stack([m.xCell, m.yCell, m.zCell], 1)
    xv = np.stack([m.xVertex, m.yVertex, m.zVertex], 1)
    xe = np.stack([m.xEdge, m.yEdge, m.zEdge], 1)
    n = xc[m.cellsOnEdge[:, 1] - 1] - xc[m.cellsOnEdge[:, 0] - 1]
    d = xv[m.verticesOnEdge[:, 1] - 1] - xv[m.verticesOnEdge[:, 0] - 1]
    assert np.all(np.sum(np.cross(xe, n) * d, 1) > 0)  # tangent k x n from vertex 1 to 2
    ae = m.dvEdge * m.dcEdge
    eoe, w, cnt = m.edgesOnEdge - 1, m.weightsOnEdge, m.nEdgesOnEdge
    wmax = np.abs(w).max()
    for e in range(ne):
        for j in range(cnt[e]):
            ep = eoe[e, j]
            k = list(eoe[ep, :cnt[ep]]).index(e)
            assert abs(ae[e] * w[e, j] + ae[ep] * w[ep, k]) <= 1e-13 * ae[e] * wmax
