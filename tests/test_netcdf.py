"""The library's NetCDF-classic MPAS grid reader and writer (no GPU needed),
against scipy's reader and writer."""
import os

import numpy as np
import pytest


def _same(a, b):
    return a.shape == b.shape and np.array_equal(np.asarray(a), np.asarray(b))


def test_write_then_read_both_ways(tmp_path):
    from conftest import icos
    from tmcore_gb300 import mesh
    from tmcore_gb300.gpu import read_mesh_file, write_mesh_file

    m = icos(3)
    p = os.path.join(tmp_path, "x1.642.grid.nc")
    write_mesh_file(p, m)
    a = mesh.read_mpas(p)        # scipy reads the library's file
    b = read_mesh_file(p)        # the library reads its own file
    for k in ("nCells", "nEdges", "nVertices", "maxEdges", "maxEdges2", "vertexDegree"):
        assert a.dims[k] == m.dims[k] == b.dims[k]
    for name in ("cellsOnEdge", "edgesOnEdge", "weightsOnEdge", "kiteAreasOnVertex", "xCell", "lonVertex",
                 "areaTriangle", "nEdgesOnCell"):
        ref = np.asarray(m.vars[name])
        assert np.array_equal(np.asarray(a.vars[name]).reshape(ref.shape), ref), name
        assert np.array_equal(np.asarray(b.vars[name]).reshape(ref.shape), ref), name


@pytest.mark.parametrize("version", [1, 2])
def test_reads_a_scipy_written_file(tmp_path, version):
    """CDF-1 (32-bit offsets) and CDF-2 (64-bit offsets) files from scipy."""
    from conftest import icos
    from tmcore_gb300.gpu import read_mesh_file

    m = icos(2)
    p = os.path.join(tmp_path, "x1.162.grid.nc")
    m.write(p, version=version)
    with open(p, "rb") as f:
        assert f.read(4) == b"CDF" + bytes([version])
    b = read_mesh_file(p)
    for name in ("verticesOnEdge", "cellsOnVertex", "dvEdge", "latCell", "zVertex", "weightsOnEdge",
                 "kiteAreasOnVertex", "nEdgesOnCell"):
        ref = np.asarray(m.vars[name])
        assert np.array_equal(np.asarray(b.vars[name]).reshape(ref.shape), ref), name
