"""MPAS spherical Voronoi meshes: generation, NetCDF grid files, host arrays.

The arrays follow the MPAS grid-file layout that TMCORE's ``mesh_init`` reads
(src/core/mesh_mod.F90:130-167): connectivity is int32 and 1-based, 2-D
fields are stored element-major (numpy shape ``(n, k)``, C order), which is
the Fortran ``(k, n)`` column-major array the reference reads.  Coordinates,
lengths and areas are on the unit sphere; ``mesh_init`` multiplies them by the
radius (mesh_mod.F90:205-222), and so does :func:`tmcore_gb300.model` when it
hands them to the GPU library.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

from . import _lib

# Variables mesh_init reads (mesh_mod.F90:131-167) plus a few MPAS extras.
INT_VARS_2D = {
    "cellsOnCell": ("nCells", "maxEdges"),
    "edgesOnCell": ("nCells", "maxEdges"),
    "verticesOnCell": ("nCells", "maxEdges"),
    "cellsOnEdge": ("nEdges", "TWO"),
    "verticesOnEdge": ("nEdges", "TWO"),
    "edgesOnEdge": ("nEdges", "maxEdges2"),
    "cellsOnVertex": ("nVertices", "vertexDegree"),
    "edgesOnVertex": ("nVertices", "vertexDegree"),
}
INT_VARS_1D = {"nEdgesOnCell": "nCells", "nEdgesOnEdge": "nEdges",
               "indexToCellID": "nCells", "indexToEdgeID": "nEdges", "indexToVertexID": "nVertices"}
F64_VARS_1D = {
    **{f"{a}Cell": "nCells" for a in ("x", "y", "z", "lat", "lon")},
    **{f"{a}Edge": "nEdges" for a in ("x", "y", "z", "lat", "lon")},
    **{f"{a}Vertex": "nVertices" for a in ("x", "y", "z", "lat", "lon")},
    "dcEdge": "nEdges", "dvEdge": "nEdges", "dv1Edge": "nEdges", "dv2Edge": "nEdges",
    "angleEdge": "nEdges", "areaCell": "nCells", "areaTriangle": "nVertices",
    "meshDensity": "nCells",
}
F64_VARS_2D = {
    "weightsOnEdge": ("nEdges", "maxEdges2"),
    "kiteAreasOnVertex": ("nVertices", "vertexDegree"),
}


@dataclass
class MPASMesh:
    """An MPAS grid held as host numpy arrays in grid-file layout (see module doc)."""

    dims: dict
    vars: dict = field(default_factory=dict)
    attrs: dict = field(default_factory=dict)

    def __getattr__(self, name):
        v = self.__dict__.get("vars", {})
        if name in v:
            return v[name]
        d = self.__dict__.get("dims", {})
        if name in d:
            return d[name]
        raise AttributeError(name)

    @property
    def level(self) -> int | None:
        n = self.dims["nCells"] - 2
        lev = 0
        while n > 10:
            n //= 4
            lev += 1
        return lev if 10 * 4 ** lev + 2 == self.dims["nCells"] else None

    # ------------------------------------------------------------------ I/O
    def write(self, path: str, version: int = 2) -> None:
        """Write an MPAS grid NetCDF file (version 2: CDF-2, 64-bit offsets;
        1: CDF-1, 32-bit offsets)."""
        from scipy.io import netcdf_file

        with netcdf_file(path, "w", version=version) as f:
            for k, n in self.dims.items():
                f.createDimension(k, n)
            if "TWO" not in self.dims:
                f.createDimension("TWO", 2)
            for k, v in self.attrs.items():
                setattr(f, k, v)
            for name, arr in self.vars.items():
                if name in INT_VARS_2D:
                    dd = INT_VARS_2D[name]
                elif name in INT_VARS_1D:
                    dd = (INT_VARS_1D[name],)
                elif name in F64_VARS_1D:
                    dd = (F64_VARS_1D[name],)
                elif name in F64_VARS_2D:
                    dd = F64_VARS_2D[name]
                else:
                    continue
                var = f.createVariable(name, arr.dtype, dd)
                var[...] = arr


def read_mpas(path: str) -> MPASMesh:
    """Read the variables mesh_init reads from an MPAS grid file."""
    from scipy.io import netcdf_file

    with netcdf_file(path, "r", mmap=False) as f:
        dims = {k: int(f.dimensions[k]) for k in
                ("nCells", "nEdges", "nVertices", "maxEdges", "maxEdges2", "vertexDegree")}
        vars_ = {}
        for name in list(INT_VARS_2D) + list(INT_VARS_1D) + list(F64_VARS_1D) + list(F64_VARS_2D):
            if name in f.variables:
                a = np.array(f.variables[name][...])
                want = np.int32 if (name in INT_VARS_2D or name in INT_VARS_1D) else np.float64
                vars_[name] = np.ascontiguousarray(a.astype(want, copy=False))
        attrs = {k: v for k, v in f._attributes.items()}
    return MPASMesh(dims=dims, vars=vars_, attrs=attrs)


def generate_icos(level: int, lloyd_iters: int = 20) -> MPASMesh:
    """Generate a level-``level`` icosahedral SCVT (nCells = 10*4**level + 2).

    The generator is the native ``tmc_meshgen_create`` (csrc/meshgen.cpp).
    Returned arrays use the MPAS file convention: 1-based int32 connectivity
    with 0 in unused slots, unit-sphere geometry.
    """
    lib = _lib.meshgen()
    h = ctypes.c_void_p()
    rc = lib.tmc_meshgen_create(int(level), int(lloyd_iters), ctypes.byref(h))
    if rc != 0:
        msg = lib.tmc_meshgen_error(h).decode() if h.value else "bad arguments"
        if h.value:
            lib.tmc_meshgen_destroy(h)
        raise RuntimeError(f"tmc_meshgen_create failed ({rc}): {msg}")
    try:
        d = (ctypes.c_int32 * 6)()
        lib.tmc_meshgen_dims(h, d)
        nc, ne, nv, me, me2, vd = list(d)
        dims = dict(nCells=nc, nEdges=ne, nVertices=nv, maxEdges=me, maxEdges2=me2, vertexDegree=vd)
        vars_: dict[str, np.ndarray] = {}
        shapes = {"nCells": nc, "nEdges": ne, "nVertices": nv, "maxEdges": me,
                  "maxEdges2": me2, "vertexDegree": vd, "TWO": 2}
        for name, dd in INT_VARS_2D.items():
            a = np.empty((shapes[dd[0]], shapes[dd[1]]), np.int32)
            n = lib.tmc_meshgen_get_i32(h, name.encode(), a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
            assert n == a.size, name
            vars_[name] = a + 1  # 0-based -> 1-based; unused slots (-1) become 0
        for name in ("nEdgesOnCell", "nEdgesOnEdge"):
            a = np.empty(shapes[INT_VARS_1D[name]], np.int32)
            n = lib.tmc_meshgen_get_i32(h, name.encode(), a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
            assert n == a.size, name
            vars_[name] = a
        for name, dim in F64_VARS_1D.items():
            a = np.empty(shapes[dim], np.float64)
            n = lib.tmc_meshgen_get_f64(h, name.encode(), a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
            assert n == a.size, name
            vars_[name] = a
        for name, dd in F64_VARS_2D.items():
            a = np.empty((shapes[dd[0]], shapes[dd[1]]), np.float64)
            n = lib.tmc_meshgen_get_f64(h, name.encode(), a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
            assert n == a.size, name
            vars_[name] = a
        vars_["indexToCellID"] = np.arange(1, nc + 1, dtype=np.int32)
        vars_["indexToEdgeID"] = np.arange(1, ne + 1, dtype=np.int32)
        vars_["indexToVertexID"] = np.arange(1, nv + 1, dtype=np.int32)
    finally:
        lib.tmc_meshgen_destroy(h)
    attrs = {"on_a_sphere": b"YES", "sphere_radius": 1.0, "mesh_spec": b"1.0",
             "source": b"tmcore_gb300 icosahedral SCVT generator",
             "icosahedral_level": int(level), "lloyd_iterations": int(lloyd_iters)}
    return MPASMesh(dims=dims, vars=vars_, attrs=attrs)


_CACHE: dict = {}


def icos_mesh(level: int, lloyd_iters: int = 20, cache_dir: str | None = None) -> MPASMesh:
    """Generated mesh with an in-process cache and an optional on-disk cache."""
    key = (int(level), int(lloyd_iters))
    if key in _CACHE:
        return _CACHE[key]
    m = None
    if cache_dir:
        p = os.path.join(cache_dir, f"x1.{10 * 4 ** level + 2}.L{level}.it{lloyd_iters}.grid.nc")
        if os.path.exists(p):
            m = read_mpas(p)
    if m is None:
        m = generate_icos(level, lloyd_iters)
        if cache_dir:
            os.makedirs(cache_dir, exist_ok=True)
            m.write(os.path.join(cache_dir, f"x1.{m.nCells}.L{level}.it{lloyd_iters}.grid.nc"))
    _CACHE[key] = m
    return m
