"""TEST INFRASTRUCTURE ONLY: ctypes front end of the C FP64 oracle.

The oracle restates TMCORE's Fortran hot path (see tmc_oracle.h for the file
and line map).  Parity is UNPINNED: the reference cannot be compiled here and
ships no golden vectors; physics-level known answers stand in (tests/).

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libtmc_oracle.so")
SRC = [os.path.join(HERE, "tmc_oracle.c")]
HDR = os.path.join(HERE, "tmc_oracle.h")
CFLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-fopenmp", "-std=c11", "-Wall"]


def build(force: bool = False) -> str:
    """Compile the oracle (gcc, no FMA contraction) into oracle/_build/."""
    os.makedirs(BUILD, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in SRC + [HDR])
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = ["gcc", *CFLAGS, "-shared", *SRC, "-o", LIB, "-lm"]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stdout)
    return LIB


_lib = None


class MeshIn(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in
                ("nCells", "nEdges", "nVertices", "maxEdges", "maxEdges2", "vertexDegree")] + \
               [(n, ctypes.c_void_p) for n in
                ("nEdgesOnCell", "nEdgesOnEdge", "cellsOnCell", "edgesOnCell", "verticesOnCell",
                 "cellsOnEdge", "verticesOnEdge", "edgesOnEdge", "cellsOnVertex", "edgesOnVertex",
                 "xCell", "yCell", "zCell", "latCell", "lonCell",
                 "xEdge", "yEdge", "zEdge", "latEdge", "lonEdge",
                 "xVertex", "yVertex", "zVertex", "latVertex", "lonVertex",
                 "dvEdge", "dcEdge", "areaCell", "areaTriangle", "kiteAreasOnVertex", "weightsOnEdge")]


class Params(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_double), ("time_scheme", ctypes.c_int32), ("pv_scheme", ctypes.c_int32),
                ("conserve_energy", ctypes.c_int32), ("flux_4th_order_correct", ctypes.c_int32),
                ("apvm_weight", ctypes.c_double), ("adv_order", ctypes.c_int32), ("adv_mono", ctypes.c_int32),
                ("interp_pv_order", ctypes.c_int32), ("radius", ctypes.c_double), ("g", ctypes.c_double),
                ("omega", ctypes.c_double), ("n_tracers", ctypes.c_int32), ("tracer_adv_order", ctypes.c_int32),
                ("tracer_adv_mono", ctypes.c_int32), ("nthreads", ctypes.c_int32)]


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        L = _lib
        vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int
        L.orc_create.restype = vp
        L.orc_create.argtypes = [ctypes.POINTER(MeshIn), ctypes.POINTER(Params)]
        L.orc_destroy.argtypes = [vp]
        L.orc_default_params.argtypes = [ctypes.POINTER(Params)]
        L.orc_error.restype = ctypes.c_char_p
        L.orc_error.argtypes = [vp]
        for n in ("orc_areaEdge", "orc_fVertex"):
            getattr(L, n).restype = dp
            getattr(L, n).argtypes = [vp]
        for n in ("orc_nSignEdge", "orc_tSignEdge"):
            getattr(L, n).restype = ctypes.POINTER(ctypes.c_int32)
            getattr(L, n).argtypes = [vp]
        L.orc_totalArea.restype = ctypes.c_double
        L.orc_totalArea.argtypes = [vp]
        L.orc_poly_fit_table.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_int64)]
        for n in ("orc_op_div", "orc_op_curl", "orc_op_c2e", "orc_op_c2v", "orc_op_v2c", "orc_op_v2e",
                  "orc_op_kinetic_energy", "orc_op_tangent_wind"):
            getattr(L, n).argtypes = [vp, vp, vp]
        L.orc_op_tangent_vor_flux.argtypes = [vp, vp, vp, vp, vp]
        L.orc_op_upwind_correction.argtypes = [vp, vp, vp, vp, ip, ip]
        L.orc_swm_set_initial.argtypes = [vp, vp, vp, vp]
        L.orc_swm_set_state.argtypes = [vp, vp, vp]
        L.orc_swm_spatial_operators.argtypes = [vp, vp, vp, vp, vp]
        L.orc_swm_step.argtypes = [vp, ip]
        L.orc_swm_get_state.argtypes = [vp, vp, vp, vp]
        L.orc_swm_get_vertex.argtypes = [vp, vp, vp]
        L.orc_swm_get_diag.argtypes = [vp, vp]
        L.orc_set_tracers.argtypes = [vp, vp]
        L.orc_get_tracers.argtypes = [vp, vp]
        L.orc_adv_set_initial.argtypes = [vp, vp, ip]
        L.orc_adv_step.argtypes = [vp, ip]
        L.orc_adv_get.argtypes = [vp, vp, vp]
        L.orc_reconstruct.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        L.orc_adv_elapsed.restype = ctypes.c_double
        L.orc_adv_elapsed.argtypes = [vp]
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def default_params(**kw) -> Params:
    p = Params()
    lib().orc_default_params(ctypes.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


class Oracle:
    """One oracle model on one MPAS mesh (unit-sphere file arrays)."""

    def __init__(self, mesh, params: Params | None = None, **kw):
        self.L = lib()
        self.params = params if params is not None else default_params(**kw)
        self.mesh = mesh
        self._keep = {}
        mi = MeshIn()
        for k in ("nCells", "nEdges", "nVertices", "maxEdges", "maxEdges2", "vertexDegree"):
            setattr(mi, k, int(mesh.dims[k]))
        for name, _ in MeshIn._fields_[6:]:
            a = mesh.vars[name]
            a = np.ascontiguousarray(a, dtype=np.int32 if a.dtype.kind == "i" else np.float64)
            self._keep[name] = a
            setattr(mi, name, a.ctypes.data)
        self.nc, self.ne, self.nv = mesh.nCells, mesh.nEdges, mesh.nVertices
        self.h = self.L.orc_create(ctypes.byref(mi), ctypes.byref(self.params))
        if not self.h:
            raise RuntimeError("orc_create failed")

    def close(self):
        if getattr(self, "h", None):
            self.L.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    # derived mesh
    def area_edge(self):
        return np.ctypeslib.as_array(self.L.orc_areaEdge(self.h), (self.ne,)).copy()

    def f_vertex(self):
        return np.ctypeslib.as_array(self.L.orc_fVertex(self.h), (self.nv,)).copy()

    def total_area(self):
        return self.L.orc_totalArea(self.h)

    def poly_table(self, name: str) -> np.ndarray:
        d, n = ctypes.c_void_p(), ctypes.c_int64()
        if self.L.orc_poly_fit_table(self.h, name.encode(), ctypes.byref(d), ctypes.byref(n)) != 0:
            raise KeyError(name)
        ct = ctypes.c_double if name.startswith("deriv") else ctypes.c_int32
        return np.ctypeslib.as_array(ctypes.cast(d, ctypes.POINTER(ct)), (n.value,)).copy()

    # operators
    def op(self, name: str, *args, out_size: int):
        out = np.zeros(out_size)
        ins = [np.ascontiguousarray(a, dtype=np.float64) for a in args]
        getattr(self.L, "orc_op_" + name)(self.h, *[_p(a) for a in ins], _p(out))
        return out

    def upwind_correction(self, f_cell, u_edge, f_edge, order, mono=0):
        fe = np.array(f_edge, dtype=np.float64)
        self.L.orc_op_upwind_correction(self.h, _p(np.ascontiguousarray(f_cell, np.float64)),
                                        _p(np.ascontiguousarray(u_edge, np.float64)), _p(fe), order, mono)
        return fe

    # swm
    def set_initial(self, gd, u, ghs):
        self.L.orc_swm_set_initial(self.h, _p(np.ascontiguousarray(gd, np.float64)),
                                   _p(np.ascontiguousarray(u, np.float64)), _p(np.ascontiguousarray(ghs, np.float64)))

    def set_state(self, gd, iap_u):
        self.L.orc_swm_set_state(self.h, _p(np.ascontiguousarray(gd, np.float64)),
                                 _p(np.ascontiguousarray(iap_u, np.float64)))

    def spatial_operators(self, gd, iap_u):
        tg, tu = np.zeros(self.nc), np.zeros(self.ne)
        self.L.orc_swm_spatial_operators(self.h, _p(np.ascontiguousarray(gd, np.float64)),
                                         _p(np.ascontiguousarray(iap_u, np.float64)), _p(tg), _p(tu))
        return tg, tu

    def step(self, n=1):
        self.L.orc_swm_step(self.h, int(n))
        err = self.L.orc_error(self.h)
        if err:
            raise RuntimeError(err.decode())

    def state(self):
        gd, iap, u = np.zeros(self.nc), np.zeros(self.ne), np.zeros(self.ne)
        self.L.orc_swm_get_state(self.h, _p(gd), _p(iap), _p(u))
        return gd, iap, u

    def vertex(self):
        pv, vor = np.zeros(self.nv), np.zeros(self.nv)
        self.L.orc_swm_get_vertex(self.h, _p(pv), _p(vor))
        return pv, vor

    def diag(self):
        d = np.zeros(5)
        self.L.orc_swm_get_diag(self.h, _p(d))
        return d

    def set_tracers(self, qgd):
        self.L.orc_set_tracers(self.h, _p(np.ascontiguousarray(qgd, np.float64)))

    def tracers(self):
        q = np.zeros((self.params.n_tracers, self.nc))
        self.L.orc_get_tracers(self.h, _p(q))
        return q

    # adv
    def reconstruct(self, u):
        """(uX, uY, uZ, zonal, meridional) on cells from u on edges (mpas_reconstruct_1d)."""
        out = [np.empty(self.nc) for _ in range(5)]
        self.L.orc_reconstruct(self.h, _p(np.ascontiguousarray(u, np.float64)), *[_p(a) for a in out])
        return tuple(out)

    def adv_set_initial(self, q, wind_case: int):
        self.L.orc_adv_set_initial(self.h, _p(np.ascontiguousarray(q, np.float64)), int(wind_case))

    def adv_step(self, n=1):
        self.L.orc_adv_step(self.h, int(n))

    def adv_state(self):
        q, u = np.zeros(self.nc), np.zeros(self.ne)
        self.L.orc_adv_get(self.h, _p(q), _p(u))
        return q, u
