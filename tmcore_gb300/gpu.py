"""Python host mirror of the C ABI: one shallow-water model on one GPU.

Method names follow the reference's integrator/operator interface
(src/core/time_scheme_mod.F90:14-43, src/core/operators_mod.F90:15-30);
arrays are numpy float64 in the mesh file's element order.  There is no CPU
path: if the CUDA library or a GPU is missing, construction raises.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib, abi

REF_RADIUS = 6371220.0  # src/utils/const_mod.F90:11
REF_G = 9.80616
REF_OMEGA = 7.292e-5


class TMCError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"tmcore_gpu error {code}: {msg}")
        self.code = code


def default_params(**kw) -> abi.Params:
    """tmc_params with the shipped SWM namelist defaults, overridden by ``kw``."""
    p = abi.Params()
    lib = _lib.gpu()
    lib.tmc_default_params(ctypes.byref(p))
    for k, v in kw.items():
        if not any(f[0] == k for f in abi.Params._fields_):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a):
    return None if a is None else a.ctypes.data


def mesh_desc(mesh):
    """tmc_mesh_desc of an MPASMesh; returns (desc, arrays to keep alive)."""
    d = abi.MeshDesc()
    for k in ("nCells", "nEdges", "nVertices", "maxEdges", "maxEdges2", "vertexDegree"):
        setattr(d, k, int(mesh.dims[k]))
    keep = []
    for name, _ in abi.MeshDesc._fields_[6:]:
        if name not in mesh.vars and name in ("lonCell", "lonVertex"):
            continue  # optional: NULL
        a = mesh.vars[name]
        a = np.ascontiguousarray(a, dtype=np.int32 if a.dtype.kind == "i" else np.float64)
        keep.append(a)
        setattr(d, name, a.ctypes.data)
    return d, keep


class TMCoreGPU:
    """A device-resident shallow-water model (handle of the C ABI)."""

    def __init__(self, mesh, params: abi.Params | None = None, **kw):
        self.lib = _lib.gpu()
        self.params = params if params is not None else default_params(**kw)
        self.mesh = mesh
        self.nc, self.ne, self.nv = mesh.nCells, mesh.nEdges, mesh.nVertices
        d, self._keep = mesh_desc(mesh)
        h = ctypes.c_void_p()
        rc = self.lib.tmc_create(ctypes.byref(d), ctypes.byref(self.params), ctypes.byref(h))
        self.h = h
        if rc != 0:
            msg = self.lib.tmc_last_error(h).decode() if h.value else "tmc_create failed"
            self.close()
            raise TMCError(rc, msg)
        self.n_tracers = int(self.params.n_tracers)

    # ------------------------------------------------------------------
    def _chk(self, rc):
        if rc != 0:
            raise TMCError(rc, self.lib.tmc_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.tmc_destroy(self.h)
        self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ------------------------------------------------------------------ state
    def set_initial(self, gd, u, ghs):
        self._chk(self.lib.tmc_set_initial(self.h, _ptr(_f64(gd)), _ptr(_f64(u)), _ptr(_f64(ghs))))

    def set_state(self, gd, iap_u):
        self._chk(self.lib.tmc_set_state(self.h, _ptr(_f64(gd)), _ptr(_f64(iap_u))))

    def get_state(self, with_u: bool = True):
        gd, iap = np.empty(self.nc), np.empty(self.ne)
        u = np.empty(self.ne) if with_u else None
        self._chk(self.lib.tmc_get_state(self.h, _ptr(gd), _ptr(iap), _ptr(u)))
        return (gd, iap, u) if with_u else (gd, iap)

    def get_vertex(self):
        pv, vor = np.empty(self.nv), np.empty(self.nv)
        self._chk(self.lib.tmc_get_vertex(self.h, _ptr(pv), _ptr(vor)))
        return pv, vor

    def set_tracers(self, qgd):
        self._chk(self.lib.tmc_set_tracers(self.h, _ptr(_f64(qgd))))

    def get_tracers(self):
        q = np.empty((self.n_tracers, self.nc))
        self._chk(self.lib.tmc_get_tracers(self.h, _ptr(q)))
        return q

    def autotune(self, steps: int = 3):
        """Per-pass block sizes by timing (tmc_autotune); returns
        {cell, vertex, edge_pv, edge_flux, final}."""
        out = (ctypes.c_int32 * 5)()
        self._chk(self.lib.tmc_autotune(self.h, int(steps), out))
        return dict(zip(("cell", "vertex", "edge_pv", "edge_flux", "final"), list(out)))

    # ------------------------------------------------------------------ history diagnostics
    def history_fields(self):
        """dict of the history fields of state(old): u, zonal, meridional, h, div, pv, vor."""
        out = {"u": np.empty(self.ne), "zonal": np.empty(self.nc), "meridional": np.empty(self.nc),
               "h": np.empty(self.nc), "div": np.empty(self.nc), "pv": np.empty(self.nv), "vor": np.empty(self.nv)}
        self._chk(self.lib.tmc_history_fields(self.h, *[_ptr(out[k]) for k in
                                                        ("u", "zonal", "meridional", "h", "div", "pv", "vor")]))
        return out

    def reconstruct(self, u):
        """(uX, uY, uZ, zonal, meridional) on cells from u on edges (mpas_reconstruct_1d)."""
        out = [np.empty(self.nc) for _ in range(5)]
        self._chk(self.lib.tmc_reconstruct(self.h, _ptr(_f64(u)), *[_ptr(a) for a in out]))
        return tuple(out)

    # ------------------------------------------------------------------ learned closure
    def set_closure(self, net):
        """Apply `net` (a ClosureMLP, or None) to pv_edge in every stage."""
        self._closure = net
        self._chk(self.lib.tmc_set_closure(self.h, None if net is None else net.n))

    def set_closure_stages(self, every_stage: bool):
        """True: the network runs in every stage; False: in stage 1, its output
        held for stages 2-4."""
        self._chk(self.lib.tmc_set_closure_stages(self.h, 1 if every_stage else 0))

    def set_member_closure(self, member: int, on: bool):
        self._chk(self.lib.tmc_set_member_closure(self.h, int(member), 1 if on else 0))

    def closure_status(self) -> bool:
        v = ctypes.c_int32()
        self._chk(self.lib.tmc_closure_status(self.h, ctypes.byref(v)))
        return bool(v.value)

    def closure_correction(self):
        """[nEdges] the correction the network added to pv_edge in stage 1 of
        the last step (closure held from stage 1), selected member."""
        dq = np.empty(self.ne, np.float32)
        self._chk(self.lib.tmc_closure_correction(self.h, _ptr(dq)))
        return dq

    def closure_features(self):
        """[nEdges, 24] features and pv_edge of state(old) of the selected member."""
        f = np.empty((self.ne, abi.TMC_MLP_FEATURES), np.float32)
        pv = np.empty(self.ne)
        self._chk(self.lib.tmc_closure_features(self.h, _ptr(f), _ptr(pv)))
        return f, pv

    def pass_times(self, steps: int = 3) -> dict:
        """Mean device ms per launch of each pass of the fused step (tmc_pass_times)."""
        out = np.empty(5)
        self._chk(self.lib.tmc_pass_times(self.h, int(steps), _ptr(out)))
        return dict(zip(("cell", "vertex", "edge_pv", "edge_flux", "final"), out.tolist()))

    # ------------------------------------------------------------------ ensembles
    def select_member(self, m: int):
        """State-transfer calls address member m of an ensemble (members > 1)."""
        self._chk(self.lib.tmc_select_member(self.h, int(m)))

    # ------------------------------------------------------------------ adv model
    def adv_set_initial(self, q):
        """adv model (adv_wind 1 or 2): the advected scalar; the wind at elapsed = 0."""
        self._chk(self.lib.tmc_adv_set_initial(self.h, _ptr(_f64(q))))

    def adv_state(self):
        q, u = np.empty(self.nc), np.empty(self.ne)
        self._chk(self.lib.tmc_adv_get(self.h, _ptr(q), _ptr(u)))
        return q, u

    def adv_elapsed(self) -> float:
        t = ctypes.c_double()
        self._chk(self.lib.tmc_adv_elapsed(self.h, ctypes.byref(t)))
        return t.value

    # ------------------------------------------------------------------ stepping
    def step(self, n: int = 1):
        self._chk(self.lib.tmc_step(self.h, int(n)))

    def synchronize(self):
        self._chk(self.lib.tmc_synchronize(self.h))

    def diag(self):
        """[total_mass, total_energy, total_potential_enstrophy, total_absolute_vorticity, beta]"""
        out = np.empty(5)
        self._chk(self.lib.tmc_get_diag(self.h, _ptr(out)))
        return out

    def diag_all(self):
        """[members, 5] invariants and beta of every ensemble member."""
        m = int(self.params.members) if self.params.members > 1 else 1
        out = np.empty((m, 5))
        self._chk(self.lib.tmc_get_diag_all(self.h, _ptr(out)))
        return out

    def time_integrate(self, gd_old, iap_old, q_old=None, out=None):
        """One step with host arrays in and out (tmc_time_integrate)."""
        if out is None:
            out = (np.empty(self.nc), np.empty(self.ne),
                   np.empty((self.n_tracers, self.nc)) if self.n_tracers else None)
        gd_new, iap_new, q_new = out
        self._chk(self.lib.tmc_time_integrate(self.h, _ptr(gd_old), _ptr(iap_old), _ptr(q_old),
                                              _ptr(gd_new), _ptr(iap_new), _ptr(q_new)))
        return out

    def spatial_operators(self, gd, iap_u):
        tg, tu = np.empty(self.nc), np.empty(self.ne)
        self._chk(self.lib.tmc_spatial_operators(self.h, _ptr(_f64(gd)), _ptr(_f64(iap_u)), _ptr(tg), _ptr(tu)))
        return tg, tu

    def time_steps(self, n: int, total: bool = True, flux: bool = True):
        """Device timing of n steps: (ms_total, ms_flux_kernel, flux_launches, total_launches)."""
        a, b = ctypes.c_double(), ctypes.c_double()
        c, d = ctypes.c_int32(), ctypes.c_int32()
        self._chk(self.lib.tmc_time_steps(self.h, int(n), ctypes.byref(a) if total else None,
                                          ctypes.byref(b) if flux else None, ctypes.byref(c), ctypes.byref(d)))
        return (a.value if total else None), (b.value if flux else None), c.value, d.value

    def sizes(self):
        v = [ctypes.c_int64() for _ in range(4)]
        self._chk(self.lib.tmc_sizes(self.h, *[ctypes.byref(x) for x in v]))
        return tuple(x.value for x in v)

    # ------------------------------------------------------------------ operators
    _OUT = {"div": "c", "curl": "v", "c2e": "e", "c2v": "v", "v2c": "c", "v2e": "e",
            "kinetic_energy": "c", "tangent_wind": "e"}

    def op(self, name: str, f):
        n = {"c": self.nc, "e": self.ne, "v": self.nv}[self._OUT[name]]
        out = np.empty(n)
        self._chk(getattr(self.lib, "tmc_op_" + name)(self.h, _ptr(_f64(f)), _ptr(out)))
        return out

    def tangent_vor_flux(self, u, gd_e, pv_e):
        out = np.empty(self.ne)
        self._chk(self.lib.tmc_op_tangent_vor_flux(self.h, _ptr(_f64(u)), _ptr(_f64(gd_e)), _ptr(_f64(pv_e)),
                                                   _ptr(out)))
        return out

    def upwind_correction(self, f_cell, u_edge, f_edge, order: int, mono: int = 0):
        fe = np.array(f_edge, dtype=np.float64)
        self._chk(self.lib.tmc_op_upwind_correction(self.h, _ptr(_f64(f_cell)), _ptr(_f64(u_edge)), _ptr(fe),
                                                    int(order), int(mono)))
        return fe


class TMCoreGroup:
    """Several models (different meshes and dt) advanced together: one CUDA
    graph per cycle of ``cycle_seconds`` (tmc_group_*).  mode 0: one branch
    per model; mode 1: one launch per pass over all models (member-innermost
    ensembles of one member count and pv scheme, tmc_group_create_ex)."""

    def __init__(self, models, cycle_seconds: float, mode: int = 0):
        self.lib = _lib.gpu()
        self.models = list(models)
        self.mode = int(mode)
        arr = (ctypes.c_void_p * len(self.models))(*[m.h.value for m in self.models])
        g = ctypes.c_void_p()
        rc = self.lib.tmc_group_create_ex(arr, len(self.models), float(cycle_seconds), self.mode, ctypes.byref(g))
        self.g = g
        if rc != 0:
            msg = self.lib.tmc_group_last_error(g).decode() if g.value else \
                "; ".join(m.lib.tmc_last_error(m.h).decode() for m in self.models)
            self.close()
            raise TMCError(rc, msg)

    def run(self, cycles: int = 1):
        rc = self.lib.tmc_group_run(self.g, int(cycles))
        if rc != 0:
            raise TMCError(rc, self.lib.tmc_group_last_error(self.g).decode())

    def synchronize(self):
        rc = self.lib.tmc_group_synchronize(self.g)
        if rc != 0:
            raise TMCError(rc, self.lib.tmc_group_last_error(self.g).decode())

    def close(self):
        if getattr(self, "g", None) is not None and self.g.value:
            self.lib.tmc_group_destroy(self.g)
        self.g = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ClosureMLP:
    """The 24-64-64-64-1 GELU network of the learned PV-on-edge closure
    (tmc_mlp_*): BF16 weights, FP32 accumulation, tensor-core forward,
    Adam training on the device (forward and backward on the tensor cores,
    or on the CUDA cores in FP32 after ``set_train_mode(False)``)."""

    def __init__(self, device: int = 0, seed: int = 0):
        self.lib = _lib.gpu()
        self.head, self.head_dt = 0, 0.0
        n = ctypes.c_void_p()
        rc = self.lib.tmc_mlp_create(int(device), int(seed), ctypes.byref(n))
        self.n = n
        if rc != 0:
            msg = self.lib.tmc_mlp_last_error(n).decode() if n.value else "tmc_mlp_create failed"
            self.close()
            raise TMCError(rc, msg)

    def _chk(self, rc):
        if rc != 0:
            raise TMCError(rc, self.lib.tmc_mlp_last_error(self.n).decode())

    def close(self):
        if getattr(self, "n", None) is not None and self.n.value:
            self.lib.tmc_mlp_destroy(self.n)
        self.n = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self) -> np.ndarray:
        p = np.empty(abi.TMC_MLP_PARAMS, np.float32)
        self._chk(self.lib.tmc_mlp_get_params(self.n, _ptr(p)))
        return p

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == abi.TMC_MLP_PARAMS
        self._chk(self.lib.tmc_mlp_set_params(self.n, _ptr(p)))

    def set_scaling(self, x_mean, x_inv_std, y_scale: float):
        xm = np.ascontiguousarray(x_mean, np.float32)
        xi = np.ascontiguousarray(x_inv_std, np.float32)
        self._chk(self.lib.tmc_mlp_set_scaling(self.n, _ptr(xm), _ptr(xi), float(y_scale)))

    def forward(self, x, tensor_cores: bool = True) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32).reshape(-1, abi.TMC_MLP_FEATURES)
        y = np.empty(x.shape[0], np.float32)
        self._chk(self.lib.tmc_mlp_forward(self.n, _ptr(x), x.shape[0], _ptr(y), 1 if tensor_cores else 0))
        return y

    def set_dataset(self, x, y):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, abi.TMC_MLP_FEATURES)
        y = np.ascontiguousarray(y, np.float32).reshape(-1)
        self._keep = (x, y)
        self._chk(self.lib.tmc_mlp_set_dataset(self.n, _ptr(x), _ptr(y), x.shape[0]))

    def set_train_mode(self, tensor_cores: bool):
        """Run train() and gradient() on the tensor cores (True) or the CUDA cores."""
        self._chk(self.lib.tmc_mlp_set_train_mode(self.n, 1 if tensor_cores else 0))

    def set_head(self, head: int, dt: float = 0.0):
        """Output head: 0 the correction is y * y_scale; 1 it is
        -softplus(y) dt (v dq/dt + u dq/dn), a learned non-negative APVM weight;
        2 it is y * y_scale where y v dq/dt <= 0 (APVM's sign), else 0."""
        self.head, self.head_dt = int(head), float(dt)
        self._chk(self.lib.tmc_mlp_set_head(self.n, int(head), float(dt)))

    def set_wait_limit(self, polls: int):
        """Poll limit of the tensor-core completion waits (< 0: the default);
        0 makes every wait run out at once, to exercise the error path."""
        self._chk(self.lib.tmc_mlp_set_wait_limit(self.n, int(polls)))

    def train(self, steps: int, batch: int = 65536, lr: float = 1e-3) -> np.ndarray:
        losses = np.empty(max(int(steps), 1), np.float32)
        self._chk(self.lib.tmc_mlp_train(self.n, int(batch), int(steps), float(lr), _ptr(losses)))
        return losses[:steps]

    def gradient(self, x, y):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, abi.TMC_MLP_FEATURES)
        y = np.ascontiguousarray(y, np.float32).reshape(-1)
        g = np.empty(abi.TMC_MLP_PARAMS, np.float32)
        loss = ctypes.c_double()
        self._chk(self.lib.tmc_mlp_gradient(self.n, _ptr(x), _ptr(y), x.shape[0], _ptr(g), ctypes.byref(loss)))
        return g, loss.value


class Coarsener:
    """Coarse-graining of fine-mesh fields onto a coarser mesh (tmc_coarsen_*);
    device < 0 builds the maps only (``rows``), without CUDA."""

    def __init__(self, fine, coarse, device: int = 0):
        self.lib = _lib.gpu()
        self.fine, self.coarse = fine, coarse
        df, kf = mesh_desc(fine)
        dc, kc = mesh_desc(coarse)
        c = ctypes.c_void_p()
        rc = self.lib.tmc_coarsen_create(ctypes.byref(df), ctypes.byref(dc), int(device), ctypes.byref(c))
        self.c = c
        if rc != 0:
            msg = self.lib.tmc_coarsen_last_error(c).decode() if c.value else "tmc_coarsen_create failed"
            self.close()
            raise TMCError(rc, msg)

    def rows(self, which: int):
        """Map `which` (0 cells, 1 normal velocity, 2 edge scalars) as CSR
        arrays (start, idx, w) over the fine array."""
        n = ctypes.c_int64()
        self.lib.tmc_coarsen_rows(self.c, int(which), ctypes.byref(n), None, None, None)
        rows = self.coarse.nCells if which == 0 else self.coarse.nEdges
        start, idx, w = np.empty(rows + 1, np.int32), np.empty(n.value, np.int32), np.empty(n.value)
        rc = self.lib.tmc_coarsen_rows(self.c, int(which), ctypes.byref(n), _ptr(start), _ptr(idx), _ptr(w))
        if rc != 0:
            raise TMCError(rc, "tmc_coarsen_rows")
        return start, idx, w

    def unmatched(self) -> int:
        n = ctypes.c_int64()
        self.lib.tmc_coarsen_unmatched(self.c, ctypes.byref(n))
        return n.value

    def cell_map(self) -> np.ndarray:
        """0-based coarse cell of every fine cell."""
        m = np.empty(self.fine.nCells, np.int32)
        self.lib.tmc_coarsen_cell_map(self.c, _ptr(m))
        return m - 1

    def __call__(self, gd=None, u=None, pv_edge=None):
        nc, ne = self.coarse.nCells, self.coarse.nEdges
        og = np.empty(nc) if gd is not None else None
        ou = np.empty(ne) if u is not None else None
        op = np.empty(ne) if pv_edge is not None else None
        a = [None if v is None else _f64(v) for v in (gd, u, pv_edge)]
        rc = self.lib.tmc_coarsen_apply(self.c, _ptr(a[0]), _ptr(a[1]), _ptr(a[2]), _ptr(og), _ptr(ou), _ptr(op))
        if rc != 0:
            raise TMCError(rc, self.lib.tmc_coarsen_last_error(self.c).decode())
        return og, ou, op

    def close(self):
        if getattr(self, "c", None) is not None and self.c.value:
            self.lib.tmc_coarsen_destroy(self.c)
        self.c = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def read_mesh_file(path: str):
    """An MPAS grid file read by the library's NetCDF-classic reader
    (tmc_mesh_file_open), as an MPASMesh (arrays copied)."""
    from .mesh import MPASMesh

    lib = _lib.gpu()
    d = abi.MeshDesc()
    f = ctypes.c_void_p()
    rc = lib.tmc_mesh_file_open(str(path).encode(), ctypes.byref(f), ctypes.byref(d))
    try:
        if rc != 0:
            raise TMCError(rc, lib.tmc_mesh_file_error(f).decode() if f.value else "tmc_mesh_file_open failed")
        dims = {k: int(getattr(d, k)) for k in ("nCells", "nEdges", "nVertices", "maxEdges", "maxEdges2",
                                                 "vertexDegree")}
        n = {"Cell": dims["nCells"], "Edge": dims["nEdges"], "Vertex": dims["nVertices"]}
        shapes = {"nEdgesOnCell": (n["Cell"],), "nEdgesOnEdge": (n["Edge"],),
                  "cellsOnCell": (n["Cell"], dims["maxEdges"]), "edgesOnCell": (n["Cell"], dims["maxEdges"]),
                  "verticesOnCell": (n["Cell"], dims["maxEdges"]), "cellsOnEdge": (n["Edge"], 2),
                  "verticesOnEdge": (n["Edge"], 2), "edgesOnEdge": (n["Edge"], dims["maxEdges2"]),
                  "cellsOnVertex": (n["Vertex"], dims["vertexDegree"]),
                  "edgesOnVertex": (n["Vertex"], dims["vertexDegree"]),
                  "kiteAreasOnVertex": (n["Vertex"], dims["vertexDegree"]),
                  "weightsOnEdge": (n["Edge"], dims["maxEdges2"])}
        vars_ = {}
        for name, ctype in abi.MeshDesc._fields_[6:]:
            ptr = getattr(d, name)
            if not ptr:
                continue
            if name in shapes:
                shape = shapes[name]
            else:
                kind = "Vertex" if name == "areaTriangle" else [k for k in ("Cell", "Edge", "Vertex")
                                                                   if name.endswith(k)][0]
                shape = (n[kind],)
            size = int(np.prod(shape))
            is_int = name.startswith("n") or name.endswith(("OnCell", "OnEdge", "OnVertex")) and name not in (
                "kiteAreasOnVertex", "weightsOnEdge")
            ct = ctypes.c_int32 if is_int else ctypes.c_double
            arr = np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ct)), shape=(size,)).copy()
            vars_[name] = arr.reshape(shape)
        return MPASMesh(dims, vars_, {})
    finally:
        if f.value:
            lib.tmc_mesh_file_close(f)


def write_mesh_file(path: str, mesh):
    """Write an MPASMesh with the library's NetCDF-classic writer (tmc_mesh_file_write)."""
    lib = _lib.gpu()
    d, keep = mesh_desc(mesh)
    rc = lib.tmc_mesh_file_write(str(path).encode(), ctypes.byref(d))
    del keep
    if rc != 0:
        raise TMCError(rc, f"tmc_mesh_file_write({path}) failed")


class HistoryWriter:
    """History file of history_mod.F90 written by the library (tmc_history_*)."""

    def __init__(self, path: str, mesh):
        self.lib = _lib.gpu()
        d, self._keep = mesh_desc(mesh)
        hw = ctypes.c_void_p()
        rc = self.lib.tmc_history_create(str(path).encode(), ctypes.byref(d), ctypes.byref(hw))
        if rc != 0:
            raise TMCError(rc, f"tmc_history_create({path}) failed")
        self.hw = hw

    def write(self, model: TMCoreGPU, seconds: float):
        rc = self.lib.tmc_history_write(self.hw, model.h, float(seconds))
        if rc != 0:
            raise TMCError(rc, model.lib.tmc_last_error(model.h).decode())

    def close(self):
        if getattr(self, "hw", None) is not None and self.hw.value:
            self.lib.tmc_history_close(self.hw)
        self.hw = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
