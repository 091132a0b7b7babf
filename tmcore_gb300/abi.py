"""ctypes declarations of the C ABI in ``include/tmcore_gpu.h``.

Every exported symbol the header declares is listed in :data:`SYMBOLS`; the
CPU test-suite checks that the built library exports each of them.
"""
from __future__ import annotations

import ctypes

vp = ctypes.c_void_p
dp = ctypes.POINTER(ctypes.c_double)
i32 = ctypes.c_int32
i64p = ctypes.POINTER(ctypes.c_int64)

TMC_OK = 0
TMC_E_ARG = -1
TMC_E_CUDA = -2
TMC_E_HEALTH = -3
TMC_E_UNSUP = -4
TMC_E_STATE = -5
TMC_FP64 = 0
TMC_FP32 = 1


class MeshDesc(ctypes.Structure):
    """tmc_mesh_desc: the MPAS arrays as mesh_init reads them."""

    _fields_ = [(n, i32) for n in ("nCells", "nEdges", "nVertices", "maxEdges", "maxEdges2", "vertexDegree")] + \
               [(n, vp) for n in ("nEdgesOnCell", "nEdgesOnEdge", "cellsOnCell", "edgesOnCell", "verticesOnCell",
                                  "cellsOnEdge", "verticesOnEdge", "edgesOnEdge", "cellsOnVertex", "edgesOnVertex",
                                  "xCell", "yCell", "zCell", "latCell", "xEdge", "yEdge", "zEdge",
                                  "xVertex", "yVertex", "zVertex", "latVertex",
                                  "dvEdge", "dcEdge", "areaCell", "areaTriangle", "kiteAreasOnVertex",
                                  "weightsOnEdge", "lonCell", "lonVertex")]


class Params(ctypes.Structure):
    """tmc_params."""

    _fields_ = [("dt", ctypes.c_double), ("time_scheme", i32), ("pv_scheme", i32), ("conserve_energy", i32),
                ("flux_4th_order_correct", i32), ("apvm_weight", ctypes.c_double), ("adv_order", i32),
                ("adv_mono", i32), ("interp_pv_order", i32), ("radius", ctypes.c_double), ("g", ctypes.c_double),
                ("omega", ctypes.c_double), ("n_tracers", i32), ("tracer_adv_order", i32),
                ("tracer_adv_mono", i32), ("precision", i32), ("renumber", i32), ("use_graph", i32),
                ("diag_every", i32), ("device", i32), ("block_size", i32), ("stencils", i32),
                ("adv_wind", i32), ("members", i32), ("member_layout", i32),
                ("member_lanes", i32), ("reserved", i32 * 2)]


# name -> (restype, argtypes)
SYMBOLS = {
    "tmc_default_params": (ctypes.c_int, [ctypes.POINTER(Params)]),
    "tmc_create": (ctypes.c_int, [ctypes.POINTER(MeshDesc), ctypes.POINTER(Params), ctypes.POINTER(vp)]),
    "tmc_destroy": (ctypes.c_int, [vp]),
    "tmc_last_error": (ctypes.c_char_p, [vp]),
    "tmc_set_initial": (ctypes.c_int, [vp, vp, vp, vp]),
    "tmc_set_state": (ctypes.c_int, [vp, vp, vp]),
    "tmc_get_state": (ctypes.c_int, [vp, vp, vp, vp]),
    "tmc_get_vertex": (ctypes.c_int, [vp, vp, vp]),
    "tmc_set_tracers": (ctypes.c_int, [vp, vp]),
    "tmc_get_tracers": (ctypes.c_int, [vp, vp]),
    "tmc_step": (ctypes.c_int, [vp, i32]),
    "tmc_get_diag": (ctypes.c_int, [vp, vp]),
    "tmc_get_diag_all": (ctypes.c_int, [vp, vp]),
    "tmc_synchronize": (ctypes.c_int, [vp]),
    "tmc_time_integrate": (ctypes.c_int, [vp, vp, vp, vp, vp, vp, vp]),
    "tmc_spatial_operators": (ctypes.c_int, [vp, vp, vp, vp, vp]),
    "tmc_op_div": (ctypes.c_int, [vp, vp, vp]),
    "tmc_op_curl": (ctypes.c_int, [vp, vp, vp]),
    "tmc_op_c2e": (ctypes.c_int, [vp, vp, vp]),
    "tmc_op_c2v": (ctypes.c_int, [vp, vp, vp]),
    "tmc_op_v2c": (ctypes.c_int, [vp, vp, vp]),
    "tmc_op_v2e": (ctypes.c_int, [vp, vp, vp]),
    "tmc_op_kinetic_energy": (ctypes.c_int, [vp, vp, vp]),
    "tmc_op_tangent_wind": (ctypes.c_int, [vp, vp, vp]),
    "tmc_op_tangent_vor_flux": (ctypes.c_int, [vp, vp, vp, vp, vp]),
    "tmc_op_upwind_correction": (ctypes.c_int, [vp, vp, vp, vp, i32, i32]),
    "tmc_time_steps": (ctypes.c_int, [vp, i32, dp, dp, ctypes.POINTER(i32), ctypes.POINTER(i32)]),
    "tmc_sizes": (ctypes.c_int, [vp, i64p, i64p, i64p, i64p]),
    "tmc_select_member": (ctypes.c_int, [vp, i32]),
    "tmc_history_fields": (ctypes.c_int, [vp, vp, vp, vp, vp, vp, vp, vp]),
    "tmc_reconstruct": (ctypes.c_int, [vp, vp, vp, vp, vp, vp, vp]),
    "tmc_autotune": (ctypes.c_int, [vp, i32, ctypes.POINTER(i32)]),
    "tmc_pass_times": (ctypes.c_int, [vp, i32, vp]),
    "tmc_group_create": (ctypes.c_int, [ctypes.POINTER(vp), i32, ctypes.c_double, ctypes.POINTER(vp)]),
    "tmc_group_create_ex": (ctypes.c_int, [ctypes.POINTER(vp), i32, ctypes.c_double, i32, ctypes.POINTER(vp)]),
    "tmc_group_run": (ctypes.c_int, [vp, i32]),
    "tmc_group_synchronize": (ctypes.c_int, [vp]),
    "tmc_group_last_error": (ctypes.c_char_p, [vp]),
    "tmc_group_destroy": (ctypes.c_int, [vp]),
    "tmc_mlp_create": (ctypes.c_int, [i32, ctypes.c_uint64, ctypes.POINTER(vp)]),
    "tmc_mlp_destroy": (ctypes.c_int, [vp]),
    "tmc_mlp_last_error": (ctypes.c_char_p, [vp]),
    "tmc_mlp_get_params": (ctypes.c_int, [vp, vp]),
    "tmc_mlp_set_params": (ctypes.c_int, [vp, vp]),
    "tmc_mlp_set_scaling": (ctypes.c_int, [vp, vp, vp, ctypes.c_float]),
    "tmc_mlp_forward": (ctypes.c_int, [vp, vp, ctypes.c_int64, vp, i32]),
    "tmc_mlp_set_dataset": (ctypes.c_int, [vp, vp, vp, ctypes.c_int64]),
    "tmc_mlp_train": (ctypes.c_int, [vp, i32, i32, ctypes.c_float, vp]),
    "tmc_mlp_gradient": (ctypes.c_int, [vp, vp, vp, ctypes.c_int64, vp, dp]),
    "tmc_mlp_set_train_mode": (ctypes.c_int, [vp, i32]),
    "tmc_mlp_set_wait_limit": (ctypes.c_int, [vp, i32]),
    "tmc_mlp_set_head": (ctypes.c_int, [vp, i32, ctypes.c_double]),
    "tmc_set_closure": (ctypes.c_int, [vp, vp]),
    "tmc_set_closure_stages": (ctypes.c_int, [vp, i32]),
    "tmc_set_member_closure": (ctypes.c_int, [vp, i32, i32]),
    "tmc_closure_status": (ctypes.c_int, [vp, ctypes.POINTER(i32)]),
    "tmc_closure_features": (ctypes.c_int, [vp, vp, vp]),
    "tmc_closure_correction": (ctypes.c_int, [vp, vp]),
    "tmc_coarsen_create": (ctypes.c_int, [ctypes.POINTER(MeshDesc), ctypes.POINTER(MeshDesc), i32,
                                           ctypes.POINTER(vp)]),
    "tmc_coarsen_apply": (ctypes.c_int, [vp, vp, vp, vp, vp, vp, vp]),
    "tmc_coarsen_rows": (ctypes.c_int, [vp, i32, i64p, vp, vp, vp]),
    "tmc_coarsen_unmatched": (ctypes.c_int, [vp, i64p]),
    "tmc_coarsen_cell_map": (ctypes.c_int, [vp, vp]),
    "tmc_coarsen_last_error": (ctypes.c_char_p, [vp]),
    "tmc_coarsen_destroy": (ctypes.c_int, [vp]),
    "tmc_mesh_file_open": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(vp), ctypes.POINTER(MeshDesc)]),
    "tmc_mesh_file_error": (ctypes.c_char_p, [vp]),
    "tmc_mesh_file_close": (ctypes.c_int, [vp]),
    "tmc_mesh_file_write": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(MeshDesc)]),
    "tmc_history_create": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(MeshDesc), ctypes.POINTER(vp)]),
    "tmc_history_write": (ctypes.c_int, [vp, vp, ctypes.c_double]),
    "tmc_history_close": (ctypes.c_int, [vp]),
    "tmc_adv_set_initial": (ctypes.c_int, [vp, vp]),
    "tmc_adv_get": (ctypes.c_int, [vp, vp, vp]),
    "tmc_adv_elapsed": (ctypes.c_int, [vp, dp]),
    "tmc_mass_energy_noalloc": (ctypes.c_int, [vp, vp, vp, ctypes.c_int64, vp, vp, ctypes.c_int64, vp, vp]),
}
TMC_NOALLOC_MAX_ELEMENTS = 8388608
TMC_MLP_PARAMS = 9985
TMC_MLP_FEATURES = 24


def declare(lib: ctypes.CDLL) -> ctypes.CDLL:
    for name, (res, args) in SYMBOLS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


def header_symbols(header_text: str) -> list[str]:
    """Function names declared in a C header (``int tmc_x(`` / ``const char* tmc_x(``)."""
    import re

    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(tmc_\w+)\s*\(", header_text, flags=re.M)))
