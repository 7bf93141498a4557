"""ctypes declarations of the C ABI in include/swgpu.h.

The shared library is built in-tree (``_lib/libswgpu.so``) by
``omega_playground_gb300._build``.  There is no fallback: if the library is
missing or a call fails, an exception is raised.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _build

_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)
_vp = C.c_void_p

SWG_OK = 0
ERRORS = {1: "bad argument", 2: "out of memory", 3: "CUDA error",
          4: "device wait timed out", 5: "checkpoint budget", 6: "bad state"}


class SwgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{ERRORS.get(code, code)}] {msg}")
        self.code = code


class MeshDesc(C.Structure):
    _fields_ = [("ncells", C.c_int), ("nedges", C.c_int),
                ("nvertices", C.c_int), ("nlayers", C.c_int),
                ("nedges_on_cell", _ip), ("edges_on_cell", _ip),
                ("nedges_on_edge", _ip), ("edges_on_edge", _ip),
                ("cells_on_edge", _ip), ("vertices_on_edge", _ip),
                ("edges_on_vertex", _ip), ("cells_on_vertex", _ip),
                ("area_cell", _dp), ("edge_sign_on_cell", _dp),
                ("dc_edge", _dp), ("dv_edge", _dp), ("weights_on_edge", _dp),
                ("area_triangle", _dp), ("kiteareas_on_vertex", _dp),
                ("edge_sign_on_vertex", _dp), ("mesh_scaling_del2", _dp),
                ("mesh_scaling_del4", _dp), ("edge_mask", _dp),
                ("max_level_cell", _ip), ("max_level_vertex_bot", _ip)]


HEX_INT = ["nedges_on_cell", "edges_on_cell", "cells_on_cell",
           "vertices_on_cell", "kite_index_on_cell", "nedges_on_edge",
           "edges_on_edge", "cells_on_edge", "vertices_on_edge",
           "edges_on_vertex", "cells_on_vertex"]
HEX_DBL = ["area_cell", "x_cell", "y_cell", "edge_sign_on_cell", "dc_edge",
           "dv_edge", "angle_edge", "x_edge", "y_edge", "weights_on_edge",
           "area_triangle", "x_vertex", "y_vertex", "kiteareas_on_vertex",
           "edge_sign_on_vertex"]
# (entity, width) of every hex table
HEX_SHAPE = {
    "nedges_on_cell": ("C", 1), "edges_on_cell": ("C", 6),
    "cells_on_cell": ("C", 6), "vertices_on_cell": ("C", 6),
    "kite_index_on_cell": ("C", 6), "nedges_on_edge": ("E", 1),
    "edges_on_edge": ("E", 12), "cells_on_edge": ("E", 2),
    "vertices_on_edge": ("E", 2), "edges_on_vertex": ("V", 3),
    "cells_on_vertex": ("V", 3), "area_cell": ("C", 1), "x_cell": ("C", 1),
    "y_cell": ("C", 1), "edge_sign_on_cell": ("C", 6), "dc_edge": ("E", 1),
    "dv_edge": ("E", 1), "angle_edge": ("E", 1), "x_edge": ("E", 1),
    "y_edge": ("E", 1), "weights_on_edge": ("E", 12),
    "area_triangle": ("V", 1), "x_vertex": ("V", 1), "y_vertex": ("V", 1),
    "kiteareas_on_vertex": ("V", 3), "edge_sign_on_vertex": ("V", 3),
}


class HexTables(C.Structure):
    _fields_ = [(n, _ip) for n in HEX_INT] + [(n, _dp) for n in HEX_DBL]


class Params(C.Structure):
    _fields_ = [("f0", C.c_double), ("grav", C.c_double),
                ("drag_coeff", C.c_double), ("visc_del2", C.c_double),
                ("visc_del4", C.c_double), ("eddy_diff2", C.c_double),
                ("eddy_diff4", C.c_double), ("ntracers", C.c_int),
                ("disable_h_tendency", C.c_int),
                ("disable_vn_tendency", C.c_int)]


class ModelOptions(C.Structure):
    _fields_ = [("linear", C.c_int), ("h0", C.c_double),
                ("apply_drag", C.c_int)]


FORCING_FN = C.CFUNCTYPE(None, _vp, _dp, _dp, _dp, _dp, C.c_double, _vp)

# name -> (restype, argtypes)
_SIGS = {
    "swg_last_error": (C.c_char_p, []),
    "swg_version": (C.c_char_p, []),
    "swg_kernel_launches": (C.c_longlong, []),
    "swg_planar_hex_mesh_build": (C.c_int, [C.c_int, C.c_int, C.c_double,
                                            C.POINTER(HexTables), _dp, _dp]),
    "swg_mesh_create": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(_vp)]),
    "swg_mesh_destroy": (C.c_int, [_vp]),
    "swg_state_create": (C.c_int, [_vp, C.c_int, C.POINTER(_vp)]),
    "swg_state_destroy": (C.c_int, [_vp]),
    "swg_state_upload": (C.c_int, [_vp, _dp, _dp, _dp, _vp]),
    "swg_state_download": (C.c_int, [_vp, _dp, _dp, _dp, _vp]),
    "swg_state_device_ptrs": (C.c_int, [_vp, C.POINTER(_dp), C.POINTER(_dp),
                                        C.POINTER(_dp)]),
    "swg_state_copy": (C.c_int, [_vp, _vp, _vp]),
    "swg_state_fill": (C.c_int, [_vp, C.c_double, _vp]),
    "swg_model_create": (C.c_int, [_vp, C.POINTER(Params), C.POINTER(_vp)]),
    "swg_model_set_term_enabled": (C.c_int, [_vp, C.c_int, C.c_int]),
    "swg_model_term_enabled": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int)]),
    "swg_model_create_ex": (C.c_int, [_vp, C.POINTER(Params),
                                      C.POINTER(ModelOptions),
                                      C.POINTER(_vp)]),
    "swg_linear_model_create": (C.c_int, [_vp, C.POINTER(Params), C.c_double,
                                          C.POINTER(_vp)]),
    "swg_model_destroy": (C.c_int, [_vp]),
    "swg_model_set_forcing": (C.c_int, [_vp, FORCING_FN, _vp]),
    "swg_compute_tendency": (C.c_int, [_vp, _vp, _vp, C.c_double, C.c_int,
                                       _vp]),
    "swg_model_compute_aux": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "swg_compute_h_tendency": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, _vp]),
    "swg_compute_vn_tendency": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, _vp]),
    "swg_compute_tr_tendency": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, _vp]),
    "swg_compute_tendency_noalloc": (C.c_int, [_vp, C.POINTER(Params), _vp,
                                               _vp, _vp, _vp, _vp, _vp,
                                               C.c_int, _vp]),
    "swg_model_aux": (C.c_int, [_vp, C.c_char_p, C.POINTER(_dp),
                                C.POINTER(C.c_longlong)]),
    "swg_stepper_create": (C.c_int, [_vp, C.c_int, C.c_int, C.POINTER(_vp)]),
    "swg_stepper_destroy": (C.c_int, [_vp]),
    "swg_step": (C.c_int, [_vp, _vp, C.c_double, C.c_double, C.c_int,
                           C.c_int, _vp]),
    "swg_host_stepper_create": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int,
                                          C.POINTER(_vp)]),
    "swg_host_stepper_create_levels": (C.c_int, [_vp, C.c_int, C.c_int,
                                                 C.c_int, C.POINTER(C.c_int),
                                                 C.POINTER(_vp)]),
    "swg_host_stepper_destroy": (C.c_int, [_vp]),
    "swg_host_stepper_chunks": (C.c_int, [_vp, C.POINTER(C.c_int),
                                          C.POINTER(C.c_int)]),
    "swg_host_step": (C.c_int, [_vp, _dp, _dp, _dp, C.c_double, C.c_double,
                                C.c_int, _vp]),
    "swg_host_alloc": (C.c_int, [C.c_ulonglong, C.POINTER(_vp)]),
    "swg_host_free": (C.c_int, [_vp]),
    "swg_batch_create": (C.c_int, [C.c_int, C.POINTER(_vp), C.POINTER(_vp),
                                   C.c_int, C.c_int, C.POINTER(_vp)]),
    "swg_batch_destroy": (C.c_int, [_vp]),
    "swg_batch_step": (C.c_int, [_vp, C.c_double, C.c_double, C.c_int,
                                 C.c_int, _vp]),
    "swg_batch_check": (C.c_int, [_vp, _vp]),
    "swg_batch_config_count": (C.c_int, []),
    "swg_batch_set_config": (C.c_int, [_vp, C.c_int]),
    "swg_batch_autotune": (C.c_int, [_vp, C.c_double, C.c_int, _vp,
                                     C.POINTER(C.c_int), _dp]),
    "swg_batch_selftest_timeout": (C.c_int, [_vp, C.c_double, _vp]),
    "swg_adjoint_create": (C.c_int, [_vp, C.c_int, C.POINTER(_vp)]),
    "swg_adjoint_create_stepper": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int,
                                             C.POINTER(_vp)]),
    "swg_adjoint_destroy": (C.c_int, [_vp]),
    "swg_tlm_tendency": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "swg_adj_tendency": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "swg_tlm_apply": (C.c_int, [_vp, _vp, _vp, C.c_double, C.c_double,
                                C.c_int, _vp]),
    "swg_adj_forward": (C.c_int, [_vp, _vp, C.c_double, C.c_double, C.c_int,
                                  _vp, _vp]),
    "swg_adj_backward": (C.c_int, [_vp, _vp, _vp]),
    "swg_adj_info": (C.c_int, [_vp, C.POINTER(C.c_longlong),
                               C.POINTER(C.c_longlong)]),
    "swg_adj_info_ex": (C.c_int, [_vp, C.POINTER(C.c_longlong),
                                  C.POINTER(C.c_longlong),
                                  C.POINTER(C.c_longlong)]),
    "swg_adj_memory": (C.c_int, [_vp, C.POINTER(C.c_longlong),
                                 C.POINTER(C.c_longlong),
                                 C.POINTER(C.c_longlong)]),
    "swg_checkpoint_cost": (C.c_longlong, [C.c_int, C.c_int]),
    "swg_fp64_issue_rate": (C.c_int, [C.c_int, C.c_int, _dp, _dp, _vp]),
    "swg_adj_plan": (C.c_int, [C.c_int, C.c_int, C.c_int,
                               C.POINTER(C.c_longlong),
                               C.POINTER(C.c_longlong)]),
    "swg_adj_schedule": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int,
                                   C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "swg_adj_grad_visc": (C.c_int, [_vp, _dp, _dp, _vp]),
    "swg_adj_batch_forward": (C.c_int, [C.c_int, C.POINTER(_vp),
                                        C.POINTER(_vp), C.c_double,
                                        C.c_double, C.c_int, C.POINTER(_vp),
                                        C.POINTER(_vp)]),
    "swg_adj_batch_backward": (C.c_int, [C.c_int, C.POINTER(_vp),
                                         C.POINTER(_vp), C.POINTER(_vp)]),
    "swg_adj_ensemble_create": (C.c_int, [C.c_int, C.POINTER(_vp),
                                          C.POINTER(_vp)]),
    "swg_adj_ensemble_destroy": (C.c_int, [_vp]),
    "swg_adj_ensemble_forward": (C.c_int, [_vp, C.POINTER(_vp), C.c_double,
                                           C.c_double, C.c_int,
                                           C.POINTER(_vp), _vp]),
    "swg_adj_ensemble_backward": (C.c_int, [_vp, C.POINTER(_vp), _vp]),
    "swg_adj_ensemble_groups": (C.c_int, [_vp, C.POINTER(C.c_int),
                                          C.POINTER(C.c_int)]),
    "swg_diag_mass": (C.c_int, [_vp, _vp, _dp, _vp]),
    "swg_diag_energy": (C.c_int, [_vp, _vp, _dp, _vp]),
    "swg_diag_circulation": (C.c_int, [_vp, _vp, _dp, _vp]),
    "swg_profile_enable": (C.c_int, [C.c_int]),
    "swg_profile_read": (C.c_int, [C.c_int, C.c_char_p, _dp,
                                   C.POINTER(C.c_longlong),
                                   C.POINTER(C.c_int)]),
    "swg_sync": (C.c_int, [_vp]),
}

_lib = None


def exported_symbols() -> list:
    """Every entry point declared in include/swgpu.h."""
    return list(_SIGS)


def lib() -> C.CDLL:
    """Load the in-tree CUDA library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(_build.LIB):
            raise RuntimeError(
                f"{_build.LIB} is missing: build the CUDA extension first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        L = C.CDLL(_build.LIB)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != SWG_OK:
        raise SwgError(rc, lib().swg_last_error().decode())
