"""The C-ABI library loads on a machine without a GPU, exports every entry
point include/swgpu.h declares, and rejects bad input on the host before any
CUDA call."""
import ctypes as C
import os
import re

import numpy as np

from omega_playground_gb300 import _build, _capi

HEADER = os.path.join(os.path.dirname(_build.PKG), "include", "swgpu.h")


def declared():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(swg_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    lib = _capi.lib()
    names = declared()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_capi.exported_symbols())


def test_version_and_launch_counter():
    assert b"sm_103a" in _capi.lib().swg_version()
    assert _capi.lib().swg_kernel_launches() >= 0


def _desc_for(nx, ny, K):
    from test_mesh_builder import product_tables
    t, _, _ = product_tables(nx, ny, 1.0)
    d = _capi.MeshDesc()
    d.ncells, d.nedges, d.nvertices, d.nlayers = nx * ny, 3 * nx * ny, \
        2 * nx * ny, K
    for n in ("nedges_on_cell", "edges_on_cell", "nedges_on_edge",
              "edges_on_edge", "cells_on_edge", "vertices_on_edge",
              "edges_on_vertex", "cells_on_vertex"):
        setattr(d, n, t[n].ctypes.data_as(C.POINTER(C.c_int)))
    for n in ("area_cell", "edge_sign_on_cell", "dc_edge", "dv_edge",
              "weights_on_edge", "area_triangle", "kiteareas_on_vertex",
              "edge_sign_on_vertex"):
        setattr(d, n, t[n].ctypes.data_as(C.POINTER(C.c_double)))
    return d, t


def test_mesh_create_rejects_out_of_range_connectivity():
    d, t = _desc_for(4, 4, 2)
    t["cells_on_edge"][5, 1] = 16  # == ncells: out of range
    out = C.c_void_p()
    rc = _capi.lib().swg_mesh_create(C.byref(d), C.byref(out))
    assert rc == 1 and not out.value
    assert b"out of range" in _capi.lib().swg_last_error()


def test_mesh_create_rejects_bad_sizes_and_nulls():
    d, _ = _desc_for(4, 4, 2)
    d.nlayers = 0
    out = C.c_void_p()
    assert _capi.lib().swg_mesh_create(C.byref(d), C.byref(out)) == 1
    d, _ = _desc_for(4, 4, 2)
    d.dc_edge = None
    assert _capi.lib().swg_mesh_create(C.byref(d), C.byref(out)) == 1
    assert b"NULL" in _capi.lib().swg_last_error()
    d, t = _desc_for(4, 4, 2)
    t["nedges_on_cell"][3] = 7
    assert _capi.lib().swg_mesh_create(C.byref(d), C.byref(out)) == 1


def test_mesh_create_rejects_max_levels_out_of_range():
    d, t = _desc_for(4, 4, 2)
    ml = np.full(16, 2, np.int32)
    ml[7] = 3  # > nlayers
    d.max_level_cell = ml.ctypes.data_as(C.POINTER(C.c_int))
    out = C.c_void_p()
    assert _capi.lib().swg_mesh_create(C.byref(d), C.byref(out)) == 1
    assert b"max level" in _capi.lib().swg_last_error()
    d, t = _desc_for(4, 4, 2)
    mv = np.full(32, -1, np.int32)
    d.max_level_vertex_bot = mv.ctypes.data_as(C.POINTER(C.c_int))
    assert _capi.lib().swg_mesh_create(C.byref(d), C.byref(out)) == 1


def test_null_handles_are_errors_not_crashes():
    lib = _capi.lib()
    assert lib.swg_state_create(None, 0, C.byref(C.c_void_p())) == 1
    assert lib.swg_model_create(None, None, C.byref(C.c_void_p())) == 1
    assert lib.swg_stepper_create(None, 0, 4, C.byref(C.c_void_p())) == 1
    assert lib.swg_step(None, None, 0.0, 1.0, 1, 0, None) == 1
    assert lib.swg_compute_tendency(None, None, None, 0.0, 0, None) == 1
    assert lib.swg_mesh_destroy(None) == 0
    # host-resident states
    out = C.c_void_p()
    assert lib.swg_host_stepper_create(None, 1, 5, 16, C.byref(out)) == 1
    assert not out.value
    levels = (C.c_int * 2)(3, 4)
    assert lib.swg_host_stepper_create_levels(None, 1, 5, 2, levels,
                                              C.byref(out)) == 1
    assert lib.swg_host_step(None, None, None, None, 0.0, 1.0, 1, None) == 1
    n = C.c_int(0)
    assert lib.swg_host_stepper_chunks(None, None, C.byref(n)) == 1
    assert lib.swg_host_stepper_destroy(None) == 0
    assert lib.swg_host_alloc(8, None) == 1
    assert lib.swg_host_free(None) == 0


def test_checkpoint_cost_matches_binomial_formula():
    """Plain advances of the optimal schedule equal Griewank-Walther's
    t(n, s) = r n - C(s + r, s + 1) with C(s + r - 1, s) < n <= C(s + r, s)
    (host-only planner, no GPU)."""
    from math import comb
    lib = _capi.lib()
    for n, s in [(1000, 32), (100, 5), (50, 1), (7, 3), (20, 4), (12, 12),
                 (300, 10)]:
        r = 0
        while comb(s + r, s) < n:
            r += 1
        t = r * n - comb(s + r, s + 1) if r > 0 else 0
        assert lib.swg_checkpoint_cost(n, s) == t, (n, s)
    assert lib.swg_checkpoint_cost(1000, 32) == 2405
    # outside the planner's range
    assert lib.swg_checkpoint_cost(10001, 32) == -1
    assert lib.swg_checkpoint_cost(0, 32) == -1
    assert lib.swg_checkpoint_cost(10, 0) == -1


def test_host_stepper_edge_layout():
    """Chunk layouts with small end chunks (host-state stepper autotuning)."""
    import omega_playground_gb300 as og
    assert og.HostStepper.edge_layout(64, 16, 8) == [8, 16, 16, 16, 8]
    assert og.HostStepper.edge_layout(64, 16, 4) == [4, 16, 16, 16, 8, 4]
    assert og.HostStepper.edge_layout(7, 3, 1) == [1, 3, 2, 1]
    assert og.HostStepper.edge_layout(6, 3, 3) == [6]
