"""Python mirror of omega_playground's C++ interface over the C ABI.

Class and member names follow the reference (src/mesh, src/model,
src/time_integration) so code written against it reads the same:

    mesh = PlanarHexagonalMesh(nx, ny, dc, nlayers)        # planar_hexagonal_mesh.hpp:8-28
    params = ShallowWaterParams(m_f0=1e-4, m_ntracers=1)   # shallow_water_params.hpp:7-18
    model = ShallowWaterModel(mesh, params)                # shallow_water_model.hpp:14-51
    state = ShallowWaterState(mesh, params)                # shallow_water_state.hpp:9-16
    stepper = LSRKStepper(model, 5)                        # time_stepper.hpp:16-25
    stepper.do_step(t, dt, state)                          # time_stepper.hpp:10-11
    mass_integral(state, model)                            # shallow_water_diagnostics.hpp:7-12

The state lives on the GPU; ``upload`` / ``download`` move numpy arrays
(FP64, [entity][k], tracers [l][cell][k]).  Every compute call is a CUDA
launch on ``stream`` (a raw cudaStream_t as int, default the legacy stream).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import enum
import weakref

import numpy as np

from . import _capi
from ._capi import check, lib

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def _d(a):
    if a is None:
        return None
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous float64 array")
    return a.ctypes.data_as(_dp)


def _i(a):
    if a is None:
        return None
    if a.dtype != np.int32 or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous int32 array")
    return a.ctypes.data_as(_ip)


def _s(stream):
    return C.c_void_p(int(stream)) if stream else None


class AddMode(enum.IntEnum):
    """shallow_water_model.hpp:11"""
    replace = 0
    increment = 1


class MPASMesh:
    """MPAS mesh tables (mpas_mesh.hpp:7-71) uploaded to the GPU.

    Subclasses (PlanarHexagonalMesh) fill ``tables``; ``finalize`` uploads
    them.  ``mesh_scaling_del2/4`` and ``edge_mask`` default to ones as in
    MPASMesh::finalize_mesh (mpas_mesh.cpp:48-50)."""

    maxedges = 6

    def __init__(self):
        self.tables = {}
        self._h = None

    @classmethod
    def from_tables(cls, tables: dict, nlayers: int, **finalize_kw):
        """A mesh from arbitrary MPAS tables (numpy arrays named like the
        reference's members without ``m_``: nedges_on_cell [C], edges_on_cell
        [C][6], nedges_on_edge [E], edges_on_edge [E][12], cells_on_edge,
        vertices_on_edge [E][2], edges_on_vertex, cells_on_vertex [V][3],
        area_cell, edge_sign_on_cell, dc_edge, dv_edge, weights_on_edge,
        area_triangle, kiteareas_on_vertex, edge_sign_on_vertex)."""
        m = cls.__new__(cls)
        MPASMesh.__init__(m)
        for k, v in tables.items():
            dt = np.int32 if np.asarray(v).dtype.kind in "iu" else np.float64
            m.tables[k] = np.ascontiguousarray(v, dt)
        m.m_ncells = len(m.tables["nedges_on_cell"])
        m.m_nedges = len(m.tables["nedges_on_edge"])
        m.m_nvertices = len(m.tables["area_triangle"])
        m.m_nlayers = int(nlayers)
        m.finalize(**finalize_kw)
        return m

    def finalize(self, mesh_scaling_del2=None, mesh_scaling_del4=None,
                 edge_mask=None, max_level_cell=None,
                 max_level_vertex_bot=None):
        t = self.tables
        d = _capi.MeshDesc()
        d.ncells, d.nedges, d.nvertices = self.m_ncells, self.m_nedges, \
            self.m_nvertices
        d.nlayers = self.m_nlayers
        for n in ("nedges_on_cell", "edges_on_cell", "nedges_on_edge",
                  "edges_on_edge", "cells_on_edge", "vertices_on_edge",
                  "edges_on_vertex", "cells_on_vertex"):
            setattr(d, n, _i(t[n]))
        for n in ("area_cell", "edge_sign_on_cell", "dc_edge", "dv_edge",
                  "weights_on_edge", "area_triangle", "kiteareas_on_vertex",
                  "edge_sign_on_vertex"):
            setattr(d, n, _d(t[n]))
        self._keep = [np.ascontiguousarray(x, np.float64) if x is not None
                      else None for x in (mesh_scaling_del2,
                                          mesh_scaling_del4, edge_mask)]
        d.mesh_scaling_del2 = _d(self._keep[0])
        d.mesh_scaling_del4 = _d(self._keep[1])
        d.edge_mask = _d(self._keep[2])
        self._keep_i = [np.ascontiguousarray(x, np.int32) if x is not None
                        else None for x in (max_level_cell,
                                            max_level_vertex_bot)]
        d.max_level_cell = _i(self._keep_i[0])
        d.max_level_vertex_bot = _i(self._keep_i[1])
        h = C.c_void_p()
        check(lib().swg_mesh_create(C.byref(d), C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def __getattr__(self, name):
        t = self.__dict__.get("tables")
        if t is not None and name.startswith("m_") and name[2:] in t:
            return t[name[2:]]
        raise AttributeError(name)

    def __del__(self):
        if getattr(self, "_h", None) and _capi._lib is not None:
            _capi._lib.swg_mesh_destroy(self._h)
            self._h = None


class PlanarHexagonalMesh(MPASMesh):
    """Doubly periodic planar hexagonal mesh (planar_hexagonal_mesh.cpp:5-62).

    ``dc`` defaults to 1/nx like the reference's 3-argument constructor."""

    def __init__(self, nx: int, ny: int, dc: float | None = None,
                 nlayers: int = 1, **finalize_kw):
        super().__init__()
        self.m_nx, self.m_ny = int(nx), int(ny)
        self.m_dc = float(1.0 / nx if dc is None else dc)
        self.m_nlayers = int(nlayers)
        self.m_ncells = nx * ny
        self.m_nedges = 3 * nx * ny
        self.m_nvertices = 2 * nx * ny
        sizes = {"C": self.m_ncells, "E": self.m_nedges, "V": self.m_nvertices}
        ht = _capi.HexTables()
        for name, (ent, w) in _capi.HEX_SHAPE.items():
            dt = np.int32 if name in _capi.HEX_INT else np.float64
            shape = (sizes[ent], w) if w > 1 else (sizes[ent],)
            self.tables[name] = np.zeros(shape, dt)
            setattr(ht, name, (_i if dt == np.int32 else _d)(self.tables[name]))
        px, py = C.c_double(), C.c_double()
        check(lib().swg_planar_hex_mesh_build(self.m_nx, self.m_ny, self.m_dc,
                                              C.byref(ht), C.byref(px),
                                              C.byref(py)))
        self.m_period_x, self.m_period_y = px.value, py.value
        self.finalize(**finalize_kw)

    @property
    def odd_row_seam(self) -> bool:
        """True for odd ny: the half-cell shift of alternate rows does not
        alternate across the periodic y boundary, so the reference's
        parallel construction writes some table slots twice (a race) and
        the rows meet irregularly there.  The tables are the reference's
        serial result."""
        return self.m_ny % 2 == 1


@dataclasses.dataclass
class ShallowWaterParams:
    """shallow_water_params.hpp:7-18"""
    m_f0: float = 0.0
    m_grav: float = 9.81
    m_drag_coeff: float = 0.0
    m_visc_del2: float = 0.0
    m_visc_del4: float = 0.0
    m_eddy_diff2: float = 0.0
    m_eddy_diff4: float = 0.0
    m_ntracers: int = 0
    m_disable_h_tendency: bool = False
    m_disable_vn_tendency: bool = False

    def _c(self):
        return _capi.Params(self.m_f0, self.m_grav, self.m_drag_coeff,
                            self.m_visc_del2, self.m_visc_del4,
                            self.m_eddy_diff2, self.m_eddy_diff4,
                            self.m_ntracers, int(self.m_disable_h_tendency),
                            int(self.m_disable_vn_tendency))


class _DeviceArray:
    """A dense float64 device array in the CUDA array interface (version 3)
    with a reference to the object that owns the memory."""

    def __init__(self, owner, ptr, shape):
        self.owner = owner
        self.__cuda_array_interface__ = {
            "shape": tuple(int(n) for n in shape), "typestr": "<f8",
            "data": (int(ptr), False), "strides": None, "version": 3,
            "stream": None}


class ShallowWaterState:
    """h_cell [C][K], vn_edge [E][K], tr_cell [T][C][K] on the GPU
    (shallow_water_state.cpp:7-14)."""

    def __init__(self, mesh: MPASMesh, params_or_ntracers=0):
        nt = (params_or_ntracers.m_ntracers
              if isinstance(params_or_ntracers, ShallowWaterParams)
              else int(params_or_ntracers))
        self.mesh, self.ntracers = mesh, nt
        h = C.c_void_p()
        check(lib().swg_state_create(mesh.handle, nt, C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def shapes(self):
        m = self.mesh
        return ((m.m_ncells, m.m_nlayers), (m.m_nedges, m.m_nlayers),
                (self.ntracers, m.m_ncells, m.m_nlayers))

    def upload(self, h, vn, tr=None, stream=None):
        sh, sv, st = self.shapes()
        h = np.ascontiguousarray(h, np.float64).reshape(sh)
        vn = np.ascontiguousarray(vn, np.float64).reshape(sv)
        tr = (np.ascontiguousarray(tr, np.float64).reshape(st)
              if self.ntracers else None)
        check(lib().swg_state_upload(self._h, _d(h), _d(vn), _d(tr),
                                     _s(stream)))
        lib().swg_sync(_s(stream))  # host arrays may be temporaries

    def download(self, stream=None, out=None):
        """Synchronous copy to host; `out` = (h, vn, tr) preallocated
        C-contiguous float64 arrays (e.g. pinned) or None for new ones."""
        sh, sv, st = self.shapes()
        if out is None:
            out = (np.empty(sh), np.empty(sv), np.empty(st))
        h, vn, tr = out
        check(lib().swg_state_download(self._h, _d(h), _d(vn),
                                       _d(tr) if self.ntracers else None,
                                       _s(stream)))
        return h, vn, tr

    def device_ptrs(self):
        p = [_dp(), _dp(), _dp()]
        check(lib().swg_state_device_ptrs(self._h, *[C.byref(x) for x in p]))
        return tuple(C.cast(x, C.c_void_p).value for x in p)

    def as_tensors(self):
        """Zero-copy torch views (h [C][K], vn [E][K], tr [T][C][K]) of the
        state's device memory, float64 on the state's GPU, valid while
        this state is alive.  The views carry no stream: order torch work
        against the state's own calls by running both on the same
        stream."""
        import torch
        out = []
        for ptr, shape in zip(self.device_ptrs(), self.shapes()):
            if int(np.prod(shape)) == 0:
                out.append(torch.empty(shape, dtype=torch.float64,
                                       device="cuda"))
            else:
                out.append(torch.as_tensor(_DeviceArray(self, ptr, shape),
                                           device="cuda"))
        return tuple(out)

    def copy_from(self, other: "ShallowWaterState", stream=None):
        check(lib().swg_state_copy(self._h, other._h, _s(stream)))

    def fill(self, value: float, stream=None):
        check(lib().swg_state_fill(self._h, float(value), _s(stream)))

    def __del__(self):
        if getattr(self, "_h", None) and _capi._lib is not None:
            _capi._lib.swg_state_destroy(self._h)
            self._h = None


# the reference's tendency-term members (shallow_water_model.hpp:19-29), in
# the order of swgpu.h's SWG_TERM_* numbers
TERMS = ("m_thickness_hadv_cell", "m_pv_flux_edge", "m_ke_grad_edge",
         "m_ssh_grad_edge", "m_vel_diff_edge", "m_vel_hyperdiff_edge",
         "m_tracer_hadv_cell", "m_tracer_diff_cell", "m_tracer_hyperdiff_cell")


class TendencyTerm:
    """One of the model's tendency terms; ``m_enabled`` reads and switches it
    like the reference member's flag (read at compute time)."""

    def __init__(self, model, term: int):
        # weak: the model owns its terms, a strong back-reference would make
        # a cycle and delay the model's release
        self._model, self._term = weakref.ref(model), term

    @property
    def m_enabled(self) -> bool:
        out = C.c_int()
        check(lib().swg_model_term_enabled(self._model().handle, self._term,
                                           C.byref(out)))
        return bool(out.value)

    @m_enabled.setter
    def m_enabled(self, on: bool):
        check(lib().swg_model_set_term_enabled(self._model().handle,
                                               self._term, int(bool(on))))


class ShallowWaterModel:
    """shallow_water_model.hpp:14-51.  Override ``additional_tendency`` to
    add forcing (it receives device pointers and the CUDA stream).

    ``apply_drag`` turns on the bottom drag with ``params.m_drag_coeff``
    (the term commented out at shallow_water_hierarchical.cpp:479-486); the
    reference's live model ignores the coefficient, and so does this one by
    default."""

    _linear_h0 = None

    def __init__(self, mesh: MPASMesh, params: ShallowWaterParams,
                 apply_drag: bool = False):
        self.m_mesh, self.m_params = mesh, params
        p = params._c()
        o = _capi.ModelOptions(int(self._linear_h0 is not None),
                               float(self._linear_h0 or 0.0), int(apply_drag))
        h = C.c_void_p()
        check(lib().swg_model_create_ex(mesh.handle, C.byref(p), C.byref(o),
                                        C.byref(h)))
        self._h = h
        for t, name in enumerate(TERMS):
            setattr(self, name, TendencyTerm(self, t))
        self._cb = None
        if type(self).additional_tendency is not \
                ShallowWaterModel.additional_tendency:
            def tramp(user, ht, vt, hp, vp, t, stream):
                self.additional_tendency(C.cast(ht, C.c_void_p).value,
                                         C.cast(vt, C.c_void_p).value,
                                         C.cast(hp, C.c_void_p).value,
                                         C.cast(vp, C.c_void_p).value, t,
                                         stream or 0)
            self._cb = _capi.FORCING_FN(tramp)
            check(lib().swg_model_set_forcing(self._h, self._cb, None))

    @property
    def handle(self):
        return self._h

    def additional_tendency(self, h_tend, vn_tend, h, vn, t, stream):
        """shallow_water_model.hpp:42-44 (no-op)."""

    def compute_tendency(self, tend: ShallowWaterState,
                         state: ShallowWaterState, t: float,
                         add_mode: AddMode = AddMode.replace, stream=None):
        check(lib().swg_compute_tendency(self._h, tend.handle, state.handle,
                                         float(t), int(add_mode), _s(stream)))

    def compute_aux(self, h, vn, tr=None, stream=None):
        """m_aux_state.compute(h, vn, tr, f_vertex, mesh)
        (shallow_water_auxstate.cpp:12-50) on device arrays: a
        ShallowWaterState's fields (state.device_ptrs()), torch tensors or
        raw device pointers; f_vertex is the model's own m_f_vertex."""
        check(lib().swg_model_compute_aux(self._h, _dev(h), _dev(vn),
                                          _dev(tr), _s(stream)))

    def compute_h_tendency(self, h_tend, h, vn, add_mode=AddMode.replace,
                           stream=None):
        """shallow_water_model.hpp:36-37: the thickness tendency from the
        last auxiliary state (its mean thickness) and vn."""
        check(lib().swg_compute_h_tendency(self._h, _dev(h_tend), _dev(h),
                                           _dev(vn), int(add_mode),
                                           _s(stream)))

    def compute_vn_tendency(self, vn_tend, h, vn, add_mode=AddMode.replace,
                            stream=None):
        """shallow_water_model.hpp:38-39: the normal-velocity tendency from
        the last auxiliary state, vn (PV flux) and h (SSH gradient)."""
        check(lib().swg_compute_vn_tendency(self._h, _dev(vn_tend), _dev(h),
                                            _dev(vn), int(add_mode),
                                            _s(stream)))

    def compute_tr_tendency(self, tr_tend, tr, vn, add_mode=AddMode.replace,
                            stream=None):
        """shallow_water_model.hpp:40-41: the tracer tendencies from the
        last auxiliary state (normalised tracers, mean thickness) and vn;
        tr is not read, as in the reference."""
        check(lib().swg_compute_tr_tendency(self._h, _dev(tr_tend), _dev(tr),
                                            _dev(vn), int(add_mode),
                                            _s(stream)))

    @property
    def m_aux_state(self):
        """Read-only view of the auxiliary state of the last evaluation:
        reference-named members holding host copies (see AuxStateView)."""
        return AuxStateView(self)

    def aux(self, name: str) -> np.ndarray:
        """Copy of a named intermediate of the last tendency evaluation."""
        p, n = _dp(), C.c_longlong()
        check(lib().swg_model_aux(self._h, name.encode(), C.byref(p),
                                  C.byref(n)))
        out = np.empty(n.value)
        cudart = _cudart()
        err = cudart.cudaMemcpy(out.ctypes.data_as(C.c_void_p),
                                C.cast(p, C.c_void_p), C.c_size_t(8 * n.value),
                                C.c_int(2))
        if err:
            raise _capi.SwgError(3, f"cudaMemcpy failed ({err})")
        return out

    @property
    def m_f_vertex(self) -> np.ndarray:
        """Copy of the Coriolis parameter per vertex (the reference's
        m_f_vertex, f0 after construction)."""
        return self.aux("f_vertex")

    @m_f_vertex.setter
    def m_f_vertex(self, f):
        """Writes the Coriolis parameter per vertex (e.g. a beta plane);
        every later evaluation reads it."""
        p, n = _dp(), C.c_longlong()
        check(lib().swg_model_aux(self._h, b"f_vertex", C.byref(p),
                                  C.byref(n)))
        f = np.ascontiguousarray(f, np.float64)
        if f.size != n.value:
            raise ValueError(f"f_vertex needs {n.value} values")
        err = _cudart().cudaMemcpy(C.cast(p, C.c_void_p),
                                   f.ctypes.data_as(C.c_void_p),
                                   C.c_size_t(8 * n.value), C.c_int(1))
        if err:
            raise _capi.SwgError(3, f"cudaMemcpy failed ({err})")

    def __del__(self):
        if getattr(self, "_h", None) and _capi._lib is not None:
            _capi._lib.swg_model_destroy(self._h)
            self._h = None


def _dev(x):
    """Device address of x: None, an int pointer, a torch tensor or an
    object with __cuda_array_interface__."""
    if x is None:
        return None
    if isinstance(x, int):
        return C.c_void_p(x)
    if hasattr(x, "data_ptr"):
        return C.c_void_p(x.data_ptr())
    if hasattr(x, "__cuda_array_interface__"):
        return C.c_void_p(x.__cuda_array_interface__["data"][0])
    raise TypeError(f"not a device array: {type(x).__name__}")


class AuxStateView:
    """The reference's ShallowWaterAuxiliaryState member groups
    (shallow_water_auxstate.hpp) over the model's intermediates, read when
    accessed (host copies).  The mean thickness is kept once
    (m_mean_h_edge is m_flux_h_edge); the vorticity terms are kept summed:
    m_pv_vertex = norm_rvort_vertex + norm_pvort_vertex and m_pv_edge =
    2 (norm_rvort_edge + norm_pvort_edge).  A member the configuration does
    not compute is None."""

    _GROUPS = {
        "m_thickness_aux": {"m_mean_h_edge": "mean_h_edge",
                            "m_flux_h_edge": "mean_h_edge"},
        "m_vorticity_aux": {"m_rvort_vertex": "rvort_vertex",
                            "m_pv_vertex": "q_vertex",
                            "m_pv_edge": "pv_edge"},
        "m_kinetic_aux": {"m_ke_cell": "ke_cell",
                          "m_vel_div_cell": "vel_div_cell"},
        "m_tracer_aux": {"m_norm_tr_cell": "norm_tr_cell"},
    }

    def __init__(self, model):
        self._model = model

    def compute(self, h, vn, tr=None, f_vertex=None, mesh=None, stream=None):
        """shallow_water_auxstate.cpp:12-50 (f_vertex: the model's own)."""
        self._model.compute_aux(h, vn, tr, stream)

    def __getattr__(self, group):
        names = AuxStateView._GROUPS.get(group)
        if names is None:
            raise AttributeError(group)
        model = self._model
        me = model.m_mesh
        rows = {"edge": me.m_nedges, "vertex": me.m_nvertices,
                "cell": me.m_ncells}

        class _Group:
            pass
        g = _Group()
        for member, name in names.items():
            try:
                a = model.aux(name)
            except _capi.SwgError:
                a = None
            if a is not None:
                n = rows[name.rsplit("_", 1)[1]]
                a = a.reshape(-1, n, me.m_nlayers) if name == "norm_tr_cell" \
                    else a.reshape(n, me.m_nlayers)
            setattr(g, member, a)
        return g


_cudart_lib = None


def _cudart():
    global _cudart_lib
    if _cudart_lib is None:
        lib()  # loads libcudart.so.13 as a dependency
        _cudart_lib = C.CDLL("libcudart.so.13")
        _cudart_lib.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t,
                                           C.c_int]
        _cudart_lib.cudaDeviceGetPCIBusId.argtypes = [C.c_char_p, C.c_int,
                                                      C.c_int]
    return _cudart_lib


@dataclasses.dataclass
class LinearShallowWaterParams(ShallowWaterParams):
    """ShallowWaterParams plus the resting thickness m_h0 of the linear
    model (shallow_water_hierarchical.cpp:676-678)."""
    m_h0: float = 1000.0


class LinearShallowWaterModel(ShallowWaterModel):
    """LinearShallowWaterModel (shallow_water_hierarchical.cpp:676-775):
    h_t = -h0 div(vn), vn_t = f0 sum_j w_j vn_j - g grad h; no tracers, no
    dissipation.  Same state, steppers and diagnostics as the nonlinear
    model; its energy integral weights the kinetic energy by h0."""

    def __init__(self, mesh: MPASMesh, params: LinearShallowWaterParams):
        self._linear_h0 = float(params.m_h0)
        super().__init__(mesh, params)


class TimeStepper:
    """time_stepper.hpp:8-14"""

    _kind = None

    def __init__(self, shallow_water: ShallowWaterModel, nstages: int = 0):
        self.m_shallow_water = shallow_water
        h = C.c_void_p()
        check(lib().swg_stepper_create(shallow_water.handle, self._kind,
                                       int(nstages), C.byref(h)))
        self._h = h

    def do_step(self, t: float, dt: float, state: ShallowWaterState,
                stream=None):
        check(lib().swg_step(self._h, state.handle, float(t), float(dt), 1, 0,
                             _s(stream)))

    def step(self, state: ShallowWaterState, t0: float, dt: float,
             nsteps: int, use_graph: bool = True, stream=None):
        """nsteps do_step calls (t0 + s*dt); replays a CUDA graph of one
        step when no forcing hook is set."""
        check(lib().swg_step(self._h, state.handle, float(t0), float(dt),
                             int(nsteps), int(use_graph), _s(stream)))

    def __del__(self):
        if getattr(self, "_h", None) and _capi._lib is not None:
            _capi._lib.swg_stepper_destroy(self._h)
            self._h = None


class RK4Stepper(TimeStepper):
    """time_stepper.hpp:27-38, rk4.cpp"""
    _kind = 0
    nstages = 4

    def __init__(self, shallow_water: ShallowWaterModel):
        super().__init__(shallow_water, 4)


class LSRKStepper(TimeStepper):
    """time_stepper.hpp:16-25, lsrk.cpp (nstages 5 or 1)"""
    _kind = 1

    def __init__(self, shallow_water: ShallowWaterModel, nstages: int = 5):
        self.m_nstages = nstages
        super().__init__(shallow_water, nstages)


def gpu_numa_node(device: int | None = None):
    """(NUMA node of the current GPU's PCI function, number of host NUMA
    nodes with CPUs); the node is None where the system does not say."""
    import glob
    import os
    nodes = [n for n in glob.glob("/sys/devices/system/node/node[0-9]*")
             if open(os.path.join(n, "cpulist")).read().strip()]
    node = None
    try:
        cudart = _cudart()
        dev = C.c_int(0)
        if device is None:
            cudart.cudaGetDevice(C.byref(dev))
        else:
            dev.value = int(device)
        bus = C.create_string_buffer(64)
        if cudart.cudaDeviceGetPCIBusId(bus, 64, dev) == 0:
            path = ("/sys/bus/pci/devices/" + bus.value.decode().lower()
                    + "/numa_node")
            v = int(open(path).read().strip())
            node = v if v >= 0 else None
    except Exception:
        node = None
    if node is None and len(nodes) == 1:
        node = int(nodes[0].rsplit("node", 1)[1])
    return node, len(nodes)


def _node_cpus(node: int):
    cpus = set()
    text = open(f"/sys/devices/system/node/node{node}/cpulist").read().strip()
    for part in text.split(","):
        if part:
            a, _, b = part.partition("-")
            cpus |= set(range(int(a), int(b or a) + 1))
    return cpus


def pinned_empty(shape) -> np.ndarray:
    """An uninitialised float64 array in page-locked host memory
    (swg_host_alloc), freed when the last array viewing it goes away.  On a
    host with several NUMA nodes the calling thread runs on the CPUs of the
    GPU's node while the memory is allocated and locked, so its pages come
    from the memory nearest the GPU (the thread's CPU set is restored
    afterwards; no GPU setting changes)."""
    import os
    shape = tuple(int(n) for n in np.atleast_1d(shape))
    n = int(np.prod(shape))
    p = C.c_void_p()
    node, nnodes = gpu_numa_node()
    saved = None
    if node is not None and nnodes > 1 and hasattr(os, "sched_setaffinity"):
        try:
            saved = os.sched_getaffinity(0)
            near = _node_cpus(node) & saved
            if near:
                os.sched_setaffinity(0, near)
            else:
                saved = None
        except OSError:
            saved = None
    try:
        check(lib().swg_host_alloc(max(n, 1) * 8, C.byref(p)))
    finally:
        if saved is not None:
            os.sched_setaffinity(0, saved)
    buf = (C.c_double * max(n, 1)).from_address(p.value)
    buf._owner = _PinnedBlock(p.value)
    return np.frombuffer(buf, np.float64, n).reshape(shape)


class _PinnedBlock:
    def __init__(self, ptr):
        self.ptr = ptr

    def __del__(self):
        if _capi._lib is not None:
            _capi._lib.swg_host_free(C.c_void_p(self.ptr))


class HostStepper:
    """Steps a state held in host arrays (h [C][K], vn [E][K], tr [T][C][K],
    C-contiguous float64) in place, in chunks of `level_chunk` levels whose
    copies overlap the other chunks' compute (swg_host_stepper_* in
    swgpu.h).  Bitwise equal to upload + step + download; arrays from
    pinned_empty let the copies overlap.  stepper is "rk4" or "lsrk"."""

    def __init__(self, model: ShallowWaterModel, stepper: str = "lsrk",
                 nstages: int = 5, level_chunk: int = 0, levels=None):
        """level_chunk: levels per chunk (0: one chunk); or levels: the
        chunk sizes one by one, adding up to the level count."""
        self.model = model
        h = C.c_void_p()
        kind = 0 if stepper == "rk4" else 1
        if levels is not None:
            arr = (C.c_int * len(levels))(*[int(n) for n in levels])
            check(lib().swg_host_stepper_create_levels(
                model.handle, kind, int(nstages), len(levels), arr,
                C.byref(h)))
        else:
            check(lib().swg_host_stepper_create(
                model.handle, kind, int(nstages), int(level_chunk),
                C.byref(h)))
        self._h = h

    @staticmethod
    def edge_layout(nlayers: int, chunk: int, edge: int):
        """Chunk sizes with `edge` levels first and last and chunks of
        `chunk` levels between them (the last of those ragged): the small
        end chunks shorten the copy-in before the first compute and the
        copy-out after the last."""
        K, c, e = int(nlayers), int(chunk), int(edge)
        if K <= 2 * e or c < 1:
            return [K]
        mid = [min(c, K - 2 * e - k) for k in range(0, K - 2 * e, c)]
        return [e] + mid + [e]

    @classmethod
    def autotuned(cls, model: ShallowWaterModel, stepper: str = "lsrk",
                  nstages: int = 5, state=None, dt: float = 1.0,
                  candidates=None, reps: int = 5):
        """The stepper whose chunk layout steps fastest on this machine,
        and {layout: ms per step}.  A candidate is a level chunk (int, 0:
        one chunk) or a list of chunk sizes; the default tries one chunk,
        chunks of 32, 16 and 8, chunks of 16 or 32 between end chunks of 4
        or 8 levels, and chunks of 12 or 8 between end chunks of 4.  Each candidate is timed (host wall clock, the call
        being synchronous) over `reps` one-step calls after one untimed
        call, on page-locked copies of `state` = (h, vn, tr) host arrays,
        which are left unchanged; a candidate's figure is the median of its
        calls, the figure back-to-back calls reach (the fastest single call
        overstates it when the host link is shared).  The fastest layout
        depends on the host link."""
        import time
        K = model.m_mesh.m_nlayers
        if candidates is None:
            candidates = [0, 32, 16, 8] + [cls.edge_layout(K, c, e)
                                           for c, e in ((16, 4), (16, 8),
                                                        (32, 8), (12, 4),
                                                        (8, 4))]
        layouts = {}
        for c in candidates:
            if isinstance(c, (list, tuple)):
                layout = [int(n) for n in c]
            else:
                c = min(int(c), K) if c > 0 else K
                layout = [min(c, K - k) for k in range(0, K, c)]
            layouts[",".join(map(str, layout))] = layout
        best, table = None, {}
        for key, layout in layouts.items():
            hs = cls(model, stepper, nstages, levels=layout)
            arrs = hs.pinned_state()
            if state is not None:
                for a, b in zip(arrs, state):
                    if a.size:
                        a[...] = b
            else:
                for a in arrs:
                    a.fill(1.0)
            hs.step(*arrs, 0.0, dt, 1)
            times = []
            for _ in range(reps):  # one call per step: copies every step
                t0 = time.perf_counter()
                hs.step(*arrs, 0.0, dt, 1)
                times.append((time.perf_counter() - t0) * 1e3)
            table[key] = float(np.median(times))
            if best is None or table[key] < table[best[0]]:
                best = (key, hs)
        return best[1], table

    @property
    def chunks(self):
        """Levels of each chunk."""
        n = C.c_int(0)
        check(lib().swg_host_stepper_chunks(self._h, None, C.byref(n)))
        out = (C.c_int * n.value)()
        check(lib().swg_host_stepper_chunks(self._h, out, C.byref(n)))
        return list(out)

    def pinned_state(self):
        """(h, vn, tr) page-locked host arrays of the model's state shapes."""
        m, T = self.model.m_mesh, self.model.m_params.m_ntracers
        return (pinned_empty((m.m_ncells, m.m_nlayers)),
                pinned_empty((m.m_nedges, m.m_nlayers)),
                pinned_empty((T, m.m_ncells, m.m_nlayers)))

    def step(self, h, vn, tr, t0: float, dt: float, nsteps: int = 1,
             stream=None):
        m, T = self.model.m_mesh, self.model.m_params.m_ntracers
        want = ((m.m_ncells, m.m_nlayers), (m.m_nedges, m.m_nlayers),
                (T, m.m_ncells, m.m_nlayers))
        arrs = (h, vn, tr)
        for name, a, shape in zip(("h", "vn", "tr"), arrs, want):
            if a is None and name == "tr" and T == 0:
                continue
            if not isinstance(a, np.ndarray) or a.dtype != np.float64 or \
                    not a.flags.c_contiguous or not a.flags.writeable or \
                    a.size != int(np.prod(shape)):
                raise TypeError(f"{name}: expected a writeable C-contiguous "
                                f"float64 array of shape {shape}")
        check(lib().swg_host_step(self._h, _d(h), _d(vn),
                                  _d(tr) if T else None, float(t0),
                                  float(dt), int(nsteps), _s(stream)))

    def __del__(self):
        if getattr(self, "_h", None) and _capi._lib is not None:
            _capi._lib.swg_host_stepper_destroy(self._h)
            self._h = None


class Batch:
    """Ensemble of independent members (uneven nx, levels, tracers) advanced
    together by one persistent kernel per RK stage (swg_batch_* in swgpu.h).
    Members are (ShallowWaterModel, ShallowWaterState) pairs."""

    def __init__(self, models, states, kind: str = "rk4", nstages: int = 4):
        n = len(models)
        assert n == len(states) and n > 0
        self.models, self.states = list(models), list(states)
        mh = (C.c_void_p * n)(*[m.handle.value for m in models])
        sh = (C.c_void_p * n)(*[s.handle.value for s in states])
        h = C.c_void_p()
        check(lib().swg_batch_create(n, mh, sh, 0 if kind == "rk4" else 1,
                                     int(nstages), C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def step(self, t0: float, dt: float, nsteps: int, use_graph: bool = True,
             stream=None, check_status: bool = True):
        check(lib().swg_batch_step(self._h, float(t0), float(dt), int(nsteps),
                                   int(use_graph), _s(stream)))
        if check_status:
            self.check(stream)

    def check(self, stream=None):
        check(lib().swg_batch_check(self._h, _s(stream)))

    @staticmethod
    def config_count() -> int:
        return int(lib().swg_batch_config_count())

    def set_config(self, config: int):
        check(lib().swg_batch_set_config(self._h, int(config)))

    def autotune(self, dt: float, reps: int = 2, stream=None):
        """Times every launch configuration and keeps the fastest; returns
        (config, ms per step).  The tuning steps advance the members."""
        best, ms = C.c_int(), C.c_double()
        check(lib().swg_batch_autotune(self._h, float(dt), int(reps),
                                       _s(stream), C.byref(best), C.byref(ms)))
        return best.value, ms.value

    def selftest_timeout(self, limit_ms: float = 50.0, stream=None) -> int:
        """Status code of a barrier wait that nothing releases."""
        return int(lib().swg_batch_selftest_timeout(self._h, float(limit_ms),
                                                    _s(stream)))

    def __del__(self):
        if getattr(self, "_h", None) and _capi._lib is not None:
            _capi._lib.swg_batch_destroy(self._h)
            self._h = None


class Adjoint:
    """Tangent-linear and adjoint models of the RK4 step, or of the
    low-storage RK step (stepper="lsrk", nstages 5 or 1), with binomial
    checkpointing (swg_adjoint_* / swg_tlm_* / swg_adj_* in swgpu.h)."""

    def __init__(self, model: ShallowWaterModel, nsnapshots: int = 32,
                 stepper: str = "rk4", nstages: int = 4):
        self.model = model
        h = C.c_void_p()
        kind = 0 if stepper == "rk4" else 1
        check(lib().swg_adjoint_create_stepper(model.handle, int(nsnapshots),
                                               kind, int(nstages),
                                               C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def tlm_tendency(self, x, dx, dtend, stream=None):
        check(lib().swg_tlm_tendency(self._h, x.handle, dx.handle,
                                     dtend.handle, _s(stream)))

    def adj_tendency(self, x, mu, lam, stream=None):
        check(lib().swg_adj_tendency(self._h, x.handle, mu.handle, lam.handle,
                                     _s(stream)))

    def tlm_apply(self, x0, dx, t0, dt, nsteps, stream=None):
        check(lib().swg_tlm_apply(self._h, x0.handle, dx.handle, float(t0),
                                  float(dt), int(nsteps), _s(stream)))

    def forward(self, state0, t0, dt, nsteps, final, stream=None):
        check(lib().swg_adj_forward(self._h, state0.handle, float(t0),
                                    float(dt), int(nsteps), final.handle,
                                    _s(stream)))

    def backward(self, lam, stream=None):
        check(lib().swg_adj_backward(self._h, lam.handle, _s(stream)))

    def grad_visc(self, stream=None):
        """(dL/dvisc per edge, dL/dvisc per cell) of the last backward."""
        me = self.model.m_mesh
        ge = np.empty(me.m_nedges)
        gc = np.empty(me.m_ncells)
        check(lib().swg_adj_grad_visc(self._h, _d(ge), _d(gc), _s(stream)))
        return ge, gc

    def info(self):
        """(plain re-advanced steps, taped steps) of the last sweep pair."""
        a, b = C.c_longlong(), C.c_longlong()
        check(lib().swg_adj_info(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def info_ex(self):
        """(plain steps, taped steps, taped advances among them)."""
        a, b, c = C.c_longlong(), C.c_longlong(), C.c_longlong()
        check(lib().swg_adj_info_ex(self._h, C.byref(a), C.byref(b),
                                    C.byref(c)))
        return a.value, b.value, c.value

    def memory(self):
        """Device bytes: (one snapshot, one tape, everything held)."""
        a, b, c = C.c_longlong(), C.c_longlong(), C.c_longlong()
        check(lib().swg_adj_memory(self._h, C.byref(a), C.byref(b),
                                   C.byref(c)))
        return a.value, b.value, c.value

    def __del__(self):
        if getattr(self, "_h", None) and _capi._lib is not None:
            _capi._lib.swg_adjoint_destroy(self._h)
            self._h = None


def _handles(objs):
    return (C.c_void_p * len(objs))(*[o.handle.value for o in objs])


def _streams(streams, n):
    if streams is None:
        return None
    return (C.c_void_p * n)(*[int(s) if s else None for s in streams])


def adjoint_batch_forward(adjs, states0, t0, dt, nsteps, finals,
                          streams=None):
    """Forward sweeps of several members' adjoints, interleaved, member m on
    streams[m] (raw cudaStream_t ints)."""
    n = len(adjs)
    check(lib().swg_adj_batch_forward(n, _handles(adjs), _handles(states0),
                                      float(t0), float(dt), int(nsteps),
                                      _handles(finals), _streams(streams, n)))


def adjoint_batch_backward(adjs, lambdas, streams=None):
    n = len(adjs)
    check(lib().swg_adj_batch_backward(n, _handles(adjs), _handles(lambdas),
                                       _streams(streams, n)))


class AdjointEnsemble:
    """The members' checkpointed adjoints advanced together: every action of
    the checkpoint schedule is one batched launch per pass over the members
    (swg_adj_ensemble_* in swgpu.h).  Members are Adjoint objects with
    distinct models; each keeps its own snapshot budget."""

    def __init__(self, adjoints):
        self.adjoints = list(adjoints)
        h = C.c_void_p()
        check(lib().swg_adj_ensemble_create(len(self.adjoints),
                                            _handles(self.adjoints),
                                            C.byref(h)))
        self._h = h

    def forward(self, states0, t0, dt, nsteps, finals, stream=None):
        check(lib().swg_adj_ensemble_forward(self._h, _handles(states0),
                                             float(t0), float(dt),
                                             int(nsteps), _handles(finals),
                                             _s(stream)))

    def backward(self, lambdas, stream=None):
        check(lib().swg_adj_ensemble_backward(self._h, _handles(lambdas),
                                              _s(stream)))

    def groups(self):
        """(number of lockstep groups, each member's group)."""
        n = C.c_int()
        of = (C.c_int * len(self.adjoints))()
        check(lib().swg_adj_ensemble_groups(self._h, C.byref(n), of))
        return n.value, list(of)

    def __del__(self):
        if getattr(self, "_h", None) and _capi._lib is not None:
            _capi._lib.swg_adj_ensemble_destroy(self._h)
            self._h = None


def checkpoint_cost(nsteps: int, nsnapshots: int) -> int:
    """Plain forward steps of the classic optimal binomial checkpointing
    schedule with one tape (Griewank-Walther)."""
    return int(lib().swg_checkpoint_cost(int(nsteps), int(nsnapshots)))


def adjoint_plan(nsteps: int, nsnapshots: int, nstages: int = 4):
    """(plain advances, taped advances) of the schedule the adjoint runs
    for nsteps steps and nsnapshots snapshots (nstages 4: RK4; 5, 1: LSRK)."""
    a, b = C.c_longlong(), C.c_longlong()
    check(lib().swg_adj_plan(int(nsteps), int(nsnapshots), int(nstages),
                             C.byref(a), C.byref(b)))
    return a.value, b.value


def fp64_issue_rate(op: str = "dfma", iters: int = 20000, stream=None):
    """(thread-instructions/s, kernel ms) of FP64 `op` ('dfma', 'dadd',
    'dmul') on the current GPU, every SM filled (blocking)."""
    code = {"dfma": 0, "dadd": 1, "dmul": 2}[op]
    r, ms = C.c_double(), C.c_double()
    check(lib().swg_fp64_issue_rate(code, int(iters), C.byref(r), C.byref(ms),
                                    _s(stream)))
    return r.value, ms.value


def _diag(fn, state, model, stream=None):
    out = C.c_double()
    check(fn(model.handle, state.handle, C.byref(out), _s(stream)))
    return out.value


def mass_integral(state, model, stream=None):
    """shallow_water_diagnostics.cpp:40-58"""
    return _diag(lib().swg_diag_mass, state, model, stream)


def energy_integral(state, model, stream=None):
    """shallow_water_diagnostics.cpp:5-38"""
    return _diag(lib().swg_diag_energy, state, model, stream)


def circulation_integral(state, model, stream=None):
    """shallow_water_diagnostics.cpp:60-89"""
    return _diag(lib().swg_diag_circulation, state, model, stream)


def sync(stream=None):
    check(lib().swg_sync(_s(stream)))


def kernel_launches() -> int:
    return int(lib().swg_kernel_launches())


def profile_enable(on: bool = True) -> None:
    """Per-kernel CUDA-event timing of subsequent tendency launches."""
    check(lib().swg_profile_enable(int(on)))


def profile_read(max_kernels: int = 16) -> dict:
    """{kernel name: (total ms, launches)} recorded since the last read."""
    names = C.create_string_buffer(32 * max_kernels)
    ms = (C.c_double * max_kernels)()
    n = (C.c_longlong * max_kernels)()
    cnt = C.c_int()
    check(lib().swg_profile_read(max_kernels, names, ms, n, C.byref(cnt)))
    out = {}
    for j in range(cnt.value):
        nm = names.raw[32 * j:32 * j + 32].split(b"\0")[0].decode()
        out[nm] = (ms[j], int(n[j]))
    return out
