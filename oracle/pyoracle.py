"""ctypes binding for the CPU oracle (``swe_oracle.c``).

TEST INFRASTRUCTURE ONLY.  Imported by ``tests/``, ``__graft_entry__.smoke``
and the CPU-baseline leg of ``bench.py``; the product package never imports
it.  The oracle restates the omega_playground reference (see
``swe_oracle.h``); this module builds it, builds planar hexagonal meshes with
it and runs tendencies, steppers and diagnostics on numpy arrays.

It also reads and writes the named-array files exchanged with
``oracle/_ref/ref_driver`` (the reference's own sources compiled against the
host-only Kokkos shim), which ``tests/golden/make_golden.py`` uses to record
golden vectors.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libswe_oracle.so")
REF_DRIVER = os.path.join(HERE, "_ref", "ref_driver")

_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)

_MESH_INT = [
    ("nedges_on_cell", "C", 1), ("edges_on_cell", "C", 6),
    ("cells_on_cell", "C", 6), ("vertices_on_cell", "C", 6),
    ("kite_index_on_cell", "C", 6), ("nedges_on_edge", "E", 1),
    ("edges_on_edge", "E", 12), ("cells_on_edge", "E", 2),
    ("vertices_on_edge", "E", 2), ("edges_on_vertex", "V", 3),
    ("cells_on_vertex", "V", 3),
]
_MESH_DBL = [
    ("area_cell", "C", 1), ("x_cell", "C", 1), ("y_cell", "C", 1),
    ("edge_sign_on_cell", "C", 6), ("dc_edge", "E", 1), ("dv_edge", "E", 1),
    ("angle_edge", "E", 1), ("x_edge", "E", 1), ("y_edge", "E", 1),
    ("weights_on_edge", "E", 12), ("mesh_scaling_del2", "E", 1),
    ("mesh_scaling_del4", "E", 1), ("edge_mask", "E", "K"),
    ("area_triangle", "V", 1), ("x_vertex", "V", 1), ("y_vertex", "V", 1),
    ("kiteareas_on_vertex", "V", 3), ("edge_sign_on_vertex", "V", 3),
]


class _Mesh(C.Structure):
    _fields_ = ([("nx", C.c_int), ("ny", C.c_int), ("ncells", C.c_int),
                 ("nedges", C.c_int), ("nvertices", C.c_int),
                 ("nlayers", C.c_int), ("dc", C.c_double),
                 ("period_x", C.c_double), ("period_y", C.c_double)]
                + [(n, _ip) for n, _, _ in _MESH_INT]
                + [(n, _dp) for n, _, _ in _MESH_DBL]
                + [("max_level_cell", _ip), ("max_level_vertex_bot", _ip)])


class _Params(C.Structure):
    _fields_ = [("f0", C.c_double), ("grav", C.c_double),
                ("drag_coeff", C.c_double), ("visc_del2", C.c_double),
                ("visc_del4", C.c_double), ("eddy_diff2", C.c_double),
                ("eddy_diff4", C.c_double), ("ntracers", C.c_int),
                ("disable_h_tendency", C.c_int),
                ("disable_vn_tendency", C.c_int)]


def build(with_reference: bool | None = None) -> None:
    """Compile the oracle (and, where the reference checkout is present, the
    reference-against-shim driver) with the Makefile in this directory."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    ref = os.environ.get("OMEGA_REFERENCE", "/root/reference")
    if with_reference is None:
        with_reference = os.path.isdir(os.path.join(ref, "src"))
    if with_reference:
        subprocess.run(["make", "-s", "-C", HERE, f"REF={ref}", "ref", "-j8"],
                       check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(with_reference=False)
        L = C.CDLL(LIB_PATH)
        L.or_planar_hex_build.argtypes = [C.POINTER(_Mesh), C.c_int, C.c_int,
                                          C.c_double, C.c_int]
        L.or_model_create.argtypes = [C.POINTER(_Mesh), C.POINTER(_Params)]
        L.or_model_create.restype = C.c_void_p
        L.or_model_create_ex.argtypes = [C.POINTER(_Mesh), C.POINTER(_Params),
                                         C.c_int, C.c_double, C.c_int]
        L.or_model_create_ex.restype = C.c_void_p
        L.or_model_set_term.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.or_model_set_term.restype = C.c_int
        L.or_model_destroy.argtypes = [C.c_void_p]
        L.or_model_aux.argtypes = [C.c_void_p, C.c_char_p,
                                   C.POINTER(C.c_size_t)]
        L.or_model_aux.restype = _dp
        L.or_compute_tendency.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp,
                                          _dp, _dp, C.c_double, C.c_int]
        L.or_aux_compute.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.or_h_tendency.argtypes = [C.c_void_p, _dp, _dp, C.c_int]
        L.or_vn_tendency.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_int]
        L.or_tr_tendency.argtypes = [C.c_void_p, _dp, _dp, C.c_int]
        L.or_step.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _dp,
                              C.c_double, C.c_double, C.c_int]
        L.or_step.restype = C.c_int
        for f in ("or_mass_integral", "or_circulation_integral"):
            getattr(L, f).argtypes = [C.c_void_p, _dp]
            getattr(L, f).restype = C.c_double
        L.or_energy_integral.argtypes = [C.c_void_p, _dp, _dp]
        L.or_energy_integral.restype = C.c_double
        L.or_num_threads.restype = C.c_int
        _lib = L
    return _lib


def _ptr(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def _dptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return _ptr(a, C.c_double)


class OracleMesh:
    """PlanarHexagonalMesh(nx, ny, dc, nlayers) built by the oracle; the
    tables are numpy arrays named like the reference's MPASMesh members."""

    def __init__(self, nx: int, ny: int, dc: float, nlayers: int = 1):
        self.nx, self.ny, self.dc, self.nlayers = nx, ny, float(dc), nlayers
        C_, E, V = nx * ny, 3 * nx * ny, 2 * nx * ny
        dims = {"C": C_, "E": E, "V": V, "K": nlayers}
        self.ncells, self.nedges, self.nvertices = C_, E, V
        self.tables = {}
        for name, ent, w in _MESH_INT:
            w = dims[w] if isinstance(w, str) else w
            self.tables[name] = np.zeros((dims[ent], w) if w > 1 else dims[ent],
                                         np.int32)
        for name, ent, w in _MESH_DBL:
            w = dims[w] if isinstance(w, str) else w
            self.tables[name] = np.zeros((dims[ent], w) if w > 1 else dims[ent],
                                         np.float64)
        self._s = _Mesh()
        for name, _, _ in _MESH_INT:
            setattr(self._s, name, _ptr(self.tables[name], C.c_int))
        for name, _, _ in _MESH_DBL:
            setattr(self._s, name, _ptr(self.tables[name], C.c_double))
        lib().or_planar_hex_build(C.byref(self._s), nx, ny, self.dc, nlayers)
        self.period_x, self.period_y = self._s.period_x, self._s.period_y

    def set_max_levels(self, max_level_cell=None, max_level_vertex_bot=None):
        """Per-column level counts for the diagnostics (None = nlayers)."""
        for name, a in (("max_level_cell", max_level_cell),
                        ("max_level_vertex_bot", max_level_vertex_bot)):
            if a is None:
                self.tables.pop(name, None)
                setattr(self._s, name, None)
            else:
                self.tables[name] = np.ascontiguousarray(a, np.int32)
                setattr(self._s, name, _ptr(self.tables[name], C.c_int))

    def __getattr__(self, name):
        t = self.__dict__.get("tables")
        if t is not None and name in t:
            return t[name]
        raise AttributeError(name)


class OracleModel:
    """ShallowWaterModel + its steppers on the oracle."""

    def __init__(self, mesh: OracleMesh, *, f0=0.0, grav=9.81, visc_del2=0.0,
                 visc_del4=0.0, eddy_diff2=0.0, eddy_diff4=0.0, ntracers=0,
                 disable_h_tendency=False, disable_vn_tendency=False,
                 drag_coeff=0.0, apply_drag=False, linear_h0=None):
        """linear_h0: the linear model with that resting thickness;
        apply_drag: the opt-in bottom drag with drag_coeff."""
        self.mesh = mesh
        self.ntracers = ntracers
        self._p = _Params(f0, grav, drag_coeff, visc_del2, visc_del4,
                          eddy_diff2, eddy_diff4, ntracers,
                          int(disable_h_tendency), int(disable_vn_tendency))
        self._h = lib().or_model_create_ex(
            C.byref(mesh._s), C.byref(self._p), int(linear_h0 is not None),
            float(linear_h0 or 0.0), int(apply_drag))

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.or_model_destroy(self._h)
            self._h = None

    def shapes(self):
        m = self.mesh
        return ((m.ncells, m.nlayers), (m.nedges, m.nlayers),
                (self.ntracers, m.ncells, m.nlayers))

    def aux(self, name: str) -> np.ndarray:
        n = C.c_size_t()
        p = lib().or_model_aux(self._h, name.encode(), C.byref(n))
        if not p:
            raise KeyError(name)
        return np.ctypeslib.as_array(p, shape=(n.value,)).copy()

    def set_f_vertex(self, f):
        """Writes the Coriolis parameter per vertex (m_f_vertex)."""
        n = C.c_size_t()
        p = lib().or_model_aux(self._h, b"f_vertex", C.byref(n))
        np.ctypeslib.as_array(p, shape=(n.value,))[:] = f

    def set_term(self, term: int, enabled: bool):
        """A term member's m_enabled (terms numbered as SWG_TERM_*)."""
        if lib().or_model_set_term(self._h, int(term), int(bool(enabled))):
            raise ValueError("unknown term")

    def compute_tendency(self, h, vn, tr, t=0.0, add_mode=0, tend=None):
        sh, sv, st = self.shapes()
        if tend is None:
            tend = (np.zeros(sh), np.zeros(sv), np.zeros(st))
        th, tv, tt = tend
        tr = tr if tr is not None else np.zeros(st)
        lib().or_compute_tendency(self._h, _dptr(th), _dptr(tv), _dptr(tt),
                                  _dptr(h), _dptr(vn), _dptr(tr), t, add_mode)
        return th, tv, tt

    def compute_aux(self, h, vn, tr):
        """m_aux_state.compute (shallow_water_auxstate.cpp:12-50)."""
        tr = tr if tr is not None else np.zeros(self.shapes()[2])
        lib().or_aux_compute(self._h, _dptr(h), _dptr(vn), _dptr(tr))

    def compute_h_tendency(self, h_tend, vn, add_mode=0):
        """compute_h_tendency (shallow_water_model.cpp:43-84) from the last
        auxiliary state and vn; h_tend in place."""
        lib().or_h_tendency(self._h, _dptr(h_tend), _dptr(vn), add_mode)
        return h_tend

    def compute_vn_tendency(self, vn_tend, h, vn, add_mode=0):
        """compute_vn_tendency (shallow_water_model.cpp:86-219)."""
        lib().or_vn_tendency(self._h, _dptr(vn_tend), _dptr(h), _dptr(vn),
                             add_mode)
        return vn_tend

    def compute_tr_tendency(self, tr_tend, vn, add_mode=0):
        """compute_tr_tendency (shallow_water_model.cpp:221-311): the
        normalised tracers come from the auxiliary state."""
        lib().or_tr_tendency(self._h, _dptr(tr_tend), _dptr(vn), add_mode)
        return tr_tend

    def step(self, h, vn, tr, t0, dt, nsteps, kind="lsrk", nstages=5):
        """In place on (h, vn, tr); kind 'rk4' or 'lsrk'."""
        tr = tr if tr is not None else np.zeros(self.shapes()[2])
        rc = lib().or_step(self._h, 0 if kind == "rk4" else 1, nstages,
                           _dptr(h), _dptr(vn), _dptr(tr), t0, dt, nsteps)
        if rc:
            raise ValueError("unsupported stepper")
        return h, vn, tr

    def mass(self, h):
        return lib().or_mass_integral(self._h, _dptr(h))

    def energy(self, h, vn):
        return lib().or_energy_integral(self._h, _dptr(h), _dptr(vn))

    def circulation(self, vn):
        return lib().or_circulation_integral(self._h, _dptr(vn))


# ----------------------------------------------------- named-array files ---

def write_named(path: str, arrays: dict) -> None:
    with open(path, "wb") as f:
        for name, a in arrays.items():
            a = np.ascontiguousarray(a)
            if a.dtype.kind in "iu":
                a, dt = a.astype(np.int32), b"i"
            else:
                a, dt = a.astype(np.float64), b"d"
            f.write(name.encode().ljust(32, b"\0")[:32])
            f.write(dt)
            f.write(np.int32(a.ndim).tobytes())
            f.write(np.asarray(a.shape, np.int64).tobytes())
            f.write(a.tobytes())


def read_named(path: str) -> dict:
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    while pos < len(data):
        name = data[pos:pos + 32].split(b"\0")[0].decode()
        dt = data[pos + 32:pos + 33]
        nd = int(np.frombuffer(data, np.int32, 1, pos + 33)[0])
        dims = tuple(np.frombuffer(data, np.int64, nd, pos + 37))
        pos += 37 + 8 * nd
        n = int(np.prod(dims)) if nd else 1
        typ, sz = (np.float64, 8) if dt == b"d" else (np.int32, 4)
        out[name] = np.frombuffer(data, typ, n, pos).reshape(dims).copy()
        pos += n * sz
    return out


def run_ref_driver(inputs: dict, workdir: str) -> dict:
    """Run oracle/_ref/ref_driver on one scenario (see ref_driver.cpp)."""
    inp = os.path.join(workdir, "in.bin")
    out = os.path.join(workdir, "out.bin")
    write_named(inp, inputs)
    subprocess.run([REF_DRIVER, inp, out], check=True)
    return read_named(out)
