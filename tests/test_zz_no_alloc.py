"""swg_compute_tendency_noalloc: the tendency entry point for callers that
cannot allocate device memory while they run.  It keeps its parameter tables
and intermediate fields in a static 64 MiB device array instead of
model-owned buffers, so here it is checked through the C ABI against the
allocating entry point, swg_compute_tendency, on two calls in a row (the
second reuses the array the first one wrote); its size limit is checked, and
so is the reason it exists: a warm call at the largest documented size
leaves the device's free memory unchanged.

This file is named to be collected last so that a run stopping at its first
failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

import omega_playground_gb300 as og
from helpers import load_golden, rel_diff
from omega_playground_gb300 import _capi
from omega_playground_gb300.workloads import WORKLOADS, initial_state

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _setup(cfg):
    mesh = og.PlanarHexagonalMesh(cfg["nx"], cfg["ny"], cfg["dc"], cfg["K"])
    params = og.ShallowWaterParams(
        m_f0=cfg["f0"], m_grav=cfg["grav"], m_visc_del2=cfg["visc_del2"],
        m_visc_del4=cfg["visc_del4"], m_eddy_diff2=cfg["eddy_diff2"],
        m_eddy_diff4=cfg["eddy_diff4"], m_ntracers=cfg["T"],
        m_disable_h_tendency=cfg.get("disable_h", False),
        m_disable_vn_tendency=cfg.get("disable_vn", False))
    return mesh, params


def _noalloc(mesh, params, state, tend, add_mode=0):
    h, vn, tr = state.device_ptrs()
    th, tv, tt = tend.device_ptrs()
    p = params._c()
    T = params.m_ntracers
    rc = _capi.lib().swg_compute_tendency_noalloc(
        mesh.handle, C.byref(p), C.c_void_p(h), C.c_void_p(vn),
        C.c_void_p(tr) if T else None, C.c_void_p(th), C.c_void_p(tv),
        C.c_void_p(tt) if T else None, add_mode, None)
    return rc


def _free_device_bytes():
    """cudaMemGetInfo's free byte count of the current device."""
    from omega_playground_gb300.shallow_water import _cudart
    free, total = C.c_size_t(0), C.c_size_t(0)
    assert _cudart().cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value


def _allocating(mesh, params, state):
    model = og.ShallowWaterModel(mesh, params)
    tend = og.ShallowWaterState(mesh, params)
    model.compute_tendency(tend, state, 0.0)
    return tend.download()


def test_noalloc_matches_compute_tendency_two_calls():
    # call 1: every term on, two tracers (golden inputs)
    g = load_golden("rk4_all_terms")
    cfg = g["cfg"]
    mesh1, params1 = _setup(cfg)
    s1 = og.ShallowWaterState(mesh1, params1)
    s1.upload(g["in_h"], g["in_vn"], g["in_tr"])
    # call 2: a different mesh, parameter set and state (three tracers,
    # velocity noise), so the second call reuses the array differently
    wl = WORKLOADS["lsrk5_512x512"].scaled(nx=24, ny=20, nlayers=37,
                                           ntracers=3)
    cfg2 = dict(nx=wl.nx, ny=wl.ny, dc=wl.dc, K=wl.nlayers, T=wl.ntracers,
                f0=wl.f0, grav=wl.grav, visc_del2=wl.visc_del2,
                visc_del4=wl.visc_del4, eddy_diff2=wl.eddy_diff2,
                eddy_diff4=wl.eddy_diff4)
    mesh2, params2 = _setup(cfg2)
    s2 = og.ShallowWaterState(mesh2, params2)
    s2.upload(*initial_state(mesh2, wl))

    results = []
    for mesh, params, state in ((mesh1, params1, s1), (mesh2, params2, s2)):
        tend = og.ShallowWaterState(mesh, params)
        assert _noalloc(mesh, params, state, tend) == 0, \
            _capi.lib().swg_last_error()
        results.append((tend.download(), mesh, params, state))
    og.sync()
    for got, mesh, params, state in results:
        ref = _allocating(mesh, params, state)
        for a, b in zip(got, ref):
            assert rel_diff(a, b) <= TOL
    # and the golden tendency itself
    (th, tv, tt) = results[0][0]
    assert rel_diff(th, g["tend_h"]) <= TOL
    assert rel_diff(tv, g["tend_vn"]) <= TOL
    assert rel_diff(tt, g["tend_tr"]) <= TOL


def test_noalloc_increment_and_size_limit():
    g = load_golden("lsrk5_all_terms")
    cfg = g["cfg"]
    mesh, params = _setup(cfg)
    state = og.ShallowWaterState(mesh, params)
    state.upload(g["in_h"], g["in_vn"], g["in_tr"])
    tend = og.ShallowWaterState(mesh, params)
    assert _noalloc(mesh, params, state, tend, 0) == 0
    assert _noalloc(mesh, params, state, tend, 1) == 0
    th, tv, tt = tend.download()
    assert rel_diff(th, 2 * g["tend_h"]) <= TOL
    assert rel_diff(tv, 2 * g["tend_vn"]) <= TOL
    assert rel_diff(tt, 2 * g["tend_tr"]) <= TOL
    # 128x128 cells x 64 levels x 8 tracers needs far more than 64 MiB
    big = dict(nx=128, ny=128, dc=1e4, K=64, T=8, f0=1e-4, grav=9.81,
               visc_del2=1e3, visc_del4=1e9, eddy_diff2=1e3, eddy_diff4=1e9)
    mesh_b, params_b = _setup(big)
    sb = og.ShallowWaterState(mesh_b, params_b)
    tb = og.ShallowWaterState(mesh_b, params_b)
    rc = _noalloc(mesh_b, params_b, sb, tb)
    assert rc == 1
    msg = _capi.lib().swg_last_error().decode()
    assert "static maximum" in msg and "64 MiB" in msg
    h, vn, tr = tb.download()
    assert not h.any() and not vn.any() and not tr.any()


@pytest.mark.parametrize("name", ["h_frozen", "vn_frozen", "no_tracers",
                                  "del2_only", "del4_only", "tracer_del4_only",
                                  "inviscid", "many_tracers"])
def test_noalloc_enabled_sets(name):
    """Each enabled set (frozen fields, no tracers, single dissipation terms)
    in both add modes, against the allocating entry point."""
    from test_config_matrix_gpu import CONFIGS, state
    c = dict(CONFIGS[name])
    cfg = dict(nx=10, ny=8, dc=1e4, K=5, T=c.pop("T", 2),
               disable_h=c.pop("disable_h", False),
               disable_vn=c.pop("disable_vn", False),
               f0=c.get("f0", 0.0), grav=c.get("grav", 9.81),
               visc_del2=c.get("visc_del2", 0.0),
               visc_del4=c.get("visc_del4", 0.0),
               eddy_diff2=c.get("eddy_diff2", 0.0),
               eddy_diff4=c.get("eddy_diff4", 0.0))
    mesh, params = _setup(cfg)
    S = og.ShallowWaterState(mesh, params)
    S.upload(*state(mesh, cfg["T"], 23))
    ref = _allocating(mesh, params, S)
    tend = og.ShallowWaterState(mesh, params)
    assert _noalloc(mesh, params, S, tend, 0) == 0
    for a, b in zip(tend.download(), ref):
        assert rel_diff(a, b) <= TOL, name
    assert _noalloc(mesh, params, S, tend, 1) == 0
    for a, b in zip(tend.download(), ref):
        assert rel_diff(a, 2 * b) <= TOL, name


def test_noalloc_allocates_nothing_and_largest_documented_size():
    """The property the entry point exists for: a warm call on a mesh and
    parameter set it has not seen before leaves the device's free memory
    unchanged.  It runs at the size the header documents as fitting (64x64
    cells x 64 levels, one tracer, del2 viscosity), twice in a row, and each
    result equals swg_compute_tendency's."""
    # warm-up on another configuration: loads the module (and with it the
    # static array) and every kernel of the path
    g = load_golden("rk4_all_terms")
    mesh0, params0 = _setup(g["cfg"])
    s0 = og.ShallowWaterState(mesh0, params0)
    s0.upload(g["in_h"], g["in_vn"], g["in_tr"])
    t0 = og.ShallowWaterState(mesh0, params0)
    assert _noalloc(mesh0, params0, s0, t0) == 0
    og.sync()
    wl = WORKLOADS["rk4_64x64"]
    assert (wl.nx, wl.ny, wl.nlayers, wl.ntracers) == (64, 64, 64, 1)
    cfg = dict(nx=64, ny=64, dc=wl.dc, K=64, T=1, f0=wl.f0, grav=wl.grav,
               visc_del2=1e3, visc_del4=0.0, eddy_diff2=0.0, eddy_diff4=0.0)
    mesh, params = _setup(cfg)
    state = og.ShallowWaterState(mesh, params)
    state.upload(*initial_state(mesh, wl))
    tend = og.ShallowWaterState(mesh, params)
    og.sync()
    outs = []
    for call in range(2):
        before = _free_device_bytes()
        assert _noalloc(mesh, params, state, tend) == 0, \
            _capi.lib().swg_last_error()
        og.sync()
        assert _free_device_bytes() == before, f"call {call} allocated"
        outs.append(tend.download())
    ref = _allocating(mesh, params, state)
    for out in outs:
        for a, b in zip(out, ref):
            assert rel_diff(a, b) <= TOL
