"""Entry points that the other tests reach only indirectly: the RK4
shortcut swg_adjoint_create, state copy and fill, and the per-kernel
profiler (swg_profile_enable / swg_profile_read) that bench.py uses for its
kernel shares."""
import ctypes as C

import numpy as np
import pytest

import omega_playground_gb300 as og
from omega_playground_gb300 import _capi
from omega_playground_gb300.workloads import WORKLOADS, initial_state

pytestmark = pytest.mark.gpu

WL = WORKLOADS["lsrk5_512x512"].scaled(nx=10, ny=8, nlayers=4, ntracers=2)


def setup():
    mesh = og.PlanarHexagonalMesh(WL.nx, WL.ny, WL.dc, WL.nlayers)
    params = WL.params()
    return mesh, params, og.ShallowWaterModel(mesh, params)


def test_adjoint_create_is_the_rk4_adjoint():
    mesh, params, model = setup()
    x = initial_state(mesh, WL)
    h = C.c_void_p()
    _capi.check(_capi.lib().swg_adjoint_create(model.handle, 3, C.byref(h)))
    keep = og.Adjoint(model, 3, "rk4", 4)      # owns its handle
    results = []
    for handle in (h, keep.handle):
        X0 = og.ShallowWaterState(mesh, params)
        X0.upload(*x)
        XN = og.ShallowWaterState(mesh, params)
        _capi.check(_capi.lib().swg_adj_forward(handle, X0.handle, 0.0, WL.dt,
                                                7, XN.handle, None))
        L = og.ShallowWaterState(mesh, params)
        L.upload(*initial_state(mesh, WL.scaled(seed=WL.seed + 1)))
        _capi.check(_capi.lib().swg_adj_backward(handle, L.handle, None))
        results.append((XN.download(), L.download()))
    _capi.lib().swg_adjoint_destroy(h)
    for a, b in zip(results[0], results[1]):
        for u, v in zip(a, b):
            np.testing.assert_array_equal(u, v)


def test_state_copy_and_fill():
    mesh, params, _ = setup()
    x = initial_state(mesh, WL)
    A, B = og.ShallowWaterState(mesh, params), og.ShallowWaterState(mesh, params)
    A.upload(*x)
    B.copy_from(A)
    for u, v in zip(B.download(), x):
        np.testing.assert_array_equal(u, v)
    B.fill(2.5)
    for u in B.download():
        np.testing.assert_array_equal(u, 2.5)
    other = og.ShallowWaterState(og.PlanarHexagonalMesh(6, 6, 1e4, 4), params)
    with pytest.raises(og.SwgError):
        other.copy_from(A)                  # another mesh


def test_profiler_counts_the_passes_of_a_step():
    mesh, params, model = setup()
    S = og.ShallowWaterState(mesh, params)
    S.upload(*initial_state(mesh, WL))
    og.profile_read()                           # drop earlier records
    og.profile_enable(True)
    og.LSRKStepper(model, 5).step(S, 0.0, WL.dt, 2, use_graph=False)
    prof = og.profile_read()
    og.profile_enable(False)
    want = {"k_vertex", "k_cell1", "k_edge1", "k_aux2", "k_edge_final",
            "k_cell_final"}
    assert want <= set(prof), prof
    for k in want:
        ms, n = prof[k]
        assert n == 2 * 5 and ms > 0, (k, prof[k])
    assert og.profile_read() == {}              # read resets the records
