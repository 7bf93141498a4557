"""Host-resident states stepped in level chunks (swg_host_stepper_* /
og.HostStepper): bitwise equal to upload + swg_step + download on the same
model, for ragged chunkings, both steppers, pinned and pageable arrays,
general tables with a per-level edge mask, the linear model, the drag, the
model's term switches and f_vertex read at each call, and the full-size
512x512x64, 8-tracer workload."""
import numpy as np
import pytest

import omega_playground_gb300 as og
from omega_playground_gb300.workloads import WORKLOADS, initial_state

pytestmark = pytest.mark.gpu

WL = WORKLOADS["lsrk5_512x512"].scaled(nx=10, ny=8, nlayers=7, ntracers=2)


def device_run(model, mesh, params, x, kind, nstages, t0, dt, nsteps):
    S = og.ShallowWaterState(mesh, params)
    S.upload(*x)
    st = og.RK4Stepper(model) if kind == "rk4" else og.LSRKStepper(model,
                                                                   nstages)
    st.step(S, t0, dt, nsteps)
    return S.download()


def host_run(model, x, kind, nstages, chunk, t0, dt, nsteps, pinned=True):
    hs = og.HostStepper(model, kind, nstages, chunk)
    if pinned:
        arrs = hs.pinned_state()
        for a, b in zip(arrs, x):
            a[...] = b
    else:
        arrs = tuple(np.array(a, copy=True) for a in x)
    hs.step(*arrs, t0, dt, nsteps)
    return arrs, hs


def assert_bitwise(got, want):
    for g, w in zip(got, want):
        assert np.all(np.isfinite(w))
        np.testing.assert_array_equal(g, w)


@pytest.mark.parametrize("kind,nstages", [("rk4", 4), ("lsrk", 5),
                                          ("lsrk", 1)])
@pytest.mark.parametrize("chunk,want_chunks", [(0, [7]), (3, [3, 3, 1]),
                                               (1, [1] * 7), (7, [7]),
                                               (50, [7])])
def test_bitwise_equal_to_device_stepper(kind, nstages, chunk, want_chunks):
    mesh = og.PlanarHexagonalMesh(WL.nx, WL.ny, WL.dc, WL.nlayers)
    params = WL.params()
    model = og.ShallowWaterModel(mesh, params)
    x = initial_state(mesh, WL)
    want = device_run(model, mesh, params, x, kind, nstages, 5.0, WL.dt, 3)
    got, hs = host_run(model, x, kind, nstages, chunk, 5.0, WL.dt, 3)
    assert hs.chunks == want_chunks
    assert_bitwise(got, want)
    # a second call replays the chunks' graphs from the new host state
    want2 = device_run(model, mesh, params, want, kind, nstages, 5.0, WL.dt, 2)
    hs.step(*got, 5.0, WL.dt, 2)
    assert_bitwise(got, want2)


def test_explicit_chunk_sizes():
    mesh = og.PlanarHexagonalMesh(WL.nx, WL.ny, WL.dc, WL.nlayers)
    params = WL.params()
    model = og.ShallowWaterModel(mesh, params)
    x = initial_state(mesh, WL)
    want = device_run(model, mesh, params, x, "lsrk", 5, 0.0, WL.dt, 2)
    for levels in ([1, 5, 1], [2, 2, 3], [7]):
        hs = og.HostStepper(model, "lsrk", 5, levels=levels)
        assert hs.chunks == levels
        arrs = hs.pinned_state()
        for a, b in zip(arrs, x):
            a[...] = b
        hs.step(*arrs, 0.0, WL.dt, 2)
        assert_bitwise(arrs, want)
    for bad in ([3, 3], [4, 4], [0, 7], [-1, 8]):
        with pytest.raises(og.SwgError):
            og.HostStepper(model, "lsrk", 5, levels=bad)


def test_pageable_arrays_no_tracers_and_zero_steps():
    wl = WL.scaled(ntracers=0)
    mesh = og.PlanarHexagonalMesh(wl.nx, wl.ny, wl.dc, wl.nlayers)
    params = wl.params()
    model = og.ShallowWaterModel(mesh, params)
    x = initial_state(mesh, wl)
    want = device_run(model, mesh, params, x, "rk4", 4, 0.0, wl.dt, 4)
    got, hs = host_run(model, x, "rk4", 4, 2, 0.0, wl.dt, 4, pinned=False)
    assert_bitwise(got[:2], want[:2])
    before = tuple(a.copy() for a in got)
    hs.step(got[0], got[1], None, 0.0, wl.dt, 0)
    assert_bitwise(got[:2], before[:2])
    with pytest.raises(TypeError):
        hs.step(got[0].astype(np.float32), got[1], None, 0.0, wl.dt, 1)


def test_general_tables_with_edge_mask():
    from test_general_mesh_gpu import general_mesh, models, state
    om, gm = general_mesh(10, 8, 7, 919)
    T = 2
    _, gp, model = models(om, gm, T)
    x = state(om, T, 3)
    want = device_run(model, gm, gp, x, "lsrk", 5, 0.0, 5.0, 3)
    got, _ = host_run(model, x, "lsrk", 5, 3, 0.0, 5.0, 3)
    assert_bitwise(got, want)


def test_term_switches_and_f_vertex_are_read_at_each_call():
    mesh = og.PlanarHexagonalMesh(WL.nx, WL.ny, WL.dc, WL.nlayers)
    params = WL.params()
    model = og.ShallowWaterModel(mesh, params)
    x = initial_state(mesh, WL)
    hs = og.HostStepper(model, "lsrk", 5, 4)
    arrs = hs.pinned_state()
    for a, b in zip(arrs, x):
        a[...] = b
    hs.step(*arrs, 0.0, WL.dt, 1)                 # graphs captured, all on
    model.m_pv_flux_edge.m_enabled = False
    model.m_tracer_hyperdiff_cell.m_enabled = False
    f = model.m_f_vertex
    model.m_f_vertex = f * (1.0 + 0.1 * np.sin(np.arange(f.size)))
    for a, b in zip(arrs, x):
        a[...] = b
    hs.step(*arrs, 0.0, WL.dt, 3)
    want = device_run(model, mesh, params, x, "lsrk", 5, 0.0, WL.dt, 3)
    assert_bitwise(arrs, want)


def test_linear_model_and_drag():
    mesh = og.PlanarHexagonalMesh(WL.nx, WL.ny, WL.dc, WL.nlayers)
    lp = og.LinearShallowWaterParams(m_h0=1000.0, m_f0=1e-4, m_grav=9.81)
    lin = og.LinearShallowWaterModel(mesh, lp)
    x = initial_state(mesh, WL.scaled(ntracers=0))
    x = (x[0], x[1], np.zeros((0,) + x[0].shape))
    want = device_run(lin, mesh, og.ShallowWaterParams(), x, "rk4", 4, 0.0,
                      WL.dt, 3)
    got, _ = host_run(lin, x, "rk4", 4, 2, 0.0, WL.dt, 3)
    assert_bitwise(got[:2], want[:2])
    params = WL.params()
    params.m_drag_coeff = 2e-3
    drag = og.ShallowWaterModel(mesh, params, apply_drag=True)
    x = initial_state(mesh, WL)
    want = device_run(drag, mesh, params, x, "lsrk", 5, 0.0, WL.dt, 3)
    got, _ = host_run(drag, x, "lsrk", 5, 2, 0.0, WL.dt, 3)
    assert_bitwise(got, want)


def test_hooked_model_is_rejected():
    mesh = og.PlanarHexagonalMesh(6, 6, 1e4, 2)
    params = og.ShallowWaterParams(m_f0=1e-4)

    class Forced(og.ShallowWaterModel):
        def additional_tendency(self, h_tend, vn_tend, h, vn, t, stream):
            pass

    with pytest.raises(og.SwgError, match="forcing hook"):
        og.HostStepper(Forced(mesh, params), "rk4", 4, 1)


def test_full_size_workload_one_step():
    wl = WORKLOADS["lsrk5_512x512"]
    mesh = og.PlanarHexagonalMesh(wl.nx, wl.ny, wl.dc, wl.nlayers)
    params = wl.params()
    model = og.ShallowWaterModel(mesh, params)
    x = initial_state(mesh, wl)
    want = device_run(model, mesh, params, x, "lsrk", 5, 0.0, wl.dt, 1)
    got, hs = host_run(model, x, "lsrk", 5, 16, 0.0, wl.dt, 1)
    assert hs.chunks == [16] * 4
    assert_bitwise(got, want)


def test_autotuned_picks_a_timed_candidate_and_leaves_the_state():
    mesh = og.PlanarHexagonalMesh(WL.nx, WL.ny, WL.dc, WL.nlayers)
    params = WL.params()
    model = og.ShallowWaterModel(mesh, params)
    x = initial_state(mesh, WL)
    keep = tuple(a.copy() for a in x)
    hs, table = og.HostStepper.autotuned(model, "lsrk", 5, x, WL.dt,
                                         candidates=(0, 4, 2, 50, [1, 5, 1]))
    assert set(table) == {"7", "4,3", "2,2,2,1", "1,5,1"}
    best = min(table, key=table.get)
    assert hs.chunks == [int(n) for n in best.split(",")]
    assert_bitwise(x, keep)
    want = device_run(model, mesh, params, x, "lsrk", 5, 0.0, WL.dt, 2)
    arrs = hs.pinned_state()
    for a, b in zip(arrs, x):
        a[...] = b
    hs.step(*arrs, 0.0, WL.dt, 2)
    assert_bitwise(arrs, want)


def test_call_graph_cache():
    """With page-locked arrays each call of up to 4 steps replays one
    captured graph of the whole call, cached per array set, dt, step count
    and term version.  Six array sets used in turn twice (the cache holds
    four), a term switched between two one-step calls on the same arrays, a
    new dt and a call of more steps than the cache takes (direct launches)
    all equal the device stepper bit for bit, and a replay counts the same
    kernels as the call that captured it."""
    mesh = og.PlanarHexagonalMesh(WL.nx, WL.ny, WL.dc, WL.nlayers)
    params = WL.params()
    model = og.ShallowWaterModel(mesh, params)
    x = initial_state(mesh, WL)
    hs = og.HostStepper(model, "lsrk", 5, 3)
    rng = np.random.default_rng(17)
    sets, starts = [], []
    for _ in range(6):
        arrs = hs.pinned_state()
        x0 = [x[0] * (1 + 1e-3 * rng.standard_normal(x[0].shape)),
              x[1] + 0.01 * rng.standard_normal(x[1].shape), x[2].copy()]
        for a, b in zip(arrs, x0):
            a[...] = b
        sets.append(arrs)
        starts.append(x0)
    # six array sets, two rounds: the second round's sets were evicted
    # from the cache, or (the last four) replay their captured call
    for rnd in range(2):
        for arrs in sets:
            n0 = og.kernel_launches()
            hs.step(*arrs, 0.0, WL.dt, 2)
            n1 = og.kernel_launches()
            hs.step(*arrs, 2 * WL.dt, WL.dt, 2)
            assert og.kernel_launches() - n1 == n1 - n0 > 0
    for arrs, x0 in zip(sets, starts):
        want = device_run(model, mesh, params, x0, "lsrk", 5, 0.0, WL.dt, 8)
        assert_bitwise(arrs, want)
    # a term switched between two one-step calls on the same arrays
    arrs, x0 = sets[0], starts[0]
    for a, b in zip(arrs, x0):
        a[...] = b
    hs.step(*arrs, 0.0, WL.dt, 1)
    model.m_ke_grad_edge.m_enabled = False
    hs.step(*arrs, WL.dt, WL.dt, 1)
    model.m_ke_grad_edge.m_enabled = True
    S = og.ShallowWaterState(mesh, params)
    S.upload(*x0)
    st = og.LSRKStepper(model, 5)
    st.step(S, 0.0, WL.dt, 1)
    model.m_ke_grad_edge.m_enabled = False
    st.step(S, WL.dt, WL.dt, 1)
    model.m_ke_grad_edge.m_enabled = True
    assert_bitwise(arrs, S.download())
    # a new dt, then more steps per call than the cache takes
    for a, b in zip(arrs, x0):
        a[...] = b
    hs.step(*arrs, 0.0, 0.5 * WL.dt, 1)
    hs.step(*arrs, 0.5 * WL.dt, WL.dt, 6)
    S.upload(*x0)
    st.step(S, 0.0, 0.5 * WL.dt, 1)
    st.step(S, 0.5 * WL.dt, WL.dt, 6)
    assert_bitwise(arrs, S.download())
