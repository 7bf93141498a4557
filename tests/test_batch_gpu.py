"""Batched ensembles: every member advanced in a batch (one persistent
kernel per RK stage, or one launch per pass, in every launch configuration)
is bitwise equal to the same member advanced alone by the single-instance
stepper, which is itself checked against the oracle elsewhere."""
import numpy as np
import pytest

import omega_playground_gb300 as og
from omega_playground_gb300.workloads import ensemble, initial_state

pytestmark = pytest.mark.gpu


def build_members(wls):
    out = []
    for wl in wls:
        mesh = og.PlanarHexagonalMesh(wl.nx, wl.ny, wl.dc, wl.nlayers)
        params = wl.params()
        model = og.ShallowWaterModel(mesh, params)
        ic = initial_state(mesh, wl)
        out.append((mesh, params, model, ic))
    return out


def run_single(members, wls, kind, nstages, nsteps):
    res = []
    for (mesh, params, model, ic), wl in zip(members, wls):
        st = og.ShallowWaterState(mesh, params)
        st.upload(*ic)
        stp = og.RK4Stepper(model) if kind == "rk4" else og.LSRKStepper(model, nstages)
        stp.step(st, 0.0, wl.dt, nsteps, use_graph=False)
        res.append(st.download())
    return res


def run_batch(members, wls, kind, nstages, nsteps, config=None, use_graph=False):
    states = []
    for mesh, params, model, ic in members:
        st = og.ShallowWaterState(mesh, params)
        st.upload(*ic)
        states.append(st)
    b = og.Batch([m[2] for m in members], states, kind, nstages)
    if config is not None:
        b.set_config(config)
    b.step(0.0, wls[0].dt, nsteps, use_graph=use_graph)
    return [s.download() for s in states], b


SMALL = ensemble(n=6, nx_choices=(8, 12, 16), levels=(16, 40), tracers=(1, 4))


@pytest.mark.parametrize("kind,nstages", [("rk4", 4), ("lsrk", 5)])
def test_every_config_matches_single_instance_bitwise(kind, nstages):
    members = build_members(SMALL)
    ref = run_single(members, SMALL, kind, nstages, 3)
    for cfg in range(og.Batch.config_count()):
        got, _ = run_batch(members, SMALL, kind, nstages, 3, config=cfg)
        for m, (a, b) in enumerate(zip(got, ref)):
            for x, y in zip(a, b):
                np.testing.assert_array_equal(x, y, err_msg=f"config {cfg} member {m}")


def test_graph_replay_matches_direct():
    members = build_members(SMALL)
    a, _ = run_batch(members, SMALL, "rk4", 4, 4, use_graph=False)
    b, _ = run_batch(members, SMALL, "rk4", 4, 4, use_graph=True)
    for x, y in zip(a, b):
        for u, v in zip(x, y):
            np.testing.assert_array_equal(u, v)


def test_ensemble64_members_match_single_instance():
    """64 members with the ensemble's distribution of levels (16-96) and
    tracers (1-4) on smaller meshes, two RK4 steps, after autotuning."""
    wls = ensemble(n=64, nx_choices=(8, 12, 16, 24, 32, 48))
    members = build_members(wls)
    ref = run_single(members, wls, "rk4", 4, 2)
    states = []
    for mesh, params, model, ic in members:
        st = og.ShallowWaterState(mesh, params)
        states.append(st)
    for st, (mesh, params, model, ic) in zip(states, members):
        st.upload(*ic)
    b = og.Batch([m[2] for m in members], states, "rk4", 4)
    cfg, ms = b.autotune(wls[0].dt, reps=1)
    assert 0 <= cfg < og.Batch.config_count() and ms > 0
    for st, (mesh, params, model, ic) in zip(states, members):
        st.upload(*ic)
    b.step(0.0, wls[0].dt, 2, use_graph=True)
    for m, (st, r) in enumerate(zip(states, ref)):
        for x, y in zip(st.download(), r):
            np.testing.assert_array_equal(x, y, err_msg=f"member {m}")


def test_ensemble64_full_size_workload_matches_single_instance():
    """The 64-member ensemble workload at full size (nx in {32..192}, 16-96
    levels, 1-4 tracers; 32.5 M cell-levels), two RK4 steps with the
    autotuned configuration, every member bitwise equal to its own
    single-instance run."""
    wls = ensemble()
    members = build_members(wls)
    ref = run_single(members, wls, "rk4", 4, 2)
    states = [og.ShallowWaterState(m[0], m[1]) for m in members]
    b = og.Batch([m[2] for m in members], states, "rk4", 4)
    for st, m in zip(states, members):
        st.upload(*m[3])
    b.autotune(wls[0].dt, reps=1)
    for st, m in zip(states, members):
        st.upload(*m[3])
    b.step(0.0, wls[0].dt, 2, use_graph=True)
    for i, (st, r) in enumerate(zip(states, ref)):
        for x, y in zip(st.download(), r):
            np.testing.assert_array_equal(x, y, err_msg=f"member {i}")


def test_barrier_wait_limit_reports_timeout_and_context_survives():
    members = build_members(SMALL[:2])
    got, b = run_batch(members, SMALL[:2], "rk4", 4, 1)
    assert b.selftest_timeout(50.0) == 4  # SWG_ERR_TIMEOUT
    b.check()  # status cleared
    # the context is still usable: the batch steps and matches again
    ref = run_single(members, SMALL[:2], "rk4", 4, 2)
    got2, _ = run_batch(members, SMALL[:2], "rk4", 4, 2)
    for x, y in zip(got2, ref):
        for u, v in zip(x, y):
            np.testing.assert_array_equal(u, v)


def test_batch_rejects_hooked_members():
    class Forced(og.ShallowWaterModel):
        def additional_tendency(self, *a):
            pass
    mesh = og.PlanarHexagonalMesh(8, 8, 1e4, 4)
    params = og.ShallowWaterParams(m_f0=1e-4)
    st = og.ShallowWaterState(mesh, params)
    with pytest.raises(og.SwgError):
        og.Batch([Forced(mesh, params)], [st])


def test_batch_rejects_shared_models_and_states():
    """Members run concurrently, so a model (its intermediates) or a state
    shared by two members would be written by both: refused on the host."""
    mesh = og.PlanarHexagonalMesh(8, 8, 1e4, 4)
    params = og.ShallowWaterParams(m_f0=1e-4)
    model = og.ShallowWaterModel(mesh, params)
    other = og.ShallowWaterModel(mesh, params)
    a, b = og.ShallowWaterState(mesh, params), og.ShallowWaterState(mesh, params)
    with pytest.raises(og.SwgError):
        og.Batch([model, model], [a, b])
    with pytest.raises(og.SwgError):
        og.Batch([model, other], [a, a])
    og.Batch([model, other], [a, b])  # distinct members are fine


def test_tiny_members_match_single_instance_bitwise():
    """The smallest meshes as members (one column of cells, each cell its own
    east and west neighbour; an odd 2x3 mesh; one level, no tracers) beside
    a regular one, in every launch configuration."""
    from omega_playground_gb300.workloads import WORKLOADS
    base = WORKLOADS["lsrk5_512x512"]
    wls = [base.scaled(nx=1, ny=2, nlayers=1, ntracers=0, seed=71),
           base.scaled(nx=2, ny=3, nlayers=3, ntracers=2, seed=72),
           base.scaled(nx=1, ny=1, nlayers=5, ntracers=1, seed=73),
           base.scaled(nx=8, ny=6, nlayers=33, ntracers=3, seed=74)]
    members = build_members(wls)
    ref = run_single(members, wls, "lsrk", 5, 3)
    assert all(np.all(np.isfinite(x)) for r in ref for x in r)
    for cfg in range(og.Batch.config_count()):
        got, _ = run_batch(members, wls, "lsrk", 5, 3, config=cfg)
        for m, (a, b) in enumerate(zip(got, ref)):
            for x, y in zip(a, b):
                np.testing.assert_array_equal(x, y, err_msg=f"config {cfg} member {m}")


def test_term_switch_after_first_batch_step_is_followed():
    """A member's model switches terms between batch steps (the reference's
    m_enabled members): the batch takes the new set at its next step, graph
    path included, bitwise equal to the single-instance stepper doing the
    same."""
    members = build_members(SMALL)
    states = []
    for mesh, params, model, ic in members:
        st = og.ShallowWaterState(mesh, params)
        st.upload(*ic)
        states.append(st)
    b = og.Batch([m[2] for m in members], states, "rk4", 4)
    b.step(0.0, SMALL[0].dt, 2)
    singles = []
    for mesh, params, model, ic in members:
        st = og.ShallowWaterState(mesh, params)
        st.upload(*ic)
        og.RK4Stepper(model).step(st, 0.0, SMALL[0].dt, 2, use_graph=False)
        singles.append(st)
    m1 = members[1][2]
    m1.m_pv_flux_edge.m_enabled = False
    m1.m_tracer_hadv_cell.m_enabled = False
    members[3][2].m_vel_diff_edge.m_enabled = False
    b.step(0.0, SMALL[0].dt, 3)
    for (mesh, params, model, ic), st in zip(members, singles):
        og.RK4Stepper(model).step(st, 0.0, SMALL[0].dt, 3, use_graph=False)
    for m, (a, s) in enumerate(zip(states, singles)):
        for x, y in zip(a.download(), s.download()):
            assert np.all(np.isfinite(y))
            np.testing.assert_array_equal(x, y, err_msg=f"member {m}")
    # and back on
    m1.m_pv_flux_edge.m_enabled = True
    b.step(0.0, SMALL[0].dt, 1)
    og.RK4Stepper(m1).step(singles[1], 0.0, SMALL[0].dt, 1, use_graph=False)
    for x, y in zip(states[1].download(), singles[1].download()):
        np.testing.assert_array_equal(x, y)
